"""The command-line tool's argument checks (tapkee_gb300.cli, in the shape of
src/cli/main.cpp:351-422): CPU only, nothing reaches the GPU."""
import pytest

from tapkee_gb300 import cli


@pytest.mark.parametrize("args,msg", [
    (["-m", "isomapp"], "Unknown method isomapp"),
    (["-nm", "kdtree"], "Unknown neighbors method kdtree"),
    (["-nm", "covertree"], "not provided by this library"),
    (["-em", "lapack"], "Unknown eigendecomposition method lapack"),
    (["-em", "randomized"], "not provided by this library"),
    (["-td", "0"], "positive target dimensionality"),
    (["-k", "2"], "The provided number of neighbors is too small, consider at least 3."),
])
def test_cli_rejections(tmp_path, capsys, args, msg):
    f = tmp_path / "in.csv"
    f.write_text("1,2,3\n4,5,6\n")
    assert cli.main(["-i", str(f), "-o", str(tmp_path / "out.csv")] + args) == 1
    assert msg in capsys.readouterr().err
    assert not (tmp_path / "out.csv").exists()


def test_cli_defaults_match_the_reference_tool():
    a = cli.parser().parse_args([])
    assert (a.input_file, a.output_file, a.delimiter) == ("/dev/stdin", "/dev/stdout", ",")
    assert (a.method, a.target_dimension, a.num_neighbors, a.eigenshift) == ("locally_linear_embedding", 2, 10, 1e-9)
