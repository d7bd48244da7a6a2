"""Delimiter-separated matrix files (src/cli/util.hpp:73-130 semantics)."""
import numpy as np
import pytest

from tapkee_gb300 import io as tkio


def test_round_trip_and_layout(tmp_path):
    rng = np.random.default_rng(0)
    X = rng.normal(size=(7, 3))
    p = tmp_path / "x.csv"
    tkio.write_matrix(p, X)
    lines = p.read_text().splitlines()
    assert len(lines) == 7 and all(len(l.split(",")) == 3 for l in lines)
    back = tkio.read_data(p)
    assert back.shape == (7, 3)
    assert np.allclose(back, X, rtol=1e-5, atol=1e-6)  # 6 significant digits, like a C++ stream
    assert tkio.as_points(back).shape == (7, 3)
    assert tkio.as_points(back, transposed=True).shape == (3, 7)
    assert tkio.from_embedding(back, transposed=True).shape == (3, 7)


def test_reader_leniency_and_errors(tmp_path):
    p = tmp_path / "m.txt"
    # blank lines are skipped; a field that does not parse (including inf / nan,
    # which istream >> double rejects) is dropped; a field keeps its leading number
    p.write_text("1;2;3\n\n4;x;5;6\n7e-1;8abc; 9\ninf;-2.5;nan;1;+3\n")
    m = tkio.read_data(p, delimiter=";")
    assert m.shape == (4, 3)
    assert np.array_equal(m, [[1, 2, 3], [4, 5, 6], [0.7, 8, 9], [-2.5, 1, 3]])
    p.write_text("1,2,3\n4,5\n")
    with pytest.raises(ValueError, match="Wrong data at line 1"):
        tkio.read_data(p)
    p.write_text("\n\n")
    assert tkio.read_data(p).shape == (0, 0)


def test_writer_format(tmp_path):
    p = tmp_path / "w.txt"
    tkio.write_matrix(p, [[1.0, 0.1234567, 1e-7], [123456789.0, -np.inf, 2.0]], delimiter=" ")
    assert p.read_text() == "1 0.123457 1e-07\n1.23457e+08 -inf 2\n"
