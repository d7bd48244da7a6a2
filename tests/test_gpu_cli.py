"""The command-line tool end to end on the GPU: a delimited file of the C1 Swiss
roll (one point per line, then transposed), KLLE with k = 12, and the written
embedding against the oracle's dense FP64 embedding of the same file data
(principal angles <= 1e-4 rad)."""
import numpy as np
import pytest

from oracle import oracle
from tapkee_gb300 import cli, datasets, io

pytestmark = pytest.mark.gpu


def _angles(A, B):
    qa, _ = np.linalg.qr(A - A.mean(0))
    qb, _ = np.linalg.qr(B - B.mean(0))
    return np.arccos(np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False), -1.0, 1.0))


@pytest.mark.parametrize("transposed", [False, True])
def test_cli_lle_embedding(ctx, tmp_path, transposed):
    X = datasets.swiss_roll(2000, seed=0)
    src = tmp_path / "roll.csv"
    io.write_matrix(str(src), X.T if transposed else X, ";")
    out = tmp_path / "emb.csv"
    args = ["-i", str(src), "-o", str(out), "-d", ";", "-m", "lle", "-k", "12", "-td", "2", "-em", "dense"]
    if transposed:
        args += ["--transpose-input", "--transpose-output"]
    assert cli.main(args) == 0
    E = io.read_data(str(out), ";")
    E = E.T if transposed else E
    assert E.shape == (2000, 2)
    Xf = io.as_points(io.read_data(str(src), ";"), transposed=transposed)  # the data as the file holds it
    idx, k = oracle.find_neighbors(Xf, 12)
    rp, col, vals = oracle.assemble(0, idx, oracle.lle_weights(Xf, idx, 1e-3), 1e-9)
    E_ref, _ = oracle.dense_embedding(rp, col, vals, 2)
    assert _angles(E, E_ref).max() < 1e-4
