"""NPE / LLTSA dense eigenproblem pair (routines/locally_linear.hpp:257-338).

CPU: the oracle's restatement against a numpy statement of the same algebra.
GPU: tk_eigenproblem_pair against the oracle on the operators of the C1-style
workloads, float32 and float64 input; the sums run in a different order, so
the bar is 1e-10 relative to the largest entry."""
import numpy as np
import pytest

from oracle import oracle
from tapkee_gb300 import datasets


def _numpy_pair(kind, X, rp, col, vals):
    import scipy.sparse as sp
    X = np.asarray(X, np.float64)
    N, D = X.shape
    M = sp.csr_matrix((vals, col, rp), shape=(N, N))
    XMX = X.T @ (M @ X)
    s = X.sum(0)
    L = XMX + XMX.T
    R = X.T @ X
    if kind == 1:
        L = L - np.outer(s, s) / N
        R = R - np.outer(s, s) / N
    L = np.triu(L)
    U = np.triu(R)
    return L, (U + U.T) / 2


@pytest.mark.parametrize("kind", [0, 1])
def test_oracle_pair_matches_numpy(kind):
    rng = np.random.default_rng(3)
    N, D, k = 300, 5, 6
    X = rng.normal(size=(N, D))
    idx, _, _ = oracle.knn_brute(X, k)
    if kind == 0:
        w = oracle.lle_weights(X, idx, 1e-3)
    else:
        w = oracle.ltsa_basis(X, idx, 2)
    rp, col, vals = oracle.assemble(kind, idx, w, 1e-9)
    L, R = oracle.eigenproblem_pair(kind, X, rp, col, vals)
    Ln, Rn = _numpy_pair(kind, X, rp, col, vals)
    assert np.abs(L - Ln).max() <= 1e-11 * np.abs(Ln).max()
    assert np.abs(R - Rn).max() <= 1e-11 * np.abs(Rn).max()
    assert np.all(np.tril(L, -1) == 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,dtype", [("npe", np.float64), ("npe", np.float32), ("lltsa", np.float32)])
def test_gpu_pair_matches_oracle(ctx, kind, dtype):
    if kind == "npe":
        X = datasets.lifted_swiss_roll(3000, 16, seed=4, dtype=dtype)
        op = ctx.local_operator(X, "lle", num_neighbors=12, klle_shift=1e-3, check_connectivity=False)
    else:
        X = datasets.lifted_s_curve(2500, 32, seed=9, dtype=dtype)
        op = ctx.local_operator(X, "ltsa", num_neighbors=14, target_dimension=2, check_connectivity=False)
    L, R = ctx.eigenproblem_pair(kind, X, op.row_ptr, op.col_idx, op.vals)
    Lr, Rr = oracle.eigenproblem_pair(0 if kind == "npe" else 1, X.astype(np.float64), op.row_ptr, op.col_idx,
                                      op.vals)
    assert np.abs(L - Lr).max() <= 1e-10 * np.abs(Lr).max()
    assert np.abs(R - Rr).max() <= 1e-10 * np.abs(Rr).max()
    assert np.all(np.tril(L, -1) == 0.0)


@pytest.mark.gpu
def test_gpu_pair_device_inputs_and_wide_d(ctx):
    torch = pytest.importorskip("torch")
    X = datasets.lifted_swiss_roll(2000, 96, seed=2)
    op = ctx.local_operator(X, "lle", num_neighbors=10, klle_shift=1e-3, check_connectivity=False)
    Xd = torch.from_numpy(X).cuda()
    L, R = ctx.eigenproblem_pair("npe", Xd, torch.from_numpy(op.row_ptr).cuda(), torch.from_numpy(op.col_idx).cuda(),
                                 torch.from_numpy(op.vals).cuda())
    Lr, Rr = oracle.eigenproblem_pair(0, X.astype(np.float64), op.row_ptr, op.col_idx, op.vals)
    assert np.abs(L - Lr).max() <= 1e-10 * np.abs(Lr).max()
    assert np.abs(R - Rr).max() <= 1e-10 * np.abs(Rr).max()


@pytest.mark.gpu
def test_gpu_pair_rejects_bad_row_pointers(ctx):
    import tapkee_gb300 as tk
    X = datasets.swiss_roll(500, seed=3)
    op = ctx.local_operator(X, "lle", num_neighbors=8, klle_shift=1e-3)
    rp_bad = op.row_ptr.copy()
    rp_bad[20], rp_bad[21] = rp_bad[21], rp_bad[20]
    with pytest.raises(tk.WrongParameterError, match="index out of range"):
        ctx.eigenproblem_pair("npe", X, rp_bad, op.col_idx, op.vals)
    L, _ = ctx.eigenproblem_pair("npe", X, op.row_ptr, op.col_idx, op.vals)  # the context stays usable
    assert L.shape == (3, 3)
