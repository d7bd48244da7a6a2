"""Hessian LLE on the GPU (hessian_weight_matrix, routines/locally_linear.hpp:161-255)
against the oracle, through the C ABI.

Tolerances: the blocks B = Yr Yr^T within 1e-5 of the oracle's FP64 blocks (max
|err| / max |B|); M's CSR structure equal, values within 1e-5; the embedding
within 1e-4 rad (principal angles) of the committed golden embedding."""
import numpy as np
import pytest

from oracle import oracle
from tapkee_gb300 import datasets

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _blocks(Y):
    return np.einsum("naq,nbq->nab", Y, Y)


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def _angles(A, B):
    qa, _ = np.linalg.qr(A - A.mean(0))
    qb, _ = np.linalg.qr(B - B.mean(0))
    s = np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False), -1.0, 1.0)
    return np.arccos(s)


def test_hessian_blocks_golden_s_curve(ctx, golden):
    X = datasets.lifted_s_curve(1500, d=8, seed=11, noise=0.02, dtype=np.float64)
    idx = golden["ltsa_idx_oracle_order"]
    Y = ctx.hessian_basis(X, idx, 2)
    assert Y.shape == (1500, 12, 3)
    B = _blocks(Y)
    ref = oracle.hessian_blocks(X, idx, 2)
    assert _rel(B, ref) < TOL, _rel(B, ref)
    assert _rel(B[:64], golden["hlle_B"]) < TOL
    # each block is an orthogonal projector of rank dp = 3
    assert np.abs(np.einsum("nab,nbc->nac", B, B) - B).max() < 1e-6
    np.testing.assert_allclose(np.trace(B, axis1=1, axis2=2), 3.0, atol=1e-6)


@pytest.mark.parametrize("n,d,k,td,dtype", [(3000, 32, 20, 2, np.float32), (2000, 16, 12, 1, np.float32),
                                            (1200, 8, 30, 2, np.float64), (1500, 64, 48, 2, np.float32),
                                            (1500, 64, 64, 2, np.float32), (900, 16, 40, 1, np.float64)])
def test_hessian_blocks_lifted(ctx, n, d, k, td, dtype):
    X = datasets.lifted_s_curve(n, d, seed=n + k, noise=0.02, dtype=dtype)
    idx, _, _ = oracle.knn_brute(X, k)
    B = _blocks(ctx.hessian_basis(X, idx, td))
    ref = oracle.hessian_blocks(X, idx, td)
    assert _rel(B, ref) < TOL, _rel(B, ref)


def test_hessian_assembly_and_embedding(ctx, golden):
    X = datasets.lifted_s_curve(1500, d=8, seed=11, noise=0.02, dtype=np.float64)
    idx = golden["ltsa_idx_oracle_order"]
    Y = ctx.hessian_basis(X, idx, 2)
    rp, col, vals = ctx.assemble("hlle", idx, Y, 0.0)
    rr, rc, rv = oracle.assemble(2, idx, oracle.hessian_blocks(X, idx, 2), 0.0)
    assert np.array_equal(rp, rr) and np.array_equal(col, rc)
    assert _rel(vals, rv) < TOL
    assert int(rp[-1]) == int(golden["hlle_nnz"])
    # the whole stage (kNN on the GPU, rows in (distance, index) order) and the
    # dense FP64 embedding of its M
    op = ctx.local_operator(X, "hlle", num_neighbors=12, target_dimension=2, check_connectivity=False)
    assert op.weights.shape == (1500, 12, 3)
    assert np.array_equal(op.row_ptr, rr) and np.array_equal(op.col_idx, rc)
    assert _rel(op.vals, rv) < TOL
    E, _ = oracle.dense_embedding(op.row_ptr, op.col_idx, op.vals, 2)
    assert _angles(E, golden["hlle_embedding"]).max() < 1e-4


def test_hessian_rejections(ctx):
    import tapkee_gb300 as tk
    X = datasets.lifted_s_curve(400, 8, seed=1, noise=0.02)
    idx, _, _ = oracle.knn_brute(X, 12)
    with pytest.raises(tk.UnsupportedMethodError, match="target_dimension 1 or 2"):
        ctx.hessian_basis(X, idx, 3)
    with pytest.raises(tk.WrongParameterError):
        ctx.hessian_basis(X, idx[:, :5], 2)  # k must exceed td + td (td + 1) / 2
    bad = idx.copy()
    bad[7, 2] = 400
    with pytest.raises(tk.WrongParameterError, match="index out of range"):
        ctx.hessian_basis(X, bad, 2)
