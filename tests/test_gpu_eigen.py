"""tk_smallest_eigenvectors (the GPU eigensolver on the CSR of M) against the
oracle's dense eigendecomposition of the same matrix
(routines/eigendecomposition.hpp:56-87, columns skip..skip+td): principal angles
of the embedding subspace <= 1e-4, eigenvalues to 1e-6 relative. Plus its
argument checks, the non-convergence status, host/device pointer agreement and
run-to-run identity."""
import numpy as np
import pytest

import tapkee_gb300 as tk
from oracle import oracle
from tapkee_gb300 import datasets

pytestmark = pytest.mark.gpu

ANGLE_TOL = 1e-4
# eigenvalues: 1e-6 relative, plus the rounding of the float-float products with
# M (about 2^-46 of the row sums |M| |x|), 1e-14 x the spectrum bound
VALUE_RTOL = 1e-6
VALUE_ATOL_OF_BOUND = 1e-14


def _angles(A, B):
    qa, _ = np.linalg.qr(A)
    qb, _ = np.linalg.qr(B)
    return np.arccos(np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False), -1, 1))


def _dense(rp, col, vals, td, skip):
    N = len(rp) - 1
    M = np.zeros((N, N))
    for r in range(N):
        M[r, col[rp[r]:rp[r + 1]]] = vals[rp[r]:rp[r + 1]]
    w, V = np.linalg.eigh((M + M.T) / 2)
    return V[:, skip:skip + td], w[skip:skip + td], w


def _check_against_dense(E, lam, rp, col, vals, td, skip):
    Ed, wd, w = _dense(rp, col, vals, td, skip)
    assert E.shape == (len(rp) - 1, td)
    assert _angles(E, Ed).max() < ANGLE_TOL
    bound = np.abs(w).max()
    assert np.all(np.abs(lam - wd) <= VALUE_RTOL * np.abs(wd) + VALUE_ATOL_OF_BOUND * bound)
    # each vector: unit norm, entry of largest magnitude positive
    assert np.allclose(np.linalg.norm(E, axis=0), 1.0, atol=1e-10)
    for c in range(td):
        assert E[np.argmax(np.abs(E[:, c])), c] > 0


def test_lle_c1_matches_dense_oracle(ctx):
    X = datasets.swiss_roll(2000, seed=0)
    op = ctx.local_operator(X, "lle", num_neighbors=12, klle_shift=1e-3)
    E, lam, info = ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 2, 1, return_info=True)
    assert info["converged"] and info["block"] == 32
    assert info["max_residual"] <= 1e-12 * info["spectrum_bound"]
    _check_against_dense(E, lam, op.row_ptr, op.col_idx, op.vals, 2, 1)
    # the same as the dense path of the Python helper and of the oracle
    Eo, _ = oracle.dense_embedding(op.row_ptr, op.col_idx, op.vals, 2)
    assert _angles(E, Eo).max() < ANGLE_TOL


def test_ltsa_matches_dense_oracle(ctx):
    X = datasets.lifted_s_curve(1500, d=8, seed=11, noise=0.02, dtype=np.float64)
    op = ctx.local_operator(X, "ltsa", num_neighbors=12, target_dimension=2)
    E, lam = ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 2, 1)
    _check_against_dense(E, lam, op.row_ptr, op.col_idx, op.vals, 2, 1)


def test_wide_block_and_other_skip(ctx):
    # td + skip = 7 (more wanted pairs); skip = 0 keeps the null vector
    X = datasets.lifted_s_curve(1200, d=6, seed=5, noise=0.02, dtype=np.float64)
    op = ctx.local_operator(X, "ltsa", num_neighbors=10, target_dimension=2)
    E, lam, info = ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 6, 1, return_info=True)
    assert info["block"] == 32
    _, _, w = _dense(op.row_ptr, op.col_idx, op.vals, 6, 1)
    assert w[7] - w[6] > 1e-3 * (w[7] - w[0])  # a clean gap after the wanted pairs
    _check_against_dense(E, lam, op.row_ptr, op.col_idx, op.vals, 6, 1)
    E0, lam0 = ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 2, 0)
    _check_against_dense(E0, lam0, op.row_ptr, op.col_idx, op.vals, 2, 0)


def test_host_and_device_pointers_agree_and_repeat(ctx):
    torch = pytest.importorskip("torch")
    X = datasets.swiss_roll(1500, seed=4)
    op = ctx.local_operator(X, "lle", num_neighbors=10)
    E1, l1 = ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 2, 1)
    E2, l2 = ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 2, 1)
    assert np.array_equal(E1, E2) and np.array_equal(l1, l2)
    Ed, ld = ctx.smallest_eigenvectors(torch.from_numpy(op.row_ptr).cuda(), torch.from_numpy(op.col_idx).cuda(),
                                       torch.from_numpy(op.vals).cuda(), 2, 1)
    assert Ed.is_cuda
    assert np.array_equal(Ed.cpu().numpy(), E1) and np.array_equal(ld.cpu().numpy(), l1)


def test_argument_errors_and_non_convergence(ctx):
    X = datasets.swiss_roll(600, seed=2)
    op = ctx.local_operator(X, "lle", num_neighbors=8)
    with pytest.raises(tk.UnsupportedMethodError):
        ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 14, 1)
    with pytest.raises(tk.WrongParameterError):
        ctx.smallest_eigenvectors(op.row_ptr[:41], op.col_idx[:op.row_ptr[40]], op.vals[:op.row_ptr[40]], 2, 1)
    with pytest.raises(tk.WrongParameterError):
        ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 0, 1)
    with pytest.raises(tk.EigendecompositionError):
        ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 2, 1, max_matvecs=3)
    # a column index outside [0, N) is reported (as a bad argument), not read
    bad = op.col_idx.copy()
    bad[5] = len(op.row_ptr) + 3
    with pytest.raises(tk.WrongParameterError, match="index out of range"):
        ctx.smallest_eigenvectors(op.row_ptr, bad, op.vals, 2, 1)
    # row pointers that go backwards or past row_ptr[N] are rejected before any gather
    rp_bad = op.row_ptr.copy()
    rp_bad[10], rp_bad[11] = rp_bad[11], rp_bad[10]
    with pytest.raises(tk.WrongParameterError, match="index out of range"):
        ctx.smallest_eigenvectors(rp_bad, op.col_idx, op.vals, 2, 1)
    rp_bad = op.row_ptr.copy()
    rp_bad[7] = rp_bad[-1] + 100
    with pytest.raises(tk.WrongParameterError, match="index out of range"):
        ctx.smallest_eigenvectors(rp_bad, op.col_idx, op.vals, 2, 1)
    # the context stays usable
    E, _ = ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 2, 1)
    assert E.shape == (600, 2)


def test_default_embed_uses_sparse_solver(ctx, golden):
    X = datasets.swiss_roll(2000, seed=0)
    E = tk.embed(X.T, method="lle", neighbors_method="brute", num_neighbors=12, klle_shift=1e-3, context=ctx)
    assert _angles(E, golden["lle_embedding"]).max() < ANGLE_TOL
    Ed = tk.embed(X.T, method="lle", neighbors_method="brute", num_neighbors=12, klle_shift=1e-3,
                  eigen_method="dense", context=ctx)
    assert _angles(E, Ed).max() < ANGLE_TOL


def test_mid_size_lle_matches_shift_invert_lanczos(ctx):
    """N = 20000 points of the lifted roll (D = 64, k = 16): too large for the dense
    oracle, so the same CSR goes to scipy's shift-invert Lanczos (ARPACK with a
    sparse LU, the reference's own eigen method family)."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    sp = pytest.importorskip("scipy.sparse")
    X = datasets.lifted_swiss_roll(20000, 64, seed=1)
    op = ctx.local_operator(X, "lle", num_neighbors=16, check_connectivity=False)
    E, lam, info = ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, 2, 1, return_info=True)
    M = sp.csr_matrix((op.vals, op.col_idx, op.row_ptr), shape=(20000, 20000))
    R = M @ E - E * lam
    assert np.linalg.norm(R, axis=0).max() <= 1e-12 * info["spectrum_bound"]
    assert np.abs(E.T @ E - np.eye(2)).max() < 1e-10
    w, V = sla.eigsh(M, k=3, sigma=0, which="LM")
    o = np.argsort(w)
    w, V = w[o], V[:, o]
    assert _angles(E, V[:, 1:3]).max() < ANGLE_TOL
    assert np.all(np.abs(lam - w[1:3]) <= VALUE_RTOL * np.abs(w[1:3]) + VALUE_ATOL_OF_BOUND * info["spectrum_bound"])
