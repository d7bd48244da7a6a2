"""Full-size workloads checked through size-independent properties plus a
sample of rows against the oracle.

  * LTSA, lifted S-curve N=50000 D=32 k=20 td=2 (float32)
  * LLE, lifted Swiss roll N=200000 D=64 k=16 (float32)

Properties: neighbour sets of sampled rows equal the oracle's; tangent
projectors / weights of sampled rows within 1e-5 of FP64; M is symmetric,
sorted, and M 1 = shift 1 (every block (I - W)^T (I - W) and I - P_i
annihilates the constant vector)."""
import numpy as np
import pytest

from oracle import oracle
from tapkee_gb300 import datasets

pytestmark = pytest.mark.gpu


def _csr_checks(op, shift, tol):
    import scipy.sparse as sp
    n = op.idx.shape[0]
    rp, col, vals = op.row_ptr, op.col_idx, op.vals
    assert rp[0] == 0 and rp[-1] == len(col) and np.all(np.diff(rp) > 0)
    # columns strictly ascending within each row
    d = np.diff(col.astype(np.int64))
    starts = rp[1:-1]
    d[starts - 1] = 1  # row boundaries
    assert np.all(d > 0)
    M = sp.csr_matrix((vals, col, rp), shape=(n, n))
    asym = abs(M - M.T).max()
    assert asym <= 1e-12 * abs(M).max()
    r = M @ np.ones(n)
    assert np.abs(r - shift).max() <= tol


def test_ltsa_s_curve_50k(ctx):
    X = datasets.lifted_s_curve(50_000, 32, seed=3, noise=0.02)
    op = ctx.local_operator(X, "ltsa", num_neighbors=20, target_dimension=2, check_connectivity=False)
    assert op.idx.shape == (50_000, 20) and op.weights.shape == (50_000, 20, 2)
    rows = np.sort(np.random.default_rng(0).choice(50_000, 400, replace=False))
    ref = oracle.knn_brute_rows(X, 20, rows)
    assert all(set(a) == set(b) for a, b in zip(op.idx[rows].tolist(), ref.tolist()))
    V_ref = oracle.ltsa_basis(X, op.idx[rows], 2)
    P = np.einsum("nat,nbt->nab", op.weights[rows], op.weights[rows])
    Pr = np.einsum("nat,nbt->nab", V_ref, V_ref)
    assert np.abs(P - Pr).max() < 1e-5
    _csr_checks(op, 1e-9, 1e-5)


def test_lle_lifted_roll_200k(ctx):
    X = datasets.lifted_swiss_roll(200_000, 64, seed=1)
    op = ctx.local_operator(X, "lle", num_neighbors=16, klle_shift=1e-3, check_connectivity=False)
    rows = np.sort(np.random.default_rng(1).choice(200_000, 300, replace=False))
    ref = oracle.knn_brute_rows(X, 16, rows)
    assert all(set(a) == set(b) for a, b in zip(op.idx[rows].tolist(), ref.tolist()))
    W_ref = oracle.lle_weights_rows(X, rows, op.idx[rows], 1e-3)
    assert np.abs(op.weights[rows] - W_ref).max() / np.abs(W_ref).max() < 1e-5
    np.testing.assert_allclose(op.weights.sum(1), 1.0, atol=1e-9)
    _csr_checks(op, 1e-9, 1e-6)


@pytest.mark.parametrize("n", [25_000, 200_000])
def test_lle_tensor_screen_equals_fp32_screen(ctx, n):
    # both screens are certified exact, so the neighbour tables agree row for
    # row; at these sizes the last, partial wave of query blocks is split into
    # parts whose lists are merged (25000 points: 196 blocks, 44 split in 3)
    X = datasets.lifted_swiss_roll(n, 64, seed=1)
    a = ctx.local_operator(X, "lle", num_neighbors=16, klle_shift=1e-3, check_connectivity=False)
    b = ctx.local_operator(X, "lle", num_neighbors=16, klle_shift=1e-3, check_connectivity=False, screen="fp32")
    assert a.rows_uncertified == 0
    assert np.array_equal(a.idx, b.idx)


def test_lle_lifted_roll_200k_reference_default_connectivity(ctx):
    """The reference's default path at N=200000 (check_connectivity=true,
    defines/keywords.hpp:272): while is_connected fails, find_neighbors redoes
    the search with 2k (neighbors/neighbors.hpp:196-204). The final k equals the
    one the oracle's is_connected reaches on the same neighbour tables, every
    doubling is logged with the reference's message, and sampled rows at the
    final k match the oracle (sets exact, W within 1e-5)."""
    X = datasets.lifted_swiss_roll(200_000, 64, seed=1)
    msgs = []
    ctx.set_logger(lambda lvl, m: msgs.append(m))
    try:
        op = ctx.local_operator(X, "lle", num_neighbors=16, klle_shift=1e-3, check_connectivity=True)
    finally:
        ctx.set_logger(None)
    k, decisions = 16, []
    while True:
        conn = oracle.is_connected(ctx.knn_brute(X, k))
        decisions.append((k, conn))
        if conn:
            break
        k *= 2
    assert op.k == k and op.connectivity_retries == len(decisions) - 1, decisions
    for kk, conn in decisions[:-1]:
        assert any(f"The neighborhood graph with {kk} neighbors is not connected. Recomputing with a larger "
                   f"number of neighbors {2 * kk}." in m for m in msgs)
    assert any(f"The neighborhood graph with {k} neighbors is connected." in m for m in msgs)
    rows = np.sort(np.random.default_rng(2).choice(200_000, 300, replace=False))
    ref = oracle.knn_brute_rows(X, k, rows)
    assert all(set(a) == set(b) for a, b in zip(op.idx[rows].tolist(), ref.tolist()))
    W_ref = oracle.lle_weights_rows(X, rows, op.idx[rows], 1e-3)
    assert np.abs(op.weights[rows] - W_ref).max() / np.abs(W_ref).max() < 1e-5
    _csr_checks(op, 1e-9, 1e-6)
