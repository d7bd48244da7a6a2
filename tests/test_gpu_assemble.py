"""CSR assembly of M through the C ABI vs the oracle's setFromTriplets (GPU).
Given identical W, structure is exact and values agree to 1e-12 relative; two
runs are bit-identical."""
import numpy as np
import pytest

from oracle import oracle
from tapkee_gb300 import datasets

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["lle", "ltsa"])
def test_assembly_matches_oracle(ctx, golden, method):
    if method == "lle":
        X = datasets.swiss_roll(2000, seed=0)
        idx = golden["lle_idx_oracle_order"]
        w = oracle.lle_weights(X, idx, 1e-3)
        m = 0
    else:
        X = datasets.lifted_s_curve(1500, d=8, seed=11, noise=0.02, dtype=np.float64)
        idx = golden["ltsa_idx_oracle_order"]
        w = golden["ltsa_V"]
        m = 1
    rp, col, vals = ctx.assemble(method, idx, w, 1e-9)
    rr, rc, rv = oracle.assemble(m, idx, w, 1e-9)
    assert np.array_equal(rp, rr)
    assert np.array_equal(col, rc)
    assert np.abs(vals - rv).max() <= 1e-12 * np.abs(rv).max()


def test_assembly_is_deterministic_and_symmetric(ctx):
    X = datasets.lifted_swiss_roll(6000, 64, seed=3)
    idx, _, _ = oracle.knn_brute(X, 16)
    W = oracle.lle_weights(X, idx, 1e-3)
    a = ctx.assemble("lle", idx, W, 1e-9)
    b = ctx.assemble("lle", idx, W, 1e-9)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    import scipy.sparse as sp
    M = sp.csr_matrix((a[2], a[1], a[0]), shape=(6000, 6000))
    assert abs(M - M.T).max() == 0.0


def test_hub_rows_use_the_large_table(ctx):
    # a hub: point 0 is every other point's neighbour -> in-degree N-1
    rng = np.random.default_rng(0)
    N, k = 1200, 8
    idx = np.zeros((N, k), np.int32)
    for i in range(N):
        pool = np.setdiff1d(np.arange(N), [i, 0])
        rest = rng.choice(pool, size=k - 1, replace=False)
        idx[i] = np.concatenate([[0], rest]) if i != 0 else rng.choice(pool, size=k, replace=False)
    W = rng.random((N, k))
    W /= W.sum(1, keepdims=True)
    rp, col, vals = ctx.assemble("lle", idx, W, 1e-9)
    rr, rc, rv = oracle.assemble(0, idx, W, 1e-9)
    assert np.array_equal(rp, rr) and np.array_equal(col, rc)
    assert np.abs(vals - rv).max() <= 1e-12 * np.abs(rv).max()


@pytest.mark.parametrize("method,k", [("lle", 12), ("ltsa", 33), ("lle", 48), ("lle", 64), ("ltsa", 50)])
def test_assembly_wide_rows_and_long_sources(ctx, method, k):
    # skewed in-degree (neighbour j drawn with probability ~ 1 / (1 + j)): rows
    # from a dozen columns to past the 128-entry row scratch and the 256-slot
    # table; LTSA k=33 sources hold more contributions than a warp has lanes;
    # k > 40 takes the 512-entry row scratch, and rows past it the large table
    rng = np.random.default_rng(7)
    N, td = 900, 2
    p = 1.0 / (1.0 + np.arange(N))
    p /= p.sum()
    idx = np.stack([rng.choice(N, size=k, replace=False, p=p) for _ in range(N)]).astype(np.int32)
    if method == "lle":
        w = rng.random((N, k))
        w /= w.sum(1, keepdims=True)
        m = 0
    else:
        w = rng.standard_normal((N, k, td)) / np.sqrt(k)
        m = 1
    rp, col, vals = ctx.assemble(method, idx, w, 1e-9)
    rr, rc, rv = oracle.assemble(m, idx, w, 1e-9)
    d = np.diff(rr)
    if k <= 40:
        assert (d <= 128).any() and ((d > 128) & (d <= 256)).any() and (d > 256).any()
    else:
        assert ((d > 256) & (d <= 512)).any() and (d > 512).any()
    assert np.array_equal(rp, rr) and np.array_equal(col, rc)
    assert np.abs(vals - rv).max() <= 1e-12 * np.abs(rv).max()


def test_assembly_self_loops(ctx):
    # a caller's idx may list a point as its own neighbour
    rng = np.random.default_rng(3)
    N, k = 500, 6
    idx = np.stack([rng.choice(N, size=k, replace=False) for _ in range(N)]).astype(np.int32)
    idx[::7, 0] = np.arange(0, N, 7)
    w = rng.random((N, k))
    w /= w.sum(1, keepdims=True)
    rp, col, vals = ctx.assemble("lle", idx, w, 1e-9)
    rr, rc, rv = oracle.assemble(0, idx, w, 1e-9)
    assert np.array_equal(rp, rr) and np.array_equal(col, rc)
    assert np.abs(vals - rv).max() <= 1e-12 * np.abs(rv).max()


@pytest.mark.parametrize("method", ["lle", "ltsa"])
def test_assembly_out_of_range_neighbours_are_reported(ctx, method):
    """A neighbour index outside [0, N) in a caller's list is reported as a bad
    argument by assembly (never used as an address), and the context stays
    usable."""
    import tapkee_gb300 as tk
    rng = np.random.default_rng(9)
    N, k, td = 700, 8, 2
    idx = np.stack([rng.choice(N, size=k, replace=False) for _ in range(N)]).astype(np.int32)
    w = rng.random((N, k)) if method == "lle" else rng.standard_normal((N, k, td))
    bad = idx.copy()
    bad[11, 2] = N + 5
    bad[600, 0] = -3
    with pytest.raises(tk.WrongParameterError, match="index out of range"):
        ctx.assemble(method, bad, w, 1e-9)
    rp, col, vals = ctx.assemble(method, idx, w, 1e-9)
    rr, rc, rv = oracle.assemble(0 if method == "lle" else 1, idx, w, 1e-9)
    assert np.array_equal(rp, rr) and np.array_equal(col, rc)
