"""Brute kNN through the C ABI vs the CPU oracle (GPU).

Bar: neighbour index sets bit-exact; rows ordered by (FP64 distance, index),
except tie rows, which hold the reference's partition order; squared distances
equal to FP64 within 1e-12 relative."""
import numpy as np
import pytest

from oracle import oracle
from tapkee_gb300 import datasets

pytestmark = pytest.mark.gpu
SCREENS = ["tensor", "fp32"]


def _ordered(X, idx):
    X = np.asarray(X, np.float64)
    d = ((X[idx] - X[:, None, :]) ** 2).sum(-1)
    order = np.array([np.lexsort((idx[i], d[i])) for i in range(len(idx))])
    return np.take_along_axis(idx, order, 1), np.take_along_axis(d, order, 1)


@pytest.mark.parametrize("screen", SCREENS)
def test_line_known_answer(ctx, screen):
    # test/unit/neighbors.cpp:92-127 through the GPU path
    N, k = 100, 10
    X = np.arange(N, dtype=np.float32).reshape(N, 1)
    idx = ctx.knn_brute(X, k, screen=screen)
    for i in range(N):
        s = set(idx[i].tolist())
        assert len(s) == k and i not in s
        for j in range(min(i, k // 2)):
            assert i - j - 1 in s
        for j in range(min(N - i - 1, k // 2)):
            assert i + j + 1 in s


@pytest.mark.parametrize("screen", SCREENS)
def test_swiss_roll_2000_bit_exact(ctx, golden, screen):
    X = datasets.swiss_roll(2000, seed=0)
    idx, d2, st = ctx.knn_brute(X, 12, screen=screen, return_distances=True, return_stats=True)
    ref = golden["lle_idx"]  # oracle sets ordered by (distance, index)
    assert np.array_equal(idx, ref)
    _, dref = _ordered(X, ref)
    assert np.abs(d2 - dref).max() <= 1e-12 * dref.max()


@pytest.mark.parametrize("screen", SCREENS)
@pytest.mark.parametrize("n,d,k,dtype", [(3000, 64, 16, np.float32), (2500, 32, 20, np.float32),
                                         (1800, 128, 24, np.float64), (1200, 16, 40, np.float32),
                                         (3000, 64, 64, np.float32), (2000, 100, 100, np.float32),
                                         (1500, 64, 130, np.float64)])
def test_lifted_rolls_match_oracle(ctx, screen, n, d, k, dtype):
    X = datasets.lifted_swiss_roll(n, d, seed=n + d, dtype=dtype)
    idx = ctx.knn_brute(X, k, screen=screen)
    ref, _, _ = oracle.knn_brute(X, k)
    ref_sorted, _ = _ordered(X, ref)
    assert np.array_equal(idx, ref_sorted)


@pytest.mark.parametrize("screen", SCREENS)
def test_small_and_ragged_sizes(ctx, screen):
    for n, k in [(2, 1), (3, 2), (33, 5), (257, 31), (300, 56), (400, 100), (600, 200)]:
        X = np.random.default_rng(n).normal(size=(n, 5)).astype(np.float32)
        idx = ctx.knn_brute(X, k, screen=screen)
        ref, _, _ = oracle.knn_brute(X, k)
        assert np.array_equal(idx, _ordered(X, ref)[0]), (n, k)


def _tie_rows(X, k):
    """Rows whose k-th and (k+1)-th nearest other points are at distances within
    1e-12 relative (exact squared distances, numpy FP64)."""
    X = np.asarray(X, np.float64)
    d = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d, np.inf)
    d.sort(axis=1)
    if k >= len(X) - 1:
        return np.zeros(len(X), bool)
    return d[:, k] - d[:, k - 1] <= 1e-12 * d[:, k]


def _lattice(shape, dtype):
    g = np.stack(np.meshgrid(*[np.arange(s) for s in shape], indexing="ij"), -1).reshape(-1, len(shape))
    return np.ascontiguousarray(g[np.random.default_rng(3).permutation(len(g))], dtype=dtype)


def _duplicates(dtype):
    base = np.random.default_rng(1).normal(size=(5, 3))
    return np.ascontiguousarray(np.repeat(base, 40, axis=0), dtype=dtype)


def _copies4(dtype):
    base = np.random.default_rng(4).normal(size=(50, 8))
    return np.ascontiguousarray(np.repeat(base, 4, axis=0), dtype=dtype)


def _copies(n_base, copies, dim, seed, dtype):
    base = np.random.default_rng(seed).normal(size=(n_base, dim))
    return np.ascontiguousarray(np.repeat(base, copies, axis=0), dtype=dtype)


TIE_CASES = [
    # the nearest other point's 4 copies straddle ranks k - 1, k and k + 1: equal
    # FP32 distances past rank k must be refined with the others
    ("4 copies of 50 points, k=5", lambda dt: _copies4(dt), 5),
    ("40 copies of 5 points, k=3", lambda dt: _duplicates(dt), 3),
    ("40 copies of 5 points, k=6", lambda dt: _duplicates(dt), 6),
    ("40 copies of 5 points, k=45", lambda dt: _duplicates(dt), 45),
    ("integer line, k=3", lambda dt: np.arange(300, dtype=dt).reshape(300, 1), 3),
    ("integer line, k=11", lambda dt: np.arange(300, dtype=dt).reshape(300, 1), 11),
    ("2-D integer grid 40x40, k=10", lambda dt: _lattice((40, 40), dt), 10),
    ("2-D integer grid 40x40, k=6", lambda dt: _lattice((40, 40), dt), 6),
    ("3-D integer grid 12^3, k=12", lambda dt: _lattice((12, 12, 12), dt), 12),
    # lists longer than 64 are screened in passes of 64: equal screened values
    # straddle the passes (2 passes at k=70, 4 at k=150)
    ("100 copies of 3 points, k=70", lambda dt: _copies(3, 100, 6, 5, dt), 70),
    ("150 copies of 3 points, k=150", lambda dt: _copies(3, 150, 6, 6, dt), 150),
    ("3-D integer grid 12^3, k=80", lambda dt: _lattice((12, 12, 12), dt), 80),
]


@pytest.mark.parametrize("screen", SCREENS)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("case", range(len(TIE_CASES)))
def test_ties_follow_the_reference_partition(ctx, screen, dtype, case):
    """Exact ties at the k-boundary (duplicated points, integer lattices): every
    row's set equals the oracle's (std::nth_element at k + 1 over the row's
    records in index order, minus the query: neighbors/neighbors.hpp:129-146);
    tie rows keep the partition order itself; the tie rows are counted; and the
    rows for which the reference returns k + 1 neighbours are listed with their
    (k + 1)-th neighbour."""
    name, make, k = TIE_CASES[case]
    X = make(dtype)
    idx, st = ctx.knn_brute(X, k, screen=screen, return_stats=True)
    ref, _, cnt, extra = oracle.knn_brute(X, k, return_extra=True)
    for i in range(len(X)):
        assert set(idx[i].tolist()) == set(ref[i].tolist()), (name, i)
    ties = _tie_rows(X, k)
    assert st["tie_rows"] == int(ties.sum()) and ties.sum() > 0, name
    assert np.array_equal(idx[ties], ref[ties]), name  # partition order on tie rows
    want = [(int(i), int(extra[i])) for i in np.nonzero(cnt == k + 1)[0]]
    assert st["extra_rows"] == len(want), name
    assert st.get("extra", []) == want, name


def test_continuous_data_has_no_tie_rows(ctx):
    X = datasets.lifted_swiss_roll(20_000, 64, seed=4)
    _, st = ctx.knn_brute(X, 16, return_stats=True)
    assert st["tie_rows"] == 0 and st["extra_rows"] == 0


def test_wide_dimensions_take_the_fp32_screen(ctx):
    """D = 300: the tensor-core screen (padded D <= 128) refuses it; the FP32
    screen and the re-rank's dimension-parallel path (D > 256) match the oracle."""
    import tapkee_gb300 as tk
    X = datasets.lifted_swiss_roll(700, 300, seed=5)
    with pytest.raises(tk.UnsupportedMethodError):
        ctx.knn_brute(X, 12, screen="tensor")
    idx = ctx.knn_brute(X, 12, screen="fp32")
    ref, _, _ = oracle.knn_brute(X, 12)
    assert np.array_equal(idx, _ordered(X, ref)[0])


def test_invalid_arguments(ctx):
    import tapkee_gb300 as tk
    X = np.zeros((10, 3), np.float32)
    with pytest.raises(tk.WrongParameterError):
        ctx.knn_brute(X, 10)
    with pytest.raises(tk.WrongParameterError):
        ctx.knn_brute(X, 0)
    with pytest.raises(tk.NoDataError):
        ctx.knn_brute(np.zeros((0, 3), np.float32), 1)
    with pytest.raises(tk.UnsupportedMethodError):
        ctx.knn_brute(np.random.default_rng(0).normal(size=(300, 3)), 250)


def test_device_resident_inputs(ctx):
    import torch
    X = datasets.lifted_swiss_roll(2048, 64, seed=9)
    Xd = torch.from_numpy(X).cuda()
    idx_d = ctx.knn_brute(Xd, 16)
    assert idx_d.is_cuda
    idx_h = ctx.knn_brute(X, 16)
    assert np.array_equal(idx_d.cpu().numpy(), idx_h)


@pytest.mark.parametrize("n", [1290, 1300, 1345, 1353])
def test_wide_screen_short_last_block(ctx, n):
    # the last 128-query block holds 10, 20, 65 and 73 rows: the block-mate
    # bound of its k-th neighbour distance is infinite (every tile near), taken
    # over all of its rows, or over a 64-row window
    X = datasets.lifted_swiss_roll(n, 64, seed=n)
    idx = ctx.knn_brute(X, 16, screen="tensor")
    ref, _, _ = oracle.knn_brute(X, 16)
    assert np.array_equal(idx, _ordered(X, ref)[0])


def test_wide_screen_tail_blocks_split_in_eight(ctx):
    # 19600 points: 154 query blocks, the 2 after the first 152 split in 8 parts
    X = datasets.lifted_swiss_roll(19_600, 64, seed=5)
    a = ctx.knn_brute(X, 16, screen="tensor")
    b = ctx.knn_brute(X, 16, screen="fp32")
    assert np.array_equal(a, b)


def test_find_neighbors_for_plain_distance_callers(ctx):
    """find_neighbors (neighbors/neighbors.hpp:173-213) as the plain-distance
    callers (Isomap, Laplacian Eigenmaps, LPP, SPE, Manifold Sculpting) use it:
    the connectivity retry and the k clamp of the reference, and distances equal
    to eigen_distance_callback's (x_a - x_b).norm() (callbacks/eigen_callbacks.hpp:52-64)."""
    rng = np.random.default_rng(0)
    X = np.concatenate([rng.normal(size=(60, 2)), rng.normal(size=(60, 2)) + 100.0])
    msgs = []
    ctx.set_logger(lambda lvl, m: msgs.append((lvl, m)))
    try:
        idx, dist, k = ctx.find_neighbors(X, 5, return_distances=True)
        idx_small, k_small = ctx.find_neighbors(X[:8], 20)
    finally:
        ctx.set_logger(None)
    ref_idx, k_ref = oracle.find_neighbors(X, 5)
    assert k == k_ref == 80
    assert all(set(a) == set(b) for a, b in zip(idx.tolist(), ref_idx.tolist()))
    plain = np.linalg.norm(X[:, None, :] - X[idx], axis=2)
    assert np.allclose(dist, plain, rtol=1e-12, atol=1e-12)
    assert np.all(np.diff(dist, axis=1) >= 0)
    assert k_small == 7 and idx_small.shape == (8, 7)
    assert any("not connected" in m for _, m in msgs)
    assert any("greater than number of objects" in m for _, m in msgs)
