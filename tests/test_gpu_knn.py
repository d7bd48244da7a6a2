"""Brute kNN through the C ABI vs the CPU oracle (GPU).

Bar: neighbour index sets bit-exact; rows ordered by (FP64 distance, index);
squared distances equal to FP64 within 1e-12 relative."""
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
                                         (1800, 128, 24, np.float64), (1200, 16, 40, np.float32)])
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


@pytest.mark.parametrize("screen", SCREENS)
def test_duplicate_points_tie_break_by_index(ctx, screen):
    # 40 copies of 5 distinct points: many exact ties; ties resolve by index
    base = np.random.default_rng(1).normal(size=(5, 3))
    X = np.repeat(base, 40, axis=0).astype(np.float64)
    k = 6
    idx = ctx.knn_brute(X, k, screen=screen)
    for i in range(len(X)):
        same = [j for j in range(len(X)) if j != i and (X[j] == X[i]).all()]
        assert idx[i].tolist() == same[:k]


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
