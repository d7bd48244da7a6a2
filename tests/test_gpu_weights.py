"""LLE weights and LTSA bases through the C ABI vs the CPU oracle (GPU).
Tolerance: 1e-5 relative (max |err| / max |ref|) for W and for P = V V^T."""
import numpy as np
import pytest

from oracle import oracle
from tapkee_gb300 import datasets

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_lle_weights_k_greater_than_d(ctx, golden):
    # Swiss roll D=3, k=12: rank-deficient Gram, conditioning set by klle_shift
    X = datasets.swiss_roll(2000, seed=0)
    idx = golden["lle_idx"]
    W = ctx.lle_weights(X, idx, 1e-3)
    ref = oracle.lle_weights(X, idx, 1e-3)
    assert _rel(W, ref) < TOL
    assert np.allclose(W.sum(1), 1.0, atol=1e-12)


@pytest.mark.parametrize("n,d,k,dtype", [(4000, 64, 16, np.float32), (3000, 128, 24, np.float32),
                                         (2000, 32, 20, np.float32), (1500, 16, 32, np.float32),
                                         (800, 8, 48, np.float32), (3000, 64, 64, np.float32),
                                         (2000, 128, 40, np.float32), (1500, 16, 60, np.float32),
                                         (1200, 32, 50, np.float64), (900, 100, 33, np.float32),
                                         (1000, 16, 100, np.float32), (700, 8, 90, np.float64),
                                         (600, 300, 12, np.float32), (500, 300, 40, np.float32)])
def test_lle_weights_lifted(ctx, n, d, k, dtype):
    X = datasets.lifted_swiss_roll(n, d, seed=n, dtype=dtype)
    idx, _, _ = oracle.knn_brute(X, k)
    W = ctx.lle_weights(X, idx, 1e-3)
    ref = oracle.lle_weights(X, idx, 1e-3)
    assert _rel(W, ref) < TOL, _rel(W, ref)


def _P(V, k):
    return np.einsum("nat,nbt->nab", V, V) + 1.0 / k


@pytest.mark.parametrize("n,d,k,td,dtype", [(1500, 8, 12, 2, np.float32), (3000, 32, 20, 2, np.float32),
                                            (2000, 16, 10, 3, np.float32), (1000, 64, 30, 2, np.float32),
                                            (1500, 16, 40, 2, np.float32), (1200, 8, 64, 3, np.float32),
                                            (1500, 32, 22, 2, np.float32), (900, 16, 40, 2, np.float64),
                                            (700, 32, 64, 4, np.float64)])
def test_ltsa_basis(ctx, n, d, k, td, dtype):
    X = datasets.lifted_s_curve(n, d, seed=n, noise=0.02, dtype=dtype)
    idx, _, _ = oracle.knn_brute(X, k)
    V = ctx.ltsa_basis(X, idx, td)
    ref = oracle.ltsa_basis(X, idx, td)
    assert _rel(_P(V, k), _P(ref, k)) < TOL
    # orthonormal columns
    assert np.abs(np.einsum("nat,nas->nts", V, V) - np.eye(td)).max() < 1e-5


def test_out_of_range_neighbours_are_reported(ctx):
    """A neighbour index outside [0, N) in a caller's list is reported as a bad
    argument by both weight routines, never read."""
    import tapkee_gb300 as tk
    X = datasets.lifted_s_curve(800, 8, seed=5, noise=0.02)
    idx, _, _ = oracle.knn_brute(X, 12)
    bad = idx.copy()
    bad[17, 3] = 800
    bad[400, 0] = -5
    with pytest.raises(tk.WrongParameterError, match="index out of range"):
        ctx.ltsa_basis(X, bad, 2)
    with pytest.raises(tk.WrongParameterError, match="index out of range"):
        ctx.lle_weights(X, bad)
    V = ctx.ltsa_basis(X, idx, 2)  # the context stays usable
    assert V.shape == (800, 12, 2)


@pytest.mark.parametrize("n,d,k", [(3001, 64, 16), (2001, 4, 12), (1999, 36, 8), (1500, 100, 15), (1200, 128, 16),
                                   (999, 8, 3), (1000, 20, 16)])
def test_lle_weights_pair_kernel(ctx, n, d, k):
    """The two-points-per-warp solve (float32, k <= 16, 16-byte aligned rows):
    odd N (the last pair has one point), D with a ragged last float4 and chunk,
    D over two chunks, k > D (two refinement steps), small k."""
    X = datasets.lifted_swiss_roll(n, d, seed=n + d, dtype=np.float32)
    idx, _, _ = oracle.knn_brute(X, k)
    W = ctx.lle_weights(X, idx, 1e-3)
    ref = oracle.lle_weights(X, idx, 1e-3)
    assert _rel(W, ref) < TOL, _rel(W, ref)
    assert np.allclose(W.sum(1), 1.0, atol=1e-12)


def test_lle_weights_pair_kernel_bad_index(ctx):
    import tapkee_gb300 as tk
    X = datasets.lifted_swiss_roll(800, 16, seed=5)
    idx, _, _ = oracle.knn_brute(X, 12)
    bad = idx.copy()
    bad[401, 5] = 800
    with pytest.raises(tk.WrongParameterError, match="index out of range"):
        ctx.lle_weights(X, bad)
    assert _rel(ctx.lle_weights(X, idx), oracle.lle_weights(X, idx, 1e-3)) < TOL
