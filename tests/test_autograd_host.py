"""The adjoint of the LLE weight solve, checked on the CPU in FP64: the oracle's
weights, the dense torch reference, its autograd gradient, the adjoint formula
of the CUDA kernel, and central finite differences (h = 1e-4)."""
import numpy as np
import pytest
import torch

from lle_torch_ref import adjoint_numpy, lle_weights_dense
from oracle import oracle
from tapkee_gb300 import datasets


@pytest.mark.parametrize("n,d,k", [(300, 10, 6), (300, 3, 8)])  # k < D and k > D (rank-deficient Gram)
def test_adjoint_formula_matches_autograd_and_fd(n, d, k):
    rng = np.random.default_rng(n + d + k)
    X = datasets.cluster_curve(n, d, n_clusters=4, sigma=0.3, seed=11, dtype=np.float64)
    idx = np.ascontiguousarray(oracle.knn_brute(X, k)[0], dtype=np.int32)
    shift = 1e-3
    Xt = torch.tensor(X, requires_grad=True)
    W = lle_weights_dense(Xt, torch.tensor(idx), shift)
    W_or = oracle.lle_weights(X, idx, shift)
    assert np.abs(W.detach().numpy() - W_or).max() < 1e-9
    R = torch.tensor(rng.normal(size=(n, k)))
    (W * R).sum().backward()
    g_auto = Xt.grad.numpy()
    g_adj = adjoint_numpy(X, idx, shift, W.detach().numpy(), R.numpy())
    assert np.abs(g_adj - g_auto).max() <= 1e-8 * np.abs(g_auto).max()
    # central differences on a few coordinates
    h = 1e-4
    for (i, j) in [(0, 0), (5, 1), (n - 1, d - 1), (17, 2)]:
        Xp = X.copy()
        Xp[i, j] += h
        Xm = X.copy()
        Xm[i, j] -= h
        fp = (lle_weights_dense(torch.tensor(Xp), torch.tensor(idx), shift) * R).sum().item()
        fm = (lle_weights_dense(torch.tensor(Xm), torch.tensor(idx), shift) * R).sum().item()
        fd = (fp - fm) / (2 * h)
        assert abs(fd - g_auto[i, j]) <= 1e-5 * max(1.0, np.abs(g_auto).max())
