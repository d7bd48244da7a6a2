"""FP64 dense-autograd reference of the LLE weights (test helper).

Restates the per-point solve of linear_weight_matrix
(routines/locally_linear.hpp:117-131) with batched dense torch ops, so torch's
own autograd gives the reference gradient: C_ab = (n_a - x).(n_b - x),
C += klle_shift tr(C) I, w = C^{-1} 1 / sum.
"""
import numpy as np
import torch


def lle_weights_dense(X: torch.Tensor, idx: torch.Tensor, klle_shift: float) -> torch.Tensor:
    Z = X[idx.long()] - X[:, None, :]
    C = Z @ Z.transpose(1, 2)
    tr = C.diagonal(dim1=1, dim2=2).sum(-1)
    k = idx.shape[1]
    eye = torch.eye(k, dtype=X.dtype, device=X.device)
    Cr = C + klle_shift * tr[:, None, None] * eye
    u = torch.linalg.solve(Cr, torch.ones(X.shape[0], k, 1, dtype=X.dtype, device=X.device))[..., 0]
    return u / u.sum(-1, keepdim=True)


def adjoint_numpy(X, idx, klle_shift, W, G):
    """dL/dX by the adjoint formula the CUDA kernel implements (FP64 numpy)."""
    N, D = X.shape
    gX = np.zeros_like(X, dtype=np.float64)
    for i in range(N):
        Z = X[idx[i]] - X[i]
        C = Z @ Z.T
        Cr = C + klle_shift * np.trace(C) * np.eye(len(idx[i]))
        w = W[i]
        g = G[i]
        mu = np.linalg.solve(Cr, g - (g @ w))
        p = w @ Z
        q = mu @ Z
        dZ = -np.outer(mu, p) - np.outer(w, q) - 2.0 * klle_shift * (mu @ w) * Z
        np.add.at(gX, idx[i], dZ)
        gX[i] -= dZ.sum(0)
    return gX
