"""Differentiable LLE weights on the GPU (torch.autograd.Function over
tk_lle_weights / tk_lle_weights_grad) against the FP64 dense-autograd reference
and central finite differences (h = 1e-4, FP64).

Workload: 10 Gaussian clusters (sigma 0.3) on a seeded random curve in R^128,
N = 20000, float32, a learnable per-feature scale s (s0 = 1) applied before the
weights, neighbour sets fixed (computed once at s0), k = 12."""
import numpy as np
import pytest
import torch

from lle_torch_ref import lle_weights_dense
from tapkee_gb300 import autograd as tka
from tapkee_gb300 import datasets

pytestmark = pytest.mark.gpu

SHIFT = 1e-3


def _setup(ctx, n=20000, d=128, k=12):
    X = datasets.cluster_curve(n, d, n_clusters=10, sigma=0.3, seed=5)
    idx = ctx.knn_brute(X, k)
    Xd = torch.from_numpy(X).cuda()
    idd = torch.from_numpy(idx).cuda()
    return Xd, idd


def _grads(ctx, Xd, idd, loss_kind, R=None):
    s = torch.ones(Xd.shape[1], dtype=torch.float32, device="cuda", requires_grad=True)
    Xs = Xd * s
    W = tka.lle_weights(Xs, idd, SHIFT, context=ctx)
    loss = tka.reconstruction_loss(Xs, idd, W) if loss_kind == "recon" else (W * R).sum()
    loss.backward()
    g = s.grad.double()

    s64 = torch.ones(Xd.shape[1], dtype=torch.float64, device="cuda", requires_grad=True)

    def ref_loss(s_):
        Xs_ = Xd.double() * s_
        W_ = lle_weights_dense(Xs_, idd, SHIFT)
        if loss_kind == "recon":
            return tka.reconstruction_loss(Xs_, idd, W_)
        return (W_ * R).sum()

    ref_loss(s64).backward()
    return g, s64.grad, ref_loss, W


@pytest.mark.parametrize("loss_kind", ["recon", "random_functional"])
def test_lle_weights_gradient_vs_fp64_reference_and_fd(ctx, loss_kind):
    Xd, idd = _setup(ctx)
    R = torch.randn(idd.shape, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(3))
    g, g_ref, ref_loss, W = _grads(ctx, Xd, idd, loss_kind, R)
    # forward: W within 1e-5 of the FP64 reference
    W_ref = lle_weights_dense(Xd.double(), idd, SHIFT)
    assert (W - W_ref).abs().max().item() / W_ref.abs().max().item() < 1e-5
    # gradient vs FP64 dense autograd
    rel = ((g - g_ref).norm() / g_ref.norm()).item()
    assert rel < 1e-4, rel
    # central differences (h = 1e-4, FP64) on a few coordinates of s
    h = 1e-4
    with torch.no_grad():
        for j in (0, 17, 64, 127):
            e = torch.zeros(Xd.shape[1], dtype=torch.float64, device="cuda")
            e[j] = h
            one = torch.ones_like(e)
            fd = (ref_loss(one + e) - ref_loss(one - e)).item() / (2 * h)
            scale = g_ref.abs().max().item()
            assert abs(fd - g_ref[j].item()) <= 1e-4 * scale, (j, fd, g_ref[j].item())
            assert abs(fd - g[j].item()) <= 2e-4 * scale, (j, fd, g[j].item())


def test_lle_weights_grad_entry_point_matches_adjoint_formula(ctx):
    """tk_lle_weights_grad on a small k > D case (rank-deficient Gram) against the
    FP64 numpy restatement of the adjoint."""
    from lle_torch_ref import adjoint_numpy
    from oracle import oracle
    X = datasets.swiss_roll(2000, seed=0)
    idx = ctx.knn_brute(X, 12)
    W = oracle.lle_weights(X, idx, SHIFT)
    G = np.random.default_rng(1).normal(size=W.shape)
    Xd = torch.from_numpy(X).cuda().requires_grad_(True)
    Wd = tka.lle_weights(Xd, torch.from_numpy(idx).cuda(), SHIFT, context=ctx)
    (Wd * torch.from_numpy(G).cuda()).sum().backward()
    g_ref = adjoint_numpy(X, idx, SHIFT, W, G)
    err = np.abs(Xd.grad.cpu().numpy() - g_ref).max() / np.abs(g_ref).max()
    assert err < 1e-4, err


def test_lle_weights_grad_is_bit_reproducible(ctx):
    """dL/dX is a pull over reverse neighbour lists in a fixed order (no atomics):
    repeated calls give bit-identical gradients."""
    X = datasets.lifted_swiss_roll(6000, 32, seed=2)
    idx = ctx.knn_brute(X, 16)
    Xd = torch.from_numpy(X).cuda()
    idd = torch.from_numpy(idx).cuda()
    G = torch.from_numpy(np.random.default_rng(4).normal(size=idx.shape)).cuda()
    grads = []
    for _ in range(3):
        Xg = Xd.clone().requires_grad_(True)
        (tka.lle_weights(Xg, idd, SHIFT, context=ctx) * G).sum().backward()
        grads.append(Xg.grad.clone())
    assert torch.equal(grads[0], grads[1]) and torch.equal(grads[0], grads[2])
