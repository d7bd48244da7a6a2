"""Differentiable LLE reconstruction weights.

LLEWeights is a torch.autograd.Function over the C ABI: the forward runs
tk_lle_weights (routines/locally_linear.hpp:107-131 restated on the GPU) and the
backward runs tk_lle_weights_grad, the hand-written adjoint of the regularised
solve (mu = C^{-1} (g - (g.w) 1), scattered to dL/dX through the neighbour
differences). The neighbour sets are inputs, not outputs: they are held fixed.
"""
from __future__ import annotations

import ctypes

import torch

from . import _capi as C
from .api import default_context

_DT = {torch.float32: C.TK_F32, torch.float64: C.TK_F64}


def _check_inputs(X, idx):
    if not (X.is_cuda and idx.is_cuda):
        raise ValueError("X and idx must be CUDA tensors")
    if X.dtype not in _DT:
        raise ValueError("X must be float32 or float64")
    if X.dim() != 2 or idx.dim() != 2 or idx.shape[0] != X.shape[0]:
        raise ValueError("X is (N, D) and idx is (N, k)")


class LLEWeights(torch.autograd.Function):
    """W = LLEWeights.apply(X, idx, klle_shift, context): X (N, D) float32/64 on
    the context's GPU, idx (N, k) int32 neighbour indices; W (N, k) float64."""

    @staticmethod
    def forward(fctx, X, idx, klle_shift, context):
        _check_inputs(X, idx)
        ctx = context or default_context()
        Xc = X.detach().contiguous()
        ic = idx.to(torch.int32).contiguous()
        N, D = Xc.shape
        k = ic.shape[1]
        W = torch.empty((N, k), dtype=torch.float64, device=X.device)
        torch.cuda.current_stream(X.device).synchronize()  # inputs were written on torch's stream
        ctx._check(ctx.lib.tk_lle_weights(ctx.ptr, ctypes.c_void_p(Xc.data_ptr()), _DT[Xc.dtype], N, D, D,
                                          ctypes.c_void_p(ic.data_ptr()), k, float(klle_shift),
                                          ctypes.c_void_p(W.data_ptr())))
        fctx.save_for_backward(Xc, ic, W)
        fctx.klle_shift = float(klle_shift)
        fctx.context = ctx
        return W

    @staticmethod
    def backward(fctx, gW):
        Xc, ic, W = fctx.saved_tensors
        ctx = fctx.context
        N, D = Xc.shape
        k = ic.shape[1]
        g = gW.to(torch.float64).contiguous()
        gX = torch.empty((N, D), dtype=torch.float64, device=Xc.device)
        torch.cuda.current_stream(Xc.device).synchronize()
        ctx._check(ctx.lib.tk_lle_weights_grad(ctx.ptr, ctypes.c_void_p(Xc.data_ptr()), _DT[Xc.dtype], N, D, D,
                                               ctypes.c_void_p(ic.data_ptr()), k, fctx.klle_shift,
                                               ctypes.c_void_p(W.data_ptr()), ctypes.c_void_p(g.data_ptr()),
                                               ctypes.c_void_p(gX.data_ptr())))
        return gX.to(Xc.dtype), None, None, None


def lle_weights(X: torch.Tensor, idx: torch.Tensor, klle_shift: float = 1e-3, context=None) -> torch.Tensor:
    """Differentiable LLE weights (N, k) float64 of X (N, D) for fixed neighbours idx."""
    return LLEWeights.apply(X, idx, klle_shift, context)


def reconstruction_loss(X: torch.Tensor, idx: torch.Tensor, W: torch.Tensor) -> torch.Tensor:
    """sum_i || x_i - sum_a W_ia x_{idx_ia} ||^2 (in float64)."""
    X64 = X.to(torch.float64)
    rec = torch.einsum("nk,nkd->nd", W, X64[idx.long()])
    return ((X64 - rec) ** 2).sum()
