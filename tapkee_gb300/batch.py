"""Batches of independent KLLE problems (tk_batch_* of the C ABI).

A Batch plans many problems of uneven N, D and k once, captures the whole
stage for all of them as one CUDA graph, and replays it with run(). Tile shapes
come from the autotuner's table (tapkee_gb300/tuning/gb300_batch.json, written
by tapkee_gb300/autotune.py) unless given explicitly.
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

from . import _capi as C
from .api import LocalOperator, default_context

HERE = os.path.dirname(os.path.abspath(__file__))
TUNING_PATH = os.path.join(HERE, "tuning", "gb300_batch.json")
_DT = {"float32": C.TK_F32, "float64": C.TK_F64}


def default_tuning() -> dict:
    """The autotuned tile shapes if the table exists, else the library defaults."""
    lib = C.load()
    t = C.tk_batch_tuning()
    lib.tk_batch_tuning_default(ctypes.byref(t))
    out = {"screen_qt": [t.screen_qt[0], t.screen_qt[1]], "lle_warps": t.lle_warps, "wide_lists": t.wide_lists}
    try:
        with open(TUNING_PATH) as f:
            best = json.load(f).get("best", {})
        out.update({k: v for k, v in best.items() if k in out})
    except (OSError, ValueError):
        pass
    return out


def _tuning_struct(t: dict):
    s = C.tk_batch_tuning()
    s.screen_qt[0], s.screen_qt[1] = int(t["screen_qt"][0]), int(t["screen_qt"][1])
    s.lle_warps = int(t["lle_warps"])
    s.wide_lists = int(t["wide_lists"])
    return s


class Batch:
    """problems: sequence of CUDA tensors (N_i, D_i), float32 or float64, kept
    alive by the batch; ks: one k per problem (or one int for all)."""

    def __init__(self, problems, ks, klle_shift=1e-3, nullspace_shift=1e-9, tuning=None, context=None):
        import torch
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        self._keep = [p.contiguous() for p in problems]
        if isinstance(ks, int):
            ks = [ks] * len(self._keep)
        if len(ks) != len(self._keep):
            raise ValueError("one k per problem")
        arr = (C.tk_batch_problem * len(self._keep))()
        for a, X, k in zip(arr, self._keep, ks):
            if not X.is_cuda or X.dim() != 2 or X.dtype not in (torch.float32, torch.float64):
                raise ValueError("each problem is a 2-D float32/float64 CUDA tensor")
            a.X = X.data_ptr()
            a.dtype = C.TK_F32 if X.dtype == torch.float32 else C.TK_F64
            a.N, a.D = X.shape
            a.ldx = X.shape[1]
            a.k = int(k)
        self.tuning = dict(tuning) if tuning is not None else default_tuning()
        ts = _tuning_struct(self.tuning)
        self.ptr = ctypes.c_void_p()
        torch.cuda.current_stream().synchronize()  # problem data was written on torch's stream
        self.ctx._check(self.lib.tk_batch_create(self.ctx.ptr, arr, len(self._keep), float(klle_shift),
                                                 float(nullspace_shift), ctypes.byref(ts), ctypes.byref(self.ptr)))
        self.ks = list(ks)

    def __len__(self):
        return len(self._keep)

    def run(self) -> float:
        """Replays the captured graph; returns its device time in ms."""
        ms = ctypes.c_float()
        self.ctx._check(self.lib.tk_batch_run(self.ptr, ctypes.byref(ms)))
        return ms.value

    def result(self, p: int) -> LocalOperator:
        info = C.tk_operator_info()
        self.ctx._check(self.lib.tk_batch_get_info(self.ptr, p, ctypes.byref(info)))
        n, k, nnz = int(info.n), int(info.k), int(info.nnz)
        idx = np.empty((n, k), np.int32)
        w = np.empty((n, k), np.float64)
        rp = np.empty(n + 1, np.int64)
        col = np.empty(nnz, np.int32)
        val = np.empty(nnz, np.float64)
        self.ctx._check(self.lib.tk_batch_copy(self.ptr, p, idx.ctypes.data, w.ctypes.data, rp.ctypes.data,
                                               col.ctypes.data, val.ctypes.data))
        return LocalOperator(idx=idx, weights=w, row_ptr=rp, col_idx=col, vals=val, k=k, method=C.TK_METHOD_KLLE,
                             target_dimension=0, connectivity_retries=0, rows_uncertified=int(info.rows_uncertified))

    def close(self):
        if self.ptr:
            self.lib.tk_batch_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
