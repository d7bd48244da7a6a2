"""ctypes binding of the C ABI (include/tapkee_gb300.h).

The shared library is built in-tree by tapkee_gb300/build.py. Loading fails
loudly when it is missing: there is no CPU implementation behind this package.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libtapkee_gb300.so")

TK_OK = 0
TK_ERR_INVALID_ARG = 1
TK_ERR_NO_DATA = 2
TK_ERR_OOM = 3
TK_ERR_CUDA = 4
TK_ERR_TIMEOUT = 5
TK_ERR_CANCELLED = 6
TK_ERR_BUFFER_TOO_SMALL = 7
TK_ERR_UNSUPPORTED = 8
TK_ERR_NO_DEVICE = 9
TK_PAIR_NPE = 0
TK_PAIR_LLTSA = 1
TK_ERR_INTERNAL = 10
TK_ERR_NOT_CONVERGED = 11

TK_F32, TK_F64 = 0, 1
TK_NOALLOC_MAX_POINTS = 2097152
TK_METHOD_KLLE, TK_METHOD_KLTSA, TK_METHOD_HLLE = 0, 1, 2
TK_SCREEN_TENSOR, TK_SCREEN_FP32 = 0, 1

CANCEL_FN = ctypes.CFUNCTYPE(ctypes.c_int)
LOG_FN = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p)


class tk_params(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int),
        ("num_neighbors", ctypes.c_int),
        ("target_dimension", ctypes.c_int),
        ("klle_shift", ctypes.c_double),
        ("nullspace_shift", ctypes.c_double),
        ("check_connectivity", ctypes.c_int),
        ("screen", ctypes.c_int),
        ("cancel_function", CANCEL_FN),
    ]


class tk_knn_stats(ctypes.Structure):
    _fields_ = [("rows_uncertified", ctypes.c_int64), ("candidates", ctypes.c_int32), ("screen", ctypes.c_int32),
                ("tie_rows", ctypes.c_int64), ("extra_rows", ctypes.c_int64)]


class tk_batch_problem(ctypes.Structure):
    _fields_ = [("X", ctypes.c_void_p), ("dtype", ctypes.c_int), ("N", ctypes.c_int64), ("D", ctypes.c_int),
                ("ldx", ctypes.c_int64), ("k", ctypes.c_int)]


class tk_batch_tuning(ctypes.Structure):
    _fields_ = [("screen_qt", ctypes.c_int * 2), ("lle_warps", ctypes.c_int), ("wide_lists", ctypes.c_int)]


class tk_operator_info(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("k", ctypes.c_int32),
        ("method", ctypes.c_int32),
        ("target_dimension", ctypes.c_int32),
        ("connectivity_retries", ctypes.c_int32),
        ("nnz", ctypes.c_int64),
        ("rows_uncertified", ctypes.c_int64),
        ("stage_ms", ctypes.c_float * 6),
        ("tie_rows", ctypes.c_int64),
        ("extra_rows", ctypes.c_int64),
        ("kernel_ms", ctypes.c_float * 8),
    ]


class tk_eig_info(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int32),
        ("block", ctypes.c_int32),
        ("matvecs", ctypes.c_int64),
        ("spectrum_bound", ctypes.c_double),
        ("max_residual", ctypes.c_double),
        ("converged", ctypes.c_int32),
        ("ms", ctypes.c_float),
    ]


# Every symbol the header declares, with its ctypes signature.
_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double
SIGNATURES = {
    "tk_params_default": (None, [ctypes.POINTER(tk_params)]),
    "tk_ctx_create": (_I, [_I, _P, ctypes.POINTER(_P)]),
    "tk_ctx_destroy": (_I, [_P]),
    "tk_last_error": (ctypes.c_char_p, [_P]),
    "tk_status_string": (ctypes.c_char_p, [_I]),
    "tk_set_log_callback": (_I, [_P, LOG_FN, _P]),
    "tk_version": (ctypes.c_char_p, []),
    "tk_kernel_launch_count": (ctypes.c_longlong, []),
    "tk_knn_brute": (_I, [_P, _P, _I, _I64, _I, _I64, _I, _I, _P, _P, ctypes.POINTER(tk_knn_stats)]),
    "tk_knn_extra_rows": (_I, [_P, _P, _P, _I64, ctypes.POINTER(_I64)]),
    "tk_check_connected": (_I, [_P, _I64, _I, _P, ctypes.POINTER(_I)]),
    "tk_lle_weights": (_I, [_P, _P, _I, _I64, _I, _I64, _P, _I, _D, _P]),
    "tk_lle_weights_grad": (_I, [_P, _P, _I, _I64, _I, _I64, _P, _I, _D, _P, _P, _P]),
    "tk_ltsa_basis": (_I, [_P, _P, _I, _I64, _I, _I64, _P, _I, _I, _P]),
    "tk_hessian_basis": (_I, [_P, _P, _I, _I64, _I, _I64, _P, _I, _I, _P]),
    "tk_assemble": (_I, [_P, _I, _I64, _I, _I, _P, _P, _D, _P, _P, _P, ctypes.POINTER(_I64)]),
    "tk_eigenproblem_pair": (_I, [_P, _I, _P, _I, _I64, _I, _I64, _P, _P, _P, _P, _P]),
    "tk_smallest_eigenvectors": (_I, [_P, _I64, _P, _P, _P, _I, _I, _D, _I64, _P, _P,
                                      ctypes.POINTER(tk_eig_info)]),
    "tk_local_operator": (_I, [_P, ctypes.POINTER(tk_params), _P, _I, _I64, _I, _I64,
                               ctypes.POINTER(tk_operator_info)]),
    "tk_operator_copy": (_I, [_P, _P, _P, _P, _P, _P]),
    "tk_operator_device_views": (_I, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P),
                                      ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "tk_operator_get_info": (_I, [_P, ctypes.POINTER(tk_operator_info)]),
    "tk_ctx_synchronize": (_I, [_P]),
    "tk_selftest_bounded_wait": (_I, [_P, ctypes.POINTER(_I)]),
    "tk_selftest_grid_barrier": (_I, [_P, ctypes.POINTER(_I)]),
    "tk_batch_tuning_default": (None, [ctypes.POINTER(tk_batch_tuning)]),
    "tk_batch_create": (_I, [_P, ctypes.POINTER(tk_batch_problem), _I, _D, _D, ctypes.POINTER(tk_batch_tuning),
                             ctypes.POINTER(_P)]),
    "tk_batch_run": (_I, [_P, ctypes.POINTER(ctypes.c_float)]),
    "tk_batch_count": (_I, [_P]),
    "tk_batch_get_info": (_I, [_P, _I, ctypes.POINTER(tk_operator_info)]),
    "tk_batch_copy": (_I, [_P, _I, _P, _P, _P, _P, _P]),
    "tk_batch_destroy": (_I, [_P]),
    "tk_check_connected_noalloc": (_I, [_I, _P, _I64, _I, _P, ctypes.POINTER(_I), ctypes.c_char_p,
                                        ctypes.c_size_t]),
}

_lib = None


def library_path() -> str:
    return LIB_PATH


def load(path: str | None = None) -> ctypes.CDLL:
    """Loads the CUDA library (building it first is the caller's job)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"tapkee_gb300 CUDA library not found at {p}; build it with "
            "`python -c \"import __graft_entry__ as g; g.build()\"` or `python tapkee_gb300/build.py`")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
