"""Host-side mirror of the reference's interface for the local-neighborhood stage.

* ``Context`` -- one GPU context (CUDA stream + scratch) with one method per C ABI
  stage: ``knn_brute``, ``check_connected``, ``lle_weights``, ``ltsa_basis``,
  ``assemble`` and the whole stage ``local_operator``.
* ``embed(data, method='lle', ...)`` -- the keyword signature of the reference's
  Python module (src/python/nanobind_extension.cpp:28-96): ``data`` is
  features x samples, the result samples x target_dimension.
* ``with_(method=..., num_neighbors=...).embed_using(matrix)`` -- the chain of
  ``tapkee::with((...)).embedUsing(matrix)`` (chain_interface.hpp:471-500).

Errors map onto the reference's exception types (exceptions.hpp:14-91).
Arrays may be numpy (host) or torch tensors (host or CUDA); outputs follow the
input: numpy in, numpy out; CUDA tensor in, CUDA tensors out.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _capi as C

# ---------------------------------------------------------------- exceptions


class TapkeeError(Exception):
    """Base class of the errors raised by this package."""


class WrongParameterError(TapkeeError, ValueError):
    """tapkee::wrong_parameter_error"""


class NoDataError(TapkeeError, ValueError):
    """tapkee::no_data_error"""


class NotEnoughMemoryError(TapkeeError, MemoryError):
    """tapkee::not_enough_memory_error"""


class CancelledError(TapkeeError):
    """tapkee::cancelled_exception"""


class UnsupportedMethodError(TapkeeError):
    """tapkee::unsupported_method_error"""


class EigendecompositionError(TapkeeError):
    """tapkee::eigendecomposition_error"""


class MultipleParameterError(TapkeeError):
    """tapkee::multiple_parameter_error"""


class MissedParameterError(TapkeeError):
    """tapkee::missed_parameter_error"""


class DeviceError(TapkeeError, RuntimeError):
    """A CUDA failure or a device-side check (including a bounded wait that expired)."""


_STATUS_EXC = {
    C.TK_ERR_INVALID_ARG: WrongParameterError,
    C.TK_ERR_NO_DATA: NoDataError,
    C.TK_ERR_OOM: NotEnoughMemoryError,
    C.TK_ERR_CUDA: DeviceError,
    C.TK_ERR_TIMEOUT: DeviceError,
    C.TK_ERR_CANCELLED: CancelledError,
    C.TK_ERR_BUFFER_TOO_SMALL: WrongParameterError,
    C.TK_ERR_UNSUPPORTED: UnsupportedMethodError,
    C.TK_ERR_NO_DEVICE: DeviceError,
    C.TK_ERR_INTERNAL: DeviceError,
    C.TK_ERR_NOT_CONVERGED: EigendecompositionError,
}

METHODS = {
    "lle": C.TK_METHOD_KLLE,
    "locally_linear_embedding": C.TK_METHOD_KLLE,
    "klle": C.TK_METHOD_KLLE,
    "ltsa": C.TK_METHOD_KLTSA,
    "local_tangent_space_alignment": C.TK_METHOD_KLTSA,
    "kltsa": C.TK_METHOD_KLTSA,
    "hlle": C.TK_METHOD_HLLE,
    "hessian_locally_linear_embedding": C.TK_METHOD_HLLE,
}
SCREENS = {"tensor": C.TK_SCREEN_TENSOR, "fp32": C.TK_SCREEN_FP32}


def _raise(ctx_ptr, status, lib):
    if status == C.TK_OK:
        return
    msg = lib.tk_last_error(ctx_ptr).decode() if ctx_ptr else lib.tk_status_string(status).decode()
    raise _STATUS_EXC.get(status, DeviceError)(msg or lib.tk_status_string(status).decode())


# ---------------------------------------------------------------- arrays


def _torch():
    try:
        import torch  # noqa: F401
        return torch
    except Exception:  # pragma: no cover
        return None


def _is_torch(x):
    t = _torch()
    return t is not None and isinstance(x, t.Tensor)


class _Buf:
    """A contiguous array and its address, numpy or torch."""

    def __init__(self, arr, kind):
        self.arr = arr
        self.kind = kind  # "np" | "torch"

    @property
    def ptr(self):
        return self.arr.ctypes.data if self.kind == "np" else self.arr.data_ptr()


def _as_points(X):
    """Points-major (N x D) contiguous float32/float64 array."""
    if _is_torch(X):
        t = X.contiguous()
        if t.dtype not in (_torch().float32, _torch().float64):
            t = t.to(_torch().float64)
        dt = C.TK_F64 if t.dtype == _torch().float64 else C.TK_F32
        return _Buf(t, "torch"), dt
    a = np.asarray(X)
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float64)
    a = np.ascontiguousarray(a)
    return _Buf(a, "np"), (C.TK_F64 if a.dtype == np.float64 else C.TK_F32)


def _as_index(idx, like):
    if _is_torch(idx):
        return _Buf(idx.to(_torch().int32).contiguous(), "torch")
    return _Buf(np.ascontiguousarray(np.asarray(idx, dtype=np.int32)), "np")


def _as_f64(a):
    if _is_torch(a):
        return _Buf(a.to(_torch().float64).contiguous(), "torch")
    return _Buf(np.ascontiguousarray(np.asarray(a, dtype=np.float64)), "np")


def _empty(shape, dtype, like: _Buf):
    if like.kind == "torch" and like.arr.is_cuda:
        torch = _torch()
        tdt = {np.int32: torch.int32, np.int64: torch.int64, np.float64: torch.float64}[dtype]
        return _Buf(torch.empty(shape, dtype=tdt, device=like.arr.device), "torch")
    return _Buf(np.empty(shape, dtype=dtype), "np")


# ---------------------------------------------------------------- context


@dataclass
class LocalOperator:
    """The operator of one stage run: neighbours, weights and M in CSR."""

    idx: object
    weights: object
    row_ptr: object
    col_idx: object
    vals: object
    k: int
    method: int
    target_dimension: int
    connectivity_retries: int
    rows_uncertified: int
    stage_ms: dict = field(default_factory=dict)
    tie_rows: int = 0
    extra_rows: int = 0

    def to_scipy(self):
        import scipy.sparse as sp
        n = len(self.row_ptr) - 1
        rp, ci, v = (np.asarray(a.cpu()) if _is_torch(a) else np.asarray(a)
                     for a in (self.row_ptr, self.col_idx, self.vals))
        return sp.csr_matrix((v, ci, rp), shape=(n, n))


class Context:
    """One GPU context: a CUDA stream plus reusable device scratch memory."""

    def __init__(self, device: int = 0, stream=None):
        self.lib = C.load()
        self.ptr = ctypes.c_void_p()
        st = ctypes.c_void_p(int(stream)) if stream is not None else None
        rc = self.lib.tk_ctx_create(int(device), st, ctypes.byref(self.ptr))
        if rc != C.TK_OK:
            raise DeviceError(f"tk_ctx_create failed: {self.lib.tk_status_string(rc).decode()}")
        self._log_cb = None

    def close(self):
        if self.ptr:
            self.lib.tk_ctx_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        _raise(self.ptr, rc, self.lib)

    def set_logger(self, fn):
        """fn(level:int, message:str) receives the library's log messages."""
        if fn is None:
            self._log_cb = None
            self._check(self.lib.tk_set_log_callback(self.ptr, C.LOG_FN(), None))
            return
        self._log_cb = C.LOG_FN(lambda lvl, msg, user: fn(lvl, msg.decode()))
        self._log_fn = fn
        self._check(self.lib.tk_set_log_callback(self.ptr, self._log_cb, None))

    def _log(self, level, message):
        fn = getattr(self, "_log_fn", None)
        if fn is not None:
            fn(level, message)

    # -- stages ---------------------------------------------------------------
    def knn_brute(self, X, k, screen="tensor", return_distances=False, return_stats=False):
        """Brute-force k nearest neighbours (neighbors/neighbors.hpp:119-149).
        Rows ordered by (FP64 squared distance, index), except tie rows (the k-th
        and (k+1)-th distances within 1e-12 relative), which hold the reference's
        nth_element selection in its partition order. return_stats adds a dict
        with rows_uncertified, candidates, tie_rows, extra_rows and, when
        extra_rows > 0, extra = [(row, (k+1)-th reference neighbour), ...]."""
        xb, dt = _as_points(X)
        N, D = xb.arr.shape
        idx = _empty((N, k), np.int32, xb)
        d2 = _empty((N, k), np.float64, xb) if return_distances else None
        st = C.tk_knn_stats()
        self._check(self.lib.tk_knn_brute(self.ptr, xb.ptr, dt, N, D, D, int(k), SCREENS[screen], idx.ptr,
                                          d2.ptr if d2 else None, ctypes.byref(st)))
        out = [idx.arr]
        if return_distances:
            out.append(d2.arr)
        if return_stats:
            stats = {"rows_uncertified": st.rows_uncertified, "candidates": st.candidates,
                     "tie_rows": st.tie_rows, "extra_rows": st.extra_rows}
            if st.extra_rows > 0:
                stats["extra"] = self.knn_extra_rows()
            out.append(stats)
        return out[0] if len(out) == 1 else tuple(out)

    def knn_extra_rows(self):
        """(row, (k+1)-th neighbour) pairs of the last brute kNN pass for which the
        reference returns k + 1 neighbours (tk_knn_extra_rows), ascending by row."""
        n = ctypes.c_int64(0)
        self._check(self.lib.tk_knn_extra_rows(self.ptr, None, None, 0, ctypes.byref(n)))
        rows = np.empty(n.value, np.int32)
        extra = np.empty(n.value, np.int32)
        if n.value:
            self._check(self.lib.tk_knn_extra_rows(self.ptr, rows.ctypes.data, extra.ctypes.data, n.value,
                                                   ctypes.byref(n)))
        return list(zip(rows.tolist(), extra.tolist()))

    def find_neighbors(self, X, k, check_connectivity=True, screen="tensor", return_distances=False):
        """find_neighbors with neighbors_method=Brute (neighbors/neighbors.hpp:173-213)
        for any caller of the brute kNN, including the plain-distance ones (Isomap,
        Laplacian Eigenmaps, LPP, SPE, Manifold Sculpting; callbacks/eigen_callbacks.hpp:52-64):
        k above N - 1 is clamped with a warning, and while the graph is not connected
        (is_connected, neighbors/connected.hpp:19-62) the search is redone with 2k.
        The ranking is by the exact squared Euclidean distance, which orders both the
        kernel-trick and the plain distance. Returns (idx N x k_used, k_used) or, with
        return_distances, (idx, distances N x k_used = sqrt(d2), k_used)."""
        xb, _ = _as_points(X)
        N = int(xb.arr.shape[0])
        if N < 2:
            raise WrongParameterError("at least 2 points are needed to find neighbours")
        k = int(k)
        if k < 1:
            raise WrongParameterError(f"num_neighbors {k} must be at least 1")
        if k > N - 1:
            self._log(1, "Number of neighbors is greater than number of objects to embed. "
                         "Using greatest possible number of neighbors.")
            k = N - 1
        while True:
            idx, d2 = self.knn_brute(X, k, screen=screen, return_distances=True)
            if not check_connectivity or self.check_connected(idx) or k >= N - 1:
                break
            self._log(1, f"The neighborhood graph with {k} neighbors is not connected. "
                         f"Recomputing with a larger number of neighbors {min(2 * k, N - 1)}.")
            k = min(2 * k, N - 1)
        if return_distances:
            dist = d2.sqrt() if _is_torch(d2) else np.sqrt(d2)
            return idx, dist, k
        return idx, k

    def check_connected(self, idx):
        """Reachability of all vertices from vertex 0 (neighbors/connected.hpp:19-62)."""
        ib = _as_index(idx, None)
        N, k = ib.arr.shape
        c = ctypes.c_int()
        self._check(self.lib.tk_check_connected(self.ptr, N, k, ib.ptr, ctypes.byref(c)))
        return bool(c.value)

    def lle_weights(self, X, idx, klle_shift=1e-3):
        """LLE reconstruction weights (routines/locally_linear.hpp:107-131)."""
        xb, dt = _as_points(X)
        ib = _as_index(idx, xb)
        N, D = xb.arr.shape
        k = ib.arr.shape[1]
        W = _empty((N, k), np.float64, xb)
        self._check(self.lib.tk_lle_weights(self.ptr, xb.ptr, dt, N, D, D, ib.ptr, k, float(klle_shift), W.ptr))
        return W.arr

    def ltsa_basis(self, X, idx, target_dimension=2):
        """LTSA tangent bases V (N x k x td) (routines/locally_linear.hpp:45-63)."""
        xb, dt = _as_points(X)
        ib = _as_index(idx, xb)
        N, D = xb.arr.shape
        k = ib.arr.shape[1]
        V = _empty((N, k, target_dimension), np.float64, xb)
        self._check(self.lib.tk_ltsa_basis(self.ptr, xb.ptr, dt, N, D, D, ib.ptr, k, int(target_dimension), V.ptr))
        return V.arr

    def hessian_basis(self, X, idx, target_dimension=2):
        """Hessian LLE product columns Yr (N x k x td(td+1)/2); the point's block
        is B = Yr Yr^T (routines/locally_linear.hpp:183-234)."""
        xb, dt = _as_points(X)
        ib = _as_index(idx, xb)
        N, D = xb.arr.shape
        k = ib.arr.shape[1]
        td = int(target_dimension)
        Y = _empty((N, k, td * (td + 1) // 2), np.float64, xb)
        self._check(self.lib.tk_hessian_basis(self.ptr, xb.ptr, dt, N, D, D, ib.ptr, k, td, Y.ptr))
        return Y.arr

    def assemble(self, method, idx, weights, shift, target_dimension=None):
        """M in CSR (routines/locally_linear.hpp:133-146 / :65-77 / :236-243 +
        utils/sparse.hpp:16-21). weights: W (N x k) for LLE, V (N x k x td) for
        LTSA, Yr (N x k x td(td+1)/2) for HLLE, whose target_dimension is derived
        from the column count unless given."""
        m = METHODS[method] if isinstance(method, str) else int(method)
        ib = _as_index(idx, None)
        wb = _as_f64(weights)
        N, k = ib.arr.shape
        td = wb.arr.shape[2] if wb.arr.ndim == 3 else 0
        if m == C.TK_METHOD_HLLE:
            td = int(target_dimension) if target_dimension is not None else {1: 1, 3: 2}.get(td, 0)
        rp = _empty((N + 1,), np.int64, wb)
        nnz = ctypes.c_int64(0)
        self._check(self.lib.tk_assemble(self.ptr, m, N, k, td, ib.ptr, wb.ptr, float(shift), rp.ptr, None, None,
                                         ctypes.byref(nnz)))
        col = _empty((nnz.value,), np.int32, wb)
        val = _empty((nnz.value,), np.float64, wb)
        self._check(self.lib.tk_assemble(self.ptr, m, N, k, td, ib.ptr, wb.ptr, float(shift), rp.ptr, col.ptr,
                                         val.ptr, ctypes.byref(nnz)))
        return rp.arr, col.arr, val.arr

    def eigenproblem_pair(self, kind, X, row_ptr, col_idx, vals):
        """The NPE ("npe", from the LLE matrix M) or LLTSA ("lltsa", from the LTSA
        matrix M) dense pair (lhs, rhs), D x D, as
        routines/locally_linear.hpp:257-338 leaves them: lhs on its upper
        triangle (lower zero), rhs symmetric with halved off-diagonal entries."""
        k = {"npe": C.TK_PAIR_NPE, "lltsa": C.TK_PAIR_LLTSA}[kind] if isinstance(kind, str) else int(kind)
        xb, dt = _as_points(X)
        if xb.arr.ndim != 2:
            raise WrongParameterError("X must be 2-D (points x features)")
        N, D = xb.arr.shape
        rp = _Buf(np.ascontiguousarray(np.asarray(row_ptr, dtype=np.int64)), "np") if not _is_torch(row_ptr) \
            else _Buf(row_ptr.to(_torch().int64).contiguous(), "torch")
        ci = _as_index(col_idx, xb)
        vb = _as_f64(vals)
        lhs = np.zeros(D * D, np.float64)
        rhs = np.zeros(D * D, np.float64)
        self._check(self.lib.tk_eigenproblem_pair(self.ptr, k, xb.ptr, dt, N, D, D, rp.ptr, ci.ptr, vb.ptr,
                                                  lhs.ctypes.data, rhs.ctypes.data))
        # column-major D x D -> [a, b]
        return lhs.reshape(D, D).T.copy(), rhs.reshape(D, D).T.copy()

    def smallest_eigenvectors(self, row_ptr, col_idx, vals, target_dimension, skip=1, tol=None, max_matvecs=None,
                              return_info=False):
        """The target_dimension smallest eigenpairs of the symmetric CSR matrix M
        after skipping `skip` (eigendecomposition(Arpack, SmallestEigenvalues, M, td),
        routines/eigendecomposition.hpp:31-50,252-266): Chebyshev-filtered subspace
        iteration on the GPU. Returns (vectors N x td, values td), each vector's
        entry of largest magnitude positive; raises EigendecompositionError when the
        residual does not reach tol * B within max_matvecs block products."""
        rp = _Buf(np.ascontiguousarray(np.asarray(row_ptr, dtype=np.int64)), "np") if not _is_torch(row_ptr) \
            else _Buf(row_ptr.to(_torch().int64).contiguous(), "torch")
        N = int(rp.arr.shape[0]) - 1
        ci = _as_index(col_idx, rp)
        vb = _as_f64(vals)
        td = int(target_dimension)
        vec = _empty((td, N), np.float64, rp)
        lam = _empty((td,), np.float64, rp)
        info = C.tk_eig_info()
        self._check(self.lib.tk_smallest_eigenvectors(self.ptr, N, rp.ptr, ci.ptr, vb.ptr, td, int(skip),
                                                      float(tol or 0.0), int(max_matvecs or 0), vec.ptr, lam.ptr,
                                                      ctypes.byref(info)))
        out = (vec.arr.T, lam.arr)
        if return_info:
            return out + ({"iterations": info.iterations, "block": info.block, "matvecs": info.matvecs,
                           "spectrum_bound": info.spectrum_bound, "max_residual": info.max_residual,
                           "converged": bool(info.converged), "ms": info.ms},)
        return out

    def local_operator(self, X, method="lle", num_neighbors=5, target_dimension=2, klle_shift=1e-3,
                       nullspace_shift=1e-9, check_connectivity=True, screen="tensor", cancel_function=None,
                       copy_out=True):
        """The whole stage of KLLE / KLTSA / HLLE embed() up to the eigensolver.
        HLLE adds no diagonal shift (nullspace_shift and klle_shift are unused)."""
        if method not in METHODS:
            raise UnsupportedMethodError(f"method {method!r} is not provided by this library")
        xb, dt = _as_points(X)
        if xb.arr.ndim != 2:
            raise WrongParameterError("X must be 2-D (points x features)")
        N, D = xb.arr.shape
        p = C.tk_params()
        self.lib.tk_params_default(ctypes.byref(p))
        p.method = METHODS[method]
        p.num_neighbors = int(num_neighbors)
        p.target_dimension = int(target_dimension)
        p.klle_shift = float(klle_shift)
        p.nullspace_shift = float(nullspace_shift)
        p.check_connectivity = 1 if check_connectivity else 0
        p.screen = SCREENS[screen]
        if cancel_function is not None:
            cb = C.CANCEL_FN(lambda: 1 if cancel_function() else 0)
            p.cancel_function = cb
        info = C.tk_operator_info()
        self._check(self.lib.tk_local_operator(self.ptr, ctypes.byref(p), xb.ptr, dt, N, D, D, ctypes.byref(info)))
        stage = dict(knn=info.stage_ms[0], connectivity=info.stage_ms[1], weights=info.stage_ms[2],
                     assembly=info.stage_ms[3], total=info.stage_ms[4])
        if not copy_out:
            return info
        k, td = info.k, info.target_dimension
        wshape = {C.TK_METHOD_KLLE: (N, k), C.TK_METHOD_KLTSA: (N, k, td)}.get(info.method, (N, k, td * (td + 1) // 2))
        idx = _empty((N, k), np.int32, xb)
        w = _empty(wshape, np.float64, xb)
        rp = _empty((N + 1,), np.int64, xb)
        col = _empty((info.nnz,), np.int32, xb)
        val = _empty((info.nnz,), np.float64, xb)
        self._check(self.lib.tk_operator_copy(self.ptr, idx.ptr, w.ptr, rp.ptr, col.ptr, val.ptr))
        return LocalOperator(idx.arr, w.arr, rp.arr, col.arr, val.arr, k, info.method, td,
                             info.connectivity_retries, info.rows_uncertified, stage, info.tie_rows,
                             info.extra_rows)

    def synchronize(self):
        self._check(self.lib.tk_ctx_synchronize(self.ptr))


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


# ---------------------------------------------------------------- eigensolver


# Largest N of the dense eigensolver path (a 16384 x 16384 FP64 matrix is 2 GiB).
DENSE_EIGEN_MAX_N = 16384


def smallest_eigenvectors(op: LocalOperator, target_dimension: int, skip: int = 1, eigen_method: str = "arpack",
                          context=None):
    """Consumes the CSR of M unchanged and returns (vectors N x td, values td) as
    numpy arrays: the eigenvectors of the target_dimension smallest eigenvalues
    after skipping `skip`.
    - "arpack", the reference default (defines/methods.hpp:198): the GPU
      Chebyshev-filtered subspace iteration of tk_smallest_eigenvectors
      (routines/eigendecomposition.hpp:31-50,252-266). Problems smaller than four
      block widths go to the dense solver below.
    - "dense" (routines/eigendecomposition.hpp:56-87): symmetrise, self-adjoint
      solve of the dense N x N matrix on the GPU in FP64, columns skip..skip+td;
      refused with WrongParameterError above N = DENSE_EIGEN_MAX_N."""
    if eigen_method not in ("arpack", "dense"):
        raise UnsupportedMethodError(f"eigen_method {eigen_method!r} is not provided (use 'arpack' or 'dense')")
    n = len(op.row_ptr) - 1
    if eigen_method == "arpack":
        if n >= 128 and target_dimension + skip <= 14:
            ctx = context or default_context()
            E, w = ctx.smallest_eigenvectors(op.row_ptr, op.col_idx, op.vals, target_dimension, skip)
            if _is_torch(E):
                E, w = E.cpu().numpy(), w.cpu().numpy()
            return np.ascontiguousarray(E), np.asarray(w)
    if n > DENSE_EIGEN_MAX_N:
        raise WrongParameterError(
            f"the dense eigensolver holds the N x N matrix in FP64 ({8 * n * n / 2**30:.1f} GiB at N = {n}); "
            f"it accepts N <= {DENSE_EIGEN_MAX_N}: use eigen_method='arpack' (td + skip <= 14)")
    torch = _torch()
    dev = "cuda"
    rp = torch.as_tensor(np.asarray(op.row_ptr.cpu() if _is_torch(op.row_ptr) else op.row_ptr)).to(dev)
    ci = torch.as_tensor(np.asarray(op.col_idx.cpu() if _is_torch(op.col_idx) else op.col_idx)).to(dev)
    v = torch.as_tensor(np.asarray(op.vals.cpu() if _is_torch(op.vals) else op.vals)).to(dev)
    M = torch.sparse_csr_tensor(rp, ci.to(torch.int64), v, size=(n, n)).to_dense()
    M = (M + M.T) / 2
    try:
        w, V = torch.linalg.eigh(M)
    except Exception as e:  # pragma: no cover
        raise EigendecompositionError(str(e))
    return V[:, skip:skip + target_dimension].cpu().numpy(), w[skip:skip + target_dimension].cpu().numpy()


# ---------------------------------------------------------------- reference-shaped entry points


_KNOWN_KW = ("method", "neighbors_method", "eigen_method", "num_neighbors", "target_dimension",
             "nullspace_shift", "klle_shift", "check_connectivity", "screen", "cancel_function")


def embed(data, method="lle", neighbors_method=None, eigen_method=None, num_neighbors=None, target_dimension=None,
          nullspace_shift=None, klle_shift=None, check_connectivity=None, screen="tensor", context=None,
          **unsupported):
    """Python signature of the reference module's ``embed`` for the methods this
    library provides (KLLE, KLTSA, HLLE with brute-force neighbours). ``data`` is
    features x samples; returns samples x target_dimension (numpy)."""
    for key, val in unsupported.items():
        if val is not None:
            raise UnsupportedMethodError(f"parameter {key!r} is not used by the local-neighborhood methods")
    if method not in METHODS:
        raise UnsupportedMethodError(f"method {method!r} is not provided by this library")
    if neighbors_method not in (None, "brute"):
        raise UnsupportedMethodError("only neighbors_method='brute' is provided")
    X = data.T if not _is_torch(data) else data.t()
    td = 2 if target_dimension is None else int(target_dimension)
    ctx = context or default_context()
    op = ctx.local_operator(X, method=method, num_neighbors=5 if num_neighbors is None else num_neighbors,
                            target_dimension=td, klle_shift=1e-3 if klle_shift is None else klle_shift,
                            nullspace_shift=1e-9 if nullspace_shift is None else nullspace_shift,
                            check_connectivity=True if check_connectivity is None else bool(check_connectivity),
                            screen=screen)
    E, _ = smallest_eigenvectors(op, td, 1, eigen_method or "arpack", ctx)
    return E


@dataclass
class TapkeeOutput:
    embedding: np.ndarray
    operator: LocalOperator | None = None


class ParametersInitializedState:
    """``tapkee::with(parameters)`` (chain_interface.hpp:497-500)."""

    def __init__(self, params: dict):
        self.params = dict(params)

    def embed_using(self, matrix, context=None) -> TapkeeOutput:
        """``embedUsing(const DenseMatrix&)`` (chain_interface.hpp:471-480): matrix is
        features x samples (column = point)."""
        p = self.params
        if "method" not in p:
            raise MissedParameterError("missed parameter: dimension reduction method")
        ctx = context or default_context()
        X = matrix.T if not _is_torch(matrix) else matrix.t()
        td = p.get("target_dimension", 2)
        op = ctx.local_operator(X, method=p["method"], num_neighbors=p.get("num_neighbors", 5),
                                target_dimension=td, klle_shift=p.get("klle_shift", 1e-3),
                                nullspace_shift=p.get("nullspace_shift", 1e-9),
                                check_connectivity=p.get("check_connectivity", True),
                                screen=p.get("screen", "tensor"), cancel_function=p.get("cancel_function"))
        E, _ = smallest_eigenvectors(op, td, 1, p.get("eigen_method", "arpack"), ctx)
        return TapkeeOutput(E, op)

    embedUsing = embed_using


def with_(*param_sets, **kwargs) -> ParametersInitializedState:
    """Keyword-set form of ``tapkee::with((kw=value, ...))``. A keyword given
    twice (across dicts and kwargs) raises MultipleParameterError, like
    ParametersSet::check (stichwort/parameter.hpp:232-310)."""
    merged = {}
    for d in list(param_sets) + [kwargs]:
        for key, val in d.items():
            if key in merged:
                raise MultipleParameterError(f"parameter {key!r} is set more than once")
            if key not in _KNOWN_KW:
                raise UnsupportedMethodError(f"parameter {key!r} is not used by the local-neighborhood methods")
            merged[key] = val
    if "neighbors_method" in merged and merged["neighbors_method"] != "brute":
        raise UnsupportedMethodError("only neighbors_method='brute' is provided")
    return ParametersInitializedState(merged)
