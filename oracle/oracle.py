"""ctypes wrapper of the CPU oracle (oracle/tapkee_oracle.cpp).

TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm may import this module. The product path
(tapkee_gb300) never does.

The oracle restates, in FP64, the reference's brute kNN
(neighbors/neighbors.hpp:119-149), connectivity DFS (neighbors/connected.hpp:19-62),
LLE weights (routines/locally_linear.hpp:90-159), LTSA tangent basis
(routines/locally_linear.hpp:20-88), Hessian LLE blocks
(routines/locally_linear.hpp:161-255) and triplet assembly (utils/sparse.hpp:16-21).
Parity status: kNN sets pinned by the reference's 1-D line known-answer test;
W / M / LTSA values unpinned by the reference (it has no golden values for them)
and cross-checked against scikit-learn fixtures in tests/golden/. The dense
eigen step (dense_embedding) reproduces the reference's sparse
smallest-eigenvector known answer (test/unit/eigendecomposition.cpp:30-50).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libtapkee_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library (g++ -O3 -fopenmp)."""
    src = os.path.join(_HERE, "tapkee_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
        subprocess.check_call(["g++", "-O3", "-fopenmp", "-fPIC", "-std=c++17", "-shared",
                               "-o", _LIB_PATH, src])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        i64, i32, dptr, iptr = ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p
        L.oracle_knn_brute.argtypes = [dptr, i64, i64, i32, iptr, dptr, iptr, iptr, i32]
        L.oracle_knn_brute.restype = i32
        L.oracle_knn_brute_rows.argtypes = [dptr, i64, i64, i32, iptr, i64, iptr, i32]
        L.oracle_knn_brute_rows.restype = i32
        L.oracle_is_connected.argtypes = [i64, i32, iptr]
        L.oracle_is_connected.restype = i32
        L.oracle_lle_weights.argtypes = [dptr, i64, i64, iptr, i32, ctypes.c_double, dptr, i32]
        L.oracle_lle_weights.restype = i32
        L.oracle_lle_weights_rows.argtypes = [dptr, i64, i64, iptr, i64, iptr, i32, ctypes.c_double, dptr, i32]
        L.oracle_lle_weights_rows.restype = i32
        L.oracle_ltsa_basis.argtypes = [dptr, i64, i64, iptr, i32, i32, dptr, dptr, i32]
        L.oracle_ltsa_basis.restype = i32
        L.oracle_hessian_blocks.argtypes = [dptr, i64, i64, iptr, i32, i32, dptr, i32]
        L.oracle_hessian_blocks.restype = i32
        L.oracle_assemble.argtypes = [i32, i64, i32, i32, iptr, dptr, ctypes.c_double, dptr, dptr, dptr, i64]
        L.oracle_assemble.restype = i64
        L.oracle_eigenproblem_pair.argtypes = [i32, i64, i32, dptr, dptr, iptr, dptr, dptr, dptr]
        L.oracle_eigenproblem_pair.restype = None
        _lib = L
    return _lib


def _threads(nthreads):
    return int(nthreads) if nthreads else (os.cpu_count() or 1)


def _X64(X):
    return np.ascontiguousarray(np.asarray(X, dtype=np.float64))


def knn_brute(X, k, nthreads=None, return_extra=False):
    """Returns (idx N x k int32 in partition order, dist N x k, row_count N) and,
    with return_extra, also extra N: the (k+1)-th reference neighbour of rows with
    row_count k + 1, -1 elsewhere."""
    X = _X64(X)
    N, D = X.shape
    idx = np.zeros((N, k), np.int32)
    dist = np.zeros((N, k), np.float64)
    cnt = np.zeros(N, np.int32)
    extra = np.full(N, -1, np.int32)
    rc = lib().oracle_knn_brute(X.ctypes.data, N, D, k, idx.ctypes.data, dist.ctypes.data, cnt.ctypes.data,
                                extra.ctypes.data, _threads(nthreads))
    if rc != 0:
        raise ValueError("oracle_knn_brute: invalid arguments")
    return (idx, dist, cnt, extra) if return_extra else (idx, dist, cnt)


def knn_brute_rows(X, k, rows, nthreads=None):
    X = _X64(X)
    N, D = X.shape
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    idx = np.zeros((len(rows), k), np.int32)
    rc = lib().oracle_knn_brute_rows(X.ctypes.data, N, D, k, rows.ctypes.data, len(rows), idx.ctypes.data,
                                     _threads(nthreads))
    if rc != 0:
        raise ValueError("oracle_knn_brute_rows: invalid arguments")
    return idx


def is_connected(idx):
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    return bool(lib().oracle_is_connected(idx.shape[0], idx.shape[1], idx.ctypes.data))


def find_neighbors(X, k, check_connectivity=True, nthreads=None):
    """neighbors/neighbors.hpp:173-213: clamp k to N-1, brute kNN, and while the
    graph is not connected recompute with 2k. Returns (idx, k_used)."""
    N = np.asarray(X).shape[0]
    if k > N - 1:
        k = N - 1
    idx, _, _ = knn_brute(X, k, nthreads)
    if check_connectivity and not is_connected(idx):
        return find_neighbors(X, 2 * k, check_connectivity, nthreads)
    return idx, k


def lle_weights(X, idx, klle_shift=1e-3, nthreads=None):
    X = _X64(X)
    N, D = X.shape
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    k = idx.shape[1]
    W = np.zeros((N, k), np.float64)
    lib().oracle_lle_weights(X.ctypes.data, N, D, idx.ctypes.data, k, float(klle_shift), W.ctypes.data,
                             _threads(nthreads))
    return W


def lle_weights_rows(X, rows, idx_rows, klle_shift=1e-3, nthreads=None):
    """LLE weights of the points `rows` (int64) with neighbour rows idx_rows."""
    X = _X64(X)
    N, D = X.shape
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    idx_rows = np.ascontiguousarray(idx_rows, dtype=np.int32)
    k = idx_rows.shape[1]
    W = np.zeros((len(rows), k), np.float64)
    lib().oracle_lle_weights_rows(X.ctypes.data, N, D, rows.ctypes.data, len(rows), idx_rows.ctypes.data, k,
                                  float(klle_shift), W.ctypes.data, _threads(nthreads))
    return W


def ltsa_basis(X, idx, td=2, nthreads=None, return_evals=False):
    """Tangent bases of the neighbourhoods idx (one row per neighbourhood; the
    rows may be any subset of the points, since LTSA's Gram uses neighbours only)."""
    X = _X64(X)
    D = X.shape[1]
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    rows, k = idx.shape
    V = np.zeros((rows, k, td), np.float64)
    ev = np.zeros((rows, k), np.float64)
    lib().oracle_ltsa_basis(X.ctypes.data, rows, D, idx.ctypes.data, k, td, V.ctypes.data, ev.ctypes.data,
                            _threads(nthreads))
    return (V, ev) if return_evals else V


def hessian_blocks(X, idx, td=2, nthreads=None):
    """Per-neighbourhood Hessian LLE blocks B (rows x k x k) of
    hessian_weight_matrix (routines/locally_linear.hpp:161-255); td is 1 or 2
    (the reference's product-column placement is defined for those only)."""
    X = _X64(X)
    D = X.shape[1]
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    rows, k = idx.shape
    B = np.zeros((rows, k, k), np.float64)
    rc = lib().oracle_hessian_blocks(X.ctypes.data, rows, D, idx.ctypes.data, k, int(td), B.ctypes.data,
                                     _threads(nthreads))
    if rc != 0:
        raise ValueError("the Hessian blocks are defined for target_dimension 1 or 2")
    return B


def assemble(method, idx, weights, shift):
    """method 0 = LLE (weights = W, N x k), 1 = LTSA (weights = V, N x k x td),
    2 = Hessian (weights = B, N x k x k; shift unused).
    Returns (row_ptr int64, col_idx int32, vals float64)."""
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    N, k = idx.shape
    weights = np.ascontiguousarray(weights, dtype=np.float64)
    td = weights.shape[2] if weights.ndim == 3 else 0
    row_ptr = np.zeros(N + 1, np.int64)
    nnz = lib().oracle_assemble(int(method), N, k, td, idx.ctypes.data, weights.ctypes.data, float(shift),
                                row_ptr.ctypes.data, None, None, 0)
    nnz = int(row_ptr[-1])
    col = np.zeros(nnz, np.int32)
    vals = np.zeros(nnz, np.float64)
    got = lib().oracle_assemble(int(method), N, k, td, idx.ctypes.data, weights.ctypes.data, float(shift),
                                row_ptr.ctypes.data, col.ctypes.data, vals.ctypes.data, nnz)
    assert got == nnz
    return row_ptr, col, vals


def eigenproblem_pair(kind, X, row_ptr, col, vals):
    """The NPE (kind 0) or LLTSA (kind 1) dense eigenproblem pair (lhs, rhs), D x D,
    built as routines/locally_linear.hpp:257-338 builds them for the linear
    kernel (X points-major, N x D; M in CSR)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    N, D = X.shape
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    ci = np.ascontiguousarray(col, dtype=np.int32)
    v = np.ascontiguousarray(vals, dtype=np.float64)
    lhs = np.zeros((D, D), np.float64, order="F")
    rhs = np.zeros((D, D), np.float64, order="F")
    lib().oracle_eigenproblem_pair(int(kind), N, D, X.ctypes.data, rp.ctypes.data, ci.ctypes.data, v.ctypes.data,
                                   lhs.ctypes.data, rhs.ctypes.data)
    return lhs, rhs


def dense_embedding(row_ptr, col, vals, td):
    """Dense smallest-eigenvalue embedding, skip 1 (routines/eigendecomposition.hpp:56-87):
    symmetrise, eigh, columns 1..td."""
    N = len(row_ptr) - 1
    M = np.zeros((N, N))
    for r in range(N):
        M[r, col[row_ptr[r]:row_ptr[r + 1]]] = vals[row_ptr[r]:row_ptr[r + 1]]
    M = (M + M.T) / 2
    w, V = np.linalg.eigh(M)
    return V[:, 1:td + 1], w[1:td + 1]
