"""tk_check_connected_noalloc (static device scratch, no allocation) against
tk_check_connected (context arena), both called through the C ABI.

Kept in its own file, collected last, so it runs both after the other GPU tests
and alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from tapkee_gb300 import _capi, datasets

pytestmark = pytest.mark.gpu

MAX_N = _capi.TK_NOALLOC_MAX_POINTS


def _heap_graph(n, cut=False):
    """k = 2 out-edges per vertex: the binary-heap children 2i+1, 2i+2 (a self
    loop where a child would be >= n). cut=True drops the edge 0 -> 2, which
    leaves the subtree under vertex 2 unreachable from vertex 0."""
    i = np.arange(n, dtype=np.int64)
    idx = np.stack([2 * i + 1, 2 * i + 2], axis=1)
    idx = np.where(idx < n, idx, i[:, None])
    if cut:
        idx[0, 1] = 0
    return idx.astype(np.int32)


def _two_clusters():
    rng = np.random.default_rng(0)
    return np.concatenate([rng.normal(size=(60, 2)), rng.normal(size=(60, 2)) + 100.0])


def _existing(ctx, idx_dev):
    N, k = idx_dev.shape
    c = ctypes.c_int(-1)
    st = ctx.lib.tk_check_connected(ctx.ptr, N, k, ctypes.c_void_p(idx_dev.data_ptr()), ctypes.byref(c))
    assert st == _capi.TK_OK, ctx.lib.tk_last_error(ctx.ptr)
    return c.value


def _noalloc(lib, idx_dev, n=None):
    N, k = idx_dev.shape
    c = ctypes.c_int(-1)
    msg = ctypes.create_string_buffer(512)
    st = lib.tk_check_connected_noalloc(0, None, N if n is None else n, k, ctypes.c_void_p(idx_dev.data_ptr()),
                                        ctypes.byref(c), msg, len(msg))
    return st, c.value, msg.value.decode()


def test_noalloc_matches_context_entry_point(ctx):
    import torch
    lib = _capi.load()
    graphs = [
        ("heap at the size limit", _heap_graph(MAX_N)),
        ("swiss roll 2000, k=12", ctx.knn_brute(datasets.swiss_roll(2000, seed=0), 12)),
        ("two clusters, k=5", ctx.knn_brute(_two_clusters(), 5)),
        ("heap at the size limit, one edge cut", _heap_graph(MAX_N, cut=True)),
        ("lifted roll 200000 x 64, k=16", ctx.knn_brute(datasets.lifted_swiss_roll(), 16)),
        ("small heap", _heap_graph(1000)),
    ]
    seen = set()
    for name, idx in graphs:
        idx_dev = torch.from_numpy(np.ascontiguousarray(idx, dtype=np.int32)).to("cuda:0")
        want = _existing(ctx, idx_dev)
        for call in range(2):
            st, got, msg = _noalloc(lib, idx_dev)
            assert st == _capi.TK_OK, (name, call, msg)
            assert msg == ""
            assert got == want, (name, call)
        seen.add(want)
    assert seen == {0, 1}


def test_noalloc_rejections(ctx):
    import torch
    lib = _capi.load()
    idx_dev = torch.from_numpy(_heap_graph(1000)).to("cuda:0")
    # beyond the static scratch: refused on the host, nothing launched
    st, c, msg = _noalloc(lib, idx_dev, n=MAX_N + 1)
    assert st == _capi.TK_ERR_INVALID_ARG and c == -1
    assert str(MAX_N) in msg and "limit" in msg
    # host memory: refused (the entry point copies nothing)
    host = np.ascontiguousarray(_heap_graph(1000))
    c = ctypes.c_int(-1)
    msg = ctypes.create_string_buffer(512)
    st = lib.tk_check_connected_noalloc(0, None, 1000, 2, host.ctypes.data_as(ctypes.c_void_p), ctypes.byref(c),
                                        msg, len(msg))
    assert st == _capi.TK_ERR_INVALID_ARG and b"device" in msg.value
    # an index outside [0, N) reachable from vertex 0: the kernel's bounds check
    # reports it, and the next call starts from a clean error word
    bad = _heap_graph(1000)
    bad[1, 0] = 1005
    st, c, msg = _noalloc(lib, torch.from_numpy(bad).to("cuda:0"))
    assert st == _capi.TK_ERR_INVALID_ARG and "out of range" in msg
    st, c, msg = _noalloc(lib, idx_dev)
    assert st == _capi.TK_OK and c == 1


def test_noalloc_calls_allocate_no_device_memory(ctx):
    """After the set-up call, calls (up to the size limit) leave the device's free
    memory unchanged: nothing is allocated, by the library or by the runtime."""
    import torch
    lib = _capi.load()
    graphs = [torch.from_numpy(g).to("cuda:0") for g in
              (_heap_graph(MAX_N), _heap_graph(MAX_N, cut=True), _heap_graph(1000))]
    torch.cuda.synchronize()
    st, _, msg = _noalloc(lib, graphs[2])  # set-up (a no-op when an earlier test made it)
    assert st == _capi.TK_OK, msg
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    results = []
    for _ in range(3):
        for g in graphs:
            st, c, msg = _noalloc(lib, g)
            assert st == _capi.TK_OK, msg
            results.append(c)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)
    assert results == [1, 0, 1] * 3
