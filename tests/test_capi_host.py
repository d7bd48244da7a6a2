"""C ABI library and host-side logic (no GPU work)."""
import ctypes
import os
import re

import numpy as np
import pytest

import tapkee_gb300 as tk
from tapkee_gb300 import _capi, datasets

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from tapkee_gb300 import build as tkbuild
    tkbuild.build()
    return _capi.load()


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "tapkee_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tk_[a-z_0-9]+)\s*\(", text)) - {"tk_log_fn"})


def test_library_exports_every_declared_symbol(lib):
    syms = _declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), f"{s} declared in include/tapkee_gb300.h but not exported"
    # the binding covers exactly the declared API
    assert set(syms) == set(_capi.SIGNATURES), set(syms) ^ set(_capi.SIGNATURES)


def test_pure_host_entry_points(lib):
    assert lib.tk_version().decode().count(".") == 2
    assert lib.tk_status_string(0) == b"ok"
    assert lib.tk_status_string(6) == b"cancelled"
    p = _capi.tk_params()
    lib.tk_params_default(ctypes.byref(p))
    # reference keyword defaults (defines/keywords.hpp)
    assert p.num_neighbors == 5 and p.target_dimension == 2
    assert p.klle_shift == 1e-3 and p.nullspace_shift == 1e-9 and p.check_connectivity == 1


def test_no_device_is_reported_not_crashed(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    ptr = ctypes.c_void_p()
    rc = lib.tk_ctx_create(0, None, ctypes.byref(ptr))
    assert rc == _capi.TK_ERR_NO_DEVICE and not ptr.value
    assert lib.tk_ctx_destroy(None) == 0


def test_with_rejects_duplicate_and_unknown_keywords():
    with pytest.raises(tk.MultipleParameterError):
        tk.with_({"num_neighbors": 6}, num_neighbors=5)
    with pytest.raises(tk.UnsupportedMethodError):
        tk.with_(method="lle", sne_perplexity=10.0)
    with pytest.raises(tk.UnsupportedMethodError):
        tk.with_(method="lle", neighbors_method="vptree")
    st = tk.with_(method="lle", neighbors_method="brute", num_neighbors=8)
    assert st.params["num_neighbors"] == 8


def test_embed_rejects_unprovided_methods():
    with pytest.raises(tk.UnsupportedMethodError):
        tk.embed(np.zeros((3, 10)), method="isomap")
    with pytest.raises(tk.UnsupportedMethodError):
        tk.embed(np.zeros((3, 10)), method="lle", neighbors_method="covertree")


def test_datasets_are_seeded_and_shaped():
    a = datasets.lifted_swiss_roll(1000, 64, seed=1)
    b = datasets.lifted_swiss_roll(1000, 64, seed=1)
    assert a.dtype == np.float32 and a.shape == (1000, 64)
    assert np.array_equal(a, b)
    c = datasets.lifted_s_curve(500, 32)
    assert c.shape == (500, 32)
    specs = datasets.batch_problems(16)
    assert all(500 <= n <= 20000 and d in (3, 16, 64, 128) and k in (8, 12, 16, 24, 32) for n, d, k, _ in specs)
    X = datasets.swiss_roll(2000, seed=0)
    assert X.shape == (2000, 3)


def test_noalloc_entry_point_host_checks(lib):
    """tk_check_connected_noalloc refuses bad sizes and arguments on the host,
    before any CUDA call, and writes the reason into the caller's buffer."""
    c = ctypes.c_int(-1)
    msg = ctypes.create_string_buffer(256)
    dummy = ctypes.c_void_p(16)  # never dereferenced: every call below fails first

    def call(n, k=2, idx=dummy, out=ctypes.byref(c), device=0):
        msg.value = b"stale"
        return lib.tk_check_connected_noalloc(device, None, n, k, idx, out, msg, len(msg))

    assert call(0) == _capi.TK_ERR_NO_DATA and msg.value == b"No data"
    assert call(10, k=0) == _capi.TK_ERR_INVALID_ARG
    assert call(10, idx=None) == _capi.TK_ERR_INVALID_ARG
    assert call(10, out=None) == _capi.TK_ERR_INVALID_ARG
    st = call(_capi.TK_NOALLOC_MAX_POINTS + 1)
    assert st == _capi.TK_ERR_INVALID_ARG
    assert str(_capi.TK_NOALLOC_MAX_POINTS) in msg.value.decode() and b"limit" in msg.value
    assert call(10, device=-1) == _capi.TK_ERR_NO_DEVICE
    assert c.value == -1
    # a NULL or empty message buffer is allowed
    assert lib.tk_check_connected_noalloc(0, None, 0, 2, dummy, ctypes.byref(c), None, 0) == _capi.TK_ERR_NO_DATA
    import torch
    if not torch.cuda.is_available():
        assert call(10) == _capi.TK_ERR_NO_DEVICE and msg.value.startswith(b"no CUDA device")
