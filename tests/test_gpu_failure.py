"""The failure path of the bounded device waits, made to run out on purpose
without faulting the GPU: one CTA waits with the distance screen's own wait
helper on an mbarrier that nothing arrives at. The wait gives up after its
limit, the kernel records the timeout and returns, the host reads TK_ERR_TIMEOUT,
and the context keeps working afterwards."""
import ctypes
import time

import numpy as np
import pytest

import tapkee_gb300 as tk
from tapkee_gb300 import _capi as C
from tapkee_gb300 import datasets

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_context_survives(ctx, golden):
    outcome = ctypes.c_int(0)
    t0 = time.perf_counter()
    st = ctx.lib.tk_selftest_bounded_wait(ctx.ptr, ctypes.byref(outcome))
    elapsed = time.perf_counter() - t0
    assert st == C.TK_ERR_TIMEOUT
    assert outcome.value == 1  # the wait expired; it did not complete
    assert "bounded wait expired" in ctx.lib.tk_last_error(ctx.ptr).decode()
    assert 1.5 < elapsed < 30.0  # the 2 s limit, not a hang
    # the error word was cleared and the context still computes the right thing
    X = datasets.swiss_roll(2000, seed=0)
    op = ctx.local_operator(X, "lle", num_neighbors=12, klle_shift=1e-3)
    assert np.array_equal(op.idx, golden["lle_idx"])
    # and through the Python error mapping
    with pytest.raises(tk.DeviceError, match="bounded wait expired"):
        ctx._check(ctx.lib.tk_selftest_bounded_wait(ctx.ptr, None))


def test_grid_barrier_wait_expires_and_context_survives(ctx, golden):
    """The connectivity check's grid barrier (cooperative launch): CTA 0 never
    arrives, the other CTAs give up after the 2 s limit, and the next check on the
    same context is right (its state is cleared per call)."""
    outcome = ctypes.c_int(0)
    t0 = time.perf_counter()
    st = ctx.lib.tk_selftest_grid_barrier(ctx.ptr, ctypes.byref(outcome))
    elapsed = time.perf_counter() - t0
    assert st == C.TK_ERR_TIMEOUT
    assert outcome.value == 1
    assert "bounded wait expired" in ctx.lib.tk_last_error(ctx.ptr).decode()
    assert 1.5 < elapsed < 30.0
    assert ctx.check_connected(golden["lle_idx"]) is True
    rng = np.random.default_rng(0)
    two = np.concatenate([rng.normal(size=(60, 2)), rng.normal(size=(60, 2)) + 100.0])
    assert ctx.check_connected(ctx.knn_brute(two, 5)) is False
