"""Bounded device-side waits: a wait that nothing satisfies gives up after its
limit, the kernel returns, and the call reports JC_DEVICE_TIMEOUT (the status
every batch, rollout and serving call maps a stalled device wait to, the
counterpart of lean_runtime::Error::Poll in crates/lean-runtime/src/error.rs:6-13).
The limit here is 1 ms; the production limit is 2 s. Nothing faults or hangs:
afterwards the same process still runs a forward on the GPU."""

import ctypes as C
import time

import numpy as np
import pytest

from jacobi2000_gb300 import engine

pytestmark = pytest.mark.gpu


def _lib():
    L = engine.load_library()
    L.jc_selftest_device_wait.argtypes = [C.c_int32, C.c_uint32]
    L.jc_selftest_device_wait.restype = C.c_int
    return L


def test_unsatisfied_wait_times_out_and_the_context_stays_usable(pt_tiny):
    L = _lib()
    t0 = time.perf_counter()
    status = L.jc_selftest_device_wait(0, 1000)
    elapsed = time.perf_counter() - t0
    assert engine.STATUS[status] == "DEVICE_TIMEOUT"
    assert "time limit" in L.jc_last_error().decode()
    assert elapsed < 5.0
    # the control case: the barrier completes, no timeout
    assert L.jc_selftest_device_wait(1, 1000) == 0
    # the context is intact: a forward still matches the golden vectors
    with engine.Model.from_bytes(pt_tiny["st_bytes"], pt_tiny["config"]) as m:
        out = m.forward(pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"])
    assert np.abs(out - pt_tiny["ref"]["forward_stencil"]).max() < 1e-5
