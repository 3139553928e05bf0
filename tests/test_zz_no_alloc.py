"""The forward entry point that allocates nothing (jc_forward_device_noalloc).

It serves callers that cannot call cudaMalloc when they run the model: host
applications whose own pool allocator has reserved the whole device, and
plugins that work only in the buffers their host hands them. Its buffers
live in a fixed 12 MiB device array inside the library. Here it is called
through the C ABI and compared with jc_forward_device (which uses the model's
own allocated workspace), on two calls in a row, up to the largest grid the
array holds (128 x 128 at dim 128); grids that need more are refused with
JC_LIMIT, and the device's free memory is unchanged across calls.
"""

import ctypes as C

import numpy as np
import pytest

from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import meta_of, parse_config, synthetic_checkpoint, write_safetensors_bytes
from jacobi2000_gb300.ic import random_drops

pytestmark = pytest.mark.gpu

# the FP32 forward tests hold the path to 1e-5 max abs against the golden
# vectors; both entry points run the same kernels, so that tolerance is ample
TOL = 1e-5


def _lib():
    L = engine.load_library()
    L.jc_forward_device_noalloc.argtypes = [C.c_void_p] * 5
    L.jc_forward_device_noalloc.restype = C.c_int
    return L


def _cases(pt_tiny, extra):
    t, cj = synthetic_checkpoint(32, 128, 4, 0)
    # 128 x 128 at dim 128: the largest grid the 12 MiB array holds
    t128, cj128 = synthetic_checkpoint(128, 128, 4, 0)
    cfg128 = parse_config(cj128, t128)
    return [
        (pt_tiny["st_bytes"], pt_tiny["config"], pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"]),
        (write_safetensors_bytes(t), cj, extra["c1_state"], extra["c1_meta"]),
        (write_safetensors_bytes(t128), cj128, random_drops(cfg128, seed=3), meta_of(cfg128)),
    ]


def test_noalloc_forward_matches_forward_device(pt_tiny, extra):
    torch = pytest.importorskip("torch")
    L = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    for st, cj, state, meta in _cases(pt_tiny, extra):
        with engine.Model.from_bytes(st, cj, engine.FP32) as m:
            ds = torch.from_numpy(np.ascontiguousarray(state)).cuda()
            dm = torch.from_numpy(np.ascontiguousarray(meta)).cuda()
            want_d = torch.empty_like(ds)
            engine._check(L.jc_forward_device(m._h, ds.data_ptr(), dm.data_ptr(), want_d.data_ptr(), stream))
            torch.cuda.synchronize()
            want = want_d.cpu().numpy()
            for _ in range(2):  # two calls in a row share the library's array
                got_d = torch.full_like(ds, float("nan"))
                status = L.jc_forward_device_noalloc(m._h, ds.data_ptr(), dm.data_ptr(), got_d.data_ptr(), stream)
                engine._check(status)
                torch.cuda.synchronize()
                got = got_d.cpu().numpy()
                assert np.all(np.isfinite(got))
                assert np.abs(got - want).max() <= TOL


def test_noalloc_bf16_model_runs_the_fp32_kernels_and_allocates_nothing(extra):
    """A model created with BF16 precision keeps its f32 weights; this entry
    point runs the FP32 kernels on them, so its result equals the FP32
    model's jc_forward_device. After a first call (which looks up the
    array's address), further calls leave the device's free memory as it
    was."""
    torch = pytest.importorskip("torch")
    L = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    t, cj = synthetic_checkpoint(32, 128, 4, 0)
    st = write_safetensors_bytes(t)
    ds = torch.from_numpy(np.ascontiguousarray(extra["c1_state"])).cuda()
    dm = torch.from_numpy(np.ascontiguousarray(extra["c1_meta"])).cuda()
    want_d, got_d = torch.empty_like(ds), torch.empty_like(ds)
    with engine.Model.from_bytes(st, cj, engine.FP32) as m32:
        engine._check(L.jc_forward_device(m32._h, ds.data_ptr(), dm.data_ptr(), want_d.data_ptr(), stream))
    with engine.Model.from_bytes(st, cj, engine.BF16) as m16:
        engine._check(L.jc_forward_device_noalloc(m16._h, ds.data_ptr(), dm.data_ptr(), got_d.data_ptr(), stream))
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            engine._check(L.jc_forward_device_noalloc(m16._h, ds.data_ptr(), dm.data_ptr(), got_d.data_ptr(),
                                                      stream))
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert np.abs(got_d.cpu().numpy() - want_d.cpu().numpy()).max() <= TOL


def test_noalloc_refuses_grids_beyond_its_array():
    torch = pytest.importorskip("torch")
    L = _lib()
    t, cj = synthetic_checkpoint(256, 128, 4, 0)
    with engine.Model.from_bytes(write_safetensors_bytes(t), cj, engine.FP32) as m:
        ds = torch.zeros((3, 256, 256), device="cuda")
        dm = torch.zeros(5, device="cuda")
        out = torch.zeros_like(ds)
        status = L.jc_forward_device_noalloc(m._h, ds.data_ptr(), dm.data_ptr(), out.data_ptr(),
                                             torch.cuda.current_stream().cuda_stream)
        assert engine.STATUS[status] == "LIMIT"
        assert "12 MiB" in L.jc_last_error().decode()
