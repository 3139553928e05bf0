"""The C ABI without a GPU: the library loads and exports every symbol
include/jacobi2000.h declares; checkpoint errors map to status codes before
any device work; the host projections agree with the oracle."""

import ctypes as C
import json
import re

import numpy as np
import pytest

from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import read_safetensors, write_safetensors_bytes
from conftest import ROOT
from oracle.oracle import identity_config, projection_only


def test_header_symbols_are_exported():
    header = (ROOT / "include" / "jacobi2000.h").read_text()
    declared = set(re.findall(r"\b(jc_[a-z_0-9]+)\s*\(", header))
    L = engine.load_library()
    missing = [s for s in sorted(declared) if not hasattr(L, s)]
    assert not missing, missing
    assert declared >= set(engine.EXPORTED)


def test_device_wait_selftest_validates_its_limit():
    # argument checks happen on the host, before any device work
    L = engine.load_library()
    L.jc_selftest_device_wait.argtypes = [C.c_int32, C.c_uint32]
    assert engine.STATUS[L.jc_selftest_device_wait(0, 0)] == "BAD_ARGUMENT"
    assert engine.STATUS[L.jc_selftest_device_wait(0, 3_000_000)] == "BAD_ARGUMENT"


def _create(st: bytes, cj: str):
    L = engine.load_library()
    h = C.c_void_p()
    status = L.jc_model_create(st, len(st), cj.encode(), 0, C.byref(h))
    return status, L.jc_last_error().decode()


def test_truncated_safetensors_is_a_bad_checkpoint(pt_tiny):
    status, msg = _create(pt_tiny["st_bytes"][:100], pt_tiny["config"])
    assert engine.STATUS[status] == "BAD_CHECKPOINT", msg
    status, msg = _create(b"\x01\x02", pt_tiny["config"])
    assert engine.STATUS[status] == "BAD_CHECKPOINT"


def test_non_f32_tensor_is_rejected(pt_tiny):
    st = pt_tiny["st_bytes"]
    (hlen,) = np.frombuffer(st[:8], dtype="<u8")
    header = json.loads(st[8:8 + int(hlen)])
    header["pos"]["dtype"] = "F16"
    hb = json.dumps(header).encode()
    bad = np.uint64(len(hb)).tobytes() + hb + st[8 + int(hlen):]
    status, msg = _create(bad, pt_tiny["config"])
    assert engine.STATUS[status] == "BAD_CHECKPOINT" and "F32" in msg


def test_missing_tensor_is_named(pt_tiny):
    t = dict(pt_tiny["tensors"])
    del t["blocks.1.ff2.bias"]
    status, msg = _create(write_safetensors_bytes(t), pt_tiny["config"])
    assert engine.STATUS[status] == "BAD_CHECKPOINT" and "blocks.1.ff2.bias" in msg


def test_grid_not_divisible_by_patch_is_a_bad_shape(pt_tiny):
    c = json.loads(pt_tiny["config"])
    c["nx"] = 18
    status, msg = _create(pt_tiny["st_bytes"], json.dumps(c))
    assert engine.STATUS[status] == "BAD_SHAPE", msg


def test_missing_config_field_and_bad_json(pt_tiny):
    c = json.loads(pt_tiny["config"])
    del c["dt"]
    status, msg = _create(pt_tiny["st_bytes"], json.dumps(c))
    assert engine.STATUS[status] == "BAD_CHECKPOINT" and "dt" in msg
    status, _ = _create(pt_tiny["st_bytes"], "{not json")
    assert engine.STATUS[status] == "BAD_CHECKPOINT"


def test_pos_shape_must_match_the_grid(pt_tiny):
    c = json.loads(pt_tiny["config"])
    c["nx"] = c["ny"] = 32
    status, msg = _create(pt_tiny["st_bytes"], json.dumps(c))
    assert engine.STATUS[status] == "BAD_SHAPE" and "pos" in msg


def test_null_out_pointer_is_a_bad_argument(pt_tiny):
    L = engine.load_library()
    st = pt_tiny["st_bytes"]
    assert engine.STATUS[L.jc_model_create(st, len(st), pt_tiny["config"].encode(), 0, None)] == "BAD_ARGUMENT"
    h = C.c_void_p()
    assert engine.STATUS[L.jc_model_create(st, len(st), pt_tiny["config"].encode(), 7, C.byref(h))] == "BAD_ARGUMENT"


def test_host_projections_match_the_oracle():
    rng = np.random.default_rng(3)
    n = 300
    cfg = identity_config(n, r_max=1.0)
    cfg.norm_mean = (0.1, -0.05, 0.02)
    cfg.norm_std = (0.3, 0.2, 0.2)
    cfg.norm_depth = 1.0
    orc = projection_only(cfg)
    x = (0.5 * rng.standard_normal(3 * n)).astype(np.float32)
    jcfg = engine.JcConfig()
    jcfg.norm_mean[:] = cfg.norm_mean
    jcfg.norm_std[:] = cfg.norm_std
    jcfg.norm_depth, jcfg.g, jcfg.energy_r_max = 1.0, 9.81, 1.0
    assert engine.mass(x, n) == pytest.approx(orc.mass_sum64(x), rel=0, abs=1e-15)
    assert engine.energy(x, jcfg, n) == pytest.approx(orc.energy_sum64(x), rel=1e-15)
    y = engine.project_mass(x, 0.25, n)
    assert np.array_equal(y, orc.project_mass(x, 0.25, sum64=True))
    e0 = orc.energy_sum64(x)
    y = engine.project_energy(x, 0.999 * e0, jcfg, n)
    assert np.array_equal(y, orc.project_energy(x, 0.999 * e0, sum64=True))
    assert engine.energy(y, jcfg, n) <= 0.999 * e0 * (1 + 1e-6)


def test_solver_and_scoring_arguments_are_checked_before_device_work():
    L = engine.load_library()
    engine._declare_eval(L)
    s = np.zeros(3 * 16, dtype=np.float32)
    bad = engine.JcSwParams(0, 16, 1.0, 0.1, 9.81, 1.0, 0.0)
    assert engine.STATUS[L.jc_sw_run(C.byref(bad), s, 1, 3)] == "BAD_SHAPE"
    bad = engine.JcSwParams(4, 4, 0.0, 0.1, 9.81, 1.0, 0.0)
    assert engine.STATUS[L.jc_sw_run(C.byref(bad), s, 1, 3)] == "BAD_ARGUMENT"
    ok = engine.JcSwParams(4, 4, 1.0, 0.1, 9.81, 1.0, 0.0)
    assert engine.STATUS[L.jc_sw_run(C.byref(ok), s, 1, -1)] == "BAD_ARGUMENT"
    assert engine.STATUS[L.jc_sw_run(C.byref(ok), s, 1, 0)] == "OK"  # nothing to do
    rows = (engine.JcEvalRow * 1)()
    cfg = engine.JcConfig()
    cfg.nx, cfg.ny = 4, 4
    cfg.norm_std[:] = [1.0, 1.0, 1.0]
    x = np.zeros(48, dtype=np.float32)
    c = np.array([1e9, 2.0], dtype=np.float32)
    assert engine.STATUS[L.jc_eval_score(C.byref(cfg), x, x, c, 1, rows)] == "BAD_ARGUMENT"
    assert engine.STATUS[L.jc_eval_score(C.byref(cfg), x, x, c, 0, rows)] == "OK"


def test_host_add_drop_matches_the_oracle():
    from oracle import oracle as O

    p = engine.JcSwParams(33, 21, 1.0, 0.0903, 9.81, 1.0, 1e-3)
    a = engine.sw_flat(p)[0]
    engine.sw_add_drop(p, a[0], 12.7, 9.1, 0.06, 4.2)
    q = O._SwParams()
    q.nx, q.ny, q.dx, q.dt, q.g, q.depth, q.nu = 33, 21, 1.0, 0.0903, 9.81, 1.0, 1e-3
    b = O.sw_flat(q)[0]
    O.sw_add_drop(q, b[0], 12.7, 9.1, 0.06, 4.2)
    np.testing.assert_array_equal(a, b)


def test_eval_drop_sampler_keeps_waves_off_the_walls():
    from jacobi2000_gb300.evaluate import cells_per_tick, draw_drops, horizon_ticks

    cfg = engine.JcConfig()
    cfg.nx, cfg.ny, cfg.dx, cfg.dt, cfg.g, cfg.depth = 128, 96, 1.0, 0.0903, 9.81, 1.0
    drops, skipped = draw_drops(cfg, 20, 0, 50.0)
    assert len(drops) == 20 and skipped > 0
    for cx, cy, amp, sigma in drops:
        assert 8.0 <= cx < 120.0 and 8.0 <= cy < 88.0 and 0.03 <= amp < 0.07 and 3.0 <= sigma < 5.5
        assert horizon_ticks(cfg, cx, cy) >= 50.0
    assert abs(float(cells_per_tick(cfg)) - np.sqrt(9.81) * 0.0903) < 1e-6
    assert draw_drops(cfg, 20, 0, 50.0) == (drops, skipped)


def test_packed_checkpoint_header_is_checked_before_device_work(pt_tiny):
    L = engine.load_library()
    engine._declare_pack(L)
    h = C.c_void_p()
    for bad in (b"", b"JCPACK01", b"NOTAPACK" + bytes(64), b"JCPACK01" + (1).to_bytes(4, "little") + bytes(64)):
        assert engine.STATUS[L.jc_model_create_packed(bad, len(bad), C.byref(h))] == "BAD_CHECKPOINT"
    st, cj = pt_tiny["st_bytes"], pt_tiny["config"]
    a = engine.source_hash(st, cj)
    assert a == engine.source_hash(st, cj)
    assert a != engine.source_hash(st[:-1] + bytes([st[-1] ^ 1]), cj)
    assert a != engine.source_hash(st, cj + " ")
