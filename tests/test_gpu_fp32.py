"""FP32 CUDA path against the oracle and the reference's golden vectors.

Gates: the reference's own GPU gates (crates/engine/tests/parity.rs:93,101,
128,136: 1e-4 forward, 1e-3 rollout, max abs) are the floor; the FP32 path is
held to the tighter CPU gates (1e-5 forward, 1e-4 rollout) and, at the
128x128 size, to a per-forward normwise relative error <= 1e-4 per field and an
energy violation <= 1e-6."""

import json

import numpy as np
import pytest

from helpers import field_errors, r2d2_config
from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import (parse_config, synthetic_checkpoint, synthetic_family,
                                         write_safetensors_bytes, meta_of)
from jacobi2000_gb300.ic import random_drops
from oracle.oracle import ENERGY, MASS, SUM64, OracleModel

pytestmark = pytest.mark.gpu

MASS_ENERGY = engine.PROJECT_MASS | engine.PROJECT_ENERGY


def _pair(tensors, cj, precision=engine.FP32):
    return (engine.Model.from_bytes(write_safetensors_bytes(tensors), cj, precision),
            OracleModel(parse_config(cj, tensors), tensors))


def test_pt_tiny_forward_stencil(pt_tiny):
    with engine.Model.from_bytes(pt_tiny["st_bytes"], pt_tiny["config"]) as m:
        out = m.forward(pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"])
    assert np.abs(out - pt_tiny["ref"]["forward_stencil"]).max() < 1e-5


def test_pt_tiny_forward_full(pt_tiny):
    with engine.Model.from_bytes(pt_tiny["st_bytes"], pt_tiny["config_full"]) as m:
        out = m.forward(pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"])
    assert np.abs(out - pt_tiny["ref"]["forward_full"]).max() < 1e-5


def test_pt_tiny_r2d2_edge_clip(pt_tiny, extra):
    with engine.Model.from_bytes(pt_tiny["st_bytes"], r2d2_config(pt_tiny["config"])) as m:
        out = m.forward(pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"])
    assert np.abs(out - extra["r2d2_forward"]).max() < 1e-5


def test_pt_tiny_fifty_step_rollout(pt_tiny):
    r = pt_tiny["ref"]
    with engine.Model.from_bytes(pt_tiny["st_bytes"], pt_tiny["config"]) as m:
        x = r["state"]
        for i in range(1, 51):
            x = m.step(x, r["meta"])
            if i in (1, 10, 50):
                assert np.abs(x - r[f"rollout_{i}"]).max() < 1e-4
        final, energies, traj = m.rollout(r["state"], r["meta"], 50, 0, trajectory=True)
    for i in (1, 10, 50):
        assert np.abs(traj[i] - r[f"rollout_{i}"]).max() < 1e-4
    assert np.array_equal(traj[50], final)
    assert np.array_equal(traj[0], r["state"])


def test_non_square_grid(extra):
    t, cj = synthetic_family(32, 2, 5, [], rect=[(24, 16)])[(24, 16)]
    with engine.Model.from_bytes(write_safetensors_bytes(t), cj) as m:
        out = m.forward(extra["rect_state"], extra["rect_meta"])
    assert np.abs(out - extra["rect_forward_f32"]).max() < 1e-5


def test_model20_shape_forward_and_projected_rollout(extra):
    t, cj = synthetic_checkpoint(32, 128, 4, 0)
    m, orc = _pair(t, cj)
    with m:
        s, meta = extra["c1_state"], extra["c1_meta"]
        assert np.abs(m.forward(s, meta) - extra["c1_forward_f32"]).max() < 1e-5
        final, energies = m.rollout(s, meta, 10, MASS_ENERGY)
    want, e_want, viol = orc.rollout(s, meta, 10, MASS | ENERGY | SUM64)
    assert np.abs(final - want).max() < 1e-4
    assert np.abs(final - extra["c1_rollout10_projected"]).max() < 1e-4
    assert np.allclose(energies, e_want, rtol=1e-7, atol=0)


def test_energy_projection_engages_and_holds_the_bound(pt_tiny):
    # pt-tiny has energy_r_max 0.999: the bound shrinks every tick, so the
    # projection must scale (u, v) down
    r = pt_tiny["ref"]
    t = pt_tiny["tensors"]
    m, orc = _pair(t, pt_tiny["config"])
    with m:
        final, energies = m.rollout(r["state"], r["meta"], 20, MASS_ENERGY)
    want, e_want, viol_want = orc.rollout(r["state"], r["meta"], 20, MASS | ENERGY | SUM64)
    assert np.abs(final - want).max() < 1e-4
    assert np.allclose(energies, e_want, rtol=1e-6)
    # scaling (u, v) cannot remove potential energy: where the potential alone
    # exceeds the bound the reference's projection leaves a violation, and the
    # GPU must leave the same one
    viol = np.max(np.maximum((energies[1:] - energies[:-1] * 0.999) / energies[:-1], 0))
    assert abs(viol - viol_want) <= 1e-6
    free, _, _ = orc.rollout(r["state"], r["meta"], 20, MASS | SUM64)
    assert np.abs(final[1:] - free[1:]).max() > 1e-3  # the projection changed u, v


@pytest.fixture(scope="module")
def c2_model():
    t, cj = synthetic_checkpoint(128, 128, 4, 0)
    m, orc = _pair(t, cj)
    yield m, orc
    m.close()


def test_128_grid_per_forward_error(c2_model):
    """Config C2: 128x128, 8 drops; teacher-forced per-forward error <= 1e-4
    normwise per field against the f32 oracle, at the initial state and at
    states 10 and 25 ticks along the GPU rollout."""
    m, orc = c2_model
    cfg = orc.cfg
    x0 = random_drops(cfg, seed=0)
    meta = meta_of(cfg)
    _, _, traj = m.rollout(x0, meta, 25, MASS_ENERGY, trajectory=True)
    for t in (0, 10, 25):
        got = m.forward(traj[t], meta)
        want = orc.forward(traj[t], meta)
        errs = field_errors(got, want)
        assert max(errs) <= 1e-4, (t, errs)


def test_128_grid_fifty_tick_rollout_energy(c2_model):
    m, orc = c2_model
    cfg = orc.cfg
    x0 = random_drops(cfg, seed=1)
    meta = meta_of(cfg)
    final, energies = m.rollout(x0, meta, 50, MASS_ENERGY)
    viol = np.max(np.maximum((energies[1:] - energies[:-1] * cfg.energy_r_max) / energies[:-1], 0))
    assert viol <= 1e-6
    assert np.all(np.isfinite(final))
    # mass is held to the initial box mean of channel 0
    assert abs(final[0].astype(np.float64).mean() - x0[0].astype(np.float64).mean()) < 1e-4


def test_rollout_is_deterministic(c2_model):
    m, orc = c2_model
    x0 = random_drops(orc.cfg, seed=2)
    meta = meta_of(orc.cfg)
    a, ea = m.rollout(x0, meta, 5, MASS_ENERGY)
    b, eb = m.rollout(x0, meta, 5, MASS_ENERGY)
    assert np.array_equal(a, b) and np.array_equal(ea, eb)
