"""The oracle against the reference's golden vectors and unit cases.

Gates are the reference's own: crates/engine/tests/parity.rs:43,53 (forward,
1e-5 max abs) and :67 (rollout, 1e-4 max abs)."""

import json

import numpy as np
import pytest

from helpers import r2d2_config
from jacobi2000_gb300.checkpoint import checksum, parse_config, synthetic_checkpoint, synthetic_family
from oracle.oracle import (ENERGY, MASS, SUM64, OracleModel, identity_config, projection_only,
                           set_attention_mode)


def _model(tensors, config_json):
    return OracleModel(parse_config(config_json, tensors), tensors)


@pytest.mark.parametrize("mode", ["scan", "gather"])
def test_forward_stencil_matches_pt_tiny(pt_tiny, mode):
    set_attention_mode(mode)
    try:
        m = _model(pt_tiny["tensors"], pt_tiny["config"])
        out = m.forward(pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"])
    finally:
        set_attention_mode("gather")
    assert np.abs(out - pt_tiny["ref"]["forward_stencil"]).max() < 1e-5


def test_forward_full_matches_pt_tiny(pt_tiny):
    m = _model(pt_tiny["tensors"], pt_tiny["config_full"])
    out = m.forward(pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"])
    assert np.abs(out - pt_tiny["ref"]["forward_full"]).max() < 1e-5


def test_scan_and_gather_give_identical_bits(pt_tiny):
    m = _model(pt_tiny["tensors"], r2d2_config(pt_tiny["config"]))
    set_attention_mode("scan")
    a = m.forward(pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"])
    set_attention_mode("gather")
    b = m.forward(pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"])
    assert np.array_equal(a, b)


def test_fifty_step_rollout_matches_pt_tiny(pt_tiny):
    m = _model(pt_tiny["tensors"], pt_tiny["config"])
    meta = pt_tiny["ref"]["meta"]
    x = pt_tiny["ref"]["state"]
    for i in range(1, 51):
        x = m.step(x, meta)
        if i in (1, 10, 50):
            assert np.abs(x - pt_tiny["ref"][f"rollout_{i}"]).max() < 1e-4
    final, _, _ = m.rollout(pt_tiny["ref"]["state"], meta, 50, 0)
    assert np.array_equal(final, x)


def test_r2d2_edge_clip_matches_pytorch(pt_tiny, extra):
    m = _model(pt_tiny["tensors"], r2d2_config(pt_tiny["config"]))
    out = m.forward(pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"])
    assert np.abs(out - extra["r2d2_forward"]).max() < 1e-5


def test_synthetic_checkpoints_are_reproducible(extra):
    t, _ = synthetic_family(32, 2, 5, [], rect=[(24, 16)])[(24, 16)]
    assert np.array_equal(checksum(t), extra["rect_checksum"])
    t, _ = synthetic_checkpoint(32, 128, 4, 0)
    assert np.array_equal(checksum(t), extra["c1_checksum"])


def test_non_square_grid_f32_and_f64(extra):
    t, cj = synthetic_family(32, 2, 5, [], rect=[(24, 16)])[(24, 16)]
    m = _model(t, cj)
    assert np.abs(m.forward(extra["rect_state"], extra["rect_meta"]) - extra["rect_forward_f32"]).max() < 1e-5
    o64 = m.forward(extra["rect_state"].astype(np.float64), extra["rect_meta"].astype(np.float64), f64=True)
    assert np.abs(o64 - extra["rect_forward_f64"]).max() < 1e-12


def test_model20_shape_forward_and_rollouts(extra):
    t, cj = synthetic_checkpoint(32, 128, 4, 0)
    m = _model(t, cj)
    s, meta = extra["c1_state"], extra["c1_meta"]
    assert np.abs(m.forward(s, meta) - extra["c1_forward_f32"]).max() < 1e-5
    o64 = m.forward(s.astype(np.float64), meta.astype(np.float64), f64=True)
    assert np.abs(o64 - extra["c1_forward_f64"]).max() < 1e-12
    fin, _, _ = m.rollout(s, meta, 10, 0)
    assert np.abs(fin - extra["c1_rollout10_plain"]).max() < 1e-4
    fin, energies, viol = m.rollout(s, meta, 10, MASS | ENERGY | SUM64)
    assert np.abs(fin - extra["c1_rollout10_projected"]).max() < 1e-4
    assert viol <= 1e-6


# crates/engine/src/project.rs:64-102, restated.

def test_mass_projection_restores_target_and_leaves_uv_alone():
    p = projection_only(identity_config(4))
    x = np.array([0.1, 0.2, 0.3, 0.4, 5, 5, 5, 5, -1, -1, -1, -1], dtype=np.float32)
    for sum64 in (False, True):
        y = p.project_mass(x, 0.0, sum64=sum64)
        assert abs(p.mass(y)) < 1e-6
        assert np.array_equal(y[4:8], x[4:8])


def test_energy_projection_scales_down_to_the_bound():
    n = 16
    p = projection_only(identity_config(n, r_max=100.0))
    x = np.concatenate([np.ones(n), 2 * np.ones(n), 2 * np.ones(n)]).astype(np.float32)
    for sum64 in (False, True):
        y = p.project_energy(x, 1.0, sum64=sum64)
        e = p.energy(y)
        assert e <= 100.0 + 1e-3 and e > 99.0
        assert abs(p.mass(y) - 1.0) < 1e-6


def test_energy_projection_is_identity_within_the_bound():
    n = 16
    p = projection_only(identity_config(n, r_max=100.0))
    x = np.concatenate([np.ones(n), 2 * np.ones(n), 2 * np.ones(n)]).astype(np.float32)
    for sum64 in (False, True):
        assert np.array_equal(p.project_energy(x, 2.0, sum64=sum64), x)
