"""Batched rollouts: many instances of different grids and horizons in one
graph-captured launch sequence. Each instance's result must be the same
alone and in the mix, and match the oracle."""

import numpy as np
import pytest

from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import (parse_config, synthetic_family, write_safetensors_bytes, meta_of)
from jacobi2000_gb300.ic import random_drops
from oracle.oracle import ENERGY, MASS, SUM64, OracleModel

pytestmark = pytest.mark.gpu

SIDES = [32, 64, 96]


@pytest.fixture(scope="module")
def family():
    fam = synthetic_family(128, 4, 0, SIDES)
    models, oracles, cfgs = [], [], []
    for s in SIDES:
        t, cj = fam[(s, s)]
        models.append(engine.Model.from_bytes(write_safetensors_bytes(t), cj))
        cfg = parse_config(cj, t)
        oracles.append(OracleModel(cfg, t))
        cfgs.append(cfg)
    yield models, oracles, cfgs
    for m in models:
        m.close()


def _items(cfgs, spec):
    items = []
    for k, (mi, ticks, flags) in enumerate(spec):
        cfg = cfgs[mi]
        items.append((mi, random_drops(cfg, seed=100 + k), meta_of(cfg), ticks, flags))
    return items


def test_batch_equals_single_instance_rollouts(family):
    models, oracles, cfgs = family
    me = engine.PROJECT_MASS | engine.PROJECT_ENERGY
    spec = [(0, 7, me), (1, 3, me), (2, 5, 0), (0, 0, me), (1, 9, engine.PROJECT_MASS), (2, 1, me)]
    items = _items(cfgs, spec)
    with engine.Batch(models, max_instances=16, max_cells=200_000) as b:
        res = b.rollout(items)
        res2 = b.rollout(items)  # graph replay
    for (mi, x0, meta, ticks, flags), (final, e, viol), (final2, _, _) in zip(items, res, res2):
        alone, energies = models[mi].rollout(x0, meta, ticks, flags)
        assert np.array_equal(final, alone), (mi, ticks)
        assert np.array_equal(final2, alone)
        assert e == energies[-1]


def test_batch_matches_oracle(family):
    models, oracles, cfgs = family
    me = engine.PROJECT_MASS | engine.PROJECT_ENERGY
    spec = [(0, 4, me), (1, 2, me)]
    items = _items(cfgs, spec)
    with engine.Batch(models, max_instances=4, max_cells=50_000) as b:
        res = b.rollout(items)
    for (mi, x0, meta, ticks, flags), (final, e, viol) in zip(items, res):
        want, ew, _ = oracles[mi].rollout(x0, meta, ticks, MASS | ENERGY | SUM64)
        assert np.abs(final - want).max() / np.abs(want).max() < 1e-5
        assert abs(e - ew[-1]) / ew[-1] < 1e-7


def test_batch_capacity_is_enforced(family):
    models, oracles, cfgs = family
    items = _items(cfgs, [(2, 1, 0)] * 3)
    with engine.Batch(models, max_instances=2, max_cells=1_000_000) as b:
        with pytest.raises(engine.JcError) as e:
            b.rollout(items)
        assert e.value.name == "OVER_BUDGET"
    with engine.Batch(models, max_instances=8, max_cells=96 * 96) as b:
        with pytest.raises(engine.JcError) as e:
            b.rollout(items)
        assert e.value.name == "OVER_BUDGET"


def test_profile_reports_every_kernel(family):
    models, oracles, cfgs = family
    items = _items(cfgs, [(0, 2, 3), (1, 2, 3)])
    with engine.Batch(models, max_instances=4, max_cells=50_000) as b:
        prof = b.profile(items)
    assert prof["f32_ln_qkv"][0] == 2 * 4
    assert prof["projection"][0] == 1 + 2
    assert all(ms > 0 for _, ms in prof.values())
