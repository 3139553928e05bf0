"""BF16 tensor-core path against the f64 oracle (the precision form's
tolerance reference): per-field normwise error <= 1e-2 per forward and along
rollouts, relative energy violation <= 1e-6, and batch results identical to
single-instance results."""

import numpy as np
import pytest

from helpers import field_errors
from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import (parse_config, synthetic_checkpoint, synthetic_family,
                                         write_safetensors_bytes, meta_of)
from jacobi2000_gb300.ic import random_drops, single_drop
from oracle.oracle import ENERGY, MASS, OracleModel

pytestmark = pytest.mark.gpu

TOL = 1e-2
ME = engine.PROJECT_MASS | engine.PROJECT_ENERGY


def _pair(side, dim=128, layers=4, seed=0):
    t, cj = synthetic_checkpoint(side, dim, layers, seed)
    cfg = parse_config(cj, t)
    return engine.Model.from_bytes(write_safetensors_bytes(t), cj, engine.BF16), OracleModel(cfg, t), cfg


@pytest.mark.parametrize("side", [32, 96, 128])
def test_bf16_forward_against_f64_oracle(side):
    m, orc, cfg = _pair(side)
    with m:
        x = random_drops(cfg, seed=side)
        meta = meta_of(cfg)
        got = m.forward(x, meta)
    want = orc.forward(x.astype(np.float64), meta.astype(np.float64), f64=True)
    errs = field_errors(got, want)
    assert max(errs) <= TOL, errs


def test_bf16_forward_pt_tiny(pt_tiny):
    from jacobi2000_gb300.checkpoint import parse_config as pc
    with engine.Model.from_bytes(pt_tiny["st_bytes"], pt_tiny["config"], engine.BF16) as m:
        got = m.forward(pt_tiny["ref"]["state"], pt_tiny["ref"]["meta"])
    want = pt_tiny["ref"]["forward_stencil"]
    assert max(field_errors(got, want)) <= 3e-2


def test_bf16_rollout_against_f64_oracle():
    m, orc, cfg = _pair(64)
    with m:
        x0 = random_drops(cfg, seed=3)
        meta = meta_of(cfg)
        final, energies, traj = m.rollout(x0, meta, 10, ME, trajectory=True)
    want, e_want, viol_want, wtraj = orc.rollout(x0.astype(np.float64), meta.astype(np.float64), 10, MASS | ENERGY,
                                                 f64=True, trajectory=True)
    for t in (1, 5, 10):
        assert max(field_errors(traj[t], wtraj[t])) <= TOL, t
    viol = np.max(np.maximum((energies[1:] - energies[:-1] * cfg.energy_r_max) / energies[:-1], 0))
    assert viol <= 1e-6
    assert abs(energies[-1] - e_want[-1]) / e_want[-1] < 1e-4


def test_bf16_wide_model_forward():
    m, orc, cfg = _pair(64, dim=256, layers=6, seed=1)
    with m:
        x = random_drops(cfg, seed=9)
        meta = meta_of(cfg)
        got = m.forward(x, meta)
    want = orc.forward(x.astype(np.float64), meta.astype(np.float64), f64=True)
    assert max(field_errors(got, want)) <= TOL


def test_bf16_batch_equals_single():
    sides = [32, 64, 96]
    fam = synthetic_family(128, 4, 0, sides)
    models, cfgs = [], []
    for s in sides:
        t, cj = fam[(s, s)]
        models.append(engine.Model.from_bytes(write_safetensors_bytes(t), cj, engine.BF16))
        cfgs.append(parse_config(cj, t))
    spec = [(0, 4, ME), (1, 2, ME), (2, 3, 0), (0, 1, ME), (2, 5, ME)]
    items = [(mi, random_drops(cfgs[mi], seed=50 + k), meta_of(cfgs[mi]), ticks, fl)
             for k, (mi, ticks, fl) in enumerate(spec)]
    with engine.Batch(models, max_instances=8, max_cells=100_000) as b:
        res = b.rollout(items)
        res2 = b.rollout(items)
    for (mi, x0, meta, ticks, fl), (final, e, v), (final2, _, _) in zip(items, res, res2):
        alone, _ = models[mi].rollout(x0, meta, ticks, fl)
        assert np.array_equal(final, alone)
        assert np.array_equal(final2, alone)
    for m in models:
        m.close()


@pytest.mark.parametrize("dim,layers,seed", [(128, 4, 0), (256, 6, 1)])
def test_bf16_and_fp32_forward_256x256_against_f64_oracle(dim, layers, seed):
    """The 256x256 checkpoints (dim 128 / 4 layers and dim 256 / 6 layers):
    one forward of each path against the f64 oracle (BF16 <= 1e-2, FP32 <=
    1e-4 per field)."""
    import os

    from oracle import oracle as orc_mod

    orc_mod.set_threads(os.cpu_count() or 1)
    orc_mod.set_attention_mode("gather")
    t, cj = synthetic_checkpoint(256, dim, layers, seed)
    cfg = parse_config(cj, t)
    x = random_drops(cfg, seed=11)
    meta = meta_of(cfg)
    want = OracleModel(cfg, t).forward(x.astype(np.float64), meta.astype(np.float64), f64=True)
    for prec, tol in ((engine.BF16, TOL), (engine.FP32, 1e-4)):
        with engine.Model.from_bytes(write_safetensors_bytes(t), cj, prec) as m:
            got = m.forward(x, meta)
        assert max(field_errors(got, want)) <= tol, (prec, field_errors(got, want))
