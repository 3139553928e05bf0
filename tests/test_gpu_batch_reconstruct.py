"""Reconstruct instances in the batch runner: the Jacobi sweeps run inside one
CUDA-graph conditional while loop that ends on the device; rollouts in the
same call are unaffected; results agree with the server's reconstruct and
with the rule restated on the oracle."""

import numpy as np
import pytest

from helpers import field_errors
from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import parse_config, synthetic_family, write_safetensors_bytes, meta_of
from jacobi2000_gb300.ic import random_drops
from oracle.oracle import OracleModel
from test_gpu_server import _reconstruct_oracle

pytestmark = pytest.mark.gpu

SIDES = [32, 64]


@pytest.fixture(scope="module")
def fam():
    models, oracles, cfgs = [], [], []
    for seed in (0, 1):  # forward family, reverse family
        f = synthetic_family(128, 4, seed, SIDES)
        for s in SIDES:
            t, cj = f[(s, s)]
            models.append(engine.Model.from_bytes(write_safetensors_bytes(t), cj, engine.FP32))
            cfg = parse_config(cj, t)
            oracles.append(OracleModel(cfg, t))
            cfgs.append(cfg)
    yield models, oracles, cfgs  # index: seed * 2 + side index
    for m in models:
        m.close()


def _recon_item(cfg, g, rg, H, seed, sweeps, tol):
    rng = np.random.default_rng(seed)
    known = rng.random((H + 1, cfg.ny, cfg.nx)) < 0.05
    known[0] = True
    vals = np.stack([random_drops(cfg, seed=seed * 10 + t) for t in range(H + 1)]).astype(np.float32)
    vals = np.where(known[:, None], vals, 0).astype(np.float32)
    return {"task": 2, "model": g, "reverse_model": rg, "x": vals, "known": known.astype(np.uint8),
            "meta": meta_of(cfg), "ticks": H, "max_sweeps": sweeps, "tol": tol}


def test_batch_reconstruct_with_rollouts(fam):
    models, oracles, cfgs = fam
    rec = [_recon_item(cfgs[0], 0, 2, 3, 1, 3, 0.0), _recon_item(cfgs[1], 1, 3, 2, 2, 2, 0.0)]
    rolls = [(0, random_drops(cfgs[0], seed=9), meta_of(cfgs[0]), 4, 3),
             (3, random_drops(cfgs[3], seed=8), meta_of(cfgs[3]), 2, 3)]  # a rewind on the reverse 64 grid
    with engine.Batch(models, max_instances=64, max_cells=400_000) as b:
        res = b.rollout(rolls + rec)
        res2 = b.rollout(rolls + rec)  # the cached graph, replayed
    for (mi, x0, meta, ticks, fl), (final, e, v) in zip(rolls, res[:2]):
        alone, _ = models[mi].rollout(x0, meta, ticks, fl)
        assert np.array_equal(final, alone)
    for it, (vol, sweeps, resid), (vol2, sweeps2, _) in zip(rec, res[2:], res2[2:]):
        assert sweeps == it["max_sweeps"] and sweeps2 == sweeps
        assert np.array_equal(vol, vol2)
        g, rg, H = it["model"], it["reverse_model"], it["ticks"]
        want = _reconstruct_oracle(oracles[g], oracles[rg], it["x"], it["known"].astype(bool), it["meta"], H,
                                   it["max_sweeps"])
        for t in range(H + 1):
            assert max(field_errors(vol[t], want[t])) <= 1e-4
    # the same reconstruct through the serving loop gives the same bits
    it = rec[0]
    with engine.Server([models[0], models[1]], [models[2], models[3]], max_active_cells=1 << 18) as srv:
        rid = srv.submit(engine.TASK_RECONSTRUCT, 0, it["x"], it["meta"], it["ticks"], known=it["known"],
                         max_sweeps=it["max_sweeps"], tol=0.0)
        served, _ = srv.wait(rid, engine.TASK_RECONSTRUCT, 0, it["ticks"], timeout=60)
    assert np.array_equal(served, res[2][0])


def test_device_side_loop_stops_on_convergence(fam):
    models, oracles, cfgs = fam
    loose = _recon_item(cfgs[0], 0, 2, 2, 3, 50, 1e9)   # converged after its first sweep
    tight = _recon_item(cfgs[0], 0, 2, 2, 4, 3, 0.0)    # runs its 3 sweeps
    with engine.Batch(models, max_instances=32, max_cells=200_000) as b:
        (v1, s1, r1), (v2, s2, r2) = b.rollout([loose, tight])
    assert s1 == 1 and s2 == 3
    with engine.Batch(models, max_instances=32, max_cells=200_000) as b:
        (v2b, s2b, _), = b.rollout([tight])
    assert np.array_equal(v2, v2b) and s2b == 3  # the same alone and in the mix
