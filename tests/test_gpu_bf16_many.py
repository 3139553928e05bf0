"""A BF16 batch of many instances (more than one 32-way round of the kernels'
warp-wide instance search): every instance's result equals its own rollout
bit for bit, whatever its place in the pack."""

import numpy as np
import pytest

from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import meta_of, parse_config, synthetic_family, write_safetensors_bytes
from jacobi2000_gb300.ic import random_drops

pytestmark = pytest.mark.gpu

SIDES = [32, 36, 48, 64]
N_INST = 70


def test_seventy_instances_equal_single_rollouts():
    fam = synthetic_family(128, 4, 0, SIDES)
    models, cfgs = [], []
    for s in SIDES:
        t, cj = fam[(s, s)]
        models.append(engine.Model.from_bytes(write_safetensors_bytes(t), cj, engine.BF16))
        cfgs.append(parse_config(cj, t))
    me = engine.PROJECT_MASS | engine.PROJECT_ENERGY
    rng = np.random.default_rng(5)
    items = []
    for k in range(N_INST):
        mi = int(rng.integers(0, len(SIDES)))
        ticks = int(rng.integers(1, 4))
        items.append((mi, random_drops(cfgs[mi], seed=500 + k), meta_of(cfgs[mi]), ticks, me))
    try:
        cells = sum(cfgs[mi].nx * cfgs[mi].ny for mi, *_ in items)
        with engine.Batch(models, max_instances=N_INST, max_cells=cells) as b:
            res = b.rollout(items)
        for k, ((mi, x0, meta, ticks, flags), (final, e, _)) in enumerate(zip(items, res)):
            alone, energies = models[mi].rollout(x0, meta, ticks, flags)
            assert np.array_equal(final, alone), (k, mi, ticks)
            assert e == energies[-1]
    finally:
        for m in models:
            m.close()
