"""BF16 schedule autotuning: every schedule gives bit-identical results (the
candidates change tiling and CTA size, never the order of a sum, so a result
does not depend on the batch it runs in), the tuned choice persists through
the JC_AUTOTUNE_CACHE file, and a schedule read from that file is the one the
launches use."""

import json

import numpy as np
import pytest

from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import parse_config, synthetic_family, write_safetensors_bytes, meta_of
from jacobi2000_gb300.ic import random_drops

pytestmark = pytest.mark.gpu

ME = engine.PROJECT_MASS | engine.PROJECT_ENERGY
SIDES = [64, 128]


def _family(dim=128, layers=2):
    fam = synthetic_family(dim, layers, 3, SIDES)
    out = []
    for s in SIDES:
        t, cj = fam[(s, s)]
        out.append((write_safetensors_bytes(t), cj, parse_config(cj, t)))
    return out


def _key(c):
    return f"d{c.dim}_l{c.layers}_f{c.ff_inner}_r{c.radius}_k{c.mask_kind}_g{c.dilation}"


def _run(fam, items_spec):
    models = [engine.Model.from_bytes(st, cj, engine.BF16) for st, cj, _ in fam]
    try:
        items = [(mi, random_drops(fam[mi][2], seed=70 + k), meta_of(fam[mi][2]), ticks, ME)
                 for k, (mi, ticks) in enumerate(items_spec)]
        with engine.Batch(models, max_instances=16, max_cells=200_000) as b:
            res = b.rollout(items)
        x1 = next(it for it in items if it[0] == 1)
        single = models[1].forward(x1[1], x1[2])
        return [r[0] for r in res], single
    finally:
        for m in models:
            m.close()


@pytest.mark.parametrize("dim", [32, 128])
def test_every_schedule_gives_identical_results(tmp_path, monkeypatch, dim):
    fam = _family(dim)
    spec = [(0, 3), (1, 2), (1, 3), (0, 1)]
    prev = engine.autotune(False)
    try:
        base, base1 = _run(fam, spec)
        cache = tmp_path / "tune.txt"
        monkeypatch.setenv("JC_AUTOTUNE_CACHE", str(cache))
        engine.autotune(True)
        scheds = [(32, 256), (64, 256), (64, 64), (64, 128), (64, 0)]
        for nc, threads in scheds:
            # a cache file written beforehand fixes the schedule of every row bucket
            key = _key(fam[0][2])
            cache.write_text("".join(json.dumps({"model": key, "rows": 1 << b, "nc": nc, "attn_threads": threads})
                                     + "\n" for b in range(7, 25)))
            got, got1 = _run(fam, spec)
            for a, g in zip(base, got):
                assert np.array_equal(a, g), (nc, threads)
            assert np.array_equal(base1, got1), (nc, threads)
    finally:
        engine.autotune(prev)


def test_tuning_is_recorded_and_reused(tmp_path, monkeypatch):
    fam = _family()
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("JC_AUTOTUNE_CACHE", str(cache))
    prev = engine.autotune(True)
    try:
        first, _ = _run(fam, [(1, 2), (1, 2), (0, 2)])
        rows = [json.loads(ln) for ln in cache.read_text().splitlines()]
        assert len(rows) >= 2  # the batch's row bucket and the single forward's
        assert all(r["model"] == _key(fam[0][2]) for r in rows)
        assert all(r["nc"] in (32, 64) and r["attn_threads"] in (0, 64, 128, 256) for r in rows)
        size = cache.stat().st_size
        again, _ = _run(fam, [(1, 2), (1, 2), (0, 2)])
        assert cache.stat().st_size == size  # read back, not tuned again
        for a, b in zip(first, again):
            assert np.array_equal(a, b)
    finally:
        engine.autotune(prev)


def test_autotune_switch():
    prev = engine.autotune(False)
    assert engine.autotune(None) is False
    engine.autotune(True)
    assert engine.autotune(None) is True
    engine.autotune(prev)
