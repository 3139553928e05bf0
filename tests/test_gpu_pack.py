"""Pre-packed checkpoints (jc_model_pack / jc_model_create_packed): a model
loaded from its device weight image must give the same bits as the model
converted from model.safetensors, and the cache beside the checkpoint must be
used only while it records the current source."""

import time

import numpy as np
import pytest

from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import meta_of, parse_config, synthetic_checkpoint, write_safetensors_bytes
from jacobi2000_gb300.ic import random_drops

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [engine.FP32, engine.BF16])
@pytest.mark.parametrize("side,dim,layers", [(64, 128, 4), (32, 256, 6)])
def test_packed_model_gives_the_same_bits(prec, side, dim, layers):
    t, cj = synthetic_checkpoint(side, dim, layers, 3)
    cfg = parse_config(cj, t)
    x0 = random_drops(cfg, seed=5)
    meta = meta_of(cfg)
    with engine.Model.from_bytes(write_safetensors_bytes(t), cj, prec) as m:
        packed = m.pack()
        want_f = m.forward(x0, meta)
        want_r, want_e = m.rollout(x0, meta, 6)
    with engine.Model.from_packed(packed) as p:
        assert p.precision == prec
        assert (p.config.nx, p.config.dim, p.config.layers) == (side, dim, layers)
        np.testing.assert_array_equal(p.forward(x0, meta), want_f)
        got_r, got_e = p.rollout(x0, meta, 6)
        np.testing.assert_array_equal(got_r, want_r)
        np.testing.assert_array_equal(got_e, want_e)
        assert p.pack() == packed


def test_packed_models_share_batch_launches():
    fam = {}
    for s in (32, 64):
        t, cj = synthetic_checkpoint(s, 128, 4, 0)
        fam[s] = (t, cj)
    src = [engine.Model.from_bytes(write_safetensors_bytes(t), cj, engine.BF16) for t, cj in fam.values()]
    packed = [engine.Model.from_packed(m.pack()) for m in src]
    items = []
    for i, (t, cj) in enumerate(fam.values()):
        cfg = parse_config(cj, t)
        items.append((i, random_drops(cfg, seed=i), meta_of(cfg), 4, 3))
    with engine.Batch(src, 4, 8192) as a, engine.Batch(packed, 4, 8192) as b:
        ra, rb = a.rollout(items), b.rollout(items)
    for (fa, ea, va), (fb, eb, vb) in zip(ra, rb):
        np.testing.assert_array_equal(fa, fb)
        assert ea == eb
    for m in src + packed:
        m.close()


def test_cache_beside_the_checkpoint(tmp_path):
    t, cj = synthetic_checkpoint(64, 256, 6, 1)
    (tmp_path / "model.safetensors").write_bytes(write_safetensors_bytes(t))
    (tmp_path / "config.json").write_text(cj)
    cfg = parse_config(cj, t)
    x0, meta = random_drops(cfg, seed=2), meta_of(cfg)
    t0 = time.perf_counter()
    with engine.Model.load_cached(tmp_path, engine.BF16) as m:
        first = time.perf_counter() - t0
        want = m.forward(x0, meta)
    cache = tmp_path / "model.bf16.jcpack"
    assert cache.exists()
    stamp = cache.stat().st_mtime_ns
    t0 = time.perf_counter()
    with engine.Model.load_cached(tmp_path, engine.BF16) as m:
        second = time.perf_counter() - t0
        np.testing.assert_array_equal(m.forward(x0, meta), want)
    assert cache.stat().st_mtime_ns == stamp  # used, not rewritten
    assert second < first
    # a changed source invalidates the cache
    t2, cj2 = synthetic_checkpoint(64, 256, 6, 2)
    (tmp_path / "model.safetensors").write_bytes(write_safetensors_bytes(t2))
    with engine.Model.load_cached(tmp_path, engine.BF16) as m:
        with engine.Model.from_bytes(write_safetensors_bytes(t2), cj2, engine.BF16) as ref:
            np.testing.assert_array_equal(m.forward(x0, meta), ref.forward(x0, meta))
    assert cache.stat().st_mtime_ns != stamp


def test_corrupt_pack_is_a_bad_checkpoint():
    t, cj = synthetic_checkpoint(32, 128, 4, 0)
    with engine.Model.from_bytes(write_safetensors_bytes(t), cj) as m:
        packed = bytearray(m.pack())
    for cut in (len(packed) - 1, 100, 20):
        with pytest.raises(engine.JcError) as e:
            engine.Model.from_packed(bytes(packed[:cut]))
        assert e.value.name == "BAD_CHECKPOINT"
