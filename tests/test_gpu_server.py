"""The serving loop: continuous batching of forward, rewind and reconstruct
requests of several grid sizes. Results must not depend on what else runs in
the same launches, and must match the single-request paths and the oracle."""

import threading
import time

import numpy as np
import pytest

from helpers import field_errors
from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import parse_config, synthetic_family, write_safetensors_bytes, meta_of
from jacobi2000_gb300.ic import random_drops
from oracle.oracle import OracleModel

pytestmark = pytest.mark.gpu

SIDES = [32, 48, 64]
ME = engine.PROJECT_MASS | engine.PROJECT_ENERGY


def _family(seed, precision):
    fam = synthetic_family(128, 4, seed, SIDES)
    models, oracles, cfgs = [], [], []
    for s in SIDES:
        t, cj = fam[(s, s)]
        models.append(engine.Model.from_bytes(write_safetensors_bytes(t), cj, precision))
        cfg = parse_config(cj, t)
        oracles.append(OracleModel(cfg, t))
        cfgs.append(cfg)
    return models, oracles, cfgs


@pytest.fixture(scope="module", params=[engine.FP32, engine.BF16], ids=["fp32", "bf16"])
def families(request):
    fwd = _family(0, request.param)
    rev = _family(1, request.param)  # the reverse checkpoints: a second seeded family
    yield fwd, rev
    for m in fwd[0] + rev[0]:
        m.close()


def test_mixed_requests_match_single_runs(families):
    (fm, _, cfgs), (rm, _, _) = families
    rng = np.random.default_rng(7)
    reqs = []
    for k in range(12):
        task = engine.TASK_FORWARD if k % 2 == 0 else engine.TASK_REWIND
        g = int(rng.integers(0, len(SIDES)))
        ticks = int(rng.integers(2, 9))
        x = random_drops(cfgs[g], seed=200 + k)
        reqs.append((task, g, ticks, x, meta_of(cfgs[g])))
    with engine.Server(fm, rm, max_active_cells=6 * 64 * 64) as srv:
        ids = []
        for k, (task, g, ticks, x, meta) in enumerate(reqs):
            ids.append(srv.submit(task, g, x, meta, ticks, ME))
            if k % 3 == 2:
                time.sleep(0.002)  # later requests arrive while earlier ones run
        outs = [srv.wait(i, task, g, ticks, timeout=60) for i, (task, g, ticks, _, _) in zip(ids, reqs)]
        st = srv.stats()
    assert st["completed"] == len(reqs)
    for (task, g, ticks, x, meta), (out, info) in zip(reqs, outs):
        model = fm[g] if task == engine.TASK_FORWARD else rm[g]
        alone, energies = model.rollout(x, meta, ticks, ME)
        assert np.array_equal(out, alone), (task, g, ticks)
        assert info["energy"] == energies[-1]
        assert info["latency_s"] >= info["queue_s"] >= 0


def _reconstruct_oracle(fo, ro, vals, known, meta, H, sweeps):
    """The reconstruct rule restated with the f32 oracle's steps."""
    X = np.where(known[:, None], vals, 0.0).astype(np.float32)
    for _ in range(sweeps):
        F = [fo.step(X[t - 1], meta) for t in range(1, H + 1)]
        R = [ro.step(X[t + 1], meta) for t in range(0, H)]
        new = np.empty_like(X)
        for t in range(H + 1):
            if t == 0:
                v = R[0]
            elif t == H:
                v = F[H - 1]
            else:
                v = np.float32(0.5) * (F[t - 1] + R[t])
            new[t] = np.where(known[t][None], vals[t], v)
        X = new
    return X


def test_reconstruct_matches_oracle(families):
    (fm, fo, cfgs), (rm, ro, _) = families
    g, H, sweeps = 0, 3, 3
    cfg = cfgs[g]
    rng = np.random.default_rng(3)
    truth = np.stack([random_drops(cfg, seed=t) for t in range(H + 1)])
    known = rng.random((H + 1, cfg.ny, cfg.nx)) < 0.02
    known[0] = True  # a fully known first slice plus sparse readings
    vals = np.where(known[:, None], truth, 0).astype(np.float32)
    meta = meta_of(cfg)
    with engine.Server(fm, rm, max_active_cells=1 << 18) as srv:
        rid = srv.submit(engine.TASK_RECONSTRUCT, g, vals, meta, H, known=known, max_sweeps=sweeps, tol=0.0)
        out, info = srv.wait(rid, engine.TASK_RECONSTRUCT, g, H, timeout=60)
    assert info["sweeps"] == sweeps
    want = _reconstruct_oracle(fo[g], ro[g], vals, known, meta, H, sweeps)
    tol = 1e-4 if fm[g].precision == engine.FP32 else 2e-2
    for t in range(H + 1):
        assert max(field_errors(out[t], want[t])) <= tol, t
    assert np.array_equal(out[0], vals[0])  # the fully known first slice is kept


def test_reconstruct_in_the_mix_equals_alone(families):
    (fm, _, cfgs), (rm, _, _) = families
    g, H = 1, 2
    cfg = cfgs[g]
    rng = np.random.default_rng(5)
    known = rng.random((H + 1, cfg.ny, cfg.nx)) < 0.05
    vals = np.stack([random_drops(cfg, seed=40 + t) for t in range(H + 1)]).astype(np.float32)
    meta = meta_of(cfg)
    with engine.Server(fm, rm, max_active_cells=1 << 18) as srv:
        rid = srv.submit(engine.TASK_RECONSTRUCT, g, vals, meta, H, known=known, max_sweeps=2, tol=0.0)
        alone, _ = srv.wait(rid, engine.TASK_RECONSTRUCT, g, H, timeout=60)
        others = [srv.submit(engine.TASK_FORWARD, k % 3, random_drops(cfgs[k % 3], seed=k), meta_of(cfgs[k % 3]), 5)
                  for k in range(5)]
        rid = srv.submit(engine.TASK_RECONSTRUCT, g, vals, meta, H, known=known, max_sweeps=2, tol=0.0)
        mixed, _ = srv.wait(rid, engine.TASK_RECONSTRUCT, g, H, timeout=60)
        for i, k in zip(others, range(5)):
            srv.wait(i, engine.TASK_FORWARD, k % 3, 5, timeout=60)
    assert np.array_equal(alone, mixed)


def test_admission_limits(families):
    (fm, _, cfgs), (rm, _, _) = families
    cfg = cfgs[2]
    with engine.Server(fm, rm, max_active_cells=64 * 64) as srv:
        # one request per tick fits; a reconstruct of 2 x 4 instances does not
        with pytest.raises(engine.JcError) as e:
            srv.submit(engine.TASK_RECONSTRUCT, 2, np.zeros((5, 3, 64, 64), np.float32), meta_of(cfg), 4,
                       known=np.zeros((5, 64, 64), np.uint8))
        assert e.value.name == "OVER_BUDGET"
        # several requests queue behind the one that runs and all complete
        ids = [srv.submit(engine.TASK_FORWARD, 2, random_drops(cfg, seed=k), meta_of(cfg), 3) for k in range(4)]
        for i in ids:
            out, info = srv.wait(i, engine.TASK_FORWARD, 2, 3, timeout=60)
            assert np.all(np.isfinite(out))
        with pytest.raises(engine.JcError) as e:
            srv.wait(12345, engine.TASK_FORWARD, 2, 3, timeout=1)
        assert e.value.name == "NOT_FOUND"


def test_submissions_from_many_threads(families):
    (fm, _, cfgs), (rm, _, _) = families
    results = {}

    def client(k):
        g = k % 3
        x = random_drops(cfgs[g], seed=500 + k)
        with lock:
            pass
        rid = srv.submit(engine.TASK_FORWARD, g, x, meta_of(cfgs[g]), 4)
        results[k] = (g, x, srv.wait(rid, engine.TASK_FORWARD, g, 4, timeout=60)[0])

    lock = threading.Lock()
    with engine.Server(fm, rm, max_active_cells=1 << 18) as srv:
        th = [threading.Thread(target=client, args=(k,)) for k in range(8)]
        for t in th:
            t.start()
        for t in th:
            t.join()
    for k, (g, x, out) in results.items():
        alone, _ = fm[g].rollout(x, meta_of(cfgs[g]), 4, ME)
        assert np.array_equal(out, alone)


def test_device_buffer_requests_equal_host_requests(families):
    """Requests whose inputs and results are the caller's buffers
    (JC_REQUEST_DEVICE_BUFFERS), device memory or page-locked host memory,
    give the same bits as host-buffer requests (staged by the server) and as
    the model's own rollout; the server's device-timed span covers the
    work."""
    torch = pytest.importorskip("torch")
    (fm, _, cfgs), (rm, _, _) = families
    rng = np.random.default_rng(11)
    reqs = []
    for k in range(6):
        task = (engine.TASK_FORWARD, engine.TASK_REWIND, engine.TASK_RECONSTRUCT)[k % 3]
        g = int(rng.integers(0, len(SIDES)))
        cfg = cfgs[g]
        H = int(rng.integers(2, 7))
        if task == engine.TASK_RECONSTRUCT:
            known = (rng.random((H + 1, cfg.ny, cfg.nx)) < 0.05).astype(np.uint8)
            x = np.where(known[:, None], 0.3 * rng.standard_normal((H + 1, 3, cfg.ny, cfg.nx)), 0).astype(np.float32)
        else:
            known, x = None, random_drops(cfg, seed=300 + k)
        reqs.append((task, g, H, x, known, meta_of(cfg)))
    with engine.Server(fm, rm, max_active_cells=1 << 18) as srv:
        host = []
        for task, g, H, x, known, meta in reqs:
            rid = srv.submit(task, g, x, meta, H, ME, known=known, max_sweeps=3, tol=0.0)
            host.append(srv.wait(rid, task, g, H, timeout=60)[0])
        srv.reset_stats()
        dev_in = [(torch.from_numpy(np.ascontiguousarray(x)).cuda(),
                   torch.from_numpy(np.ascontiguousarray(known)).cuda() if known is not None else None,
                   torch.from_numpy(np.ascontiguousarray(meta)).cuda()) for _, _, _, x, known, meta in reqs]
        outs = [torch.empty(srv.out_shape(task, g, H), device="cuda") for task, g, H, _, _, _ in reqs]
        torch.cuda.synchronize()
        ids = [srv.submit_device(task, g, dx.data_ptr(), dm.data_ptr(), H, ME,
                                 known_ptr=dk.data_ptr() if dk is not None else None, max_sweeps=3, tol=0.0)
               for (task, g, H, _, _, _), (dx, dk, dm) in zip(reqs, dev_in)]
        for rid, o in zip(ids, outs):
            srv.wait_device(rid, o.data_ptr(), o.numel(), timeout=60)
        st = srv.stats()
        # the same flag with page-locked host buffers: copied by DMA, no staging
        pin_in = [(torch.from_numpy(np.ascontiguousarray(x)).pin_memory(),
                   torch.from_numpy(np.ascontiguousarray(known)).pin_memory() if known is not None else None,
                   torch.from_numpy(np.ascontiguousarray(meta)).pin_memory()) for _, _, _, x, known, meta in reqs]
        pin_out = [torch.empty(srv.out_shape(task, g, H), pin_memory=True) for task, g, H, _, _, _ in reqs]
        ids = [srv.submit_device(task, g, px.data_ptr(), pm.data_ptr(), H, ME,
                                 known_ptr=pk.data_ptr() if pk is not None else None, max_sweeps=3, tol=0.0)
               for (task, g, H, _, _, _), (px, pk, pm) in zip(reqs, pin_in)]
        for rid, o in zip(ids, pin_out):
            srv.wait_device(rid, o.data_ptr(), o.numel(), timeout=60)
    for (task, g, H, x, known, meta), h, o, po in zip(reqs, host, outs, pin_out):
        assert np.array_equal(o.cpu().numpy(), h), (task, g, H)
        assert np.array_equal(po.numpy(), h), (task, g, H)
        if task != engine.TASK_RECONSTRUCT:
            model = fm[g] if task == engine.TASK_FORWARD else rm[g]
            assert np.array_equal(h, model.rollout(x, meta, H, ME)[0])
    assert st["completed"] == len(reqs)
    assert 0 < st["device_span_s"] <= st["span_s"] + 1e-3


def test_reconstruct_that_converges_early_matches_the_batch_runner(families):
    """A tolerance that stops the sweeps before max_sweeps: the server (where
    the request may freeze in the middle of a chunk while other requests run
    on) and the batch runner (a graph while loop that ends on the device)
    apply the same rule, so their volumes, sweep counts and residuals agree
    bit for bit, alone and in a mix."""
    (fm, _, cfgs), (rm, _, _) = families
    g, H = 0, 3
    cfg = cfgs[g]
    rng = np.random.default_rng(9)
    known = (rng.random((H + 1, cfg.ny, cfg.nx)) < 0.1).astype(np.uint8)
    known[0] = 1
    vals = np.where(known[:, None], np.stack([random_drops(cfg, seed=60 + t) for t in range(H + 1)]), 0)
    vals = vals.astype(np.float32)
    meta = meta_of(cfg)
    n = len(SIDES)
    with engine.Batch(fm + rm, max_instances=64, max_cells=1 << 16) as b:
        # the residual after each sweep count, with a tolerance of 0; a
        # tolerance just above the fifth makes the sweeps stop early
        item = {"task": engine.TASK_RECONSTRUCT, "model": g, "reverse_model": g + n, "x": vals, "known": known,
                "meta": meta, "ticks": H, "max_sweeps": 12, "tol": 0.0}
        sweeps_res = []
        for s in range(1, 13):
            item["max_sweeps"] = s
            sweeps_res.append(b.rollout([item])[0][2])
        tol = float(sweeps_res[4]) * 1.0001
        item["max_sweeps"], item["tol"] = 12, tol
        (want, w_sweeps, w_resid), = b.rollout([item])
    assert int(w_sweeps) < 12
    with engine.Server(fm, rm, max_active_cells=1 << 18) as srv:
        rid = srv.submit(engine.TASK_RECONSTRUCT, g, vals, meta, H, known=known, max_sweeps=12, tol=tol)
        alone, info = srv.wait(rid, engine.TASK_RECONSTRUCT, g, H, timeout=60)
        others = [srv.submit(engine.TASK_FORWARD, k % 3, random_drops(cfgs[k % 3], seed=k), meta_of(cfgs[k % 3]),
                             20) for k in range(4)]
        rid = srv.submit(engine.TASK_RECONSTRUCT, g, vals, meta, H, known=known, max_sweeps=12, tol=tol)
        mixed, info2 = srv.wait(rid, engine.TASK_RECONSTRUCT, g, H, timeout=60)
        for i, k in zip(others, range(4)):
            srv.wait(i, engine.TASK_FORWARD, k % 3, 20, timeout=60)
    assert np.array_equal(alone, want) and np.array_equal(mixed, want)
    assert info["sweeps"] == info2["sweeps"] == int(w_sweeps)
    assert info["residual"] == info2["residual"] == np.float32(w_resid)


def test_loop_profile_reports_its_kernels(families):
    """jc_server_profile: per-kernel device times of the loop's launches
    between start and stop; nothing is recorded once stopped."""
    (fm, _, cfgs), (rm, _, _) = families
    with engine.Server(fm, rm, max_active_cells=1 << 18) as srv:
        srv.profile_start()
        rid = srv.submit(engine.TASK_FORWARD, 1, random_drops(cfgs[1], seed=3), meta_of(cfgs[1]), 4)
        srv.wait(rid, engine.TASK_FORWARD, 1, 4, timeout=60)
        prof = srv.profile_stop()
        rid = srv.submit(engine.TASK_FORWARD, 1, random_drops(cfgs[1], seed=4), meta_of(cfgs[1]), 4)
        srv.wait(rid, engine.TASK_FORWARD, 1, 4, timeout=60)
        assert srv.profile_stop() == {}
    assert "projection" in prof and all(n > 0 and ms > 0 for n, ms in prof.values())
    per_tick = "tc_qkv" if fm[1].precision == engine.BF16 else "f32_attention"
    assert prof[per_tick][0] == 4 * fm[1].config.layers  # one launch per layer and tick
