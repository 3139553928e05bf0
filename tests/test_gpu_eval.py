"""Evaluation on the GPU: the reference solver (jc_sw_run), the eval-metrics
scores (jc_eval_score) and the evaluator (jc_eval_run), against the oracle's
restatement of crates/solvers/src/shallow_water.rs, crates/engine/src/metrics.rs
and the eval-metrics loop of crates/engine-cli/src/eval.rs."""

from pathlib import Path

import numpy as np
import pytest

from jacobi2000_gb300 import engine
from jacobi2000_gb300.checkpoint import meta_of, parse_config, synthetic_checkpoint, write_safetensors_bytes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def _sw(nx, ny, nu=1e-3, dt=0.0903, g=9.81, depth=1.0, dx=1.0):
    return engine.JcSwParams(nx, ny, dx, dt, g, depth, nu)


def _orc_sw(p):
    q = O._SwParams()
    q.nx, q.ny, q.dx, q.dt, q.g, q.depth, q.nu = p.nx, p.ny, p.dx, p.dt, p.g, p.depth, p.nu
    return q


def _states(p, count, seed):
    rng = np.random.default_rng(seed)
    s = engine.sw_flat(p, count)
    for k in range(count):
        engine.sw_add_drop(p, s[k, 0], rng.uniform(0, p.nx), rng.uniform(0, p.ny), rng.uniform(0.02, 0.1),
                           rng.uniform(1.5, 5.0))
        s[k, 1] = (0.02 * rng.standard_normal((p.ny, p.nx))).astype(np.float32)
        s[k, 2] = (0.02 * rng.standard_normal((p.ny, p.nx))).astype(np.float32)
    return s


@pytest.mark.parametrize("nx,ny,steps", [(64, 64, 25), (37, 23, 8), (1, 5, 3), (6, 1, 4), (130, 70, 7),
                                         (256, 256, 10)])
def test_solver_matches_oracle_bit_for_bit(nx, ny, steps):
    p = _sw(nx, ny)
    s0 = _states(p, 3, nx * 7 + ny)
    got = engine.sw_run(p, s0, steps)
    q = _orc_sw(p)
    for k in range(3):
        want = s0[k].copy()
        O.sw_steps(q, want, steps)
        np.testing.assert_array_equal(got[k], want)


def test_add_drop_matches_oracle_bit_for_bit():
    p = _sw(48, 40)
    a = engine.sw_flat(p)[0]
    engine.sw_add_drop(p, a[0], 17.3, 22.9, 0.05, 3.7)
    b = O.sw_flat(_orc_sw(p))[0]
    O.sw_add_drop(_orc_sw(p), b[0], 17.3, 22.9, 0.05, 3.7)
    np.testing.assert_array_equal(a, b)


# crates/solvers/src/shallow_water.rs:260-322 on the GPU solver. Params::default
# with dt = with_cfl_dt(0.4) (:31-44), in f32.
def _cfl_params(nu=0.0):
    c = np.sqrt(np.float32(9.81) * np.float32(1.0), dtype=np.float32)
    dt = float(np.float32(0.4) * np.float32(1.0) / (c * np.float32(np.sqrt(2.0))))
    return _sw(64, 64, nu=nu, dt=dt)


def test_reference_solver_properties_on_the_gpu():
    p = _cfl_params()
    flat = engine.sw_run(p, engine.sw_flat(p), 200)[0]
    assert np.all(flat[0] == np.float32(1.0)) and not flat[1].any() and not flat[2].any()

    s = engine.sw_flat(p)
    engine.sw_add_drop(p, s[0, 0], 20.0, 30.0, 0.05, 4.0)
    m0 = float(np.sum(s[0, 0], dtype=np.float64))
    s = engine.sw_run(p, s, 500)
    assert abs((float(np.sum(s[0, 0], dtype=np.float64)) - m0) / m0) < 1e-7

    s = engine.sw_flat(p)
    engine.sw_add_drop(p, s[0, 0], 31.5, 31.5, 0.05, 5.0)
    h, u, v = engine.sw_run(p, s, 120)[0]
    assert np.abs(h - h[:, ::-1]).max() < 1e-6 and np.abs(h - h[::-1, :]).max() < 1e-6
    assert np.abs(u + u[:, ::-1]).max() < 1e-6 and np.abs(v + v[::-1, :]).max() < 1e-6

    p = _cfl_params(nu=1e-3)
    s = engine.sw_flat(p)
    engine.sw_add_drop(p, s[0, 0], 24.0, 40.0, 0.08, 4.0)
    s = engine.sw_run(p, s, 2000)
    amp = np.abs(s[0, 0] - np.float32(1.0)).max()
    assert np.isfinite(amp) and amp < 0.08


def test_solver_on_device_buffers():
    torch = pytest.importorskip("torch")
    p = _sw(96, 80)
    s0 = _states(p, 2, 3)
    want = engine.sw_run(p, s0, 11)
    d = torch.from_numpy(s0.copy()).cuda()
    L = engine.load_library()
    engine._declare_eval(L)
    engine._check(L.jc_sw_run_device(engine.C.byref(p), d.data_ptr(), 2, 11, None))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.cpu().numpy(), want)


class _Cfg:
    pass


def _cfg_of(nx, ny, mean, std, depth):
    c = engine.JcConfig()
    c.nx, c.ny = nx, ny
    c.norm_mean[:] = [float(v) for v in mean]
    c.norm_std[:] = [float(v) for v in std]
    c.norm_depth = float(depth)
    o = _Cfg()
    o.nx, o.ny, o.norm_mean, o.norm_std, o.norm_depth = nx, ny, mean, std, float(depth)
    return c, o


def _check_rows(got, want, exact_bias=True):
    """Peaks, profiles and the f32 bias sums follow the reference's order on
    both sides; the correlations' f64 sums are tree-ordered on the GPU, which
    can move a correlation by one f32 step."""
    for k in range(len(want)):
        g, w = got[k], want[k]
        assert abs(g["corr"] - w[0]) <= 2.5e-7, (k, g["corr"], w[0])
        assert abs(g["corr_h"] - w[1]) <= 2.5e-7, (k, g["corr_h"], w[1])
        assert g["amplitude_ratio"] == np.float32(w[2]), k
        assert abs(g["lag"] - w[3]) <= 1e-5, (k, g["lag"], w[3])
        if exact_bias:
            assert g["bias"] == np.float32(w[4]), (k, g["bias"], w[4])


def test_eval_score_matches_oracle_on_the_golden_fields():
    g = np.load(GOLDEN / "metrics.npz")
    nx, ny = int(g["nx"]), int(g["ny"])
    c, o = _cfg_of(nx, ny, g["norm_mean"], g["norm_std"], g["norm_depth"])
    cx, cy = float(g["cx"]), float(g["cy"])
    got = engine.eval_score(c, g["x"][None], g["truth"][None], np.array([[cx, cy]], np.float32))
    want = O.eval_score(o, g["x"], g["truth"], cx, cy)
    _check_rows(got, [want])


@pytest.mark.parametrize("nx,ny", [(128, 128), (96, 64), (256, 256), (20, 36)])
def test_eval_score_matches_oracle_on_solver_states(nx, ny):
    mean = np.array([0.0008, 0.0004, 0.0005], np.float32)
    std = np.array([0.0063, 0.0138, 0.0135], np.float32)
    c, o = _cfg_of(nx, ny, mean, std, 1.0)
    p = _sw(nx, ny)
    rng = np.random.default_rng(nx + ny)
    count = 4
    truth = engine.sw_flat(p, count)
    centres = np.zeros((count, 2), np.float32)
    for k in range(count):
        cx, cy = rng.uniform(2, nx - 2), rng.uniform(2, ny - 2)
        if k == 3:
            cx, cy = float(nx // 2), float(ny // 2)  # integer centre: many cells on bin boundaries
        centres[k] = (cx, cy)
        engine.sw_add_drop(p, truth[k, 0], cx, cy, 0.05, 3.0)
    truth = engine.sw_run(p, truth, 12)
    x = np.stack([O.encode(o, truth[k]) for k in range(count)])
    x = (x + 0.3 * rng.standard_normal(x.shape)).astype(np.float32)  # a model that is off
    got = engine.eval_score(c, x, truth, centres)
    want = [O.eval_score(o, x[k], truth[k], float(centres[k, 0]), float(centres[k, 1])) for k in range(count)]
    _check_rows(got, want)


@pytest.fixture(scope="module")
def model64():
    t, cj = synthetic_checkpoint(64, 128, 4, 0)
    cfg = parse_config(cj, t)
    m = engine.Model.from_bytes(write_safetensors_bytes(t), cj)
    yield m, cfg, O.OracleModel(cfg, t)
    m.close()


DROPS = [(30.5, 28.0, 0.05, 4.0), (22.0, 40.3, 0.035, 3.2), (33.3, 31.1, 0.06, 5.1)]


def test_evaluator_matches_oracle_eval_loop(model64):
    m, cfg, om = model64
    horizons = [2, 5, 9]
    with engine.Evaluator(m, 4) as ev:
        rows, viol = ev.run(DROPS, horizons, engine.PROJECT_MASS | engine.PROJECT_ENERGY)
    want, wviol = O.eval_metrics(om, DROPS, horizons, O.MASS | O.ENERGY | O.SUM64, meta_of(cfg))
    # the FP32 model path differs from the oracle's f32 forward by ~1e-6 per
    # tick, which the scores carry; the solver and the scoring are exact
    for i in range(len(horizons)):
        for k in range(len(DROPS)):
            g, w = rows[i, k], want[i, k]
            assert abs(g["corr"] - w[0]) < 1e-5
            assert abs(g["corr_h"] - w[1]) < 1e-5
            assert abs(g["amplitude_ratio"] - w[2]) < 1e-4 * abs(w[2])
            assert abs(g["lag"] - w[3]) < 1e-3
            assert abs(g["bias"] - w[4]) < 1e-3 * abs(w[4]) + 1e-5
    assert viol <= 1e-6 and wviol <= 1e-6


def test_evaluator_rows_do_not_depend_on_the_batch(model64):
    m, cfg, om = model64
    horizons = [3, 7]
    with engine.Evaluator(m, 4) as ev:
        all_rows, _ = ev.run(DROPS, horizons)
        again, _ = ev.run(DROPS, horizons)  # graph replay
        alone, _ = ev.run(DROPS[1:2], horizons)
    np.testing.assert_array_equal(all_rows, again)
    np.testing.assert_array_equal(all_rows[:, 1:2], alone)


def test_evaluator_bf16_close_to_fp32(model64):
    m, cfg, om = model64
    t, cj = synthetic_checkpoint(64, 128, 4, 0)
    with engine.Model.from_bytes(write_safetensors_bytes(t), cj, engine.BF16) as mb:
        with engine.Evaluator(m, 4) as e32, engine.Evaluator(mb, 4) as e16:
            r32, _ = e32.run(DROPS, [4, 8])
            r16, v16 = e16.run(DROPS, [4, 8], engine.PROJECT_MASS | engine.PROJECT_ENERGY)
    assert np.abs(r32["corr"] - r16["corr"]).max() < 1e-2
    assert np.abs(r32["corr_h"] - r16["corr_h"]).max() < 1e-2
    assert v16 <= 1e-6


def test_evaluator_rejects_bad_arguments(model64):
    m, cfg, om = model64
    with engine.Evaluator(m, 2) as ev:
        for drops, hz in [(DROPS, [3]), (DROPS[:1], [3, 3]), (DROPS[:1], [0, 2]), ([], [2]),
                          ([(float("nan"), 3.0, 0.05, 3.0)], [2])]:
            with pytest.raises(engine.JcError) as e:
                ev.run(drops, hz)
            assert e.value.name == "BAD_ARGUMENT"


def test_eval_metrics_command(tmp_path, capsys):
    from jacobi2000_gb300 import evaluate

    t, cj = synthetic_checkpoint(128, 128, 4, 0)
    (tmp_path / "model.safetensors").write_bytes(write_safetensors_bytes(t))
    (tmp_path / "config.json").write_text(cj)
    assert evaluate.main(["--model", str(tmp_path), "--horizons", "5,10", "--trajectories", "3",
                          "--project-energy", "true"]) == 0
    out = capsys.readouterr().out
    assert "3 single-drop trajectories" in out and "| 10 |" in out
    assert "max relative energy violation" in out


@pytest.fixture(scope="module")
def pair64():
    tf, cjf = synthetic_checkpoint(64, 128, 4, 0)
    tr, cjr = synthetic_checkpoint(64, 128, 4, 1)
    cfg = parse_config(cjf, tf)
    f = engine.Model.from_bytes(write_safetensors_bytes(tf), cjf)
    r = engine.Model.from_bytes(write_safetensors_bytes(tr), cjr)
    yield f, r, cfg, O.OracleModel(cfg, tf), O.OracleModel(parse_config(cjr, tr), tr), (tf, cjf, tr, cjr)
    f.close()
    r.close()


def test_roundtrip_matches_oracle(pair64):
    f, r, cfg, of, orv, _ = pair64
    horizons = [2, 5]
    flags = engine.PROJECT_MASS | engine.PROJECT_ENERGY
    with engine.RoundTrip(f, r, 4, 2) as rt:
        rows = rt.run(DROPS, horizons, flags)
    want = O.roundtrip(of, orv, DROPS, horizons, O.MASS | O.ENERGY | O.SUM64, meta_of(cfg))
    for i in range(len(horizons)):
        for k in range(len(DROPS)):
            g, w = rows[i, k], want[i, k]
            assert abs(g["corr"] - w[0]) < 1e-5
            assert abs(g["amplitude_ratio"] - w[1]) < 1e-4 * abs(w[1])
            assert abs(g["rmse"] - w[2]) < 1e-4 * abs(w[2]) + 1e-6
            assert abs(g["change_rmse"] - w[3]) < 1e-4 * abs(w[3]) + 1e-6


def test_roundtrip_rows_do_not_depend_on_the_batch(pair64):
    f, r, cfg, of, orv, _ = pair64
    with engine.RoundTrip(f, r, 4, 3) as rt:
        a = rt.run(DROPS, [1, 3, 6])
        b = rt.run(DROPS, [1, 3, 6])
        c = rt.run(DROPS[2:], [3])
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a[1, 2:], c[0])


def test_roundtrip_bf16_close_to_fp32(pair64):
    f, r, cfg, of, orv, (tf, cjf, tr, cjr) = pair64
    with engine.Model.from_bytes(write_safetensors_bytes(tf), cjf, engine.BF16) as fb, \
            engine.Model.from_bytes(write_safetensors_bytes(tr), cjr, engine.BF16) as rb:
        with engine.RoundTrip(f, r, 4, 2) as r32, engine.RoundTrip(fb, rb, 4, 2) as r16:
            a = r32.run(DROPS, [2, 4])
            b = r16.run(DROPS, [2, 4])
    assert np.abs(a["corr"] - b["corr"]).max() < 1e-2
    assert np.abs(a["change_rmse"] - b["change_rmse"]).max() < 1e-2 * np.abs(a["change_rmse"]).max()


def test_roundtrip_rejects_bad_arguments(pair64):
    f, r, cfg, of, orv, _ = pair64
    with engine.RoundTrip(f, r, 2, 2) as rt:
        for drops, hz in [(DROPS, [3]), (DROPS[:1], [1, 2, 3]), (DROPS[:1], [2, 2]), (DROPS[:1], [0])]:
            with pytest.raises(engine.JcError) as e:
                rt.run(drops, hz)
            assert e.value.name == "BAD_ARGUMENT"
    t, cj = synthetic_checkpoint(32, 128, 4, 1)
    with engine.Model.from_bytes(write_safetensors_bytes(t), cj) as other:
        with pytest.raises(engine.JcError) as e:
            engine.RoundTrip(f, other, 2, 2)
        assert e.value.name == "BAD_SHAPE"


def test_roundtrip_command(tmp_path, capsys):
    from jacobi2000_gb300 import roundtrip

    for name, seed in (("fwd", 0), ("rev", 1)):
        t, cj = synthetic_checkpoint(128, 128, 4, seed)
        (tmp_path / name).mkdir()
        (tmp_path / name / "model.safetensors").write_bytes(write_safetensors_bytes(t))
        (tmp_path / name / "config.json").write_text(cj)
    assert roundtrip.main(["--forward", str(tmp_path / "fwd"), "--reverse", str(tmp_path / "rev"),
                           "--horizons", "3,6", "--trajectories", "3"]) == 0
    out = capsys.readouterr().out
    assert "| 6 |" in out and "round-trip RMSE" in out


def _oracle_trajectory(p, x0, ticks, drops):
    """dump_dataset.rs:164-175 on the oracle: frames [3, ticks + 1, ny, nx]."""
    q = _orc_sw(p)
    s = np.array(x0, dtype=np.float32, copy=True)
    frames = np.empty((3, ticks + 1, p.ny, p.nx), dtype=np.float32)
    frames[:, 0] = s
    for t in range(1, ticks + 1):
        O.sw_steps(q, s, 1)
        for tick, f in drops:  # apply_pending, in order
            if tick == t:
                s[0] = s[0] + f
        frames[:, t] = s
    return frames


def test_solver_trajectories_match_oracle_bit_for_bit():
    p = _sw(40, 24)
    rng = np.random.default_rng(3)
    items = []
    for k, ticks in enumerate([9, 3, 14, 0]):
        x0 = engine.sw_flat(p)[0]
        engine.sw_add_drop(p, x0[0], rng.uniform(5, 35), rng.uniform(5, 19), 0.05, 3.0)
        drops = []
        for tick in ([2, 2, 7] if k == 0 else ([ticks] if ticks > 0 else [])):
            f = np.zeros((p.ny, p.nx), np.float32)
            engine.sw_add_drop(p, f, rng.uniform(5, 35), rng.uniform(5, 19), rng.uniform(-0.1, 0.1), 2.5)
            drops.append((tick, f))
        items.append((x0, ticks, drops))
    got = engine.sw_trajectories(p, items)
    for (x0, ticks, drops), fr in zip(items, got):
        np.testing.assert_array_equal(fr, _oracle_trajectory(p, x0, ticks, drops))


def test_dump_dataset_command(tmp_path, capsys):
    import json
    from jacobi2000_gb300 import dump_dataset as D

    assert D.main(["--out", str(tmp_path), "--pool", "5", "--seed", "3", "--chunk", "2"]) == 0
    assert "5 trajectories" in capsys.readouterr().out
    manifest = json.loads((tmp_path / "manifest.json").read_text())
    assert [h["index"] for h in manifest] == list(range(5))
    cfg = D.DumpConfig(pool=5, seed=3)
    p = cfg.params()
    rng = np.random.default_rng(3)
    trajs = [D.draw(cfg, rng) for _ in range(5)]
    for h, t in zip(manifest, trajs):
        assert json.loads((tmp_path / f"traj-{h['index']:05d}.json").read_text()) == h
        raw = np.fromfile(tmp_path / f"traj-{h['index']:05d}.f32", dtype="<f4")
        assert raw.size == 3 * h["ticks"] * 64 * 64 and h["ticks"] == t.ticks + 1
        x0 = engine.sw_flat(p)[0]
        engine.sw_add_drop(p, x0[0], t.cx, t.cy, t.amp, t.sigma)
        drops = []
        for (tick, cx, cy, amp, sigma) in t.pending:
            f = np.zeros((64, 64), np.float32)
            engine.sw_add_drop(p, f, cx, cy, amp, sigma)
            drops.append((tick, f))
        np.testing.assert_array_equal(raw.reshape(3, t.ticks + 1, 64, 64), _oracle_trajectory(p, x0, t.ticks, drops))
