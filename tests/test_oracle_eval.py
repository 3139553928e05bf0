"""The CPU oracle of the evaluation path (oracle/solver.c): the shallow-water
solver and the eval-metrics scores, pinned against

* the reference solver's own unit tests (crates/solvers/src/shallow_water.rs:
  260-322: flat stays flat, mass is conserved, a symmetric drop stays
  symmetric, a long run stays bounded),
* the reference metrics' unit tests (crates/engine/src/metrics.rs:118-135),
* golden scores from the reference's Python scoring twin
  (tests/golden/metrics.npz, written by tests/golden/make_golden.py), and
* an independent vectorised numpy restatement of ShallowWater::step in f32
  (every operation separately rounded, as in the reference), which must agree
  bit for bit.
"""

from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


class _P:
    """solvers::Params fields (shallow_water.rs:16-29)."""

    def __init__(self, nx=64, ny=64, dx=1.0, dt=None, g=9.81, depth=1.0, nu=0.0):
        self.nx, self.ny, self.dx, self.g, self.depth, self.nu = nx, ny, dx, g, depth, nu
        if dt is None:  # Params::with_cfl_dt(0.4), shallow_water.rs:49-57, in f32
            c = np.sqrt(np.float32(g) * np.float32(depth), dtype=np.float32)
            dt = np.float32(0.4) * np.float32(dx) / (c * np.float32(np.sqrt(2.0)))
        self.dt = float(np.float32(dt))


def _params(**kw):
    return O.sw_params(_P(**kw))


def numpy_step(p, s):
    """ShallowWater::step (shallow_water.rs:149-238) vectorised in numpy f32."""
    f = np.float32
    h, u, v = s[0], s[1], s[2]
    nx, ny = p.nx, p.ny
    fx = np.zeros((ny, nx + 1), np.float32)
    fx[:, 1:nx] = f(0.5) * (h[:, :-1] + h[:, 1:]) * f(0.5) * (u[:, :-1] + u[:, 1:])
    fy = np.zeros((ny + 1, nx), np.float32)
    fy[1:ny, :] = f(0.5) * (h[:-1, :] + h[1:, :]) * f(0.5) * (v[:-1, :] + v[1:, :])
    r = f(p.dt) / f(p.dx)
    hn = h - r * ((fx[:, 1:] - fx[:, :-1]) + (fy[1:, :] - fy[:-1, :]))
    xm = np.maximum(np.arange(nx) - 1, 0)
    xp = np.minimum(np.arange(nx) + 1, nx - 1)
    ym = np.maximum(np.arange(ny) - 1, 0)
    yp = np.minimum(np.arange(ny) + 1, ny - 1)
    sxm = np.where(np.arange(nx) == 0, f(-1), f(1)).astype(np.float32)[None, :]
    sxp = np.where(np.arange(nx) == nx - 1, f(-1), f(1)).astype(np.float32)[None, :]
    sym = np.where(np.arange(ny) == 0, f(-1), f(1)).astype(np.float32)[:, None]
    syp = np.where(np.arange(ny) == ny - 1, f(-1), f(1)).astype(np.float32)[:, None]
    hl, hr, hd, hu = hn[:, xm], hn[:, xp], hn[ym, :], hn[yp, :]
    ul, ur, ud, uu = sxm * u[:, xm], sxp * u[:, xp], u[ym, :], u[yp, :]
    vl, vr, vd, vu = v[:, xm], v[:, xp], sym * v[ym, :], syp * v[yp, :]
    inv2dx = f(1) / (f(2) * f(p.dx))
    invdx2 = f(1) / (f(p.dx) * f(p.dx))
    dudx, dudy = (ur - ul) * inv2dx, (uu - ud) * inv2dx
    dvdx, dvdy = (vr - vl) * inv2dx, (vu - vd) * inv2dx
    dhdx, dhdy = (hr - hl) * inv2dx, (hu - hd) * inv2dx
    lap_u = ((((ul + ur) + ud) + uu) - f(4) * u) * invdx2
    lap_v = ((((vl + vr) + vd) + vu) - f(4) * v) * invdx2
    dt, g, nu = f(p.dt), f(p.g), f(p.nu)
    un = u + dt * ((((-u) * dudx - v * dudy) - g * dhdx) + nu * lap_u)
    vn = v + dt * ((((-u) * dvdx - v * dvdy) - g * dhdy) + nu * lap_v)
    return np.stack([hn, un, vn]).astype(np.float32)


def test_flat_stays_flat():
    p = _params()
    s = O.sw_flat(p)[0]
    O.sw_steps(p, s, 200)
    assert np.all(s[0] == np.float32(p.depth)) and not s[1].any() and not s[2].any()


def test_mass_is_conserved():
    p = _params()
    s = O.sw_flat(p)[0]
    O.sw_add_drop(p, s[0], 20.0, 30.0, 0.05, 4.0)
    m0 = O.sw_mass(s[0])
    O.sw_steps(p, s, 500)
    assert abs((O.sw_mass(s[0]) - m0) / m0) < 1e-7


def test_symmetric_drop_stays_symmetric():
    p = _params()
    s = O.sw_flat(p)[0]
    O.sw_add_drop(p, s[0], 31.5, 31.5, 0.05, 5.0)
    O.sw_steps(p, s, 120)
    h, u, v = s
    assert np.abs(h - h[:, ::-1]).max() < 1e-6 and np.abs(h - h[::-1, :]).max() < 1e-6
    assert np.abs(u + u[:, ::-1]).max() < 1e-6 and np.abs(v + v[::-1, :]).max() < 1e-6


def test_drop_stays_bounded_over_a_long_run():
    p = _params(nu=1e-3)
    s = O.sw_flat(p)[0]
    O.sw_add_drop(p, s[0], 24.0, 40.0, 0.08, 4.0)
    O.sw_steps(p, s, 2000)
    amp = np.abs(s[0] - np.float32(p.depth)).max()
    assert np.isfinite(amp) and amp < 0.08


@pytest.mark.parametrize("nx,ny,nu", [(64, 64, 0.0), (37, 23, 1e-3), (1, 5, 0.0), (6, 1, 2e-3)])
def test_step_matches_numpy_restatement_bit_for_bit(nx, ny, nu):
    p = _params(nx=nx, ny=ny, nu=nu)
    s = O.sw_flat(p)[0]
    rng = np.random.default_rng(nx * 100 + ny)
    O.sw_add_drop(p, s[0], nx * 0.4, ny * 0.6, 0.07, 3.0)
    s[1] = (0.01 * rng.standard_normal((ny, nx))).astype(np.float32)
    s[2] = (0.01 * rng.standard_normal((ny, nx))).astype(np.float32)
    ref = s.copy()
    for _ in range(7):
        ref = numpy_step(p, ref)
    O.sw_steps(p, s, 7)
    np.testing.assert_array_equal(s, ref)


def test_add_drop_matches_expf_formula():
    p = _params(nx=19, ny=11)
    s = O.sw_flat(p)[0]
    O.sw_add_drop(p, s[0], 7.25, 4.5, 0.05, 2.5)
    f = np.float32
    yy, xx = np.meshgrid(np.arange(11, dtype=np.float32), np.arange(19, dtype=np.float32), indexing="ij")
    inv = f(1) / (f(2) * f(2.5) * f(2.5))
    dx, dy = xx - f(7.25), yy - f(4.5)
    want = f(1) + f(0.05) * np.exp(-(dx * dx + dy * dy) * inv)
    # numpy's float32 exp and the C library's expf may differ in the last place
    np.testing.assert_allclose(s[0], want, rtol=2e-7, atol=0)


def test_metrics_unit_cases():
    """crates/engine/src/metrics.rs:118-135."""
    a = np.array([0.1, 0.5, -0.3, 0.9, -0.7], dtype=np.float32)
    assert abs(O.correlation(a, a) - 1.0) < 1e-6
    assert O.correlation(np.ones(5, np.float32), a) == 0.0
    assert O.bias(a, a) == 0.0


def _golden():
    g = np.load(GOLDEN / "metrics.npz")

    class Cfg:
        pass

    c = Cfg()
    c.nx, c.ny = int(g["nx"]), int(g["ny"])
    c.norm_mean, c.norm_std, c.norm_depth = g["norm_mean"], g["norm_std"], float(g["norm_depth"])
    return g, c


def test_encode_matches_golden_bit_for_bit():
    g, c = _golden()
    np.testing.assert_array_equal(O.encode(c, g["truth"]), g["target"])


def test_eval_score_matches_python_twin():
    """The Python twin computes radii and profile correlations in f64 where
    metrics.rs uses f32 (5 of the 1,920 cells fall in a neighbouring radius
    bin), and averages with numpy's pairwise sums where metrics.rs adds
    sequentially in f32; the tolerances cover exactly those differences."""
    g, c = _golden()
    row = O.eval_score(c, g["x"], g["truth"], float(g["cx"]), float(g["cy"]))
    want = g["row"]
    assert abs(row[0] - want[0]) < 1e-6
    assert abs(row[1] - want[1]) < 1e-6
    assert abs(row[2] - want[2]) < 1e-6
    assert abs(row[3] - want[3]) < 5e-3
    assert abs(row[4] - want[4]) < 1e-4 * abs(want[4]) + 1e-6


def _profile(f, nx, ny, cx, cy, dt):
    """metrics.rs:45-61 in numpy with radii computed in `dt`."""
    ys, xs = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    dx, dy = xs.astype(dt) - dt(cx), ys.astype(dt) - dt(cy)
    bins = (np.sqrt(dx * dx + dy * dy) + dt(0.5)).astype(np.int64).ravel()
    rmax = int(max(np.floor(np.float32(min(cx, cy, nx - np.float32(cx), ny - np.float32(cy)))), 1))
    sums = np.zeros(rmax + 1)
    counts = np.zeros(rmax + 1)
    ok = bins <= rmax
    np.add.at(sums, bins[ok], np.abs(f[ok]).astype(np.float64))
    np.add.at(counts, bins[ok], 1)
    return np.where(counts > 0, sums / np.maximum(counts, 1), 0.0)


def _ph(g, c):
    n = c.nx * c.ny
    return (g["x"].ravel()[:n] * g["norm_std"][0] + g["norm_mean"][0]).astype(np.float32)


def test_radial_profile_differs_from_the_twin_only_by_radius_precision():
    g, c = _golden()
    cx, cy, f = float(g["cx"]), float(g["cy"]), _ph(g, c)
    np.testing.assert_allclose(_profile(f, c.nx, c.ny, cx, cy, np.float64), g["prof_model"], rtol=1e-12)
    np.testing.assert_array_equal(O.radial_profile(f, c.nx, c.ny, cx, cy),
                                  _profile(f, c.nx, c.ny, cx, cy, np.float32))


def test_xcorr_lag_recovers_a_shift():
    r = np.arange(40, dtype=np.float64)
    truth = np.exp(-((r - 15.0) ** 2) / 8.0)
    model = np.exp(-((r - 17.0) ** 2) / 8.0)
    lag = O.xcorr_lag(model, truth, 8)
    assert abs(lag - 2.0) < 0.05
    assert O.xcorr_lag(truth, truth, 8) == 0.0


def test_dump_dataset_draws_follow_the_reference_distribution():
    from jacobi2000_gb300 import dump_dataset as D

    cfg = D.DumpConfig(pool=400)
    rng = np.random.default_rng(20)
    ts = [D.draw(cfg, rng) for _ in range(400)]
    longs = [t for t in ts if t.ticks == 400]
    shorts = [t for t in ts if t.ticks != 400]
    assert 0.1 < len(longs) / 400 < 0.3 and all(60 <= t.ticks <= 80 for t in shorts)
    cpt = 0.4 / np.sqrt(2.0)  # cells per tick at the CFL dt
    for t in ts:
        assert 0.02 <= abs(t.amp) < 0.3 and 2.5 <= t.sigma < 6.0
        assert 8.0 <= t.cx < 56.0 and 8.0 <= t.cy < 56.0
        assert len(t.pending) <= 2 and all(1 <= d[0] < t.ticks for d in t.pending)
    # short, non-extended lives keep the pre-reflection margin
    assert any(min(t.cx, t.cy, 64 - t.cx, 64 - t.cy) >= t.ticks * cpt - 1e-3 for t in shorts)
    assert any(t.amp < 0 for t in ts) and any(t.pending for t in ts)


def test_dump_dataset_header_layout():
    from jacobi2000_gb300 import dump_dataset as D

    h = {"index": 3, "ticks": 61, "nx": 64, "dx": 1.0, "dt": float(np.float32(0.09032)), "cx": float(np.float32(30.2))}
    assert D.header_json(h) == '{"index":3,"ticks":61,"nx":64,"dx":1.0,"dt":0.09032,"cx":30.2}'
