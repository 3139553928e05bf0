"""ctypes wrapper of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by ``bench.py``'s CPU-baseline leg, as the checker and the timed CPU
baseline. The product library never imports, links or calls it.

The oracle restates crates/engine/src/cpu.rs:26-352 and project.rs:9-54;
see oracle.h for the function-by-function mapping.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

MASS, ENERGY, SUM64 = 1, 2, 4
MAX_LAYERS = 32


class _Config(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nx", "ny", "patch", "channels", "dim", "layers", "heads", "head_dim",
                                       "ff_inner", "meta_dim", "mask_kind", "radius", "dilation")] + [
        ("norm_mean", C.c_float * 3), ("norm_std", C.c_float * 3), ("norm_depth", C.c_float),
        ("g", C.c_float), ("energy_r_max", C.c_float)]


_FP = C.POINTER(C.c_float)


class _Block(C.Structure):
    _fields_ = [(n, _FP) for n in ("n1g", "n1b", "qw", "qb", "kw", "kb", "vw", "vb", "pw", "pb",
                                   "n2g", "n2b", "f1w", "f1b", "f2w", "f2b")]


class _Weights(C.Structure):
    _fields_ = [(n, _FP) for n in ("embed_w", "embed_b", "meta_w", "meta_b", "pos")] + [
        ("blk", _Block * MAX_LAYERS)] + [(n, _FP) for n in ("norm_g", "norm_b", "tm_w", "tm_b", "tc_w", "tc_b",
                                                             "c1_w", "c1_b", "c2_w", "c2_b")]


def build(quiet: bool = True) -> Path:
    """Compile oracle.c with its Makefile (gcc, OpenMP, no FMA contraction)."""
    srcs = [HERE / "oracle.c", HERE / "oracle_impl.inc", HERE / "solver.c", HERE / "oracle.h"]
    if LIB_PATH.exists() and all(LIB_PATH.stat().st_mtime >= s.stat().st_mtime for s in srcs):
        return LIB_PATH
    out = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        cfgp, wp = C.POINTER(_Config), C.POINTER(_Weights)
        L.orc_forward_f32.argtypes = [cfgp, wp, f32p, f32p, f32p]
        L.orc_forward_f64.argtypes = [cfgp, wp, f64p, f64p, f64p]
        L.orc_rollout_f32.argtypes = [cfgp, wp, f32p, f32p, C.c_int, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_rollout_f32.restype = C.c_double
        L.orc_rollout_f64.argtypes = [cfgp, wp, f64p, f64p, C.c_int, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_rollout_f64.restype = C.c_double
        L.orc_mass_f32.argtypes = [f32p, C.c_int]
        L.orc_mass_f32.restype = C.c_float
        L.orc_energy_f32.argtypes = [f32p, cfgp, C.c_int]
        L.orc_energy_f32.restype = C.c_float
        L.orc_project_mass_f32.argtypes = [f32p, C.c_float, C.c_int]
        L.orc_project_energy_f32.argtypes = [f32p, C.c_float, cfgp, C.c_int]
        L.orc_mass_sum64.argtypes = [f32p, C.c_int]
        L.orc_mass_sum64.restype = C.c_double
        L.orc_energy_sum64.argtypes = [f32p, cfgp, C.c_int]
        L.orc_energy_sum64.restype = C.c_double
        L.orc_project_mass_sum64.argtypes = [f32p, C.c_double, C.c_int]
        L.orc_project_energy_sum64.argtypes = [f32p, C.c_double, cfgp, C.c_int]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int
        L.orc_set_attention_mode.argtypes = [C.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return lib().orc_get_threads()


def set_attention_mode(mode: str) -> None:
    """"scan": every key tested with the mask predicate (the reference's
    O(T^2) cost); "gather": only the stencil candidates (same bits)."""
    lib().orc_set_attention_mode({"scan": 0, "gather": 1}[mode])


class OracleModel:
    """A checkpoint bound to the oracle: ``cfg`` is a ModelConfig, ``tensors``
    the checkpoint's F32 tensors by name."""

    def __init__(self, cfg, tensors):
        self.cfg = cfg
        self._keep = {k: np.ascontiguousarray(v, dtype=np.float32) for k, v in tensors.items()}
        c = _Config()
        for n in ("nx", "ny", "patch", "channels", "dim", "layers", "heads", "head_dim", "ff_inner", "meta_dim",
                  "mask_kind", "radius", "dilation"):
            setattr(c, n, int(getattr(cfg, n)))
        c.norm_mean[:] = [float(v) for v in cfg.norm_mean]
        c.norm_std[:] = [float(v) for v in cfg.norm_std]
        c.norm_depth, c.g, c.energy_r_max = cfg.norm_depth, cfg.g, cfg.energy_r_max
        self._c = c
        w = _Weights()

        def P(name):
            if name not in self._keep:
                raise KeyError(f"missing tensor `{name}`")
            return self._keep[name].ctypes.data_as(_FP)

        w.embed_w, w.embed_b, w.meta_w, w.meta_b, w.pos = (P("embed.weight"), P("embed.bias"), P("meta.weight"),
                                                           P("meta.bias"), P("pos"))
        if cfg.layers > MAX_LAYERS:
            raise ValueError("too many layers for the oracle")
        for i in range(cfg.layers):
            b = w.blk[i]
            p = f"blocks.{i}."
            (b.n1g, b.n1b, b.qw, b.qb, b.kw, b.kb, b.vw, b.vb, b.pw, b.pb, b.n2g, b.n2b, b.f1w, b.f1b, b.f2w,
             b.f2b) = [P(p + s) for s in ("norm1.gamma", "norm1.beta", "q.weight", "q.bias", "k.weight", "k.bias",
                                           "v.weight", "v.bias", "proj.weight", "proj.bias", "norm2.gamma",
                                           "norm2.beta", "ff1.weight", "ff1.bias", "ff2.weight", "ff2.bias")]
        (w.norm_g, w.norm_b, w.tm_w, w.tm_b, w.tc_w, w.tc_b, w.c1_w, w.c1_b, w.c2_w, w.c2_b) = [
            P(n) for n in ("norm.gamma", "norm.beta", "head.token_mix.weight", "head.token_mix.bias",
                           "head.to_cells.weight", "head.to_cells.bias", "head.conv1.weight", "head.conv1.bias",
                           "head.conv2.weight", "head.conv2.bias")]
        self._w = w

    @property
    def state_shape(self):
        return (self.cfg.channels, self.cfg.ny, self.cfg.nx)

    def forward(self, state, meta, f64: bool = False) -> np.ndarray:
        dt = np.float64 if f64 else np.float32
        s = np.ascontiguousarray(state, dtype=dt).reshape(self.state_shape)
        m = np.ascontiguousarray(meta, dtype=dt)
        out = np.empty(self.state_shape, dtype=dt)
        fn = lib().orc_forward_f64 if f64 else lib().orc_forward_f32
        fn(C.byref(self._c), C.byref(self._w), s, m, out)
        return out

    def step(self, state, meta, f64: bool = False) -> np.ndarray:
        """cpu.rs:84-88."""
        s = np.asarray(state, dtype=np.float64 if f64 else np.float32)
        out = self.forward(s, meta, f64)
        out += s.reshape(out.shape)
        return out

    def rollout(self, x0, meta, ticks: int, flags: int = 0, f64: bool = False, trajectory: bool = False):
        """Returns (final_state, energies[ticks+1], max_violation[, trajectory])."""
        dt = np.float64 if f64 else np.float32
        s = np.ascontiguousarray(x0, dtype=dt).reshape(self.state_shape)
        m = np.ascontiguousarray(meta, dtype=dt)
        final = np.empty(self.state_shape, dtype=dt)
        energies = np.empty(ticks + 1, dtype=np.float64)
        traj = np.empty((ticks + 1,) + self.state_shape, dtype=dt) if trajectory else None
        fn = lib().orc_rollout_f64 if f64 else lib().orc_rollout_f32
        viol = fn(C.byref(self._c), C.byref(self._w), s, m, int(ticks), int(flags),
                  traj.ctypes.data if traj is not None else None, final.ctypes.data, energies.ctypes.data)
        if trajectory:
            return final, energies, viol, traj
        return final, energies, viol

    # project.rs, reference arithmetic
    def mass(self, x) -> float:
        return lib().orc_mass_f32(np.ascontiguousarray(x, dtype=np.float32).ravel(), self.cfg.cells)

    def energy(self, x) -> float:
        return lib().orc_energy_f32(np.ascontiguousarray(x, dtype=np.float32).ravel(), C.byref(self._c), self.cfg.cells)

    def energy_sum64(self, x) -> float:
        return lib().orc_energy_sum64(np.ascontiguousarray(x, dtype=np.float32).ravel(), C.byref(self._c),
                                      self.cfg.cells)

    def mass_sum64(self, x) -> float:
        return lib().orc_mass_sum64(np.ascontiguousarray(x, dtype=np.float32).ravel(), self.cfg.cells)

    def project_mass(self, x, target, sum64: bool = False) -> np.ndarray:
        y = np.array(x, dtype=np.float32, copy=True).ravel()
        if sum64:
            lib().orc_project_mass_sum64(y, float(target), self.cfg.cells)
        else:
            lib().orc_project_mass_f32(y, float(target), self.cfg.cells)
        return y.reshape(np.shape(x))

    def project_energy(self, x, prev_energy, sum64: bool = False) -> np.ndarray:
        y = np.array(x, dtype=np.float32, copy=True).ravel()
        if sum64:
            lib().orc_project_energy_sum64(y, float(prev_energy), C.byref(self._c), self.cfg.cells)
        else:
            lib().orc_project_energy_f32(y, float(prev_energy), C.byref(self._c), self.cfg.cells)
        return y.reshape(np.shape(x))


# ---- evaluation path (solver.c): the reference solver and the metrics ----

class _SwParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int)] + [(n, C.c_float) for n in ("dx", "dt", "g", "depth", "nu")]


def _bind_eval(L):
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    swp = C.POINTER(_SwParams)
    L.orc_sw_add_drop.argtypes = [swp, f32p, C.c_float, C.c_float, C.c_float, C.c_float]
    L.orc_sw_mass.argtypes = [f32p, C.c_int]
    L.orc_sw_mass.restype = C.c_double
    L.orc_sw_steps.argtypes = [swp, f32p, f32p, f32p, C.c_int]
    for fn in ("orc_correlation", "orc_bias"):
        getattr(L, fn).argtypes = [f32p, f32p, C.c_int]
        getattr(L, fn).restype = C.c_float
    for fn in ("orc_peak", "orc_mean", "orc_std_dev"):
        getattr(L, fn).argtypes = [f32p, C.c_int]
        getattr(L, fn).restype = C.c_float
    L.orc_radial_profile.argtypes = [f32p, C.c_int, C.c_int, C.c_float, C.c_float, f64p, C.c_int]
    L.orc_radial_profile.restype = C.c_int
    L.orc_rmse.argtypes = [f32p, f32p, C.c_int]
    L.orc_rmse.restype = C.c_float
    L.orc_xcorr_lag.argtypes = [f64p, f64p, C.c_int, C.c_int]
    L.orc_xcorr_lag.restype = C.c_float
    fa3 = C.c_float * 3
    L.orc_encode.argtypes = [fa3, fa3, C.c_float, f32p, f32p, f32p, C.c_int, f32p]
    L.orc_eval_score.argtypes = [fa3, fa3, C.c_float, C.c_int, C.c_int, f32p, f32p, f32p, f32p, C.c_float,
                                 C.c_float, f32p]


def _elib():
    L = lib()
    if not getattr(L, "_eval_bound", False):
        _bind_eval(L)
        L._eval_bound = True
    return L


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def sw_params(cfg) -> _SwParams:
    """solvers::Params of a model config (crates/engine/src/config.rs:102-104)."""
    p = _SwParams()
    p.nx, p.ny = int(cfg.nx), int(cfg.ny)
    p.dx, p.dt, p.g, p.depth, p.nu = float(cfg.dx), float(cfg.dt), float(cfg.g), float(cfg.depth), float(cfg.nu)
    return p


def sw_flat(p: _SwParams, count: int = 1) -> np.ndarray:
    """State::flat for `count` states: [count, 3, ny, nx] (h = depth, u = v = 0)."""
    s = np.zeros((count, 3, p.ny, p.nx), dtype=np.float32)
    s[:, 0] = np.float32(p.depth)
    return s


def sw_add_drop(p: _SwParams, h: np.ndarray, cx: float, cy: float, amp: float, sigma: float) -> None:
    """In place on the h plane [ny, nx] (float32, contiguous)."""
    assert h.dtype == np.float32 and h.flags.c_contiguous
    _elib().orc_sw_add_drop(C.byref(p), h.reshape(-1), cx, cy, amp, sigma)


def sw_steps(p: _SwParams, state: np.ndarray, steps: int) -> None:
    """`steps` solver ticks in place on one state [3, ny, nx] (float32)."""
    assert state.dtype == np.float32 and state.flags.c_contiguous and state.shape == (3, p.ny, p.nx)
    h, u, v = state[0], state[1], state[2]
    _elib().orc_sw_steps(C.byref(p), h, u, v, int(steps))


def sw_mass(h) -> float:
    h = _f32(h).ravel()
    return _elib().orc_sw_mass(h, h.size)


def correlation(a, b) -> float:
    a, b = _f32(a).ravel(), _f32(b).ravel()
    return _elib().orc_correlation(a, b, a.size)


def peak(f) -> float:
    f = _f32(f).ravel()
    return _elib().orc_peak(f, f.size)


def mean(f) -> float:
    f = _f32(f).ravel()
    return _elib().orc_mean(f, f.size)


def std_dev(f) -> float:
    f = _f32(f).ravel()
    return _elib().orc_std_dev(f, f.size)


def bias(model, solver) -> float:
    a, b = _f32(model).ravel(), _f32(solver).ravel()
    return _elib().orc_bias(a, b, a.size)


def radial_profile(f, nx: int, ny: int, cx: float, cy: float) -> np.ndarray:
    out = np.zeros(nx + ny + 2, dtype=np.float64)
    k = _elib().orc_radial_profile(_f32(f).ravel(), nx, ny, cx, cy, out, out.size)
    return out[:k]


def xcorr_lag(model_prof, solver_prof, max_lag: int = 8) -> float:
    m = np.ascontiguousarray(model_prof, dtype=np.float64)
    s = np.ascontiguousarray(solver_prof, dtype=np.float64)
    return _elib().orc_xcorr_lag(m, s, m.size, int(max_lag))


def _norm_args(cfg):
    fa3 = C.c_float * 3
    return fa3(*[float(v) for v in cfg.norm_mean]), fa3(*[float(v) for v in cfg.norm_std]), float(cfg.norm_depth)


def encode(cfg, truth) -> np.ndarray:
    """Normalizer::encode of a solver state [3, ny, nx] -> [3, ny, nx]."""
    t = _f32(truth).reshape(3, -1)
    out = np.empty(t.size, dtype=np.float32)
    nm, ns, nd = _norm_args(cfg)
    _elib().orc_encode(nm, ns, nd, t[0], t[1], t[2], t.shape[1], out)
    return out.reshape(np.shape(truth))


def eval_score(cfg, x, truth, cx: float, cy: float) -> np.ndarray:
    """(corr, corr_h, amplitude_ratio, lag, bias) of model state x against the
    solver state `truth` (eval.rs:158-171)."""
    x = _f32(x).ravel()
    t = _f32(truth).reshape(3, -1)
    row = np.zeros(5, dtype=np.float32)
    nm, ns, nd = _norm_args(cfg)
    _elib().orc_eval_score(nm, ns, nd, int(cfg.nx), int(cfg.ny), x, t[0], t[1], t[2], cx, cy, row)
    return row


def eval_metrics(model: "OracleModel", drops, horizons, flags: int, meta):
    """The eval-metrics loop (crates/engine-cli/src/eval.rs:126-176) for the
    given drops (cx, cy, amp, sigma): returns rows [len(horizons), len(drops), 5]
    and the largest relative energy violation over all rollouts."""
    cfg = model.cfg
    p = sw_params(cfg)
    horizons = sorted(int(h) for h in horizons)
    last = horizons[-1]
    rows = np.zeros((len(horizons), len(drops), 5), dtype=np.float32)
    worst = 0.0
    for j, (cx, cy, amp, sigma) in enumerate(drops):
        truth = sw_flat(p)[0]
        sw_add_drop(p, truth[0], cx, cy, amp, sigma)
        x0 = encode(cfg, truth)
        _, _, viol, traj = model.rollout(x0, meta, last, flags, trajectory=True)
        worst = max(worst, viol)
        t_done = 0
        for i, hz in enumerate(horizons):
            sw_steps(p, truth, hz - t_done)
            t_done = hz
            rows[i, j] = eval_score(cfg, traj[hz], truth, cx, cy)
    return rows, worst


def rmse(a, b) -> float:
    a, b = _f32(a).ravel(), _f32(b).ravel()
    return _elib().orc_rmse(a, b, a.size)


def initial_state(cfg, drop) -> np.ndarray:
    """State::flat plus one drop, encoded: the start of an eval or round-trip
    trajectory (eval.rs:135-139)."""
    p = sw_params(cfg)
    truth = sw_flat(p)[0]
    sw_add_drop(p, truth[0], *drop)
    return encode(cfg, truth)


def roundtrip(forward: "OracleModel", reverse: "OracleModel", drops, horizons, flags: int, meta):
    """Forward N ticks, reverse N ticks, scored against the start: rows
    [len(horizons), len(drops), 4] of (corr, amplitude ratio, round-trip RMSE,
    N-tick change RMSE), with metrics.rs's correlation, peak, decode_h and
    rmse."""
    cfg = forward.cfg
    n = cfg.nx * cfg.ny
    horizons = sorted(int(h) for h in horizons)
    rows = np.zeros((len(horizons), len(drops), 4), dtype=np.float32)
    s0, m0 = np.float32(cfg.norm_std[0]), np.float32(cfg.norm_mean[0])
    for j, drop in enumerate(drops):
        x0 = initial_state(cfg, drop)
        _, _, _, traj = forward.rollout(x0, meta, horizons[-1], flags, trajectory=True)
        for i, hz in enumerate(horizons):
            xn = traj[hz]
            y, _, _ = reverse.rollout(xn, meta, hz, flags)
            rows[i, j] = (correlation(y, x0), peak(y.ravel()[:n] * s0 + m0) / peak(x0.ravel()[:n] * s0 + m0),
                          rmse(y, x0), rmse(xn, x0))
    return rows


def reconstruct(forward: "OracleModel", reverse: "OracleModel", vals, known, meta, sweeps: int, tol: float = 0.0):
    """The reconstruct rule on the f32 oracle (no reference counterpart; the
    library's JC_TASK_RECONSTRUCT): from X = known ? value : 0, each sweep
    sets X_t <- known_t ? value : mean of step_F(X_{t-1}) and step_R(X_{t+1})
    where they exist (one-sided at t = 0 and t = H), until the largest change
    of an unknown value is below tol or `sweeps` sweeps ran. Returns (X,
    sweeps run, last largest change)."""
    vals = np.asarray(vals, dtype=np.float32)
    known = np.asarray(known).astype(bool)
    H = vals.shape[0] - 1
    X = np.where(known[:, None], vals, np.float32(0.0)).astype(np.float32)
    resid, k = 0.0, 0
    for k in range(1, sweeps + 1):
        F = [forward.step(X[t - 1], meta) for t in range(1, H + 1)]
        R = [reverse.step(X[t + 1], meta) for t in range(0, H)]
        new = np.empty_like(X)
        for t in range(H + 1):
            if t == 0:
                v = R[0]
            elif t == H:
                v = F[H - 1]
            else:
                v = np.float32(0.5) * (F[t - 1] + R[t])
            new[t] = np.where(known[t][None], vals[t], v)
        unknown = ~np.broadcast_to(known[:, None], X.shape)
        resid = float(np.abs(new - X)[unknown].max()) if unknown.any() else 0.0
        X = new
        if resid < tol:
            break
    return X, k, resid


def identity_config(n: int, g: float = 9.81, r_max: float = 1.0):
    """A config with identity normalization over an n-cell strip, for the
    projection unit cases of crates/engine/src/project.rs:64-102."""
    from jacobi2000_gb300.checkpoint import ModelConfig

    return ModelConfig(nx=n, ny=1, patch=1, channels=3, dim=1, layers=0, heads=1, meta_dim=0, head_dim=1,
                       ff_inner=1, norm_mean=(0.0, 0.0, 0.0), norm_std=(1.0, 1.0, 1.0), norm_depth=0.0,
                       dx=1.0, dt=1.0, g=g, depth=1.0, nu=0.0, energy_r_max=r_max)


class _ProjOnly(OracleModel):
    def __init__(self, cfg):  # noqa: D401 - projection-only binding, no weights
        self.cfg = cfg
        c = _Config()
        c.nx, c.ny, c.channels = cfg.nx, cfg.ny, cfg.channels
        c.norm_mean[:] = list(cfg.norm_mean)
        c.norm_std[:] = list(cfg.norm_std)
        c.norm_depth, c.g, c.energy_r_max = cfg.norm_depth, cfg.g, cfg.energy_r_max
        self._c = c


def projection_only(cfg) -> OracleModel:
    return _ProjOnly(cfg)


if __name__ == "__main__":
    print(build())
    print("threads:", get_threads(), "cores:", os.cpu_count())
