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
    srcs = [HERE / "oracle.c", HERE / "oracle_impl.inc", HERE / "oracle.h"]
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
