"""Python binding of the C ABI (include/jacobi2000.h) through ctypes.

Mirrors the reference engine crate's model API (crates/engine/src/lib.rs:30-68,
gpu.rs:211-438): ``Model.load`` / ``Model.from_bytes``, ``forward``, ``step``,
plus the tick loop of crates/engine-cli/src/eval.rs:144-157 as ``rollout``
and the projections of crates/engine/src/project.rs as module functions.
Every call goes to the CUDA library; there is no CPU fallback. If the library
cannot be loaded, importing this module raises.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

PROJECT_MASS = 1
PROJECT_ENERGY = 2
FP32 = 0
BF16 = 1

STATUS = {0: "OK", 1: "NO_DEVICE", 2: "LIMIT", 3: "MAP", 4: "POLL", 5: "BAD_CHECKPOINT", 6: "BAD_SHAPE",
          7: "OVER_BUDGET", 8: "DEVICE_TIMEOUT", 9: "BAD_ARGUMENT", 10: "CUDA_ERROR", 11: "NOT_FOUND"}


class JcError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status
        self.name = STATUS.get(status, str(status))


class JcConfig(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("nx", "ny", "patch", "channels", "dim", "layers", "heads", "head_dim",
                                         "ff_inner", "meta_dim", "mask_kind", "mask_radius", "mask_dilation")] + [
        ("norm_mean", C.c_float * 3), ("norm_std", C.c_float * 3), ("norm_depth", C.c_float),
        ("dx", C.c_float), ("dt", C.c_float), ("g", C.c_float), ("depth", C.c_float), ("nu", C.c_float),
        ("energy_r_max", C.c_float)]


# Every symbol include/jacobi2000.h declares.
EXPORTED = ["jc_model_create", "jc_model_destroy", "jc_model_config", "jc_meta_of", "jc_forward", "jc_step",
            "jc_rollout", "jc_forward_device", "jc_rollout_device", "jc_mass", "jc_energy", "jc_project_mass",
            "jc_project_energy", "jc_last_error", "jc_version", "jc_autotune"]

_lib = None


def load_library(path: str | Path | None = None):
    """Loads (building first if needed) libjacobi2000.so and declares its
    signatures."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else _build.build()
    L = C.CDLL(str(p))
    F = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    D = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    vp = C.c_void_p
    L.jc_model_create.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_int32, C.POINTER(vp)]
    L.jc_model_destroy.argtypes = [vp]
    L.jc_model_destroy.restype = None
    L.jc_model_config.argtypes = [vp, C.POINTER(JcConfig)]
    L.jc_meta_of.argtypes = [vp, F]
    L.jc_forward.argtypes = [vp, F, F, F]
    L.jc_step.argtypes = [vp, F, F, F]
    L.jc_rollout.argtypes = [vp, F, F, C.c_int32, C.c_uint32, F, vp, vp]
    L.jc_forward_device.argtypes = [vp, vp, vp, vp, vp]
    L.jc_rollout_device.argtypes = [vp, vp, vp, C.c_int32, C.c_uint32, vp, vp, vp]
    L.jc_mass.argtypes = [F, C.c_int64]
    L.jc_mass.restype = C.c_double
    L.jc_energy.argtypes = [F, C.POINTER(JcConfig), C.c_int64]
    L.jc_energy.restype = C.c_double
    L.jc_project_mass.argtypes = [F, C.c_double, C.c_int64]
    L.jc_project_mass.restype = None
    L.jc_project_energy.argtypes = [F, C.c_double, C.POINTER(JcConfig), C.c_int64]
    L.jc_project_energy.restype = None
    L.jc_last_error.restype = C.c_char_p
    L.jc_version.restype = C.c_char_p
    for name in EXPORTED:
        if name.startswith("jc_") and not name.endswith("_destroy") and name not in (
                "jc_mass", "jc_energy", "jc_project_mass", "jc_project_energy", "jc_last_error", "jc_version"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _check(status: int) -> None:
    if status != 0:
        raise JcError(status, load_library().jc_last_error().decode())


class Model:
    """A checkpoint on the GPU (engine::Model + GpuModel in one)."""

    def __init__(self, safetensors: bytes, config_json: str, precision: int = FP32):
        L = load_library()
        h = C.c_void_p()
        _check(L.jc_model_create(safetensors, len(safetensors), config_json.encode(), int(precision), C.byref(h)))
        self._h = h
        self._L = L
        c = JcConfig()
        _check(L.jc_model_config(h, C.byref(c)))
        self.config = c
        self.precision = precision
        self.shape = (c.channels, c.ny, c.nx)
        self.cells = c.nx * c.ny

    @classmethod
    def load(cls, directory: str | Path, precision: int = FP32) -> "Model":
        """engine::Model::load (lib.rs:36-40): model.safetensors + config.json."""
        d = Path(directory)
        return cls((d / "model.safetensors").read_bytes(), (d / "config.json").read_text(), precision)

    @classmethod
    def from_bytes(cls, safetensors: bytes, config_json: str, precision: int = FP32) -> "Model":
        return cls(safetensors, config_json, precision)

    @classmethod
    def from_packed(cls, packed: bytes) -> "Model":
        """A model from a pre-packed checkpoint (jc_model_create_packed)."""
        L = load_library()
        _declare_pack(L)
        self = cls.__new__(cls)
        h = C.c_void_p()
        _check(L.jc_model_create_packed(packed, len(packed), C.byref(h)))
        self._h = h
        self._L = L
        c = JcConfig()
        _check(L.jc_model_config(h, C.byref(c)))
        self.config = c
        self.precision = packed_precision(packed)
        self.shape = (c.channels, c.ny, c.nx)
        self.cells = c.nx * c.ny
        return self

    def pack(self) -> bytes:
        """The pre-packed checkpoint of this model (jc_model_pack)."""
        _declare_pack(self._L)
        n = C.c_size_t()
        _check(self._L.jc_model_pack(self._h, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        _check(self._L.jc_model_pack(self._h, buf, n.value, C.byref(n)))
        return buf.raw[:n.value]

    @classmethod
    def load_cached(cls, directory: str | Path, precision: int = FP32) -> "Model":
        """Model.load through the pre-packed cache beside the checkpoint:
        ``model.fp32.jcpack`` / ``model.bf16.jcpack`` is used when it records
        the current model.safetensors and config.json, else rebuilt from them."""
        d = Path(directory)
        st = (d / "model.safetensors").read_bytes()
        cj = (d / "config.json").read_text()
        cache = d / f"model.{'bf16' if precision == BF16 else 'fp32'}.jcpack"
        if cache.exists():
            packed = cache.read_bytes()
            try:
                if packed_source_hash(packed) == source_hash(st, cj) and packed_precision(packed) == precision:
                    return cls.from_packed(packed)
            except JcError:
                pass
        m = cls(st, cj, precision)
        tmp = cache.with_suffix(".tmp")
        tmp.write_bytes(m.pack())
        tmp.replace(cache)
        return m

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.jc_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _state(self, x) -> np.ndarray:
        a = np.ascontiguousarray(x, dtype=np.float32)
        if a.size != int(np.prod(self.shape)):
            raise JcError(6, f"state has {a.size} elements, expected {int(np.prod(self.shape))}")
        return a.reshape(self.shape)

    def _meta(self, m) -> np.ndarray:
        a = np.ascontiguousarray(m, dtype=np.float32).ravel()
        if a.size != self.config.meta_dim:
            raise JcError(6, f"meta has {a.size} elements, expected {self.config.meta_dim}")
        return a

    def meta_of(self) -> np.ndarray:
        out = np.zeros(self.config.meta_dim, dtype=np.float32)
        _check(self._L.jc_meta_of(self._h, out))
        return out

    def forward(self, state, meta) -> np.ndarray:
        """The predicted increment (cpu.rs:249-352)."""
        out = np.empty(self.shape, dtype=np.float32)
        _check(self._L.jc_forward(self._h, self._state(state), self._meta(meta), out))
        return out

    def step(self, state, meta) -> np.ndarray:
        """state + forward(state, meta) (cpu.rs:84-88)."""
        out = np.empty(self.shape, dtype=np.float32)
        _check(self._L.jc_step(self._h, self._state(state), self._meta(meta), out))
        return out

    def rollout(self, x0, meta, ticks: int, flags: int = PROJECT_MASS | PROJECT_ENERGY, trajectory: bool = False):
        """``ticks`` ticks of step + projections. Returns (final, energies[,
        trajectory])."""
        final = np.empty(self.shape, dtype=np.float32)
        energies = np.empty(ticks + 1, dtype=np.float64)
        traj = np.empty((ticks + 1,) + self.shape, dtype=np.float32) if trajectory else None
        _check(self._L.jc_rollout(self._h, self._state(x0), self._meta(meta), int(ticks), int(flags), final,
                                  traj.ctypes.data if traj is not None else None, energies.ctypes.data))
        return (final, energies, traj) if trajectory else (final, energies)


def mass(x, cells: int) -> float:
    return load_library().jc_mass(np.ascontiguousarray(x, dtype=np.float32).ravel(), int(cells))


def energy(x, config: JcConfig, cells: int) -> float:
    return load_library().jc_energy(np.ascontiguousarray(x, dtype=np.float32).ravel(), C.byref(config), int(cells))


def project_mass(x, target: float, cells: int) -> np.ndarray:
    y = np.array(x, dtype=np.float32, copy=True)
    load_library().jc_project_mass(y.reshape(-1), float(target), int(cells))
    return y


def project_energy(x, prev_energy: float, config: JcConfig, cells: int) -> np.ndarray:
    y = np.array(x, dtype=np.float32, copy=True)
    load_library().jc_project_energy(y.reshape(-1), float(prev_energy), C.byref(config), int(cells))
    return y


def autotune(enable: bool | None = None) -> bool:
    """Turns the BF16 schedule autotuner on or off (None: query only);
    returns the previous setting."""
    L = load_library()
    L.jc_autotune.argtypes = [C.c_int32]
    return bool(L.jc_autotune(-1 if enable is None else int(bool(enable))))


class JcInstance(C.Structure):
    _fields_ = [("model", C.c_int32), ("ticks", C.c_int32), ("flags", C.c_uint32), ("task", C.c_int32),
                ("x0", C.c_void_p), ("meta", C.c_void_p), ("final_state", C.c_void_p), ("energy", C.c_void_p),
                ("known", C.c_void_p), ("reverse_model", C.c_int32), ("max_sweeps", C.c_int32), ("tol", C.c_float),
                ("reserved", C.c_int32)]


def _declare_batch(L):
    if getattr(L, "_batch_declared", False):
        return
    vp = C.c_void_p
    L.jc_batch_create.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.c_int64, C.POINTER(vp)]
    L.jc_batch_create.restype = C.c_int
    L.jc_batch_destroy.argtypes = [vp]
    L.jc_batch_destroy.restype = None
    L.jc_batch_rollout.argtypes = [vp, C.POINTER(JcInstance), C.c_int32, C.c_int32, vp]
    L.jc_batch_rollout.restype = C.c_int
    L.jc_batch_profile.argtypes = [vp, C.POINTER(JcInstance), C.c_int32, C.c_int32, C.c_char_p, C.c_size_t]
    L.jc_batch_profile.restype = C.c_int
    L._batch_declared = True


EXPORTED += ["jc_batch_create", "jc_batch_destroy", "jc_batch_rollout", "jc_batch_profile",
             "jc_forward_device_noalloc", "jc_selftest_device_wait"]


class Batch:
    """Many rollouts stepped together (jc_batch_*). ``models`` share every
    hyper-parameter; instances are (model index, x0, meta, ticks, flags)."""

    def __init__(self, models, max_instances: int, max_cells: int):
        L = load_library()
        _declare_batch(L)
        self._L = L
        self.models = list(models)
        arr = (C.c_void_p * len(self.models))(*[m._h.value for m in self.models])
        h = C.c_void_p()
        _check(L.jc_batch_create(arr, len(self.models), int(max_instances), int(max_cells), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.jc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _instances(self, items, device: bool):
        """Items are tuples (model, x0, meta, ticks[, flags[, final_device_ptr]])
        for rollouts, or dicts with task=2 (reconstruct): model,
        reverse_model, x (values [H+1,3,ny,nx]), known ([H+1,ny,nx]), meta,
        ticks, max_sweeps, tol."""
        n = len(items)
        arr = (JcInstance * n)()
        keep = []
        outs = []
        for k, it in enumerate(items):
            e = np.zeros(2, dtype=np.float64)
            keep.append(e)
            if isinstance(it, dict):
                m = self.models[it["model"]]
                c = m.config
                H = int(it["ticks"])
                xa = np.ascontiguousarray(it["x"], dtype=np.float32).reshape(H + 1, 3, c.ny, c.nx)
                ka = np.ascontiguousarray(it["known"], dtype=np.uint8).reshape(H + 1, c.ny, c.nx)
                ma = m._meta(it["meta"])
                out = np.empty_like(xa)
                keep += [xa, ka, ma]
                arr[k] = JcInstance(int(it["model"]), H, 0, TASK_RECONSTRUCT, xa.ctypes.data, ma.ctypes.data,
                                    out.ctypes.data, e.ctypes.data, ka.ctypes.data, int(it["reverse_model"]),
                                    int(it.get("max_sweeps", 4)), float(it.get("tol", 1e-3)), 0)
                outs.append((out, e))
                continue
            mi, x0, meta, ticks = it[0], it[1], it[2], it[3]
            flags = it[4] if len(it) > 4 else PROJECT_MASS | PROJECT_ENERGY
            m = self.models[mi]
            if device:
                # (x0, meta, final) are device pointers (ints)
                x0p, metap, outp = int(x0), int(meta), int(it[5])
                out = None
            else:
                xa = m._state(x0)
                ma = m._meta(meta)
                out = np.empty(m.shape, dtype=np.float32)
                keep += [xa, ma]
                x0p, metap, outp = xa.ctypes.data, ma.ctypes.data, out.ctypes.data
            arr[k] = JcInstance(int(mi), int(ticks), int(flags), 0, x0p, metap, outp, e.ctypes.data, None, 0, 0, 0.0, 0)
            outs.append((out, e))
        return arr, keep, outs

    def rollout(self, items, device: bool = False, stream: int | None = None):
        """Returns [(final_state, final_energy, max_violation)] in input order
        (final_state is None with device pointers); for reconstruct items
        [(volume, sweeps, last_residual)]."""
        arr, keep, outs = self._instances(items, device)
        _check(self._L.jc_batch_rollout(self._h, arr, len(items), int(device), stream))
        return [(o, float(e[0]), float(e[1])) for o, e in outs]

    def profile(self, items, device: bool = False) -> dict:
        """{kernel name: (launches, total device ms)} for one run of ``items``."""
        arr, keep, outs = self._instances(items, device)
        buf = C.create_string_buffer(1 << 16)
        _check(self._L.jc_batch_profile(self._h, arr, len(items), int(device), buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms = line.split(",")
            out[name] = (int(n), float(ms))
        return out


TASK_FORWARD, TASK_REWIND, TASK_RECONSTRUCT = 0, 1, 2


class JcRequest(C.Structure):
    _fields_ = [("task", C.c_int32), ("grid", C.c_int32), ("ticks", C.c_int32), ("flags", C.c_uint32),
                ("x", C.c_void_p), ("known", C.c_void_p), ("meta", C.c_void_p), ("max_sweeps", C.c_int32),
                ("tol", C.c_float)]


class JcResult(C.Structure):
    _fields_ = [("latency_s", C.c_double), ("queue_s", C.c_double), ("sweeps", C.c_int32), ("residual", C.c_float),
                ("energy", C.c_double), ("max_violation", C.c_double), ("out_len", C.c_int64)]


class JcServerStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("cell_ticks", C.c_double), ("busy_s", C.c_double), ("span_s", C.c_double),
                ("iterations", C.c_int32), ("active", C.c_int32), ("pending", C.c_int32),
                ("device_span_s", C.c_double), ("launches", C.c_int64)]


REQUEST_DEVICE_BUFFERS = 0x100

EXPORTED += ["jc_server_create", "jc_server_destroy", "jc_server_submit", "jc_server_wait", "jc_server_get_stats",
             "jc_server_reset_stats", "jc_server_profile"]


def _declare_server(L):
    if getattr(L, "_server_declared", False):
        return
    vp = C.c_void_p
    L.jc_server_create.argtypes = [C.POINTER(vp), C.POINTER(vp), C.c_int32, C.c_int64, C.c_double, C.POINTER(vp)]
    L.jc_server_create.restype = C.c_int
    L.jc_server_destroy.argtypes = [vp]
    L.jc_server_destroy.restype = None
    L.jc_server_submit.argtypes = [vp, C.POINTER(JcRequest), C.POINTER(C.c_uint64)]
    L.jc_server_submit.restype = C.c_int
    L.jc_server_wait.argtypes = [vp, C.c_uint64, vp, C.c_size_t, C.POINTER(JcResult), C.c_double]
    L.jc_server_wait.restype = C.c_int
    L.jc_server_get_stats.argtypes = [vp, C.POINTER(JcServerStats)]
    L.jc_server_get_stats.restype = C.c_int
    L.jc_server_reset_stats.argtypes = [vp]
    L.jc_server_reset_stats.restype = C.c_int
    L.jc_server_profile.argtypes = [vp, C.c_int32, C.c_char_p, C.c_size_t]
    L.jc_server_profile.restype = C.c_int
    L._server_declared = True


class Server:
    """Continuous-batching request loop (jc_server_*). ``forward_models[i]``
    and ``reverse_models[i]`` hold grid i."""

    def __init__(self, forward_models, reverse_models=None, max_active_cells: int = 1 << 22,
                 hbm_fraction: float = 0.8):
        L = load_library()
        _declare_server(L)
        self._L = L
        self.forward_models = list(forward_models)
        self.reverse_models = list(reverse_models) if reverse_models else None
        n = len(self.forward_models)
        fa = (C.c_void_p * n)(*[m._h.value for m in self.forward_models])
        ra = (C.c_void_p * n)(*[m._h.value for m in self.reverse_models]) if self.reverse_models else None
        h = C.c_void_p()
        _check(L.jc_server_create(fa, ra, n, int(max_active_cells), float(hbm_fraction), C.byref(h)))
        self._h = h
        self._keep = {}

    def close(self):
        if getattr(self, "_h", None):
            self._L.jc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _submit(self, req: JcRequest) -> int:
        i = C.c_uint64()
        _check(self._L.jc_server_submit(self._h, C.byref(req), C.byref(i)))
        return int(i.value)

    def submit(self, task: int, grid: int, x, meta, ticks: int, flags: int = PROJECT_MASS | PROJECT_ENERGY,
               known=None, max_sweeps: int = 4, tol: float = 1e-3) -> int:
        xa = np.ascontiguousarray(x, dtype=np.float32)
        ma = np.ascontiguousarray(meta, dtype=np.float32)
        ka = np.ascontiguousarray(known, dtype=np.uint8) if known is not None else None
        req = JcRequest(int(task), int(grid), int(ticks), int(flags), xa.ctypes.data,
                        ka.ctypes.data if ka is not None else None, ma.ctypes.data, int(max_sweeps), float(tol))
        return self._submit(req)  # inputs are copied by the call

    def submit_device(self, task: int, grid: int, x_ptr: int, meta_ptr: int, ticks: int,
                      flags: int = PROJECT_MASS | PROJECT_ENERGY, known_ptr: int | None = None, max_sweeps: int = 4,
                      tol: float = 1e-3) -> int:
        """submit() with caller-owned inputs: device pointers, or page-locked
        host pointers (copied by DMA), that must stay valid until the request
        is done; collect with wait_device()."""
        req = JcRequest(int(task), int(grid), int(ticks), int(flags) | REQUEST_DEVICE_BUFFERS, int(x_ptr),
                        int(known_ptr) if known_ptr else None, int(meta_ptr), int(max_sweeps), float(tol))
        return self._submit(req)

    def wait_device(self, rid: int, out_ptr: int | None, out_len: int, timeout: float = -1.0) -> dict:
        """Waits for a request submitted with submit_device and copies its
        result to `out_ptr`, a device or page-locked host pointer (out_len
        floats; None: drop it)."""
        info = JcResult()
        _check(self._L.jc_server_wait(self._h, int(rid), int(out_ptr) if out_ptr else None, int(out_len),
                                      C.byref(info), float(timeout)))
        return {f: getattr(info, f) for f, _ in JcResult._fields_}

    def reset_stats(self) -> None:
        _check(self._L.jc_server_reset_stats(self._h))

    def profile_start(self) -> None:
        """Per-kernel timing of the loop's launches from now on (jc_server_profile)."""
        _check(self._L.jc_server_profile(self._h, 1, None, 0))

    def profile_stop(self) -> dict:
        """{kernel name: (launches, total device ms)} since profile_start()."""
        buf = C.create_string_buffer(1 << 16)
        _check(self._L.jc_server_profile(self._h, 0, buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms = line.split(",")
            out[name] = (int(n), float(ms))
        return out

    def out_shape(self, task: int, grid: int, ticks: int):
        c = self.forward_models[grid].config
        return ((ticks + 1, 3, c.ny, c.nx) if task == TASK_RECONSTRUCT else (3, c.ny, c.nx))

    def wait(self, rid: int, task: int, grid: int, ticks: int, timeout: float = -1.0):
        out = np.empty(self.out_shape(task, grid, ticks), dtype=np.float32)
        info = JcResult()
        _check(self._L.jc_server_wait(self._h, int(rid), out.ctypes.data, out.size, C.byref(info), float(timeout)))
        return out, {f: getattr(info, f) for f, _ in JcResult._fields_}

    def stats(self) -> dict:
        st = JcServerStats()
        _check(self._L.jc_server_get_stats(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in JcServerStats._fields_}


# ---- evaluation on the device (jc_sw_*, jc_eval_*) -------------------------------

class JcSwParams(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32)] + [(n, C.c_float) for n in ("dx", "dt", "g", "depth", "nu")]


class JcDrop(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("cx", "cy", "amp", "sigma")]


class JcEvalRow(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("corr", "corr_h", "amplitude_ratio", "lag", "bias")]


EVAL_FIELDS = [f for f, _ in JcEvalRow._fields_]
EXPORTED += ["jc_sw_run", "jc_sw_run_device", "jc_sw_add_drop", "jc_eval_score", "jc_eval_create", "jc_eval_destroy",
             "jc_eval_run"]


def _declare_eval(L):
    if getattr(L, "_eval_declared", False):
        return
    vp = C.c_void_p
    F = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    swp = C.POINTER(JcSwParams)
    L.jc_sw_run.argtypes = [swp, F, C.c_int32, C.c_int32]
    L.jc_sw_run_device.argtypes = [swp, vp, C.c_int32, C.c_int32, vp]
    L.jc_sw_add_drop.argtypes = [swp, F, C.c_float, C.c_float, C.c_float, C.c_float]
    L.jc_eval_score.argtypes = [C.POINTER(JcConfig), F, F, F, C.c_int32, C.POINTER(JcEvalRow)]
    L.jc_eval_create.argtypes = [vp, C.c_int32, C.POINTER(vp)]
    L.jc_eval_destroy.argtypes = [vp]
    L.jc_eval_destroy.restype = None
    L.jc_eval_run.argtypes = [vp, C.POINTER(JcDrop), C.c_int32, C.POINTER(C.c_int32), C.c_int32, C.c_uint32,
                              C.POINTER(JcEvalRow), C.POINTER(C.c_double)]
    for fn in ("jc_sw_run", "jc_sw_run_device", "jc_sw_add_drop", "jc_eval_score", "jc_eval_create", "jc_eval_run"):
        getattr(L, fn).restype = C.c_int
    L._eval_declared = True


def sw_params(config: JcConfig) -> JcSwParams:
    """solvers::Params of a model's config (crates/engine/src/config.rs:102-104)."""
    return JcSwParams(config.nx, config.ny, config.dx, config.dt, config.g, config.depth, config.nu)


def sw_flat(p: JcSwParams, count: int = 1) -> np.ndarray:
    """State::flat for `count` solver states: [count, 3, ny, nx], h = depth."""
    s = np.zeros((count, 3, p.ny, p.nx), dtype=np.float32)
    s[:, 0] = np.float32(p.depth)
    return s


def sw_add_drop(p: JcSwParams, h: np.ndarray, cx: float, cy: float, amp: float, sigma: float) -> None:
    """State::add_drop in place on an h plane [ny, nx] (float32, contiguous)."""
    L = load_library()
    _declare_eval(L)
    if h.dtype != np.float32 or not h.flags.c_contiguous or h.size != p.nx * p.ny:
        raise ValueError("h must be a contiguous float32 [ny, nx] plane")
    _check(L.jc_sw_add_drop(C.byref(p), h.reshape(-1), cx, cy, amp, sigma))


def sw_run(p: JcSwParams, states: np.ndarray, steps: int) -> np.ndarray:
    """`steps` reference solver ticks of every state ([count, 3, ny, nx] or
    [3, ny, nx]) on the GPU; returns the advanced states."""
    L = load_library()
    _declare_eval(L)
    s = np.array(states, dtype=np.float32, copy=True, order="C")
    count = s.size // (3 * p.nx * p.ny)
    if count * 3 * p.nx * p.ny != s.size:
        raise ValueError("states must be [count, 3, ny, nx]")
    _check(L.jc_sw_run(C.byref(p), s.reshape(-1), count, int(steps)))
    return s


def eval_score(config: JcConfig, x, truth, centres) -> np.ndarray:
    """Scores model states x [count, 3, ny, nx] (normalized) against solver
    states [count, 3, ny, nx] about centres [count, 2]; returns a structured
    array with the fields of EVAL_FIELDS."""
    L = load_library()
    _declare_eval(L)
    n = config.nx * config.ny
    xa = np.ascontiguousarray(x, dtype=np.float32).reshape(-1)
    ta = np.ascontiguousarray(truth, dtype=np.float32).reshape(-1)
    ca = np.ascontiguousarray(centres, dtype=np.float32).reshape(-1)
    count = xa.size // (3 * n)
    if xa.size != count * 3 * n or ta.size != xa.size or ca.size != 2 * count:
        raise ValueError("shape mismatch")
    rows = (JcEvalRow * max(count, 1))()
    _check(L.jc_eval_score(C.byref(config), xa, ta, ca, count, rows))
    return _rows_array(rows, count)


def _rows_array(rows, count: int) -> np.ndarray:
    out = np.zeros(count, dtype=[(f, np.float32) for f in EVAL_FIELDS])
    for k in range(count):
        for f in EVAL_FIELDS:
            out[f][k] = getattr(rows[k], f)
    return out


class Evaluator:
    """eval-metrics on the device for one model (jc_eval_*): the reference
    solver and the model advance side by side and every trajectory is scored
    at each horizon."""

    def __init__(self, model: Model, max_trajectories: int):
        L = load_library()
        _declare_eval(L)
        self._L = L
        self.model = model
        self.max_trajectories = int(max_trajectories)
        h = C.c_void_p()
        _check(L.jc_eval_create(model._h, self.max_trajectories, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.jc_eval_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, drops, horizons, flags: int = PROJECT_MASS):
        """drops: [(cx, cy, amp, sigma)]. Returns (rows [len(horizons),
        len(drops)] structured by EVAL_FIELDS, max relative energy violation)."""
        n, nh = len(drops), len(horizons)
        d = (JcDrop * max(n, 1))(*[JcDrop(*map(float, dr)) for dr in drops])
        hz = (C.c_int32 * max(nh, 1))(*[int(h) for h in horizons])
        rows = (JcEvalRow * max(n * nh, 1))()
        viol = C.c_double(0.0)
        _check(self._L.jc_eval_run(self._h, d, n, hz, nh, int(flags), rows, C.byref(viol)))
        return _rows_array(rows, n * nh).reshape(nh, n), float(viol.value)


# ---- rewind round trip (jc_roundtrip_*) --------------------------------------------

class JcRoundTripRow(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("corr", "amplitude_ratio", "rmse", "change_rmse")]


ROUNDTRIP_FIELDS = [f for f, _ in JcRoundTripRow._fields_]
EXPORTED += ["jc_roundtrip_create", "jc_roundtrip_destroy", "jc_roundtrip_run"]


def _declare_roundtrip(L):
    if getattr(L, "_rt_declared", False):
        return
    _declare_eval(L)
    vp = C.c_void_p
    L.jc_roundtrip_create.argtypes = [vp, vp, C.c_int32, C.c_int32, C.POINTER(vp)]
    L.jc_roundtrip_create.restype = C.c_int
    L.jc_roundtrip_destroy.argtypes = [vp]
    L.jc_roundtrip_destroy.restype = None
    L.jc_roundtrip_run.argtypes = [vp, C.POINTER(JcDrop), C.c_int32, C.POINTER(C.c_int32), C.c_int32, C.c_uint32,
                                   C.POINTER(JcRoundTripRow)]
    L.jc_roundtrip_run.restype = C.c_int
    L._rt_declared = True


class RoundTrip:
    """Forward N ticks with `forward`, back N ticks with `reverse`, scored
    against the start (jc_roundtrip_*)."""

    def __init__(self, forward: Model, reverse: Model, max_trajectories: int, max_horizons: int = 4):
        L = load_library()
        _declare_roundtrip(L)
        self._L = L
        self.forward, self.reverse = forward, reverse
        h = C.c_void_p()
        _check(L.jc_roundtrip_create(forward._h, reverse._h, int(max_trajectories), int(max_horizons), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.jc_roundtrip_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, drops, horizons, flags: int = PROJECT_MASS) -> np.ndarray:
        """drops: [(cx, cy, amp, sigma)]; returns rows [len(horizons),
        len(drops)] structured by ROUNDTRIP_FIELDS."""
        n, nh = len(drops), len(horizons)
        d = (JcDrop * max(n, 1))(*[JcDrop(*map(float, dr)) for dr in drops])
        hz = (C.c_int32 * max(nh, 1))(*[int(h) for h in horizons])
        rows = (JcRoundTripRow * max(n * nh, 1))()
        _check(self._L.jc_roundtrip_run(self._h, d, n, hz, nh, int(flags), rows))
        out = np.zeros(n * nh, dtype=[(f, np.float32) for f in ROUNDTRIP_FIELDS])
        for k in range(n * nh):
            for f in ROUNDTRIP_FIELDS:
                out[f][k] = getattr(rows[k], f)
        return out.reshape(nh, n)


# ---- pre-packed checkpoints (jc_model_pack, jc_model_create_packed) ----------------

EXPORTED += ["jc_model_pack", "jc_model_create_packed", "jc_source_hash", "jc_packed_source_hash"]


def _declare_pack(L):
    if getattr(L, "_pack_declared", False):
        return
    vp = C.c_void_p
    L.jc_model_pack.argtypes = [vp, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]
    L.jc_model_pack.restype = C.c_int
    L.jc_model_create_packed.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(vp)]
    L.jc_model_create_packed.restype = C.c_int
    L.jc_source_hash.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.POINTER(C.c_uint64)]
    L.jc_source_hash.restype = C.c_int
    L.jc_packed_source_hash.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_uint64)]
    L.jc_packed_source_hash.restype = C.c_int
    L._pack_declared = True


def source_hash(safetensors: bytes, config_json: str) -> int:
    L = load_library()
    _declare_pack(L)
    out = C.c_uint64()
    _check(L.jc_source_hash(safetensors, len(safetensors), config_json.encode(), C.byref(out)))
    return out.value


def packed_source_hash(packed: bytes) -> int:
    L = load_library()
    _declare_pack(L)
    out = C.c_uint64()
    _check(L.jc_packed_source_hash(packed, len(packed), C.byref(out)))
    return out.value


def packed_precision(packed: bytes) -> int:
    """The precision field of a pre-packed checkpoint's header (after the
    8-byte magic and the u32 version)."""
    packed_source_hash(packed)  # validates the header
    return int.from_bytes(packed[12:16], "little")


# ---- solver trajectories (jc_sw_trajectories) ---------------------------------------

class JcSwTrajectory(C.Structure):
    _fields_ = [("ticks", C.c_int32), ("x0", C.c_void_p), ("n_drops", C.c_int32), ("drop_ticks", C.c_void_p),
                ("drop_fields", C.c_void_p), ("frames", C.c_void_p)]


EXPORTED += ["jc_sw_trajectories"]


def sw_trajectories(p: JcSwParams, trajectories):
    """trajectories: [(x0 [3, ny, nx], ticks, [(tick, field [ny, nx]), ...])].
    Returns frames [3, ticks + 1, ny, nx] per trajectory (the traj-NNNNN.f32
    layout), all computed in one device batch."""
    L = load_library()
    _declare_eval(L)
    if not getattr(L, "_traj_declared", False):
        L.jc_sw_trajectories.argtypes = [C.POINTER(JcSwParams), C.POINTER(JcSwTrajectory), C.c_int32]
        L.jc_sw_trajectories.restype = C.c_int
        L._traj_declared = True
    n = len(trajectories)
    arr = (JcSwTrajectory * max(n, 1))()
    keep, outs = [], []
    for k, (x0, ticks, drops) in enumerate(trajectories):
        xa = np.ascontiguousarray(x0, dtype=np.float32).reshape(3, p.ny, p.nx)
        dt = np.ascontiguousarray([int(t) for t, _ in drops], dtype=np.int32)
        df = np.ascontiguousarray(np.stack([np.asarray(f, np.float32).reshape(p.ny, p.nx) for _, f in drops])
                                  if drops else np.zeros((1, p.ny, p.nx), np.float32))
        fr = np.empty((3, int(ticks) + 1, p.ny, p.nx), dtype=np.float32)
        keep += [xa, dt, df]
        outs.append(fr)
        arr[k] = JcSwTrajectory(int(ticks), xa.ctypes.data, len(drops), dt.ctypes.data if len(drops) else None,
                                df.ctypes.data if len(drops) else None, fr.ctypes.data)
    _check(L.jc_sw_trajectories(C.byref(p), arr, n))
    return outs
