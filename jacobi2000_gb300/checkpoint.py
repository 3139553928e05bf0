"""Checkpoint format: ``model.safetensors`` + ``config.json``.

The format is the reference's weight exchange format (docs/pytorch-training.md:25-47,
written by training/jacobi2000_pt/export.py:22-70, read by
crates/engine/src/weights.rs:29-48 and crates/engine/src/config.rs:70-100):

* safetensors: an 8-byte little-endian header length, a JSON header
  ``{name: {dtype, shape, data_offsets}}``, then the raw little-endian payload.
  Only ``F32`` tensors are accepted (weights.rs:39).
* config.json: ``nx, ny, patch, channels, dim, layers, heads, meta_dim, norm
  {mean[3], std[3], depth}, dx, dt, g, depth, nu`` are required;
  ``energy_r_max`` defaults to 1.0 and ``mask`` to ``"Full"`` (config.rs:29-41).
  ``head_dim`` and ``ff_inner`` come from tensor shapes (config.rs:72-73).

This module also builds synthetic seeded checkpoint *families*: every tensor
except ``pos`` is shared across grid sides, ``pos`` is seeded per side, since
``pos`` is the only tensor whose shape depends on the grid.
"""

from __future__ import annotations

import hashlib
import json
import math
import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

__all__ = [
    "read_safetensors_bytes",
    "read_safetensors",
    "write_safetensors_bytes",
    "write_safetensors",
    "ModelConfig",
    "parse_config",
    "synthetic_family",
    "synthetic_checkpoint",
    "meta_of",
    "tensor_names",
    "checksum",
]


def read_safetensors_bytes(buf: bytes) -> dict[str, np.ndarray]:
    """weights.rs:29-48: header length, JSON header, F32 payload."""
    if len(buf) < 8:
        raise ValueError("safetensors: truncated header length")
    (hlen,) = struct.unpack("<Q", buf[:8])
    if 8 + hlen > len(buf):
        raise ValueError("safetensors: header runs past the end of the file")
    header = json.loads(buf[8 : 8 + hlen])
    start = 8 + hlen
    out: dict[str, np.ndarray] = {}
    for name, v in header.items():
        if name == "__metadata__":
            continue
        if v["dtype"] != "F32":
            raise ValueError(f"tensor `{name}`: only F32 is supported")
        a, b = v["data_offsets"]
        shape = tuple(int(s) for s in v["shape"])
        if b - a != 4 * int(np.prod(shape, dtype=np.int64)) or start + b > len(buf):
            raise ValueError(f"tensor `{name}`: data_offsets do not match its shape")
        out[name] = np.frombuffer(buf, dtype="<f4", count=(b - a) // 4, offset=start + a).reshape(shape).astype(np.float32)
    return out


def read_safetensors(path: str | Path) -> dict[str, np.ndarray]:
    return read_safetensors_bytes(Path(path).read_bytes())


def write_safetensors_bytes(tensors: dict[str, np.ndarray]) -> bytes:
    header = {}
    off = 0
    blobs = []
    for name in sorted(tensors):
        a = np.ascontiguousarray(tensors[name], dtype="<f4")
        header[name] = {"dtype": "F32", "shape": list(a.shape), "data_offsets": [off, off + a.nbytes]}
        blobs.append(a.tobytes())
        off += a.nbytes
    hb = json.dumps(header, separators=(",", ":")).encode()
    hb += b" " * ((8 - len(hb) % 8) % 8)
    return struct.pack("<Q", len(hb)) + hb + b"".join(blobs)


def write_safetensors(path: str | Path, tensors: dict[str, np.ndarray]) -> None:
    Path(path).write_bytes(write_safetensors_bytes(tensors))


@dataclass
class ModelConfig:
    """config.rs:43-67, with the mask flattened to (kind, radius, dilation)."""

    nx: int
    ny: int
    patch: int
    channels: int
    dim: int
    layers: int
    heads: int
    meta_dim: int
    head_dim: int
    ff_inner: int
    norm_mean: tuple
    norm_std: tuple
    norm_depth: float
    dx: float
    dt: float
    g: float
    depth: float
    nu: float
    energy_r_max: float = 1.0
    mask_kind: int = 0  # 0 Full, 1 Stencil
    radius: int = 0
    dilation: int = 1
    raw: dict = field(default_factory=dict, repr=False)

    @property
    def tokens_x(self) -> int:
        return self.nx // self.patch

    @property
    def tokens_y(self) -> int:
        return self.ny // self.patch

    @property
    def tokens(self) -> int:
        return self.tokens_x * self.tokens_y

    @property
    def cells(self) -> int:
        return self.nx * self.ny


_REQUIRED = ("nx", "ny", "patch", "channels", "dim", "layers", "heads", "meta_dim", "norm", "dx", "dt", "g", "depth", "nu")


def parse_config(config_json: str | dict, tensors: dict[str, np.ndarray]) -> ModelConfig:
    """config.rs:70-100: required fields, defaults, shapes inferred from tensors."""
    raw = json.loads(config_json) if isinstance(config_json, str) else dict(config_json)
    for k in _REQUIRED:
        if k not in raw:
            raise ValueError(f"config.json: missing field `{k}`")
    mask = raw.get("mask", "Full")
    if mask == "Full":
        mk, r, d = 0, 0, 1
    elif isinstance(mask, dict) and "Stencil" in mask:
        mk, r, d = 1, int(mask["Stencil"]["radius"]), int(mask["Stencil"]["dilation"])
    else:
        raise ValueError(f"config.json: unrecognized mask {mask!r}")
    for name in ("head.to_cells.weight", "blocks.0.ff1.weight"):
        if name not in tensors:
            raise ValueError(f"missing tensor `{name}`")
    n = raw["norm"]
    return ModelConfig(
        nx=int(raw["nx"]), ny=int(raw["ny"]), patch=int(raw["patch"]), channels=int(raw["channels"]),
        dim=int(raw["dim"]), layers=int(raw["layers"]), heads=int(raw["heads"]), meta_dim=int(raw["meta_dim"]),
        head_dim=int(tensors["head.to_cells.weight"].shape[0]), ff_inner=int(tensors["blocks.0.ff1.weight"].shape[1]),
        norm_mean=tuple(float(v) for v in n["mean"]), norm_std=tuple(float(v) for v in n["std"]),
        norm_depth=float(n["depth"]), dx=float(raw["dx"]), dt=float(raw["dt"]), g=float(raw["g"]),
        depth=float(raw["depth"]), nu=float(raw["nu"]), energy_r_max=float(raw.get("energy_r_max", 1.0)),
        mask_kind=mk, radius=r, dilation=d, raw=raw,
    )


def meta_of(cfg: ModelConfig) -> np.ndarray:
    """crates/engine/src/solver_meta.rs:9-11: [ln dx, ln dt, ln g, ln depth, ln(nu + 1e-6)], in f32."""
    f = np.float32
    return np.array([np.log(f(cfg.dx)), np.log(f(cfg.dt)), np.log(f(cfg.g)), np.log(f(cfg.depth)),
                     np.log(f(cfg.nu) + f(1e-6))], dtype=np.float32)


def tensor_names(layers: int) -> list[str]:
    names = ["embed.weight", "embed.bias", "meta.weight", "meta.bias", "pos"]
    for i in range(layers):
        for s in ("norm1.gamma", "norm1.beta", "q.weight", "q.bias", "k.weight", "k.bias", "v.weight", "v.bias",
                  "proj.weight", "proj.bias", "norm2.gamma", "norm2.beta", "ff1.weight", "ff1.bias",
                  "ff2.weight", "ff2.bias"):
            names.append(f"blocks.{i}.{s}")
    names += ["norm.gamma", "norm.beta", "head.token_mix.weight", "head.token_mix.bias",
              "head.to_cells.weight", "head.to_cells.bias", "head.conv1.weight", "head.conv1.bias",
              "head.conv2.weight", "head.conv2.bias"]
    return names


# Normalizer of the synthetic checkpoints: D20-like statistics.
SYNTH_NORM = {"mean": [0.0008, 0.0004, 0.0005], "std": [0.0063, 0.0138, 0.0135], "depth": 1.0}


def _shared_tensors(dim: int, layers: int, heads: int, seed: int, head_dim: int = 32, channels: int = 3,
                    patch: int = 4, meta_dim: int = 5, ff_mult: int = 4) -> dict[str, np.ndarray]:
    """The init recipe of training/jacobi2000_pt/model.py:52-85 (uniform
    +-1/sqrt(fan_in) for Lin/Conv, LayerNorm gamma 1 beta 0) followed by the
    fixture recipe of training/jacobi2000_pt/parity.py:63-74 (every tensor gets
    0.05 N(0,1) noise; head.conv2 scaled by 0.05 so long rollouts stay bounded).
    Random numbers come from numpy's PCG64 so they are the same on every host."""
    rng = np.random.default_rng(seed)
    t: dict[str, np.ndarray] = {}
    pd = channels * patch * patch

    def lin(name, din, dout):
        k = 1.0 / math.sqrt(din)
        t[name + ".weight"] = rng.uniform(-k, k, size=(din, dout))
        t[name + ".bias"] = rng.uniform(-k, k, size=(dout,))

    def conv(name, cin, cout, k):
        b = math.sqrt(1.0 / (cin * k * k))
        t[name + ".weight"] = rng.uniform(-b, b, size=(cout, cin, k, k))
        t[name + ".bias"] = rng.uniform(-b, b, size=(cout,))

    def norm(name):
        t[name + ".gamma"] = np.ones(dim)
        t[name + ".beta"] = np.zeros(dim)

    lin("embed", pd, dim)
    lin("meta", meta_dim, dim)
    for i in range(layers):
        p = f"blocks.{i}."
        norm(p + "norm1")
        lin(p + "q", dim, dim)
        lin(p + "k", dim, dim)
        lin(p + "v", dim, dim)
        lin(p + "proj", dim, dim)
        norm(p + "norm2")
        lin(p + "ff1", dim, dim * ff_mult)
        lin(p + "ff2", dim * ff_mult, dim)
    norm("norm")
    conv("head.token_mix", dim, dim, 3)
    conv("head.to_cells", dim, head_dim, 1)
    conv("head.conv1", head_dim + channels, head_dim, 3)
    conv("head.conv2", head_dim, channels, 3)
    for name in sorted(t):
        t[name] = t[name] + 0.05 * rng.standard_normal(t[name].shape)
    t["head.conv2.weight"] *= 0.05
    t["head.conv2.bias"] *= 0.05
    return {k: v.astype(np.float32) for k, v in t.items()}


def _pos_tensor(dim: int, tokens: int, seed: int, side_key: int) -> np.ndarray:
    """pos starts at zero (model.py:165); the fixture recipe adds 0.05 N(0,1)."""
    rng = np.random.default_rng([seed, 7919, side_key])
    return (0.05 * rng.standard_normal((1, tokens, dim))).astype(np.float32)


def _config_dict(nx, ny, dim, layers, heads, mask, energy_r_max, dt=0.0903, norm=None):
    return {
        "nx": nx, "ny": ny, "patch": 4, "channels": 3, "dim": dim, "layers": layers, "heads": heads,
        "ff_mult": 4, "meta_dim": 5, "norm": norm or SYNTH_NORM, "dx": 1.0, "dt": dt, "g": 9.81,
        "depth": 1.0, "nu": 1e-3, "mask": mask, "energy_r_max": energy_r_max,
    }


def synthetic_family(dim: int, layers: int, seed: int, sides, heads: int = 4, mask=None,
                     energy_r_max: float = 1.0001, rect: dict | None = None):
    """A checkpoint family: {(nx, ny): (tensors, config_json_str)} sharing every
    tensor but ``pos``. ``sides`` are square sides; ``rect`` adds (nx, ny) pairs."""
    if mask is None:
        mask = {"Stencil": {"radius": 1, "dilation": 1}}
    shared = _shared_tensors(dim, layers, heads, seed)
    shapes = [(s, s) for s in sides] + list(rect or [])
    fam = {}
    for nx, ny in shapes:
        if nx % 4 or ny % 4:
            raise ValueError(f"grid {nx}x{ny} is not divisible by the patch size 4")
        t = dict(shared)
        t["pos"] = _pos_tensor(dim, (nx // 4) * (ny // 4), seed, nx * 100003 + ny)
        fam[(nx, ny)] = (t, json.dumps(_config_dict(nx, ny, dim, layers, heads, mask, energy_r_max), indent=2))
    return fam


def synthetic_checkpoint(side: int, dim: int = 128, layers: int = 4, seed: int = 0, **kw):
    return synthetic_family(dim, layers, seed, [side], **kw)[(side, side)]


def checksum(tensors: dict) -> np.ndarray:
    """First 16 bytes of a SHA-256 over the tensors' names and F32 bytes, as
    f32 values (so the digest fits in a safetensors fixture)."""
    h = hashlib.sha256()
    for k in sorted(tensors):
        h.update(k.encode())
        h.update(np.ascontiguousarray(tensors[k], dtype="<f4").tobytes())
    return np.frombuffer(h.digest()[:16], dtype=np.uint8).astype(np.float32)
