"""dump-dataset on the GPU: the command of crates/engine-cli/src/dump_dataset.rs
over the library's batched reference solver (jc_sw_trajectories).

    python -m jacobi2000_gb300.dump_dataset --out <dir> [--pool N] [--nu V] [--seed S]
        [--long-fraction F] [--amplitude-max A] [--extra-drop-prob P]
        [--no-horizon-fraction F] [--extended-fraction F] [--chunk K]

Writes, as the reference does, one traj-NNNNN.f32 per trajectory (little-endian
f32, all h frames, then all u, then all v, tick-major within each channel), a
traj-NNNNN.json header and manifest.json. The trajectory distribution is the
reference's (dump_dataset.rs:104-155: short lives of 60-80 ticks with the
pre-reflection margin, a long minority of 400 ticks, an extended share with
larger and negative amplitudes and up to two extra drops landing later); the
random stream is numpy's PCG64 seeded with --seed where the reference uses
Rust's StdRng, so the same seed draws different trajectories. Trajectories run
in device batches of --chunk; the frames are bit-identical to the reference
solver's for the same drops.
"""

from __future__ import annotations

import argparse
import json
import sys
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import engine


@dataclass
class DumpConfig:
    """dump_dataset.rs:211-225 defaults; params = Params::default() with nu 1e-3."""
    nx: int = 64
    ny: int = 64
    dx: float = 1.0
    g: float = 9.81
    depth: float = 1.0
    nu: float = 1e-3
    pool: int = 2000
    short_ticks: tuple = (60, 80)
    long_ticks: int = 400
    long_fraction: float = 0.2
    amplitude: tuple = (0.02, 0.08)
    sigma: tuple = (2.5, 6.0)
    amplitude_max: float = 0.3
    extra_drop_prob: float = 0.3
    no_horizon_fraction: float = 0.3
    extended_fraction: float = 0.3
    seed: int = 20

    def params(self) -> engine.JcSwParams:
        f = np.float32
        c = np.sqrt(f(self.g) * f(self.depth), dtype=np.float32)
        dt = f(0.4) * f(self.dx) / (c * f(np.sqrt(2.0)))  # Params::with_cfl_dt(0.4)
        return engine.JcSwParams(self.nx, self.ny, self.dx, float(dt), self.g, self.depth, self.nu)


@dataclass
class Trajectory:
    ticks: int
    cx: float
    cy: float
    amp: float
    sigma: float
    pending: list = field(default_factory=list)  # (tick, cx, cy, amp, sigma)


def _f32(v) -> float:
    return float(np.float32(v))


def draw(cfg: DumpConfig, rng: np.random.Generator) -> Trajectory:
    """draw_single_drop (dump_dataset.rs:104-155)."""
    p = cfg.params()
    cpt = np.sqrt(np.float32(p.g) * np.float32(p.depth), dtype=np.float32) * np.float32(p.dt) / np.float32(p.dx)
    extended = rng.random() < cfg.extended_fraction
    amax, extra_p, noh = (cfg.amplitude_max, cfg.extra_drop_prob, cfg.no_horizon_fraction) if extended else (0.08, 0.0, 0.0)
    long = rng.random() < cfg.long_fraction
    ticks = cfg.long_ticks if long else int(rng.integers(cfg.short_ticks[0], cfg.short_ticks[1] + 1))
    no_horizon = rng.random() < noh
    margin = 8.0 if (long or no_horizon) else float(np.float32(ticks) * cpt)

    def log_uniform(lo, hi):
        return _f32(np.exp(rng.uniform(np.log(lo), np.log(hi))))

    def sign():
        return -1.0 if rng.random() < 0.25 else 1.0

    cx = _f32(rng.uniform(margin, p.nx - margin))
    cy = _f32(rng.uniform(margin, p.ny - margin))
    amp = _f32(log_uniform(cfg.amplitude[0], amax) * sign())
    sigma = _f32(rng.uniform(*cfg.sigma))
    t = Trajectory(ticks, cx, cy, amp, sigma)
    for _ in range(2):
        if ticks < 2 or not (rng.random() < extra_p):
            break
        if rng.random() < 0.5:
            dcx, dcy = cx, cy
        else:
            dcx, dcy = _f32(rng.uniform(margin, p.nx - margin)), _f32(rng.uniform(margin, p.ny - margin))
        t.pending.append((int(rng.integers(1, ticks)), dcx, dcy, _f32(log_uniform(cfg.amplitude[0], amax) * sign()),
                          _f32(rng.uniform(*cfg.sigma))))
    return t


def run_chunk(cfg: DumpConfig, trajs):
    """Frames [3, ticks + 1, ny, nx] of each trajectory, from the device."""
    p = cfg.params()
    items = []
    for t in trajs:
        x0 = engine.sw_flat(p)[0]
        engine.sw_add_drop(p, x0[0], t.cx, t.cy, t.amp, t.sigma)
        drops = []
        for (tick, cx, cy, amp, sigma) in t.pending:
            f = np.zeros((p.ny, p.nx), dtype=np.float32)
            engine.sw_add_drop(p, f, cx, cy, amp, sigma)  # exactly amp * exp(...) as add_drop forms it
            drops.append((tick, f))
        items.append((x0, t.ticks, drops))
    return engine.sw_trajectories(p, items)


def _num(v) -> str:
    return str(np.float32(v)) if isinstance(v, float) else str(v)


def header_json(h: dict, indent: str = "") -> str:
    """The serde layout of dump_dataset.rs:63-78 (f32 fields in shortest form)."""
    return "{" + ",".join(f'"{k}":{_num(v)}' for k, v in h.items()) + "}"


def dump(cfg: DumpConfig, out: Path, chunk: int = 256):
    out.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(cfg.seed)
    p = cfg.params()
    headers = []
    trajs = [draw(cfg, rng) for _ in range(cfg.pool)]
    for c0 in range(0, len(trajs), chunk):
        frames = run_chunk(cfg, trajs[c0:c0 + chunk])
        for k, fr in enumerate(frames):
            index = c0 + k
            t = trajs[index]
            (out / f"traj-{index:05d}.f32").write_bytes(np.ascontiguousarray(fr, dtype="<f4").tobytes())
            h = {"index": index, "ticks": t.ticks + 1, "nx": p.nx, "ny": p.ny, "dx": _f32(p.dx), "dt": _f32(p.dt),
                 "g": _f32(p.g), "depth": _f32(p.depth), "nu": _f32(p.nu), "cx": t.cx, "cy": t.cy, "amp": t.amp,
                 "sigma": t.sigma}
            (out / f"traj-{index:05d}.json").write_text(header_json(h))
            headers.append(h)
    manifest = "[\n" + ",\n".join(
        "  {\n" + ",\n".join(f'    "{k}": {_num(v)}' for k, v in h.items()) + "\n  }" for h in headers) + "\n]"
    (out / "manifest.json").write_text(manifest)
    return headers


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="dump-dataset")
    ap.add_argument("--out", required=True)
    ap.add_argument("--pool", type=int, default=2000)
    ap.add_argument("--long-fraction", type=float, default=0.2)
    ap.add_argument("--amplitude-max", type=float, default=0.3)
    ap.add_argument("--extra-drop-prob", type=float, default=0.3)
    ap.add_argument("--no-horizon-fraction", type=float, default=0.3)
    ap.add_argument("--extended-fraction", type=float, default=0.3)
    ap.add_argument("--nu", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=20)
    ap.add_argument("--chunk", type=int, default=256)
    a = ap.parse_args(argv)
    cfg = DumpConfig(pool=a.pool, long_fraction=a.long_fraction, amplitude_max=a.amplitude_max,
                     extra_drop_prob=a.extra_drop_prob, no_horizon_fraction=a.no_horizon_fraction,
                     extended_fraction=a.extended_fraction, nu=a.nu, seed=a.seed)
    headers = dump(cfg, Path(a.out), a.chunk)
    print(f"{len(headers)} trajectories, {sum(h['ticks'] for h in headers)} total ticks, written to {a.out}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
