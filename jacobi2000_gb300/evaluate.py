"""eval-metrics on the GPU: the command of crates/engine-cli/src/eval.rs:1-202
over the library's evaluator (jc_eval_*).

    python -m jacobi2000_gb300.evaluate --model <checkpoint-dir> [--horizons 10,25,50]
        [--trajectories 16] [--seed 0] [--project true|false]
        [--project-energy true|false] [--precision fp32|bf16]

Each trajectory is one drop placed so that its wave has not met a wall by the
last horizon (or 50 ticks, whichever is later); drops that cannot answer that
are redrawn (eval.rs:126-134). The drop distribution is the reference's (centre
uniform in [8, n - 8), amplitude in [0.03, 0.07), radius in [3, 5.5)); the
random stream is numpy's PCG64 seeded with --seed, where the reference uses
Rust's StdRng, so the same seed draws different drops. All trajectories run
as one batch on the device; the table is the mean over trajectories.
"""

from __future__ import annotations

import argparse
import sys

import numpy as np

from . import engine


def cells_per_tick(cfg) -> np.float32:
    """Params::cells_per_tick (crates/solvers/src/shallow_water.rs:64-66), f32."""
    f = np.float32
    return np.sqrt(f(cfg.g) * f(cfg.depth), dtype=np.float32) * f(cfg.dt) / f(cfg.dx)


def horizon_ticks(cfg, cx: float, cy: float) -> np.float32:
    """Params::horizon_ticks (shallow_water.rs:71-77), f32."""
    f = np.float32
    dist = min(f(cx), f(cy), f(cfg.nx) - f(cx), f(cfg.ny) - f(cy))
    return f(dist) / cells_per_tick(cfg)


def draw_drops(cfg, trajectories: int, seed: int, need: float):
    """Single drops that stay clear of the walls for `need` ticks; returns
    (drops, skipped)."""
    rng = np.random.default_rng(seed)
    drops, skipped = [], 0
    while len(drops) < trajectories:
        cx = float(np.float32(rng.uniform(8.0, cfg.nx - 8.0)))
        cy = float(np.float32(rng.uniform(8.0, cfg.ny - 8.0)))
        amp = float(np.float32(rng.uniform(0.03, 0.07)))
        sigma = float(np.float32(rng.uniform(3.0, 5.5)))
        if horizon_ticks(cfg, cx, cy) < need:
            skipped += 1
            if skipped > 100000:
                raise ValueError("the grid is too small for single-drop trajectories of this horizon")
            continue
        drops.append((cx, cy, amp, sigma))
    return drops, skipped


def evaluate(model: engine.Model, horizons=(10, 25, 50), trajectories: int = 16, seed: int = 0,
             project: bool = True, project_energy: bool = False):
    """Returns ({horizon: {metric: mean over trajectories}}, max energy
    violation, drops used, drops skipped)."""
    horizons = sorted(int(h) for h in horizons)
    need = float(max(horizons[-1], 50))
    drops, skipped = draw_drops(model.config, trajectories, seed, need)
    flags = (engine.PROJECT_MASS if project else 0) | (engine.PROJECT_ENERGY if project_energy else 0)
    with engine.Evaluator(model, len(drops)) as ev:
        rows, viol = ev.run(drops, horizons, flags)
    table = {h: {f: float(np.mean(rows[i][f], dtype=np.float32)) for f in engine.EVAL_FIELDS}
             for i, h in enumerate(horizons)}
    return table, viol, len(drops), skipped


def _bool(s: str) -> bool:
    if s not in ("true", "false"):
        raise argparse.ArgumentTypeError(f"expected true or false, got `{s}`")
    return s == "true"


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="eval-metrics")
    ap.add_argument("--model", required=True)
    ap.add_argument("--horizons", default="10,25,50")
    ap.add_argument("--trajectories", type=int, default=16)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--project", type=_bool, default=True)
    ap.add_argument("--project-energy", type=_bool, default=False)
    ap.add_argument("--precision", choices=("fp32", "bf16"), default="fp32")
    a = ap.parse_args(argv)
    horizons = [int(s) for s in a.horizons.split(",") if s.strip()]
    if not horizons:
        ap.error("--horizons is empty")
    prec = engine.BF16 if a.precision == "bf16" else engine.FP32
    with engine.Model.load(a.model, prec) as m:
        table, viol, used, skipped = evaluate(m, horizons, a.trajectories, a.seed, a.project, a.project_energy)
        c = m.config
        mask = "Full" if c.mask_kind == 0 else f"Stencil {{ radius: {c.mask_radius}, dilation: {c.mask_dilation} }}"
        print(f"backend: cuda ({a.precision}), mass projection: {str(a.project).lower()}, energy projection: "
              f"{str(a.project_energy).lower()} (r_max {c.energy_r_max:g}), mask: {mask}")
    need = max(max(horizons), 50)
    print(f"{used} single-drop trajectories, {skipped} skipped (horizon < {need} ticks)\n")
    print("| ticks | corr (h,u,v) | corr (h) | amplitude ratio | wavefront lag (cells) | bias |")
    print("|---:|---:|---:|---:|---:|---:|")
    for h in sorted(table):
        r = table[h]
        print(f"| {h} | {r['corr']:.4f} | {r['corr_h']:.4f} | {r['amplitude_ratio']:.4f} | {r['lag']:+.3f} | "
              f"{r['bias']:+.3f} |")
    if a.project_energy:
        print(f"\nmax relative energy violation along the projected rollout: {viol:.3e} (bound: <= 1e-6)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
