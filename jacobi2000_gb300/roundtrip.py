"""Rewind round trip on the GPU: forward N ticks with a forward checkpoint,
then N ticks back with its reverse checkpoint, scored against the start (the
round-trip runs of docs/runs/2026-09-20-rewind-round-trip.md:17-32).

    python -m jacobi2000_gb300.roundtrip --forward <dir> --reverse <dir>
        [--horizons 10,25,50] [--trajectories 24] [--seed 0]
        [--project true|false] [--project-energy true|false] [--precision fp32|bf16]

Trajectories are single drops drawn as eval-metrics draws them
(jacobi2000_gb300.evaluate.draw_drops). The table is the mean over
trajectories of the correlation and amplitude ratio of the rewound state
against the start, the round-trip RMSE and the RMSE of the N-tick change (what
a rewind that changes nothing would score), in normalized units.
"""

from __future__ import annotations

import argparse
import sys

import numpy as np

from . import engine
from .evaluate import _bool, draw_drops


def roundtrip(forward: engine.Model, reverse: engine.Model, horizons=(10, 25, 50), trajectories: int = 24,
              seed: int = 0, project: bool = True, project_energy: bool = False):
    """Returns {horizon: {metric: mean over trajectories}}."""
    horizons = sorted(int(h) for h in horizons)
    drops, _ = draw_drops(forward.config, trajectories, seed, float(max(horizons[-1], 50)))
    flags = (engine.PROJECT_MASS if project else 0) | (engine.PROJECT_ENERGY if project_energy else 0)
    with engine.RoundTrip(forward, reverse, len(drops), len(horizons)) as rt:
        rows = rt.run(drops, horizons, flags)
    return {h: {f: float(np.mean(rows[i][f], dtype=np.float32)) for f in engine.ROUNDTRIP_FIELDS}
            for i, h in enumerate(horizons)}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="round-trip")
    ap.add_argument("--forward", required=True)
    ap.add_argument("--reverse", required=True)
    ap.add_argument("--horizons", default="10,25,50")
    ap.add_argument("--trajectories", type=int, default=24)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--project", type=_bool, default=True)
    ap.add_argument("--project-energy", type=_bool, default=False)
    ap.add_argument("--precision", choices=("fp32", "bf16"), default="fp32")
    a = ap.parse_args(argv)
    horizons = [int(s) for s in a.horizons.split(",") if s.strip()]
    if not horizons:
        ap.error("--horizons is empty")
    prec = engine.BF16 if a.precision == "bf16" else engine.FP32
    with engine.Model.load(a.forward, prec) as f, engine.Model.load(a.reverse, prec) as r:
        table = roundtrip(f, r, horizons, a.trajectories, a.seed, a.project, a.project_energy)
    print(f"{a.trajectories} single-drop trajectories, backend: cuda ({a.precision})\n")
    print("| horizon | corr | amplitude ratio | round-trip RMSE | N-tick change RMSE |")
    print("|---:|---:|---:|---:|---:|")
    for h in sorted(table):
        t = table[h]
        print(f"| {h} | {t['corr']:.4f} | {t['amplitude_ratio']:.4f} | {t['rmse']:.3f} | {t['change_rmse']:.3f} |")
    return 0


if __name__ == "__main__":
    sys.exit(main())
