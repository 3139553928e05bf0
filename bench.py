"""Throughput of the shallow-water transformer rollout on GB300.

Workload (default): B instances of a 128x128 grid, model20-shaped checkpoint
(dim 128, 4 layers, 4 heads, stencil r1 d1, random init seed 0), 8 seeded
Gaussian drops per instance (amplitude U[0.02, 0.15], sigma U[2, 6] cells,
periodic images), a 50-tick rollout with mass and energy projection per
instance. One step = one batched rollout of all B instances. Metric:
cell-ticks/s = sum over instances of nx * ny * ticks / seconds.

* ``value``: device-resident inputs (x0/meta already in HBM), timed with CUDA
  events on the launching stream.
* ``e2e``: the same rollouts through the C ABI with host buffers; host->device
  copies of x0/meta and device->host copies of the final states and energies
  are inside the timed region.
* ``fp32_plain``: the FP32 single-request path, one rollout at a time.
* ``--impl reference``: the reference's CPU forward pass and projections
  (the C restatement of crates/engine/src/cpu.rs and project.rs, with the
  reference's own O(T^2) masked attention scan) on the host cores.

Under torchrun each rank runs its own B instances (no exchange step):
weak scaling, barrier + max over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-ticks/s BF16 served vs FP32 plain on 1 GB300 at stated error; p50/p99 lat"
UNIT = "cell-ticks/s"
FLOP_PER_CELL_TICK = {(128, 4): 141_056, (256, 6): 691_456}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16", choices=["fp32", "bf16"])
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--side", type=int, default=128)
    ap.add_argument("--ticks", type=int, default=50)
    ap.add_argument("--dim", type=int, default=128)
    ap.add_argument("--layers", type=int, default=4)
    ap.add_argument("--cpu-sample-ticks", type=int, default=300,
                    help="ticks of one instance timed on the host cores for cpu_baseline (about 10 s)")
    ap.add_argument("--cpu-sample-ticks-1t", type=int, default=20,
                    help="ticks of the same instance timed on one host thread (about 10 s); 0 to skip")
    ap.add_argument("--ref-step-ticks", type=int, default=50,
                    help="ticks of one instance per step of the --impl reference arm")
    ap.add_argument("--served-rates", default="100,400,1600",
                    help="request arrival rates (req/s) of the served-form run; empty to skip")
    ap.add_argument("--served-requests", type=int, default=240)
    ap.add_argument("--served-fp32-requests", type=int, default=24)
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-task batch measurement")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the 256x256 error report against the f64 oracle")
    ap.add_argument("--no-eval", action="store_true", help="skip the eval-metrics measurement")
    return ap.parse_args()


def workload(args):
    from jacobi2000_gb300.checkpoint import parse_config, synthetic_checkpoint, meta_of
    from jacobi2000_gb300.ic import random_drops

    t, cj = synthetic_checkpoint(args.side, args.dim, args.layers, 0)
    cfg = parse_config(cj, t)
    rank = int(os.environ.get("RANK", "0"))
    x0s = [random_drops(cfg, seed=rank * 100_000 + i) for i in range(args.instances)]
    return t, cj, cfg, x0s, meta_of(cfg)


def config_dict(args, cfg):
    return {"workload": f"rollout {args.instances}x {args.side}x{args.side} grids, {args.ticks} ticks, "
                        f"mass+energy projection, 8 drops/instance",
            "model": f"jacobi2000 dim {args.dim}, {args.layers} layers, 4 heads, stencil r1 d1, seed 0",
            "grid": [args.side, args.side], "instances_per_step": args.instances, "ticks": args.ticks,
            "l2": "per-tick working set > 129 MB L2 (no flush needed)", "parallelism": "replicas"}


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, out: Path):
        self.out = out
        self.p = None

    def __enter__(self):
        try:
            self.f = open(self.out, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()
            self.f.close()

    def summary(self, gpu_index: int = 0):
        try:
            rows = [r.split(", ") for r in self.out.read_text().strip().splitlines()]
        except OSError:
            return None
        rows = [r for r in rows if len(r) >= 9 and r[0].strip() == str(gpu_index)]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        reasons = set()
        for r in rows:
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), r[5:9]):
                if v.strip() == "Active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "samples": len(rows),
                "reasons": sorted(reasons)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0}, "fallback"


def ncu_traffic() -> dict:
    """Per-launch DRAM bytes of kernels from the committed ncu summary
    (profiles/ncu_traffic.txt: `kernel bytes_per_launch` lines)."""
    p = ROOT / "profiles" / "ncu_traffic.txt"
    out = {}
    if p.exists():
        for line in p.read_text().splitlines():
            parts = line.split()
            if len(parts) >= 2 and not line.startswith("#"):
                try:
                    out[parts[0]] = float(parts[1])
                except ValueError:
                    pass
    return out


def kernel_work(name: str, B: int, cells: int, D: int, F: int):
    """Algorithmic work of one launch of a kernel over the whole batch:
    ("flop", useful FLOPs) for contractions, ("byte", compulsory bytes) for
    memory-bound kernels. R tokens = B cells / 16, N cells = B cells."""
    R, N = B * cells // 16, B * cells
    flop = {"tc_qkv": 2 * R * D * 3 * D, "tc_proj_ln": 2 * R * D * D, "tc_mlp": 4 * R * D * F,
            "tc_token_mix": 18 * R * D * D, "tc_to_cells": 2 * R * D * 32, "tc_conv1": 2 * N * 35 * 9 * 32,
            "f32_ln_qkv": 2 * R * D * 3 * D, "f32_proj": 2 * R * D * D, "f32_ln_ff1": 2 * R * D * F,
            "f32_ff2": 2 * R * F * D, "f32_token_mix": 18 * R * D * D, "f32_to_cells": 2 * R * D * 32,
            "f32_conv1": 2 * N * 35 * 9 * 32, "bf_conv2_step": 2 * N * 32 * 9 * 3, "f32_conv2_step": 2 * N * 32 * 9 * 3}
    byte = {"bf_attention": R * (3 * D * 2 + D * 2), "bf_embed": N * 12 + R * (4 * D + 2 * D),
            "bf_upsample": R * 32 * 4 + N * (12 + 96), "projection": N * 12 * 4 + N * 12,
            "f32_attention": R * (3 * D * 4 + D * 4), "f32_embed": N * 12 + R * 4 * D,
            "f32_upsample_concat": R * 32 * 4 + N * (12 + 144), "f32_final_ln": R * D * 8}
    if name in flop:
        return "flop", flop[name]
    if name in byte:
        return "byte", byte[name]
    return None, None


SERVED_SIDES = [32, 64, 96, 128, 160, 192, 224, 256]


def served_requests(rng, n, rate, cfgs, volumes, masks):
    """Poisson arrivals at `rate`; grid side log-uniform in [32, 256] rounded
    to a multiple of 32; horizon U[10, 50]; tasks 1/3 forward (initial state
    known), 1/3 rewind (final state known), 1/3 reconstruct (2% of the
    space-time cells known). Returns (arrival_s, task, grid, ticks, x, known)."""
    from jacobi2000_gb300 import engine
    from jacobi2000_gb300.ic import random_drops

    out, t = [], 0.0
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        side = float(np.exp(rng.uniform(np.log(32), np.log(256))))
        g = int(np.argmin([abs(side - s) for s in SERVED_SIDES]))
        ticks = int(rng.integers(10, 51))
        task = int(rng.integers(0, 3))
        if task == engine.TASK_RECONSTRUCT:
            x, known = volumes[g][: ticks + 1], masks[g][: ticks + 1]
        else:
            x, known = random_drops(cfgs[g], seed=int(rng.integers(1 << 30))), None
        out.append((t, task, g, ticks, x, known))
    return out


def run_served(srv, reqs, metas, sweeps, concurrent=True):
    """Submits at the arrival times (concurrent) or one request at a time
    after the previous result (sequential). Returns throughput and latency
    percentiles, latency measured from the scheduled arrival."""
    import threading

    from jacobi2000_gb300 import engine

    lat = [None] * len(reqs)
    cell_ticks = sum(SERVED_SIDES[g] ** 2 * ticks for _, _, g, ticks, _, _ in reqs)
    t0 = time.perf_counter()
    ids = [None] * len(reqs)

    def collect():
        for k, (arr, task, g, ticks, _, _) in enumerate(reqs):
            while ids[k] is None:
                time.sleep(0.0002)
            srv.wait(ids[k], task, g, ticks, timeout=600)
            lat[k] = time.perf_counter() - (t0 + arr)

    if concurrent:
        th = threading.Thread(target=collect)
        th.start()
        for k, (arr, task, g, ticks, x, known) in enumerate(reqs):
            delay = t0 + arr - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            ids[k] = srv.submit(task, g, x, metas[g], ticks, known=known, max_sweeps=sweeps, tol=0.0)
        th.join()
    else:
        for k, (arr, task, g, ticks, x, known) in enumerate(reqs):
            delay = t0 + arr - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            rid = srv.submit(task, g, x, metas[g], ticks, known=known, max_sweeps=sweeps, tol=0.0)
            srv.wait(rid, task, g, ticks, timeout=600)
            lat[k] = time.perf_counter() - (t0 + arr)
    span = time.perf_counter() - t0
    lat_ms = np.array(lat) * 1e3
    return {"requests": len(reqs), "cell_ticks_per_s": cell_ticks / span, "span_s": span,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99))}


def served_bench(args):
    """Config: Poisson arrivals, three task types, sides 32-256, BF16 served
    form with continuous batching vs the FP32 one-request-at-a-time path."""
    from jacobi2000_gb300 import engine
    from jacobi2000_gb300.checkpoint import parse_config, synthetic_family, write_safetensors_bytes, meta_of

    rates = [float(r) for r in args.served_rates.split(",") if r.strip()]
    if not rates:
        return None
    fam_f = synthetic_family(args.dim, args.layers, 0, SERVED_SIDES)
    fam_r = synthetic_family(args.dim, args.layers, 1, SERVED_SIDES)
    cfgs = [parse_config(fam_f[(s, s)][1], fam_f[(s, s)][0]) for s in SERVED_SIDES]
    metas = [meta_of(c) for c in cfgs]
    rng = np.random.default_rng(1234)
    volumes, masks = [], []
    for s in SERVED_SIDES:
        volumes.append((0.3 * rng.standard_normal((51, 3, s, s))).astype(np.float32))
        masks.append((rng.random((51, s, s)) < 0.02).astype(np.uint8))
    sweeps = 4
    out = {"task_mix": "1/3 forward, 1/3 rewind, 1/3 reconstruct (2% known, 4 Jacobi sweeps)",
           "sides": "log-uniform 32-256, rounded to a multiple of 32", "horizon": "U[10,50] ticks",
           "admission": "0.8 x HBM, 8M cells per tick", "bf16": []}
    for prec, key in ((engine.BF16, "bf16"), (engine.FP32, "fp32_one_at_a_time")):
        fm = [engine.Model.from_bytes(write_safetensors_bytes(fam_f[(s, s)][0]), fam_f[(s, s)][1], prec)
              for s in SERVED_SIDES]
        rm = [engine.Model.from_bytes(write_safetensors_bytes(fam_r[(s, s)][0]), fam_r[(s, s)][1], prec)
              for s in SERVED_SIDES]
        with engine.Server(fm, rm, max_active_cells=8 << 20, hbm_fraction=0.8) as srv:
            warm = served_requests(np.random.default_rng(99), 12, 1000.0, cfgs, volumes, masks)
            run_served(srv, warm, metas, sweeps)
            if prec == engine.BF16:
                for rate in rates:
                    reqs = served_requests(np.random.default_rng(int(rate)), args.served_requests, rate, cfgs,
                                           volumes, masks)
                    r = run_served(srv, reqs, metas, sweeps)
                    r["rate_req_s"] = rate
                    out["bf16"].append(r)
            else:
                reqs = served_requests(np.random.default_rng(int(rates[0])), args.served_fp32_requests, rates[0],
                                       cfgs, volumes, masks)
                r = run_served(srv, reqs, metas, sweeps, concurrent=False)
                r["rate_req_s"] = rates[0]
                out[key] = r
        for m in fm + rm:
            m.close()
    return out


MIXED_SIDES = [32, 64, 96, 128, 192]


def mixed_batch_bench(args, steps=3):
    """Config: 64 instances in one batch call, sides uniform in {32, 64, 96,
    128, 192}, horizons U[10, 50]; 1/3 forward, 1/3 rewind (the reverse
    family), 1/3 reconstruct (2% of space-time cells known, 4 Jacobi sweeps).
    Timed end to end with host buffers, with the autotuned schedules and with
    the fixed default schedule."""
    from jacobi2000_gb300 import engine
    from jacobi2000_gb300.checkpoint import parse_config, synthetic_family, write_safetensors_bytes, meta_of
    from jacobi2000_gb300.ic import random_drops

    fam_f = synthetic_family(args.dim, args.layers, 0, MIXED_SIDES)
    fam_r = synthetic_family(args.dim, args.layers, 1, MIXED_SIDES)
    cfgs = [parse_config(fam_f[(s, s)][1], fam_f[(s, s)][0]) for s in MIXED_SIDES]
    models = [engine.Model.from_bytes(write_safetensors_bytes(f[(s, s)][0]), f[(s, s)][1], engine.BF16)
              for f in (fam_f, fam_r) for s in MIXED_SIDES]
    nf = len(MIXED_SIDES)
    rng = np.random.default_rng(4)
    me = engine.PROJECT_MASS | engine.PROJECT_ENERGY
    items, useful, n_inst, recon_cells, tick_cells = [], 0, 0, 0, 0
    for k in range(64):
        g = int(rng.integers(nf))
        cfg, H = cfgs[g], int(rng.integers(10, 51))
        cells = cfg.nx * cfg.ny
        useful += cells * H
        task = k % 3
        if task < 2:
            items.append((g + nf * task, random_drops(cfg, seed=int(rng.integers(1 << 30))), meta_of(cfg), H, me))
            n_inst += 1
            tick_cells += cells
        else:
            known = rng.random((H + 1, cfg.ny, cfg.nx)) < 0.02
            vals = np.where(known[:, None], (0.3 * rng.standard_normal((H + 1, 3, cfg.ny, cfg.nx))), 0)
            items.append({"task": engine.TASK_RECONSTRUCT, "model": g, "reverse_model": g + nf,
                          "x": vals.astype(np.float32), "known": known.astype(np.uint8), "meta": meta_of(cfg),
                          "ticks": H, "max_sweeps": 4, "tol": 0.0})
            n_inst += 2 * H + 2
            recon_cells += cells * (2 * H + 2)
    out = {"instances": 64, "sides": MIXED_SIDES, "horizon": "U[10,50] ticks",
           "task_mix": "1/3 forward, 1/3 rewind, 1/3 reconstruct (2% known, 4 Jacobi sweeps)",
           "useful_cell_ticks": useful, "timing": "wall clock per batch call, host buffers in and out"}
    prev = engine.autotune(None)
    try:
        with engine.Batch(models, max_instances=n_inst, max_cells=max(tick_cells, recon_cells)) as b:
            for key, on in (("default_schedule", False), ("autotuned", True)):
                engine.autotune(on)
                b.rollout(items)  # capture (and, when on, tune) outside the timed calls
                t0 = time.perf_counter()
                for _ in range(steps):
                    b.rollout(items)
                dt = (time.perf_counter() - t0) / steps
                out[key] = {"s_per_batch": dt, "cell_ticks_per_s": useful / dt}
    finally:
        engine.autotune(prev)
        for m in models:
            m.close()
    out["autotune_speedup"] = out["default_schedule"]["s_per_batch"] / out["autotuned"]["s_per_batch"]
    return out


def accuracy_c3(ticks=(10, 25, 50)):
    """Config: 256x256 checkpoints at dim 128 / 4 layers (seed 0) and dim 256 /
    6 layers (seed 1), 8 drops, mass + energy projection each tick. Per-field
    normwise error (max|a - b| / max|b|) of the BF16 and the FP32 path against
    the f64 oracle for one forward and along a 50-tick rollout, the largest
    relative energy violation of each, and |E - E_oracle| / E_oracle at the
    reported ticks."""
    from jacobi2000_gb300 import engine
    from jacobi2000_gb300.checkpoint import parse_config, synthetic_checkpoint, write_safetensors_bytes, meta_of
    from jacobi2000_gb300.ic import random_drops
    from oracle import oracle

    def err(a, b):
        a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
        return [float(np.abs(a[i] - b[i]).max() / max(np.abs(b[i]).max(), 1e-30)) for i in range(3)]

    oracle.set_threads(os.cpu_count() or 1)
    oracle.set_attention_mode("gather")
    me = engine.PROJECT_MASS | engine.PROJECT_ENERGY
    H = max(ticks)
    out = []
    for dim, layers, seed in ((128, 4, 0), (256, 6, 1)):
        t, cj = synthetic_checkpoint(256, dim, layers, seed)
        cfg = parse_config(cj, t)
        x0 = random_drops(cfg, seed=7)
        meta = meta_of(cfg)
        t0 = time.perf_counter()
        orc = oracle.OracleModel(cfg, t)
        want_fwd = orc.forward(x0.astype(np.float64), meta.astype(np.float64), f64=True)
        _, e64, v64, traj64 = orc.rollout(x0.astype(np.float64), meta.astype(np.float64), H, oracle.MASS | oracle.ENERGY,
                                          f64=True, trajectory=True)
        oracle_s = time.perf_counter() - t0
        row = {"model": f"dim {dim}, {layers} layers, 256x256, seed {seed}", "oracle_s": oracle_s,
               "f64_max_energy_violation": float(v64), "paths": {}}
        for name, prec in (("bf16", engine.BF16), ("fp32", engine.FP32)):
            with engine.Model.from_bytes(write_safetensors_bytes(t), cj, prec) as m:
                fwd = m.forward(x0, meta)
                final, e, traj = m.rollout(x0, meta, H, me, trajectory=True)
            viol = float(np.max(np.maximum((e[1:] - e[:-1] * cfg.energy_r_max) / e[:-1], 0.0)))
            e, e64a = np.asarray(e, np.float64), np.asarray(e64, np.float64)
            row["paths"][name] = {"forward": max(err(fwd, want_fwd)),
                                  "rollout": {str(k): max(err(traj[k], traj64[k])) for k in ticks},
                                  "max_energy_violation": viol,
                                  "energy_rel_diff": {str(k): float(abs(e[k] - e64a[k]) / abs(e64a[k])) for k in ticks}}
        out.append(row)
    return {"measure": "max over fields of max|a - b| / max|b| against the f64 oracle", "ticks": list(ticks),
            "cases": out}


def eval_bench(args, steps=3):
    """The eval-metrics row (crates/engine-cli/src/eval.rs at its defaults:
    horizons 10/25/50, mass projection): 64 single-drop trajectories drawn as
    eval.rs draws them on the workload's grid, all in one jc_eval_run (model,
    solver and scoring in one captured graph), for the BF16 and the FP32
    model; the solver kernel alone on 256 states of 256x256 (24 compulsory
    bytes per cell-step, inputs larger than L2); and the oracle's eval loop
    (f32 forward with the reference's masked scan, C solver, C scores) on one
    trajectory on the host cores."""
    import torch

    from jacobi2000_gb300 import engine, evaluate
    from jacobi2000_gb300.checkpoint import meta_of, parse_config, synthetic_checkpoint, write_safetensors_bytes
    from oracle import oracle

    horizons, ntraj = [10, 25, 50], 64
    t, cj = synthetic_checkpoint(args.side, args.dim, args.layers, 0)
    cfg = parse_config(cj, t)
    out = {"config": {"grid": f"{args.side}x{args.side}", "model": f"dim {args.dim}, {args.layers} layers",
                      "trajectories": ntraj, "horizons": horizons, "flags": "mass projection"}}
    rows32 = None
    for prec, key in ((engine.BF16, "bf16"), (engine.FP32, "fp32")):
        m = engine.Model.from_bytes(write_safetensors_bytes(t), cj, prec)
        drops, skipped = evaluate.draw_drops(m.config, ntraj, 0, 50.0)
        with engine.Evaluator(m, ntraj) as ev:
            ev.run(drops, horizons)
            times = []
            for _ in range(steps):
                t0 = time.perf_counter()
                rows, viol = ev.run(drops, horizons)
                times.append(time.perf_counter() - t0)
        sec = statistics.median(times)
        out[key] = {"s_per_eval": sec, "trajectories_per_s": ntraj / sec,
                    "model_cell_ticks_per_s": ntraj * cfg.nx * cfg.ny * horizons[-1] / sec,
                    "mean_corr_at": {str(h): float(rows[i]["corr"].mean()) for i, h in enumerate(horizons)}}
        if prec == engine.FP32:
            rows32 = rows
        m.close()
    # the solver kernel alone, CUDA events on the launching stream
    L = engine.load_library()
    engine._declare_eval(L)
    count, side, nsteps = 256, 256, 50
    p = engine.JcSwParams(side, side, 1.0, cfg.dt, cfg.g, cfg.depth, cfg.nu)
    st = torch.zeros((count, 3, side, side), device="cuda")
    st[:, 0] = 1.0
    stream = torch.cuda.current_stream()
    engine._check(L.jc_sw_run_device(engine.C.byref(p), st.data_ptr(), count, 4, stream.cuda_stream))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    engine._check(L.jc_sw_run_device(engine.C.byref(p), st.data_ptr(), count, nsteps, stream.cuda_stream))
    e1.record(stream)
    torch.cuda.synchronize()
    step_s = e0.elapsed_time(e1) / nsteps / 1e3
    cells = count * side * side
    pk, pk_kind = peaks()
    gbs = cells * 24 / step_s / 1e9
    out["sw_step"] = {"workload": f"{count} states of {side}x{side}", "us_per_step": step_s * 1e6,
                      "cell_steps_per_s": cells / step_s,
                      "roofline": {"bound": "hbm", "achieved": gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
                                   "frac": gbs / pk["hbm_gbs"], "bytes_per_cell_step": 24,
                                   "peak_kind": f"{pk_kind} copy bandwidth"}}
    del st
    # the oracle's eval loop on one trajectory
    oracle.set_threads(os.cpu_count() or 1)
    oracle.set_attention_mode("scan")
    om = oracle.OracleModel(cfg, t)
    t0 = time.perf_counter()
    want, _ = oracle.eval_metrics(om, drops[:1], horizons, oracle.MASS | oracle.SUM64, meta_of(cfg))
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"trajectories_per_s": 1.0 / cpu_s, "cores": oracle.get_threads(), "kind": "port",
                           "sample": f"1 trajectory x {horizons[-1]} ticks, {cpu_s:.1f} s"}
    out["fp32_vs_oracle_max_abs_corr_diff"] = float(np.abs(rows32[:, 0]["corr"] - want[:, 0, 0]).max())

    # rewind round trip: forward N then back N with the reverse checkpoint
    # (a second seeded family), all trajectories and horizons batched
    tr, cjr = synthetic_checkpoint(args.side, args.dim, args.layers, 1)
    fm = engine.Model.from_bytes(write_safetensors_bytes(t), cj, engine.BF16)
    rm = engine.Model.from_bytes(write_safetensors_bytes(tr), cjr, engine.BF16)
    with engine.RoundTrip(fm, rm, ntraj, len(horizons)) as rt:
        rt.run(drops, horizons)
        times = []
        for _ in range(steps):
            t0 = time.perf_counter()
            rrows = rt.run(drops, horizons)
            times.append(time.perf_counter() - t0)
    fm.close()
    rm.close()
    sec = statistics.median(times)
    traj_ticks = ntraj * (horizons[-1] + sum(horizons))
    omr = oracle.OracleModel(parse_config(cjr, tr), tr)
    t0 = time.perf_counter()
    oracle.roundtrip(om, omr, drops[:1], horizons, oracle.MASS | oracle.SUM64, meta_of(cfg))
    cpu_rt = time.perf_counter() - t0
    # dump-dataset: 512 trajectories of the reference distribution on the 64x64
    # solver grid, frames to host memory (files not written), against the
    # oracle's solver on 8 of them
    from jacobi2000_gb300 import dump_dataset as dd

    dcfg = dd.DumpConfig(pool=512, seed=20)
    drng = np.random.default_rng(20)
    dtrajs = [dd.draw(dcfg, drng) for _ in range(dcfg.pool)]
    dd.run_chunk(dcfg, dtrajs[:8])
    t0 = time.perf_counter()
    for c0 in range(0, len(dtrajs), 256):
        dd.run_chunk(dcfg, dtrajs[c0:c0 + 256])
    dump_s = time.perf_counter() - t0
    frames = sum(t.ticks for t in dtrajs)
    sp = dcfg.params()
    q = oracle._SwParams()
    q.nx, q.ny, q.dx, q.dt, q.g, q.depth, q.nu = sp.nx, sp.ny, sp.dx, sp.dt, sp.g, sp.depth, sp.nu
    t0 = time.perf_counter()
    cpu_steps = 0
    for t in dtrajs[:8]:
        st = oracle.sw_flat(q)[0]
        oracle.sw_add_drop(q, st[0], t.cx, t.cy, t.amp, t.sigma)
        oracle.sw_steps(q, st, t.ticks)
        cpu_steps += t.ticks
    cpu_dump_s = time.perf_counter() - t0
    out["dump_dataset"] = {"config": "512 trajectories, 64x64, the reference distribution (60-80 and 400 ticks)",
                           "s": dump_s, "trajectories_per_s": len(dtrajs) / dump_s,
                           "solver_cell_steps_per_s": frames * 64 * 64 / dump_s,
                           "cpu_baseline": {"solver_cell_steps_per_s": cpu_steps * 64 * 64 / cpu_dump_s, "cores": 1,
                                            "kind": "port", "sample": f"8 trajectories, {cpu_dump_s:.2f} s"}}
    out["roundtrip"] = {"config": f"{ntraj} trajectories, horizons {horizons}, bf16 forward and reverse models",
                        "s_per_run": sec, "trajectories_per_s": ntraj / sec,
                        "model_cell_ticks_per_s": traj_ticks * cfg.nx * cfg.ny / sec,
                        "mean_corr_at": {str(h): float(rrows[i]["corr"].mean()) for i, h in enumerate(horizons)},
                        "cpu_baseline": {"trajectories_per_s": 1.0 / cpu_rt, "cores": oracle.get_threads(),
                                         "kind": "port", "sample": f"1 trajectory, {cpu_rt:.1f} s"}}
    return out


def cpu_sample(cfg, t, x0, meta, ticks: int, threads: int = 0):
    """The oracle's f32 rollout (the reference's CPU arithmetic and O(T^2)
    masked scan) over `ticks` ticks of one instance, on `threads` host
    threads (0: all host cores)."""
    from oracle import oracle

    oracle.set_threads(threads or os.cpu_count() or 1)
    oracle.set_attention_mode("scan")
    m = oracle.OracleModel(cfg, t)
    t0 = time.perf_counter()
    m.rollout(x0, meta, ticks, oracle.MASS | oracle.ENERGY)
    dt = time.perf_counter() - t0
    return cfg.nx * cfg.ny * ticks / dt, oracle.get_threads(), dt


def max_over_ranks(v: float, world: int, device: str) -> float:
    """The largest of the ranks' values (a step time: the job ends with its
    slowest rank), by an all-reduce over the default process group."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, ms: float) -> float:
    """Units per second of the whole job: every rank processes the same
    number of units (replicas, weak scaling) in at most `ms` per step."""
    return units_per_rank * world / (ms / 1e3)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    t, cj, cfg, x0s, meta = workload(args)
    from oracle import oracle

    oracle.build()
    vals = []
    for i in range(args.warmup + args.steps):
        v, cores, dt = cpu_sample(cfg, t, x0s[i % len(x0s)], meta, args.ref_step_ticks)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    sample = f"1 instance x {args.ref_step_ticks} tick(s) of the {args.side}x{args.side} workload per step"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * cfg.nx * cfg.ny * args.ref_step_ticks / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(args, cfg), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from jacobi2000_gb300 import engine
    from jacobi2000_gb300.checkpoint import write_safetensors_bytes

    t, cj, cfg, x0s, meta = workload(args)
    prec = engine.BF16 if args.precision == "bf16" else engine.FP32
    model = engine.Model.from_bytes(write_safetensors_bytes(t), cj, prec)
    cells = cfg.nx * cfg.ny
    B, H = args.instances, args.ticks
    batch = engine.Batch([model], max_instances=B, max_cells=B * cells)
    me = engine.PROJECT_MASS | engine.PROJECT_ENERGY
    host_items = [(0, x, meta, H, me) for x in x0s]

    # device-resident inputs
    dx0 = [torch.from_numpy(x).cuda() for x in x0s]
    dmeta = torch.from_numpy(meta).cuda()
    dout = [torch.empty_like(x) for x in dx0]
    dev_items = [(0, x.data_ptr(), dmeta.data_ptr(), H, me, o.data_ptr()) for x, o in zip(dx0, dout)]
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        batch.rollout(dev_items, device=True, stream=sptr)
    barrier()
    # the raw nvidia-smi samples go to $JC_BENCH_OUT (default: the system's temp folder)
    out_dir = Path(os.environ.get("JC_BENCH_OUT") or tempfile.gettempdir())
    out_dir.mkdir(parents=True, exist_ok=True)
    clocks = Clocks(out_dir / f"clocks_rank{rank}.csv")
    with clocks:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            batch.rollout(dev_items, device=True, stream=sptr)
        ev1.record(stream)
        barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, world, "cuda")
    value = whole_job_rate(B * cells * H, world, ms)

    # end to end through the C ABI with host buffers
    for _ in range(2):
        batch.rollout(host_items)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batch.rollout(host_items)
    barrier()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world, "cuda")
    h2d = B * (x0s[0].nbytes + meta.nbytes)
    d2h = B * (x0s[0].nbytes + 32)

    # the plain FP32 single-request path, one rollout at a time
    plain = engine.Model.from_bytes(write_safetensors_bytes(t), cj, engine.FP32)
    plain.rollout(x0s[0], meta, H, me)
    n_plain = min(B, 8)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(n_plain):
        plain.rollout(x0s[i], meta, H, me)
    plain_s = (time.perf_counter() - t0) / n_plain
    plain_value = cells * H / plain_s

    # per-kernel device times (events on the launching stream, outside graphs)
    prof = batch.profile(dev_items, device=True)
    launches_per_step = sum(n for n, _ in prof.values())
    pk, pk_kind = peaks()
    total_ms = sum(v[1] for v in prof.values())
    table = {}
    for kname, (nl, tot) in prof.items():
        kind, amount = kernel_work(kname, B, cells, args.dim, 4 * args.dim)
        avg_s = tot / nl / 1e3
        if kind == "flop":
            table[kname] = {"tflops": amount / avg_s / 1e12, "avg_ms": avg_s * 1e3, "share": tot / total_ms}
        elif kind == "byte":
            table[kname] = {"gbs": amount / avg_s / 1e9, "avg_ms": avg_s * 1e3, "share": tot / total_ms}
    name, (nl, tot_ms) = max(prof.items(), key=lambda kv: kv[1][1])
    kind, amount = kernel_work(name, B, cells, args.dim, 4 * args.dim)
    avg_s = tot_ms / nl / 1e3
    traffic = ncu_traffic().get(name)
    if kind == "flop" and name.startswith("tc_"):
        peak = pk["bf16_tflops"]
        roof = {"bound": "tensor", "kernel": name, "achieved": amount / avg_s / 1e12, "peak": peak,
                "unit": "TFLOP/s", "frac": amount / avg_s / 1e12 / peak, "traffic": traffic,
                "peak_kind": f"{pk_kind} bf16 dense burst", "flop_per_launch": amount}
    elif kind == "flop":
        peak = 152 * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
        roof = {"bound": "fp32-simt", "kernel": name, "achieved": amount / avg_s / 1e12, "peak": peak,
                "unit": "TFLOP/s", "frac": amount / avg_s / 1e12 / peak, "traffic": traffic,
                "peak_kind": "nominal FP32 FMA rate (152 SMs x 128 lanes x 2 x max SM clock)",
                "flop_per_launch": amount}
    else:
        peak = pk["hbm_gbs"]
        roof = {"bound": "hbm", "kernel": name, "achieved": amount / avg_s / 1e9, "peak": peak, "unit": "GB/s",
                "frac": amount / avg_s / 1e9 / peak, "traffic": traffic, "peak_kind": f"{pk_kind} copy bandwidth",
                "bytes_per_launch": amount}
    roof.update({"avg_launch_ms": avg_s * 1e3, "share": tot_ms / total_ms})

    served = served_bench(args) if rank == 0 else None
    mixed = mixed_batch_bench(args) if rank == 0 and not args.no_mixed else None
    accuracy = accuracy_c3() if rank == 0 and not args.no_accuracy else None
    evalm = eval_bench(args) if rank == 0 and not args.no_eval else None

    cpu = None
    if rank == 0:
        v, cores, dt = cpu_sample(cfg, t, x0s[0], meta, args.cpu_sample_ticks)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"1 instance x {args.cpu_sample_ticks} tick(s), {dt:.1f} s"}
        if args.cpu_sample_ticks_1t > 0:
            v1, _, dt1 = cpu_sample(cfg, t, x0s[0], meta, args.cpu_sample_ticks_1t, threads=1)
            cpu["one_thread"] = {"value": v1, "unit": UNIT, "cores": 1,
                                 "sample": f"1 instance x {args.cpu_sample_ticks_1t} tick(s), {dt1:.1f} s"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32" if prec == engine.FP32 else "bf16", "data": "synthetic",
                "config": config_dict(args, cfg),
                "e2e": {"value": whole_job_rate(B * cells * H, world, 1e3 * e2e_s), "unit": UNIT,
                        "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "fp32_plain": {"value": plain_value, "unit": UNIT, "ms_per_rollout": plain_s * 1e3,
                               "note": f"one {args.side}x{args.side} rollout of {H} ticks at a time"},
                "roofline": roof, "cpu_baseline": cpu, "clocks": clocks.summary(local), "served": served,
                "mixed_batch": mixed, "accuracy": accuracy, "eval_metrics": evalm,
                "gpu_launches": launches_per_step * args.steps,
                "kernels": table, "peaks": pk_kind}
        print(json.dumps(line), flush=True)
    batch.close()
    model.close()
    plain.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
