"""Throughput of the shallow-water transformer on GB300, served.

Workload (the metric's configuration): a request loop with continuous
batching on one GPU. Requests arrive as a Poisson stream (rates swept over
10-2000 req/s); grid side log-uniform in [32, 256] rounded to a multiple of 4
(one checkpoint per side, dim 128, 4 layers, random init: a forward family,
seed 0, and a reverse family, seed 1); horizon U[10, 50] ticks; 1/3 forward,
1/3 rewind, 1/3 reconstruct (2% of the space-time cells known, 4 Jacobi
sweeps); mass and energy projection each tick; admission at 80% of HBM.
Metric: useful cell-ticks/s = sum over requests of nx * ny * horizon /
seconds. One step = one served run of N requests arriving at 2000 req/s (the
saturating rate).

* ``value``: the BF16 served form with inputs already in device memory
  (requests carry device pointers), timed on the device: CUDA events on the
  server's stream from the start of its first iteration to the end of its
  last, summed over the timed steps.
* ``e2e``: the same runs through the C ABI from the caller's page-locked
  host buffers (jc_server_submit / jc_server_wait with
  JC_REQUEST_DEVICE_BUFFERS): wall clock from the first arrival to the last
  result in host memory, every request's host->device and device->host
  copies inside. ``served.pageable_host_buffers``: the same from pageable
  numpy buffers, which the server stages.
* ``served.rates``: throughput and p50/p99 latency per arrival rate (host
  buffers).
* ``fp32_plain``: the plain FP32 kernel path, one request at a time; and
  ``served_vs_plain`` = value / its throughput.
* ``batched``: 64 instances of a 128x128 grid x 50 ticks in one batch call;
  the per-kernel table and the roofline of the dominant kernel come from it.
* ``--impl reference``: the reference's CPU forward pass and projections (the
  C restatement of crates/engine/src/cpu.rs and project.rs, with the
  reference's own O(T^2) masked attention scan) on a bounded sample of the
  same requests, on the host cores.

Under torchrun each rank serves its own requests (no exchange step): weak
scaling, barrier + max over ranks.
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
    ap.add_argument("--dim", type=int, default=128)
    ap.add_argument("--layers", type=int, default=4)
    ap.add_argument("--requests", type=int, default=400,
                    help="served requests per step at the saturating rate")
    ap.add_argument("--sweep-seconds", type=float, default=3.0,
                    help="arrival time per rate of the 10-2000 req/s sweep (at least 40 requests per rate)")
    ap.add_argument("--plain-requests", type=int, default=120,
                    help="requests of the FP32 one-request-at-a-time run")
    ap.add_argument("--cpu-requests", type=int, default=12,
                    help="requests of the served workload in the CPU sample (each at most 5 ticks)")
    ap.add_argument("--ref-requests", type=int, default=4,
                    help="requests of the served workload per step of the --impl reference arm")
    ap.add_argument("--ref-horizon", type=int, default=5,
                    help="ticks of each request run by the CPU sample (the rest of its horizon is not run)")
    # the batched extra: B instances of one grid, one rollout per step
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--side", type=int, default=128)
    ap.add_argument("--ticks", type=int, default=50)
    ap.add_argument("--no-sweep", action="store_true", help="skip the arrival-rate sweep")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-task batch measurement")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the 256x256 error report against the f64 oracle")
    ap.add_argument("--no-eval", action="store_true", help="skip the eval-metrics measurement")
    ap.add_argument("--only-served", action="store_true",
                    help="the served steps alone (for profiling): no FP32, batched, CPU or accuracy runs")
    ap.add_argument("--only-batched", action="store_true",
                    help="the batched extra alone (for profiling): --instances x --side^2 grids, --ticks ticks; "
                         "prints its JSON and exits")
    return ap.parse_args()


def workload(args):
    from jacobi2000_gb300.checkpoint import parse_config, synthetic_checkpoint, meta_of
    from jacobi2000_gb300.ic import random_drops

    t, cj = synthetic_checkpoint(args.side, args.dim, args.layers, 0)
    cfg = parse_config(cj, t)
    rank = int(os.environ.get("RANK", "0"))
    x0s = [random_drops(cfg, seed=rank * 100_000 + i) for i in range(args.instances)]
    return t, cj, cfg, x0s, meta_of(cfg)


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
            "tc_proj_mlp": 2 * R * D * D + 4 * R * D * F,
            "tc_token_mix": 18 * R * D * D, "tc_to_cells": 2 * R * D * 32, "tc_conv1": 2 * N * 35 * 9 * 32,
            "f32_ln_qkv": 2 * R * D * 3 * D, "f32_proj": 2 * R * D * D, "f32_ln_ff1": 2 * R * D * F,
            "f32_ff2": 2 * R * F * D, "f32_token_mix": 18 * R * D * D, "f32_to_cells": 2 * R * D * 32,
            "f32_conv1": 2 * N * 35 * 9 * 32, "tc_conv2": 2 * N * 32 * 9 * 3, "f32_conv2_step": 2 * N * 32 * 9 * 3}
    byte = {"bf_attention": R * (3 * D * 2 + D * 2), "bf_embed": N * 12 + R * (4 * D + 2 * D),
            "bf_upsample": R * 32 * 4 + N * (12 + 96), "projection": N * 12 * 4 + N * 12,
            "f32_attention": R * (3 * D * 4 + D * 4), "f32_embed": N * 12 + R * 4 * D,
            "f32_upsample_concat": R * 32 * 4 + N * (12 + 144), "f32_final_ln": R * D * 8}
    if name in flop:
        return "flop", flop[name]
    if name in byte:
        return "byte", byte[name]
    return None, None


PER_LAYER = ("tc_qkv", "bf_attention", "tc_proj_ln", "tc_mlp", "tc_proj_mlp")


def work_table(prof, cells, proj_cells, D, F, L, pk, pk_kind, where):
    """Per-kernel rates from a profile {name: (launches, total ms)} of work that
    stepped `cells` forward cell-ticks in all (`proj_cells` of them projected):
    algorithmic FLOPs (contractions) or compulsory bytes (memory-bound
    kernels) summed over the launches, over the kernel's total device time;
    and the roofline of the kernel with the largest share."""
    total_ms = sum(v[1] for v in prof.values())
    table, best = {}, None
    for name, (n, ms) in prof.items():
        kind, amount = kernel_work(name, 1, proj_cells if name == "projection" else cells, D, F)
        if kind is None:
            table[name] = {"launches": n, "total_ms": ms, "share": ms / total_ms}
            continue
        amount *= L if name in PER_LAYER else 1
        rate = amount / (ms / 1e3)
        row = {"launches": n, "total_ms": ms, "avg_ms": ms / n, "share": ms / total_ms}
        row.update({"tflops": rate / 1e12} if kind == "flop" else {"gbs": rate / 1e9})
        table[name] = row
        if best is None or ms > best[2]:
            best = (name, kind, ms, amount, n)
    name, kind, ms, amount, n = best
    traffic = ncu_traffic().get(name)
    if traffic is not None:  # ncu bytes of one launch over 64 x 128x128 cells, scaled to this run's average launch
        traffic *= (amount / n) / (kernel_work(name, 64, 128 * 128, D, F)[1])
    if kind == "flop":
        ach = amount / (ms / 1e3) / 1e12
        roof = {"bound": "tensor", "kernel": name, "achieved": ach, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": ach / pk["bf16_tflops"], "traffic": traffic, "peak_kind": f"{pk_kind} bf16 dense burst",
                "flop_per_launch": amount / n}
    else:
        ach = amount / (ms / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": name, "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": ach / pk["hbm_gbs"], "traffic": traffic, "peak_kind": f"{pk_kind} copy bandwidth",
                "bytes_per_launch": amount / n}
    roof.update({"avg_launch_ms": ms / n, "share": ms / total_ms, "measured_on": where})
    return table, roof


# ---- the served workload (the metric's configuration) ------------------------------------

C5_SIDES = list(range(32, 257, 4))  # grid sides: log-uniform in [32, 256], rounded to a multiple of 4
C5_RATES = [10.0, 40.0, 100.0, 400.0, 1000.0, 2000.0]
C5_SWEEPS = 4         # reconstruct: Jacobi sweeps (tolerance 0: every sweep runs)
C5_KNOWN = 0.02       # reconstruct: fraction of space-time cells known
C5_MAX_CELLS = 8 << 20
C5_HBM = 0.8


class C5:
    """Requests of the serving configuration: Poisson arrivals at `rate`;
    grid side log-uniform in [32, 256] rounded to a multiple of 4; horizon
    U[10, 50] ticks; tasks 1/3 forward (initial state known), 1/3 rewind
    (final state known), 1/3 reconstruct (2% of the space-time cells known as
    sensor readings of a drop field, the rest blank). Inputs are made from the
    request's own seed, so a request list is reproducible."""

    def __init__(self, cfgs):
        self.cfgs = cfgs
        self._states = {}

    @staticmethod
    def draw(seed: int, n: int, rate: float):
        rng = np.random.default_rng(seed)
        out, t = [], 0.0
        for _ in range(n):
            t += rng.exponential(1.0 / rate)
            side = float(np.exp(rng.uniform(np.log(32.0), np.log(256.0))))
            g = int(np.clip(round(side / 4.0) * 4, 32, 256) - 32) // 4
            out.append({"arrival": t, "task": int(rng.integers(0, 3)), "g": g, "ticks": int(rng.integers(10, 51)),
                        "seed": int(rng.integers(1 << 30))})
        return out

    def side(self, r):
        return C5_SIDES[r["g"]]

    def state(self, g: int, k: int):
        from jacobi2000_gb300.ic import random_drops

        key = (g, k % 2)
        if key not in self._states:
            self._states[key] = random_drops(self.cfgs[g], seed=1000 * g + k % 2)
        return self._states[key]

    def inputs(self, r):
        """(x, known): x is [3, n, n] (forward / rewind) or the values [H+1, 3,
        n, n] (reconstruct, zero where unknown) with its mask known [H+1, n, n]."""
        from jacobi2000_gb300 import engine

        if r["task"] != engine.TASK_RECONSTRUCT:
            return self.state(r["g"], r["seed"]), None
        n, H = self.side(r), r["ticks"]
        known = (np.random.default_rng(r["seed"]).random((H + 1, n, n)) < C5_KNOWN).astype(np.uint8)
        vals = np.where(known[:, None], self.state(r["g"], r["seed"])[None], np.float32(0.0)).astype(np.float32)
        return vals, known

    def useful(self, reqs):
        return sum(self.side(r) ** 2 * r["ticks"] for r in reqs)

    def projected(self, reqs):
        """Cell-ticks of the forward and rewind requests (the projected ones)."""
        from jacobi2000_gb300 import engine

        return sum(self.side(r) ** 2 * r["ticks"] for r in reqs if r["task"] != engine.TASK_RECONSTRUCT)

    def work(self, reqs):
        """Forward cell-ticks the requests cost (a reconstruct sweep steps 2H slices)."""
        from jacobi2000_gb300 import engine

        return sum(self.side(r) ** 2 * r["ticks"] * (2 * C5_SWEEPS if r["task"] == engine.TASK_RECONSTRUCT else 1)
                   for r in reqs)


def c5_models(args, precision):
    """The forward and the reverse checkpoint family (seeds 0 and 1; one model
    per grid side, every tensor but `pos` shared) at `precision`."""
    from jacobi2000_gb300 import engine
    from jacobi2000_gb300.checkpoint import synthetic_family, write_safetensors_bytes

    fams = [synthetic_family(args.dim, args.layers, seed, C5_SIDES) for seed in (0, 1)]
    return [[engine.Model.from_bytes(write_safetensors_bytes(f[(s, s)][0]), f[(s, s)][1], precision)
             for s in C5_SIDES] for f in fams]


def c5_configs(args):
    from jacobi2000_gb300.checkpoint import parse_config, synthetic_family

    fam = synthetic_family(args.dim, args.layers, 0, C5_SIDES)
    return [parse_config(fam[(s, s)][1], fam[(s, s)][0]) for s in C5_SIDES]


def run_served(srv, wl, reqs, metas, device=False, concurrent=True, pinned=False):
    """Submits `reqs` at their arrival times (concurrent) or one after the
    previous result (sequential) and collects every result. Host mode: host
    buffers (numpy, pageable) in and out through jc_server_submit /
    jc_server_wait, which stage them. Pinned mode: the caller's page-locked
    host buffers, read and written by DMA (JC_REQUEST_DEVICE_BUFFERS). Device
    mode: inputs already in device memory, results copied to device memory.
    Latency per request is the server's submit to completion time plus how
    late the submission was."""
    import threading

    from jacobi2000_gb300 import engine

    ins = [wl.inputs(r) for r in reqs]
    h2d = sum(x.nbytes + (k.nbytes if k is not None else 0) + metas[r["g"]].nbytes for r, (x, k) in zip(reqs, ins))
    d2h = sum(x.nbytes for x, _ in ins)
    dev = None
    if device or pinned:
        import torch

        put = (lambda a: torch.from_numpy(a).pin_memory()) if pinned else (lambda a: torch.from_numpy(a).cuda())
        dev = [(put(x), put(k) if k is not None else None, put(metas[r["g"]]),
                torch.empty(x.shape, pin_memory=True) if pinned else torch.empty(x.shape, device="cuda"))
               for r, (x, k) in zip(reqs, ins)]
        torch.cuda.synchronize()
        device = True
    srv.reset_stats()
    lat = [None] * len(reqs)
    ids = [None] * len(reqs)
    late = [0.0] * len(reqs)

    def submit(k, r):
        x, known = ins[k]
        if device:
            dx, dk, dm, _ = dev[k]
            return srv.submit_device(r["task"], r["g"], dx.data_ptr(), dm.data_ptr(), r["ticks"],
                                     known_ptr=dk.data_ptr() if dk is not None else None, max_sweeps=C5_SWEEPS,
                                     tol=0.0)
        return srv.submit(r["task"], r["g"], x, metas[r["g"]], r["ticks"], known=known, max_sweeps=C5_SWEEPS, tol=0.0)

    def collect(k, r):
        if device:
            o = dev[k][3]
            info = srv.wait_device(ids[k], o.data_ptr(), o.numel(), timeout=600)
        else:
            _, info = srv.wait(ids[k], r["task"], r["g"], r["ticks"], timeout=600)
        lat[k] = info["latency_s"] + late[k]

    t0 = time.perf_counter()
    if concurrent:
        def collector():
            for k, r in enumerate(reqs):
                while ids[k] is None:
                    time.sleep(0.0002)
                collect(k, r)

        th = threading.Thread(target=collector)
        th.start()
        for k, r in enumerate(reqs):
            delay = t0 + r["arrival"] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            late[k] = max(0.0, time.perf_counter() - (t0 + r["arrival"]))
            ids[k] = submit(k, r)
        th.join()
    else:
        for k, r in enumerate(reqs):
            ids[k] = submit(k, r)
            collect(k, r)
    wall = time.perf_counter() - t0
    st = srv.stats()
    useful = wl.useful(reqs)
    lat_ms = np.array(lat) * 1e3
    return {"requests": len(reqs), "useful_cell_ticks": useful, "work_cell_ticks": wl.work(reqs),
            "wall_s": wall, "device_span_s": st["device_span_s"], "cell_ticks_per_s_wall": useful / wall,
            "cell_ticks_per_s_device": useful / st["device_span_s"] if st["device_span_s"] > 0 else None,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
            "iterations": st["iterations"], "launches": st["launches"], "h2d_bytes": h2d, "d2h_bytes": d2h}


def cpu_served_sample(args, n_requests: int, seed: int, threads: int = 0, horizon_cap: int = 5):
    """The reference's CPU forward (the oracle's f32 restatement with the
    reference's O(T^2) masked attention scan) on a bounded sample of the
    served workload, one request at a time on `threads` host threads (0: all
    cores). Each request runs at most `horizon_cap` ticks of its horizon (a
    reconstruct: one of its sweeps over that window) and is credited with the
    useful cell-ticks that part of it is worth (a reconstruct sweep 1/4 of its
    window's cell-ticks), so the rate is the full workload's rate."""
    from jacobi2000_gb300 import engine
    from jacobi2000_gb300.checkpoint import meta_of, parse_config, synthetic_family
    from oracle import oracle

    oracle.set_threads(threads or os.cpu_count() or 1)
    oracle.set_attention_mode("scan")
    reqs = C5.draw(seed, n_requests, 1000.0)
    sides = sorted({C5_SIDES[r["g"]] for r in reqs})
    fams = [synthetic_family(args.dim, args.layers, s, sides) for s in (0, 1)]
    cfgs = {sd: parse_config(fams[0][(sd, sd)][1], fams[0][(sd, sd)][0]) for sd in sides}
    wl = C5([cfgs.get(sd) for sd in C5_SIDES])
    credited, elapsed = 0.0, 0.0
    for r in reqs:
        sd, H = C5_SIDES[r["g"]], min(r["ticks"], horizon_cap)
        fo = oracle.OracleModel(cfgs[sd], fams[0][(sd, sd)][0])
        ro = oracle.OracleModel(cfgs[sd], fams[1][(sd, sd)][0])
        meta = meta_of(cfgs[sd])
        x, known = wl.inputs(dict(r, ticks=H))
        t0 = time.perf_counter()
        if r["task"] == engine.TASK_RECONSTRUCT:
            oracle.reconstruct(fo, ro, x, known, meta, 1)
            credited += sd * sd * H / C5_SWEEPS
        else:
            (fo if r["task"] == engine.TASK_FORWARD else ro).rollout(x, meta, H, oracle.MASS | oracle.ENERGY)
            credited += sd * sd * H
        elapsed += time.perf_counter() - t0
    return credited / elapsed, oracle.get_threads(), elapsed, len(reqs)


def served_config(n_requests: int):
    return {"workload": f"served: Poisson arrivals at {C5_RATES[-1]:.0f} req/s (the saturating rate of the 10-2000 "
                        f"req/s sweep), {n_requests} requests per step; grid side log-uniform 32-256 rounded to a "
                        f"multiple of 4, horizon U[10,50] ticks; 1/3 forward, 1/3 rewind, 1/3 reconstruct "
                        f"({C5_KNOWN:.0%} of space-time cells known, {C5_SWEEPS} Jacobi sweeps); mass+energy "
                        f"projection; continuous batching, admission at {C5_HBM:.0%} of HBM and "
                        f"{C5_MAX_CELLS >> 20}M cells per tick",
            "model": "jacobi2000 dim 128, 4 layers, 4 heads, stencil r1 d1; forward family seed 0, reverse family "
                     "seed 1 (one checkpoint per side, every tensor but pos shared)",
            "sides": [C5_SIDES[0], C5_SIDES[-1], 4], "requests_per_step": n_requests,
            "l2": "per-tick working set of the active requests > 129 MB L2 (no flush needed)",
            "parallelism": "replicas"}


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
    """The reference arm: the reference's CPU forward (the oracle's f32
    restatement, O(T^2) masked attention scan) on a bounded sample of the
    served workload per step, on every host core; rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle

    oracle.build()
    vals, cores, secs = [], 1, 0.0
    for i in range(args.warmup + args.steps):
        v, cores, dt, n = cpu_served_sample(args, args.ref_requests, seed=500 + i, horizon_cap=args.ref_horizon)
        if i >= args.warmup:
            vals.append(v)
            secs += dt
    value = statistics.median(vals)
    sample = (f"{args.ref_requests} requests of the served workload per step, one at a time, each at most "
              f"{args.ref_horizon} ticks "
              f"(a reconstruct: one sweep of that window, credited 1/4 of its cell-ticks)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / max(1, args.steps),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": served_config(args.requests), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batched_bench(args, world, barrier):
    """The batched extra: B instances of one grid (side x side), `ticks`
    ticks with mass+energy projection, one batch call per step, device
    buffers (CUDA events) and host buffers (wall clock); the per-kernel table
    and the roofline of the dominant kernel."""
    import torch

    from jacobi2000_gb300 import engine
    from jacobi2000_gb300.checkpoint import write_safetensors_bytes

    t, cj, cfg, x0s, meta = workload(args)
    model = engine.Model.from_bytes(write_safetensors_bytes(t), cj, engine.BF16)
    cells = cfg.nx * cfg.ny
    B, H = args.instances, args.ticks
    batch = engine.Batch([model], max_instances=B, max_cells=B * cells)
    me = engine.PROJECT_MASS | engine.PROJECT_ENERGY
    host_items = [(0, x, meta, H, me) for x in x0s]
    dx0 = [torch.from_numpy(x).cuda() for x in x0s]
    dmeta = torch.from_numpy(meta).cuda()
    dout = [torch.empty_like(x) for x in dx0]
    dev_items = [(0, x.data_ptr(), dmeta.data_ptr(), H, me, o.data_ptr()) for x, o in zip(dx0, dout)]
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    for _ in range(2):
        batch.rollout(dev_items, device=True, stream=sptr)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = 5
    ev0.record(stream)
    for _ in range(steps):
        batch.rollout(dev_items, device=True, stream=sptr)
    ev1.record(stream)
    barrier()
    ms = ev0.elapsed_time(ev1) / steps
    batch.rollout(host_items)
    t0 = time.perf_counter()
    for _ in range(2):
        batch.rollout(host_items)
    e2e_s = (time.perf_counter() - t0) / 2
    prof = batch.profile(dev_items, device=True)
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
    if kind == "flop":
        peak = pk["bf16_tflops"]
        roof = {"bound": "tensor", "kernel": name, "achieved": amount / avg_s / 1e12, "peak": peak,
                "unit": "TFLOP/s", "frac": amount / avg_s / 1e12 / peak, "traffic": traffic,
                "peak_kind": f"{pk_kind} bf16 dense burst", "flop_per_launch": amount}
    else:
        peak = pk["hbm_gbs"]
        roof = {"bound": "hbm", "kernel": name, "achieved": amount / avg_s / 1e9, "peak": peak, "unit": "GB/s",
                "frac": amount / avg_s / 1e9 / peak, "traffic": traffic, "peak_kind": f"{pk_kind} copy bandwidth",
                "bytes_per_launch": amount}
    roof.update({"avg_launch_ms": avg_s * 1e3, "share": tot_ms / total_ms,
                 "measured_on": f"the batched extra ({B} x {args.side}x{args.side}, one tick's launches timed with "
                                f"CUDA events on the launching stream)"})
    rate = B * cells * H / (ms / 1e3)
    flop = FLOP_PER_CELL_TICK.get((args.dim, args.layers))
    out = {"workload": f"rollout {B}x {args.side}x{args.side} grids, {H} ticks, mass+energy projection, "
                       f"8 drops/instance, one batch call per step",
           "value": rate, "ms_per_step": ms, "e2e": B * cells * H / e2e_s,
           "tick_tflops": rate * flop / 1e12 if flop else None,
           "tick_frac_of_bf16_peak": rate * flop / 1e12 / pk["bf16_tflops"] if flop else None,
           "launches_per_step": sum(n for n, _ in prof.values())}
    batch.close()
    model.close()
    return out, roof, table


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
    from jacobi2000_gb300.checkpoint import meta_of

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    if args.only_batched:
        batched, broof, btable = batched_bench(args, world, barrier)
        if rank == 0:
            batched.update({"roofline": broof, "kernels": btable})
            print(json.dumps(batched), flush=True)
        return
    pk, pk_kind = peaks()
    cfgs = c5_configs(args)
    metas = [meta_of(c) for c in cfgs]
    wl = C5(cfgs)
    fm, rm = c5_models(args, engine.BF16)
    srv = engine.Server(fm, rm, max_active_cells=C5_MAX_CELLS, hbm_fraction=C5_HBM)
    rate = C5_RATES[-1]
    step_reqs = C5.draw(7 + 1000 * rank, args.requests, rate)
    # warm-up: the same requests (tunes and allocates outside the timed steps),
    # then requests one at a time, so the row buckets of small batches (low
    # arrival rates) are tuned before the rate sweep measures latency
    for _ in range(args.warmup):
        run_served(srv, wl, step_reqs, metas, device=True)
    run_served(srv, wl, C5.draw(3 + 1000 * rank, 24, rate), metas, concurrent=False)
    barrier()
    out_dir = Path(os.environ.get("JC_BENCH_OUT") or tempfile.gettempdir())
    out_dir.mkdir(parents=True, exist_ok=True)
    clocks = Clocks(out_dir / f"clocks_rank{rank}.csv")
    runs = []
    with clocks:
        for _ in range(args.steps):
            runs.append(run_served(srv, wl, step_reqs, metas, device=True))
        barrier()
    dev_s = sum(r["device_span_s"] for r in runs)
    ms = max_over_ranks(1e3 * dev_s / args.steps, world, "cuda")
    useful = wl.useful(step_reqs)
    value = whole_job_rate(useful, world, ms)
    launches = sum(r["launches"] for r in runs)
    # end to end through the C ABI from page-locked host buffers: every
    # request's inputs copied host -> device and its result device -> host
    # inside the timed wall time (after one untimed run of the same kind)
    run_served(srv, wl, step_reqs, metas, pinned=True)
    e2e_runs = [run_served(srv, wl, step_reqs, metas, pinned=True) for _ in range(2)]
    # and from pageable host buffers, which the server stages (one untimed run
    # first: its page-locked staging buffers are allocated on first use)
    run_served(srv, wl, step_reqs, metas, device=False)
    staged = run_served(srv, wl, step_reqs, metas, device=False)
    e2e_ms = max_over_ranks(1e3 * statistics.mean(r["wall_s"] for r in e2e_runs), world, "cuda")
    # one more step with CUDA events around every launch of the loop: the
    # per-kernel table and the roofline of the served workload's top kernel
    srv.profile_start()
    run_served(srv, wl, step_reqs, metas, device=True)
    sprof = srv.profile_stop()
    table, roof = work_table(sprof, wl.work(step_reqs), wl.projected(step_reqs), args.dim, 4 * args.dim,
                             args.layers, pk, pk_kind,
                             f"one served step ({args.requests} requests), CUDA events around each launch on the "
                             f"server's stream, outside the timed steps")

    served = None
    if rank == 0:
        served = {"saturating_rate_req_s": rate,
                  "device_buffers": {"p50_ms": statistics.median(r["p50_ms"] for r in runs),
                                     "p99_ms": statistics.median(r["p99_ms"] for r in runs),
                                     "iterations_per_step": statistics.mean(r["iterations"] for r in runs),
                                     "wall_s": statistics.mean(r["wall_s"] for r in runs),
                                     "work_cell_ticks_per_s": wl.work(step_reqs) / (dev_s / args.steps)},
                  "pinned_host_buffers": {k: e2e_runs[-1][k] for k in ("cell_ticks_per_s_wall", "p50_ms",
                                                                         "p99_ms", "wall_s", "device_span_s")},
                  "pageable_host_buffers": {k: staged[k] for k in ("cell_ticks_per_s_wall", "p50_ms", "p99_ms",
                                                                   "wall_s", "device_span_s")},
                  "rates": []}
        if not args.no_sweep:
            for r_ in C5_RATES:
                n = max(40, int(r_ * args.sweep_seconds))
                n = min(n, args.requests)
                res = run_served(srv, wl, C5.draw(int(r_) + 17, n, r_), metas)
                res["rate_req_s"] = r_
                served["rates"].append({k: res[k] for k in ("rate_req_s", "requests", "cell_ticks_per_s_wall",
                                                             "cell_ticks_per_s_device", "p50_ms", "p99_ms",
                                                             "wall_s")})
        served["work_per_useful"] = wl.work(step_reqs) / useful
    srv.close()
    for m in fm + rm:
        m.close()

    plain = None
    if rank == 0 and not args.only_served:
        fm32, rm32 = c5_models(args, engine.FP32)
        with engine.Server(fm32, rm32, max_active_cells=C5_MAX_CELLS, hbm_fraction=C5_HBM) as s32:
            preqs = C5.draw(99, args.plain_requests, rate)
            run_served(s32, wl, preqs[:6], metas, concurrent=False)
            r32 = run_served(s32, wl, preqs, metas, concurrent=False)
        for m in fm32 + rm32:
            m.close()
        flop = FLOP_PER_CELL_TICK.get((args.dim, args.layers))
        fp32_peak = 152 * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
        work_rate = r32["work_cell_ticks"] / r32["wall_s"]
        plain = {"value": r32["cell_ticks_per_s_wall"], "unit": UNIT, "requests": r32["requests"],
                 "p50_ms": r32["p50_ms"], "p99_ms": r32["p99_ms"],
                 "note": "FP32 kernels, one request at a time (each submitted after the previous result), "
                         "same request distribution, host buffers",
                 "roofline": {"bound": "fp32-simt", "achieved": work_rate * flop / 1e12 if flop else None,
                              "peak": fp32_peak, "unit": "TFLOP/s",
                              "frac": work_rate * flop / 1e12 / fp32_peak if flop else None,
                              "peak_kind": "nominal FP32 FMA rate (152 SMs x 128 lanes x 2 x max SM clock)",
                              "flop_per_cell_tick": flop}}
    batched = broof = btable = None
    if not args.only_served:
        batched, broof, btable = batched_bench(args, world, barrier)
        batched.update({"roofline": broof, "kernels": btable})
    extras = rank == 0 and not args.only_served
    mixed = mixed_batch_bench(args) if extras and not args.no_mixed else None
    accuracy = accuracy_c3() if extras and not args.no_accuracy else None
    evalm = eval_bench(args) if extras and not args.no_eval else None

    cpu = None
    if extras:
        v, cores, dt, n = cpu_served_sample(args, args.cpu_requests, seed=31)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{n} requests of the served workload, one at a time, each at most 5 ticks (a "
                         f"reconstruct: one sweep of that window, credited 1/4 of its cell-ticks), {dt:.1f} s"}
        v1, _, dt1, n1 = cpu_served_sample(args, 3, seed=32, threads=1, horizon_cap=2)
        cpu["one_thread"] = {"value": v1, "unit": UNIT, "cores": 1,
                             "sample": f"{n1} requests, each at most 2 ticks, {dt1:.1f} s"}

    if rank == 0:
        flop = FLOP_PER_CELL_TICK.get((args.dim, args.layers))
        h2d = e2e_runs[-1]["h2d_bytes"]
        d2h = e2e_runs[-1]["d2h_bytes"]
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "bf16", "data": "synthetic (seeded drops and sensor masks, "
                "random-init checkpoints)", "config": served_config(args.requests),
                "e2e": {"value": whole_job_rate(useful, world, e2e_ms), "unit": UNIT,
                        "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "served_vs_plain": value / plain["value"] if plain else None,
                "fp32_plain": plain, "served": served,
                "served_roofline": {"bound": "tensor", "achieved": served["device_buffers"]["work_cell_ticks_per_s"]
                                    * flop / 1e12 if flop else None, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                                    "frac": served["device_buffers"]["work_cell_ticks_per_s"] * flop / 1e12
                                    / pk["bf16_tflops"] if flop else None,
                                    "note": "every forward the served steps ran (reconstruct sweeps included) "
                                            "x useful FLOP per cell-tick, over the device span"},
                "roofline": roof, "cpu_baseline": cpu, "clocks": clocks.summary(local),
                "batched": batched, "kernels": table, "mixed_batch": mixed, "accuracy": accuracy,
                "eval_metrics": evalm, "gpu_launches": launches, "peaks": pk_kind}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
