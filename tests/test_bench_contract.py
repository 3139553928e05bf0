"""The bench's JSON line contract, checked through its CPU reference arm (the
oracle's f32 rollout on the host cores): one line with the metric, the
timing keys, the configuration and the CPU baseline; ranks other than 0 of a
multi-process launch print nothing. The multi-rank timing (the slowest rank's
step, whole-job units) runs on two gloo processes."""

import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _run(extra_env=None, *args):
    env = dict(os.environ)
    env.update(extra_env or {})
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
           "--ref-requests", "2", "--ref-horizon", "1", *args]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_reference_arm_prints_one_contract_line():
    lines = _run()
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["unit"] == "cell-ticks/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1 and line["n_gpus"] == 1
    assert line["config"]["workload"] and line["config"]["sides"] == [32, 256, 4]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_print_nothing():
    assert _run({"RANK": "1", "WORLD_SIZE": "2"}) == []


def _ranks_worker(rank, world, port, q):
    import importlib.util

    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    ms = b.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")  # rank 1 is the slower one
    q.put((rank, ms, b.whole_job_rate(1000.0, world, ms)))
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_step_and_count_every_rank():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_ranks_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's 15 ms; 2 x 1000 units in 15 ms
    assert got == [(0, 15.0, 2000.0 / 0.015), (1, 15.0, 2000.0 / 0.015)]


def test_profiled_kernel_names_are_known_to_the_roofline():
    """Every kernel of the committed ncu traffic table has algorithmic work in
    the bench (so the roofline's `traffic` is found for it), and the per-layer
    kernels count once per layer."""
    sys.path.insert(0, str(ROOT))
    import bench

    traffic = bench.ncu_traffic()
    assert {"tc_proj_mlp", "bf_attention", "tc_qkv", "tc_conv1", "tc_conv2"} <= set(traffic)
    for name, nbytes in traffic.items():
        kind, amount = bench.kernel_work(name, 64, 128 * 128, 128, 512)
        assert kind in ("flop", "byte") and amount > 0, name
        assert nbytes > 0
    assert {"tc_qkv", "bf_attention", "tc_proj_mlp"} <= set(bench.PER_LAYER)
