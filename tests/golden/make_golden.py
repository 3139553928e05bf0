"""Regenerates the golden fixtures in this directory. Runs only where the
reference checkout is present (it reads it, read-only); the fixtures it writes
are committed so the tests never need the reference at run time.

1. ``pt-tiny/``: the reference's own parity fixture, copied byte for byte from
   crates/engine/tests/fixtures/pt-tiny (checkpoint, both mask configs, and
   reference.safetensors with PyTorch's forward and 1/10/50-step rollouts,
   written by training/jacobi2000_pt/parity.py:77-109).
2. ``extra.safetensors``: further cases computed by importing the reference's
   PyTorch twin (training/jacobi2000_pt/model.py and project.py) on CPU:
   * ``r2d2_forward``: pt-tiny with a Stencil{radius 2, dilation 2} mask, the
     edge-clipping case crates/engine/tests/parity.rs:130-136 checks;
   * ``rect_*``: a 24x16 non-square synthetic checkpoint (dim 32, 2 layers,
     seed 5), forward in f32 and f64;
   * ``c1_*``: the 32x32 model20-shaped synthetic checkpoint (dim 128, 4 layers,
     seed 0) on a single drop: forward in f32 and f64, and 10 ticks of rollout
     without projection and with mass + energy projection (project.py's
     formulas evaluated in float64, state kept in f32).
   Synthetic checkpoints are regenerated at test time from their seeds by
   jacobi2000_gb300.checkpoint; ``extra.safetensors`` stores a checksum of
   each so a generator drift is caught.

Usage: python tests/golden/make_golden.py /path/to/reference
"""

from __future__ import annotations

import shutil
import sys
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from jacobi2000_gb300.checkpoint import (checksum, parse_config, read_safetensors, synthetic_checkpoint,  # noqa: E402
                                         synthetic_family, write_safetensors, meta_of)
from jacobi2000_gb300.ic import single_drop  # noqa: E402


def torch_model(ref_root: Path, cfg, tensors, dtype=torch.float32):
    sys.path.insert(0, str(ref_root / "training"))
    from jacobi2000_pt.model import Jacobi2000, Jacobi2000Config

    m = Jacobi2000(Jacobi2000Config(nx=cfg.nx, ny=cfg.ny, patch=cfg.patch, channels=cfg.channels, dim=cfg.dim,
                                    layers=cfg.layers, heads=cfg.heads, ff_mult=cfg.ff_inner // cfg.dim,
                                    meta_dim=cfg.meta_dim, head_dim=cfg.head_dim))
    m.load_state_dict({k: torch.from_numpy(np.array(v)) for k, v in tensors.items()}, strict=True)
    return m.to(dtype).eval()


def mask_for(ref_root: Path, m, cfg, dtype):
    from jacobi2000_pt.model import stencil_mask

    if cfg.mask_kind == 0:
        return None
    return stencil_mask(m.cfg, cfg.radius, cfg.dilation).to(dtype)


def main(ref_root: Path) -> None:
    src = ref_root / "crates/engine/tests/fixtures/pt-tiny"
    dst = HERE / "pt-tiny"
    dst.mkdir(exist_ok=True)
    for f in ("model.safetensors", "config.json", "config-full.json", "reference.safetensors"):
        shutil.copyfile(src / f, dst / f)

    out: dict[str, np.ndarray] = {}
    with torch.no_grad():
        # 1. pt-tiny, Stencil r2 d2
        t = read_safetensors(dst / "model.safetensors")
        r = read_safetensors(dst / "reference.safetensors")
        import json
        cj = json.loads((dst / "config.json").read_text())
        cj["mask"] = {"Stencil": {"radius": 2, "dilation": 2}}
        cfg = parse_config(cj, t)
        m = torch_model(ref_root, cfg, t)
        x = torch.from_numpy(r["state"]).unsqueeze(0)
        meta = torch.from_numpy(r["meta"]).unsqueeze(0)
        out["r2d2_forward"] = m.forward(x, meta, mask_for(ref_root, m, cfg, torch.float32))[0].numpy()

        # 2. non-square synthetic checkpoint, 24 x 16
        fam = synthetic_family(32, 2, 5, [], rect=[(24, 16)])
        t, cj = fam[(24, 16)]
        cfg = parse_config(cj, t)
        rng = np.random.default_rng(11)
        state = (0.5 * rng.standard_normal((3, 16, 24))).astype(np.float32)
        meta_np = meta_of(cfg)
        out["rect_state"] = state
        out["rect_meta"] = meta_np
        out["rect_checksum"] = checksum(t)
        for dt, name in ((torch.float32, "rect_forward_f32"), (torch.float64, "rect_forward_f64")):
            m = torch_model(ref_root, cfg, t, dt)
            out[name] = m.forward(torch.from_numpy(state).to(dt).unsqueeze(0),
                                  torch.from_numpy(meta_np).to(dt).unsqueeze(0),
                                  mask_for(ref_root, m, cfg, dt))[0].numpy().astype(
                np.float32 if dt == torch.float32 else np.float64)

        # 3. model20-shaped 32x32 synthetic checkpoint, one drop
        t, cj = synthetic_checkpoint(32, 128, 4, 0)
        cfg = parse_config(cj, t)
        state = single_drop(cfg, seed=0)
        meta_np = meta_of(cfg)
        out["c1_state"] = state
        out["c1_meta"] = meta_np
        out["c1_checksum"] = checksum(t)
        for dt, name in ((torch.float32, "c1_forward_f32"), (torch.float64, "c1_forward_f64")):
            m = torch_model(ref_root, cfg, t, dt)
            out[name] = m.forward(torch.from_numpy(state).to(dt).unsqueeze(0),
                                  torch.from_numpy(meta_np).to(dt).unsqueeze(0),
                                  mask_for(ref_root, m, cfg, dt))[0].numpy().astype(
                np.float32 if dt == torch.float32 else np.float64)

        from jacobi2000_pt.project import Denorm, energy, project_energy, project_mass, mass

        m = torch_model(ref_root, cfg, t, torch.float32)
        mask = mask_for(ref_root, m, cfg, torch.float32)
        tmeta = torch.from_numpy(meta_np).unsqueeze(0)
        x = torch.from_numpy(state).unsqueeze(0)
        for i in range(10):
            x = m.step(x, tmeta, mask)
        out["c1_rollout10_plain"] = x[0].numpy()

        d = Denorm(tuple(cfg.norm_mean), tuple(cfg.norm_std), cfg.norm_depth)
        x = torch.from_numpy(state).unsqueeze(0)
        x64 = x.double()
        mass0 = mass(x64)
        e_prev = energy(x64, d, cfg.g)
        for i in range(10):
            nxt = m.step(x, tmeta, mask).double()
            nxt = project_mass(nxt, mass0)
            nxt = project_energy(nxt, e_prev, d, cfg.g, cfg.energy_r_max)
            x = nxt.float()
            e_prev = energy(x.double(), d, cfg.g)
        out["c1_rollout10_projected"] = x[0].numpy()

    write_safetensors(HERE / "extra.safetensors", {k: np.asarray(v, dtype=np.float32) for k, v in out.items()
                                                    if not k.endswith("_f64")})
    np.savez_compressed(HERE / "extra_f64.npz", **{k: v for k, v in out.items() if k.endswith("_f64")})
    print("wrote", sorted(out))
    metrics_golden(ref_root)


def metrics_golden(ref_root: Path) -> None:
    """3. ``metrics.npz``: the eval-metrics scores of fixed fields, computed by
    the reference's Python scoring twin (training/jacobi2000_pt/metrics.py,
    the formulas of crates/engine/src/metrics.rs). A 48x40 solver-like state
    (two Gaussian drops on depth 1, small seeded u and v) is the truth; the
    model state is the same with the drops widened and shifted (a lagging,
    weaker wave) plus seeded noise."""
    sys.path.insert(0, str(ref_root / "training"))
    from jacobi2000_pt import metrics as M

    nx, ny, cx, cy = 48, 40, 22.3, 19.6
    mean = np.array([0.0008, 0.0004, 0.0005], dtype=np.float32)
    std = np.array([0.0063, 0.0138, 0.0135], dtype=np.float32)
    depth = np.float32(1.0)
    rng = np.random.default_rng(11)
    yy, xx = np.meshgrid(np.arange(ny, dtype=np.float32), np.arange(nx, dtype=np.float32), indexing="ij")

    def ring(r0, w, amp):
        r = np.sqrt((xx - np.float32(cx)) ** 2 + (yy - np.float32(cy)) ** 2)
        return (amp * np.exp(-((r - r0) ** 2) / (2 * w * w))).astype(np.float32)

    truth = np.zeros((3, ny, nx), dtype=np.float32)
    truth[0] = depth + ring(6.0, 1.5, 0.03) + ring(0.0, 2.0, -0.01)
    truth[1] = (0.01 * rng.standard_normal((ny, nx))).astype(np.float32)
    truth[2] = (0.01 * rng.standard_normal((ny, nx))).astype(np.float32)
    model_phys = np.zeros_like(truth)
    model_phys[0] = depth + ring(7.3, 1.8, 0.024) + ring(0.0, 2.2, -0.008) + \
        (0.001 * rng.standard_normal((ny, nx))).astype(np.float32)
    model_phys[1] = truth[1] + (0.002 * rng.standard_normal((ny, nx))).astype(np.float32)
    model_phys[2] = truth[2] + (0.002 * rng.standard_normal((ny, nx))).astype(np.float32)

    def encode(s):  # norm.rs:27-34, f32 element by element
        out = np.empty_like(s)
        out[0] = ((s[0] - depth) - mean[0]) / std[0]
        out[1] = (s[1] - mean[1]) / std[1]
        out[2] = (s[2] - mean[2]) / std[2]
        return out

    x = encode(model_phys)
    target = encode(truth)
    n = nx * ny
    sc = M.score(x.ravel(), target.ravel(), float(mean[0]), float(std[0]), nx, ny, cx, cy)
    ph = M.decode_h(x.ravel(), mean[0], std[0], n)
    th = M.decode_h(target.ravel(), mean[0], std[0], n)
    np.savez_compressed(HERE / "metrics.npz", nx=nx, ny=ny, cx=cx, cy=cy, norm_mean=mean, norm_std=std,
                        norm_depth=depth, truth=truth, x=x, target=target,
                        prof_model=M.radial_profile(ph, nx, ny, cx, cy), prof_truth=M.radial_profile(th, nx, ny, cx, cy),
                        row=np.array([sc.corr, sc.corr_h, sc.amplitude_ratio, sc.xcorr_lag, sc.bias], dtype=np.float64))
    print("wrote metrics.npz", sc)


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
