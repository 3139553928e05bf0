"""Synthetic shallow-water initial conditions, normalized for the model.

A drop is the reference solver's Gaussian bump (crates/solvers/src/shallow_water.rs:102-111:
``h += amp * exp(-(dx^2 + dy^2) / (2 sigma^2))`` with cell-unit offsets), summed
over the periodic images of the box so the field wraps. The normalized state is
``norm.rs:27-34``'s encoding: ``[(h - depth - mean0)/std0, (u - mean1)/std1,
(v - mean2)/std2]`` in a ``[3, ny, nx]`` f32 array.
"""

from __future__ import annotations

import numpy as np

from .checkpoint import ModelConfig


def drops_field(nx: int, ny: int, drops, depth: float = 1.0) -> np.ndarray:
    """Physical h [ny, nx] (f32) for a list of (cx, cy, amp, sigma) drops."""
    h = np.full((ny, nx), np.float32(depth), dtype=np.float32)
    ys, xs = np.meshgrid(np.arange(ny, dtype=np.float32), np.arange(nx, dtype=np.float32), indexing="ij")
    for cx, cy, amp, sigma in drops:
        inv = np.float32(1.0) / (np.float32(2.0) * np.float32(sigma) * np.float32(sigma))
        for ox in (-nx, 0, nx):
            for oy in (-ny, 0, ny):
                dx = xs - np.float32(cx + ox)
                dy = ys - np.float32(cy + oy)
                h += np.float32(amp) * np.exp(-(dx * dx + dy * dy) * inv)
    return h


def encode(cfg: ModelConfig, h: np.ndarray, u: np.ndarray | None = None, v: np.ndarray | None = None) -> np.ndarray:
    """norm.rs:27-34."""
    u = np.zeros_like(h) if u is None else u
    v = np.zeros_like(h) if v is None else v
    f = np.float32
    m, s, d = cfg.norm_mean, cfg.norm_std, cfg.norm_depth
    x = np.empty((3,) + h.shape, dtype=np.float32)
    x[0] = (h - f(d) - f(m[0])) / f(s[0])
    x[1] = (u - f(m[1])) / f(s[1])
    x[2] = (v - f(m[2])) / f(s[2])
    return x


def single_drop(cfg: ModelConfig, seed: int, amp: float = 0.1, sigma: float = 3.0) -> np.ndarray:
    """One drop of fixed amplitude and width, centre uniform from ``seed``."""
    rng = np.random.default_rng(seed)
    cx, cy = rng.uniform(0, cfg.nx), rng.uniform(0, cfg.ny)
    return encode(cfg, drops_field(cfg.nx, cfg.ny, [(cx, cy, amp, sigma)], cfg.depth))


def random_drops(cfg: ModelConfig, seed: int, n_drops: int = 8, amp=(0.02, 0.15), sigma=(2.0, 6.0)) -> np.ndarray:
    """``n_drops`` drops, amplitude U[amp], sigma U[sigma] cells, centres uniform."""
    rng = np.random.default_rng(seed)
    drops = [(rng.uniform(0, cfg.nx), rng.uniform(0, cfg.ny), rng.uniform(*amp), rng.uniform(*sigma))
             for _ in range(n_drops)]
    return encode(cfg, drops_field(cfg.nx, cfg.ny, drops, cfg.depth))


def probe_input(channels: int, nx: int, ny: int) -> np.ndarray:
    """The sinusoid probe of training/jacobi2000_pt/parity.py:34-46 and
    crates/engine/examples/bench.rs:16-25."""
    x = np.zeros((channels, ny, nx), dtype=np.float32)
    ys, xs = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    for c in range(channels):
        x[c] = ((c + 1) * 0.05 * np.sin(2 * np.pi * (c + 1) * xs / nx) * np.cos(2 * np.pi * ys / ny)).astype(np.float32)
    return x
