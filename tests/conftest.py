"""Shared fixtures. Tests marked ``gpu`` need a CUDA device and the built
library; everything else runs on the CPU."""

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA library")


@pytest.fixture(scope="session")
def pt_tiny():
    """The reference's pt-tiny parity fixture (crates/engine/tests/fixtures/pt-tiny)."""
    from jacobi2000_gb300.checkpoint import read_safetensors

    d = GOLDEN / "pt-tiny"
    return {
        "dir": d,
        "tensors": read_safetensors(d / "model.safetensors"),
        "st_bytes": (d / "model.safetensors").read_bytes(),
        "config": (d / "config.json").read_text(),
        "config_full": (d / "config-full.json").read_text(),
        "ref": read_safetensors(d / "reference.safetensors"),
    }


@pytest.fixture(scope="session")
def extra():
    from jacobi2000_gb300.checkpoint import read_safetensors

    g = read_safetensors(GOLDEN / "extra.safetensors")
    g.update(dict(np.load(GOLDEN / "extra_f64.npz")))
    return g
