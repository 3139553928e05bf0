"""Helpers shared by the tests."""

import json

import numpy as np


def r2d2_config(config_json: str) -> str:
    c = json.loads(config_json)
    c["mask"] = {"Stencil": {"radius": 2, "dilation": 2}}
    return json.dumps(c)


def normwise(a, b) -> float:
    """max|a - b| / max|b|, the per-field error measure."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def field_errors(a, b):
    """normwise error of each of the h, u, v fields of [3, ny, nx] states."""
    return [normwise(a[i], b[i]) for i in range(3)]
