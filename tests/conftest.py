"""Shared pytest configuration.

Tests marked ``gpu`` need a CUDA device and the compiled ``libpynof_gb300.so``;
everything else runs on the CPU.
"""
import os
import sys
import types

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the compiled CUDA library")
    config.addinivalue_line("markers", "slow: larger CPU cases")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


def param_for(name, **over):
    from pynof_gb300 import synthetic

    st = synthetic.structure(name)
    for k, v in over.items():
        setattr(st, k, v)
    return st


def nrel(a, b):
    """Normwise relative error max|a-b| / max|b|.

    Element-wise relative error is ill-posed for these arrays (entries span
    tens of decades and K_i has exact zeros), so every parity check uses this
    normwise measure.
    """
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


GOLDEN_CASES = {"c1": "c1", "water": "water", "ragged": "ragged"}
