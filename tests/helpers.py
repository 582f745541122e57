"""Shared helpers of the test suite."""
from __future__ import annotations

import glob
import os
import types

import numpy as np

from conftest import GOLDEN

import fixture_io  # noqa: E402  (tests/golden)


def fixtures():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_fixture(name):
    return fixture_io.load(os.path.join(GOLDEN, f"{name}.npz"))


def package_ns(device="cuda"):
    import diff_2d_fem_gb300 as D
    return types.SimpleNamespace(Model=D.Model, ImplicitIntegrator=D.ImplicitIntegrator, device=device)


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
