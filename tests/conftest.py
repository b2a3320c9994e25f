"""Shared test setup.

`-m "not gpu"` runs here without a GPU: the oracle against the reference's
golden fixtures, the scene generator, host-side logic, and that the built
libraries load and export what include/*.h declares.  `-m gpu` runs the
CUDA path through the C ABI against the oracle and the fixtures.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "4d-image-segmentation-algorithm_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the product path")


@pytest.fixture(scope="session")
def built():
    """Build (incrementally) the solver libraries and the oracle."""
    import build as pkg_build
    import oracle as orc

    pkg_build.build()
    orc.build()
    return True


@pytest.fixture(scope="session")
def ss4d(built):
    import ss4d as m

    return m


@pytest.fixture(scope="session")
def oracle(built):
    import oracle as orc

    orc.set_threads(1)
    return orc


@pytest.fixture(scope="session")
def cuda(ss4d):
    """torch with a CUDA device, or skip (only ever reached by gpu tests)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name)) as d:
        return {k: d[k] for k in d.files}


def params_from_golden(ss4d_mod, d: dict):
    names = [str(n) for n in d["param_names"]]
    vals = d["params"]
    p = ss4d_mod.Params()
    for n, v in zip(names, vals):
        setattr(p, n, int(v) if n in ("maxNoGSIteration", "maxNoOfTimeSteps") else float(v))
    return p


def rel_err(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / den)
