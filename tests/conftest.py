import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")
    config.addinivalue_line("markers", "slow: takes tens of seconds on the CPU")


@pytest.fixture(scope="session")
def native_lib():
    """Path of libamcl3d_gpu.so, built in-tree if missing (nvcc cross-compiles)."""
    from amcl3d_gb300 import build

    so = build.LIB / "libamcl3d_gpu.so"
    if not so.exists():
        build.build_gpu()
    return so


@pytest.fixture(scope="session")
def refdata():
    return np.load(GOLDEN / "refdata.npz")


@pytest.fixture(scope="session")
def ref_small():
    return np.load(GOLDEN / "ref_small.npz")


@pytest.fixture(scope="session")
def ref_kat():
    import json

    return json.loads((GOLDEN / "ref_kat.json").read_text())


@pytest.fixture(scope="session")
def amcl(native_lib):
    import amcl3d_gb300

    return amcl3d_gb300


def small_grid_data(ref_small):
    """GridData of the golden synthetic case, cells from the oracle (exp as on the GPU)."""
    import oracle as O

    b = ref_small["bounds"]
    mn, mx, res = tuple(b[:3]), tuple(b[3:6]), float(b[6])
    d, p = O.compute_grid(ref_small["points"], mn, mx, res, 0.05, exp_mode=1)
    return O.GridData(mn, mx, res, tuple(int(v) for v in ref_small["dims"]), p.ravel(), d.ravel())
