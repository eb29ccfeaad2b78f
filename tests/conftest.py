import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
for _p in (ROOT, ROOT / "tests"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libcyclix_gpu.so")
    config.addinivalue_line("markers", "slow: longer CPU-oracle runs")


def gpu_available() -> bool:
    try:
        import ctypes
        lib = ctypes.CDLL("libcudart.so") if False else None  # noqa: F841
        import subprocess
        r = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True, timeout=20)
        return r.returncode == 0 and "GPU" in r.stdout
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no GPU on this machine")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def small_cyclic():
    """The 40 x 12 x 20 cyclic workload (24 atoms, one Bloch block nu = 1, Ns = 48)."""
    from cyclix_msparc_gb300.workloads import WORKLOADS, make_system
    return make_system(WORKLOADS["cyclic-40x12x20-ns48-m20"])


@pytest.fixture(scope="session")
def small_helical():
    """A small helical cell (twist 0.05 rad/bohr) with two Bloch blocks and two spins."""
    from cyclix_msparc_gb300.workloads import Workload, make_system
    wl = Workload("helical-test-24x16x16", 24, 16, 16, (12, 10, 12, 10), ((0.0, 1.0, 0.0), (0.0, 2.0, 0.7)), 2, 8, 6, 4,
                  twist=0.05, L1=5.0)
    return make_system(wl)


@pytest.fixture(scope="session")
def tiny_helical():
    """A tiny helical cell whose dense Hamiltonian is cheap (1280 points, 2 atoms, 2 blocks)."""
    from cyclix_msparc_gb300.workloads import make_system
    from kat_systems import tiny_helical_workload
    return make_system(tiny_helical_workload())


@pytest.fixture(scope="session")
def tiny_cyclic():
    """A tiny cyclic cell (1280 points, 2 atoms, one block nu = 1, eta = 0.9)."""
    from cyclix_msparc_gb300.workloads import make_system
    from kat_systems import tiny_cyclic_workload
    return make_system(tiny_cyclic_workload())
