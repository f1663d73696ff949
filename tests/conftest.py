"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; everything else
runs on the CPU (oracle pins, host-side integer set-up, ABI exports)."""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _ensure_lib():
    lib = os.path.join(ROOT, "schwarz_gmres_dashboard_gb300", "_build", "libsgmres.so")
    if not os.path.exists(lib):
        subprocess.run([sys.executable, os.path.join(ROOT, "schwarz_gmres_dashboard_gb300",
                                                     "build.py")], check=True)


@pytest.fixture(scope="session")
def sg():
    _ensure_lib()
    import schwarz_gmres_dashboard_gb300 as mod
    return mod


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    orc.build()
    return orc.Oracle()


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


class HostCSR:
    """Plain CSR holder for the oracle."""

    def __init__(self, row_ptr, col_idx, vals):
        self.row_ptr = np.ascontiguousarray(row_ptr, np.int32)
        self.col_idx = np.ascontiguousarray(col_idx, np.int32)
        self.vals = np.ascontiguousarray(vals, np.float64)
        self.nrows = self.ncols = len(self.row_ptr) - 1


def golden_matrix(golden, name):
    return HostCSR(golden[f"{name}/row_ptr"], golden[f"{name}/col_idx"], golden[f"{name}/vals"])


@pytest.fixture(scope="session")
def gpu_ctx(sg):
    """The package's default context (skips nothing: a gpu test without a
    device fails loudly)."""
    return sg.default_context()
