"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def cdx():
    """The product package with its library built and loaded."""
    import cudadecon_gb300 as c
    if not c.lib_path().exists():
        c.build()
    c.lib()
    return c


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="session")
def oracle():
    from oracle import rl_oracle
    return rl_oracle


def rel_l2(a, b):
    """||a - b|| / ||b|| in double (complex arrays compared as complex)."""
    cplx = np.iscomplexobj(a) or np.iscomplexobj(b)
    dt = np.complex128 if cplx else np.float64
    a = np.asarray(a, dtype=dt)
    b = np.asarray(b, dtype=dt)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
