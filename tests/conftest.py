"""Shared fixtures.  `-m gpu` tests need a CUDA device; the rest run on CPU."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build_oracle()
    return oracle


@pytest.fixture(scope="session")
def golden_c1():
    return load_golden("golden_c1.npz")


@pytest.fixture(scope="session")
def golden_ellip():
    return load_golden("golden_ellip.npz")


@pytest.fixture(scope="session")
def golden_healpix():
    return load_golden("golden_healpix.npz")


def has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # noqa: BLE001
        return False


@pytest.fixture(scope="session")
def gpu():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from pisco4cmb_gb300 import _lib

    _lib.load()
    return True


def rel_rms(x, ref):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.sqrt(np.mean((x - ref) ** 2)) / max(np.sqrt(np.mean(ref ** 2)), 1e-300))


def rel_max(x, ref):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.max(np.abs(x - ref)) / max(np.sqrt(np.mean(ref ** 2)), 1e-300))
