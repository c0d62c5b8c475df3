"""Shared test set-up.

Markers:
  gpu  -- needs a CUDA GPU and the built libcgsense.so (parity tests proper).
Everything else runs on the CPU: the oracle against the reference's golden
vectors, host-side logic, and the C ABI's exports.
"""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libcgsense.so")


@pytest.fixture(scope="session")
def cgs():
    """The product package (4d_lung_gb300)."""
    return importlib.import_module("4d_lung_gb300")


@pytest.fixture(scope="session")
def synth():
    return importlib.import_module("4d_lung_gb300.synth")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle_py
    return oracle_py


@pytest.fixture(scope="session")
def o64(oracle_mod):
    return oracle_mod.Oracle(64)


@pytest.fixture(scope="session")
def o32(oracle_mod):
    return oracle_mod.Oracle(32)


@pytest.fixture(scope="session")
def gpu_lib(cgs):
    """Loads libcgsense.so (building it when absent) and checks for a GPU."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    if not os.path.exists(cgs.LIB_PATH):
        cgs.build()
    return cgs.lib()


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=True)


def rel_l2(a, b):
    a = np.asarray(a).ravel().astype(np.complex128)
    b = np.asarray(b).ravel().astype(np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
