"""Test configuration: the `gpu` marker (tests that need a GB300 and the CUDA
engine) and shared helpers.  CPU tests (-m "not gpu") cover the oracle
against the golden fixtures, the host-side policy, the C ABI's exported
symbols and the sort emulation; GPU tests compare the engine with the oracle
through the C ABI."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libncvis_gb300.so")


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def gmm(N, D, n_comp, center_std, seed, sigma=1.0):
    """Isotropic Gaussian mixture with equal weights (the synthetic shape of
    the small configurations)."""
    rng = np.random.default_rng(seed)
    centers = rng.normal(0.0, center_std, size=(n_comp, D))
    labels = rng.integers(0, n_comp, size=N)
    return (centers[labels] + rng.normal(0.0, sigma, size=(N, D))).astype(np.float32), labels


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from ncvis_gb300 import _lib
    _lib.lib()
    return torch
