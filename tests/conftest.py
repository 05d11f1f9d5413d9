import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    """The reference's fixture for the decomposition path (test/test_data/, used by
    test/python/decomposition_test.py:8-20)."""
    return {
        "correction_factor": 5535184878.03 / (2500 ** 3 * 4 / 3 * np.pi),
        "xyz": np.loadtxt(os.path.join(GOLDEN, "gaussian_catalog.txt"))[:, :3],
        "c_ln": np.loadtxt(os.path.join(GOLDEN, "gaussian_catalog.python.c_ln")),
        "c_ln_rev": np.loadtxt(os.path.join(GOLDEN, "gaussian_catalog.pythonrev.c_ln")),
        "k_ln": np.loadtxt(os.path.join(GOLDEN, "gaussian_catalog.python.k_ln")),
        "k_ln_rev": np.loadtxt(os.path.join(GOLDEN, "gaussian_catalog.pythonrev.k_ln")),
    }


def uniform_ball(n, rmax, seed):
    """Points uniform in a ball: r = rmax u^(1/3), cos(theta) ~ U[-1,1], phi ~ U[0,2pi)."""
    rng = np.random.default_rng(seed)
    r = rmax * rng.random(n) ** (1.0 / 3.0)
    th = np.arccos(rng.uniform(-1.0, 1.0, n))
    ph = rng.uniform(0.0, 2.0 * np.pi, n)
    return np.ascontiguousarray(np.stack([r, th, ph], axis=1))


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch.cuda.get_device_capability(0)
