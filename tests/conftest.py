"""Shared test configuration and helpers.

GPU tests are marked ``@pytest.mark.gpu``; everything else runs on CPU.
"""

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built extension")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        return {k: f[k] for k in f.files}


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def create_input_plus_noise(shape, is_complex, gen=None):
    """Ramp plus Gaussian noise, as the reference tests build inputs (tests/conftest.py:28-37)."""
    import torch

    x = torch.arange(int(np.prod(shape)), dtype=torch.float64).reshape(shape)
    if is_complex:
        x = x + torch.randn(x.shape, generator=gen, dtype=torch.float64) + 1j * torch.randn(
            x.shape, generator=gen, dtype=torch.float64)
    else:
        x = x + torch.randn(x.shape, generator=gen, dtype=torch.float64)
    return x


def create_ktraj(ndims, klength, gen=None, batch=None, dtype=None):
    import torch

    shape = (ndims, klength) if batch is None else (batch, ndims, klength)
    return (torch.rand(shape, generator=gen, dtype=torch.float64) * 2 * np.pi - np.pi).to(dtype or torch.float64)
