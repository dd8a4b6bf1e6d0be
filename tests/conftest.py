import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built sm_103a library")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def igf_extended(shape, h):
    """sym_kernel's formula (sc.py:109-133) in np.longdouble: the 8-corner
    difference cancels catastrophically, so FP64 results (the reference's and
    ours) carry ~1e-12..1e-10 relative noise; this is the yardstick."""
    L = np.longdouble
    i2, j2, k2 = (int(v) for v in shape)
    hx, hy, hz = (L(float(v)) for v in h)
    x = hx * np.arange(i2 + 1, dtype=L) - hx / 2
    y = hy * np.arange(j2 + 1, dtype=L) - hy / 2
    z = hz * np.arange(k2 + 1, dtype=L) - hz / 2
    x, y, z = np.ix_(x, y, z)
    r = np.sqrt(x * x + y * y + z * z)
    IG = (-x * x * L(0.5) * np.arctan(y * z / (x * r)) + y * z * np.log(x + r)
          - y * y * L(0.5) * np.arctan(z * x / (y * r)) + z * x * np.log(y + r)
          - z * z * L(0.5) * np.arctan(x * y / (z * r)) + x * y * np.log(z + r))
    return (IG[1:, 1:, 1:] - IG[:-1, 1:, 1:] - IG[1:, :-1, 1:] + IG[:-1, :-1, 1:]
            - IG[1:, 1:, :-1] + IG[:-1, 1:, :-1] + IG[1:, :-1, :-1] - IG[:-1, :-1, :-1])
