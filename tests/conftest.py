"""Test configuration.

Tests that need a GPU are marked ``gpu``; everything else runs on the CPU.
The DYFOX reference is never read at test time: its answers are the golden
vectors under tests/golden (made by tests/golden/make_golden.py) and the
oracle under oracle/.
"""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device")
    config.addinivalue_line("markers", "slow: more than about ten seconds")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    """The CUDA path, built and loaded; fails (not skips) when a GPU is
    visible but the library cannot be loaded."""
    if not has_gpu():
        pytest.skip("no CUDA device")
    from dyfox_gb300 import _lib, build
    if not os.path.exists(build.LIB):
        build.build()
    _lib.lib()
    import torch
    return torch


@pytest.fixture
def rng():
    return np.random.default_rng(20260909)


@pytest.fixture(scope="session")
def diamond400():
    from dyfox_gb300.crystal import diamond_400
    return diamond_400()


@pytest.fixture(scope="session")
def small_grid(diamond400):
    from dyfox_gb300.grid import LaueGrid
    return LaueGrid(diamond400, t_crystal=40e-6, dx=0.25e-6,
                    beam_width=8e-6, beam_thickness=1e-6)


def golden(name):
    path = os.path.join(GOLDEN, name + ".npz")
    if not os.path.exists(path):
        pytest.fail(f"golden fixture {path} is missing")
    return np.load(path, allow_pickle=False)


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
