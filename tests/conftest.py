"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the built
libgalaxcu.so; everything else runs on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libgalaxcu.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def G():
    import galax_gb300
    from galax_gb300 import build
    build.build()
    galax_gb300.lib()
    return galax_gb300


def rel_vec_err(ax, ay, rx, ry):
    """Per-body |a - a*| / max(|a*|, 1e-30) (vector metric)."""
    den = np.maximum(np.hypot(rx, ry), 1e-30)
    return np.hypot(np.asarray(ax) - rx, np.asarray(ay) - ry) / den
