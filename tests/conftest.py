"""Shared test setup: the `gpu` marker, library builds, common fixtures."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    from dgtd_gb300 import build as pkg_build
    from oracle import pyoracle
    pkg_build.build()
    pyoracle.build()


_ensure_built()


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel_l2(a, b):
    import numpy as np
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


SPEED_OF_LIGHT_SI = 299792458.0


def read_point_probe(path):
    """A point-probe file in the reference's format (ProbesManager.cpp:203-215, 400-407): four
    header lines (ID, "Spatial Position (X, Y, Z)", the position, the column names), then rows
    t[s] Ex Ey Ez Hx Hy Hz. Returned as an array with t back in normalised units (t[s] * c)."""
    import numpy as np
    lines = Path(path).read_text().splitlines()
    assert lines[0].startswith("PointProbe ID ")
    assert lines[1].startswith("Spatial Position (X, Y, Z)")
    assert len(lines[2].split()) == 3
    assert lines[3].startswith("Time (s) // Ex // Ey // Ez // Hx // Hy // Hz")
    rows = np.loadtxt(path, skiprows=4, ndmin=2)
    rows[:, 0] *= SPEED_OF_LIGHT_SI
    return rows
