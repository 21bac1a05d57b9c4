"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on a
CPU-only machine."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Build libebsdgpu.so and the CPU oracle once per session."""
    from ctemsoft_gb300 import build
    build.build_library()
    build.build_oracle()
    return True


_CACHE = {}


def workload_data(wl):
    """(master, accum_e) of a synthetic workload, cached per session."""
    key = wl.name
    if key not in _CACHE:
        _CACHE[key] = (wl.master(), wl.mc())
    return _CACHE[key]
