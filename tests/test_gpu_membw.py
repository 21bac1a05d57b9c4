"""The memory-hierarchy read-bandwidth probes behind the pattern kernel's
roofline (ebsd_measure_bandwidth), on the GPU."""
from __future__ import annotations

import pytest

from ctemsoft_gb300 import capi

pytestmark = pytest.mark.gpu


def test_bandwidth_levels_are_ordered(built):
    """L1 hits outrun an L2-resident sweep, which outruns an HBM sweep; all
    three are positive and finite."""
    l1 = capi.measure_bandwidth(0, capi.BW_L1, 16, 3)
    l2 = capi.measure_bandwidth(0, capi.BW_L2, 48 << 20, 3)
    hbm = capi.measure_bandwidth(0, capi.BW_HBM, 2 << 30, 2)
    print(f"read bandwidth GB/s: L1 {l1:.0f}, L2 (48 MB) {l2:.0f}, HBM (2 GB) {hbm:.0f}")
    assert l1 > l2 > hbm > 100.0
