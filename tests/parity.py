"""Parity measures used by the tests (GPU results against the oracle)."""
from __future__ import annotations

import numpy as np

# Tolerances: Lambert cells bit-exact except pixels within float rounding
# of a cell edge (counted); intensities within 1e-5 relative of the FP64
# re-evaluation and within 1e-4 of the FP32 reference.
#
# "Relative" for a pattern is its relative L2 error.  In the default
# (reference) arithmetic, single pixels near the Lambert poles differ from
# FP64 by up to ~1e-4 of the pattern maximum because the reference computes
# 1 - z in single precision (Lambert.f90:427,430); TOL_PIXEL_REF bounds that
# pixel-wise error.  The optional accurate Lambert arithmetic removes the
# cancellation and meets TOL_FP64 pixel-wise.
TOL_FP64 = 1e-5
TOL_REF = 1e-4
TOL_PIXEL_REF = 1e-4
EDGE_ULPS = 4


def rel_errors(a: np.ndarray, ref: np.ndarray):
    """Per-pattern relative L2 error and max|a-ref| / max|ref| (pattern
    axes are the last two)."""
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    d = a - ref
    ax = tuple(range(a.ndim - 2, a.ndim))
    l2 = np.sqrt((d * d).sum(axis=ax) / np.maximum((ref * ref).sum(axis=ax), 1e-300))
    mx = np.abs(d).max(axis=ax) / np.maximum(np.abs(ref).max(axis=ax), 1e-300)
    return l2, mx


def near_edge(n: int, ixy: np.ndarray, ulps: int = EDGE_ULPS) -> np.ndarray:
    """True where float32(n) + ixy lies within `ulps` ulps of an integer,
    i.e. where int(n + ixy) can flip between two correct float results."""
    a = np.float32(n) + np.asarray(ixy, np.float32)
    dist = np.abs(a.astype(np.float64) - np.round(a.astype(np.float64)))
    return dist <= ulps * np.spacing(np.abs(a)).astype(np.float64)


def cell_report(gpu, ora, npx: int, npy: int) -> dict:
    """Compare (nix, niy, ixy0, ixy1) tuples.  Returns counts of all
    pixels, mismatching pixels, mismatches at a cell edge and mismatches
    elsewhere (which must be zero)."""
    gnix, gniy, g0, g1 = gpu
    onix, oniy, o0, o1 = ora
    mism = (gnix != onix) | (gniy != oniy)
    edge = near_edge(npx, o0) | near_edge(npx, g0) | near_edge(npy, o1) | near_edge(npy, g1)
    close = (np.abs(g0 - o0) <= EDGE_ULPS * np.spacing(np.abs(o0) + 1)) & \
            (np.abs(g1 - o1) <= EDGE_ULPS * np.spacing(np.abs(o1) + 1))
    return {
        "pixels": int(mism.size),
        "mismatch": int(mism.sum()),
        "edge": int((mism & edge & close).sum()),
        "non_edge": int((mism & ~(edge & close)).sum()),
        "ixy_max_ulps": float(max(
            (np.abs(g0 - o0) / np.spacing(np.abs(o0) + 1)).max(),
            (np.abs(g1 - o1) / np.spacing(np.abs(o1) + 1)).max())),
    }
