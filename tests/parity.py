"""Parity measures used by the tests (GPU results against the oracle)."""
from __future__ import annotations

import numpy as np

# Gates.  Lambert cells are bit-exact except pixels within float rounding of
# a cell edge (counted).  Intensities: within 1e-5 relative of the FP64
# re-evaluation and within 1e-4 of the FP32 reference restatement.
#
# Two error measures per pattern: its relative L2 error, and the pixel-wise
# max |a - ref| / max |ref| (the largest pixel error against the pattern's
# scale).  Which arithmetic meets which gate:
#
# * reference arithmetic (options weights_fp64 = 0, strict_order = 1): the
#   GPU repeats the reference's single-precision operations in its order, so
#   against the FP32 restatement it is within TOL_REF pixel-wise (measured
#   ~1e-6: only CUDA's atanf differs from the C library's).
# * accurate Lambert arithmetic (lambert_accurate = 1, with the default
#   binary64 weights): within TOL_FP64 of FP64 pixel-wise on the 501^2
#   master (measured 7.4e-6 at 80x60); on the 1001^2 master it meets
#   TOL_FP64 as relative L2 (2.2e-6) and TOL_PIXEL_REF pixel-wise (8.7e-5,
#   the same pixel error as the default): a single-precision Lambert
#   coordinate near |ixy| = 500 resolves 3e-5 of a cell (one ulp), so a
#   few ulps of binary32 geometry move a pixel on a sharp band edge by
#   ~1e-4 of the pattern maximum whatever 1 - z is computed as.
# * binary64 geometry (lambert_accurate = 2): the rotation, normalisation,
#   Lambert map and cell of every pixel in binary64 from binary64 detector
#   directions, the gather in binary32: within TOL_FP64 of FP64 pixel-wise
#   on both masters.
# * the default (binary64 weights, the reference's 1 - z): within TOL_FP64
#   of FP64 as relative L2 and TOL_PIXEL_REF pixel-wise.  Single pixels near
#   the Lambert poles differ from FP64 by up to ~1e-4 of the pattern maximum
#   because the reference computes 1 - z in single precision
#   (Lambert.f90:427,430), which the default keeps so that its cells stay
#   the reference's.  Against the FP32 restatement the default is within
#   TOL_REF as relative L2; pixel-wise it differs by the reference's own
#   single-precision weight error (~1e-4 on sparse MC histograms), which the
#   binary64 weights do not have.
TOL_FP64 = 1e-5
TOL_REF = 1e-4
TOL_PIXEL_REF = 1e-4
EDGE_ULPS = 4
# The binary32 adjoint against the oracle's binary64 analytic gradient: the
# largest error of each kind (rotation, xpc, ypc, L) relative to the largest
# component of that kind over the batch.
TOL_GRAD = 1e-4     # measured <= 1.3e-5 on the small detectors
TOL_GRAD_C4 = 6e-4  # 480x480 on the 1001^2 master: measured 6.3e-5 (rotation)
# The loss 1 - <O,T>/(|O||T|) against the binary64 loss, relative.
TOL_LOSS = 1e-4


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
