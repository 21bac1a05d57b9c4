"""The pattern kernels take the cell index int(npx + ixy) (CTEMEBSD.f90:593)
without float/integer conversion instructions: with t = npx + ixy (the
reference's binary32 sum), max(t, 0) + 2^23 rounded toward zero is 2^23 +
int(t), whose low mantissa bits are int(t), and (that sum - 2^23) - npx is
the reference's real(nix) exactly.  This restates the device arithmetic in
numpy (binary32 operations, the round-toward-zero add emulated from the
exact binary64 sum) and checks it against truncation on random coordinates
of every magnitude the Lambert map produces, on values next to integers,
and on the small negative sums float rounding can give at the grid's edge."""
from __future__ import annotations

import numpy as np

TWO23 = np.float32(8388608.0)


def _fadd_rz(a: np.ndarray, b: np.float32) -> np.ndarray:
    exact = a.astype(np.float64) + np.float64(b)       # exact for these magnitudes
    r = exact.astype(np.float32)                       # round to nearest
    away = np.abs(r.astype(np.float64)) > np.abs(exact)
    r[away] = np.nextafter(r[away], np.float32(0))     # one step toward zero
    return r


def _cell(ixy: np.ndarray, npx: int):
    t = np.float32(npx) + ixy                          # binary32 add
    tt = _fadd_rz(np.maximum(t, np.float32(0)), TWO23)
    it = tt.view(np.int32) - np.int32(0x4B000000)
    ni = it - npx
    d = ixy - ((tt - TWO23) - np.float32(npx))
    return ni, d, np.minimum(it, 2 * npx)


def _reference(ixy: np.ndarray, npx: int):
    t = np.float32(npx) + ixy
    ni = np.trunc(t.astype(np.float64)).astype(np.int64) - npx   # Fortran int()
    d = ixy - ni.astype(np.float32)
    i0 = np.clip(ni + npx, 0, 2 * npx)
    return ni, d, i0


def test_conversion_free_cell_matches_truncation():
    rng = np.random.default_rng(0)
    for npx in (40, 250, 500, 750, 4000):
        parts = [rng.uniform(-npx, npx, 200000),
                 # next to the integers
                 np.repeat(np.arange(-npx, npx + 1), 3)
                 + np.tile([-1e-4, 0.0, 1e-4], 2 * npx + 1),
                 # below -npx by float rounding (t slightly negative) and at +npx
                 [-npx - 1e-4, -npx - 3e-5, -float(npx), float(npx), npx + 1e-5]]
        ixy = np.concatenate([np.asarray(p, np.float64) for p in parts]).astype(np.float32)
        ixy = np.concatenate([ixy, np.nextafter(ixy, np.float32(np.inf)),
                              np.nextafter(ixy, np.float32(-np.inf))])
        ixy = ixy[np.float32(npx) + ixy > np.float32(-1.0)]   # the Lambert map's range
        ni, d, i0 = _cell(ixy, npx)
        rni, rd, ri0 = _reference(ixy, npx)
        assert np.array_equal(ni, rni), npx
        assert np.array_equal(i0, ri0), npx
        assert np.array_equal(d.view(np.int32), rd.view(np.int32)), npx   # bit for bit
