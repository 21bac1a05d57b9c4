"""ctypes wrapper of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY -- the checker for the GPU library.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
PARITY UNPINNED: the reference has no tests, fixtures or runnable build for
this path; see ebsd_oracle.c.

Array layouts (numpy, C order) match the Fortran arrays with the first
Fortran index last: detector arrays (numsy, numsx), W (numsy, numsx, nE),
accum_e (2nsy+1, 2nsx+1, nE), master sr (nE, 2npy+1, 2npx+1), patterns
(N, numsy, numsx).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"


class Geometry(C.Structure):
    _fields_ = [("L", C.c_float), ("thetac", C.c_float), ("delta", C.c_float),
                ("numsx", C.c_int32), ("numsy", C.c_int32), ("xpc", C.c_float),
                ("ypc", C.c_float), ("sig", C.c_double)]


class GeometryD(C.Structure):
    _fields_ = [("L", C.c_double), ("thetac", C.c_double), ("delta", C.c_double),
                ("numsx", C.c_int32), ("numsy", C.c_int32), ("xpc", C.c_double),
                ("ypc", C.c_double), ("sig", C.c_double)]


_P = C.c_void_p
_SIGS = {
    "oracle_lambert_inverse_f32": (C.c_int, [_P, _P]),
    "oracle_lambert_inverse_f64": (C.c_int, [_P, _P]),
    "oracle_lambert_forward_f64": (C.c_int, [_P, _P]),
    "oracle_quat_mult_f32": (None, [_P, _P, _P]),
    "oracle_eu2qu_f32": (None, [_P, _P]),
    "oracle_ax2qu_f32": (None, [_P, _P]),
    "oracle_angles_to_quats_f32": (None, [_P, C.c_int64, C.c_int, C.c_int, _P, _P]),
    "oracle_detector_f32": (None, [C.POINTER(Geometry), _P, _P, _P]),
    "oracle_detector_f64": (None, [C.POINTER(GeometryD), _P, _P, _P]),
    "oracle_mc_weights_f32": (C.c_int32, [C.POINTER(Geometry), _P, _P, _P, _P, C.c_int, C.c_int,
                                          C.c_int, C.c_int, C.c_int, _P]),
    "oracle_mc_weights_f64": (C.c_double, [C.POINTER(GeometryD), _P, _P, _P, _P, C.c_int,
                                           C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "oracle_prefactor": (C.c_double, [C.c_double, C.c_double, C.c_int32]),
    "oracle_energy_window": (None, [C.c_float, C.c_float, C.c_double, C.c_double, C.c_int,
                                    C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "oracle_master_scale_f32": (C.c_float, [C.c_int]),
    "oracle_cells_f32": (None, [C.POINTER(Geometry), _P, _P, _P, _P, C.c_int64, C.c_int, C.c_int,
                                _P, _P, _P, _P]),
    "oracle_patterns_f32": (None, [C.POINTER(Geometry), _P, _P, _P, _P, C.c_int, C.c_int,
                                   C.c_int, _P, C.c_int, C.c_int, _P, C.c_int64, C.c_double, _P,
                                   C.c_int]),
    "oracle_patterns_f64": (None, [C.POINTER(GeometryD), _P, _P, _P, _P, C.c_int, C.c_int,
                                   C.c_int, _P, C.c_int, C.c_int, _P, C.c_int64, C.c_double, _P,
                                   C.c_int]),
    "oracle_vjp_f64": (None, [C.POINTER(GeometryD), _P, C.c_int, C.c_int, C.c_int, C.c_int,
                              C.c_int, _P, C.c_int, C.c_int, _P, C.c_int64, C.c_double, C.c_int,
                              C.c_int, _P, _P, _P, C.c_int]),
    "oracle_epilogue_f32": (None, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, _P]),
    "oracle_epilogue_f64": (None, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _P]),
    "oracle_max_threads": (C.c_int, []),
    "oracle_so3_constants": (None, [_P]),
    "oracle_cu2ho_d": (C.c_int, [_P, _P]),
    "oracle_ho2cu_d": (C.c_int, [_P, _P]),
    "oracle_ho2ro_d": (None, [_P, _P]),
    "oracle_cu2ro_d": (None, [_P, _P]),
    "oracle_ro2qu_d": (None, [_P, _P]),
    "oracle_fz_type": (C.c_int, [C.c_int, C.POINTER(C.c_int)]),
    "oracle_fz_code": (C.c_int, [_P, C.c_int, C.c_int]),
    "oracle_rfz_axis": (C.c_int64, [C.c_int, _P, C.c_int64]),
    "oracle_sample_rfz": (C.c_int64, [C.c_int, C.c_int, _P, C.c_int64]),
    "oracle_mc_dims": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "oracle_mc_philox": (C.c_int64, [_P, C.c_uint64, C.c_int64, C.c_int64, _P, _P]),
    "oracle_mc_reference_rng": (C.c_int64, [_P, C.c_int32, C.c_int, C.c_int64, _P, _P]),
    "oracle_mc_uniforms": (None, [C.c_int, C.c_uint64, C.c_int64, C.c_int, _P]),
    "oracle_philox4x32_10": (None, [_P, _P, _P]),
}

_lib = None


def build() -> Path:
    srcs = [HERE / n for n in ("ebsd_oracle.c", "ebsd_oracle_grad.c", "ebsd_oracle_so3.c",
                               "ebsd_oracle_mc.c", "ebsd_oracle.h")]
    if not LIB.exists() or LIB.stat().st_mtime < max(s.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


def geometry(g: dict) -> Geometry:
    return Geometry(g["L"], g["thetac"], g["delta"], g["numsx"], g["numsy"], g["xpc"], g["ypc"],
                    g["sig"])


def geometry_d(g: dict) -> GeometryD:
    """Binary64 geometry.  The float fields of the reference's namelist are
    taken at their float values unless the dict holds exact=True (finite
    differences step the geometry in binary64)."""
    f = (lambda v: float(v)) if g.get("exact") else (lambda v: float(np.float32(v)))
    return GeometryD(f(g["L"]), f(g["thetac"]), f(g["delta"]), g["numsx"], g["numsy"],
                     f(g["xpc"]), f(g["ypc"]), float(np.float32(g["sig"])))


def lambert_inverse_f32(xyz):
    v = np.asarray(xyz, np.float32)
    r = np.zeros(2, np.float32)
    ierr = lib().oracle_lambert_inverse_f32(_p(v), _p(r))
    return r, ierr


def lambert_inverse_f64(xyz):
    v = np.asarray(xyz, np.float64)
    r = np.zeros(2, np.float64)
    ierr = lib().oracle_lambert_inverse_f64(_p(v), _p(r))
    return r, ierr


def lambert_forward_f64(xy):
    v = np.asarray(xy, np.float64)
    r = np.zeros(3, np.float64)
    ierr = lib().oracle_lambert_forward_f64(_p(v), _p(r))
    return r, ierr


def quat_mult_f32(x, y):
    a, b = np.asarray(x, np.float32), np.asarray(y, np.float32)
    r = np.zeros(4, np.float32)
    lib().oracle_quat_mult_f32(_p(a), _p(b), _p(r))
    return r


def eu2qu_f32(e):
    a = np.asarray(e, np.float32)
    r = np.zeros(4, np.float32)
    lib().oracle_eu2qu_f32(_p(a), _p(r))
    return r


def ax2qu_f32(a):
    v = np.asarray(a, np.float32)
    r = np.zeros(4, np.float32)
    lib().oracle_ax2qu_f32(_p(v), _p(r))
    return r


def angles_to_quats(rows, mode: str, hkl: bool = False, axisangle=(0, 0, 0, 0)):
    r = np.ascontiguousarray(rows, np.float32)
    n = r.shape[0]
    q = np.zeros((n, 4), np.float32)
    aa = np.asarray(axisangle, np.float32)
    lib().oracle_angles_to_quats_f32(_p(r), n, 0 if mode == "eu" else 1, int(hkl), _p(aa), _p(q))
    return q


def energy_window(energymin, energymax, Ehistmin, Ebinsize, numEbins):
    a, b = C.c_int(), C.c_int()
    lib().oracle_energy_window(energymin, energymax, Ehistmin, Ebinsize, numEbins, C.byref(a),
                               C.byref(b))
    return a.value, b.value


def prefactor(beamcurrent, dwelltime, num_el):
    return lib().oracle_prefactor(beamcurrent, dwelltime, num_el)


class Detector:
    """Detector set-up in FP32 (reference semantics) and FP64."""

    def __init__(self, geom: dict, accum_e: np.ndarray, Emin: int, Emax: int):
        self.geom = dict(geom)
        g = geometry(geom)
        self._g = g
        ny, nx = geom["numsy"], geom["numsx"]
        self.rg32 = [np.zeros((ny, nx), np.float32) for _ in range(3)]
        lib().oracle_detector_f32(C.byref(g), *(_p(a) for a in self.rg32))
        self._gd = geometry_d(geom)
        self.rg64 = [np.zeros((ny, nx), np.float64) for _ in range(3)]
        lib().oracle_detector_f64(C.byref(self._gd), *(_p(a) for a in self.rg64))
        acc = np.ascontiguousarray(accum_e, np.int32)
        gy, gx, nE = acc.shape
        self.nE, self.Emin, self.Emax = nE, Emin, Emax
        self.nsx, self.nsy = (gx - 1) // 2, (gy - 1) // 2
        self.W32 = np.zeros((ny, nx, nE), np.float32)
        self.num_el = lib().oracle_mc_weights_f32(C.byref(g), *(_p(a) for a in self.rg32), _p(acc),
                                                  nE, self.nsx, self.nsy, Emin, Emax, _p(self.W32))
        self.W64 = np.zeros((ny, nx, nE), np.float64)
        self.accum_e = acc
        self.Wsum64 = lib().oracle_mc_weights_f64(C.byref(self._gd), *(_p(a) for a in self.rg64),
                                                  _p(acc), nE, self.nsx, self.nsy, Emin, Emax,
                                                  _p(self.W64))

    def cells(self, quats, npx, npy=None):
        npy = npx if npy is None else npy
        q = np.ascontiguousarray(quats, np.float32)
        n = q.shape[0]
        ny, nx = self.geom["numsy"], self.geom["numsx"]
        nix = np.zeros((n, ny, nx), np.int32)
        niy = np.zeros_like(nix)
        i0 = np.zeros((n, ny, nx), np.float32)
        i1 = np.zeros_like(i0)
        lib().oracle_cells_f32(C.byref(self._g), *(_p(a) for a in self.rg32), _p(q), n, npx, npy,
                               _p(nix), _p(niy), _p(i0), _p(i1))
        return nix, niy, i0, i1

    def patterns_f32(self, sr, quats, prefactor, nthreads=1):
        s = np.ascontiguousarray(sr, np.float32)
        nE, gy, gx = s.shape
        q = np.ascontiguousarray(quats, np.float32)
        n = q.shape[0]
        ny, nx = self.geom["numsy"], self.geom["numsx"]
        out = np.zeros((n, ny, nx), np.float32)
        lib().oracle_patterns_f32(C.byref(self._g), *(_p(a) for a in self.rg32), _p(self.W32),
                                  self.nE, self.Emin, self.Emax, _p(s), (gx - 1) // 2,
                                  (gy - 1) // 2, _p(q), n, prefactor, _p(out), nthreads)
        return out

    def patterns_f64(self, sr, quats, prefactor, nthreads=1):
        s = np.ascontiguousarray(sr, np.float32)
        nE, gy, gx = s.shape
        q = np.ascontiguousarray(quats, np.float64)
        n = q.shape[0]
        ny, nx = self.geom["numsy"], self.geom["numsx"]
        out = np.zeros((n, ny, nx), np.float64)
        lib().oracle_patterns_f64(C.byref(self._gd), *(_p(a) for a in self.rg64), _p(self.W64),
                                  self.nE, self.Emin, self.Emax, _p(s), (gx - 1) // 2,
                                  (gy - 1) // 2, _p(q), n, prefactor, _p(out), nthreads)
        return out


def vjp_f64(geom: dict, accum_e, Emin, Emax, sr, quats, prefactor, binning, mode, data,
            nthreads=None):
    """Analytic FP64 gradient per pattern with respect to (w0, w1, w2, xpc,
    ypc, L).  mode "cot": data is the cotangent on the output records; mode
    "ndp": data are target records and the loss is 1 - normalised dot
    product.  Returns (loss[N], grad[N, 6])."""
    g = geometry_d(geom)
    acc = np.ascontiguousarray(accum_e, np.int32)
    gyy, gxx, nE = acc.shape
    s = np.ascontiguousarray(sr, np.float32)
    _, gy, gx = s.shape
    q = np.ascontiguousarray(quats, np.float64)
    n = q.shape[0]
    d = np.ascontiguousarray(data, np.float32)
    loss = np.zeros(n)
    grad = np.zeros((n, 6))
    nt = max_threads() if nthreads is None else nthreads
    lib().oracle_vjp_f64(C.byref(g), _p(acc), nE, (gxx - 1) // 2, (gyy - 1) // 2, Emin, Emax,
                         _p(s), (gx - 1) // 2, (gy - 1) // 2, _p(q), n, prefactor, binning,
                         0 if mode == "cot" else 1, _p(d), _p(loss), _p(grad), nt)
    return loss, grad


def rotate_left(q, w):
    """exp(w) (x) q in binary64 (scalar-first), the rotation tangent used by
    the derivatives: exp(w) = (cos|w|/2, sin(|w|/2) w/|w|)."""
    q = np.asarray(q, np.float64)
    w = np.asarray(w, np.float64)
    th = np.linalg.norm(w)
    e = np.array([1.0, 0.0, 0.0, 0.0]) if th == 0 else \
        np.concatenate([[np.cos(th / 2)], np.sin(th / 2) * w / th])
    x, y = e, q
    return np.array([x[0] * y[0] - x[1] * y[1] - x[2] * y[2] - x[3] * y[3],
                     x[0] * y[1] + x[1] * y[0] + x[2] * y[3] - x[3] * y[2],
                     x[0] * y[2] - x[1] * y[3] + x[2] * y[0] + x[3] * y[1],
                     x[0] * y[3] + x[1] * y[2] - x[2] * y[1] + x[3] * y[0]])


def epilogue_f32(pat, binning, mode, gammavalue):
    p = np.ascontiguousarray(pat, np.float32)
    ny, nx = p.shape
    if mode == 0 or binning == 1:
        out = np.zeros((ny, nx), np.float32)
    else:
        out = np.zeros((ny // binning, nx // binning), np.float32)
    lib().oracle_epilogue_f32(_p(p), nx, ny, binning, mode, gammavalue, _p(out))
    return out


def epilogue_f64(pat, binning, mode, gammavalue):
    p = np.ascontiguousarray(pat, np.float64)
    ny, nx = p.shape
    if mode == 0:
        out = np.zeros((ny, nx), np.float64)
    else:
        out = np.zeros((ny // binning, nx // binning), np.float64)
    lib().oracle_epilogue_f64(_p(p), nx, ny, binning, mode, gammavalue, _p(out))
    return out


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def host_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


# ---------------------------------------------------------------------------
# Cubochoric sampling of Rodrigues fundamental zones (ebsd_oracle_so3.c)

def so3_constants():
    """(cube semi-edge, sc, R1, prek, pref, rvmax2, pi8, srt) in binary64."""
    out = np.zeros(8)
    lib().oracle_so3_constants(_p(out))
    return out


def _map3(fn, xs):
    x = np.ascontiguousarray(np.atleast_2d(xs), np.float64)
    out = np.zeros_like(x)
    f = getattr(lib(), fn)
    for i in range(len(x)):
        f(_p(x[i]), _p(out[i]))
    return out


def cu2ho(c):
    return _map3("oracle_cu2ho_d", c)


def ho2cu(h):
    return _map3("oracle_ho2cu_d", h)


def ho2ro(h):
    return _map3("oracle_ho2ro_d", h)


def cu2ro(c):
    return _map3("oracle_cu2ro_d", c)


def ro2qu(r):
    x = np.ascontiguousarray(np.atleast_2d(r), np.float64)
    out = np.zeros((len(x), 4))
    for i in range(len(x)):
        lib().oracle_ro2qu_d(_p(x[i]), _p(out[i]))
    return out


def fz_type(pgnum):
    o = C.c_int()
    t = lib().oracle_fz_type(pgnum, C.byref(o))
    return t, o.value


def fz_code(rod, pgnum):
    t, o = fz_type(pgnum)
    r = np.ascontiguousarray(rod, np.float64)
    return lib().oracle_fz_code(_p(r), t, o)


def rfz_axis(nsteps):
    m = lib().oracle_rfz_axis(nsteps, None, 0)
    xs = np.zeros(m)
    lib().oracle_rfz_axis(nsteps, _p(xs), m)
    return xs


def sample_rfz(nsteps, pgnum):
    """Rodrigues vectors (count, 3) of SampleRFZ(nsteps, pgnum), loop order."""
    n = lib().oracle_sample_rfz(nsteps, pgnum, None, 0)
    if n < 0:
        raise ValueError("bad point group or step count")
    rods = np.zeros((max(n, 1), 3))
    lib().oracle_sample_rfz(nsteps, pgnum, _p(rods), n)
    return rods[:n]


# ---------------------------------------------------------------------------
# Monte-Carlo backscatter histogram (ebsd_oracle_mc.c)

class MCParams(C.Structure):
    _fields_ = [("sig", C.c_double), ("omega", C.c_double), ("EkeV", C.c_double),
                ("Ehistmin", C.c_double), ("Ebinsize", C.c_double), ("depthmax", C.c_double),
                ("depthstep", C.c_double), ("Ze", C.c_double), ("density", C.c_double),
                ("at_wt", C.c_double), ("numsx", C.c_int32)]


def mc_params(**kw) -> MCParams:
    d = dict(sig=70.0, omega=0.0, EkeV=20.0, Ehistmin=10.0, Ebinsize=1.0, depthmax=100.0,
             depthstep=1.0, Ze=28.0, density=8.9, at_wt=58.69, numsx=101)
    d.update(kw)
    return MCParams(**d)


def mc_dims(p: MCParams):
    a, b = C.c_int(), C.c_int()
    if lib().oracle_mc_dims(C.byref(p), C.byref(a), C.byref(b)):
        raise ValueError("bad Monte-Carlo parameters")
    return a.value, b.value


def _mc_arrays(p):
    nE, nz = mc_dims(p)
    nx = (p.numsx - 1) // 2
    n10 = nx // 10
    acc = np.zeros((2 * nx + 1, 2 * nx + 1, nE), np.int32)          # Fortran (E, x, y)
    accz = np.zeros((2 * n10 + 1, 2 * n10 + 1, nz, nE), np.int32)   # Fortran (E, z, x, y)
    return acc, accz


def mc_philox(p: MCParams, seed: int, e0: int, e1: int):
    """Histograms of electrons [e0, e1) on the GPU's Philox stream."""
    acc, accz = _mc_arrays(p)
    n = lib().oracle_mc_philox(C.byref(p), seed, e0, e1, _p(acc), _p(accz))
    return acc, accz, n


def mc_reference_rng(p: MCParams, primeseed: int, nthreads: int, num_el: int):
    """Histograms with the reference's own generator streams."""
    acc, accz = _mc_arrays(p)
    n = lib().oracle_mc_reference_rng(C.byref(p), primeseed, nthreads, num_el, _p(acc), _p(accz))
    return acc, accz, n


def mc_uniforms(kind: int, seed: int, electron: int, count: int):
    u = np.zeros(count, np.float32)
    lib().oracle_mc_uniforms(kind, seed, electron, count, _p(u))
    return u


def philox4x32_10(ctr, key):
    """One Philox4x32-10 block: four 32-bit counter words, two key words."""
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().oracle_philox4x32_10(_p(c), _p(k), _p(out))
    return out
