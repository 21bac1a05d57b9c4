"""ctypes binding of libebsdgpu.so (include/ebsd_gpu.h).

This is the Python face of the C ABI: the same entry points, argument
meanings and error codes, with numpy arrays in place of raw pointers.  There
is no fallback: if the library is missing, importing the binding fails.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libebsdgpu.so"

EBSD_OK = 0
EBSD_EINVAL = -1
EBSD_ECUDA = -2
EBSD_ENOMEM = -3
EBSD_ESTATE = -4
EBSD_EIO = -5
EBSD_EFORMAT = -6
EBSD_EUNSUPPORTED = -7
EBSD_ETIMEOUT = -8

SCALING = {"not": 0, "lin": 1, "gam": 2}
VJP_COTANGENT = 0
VJP_NDP = 1


class EBSDError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (code {code})")
        self.code = code


class Geometry(C.Structure):
    _fields_ = [("L", C.c_float), ("thetac", C.c_float), ("delta", C.c_float),
                ("numsx", C.c_int32), ("numsy", C.c_int32), ("xpc", C.c_float),
                ("ypc", C.c_float), ("sig", C.c_double)]


class Epilogue(C.Structure):
    _fields_ = [("prefactor", C.c_double), ("binning", C.c_int32), ("scalingmode", C.c_int32),
                ("gammavalue", C.c_float), ("poisson", C.c_int32), ("seed", C.c_uint64)]


class Job(C.Structure):
    _fields_ = [("source", C.c_void_p), ("quats", C.c_void_p), ("n", C.c_int64),
                ("epilogue", Epilogue), ("out", C.c_void_p)]


BATCH_GRAPH = 1
BATCH_QUEUE_ALL = 2


class GNOptions(C.Structure):
    _fields_ = [("max_iterations", C.c_int32), ("refine_pc", C.c_int32), ("damping", C.c_double),
                ("tol_rad", C.c_double), ("tol_pc", C.c_double)]


class MCHeader(C.Structure):
    _fields_ = [("numEbins", C.c_int32), ("numzbins", C.c_int32), ("numsx", C.c_int32),
                ("numsy", C.c_int32), ("num_el_total", C.c_int64), ("nthreads", C.c_int32),
                ("EkeV", C.c_double), ("Ehistmin", C.c_double), ("Ebinsize", C.c_double),
                ("depthmax", C.c_double), ("depthstep", C.c_double), ("sig", C.c_double),
                ("omega", C.c_double), ("MCmode", C.c_char * 5)]


class MasterHeader(C.Structure):
    _fields_ = [("npx", C.c_int32), ("npy", C.c_int32), ("nE", C.c_int32),
                ("numset", C.c_int32), ("sqorhe", C.c_char * 7)]


class Namelist(C.Structure):
    _fields_ = [("L", C.c_float), ("thetac", C.c_float), ("delta", C.c_float),
                ("numsx", C.c_int32), ("numsy", C.c_int32), ("xpc", C.c_float),
                ("ypc", C.c_float), ("anglefile", C.c_char * 512),
                ("eulerconvention", C.c_char * 4), ("FZfile", C.c_char * 512),
                ("energyfile", C.c_char * 512), ("datafile", C.c_char * 512),
                ("beamcurrent", C.c_double), ("dwelltime", C.c_double),
                ("energymin", C.c_float), ("energymax", C.c_float), ("binning", C.c_int32),
                ("gammavalue", C.c_float), ("scalingmode", C.c_char * 4),
                ("axisangle", C.c_float * 4), ("poisson", C.c_int32), ("seed", C.c_int64),
                ("resume", C.c_int32), ("ncubochoric", C.c_int32), ("pgnum", C.c_int32)]


class MCNamelist(C.Structure):
    _fields_ = [("xtalname", C.c_char * 512), ("sig", C.c_double), ("omega", C.c_double),
                ("numsx", C.c_int32), ("num_el", C.c_int64), ("primeseed", C.c_int32),
                ("EkeV", C.c_double), ("dataname", C.c_char * 512), ("nthreads", C.c_int32),
                ("Ehistmin", C.c_double), ("Ebinsize", C.c_double), ("depthmax", C.c_double),
                ("depthstep", C.c_double), ("MCmode", C.c_char * 5), ("density", C.c_double),
                ("Ze", C.c_double), ("at_wt", C.c_double)]


class MCParams(C.Structure):
    """ebsd_mc_params: namelist MCdata plus the crystal's density, average Z
    and average atomic weight."""
    _fields_ = [("sig", C.c_double), ("omega", C.c_double), ("EkeV", C.c_double),
                ("Ehistmin", C.c_double), ("Ebinsize", C.c_double), ("depthmax", C.c_double),
                ("depthstep", C.c_double), ("Ze", C.c_double), ("density", C.c_double),
                ("at_wt", C.c_double), ("numsx", C.c_int32)]


def mc_params(**kw) -> MCParams:
    """MCParams with CTEMMC's namelist defaults (CTEMMC.f90:171-181) for the
    keys not given; Ze, density and at_wt default to nickel."""
    d = dict(sig=70.0, omega=0.0, EkeV=30.0, Ehistmin=20.0, Ebinsize=0.25, depthmax=50.0,
             depthstep=1.0, Ze=28.0, density=8.908, at_wt=58.6934, numsx=1501)
    d.update(kw)
    return MCParams(**d)


def mc_dims(p: MCParams):
    a, b = C.c_int32(), C.c_int32()
    _check(lib().ebsd_mc_dims(C.byref(p), C.byref(a), C.byref(b)))
    return a.value, b.value


_P = C.c_void_p
_SIGS = {
    "ebsd_version": (C.c_int, []),
    "ebsd_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "ebsd_destroy": (None, [_P]),
    "ebsd_last_error": (C.c_char_p, [_P]),
    "ebsd_set_stream": (C.c_int, [_P, _P]),
    "ebsd_set_option": (C.c_int, [_P, C.c_char_p, C.c_int64]),
    "ebsd_set_master": (C.c_int, [_P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "ebsd_share_master": (C.c_int, [_P, _P]),
    "ebsd_share_detector": (C.c_int, [_P, _P]),
    "ebsd_set_detector": (C.c_int, [_P, C.POINTER(Geometry), _P, C.c_int32, C.c_int32,
                                    C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
    "ebsd_energy_window": (C.c_int, [C.c_float, C.c_float, C.c_double, C.c_double, C.c_int32,
                                     C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ebsd_prefactor": (C.c_double, [C.c_double, C.c_double, C.c_int32]),
    "ebsd_output_dims": (C.c_int, [_P, C.POINTER(Epilogue), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int32)]),
    "ebsd_forward": (C.c_int, [_P, _P, C.c_int64, C.POINTER(Epilogue), _P]),
    "ebsd_cells": (C.c_int, [_P, _P, C.c_int64, _P, _P, _P, _P]),
    "ebsd_forward_cells": (C.c_int, [_P, _P, C.c_int64, C.POINTER(Epilogue), _P, _P, _P, _P,
                                     _P]),
    "ebsd_forward_batched": (C.c_int, [_P, C.POINTER(Job), C.c_int32, C.c_int32]),
    "ebsd_gn_accumulate": (C.c_int, [_P, _P, C.c_int64, C.POINTER(Epilogue), _P, C.c_double,
                                     _P, _P]),
    "ebsd_gn_apply": (C.c_int, [_P, _P, C.c_int64, C.c_double, _P, C.POINTER(C.c_double)]),
    "ebsd_refine": (C.c_int, [_P, _P, C.c_int64, C.POINTER(Epilogue), _P, C.POINTER(GNOptions),
                              _P, C.POINTER(Geometry), C.POINTER(C.c_int32)]),
    "ebsd_refine_sharded": (C.c_int, [C.POINTER(_P), C.c_int32, C.POINTER(_P),
                                      C.POINTER(C.c_int64), C.POINTER(Epilogue), C.POINTER(_P),
                                      C.POINTER(GNOptions), C.POINTER(_P), C.POINTER(Geometry),
                                      C.POINTER(C.c_int32)]),
    "ebsd_autotune": (C.c_int, [_P, C.POINTER(Epilogue), C.c_int64, C.c_char_p,
                                C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                C.POINTER(C.c_float)]),
    "ebsd_vjp": (C.c_int, [_P, _P, C.c_int64, C.POINTER(Epilogue), C.c_int32, _P, _P, _P]),
    "ebsd_vjp_noalloc": (C.c_int, [_P, _P, C.c_int64, C.POINTER(Epilogue), C.c_int32, _P, _P,
                                   _P]),
    "ebsd_get_detector": (C.c_int, [_P, _P, _P, _P, _P]),
    "ebsd_measure_bandwidth": (C.c_int, [C.c_int32, C.c_int32, C.c_int64, C.c_int32,
                                         C.POINTER(C.c_double)]),
    "ebsd_sample_rfz": (C.c_int, [_P, C.c_int32, C.c_int32, _P, _P, C.c_int64,
                                  C.POINTER(C.c_int64)]),
    "ebsd_mc_dims": (C.c_int, [C.POINTER(MCParams), C.POINTER(C.c_int32),
                               C.POINTER(C.c_int32)]),
    "ebsd_mc_run": (C.c_int, [_P, C.POINTER(MCParams), C.c_uint64, C.c_int64, C.c_int64, _P, _P,
                              C.POINTER(C.c_int64)]),
    "ebsd_read_mc_namelist": (C.c_int, [C.c_char_p, C.POINTER(MCNamelist)]),
    "ebsd_run_mc_namelist": (C.c_int, [C.c_char_p, C.c_int, C.c_int]),
    "ebsd_run_mc_namelist_devices": (C.c_int, [C.c_char_p, C.POINTER(C.c_int32), C.c_int32,
                                               C.c_int]),
    "ebsd_run_namelist": (C.c_int, [C.c_char_p, C.c_int, C.c_int]),
    "ebsd_run_namelist_devices": (C.c_int, [C.c_char_p, C.POINTER(C.c_int32), C.c_int32,
                                            C.c_int]),
    "ebsd_read_mc_file": (C.c_int, [C.c_char_p, C.POINTER(MCHeader), _P]),
    "ebsd_read_master_file": (C.c_int, [C.c_char_p, C.POINTER(MasterHeader), _P, _P, _P]),
    "ebsd_read_namelist": (C.c_int, [C.c_char_p, C.POINTER(Namelist)]),
    "ebsd_read_angle_file": (C.c_int, [C.c_char_p, C.c_char_p, _P, C.POINTER(C.c_int64), _P]),
}

_lib = None


def lib() -> C.CDLL:
    """Load libebsdgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() or "
                              "python ctemsoft_gb300/build.py")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def _check(rc: int, handle=None) -> None:
    if rc != EBSD_OK:
        msg = lib().ebsd_last_error(handle).decode(errors="replace")
        raise EBSDError(rc, msg)


def _ptr(a) -> int | None:
    """Raw address of a numpy array, a torch tensor, or an int."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    raise TypeError(f"cannot take the address of {type(a)}")


def energy_window(energymin, energymax, Ehistmin, Ebinsize, numEbins):
    a, b = C.c_int32(), C.c_int32()
    _check(lib().ebsd_energy_window(energymin, energymax, Ehistmin, Ebinsize, numEbins,
                                    C.byref(a), C.byref(b)))
    return a.value, b.value


BW_L1, BW_L2, BW_HBM = 1, 2, 3


def measure_bandwidth(device: int, level: int, nbytes: int, repeats: int = 5) -> float:
    """Read bandwidth (GB/s) of one memory level of a device: BW_L1 (L1 hits,
    128-bit loads), BW_L2 (an L2-resident working set of nbytes, L1
    bypassed) or BW_HBM (nbytes larger than L2)."""
    v = C.c_double()
    _check(lib().ebsd_measure_bandwidth(device, level, int(nbytes), repeats, C.byref(v)))
    return v.value


def prefactor(beamcurrent, dwelltime, num_el):
    return lib().ebsd_prefactor(beamcurrent, dwelltime, num_el)


def epilogue(prefactor=1.0, binning=1, scalingmode="not", gammavalue=1.0, poisson=False,
             seed=1) -> Epilogue:
    mode = SCALING[scalingmode] if isinstance(scalingmode, str) else int(scalingmode)
    return Epilogue(prefactor, binning, mode, gammavalue, int(bool(poisson)), seed)


class Handle:
    """One device, one stream, the master pattern and one detector."""

    def __init__(self, device: int = 0):
        self._h = _P()
        _check(lib().ebsd_create(C.byref(self._h), device))
        self.num_el = None
        self.geometry = None

    def close(self):
        if self._h:
            lib().ebsd_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def raw(self):
        return self._h

    def set_stream(self, stream_ptr: int | None):
        _check(lib().ebsd_set_stream(self._h, stream_ptr), self._h)

    def set_option(self, key: str, value: int):
        _check(lib().ebsd_set_option(self._h, key.encode(), int(value)), self._h)

    def set_master(self, srtmp: np.ndarray):
        """srtmp: array shaped (numset, nE, 2npy+1, 2npx+1), i.e. the Fortran
        srtmp(-npx:npx,-npy:npy,nE,numset) in C order (x fastest)."""
        sr = np.ascontiguousarray(srtmp, dtype=np.float32)
        if sr.ndim == 3:
            sr = sr[None]
        numset, nE, gy, gx = sr.shape
        _check(lib().ebsd_set_master(self._h, _ptr(sr), (gx - 1) // 2, (gy - 1) // 2, nE, numset),
               self._h)

    def share_master(self, other: "Handle"):
        """Use other's master pattern (same device, no copy)."""
        _check(lib().ebsd_share_master(self._h, other._h), self._h)

    def share_detector(self, other: "Handle"):
        """Use other's master and detector set-up (same device, no copy)."""
        _check(lib().ebsd_share_detector(self._h, other._h), self._h)
        self.geometry = dict(other.geometry)
        self.num_el = other.num_el
        if hasattr(other, "_nbins"):
            self._nbins = other._nbins

    def set_detector(self, geom: dict, accum_e: np.ndarray, Emin: int, Emax: int) -> int:
        """accum_e: array shaped (2nsy+1, 2nsx+1, numEbins) = Fortran
        accum_e(numEbins,-nsx:nsx,-nsy:nsy).  Returns num_el."""
        acc = np.ascontiguousarray(accum_e, dtype=np.int32)
        gy, gx, nE = acc.shape
        g = Geometry(geom["L"], geom["thetac"], geom["delta"], geom["numsx"], geom["numsy"],
                     geom["xpc"], geom["ypc"], geom["sig"])
        ne = C.c_int32()
        _check(lib().ebsd_set_detector(self._h, C.byref(g), _ptr(acc), (gx - 1) // 2,
                                       (gy - 1) // 2, nE, Emin, Emax, C.byref(ne)), self._h)
        self.num_el = ne.value
        self.geometry = dict(geom)
        return ne.value

    def output_dims(self, epi: Epilogue):
        nx, ny = C.c_int32(), C.c_int32()
        _check(lib().ebsd_output_dims(self._h, C.byref(epi), C.byref(nx), C.byref(ny)), self._h)
        return nx.value, ny.value

    def forward(self, quats, epi: Epilogue, out=None):
        """Patterns for quats (n x 4, scalar first).  quats/out may be numpy
        arrays (host) or torch CUDA tensors (device).  Returns out shaped
        (n, ny, nx)."""
        n = int(quats.shape[0])
        nx, ny = self.output_dims(epi)
        if isinstance(quats, np.ndarray):
            quats = np.ascontiguousarray(quats, dtype=np.float32)
        if out is None:
            out = np.empty((n, ny, nx), dtype=np.float32)
        _check(lib().ebsd_forward(self._h, _ptr(quats), n, C.byref(epi), _ptr(out)), self._h)
        return out

    def vjp(self, quats, epi: Epilogue, data, mode: str = "ndp", loss=None, grad=None):
        """Adjoint of the pattern loop.  mode "ndp": data are target records,
        returns (loss[n], grad[n, 6]) of 1 - normalised dot product; mode
        "cot": data is the cotangent, returns (None, grad).  grad columns:
        rotation tangent w0, w1, w2 [rad], xpc, ypc [px], L [um]."""
        n = int(quats.shape[0])
        if isinstance(quats, np.ndarray):
            quats = np.ascontiguousarray(quats, dtype=np.float32)
        if isinstance(data, np.ndarray):
            data = np.ascontiguousarray(data, dtype=np.float32)
        m = VJP_NDP if mode == "ndp" else VJP_COTANGENT
        if grad is None:
            grad = np.zeros((n, 6), np.float32)
        if loss is None and m == VJP_NDP:
            loss = np.zeros(n, np.float32)
        _check(lib().ebsd_vjp(self._h, _ptr(quats), n, C.byref(epi), m, _ptr(data), _ptr(loss),
                              _ptr(grad)), self._h)
        return loss, grad

    def autotune(self, epi: Epilogue, n_sample: int = 64, cache_path=None):
        """Pick (and apply) the fastest launch shape; returns (tile_y,
        orient_per_cta, us_per_pattern)."""
        ty, oc, us = C.c_int32(), C.c_int32(), C.c_float()
        _check(lib().ebsd_autotune(self._h, C.byref(epi), n_sample,
                                   None if cache_path is None else str(cache_path).encode(),
                                   C.byref(ty), C.byref(oc), C.byref(us)), self._h)
        return ty.value, oc.value, us.value

    def forward_batched(self, jobs, graph: bool = False, queue_all: bool = False):
        """jobs: list of (source Handle, device quats tensor, Epilogue, device
        out tensor).  Queued on this handle's stream.  queue_all: every job
        through the persistent queue kernel (default: jobs that fill the GPU
        by themselves run as their own launches)."""
        arr = (Job * max(1, len(jobs)))()
        for i, (src, q, epi, out) in enumerate(jobs):
            arr[i] = Job(src.raw.value if hasattr(src.raw, "value") else src.raw, _ptr(q),
                         int(q.shape[0]), epi, _ptr(out))
        flags = (BATCH_GRAPH if graph else 0) | (BATCH_QUEUE_ALL if queue_all else 0)
        _check(lib().ebsd_forward_batched(self._h, arr, len(jobs), flags), self._h)

    def gn_accumulate(self, quats, epi: Epilogue, targets, damping=1e-3, pc_system=False,
                      loss=None):
        """Phase 1 of a Gauss-Newton step (device tensors).  Returns the
        12-number centre system (numpy) when pc_system is true."""
        sysc = np.zeros(12) if pc_system else None
        _check(lib().ebsd_gn_accumulate(self._h, _ptr(quats), int(quats.shape[0]), C.byref(epi),
                                        _ptr(targets), damping, _ptr(sysc), _ptr(loss)), self._h)
        return sysc

    def gn_apply(self, quats, damping=1e-3, dpc=None):
        """Phase 2: update quats in place; returns the largest step (rad)."""
        d = None if dpc is None else np.ascontiguousarray(dpc, np.float64)
        ms = C.c_double()
        _check(lib().ebsd_gn_apply(self._h, _ptr(quats), int(quats.shape[0]), damping, _ptr(d),
                                   C.byref(ms)), self._h)
        return ms.value

    def refine(self, quats, epi: Epilogue, targets, max_iterations=20, refine_pc=False,
               damping=1e-3, tol_rad=1e-6, tol_pc=1e-4, loss=None):
        """Gauss-Newton refinement on the device (quats updated in place).
        Returns (iterations, refined geometry dict)."""
        opt = GNOptions(max_iterations, int(refine_pc), damping, tol_rad, tol_pc)
        g = Geometry()
        it = C.c_int32()
        _check(lib().ebsd_refine(self._h, _ptr(quats), int(quats.shape[0]), C.byref(epi),
                                 _ptr(targets), C.byref(opt), _ptr(loss), C.byref(g),
                                 C.byref(it)), self._h)
        geom = {k: getattr(g, k) for k, _ in Geometry._fields_}
        self.geometry = dict(geom)
        return it.value, geom

    def cells(self, quats: np.ndarray):
        q = np.ascontiguousarray(quats, dtype=np.float32)
        n = q.shape[0]
        ny, nx = self.geometry["numsy"], self.geometry["numsx"]
        nix = np.empty((n, ny, nx), np.int32)
        niy = np.empty_like(nix)
        i0 = np.empty((n, ny, nx), np.float32)
        i1 = np.empty_like(i0)
        _check(lib().ebsd_cells(self._h, _ptr(q), n, _ptr(nix), _ptr(niy), _ptr(i0), _ptr(i1)),
               self._h)
        return nix, niy, i0, i1

    def forward_cells(self, quats, epi):
        """Patterns and Lambert cells from one launch of the pattern kernel
        (device tensors; returns numpy arrays: out, (nix, niy, ixy0, ixy1))."""
        import torch
        q = torch.as_tensor(np.ascontiguousarray(quats, dtype=np.float32)).cuda()
        n = q.shape[0]
        ny, nx = self.geometry["numsy"], self.geometry["numsx"]
        ox, oy = self.output_dims(epi)
        out = torch.empty((n, oy, ox), dtype=torch.float32, device=q.device)
        nix = torch.empty((n, ny, nx), dtype=torch.int32, device=q.device)
        niy = torch.empty_like(nix)
        i0 = torch.empty((n, ny, nx), dtype=torch.float32, device=q.device)
        i1 = torch.empty_like(i0)
        _check(lib().ebsd_forward_cells(self._h, _ptr(q), n, C.byref(epi), _ptr(out), _ptr(nix),
                                        _ptr(niy), _ptr(i0), _ptr(i1)), self._h)
        torch.cuda.synchronize()
        return out.cpu().numpy(), tuple(t.cpu().numpy() for t in (nix, niy, i0, i1))

    def get_detector(self, nE: int):
        ny, nx = self.geometry["numsy"], self.geometry["numsx"]
        W = np.empty((ny, nx, nE), np.float32)
        rgx = np.empty((ny, nx), np.float32)
        rgy = np.empty_like(rgx)
        rgz = np.empty_like(rgx)
        _check(lib().ebsd_get_detector(self._h, _ptr(W), _ptr(rgx), _ptr(rgy), _ptr(rgz)),
               self._h)
        return W, rgx, rgy, rgz

    def mc_run(self, p: MCParams, seed: int, first: int, n: int, accum_e=None, accum_z=False):
        """Monte-Carlo histograms of electrons [first, first + n).  Returns
        (accum_e (2nx+1, 2nx+1, numEbins), accum_z or None, counted); device
        tensors passed as accum_e / accum_z are filled in place."""
        nE, nz = mc_dims(p)
        nx = (p.numsx - 1) // 2
        n10 = nx // 10
        if accum_e is None:
            accum_e = np.empty((2 * nx + 1, 2 * nx + 1, nE), np.int32)
        if accum_z is True:
            accum_z = np.empty((2 * n10 + 1, 2 * n10 + 1, nz, nE), np.int32)
        elif accum_z is False:
            accum_z = None
        cnt = C.c_int64()
        _check(lib().ebsd_mc_run(self._h, C.byref(p), seed, first, n, _ptr(accum_e),
                                 _ptr(accum_z), C.byref(cnt)), self._h)
        return accum_e, accum_z, cnt.value

    def sample_rfz(self, nsteps: int, pgnum: int):
        """Cubochoric sampling of the Rodrigues fundamental zone of point
        group pgnum (SampleRFZ).  Returns (rods (n, 3) float64, quats (n, 4)
        float32), in the reference's grid order."""
        cnt = C.c_int64()
        _check(lib().ebsd_sample_rfz(self._h, nsteps, pgnum, None, None, 0, C.byref(cnt)),
               self._h)
        n = cnt.value
        r = np.empty((n, 3), np.float64)
        q = np.empty((n, 4), np.float32)
        _check(lib().ebsd_sample_rfz(self._h, nsteps, pgnum, _ptr(r), _ptr(q), n,
                                     C.byref(cnt)), self._h)
        return r, q


def refine_sharded(handles, quats, epi: Epilogue, targets, max_iterations=20, refine_pc=False,
                   damping=1e-3, tol_rad=1e-6, tol_pc=1e-4, losses=None):
    """Gauss-Newton refinement over several handles, each with its shard of
    device orientations (updated in place) and targets; the pattern-centre
    system is summed over the shards in this process.  Returns (iterations,
    refined geometry dict); every handle ends on that geometry."""
    nh = len(handles)
    hs = (_P * nh)(*[h.raw.value if hasattr(h.raw, "value") else h.raw for h in handles])
    qs = (_P * nh)(*[_ptr(q) for q in quats])
    ts = (_P * nh)(*[_ptr(t) for t in targets])
    ns = (C.c_int64 * nh)(*[int(q.shape[0]) for q in quats])
    ls = None if losses is None else (_P * nh)(*[_ptr(x) for x in losses])
    opt = GNOptions(max_iterations, int(refine_pc), damping, tol_rad, tol_pc)
    g = Geometry()
    it = C.c_int32()
    _check(lib().ebsd_refine_sharded(hs, nh, qs, ns, C.byref(epi), ts, C.byref(opt), ls,
                                     C.byref(g), C.byref(it)), handles[0].raw)
    geom = {k: getattr(g, k) for k, _ in Geometry._fields_}
    for h in handles:
        h.geometry = dict(geom)
    return it.value, geom


def run_namelist(path: str, device=0, quiet: bool = True) -> None:
    """The CTEMEBSD program for a namelist file; device is one index or a
    list of indices (the orientations are split over them)."""
    if isinstance(device, (list, tuple)):
        arr = (C.c_int32 * len(device))(*device)
        _check(lib().ebsd_run_namelist_devices(str(path).encode(), arr, len(device), int(quiet)))
    else:
        _check(lib().ebsd_run_namelist(str(path).encode(), device, int(quiet)))


def run_mc_namelist(path: str, device=0, quiet: bool = True) -> None:
    """The CTEMMC program for a namelist file; device is one index or a list
    of indices (the electrons are split over them)."""
    if isinstance(device, (list, tuple)):
        arr = (C.c_int32 * len(device))(*device)
        _check(lib().ebsd_run_mc_namelist_devices(str(path).encode(), arr, len(device),
                                                  int(quiet)))
    else:
        _check(lib().ebsd_run_mc_namelist(str(path).encode(), device, int(quiet)))


def read_mc_namelist(path: str) -> dict:
    n = MCNamelist()
    _check(lib().ebsd_read_mc_namelist(str(path).encode(), C.byref(n)))
    out = {}
    for name, _ in MCNamelist._fields_:
        v = getattr(n, name)
        out[name] = v.decode() if isinstance(v, bytes) else v
    return out


def read_mc_file(path: str, with_data: bool = True):
    h = MCHeader()
    _check(lib().ebsd_read_mc_file(str(path).encode(), C.byref(h), None))
    if not with_data:
        return h, None
    nsx, nsy = (h.numsx - 1) // 2, (h.numsy - 1) // 2
    acc = np.empty((2 * nsy + 1, 2 * nsx + 1, h.numEbins), np.int32)
    _check(lib().ebsd_read_mc_file(str(path).encode(), C.byref(h), _ptr(acc)))
    return h, acc


def read_master_file(path: str, with_data: bool = True):
    h = MasterHeader()
    _check(lib().ebsd_read_master_file(str(path).encode(), C.byref(h), None, None, None))
    ek = np.empty(h.nE, np.float32)
    at = np.empty(h.numset, np.int32)
    sr = None
    if with_data:
        sr = np.empty((h.numset, h.nE, 2 * h.npy + 1, 2 * h.npx + 1), np.float32)
    _check(lib().ebsd_read_master_file(str(path).encode(), C.byref(h), _ptr(ek), _ptr(at),
                                       _ptr(sr)))
    return h, ek, at, sr


def read_namelist(path: str) -> dict:
    n = Namelist()
    _check(lib().ebsd_read_namelist(str(path).encode(), C.byref(n)))
    out = {}
    for name, _ in Namelist._fields_:
        v = getattr(n, name)
        if isinstance(v, bytes):
            v = v.decode()
        elif name == "axisangle":
            v = list(v)
        out[name] = v
    return out


def read_angle_file(path: str, eulerconvention: str = "tsl", axisangle=(0, 0, 0, 0)):
    aa = (C.c_float * 4)(*axisangle)
    n = C.c_int64(0)
    _check(lib().ebsd_read_angle_file(str(path).encode(), eulerconvention.encode(), aa,
                                      C.byref(n), None))
    q = np.empty((n.value, 4), np.float32)
    _check(lib().ebsd_read_angle_file(str(path).encode(), eulerconvention.encode(), aa,
                                      C.byref(n), _ptr(q)))
    return q
