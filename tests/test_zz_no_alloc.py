"""ebsd_vjp_noalloc: the adjoint for callers that cannot let the library
allocate device memory (their GPU memory belongs to their own pool, or
their refinement loop cannot take the synchronisation an allocation may
cause).  Called through the C ABI with device buffers, it must agree with
ebsd_vjp on two calls in a row.  This file is collected last on purpose."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from ctemsoft_gb300 import capi, synth

pytestmark = pytest.mark.gpu

TOL = 2e-3  # the adjoint tolerance of tests/test_gpu_vjp.py


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


@pytest.mark.parametrize("mode", ["ndp", "cot"])
def test_noalloc_matches_vjp_twice(built, mode):
    torch = pytest.importorskip("torch")
    wl = synth.tiny(seed=5, numsx=64, numsy=48, npx=60, nE=5, mc_nsx=80, n_orient=300)
    sr, acc = wl.master(), wl.mc()
    q = wl.quaternions()
    h = capi.Handle(0)
    h.set_master(sr)
    num_el = h.set_detector(wl.geometry(), acc, 1, wl.nEbins)
    epi = capi.epilogue(capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el))
    rng = np.random.default_rng(4)
    data = rng.uniform(0.5, 1.5, (len(q), wl.numsy, wl.numsx)).astype(np.float32)
    ref_loss, ref_grad = h.vjp(q, epi, data, mode)

    dq = torch.from_numpy(q).cuda()
    dd = torch.from_numpy(data).cuda()
    m = capi.VJP_NDP if mode == "ndp" else capi.VJP_COTANGENT
    lib = capi.lib()
    for call in range(2):
        dl = torch.full((len(q),), float("nan"), device="cuda")
        dg = torch.full((len(q), 6), float("nan"), device="cuda")
        rc = lib.ebsd_vjp_noalloc(h.raw, dq.data_ptr(), len(q), C.byref(epi), m, dd.data_ptr(),
                                  dl.data_ptr() if mode == "ndp" else None, dg.data_ptr())
        assert rc == capi.EBSD_OK, lib.ebsd_last_error(h.raw)
        torch.cuda.synchronize()
        g = dg.cpu().numpy()
        assert np.isfinite(g).all()
        assert _rel(g, ref_grad) <= TOL, (call, _rel(g, ref_grad))
        if mode == "ndp":
            assert _rel(dl.cpu().numpy(), ref_loss) <= TOL
    h.close()


def test_noalloc_rejects_host_buffers_and_oversized_detectors(built):
    torch = pytest.importorskip("torch")
    wl = synth.tiny(seed=5, numsx=64, numsy=48, npx=60, nE=5, mc_nsx=80, n_orient=4)
    sr, acc = wl.master(), wl.mc()
    h = capi.Handle(0)
    h.set_master(sr)
    h.set_detector(wl.geometry(), acc, 1, wl.nEbins)
    epi = capi.epilogue(1.0)
    q = wl.quaternions()
    data = np.ones((len(q), wl.numsy, wl.numsx), np.float32)
    grad = np.zeros((len(q), 6), np.float32)
    lib = capi.lib()
    rc = lib.ebsd_vjp_noalloc(h.raw, q.ctypes.data, len(q), C.byref(epi), capi.VJP_NDP,
                              data.ctypes.data, None, grad.ctypes.data)
    assert rc == capi.EBSD_EINVAL and b"device memory" in lib.ebsd_last_error(h.raw)
    # a detector whose single orientation exceeds the fixed scratch array:
    # 256 x 560 tiles x 15 floats > 2^21
    big = dict(wl.geometry(), numsx=8192, numsy=4480)
    h.set_detector(big, acc, 1, wl.nEbins)
    dq = torch.from_numpy(q).cuda()
    dd = torch.zeros(1, device="cuda")
    dg = torch.zeros((len(q), 6), device="cuda")
    rc = lib.ebsd_vjp_noalloc(h.raw, dq.data_ptr(), len(q), C.byref(epi), capi.VJP_NDP,
                              dd.data_ptr(), None, dg.data_ptr())
    assert rc == capi.EBSD_EUNSUPPORTED and b"scratch" in lib.ebsd_last_error(h.raw)
    h.close()
