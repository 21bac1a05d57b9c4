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

from tests.parity import TOL_GRAD as TOL  # the adjoint's tolerance against its references
from tests.parity import TOL_LOSS


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


def _grad_err(g, ref):
    g = np.asarray(g, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.array([np.abs(g[:, c] - ref[:, c]).max() / max(np.abs(ref[:, c]).max(), 1e-300)
                     for c in ((0, 1, 2), (3,), (4,), (5,))])


def test_noalloc_many_launches_against_the_oracle(built):
    """A 640x480 detector needs 20 x 60 tiles x 15 floats of scratch per
    orientation, so the fixed array holds 116 orientations per launch: 300
    orientations run as three launches that reuse the same array.  Every
    orientation agrees with ebsd_vjp, and orientations on both sides of each
    launch boundary agree with the oracle's binary64 gradient."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    wl = synth.tiny(seed=6, numsx=640, numsy=480, npx=60, nE=5, mc_nsx=80, n_orient=300)
    wl.delta = 20.0
    sr, acc = wl.master(), wl.mc()
    q = wl.quaternions()
    h = capi.Handle(0)
    h.set_master(sr)
    num_el = h.set_detector(wl.geometry(), acc, 1, wl.nEbins)
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    epi = capi.epilogue(pref)
    # targets: the patterns at orientations rotated by (0.4, -0.3, 0.2) deg
    qt = np.stack([O.rotate_left(x, np.radians([0.4, -0.3, 0.2]))
                   for x in q.astype(np.float64)]).astype(np.float32)
    data = h.forward(qt, epi)
    ref_loss, ref_grad = h.vjp(q, epi, data, "ndp")
    lib = capi.lib()
    dq = torch.from_numpy(q).cuda()
    dd = torch.from_numpy(data).cuda()
    dl = torch.full((len(q),), float("nan"), device="cuda")
    dg = torch.full((len(q), 6), float("nan"), device="cuda")
    rc = lib.ebsd_vjp_noalloc(h.raw, dq.data_ptr(), len(q), C.byref(epi), capi.VJP_NDP,
                              dd.data_ptr(), dl.data_ptr(), dg.data_ptr())
    assert rc == capi.EBSD_OK, lib.ebsd_last_error(h.raw)
    torch.cuda.synchronize()
    g, lo = dg.cpu().numpy(), dl.cpu().numpy()
    assert np.isfinite(g).all() and np.isfinite(lo).all()
    assert _rel(g, ref_grad) <= TOL and _rel(lo, ref_loss) <= TOL
    sel = [0, 115, 116, 231, 232, 299]
    rloss, rg = O.vjp_f64(wl.geometry(), acc, 1, wl.nEbins, sr, q[sel], pref, 1, "ndp",
                          data[sel])
    err = _grad_err(g[sel], rg)
    print("no-alloc, three launches: grad rel err vs FP64 (rot, xpc, ypc, L):", err)
    assert (err <= TOL).all(), err
    np.testing.assert_allclose(lo[sel], rloss, rtol=TOL_LOSS)
    h.close()


def test_noalloc_refuses_memory_of_another_gpu(built):
    """Buffers on a GPU other than the handle's are refused before any
    launch (needs two GPUs)."""
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    wl = synth.tiny(seed=5, numsx=64, numsy=48, npx=60, nE=5, mc_nsx=80, n_orient=4)
    h = capi.Handle(0)
    h.set_master(wl.master())
    h.set_detector(wl.geometry(), wl.mc(), 1, wl.nEbins)
    epi = capi.epilogue(1.0)
    q = torch.from_numpy(wl.quaternions()).to("cuda:1")
    dd = torch.ones((4, wl.numsy, wl.numsx), device="cuda:1")
    dg = torch.zeros((4, 6), device="cuda:1")
    lib = capi.lib()
    rc = lib.ebsd_vjp_noalloc(h.raw, q.data_ptr(), 4, C.byref(epi), capi.VJP_NDP,
                              dd.data_ptr(), None, dg.data_ptr())
    assert rc == capi.EBSD_EINVAL and b"device 1" in lib.ebsd_last_error(h.raw)
    h.close()
