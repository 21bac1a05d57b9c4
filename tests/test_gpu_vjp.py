"""GPU adjoint (ebsd_vjp) against the FP64 analytic gradient of the oracle
and against central finite differences of the FP64 forward."""
from __future__ import annotations

import numpy as np
import pytest

from ctemsoft_gb300 import capi, synth
from tests.conftest import workload_data
from tests.parity import TOL_GRAD, TOL_GRAD_C4, TOL_LOSS

pytestmark = pytest.mark.gpu

# against central differences at h = 1e-4 rad / 1e-3 px / 1e-2 um: the
# bilinear interpolation has kinks at cell edges, which the finite
# difference averages over (measured 1.1e-3 and 1.4e-3)
TOL_FD = 1e-2


def _grad_err(g, ref):
    g = np.asarray(g, np.float64)
    ref = np.asarray(ref, np.float64)
    errs = []
    for cols in ((0, 1, 2), (3,), (4,), (5,)):
        scale = np.abs(ref[:, cols]).max()
        errs.append(np.abs(g[:, cols] - ref[:, cols]).max() / max(scale, 1e-300))
    return np.array(errs)


def _wl():
    wl = synth.tiny(seed=5, numsx=64, numsy=48, npx=60, nE=5, mc_nsx=80, n_orient=8)
    wl.delta = 120.0
    return wl


def _handle(wl, sr, acc):
    h = capi.Handle(0)
    h.set_master(sr)
    num_el = h.set_detector(wl.geometry(), acc, 1, wl.nEbins)
    return h, capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)


def _targets(O, wl, sr, acc, q, b):
    det = O.Detector(wl.geometry(), acc, 1, wl.nEbins)
    qt = np.stack([O.rotate_left(x, np.radians([0.4, -0.3, 0.2])) for x in q.astype(np.float64)])
    T = det.patterns_f64(sr, qt, 1.0)
    if b > 1:
        T = np.stack([O.epilogue_f64(t, b, 1, 1.0) for t in T])
    return T.astype(np.float32)


@pytest.mark.parametrize("binning", [1, 2, 4, 8])
def test_ndp_matches_fp64_analytic(built, binning):
    from oracle import oracle as O
    wl = _wl()
    sr, acc = wl.master(), wl.mc()
    q = wl.quaternions()
    h, pref = _handle(wl, sr, acc)
    T = _targets(O, wl, sr, acc, q, binning)
    mode = "lin" if binning > 1 else "not"
    loss, g = h.vjp(q, capi.epilogue(pref, binning=binning, scalingmode=mode), T, "ndp")
    rloss, rg = O.vjp_f64(wl.geometry(), acc, 1, wl.nEbins, sr, q, pref, binning, "ndp", T)
    np.testing.assert_allclose(loss, rloss, rtol=TOL_LOSS, atol=1e-7)
    err = _grad_err(g, rg)
    print("binning", binning, "grad rel err (rot, xpc, ypc, L):", err)
    assert (err < TOL_GRAD).all(), err
    h.close()


@pytest.mark.parametrize("binning", [1, 2, 4])
def test_ragged_detector_matches_fp64_analytic(built, binning):
    """A detector whose sides are not multiples of the tile (70 x 45): partial
    tiles, and binning blocks cropped to the floor (CTEMEBSD.f90:630-651)."""
    from oracle import oracle as O
    wl = synth.tiny(seed=5, numsx=70, numsy=45, npx=60, nE=5, mc_nsx=80, n_orient=6)
    wl.delta = 110.0
    sr, acc = wl.master(), wl.mc()
    q = wl.quaternions()
    h, pref = _handle(wl, sr, acc)
    T = _targets(O, wl, sr, acc, q, binning)
    mode = "lin" if binning > 1 else "not"
    loss, g = h.vjp(q, capi.epilogue(pref, binning=binning, scalingmode=mode), T, "ndp")
    rloss, rg = O.vjp_f64(wl.geometry(), acc, 1, wl.nEbins, sr, q, pref, binning, "ndp", T)
    np.testing.assert_allclose(loss, rloss, rtol=TOL_LOSS, atol=1e-7)
    err = _grad_err(g, rg)
    print("ragged binning", binning, "grad rel err (rot, xpc, ypc, L):", err)
    assert (err < TOL_GRAD).all(), err
    h.close()


@pytest.mark.parametrize("tile_y,opc", [(4, 1), (8, 3), (16, 16), (32, 5)])
@pytest.mark.parametrize("mode", ["ndp", "cot"])
def test_every_unbinned_tile_shape_matches_fp64_analytic(built, tile_y, opc, mode):
    """The unbinned adjoint at each tile height (1, 2, 4 and 8 pixel rows per
    thread) and odd orientation counts per CTA, on the ragged 70 x 45
    detector (partial tiles), against the oracle's binary64 gradient."""
    from oracle import oracle as O
    wl = synth.tiny(seed=5, numsx=70, numsy=45, npx=60, nE=5, mc_nsx=80, n_orient=7)
    wl.delta = 110.0
    sr, acc = wl.master(), wl.mc()
    q = wl.quaternions()
    h, pref = _handle(wl, sr, acc)
    h.set_option("vjp_tile_y", tile_y)
    h.set_option("vjp_orient_per_cta", opc)
    if mode == "ndp":
        data = _targets(O, wl, sr, acc, q, 1)
    else:
        data = np.random.default_rng(1).standard_normal((len(q), 45, 70)).astype(np.float32)
    loss, g = h.vjp(q, capi.epilogue(pref), data, mode)
    rloss, rg = O.vjp_f64(wl.geometry(), acc, 1, wl.nEbins, sr, q, pref, 1, mode, data)
    if mode == "ndp":
        np.testing.assert_allclose(loss, rloss, rtol=TOL_LOSS, atol=1e-7)
    err = _grad_err(g, rg)
    print("tile", tile_y, "opc", opc, mode, "grad rel err (rot, xpc, ypc, L):", err)
    assert (err < TOL_GRAD).all(), err
    h.close()


def test_cotangent_matches_fp64_analytic(built):
    from oracle import oracle as O
    wl = _wl()
    sr, acc = wl.master(), wl.mc()
    q = wl.quaternions()
    h, pref = _handle(wl, sr, acc)
    rng = np.random.default_rng(0)
    cot = rng.standard_normal((len(q), wl.numsy, wl.numsx)).astype(np.float32)
    _, g = h.vjp(q, capi.epilogue(pref), cot, "cot")
    _, rg = O.vjp_f64(wl.geometry(), acc, 1, wl.nEbins, sr, q, pref, 1, "cot", cot)
    err = _grad_err(g, rg)
    print("cotangent grad rel err (rot, xpc, ypc, L):", err)
    assert (err < TOL_GRAD).all(), err
    h.close()


def test_ndp_matches_finite_differences(built):
    """Central FP64 finite differences of the loss (h = 1e-4 rad, 1e-3 px,
    1e-2 um), the detector re-evaluated for every pattern-centre step."""
    from oracle import oracle as O
    wl = _wl()
    sr, acc = wl.master(), wl.mc()
    q = wl.quaternions(4)
    h, pref = _handle(wl, sr, acc)
    T = _targets(O, wl, sr, acc, q, 1)
    loss, g = h.vjp(q, capi.epilogue(pref), T, "ndp")
    geom = dict(wl.geometry(), exact=True)

    def L(gm, qs):
        det = O.Detector(gm, acc, 1, wl.nEbins)
        P = det.patterns_f64(sr, qs, 1.0)
        return np.array([1 - (p * t).sum() / np.sqrt((p * p).sum() * (t * t).sum())
                         for p, t in zip(P, T.astype(np.float64))])

    qd = q.astype(np.float64)
    fd = np.zeros((len(q), 6))
    for a in range(3):
        w = np.zeros(3)
        w[a] = 1e-4
        qp = np.stack([O.rotate_left(x, w) for x in qd])
        qm = np.stack([O.rotate_left(x, -w) for x in qd])
        fd[:, a] = (L(geom, qp) - L(geom, qm)) / 2e-4
    for a, (k, st) in enumerate((("xpc", 1e-3), ("ypc", 1e-3), ("L", 1e-2))):
        gp, gm = dict(geom), dict(geom)
        gp[k] += st
        gm[k] -= st
        fd[:, 3 + a] = (L(gp, qd) - L(gm, qd)) / (2 * st)
    err = _grad_err(g, fd)
    print("FD rel err (rot, xpc, ypc, L):", err)
    assert (err < TOL_FD).all(), err
    h.close()


def test_vjp_deterministic_and_pointer_kinds(built):
    torch = pytest.importorskip("torch")
    wl = _wl()
    sr, acc = wl.master(), wl.mc()
    q = wl.quaternions()
    h, pref = _handle(wl, sr, acc)
    rng = np.random.default_rng(1)
    T = rng.uniform(0.5, 1.5, (len(q), wl.numsy, wl.numsx)).astype(np.float32)
    epi = capi.epilogue(pref)
    l1, g1 = h.vjp(q, epi, T, "ndp")
    l2, g2 = h.vjp(q, epi, T, "ndp")
    assert np.array_equal(g1, g2) and np.array_equal(l1, l2)
    dq, dT = torch.from_numpy(q).cuda(), torch.from_numpy(T).cuda()
    dl = torch.zeros(len(q), device="cuda")
    dg = torch.zeros((len(q), 6), device="cuda")
    h.vjp(dq, epi, dT, "ndp", loss=dl, grad=dg)
    torch.cuda.synchronize()
    assert np.array_equal(dg.cpu().numpy(), g1) and np.array_equal(dl.cpu().numpy(), l1)
    h.close()


def test_vjp_rejects_gamma(built):
    wl = _wl()
    sr, acc = wl.master(), wl.mc()
    h, pref = _handle(wl, sr, acc)
    q = wl.quaternions(2)
    T = np.ones((2, wl.numsy, wl.numsx), np.float32)
    with pytest.raises(capi.EBSDError) as e:
        h.vjp(q, capi.epilogue(pref, scalingmode="gam", gammavalue=0.5), T, "ndp")
    assert e.value.code == capi.EBSD_EUNSUPPORTED
    h.close()


def test_adjoint_480x480_npx500(built):
    """The adjoint configuration: 480x480 detector, 1001^2 x 11 master, targets
    simulated at orientations perturbed by N(0, 0.5 deg) and pattern centres
    perturbed by N(0, 2 px) in xpc/ypc and N(0, 50 um) in L; loss 1 - normalised
    dot product; FP32 adjoint against the FP64 analytic gradient and central
    FP64 finite differences (h = 1e-4 rad, 1e-3 px, 1e-2 um)."""
    from oracle import oracle as O
    wl = synth.C4
    sr, acc = workload_data(wl)
    q = wl.quaternions(6)
    h, pref = _handle(wl, sr, acc)
    rng = np.random.default_rng(3)
    geom = dict(wl.geometry(), exact=True)
    T = []
    for x in q.astype(np.float64):
        gt = dict(geom)
        gt["xpc"] += rng.normal(0, 2.0)
        gt["ypc"] += rng.normal(0, 2.0)
        gt["L"] += rng.normal(0, 50.0)
        qt = O.rotate_left(x, np.radians(rng.normal(0, 0.5, 3)))
        T.append(O.Detector(gt, acc, 1, wl.nEbins).patterns_f64(sr, qt[None], 1.0)[0])
    T = np.stack(T).astype(np.float32)
    loss, g = h.vjp(q, capi.epilogue(pref), T, "ndp")
    rloss, rg = O.vjp_f64(wl.geometry(), acc, 1, wl.nEbins, sr, q, pref, 1, "ndp", T)
    np.testing.assert_allclose(loss, rloss, rtol=TOL_LOSS)
    err = _grad_err(g, rg)
    print("480x480 grad rel err vs FP64 analytic (rot, xpc, ypc, L):", err)
    assert (err < TOL_GRAD_C4).all(), err

    def L(gm, qs):
        P = O.Detector(gm, acc, 1, wl.nEbins).patterns_f64(sr, qs, 1.0,
                                                            nthreads=O.max_threads())
        return np.array([1 - (a * t).sum() / np.sqrt((a * a).sum() * (t * t).sum())
                         for a, t in zip(P, T.astype(np.float64))])

    qd = q.astype(np.float64)
    fd = np.zeros((len(q), 6))
    for a in range(3):
        w = np.zeros(3)
        w[a] = 1e-4
        fd[:, a] = (L(geom, np.stack([O.rotate_left(x, w) for x in qd])) -
                    L(geom, np.stack([O.rotate_left(x, -w) for x in qd]))) / 2e-4
    for a, (k, st) in enumerate((("xpc", 1e-3), ("ypc", 1e-3), ("L", 1e-2))):
        gp, gm = dict(geom), dict(geom)
        gp[k] += st
        gm[k] -= st
        fd[:, 3 + a] = (L(gp, qd) - L(gm, qd)) / (2 * st)
    err = _grad_err(g, fd)
    print("480x480 grad rel err vs FP64 central differences:", err)
    assert (err < TOL_FD).all(), err
    h.close()
