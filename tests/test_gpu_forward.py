"""GPU parity of the pattern loop against the CPU oracle, through the C ABI."""
from __future__ import annotations

import numpy as np
import pytest

from ctemsoft_gb300 import capi, synth
from tests.conftest import workload_data
from tests.parity import TOL_FP64, TOL_PIXEL_REF, TOL_REF, cell_report, rel_errors

pytestmark = pytest.mark.gpu


def _oracle():
    from oracle import oracle as O
    return O


def _setup(wl, Emin=1, Emax=None, fp64=True, master=None, acc=None, accurate=False):
    O = _oracle()
    sr, accum = workload_data(wl)
    if master is not None:
        sr = master
    if acc is not None:
        accum = acc
    Emax = wl.nEbins if Emax is None else Emax
    h = capi.Handle(0)
    h.set_option("weights_fp64", int(fp64))
    h.set_option("lambert_accurate", int(accurate))
    h.set_master(sr)
    num_el = h.set_detector(wl.geometry(), accum, Emin, Emax)
    det = O.Detector(wl.geometry(), accum, Emin, Emax)
    return h, det, sr, num_el


@pytest.mark.parametrize("wl", [synth.tiny(), synth.tiny(seed=11, numsx=37, numsy=29, npx=33,
                                                          nE=7, phase="Ti")],
                         ids=["tiny-Ni", "tiny-Ti-ragged"])
def test_tiny_parity(built, wl):
    h, det, sr, num_el = _setup(wl)
    q = wl.quaternions(wl.n_orient)
    assert num_el == det.num_el
    # Lambert cells: bit-exact except at cell edges
    rep = cell_report(h.cells(q), det.cells(q, wl.npx), wl.npx, wl.npx)
    assert rep["non_edge"] == 0, rep
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    epi = capi.epilogue(pref)
    gpu = h.forward(q, epi)
    p64 = det.patterns_f64(sr, q, pref)
    p32 = det.patterns_f32(sr, q, pref)
    l2, mx = rel_errors(gpu, p32)
    assert l2.max() <= TOL_REF and mx.max() <= TOL_REF, (l2.max(), mx.max())
    # accurate Lambert arithmetic: within 1e-5 of FP64 pixel by pixel (these
    # coarse 400 um detectors put many pixels near a pole, where the
    # reference arithmetic itself is ~3e-4 off FP64)
    h.set_option("lambert_accurate", 1)
    acc_out = h.forward(q, epi)
    l2, mx = rel_errors(acc_out, p64)
    assert l2.max() <= TOL_FP64 and mx.max() <= TOL_FP64, (l2.max(), mx.max())
    h.close()


def test_tiny_reference_weights_mode(built):
    """With single-precision weights the GPU follows the FP32 reference
    operation by operation; differences come only from atanf."""
    wl = synth.tiny()
    h, det, sr, num_el = _setup(wl, fp64=False)
    h.set_option("strict_order", 1)
    q = wl.quaternions(wl.n_orient)
    W, rgx, rgy, rgz = h.get_detector(wl.nEbins)
    assert np.array_equal(rgx, det.rg32[0]) and np.array_equal(rgy, det.rg32[1]) \
        and np.array_equal(rgz, det.rg32[2])
    l2, mx = rel_errors(W[None], det.W32[None])
    assert mx.max() < 1e-5
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    gpu = h.forward(q, capi.epilogue(pref))
    p32 = det.patterns_f32(sr, q, pref)
    l2, mx = rel_errors(gpu, p32)
    assert mx.max() <= 1e-5, mx.max()
    # most pixels bit-identical to the FP32 reference restatement
    assert np.mean(gpu == p32) > 0.5
    h.close()


@pytest.mark.parametrize("binning", [2, 4, 8])
def test_reference_order_binning(built, binning):
    """strict_order keeps the block sums of CTEMEBSD.f90:636 in the
    reference's order (x fastest, one addition at a time), whether the
    block is summed within a warp (2, 4) or through shared memory (8)."""
    O = _oracle()
    wl = synth.tiny(seed=9, numsx=64, numsy=48)
    h, det, sr, num_el = _setup(wl, fp64=False)
    h.set_option("strict_order", 1)
    q = wl.quaternions(wl.n_orient)
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    gpu = h.forward(q, capi.epilogue(pref, binning=binning, scalingmode="lin"))
    p32 = det.patterns_f32(sr, q, pref)
    ref = np.stack([O.epilogue_f32(p, binning, 1, 1.0) for p in p32])
    assert gpu.shape == ref.shape
    l2, mx = rel_errors(gpu, ref)
    assert mx.max() <= 1e-5, mx.max()
    assert np.mean(gpu == ref) > 0.5
    h.close()


def _three_modes(wl, q, n_f32=None):
    """Patterns of one workload in the three arithmetic modes and the oracle's
    FP64 and FP32 patterns.  The default mode's patterns and cells come from
    one launch of the pattern kernel (its cells instantiation), checked bit
    for bit against the plain launch that the bench times."""
    O = _oracle()
    h, det, sr, num_el = _setup(wl)
    assert num_el == det.num_el
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    epi = capi.epilogue(pref)
    out, cells = h.forward_cells(q, epi)
    assert np.array_equal(out, h.forward(q, epi))
    rep = cell_report(cells, det.cells(q, wl.npx), wl.npx, wl.npx)
    h.set_option("lambert_accurate", 1)
    acc_out = h.forward(q, epi)
    h.set_option("lambert_accurate", 2)
    g64_out = h.forward(q, epi)
    h.close()
    # reference arithmetic: single-precision weights, reference summation order
    hr, detr, _, num_el_r = _setup(wl, fp64=False)
    hr.set_option("strict_order", 1)
    assert num_el_r == num_el
    ref_out = hr.forward(q, epi)
    hr.close()
    nt = O.max_threads()
    p64 = det.patterns_f64(sr, q, pref, nthreads=nt)
    p32 = det.patterns_f32(sr, q, pref, nthreads=nt)
    return dict(default=out, accurate=acc_out, binary64=g64_out, reference=ref_out, p64=p64,
                p32=p32, cells=rep, pref=pref, det=det, sr=sr)


def _gate_three_modes(tag, r, accurate_pixel=TOL_FP64):
    print(tag, "cells", r["cells"])
    assert r["cells"]["non_edge"] == 0, r["cells"]
    l2, mx = rel_errors(r["default"], r["p64"])
    print(tag, "default vs FP64: relL2 %.3g pixel %.3g" % (l2.max(), mx.max()))
    assert l2.max() <= TOL_FP64 and mx.max() <= TOL_PIXEL_REF
    l2, mx = rel_errors(r["default"], r["p32"])
    print(tag, "default vs FP32 reference: relL2 %.3g pixel %.3g" % (l2.max(), mx.max()))
    assert l2.max() <= TOL_REF
    l2, mx = rel_errors(r["reference"], r["p32"])
    print(tag, "reference arithmetic vs FP32 reference: relL2 %.3g pixel %.3g"
          % (l2.max(), mx.max()))
    assert l2.max() <= TOL_REF and mx.max() <= TOL_REF
    l2, mx = rel_errors(r["accurate"], r["p64"])
    print(tag, "accurate vs FP64: relL2 %.3g pixel %.3g" % (l2.max(), mx.max()))
    assert l2.max() <= TOL_FP64 and mx.max() <= accurate_pixel
    l2, mx = rel_errors(r["binary64"], r["p64"])
    print(tag, "binary64 geometry vs FP64: relL2 %.3g pixel %.3g" % (l2.max(), mx.max()))
    assert l2.max() <= TOL_FP64 and mx.max() <= TOL_FP64


def test_c1_parity(built):
    """80x60 detector, 501^2 x 11 master, all 100 orientations: cells from the
    pattern kernel, the three arithmetic modes against the oracle pixel by
    pixel, and the gamma epilogue."""
    O = _oracle()
    wl = synth.C1
    q = wl.quaternions()
    r = _three_modes(wl, q)
    _gate_three_modes("C1", r)
    h, det, sr, num_el = _setup(wl)
    gam = h.forward(q, capi.epilogue(r["pref"], scalingmode="gam", gammavalue=wl.gammavalue))
    ref = np.stack([O.epilogue_f64(p, 1, 2, wl.gammavalue) for p in r["p64"]])
    l2, mx = rel_errors(gam, ref)
    assert l2.max() <= TOL_FP64 and mx.max() <= TOL_PIXEL_REF
    h.close()


@pytest.mark.parametrize("binning", [1, 2, 4, 8])
@pytest.mark.parametrize("mode", ["not", "lin", "gam"])
def test_epilogue_binning(built, binning, mode):
    O = _oracle()
    wl = synth.tiny(seed=5, numsx=44, numsy=35, npx=30, nE=4, n_orient=5)
    h, det, sr, num_el = _setup(wl, accurate=True)
    q = wl.quaternions()
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    out = h.forward(q, capi.epilogue(pref, binning=binning, scalingmode=mode, gammavalue=0.33))
    p64 = det.patterns_f64(sr, q, pref)
    m = capi.SCALING[mode]
    ref = np.stack([O.epilogue_f64(p, binning, m, 0.33) for p in p64])
    assert out.shape == ref.shape
    l2, mx = rel_errors(out, ref)
    assert l2.max() <= TOL_FP64 and mx.max() <= TOL_FP64, (l2.max(), mx.max())
    h.close()


def test_q_and_minus_q_identical(built):
    wl = synth.tiny()
    h, det, sr, num_el = _setup(wl)
    q = wl.quaternions()
    epi = capi.epilogue(1.0)
    assert np.array_equal(h.forward(q, epi), h.forward(-q, epi))
    h.close()


def test_uniform_master(built):
    """A constant master pattern c gives prefactor * c * sum_k W_k."""
    wl = synth.tiny()
    sr, acc = workload_data(wl)
    const = np.full_like(sr, 2.5)
    h, det, _, num_el = _setup(wl, master=const)
    q = wl.quaternions()
    out = h.forward(q, capi.epilogue(1.0))
    W, *_ = h.get_detector(wl.nEbins)
    expect = 2.5 * W.astype(np.float64).sum(axis=-1)
    np.testing.assert_allclose(out, np.broadcast_to(expect, out.shape), rtol=2e-6, atol=1e-30)
    h.close()


def test_identity_quaternion_is_detector_frame(built):
    """q = (1,0,0,0) gathers along the detector directions themselves."""
    wl = synth.tiny()
    h, det, sr, num_el = _setup(wl, accurate=True)
    q = np.array([[1, 0, 0, 0]], np.float32)
    out = h.forward(q, capi.epilogue(1.0))
    ref = det.patterns_f64(sr, q, 1.0)
    l2, mx = rel_errors(out, ref)
    assert mx.max() <= TOL_FP64
    h.close()


def test_device_and_host_buffers_agree(built):
    torch = pytest.importorskip("torch")
    wl = synth.tiny()
    h, det, sr, num_el = _setup(wl)
    q = wl.quaternions()
    epi = capi.epilogue(3.0, scalingmode="gam", gammavalue=0.5)
    host = h.forward(q, epi)
    dq = torch.from_numpy(q).cuda()
    dout = torch.empty(host.shape, dtype=torch.float32, device="cuda")
    h.forward(dq, epi, out=dout)
    torch.cuda.synchronize()
    assert np.array_equal(dout.cpu().numpy(), host)
    pinned = torch.empty(host.shape, dtype=torch.float32).pin_memory()
    h.forward(q, epi, out=pinned)
    assert np.array_equal(pinned.numpy(), host)
    h.close()


def test_many_chunks_pageable(built):
    """More orientations than one device chunk: the double-buffered host
    path must keep every record in place."""
    wl = synth.tiny(numsx=640, numsy=480, npx=40, nE=5, n_orient=300)
    h, det, sr, num_el = _setup(wl, accurate=True)
    q = wl.quaternions()
    epi = capi.epilogue(1.0)
    out = h.forward(q, epi)
    import torch
    dout = torch.empty(out.shape, dtype=torch.float32, device="cuda")
    h.forward(torch.from_numpy(q).cuda(), epi, out=dout)
    torch.cuda.synchronize()
    assert np.array_equal(dout.cpu().numpy(), out)
    sel = [0, 137, 299]
    ref = det.patterns_f64(sr, q[sel], 1.0)
    l2, mx = rel_errors(out[sel], ref)
    assert mx.max() <= TOL_FP64
    h.close()


def test_edge_cases(built):
    wl = synth.tiny()
    h, det, sr, num_el = _setup(wl, accurate=True)
    epi = capi.epilogue(1.0)
    # zero orientations is a no-op
    out = h.forward(np.zeros((0, 4), np.float32), epi)
    assert out.shape == (0, wl.numsy, wl.numsx)
    # a single orientation
    q = wl.quaternions(1)
    assert h.forward(q, epi).shape == (1, wl.numsy, wl.numsx)
    # non-finite quaternions are rejected before any launch
    bad = q.copy()
    bad[0, 2] = np.nan
    with pytest.raises(capi.EBSDError) as e:
        h.forward(bad, epi)
    assert e.value.code == capi.EBSD_EINVAL
    # unsupported binning
    with pytest.raises(capi.EBSDError) as e:
        h.forward(q, capi.epilogue(1.0, binning=3, scalingmode="lin"))
    assert e.value.code == capi.EBSD_EUNSUPPORTED
    # a non-unit quaternion is used as given (the reference does not
    # normalise); the direction is renormalised, so the pattern is the same
    out2 = h.forward(q * 2.0, epi)
    ref = det.patterns_f64(sr, q * 2.0, 1.0)
    l2, mx = rel_errors(out2, ref)
    assert mx.max() <= TOL_FP64
    h.close()


def test_call_order_and_mismatch_errors(built):
    wl = synth.tiny()
    sr, acc = workload_data(wl)
    h = capi.Handle(0)
    with pytest.raises(capi.EBSDError) as e:
        h.forward(wl.quaternions(1), capi.epilogue(1.0))
    assert e.value.code == capi.EBSD_ESTATE
    with pytest.raises(capi.EBSDError) as e:
        h.set_detector(wl.geometry(), acc, 1, wl.nEbins)
    assert e.value.code == capi.EBSD_ESTATE
    h.set_master(sr[:-1])  # one energy bin fewer than the MC histogram
    with pytest.raises(capi.EBSDError) as e:
        h.set_detector(wl.geometry(), acc, 1, wl.nEbins)
    assert e.value.code == capi.EBSD_EINVAL and "energy dimension" in str(e.value)
    h.close()


def test_c2_parity_64_orientations(built):
    """640x480 detector, 1001^2 x 11 master: the first 64 of the 10 000
    orientations in the three arithmetic modes against the oracle pixel by
    pixel, Lambert cells of all 64 x 307 200 pixel-orientations read out of
    the pattern kernel, and size-independent properties on the batch."""
    wl = synth.C2
    q = wl.quaternions(64)
    r = _three_modes(wl, q)
    # on the 1001^2 master a binary32 Lambert coordinate resolves 3e-5 of a
    # cell, so the accurate mode meets 1e-5 of FP64 as relative L2 only
    _gate_three_modes("C2", r, accurate_pixel=TOL_PIXEL_REF)
    assert r["cells"]["pixels"] == 64 * wl.numsx * wl.numsy
    # q and -q, and repeat determinism, on the whole batch
    h, det, sr, num_el = _setup(wl)
    epi = capi.epilogue(r["pref"])
    assert np.array_equal(r["default"], h.forward(-q, epi))
    assert np.array_equal(r["default"], h.forward(q, epi))
    h.close()


def test_forward_cells_match_at_every_launch_shape(built):
    """The cells instantiation stores the same cells and patterns whatever
    the launch shape (tile height, orientations per CTA, binning)."""
    O = _oracle()
    wl = synth.tiny(seed=3, numsx=100, numsy=70, npx=60, nE=6, mc_nsx=80, n_orient=21)
    h, det, sr, num_el = _setup(wl)
    q = wl.quaternions()
    ocells = det.cells(q, wl.npx)
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    for ty, oc, b in ((4, 1, 1), (8, 4, 2), (16, 64, 4), (4, 8, 8)):
        h.set_option("tile_y", ty)
        h.set_option("orient_per_cta", oc)
        epi = capi.epilogue(pref, binning=b, scalingmode="lin" if b > 1 else "not")
        out, cells = h.forward_cells(q, epi)
        assert np.array_equal(out, h.forward(q, epi)), (ty, oc, b)
        rep = cell_report(cells, ocells, wl.npx, wl.npx)
        assert rep["non_edge"] == 0, (ty, oc, b, rep)
    h.close()


def test_misaligned_device_quaternions_are_refused(built):
    """Kernels read quaternions as float4: a device pointer off a 16-byte
    boundary is refused before any launch (forward, adjoint, cells)."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    wl = synth.tiny()
    h, det, sr, num_el = _setup(wl)
    epi = capi.epilogue(capi.prefactor(15.0, 100.0, num_el))
    buf = torch.zeros(4 * 3 + 1, device="cuda")
    bad = buf.data_ptr() + 4
    out = torch.zeros((3, wl.numsy, wl.numsx), device="cuda")
    L = capi.lib()
    assert L.ebsd_forward(h.raw, bad, 3, C.byref(epi), capi._ptr(out)) == capi.EBSD_EINVAL
    assert "aligned" in L.ebsd_last_error(h.raw).decode()
    grad = torch.zeros((3, 6), device="cuda")
    assert L.ebsd_vjp(h.raw, bad, 3, C.byref(epi), 0, capi._ptr(out), None,
                      capi._ptr(grad)) == capi.EBSD_EINVAL
    nix = torch.zeros((3, wl.numsy, wl.numsx), dtype=torch.int32, device="cuda")
    fl = torch.zeros((3, wl.numsy, wl.numsx), device="cuda")
    assert L.ebsd_cells(h.raw, bad, 3, capi._ptr(nix), capi._ptr(nix), capi._ptr(fl),
                        capi._ptr(fl)) == capi.EBSD_EINVAL
    # the aligned start of the same buffer works
    good = buf[:12].view(3, 4)
    good[:, 0] = 1.0
    assert L.ebsd_forward(h.raw, good.data_ptr(), 3, C.byref(epi), capi._ptr(out)) == 0
    h.close()


def test_host_direct_matches_the_copy_path(built):
    """Option host_direct: the kernel stores into the pinned destination
    directly; the records are identical to the staged-copy path."""
    torch = pytest.importorskip("torch")
    wl = synth.tiny(seed=9, numsx=64, numsy=48, npx=60, nE=5, mc_nsx=80, n_orient=37)
    h, det, sr, num_el = _setup(wl)
    epi = capi.epilogue(capi.prefactor(15.0, 100.0, num_el), binning=2, scalingmode="gam",
                        gammavalue=0.33)
    q = wl.quaternions()
    ox, oy = h.output_dims(epi)
    hq = torch.from_numpy(q).pin_memory()
    a = torch.full((len(q), oy, ox), -1.0).pin_memory()
    b = torch.full((len(q), oy, ox), -2.0).pin_memory()
    h.set_option("host_direct", 0)
    h.forward(hq, epi, out=a)
    h.set_option("host_direct", 1)
    h.forward(hq, epi, out=b)
    assert torch.equal(a, b)
    dq = torch.from_numpy(q).cuda()
    c = torch.full((len(q), oy, ox), -3.0).pin_memory()
    h.forward(dq, epi, out=c)  # device quaternions, pinned output
    assert torch.equal(a, c)
    h.close()


def test_binning_8_with_a_four_row_tile(built):
    """A 4-row tile cannot hold an 8x8 block: the launch raises the tile height,
    so the records equal those of an 8-row tile."""
    wl = synth.tiny(seed=4, numsx=80, numsy=64, npx=60, nE=5, mc_nsx=80, n_orient=9)
    h, det, sr, num_el = _setup(wl)
    q = wl.quaternions()
    epi = capi.epilogue(capi.prefactor(15.0, 100.0, num_el), binning=8, scalingmode="lin")
    h.set_option("tile_y", 8)
    a = h.forward(q, epi)
    h.set_option("tile_y", 4)
    b = h.forward(q, epi)
    assert np.array_equal(a, b) and np.abs(a).max() > 0
    h.close()


def test_shared_detector_matches_own_setup_and_copies_on_write(built):
    """ebsd_share_detector: a handle on another handle's detector makes the
    same records as the source; when a holder changes its geometry (a new
    set-up, or a pattern-centre refinement) it takes tables of its own and
    the other holders keep theirs; the tables outlive the source handle."""
    torch = pytest.importorskip("torch")
    wl = synth.tiny(seed=9, numsx=64, numsy=48, npx=60, nE=5, mc_nsx=80, n_orient=7)
    sr, acc = workload_data(wl)
    h, det, _, num_el = _setup(wl)
    q = wl.quaternions()
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    epi = capi.epilogue(pref, binning=2, scalingmode="gam", gammavalue=0.33)
    own = h.forward(q, epi)
    s = capi.Handle(0)
    s.share_detector(h)
    assert np.array_equal(s.forward(q, epi), own)
    # the source moves its pattern centre: the sharing handle is unaffected
    h.set_detector(dict(wl.geometry(), xpc=wl.xpc + 3.0), acc, 1, wl.nEbins)
    assert not np.array_equal(h.forward(q, epi), own)
    assert np.array_equal(s.forward(q, epi), own)
    h.close()
    assert np.array_equal(s.forward(q, epi), own)
    # a second holder, then a pattern-centre refinement on the first
    s2 = capi.Handle(0)
    s2.share_detector(s)
    lin = capi.epilogue(pref)
    dq = torch.from_numpy(q).cuda()
    targets = torch.from_numpy(s.forward(q, lin)).cuda()
    s.refine(dq, lin, targets, max_iterations=2, refine_pc=True)
    assert np.array_equal(s2.forward(q, epi), own)
    s.close()
    s2.close()


def test_binary64_geometry_epilogues_batch_and_refusals(built):
    """Option lambert_accurate = 2 (binary64 geometry): every epilogue
    against the FP64 oracle pixel by pixel, a batched job equal to its own
    launch, and the cells diagnostic refused."""
    torch = pytest.importorskip("torch")
    O = _oracle()
    wl = synth.tiny(seed=5, numsx=64, numsy=48, npx=60, nE=5, mc_nsx=80, n_orient=9)
    wl.delta = 60.0
    wl.name = wl.name + "-b64"
    h, det, sr, num_el = _setup(wl)
    h.set_option("lambert_accurate", 2)
    q = wl.quaternions()
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    p64 = det.patterns_f64(sr, q, pref)
    for b, mode in ((1, "not"), (1, "gam"), (2, "lin"), (4, "gam"), (8, "lin"), (8, "gam")):
        out = h.forward(q, capi.epilogue(pref, binning=b, scalingmode=mode, gammavalue=0.33))
        ref = np.stack([O.epilogue_f64(p, b, capi.SCALING[mode], 0.33) for p in p64])
        l2, mx = rel_errors(out, ref)
        assert l2.max() <= TOL_FP64 and mx.max() <= TOL_FP64, (b, mode, l2.max(), mx.max())
    epi = capi.epilogue(pref, binning=2, scalingmode="gam", gammavalue=0.33)
    dq = torch.from_numpy(q).cuda()
    ox, oy = h.output_dims(epi)
    out = torch.full((len(q), oy, ox), -1.0, device="cuda")
    capi.Handle(0).forward_batched([(h, dq, epi, out)], graph=True, queue_all=True)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), h.forward(q, epi))
    with pytest.raises(capi.EBSDError) as e:
        h.cells(q)
    assert e.value.code == capi.EBSD_EUNSUPPORTED
    with pytest.raises(capi.EBSDError):
        h.set_option("lambert_accurate", 3)
    h.close()


@pytest.mark.parametrize("nE", [40, 64])
def test_wide_energy_windows(built, nE):
    """Energy windows of 40 and 64 bins (10 and 16 float4 per master node, the
    widest the pattern kernel is built for) against the FP64 oracle, with a
    window that leaves out the first and last bins (CTEMEBSD.f90:361-367)."""
    O = _oracle()
    wl = synth.tiny(seed=13, numsx=48, numsy=40, npx=40, nE=nE, mc_nsx=60, n_orient=5)
    wl.name = f"{wl.name}-nE{nE}-wide"
    Emin, Emax = 2, nE - 1
    h, det, sr, num_el = _setup(wl, Emin=Emin, Emax=Emax, accurate=True)
    assert num_el == det.num_el
    q = wl.quaternions()
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    for kw in (dict(), dict(binning=2, scalingmode="gam", gammavalue=0.4)):
        out = h.forward(q, capi.epilogue(pref, **kw))
        p64 = det.patterns_f64(sr, q, pref)
        if kw:
            p64 = np.stack([O.epilogue_f64(p, 2, 2, 0.4) for p in p64])
        l2, mx = rel_errors(out, p64)
        assert l2.max() <= TOL_FP64 and mx.max() <= TOL_FP64, (nE, kw, l2.max(), mx.max())
    with pytest.raises(capi.EBSDError) as e:  # the adjoint serves windows of up to 32 bins
        h.vjp(q, capi.epilogue(pref), np.ones((len(q), 40, 48), np.float32), "ndp")
    assert e.value.code == capi.EBSD_EUNSUPPORTED
    h.close()
