"""ebsd_mc_run and the ctemmc program on the GPU: electron-by-electron
agreement with the oracle on the same Philox streams, range additivity,
pointer kinds, statistics against the reference's own generator, and an
MC file feeding the EBSD pattern loop."""
from __future__ import annotations

import numpy as np
import pytest

from ctemsoft_gb300 import capi, formats
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NI = dict(Ze=28.0, density=8.908, at_wt=58.6934)


def _pair(**kw):
    d = dict(EkeV=20.0, Ehistmin=10.0, Ebinsize=1.0, depthmax=100.0, depthstep=1.0, numsx=101,
             **NI)
    d.update(kw)
    return capi.mc_params(**d), O.mc_params(**d)


@pytest.mark.parametrize("sig,omega", [(70.0, 0.0), (0.0, 0.0), (60.0, 5.0)])
def test_matches_oracle_electron_by_electron(built, sig, omega):
    cp, op = _pair(sig=sig, omega=omega)
    h = capi.Handle(0)
    acc, accz, n = h.mc_run(cp, 21, 0, 20000, accum_z=True)
    ref, refz, nref = O.mc_philox(op, 21, 0, 20000)
    # the same draws for the same electrons; CUDA's and the C library's
    # binary64 transcendental functions differ in the last bits, which moves
    # an electron into another bin only rarely
    moved = np.abs(acc.astype(np.int64) - ref).sum() / 2
    print("counted", n, nref, "moved", moved)
    assert abs(n - nref) <= max(3, 0.002 * nref)
    assert moved <= max(5, 0.003 * nref)
    assert np.abs(accz.astype(np.int64) - refz).sum() / 2 <= max(5, 0.003 * nref)


def test_ranges_add_up_and_repeat(built):
    cp, _ = _pair()
    h = capi.Handle(0)
    a, z, n = h.mc_run(cp, 9, 0, 30000, accum_z=True)
    a1, z1, n1 = h.mc_run(cp, 9, 0, 12345, accum_z=True)
    a2, z2, n2 = h.mc_run(cp, 9, 12345, 30000 - 12345, accum_z=True)
    assert np.array_equal(a1 + a2, a) and np.array_equal(z1 + z2, z) and n1 + n2 == n
    b, y, m = h.mc_run(cp, 9, 0, 30000, accum_z=True)
    assert np.array_equal(a, b) and np.array_equal(z, y) and m == n
    assert a.sum() == n


def test_device_buffers(built):
    torch = pytest.importorskip("torch")
    cp, _ = _pair()
    h = capi.Handle(0)
    a, _, n = h.mc_run(cp, 4, 0, 10000)
    nE, nz = capi.mc_dims(cp)
    d = torch.full((101, 101, nE), 7, dtype=torch.int32, device="cuda")
    _, _, m = h.mc_run(cp, 4, 0, 10000, accum_e=d)
    torch.cuda.synchronize()
    assert m == n and np.array_equal(d.cpu().numpy(), a)


def test_errors(built):
    import ctypes as C
    h = capi.Handle(0)
    L = capi.lib()
    acc = np.zeros(10, np.int32)
    bad = capi.mc_params(numsx=100)
    assert L.ebsd_mc_run(h.raw, C.byref(bad), 1, 0, 10, capi._ptr(acc), None, None) == capi.EBSD_EINVAL
    bad = capi.mc_params(density=0.0)
    assert L.ebsd_mc_run(h.raw, C.byref(bad), 1, 0, 10, capi._ptr(acc), None, None) == capi.EBSD_EINVAL
    good = capi.mc_params(numsx=101)
    assert L.ebsd_mc_run(h.raw, C.byref(good), 1, -1, 10, capi._ptr(acc), None, None) == capi.EBSD_EINVAL


def test_statistics_against_the_reference_generator(built):
    """GPU (Philox) against the oracle with the reference's own streams:
    backscatter fraction within 4 sigma, energy spectrum chi-square."""
    cp, op = _pair()
    h = capi.Handle(0)
    a, _, n = h.mc_run(cp, 77, 0, 400000)
    b, _, nb = O.mc_reference_rng(op, 932117, 4, 5000)
    fa, fb = n / 400000, nb / 20000
    assert abs(fa - fb) < 4 * np.sqrt(fb * (1 - fb) / 20000)
    ea = a.sum(axis=(0, 1)) / 400000 * 20000
    eb = b.sum(axis=(0, 1)).astype(float)
    m = eb > 20
    chi2 = (((ea - eb) ** 2) / (eb + ea / 20))[m].sum()
    assert chi2 < 3 * m.sum(), chi2


def test_ctemmc_program_feeds_the_pattern_loop(built, tmp_path, monkeypatch):
    # dataname is character(60) in the reference: a relative name in the run folder
    monkeypatch.chdir(tmp_path)
    (tmp_path / "mc.nml").write_text(
        "&MCdata xtalname = 'Ni.xtal', density = 8.908, Ze = 28.0, at_wt = 58.6934,\n"
        " sig = 70.0, numsx = 121, num_el = 50000, nthreads = 2, primeseed = 5,\n"
        " EkeV = 20.0, Ehistmin = 16.0, Ebinsize = 1.0, depthmax = 100.0, depthstep = 1.0,\n"
        " dataname = 'MC.data' /\n")
    capi.run_mc_namelist(tmp_path / "mc.nml")
    hdr, acc = capi.read_mc_file(tmp_path / "MC.data")
    assert (hdr.numEbins, hdr.numsx, hdr.numsy, hdr.num_el_total, hdr.nthreads) == (5, 121, 121,
                                                                                  100000, 2)
    assert hdr.EkeV == 20.0 and hdr.sig == 70.0
    # the same histogram as the library call with the same seed and count
    cp = capi.mc_params(EkeV=20.0, Ehistmin=16.0, Ebinsize=1.0, depthmax=100.0, depthstep=1.0,
                        numsx=121, sig=70.0, **NI)
    h = capi.Handle(0)
    ref, _, _ = h.mc_run(cp, 5, 0, 100000)
    assert np.array_equal(acc, ref)
    recs = formats.read_records(tmp_path / "MC.data")
    assert recs[0][:10] == b"CTEMMC.f90" and recs[1] == b"2.0/2013"
    # the histogram drives a detector
    from ctemsoft_gb300 import synth
    wl = synth.tiny(seed=3, numsx=32, numsy=24, npx=60, nE=5)
    h.set_master(wl.master())
    num_el = h.set_detector(wl.geometry(), acc, 1, 5)
    assert num_el > 0
    out = h.forward(wl.quaternions(4), capi.epilogue(capi.prefactor(15.0, 100.0, num_el)))
    assert np.isfinite(out).all() and out.max() > 0


def test_ctemmc_device_list_writes_the_same_file(built, tmp_path, monkeypatch):
    """The electrons split over a device list (the one GPU listed two and
    three times: a handle and host thread each, histograms added on the
    host) give the single-device MC file byte for byte; also through the
    CLI's -d list."""
    import subprocess
    monkeypatch.chdir(tmp_path)
    (tmp_path / "mc.nml").write_text(
        "&MCdata xtalname = 'Ni.xtal', density = 8.908, Ze = 28.0, at_wt = 58.6934,\n"
        " sig = 70.0, numsx = 121, num_el = 30001, nthreads = 3, primeseed = 7,\n"
        " EkeV = 20.0, Ehistmin = 16.0, Ebinsize = 1.0, depthmax = 100.0, depthstep = 1.0,\n"
        " dataname = 'MC.data' /\n")
    capi.run_mc_namelist(tmp_path / "mc.nml", device=0)
    one = (tmp_path / "MC.data").read_bytes()
    for devs in ([0, 0], [0, 0, 0]):
        (tmp_path / "MC.data").unlink()
        capi.run_mc_namelist(tmp_path / "mc.nml", device=devs)
        assert (tmp_path / "MC.data").read_bytes() == one, devs
    (tmp_path / "MC.data").unlink()
    exe = capi.LIB_PATH.parent / "ctemmc"
    r = subprocess.run([str(exe), "-d", "0,0", "mc.nml"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "MC.data").read_bytes() == one


def test_fp32_option_is_statistically_equivalent(built):
    """mc_fp32: the same trajectory steps in binary32.  On the same streams the
    two precisions start from the same draws and drift apart only by
    rounding, so backscatter fraction, energy spectrum and the coarse angular
    distribution agree within counting noise."""
    cp, _ = _pair()
    h = capi.Handle(0)
    a64, z64, n64 = h.mc_run(cp, 31, 0, 300000, accum_z=True)
    h.set_option("mc_fp32", 1)
    a32, z32, n32 = h.mc_run(cp, 31, 0, 300000, accum_z=True)
    assert a32.sum() == n32 and abs(n32 - n64) < 4 * np.sqrt(n64)
    e64, e32 = a64.sum(axis=(0, 1)).astype(float), a32.sum(axis=(0, 1)).astype(float)
    m = (e64 + e32) > 20
    chi2 = (((e64 - e32) ** 2) / (e64 + e32))[m].sum()
    assert chi2 < 3 * m.sum(), chi2
    # angular distribution on 10x10-pixel blocks
    g64 = a64.sum(axis=2)[:100, :100].reshape(10, 10, 10, 10).sum(axis=(1, 3)).astype(float)
    g32 = a32.sum(axis=2)[:100, :100].reshape(10, 10, 10, 10).sum(axis=(1, 3)).astype(float)
    m = (g64 + g32) > 20
    chi2 = (((g64 - g32) ** 2) / (g64 + g32))[m].sum()
    assert chi2 < 3 * m.sum(), chi2
    assert abs(int(z32.sum()) - int(z64.sum())) < 4 * np.sqrt(z64.sum())
    h.set_option("mc_fp32", 0)
    b64, _, m64 = h.mc_run(cp, 31, 0, 300000)
    assert np.array_equal(b64, a64) and m64 == n64
