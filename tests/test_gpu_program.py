"""The drop-in program end to end on the GPU: namelist + angle/MC/master
files in, the reference's unformatted output file out, checked against the
oracle (noise off); the CLI, the 'not'+binning header quirk and resume."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from ctemsoft_gb300 import capi, formats, synth
from tests.parity import TOL_REF, rel_errors

pytestmark = pytest.mark.gpu


def _inputs(tmp_path, **over):
    wl = synth.tiny(seed=8, numsx=64, numsy=48, npx=60, nE=5, mc_nsx=80)
    sr, acc = wl.master(), wl.mc()
    formats.write_mc_file(tmp_path / "mc.data", acc, EkeV=20.0, Ehistmin=16.0, Ebinsize=1.0,
                          sig=70.0)
    formats.write_master_file(tmp_path / "master.data", sr, wl.energies)
    rng = np.random.default_rng(3)
    eul = rng.uniform(0, 360, (13, 3)).astype(np.float32)
    eul[:, 1] = rng.uniform(0, 180, 13)
    formats.write_angle_file(tmp_path / "angles.txt", eulers=eul)
    nml = dict(L=wl.L, thetac=wl.thetac, delta=wl.delta, numsx=wl.numsx, numsy=wl.numsy,
               xpc=wl.xpc, ypc=wl.ypc, anglefile=str(tmp_path / "angles.txt"),
               eulerconvention="hkl", FZfile=str(tmp_path / "master.data"),
               energyfile=str(tmp_path / "mc.data"), datafile=str(tmp_path / "out.data"),
               beamcurrent=15.0, dwelltime=100.0, energymin=16.0, energymax=20.0, binning=2,
               scalingmode="gam", gammavalue=0.4, axisangle=[1.0, 0.0, 1.0, 20.0],
               poisson=False)
    nml.update(over)
    formats.write_namelist(tmp_path / "run.nml", **nml)
    return wl, sr, acc, eul, nml


def _expected(wl, sr, acc, eul, nml):
    from oracle import oracle as O
    q = O.angles_to_quats(eul, "eu", hkl=nml["eulerconvention"] == "hkl",
                          axisangle=nml["axisangle"])
    Emin, Emax = O.energy_window(nml["energymin"], nml["energymax"], 16.0, 1.0, wl.nEbins)
    det = O.Detector(wl.geometry(), acc, Emin, Emax)
    pref = O.prefactor(nml["beamcurrent"], nml["dwelltime"], det.num_el)
    p32 = det.patterns_f32(sr, q, pref)
    mode = capi.SCALING[nml["scalingmode"]]
    return np.stack([O.epilogue_f32(p, nml["binning"], mode, nml["gammavalue"]) for p in p32])


def test_program_matches_oracle(built, tmp_path):
    wl, sr, acc, eul, nml = _inputs(tmp_path)
    capi.run_namelist(tmp_path / "run.nml")
    hdr, recs = formats.read_output_file(tmp_path / "out.data")
    assert hdr == (32, 24, 13)
    out = np.stack([r.reshape(24, 32) for r in recs])
    l2, mx = rel_errors(out, _expected(wl, sr, acc, eul, nml))
    assert l2.max() <= TOL_REF, l2.max()


def test_cli_writes_the_same_file(built, tmp_path):
    _inputs(tmp_path)
    capi.run_namelist(tmp_path / "run.nml")
    a = (tmp_path / "out.data").read_bytes()
    (tmp_path / "out.data").unlink()
    exe = capi.LIB_PATH.parent / "ctemebsd"
    r = subprocess.run([str(exe), str(tmp_path / "run.nml")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Total computation time" in r.stdout and "intensity prefactor" in r.stdout
    assert (tmp_path / "out.data").read_bytes() == a


def test_not_mode_header_quirk(built, tmp_path):
    """scalingmode 'not' with binning 2: binned header, full-size records
    (CTEMEBSD.f90:557-561 vs :654-655)."""
    _inputs(tmp_path, scalingmode="not")
    capi.run_namelist(tmp_path / "run.nml")
    hdr, recs = formats.read_output_file(tmp_path / "out.data")
    assert hdr == (32, 24, 13)
    assert all(r.size == 64 * 48 for r in recs)


def test_resume_completes_an_interrupted_file(built, tmp_path):
    _inputs(tmp_path)
    capi.run_namelist(tmp_path / "run.nml")
    full = (tmp_path / "out.data").read_bytes()
    rec = 4 * 32 * 24 + 8
    cut = 20 + 5 * rec + rec // 2          # five records and half of the sixth
    (tmp_path / "out.data").write_bytes(full[:cut])
    _inputs(tmp_path, resume=True)
    capi.run_namelist(tmp_path / "run.nml")
    assert (tmp_path / "out.data").read_bytes() == full


def test_program_errors(built, tmp_path):
    _inputs(tmp_path, FZfile=str(tmp_path / "missing.data"))
    with pytest.raises(capi.EBSDError) as e:
        capi.run_namelist(tmp_path / "run.nml")
    assert e.value.code == capi.EBSD_EIO
    # master with a different number of energy bins than the MC file
    wl = synth.tiny(seed=8, numsx=64, numsy=48, npx=60, nE=5, mc_nsx=80)
    formats.write_master_file(tmp_path / "m4.data", wl.master()[:4], wl.energies[:4])
    _inputs(tmp_path, FZfile=str(tmp_path / "m4.data"))
    with pytest.raises(capi.EBSDError) as e:
        capi.run_namelist(tmp_path / "run.nml")
    assert "energy dimension" in str(e.value)


def test_program_noise_records_are_counts(built, tmp_path):
    """With Poisson noise on and neither binning nor scaling, every record
    holds integer counts."""
    _inputs(tmp_path, binning=1, scalingmode="not", poisson=True, seed=5)
    capi.run_namelist(tmp_path / "run.nml")
    hdr, recs = formats.read_output_file(tmp_path / "out.data")
    out = np.stack(recs)
    assert np.all(out == np.round(out)) and out.max() > 0


def test_dictionary_run(built, tmp_path):
    """ncubochoric > 0: the program samples the fundamental zone of pgnum
    instead of reading an angle file and writes one record per sample."""
    from oracle import oracle as O
    wl, sr, acc, _, nml = _inputs(tmp_path, ncubochoric=5, pgnum=32, binning=1,
                                  scalingmode="not", anglefile=str(tmp_path / "absent.txt"),
                                  axisangle=[0.0, 0.0, 1.0, 0.0])
    capi.run_namelist(tmp_path / "run.nml")
    hdr, recs = formats.read_output_file(tmp_path / "out.data")
    q = O.ro2qu(O.sample_rfz(5, 32)).astype(np.float32)
    assert hdr == (64, 48, len(q))
    out = np.stack(recs).reshape(len(q), 48, 64)
    Emin, Emax = O.energy_window(16.0, 20.0, 16.0, 1.0, wl.nEbins)
    det = O.Detector(wl.geometry(), acc, Emin, Emax)
    ref = det.patterns_f32(sr, q, O.prefactor(15.0, 100.0, det.num_el))
    l2, _ = rel_errors(out, ref)
    assert l2.max() <= TOL_REF


@pytest.mark.parametrize("over", [dict(), dict(binning=1, scalingmode="not", poisson=True,
                                                seed=5)], ids=["gam-bin2", "noise"])
def test_device_list_writes_the_same_file(built, tmp_path, over):
    """The orientations split over a device list -- here the one GPU listed
    two and three times: two or three handles and host threads writing
    their shards' records concurrently at their offsets -- give the
    single-device file byte for byte, Poisson noise included (keyed by each
    pattern's index in the whole list); also through the CLI's -d list."""
    _inputs(tmp_path, **over)
    capi.run_namelist(tmp_path / "run.nml", device=0)
    a = (tmp_path / "out.data").read_bytes()
    for devs in ([0, 0], [0, 0, 0]):
        (tmp_path / "out.data").unlink()
        capi.run_namelist(tmp_path / "run.nml", device=devs)
        assert (tmp_path / "out.data").read_bytes() == a, devs
    (tmp_path / "out.data").unlink()
    exe = capi.LIB_PATH.parent / "ctemebsd"
    r = subprocess.run([str(exe), "-d", "0,0", str(tmp_path / "run.nml")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "out.data").read_bytes() == a


def test_resume_after_a_shard_stopped_early(built, tmp_path):
    """A sharded run interrupted with a record missing in the middle (one
    shard stopped, a later shard went on): resume recomputes from the first
    incomplete record and the file equals the uninterrupted one."""
    _inputs(tmp_path)
    capi.run_namelist(tmp_path / "run.nml", device=[0, 0])
    full = (tmp_path / "out.data").read_bytes()
    rec = 4 * 32 * 24 + 8
    broken = bytearray(full)
    broken[20 + 3 * rec:20 + 4 * rec] = bytes(rec)   # record 3 never written
    (tmp_path / "out.data").write_bytes(bytes(broken))
    _inputs(tmp_path, resume=True)
    capi.run_namelist(tmp_path / "run.nml", device=[0, 0])
    assert (tmp_path / "out.data").read_bytes() == full


def test_device_list_errors(built, tmp_path):
    """A device list naming a GPU that does not exist fails before any
    output is written; sharing a detector from a handle without one is a
    call-order error."""
    _inputs(tmp_path)
    with pytest.raises(capi.EBSDError) as e:
        capi.run_namelist(tmp_path / "run.nml", device=[0, 999])
    assert e.value.code in (capi.EBSD_EINVAL, capi.EBSD_ECUDA)
    assert not (tmp_path / "out.data").exists()
    a, b = capi.Handle(0), capi.Handle(0)
    with pytest.raises(capi.EBSDError) as e:
        b.share_detector(a)
    assert e.value.code == capi.EBSD_ESTATE
