"""File formats, namelist and angle files through the C ABI (no GPU)."""
from __future__ import annotations

import struct

import numpy as np
import pytest

from ctemsoft_gb300 import capi, formats, synth


@pytest.fixture(scope="module")
def lib(built):
    return capi.lib()


def test_mc_file_round_trip(lib, tmp_path):
    rng = np.random.default_rng(1)
    acc = rng.integers(0, 50, size=(41, 41, 7), dtype=np.int32)
    p = tmp_path / "mc.data"
    formats.write_mc_file(p, acc, EkeV=20.0, Ehistmin=14.0, Ebinsize=1.0, sig=70.0, omega=0.0,
                          num_el=2_000_000, nthreads=8)
    h, a = capi.read_mc_file(p)
    assert (h.numEbins, h.numsx, h.numsy) == (7, 41, 41)
    assert (h.EkeV, h.Ehistmin, h.Ebinsize, h.sig) == (20.0, 14.0, 1.0, 70.0)
    assert h.num_el_total == 2_000_000 and h.nthreads == 8 and h.MCmode == b"CSDA"
    assert np.array_equal(a, acc)
    # the 6 x int32 header variant that CTEMEBSD.f90:332 reads
    recs = formats.read_records(p)
    assert len(recs[3]) == 28


def test_master_file_round_trip(lib, tmp_path):
    rng = np.random.default_rng(2)
    sr = rng.random((2, 5, 21, 21), dtype=np.float32)
    p = tmp_path / "master.data"
    formats.write_master_file(p, sr, [16, 17, 18, 19, 20], atomtype=[28, 22])
    h, ek, at, s2 = capi.read_master_file(p)
    assert (h.npx, h.npy, h.nE, h.numset, h.sqorhe) == (10, 10, 5, 2, b"square")
    assert np.array_equal(ek, [16, 17, 18, 19, 20]) and np.array_equal(at, [28, 22])
    assert np.array_equal(s2, sr)


def test_truncated_files_are_format_errors(lib, tmp_path):
    acc = np.zeros((21, 21, 3), np.int32)
    p = tmp_path / "mc.data"
    formats.write_mc_file(p, acc, EkeV=20.0, Ehistmin=18.0, Ebinsize=1.0)
    data = p.read_bytes()
    start = sum(len(r) + 8 for r in formats.read_records(p)[:7])  # accum_e record
    (tmp_path / "cut.data").write_bytes(data[: start + 100])
    with pytest.raises(capi.EBSDError) as e:
        capi.read_mc_file(tmp_path / "cut.data")
    assert e.value.code == capi.EBSD_EFORMAT
    bad = bytearray(data)
    bad[start + 4 + len(formats.read_records(p)[7])] ^= 0x7F  # accum_e's trailing marker
    (tmp_path / "bad.data").write_bytes(bytes(bad))
    with pytest.raises(capi.EBSDError):
        capi.read_mc_file(tmp_path / "bad.data")
    with pytest.raises(capi.EBSDError) as e:
        capi.read_mc_file(tmp_path / "missing.data")
    assert e.value.code == capi.EBSD_EIO


def test_namelist_defaults(lib, tmp_path):
    p = tmp_path / "d.nml"
    p.write_text("&EBSDdata\n/\n")
    n = capi.read_namelist(p)
    # CTEMEBSD.f90:179-198
    assert n["L"] == 20000.0 and n["thetac"] == 0.0 and n["delta"] == 25.0
    assert (n["numsx"], n["numsy"]) == (640, 480)
    assert (n["energymin"], n["energymax"]) == (15.0, 30.0)
    assert n["anglefile"] == "euler.txt" and n["eulerconvention"] == "tsl"
    assert n["FZfile"] == "FZ.data" and n["energyfile"] == "energy.data"
    assert n["datafile"] == "EBSDout.data"
    assert n["beamcurrent"] == 14.513 and n["dwelltime"] == 100.0
    assert n["scalingmode"] == "not" and n["gammavalue"] == 1.0 and n["binning"] == 1
    assert n["axisangle"] == [0, 0, 0, 0]
    assert n["poisson"] == 1 and n["seed"] == 1
    assert n["resume"] == 0 and n["ncubochoric"] == 0 and n["pgnum"] == 32


def test_namelist_syntax(lib, tmp_path):
    p = tmp_path / "s.nml"
    p.write_text(
        "! leading comment\n"
        " &ebsddata  ! group names are case-insensitive\n"
        "  L = 15250.0, THETAC=10.0 delta = 4.9375D1\n"
        "  numsx = 80 numsy=60\n"
        "  xpc = 3.57, ypc = -113.45\n"
        "  anglefile = 'it''s here.txt'\n"
        "  eulerconvention = \"hkl\"\n"
        "  beamcurrent = 1.5d1, dwelltime = 1.0E2\n"
        "  axisangle = 2*0.0, 1.0, 45.0\n"
        "  axisangle(1) = 0.5\n"
        "  scalingmode = 'gamma'  ! longer than character(3): truncated\n"
        "  poisson = .false.\n"
        "  seed = 42\n"
        "  resume = .true., ncubochoric = 50, pgnum = 24\n"
        " /\n"
        "trailing text after the group is ignored\n")
    n = capi.read_namelist(p)
    assert n["L"] == 15250.0 and n["thetac"] == 10.0 and n["delta"] == 49.375
    assert (n["numsx"], n["numsy"]) == (80, 60)
    assert n["xpc"] == np.float32(3.57) and n["ypc"] == np.float32(-113.45)
    assert n["anglefile"] == "it's here.txt" and n["eulerconvention"] == "hkl"
    assert n["beamcurrent"] == 15.0 and n["dwelltime"] == 100.0
    assert n["axisangle"] == [0.5, 0.0, 1.0, 45.0]
    assert n["scalingmode"] == "gam"
    assert n["poisson"] == 0 and n["seed"] == 42
    assert n["resume"] == 1 and n["ncubochoric"] == 50 and n["pgnum"] == 24


@pytest.mark.parametrize("text,code", [
    ("&EBSDdata\n bogus = 1\n/\n", capi.EBSD_EFORMAT),
    ("&EBSDdata\n numsx = abc\n/\n", capi.EBSD_EFORMAT),
    ("&OTHERgroup\n L = 1.0\n/\n", capi.EBSD_EFORMAT),
    ("&EBSDdata\n L = \n/\n", capi.EBSD_EFORMAT),
])
def test_namelist_errors(lib, tmp_path, text, code):
    p = tmp_path / "e.nml"
    p.write_text(text)
    with pytest.raises(capi.EBSDError) as e:
        capi.read_namelist(p)
    assert e.value.code == code
    with pytest.raises(capi.EBSDError) as e:
        capi.read_namelist(tmp_path / "nope.nml")
    assert e.value.code == capi.EBSD_EIO


def test_angle_files(lib, tmp_path):
    from oracle import oracle as O
    q = synth.shoemake_quaternions(9, 5)
    formats.write_angle_file(tmp_path / "q.txt", quats=q)
    assert np.array_equal(capi.read_angle_file(tmp_path / "q.txt"), q)
    e = np.random.default_rng(0).uniform(0, 360, (7, 3)).astype(np.float32)
    formats.write_angle_file(tmp_path / "e.txt", eulers=e)
    for conv in ("tsl", "hkl"):
        for aa in ((0, 0, 0, 0), (1, 1, 0, 35.0)):
            got = capi.read_angle_file(tmp_path / "e.txt", conv, aa)
            ref = O.angles_to_quats(e, "eu", conv == "hkl", aa)
            assert np.array_equal(got, ref)
    # rows may wrap over lines and use commas (list-directed input)
    (tmp_path / "w.txt").write_text("eu\n2\n10.0, 20.0\n30.0\n 40.0 50.0 60.0 ! tail\n")
    got = capi.read_angle_file(tmp_path / "w.txt")
    ref = O.angles_to_quats(np.array([[10, 20, 30], [40, 50, 60]], np.float32), "eu")
    assert np.array_equal(got, ref)
    (tmp_path / "short.txt").write_text("qu\n3\n1 0 0 0\n")
    with pytest.raises(capi.EBSDError) as err:
        capi.read_angle_file(tmp_path / "short.txt")
    assert err.value.code == capi.EBSD_EFORMAT


def test_output_record_offsets(tmp_path):
    """Pattern k of an output file starts at byte 24 + k*(nx*ny + 2)*4, the
    offset the reference's IDL viewer uses (EBSDshowPattern.pro:81)."""
    nx, ny, n = 5, 3, 4
    pats = [np.full((ny, nx), k + 0.5, np.float32) for k in range(n)]
    p = tmp_path / "out.data"
    with open(p, "wb") as f:
        formats._record(f, struct.pack("<3i", nx, ny, n))
        for a in pats:
            formats._record(f, a.tobytes())
    data = p.read_bytes()
    for k in range(n):
        off = 24 + k * (nx * ny + 2) * 4
        assert np.frombuffer(data[off:off + 4], "<f4")[0] == k + 0.5
    hdr, recs = formats.read_output_file(p)
    assert hdr == (nx, ny, n) and all(np.array_equal(r, a.ravel()) for r, a in zip(recs, pats))


def test_host_arithmetic_matches_oracle(lib):
    from oracle import oracle as O
    for args in [(15.0, 30.0, 10.0, 1.0, 11), (5.0, 20.0, 6.0, 1.0, 15), (12.5, 13.5, 10.0, 1.0, 11)]:
        assert capi.energy_window(*args) == O.energy_window(*args)
    assert capi.prefactor(15.0, 100.0, 1234) == O.prefactor(15.0, 100.0, 1234)
