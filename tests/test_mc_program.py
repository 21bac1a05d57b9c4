"""The CTEMMC drop-in on the CPU side: the &MCdata namelist (defaults of
CTEMMC.f90:171-183, the added material keys) and the ctemmc command line."""
from __future__ import annotations

import subprocess

import pytest

from ctemsoft_gb300 import capi


@pytest.fixture(scope="module")
def lib(built):
    return capi.lib()


def test_mc_namelist_defaults(lib, tmp_path):
    p = tmp_path / "d.nml"
    p.write_text("&MCdata\n/\n")
    n = capi.read_mc_namelist(p)
    assert n["MCmode"] == "CSDA" and n["xtalname"] == "undefined"
    assert n["sig"] == 70.0 and n["omega"] == 0.0 and n["numsx"] == 1501
    assert n["primeseed"] == 932117 and n["num_el"] == 10000000 and n["nthreads"] == 4
    assert n["EkeV"] == 30.0 and n["Ehistmin"] == 20.0 and n["Ebinsize"] == 0.25
    assert n["depthmax"] == 50.0 and n["depthstep"] == 1.0
    assert n["dataname"] == "undefined.data"
    assert n["density"] == 0.0 and n["Ze"] == 0.0 and n["at_wt"] == 0.0


def test_mc_namelist_keys(lib, tmp_path):
    p = tmp_path / "k.nml"
    p.write_text("&mcdata xtalname = 'Ni.xtal', sig = 75.0D0, numsx = 501, num_el = 3000000000\n"
                 " EkeV = 25, Ehistmin = 15.0, Ebinsize = 0.5, dataname = 'out.data'\n"
                 " density = 8.9, Ze = 28, at_wt = 58.69, MCmode = 'CSDA' /\n")
    n = capi.read_mc_namelist(p)
    assert n["xtalname"] == "Ni.xtal" and n["sig"] == 75.0 and n["numsx"] == 501
    assert n["num_el"] == 3000000000 and n["EkeV"] == 25.0 and n["Ehistmin"] == 15.0
    assert n["dataname"] == "out.data" and n["density"] == 8.9 and n["Ze"] == 28.0
    # dataname is character(60) in the reference (CTEMMC.f90:135)
    p.write_text("&MCdata dataname = '" + "d" * 70 + "' /\n")
    assert capi.read_mc_namelist(p)["dataname"] == "d" * 60
    p.write_text("&MCdata bogus = 1 /\n")
    with pytest.raises(capi.EBSDError) as e:
        capi.read_mc_namelist(p)
    assert e.value.code == capi.EBSD_EFORMAT


def test_mc_dims(lib):
    p = capi.mc_params(EkeV=20.0, Ehistmin=10.0, Ebinsize=1.0, depthmax=100.0, depthstep=1.0)
    assert capi.mc_dims(p) == (11, 101)
    with pytest.raises(capi.EBSDError):
        capi.mc_dims(capi.mc_params(numsx=1500))


def test_ctemmc_template_and_help(lib, tmp_path):
    exe = capi.LIB_PATH.parent / "ctemmc"
    r = subprocess.run([str(exe), "-t"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0
    n = capi.read_mc_namelist(tmp_path / "CTEMMC.template")
    assert n["density"] > 0 and n["MCmode"] == "CSDA"
    r = subprocess.run([str(exe), "-h"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0 and "CTEMMC.nml" in r.stdout
