"""The C-ABI library loads and exports every function include/*.h declares
(no compute calls; runs without a GPU)."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from ctemsoft_gb300 import capi

ROOT = Path(__file__).resolve().parent.parent


def declared_functions() -> list[str]:
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(ebsd_[a-z0-9_]+)\s*\(", text):
            names.append(m.group(1))
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("ebsd_create", "ebsd_destroy", "ebsd_set_master", "ebsd_set_detector",
                 "ebsd_forward", "ebsd_last_error", "ebsd_run_namelist"):
        assert must in names


def test_every_declared_symbol_is_exported(built):
    lib = capi.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(capi.LIB_PATH)], capture_output=True,
                         text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    assert set(declared_functions()) <= exported


def test_binding_covers_the_header(built):
    assert set(declared_functions()) == set(capi.exported_symbols())


def test_errors_without_side_effects(built):
    lib = capi.lib()
    assert lib.ebsd_version() >= 100
    # null handles and bad arguments are reported, never crash
    assert lib.ebsd_set_master(None, None, 1, 1, 1, 1) == capi.EBSD_EINVAL
    assert lib.ebsd_forward(None, None, 1, None, None) == capi.EBSD_EINVAL
    assert b"null handle" in lib.ebsd_last_error(None)
    a, b = C.c_int32(), C.c_int32()
    assert lib.ebsd_energy_window(10.0, 20.0, 10.0, 0.0, 11, C.byref(a), C.byref(b)) == \
        capi.EBSD_EINVAL
    lib.ebsd_destroy(None)
    h = C.c_void_p()
    rc = lib.ebsd_create(C.byref(h), 0)
    if rc == capi.EBSD_OK:      # a GPU is present
        lib.ebsd_destroy(h)
    else:
        assert rc in (capi.EBSD_ECUDA, capi.EBSD_EINVAL)
        assert len(lib.ebsd_last_error(None)) > 0
    rc = lib.ebsd_create(C.byref(h), 10_000)
    assert rc in (capi.EBSD_ECUDA, capi.EBSD_EINVAL)
    # the newer entry points refuse bad arguments before any CUDA call
    assert lib.ebsd_share_detector(None, None) == capi.EBSD_EINVAL
    assert lib.ebsd_forward_cells(None, None, 1, None, None, None, None, None, None) == \
        capi.EBSD_EINVAL
    assert lib.ebsd_run_namelist_devices(b"x.nml", None, 1, 1) == capi.EBSD_EINVAL
    devs = (C.c_int32 * 1)(0)
    assert lib.ebsd_run_namelist_devices(b"x.nml", devs, 0, 1) == capi.EBSD_EINVAL
    assert lib.ebsd_run_namelist_devices(b"x.nml", devs, 65, 1) == capi.EBSD_EINVAL
    assert lib.ebsd_refine_sharded(None, 1, None, None, None, None, None, None, None,
                                   None) == capi.EBSD_EINVAL
    assert lib.ebsd_run_mc_namelist_devices(b"x.nml", None, 1, 1) == capi.EBSD_EINVAL
    # the bandwidth probe checks its arguments before any CUDA call
    v = C.c_double()
    assert lib.ebsd_measure_bandwidth(0, 9, 1 << 20, 3, C.byref(v)) == capi.EBSD_EINVAL
    assert lib.ebsd_measure_bandwidth(0, capi.BW_L2, 1 << 20, 0, C.byref(v)) == capi.EBSD_EINVAL
    assert lib.ebsd_measure_bandwidth(0, capi.BW_L2, 1 << 20, 3, None) == capi.EBSD_EINVAL
    assert lib.ebsd_measure_bandwidth(10_000, capi.BW_L2, 1 << 20, 3, C.byref(v)) == \
        capi.EBSD_EINVAL


def test_cli_help_and_template(built, tmp_path):
    exe = capi.LIB_PATH.parent / "ctemebsd"
    r = subprocess.run([str(exe), "-h"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0 and "nmlfile" in r.stdout
    r = subprocess.run([str(exe), "-t"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0
    tpl = tmp_path / "CTEMEBSD.template"
    assert tpl.exists()
    n = capi.read_namelist(tpl)  # the template parses with our own reader
    assert n["numsx"] == 640 and n["scalingmode"] == "not"
    r = subprocess.run([str(exe), str(tmp_path / "missing.nml")], capture_output=True,
                       text=True, cwd=tmp_path)
    assert r.returncode == 1 and "cannot open" in r.stderr


def test_fortran_module_binds_declared_functions():
    """Every bind(C, name=...) of the Fortran module names a function the C
    header declares, and the module's derived types mirror the C structs
    field by field."""
    src = (ROOT / "ctemsoft_gb300" / "fortran" / "ebsd_gpu.f90").read_text()
    bound = re.findall(r'bind\(C,\s*name="(ebsd_[a-z0-9_]+)"\)', src)
    assert bound and set(bound) <= set(declared_functions()), set(bound) - set(declared_functions())
    header = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "ebsd_gpu.h").read_text(), flags=re.S)
    for name in ("ebsd_geometry", "ebsd_epilogue", "ebsd_gn_options"):
        c_body = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + ";", header).group(1)
        c_fields = [f.strip().split()[-1] for decl in c_body.split(";") if decl.strip()
                    for f in decl.split(",")]
        f_body = re.search(r"type, bind\(C\) :: " + name + r"(.*?)end type", src, re.S).group(1)
        f_fields = [f.strip() for line in f_body.strip().splitlines()
                    for f in line.split("::")[1].split("!")[0].split(",")]
        assert [f.lower() for f in f_fields] == [f.lower() for f in c_fields], (name, f_fields,
                                                                                 c_fields)


def test_every_option_key_is_documented():
    """Each key ebsd_set_option accepts is described in the header, and an
    unknown key is rejected by name."""
    src = (ROOT / "ctemsoft_gb300" / "csrc" / "ebsd_capi.cu").read_text()
    body = src[src.index('extern "C" int ebsd_set_option'):]
    body = body[:body.index("\n}\n")]
    keys = sorted(set(re.findall(r'k == "([a-z0-9_]+)"', body)))
    assert "l2_persist" in keys and "orient_per_cta" in keys
    header = (ROOT / "include" / "ebsd_gpu.h").read_text()
    missing = [k for k in keys if f'"{k}"' not in header]
    assert not missing, missing
    assert "unknown option" in body
