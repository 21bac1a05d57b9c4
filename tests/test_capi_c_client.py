"""The C ABI from a C program, as a Fortran or C host would use it: the header
compiles as C99 and as C++, a client links against libebsdgpu.so, and the
host-side entry points work and report errors through return codes and
ebsd_last_error (no GPU needed: device calls are expected to fail cleanly)."""
from __future__ import annotations

import shutil
import subprocess

import pytest

from ctemsoft_gb300 import capi

ROOT = capi.LIB_PATH.parents[2]

CLIENT = r"""
#include <stdio.h>
#include <string.h>
#include "ebsd_gpu.h"

int main(void)
{
    ebsd_handle* h = NULL;
    ebsd_namelist nml;
    int32_t e0 = 0, e1 = 0;
    int rc;
    printf("version %d\n", ebsd_version());
    printf("prefactor %.17g\n", ebsd_prefactor(15.0, 100.0, 123456));
    rc = ebsd_energy_window(10.0f, 20.0f, 10.0, 1.0, 11, &e0, &e1);
    printf("window %d %d %d\n", rc, e0, e1);
    rc = ebsd_read_namelist("/nonexistent/EBSD.nml", &nml);
    printf("namelist %d %d\n", rc, (int)strlen(ebsd_last_error(NULL)) > 0);
    rc = ebsd_create(&h, 0);
    printf("create %d %d %d\n", rc, h == NULL, (int)strlen(ebsd_last_error(NULL)) > 0);
    if (rc == 0) ebsd_destroy(h);
    return 0;
}
"""


def _cc():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    return cc


def test_header_compiles_as_c99_and_cpp(tmp_path):
    cc = _cc()
    src = tmp_path / "h.c"
    src.write_text('#include "ebsd_gpu.h"\nint main(void) { return ebsd_version() > 0 ? 0 : 1; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only",
                        f"-I{ROOT / 'include'}", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cxx = shutil.which("g++")
    if cxx:
        srcp = tmp_path / "h.cpp"
        srcp.write_text(src.read_text())
        r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-fsyntax-only",
                            f"-I{ROOT / 'include'}", str(srcp)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_c_client_links_and_reports_errors(built, tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("checks the no-device error path")
    cc = _cc()
    src = tmp_path / "client.c"
    src.write_text(CLIENT)
    exe = tmp_path / "client"
    lib = capi.LIB_PATH.parent
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", str(src), f"-I{ROOT / 'include'}",
                        f"-L{lib}", "-lebsdgpu", f"-Wl,-rpath,{lib}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    assert int(out["version"]) == capi.lib().ebsd_version()
    # CTEMEBSD.f90:545: 0.25 * 6.241e18 * beamcurrent * dwelltime * 1e-15 / num_el
    assert float(out["prefactor"]) == pytest.approx(
        0.25 * 6.241e18 * 15.0 * 100.0 * 1.0e-15 / 123456, rel=1e-15)
    assert out["window"].split() == ["0", "1", "11"]
    rc, has_msg = map(int, out["namelist"].split())
    assert rc == capi.EBSD_EIO and has_msg == 1
    rc, null_handle, has_msg = map(int, out["create"].split())
    assert rc in (capi.EBSD_ECUDA, capi.EBSD_EINVAL) and null_handle == 1 and has_msg == 1
