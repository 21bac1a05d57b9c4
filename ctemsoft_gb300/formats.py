"""Writers and readers for the reference's file formats (numpy).

All binary files are gfortran unformatted sequential files: every record is
an int32 byte count, the payload, and the same count again.

  MC file      CTEMMC.f90:262-277
  master file  CTEMEBSDmaster.f90:540-568
  output file  CTEMEBSD.f90:555-561,654-658
  angle file   CTEMEBSD.f90:228-275 (text)
  namelist     CTEMEBSD.f90:169-171 (&EBSDdata, text)

Arrays use C order with the Fortran first index last, e.g. the master
sr(-npx:npx,-npy:npy,nE,numset) is a numpy array (numset, nE, 2npy+1, 2npx+1).
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

FNLEN = 132  # local.f90:84


def _record(f, payload: bytes) -> None:
    n = len(payload)
    if n > 2147483639:
        raise ValueError("record larger than a gfortran sub-record; not needed here")
    f.write(struct.pack("<i", n))
    f.write(payload)
    f.write(struct.pack("<i", n))


def _chars(s: str, n: int) -> bytes:
    return s.encode()[:n].ljust(n, b" ")


def read_records(path) -> list[bytes]:
    """All records of an unformatted sequential file (sub-records joined)."""
    out = []
    with open(path, "rb") as f:
        data = f.read()
    i = 0
    cur = b""
    while i < len(data):
        (head,) = struct.unpack_from("<i", data, i)
        n = abs(head)
        cur += data[i + 4:i + 4 + n]
        (tail,) = struct.unpack_from("<i", data, i + 4 + n)
        if abs(tail) != n:
            raise ValueError(f"bad record marker at byte {i}")
        i += 8 + n
        if head >= 0:
            out.append(cur)
            cur = b""
    return out


def write_mc_file(path, accum_e: np.ndarray, *, EkeV: float, Ehistmin: float, Ebinsize: float,
                  depthmax: float = 100.0, depthstep: float = 1.0, sig: float = 70.0,
                  omega: float = 0.0, num_el: int = 0, nthreads: int = 1,
                  numzbins: int | None = None, xtalname: str = "synthetic.xtal",
                  MCmode: str = "CSDA") -> None:
    """accum_e shaped (2nsy+1, 2nsx+1, numEbins) int32 (Fortran (E,x,y))."""
    acc = np.ascontiguousarray(accum_e, dtype="<i4")
    gy, gx, nE = acc.shape
    nz = numzbins if numzbins is not None else int(depthmax / depthstep) + 1
    with open(path, "wb") as f:
        _record(f, _chars("CTEMMC.f90", FNLEN))
        _record(f, _chars("2.0/2013", 8))
        _record(f, _chars(xtalname, FNLEN))
        _record(f, struct.pack("<iiiiqi", nE, nz, gx, gy, num_el, nthreads))
        _record(f, struct.pack("<5d", EkeV, Ehistmin, Ebinsize, depthmax, depthstep))
        _record(f, struct.pack("<2d", sig, omega))
        _record(f, _chars(MCmode, 4))
        _record(f, acc.tobytes())
        # accum_z(numEbins, numzbins, -nx/10:nx/10, -nx/10:nx/10): zeros
        nzx = 2 * (((gx - 1) // 2) // 10) + 1
        _record(f, np.zeros((nzx, nzx, nz, nE), "<i4").tobytes())


def write_master_file(path, sr: np.ndarray, EkeVs, *, atomtype=None,
                      xtalname: str = "synthetic.xtal", energyfile: str = "MC.data",
                      sqorhe: str = "square") -> None:
    """sr shaped (numset, nE, 2npy+1, 2npx+1) float32 (Fortran (x,y,E,set))."""
    s = np.ascontiguousarray(sr, dtype="<f4")
    if s.ndim == 3:
        s = s[None]
    numset, nE, gy, gx = s.shape
    at = np.asarray(atomtype if atomtype is not None else [28] * numset, "<i4")
    with open(path, "wb") as f:
        _record(f, _chars("CTEMEBSDmaster.f90", FNLEN))
        _record(f, _chars("2.0/2013", 8))
        _record(f, _chars(xtalname, FNLEN))
        _record(f, _chars(energyfile, FNLEN))
        _record(f, struct.pack("<4i", (gx - 1) // 2, (gy - 1) // 2, nE, numset))
        _record(f, np.asarray(EkeVs, "<f4").tobytes())
        _record(f, at.tobytes())
        _record(f, _chars(sqorhe, 6))
        _record(f, s.tobytes())


def write_angle_file(path, quats: np.ndarray | None = None, eulers: np.ndarray | None = None):
    """'qu' file of scalar-first quaternions or 'eu' file of Euler angles
    (degrees), written with enough digits to round-trip float32 exactly."""
    with open(path, "w") as f:
        if quats is not None:
            q = np.asarray(quats, np.float32)
            f.write("qu\n%d\n" % len(q))
            for row in q:
                f.write(" ".join(repr(float(v)) for v in row) + "\n")
        else:
            e = np.asarray(eulers, np.float32)
            f.write("eu\n%d\n" % len(e))
            for row in e:
                f.write(" ".join(repr(float(v)) for v in row) + "\n")


def write_namelist(path, **kw) -> None:
    """&EBSDdata namelist with the given keys (strings quoted, bools as
    .TRUE./.FALSE., sequences comma separated)."""
    lines = ["&EBSDdata"]
    for k, v in kw.items():
        if isinstance(v, bool):
            s = ".TRUE." if v else ".FALSE."
        elif isinstance(v, str):
            s = "'" + v.replace("'", "''") + "'"
        elif isinstance(v, (list, tuple, np.ndarray)):
            s = ", ".join(repr(float(x)) for x in v)
        elif isinstance(v, float):
            s = repr(v)
        else:
            s = str(v)
        lines.append(f" {k} = {s}")
    lines.append(" /")
    Path(path).write_text("\n".join(lines) + "\n")


def read_output_file(path):
    """Returns (header (nx, ny, N), patterns list of float32 arrays shaped
    (ny_record, nx_record)) for a CTEMEBSD output file.  Record sizes are
    taken from the records themselves (the 'not' + binning header quirk)."""
    recs = read_records(path)
    nx, ny, n = struct.unpack("<3i", recs[0][:12])
    pats = [np.frombuffer(r, "<f4") for r in recs[1:]]
    return (nx, ny, n), pats
