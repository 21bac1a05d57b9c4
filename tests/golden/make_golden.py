"""Generate the golden fixtures in this folder from the CPU oracle.

The reference ships no fixtures for this path and cannot be built here
(Fortran, no compiler), so these vectors are outputs of the oracle on small
seeded synthetic inputs; the oracle itself is pinned by the analytic
known-answer tests in tests/test_oracle_kat.py.  The fixtures freeze the
oracle's behaviour (regression) and give the GPU tests fixed inputs and
expected outputs that do not depend on re-running the oracle.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from ctemsoft_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = {
    "tiny_ni": dict(wl=synth.tiny(), binning=1, mode=2, gamma=0.33, window=None),
    "tiny_ti_bin4": dict(wl=synth.tiny(seed=11, numsx=37, numsy=29, npx=33, nE=7, phase="Ti"),
                         binning=4, mode=2, gamma=0.5, window=(2, 6)),
    "tiny_ni_lin2": dict(wl=synth.tiny(seed=3, numsx=40, numsy=32, npx=25, nE=4, mc_nsx=30,
                                       n_orient=4), binning=2, mode=1, gamma=1.0, window=None),
}


def make(name: str, spec: dict) -> dict:
    wl = spec["wl"]
    sr, acc = wl.master(), wl.mc()
    q = wl.quaternions()
    Emin, Emax = spec["window"] or (1, wl.nEbins)
    det = O.Detector(wl.geometry(), acc, Emin, Emax)
    pref = O.prefactor(wl.beamcurrent, wl.dwelltime, det.num_el)
    nix, niy, i0, i1 = det.cells(q, wl.npx)
    p32 = det.patterns_f32(sr, q, pref)
    p64 = det.patterns_f64(sr, q, pref)
    e32 = np.stack([O.epilogue_f32(p, spec["binning"], spec["mode"], spec["gamma"]) for p in p32])
    e64 = np.stack([O.epilogue_f64(p, spec["binning"], spec["mode"], spec["gamma"]) for p in p64])
    meta = dict(name=name, geometry=wl.geometry(), npx=wl.npx, Emin=Emin, Emax=Emax,
                beamcurrent=wl.beamcurrent, dwelltime=wl.dwelltime, binning=spec["binning"],
                mode=spec["mode"], gamma=spec["gamma"], num_el=int(det.num_el), prefactor=pref)
    return dict(meta=np.array(json.dumps(meta)), sr=sr, accum_e=acc, quats=q,
                rgx=det.rg32[0], rgy=det.rg32[1], rgz=det.rg32[2], W32=det.W32, W64=det.W64,
                nix=nix, niy=niy, ixy0=i0, ixy1=i1, patterns_f32=p32, patterns_f64=p64,
                epilogue_f32=e32, epilogue_f64=e64)


def main():
    for name, spec in CASES.items():
        arrays = make(name, spec)
        np.savez_compressed(HERE / f"{name}.npz", **arrays)
        print(name, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
