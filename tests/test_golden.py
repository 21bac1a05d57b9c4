"""Golden fixtures (tests/golden/*.npz, made by make_golden.py).

CPU: the oracle reproduces its committed outputs (regression pin).
GPU: the library, fed the fixture inputs through the C ABI, matches the
committed outputs -- cells bit-exact except at cell edges, intensities
within the stated tolerances.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from tests.parity import TOL_FP64, TOL_REF, cell_report, near_edge, rel_errors

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load(name):
    z = np.load(GOLDEN / f"{name}.npz")
    d = {k: z[k] for k in z.files}
    d["meta"] = json.loads(str(d["meta"]))
    return d


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(built, name):
    from oracle import oracle as O
    d = load(name)
    m = d["meta"]
    det = O.Detector(m["geometry"], d["accum_e"], m["Emin"], m["Emax"])
    assert det.num_el == m["num_el"]
    for a, k in zip(det.rg32, ("rgx", "rgy", "rgz")):
        np.testing.assert_array_equal(a, d[k])
    np.testing.assert_allclose(det.W32, d["W32"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(det.W64, d["W64"], rtol=1e-12, atol=1e-12)
    nix, niy, i0, i1 = det.cells(d["quats"], m["npx"])
    # libm may differ by an ulp across platforms: cells agree away from edges
    diff = (nix != d["nix"]) | (niy != d["niy"])
    edge = near_edge(m["npx"], d["ixy0"]) | near_edge(m["npx"], d["ixy1"])
    assert not (diff & ~edge).any()
    p32 = det.patterns_f32(d["sr"], d["quats"], m["prefactor"])
    np.testing.assert_allclose(p32, d["patterns_f32"], rtol=1e-6)
    p64 = det.patterns_f64(d["sr"], d["quats"], m["prefactor"])
    np.testing.assert_allclose(p64, d["patterns_f64"], rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_golden(built, name):
    from ctemsoft_gb300 import capi
    d = load(name)
    m = d["meta"]
    with capi.Handle(0) as h:
        h.set_master(d["sr"])
        num_el = h.set_detector(m["geometry"], d["accum_e"], m["Emin"], m["Emax"])
        assert num_el == m["num_el"]
        rep = cell_report(h.cells(d["quats"]), (d["nix"], d["niy"], d["ixy0"], d["ixy1"]),
                          m["npx"], m["npx"])
        assert rep["non_edge"] == 0, rep
        raw = h.forward(d["quats"], capi.epilogue(m["prefactor"]))
        l2, mx = rel_errors(raw, d["patterns_f32"])
        assert l2.max() <= TOL_REF and mx.max() <= TOL_REF
        h.set_option("lambert_accurate", 1)
        raw = h.forward(d["quats"], capi.epilogue(m["prefactor"]))
        l2, mx = rel_errors(raw, d["patterns_f64"])
        assert l2.max() <= TOL_FP64 and mx.max() <= TOL_FP64, (l2.max(), mx.max())
        out = h.forward(d["quats"], capi.epilogue(m["prefactor"], binning=m["binning"],
                                                  scalingmode=m["mode"], gammavalue=m["gamma"]))
        assert out.shape == d["epilogue_f64"].shape
        l2, mx = rel_errors(out, d["epilogue_f64"])
        assert l2.max() <= TOL_FP64 and mx.max() <= TOL_FP64, (l2.max(), mx.max())
