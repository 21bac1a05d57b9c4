"""The oracle's restatement of CTEMMC's Monte-Carlo backscatter histogram
(CTEMMC.f90:307-529): generator properties, accounting identities,
agreement between the GPU's Philox streams and the reference's own
generator, and backscatter physics.  The reference has no tests or fixtures
for this program."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O

NI = dict(Ze=28.0, density=8.908, at_wt=58.6934)
AL = dict(Ze=13.0, density=2.699, at_wt=26.98)
AU = dict(Ze=79.0, density=19.3, at_wt=196.97)


def test_generators_are_uniform():
    for kind, seed in ((1, 932118), (0, 7)):
        u = O.mc_uniforms(kind, seed, 3, 200000)
        assert u.min() > 0.0 and u.max() <= 1.0
        assert abs(u.mean() - 0.5) < 0.003 and abs(u.var() - 1 / 12) < 0.002
        h, _ = np.histogram(u, bins=20, range=(0, 1))
        chi2 = ((h - len(u) / 20) ** 2 / (len(u) / 20)).sum()
        assert chi2 < 50, (kind, chi2)  # 19 degrees of freedom


def test_reference_generator_streams_differ_by_seed():
    a = O.mc_uniforms(1, 932118, 0, 50)
    b = O.mc_uniforms(1, 932119, 0, 50)
    assert not np.array_equal(a, b)
    assert np.array_equal(a, O.mc_uniforms(1, 932118, 0, 50))


def test_accounting():
    p = O.mc_params(numsx=101)
    acc, accz, n = O.mc_philox(p, 3, 0, 5000)
    assert acc.sum() == n > 0
    assert 0 < accz.sum() <= n
    nE, nz = O.mc_dims(p)
    assert acc.shape == (101, 101, nE) and accz.shape == (11, 11, nz, nE)
    # disjoint electron ranges add up
    a1, z1, n1 = O.mc_philox(p, 3, 0, 2000)
    a2, z2, n2 = O.mc_philox(p, 3, 2000, 5000)
    assert np.array_equal(a1 + a2, acc) and np.array_equal(z1 + z2, accz) and n1 + n2 == n


def _yield(p, n=6000, seed=11):
    _, _, c = O.mc_philox(p, seed, 0, n)
    return c / n


def test_backscatter_physics():
    """Normal-incidence backscatter yield of Ni is about 0.3, grows with
    tilt and with atomic number (Al < Ni < Au).  The histogram records
    exits within the Lambert square (the forward hemisphere) above Emin, so
    a wide window (Ehistmin 1 keV) is used."""
    base = dict(EkeV=20.0, Ehistmin=1.5, Ebinsize=1.0, numsx=101)
    ni0 = _yield(O.mc_params(sig=0.0, **base, **NI))
    ni70 = _yield(O.mc_params(sig=70.0, **base, **NI))
    al0 = _yield(O.mc_params(sig=0.0, **base, **AL))
    au0 = _yield(O.mc_params(sig=0.0, **base, **AU))
    assert 0.22 < ni0 < 0.38, ni0
    assert ni70 > ni0 + 0.15
    assert al0 < ni0 < au0, (al0, ni0, au0)


def test_philox_and_reference_generator_agree_statistically():
    """Same physics, two generators: total counts within 4 sigma and
    energy spectra consistent (chi-square)."""
    p = O.mc_params(numsx=101)
    a, _, na = O.mc_philox(p, 5, 0, 16000)
    b, _, nb = O.mc_reference_rng(p, 932117, 2, 8000)
    frac_a, frac_b = na / 16000, nb / 16000
    sig = np.sqrt(2 * frac_a * (1 - frac_a) / 16000)
    assert abs(frac_a - frac_b) < 4 * sig
    ea, eb = a.sum(axis=(0, 1)).astype(float), b.sum(axis=(0, 1)).astype(float)
    m = (ea + eb) > 20
    chi2 = (((ea - eb) ** 2) / (ea + eb))[m].sum()
    assert chi2 < 3 * m.sum(), chi2


def test_out_of_range_parameters():
    with pytest.raises(ValueError):
        O.mc_dims(O.mc_params(numsx=100))
    with pytest.raises(ValueError):
        O.mc_dims(O.mc_params(EkeV=5.0, Ehistmin=10.0))


@pytest.mark.parametrize("ctr,key,want", [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
])
def test_philox_known_answers(ctr, key, want):
    """Philox4x32-10 against the known-answer vectors its authors publish
    with the generator (Salmon et al., SC'11; counter, key -> block)."""
    assert O.philox4x32_10(ctr, key).tolist() == list(want)
