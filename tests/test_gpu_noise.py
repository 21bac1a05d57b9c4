"""Poisson noise epilogue (the step of CTEMEBSD.f90:611-615), statistically:
per-pixel means and variances of many draws against the noise-free
intensity, for small means (inversion) and large means (PTRS)."""
from __future__ import annotations

import numpy as np
import pytest

from ctemsoft_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _setup():
    wl = synth.tiny(numsx=32, numsy=24, npx=40, nE=5)
    h = capi.Handle(0)
    h.set_master(wl.master())
    h.set_detector(wl.geometry(), wl.mc(), 1, 5)
    return wl, h


@pytest.mark.parametrize("target_mean", [3.0, 1000.0, 1.0e5])
def test_poisson_moments(built, target_mean):
    wl, h = _setup()
    q1 = wl.quaternions(1)
    clean = h.forward(q1, capi.epilogue(1.0))[0].astype(np.float64)
    pref = target_mean / clean.mean()
    lam = clean * pref
    n = 4000
    q = np.repeat(q1, n, axis=0)
    noisy = h.forward(q, capi.epilogue(pref, poisson=True, seed=123)).astype(np.float64)
    assert np.all(noisy == np.round(noisy)) and noisy.min() >= 0
    m = noisy.mean(axis=0)
    v = noisy.var(axis=0, ddof=1)
    ok = lam > 0.2
    # means: z-scores of the sample mean
    z = (m[ok] - lam[ok]) / np.sqrt(lam[ok] / n)
    assert np.abs(z).max() < 5.5, np.abs(z).max()
    assert abs(z.mean()) < 5.0 / np.sqrt(z.size)
    # variances: the sample variance of a Poisson(lam) has mean lam and
    # standard deviation ~ sqrt((lam + 2 lam^2) / n)
    zv = (v[ok] - lam[ok]) / np.sqrt((lam[ok] + 2 * lam[ok] ** 2) / n)
    assert np.abs(zv).max() < 6.0, np.abs(zv).max()
    assert abs(zv.mean()) < 6.0 / np.sqrt(zv.size)


def test_poisson_reproducible_and_chunk_independent(built):
    torch = pytest.importorskip("torch")
    wl, h = _setup()
    q = wl.quaternions(300)
    epi = capi.epilogue(50.0, poisson=True, seed=9)
    a = h.forward(q, epi)
    b = h.forward(q, epi)
    assert np.array_equal(a, b)
    c = h.forward(q, capi.epilogue(50.0, poisson=True, seed=10))
    assert not np.array_equal(a, c)
    # one device launch vs the chunked host path (640x480: 2 chunks of 218
    # patterns): the same draws
    big = synth.tiny(numsx=640, numsy=480, npx=40, nE=5)
    hb = capi.Handle(0)
    hb.share_master(h)
    hb.set_detector(big.geometry(), big.mc(), 1, 5)
    host = hb.forward(q, epi)
    dout = torch.empty(host.shape, device="cuda")
    hb.forward(torch.from_numpy(q).cuda(), epi, out=dout)
    torch.cuda.synchronize()
    assert np.array_equal(dout.cpu().numpy(), host)
    # noise, then binning and gamma, in the reference's order
    g = h.forward(q[:5], capi.epilogue(50.0, binning=4, scalingmode="gam", gammavalue=0.5,
                                       poisson=True, seed=9))
    ref = (a[:5].reshape(5, 6, 4, 8, 4).sum(axis=(2, 4)) / 16.0) ** 0.5
    np.testing.assert_allclose(g, ref, rtol=2e-6)


def test_noise_index_offset_continues_a_list(built):
    """Option noise_index_offset: a caller computing a long orientation list
    in pieces sets each piece's start index and gets the draws of one call
    over the whole list (noise is keyed by seed, pattern index and pixel)."""
    wl, h = _setup()
    q = wl.quaternions(40)
    epi = capi.epilogue(50.0, poisson=True, seed=9)
    whole = h.forward(q, epi)
    h.set_option("noise_index_offset", 17)
    tail = h.forward(q[17:], epi)
    h.set_option("noise_index_offset", 0)
    assert np.array_equal(tail, whole[17:])
    assert not np.array_equal(h.forward(q[17:], epi), whole[17:])
    with pytest.raises(capi.EBSDError):
        h.set_option("noise_index_offset", -1)


@pytest.mark.parametrize("lam", [12.5, 27.0, 29.5, 34.0, 340.0, 2.0e4, 1.0e6])
def test_poisson_distribution_shape(built, lam):
    """The whole distribution, not only its moments: a uniform master with
    uniform weights gives every pixel nearly the same mean, and 614 k draws are
    binned by standardised value and checked against the exact Poisson pmf
    (chi-square over bins with expected count >= 20)."""
    from scipy import stats
    wl = synth.tiny(numsx=64, numsy=48, npx=40, nE=5)
    sr = np.ones_like(wl.master())
    h = capi.Handle(0)
    h.set_master(sr)
    h.set_detector(wl.geometry(), wl.mc(), 1, 5)
    q = wl.quaternions(1)
    clean = h.forward(q, capi.epilogue(1.0))[0].astype(np.float64)
    inner = clean[8:-8, 8:-8]
    pref = lam / inner.mean()
    qq = np.repeat(q, 400, axis=0)
    noisy = h.forward(qq, capi.epilogue(pref, poisson=True, seed=77))[:, 8:-8, 8:-8]
    lams = (inner * pref)[None].repeat(400, 0)
    # per-pixel means differ slightly (MC weights): compare each draw's
    # Poisson CDF value, which is uniform for the exact distribution
    k = noisy.astype(np.float64).ravel()
    lv = lams.ravel()
    u_lo = stats.poisson.cdf(k - 1, lv)
    u_hi = stats.poisson.cdf(k, lv)
    rng = np.random.default_rng(1)
    u = u_lo + (u_hi - u_lo) * rng.random(u_lo.size)   # randomised PIT
    hist, _ = np.histogram(u, bins=50, range=(0, 1))
    exp = u.size / 50
    chi2 = ((hist - exp) ** 2 / exp).sum()
    assert chi2 < 100, chi2  # 49 degrees of freedom
