"""Known-answer tests that pin the CPU oracle (no GPU).

The reference has no tests or fixtures for this path, so the oracle is
pinned analytically: Lambert map identities, quaternion identities,
closed-form rotation conversions, a uniform master, and agreement of the
single-precision restatement with its binary64 re-evaluation.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from ctemsoft_gb300 import synth
from tests.conftest import workload_data
from tests.parity import TOL_FP64, rel_errors

SPIO2 = math.sqrt(math.pi / 2)


@pytest.fixture(scope="module")
def O(built):
    from oracle import oracle
    return oracle


def test_lambert_poles_and_equator(O):
    for f in (O.lambert_inverse_f32, O.lambert_inverse_f64):
        r, ierr = f([0.0, 0.0, 1.0])
        assert ierr == 0 and r[0] == 0 and r[1] == 0
        r, ierr = f([0.0, 0.0, -1.0])  # intercepted, Lambert.f90:423
        assert ierr == 0 and r[0] == 0 and r[1] == 0
    r, _ = O.lambert_inverse_f64([1.0, 0.0, 0.0])
    assert r == pytest.approx([SPIO2, 0.0], abs=1e-15)
    r, _ = O.lambert_inverse_f64([0.0, 1.0, 0.0])
    assert r == pytest.approx([0.0, SPIO2], abs=1e-15)
    r, _ = O.lambert_inverse_f64([-1.0, 0.0, 0.0])
    assert r == pytest.approx([-SPIO2, 0.0], abs=1e-15)
    r, _ = O.lambert_inverse_f32([1.0, 0.0, 0.0])
    assert r[0] == pytest.approx(SPIO2, rel=1e-7) and r[1] == 0


def test_lambert_rejects_non_unit(O):
    r, ierr = O.lambert_inverse_f32([0.5, 0.5, 0.5])
    assert ierr == 1 and r[0] == 0 and r[1] == 0
    r, ierr = O.lambert_inverse_f64([1.0, 1e-5, 0.0])
    assert ierr == 1


def test_lambert_round_trip(O):
    """inverse(forward(xy)) == xy on the square (north hemisphere)."""
    rng = np.random.default_rng(0)
    pts = rng.uniform(-SPIO2, SPIO2, size=(500, 2))
    pts = np.vstack([pts, [[0.3, 0.3], [-0.7, 0.7], [SPIO2, 0.2], [0.0, -1.1]]])
    for xy in pts:
        k, ierr = O.lambert_forward_f64(xy)
        assert ierr == 0
        assert np.linalg.norm(k) == pytest.approx(1.0, abs=1e-13)
        back, ierr = O.lambert_inverse_f64(k)
        assert ierr == 0
        assert back == pytest.approx(xy, abs=1e-11)
        b32, ierr = O.lambert_inverse_f32((k / np.linalg.norm(k)).astype(np.float32))
        assert b32 == pytest.approx(xy, abs=2e-6)


def test_lambert_forward_matches_synth_grid(O):
    X = np.array([0.1, -0.4, 1.2, 0.0])
    Y = np.array([0.5, 0.2, -0.3, 0.0])
    sx, sy, sz = synth.lambert_forward(X, Y)
    for i in range(len(X)):
        k, _ = O.lambert_forward_f64([X[i], Y[i]])
        assert k == pytest.approx([sx[i], sy[i], sz[i]], abs=1e-14)


def test_equal_area(O):
    """The Rosca map is area preserving: a uniform grid on the square
    samples the hemisphere uniformly (mean z = 1/2)."""
    n = 301
    g = (np.arange(n) + 0.5) / n * 2 * SPIO2 - SPIO2
    X, Y = np.meshgrid(g, g)
    _, _, z = synth.lambert_forward(X, Y)
    assert z.mean() == pytest.approx(0.5, abs=2e-3)


def test_quaternion_algebra(O):
    i, j, k = [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]
    assert np.array_equal(O.quat_mult_f32(i, j), [0, 0, 0, 1])
    assert np.array_equal(O.quat_mult_f32(j, k), [0, 1, 0, 0])
    assert np.array_equal(O.quat_mult_f32(k, i), [0, 0, 1, 0])
    assert np.array_equal(O.quat_mult_f32(i, i), [-1, 0, 0, 0])
    one = [1, 0, 0, 0]
    q = np.array([0.5, 0.5, -0.5, 0.5], np.float32)
    assert np.array_equal(O.quat_mult_f32(one, q), q)


def test_eu2qu_closed_forms(O):
    assert O.eu2qu_f32([0, 0, 0]) == pytest.approx([1, 0, 0, 0])
    h = math.sqrt(0.5)
    # phi1 only: (cos(phi1/2), 0, 0, -sin(phi1/2)) (passive, rotations.f90:1342-1349)
    assert O.eu2qu_f32([math.pi / 2, 0, 0]) == pytest.approx([h, 0, 0, -h], abs=1e-7)
    # Phi only: (cos(Phi/2), -sin(Phi/2), 0, 0)
    assert O.eu2qu_f32([0, math.pi / 2, 0]) == pytest.approx([h, -h, 0, 0], abs=1e-7)
    # northern hemisphere: a rotation by more than pi flips to q0 >= 0
    q = O.eu2qu_f32([3 * math.pi / 2, 0, 0])
    assert q[0] >= 0 and q == pytest.approx([h, 0, 0, h], abs=1e-7)


def test_ax2qu_closed_forms(O):
    # om2qu (rotations.f90:1584-1594) takes sqrt(|1 + x11 - x22 - x33|) in
    # single precision: a component that is zero in exact arithmetic comes
    # out as sqrt(one rounding residue)/2, up to 2^-12 ~ 2.4e-4.  The
    # restatement keeps that behaviour, so the closed forms hold to 2.5e-4.
    h = math.sqrt(0.5)
    q = O.ax2qu_f32([0, 0, 1, math.pi / 2])
    assert q == pytest.approx([h, 0, 0, -h], abs=2.5e-4)
    assert q[1] > 0 and q[1] == pytest.approx(2.0 ** -13, rel=1e-6)  # the residue itself
    q = O.ax2qu_f32([1, 0, 0, math.pi / 3])
    assert q == pytest.approx([math.cos(math.pi / 6), -math.sin(math.pi / 6), 0, 0], abs=2.5e-4)
    # ax2qu agrees with eu2qu for a rotation about z
    assert O.ax2qu_f32([0, 0, 1, 0.7]) == pytest.approx(O.eu2qu_f32([0.7, 0, 0]), abs=2.5e-4)


def test_angle_ingest(O):
    e = np.array([[0, 0, 0], [90, 0, 0]], np.float32)
    q = O.angles_to_quats(e, "eu")
    assert q[0] == pytest.approx([1, 0, 0, 0])
    q_hkl = O.angles_to_quats(e[:1], "eu", hkl=True)  # +90 deg on phi1
    assert q_hkl[0] == pytest.approx(q[1], abs=1e-7)
    # axis-angle pre-rotation by 90 deg about z composes with the rows
    qa = O.angles_to_quats(e[:1], "eu", axisangle=(0, 0, 1, 90.0))
    assert qa[0] == pytest.approx(q[1], abs=2.5e-4)  # om2qu residue, see above


def test_energy_window_and_prefactor(O):
    assert O.energy_window(15.0, 30.0, 10.0, 1.0, 11) == (6, 11)   # defaults of :186-187
    assert O.energy_window(10.0, 20.0, 10.0, 1.0, 11) == (1, 11)
    assert O.energy_window(0.0, 5.0, 10.0, 1.0, 11) == (1, 1)
    assert O.energy_window(12.5, 13.4, 10.0, 1.0, 11) == (4, 4)    # nint rounds half away
    p = O.prefactor(15.0, 100.0, 2000)
    assert p == pytest.approx(0.25 * 6.241e18 * 15.0 * 100.0 * 1e-15 / 2000, rel=1e-15)


def test_detector_geometry(O):
    g = dict(L=15000.0, thetac=10.0, delta=20.0, numsx=64, numsy=48, xpc=1.5, ypc=-3.0,
             sig=70.0)
    acc = np.ones((21, 21, 2), np.int32)
    det = O.Detector(g, acc, 1, 2)
    x, y, z = det.rg32
    assert np.allclose(x * x + y * y + z * z, 1.0, atol=3e-7)
    for a, b in zip(det.rg32, det.rg64):
        assert np.abs(a - b).max() < 3e-7
    # the pattern centre pixel looks along (sin alp, 0, cos alp), alp = 30 deg
    X, Y, Z = (np.asarray(v, np.float64) for v in det.rg64)
    ic = 64 / 2 - 0.5 + 1.5  # scin_x = 0 at i = xpc + (numsx-1)/2 (0-based)
    jc = 48 / 2 - 0.5 - 3.0
    i0, j0 = int(ic), int(jc)
    assert abs(Y[j0, i0]) < 2 * 20 / 15000


def test_uniform_histogram_weights(O):
    """A constant MC histogram c gives weights 0.25*c in every selected bin."""
    g = dict(L=15000.0, thetac=10.0, delta=50.0, numsx=20, numsy=16, xpc=0.0, ypc=0.0, sig=70.0)
    acc = np.full((41, 41, 3), 8, np.int32)
    det = O.Detector(g, acc, 2, 3)
    assert np.allclose(det.W32[..., 1:], 2.0, rtol=1e-6)
    assert np.all(det.W32[..., 0] == 0)           # bins outside the window stay zero
    assert det.num_el == round(2.0 * 2 * 20 * 16)


def test_uniform_master(O):
    wl = synth.tiny()
    sr, acc = workload_data(wl)
    det = O.Detector(wl.geometry(), acc, 1, wl.nEbins)
    q = wl.quaternions()
    c = np.full_like(sr, 3.0)
    p = det.patterns_f32(c, q, 1.0)
    expect = 3.0 * det.W32.astype(np.float64).sum(axis=-1)
    np.testing.assert_allclose(p, np.broadcast_to(expect, p.shape), rtol=2e-6)


def test_q_minus_q_and_identity(O):
    wl = synth.tiny()
    sr, acc = workload_data(wl)
    det = O.Detector(wl.geometry(), acc, 1, wl.nEbins)
    q = wl.quaternions()
    assert np.array_equal(det.patterns_f32(sr, q, 1.0), det.patterns_f32(sr, -q, 1.0))
    # identity: gather at the detector directions, checked with numpy
    p = det.patterns_f64(sr, np.array([[1, 0, 0, 0]], np.float32), 1.0)[0]
    x, y, z = (a.astype(np.float64) for a in det.rg64)
    s = np.where(z < 0, -1.0, 1.0)
    x, y, z = x * s, y * s, z * s
    r = np.sqrt(2 * (1 - z))
    br = np.abs(y) <= np.abs(x)
    sp = math.sqrt(math.pi) / 2
    with np.errstate(divide="ignore", invalid="ignore"):
        X = np.where(br, np.sign(x) * r * sp, np.sign(y) * r * np.arctan(x / y) / sp)
        Y = np.where(br, np.sign(x) * r * np.arctan(y / x) / sp, np.sign(y) * r * sp)
    scl = wl.npx / SPIO2
    ix, iy = scl * X, scl * Y
    nx = np.floor(ix).astype(int)
    ny = np.floor(iy).astype(int)
    dx, dy = ix - nx, iy - ny
    g = sr.astype(np.float64)
    n = wl.npx
    val = (g[:, ny + n, nx + n] * (1 - dx) * (1 - dy) + g[:, ny + n, nx + n + 1] * dx * (1 - dy)
           + g[:, ny + n + 1, nx + n] * (1 - dx) * dy + g[:, ny + n + 1, nx + n + 1] * dx * dy)
    ref = (det.W64.transpose(2, 0, 1) * val).sum(axis=0)
    np.testing.assert_allclose(p, ref, rtol=1e-12)


def test_single_vs_double(O):
    """The FP32 restatement of the loop agrees with the FP64 re-evaluation to
    TOL_FP64 when both use the same detector weights (the FP32 weight
    set-up adds position noise on sparse histograms; see the GPU notes)."""
    wl = synth.tiny()
    sr, acc = workload_data(wl)
    det = O.Detector(wl.geometry(), acc, 1, wl.nEbins)
    q = wl.quaternions()
    det.W32[:] = det.W64.astype(np.float32)
    l2, mx = rel_errors(det.patterns_f32(sr, q, 1.0), det.patterns_f64(sr, q, 1.0))
    assert l2.max() < TOL_FP64 and mx.max() < TOL_FP64


def test_epilogue(O):
    rng = np.random.default_rng(3)
    pat = rng.uniform(0.5, 2.0, size=(18, 26)).astype(np.float32)
    b = O.epilogue_f32(pat, 4, 1, 1.0)
    assert b.shape == (4, 6)
    ref = pat[:16, :24].reshape(4, 4, 6, 4).sum(axis=(1, 3)) / 16
    np.testing.assert_allclose(b, ref, rtol=1e-6)
    g = O.epilogue_f32(pat, 1, 2, 0.33)
    np.testing.assert_allclose(g, pat.astype(np.float64) ** 0.33, rtol=1e-6)
    n = O.epilogue_f32(pat, 8, 0, 0.33)  # 'not': untouched, full size
    assert np.array_equal(n, pat)


@pytest.mark.parametrize("b", [2, 4, 8])
def test_epilogue_reference_order_is_bit_exact(O, b):
    """The restated block sum of CTEMEBSD.f90:636-640 in single precision:
    one addition at a time, x fastest within the block, then times 1/b^2 --
    checked bit for bit against the same order written independently here."""
    rng = np.random.default_rng(10 + b)
    ny, nx = 5 * b + 3, 7 * b + 5                  # ragged: crop to whole blocks
    pat = rng.uniform(0.1, 3.0, size=(ny, nx)).astype(np.float32)
    got = O.epilogue_f32(pat, b, 1, 1.0)
    bindx = np.float32(1.0) / (np.float32(b) * np.float32(b))
    ref = np.empty((ny // b, nx // b), np.float32)
    for J in range(ny // b):
        for I in range(nx // b):
            s = np.float32(0.0)
            for jj in range(b):
                for ii in range(b):
                    s = np.float32(s + pat[J * b + jj, I * b + ii])
            ref[J, I] = np.float32(s * bindx)
    assert np.array_equal(got, ref)


def test_gradient_oracle_matches_its_finite_differences(O):
    """The analytic binary64 gradient (the adjoint's checker) against central
    binary64 finite differences of the oracle's own forward: loss 1 - the
    normalised dot product with targets, h = 1e-4 rad, 1e-3 px, 1e-2 um, the
    detector re-evaluated for every pattern-centre step.  The bilinear
    interpolation has kinks at cell edges, which the differences average
    over, hence 2e-2 relative to the largest component of each kind."""
    wl = synth.tiny(seed=5, numsx=40, numsy=30, npx=60, nE=5, mc_nsx=80, n_orient=3)
    wl.delta = 120.0
    sr, acc = wl.master(), wl.mc()
    qd = wl.quaternions(3).astype(np.float64)
    geom = dict(wl.geometry(), exact=True)
    det = O.Detector(geom, acc, 1, wl.nEbins)
    qt = np.stack([O.rotate_left(x, np.radians([0.4, -0.3, 0.2])) for x in qd])
    T = det.patterns_f64(sr, qt, 1.0).astype(np.float32)

    def L(gm, qs):
        P = O.Detector(gm, acc, 1, wl.nEbins).patterns_f64(sr, qs, 1.0)
        Td = T.astype(np.float64)
        return np.array([1 - (p * t).sum() / np.sqrt((p * p).sum() * (t * t).sum())
                         for p, t in zip(P, Td)])

    loss, g = O.vjp_f64(geom, acc, 1, wl.nEbins, sr, qd, 1.0, 1, "ndp", T, nthreads=1)
    np.testing.assert_allclose(loss, L(geom, qd), rtol=1e-12, atol=1e-15)
    fd = np.zeros((len(qd), 6))
    for a in range(3):
        w = np.zeros(3)
        w[a] = 1e-4
        qp = np.stack([O.rotate_left(x, w) for x in qd])
        qm = np.stack([O.rotate_left(x, -w) for x in qd])
        fd[:, a] = (L(geom, qp) - L(geom, qm)) / 2e-4
    for a, (k, st) in enumerate((("xpc", 1e-3), ("ypc", 1e-3), ("L", 1e-2))):
        gp, gm = dict(geom), dict(geom)
        gp[k] += st
        gm[k] -= st
        fd[:, 3 + a] = (L(gp, qd) - L(gm, qd)) / (2 * st)
    for cols in ((0, 1, 2), (3,), (4,), (5,)):
        scale = np.abs(fd[:, cols]).max()
        assert scale > 0
        err = np.abs(g[:, cols] - fd[:, cols]).max() / scale
        assert err < 2e-2, (cols, err)
