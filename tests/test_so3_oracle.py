"""The oracle's restatement of the cubochoric fundamental-zone sampler
(so3.f90, Lambert.f90 cube/ball maps, rotations.f90 ho2ro/ro2qu), checked by
round trips and analytic properties: the reference has no tests or
fixtures for this path."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

from oracle import oracle as O

# proper rotation group order of each of the 32 point groups (so3.f90:59-74)
GROUP_ORDER = {1: 1, 2: 1, 3: 2, 4: 2, 5: 2, 6: 4, 7: 4, 8: 4, 9: 4, 10: 4, 11: 4, 12: 8, 13: 8,
               14: 8, 15: 8, 16: 3, 17: 3, 18: 6, 19: 6, 20: 6, 21: 6, 22: 6, 23: 6, 24: 12,
               25: 12, 26: 12, 27: 12, 28: 12, 29: 12, 30: 24, 31: 12, 32: 24}


def test_constants():
    semi, sc, R1, prek, pref, rvmax2, pi8, srt = O.so3_constants()
    assert semi == pytest.approx(0.5 * np.pi ** (2 / 3), rel=1e-15)
    assert R1 == pytest.approx((0.75 * np.pi) ** (1 / 3), rel=1e-15)
    assert rvmax2 == pytest.approx(np.tan(np.radians(179.999) / 2) ** 2, rel=1e-12)
    assert pi8 == pytest.approx(np.tan(np.pi / 8), rel=1e-15)
    assert srt == pytest.approx(np.sqrt(3) / 2, rel=1e-15)


def test_cube_ball_round_trip():
    semi = O.so3_constants()[0]
    rng = np.random.default_rng(0)
    c = rng.uniform(-semi, semi, (3000, 3))
    c[:6] = [[0, 0, 0], [semi, semi, semi], [0.3, 0.3, 0.3], [-0.2, 0.5, 0.5],
             [0.5, -0.5, 0.1], [semi, -0.1, 0.2]]
    h = O.cu2ho(c)
    assert np.linalg.norm(h, axis=1).max() <= O.so3_constants()[2] * (1 + 1e-12)
    assert np.abs(O.ho2cu(h) - c).max() < 1e-10
    assert np.all(O.cu2ho([[semi * 1.001, 0, 0]]) == 0)  # outside the cube (ierr=1)
    # on a coordinate axis the forward map takes its pole branch; the
    # inverse divides 0/0 there (Lambert.f90:1200-1215), as the reference
    h_axis = O.cu2ho([[0, 0, 0.7]])
    assert h_axis[0, 0] == 0 and h_axis[0, 1] == 0 and h_axis[0, 2] > 0
    assert np.isnan(O.ho2cu(h_axis)).any()


def test_uniform_cube_gives_haar_angles():
    """The cube -> ball map is volume preserving and the ball is the
    homochoric image of SO(3), so uniform cube samples give rotation angles
    with the Haar CDF (w - sin w)/pi."""
    semi = O.so3_constants()[0]
    rng = np.random.default_rng(1)
    r = O.cu2ro(rng.uniform(-semi, semi, (20000, 3)))
    w = np.sort(2 * np.arctan(np.linalg.norm(r, axis=1)))
    F = (w - np.sin(w)) / np.pi
    ks = np.abs(F - (np.arange(1, len(w) + 1) - 0.5) / len(w)).max()
    assert ks < 0.015, ks


def test_ho2ro_follows_the_homochoric_angle_relation():
    rng = np.random.default_rng(2)
    h = rng.normal(size=(500, 3))
    h *= (rng.uniform(0.01, 1.3, 500) / np.linalg.norm(h, axis=1))[:, None]
    r = O.ho2ro(h)
    w = 2 * np.arctan(np.linalg.norm(r, axis=1))
    hh = (0.75 * (w - np.sin(w))) ** (1 / 3)
    assert np.abs(hh - np.linalg.norm(h, axis=1)).max() < 3e-6  # the reference's fit
    cosang = (r * h).sum(1) / (np.linalg.norm(r, axis=1) * np.linalg.norm(h, axis=1))
    assert np.all(cosang > 1 - 1e-12)  # same axis


def test_ro2qu_convention():
    """ro2qu goes through ax2om/om2qu, whose matrix convention gives the
    vector part -n sin(w/2)."""
    rng = np.random.default_rng(3)
    n = rng.normal(size=(200, 3))
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    w = rng.uniform(0.01, 3.1, 200)
    q = O.ro2qu(n * np.tan(w / 2)[:, None])
    assert np.abs(np.linalg.norm(q, axis=1) - 1).max() < 1e-15
    assert np.abs(q[:, 0] - np.cos(w / 2)).max() < 1e-12
    assert np.abs(q[:, 1:] + n * np.sin(w / 2)[:, None]).max() < 1e-12
    assert np.all(O.ro2qu([[0.0, 0.0, 0.0]]) == [[1, 0, 0, 0]])


def test_grid_axis_accumulates_like_the_reference():
    """x = -s, x = x + delta while x < s: the accumulated rounding keeps the
    last coordinate just below s, so 2N+1 values (the +s face included)."""
    for n in (1, 10, 25, 100):
        xs = O.rfz_axis(n)
        semi = O.so3_constants()[0]
        x, ref = -semi, []
        while x < semi:
            ref.append(x)
            x = x + semi / n
        assert np.array_equal(xs, ref)
        assert len(xs) in (2 * n, 2 * n + 1)


@pytest.mark.parametrize("pg", [1, 2, 3, 6, 9, 12, 16, 18, 21, 24, 28, 30, 32])
def test_fz_counts_match_group_order(pg):
    """M^3 grid points / members = the rotation group order, less the
    180-degree shell on the cube faces (about 3/M of the grid) that the zone
    tests reject."""
    rods = O.sample_rfz(16, pg)
    m = len(O.rfz_axis(16))
    ratio = m ** 3 / len(rods) / GROUP_ORDER[pg]
    assert 1.0 <= ratio <= 1.0 + 4.0 / m, (pg, ratio)


@pytest.mark.parametrize("pg", [3, 12, 18, 24, 28, 32])
def test_members_pass_the_fz_test(pg):
    rods = O.sample_rfz(12, pg)
    assert all(O.fz_code(r, pg) == 1 for r in rods[::7])


def _cubic_rotations():
    """The 24 proper rotations of the cube as unit quaternions."""
    qs = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            M = np.zeros((3, 3))
            for i, j in enumerate(perm):
                M[i, j] = signs[i]
            if np.linalg.det(M) < 0:
                continue
            w = np.sqrt(max(0.0, 1 + np.trace(M))) / 2
            if w > 1e-8:
                v = np.array([M[2, 1] - M[1, 2], M[0, 2] - M[2, 0], M[1, 0] - M[0, 1]]) / (4 * w)
            else:
                i = int(np.argmax(np.diag(M)))
                v = np.zeros(3)
                v[i] = np.sqrt((1 + M[i, i]) / 2)
                for k in range(3):
                    if k != i:
                        v[k] = M[i, k] / (2 * v[i])
            qs.append(np.concatenate([[w], v]))
    return np.array(qs)


def _qmul(a, b):
    return np.array([a[0] * b[0] - a[1:] @ b[1:],
                     *(a[0] * b[1:] + b[0] * a[1:] + np.cross(a[1:], b[1:]))])


def test_cubic_fz_is_a_fundamental_domain():
    """For m-3m, of the 24 symmetry images of a member exactly one lies in
    the zone (the member itself), away from the zone's boundary."""
    G = _cubic_rotations()
    assert len(G) == 24
    rods = O.sample_rfz(8, 32)
    rng = np.random.default_rng(4)
    pick = rods[rng.choice(len(rods), 60, replace=False)]
    for r in pick:
        q = O.ro2qu(r)[0]
        inside = 0
        for g in G:
            p = _qmul(q, g)
            if abs(p[0]) < 1e-12:
                continue
            rr = p[1:] / p[0]
            inside += O.fz_code(rr, 32) == 1
        assert inside == 1


def test_stale_flag_of_the_triclinic_zone():
    """FZ type 0 never resets insideFZ: after the first member every grid
    point is kept, including rotations of 179.999 degrees and more."""
    m = len(O.rfz_axis(6))
    rods = O.sample_rfz(6, 1)
    first = None
    xs = O.rfz_axis(6)
    for i, c in enumerate(itertools.product(xs, xs, xs)):
        if O.fz_code(O.cu2ro([c])[0], 1) == 1:
            first = i
            break
    assert len(rods) == m ** 3 - first
