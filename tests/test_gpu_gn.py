"""Gauss-Newton refinement (ebsd_refine, ebsd_gn_accumulate/apply) on the GPU:
recover orientations (and the shared pattern centre) from perturbed starts
against simulated targets."""
from __future__ import annotations

import numpy as np
import pytest

from ctemsoft_gb300 import capi, synth

pytestmark = pytest.mark.gpu


misorientation_deg = synth.misorientation_deg


def perturb(q, sigma_deg, rng):
    w = np.radians(rng.normal(0, sigma_deg, (len(q), 3)))
    th = np.linalg.norm(w, axis=1, keepdims=True)
    e = np.concatenate([np.cos(th / 2), np.sin(th / 2) * w / np.maximum(th, 1e-30)], axis=1)
    out = np.stack([e[:, 0] * q[:, 0] - (e[:, 1:] * q[:, 1:]).sum(1),
                    e[:, 0] * q[:, 1] + e[:, 1] * q[:, 0] + e[:, 2] * q[:, 3] - e[:, 3] * q[:, 2],
                    e[:, 0] * q[:, 2] - e[:, 1] * q[:, 3] + e[:, 2] * q[:, 0] + e[:, 3] * q[:, 1],
                    e[:, 0] * q[:, 3] + e[:, 1] * q[:, 2] - e[:, 2] * q[:, 1] + e[:, 3] * q[:, 0]],
                   axis=1)
    return out.astype(np.float32)


def _problem(torch, binning=1, n=64, pc_shift=(0.0, 0.0, 0.0), size=(96, 80)):
    wl = synth.tiny(seed=4, numsx=size[0], numsy=size[1], npx=120, nE=5, mc_nsx=150,
                    n_orient=n)
    wl.delta = 100.0
    wl.mc_total = 4e6
    sr, acc = wl.master(), wl.mc()
    h = capi.Handle(0)
    h.set_master(sr)
    true_geom = wl.geometry()
    num_el = h.set_detector(true_geom, acc, 1, 5)
    mode = "lin" if binning > 1 else "not"
    epi = capi.epilogue(capi.prefactor(15.0, 100.0, num_el), binning=binning, scalingmode=mode)
    qt = wl.quaternions()
    targets = torch.from_numpy(h.forward(qt, epi)).cuda()
    start_geom = dict(true_geom)
    start_geom["xpc"] += pc_shift[0]
    start_geom["ypc"] += pc_shift[1]
    start_geom["L"] += pc_shift[2]
    if any(pc_shift):
        h.set_detector(start_geom, acc, 1, 5)
    return wl, h, epi, qt, targets, true_geom


@pytest.mark.parametrize("binning", [1, 2, 4, 8])
def test_refine_orientations(built, binning):
    torch = pytest.importorskip("torch")
    wl, h, epi, qt, targets, _ = _problem(torch, binning)
    rng = np.random.default_rng(0)
    q0 = perturb(qt, 1.0, rng)
    assert misorientation_deg(q0, qt).mean() > 0.5
    dq = torch.from_numpy(q0).cuda()
    loss = torch.zeros(len(qt), device="cuda")
    it, _ = h.refine(dq, epi, targets, max_iterations=20, damping=1e-4, tol_rad=1e-7,
                     loss=loss)
    mis = misorientation_deg(dq.cpu().numpy(), qt)
    print("binning", binning, "iterations", it, "max misorientation (deg)", mis.max())
    assert mis.max() < 0.01
    assert loss.max().item() < 1e-6


@pytest.mark.parametrize("binning", [1, 2, 4])
def test_refine_on_a_ragged_detector(built, binning):
    """99 x 75 pixels: partial tiles, and binning blocks cropped to the floor."""
    torch = pytest.importorskip("torch")
    wl, h, epi, qt, targets, _ = _problem(torch, binning, n=32, size=(99, 75))
    rng = np.random.default_rng(2)
    dq = torch.from_numpy(perturb(qt, 1.0, rng)).cuda()
    it, _ = h.refine(dq, epi, targets, max_iterations=20, damping=1e-4, tol_rad=1e-7)
    mis = misorientation_deg(dq.cpu().numpy(), qt)
    print("binning", binning, "iterations", it, "max misorientation (deg)", mis.max())
    assert mis.max() < 0.01


def test_refine_orientations_and_centre(built):
    torch = pytest.importorskip("torch")
    # the normalised-dot-product loss is nearly flat once the centre is off
    # by a few pixels on this sharp synthetic master; start inside the basin
    wl, h, epi, qt, targets, true_geom = _problem(torch, 1, pc_shift=(0.5, -0.4, 10.0))
    rng = np.random.default_rng(1)
    dq = torch.from_numpy(perturb(qt, 0.5, rng)).cuda()
    it, geom = h.refine(dq, epi, targets, max_iterations=30, refine_pc=True, damping=1e-4,
                        tol_rad=1e-7, tol_pc=1e-5)
    mis = misorientation_deg(dq.cpu().numpy(), qt)
    print("iterations", it, "centre", geom, "max misorientation", mis.max())
    assert abs(geom["xpc"] - true_geom["xpc"]) < 0.02
    assert abs(geom["ypc"] - true_geom["ypc"]) < 0.02
    assert abs(geom["L"] - true_geom["L"]) < 0.5
    assert mis.max() < 0.01


@pytest.mark.parametrize("binning", [2, 4])
def test_accumulation_is_the_same_at_every_tile_shape(built, binning):
    """The Gauss-Newton accumulation for 2x2 / 4x4-binned records at each tile
    height (1, 2, 4 and 8 pixel rows per thread) and orientations per CTA:
    the pattern-centre system and the losses agree with the default shape's
    to rounding, on a detector with partial tiles."""
    torch = pytest.importorskip("torch")
    wl, h, epi, qt, targets, _ = _problem(torch, binning, n=19, size=(100, 76))
    rng = np.random.default_rng(3)
    q0 = torch.from_numpy(perturb(qt, 0.5, rng)).cuda()
    ref = None
    for tile_y, opc in [(16, 32), (4, 1), (8, 7), (32, 5)]:
        h.set_option("vjp_tile_y", tile_y)
        h.set_option("gn_orient_per_cta", opc)
        loss = torch.zeros(len(qt), device="cuda")
        sysc = h.gn_accumulate(q0, epi, targets, 1e-3, pc_system=True, loss=loss)
        cur = (sysc, loss.cpu().numpy().astype(np.float64))
        if ref is None:
            ref = cur
            continue
        scale = np.abs(ref[0]).max()
        assert np.abs(cur[0] - ref[0]).max() <= 1e-4 * scale, (tile_y, opc, cur[0], ref[0])
        np.testing.assert_allclose(cur[1], ref[1], rtol=1e-4, atol=1e-9)


def test_two_phase_api_matches_refine(built):
    """ebsd_gn_accumulate + host solve + ebsd_gn_apply (the multi-GPU form)
    takes the same step as one iteration of ebsd_refine."""
    torch = pytest.importorskip("torch")
    from ctemsoft_gb300 import sharding  # noqa: F401  (same Schur algebra as the host path)
    wl, h, epi, qt, targets, _ = _problem(torch, 1)
    rng = np.random.default_rng(2)
    q0 = perturb(qt, 0.5, rng)
    a = torch.from_numpy(q0).cuda()
    b = a.clone()
    sysc = h.gn_accumulate(a, epi, targets, 1e-3, pc_system=True)
    S, r = sysc[:9].reshape(3, 3), sysc[9:]
    A = S.copy()
    A[np.diag_indices(3)] *= 1 + 1e-3
    dpc = np.linalg.solve(A, r)
    h.gn_apply(a, 1e-3, dpc)
    h2 = capi.Handle(0)
    h2.share_master(h)
    h2.set_detector(wl.geometry(), wl.mc(), 1, 5)
    h2.refine(b, epi, targets, max_iterations=1, refine_pc=True, damping=1e-3)
    torch.cuda.synchronize()
    assert torch.allclose(a, b, atol=1e-7)


def test_sharded_refinement_matches_one_handle(built):
    """ebsd_refine_sharded: the orientations split over two and three handles
    (here all on the one GPU; on a node, one per device), their
    pattern-centre systems summed in this process each iteration, reach the
    same orientations and centre as ebsd_refine on one handle (the only
    difference is the order in which the 12-number system is summed)."""
    torch = pytest.importorskip("torch")
    wl, h, epi, qt, targets, true_geom = _problem(torch, 1, n=60, pc_shift=(0.5, -0.4, 10.0))
    rng = np.random.default_rng(5)
    q0 = perturb(qt, 0.5, rng)
    start = dict(h.geometry)
    one = torch.from_numpy(q0).cuda()
    it1, g1 = h.refine(one, epi, targets, max_iterations=8, refine_pc=True, damping=1e-4,
                       tol_rad=0.0, tol_pc=0.0)
    for parts in (2, 3):
        hs = []
        for k in range(parts):
            hk = capi.Handle(0)
            hk.share_master(h)
            hk.set_detector(start, wl.mc(), 1, 5)
            hs.append(hk)
        cuts = [len(qt) * k // parts for k in range(parts + 1)]
        qs = [torch.from_numpy(q0[a:b].copy()).cuda() for a, b in zip(cuts, cuts[1:])]
        ts = [targets[a:b].contiguous() for a, b in zip(cuts, cuts[1:])]
        losses = [torch.zeros(b - a, device="cuda") for a, b in zip(cuts, cuts[1:])]
        it, g = capi.refine_sharded(hs, qs, epi, ts, max_iterations=8, refine_pc=True,
                                    damping=1e-4, tol_rad=0.0, tol_pc=0.0, losses=losses)
        torch.cuda.synchronize()
        assert it == it1
        for k in ("xpc", "ypc", "L"):
            assert abs(g[k] - g1[k]) < 1e-3, (parts, k, g[k], g1[k])
        qs_all = torch.cat(qs).cpu().numpy()
        mis = misorientation_deg(qs_all, one.cpu().numpy())
        print(parts, "shards: centre", g, "max misorientation to one handle (deg)", mis.max())
        assert mis.max() < 1e-3
        assert misorientation_deg(qs_all, qt).max() < 0.01
        assert all(torch.isfinite(x).all() for x in losses)
        for hk in hs:
            assert hk.geometry == g
            hk.close()


def test_sharded_refinement_rejects_mixed_geometries(built):
    torch = pytest.importorskip("torch")
    wl, h, epi, qt, targets, true_geom = _problem(torch, 1, n=8)
    h2 = capi.Handle(0)
    h2.share_master(h)
    h2.set_detector(dict(true_geom, xpc=true_geom["xpc"] + 1.0), wl.mc(), 1, 5)
    q = torch.from_numpy(qt).cuda()
    with pytest.raises(capi.EBSDError) as e:
        capi.refine_sharded([h, h2], [q[:4], q[4:]], epi, [targets[:4], targets[4:]])
    assert e.value.code == capi.EBSD_EINVAL and "geometry" in str(e.value)


def test_sharded_refinement_with_an_empty_shard(built):
    """A shard with no orientations takes no part in the accumulation but
    still follows the shared pattern centre."""
    torch = pytest.importorskip("torch")
    wl, h, epi, qt, targets, true_geom = _problem(torch, 1, n=16, pc_shift=(0.3, -0.2, 5.0))
    start = dict(h.geometry)
    h2 = capi.Handle(0)
    h2.share_master(h)
    h2.set_detector(start, wl.mc(), 1, 5)
    rng = np.random.default_rng(9)
    q = torch.from_numpy(perturb(qt, 0.3, rng)).cuda()
    empty = q[:0]
    it, g = capi.refine_sharded([h, h2], [q, empty], epi, [targets, targets[:0]],
                                max_iterations=6, refine_pc=True, damping=1e-4)
    assert h2.geometry == g and h.geometry == g
    assert abs(g["xpc"] - true_geom["xpc"]) < abs(start["xpc"] - true_geom["xpc"])
