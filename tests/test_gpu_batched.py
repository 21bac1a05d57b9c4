"""Batched persistent pattern loop (ebsd_forward_batched) and the
launch-shape autotuner, on the GPU."""
from __future__ import annotations

import numpy as np
import pytest

from ctemsoft_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _mixed_jobs(torch, seed=3):
    """Jobs of different detector size, binning, epilogue, orientation count
    and phase; detectors of one phase share that phase's master."""
    ni = synth.tiny(seed=1, numsx=24, numsy=18, npx=40, nE=5, phase="Ni")
    ti = synth.tiny(seed=2, numsx=24, numsy=18, npx=40, nE=5, phase="Ti")
    masters = {}
    for ph, wl in (("Ni", ni), ("Ti", ti)):
        h = capi.Handle(0)
        h.set_master(wl.master())
        masters[ph] = (h, wl.mc())
    rng = np.random.default_rng(seed)
    shapes = [(80, 60), (37, 29), (160, 120), (64, 48), (320, 240), (101, 77)]
    jobs = []
    for j in range(10):
        nx, ny = shapes[j % len(shapes)]
        ph = "Ni" if j % 3 else "Ti"
        mh, acc = masters[ph]
        h = capi.Handle(0)
        h.share_master(mh)
        geom = dict(L=15000.0, thetac=10.0, delta=12800.0 / nx, numsx=nx, numsy=ny,
                    xpc=float(rng.normal(0, 2)), ypc=float(rng.normal(0, 2)), sig=70.0)
        num_el = h.set_detector(geom, acc, 1, 5)
        b = [1, 2, 4, 8][j % 4]
        mode = ["not", "lin", "gam"][j % 3]
        n = int(rng.integers(1, 120))
        epi = capi.epilogue(capi.prefactor(15.0, 100.0, num_el), binning=b, scalingmode=mode,
                            gammavalue=0.33)
        ox, oy = h.output_dims(epi)
        q = torch.from_numpy(synth.shoemake_quaternions(n, 100 + j)).cuda()
        out = torch.full((n, oy, ox), -1.0, device="cuda")
        jobs.append((h, q, epi, out))
    return masters, jobs


def test_batched_matches_per_job_launches(built):
    torch = pytest.importorskip("torch")
    masters, jobs = _mixed_jobs(torch)
    runner = jobs[0][0]
    runner.forward_batched(jobs)
    torch.cuda.synchronize()
    for i, (h, q, epi, out) in enumerate(jobs):
        ref = torch.empty_like(out)
        h.forward(q, epi, out=ref)
        torch.cuda.synchronize()
        assert torch.equal(out, ref), f"job {i}"


def test_batched_noise_jobs_match_per_job_launches(built):
    """Jobs with Poisson noise run in their own launch groups; the noise is
    keyed by (seed, pattern, pixel), so batched and per-job outputs agree
    bit for bit."""
    torch = pytest.importorskip("torch")
    masters, jobs = _mixed_jobs(torch, seed=5)
    noisy = []
    for i, (h, q, epi, out) in enumerate(jobs):
        if i % 2 == 0:
            epi = capi.epilogue(epi.prefactor * 50.0, binning=epi.binning,
                                scalingmode=epi.scalingmode, gammavalue=epi.gammavalue,
                                poisson=True, seed=40 + i)
        noisy.append((h, q, epi, out))
    noisy[0][0].forward_batched(noisy, graph=True)
    torch.cuda.synchronize()
    for i, (h, q, epi, out) in enumerate(noisy):
        ref = torch.empty_like(out)
        h.forward(q, epi, out=ref)
        torch.cuda.synchronize()
        assert torch.equal(out, ref), f"job {i}"
        if i % 2 == 0 and epi.scalingmode == capi.SCALING["not"]:
            v = out.cpu().numpy()
            assert np.array_equal(v, np.round(v))  # counts


def test_batched_graph_replays_new_inputs(built):
    torch = pytest.importorskip("torch")
    masters, jobs = _mixed_jobs(torch)
    runner = capi.Handle(0)
    runner.forward_batched(jobs, graph=True)
    for rep in range(2):
        # new orientations in the same buffers: the graph must pick them up
        for k, (h, q, epi, out) in enumerate(jobs):
            q.copy_(torch.from_numpy(synth.shoemake_quaternions(q.shape[0], 500 + 7 * rep + k)))
            out.fill_(-1.0)
        torch.cuda.synchronize()
        runner.forward_batched(jobs, graph=True)
        torch.cuda.synchronize()
        for i, (h, q, epi, out) in enumerate(jobs):
            ref = torch.empty_like(out)
            h.forward(q, epi, out=ref)
            torch.cuda.synchronize()
            assert torch.equal(out, ref), f"replay {rep} job {i}"


def test_batched_rejects_host_buffers_and_skips_empty_jobs(built):
    torch = pytest.importorskip("torch")
    masters, jobs = _mixed_jobs(torch)
    h, q, epi, out = jobs[0]
    empty = (h, q[:0], epi, out[:0])
    h.forward_batched([empty, jobs[1]])
    torch.cuda.synchronize()
    with pytest.raises(capi.EBSDError) as e:
        h.forward_batched([(h, q.cpu().numpy(), epi, out)])
    assert e.value.code == capi.EBSD_EINVAL


def test_autotune_and_cache(built, tmp_path):
    wl = synth.tiny(numsx=160, numsy=120, npx=60, nE=5)
    h = capi.Handle(0)
    h.set_master(wl.master())
    h.set_detector(wl.geometry(), wl.mc(), 1, 5)
    epi = capi.epilogue(1.0, binning=4, scalingmode="lin")
    cache = tmp_path / "tune.txt"
    ty, oc, us = h.autotune(epi, 32, cache)
    assert ty in (4, 8, 16) and ty % 4 == 0 and oc in (1, 2, 4, 8) and us > 0
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and lines[0].endswith(f"|{ty}|{oc}|{us:.4f}")
    # a second tuner call reads the cache instead of timing
    h2 = capi.Handle(0)
    h2.share_master(h)
    h2.set_detector(wl.geometry(), wl.mc(), 1, 5)
    assert h2.autotune(epi, 32, cache)[:2] == (ty, oc)
    assert len(cache.read_text().splitlines()) == 1
    # the tuned shape computes the same patterns as the default one
    q = wl.quaternions(7)
    h3 = capi.Handle(0)
    h3.share_master(h)
    h3.set_detector(wl.geometry(), wl.mc(), 1, 5)
    assert np.array_equal(h2.forward(q, epi), h3.forward(q, epi))


def test_batched_large_jobs_run_as_own_launches(built):
    """Jobs that fill the GPU by themselves run at their handle's launch
    shape inside the batch's graph, beside the queued small jobs; records
    equal per-job launches, also when the graph is replayed with new
    orientations and rebuilt for a new output buffer."""
    torch = pytest.importorskip("torch")
    masters, jobs = _mixed_jobs(torch, seed=7)
    mh, acc = masters["Ni"]
    for nx, ny, n, b in ((640, 480, 400, 1), (320, 240, 3000, 2)):
        h = capi.Handle(0)
        h.share_master(mh)
        geom = dict(L=15000.0, thetac=10.0, delta=12800.0 / nx, numsx=nx, numsy=ny, xpc=0.5,
                    ypc=-0.5, sig=70.0)
        num_el = h.set_detector(geom, acc, 1, 5)
        epi = capi.epilogue(capi.prefactor(15.0, 100.0, num_el), binning=b, scalingmode="gam",
                            gammavalue=0.33)
        ox, oy = h.output_dims(epi)
        q = torch.from_numpy(synth.shoemake_quaternions(n, 900 + n)).cuda()
        jobs.insert(3, (h, q, epi, torch.full((n, oy, ox), -1.0, device="cuda")))
    runner = capi.Handle(0)

    def check(tag):
        torch.cuda.synchronize()
        for i, (h, q, epi, out) in enumerate(jobs):
            ref = torch.empty_like(out)
            h.forward(q, epi, out=ref)
            torch.cuda.synchronize()
            assert torch.equal(out, ref), f"{tag} job {i}"

    runner.forward_batched(jobs, graph=True)
    check("first")
    for h, q, epi, out in jobs:
        q.copy_(torch.from_numpy(synth.shoemake_quaternions(q.shape[0], 77 + q.shape[0])))
        out.fill_(-1.0)
    runner.forward_batched(jobs, graph=True)
    check("replay")
    h, q, epi, out = jobs[3]
    jobs[3] = (h, q, epi, torch.full_like(out, -1.0))
    runner.forward_batched(jobs, graph=True)
    check("new buffer")
    # every job through the queue kernel: the same records
    for h, q, epi, out in jobs:
        out.fill_(-1.0)
    capi.Handle(0).forward_batched(jobs, graph=True, queue_all=True)
    check("queue only")


def test_batched_more_jobs_than_one_launch_carries(built):
    """A launch of the queue kernel carries at most 128 jobs in its
    parameters: 300 small jobs of one launch group run as three launches,
    with their graph replayed for new orientations; records equal per-job
    launches."""
    torch = pytest.importorskip("torch")
    wl = synth.tiny(seed=9, numsx=40, numsy=24, npx=40, nE=5)
    src = capi.Handle(0)
    src.set_master(wl.master())
    num_el = src.set_detector(wl.geometry(), wl.mc(), 1, 5)
    epi = capi.epilogue(capi.prefactor(15.0, 100.0, num_el), scalingmode="gam", gammavalue=0.33)
    rng = np.random.default_rng(11)
    jobs = []
    for j in range(300):
        n = int(rng.integers(1, 6))
        q = torch.from_numpy(synth.shoemake_quaternions(n, 2000 + j)).cuda()
        jobs.append((src, q, epi, torch.full((n, 24, 40), -1.0, device="cuda")))
    runner = capi.Handle(0)
    for rep in range(2):
        if rep:
            for j, (h, q, e, out) in enumerate(jobs):
                q.copy_(torch.from_numpy(synth.shoemake_quaternions(q.shape[0], 5000 + j)))
                out.fill_(-1.0)
        runner.forward_batched(jobs, graph=True, queue_all=True)
        torch.cuda.synchronize()
        for i, (h, q, e, out) in enumerate(jobs):
            ref = torch.empty_like(out)
            h.forward(q, e, out=ref)
            torch.cuda.synchronize()
            assert torch.equal(out, ref), f"pass {rep} job {i}"


@pytest.mark.parametrize("weights", ["fp64", "reference"])
def test_c3_shaped_jobs_against_the_oracle(built, weights):
    """Jobs shaped like the 64-job batched workload, run by ebsd_forward_batched
    and compared with the oracle itself (not with per-job launches): a
    1244x1024 detector binned 8x8, whose 1244 columns are not whole blocks
    (the record is cropped to 155 x 128, CTEMEBSD.f90:630-651); the hcp Ti
    master at half-width 500 on 640x480 binned 2; a one-orientation job; an
    unbinned 160x120 job.  Once as the default hybrid batch and once with
    every job through the persistent queue kernel.  With binary64 weights
    the records are gated against the FP64 re-evaluation; with the
    reference's single-precision weights against the FP32 restatement."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    from tests.conftest import workload_data
    from tests.parity import TOL_FP64, TOL_PIXEL_REF, TOL_REF, rel_errors
    masters = {}
    for ph in ("Ni", "Ti"):
        wl = synth.c3_phase(ph)
        sr, acc = workload_data(wl)
        mh = capi.Handle(0)
        mh.set_master(sr)
        masters[ph] = (mh, sr, acc)
    specs = [(1244, 1024, 8, "gam", 3, "Ni"), (640, 480, 2, "lin", 4, "Ti"),
             (80, 60, 4, "gam", 1, "Ti"), (160, 120, 1, "not", 2, "Ni")]
    jobs, refs = [], []
    for j, (nx, ny, b, mode, n, ph) in enumerate(specs):
        mh, sr, acc = masters[ph]
        h = capi.Handle(0)
        h.set_option("weights_fp64", int(weights == "fp64"))
        h.share_master(mh)
        geom = dict(L=15000.0, thetac=10.0, delta=12800.0 / nx, numsx=nx, numsy=ny, xpc=0.0,
                    ypc=0.0, sig=70.0)
        num_el = h.set_detector(geom, acc, 1, 11)
        pref = capi.prefactor(15.0, 100.0, num_el)
        epi = capi.epilogue(pref, binning=b, scalingmode=mode, gammavalue=0.33)
        ox, oy = h.output_dims(epi)
        assert (ox, oy) == ((nx // b, ny // b) if mode != "not" else (nx, ny))
        qn = synth.shoemake_quaternions(n, 1000 + j)
        det = O.Detector(geom, acc, 1, 11)
        assert det.num_el == num_el
        m = capi.SCALING[mode]
        if weights == "fp64":
            raw = det.patterns_f64(sr, qn, pref, nthreads=O.max_threads())
            ref = np.stack([O.epilogue_f64(p, b, m, 0.33) for p in raw])
        else:
            raw = det.patterns_f32(sr, qn, pref, nthreads=O.max_threads())
            ref = np.stack([O.epilogue_f32(p, b, m, 0.33) for p in raw])
        assert ref.shape == (n, oy, ox)
        jobs.append((h, torch.from_numpy(qn).cuda(),
                     epi, torch.full((n, oy, ox), -1.0, device="cuda")))
        refs.append(ref)
    for queue_all in (False, True):
        for *_, out in jobs:
            out.fill_(-1.0)
        capi.Handle(0).forward_batched(jobs, graph=True, queue_all=queue_all)
        torch.cuda.synchronize()
        for (h, q, epi, out), ref, sp in zip(jobs, refs, specs):
            l2, mx = rel_errors(out.cpu().numpy(), ref)
            print(weights, "queue_all" if queue_all else "hybrid", sp,
                  "relL2 %.3g pixel %.3g" % (l2.max(), mx.max()))
            if weights == "fp64":
                assert l2.max() <= TOL_FP64 and mx.max() <= TOL_PIXEL_REF, sp
            else:
                assert l2.max() <= TOL_REF and mx.max() <= TOL_REF, sp
