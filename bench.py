#!/usr/bin/env python
"""EBSD pattern synthesis throughput on GB300.

Workload: the production plain-forward case -- a 640x480 detector (20 um
pixels, L = 15000 um, xpc = 1.5, ypc = -3.0 px, tilt 10 deg, gamma 0.33) on a
1001^2 x 11-bin Ni master pattern (10-20 keV), 10 000 uniformly random
orientations (Shoemake, seed 1).  Inputs are seeded synthetic stand-ins in
the reference's formats (the reference ships no data).

A step is one pass of the pattern loop over the 10 000 orientations (one
kernel launch).  `value` is patterns/s with the master, detector weights,
quaternions and the 12.3 GB of output resident in HBM; L2 is flushed between
timed steps.  `e2e` is the same metric through the C ABI with host buffers
(quaternions uploaded from pinned memory, patterns copied back to pinned
memory each step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank computes its own 10 000 orientations
(weak scaling, no collective on the data path); rank 0 prints one JSON line.
`--impl reference` times the CPU restatement of the reference loop on the
host cores (rank 0 only).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "EBSD patterns/s 640x480 (plain forward), 1001^2 x 11-bin master"
UNIT = "patterns/s"


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--orient", type=int, default=10000)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--vjp-steps", type=int, default=3)
    ap.add_argument("--noise-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "c5", "mc", "dict"],
                    help="c2: 640x480 plain forward (default); c3: 64-job batch; "
                         "c4: 480x480 forward + adjoint; c5: Gauss-Newton refinement")
    ap.add_argument("--c3-jobs", type=int, default=64,
                    help="c3: use the first N of the 64 jobs (small profiling cases)")
    ap.add_argument("--c3-max-orient", type=int, default=0,
                    help="c3: cap each job's orientation count (0: no cap)")
    ap.add_argument("--gn-orient", type=int, default=100000)
    ap.add_argument("--mc-electrons", type=int, default=20000000,
                    help="mc: electrons per timed step")
    ap.add_argument("--dict-steps", type=int, default=100,
                    help="dict: cubochoric steps per semi-edge of the m-3m zone")
    ap.add_argument("--fd-iters", type=int, default=3)
    ap.add_argument("--legs", default="c3,c4,c5,program",
                    help="workloads added to the default line as sub-objects (comma list of "
                         "c3, c4, c5, program; empty for none)")
    ap.add_argument("--legs-fd-iters", type=int, default=2,
                    help="c5 leg of the default line: finite-difference baseline iterations")
    return ap.parse_args()


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _ncu_summary(key: str):
    """A figure of the pattern kernel's committed ncu summary (profiles/),
    written there as `key = value`, or None."""
    f = ROOT / "profiles" / "k_forward_640x480.md"
    if not f.exists():
        return None
    m = re.search(re.escape(key) + r"\s*=\s*([0-9.eE+]+)", f.read_text())
    return float(m.group(1)) if m else None


def _cache_peaks(device: int):
    """Read bandwidth of L1 (hits, 128-bit loads), of L2 (a 48 MB resident
    working set, the interleaved master's size, L1 bypassed) and of HBM (a
    2 GiB sweep), measured now on this device (GB/s)."""
    from ctemsoft_gb300 import capi
    return {"l1": capi.measure_bandwidth(device, capi.BW_L1, 16, 5),
            "l2": capi.measure_bandwidth(device, capi.BW_L2, 48 << 20, 5),
            "hbm_read": capi.measure_bandwidth(device, capi.BW_HBM, 2 << 30, 3)}


def _roofline(b_pattern: int, n: int, launch_ms: float, peaks: dict) -> dict:
    """The pattern kernel against the memory level that bounds it.  Its
    algorithmic bytes (4 corners x nE master values + one store per pixel)
    all pass through the L1 data pipe (82 % L1 hits at 640x480: neighbouring
    pixels share master nodes), so the measured L1 read rate is the roof;
    the L2 and HBM figures are the lower levels' share of the same bytes."""
    hbm_copy, hbm_kind = _peaks()
    achieved = b_pattern * n / (launch_ms / 1000.0) / 1e9
    l1, l2 = peaks["l1"], peaks["l2"]
    dram_pp = _ncu_summary("traffic_bytes_per_pattern")
    l2_pp = _ncu_summary("l2_bytes_per_pattern")
    frac = achieved / l1
    return {
        "bound": "l1", "achieved": achieved, "peak": l1, "unit": "GB/s", "frac": frac,
        "peak_kind": "measured in this run: L1-hit 128-bit loads (ebsd_measure_bandwidth)",
        "traffic": (dram_pp * n if dram_pp else None),
        "traffic_source": "ncu capture of one 256-orientation launch at 640x480 "
                          "(dram__bytes_read.sum + dram__bytes_write.sum), scaled by the "
                          "pattern count; profiles/k_forward_640x480.md",
        "algorithmic_bytes_per_pattern": b_pattern,
        "target": {"what": ">= 60 % of the gather roofline", "frac": frac,
                   "met": bool(frac >= 0.6), "level": "l1"},
        "levels": {
            "l1": {"peak": l1, "frac": frac},
            "l2": {"peak": l2, "frac_if_all_bytes_from_l2": achieved / l2,
                   "l2_bytes_per_pattern": l2_pp,
                   "frac_of_l2_peak": (l2_pp * n / (launch_ms / 1000.0) / 1e9 / l2
                                       if l2_pp else None),
                   "l2_bytes_source": "ncu lts__t_bytes of the same capture"},
            "hbm": {"peak_copy": hbm_copy, "peak_copy_kind": hbm_kind,
                    "peak_read_sweep": peaks["hbm_read"],
                    "frac_of_copy_if_all_bytes_from_hbm": achieved / hbm_copy},
        },
        "binding_unit": {"unit": "L1 data pipe (LSU wavefronts)",
                         "frac": _ncu_summary("l1_wavefront_frac"),
                         "source": "profiles/k_forward_640x480.md"},
    }


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            self.fh = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # nvidia-smi takes a moment to start: wait (at most 5 s) for its first
        # sample so that the samples cover the timed region that follows
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            self.fh.flush()
            if Path(self.path).stat().st_size > 0:
                break
            time.sleep(0.02)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _setup_data(rank: int, n: int):
    from ctemsoft_gb300 import synth
    wl = synth.C2
    sr, acc = wl.master(), wl.mc()
    q = synth.shoemake_quaternions(n, wl.seed + 7919 * rank)
    return wl, sr, acc, q


def cpu_baseline(wl, sr, acc, q, seconds: float, per_step: int | None = None, steps: int = 1,
                 warmup: int = 0):
    """Time the oracle's FP32 restatement of the loop on all host threads
    over a bounded sample of the orientations."""
    from oracle import oracle as O
    threads = O.max_threads()
    Emin, Emax = 1, wl.nEbins
    det = O.Detector(wl.geometry(), acc, Emin, Emax)
    pref = O.prefactor(wl.beamcurrent, wl.dwelltime, det.num_el)
    t = time.perf_counter()
    det.patterns_f32(sr, q[:1], pref, nthreads=1)
    t1 = time.perf_counter() - t
    if per_step is None:
        per_step = int(max(threads, min(len(q), round(seconds * threads / max(t1, 1e-6)))))
    per_step = min(per_step, len(q))
    for w in range(warmup):
        det.patterns_f32(sr, q[:threads], pref, nthreads=threads)
    total = 0.0
    done = 0
    for s in range(steps):
        lo = (s * per_step) % max(1, len(q) - per_step + 1)
        t = time.perf_counter()
        det.patterns_f32(sr, q[lo:lo + per_step], pref, nthreads=threads)
        total += time.perf_counter() - t
        done += per_step
    return {"value": done / total, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{per_step} of {len(q)} orientations x {steps} step(s), "
                      f"640x480, FP32 oracle restatement, OpenMP over orientations",
            "single_thread_patterns_per_s": 1.0 / t1}


def run_reference(args):
    rank, world, local = _dist()
    if rank != 0:
        return 0
    wl, sr, acc, q = _setup_data(0, args.orient)
    from oracle import oracle as O
    threads = O.max_threads()
    base = cpu_baseline(wl, sr, acc, q, 0.0, per_step=4 * threads, steps=args.steps,
                        warmup=args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * (4 * threads) / base["value"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": synth_name(), "orientations": args.orient,
                   "detector": "640x480", "master": "1001x1001x11"},
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def synth_name():
    from ctemsoft_gb300 import synth
    return synth.C2.name


def run_ours(args):
    import numpy as np
    import torch

    from ctemsoft_gb300 import capi

    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    wl, sr, acc, q = _setup_data(rank, args.orient)
    N = len(q)

    h = capi.Handle(local)
    h.set_master(sr)
    num_el = h.set_detector(wl.geometry(), acc, 1, wl.nEbins)
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    epi = capi.epilogue(pref, binning=1, scalingmode="gam", gammavalue=wl.gammavalue)
    nx, ny = h.output_dims(epi)
    P = wl.numsx * wl.numsy
    # the launch shape from the project's autotuner (cached per shape), as a
    # caller would run it; tuning happens before and outside the timed steps
    tuned = h.autotune(epi, 1024, Path(tempfile.gettempdir()) / f"ebsd_autotune_{local}.txt")

    # a dedicated stream: its handle is never 0, which the C ABI reads as
    # "the handle's own stream"; the events below are recorded on it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    h.set_stream(stream.cuda_stream)
    dq = torch.from_numpy(q).to(dev)
    dout = torch.empty((N, ny, nx), dtype=torch.float32, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        h.forward(dq, epi, out=dout)
    barrier()
    clocks = Clocks(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()  # evict L2 between timed steps (outside the events)
        ev[k][0].record(stream)
        h.forward(dq, epi, out=dout)
        ev[k][1].record(stream)
    barrier()
    ck = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    tot_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([tot_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        tot_ms = float(t.item())
    value = world * N * args.steps / (tot_ms / 1000.0)
    launch_ms = statistics.mean(step_ms)
    peaks = _cache_peaks(local)

    # fused forward + adjoint: the normalised-dot-product loss and its
    # gradient (3 rotation tangents + pattern centre) for every orientation
    # against target patterns, one pass per pattern
    fwd_vjp = None
    if args.vjp_steps > 0:
        fwd_vjp = _fwd_vjp(h, q, wl, pref, dout, stream, args, world, dev, barrier, value,
                           flush, peaks)

    # the same loop with the reference's Poisson noise (CTEMEBSD.f90:611-615)
    # before the gamma epilogue
    fwd_noise = None
    if args.noise_steps > 0:
        epn = capi.epilogue(pref, binning=1, scalingmode="gam", gammavalue=wl.gammavalue,
                            poisson=True, seed=7)
        h.forward(dq, epn, out=dout)
        barrier()
        evn = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.noise_steps)]
        for k in range(args.noise_steps):
            flush.zero_()
            evn[k][0].record(stream)
            h.forward(dq, epn, out=dout)
            evn[k][1].record(stream)
        barrier()
        nms = sum(a.elapsed_time(b) for a, b in evn) / args.noise_steps
        # the sampler's branches: means ~1 (inversion), ~10 (the reference's
        # beam settings: both), ~100 (PTRS), one step each
        by_mean = {}
        for scale in (0.1, 1.0, 10.0):
            eps = capi.epilogue(pref * scale, binning=1, scalingmode="gam",
                                gammavalue=wl.gammavalue, poisson=True, seed=8)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            flush.zero_()
            a.record(stream)
            h.forward(dq, eps, out=dout)
            b.record(stream)
            torch.cuda.synchronize()
            by_mean[f"prefactor x{scale:g}"] = N / (a.elapsed_time(b) / 1000.0)
        fwd_noise = {"value": world * N / (nms / 1000.0), "unit": UNIT, "ms_per_step": nms,
                     "steps": args.noise_steps, "by_prefactor_scale": by_mean,
                     "what": "forward with Poisson noise (Philox4x32-10, inversion / PTRS) "
                             "before gamma 0.33"}

    # end to end through the C ABI with host buffers
    del dout
    torch.cuda.empty_cache()
    e2e = None
    if args.e2e_steps > 0:
        e2e = _e2e(h, q, epi, N, nx, ny, args, world, dev, barrier)

    # the other workloads, one compact sub-object each (rank 0 of a 1-GPU run)
    legs = {}
    if rank == 0 and world == 1 and args.legs:
        h.close()
        h = None
        del dq
        torch.cuda.empty_cache()
        for name in [x.strip() for x in args.legs.split(",") if x.strip()]:
            try:
                if name == "c3":
                    legs["c3"] = c3_measure(args, 3)
                    legs["c3"]["small_jobs"] = small_jobs_measure(args, 5)
                elif name == "c4":
                    legs["c4"] = c4_measure(args, 5, 3)
                elif name == "program":
                    legs["program"] = program_measure(args)
                elif name == "c5":
                    legs["c5"] = c5_measure(args, args.legs_fd_iters)
                    legs["c5"]["fd_note"] = (f"forward-only finite-difference baseline capped "
                                             f"at {args.legs_fd_iters} iterations")
            except Exception as ex:  # a failed leg is reported, the headline stands
                legs[name] = {"error": f"{type(ex).__name__}: {ex}"}
            torch.cuda.empty_cache()

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline(wl, sr, acc, q, args.cpu_seconds)

    if rank == 0:
        b_pattern = P * (16 * wl.nEbins + 4)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded stand-ins in the reference's file formats)",
            "config": {"workload": wl.name, "detector": f"{wl.numsx}x{wl.numsy}",
                       "master": f"{2 * wl.npx + 1}^2 x {wl.nEbins} bins",
                       "orientations_per_gpu": N, "epilogue": "prefactor, gamma 0.33",
                       "l2": "flushed (512 MB write) between timed steps",
                       "parallelism": f"orientation shards x{world}",
                       "launch_shape": {"tile_y": tuned[0], "orient_per_cta": tuned[1],
                                        "source": "ebsd_autotune"}},
            "roofline": _roofline(b_pattern, N, launch_ms, peaks),
            "e2e": e2e,
            "fwd_vjp": fwd_vjp,
            "fwd_noise": fwd_noise,
            "gpu_launches": args.steps,
            "clocks": ck,
            "cpu_baseline": base,
        }
        line.update(legs)
        print(json.dumps(line))
    if h is not None:
        h.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def _fwd_vjp(h, q, wl, pref, dout, stream, args, world, dev, barrier, fwd_value, flush,
             peaks=None):
    import numpy as np
    import torch

    from ctemsoft_gb300 import capi, synth
    N = len(q)
    epi = capi.epilogue(pref)  # no gamma: the adjoint runs on linear patterns
    # targets: patterns at orientations rotated by ~0.5 degree
    rng = np.random.default_rng(11)
    w = np.radians(rng.normal(0.0, 0.5, (N, 3)))
    th = np.linalg.norm(w, axis=1, keepdims=True)
    e = np.concatenate([np.cos(th / 2), np.sin(th / 2) * w / np.maximum(th, 1e-30)], axis=1)
    qt = np.stack([e[:, 0] * q[:, 0] - (e[:, 1:] * q[:, 1:]).sum(1),
                   e[:, 0] * q[:, 1] + e[:, 1] * q[:, 0] + e[:, 2] * q[:, 3] - e[:, 3] * q[:, 2],
                   e[:, 0] * q[:, 2] - e[:, 1] * q[:, 3] + e[:, 2] * q[:, 0] + e[:, 3] * q[:, 1],
                   e[:, 0] * q[:, 3] + e[:, 1] * q[:, 2] - e[:, 2] * q[:, 1] + e[:, 3] * q[:, 0]],
                  axis=1).astype(np.float32)
    dq = torch.from_numpy(q).to(dev)
    h.forward(torch.from_numpy(qt).to(dev), epi, out=dout)  # targets in place
    loss = torch.zeros(N, device=dev)
    grad = torch.zeros((N, 6), device=dev)
    for _ in range(max(1, args.warmup)):
        h.vjp(dq, epi, dout, "ndp", loss=loss, grad=grad)
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.vjp_steps)]
    for k in range(args.vjp_steps):
        flush.zero_()  # evict L2 between timed steps, as in the forward leg
        ev[k][0].record(stream)
        h.vjp(dq, epi, dout, "ndp", loss=loss, grad=grad)
        ev[k][1].record(stream)
    barrier()
    tot = sum(a.elapsed_time(b) for a, b in ev)
    if world > 1:
        t = torch.tensor([tot], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        tot = float(t.item())
    v = world * N * args.vjp_steps / (tot / 1000.0)
    lh = loss.cpu().numpy()
    # algorithmic bytes: the recomputed 4-corner gather twice over (value and
    # slopes share it, the weight terms read it again per bin) + the target
    # read and the per-pattern outputs: P (2 x 16 nE + 8)
    b_vjp = wl.numsx * wl.numsy * (2 * 16 * wl.nEbins + 8)
    if peaks is None:
        peaks = _cache_peaks(dev.index if dev.index is not None else 0)
    peak = peaks["l1"]
    ach = b_vjp * (v / world) / 1e9
    return {"value": v, "unit": UNIT, "ratio_to_forward": v / fwd_value,
            "ms_per_step": tot / args.vjp_steps, "steps": args.vjp_steps,
            "l2": "flushed (512 MB write) between timed steps",
            "what": "loss 1 - normalised dot product + gradient w.r.t. 3 rotation tangents "
                    "and (xpc, ypc, L), one fused pass per pattern",
            "roofline": {"bound": "l1", "algorithmic_bytes_per_pattern": b_vjp,
                         "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "peak_kind": "measured in this run: L1-hit 128-bit loads"},
            "mean_loss": float(lh.mean()), "finite": bool(np.isfinite(lh).all())}


def _e2e(h, q, epi, N, nx, ny, args, world, dev, barrier):
    """The same metric through the C ABI with host buffers: quaternions
    uploaded from pinned memory and all patterns copied back every step."""
    import numpy as np
    import torch
    hq = torch.empty((N, 4), dtype=torch.float32, pin_memory=True)
    hq.copy_(torch.from_numpy(q))
    hout = torch.empty((N, ny, nx), dtype=torch.float32, pin_memory=True)
    h.set_stream(None)
    h.forward(hq, epi, out=hout)  # warm-up
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        h.forward(hq, epi, out=hout)
        _ = float(hout[N - 1, ny - 1, nx - 1])  # result is on the host
    barrier()
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_val = world * N * args.e2e_steps / e2e_s
    ok = bool(np.isfinite(hout[0].numpy()).all())
    # the bound of this leg: a plain device-to-host copy of 2 GiB into the
    # same pinned buffer (best of 3, CUDA events)
    n_link = min(hout.numel(), 1 << 29)
    src = torch.ones(n_link, dtype=torch.float32, device=dev)
    dst = hout.view(-1)[:n_link]
    stream = torch.cuda.current_stream(dev)
    dst.copy_(src, non_blocking=True)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(3):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        dst.copy_(src, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    link = 4 * n_link / (best / 1000.0) / 1e9
    d2h = N * nx * ny * 4
    return {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(N * 16),
            "d2h_bytes_per_step": int(d2h), "steps": args.e2e_steps, "finite": ok,
            "link": {"d2h_copy_gbs": link, "records_gbs": d2h * e2e_val / N / 1e9,
                     "frac": d2h * e2e_val / N / 1e9 / link,
                     "note": "records reach the host at this fraction of a plain "
                             "cudaMemcpy device-to-host into the same pinned memory"}}


def c4_measure(args, steps: int, vjp_steps: int) -> dict:
    """The adjoint workload: 480x480 detector, 1001^2 x 11-bin master, 4096
    orientations; the fused forward + adjoint (loss and its gradient with
    respect to 3 rotation tangents and the pattern centre) against the plain
    forward of the same patterns, both timed with L2 flushed between steps."""
    import torch

    from ctemsoft_gb300 import capi, synth
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    wl = synth.C4
    sr, acc = wl.master(), wl.mc()
    q = wl.quaternions()
    N = len(q)
    h = capi.Handle(0)
    h.set_master(sr)
    num_el = h.set_detector(wl.geometry(), acc, 1, wl.nEbins)
    pref = capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el)
    epi = capi.epilogue(pref)
    nx, ny = h.output_dims(epi)
    tuned = h.autotune(epi, 1024, Path(tempfile.gettempdir()) / "ebsd_autotune_0.txt")
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    h.set_stream(stream.cuda_stream)
    dq = torch.from_numpy(q).to(dev)
    dout = torch.empty((N, ny, nx), dtype=torch.float32, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        h.forward(dq, epi, out=dout)
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        h.forward(dq, epi, out=dout)
        b.record(stream)
        torch.cuda.synchronize()
        tot += a.elapsed_time(b)
    fwd = N * steps / (tot / 1000.0)
    sub = argparse.Namespace(warmup=args.warmup, vjp_steps=vjp_steps)
    vjp = _fwd_vjp(h, q, wl, pref, dout, stream, sub, 1, dev, torch.cuda.synchronize, fwd,
                   flush)
    torch.cuda.set_stream(torch.cuda.default_stream(dev))
    h.close()
    return {
        "metric": "EBSD fused forward + adjoint patterns/s (480x480, 4096 orientations)",
        "value": vjp["value"], "unit": UNIT, "ms_per_step": vjp["ms_per_step"],
        "steps": vjp_steps, "forward": {"value": fwd, "unit": UNIT, "steps": steps,
                                        "launch_shape": {"tile_y": tuned[0],
                                                         "orient_per_cta": tuned[1]}},
        "ratio_to_forward": vjp["ratio_to_forward"], "what": vjp["what"],
        "roofline": vjp["roofline"], "mean_loss": vjp["mean_loss"], "finite": vjp["finite"],
        "l2": "flushed (512 MB write) between timed steps of both legs",
    }


def run_c4(args):
    clocks = Clocks(0)
    clocks.start()
    res = c4_measure(args, args.steps, args.vjp_steps)
    ck = clocks.stop()
    line = dict(res, n_gpus=1, warmup=args.warmup, higher_is_better=True, dtype="f32",
                data="synthetic", gpu_launches=2 * args.vjp_steps, clocks=ck,
                config={"workload": "adjoint-480x480-npx500", "detector": "480x480",
                        "master": "1001^2 x 11 bins", "orientations": 4096})
    print(json.dumps(line))
    return 0


def c3_measure(args, steps: int) -> dict:
    """The batched uneven workload: 64 jobs (seed 2) of mixed detector size,
    binning, orientation count and phase in one CUDA graph (jobs that fill
    the GPU as their own tuned launches, the rest through one persistent
    queue kernel), against the same jobs launched one by one and with every
    job in the queue.  Set-up: one detector set-up per distinct (detector,
    phase) -- binning does not change the tables -- run concurrently on
    their own handles, then shared by every job on that detector."""
    from concurrent.futures import ThreadPoolExecutor

    import torch

    from ctemsoft_gb300 import capi, synth
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    specs = synth.c3_jobs(2)[:max(1, args.c3_jobs)]
    if args.c3_max_orient > 0:
        specs = [dict(sp, n=min(sp["n"], args.c3_max_orient)) for sp in specs]
    data = {ph: synth.c3_phase(ph) for ph in ("Ni", "Ti")}
    arrays = {ph: (wl.master(), wl.mc()) for ph, wl in data.items()}
    cache = Path(tempfile.gettempdir()) / "ebsd_autotune.txt"
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    masters = {}
    for ph, (sr, acc) in arrays.items():
        h = capi.Handle(0)
        h.set_master(sr)
        masters[ph] = h
    keys = sorted({(sp["numsx"], sp["numsy"], sp["delta"], sp["phase"]) for sp in specs})

    def setup(key):
        nx, ny, delta, ph = key
        h = capi.Handle(0)
        h.share_master(masters[ph])
        geom = dict(L=15000.0, thetac=10.0, delta=delta, numsx=nx, numsy=ny, xpc=0.0, ypc=0.0,
                    sig=70.0)
        h.set_detector(geom, arrays[ph][1], 1, 11)
        return key, h

    with ThreadPoolExecutor(max_workers=len(keys)) as ex:  # ctypes calls release the GIL
        dets = dict(ex.map(setup, keys))
    setup_s = time.perf_counter() - t0
    t1 = time.perf_counter()
    jobs = []
    shapes = {}  # tuned launch shapes (pixels x orientations per CTA) of the jobs
    for sp in specs:
        src = dets[(sp["numsx"], sp["numsy"], sp["delta"], sp["phase"])]
        h = capi.Handle(0)
        h.share_detector(src)
        epi = capi.epilogue(capi.prefactor(15.0, 100.0, src.num_el), binning=sp["binning"],
                            scalingmode="gam", gammavalue=0.33)
        ty, oc, _ = h.autotune(epi, 64, cache)
        shapes[f"32x{ty}x{oc}"] = shapes.get(f"32x{ty}x{oc}", 0) + 1
        ox, oy = h.output_dims(epi)
        q = torch.from_numpy(synth.shoemake_quaternions(sp["n"], sp["seed"])).to(dev)
        out = torch.empty((sp["n"], oy, ox), device=dev)
        jobs.append((h, q, epi, out))
    torch.cuda.synchronize()
    tune_s = time.perf_counter() - t1
    total = sum(sp["n"] for sp in specs)
    runner = capi.Handle(0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    runner.set_stream(stream.cuda_stream)
    for h, *_ in jobs:
        h.set_stream(stream.cuda_stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    # the first batch, end to end after the set-up: graph capture and launch
    t2 = time.perf_counter()
    runner.forward_batched(jobs, graph=True)
    torch.cuda.synchronize()
    first_s = time.perf_counter() - t2

    def timed(fn, n):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(n):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            tot += a.elapsed_time(b)
        return tot / n

    queue_runner = capi.Handle(0)
    queue_runner.set_stream(stream.cuda_stream)
    ms_b = timed(lambda: runner.forward_batched(jobs, graph=True), steps)
    ref = [out.clone() for *_, out in jobs]
    ms_q = timed(lambda: queue_runner.forward_batched(jobs, graph=True, queue_all=True), steps)
    same_q = all(torch.equal(r, out) for r, (*_, out) in zip(ref, jobs))

    def one_by_one():
        for h, q, epi, out in jobs:
            h.forward(q, epi, out=out)

    ms_s = timed(one_by_one, steps)
    same = all(torch.equal(r, out) for r, (*_, out) in zip(ref, jobs))
    torch.cuda.set_stream(torch.cuda.default_stream(dev))
    res = {
        "metric": f"EBSD patterns/s, batched uneven workload ({len(specs)} jobs)",
        "value": total / (ms_b / 1e3), "unit": UNIT, "ms_per_step": ms_b, "steps": steps,
        "patterns": total, "detectors": len(keys),
        "one_by_one": {"value": total / (ms_s / 1e3), "ms_per_step": ms_s,
                       "launches": len(jobs)},
        "persistent_only": {"value": total / (ms_q / 1e3), "ms_per_step": ms_q,
                            "identical": bool(same_q),
                            "what": "every job through the persistent queue kernel"},
        "identical_to_one_by_one": bool(same),
        "setup_s": setup_s, "autotune_s": tune_s, "first_batch_s": first_s,
        "tuned_shapes": shapes,
        "e2e_with_setup": {"value": total / (setup_s + tune_s + first_s), "unit": UNIT,
                           "what": "detector set-up + launch-shape tuning (cached per shape "
                                   "in a file) + the first batch (graph capture and run)"},
        "l2": "flushed (512 MB write) between timed steps",
    }
    for h, *_ in jobs:
        h.close()
    for h in list(dets.values()) + list(masters.values()) + [runner, queue_runner]:
        h.close()
    return res


def small_jobs_measure(args, steps: int, njobs: int = 256) -> dict:
    """Many small jobs -- njobs (seed 5) of 1 to 32 orientations (log-uniform)
    on 80x60 and 160x120 detectors of both phases, binning 1 or 2, gamma
    0.33 -- where one launch per job is bound by launch latency and grid
    tails: the batch (every job in the persistent queue, one CUDA graph)
    against one launch per job, and against one launch per job captured in
    a CUDA graph."""
    import numpy as np
    import torch

    from ctemsoft_gb300 import capi, synth
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    dets = {}
    for ph in ("Ni", "Ti"):
        wl = synth.c3_phase(ph)
        sr, acc = wl.master(), wl.mc()
        mh = capi.Handle(0)
        mh.set_master(sr)
        for nx, ny in ((80, 60), (160, 120)):
            h = capi.Handle(0)
            h.share_master(mh)
            h.set_detector(dict(L=15000.0, thetac=10.0, delta=12800.0 / nx, numsx=nx, numsy=ny,
                                xpc=0.0, ypc=0.0, sig=70.0), acc, 1, 11)
            dets[(ph, nx)] = h
        dets[(ph, "master")] = mh
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    jobs = []
    for j in range(njobs):
        ph = "Ni" if rng.random() < 0.5 else "Ti"
        nx = 80 if rng.random() < 0.5 else 160
        b = int(rng.choice([1, 2]))
        n = int(np.clip(np.round(np.exp(rng.uniform(0.0, np.log(32.0)))), 1, 32))
        src = dets[(ph, nx)]
        h = capi.Handle(0)
        h.share_detector(src)
        h.set_stream(stream.cuda_stream)
        epi = capi.epilogue(capi.prefactor(15.0, 100.0, src.num_el), binning=b,
                            scalingmode="gam", gammavalue=0.33)
        ox, oy = h.output_dims(epi)
        q = torch.from_numpy(synth.shoemake_quaternions(n, 5000 + j)).to(dev)
        jobs.append((h, q, epi, torch.empty((n, oy, ox), device=dev)))
    total = sum(q.shape[0] for _, q, _, _ in jobs)
    runner = capi.Handle(0)
    runner.set_stream(stream.cuda_stream)

    def one_by_one():
        for h, q, epi, out in jobs:
            h.forward(q, epi, out=out)

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps

    ms_b = timed(lambda: runner.forward_batched(jobs, graph=True))
    ref = [out.clone() for *_, out in jobs]
    ms_s = timed(one_by_one)
    same = all(torch.equal(r, out) for r, (*_, out) in zip(ref, jobs))
    # the per-job launches captured once in a CUDA graph and replayed
    try:
        graph = torch.cuda.CUDAGraph()
        one_by_one()
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=stream, capture_error_mode="thread_local"):
            one_by_one()
        ms_g = timed(graph.replay)
        graphed = {"value": total / (ms_g / 1e3), "ms_per_step": ms_g}
    except Exception as ex:
        graphed = {"error": f"{type(ex).__name__}: {ex}"}
    torch.cuda.set_stream(torch.cuda.default_stream(dev))
    res = {"jobs": njobs, "patterns": total, "value": total / (ms_b / 1e3), "unit": UNIT,
           "ms_per_step": ms_b,
           "one_by_one": {"value": total / (ms_s / 1e3), "ms_per_step": ms_s},
           "one_by_one_graph": graphed,
           "identical": bool(same),
           "what": "256 jobs of 1-32 orientations on 80x60/160x120: the persistent queue "
                   "(one graph) against one launch per job, plain and graph-captured"}
    for h, *_ in jobs:
        h.close()
    for h in list(dets.values()) + [runner]:
        h.close()
    return res


def program_measure(args, n: int = 20000, n_file: int = 4000) -> dict:
    """The drop-in program end to end (ebsd_run_namelist, the reference's
    CTEMEBSD with its namelist, angle, MC and master files): the 640x480
    detector on the 1001^2 x 11 Ni master, gamma 0.33, with and without the
    reference's Poisson noise; n orientations with the records written to
    /dev/null (compute, device-to-host, record assembly), n_file written to
    a file in the temporary directory (plus the page cache and file
    system).  Wall time of the call,
    file reading and detector set-up included, as the reference's program
    would be timed from the shell."""
    import shutil

    from ctemsoft_gb300 import capi, formats, synth
    wl = synth.C2
    d = Path(tempfile.mkdtemp(prefix="ebsd_program_"))
    try:
        sr, acc = wl.master(), wl.mc()
        formats.write_mc_file(d / "mc.data", acc, EkeV=wl.EkeV, Ehistmin=wl.Ehistmin,
                              Ebinsize=wl.Ebinsize, sig=wl.sig)
        formats.write_master_file(d / "master.data", sr, wl.energies)
        for k, m in (("angles.txt", n), ("angles_file.txt", n_file)):
            formats.write_angle_file(d / k, quats=synth.shoemake_quaternions(m, 1))
        base = dict(L=wl.L, thetac=wl.thetac, delta=wl.delta, numsx=wl.numsx, numsy=wl.numsy,
                    xpc=wl.xpc, ypc=wl.ypc, anglefile=str(d / "angles.txt"),
                    eulerconvention="tsl", FZfile=str(d / "master.data"),
                    energyfile=str(d / "mc.data"), beamcurrent=wl.beamcurrent,
                    dwelltime=wl.dwelltime, energymin=10.0, energymax=20.0, binning=1,
                    scalingmode="gam", gammavalue=wl.gammavalue)
        res = {"orientations": {"devnull": n, "file": n_file},
               "record_bytes": 4 * wl.numsx * wl.numsy,
               "what": "ebsd_run_namelist wall time: namelist, angle/MC/master file reading, "
                       "detector set-up, all patterns, records written"}
        capi.run_namelist(_nml(d, base, "/dev/null", False), 0)  # warm-up (CUDA context, build)
        for noise in (False, True):
            for dest in ("/dev/null", str(d / "out.data")):
                m = n if dest == "/dev/null" else n_file
                cfg = dict(base, anglefile=str(d / ("angles.txt" if m == n else "angles_file.txt")))
                t0 = time.perf_counter()
                capi.run_namelist(_nml(d, cfg, dest, noise), 0)
                dt = time.perf_counter() - t0
                key = ("noise" if noise else "no_noise") + \
                      ("_devnull" if dest == "/dev/null" else "_file")
                res[key] = {"value": m / dt, "unit": UNIT, "wall_s": dt,
                            "record_gbs": m * 4 * wl.numsx * wl.numsy / dt / 1e9}
                if dest != "/dev/null":
                    (d / "out.data").unlink()
        return res
    finally:
        shutil.rmtree(d, ignore_errors=True)


def _nml(d, base, dest, noise):
    from ctemsoft_gb300 import formats
    path = d / "run.nml"
    formats.write_namelist(path, **dict(base, datafile=dest, poisson=noise, seed=3))
    return path


def run_batched(args):
    res = c3_measure(args, args.steps)
    res["small_jobs"] = small_jobs_measure(args, args.steps)
    line = dict(res, n_gpus=1, warmup=args.warmup, higher_is_better=True, dtype="f32",
                data="synthetic",
                config={"workload": f"batched-{res['patterns']}-patterns-seed2",
                        "launch": "one CUDA graph: jobs that fill the GPU as their own tuned "
                                  "launches, the rest through one persistent queue kernel"})
    print(json.dumps(line))
    return 0


def _perturb(q, sigma_deg, rng):
    import numpy as np
    w = np.radians(rng.normal(0, sigma_deg, (len(q), 3)))
    th = np.linalg.norm(w, axis=1, keepdims=True)
    e = np.concatenate([np.cos(th / 2), np.sin(th / 2) * w / np.maximum(th, 1e-30)], axis=1)
    return np.stack([e[:, 0] * q[:, 0] - (e[:, 1:] * q[:, 1:]).sum(1),
                     e[:, 0] * q[:, 1] + e[:, 1] * q[:, 0] + e[:, 2] * q[:, 3] - e[:, 3] * q[:, 2],
                     e[:, 0] * q[:, 2] - e[:, 1] * q[:, 3] + e[:, 2] * q[:, 0] + e[:, 3] * q[:, 1],
                     e[:, 0] * q[:, 3] + e[:, 1] * q[:, 2] - e[:, 2] * q[:, 1] + e[:, 3] * q[:, 0]],
                    axis=1).astype(np.float32)


def _misorientation_deg(a, b):
    from ctemsoft_gb300 import synth
    return synth.misorientation_deg(a, b)


def _fd_gauss_newton(h, q, epi, targets, geom, acc, iters, damping, chunk=10000):
    """Forward-only refinement on the same GPU: the Jacobian of the
    normalised residual by one-sided finite differences (3 rotated forwards
    and 3 forwards on re-set-up detectors per iteration), then the same
    Gauss-Newton system and shared-centre elimination as the adjoint path."""
    import numpy as np
    import torch

    from ctemsoft_gb300 import sharding
    dev = targets.device
    n = q.shape[0]
    hr, hp = 1e-4, (1e-2, 1e-2, 1.0)
    g = dict(geom)
    tn = targets / targets.norm(dim=(1, 2), keepdim=True)

    def normed(qq):
        O = torch.empty_like(targets)
        h.forward(qq, epi, out=O)
        return O / O.norm(dim=(1, 2), keepdim=True)

    for _ in range(iters):
        On = normed(q)
        cols = []
        qn = q.cpu().numpy()
        for a in range(3):
            qa = torch.from_numpy(_perturb_exact(qn, a, hr)).to(dev)
            cols.append((normed(qa) - On) / hr)
        for a, k in enumerate(("xpc", "ypc", "L")):
            gg = dict(g)
            gg[k] += hp[a]
            h.set_detector(gg, acc, 1, h._nbins)
            cols.append((normed(q) - On) / hp[a])
        h.set_detector(g, acc, 1, h._nbins)
        H = np.zeros((n, 6, 6))
        gv = np.zeros((n, 6))
        for o0 in range(0, n, chunk):
            sl = slice(o0, min(n, o0 + chunk))
            J = torch.stack([c[sl].flatten(1) for c in cols], dim=2).double()
            r = (On[sl] - tn[sl]).flatten(1).double()
            H[sl] = torch.einsum("mpi,mpj->mij", J, J).cpu().numpy()
            gv[sl] = torch.einsum("mpi,mp->mi", J, r).cpu().numpy()
        del cols, On
        A, B, Cm = H[:, :3, :3].copy(), H[:, :3, 3:].copy(), H[:, 3:, 3:].copy()
        A[:, np.arange(3), np.arange(3)] *= 1 + damping
        S, rr = sharding.schur_pc_system(A, B, Cm, -gv[:, :3], -gv[:, 3:])
        S[np.diag_indices(3)] *= 1 + damping
        dpc = np.linalg.solve(S, rr)
        drot = sharding.schur_back_substitute(A, B, -gv[:, :3], dpc)
        q = torch.from_numpy(_apply_steps(qn, drot)).to(dev)
        for a, k in enumerate(("xpc", "ypc", "L")):
            g[k] += float(dpc[a])
        h.set_detector(g, acc, 1, h._nbins)
    return q, g


def _perturb_exact(q, axis, hr):
    import numpy as np
    w = np.zeros((len(q), 3))
    w[:, axis] = hr
    return _apply_steps(q, w)


def _apply_steps(q, w):
    import numpy as np
    th = np.linalg.norm(w, axis=1, keepdims=True)
    e = np.concatenate([np.cos(th / 2), np.sin(th / 2) * w / np.maximum(th, 1e-30)], axis=1)
    q = q.astype(np.float64)
    out = np.stack([e[:, 0] * q[:, 0] - (e[:, 1:] * q[:, 1:]).sum(1),
                    e[:, 0] * q[:, 1] + e[:, 1] * q[:, 0] + e[:, 2] * q[:, 3] - e[:, 3] * q[:, 2],
                    e[:, 0] * q[:, 2] - e[:, 1] * q[:, 3] + e[:, 2] * q[:, 0] + e[:, 3] * q[:, 1],
                    e[:, 0] * q[:, 3] + e[:, 1] * q[:, 2] - e[:, 2] * q[:, 1] + e[:, 3] * q[:, 0]],
                   axis=1)
    return (out / np.linalg.norm(out, axis=1, keepdims=True)).astype(np.float32)


def c5_measure(args, fd_iters: int) -> dict:
    """Gauss-Newton refinement at scale: 100 000 orientations (seed 4) on a
    120x120 detector (480x480 binned 4x4), 15 bins 6-20 keV, targets with
    Poisson noise at 1000 mean counts per detector pixel before binning,
    starts perturbed by N(0, 1 deg) per rotation axis and N(0, 3 px) in the
    pattern centre; up to 20 iterations."""
    import numpy as np
    import torch

    from ctemsoft_gb300 import capi, synth
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    wl = synth.C5
    n = args.gn_orient
    sr, acc = wl.master(), wl.mc()
    rng = np.random.default_rng(4)
    h = capi.Handle(0)
    h.set_master(sr)
    true_geom = wl.geometry()
    num_el = h.set_detector(true_geom, acc, 1, wl.nEbins)
    h._nbins = wl.nEbins
    qt = synth.shoemake_quaternions(n, wl.seed)
    probe = h.forward(qt[:16], capi.epilogue(1.0))
    pref = 1000.0 / float(probe.mean())            # 1000 counts per pixel on average
    noisy = capi.epilogue(pref, binning=4, scalingmode="lin", poisson=True, seed=44)
    clean = capi.epilogue(pref, binning=4, scalingmode="lin")
    targets = torch.empty((n, 120, 120), device=dev)
    h.forward(torch.from_numpy(qt).to(dev), noisy, out=targets)
    q0 = _perturb(qt, 1.0, rng)
    g0 = dict(true_geom)
    g0["xpc"] += float(rng.normal(0, 3))
    g0["ypc"] += float(rng.normal(0, 3))
    h.set_detector(g0, acc, 1, wl.nEbins)
    dq = torch.from_numpy(q0).to(dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    it, geom = h.refine(dq, clean, targets, max_iterations=20, refine_pc=True, damping=1e-3,
                        tol_rad=np.radians(1e-4), tol_pc=1e-3)
    torch.cuda.synchronize()
    gn_s = time.perf_counter() - t0
    mis = _misorientation_deg(dq.cpu().numpy(), qt)
    res = {"metric": "Gauss-Newton refinement: fraction of 100k orientations within 0.01 deg",
           "value": float((mis < 0.01).mean()), "unit": "fraction", "wall_s": gn_s,
           "iterations": it, "orientations": n,
           "median_misorientation_deg": float(np.median(mis)),
           "start_median_misorientation_deg": float(np.median(_misorientation_deg(q0, qt))),
           "pc_error_px": [geom["xpc"] - true_geom["xpc"], geom["ypc"] - true_geom["ypc"]],
           "L_error_um": geom["L"] - true_geom["L"],
           "config": {"workload": wl.name, "detector": "480x480 binned 4 -> 120x120",
                      "bins": wl.nEbins, "energies": "6-20 keV in 1 keV bins",
                      "noise": "Poisson, 1000 counts/px"}}
    if fd_iters > 0:
        h.set_detector(g0, acc, 1, wl.nEbins)
        dq = torch.from_numpy(q0).to(dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        qf, gf = _fd_gauss_newton(h, dq, clean, targets, g0, acc, fd_iters, 1e-3)
        torch.cuda.synchronize()
        fd_s = time.perf_counter() - t0
        misf = _misorientation_deg(qf.cpu().numpy(), qt)
        res["forward_only_fd"] = {"iterations": fd_iters, "wall_s": fd_s,
                                  "per_iteration_s": fd_s / fd_iters,
                                  "fraction_within_0.01deg": float((misf < 0.01).mean()),
                                  "gn_per_iteration_s": gn_s / max(it, 1)}
    h.close()
    return res


def run_gn(args):
    print(json.dumps(c5_measure(args, args.fd_iters)))
    return 0


def run_mc(args):
    """Monte-Carlo backscatter histograms (CTEMMC) at the program's defaults:
    Ni, 30 keV beam, 70 deg tilt, 1501^2 Lambert grid, 0.25 keV bins from
    20 keV (41 bins), exit depth to 50 nm.  value: electrons/s with the
    histograms resident on the device; e2e: the same through the C ABI into
    host arrays (370 MB copied back per step); cpu_baseline: the oracle's
    restatement with the reference's own generator streams, one OpenMP
    thread per stream as the reference runs it, on all host cores."""
    import numpy as np
    import torch

    from ctemsoft_gb300 import capi
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    p = capi.mc_params(Ze=28.0, density=8.908, at_wt=58.6934)
    nE, nz = capi.mc_dims(p)
    n10 = 750 // 10
    h = capi.Handle(0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    h.set_stream(stream.cuda_stream)
    de = torch.empty((1501, 1501, nE), dtype=torch.int32, device=dev)
    dz = torch.empty((2 * n10 + 1, 2 * n10 + 1, nz, nE), dtype=torch.int32, device=dev)
    N = args.mc_electrons
    for w in range(args.warmup):
        h.mc_run(p, 1000 + w, 0, max(1, N // 10), accum_e=de, accum_z=dz)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    counted = 0
    for k in range(args.steps):
        ev[k][0].record(stream)
        _, _, c = h.mc_run(p, 932117, k * N, N, accum_e=de, accum_z=dz)
        ev[k][1].record(stream)
        counted += c
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    value = N / (ms / 1e3)
    # the binary32 option (statistically equivalent trajectories)
    h.set_option("mc_fp32", 1)
    h.mc_run(p, 999, 0, max(1, N // 10), accum_e=de, accum_z=dz)
    a32, b32 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a32.record(stream)
    _, _, c32 = h.mc_run(p, 932117, 0, N, accum_e=de, accum_z=dz)
    b32.record(stream)
    torch.cuda.synchronize()
    fp32 = {"value": N / (a32.elapsed_time(b32) / 1e3), "unit": "electrons/s",
            "backscatter_fraction": c32 / N, "option": "mc_fp32 = 1"}
    h.set_option("mc_fp32", 0)
    # end to end: host histograms
    he = np.empty((1501, 1501, nE), np.int32)
    hz = np.empty((2 * n10 + 1, 2 * n10 + 1, nz, nE), np.int32)
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.e2e_steps, 2))
    for k in range(e2e_steps):
        h.mc_run(p, 932117, k * N, N, accum_e=he, accum_z=hz)
    e2e = e2e_steps * N / (time.perf_counter() - t0)
    base = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        threads = O.max_threads()
        op = O.mc_params(sig=p.sig, omega=p.omega, EkeV=p.EkeV, Ehistmin=p.Ehistmin,
                         Ebinsize=p.Ebinsize, depthmax=p.depthmax, depthstep=p.depthstep,
                         Ze=p.Ze, density=p.density, at_wt=p.at_wt, numsx=p.numsx)
        t = time.perf_counter()
        O.mc_reference_rng(op, 932117, 1, 2000)
        one = 2000 / (time.perf_counter() - t)
        per = int(max(2000, min(200000, one * args.cpu_seconds)))
        t = time.perf_counter()
        _, _, _ = O.mc_reference_rng(op, 932117, threads, per)
        dt = time.perf_counter() - t
        base = {"value": threads * per / dt, "unit": "electrons/s", "cores": threads,
                "kind": "port",
                "sample": f"{threads} streams x {per} electrons, the reference's generator and "
                          f"OpenMP layout (private 1501^2 x {nE} histograms), binary64 "
                          f"restatement of CTEMMC.f90:307-529",
                "single_thread_electrons_per_s": one}
    line = {
        "metric": "Monte-Carlo electrons/s (CTEMMC defaults: Ni, 30 keV, 1501^2 x 41 bins)",
        "value": value, "unit": "electrons/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": "f64",
        "data": "synthetic (material numbers of Ni)",
        "config": {"workload": "ctemmc-ni-30kev-1501", "electrons_per_step": N,
                   "backscatter_fraction": counted / (N * args.steps)},
        "e2e": {"value": e2e, "unit": "electrons/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(he.nbytes + hz.nbytes), "steps": e2e_steps},
        "fp32": fp32, "gpu_launches": 1 * args.steps, "clocks": ck, "cpu_baseline": base}
    print(json.dumps(line))
    return 0


def run_dictionary(args):
    """A dictionary: the m-3m fundamental zone sampled on the cubochoric grid
    (ebsd_sample_rfz, N steps per semi-edge) straight into the pattern loop
    on the 640x480 detector of the production workload, binned 8x8 to 80x60
    records with gamma 0.33, everything on the device.  One step = sampling
    + all patterns."""
    import torch

    from ctemsoft_gb300 import capi
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    wl, sr, acc, _ = _setup_data(0, 1)
    h = capi.Handle(0)
    h.set_master(sr)
    num_el = h.set_detector(wl.geometry(), acc, 1, wl.nEbins)
    epi = capi.epilogue(capi.prefactor(wl.beamcurrent, wl.dwelltime, num_el), binning=8,
                        scalingmode="gam", gammavalue=0.33)
    nx, ny = h.output_dims(epi)
    tuned = h.autotune(epi, 64, Path(tempfile.gettempdir()) / "ebsd_autotune.txt")
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    h.set_stream(stream.cuda_stream)
    import ctypes as C
    cnt = C.c_int64()
    N = args.dict_steps
    capi._check(capi.lib().ebsd_sample_rfz(h.raw, N, 32, None, None, 0, C.byref(cnt)), h.raw)
    n = cnt.value
    dq = torch.empty((n, 4), device=dev)
    out = torch.empty((n, ny, nx), device=dev)

    def step():
        capi._check(capi.lib().ebsd_sample_rfz(h.raw, N, 32, None, capi._ptr(dq), n,
                                               C.byref(cnt)), h.raw)
        h.forward(dq, epi, out=out)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(args.steps):
        step()
    b.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = a.elapsed_time(b) / args.steps
    t0 = time.perf_counter()
    h.sample_rfz(N, 32)
    samp_ms = (time.perf_counter() - t0) * 1e3
    line = {
        "metric": "dictionary patterns/s (m-3m zone, 640x480 binned 8 -> 80x60)",
        "value": n / (ms / 1e3), "unit": "patterns/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": "f32",
        "data": "synthetic", "config": {"workload": f"dictionary-m3m-N{N}-640x480-bin8",
                                         "orientations": n, "grid_points": (2 * N + 1) ** 3},
        "sampling_ms_host_call": samp_ms, "launch_shape": {"tile_y": tuned[0],
                                                            "orient_per_cta": tuned[1]},
        "clocks": ck, "gpu_launches": 5 * args.steps}
    print(json.dumps(line))
    return 0


def main():
    args = _args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "c3":
        return run_batched(args)
    if args.workload == "c4":
        return run_c4(args)
    if args.workload == "c5":
        return run_gn(args)
    if args.workload == "mc":
        return run_mc(args)
    if args.workload == "dict":
        return run_dictionary(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
