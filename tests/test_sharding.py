"""Host logic of the multi-GPU path, on CPU: orientation shards, in-place
record writes at the reference's file offsets, and the shared-centre
Gauss-Newton reduction across world_size 2 gloo ranks."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from ctemsoft_gb300 import formats, sharding


@pytest.mark.parametrize("n,world", [(0, 1), (1, 2), (7, 2), (10000, 8), (5, 8)])
def test_shards_cover_exactly_once(n, world):
    seen = np.zeros(n, int)
    sizes = []
    for r in range(world):
        b, e = sharding.shard_range(n, r, world)
        seen[b:e] += 1
        sizes.append(e - b)
    assert (seen == 1).all()
    assert max(sizes) - min(sizes) <= 1


def test_shard_writes_make_the_reference_file(tmp_path):
    nx, ny, n = 6, 4, 7
    rng = np.random.default_rng(0)
    recs = rng.random((n, ny, nx), dtype=np.float32)
    p = tmp_path / "out.data"
    sharding.write_header(p, nx, ny, n)
    for r in (1, 0, 2):  # any order
        b, e = sharding.shard_range(n, r, 3)
        sharding.write_shard(p, b, recs[b:e])
    hdr, pats = formats.read_output_file(p)
    assert hdr == (nx, ny, n)
    assert all(np.array_equal(a, r.ravel()) for a, r in zip(pats, recs))


def test_schur_reduction_matches_dense_solve():
    rng = np.random.default_rng(1)
    n = 5
    J = rng.standard_normal((n, 40, 6))  # per-pattern Jacobians (rot3 + pc3)
    res = rng.standard_normal((n, 40))
    # dense system with shared centre: unknowns 3n + 3
    H = np.zeros((3 * n + 3, 3 * n + 3))
    g = np.zeros(3 * n + 3)
    A = np.zeros((n, 3, 3)); B = np.zeros((n, 3, 3)); Cm = np.zeros((n, 3, 3))
    gr = np.zeros((n, 3)); gp = np.zeros((n, 3))
    for k in range(n):
        JtJ = J[k].T @ J[k]
        Jtr = J[k].T @ res[k]
        A[k], B[k], Cm[k] = JtJ[:3, :3], JtJ[:3, 3:], JtJ[3:, 3:]
        gr[k], gp[k] = Jtr[:3], Jtr[3:]
        s = slice(3 * k, 3 * k + 3)
        H[s, s] = A[k]
        H[s, -3:] = B[k]
        H[-3:, s] = B[k].T
        H[-3:, -3:] += Cm[k]
        g[s] = gr[k]
        g[-3:] += gp[k]
    x = np.linalg.solve(H, g)
    S, r = sharding.schur_pc_system(A, B, Cm, gr, gp)
    dpc = np.linalg.solve(S, r)
    drot = sharding.schur_back_substitute(A, B, gr, dpc)
    np.testing.assert_allclose(dpc, x[-3:], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(drot.ravel(), x[:-3], rtol=1e-9, atol=1e-12)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(7)
        n = 9
        A = np.stack([np.eye(3) * (2 + i) for i in range(n)])
        B = rng.standard_normal((n, 3, 3)) * 0.1
        Cm = np.stack([np.eye(3)] * n)
        gr = rng.standard_normal((n, 3))
        gp = rng.standard_normal((n, 3))
        b, e = sharding.shard_range(n, rank, world)
        S, r = sharding.schur_pc_system(A[b:e], B[b:e], Cm[b:e], gr[b:e], gp[b:e])
        S, r = sharding.allreduce_sum([S, r])
        dpc = np.linalg.solve(S, r)
        S1, r1 = sharding.schur_pc_system(A, B, Cm, gr, gp)
        q.put((rank, float(np.abs(dpc - np.linalg.solve(S1, r1)).max())))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_shared_centre():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = dict(q.get(timeout=5) for _ in range(2))
    assert max(res.values()) < 1e-12
    del torch


def _mc_worker(rank, world, port, q):
    import torch.distributed as dist
    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p = O.mc_params(numsx=61)

        def run(first, n):
            return O.mc_philox(p, 13, first, first + n)

        acc, accz, n = sharding.mc_sharded(run, 3001, rank, world)
        ref, refz, nref = O.mc_philox(p, 13, 0, 3001)
        q.put((rank, bool(np.array_equal(acc, ref) and np.array_equal(accz, refz) and n == nref)))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_monte_carlo_ranges_sum_to_one_run():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_mc_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = dict(q.get(timeout=5) for _ in range(2))
    assert all(res.values())
