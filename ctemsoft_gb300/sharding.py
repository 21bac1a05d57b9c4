"""Orientation sharding across ranks (one process per GPU).

Orientations are independent, so N ranks split the orientation list into
contiguous blocks, compute without any collective, and either concatenate
their records or write them straight into the shared output file at their
own byte offsets (the file layout of CTEMEBSD.f90:555-561,654-658: a 12-byte
header record, then one (4*nx*ny + 8)-byte record per pattern).

For Gauss-Newton refinement with one pattern centre shared by every
pattern, each rank reduces its patterns to a 3x3 Schur-complement system of
the centre; summing those 12 numbers across ranks is the only exchange.

This module serves callers that run one process per GPU.  Within one
process the C ABI does both without Python: ebsd_run_namelist_devices
(one shard and host thread per device, records written at their offsets)
and ebsd_refine_sharded (the 12 numbers summed in the process).
"""
from __future__ import annotations

import numpy as np

HEADER_BYTES = 4 + 12 + 4  # marker, (nx, ny, N) int32, marker


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """[begin, end) of rank's contiguous block of n orientations; blocks
    differ in size by at most one and cover 0..n exactly once."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def record_offset(k: int, nx: int, ny: int) -> int:
    """Byte offset of record k (its leading marker) in an output file."""
    return HEADER_BYTES + k * (4 * nx * ny + 8)


def write_shard(path, begin: int, records: np.ndarray) -> None:
    """Write this rank's records in place (the header is written by rank 0
    and the file pre-sized by write_header)."""
    recs = np.ascontiguousarray(records, "<f4")
    n, ny, nx = recs.shape
    marker = np.array([4 * nx * ny], "<i4").tobytes()
    with open(path, "r+b") as f:
        f.seek(record_offset(begin, nx, ny))
        for r in recs:
            f.write(marker)
            f.write(r.tobytes())
            f.write(marker)


def write_header(path, nx: int, ny: int, n: int, header_dims=None) -> None:
    """Create the output file with its header record and full size."""
    hx, hy = header_dims if header_dims is not None else (nx, ny)
    with open(path, "wb") as f:
        f.write(np.array([12, hx, hy, n, 12], "<i4").tobytes())
        f.truncate(record_offset(n, nx, ny))


def schur_pc_system(A: np.ndarray, B: np.ndarray, C: np.ndarray, g_rot: np.ndarray,
                    g_pc: np.ndarray, damping: float = 0.0):
    """Reduce per-pattern Gauss-Newton blocks to the shared-centre system.

    For pattern n the normal equations are
        [A_n  B_n] [d_rot_n]   [g_rot_n]
        [B_n' C_n] [d_pc   ] = [g_pc_n ]
    with d_pc shared.  Eliminating d_rot_n gives S d_pc = r with
        S = sum_n (C_n - B_n' A_n^-1 B_n),  r = sum_n (g_pc_n - B_n' A_n^-1 g_rot_n).
    Returns (S, r): 9 + 3 numbers to sum across ranks."""
    n = A.shape[0]
    Ad = A + damping * np.eye(3)[None]
    Ainv = np.linalg.inv(Ad)
    BtAi = np.einsum("nji,njk->nik", B, Ainv)
    S = (C - np.einsum("nij,njk->nik", BtAi, B)).sum(axis=0)
    r = (g_pc - np.einsum("nij,nj->ni", BtAi, g_rot)).sum(axis=0)
    return S, r


def schur_back_substitute(A, B, g_rot, d_pc, damping: float = 0.0):
    """d_rot_n = A_n^-1 (g_rot_n - B_n d_pc)."""
    Ad = A + damping * np.eye(3)[None]
    return np.linalg.solve(Ad, (g_rot - np.einsum("nij,j->ni", B, d_pc))[..., None])[..., 0]


def allreduce_sum(arrays, group=None):
    """Sum numpy arrays across torch.distributed ranks (any backend);
    identity when not initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [np.asarray(a) for a in arrays]
    flat = np.concatenate([np.asarray(a, np.float64).ravel() for a in arrays])
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.from_numpy(flat).to(dev)
    dist.all_reduce(t, group=group)
    out, i = [], 0
    flat = t.cpu().numpy()
    for a in arrays:
        a = np.asarray(a)
        out.append(flat[i:i + a.size].reshape(a.shape))
        i += a.size
    return out


def allreduce_sum_int(arrays, group=None):
    """Exact sum of integer numpy arrays across torch.distributed ranks (int64
    on the wire); identity when not initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [np.asarray(a) for a in arrays]
    flat = np.concatenate([np.asarray(a, np.int64).ravel() for a in arrays])
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.from_numpy(flat).to(dev)
    dist.all_reduce(t, group=group)
    flat = t.cpu().numpy()
    out, i = [], 0
    for a in arrays:
        a = np.asarray(a)
        out.append(flat[i:i + a.size].reshape(a.shape).astype(a.dtype))
        i += a.size
    return out


def mc_sharded(run, n_total: int, rank: int = 0, world: int = 1, group=None):
    """Monte-Carlo histograms of electrons [0, n_total) spread over ranks:
    this rank runs its contiguous range with run(first, n) -> (accum_e,
    accum_z, counted) -- e.g. a Handle.mc_run bound to the parameters and
    seed -- and the integer histograms are summed across ranks.  Each
    electron's random stream depends only on (seed, electron index), so the
    result equals a one-GPU run of all n_total electrons."""
    b, e = shard_range(n_total, rank, world)
    acc, accz, counted = run(b, e - b)
    arrays = [acc, np.array([counted], np.int64)] + ([accz] if accz is not None else [])
    summed = allreduce_sum_int(arrays, group)
    return summed[0], (summed[2] if accz is not None else None), int(summed[1][0])
