"""Particle sharding across ranks (one GPU per rank).

Particles are independent within a tracking interval
(MPathRW.F90:1207-1539), so ranks take contiguous id ranges and keep the
global particle ids as Philox keys: a particle's trajectory does not depend
on which rank tracks it.  The only exchange is the sum of the per-rank GPKDE
parts before the smoothing: the mass per bin (integer-valued for unit
masses, so the sum is exact in float64 below 2^53 particles per bin) and the
sums behind the effective mass and the coordinate statistics
(mprw_gpkde_partial); one sum-all-reduce per reconstruction, after which any
rank reconstructs (mprw_gpkde_from_counts).
"""
from __future__ import annotations

import numpy as np

from .model import Particles


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [start, stop) block of n particles for this rank."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("invalid rank/world")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard_particles(p: Particles, rank: int, world: int) -> Particles:
    a, b = shard_range(p.n, rank, world)
    ids = np.arange(p.n, dtype=np.uint64) if p.id is None else p.id
    sl = slice(a, b)
    take = lambda x: None if x is None else np.array(x[sl], copy=True)
    return Particles(cell=take(p.cell), lx=take(p.lx), ly=take(p.ly), lz=take(p.lz), t=take(p.t),
                     status=take(p.status), mass=take(p.mass), id=np.array(ids[sl], copy=True),
                     rng_ctr=take(p.rng_ctr))


def allreduce_histogram(counts: np.ndarray, group=None) -> np.ndarray:
    """Sum a per-rank histogram over all ranks (torch.distributed, any backend)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(counts, dtype=np.float64))
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy().reshape(counts.shape)


def allreduce_sums(sums, group=None):
    """Sum a GpkdeSums record over all ranks (in place) and return it."""
    import torch
    import torch.distributed as dist
    v = torch.tensor([sums.n_active, sums.sum_w, sums.sum_w2, *sums.sum_dx, *sums.sum_dx2], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        v = v.cuda()
    dist.all_reduce(v, op=dist.ReduceOp.SUM, group=group)
    v = v.cpu().tolist()
    sums.n_active, sums.sum_w, sums.sum_w2 = v[0], v[1], v[2]
    for d in range(3):
        sums.sum_dx[d], sums.sum_dx2[d] = v[3 + d], v[6 + d]
    return sums


def gpkde_allreduce(tracker, domain_size, bin_size, origin=(0.0, 0.0, 0.0), group=None, **kw):
    """GPKDE of the particles of every rank's tracker: each rank's part
    (mprw_gpkde_partial) is summed over the ranks, then every rank
    reconstructs the same density from the sums (mprw_gpkde_from_counts).
    Returns (density, histogram, loops) as Tracker.gpkde."""
    mass, sums = tracker.gpkde_partial(domain_size, bin_size, origin, **kw)
    total = allreduce_histogram(mass, group)
    allreduce_sums(sums, group)
    return tracker.gpkde_from_counts(domain_size, bin_size, total, sums, origin, **kw)
