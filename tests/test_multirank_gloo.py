"""Multi-rank path on CPU: two gloo ranks track their particle shards (with the
oracle standing in for the GPU) and sum their histograms; the result equals
the single-rank run bit for bit.  The reduce-then-reconstruct path of the
library (shard.gpkde_allreduce: each rank's mprw_gpkde_partial summed over
the ranks, then mprw_gpkde_from_counts) runs against a stand-in tracker whose
parts are the oracle's histogram and sums of its shard: the reconstruction
receives the single-rank histogram and sums."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from mprw import shard


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _workload():
    from mprw import workloads as W
    return W.lognormal_slab(n_particles=900, nlay=3, nrow=8, ncol=20, seed=5, use_torch=False)


HIST = ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (20, 8, 3))


def _hist(g, f, q):
    from oracle import gpkde_oracle as GO
    from oracle import oracle as O
    gx, gy, gz = O.global_xyz(g, f, q)
    act = q.status == 1
    c, _, _ = GO.histogram_weighted(np.stack([gx, gy, gz], 1)[act], np.ones(int(act.sum())), *HIST)
    return c


def _rank(rank, world, port, out):
    import torch.distributed as dist
    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g, f, p, opt, _ = _workload()
    q = shard.shard_particles(p, rank, world)
    q, _ = O.advance(g, f, opt, q, 0.0, 40.0, rng_kind=O.RNG_PHILOX, nthreads=2)
    total = shard.allreduce_histogram(_hist(g, f, q))
    if rank == 0:
        np.save(out, total)
    dist.destroy_process_group()


class _OracleTracker:
    """Stands in for mprw.Tracker on CPU: gpkde_partial gives the oracle's
    mass per bin and sums of the particles it holds; gpkde_from_counts records
    what it receives."""

    def __init__(self, pos):
        self.pos = pos

    def gpkde_partial(self, domain_size, bin_size, origin=(0.0, 0.0, 0.0), **kw):
        from mprw import GpkdeSums
        from oracle import gpkde_oracle as GO
        nb = tuple(int(domain_size[d] / bin_size[d] + 0.5) for d in range(3))
        c, _, _ = GO.histogram_weighted(self.pos, np.ones(len(self.pos)), origin, bin_size, nb)
        s = GpkdeSums()
        s.n_active, s.sum_w, s.sum_w2 = float(len(self.pos)), float(len(self.pos)), float(len(self.pos))
        centre = [origin[d] + 0.5 * domain_size[d] for d in range(3)]
        for d in range(3):
            dx = self.pos[:, d] - centre[d]
            s.sum_dx[d], s.sum_dx2[d] = float(dx.sum()), float((dx * dx).sum())
        return c, s

    def gpkde_from_counts(self, domain_size, bin_size, mass, sums, origin=(0.0, 0.0, 0.0), **kw):
        return mass, sums, 0


def _positions(g, f, q):
    from oracle import oracle as O
    gx, gy, gz = O.global_xyz(g, f, q)
    act = q.status == 1
    return np.stack([gx, gy, gz], 1)[act]


def _rank_reduce(rank, world, port, out):
    import torch.distributed as dist
    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g, f, p, opt, _ = _workload()
    q = shard.shard_particles(p, rank, world)
    q, _ = O.advance(g, f, opt, q, 0.0, 40.0, rng_kind=O.RNG_PHILOX, nthreads=2)
    mass, sums, _ = shard.gpkde_allreduce(_OracleTracker(_positions(g, f, q)), (20.0, 8.0, 3.0), (1.0, 1.0, 1.0))
    np.savez(out + f".{rank}.npz", mass=mass, sums=np.array([sums.n_active, sums.sum_w, sums.sum_w2,
                                                            *sums.sum_dx, *sums.sum_dx2]))
    dist.destroy_process_group()


def test_shard_range_covers():
    n = 1001
    spans = [shard.shard_range(n, r, 4) for r in range(4)]
    assert spans[0][0] == 0 and spans[-1][1] == n
    assert all(spans[i][1] == spans[i + 1][0] for i in range(3))
    with pytest.raises(ValueError):
        shard.shard_range(10, 2, 2)


def test_two_rank_histogram_equals_single_rank(tmp_path):
    from oracle import oracle as O
    out = str(tmp_path / "h.npy")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(timeout=240)
        assert pr.exitcode == 0
    g, f, p, opt, _ = _workload()
    q, _ = O.advance(g, f, opt, p, 0.0, 40.0, rng_kind=O.RNG_PHILOX, nthreads=2)
    single = _hist(g, f, q)
    np.testing.assert_array_equal(np.load(out), single)


def test_two_rank_reduce_then_reconstruct(tmp_path):
    from oracle import oracle as O
    out = str(tmp_path / "r")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_reduce, args=(r, 2, port, out)) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(timeout=240)
        assert pr.exitcode == 0
    g, f, p, opt, _ = _workload()
    q, _ = O.advance(g, f, opt, p, 0.0, 40.0, rng_kind=O.RNG_PHILOX, nthreads=2)
    mass, sums = _OracleTracker(_positions(g, f, q)).gpkde_partial((20.0, 8.0, 3.0), (1.0, 1.0, 1.0))
    want = np.array([sums.n_active, sums.sum_w, sums.sum_w2, *sums.sum_dx, *sums.sum_dx2])
    for r in range(2):
        got = np.load(out + f".{r}.npz")
        # every rank reconstructs from the same summed parts
        np.testing.assert_array_equal(got["mass"], mass)
        np.testing.assert_array_equal(got["sums"][:3], want[:3])
        np.testing.assert_allclose(got["sums"][3:], want[3:], rtol=1e-12, atol=1e-9)
