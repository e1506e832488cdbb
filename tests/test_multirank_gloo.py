"""Multi-rank path on CPU: two gloo ranks track their particle shards (with the
oracle standing in for the GPU) and sum their histograms; the result equals
the single-rank run bit for bit."""
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
