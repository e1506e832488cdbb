"""Reconstruction from summed parts: the multi-GPU collective of the GPKDE.

The particles are split into shards that keep their global ids (the
counter-based random streams), each shard tracked by its own handle; each
handle's part of the reconstruction (mprw_gpkde_partial: mass per bin and
the sums behind the effective mass and the coordinate statistics) is summed,
and mprw_gpkde_from_counts reconstructs.  Checked against one handle that
tracks every particle and reconstructs with mprw_gpkde: the histogram
identical, the same loop count, the density equal to rounding (the
statistics are summed in another order), on unit masses (lognormal field,
3-D) and on non-unit masses (uniform column, 1-D).  A world-2 gloo run
drives the same path through torch.distributed with two processes on the
one GPU (independent kernels: the exchange is a host all-reduce), with the
oracle's histogram of all particles as the check.
"""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from mprw import shard
from mprw import workloads as W
from mprw.model import ACTIVE


def _track(g, f, opt, p, t1):
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, t1)
    return tr


def _sum_parts(parts):
    mass = sum(m for m, _ in parts)
    tot = mprw.GpkdeSums()
    for _, s in parts:
        tot.n_active += s.n_active
        tot.sum_w += s.sum_w
        tot.sum_w2 += s.sum_w2
        for d in range(3):
            tot.sum_dx[d] += s.sum_dx[d]
            tot.sum_dx2[d] += s.sum_dx2[d]
    return mass, tot


@pytest.mark.parametrize("case", ["lognormal_unit_mass", "uniform_weighted"])
def test_reconstruction_from_summed_shards_equals_single_handle(gpu_lib, case):
    if case == "lognormal_unit_mass":
        g, f, p, opt, _ = W.lognormal_slab(n_particles=60_000, nlay=6, nrow=20, ncol=40, seed=1, use_torch=False)
        t1, dom = 30.0, (40.0, 20.0, 6.0)
    else:
        g, f, p, opt = W.uniform_pulse(n_particles=40_000)
        p.mass = np.random.default_rng(5).uniform(0.5, 2.0, p.n)
        t1, dom = 40.0, (200.0, 1.0, 1.0)
    bins = (1.0, 1.0, 1.0)
    single = _track(g, f, opt, p, t1)
    d1, h1, l1 = single.gpkde(dom, bins)
    single.close()
    parts, trs = [], []
    for r in range(3):
        tr = _track(g, f, opt, shard.shard_particles(p, r, 3), t1)
        parts.append(tr.gpkde_partial(dom, bins))
        trs.append(tr)
    mass, sums = _sum_parts(parts)
    assert sums.n_active == float((np.concatenate([t.get_particles()["status"] for t in trs]) == ACTIVE).sum())
    d2, h2, l2 = trs[1].gpkde_from_counts(dom, bins, mass, sums)
    for tr in trs:
        tr.close()
    assert l2 == l1
    np.testing.assert_allclose(h2, h1, rtol=1e-14, atol=0)
    np.testing.assert_allclose(d2, d1, rtol=0, atol=1e-11 * d1.max())


def test_from_counts_rejects_bad_input(gpu_lib):
    g, f, p, opt = W.uniform_pulse(n_particles=1000)
    tr = _track(g, f, opt, p, 10.0)
    mass, sums = tr.gpkde_partial((200.0, 1.0, 1.0), (1.0, 1.0, 1.0))
    sums.sum_dx[0] = float("nan")
    with pytest.raises(mprw.MprwError):
        tr.gpkde_from_counts((200.0, 1.0, 1.0), (1.0, 1.0, 1.0), mass, sums)
    with pytest.raises(ValueError):
        tr.gpkde_from_counts((200.0, 1.0, 1.0), (1.0, 1.0, 1.0), mass[:, :, :10], sums)
    tr.close()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _workload():
    return W.lognormal_slab(n_particles=30_000, nlay=4, nrow=12, ncol=30, seed=2, use_torch=False)


DOM, BINS = (30.0, 12.0, 4.0), (1.0, 1.0, 1.0)


def _rank(rank, world, port, out):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    for q in (str(root / "modpath-rw_gb300"), str(root)):
        if q not in sys.path:
            sys.path.insert(0, q)
    import torch
    import torch.distributed as dist
    import mprw as M
    from mprw import shard as S
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g, f, p, opt, _ = _workload()
    tr = M.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(S.shard_particles(p, rank, world))
    tr.advance(0.0, 25.0)
    dens, hist, loops = S.gpkde_allreduce(tr, DOM, BINS)
    q = tr.get_particles()
    tr.close()
    np.savez(f"{out}.{rank}.npz", dens=dens, hist=hist, loops=loops, gx=q["gx"], gy=q["gy"], gz=q["gz"],
             status=q["status"])
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_reconstruction(gpu_lib, tmp_path):
    import torch.multiprocessing as mp
    from oracle import gpkde_oracle as GO
    out = str(tmp_path / "r")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(timeout=300)
        assert pr.exitcode == 0
    res = [np.load(f"{out}.{r}.npz") for r in range(2)]
    # both ranks reconstructed the same density
    assert int(res[0]["loops"]) == int(res[1]["loops"])
    assert np.array_equal(res[0]["dens"], res[1]["dens"])
    # the summed histogram is the oracle's histogram of every rank's particles
    co = np.concatenate([np.stack([r["gx"], r["gy"], r["gz"]], 1)[r["status"] == ACTIVE] for r in res])
    h, _, _ = GO.histogram_weighted(co, np.ones(co.shape[0]), (0.0, 0.0, 0.0), BINS, (30, 12, 4))
    np.testing.assert_array_equal(res[0]["hist"], h)
    # and the reconstruction is the single handle's
    g, f, p, opt, _ = _workload()
    tr = _track(g, f, opt, p, 25.0)
    d1, _, l1 = tr.gpkde(DOM, BINS)
    tr.close()
    assert int(res[0]["loops"]) == l1
    np.testing.assert_allclose(res[0]["dens"], d1, rtol=0, atol=1e-11 * d1.max())
