"""Batched realizations (mprw_create_batch): several grids of different sizes
tracked in one persistent launch.  Every member's particles end exactly where
a separate single-handle run with the same particle ids puts them (the step
of a particle depends only on its own state and its cells' records), and
the per-member histogram equals the separate runs' bit for bit and the GPKDE
density to rounding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from mprw import workloads as W
from mprw.model import FP64, MIXED, Options, Particles
from oracle import oracle as O


def _members(precision):
    """Three realizations of different sizes: two lognormal fields and a uniform column."""
    out = []
    for k, (nl, nr, nc) in enumerate(((4, 12, 30), (3, 8, 20), (5, 10, 24))):
        g, f, p, opt, info = W.lognormal_slab(n_particles=1500 + 700 * k, nlay=nl, nrow=nr, ncol=nc, seed=10 + k,
                                       precision=precision, use_torch=False)
        p.id = (np.uint64(k) << np.uint64(40)) + np.arange(p.n, dtype=np.uint64)
        out.append((g, f, p))
    return out, opt


def _separate(g, f, p, opt, iv):
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    steps = sum(tr.advance(a, b) for a, b in iv)
    out = tr.get_particles()
    hist = tr.histogram((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (g.ncol, g.nrow, g.nlay))[0]
    dens = tr.gpkde((float(g.ncol), float(g.nrow), float(g.top[0] - g.botm[-1])), (1.0, 1.0, 1.0))[0]
    tr.close()
    return out, steps, hist, dens


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_batch_members_equal_separate_runs(gpu_lib, precision):
    mem, opt = _members(precision)
    iv = [(0.0, 15.0), (15.0, 40.0)]
    b = mprw.Batch([m[0] for m in mem], opt)
    for k, (g, f, p) in enumerate(mem):
        b.load_flow(k, f)
    b.set_particles([m[2] for m in mem])
    steps = sum(b.advance(t0, t1) for t0, t1 in iv)
    outs = b.get_particles()
    doms = [(float(g.ncol), float(g.nrow), float(g.top[0] - g.botm[-1])) for g, _, _ in mem]
    # every member at once, three reconstructions in flight
    dens_all, loops = b.gpkde(doms, (1.0, 1.0, 1.0), concurrency=3)
    assert (loops >= 1).all()
    # one worker for every member, twice: the executable graph of its loop
    # body, kept from one reconstruction to the next, is updated in place for
    # each member's grid -- the same densities as three workers
    for _ in range(2):
        dens_one, loops_one = b.gpkde(doms, (1.0, 1.0, 1.0), concurrency=1)
        np.testing.assert_array_equal(loops_one, loops)
        for k in range(len(mem)):
            assert np.linalg.norm(dens_one[k] - dens_all[k]) <= 1e-12 * np.linalg.norm(dens_all[k])
    total = 0
    for k, (g, f, p) in enumerate(mem):
        ref, s, hist, dens = _separate(g, f, p, opt, iv)
        assert np.linalg.norm(dens_all[k] - dens) <= 1e-9 * np.linalg.norm(dens)
        total += s
        for key in ("cell", "status", "lx", "ly", "lz", "t", "rng_ctr", "gx", "gy", "gz"):
            np.testing.assert_array_equal(outs[k][key], ref[key], err_msg=f"member {k}: {key}")
        m = b.member(k)
        h2 = m.histogram((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (g.ncol, g.nrow, g.nlay))[0]
        np.testing.assert_array_equal(h2, hist)
        d2 = m.gpkde((float(g.ncol), float(g.nrow), float(g.top[0] - g.botm[-1])), (1.0, 1.0, 1.0))[0]
        # the reconstruction's scatters add in floating point with atomics: equal to rounding
        assert np.linalg.norm(d2 - dens) <= 1e-9 * np.linalg.norm(dens)
        assert (outs[k]["cell"] >= 1).all() and (outs[k]["cell"] <= g.ncell).all()
    assert steps == total
    b.close()


def test_batch_member_against_oracle_and_without_ids(gpu_lib):
    """A member against the oracle (same ids); without ids every member draws
    the streams of its batch index, so two copies of one realization differ."""
    g, f, p, opt, info = W.lognormal_slab(n_particles=2000, nlay=4, nrow=12, ncol=30, seed=3, use_torch=False)
    u, fu = W.uniform_flow(ncol=50, q=0.3)
    pu = W.release_in_box(u, 800, 5.0, 6.0, 0.0, 1.0, 0.0, 1.0, seed=9)
    p.id = np.arange(p.n, dtype=np.uint64)
    pu.id = np.arange(pu.n, dtype=np.uint64) + np.uint64(1 << 33)
    b = mprw.Batch([u, g], opt)
    b.load_flow(0, fu)
    b.load_flow(1, f)
    b.set_particles([pu, p])
    iv = [(0.0, 20.0), (20.0, 50.0)]
    for t0, t1 in iv:
        b.advance(t0, t1)
    out = b.member(1).get_particles()
    q = p
    for t0, t1 in iv:
        q, _ = O.advance(g, f, opt, q, t0, t1, rng_kind=O.RNG_PHILOX, nthreads=8)
    same = (out["status"] == q.status) & (out["cell"] == q.cell) & (out["rng_ctr"] == q.rng_ctr)
    for a, bb in (("lx", q.lx), ("ly", q.ly), ("lz", q.lz)):
        same &= np.abs(out[a] - bb) <= 1e-6
    assert same.mean() >= 0.995
    b.close()
    # two copies of one field, no ids: independent streams
    p2 = p.copy()
    p2.id = None
    b2 = mprw.Batch([g, g], opt)
    b2.load_flow(0, f)
    b2.load_flow(1, f)
    b2.set_particles([p2, p2])
    b2.advance(0.0, 20.0)
    o0, o1 = b2.get_particles()
    assert not np.array_equal(o0["lx"], o1["lx"])
    assert abs(o0["gx"].mean() - o1["gx"].mean()) < 0.5
    b2.close()


def test_batch_state_errors(gpu_lib):
    g, f, p, opt, info = W.lognormal_slab(n_particles=100, nlay=2, nrow=4, ncol=6, seed=0, use_torch=False)
    b = mprw.Batch([g, g], opt)
    b.load_flow(0, f)
    with pytest.raises(mprw.MprwError, match="member 1"):
        b.advance(0.0, 1.0)
    b.load_flow(1, f)
    with pytest.raises(mprw.MprwError, match="advanced by its batch"):
        b.member(0).advance(0.0, 1.0)
    lib = b.lib
    assert lib.mprw_advance(b.member(0).h, 0.0, 1.0, None) == -4        # MPRW_E_STATE
    assert lib.mprw_load_flow(b.h, None) == -4
    assert lib.mprw_destroy(b.member(0).h) == -4
    q = p.copy()
    q.cell = np.where(np.arange(p.n) == 0, g.ncell + 1, p.cell).astype(np.int32)
    with pytest.raises(mprw.MprwError, match="member 1"):
        b.set_particles([p, q])
    b.set_particles([p, p])
    # a member may overwrite its particles but not change their count
    b.member(1).set_particles(p)
    with pytest.raises(mprw.MprwError):
        b.member(1).set_particles(W.release_in_box(g, 10, 0.5, 1.5, 0.5, 1.5, 0.5, 1.5))
    b.advance(0.0, 5.0)
    b.close()


def test_batch_member_observations_and_empty_member(gpu_lib):
    """Observation records of a member that does not start at cell 0 equal a
    separate handle's; a member without particles is carried along."""
    g, f, p, opt, info = W.lognormal_slab(n_particles=4000, nlay=4, nrow=12, ncol=30, seed=7, use_torch=False)
    u, fu = W.uniform_flow(ncol=20, q=0.3)
    empty = W.release_in_box(u, 0, 1.0, 2.0, 0.0, 1.0, 0.0, 1.0)
    k, i, j = np.meshgrid(np.arange(g.nlay), np.arange(g.nrow), np.arange(g.ncol), indexing="ij")
    node = (k * g.nrow * g.ncol + i * g.ncol + j + 1).ravel()
    col = j.ravel()
    cells = np.concatenate([node[col == g.ncol - 1], node[col == g.ncol // 2]]).astype(np.int32)
    obs = np.concatenate([np.zeros((col == g.ncol - 1).sum()), np.ones((col == g.ncol // 2).sum())]).astype(np.int32)
    style = np.array([2, 1], np.int32)
    ref = mprw.Tracker(g, opt)
    ref.load_flow(f)
    ref.set_particles(p)
    ref.set_observations(cells, obs, style)
    b = mprw.Batch([u, g], opt)         # the field is member 1: its cells start after the column's 20
    b.load_flow(0, fu)
    b.load_flow(1, f)
    b.set_particles([empty, p])
    m = b.member(1)
    m.set_observations(cells, obs, style)
    for t0, t1 in ((0.0, 40.0), (40.0, 120.0)):
        assert b.advance(t0, t1) == ref.advance(t0, t1)
        r1, r2 = m.observe_sinks(), ref.observe_sinks()
        for key in ("obs", "id", "time", "mass"):
            np.testing.assert_array_equal(r1[key], r2[key])
        c1, m1 = m.observe_resident()
        c2, m2 = ref.observe_resident()
        np.testing.assert_array_equal(c1, c2)
        np.testing.assert_array_equal(m1, m2)
    assert b.member(0).get_particles()["cell"].shape == (0,)
    ref.close()
    b.close()
