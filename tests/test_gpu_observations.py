"""Observation cells on the device (Observation.f90:7-60; MPathRW.F90:1337-1392
sink records, 1460-1535 resident records), through the C ABI.

* the records equal the same selection made with numpy from the particle
  state the library reports (exact: ids, times, masses, counts);
* the sink records and resident counts agree with the oracle's tracking of
  the same particles on the shared random stream (per-particle agreement
  is >= 99.5 %, so the counts agree within 1 %);
* a breakthrough curve at the outlet from the sink records of successive
  intervals holds every arrival exactly once."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from mprw import workloads as W
from mprw.model import ACTIVE
from oracle import oracle as O


def _case():
    g, f, p, opt, info = W.lognormal_slab(n_particles=6000, nlay=4, nrow=12, ncol=30, seed=0, use_torch=False)
    opt.stop_weak_sinks = True
    rng = np.random.default_rng(4)
    p.mass = rng.uniform(0.5, 1.5, p.n)
    k, i, j = np.meshgrid(np.arange(g.nlay), np.arange(g.nrow), np.arange(g.ncol), indexing="ij")
    node = (k * g.nrow * g.ncol + i * g.ncol + j + 1).ravel()
    col = j.ravel()
    sink_cells = node[col == g.ncol - 1]       # the constant-head outlet column
    res_cells = node[col == g.ncol // 2]       # a control plane across the field
    cells = np.concatenate([sink_cells, res_cells]).astype(np.int32)
    obs = np.concatenate([np.zeros(sink_cells.size), np.ones(res_cells.size)]).astype(np.int32)
    style = np.array([2, 1], np.int32)
    return g, f, p, opt, cells, obs, style


def _expected(out, cells, obs, t0, t1):
    of = np.full(int(cells.max()) + 2, -1)
    of[cells] = obs
    c1 = out["cell"]
    k = np.where(c1 < of.shape[0], of[np.minimum(c1, of.shape[0] - 1)], -1)
    st, t = out["status"], out["t"]
    sink = ((st == 3) | (st == 4)) & (t > t0) & (t <= t1) & (k == 0)
    res = (st == ACTIVE) & (k == 1)
    return sink, res


def test_observation_records_match_particle_state(gpu_lib):
    g, f, p, opt, cells, obs, style = _case()
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.set_observations(cells, obs, style)
    arrivals = []
    for t0, t1 in ((0.0, 40.0), (40.0, 120.0)):
        tr.advance(t0, t1)
        out = tr.get_particles()
        rec = tr.observe_sinks()
        cnt, mass = tr.observe_resident()
        sink, res = _expected(out, cells, obs, t0, t1)
        np.testing.assert_array_equal(rec["id"], p.id[sink])
        np.testing.assert_array_equal(rec["time"], out["t"][sink])
        np.testing.assert_array_equal(rec["mass"], p.mass[sink])
        assert np.all(rec["obs"] == 0)
        assert cnt[0] == 0 and mass[0] == 0.0     # the sink observation has no resident records
        assert cnt[1] == res.sum()
        np.testing.assert_allclose(mass[1], p.mass[res].sum(), rtol=1e-12)
        arrivals.append(rec)
    # breakthrough at the outlet: every stopped particle arrives exactly once
    ids = np.concatenate([r["id"] for r in arrivals])
    times = np.concatenate([r["time"] for r in arrivals])
    assert ids.size == np.unique(ids).size
    out = tr.get_particles()
    stopped_at_outlet = ((out["status"] == 3) | (out["status"] == 4)) & np.isin(out["cell"], cells[obs == 0])
    assert ids.size == stopped_at_outlet.sum() > 0
    assert times.min() > 0.0 and times.max() <= 120.0
    tr.close()


def test_observations_against_oracle(gpu_lib):
    g, f, p, opt, cells, obs, style = _case()
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.set_observations(cells, obs, style)
    tr.advance(0.0, 20.0)
    rec = tr.observe_sinks()
    cnt, mass = tr.observe_resident()
    tr.close()
    q, _ = O.advance(g, f, opt, p, 0.0, 20.0, rng_kind=O.RNG_PHILOX, nthreads=8)
    oq = dict(cell=q.cell, status=q.status, t=q.t)
    sink, res = _expected(oq, cells, obs, 0.0, 20.0)
    assert rec["id"].size > 1000 and res.sum() > 100
    assert abs(rec["id"].size - sink.sum()) <= max(2, 0.01 * sink.sum())
    assert abs(int(cnt[1]) - int(res.sum())) <= max(2, 0.01 * res.sum())
    common = np.intersect1d(rec["id"], p.id[sink])
    assert common.size >= 0.98 * sink.sum()
    # the same particles arrive at the same times (to the trajectories' 1e-6 agreement)
    gt = dict(zip(rec["id"].tolist(), rec["time"].tolist()))
    ot = dict(zip(p.id[sink].tolist(), q.t[sink].tolist()))
    dt = np.array([abs(gt[i] - ot[i]) for i in common.tolist()])
    assert np.quantile(dt, 0.99) <= 1e-6 * 20.0
