"""Breakthrough curves on the GPU (mprw.btc with its default reconstruction,
mprw_gpkde_series) against the same assembly over the oracle's 1-D GPKDE,
and end to end from the device's own sink records of a tracking run
(MPathRW.F90:1337-1392 records, 1759-2840 post-process)."""
import numpy as np
import pytest

import mprw
from mprw import btc as BT
from mprw import workloads as W
from oracle import series_oracle as SO

pytestmark = pytest.mark.gpu


def oracle_series(t, w, **kw):
    return SO.gpkde_series(t, w, **kw)


def close(a, b, rel):
    a = np.asarray(a)
    b = np.asarray(b)
    np.testing.assert_allclose(a, b, rtol=0, atol=rel * max(np.abs(b).max(), 1e-300))


def test_resident_btc_gpu_matches_oracle():
    rng = np.random.default_rng(0)
    tp = np.arange(1, 61) * 5.0
    t = tp[np.clip(np.round(rng.normal(25, 7, 8000)).astype(int), 0, 59)]
    groups = rng.integers(1, 3, t.shape[0])
    w = rng.uniform(0.2, 1.0, t.shape[0])
    vw = rng.uniform(5.0, 8.0, 60)
    for post in (0, 1):
        opt = BT.ObservationOptions(postprocess=post)
        g = BT.resident_btc(t, w, groups, [[1], [2]], tp, vw, opt)
        o = BT.resident_btc(t, w, groups, [[1], [2]], tp, vw, opt, series=oracle_series)
        close(g["hist"], o["hist"], 1e-12)
        if post == 1:
            close(g["gpkde"], o["gpkde"], 1e-10)
            assert [r["loops"] for r in g["raw"]] == [r["loops"] for r in o["raw"]]


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
def test_sink_btc_gpu_matches_oracle(fmt):
    rng = np.random.default_rng(fmt)
    t = rng.lognormal(np.log(50.0), 0.35, 5000)
    groups = rng.integers(1, 3, t.shape[0])
    w = np.full(t.shape[0], 0.004)
    opt = BT.ObservationOptions(histogram_bin_format=fmt, histogram_bin=1.0)
    tp = np.arange(1, 201) * 1.5
    g = BT.sink_btc(t, w, groups, [[1], [2]], opt, stoptime=300.0, time_points=tp, flow_constant=2.0)
    o = BT.sink_btc(t, w, groups, [[1], [2]], opt, stoptime=300.0, time_points=tp, flow_constant=2.0,
                    series=oracle_series)
    if g["per_solute"]:
        for s in range(2):
            close(g["time"][s], o["time"][s], 1e-13)
            close(g["hist"][s], o["hist"][s], 1e-12)
            close(g["gpkde"][s], o["gpkde"][s], 1e-10)
    else:
        close(g["hist"], o["hist"], 1e-12)
        close(g["gpkde"], o["gpkde"], 1e-10)


def test_sink_btc_from_device_records():
    """Track a heterogeneous slab to its outlet, collect the outlet's sink
    records interval by interval, and reconstruct the flux concentration:
    its integral is the arrived mass over the flow, on GPU and oracle alike."""
    g, f, p, opt, info = W.lognormal_slab(n_particles=20000, nlay=4, nrow=12, ncol=30, seed=0, use_torch=False)
    opt.stop_weak_sinks = True
    rng = np.random.default_rng(4)
    p.mass = rng.uniform(0.5, 1.5, p.n)
    k, i, j = np.meshgrid(np.arange(g.nlay), np.arange(g.nrow), np.arange(g.ncol), indexing="ij")
    node = (k * g.nrow * g.ncol + i * g.ncol + j + 1).ravel()
    outlet = node[j.ravel() == g.ncol - 1].astype(np.int32)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.set_observations(outlet, np.zeros(outlet.size, np.int32), np.array([2], np.int32))
    times, masses, ids = [], [], []
    for t0 in range(0, 400, 40):
        tr.advance(float(t0), float(t0 + 40))
        rec = tr.observe_sinks()
        times.append(rec["time"])
        masses.append(rec["mass"])
        ids.append(rec["id"])
    tr.close()
    t = np.concatenate(times)
    m = np.concatenate(masses)
    ids = np.concatenate(ids)
    assert t.shape[0] > 500 and np.unique(ids).shape[0] == ids.shape[0]
    q = 3.0
    w = m / abs(q)
    groups = np.ones(t.shape[0], np.int32)
    opt_o = BT.ObservationOptions(histogram_bin_format=1)
    gb = BT.sink_btc(t, w, groups, [[1]], opt_o, stoptime=400.0, flow_constant=q)
    ob = BT.sink_btc(t, w, groups, [[1]], opt_o, stoptime=400.0, flow_constant=q, series=oracle_series)
    b = gb["raw"][0]["bin_size"]
    binned = w[np.floor(t / b) + 1 <= gb["raw"][0]["n_bins"]].sum()
    np.testing.assert_allclose(gb["hist"][0].sum() * b, binned, rtol=1e-12)
    np.testing.assert_allclose(gb["gpkde"][0].sum() * b, binned, rtol=1e-9)
    close(gb["gpkde"][0], ob["gpkde"][0], 1e-10)
    assert gb["raw"][0]["loops"] == ob["raw"][0]["loops"]
