"""Breakthrough-curve assembly of observations (mprw.btc, host logic) on
CPU, with the oracle's 1-D GPKDE injected as the reconstruction:
interpolation (finterp's linear_interp_1d), sink-flow knots, resident
concentrations, the sink series layouts (per solute / common grid /
interpolated) and the output records (MPathRW.F90:1759-2840)."""
import io

import numpy as np
import pytest

from mprw import btc as BT
from oracle import series_oracle as SO


def oracle_series(t, w, **kw):
    return SO.gpkde_series(t, w, **kw)


def test_linear_interp_inside_outside_and_on_knots():
    xk = np.array([0.0, 1.0, 3.0, 4.0])
    fk = np.array([0.0, 2.0, 6.0, 5.0])
    x = np.array([-1.0, 0.0, 0.5, 1.0, 2.0, 3.0, 3.5, 4.0, 6.0])
    got = BT.linear_interp(xk, fk, x)
    # before the start / after the end: the first / last interval extrapolated
    np.testing.assert_array_equal(got, [-2.0, 0.0, 1.0, 2.0, 4.0, 6.0, 5.5, 5.0, 3.0])
    with pytest.raises(ValueError):
        BT.linear_interp([0.0, 0.0], [1.0, 2.0], [0.5])
    with pytest.raises(ValueError):
        BT.linear_interp([0.0], [1.0], [0.5])


def test_sink_flow_knots_forward_backward():
    tt = np.array([10.0, 20.0, 30.0, 40.0])
    q = np.array([1.0, 2.0, 3.0])
    assert BT.sink_flow_knots(tt, q[:1], 0.0, 2, 2) is None
    x, f = BT.sink_flow_knots(tt, q, 5.0, 2, 4)
    np.testing.assert_array_equal(x, [0.0, 15.0, 25.0, 35.0])
    np.testing.assert_array_equal(f, [1.0, 1.0, 2.0, 3.0])
    x, f = BT.sink_flow_knots(tt, q, 45.0, 4, 2, backward=True)
    np.testing.assert_array_equal(x, [5.0, 15.0, 25.0, 35.0])
    np.testing.assert_array_equal(f, [1.0, 2.0, 3.0, 3.0])


def resident_records(seed=0, n=4000, n_tp=50):
    rng = np.random.default_rng(seed)
    tp = np.arange(1, n_tp + 1) * 4.0
    k = np.clip(np.round(rng.normal(20, 6, n)).astype(int), 0, n_tp - 1)
    t = tp[k]
    groups = rng.integers(1, 4, n)
    w = rng.uniform(0.5, 1.0, n)
    vw = rng.uniform(10.0, 20.0, (n_tp, 3))
    vw[:3] = 0.0       # the cells were dry at the start
    return t, w, groups, tp, vw


@pytest.mark.parametrize("post", [0, 1])
def test_resident_concentrations(post):
    t, w, groups, tp, vw = resident_records()
    opt = BT.ObservationOptions(postprocess=post)
    out = BT.resident_btc(t, w, groups, [[1, 2], [3], []], tp, vw, opt, series=oracle_series)
    v = vw.sum(axis=1)
    # solute 1 = groups 1 and 2, reconstructed directly
    rows = np.isin(groups, [1, 2])
    kw = dict(domain_size=tp[-1], bin_size=4.0, bin_format=2, exact_point=True, init_selection=0, init_factor=3.0,
              apply_init_factor=True, n_opt_loops=10)
    if post == 0:
        r = SO.gpkde_series(t[rows], w[rows], only_histogram=True, **kw)
    else:
        r = SO.gpkde_series(t[rows], w[rows], unit_volume=True, rel_err=0.01, **kw)
    pos = v > 0
    np.testing.assert_array_equal(out["hist"][pos, 0], r["counts"][pos] / v[pos])
    assert np.all(out["hist"][~pos] == 0.0) and np.all(out["water_volume"][~pos] == 0.0)
    assert np.all(out["hist"][:, 2] == 0.0)                 # a solute without groups
    assert out["raw"][2] is None
    if post == 1:
        np.testing.assert_array_equal(out["gpkde"][pos, 0], r["density"][pos] / v[pos])
    else:
        assert "gpkde" not in out
    # the histogram holds the solute's mass (weights on the time points)
    np.testing.assert_allclose((out["hist"][:, 0] * v).sum(), w[rows & (t <= tp[-1])].sum()
                               - w[rows & np.isin(t, tp[~pos])].sum(), rtol=1e-12)
    buf = io.StringIO()
    assert BT.write_resident(buf, out) == tp.shape[0]
    lines = buf.getvalue().splitlines()
    width = 8 + 18 * (2 + 3 * (2 if post == 1 else 1))
    assert all(len(ln) == width for ln in lines)
    assert float(lines[0][8:26]) == 4.0 and float(lines[0][26:44]) == 0.0


def test_resident_grid_must_match_time_points():
    t, w, groups, tp, vw = resident_records(n_tp=40)
    tp2 = tp.copy()
    tp2[-1] = 400.0          # irregular time points: 100 bins for 40 records
    with pytest.raises(ValueError):
        BT.resident_btc(t, w, groups, [[1, 2, 3]], tp2, vw, BT.ObservationOptions(), series=oracle_series)


def sink_records(seed=1, n=6000):
    rng = np.random.default_rng(seed)
    t = rng.lognormal(np.log(60.0), 0.3, n)
    groups = rng.integers(1, 3, n)
    w = np.full(n, 0.01) / 2.5       # mass / |Q|
    return t, w, groups


def test_sink_per_solute_fd_bins():
    t, w, groups = sink_records()
    opt = BT.ObservationOptions(histogram_bin_format=1)
    out = BT.sink_btc(t, w, groups, [[1], [2]], opt, stoptime=300.0, flow_constant=2.5, series=oracle_series)
    assert out["per_solute"]
    for s, g in enumerate((1, 2)):
        rows = groups == g
        r = SO.gpkde_series(t[rows], w[rows], domain_size=300.0, bin_format=1, bin_size_fraction=0.75,
                            init_factor=3.0, apply_init_factor=False, raw_density=True, rel_err=0.01)
        np.testing.assert_array_equal(out["time"][s], r["coordinates"])
        np.testing.assert_array_equal(out["hist"][s], r["counts"])
        np.testing.assert_array_equal(out["gpkde"][s], r["density"])
        assert np.all(out["flow"][s] == 2.5)
        # flux concentration integrates to mass / Q
        b = r["bin_size"]
        np.testing.assert_allclose(out["hist"][s].sum() * b, w[rows].sum(), rtol=1e-12)
        np.testing.assert_allclose(out["gpkde"][s].sum() * b, w[rows].sum(), rtol=1e-9)
    buf = io.StringIO()
    nrows = BT.write_sink(buf, out, solute_ids=[7, 9])
    lines = buf.getvalue().splitlines()
    assert nrows == len(lines) == sum(x.shape[0] for x in out["time"])
    assert lines[0][:8] == "       7" and all(len(ln) == 16 + 18 * 4 for ln in lines)


def test_sink_common_grid_time_points_and_flow():
    t, w, groups = sink_records(2)
    tp = np.arange(1, 151) * 2.0
    opt = BT.ObservationOptions(histogram_bin_format=3, postprocess=1)
    knots = (np.array([0.0, 100.0, 300.0]), np.array([2.0, 2.0, 4.0]))
    out = BT.sink_btc(t, w, groups, [[1], [2]], opt, stoptime=300.0, time_points=tp, flow_knots=knots,
                      series=oracle_series)
    assert not out["per_solute"]
    assert out["hist"].shape == (150, 2)
    np.testing.assert_array_equal(out["time"], (np.arange(1, 151) - 0.5) * 2.0)
    np.testing.assert_allclose(out["flow"], BT.linear_interp(*knots, out["time"]))
    rows = groups == 1
    r = SO.gpkde_series(t[rows], w[rows], domain_size=300.0, bin_size=2.0, bin_format=3, init_factor=3.0,
                        apply_init_factor=True, raw_density=True, rel_err=0.01)
    np.testing.assert_array_equal(out["hist"][:, 0], r["counts"])
    np.testing.assert_array_equal(out["gpkde"][:, 0], r["density"])
    buf = io.StringIO()
    assert BT.write_sink(buf, out) == 150
    assert all(len(ln) == 8 + 18 * 6 for ln in buf.getvalue().splitlines())


def test_sink_interpolated_fixed_and_adapted():
    t, w, groups = sink_records(3)
    opt = BT.ObservationOptions(histogram_bin_format=2, histogram_bin=1.0, time_step_out=5.0)
    out = BT.sink_btc(t, w, groups, [[1, 2]], opt, stoptime=298.0, flow_constant=1.0, series=oracle_series)
    assert not out["per_solute"]
    ts = out["time"]
    assert ts.shape[0] == 60 and ts[0] == 5.0 and ts[-1] == 298.0
    r = out["raw"][0]
    keep = ts >= r["coordinates"][0]
    np.testing.assert_allclose(out["hist"][keep, 0], BT.linear_interp(r["coordinates"], r["counts"], ts[keep]))
    buf = io.StringIO()
    n = BT.write_sink(buf, out, skip_before=r["coordinates"])
    assert n == int(np.sum((ts >= r["coordinates"][0]) & (ts <= r["coordinates"][-1])))
    # steady state to the end: the grid adapts per solute, then interpolates
    out = BT.sink_btc(t, w, groups, [[1], [2]], opt, stoptime=1e30, adapt_grid=True, flow_constant=1.0,
                      series=oracle_series)
    assert out["per_solute"]
    for s in range(2):
        r = out["raw"][s]
        assert r["delta_bins_origin"] > 0
        ts = out["time"][s]
        assert ts[0] == 5.0 and ts.shape[0] == int(r["coordinates"].max() / 5.0)
