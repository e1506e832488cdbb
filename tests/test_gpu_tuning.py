"""Launch tuning (mprw_set_tuning / mprw_autotune): the autotuner leaves the
particles as it found them, and no tuning changes any particle's result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from mprw import workloads as W
from mprw.model import FP64, MIXED


def _state(tr):
    o = tr.get_particles()
    return {k: o[k] for k in ("cell", "status", "lx", "ly", "lz", "t", "rng_ctr")}


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_autotune_is_invisible_to_results(gpu_lib, precision):
    g, f, p, opt, info = W.lognormal_slab(n_particles=20000, nlay=4, nrow=12, ncol=30, seed=5, precision=precision,
                                   use_torch=False)
    ref = mprw.Tracker(g, opt)
    ref.load_flow(f)
    ref.set_particles(p)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    before = _state(tr)
    tun = tr.autotune(0.0, 5.0)
    after = _state(tr)
    for k in before:
        np.testing.assert_array_equal(before[k], after[k], err_msg=k)
    t = tr.tuning()
    assert t["blocks_per_sm"] == tun["blocks_per_sm"] and t["sort_interval"] == tun["sort_interval"]
    assert 1 <= t["blocks_per_sm"] <= t["max_blocks_per_sm"]
    assert all(r > 0 for r in tun["trial_rates_per_ms"][: min(t["max_blocks_per_sm"], 4) + 1])
    for t0, t1 in ((0.0, 10.0), (10.0, 20.0), (20.0, 30.0)):
        assert tr.advance(t0, t1) == ref.advance(t0, t1)
    a, b = _state(tr), _state(ref)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    # every manual setting gives the same particles too
    for bps, si in ((1, 0), (t["max_blocks_per_sm"], 3)):
        tr.set_particles(p)
        tr.set_tuning(bps, si)
        for t0, t1 in ((0.0, 10.0), (10.0, 20.0), (20.0, 30.0)):
            tr.advance(t0, t1)
        c = _state(tr)
        for k in c:
            np.testing.assert_array_equal(c[k], b[k], err_msg=f"{bps},{si}: {k}")
    with pytest.raises(mprw.MprwError):
        tr.set_tuning(t["max_blocks_per_sm"] + 1, 1)
    with pytest.raises(mprw.MprwError):
        tr.set_tuning(1, -1)
    tr.close()
    ref.close()


def test_autotune_on_a_batch(gpu_lib):
    g, f, p, opt, info = W.lognormal_slab(n_particles=5000, nlay=3, nrow=8, ncol=20, seed=6, use_torch=False)
    u, fu = W.uniform_flow(ncol=40, q=0.3)
    pu = W.release_in_box(u, 3000, 2.0, 3.0, 0.0, 1.0, 0.0, 1.0, seed=2)
    b = mprw.Batch([g, u], opt)
    b.load_flow(0, f)
    b.load_flow(1, fu)
    b.set_particles([p, pu])
    before = b.get_particles()
    b.autotune(0.0, 5.0)
    after = b.get_particles()
    for x, y in zip(before, after):
        for k in ("cell", "lx", "t", "rng_ctr"):
            np.testing.assert_array_equal(x[k], y[k])
    with pytest.raises(mprw.MprwError):
        b.member(0).autotune(0.0, 5.0)
    assert b.advance(0.0, 10.0) > 0
    b.close()
