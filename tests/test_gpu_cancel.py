"""Cancellation of an advance (mprw_set_timeout / mprw_cancel): the failure is
made on the host (a timeout that runs out, a cancel from another thread); the
kernel reads the flag, returns, and the library reports MPRW_E_ABORTED with
every particle at a valid location; the handle keeps working."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from mprw import workloads as W
from mprw.model import ACTIVE


def _tracker(n=200000):
    g, f, p, opt, info = W.lognormal_slab(n_particles=n, nlay=4, nrow=12, ncol=30, seed=0, use_torch=False)
    opt.stop_weak_sinks = False   # nothing stops: the advance runs to its end time
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    return g, tr, p


def _valid(out, g, t_hi):
    assert np.isfinite(out["lx"]).all() and np.isfinite(out["t"]).all()
    for k in ("lx", "ly", "lz"):
        assert (out[k] >= 0).all() and (out[k] <= 1).all()
    assert (out["cell"] >= 1).all() and (out["cell"] <= g.ncell).all()
    assert (out["t"] >= 0).all() and (out["t"] <= t_hi).all()


# An advance to T_LONG takes ~1e10 particle-steps (seconds of GPU time) when
# nothing stops it, so a cancel that failed would fail these tests, not hang.
T_LONG = 2.0e4


def test_timeout_stops_a_long_advance(gpu_lib):
    g, tr, p = _tracker()
    tr.set_timeout(20.0)
    t0 = time.perf_counter()
    with pytest.raises(mprw.MprwAborted, match="timeout"):
        tr.advance(0.0, T_LONG)
    assert time.perf_counter() - t0 < 1.0
    out = tr.get_particles()
    _valid(out, g, T_LONG)
    st = out["status"]
    # tracked particles are ACTIVE mid-path or stopped by the reference's rules
    # (5: a cell without exit); those the queue had not reached are unchanged
    assert np.isin(st, [0, 1, 2, 3, 4, 5, 7]).all()
    assert (st == ACTIVE).any() and (out["t"][st == ACTIVE] > 0).all()
    np.testing.assert_array_equal(out["t"][st == 0], p.t[st == 0])
    assert (out["t"] < T_LONG).all()                     # nothing reached the end time
    # the handle keeps working: a short advance after the cancelled one
    tr.set_timeout(0.0)
    t_now = float(out["t"].max())
    assert tr.advance(t_now, t_now + 1.0) > 0
    _valid(tr.get_particles(), g, t_now + 1.0)
    tr.close()


def test_cancel_from_another_thread(gpu_lib):
    g, tr, p = _tracker()
    err = []

    def run():
        try:
            tr.advance(0.0, T_LONG)
        except mprw.MprwAborted as e:
            err.append(e)

    th = threading.Thread(target=run)
    th.start()
    time.sleep(0.005)     # the cancel stops the running advance, or the one about to start
    tr.cancel()
    th.join(timeout=60.0)
    assert not th.is_alive() and len(err) == 1
    out = tr.get_particles()
    _valid(out, g, T_LONG)
    assert (out["t"] < T_LONG).all()
    tr.close()
