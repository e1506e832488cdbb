"""MIXED precision where the jump limiter and the exit loop work hardest.

The uniform pulse seldom cuts a step (its displacements stay far below half
a cell), so these cases force the paths the MIXED kernel handles differently
from FP64: the jump limiter (TrackSubCell.F90:989-1013; MIXED cuts the FP32
step copy and corrects the FP64 time once after its loop) and the exit loop
that takes back the time of a truncated step (TrackSubCell.F90:1025-1316).
On the small heterogeneous field, a FIXED time step of one day with
alphaL = 1 m makes most steps jump more than half a cell; a second case uses
the lognormal field's own MIN_ADV_DISP step with a tenfold dispersivity.
MIXED and FP64 draw the same normals, so their plumes differ by rounding
and by the few particles whose FP32 comparisons go the other way:

* every particle's time stays within the interval (t <= t_end, and ACTIVE
  particles end exactly at t_end);
* the stop-status counts agree within max(3, 0.5 %) of the particles;
* plume mean displacement within 0.5 % and variances within 1 %
  relative (the mixed-precision target's moment tolerance is 0.5 % on
  the mean);
* the limiter really cut: FP64 steps per particle at least 4x the 25 an
  uncut one-day FIXED step gives over 25 days (the oracle takes ~360).
"""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from golden_cases import hetero_flow
from mprw import workloads as W
from mprw.model import ACTIVE, EULERIAN, MIN_ADV_DISP, MIXED, Options


def _run(g, f, opt, p, iv, precision):
    o = copy.copy(opt)
    o.precision = precision
    tr = mprw.Tracker(g, o)
    tr.load_flow(f)
    tr.set_particles(p)
    steps = sum(tr.advance(a, b) for a, b in iv)
    out = tr.get_particles()
    tr.close()
    return out, steps


def _moments(out):
    act = out["status"] == ACTIVE
    return {k: (float(out[k][act].mean()), float(out[k][act].var())) for k in ("gx", "gy", "gz")}


def _compare(g, f, opt, p, iv, x0):
    o64, s64 = _run(g, f, opt, p, iv, 0)
    o32, s32 = _run(g, f, opt, p, iv, MIXED)
    t_end = iv[-1][1]
    for out in (o64, o32):
        assert np.all(out["t"] <= t_end)
        act = out["status"] == ACTIVE
        assert act.sum() > 0.3 * p.n
        assert np.all(out["t"][act] == t_end)
    for st in range(10):
        a, b = int((o64["status"] == st).sum()), int((o32["status"] == st).sum())
        assert abs(a - b) <= max(3, 0.005 * p.n), (st, a, b)
    m64, m32 = _moments(o64), _moments(o32)
    disp = m64["gx"][0] - x0
    assert abs(m32["gx"][0] - m64["gx"][0]) <= 5e-3 * abs(disp), (m32["gx"], m64["gx"])
    for k in ("gx", "gy", "gz"):
        assert abs(m32[k][1] - m64[k][1]) <= 1e-2 * m64[k][1], (k, m32[k], m64[k])
    return s64, s32


def test_mixed_fixed_step_with_limiter_cuts(gpu_lib):
    g, f = hetero_flow()
    f = copy.copy(f)
    f.uniform_dispersion = True
    f.alpha_l = np.array([1.0])
    f.alpha_t = np.array([0.1])
    f.dm_eff = np.array([1e-4])
    dt = 1.0
    opt = Options(time_step_kind=4, ts_param=(dt, 0.0), advection_kind=EULERIAN, stop_weak_sinks=True)
    p = W.release_in_box(g, 4000, 0.0, 6.0, 0.0, 12.0, 0.0, 4.0, seed=31)
    iv = [(0.0, 10.0), (10.0, 25.0)]
    s64, _ = _compare(g, f, opt, p, iv, 3.0)
    # without cuts a particle takes 25 / dt steps plus one face-truncated step per cell crossed
    assert s64 > 4 * (25.0 / dt) * p.n


def test_mixed_high_dispersivity_lognormal(gpu_lib):
    g, f = hetero_flow()
    f = copy.copy(f)
    f.uniform_dispersion = True
    f.alpha_l = np.array([5.0])
    f.alpha_t = np.array([0.5])
    f.dm_eff = np.array([1e-4])
    opt = Options(time_step_kind=MIN_ADV_DISP, ts_param=(0.5, 0.5), advection_kind=EULERIAN, stop_weak_sinks=True)
    # Under this many cuts a MIXED particle whose FP32 comparison goes the other
    # way once draws later normals at other counters and decorrelates from its
    # FP64 twin; 1e6 particles keep the sampling noise of the variance
    # difference near 0.2 %, well inside the tolerance.
    p = W.release_in_box(g, 1_000_000, 0.0, 6.0, 0.0, 12.0, 0.0, 4.0, seed=37)
    _compare(g, f, opt, p, [(0.0, 20.0)], 3.0)
