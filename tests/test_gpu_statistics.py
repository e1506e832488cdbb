"""The GPU against the reference's own random-walk statistics.

Every other parity test runs the oracle on the GPU's counter-based Philox
stream, so that trajectories can be compared one by one.  Here the oracle
runs as the reference does -- xoroshiro128+ streams seeded once per run,
Irwin-Hall(12) normals, one thread (rng_par_zig.f90:156-335,
TrackSubCell.F90:553-555, 613-620, 3631-3663) -- and its plume summaries are
stored fixtures (tests/golden/make_mc_golden.py; the oracle runs 1e6 and
2e5 particles there, too long for a test).  The GPU tracks an independent
sample with its own Philox stream, FP64 and MIXED, and the two are compared
as samples of one random-walk process (tests/mc_stats.py): every stop-status
fraction and the particles past the control plane by a two-proportion z
test, the mean and variance of each coordinate of the ACTIVE particles by z
tests with standard errors from the samples' own second and fourth moments,
the x histogram and the outlet breakthrough histogram by two-sample
chi-square tests, at |z| <= 4.5 and p >= 1e-5.

* uniform-column pulse (config 1's setting), 1,000,000 GPU particles
  against the oracle's 1,000,000, at 25, 50 and 100 days;
* the small lognormal field with weak-sink stops at the outlet (the
  lognormal-slab generator at 30x12x4 cells), 1,000,000 GPU particles
  against the oracle's 200,000, at 10, 20, 30, 45 and 60 days: status
  counts (the mass leaving through the outlet), moments, the control plane
  x = 20 m and the outlet breakthrough curve.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

import mc_stats as S  # noqa: E402
import make_mc_golden as MG  # noqa: E402
import mprw  # noqa: E402
from mprw import workloads as W  # noqa: E402
from mprw.model import FP64, MIXED  # noqa: E402


def _track(g, f, opt, p, intervals, summ, precision):
    opt.precision = precision
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    out = []
    try:
        for a, b in intervals:
            tr.advance(a, b)
            q = tr.get_particles()
            out.append(summ(q["status"], q["gx"], q["gy"], q["gz"], q["t"]))
    finally:
        tr.close()
    return out


def _check(got, fixture, label):
    bad = []
    for k, s in enumerate(got):
        bad += S.compare(s, S.from_npz(fixture, f"t{k}_"), f"{label} interval {k}")
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("precision", [FP64, MIXED], ids=["fp64", "mixed"])
def test_uniform_pulse_matches_reference_rng_statistics(gpu_lib, precision):
    fx = np.load(HERE / "golden" / "mc_uniform_pulse.npz")
    g, f, p, opt = W.uniform_pulse(n_particles=1_000_000)
    got = _track(g, f, opt, p, MG.PULSE_INTERVALS,
                 lambda st, x, y, z, t: S.summarize(st, x, y, z, t, MG.PULSE_X_EDGES), precision)
    _check(got, fx, "uniform pulse")
    # every particle stays in the column over 100 days
    assert all(int(s["status_counts"][1]) == 1_000_000 for s in got)


@pytest.mark.parametrize("precision", [FP64, MIXED], ids=["fp64", "mixed"])
def test_lognormal_field_matches_reference_rng_statistics(gpu_lib, precision):
    fx = np.load(HERE / "golden" / "mc_hetero_small.npz")
    g, f, opt, p = MG.hetero_case(1_000_000, seed=9001)   # a release independent of the oracle's
    got = _track(g, f, opt, p, MG.HETERO_INTERVALS,
                 lambda st, x, y, z, t: S.summarize(st, x, y, z, t, MG.HETERO_X_EDGES, MG.HETERO_PLANE,
                                                    MG.HETERO_T_EDGES), precision)
    _check(got, fx, "lognormal field")
    # the case exercises the weak-sink stops: most of the mass leaves by 60 days
    last = got[-1]
    assert last["status_counts"][3] > 0.5 * 1_000_000
    assert last["past_plane"] > 0.5 * 1_000_000
