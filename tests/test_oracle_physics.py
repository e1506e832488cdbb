"""The oracle against known answers (CPU).

* cell records of uniform flow in closed form (ModpathCellData.f90:2557-2564,
  TrackSubCell.F90:2557-2691, 4016-4138);
* pure advection is exact: a particle moves v*t and sits on cell faces
  exactly (ConvertFromNeighbor, RectangularGridDisMf6.f90:50-108);
* the uniform-column pulse against the analytic 1-D Gaussian ADE solution,
  with the tolerance the reference's interface-forcing scheme needs;
* release / status logic of the driver (MPathRW.F90:1256-1302);
* counter-based streams make results independent of the thread count.
"""
import numpy as np
import pytest

from mprw import workloads as W
from mprw.model import ACTIVE, INACTIVE, PENDING, UNRELEASED, WEAK_SINK, Particles
from oracle import oracle as O


def test_uniform_flow_cell_record():
    g, f, p, opt = W.uniform_pulse(n_particles=1)
    r = O.cell_record(g, f, opt, 50)
    np.testing.assert_allclose(r["vface"], [1, 1, 0, 0, 0, 0], rtol=0, atol=1e-15)
    assert r["dtcell"] == pytest.approx(0.1, rel=1e-15)
    np.testing.assert_allclose(r["qcorner"], np.tile([0.3, 0.0, 0.0, 0.3], (8, 1)), rtol=1e-15, atol=0)
    np.testing.assert_allclose(r["phicorner"], 0.3)
    D = r["D"]
    np.testing.assert_allclose(D[0], 0.01 * 0.3 + 0.09 * 0.3, rtol=1e-14)  # Dxx
    np.testing.assert_allclose(D[1], 0.01 * 0.3, rtol=1e-14)               # Dyy
    np.testing.assert_allclose(D[2], 0.01 * 0.3, rtol=1e-14)               # Dzz
    assert np.all(D[3:] == 0.0)
    # interior x faces connect, y/z faces are domain edges (defaultICBound = 1 reflects)
    assert list(r["conn"]) == [49, 51, 0, 0, 0, 0]
    assert list(r["massb"]) == [0, 0, 1, 1, 1, 1]


def test_pure_advection_exact():
    g, f, p, opt = W.uniform_pulse(n_particles=3, pure_advection=True)
    p.lx[:] = [0.0, 0.25, 0.5]
    q, steps = O.advance(g, f, opt, p, 0.0, 25.0)
    gx, gy, gz = O.global_xyz(g, f, q)
    np.testing.assert_allclose(gx, np.array([10.0, 10.25, 10.5]) + 25.0, rtol=0, atol=1e-9)
    assert np.all(q.t == 25.0) and np.all(q.status == ACTIVE)
    np.testing.assert_allclose(gy, 0.5)
    # one pass per 0.1 d plus one face-truncated pass per crossed face
    assert steps >= 3 * 250


def test_analytic_gaussian_uniform_pulse():
    """The oracle on the reference's RNG path (xoroshiro128+ thread streams,
    8 threads, 20,000 particles) against its 1,000,000-particle single-thread
    run (tests/golden/mc_uniform_pulse.npz): two samples of one process, within
    Monte-Carlo bounds (tests/mc_stats.py) at 25 and 50 days.  Against the
    analytic Gaussian the scheme is biased: the mean lags by 0.10 m at
    50 days and the variance is 4.3 % low, and both stand out against the
    large run's standard errors."""
    import math
    from pathlib import Path

    import mc_stats as S
    fx = np.load(Path(__file__).resolve().parent / "golden" / "mc_uniform_pulse.npz")
    n = 20000
    g, f, p, opt = W.uniform_pulse(n_particles=n)
    O.reset_xoroshiro()
    q = p
    for k, (a, b) in enumerate([(0.0, 25.0), (25.0, 50.0)]):
        q, _ = O.advance(g, f, opt, q, a, b, rng_kind=O.RNG_XOROSHIRO, nthreads=8)
        gx, gy, gz = O.global_xyz(g, f, q)
        assert np.all(q.status == ACTIVE)
        got = S.summarize(q.status, gx, gy, gz, q.t, np.arange(201, dtype=np.float64))
        bad = S.compare(got, S.from_npz(fx, f"t{k}_"), f"interval {k}")
        assert not bad, bad
    m, v, big = float(fx["t1_mean_x"]), float(fx["t1_var_x"]), int(fx["t1_n"])
    mean, var = 10.0 + 50.0, 2.0 * 0.1 * 1.0 * 50.0
    assert -0.15 < m - mean < -0.05 and (mean - m) > 20 * math.sqrt(v / big)
    assert -0.06 < (v - var) / var < -0.03


def test_release_and_status_logic():
    g, f, p, opt = W.uniform_pulse(n_particles=4, pure_advection=True)
    p.t[:] = [0.0, 5.0, 50.0, -1.0]      # released now, later in interval, after, before interval
    p.status[:] = PENDING
    q, _ = O.advance(g, f, opt, p, 0.0, 10.0)
    assert list(q.status) == [ACTIVE, ACTIVE, PENDING, UNRELEASED]
    gx, _, _ = O.global_xyz(g, f, q)
    assert gx[0] == pytest.approx(20.0, abs=1e-9) and gx[1] == pytest.approx(15.0, abs=1e-9)
    # inactive release cell
    f.iboundts = f.iboundts.copy()
    f.iboundts[10] = 0
    q, _ = O.advance(g, f, opt, p, 0.0, 10.0)
    assert q.status[0] == INACTIVE


def test_empty_particle_set():
    g, f, p, opt = W.uniform_pulse(n_particles=0)
    q, steps = O.advance(g, f, opt, p, 0.0, 10.0)
    assert q.n == 0 and steps == 0


def test_thread_count_invariance_with_counter_based_rng():
    g, f, p, opt, _ = W.lognormal_slab(n_particles=400, nlay=3, nrow=8, ncol=20, seed=2, use_torch=False)
    a, sa = O.advance(g, f, opt, p, 0.0, 30.0, rng_kind=O.RNG_PHILOX, nthreads=1)
    b, sb = O.advance(g, f, opt, p, 0.0, 30.0, rng_kind=O.RNG_PHILOX, nthreads=8)
    assert sa == sb
    for x, y in ((a.cell, b.cell), (a.lx, b.lx), (a.ly, b.ly), (a.lz, b.lz), (a.t, b.t), (a.status, b.status),
                 (a.rng_ctr, b.rng_ctr)):
        np.testing.assert_array_equal(x, y)


def test_heterogeneous_weak_sink_stops():
    g, f, p, opt, info = W.lognormal_slab(n_particles=600, nlay=3, nrow=8, ncol=20, seed=1, use_torch=False)
    q, _ = O.advance(g, f, opt, p, 0.0, 200.0, rng_kind=O.RNG_PHILOX, nthreads=8)
    counts = np.bincount(q.status, minlength=10)
    assert counts[WEAK_SINK] > 0
    assert counts.sum() == p.n
    # particles that stopped at the outlet sit in the last column
    col = (q.cell[q.status == WEAK_SINK] - 1) % g.ncol
    assert np.all(col == g.ncol - 1)


def test_exponential_advection_exact_in_linear_field():
    """EXPONENTIAL advection (TrackSubCell.F90:1487-1538) with the Newton exit
    time (:1895-2554) follows the exact path of a cell-wise linear velocity
    field; EULERIAN advection does not."""
    from mprw.model import EULERIAN, EXPONENTIAL, Options
    g, f, Q = W.graded_flow(ncol=40, q0=0.3, ratio=1.05)
    n = 5
    x0 = np.array([0.0, 0.2, 0.45, 0.7, 0.95])
    p = Particles(cell=np.ones(n, np.int32), lx=x0.copy(), ly=np.full(n, 0.5), lz=np.full(n, 0.5), t=np.zeros(n),
                  status=np.full(n, ACTIVE, np.int32), mass=np.ones(n), id=np.arange(n, dtype=np.uint64),
                  rng_ctr=np.zeros(n, np.uint64))
    exact = np.array([W.graded_flow_exact(a, 15.0, Q) for a in x0])
    err = {}
    for kind in (EXPONENTIAL, EULERIAN):
        opt = Options(time_step_kind=1, ts_param=(0.1, 0.1), advection_kind=kind, dim_mask=(1, 1, 1))
        q, _ = O.advance(g, f, opt, p, 0.0, 15.0)
        gx, _, _ = O.global_xyz(g, f, q)
        assert np.all(q.status == ACTIVE)
        err[kind] = np.abs(gx - exact).max()
    # exact up to rounding: Newton's exit times converge far inside their
    # relative 1e-6 tolerance here (NewtonRaphsonTimeStep..., :2451-2554)
    assert err[EXPONENTIAL] < 1e-9
    assert err[EULERIAN] > 1e-2


def test_axisymmetric_dispersion_uniform_flow():
    """Linear axisymmetric dispersion (pr_CornerDispersionAxisymmetric,
    TrackSubCell.F90:3117-3303; displacements :750-806, :3306-3604) in uniform
    flow along x: the plume spreads with alphaLH along x, alphaTH across in y
    and alphaTV across in z (the isotropic model uses alphaT for both)."""
    from mprw.model import ADV, Options
    g, f = W.uniform_flow(ncol=60, nrow=21, nlay=21, q=0.3, porosity=0.3, alpha_l=0.1, alpha_t=0.02, dm=0.0)
    f.alpha_lv = np.array([0.05])
    f.alpha_tv = np.array([0.004])
    n, t = 12000, 20.0
    node = g.node(10, 10, 10)
    p = Particles(cell=np.full(n, node, np.int32), lx=np.zeros(n), ly=np.full(n, 0.5), lz=np.full(n, 0.5),
                  t=np.zeros(n), status=np.full(n, ACTIVE, np.int32), mass=np.ones(n),
                  id=np.arange(n, dtype=np.uint64), rng_ctr=np.zeros(n, np.uint64))
    k = {}
    for model in (0, 1):
        opt = Options(time_step_kind=ADV, ts_param=(0.1, 0.1), dispersion_model=model)
        q, _ = O.advance(g, f, opt, p, 0.0, t, rng_kind=O.RNG_PHILOX, nthreads=8)
        assert np.all(q.status == ACTIVE)
        gx, gy, gz = O.global_xyz(g, f, q)
        k[model] = (gx.var() / (2 * t), gy.var() / (2 * t), gz.var() / (2 * t))
    # longitudinal: alphaLH (the interface-forcing scheme biases it low by < 12 %)
    assert abs(k[1][0] - 0.1) < 0.012 and abs(k[0][0] - 0.1) < 0.012
    assert abs(k[1][1] - 0.02) < 0.02 * 0.06        # alphaTH
    assert abs(k[1][2] - 0.004) < 0.004 * 0.06      # alphaTV
    assert abs(k[0][2] - 0.02) < 0.02 * 0.06        # isotropic: alphaT
