"""The 1-D GPKDE of observation time series on the GPU (mprw_gpkde_series)
against the numpy restatement (oracle/series_oracle.py): bin sizes, grids,
histograms, loop counts and densities for the options the observation
post-process passes (MPathRW.F90:1773-2840), and its edge cases.

Tolerances: the histogram sums weights with atomics and the kernels use the
device's erf/exp/pow, so values agree to rounding (counts 1e-12 relative to
their maximum, densities 1e-10); grid sizes, bin offsets and loop counts are
exact.  Bin sizes from Scott's rule rest on sums taken in another order
(1e-13); Freedman-Diaconis picks order statistics, so its bin size is exact.
"""
import numpy as np
import pytest

import mprw
from oracle import series_oracle as SO

pytestmark = pytest.mark.gpu


def arrivals(n, seed, mu=40.0, s=0.3):
    rng = np.random.default_rng(seed)
    t = rng.lognormal(np.log(mu), s, n)
    w = rng.uniform(0.5, 1.5, n)
    return t, w


def check(t, w, **kw):
    ref = SO.gpkde_series(t, w, **kw)
    got = mprw.gpkde_series(t, w, **kw)
    assert got["n_bins"] == ref["n_bins"]
    assert got["delta_bins_origin"] == ref["delta_bins_origin"]
    rtol_b = 1e-13 if kw.get("bin_format", 2) == 0 else 0.0
    np.testing.assert_allclose(got["bin_size"], ref["bin_size"], rtol=rtol_b, atol=0)
    np.testing.assert_allclose(got["grid_origin"], ref["grid_origin"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(got["coordinates"], ref["coordinates"], rtol=1e-13, atol=1e-12)
    c = ref["counts"]
    np.testing.assert_allclose(got["counts"], c, rtol=0, atol=1e-12 * max(np.abs(c).max(), 1e-300))
    if ref["wcounts"] is not None:
        wc = ref["wcounts"]
        np.testing.assert_allclose(got["wcounts"], wc, rtol=0, atol=1e-12 * max(np.abs(wc).max(), 1e-300))
    if ref["density"] is None:
        assert got["density"] is None
    else:
        assert got["loops"] == ref["loops"]
        d = ref["density"]
        np.testing.assert_allclose(got["density"], d, rtol=0, atol=1e-10 * max(np.abs(d).max(), 1e-300))
    return got, ref


@pytest.mark.parametrize("eff_format", [0, 1, 2, 3])
def test_weight_formats_fixed_bins(eff_format):
    t, w = arrivals(4000, 1)
    check(t, w, domain_size=120.0, bin_size=1.0, bin_format=2, eff_format=eff_format, raw_density=True,
          init_factor=3.0, apply_init_factor=True, rel_err=0.01)


@pytest.mark.parametrize("bin_format,frac", [(0, 1.0), (1, 0.75), (1, 2.0), (0, 0.5)])
def test_automatic_bin_sizes(bin_format, frac):
    t, w = arrivals(2501, 2, mu=60.0, s=0.4)
    got, ref = check(t, w, domain_size=200.0, bin_format=bin_format, bin_size_fraction=frac, raw_density=True,
                     rel_err=0.01)
    assert ref["loops"] >= 1


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6, 7, 8, 9, 1000, 1001, 1002, 1003])
def test_fd_quartile_parities(n):
    """Every branch of the Freedman-Diaconis quartile picks (n even/odd, half
    even/odd)."""
    t, w = arrivals(n, 30 + n)
    ref = SO.gpkde_series(t, w, domain_size=300.0, bin_format=1, bin_size_fraction=1.0, only_histogram=True)
    got = mprw.gpkde_series(t, w, domain_size=300.0, bin_format=1, bin_size_fraction=1.0, only_histogram=True)
    assert got["bin_size"] == ref["bin_size"] and got["n_bins"] == ref["n_bins"]


def test_adapted_grid_late_arrivals():
    """Steady state to the end of the run: the grid adapts to the data, a
    sub-grid far from the origin, kernel bounds from the whole domain."""
    t, w = arrivals(3000, 3, mu=400.0, s=0.05)
    got, ref = check(t, w, domain_size=0.0, adapt_grid=True, bin_format=1, bin_size_fraction=0.75,
                     raw_density=True, rel_err=0.01)
    assert got["delta_bins_origin"] > got["n_bins"]


def test_adapted_grid_given_bin_size():
    t, w = arrivals(2000, 4, mu=30.0, s=0.5)
    check(t, w, domain_size=0.0, adapt_grid=True, bin_format=2, bin_size=0.5, raw_density=True)


def test_resident_exact_points_unit_volume():
    """Resident records sit exactly on the time points: exactPoint opens the
    bin at its boundary, unitVolume output (MPathRW.F90:1935-1955)."""
    rng = np.random.default_rng(5)
    tp = np.arange(1, 101, dtype=np.float64) * 2.0
    t = tp[np.clip(np.round(rng.normal(50, 12, 5000)).astype(int), 0, 99)]
    w = rng.uniform(0.1, 1.0, t.shape[0])
    got, ref = check(t, w, domain_size=200.0, bin_size=2.0, bin_format=2, exact_point=True, unit_volume=True,
                     init_factor=3.0, apply_init_factor=True, rel_err=0.01)
    assert got["counts"][-1] != 0.0 or np.all(t < 200.0)


@pytest.mark.parametrize("sel,factor", [(1, 3.0), (2, 3.0), (0, 1.0), (0, 0.0)])
def test_initial_smoothing_selections(sel, factor):
    t, w = arrivals(1500, 6)
    check(t, w, domain_size=150.0, bin_size=1.0, bin_format=2, init_selection=sel, init_factor=factor,
          apply_init_factor=True, rel_err=0.01)


def test_histogram_only():
    t, w = arrivals(5000, 7)
    for fmt in (0, 1, 2, 3):
        for raw in (False, True):
            check(t, w, domain_size=100.0, bin_format=1, bin_size_fraction=0.75, eff_format=fmt, raw_density=raw,
                  only_histogram=True)


def test_skip_error_and_zero_loops():
    t, w = arrivals(2000, 8)
    got, ref = check(t, w, domain_size=120.0, bin_size=1.0, skip_error=True, n_opt_loops=6)
    assert got["loops"] == 6
    got, ref = check(t, w, domain_size=120.0, bin_size=1.0, n_opt_loops=0)
    assert got["loops"] == 0


def test_wide_kernels_fold_at_both_ends():
    """Few points on a short grid: kernels wider than the grid fold at both
    ends (the low fold first, then the high fold)."""
    t = np.array([1.2, 1.4, 2.6, 3.1, 3.3, 4.9])
    w = np.ones_like(t)
    check(t, w, domain_size=6.0, bin_size=1.0, init_factor=3.0, apply_init_factor=True)
    t = np.array([10.2, 10.4, 10.5, 11.6, 12.1])
    check(t, w[:5], domain_size=0.0, adapt_grid=True, bin_size=0.25)


def test_points_outside_and_no_active_bins():
    t, w = arrivals(500, 9, mu=500.0, s=0.01)
    got = mprw.gpkde_series(t, w, domain_size=100.0, bin_size=1.0)
    assert got["active_bins"] == 0 and got["loops"] == 0
    assert np.all(got["counts"] == 0) and np.all(got["density"] == 0)


def test_capacity_retry_many_bins():
    """More bins than the first buffer (the wrapper retries on MPRW_E_SIZE)."""
    t, w = arrivals(3000, 10, mu=1500.0, s=0.3)
    check(t, w, domain_size=5000.0, bin_size=1.0, n_opt_loops=3)


def test_invalid_inputs_rejected():
    t, w = arrivals(100, 11)
    with pytest.raises(mprw.MprwError):
        mprw.gpkde_series(t[:1], w[:1], domain_size=100.0, bin_format=1)     # FD needs two points
    with pytest.raises(mprw.MprwError):
        mprw.gpkde_series(np.full(10, 5.0), np.ones(10), domain_size=100.0, bin_format=0)   # zero variance
    bad = t.copy()
    bad[3] = np.nan
    with pytest.raises(mprw.MprwError):
        mprw.gpkde_series(bad, w, domain_size=100.0, bin_size=1.0)
    with pytest.raises(mprw.MprwError):
        mprw.gpkde_series(t, w, domain_size=1.0, bin_size=1.0)              # one bin
    with pytest.raises(mprw.MprwError):
        mprw.gpkde_series(t, w, domain_size=0.0, bin_size=1.0)              # no domain, not adapted
    with pytest.raises(mprw.MprwError):
        mprw.gpkde_series(t, w, domain_size=100.0, bin_format=1, bin_size_fraction=2.5)
    with pytest.raises(mprw.MprwError):
        mprw.gpkde_series(np.zeros(0), np.zeros(0), domain_size=100.0, bin_size=1.0)


def test_mass_conserved_at_full_size():
    """10^6 sink records: the reconstruction keeps the binned mass (the edge
    folds move kernel mass, never drop it, when kernels are narrower than
    the grid), with a plume-shaped, non-negative density."""
    t, w = arrivals(1_000_000, 12, mu=80.0, s=0.35)
    got = mprw.gpkde_series(t, w, domain_size=400.0, bin_format=1, bin_size_fraction=0.75, eff_format=0,
                            rel_err=0.01)
    b = got["bin_size"]
    mass_binned = got["counts"].sum()
    np.testing.assert_allclose(got["density"].sum() * b, mass_binned, rtol=1e-9)
    assert got["density"].min() >= -1e-12 * got["density"].max()
    assert got["loops"] >= 1


@pytest.mark.parametrize("fmt", [0, 2, 3])
def test_series_is_bitwise_repeatable(gpu_lib, fmt):
    """The same records reconstructed three times give the same counts,
    weighted counts and density to the last bit: the histogram sums are
    fixed-point integers and the density and curvature are gathered per grid
    position in ascending bin order (the reference's scatter order), so no
    result depends on the order of atomics."""
    rng = np.random.default_rng(7)
    t = rng.lognormal(np.log(60.0), 0.4, 200_000)
    w = rng.uniform(0.2, 3.0, t.size)
    kw = dict(domain_size=300.0, bin_format=1, bin_size_fraction=0.5, init_factor=3.0, raw_density=True,
              eff_format=fmt)
    runs = [mprw.gpkde_series(t, w, **kw) for _ in range(3)]
    for r in runs[1:]:
        assert r["loops"] == runs[0]["loops"] and r["n_bins"] == runs[0]["n_bins"]
        for key in ("counts", "density") + (("wcounts",) if fmt >= 2 else ()):
            assert np.array_equal(np.asarray(r[key]).view(np.uint64), np.asarray(runs[0][key]).view(np.uint64))
