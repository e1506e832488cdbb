"""The 1-D series GPKDE restatement (oracle/series_oracle.py) against known
answers (CPU): the Freedman-Diaconis quartile picks and Scott's constant of
Histogram.F90:603-720, exact-point binning, the effective-weight formats of
Histogram.F90:276-490, the adapted sub-grid of GridProjectedKDE.F90:3903-3960,
and a reconstruction of a Gaussian sample against its density."""
import math

import numpy as np
import pytest

from oracle import series_oracle as SO


@pytest.mark.parametrize("n,q1,q3", [
    (4, 1.5, 3.5),        # n even, n/2 even: averages of a(1),a(2) and a(3),a(4)
    (6, 2.0, 5.0),        # n even, n/2 odd: a(2), a(5)
    (5, 1.5, 4.5),        # n odd, (n-1)/2 even: averages of a(1),a(2) and a(4),a(5)
    (7, 2.0, 6.0),        # n odd, (n-1)/2 odd: a(2), a(6)
    (8, 2.5, 6.5),
    (9, 2.5, 7.5),
])
def test_fd_quartile_picks(n, q1, q3):
    a = np.arange(1, n + 1, dtype=np.float64)
    got = SO._fd_quartiles(a)
    assert got == (q1, q3)
    rng = np.random.default_rng(n)
    x = rng.permutation(a)
    assert SO.bin_size_fd(x) == 2.0 * (q3 - q1) / float(n) ** (1.0 / 3.0)


def test_fd_needs_two_points():
    with pytest.raises(SO.SeriesError):
        SO.bin_size_fd(np.array([3.0]))


def test_scott_constant_is_single_precision():
    assert SO.SCOTT_COEFFICIENT == 3.490000009536743
    x = np.array([0.0, 2.0])            # mean 1, population variance 1
    assert SO.bin_size_scott(x) == SO.SCOTT_COEFFICIENT * 1.0 / 2.0 ** (1.0 / 3.0)
    assert SO.bin_size_scott(np.full(5, 7.0)) == 0.0


def test_exact_point_binning():
    """exactPoint bins t at floor((t - origin)/b) (1-based), so a time on
    the edge k*b opens bin k; otherwise floor(...) + 1.  Points outside
    [1, n] are dropped."""
    t = np.array([0.0, 1.0, 2.0, 2.5, 5.0])
    w = np.ones_like(t)
    c_exact, _, _ = SO.histogram_series(t, w, 0.0, 1.0, 5, True, 2)
    c_plain, _, _ = SO.histogram_series(t, w, 0.0, 1.0, 5, False, 2)
    np.testing.assert_array_equal(c_exact, [1, 2, 0, 0, 1])       # 0.0 -> bin 0: dropped; 2.0, 2.5 -> bin 2
    np.testing.assert_array_equal(c_plain, [1, 1, 2, 0, 0])        # 5.0 -> bin 6: dropped


def test_effective_weight_formats():
    t = np.array([0.5, 0.6, 1.5, 1.7, 1.9])
    w = np.array([1.0, 3.0, 2.0, 2.0, 4.0])
    c0, wc0, eff0 = SO.histogram_series(t, w, 0.0, 1.0, 2, False, 0)
    total, sw2 = w.sum(), (w ** 2).sum()
    assert eff0 == pytest.approx(total / (total ** 2 / sw2), rel=1e-15) and wc0 is None
    np.testing.assert_allclose(c0, np.array([4.0, 8.0]) / eff0, rtol=1e-15)
    c1, _, eff1 = SO.histogram_series(t, w, 0.0, 1.0, 2, False, 1)
    assert eff1 == pytest.approx(total / 5.0, rel=1e-15)
    c2, wc2, eff2 = SO.histogram_series(t, w, 0.0, 1.0, 2, False, 2)
    np.testing.assert_array_equal(c2, [2, 3])
    np.testing.assert_array_equal(wc2, [4, 8])
    assert eff2 == 1.0
    c3, wc3, _ = SO.histogram_series(t, w, 0.0, 1.0, 2, False, 3)
    np.testing.assert_allclose(c3, [16.0 / 10.0, 64.0 / 24.0], rtol=1e-15)   # (sum w)^2 / sum w^2


def test_adapted_subgrid():
    """Data in [10, 20], bin 1: the domain is max + 0.05*delta = 20.5, the
    sub-grid [min - 0.025 delta, max + 0.025 delta] = [9.75, 20.25] on bin
    edges 9..21: 12 bins from domain bin 9 (origin 9)."""
    t = np.linspace(10.0, 20.0, 101)
    r = SO.gpkde_series(t, np.ones_like(t), domain_size=0.0, adapt_grid=True, bin_size=1.0, only_histogram=True)
    assert r["n_bins"] == 12 and r["delta_bins_origin"] == 9 and r["grid_origin"] == 9.0
    np.testing.assert_allclose(r["coordinates"], np.arange(9.5, 21.5, 1.0))
    assert r["counts"].sum() == pytest.approx(101.0)


def test_gaussian_sample_reconstruction():
    """10^4 samples of N(50, 5^2) on a 1-unit grid: the reconstruction keeps
    the mass, is within a few percent of the true density in L1, and is
    closer to it than the histogram."""
    rng = np.random.default_rng(3)
    t = rng.normal(50.0, 5.0, 10_000)
    r = SO.gpkde_series(t, np.ones_like(t), domain_size=100.0, bin_size=1.0, raw_density=True, rel_err=0.01)
    x = r["coordinates"]
    true = np.exp(-0.5 * ((x - 50.0) / 5.0) ** 2) / (5.0 * math.sqrt(2.0 * math.pi))
    dens = r["density"] / t.shape[0]
    hist = r["counts"] / t.shape[0]
    assert dens.sum() == pytest.approx(1.0, abs=1e-9)
    l1_kde = np.abs(dens - true).sum()
    l1_hist = np.abs(hist - true).sum()
    assert r["loops"] >= 1
    assert l1_kde < 0.05 and l1_kde < l1_hist


def test_rejections():
    t = np.linspace(0.0, 1.0, 10)
    w = np.ones_like(t)
    with pytest.raises(SO.SeriesError):
        SO.gpkde_series(t, w, domain_size=0.0, bin_size=0.1)                 # no domain, not adapted
    with pytest.raises(SO.SeriesError):
        SO.gpkde_series(t, w, domain_size=1.0, bin_size=1.0)                 # one bin
    with pytest.raises(SO.SeriesError):
        SO.gpkde_series(t, w, domain_size=10.0, bin_format=1, bin_size_fraction=3.0)
    with pytest.raises(SO.SeriesError):
        SO.gpkde_series(np.zeros(0), np.zeros(0), domain_size=10.0, bin_size=1.0)
