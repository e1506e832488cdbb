"""numpy restatement of the 1-D GPKDE of observation time series (TEST
INFRASTRUCTURE ONLY).

The observation post-process of MPathRW.F90:1759-2840 reconstructs each
observation's breakthrough curve from the particle arrival (or record) times
with a 1-D GPKDE whose kernel database is off.  This module follows, in the
reference's lib/gpkde (paths relative to its src/ directory):

* GridProjectedKDE.F90 prComputeDensity (3598-4392): the grid adapted to the
  data (3794-3800, 3903-3960), the automatic bin size (3806-3890), the
  weighted histogram (3962-3985), the histogram-only return (3987-4005), the
  data statistics and initial smoothing (4020-4110), the closing scalings
  (4276-4311) and the vector of bin centres (3551-3594);
* prUpdateBinSize (1129-1370) and prInitialize (354-998) for the grid size;
* prComputeDensityOptimization (4396-5160) with the brute kernel setters
  (6224-6317): the loop itself is ``gpkde_oracle.GPKDE._optimize`` with
  ``database=False``; the closing reweighting (5070-5120);
* Histogram.F90: prComputeCountsWeighted (276-350),
  prComputeCountsAndWeights (353-418), prComputeEffectiveCountsAndWeights
  (421-490), prEstimateBinSizeScott (603-641), prEstimateBinSizeFD (644-720).

Sums the reference takes in array order are taken here in array order too
(``np.cumsum`` is a running sum; ``np.add.at`` accumulates repeated indices
in array order).
"""
from __future__ import annotations

import math

import numpy as np

from oracle.gpkde_oracle import GPKDE

BORDER_FRACTION = 0.05            # defaultBorderFraction
DEFAULT_INITIAL_FACTOR = 2.0      # defaultInitialSmoothingFactor
SCOTT_COEFFICIENT = float(np.float32(3.49))   # a default-real literal in the reference


class SeriesError(ValueError):
    """An input the reference stops on (its ``stop`` statements)."""


def _seqsum(a) -> float:
    a = np.asarray(a, np.float64)
    return float(np.cumsum(a)[-1]) if a.size else 0.0


def bin_size_scott(x: np.ndarray) -> float:
    """prEstimateBinSizeScott for points (x, 0, 0)."""
    n = x.shape[0]
    avg = _seqsum(x) / float(n)
    var = _seqsum((x - avg) ** 2.0) / float(n)
    if var == 0.0:
        return 0.0
    return SCOTT_COEFFICIENT * math.sqrt(var) / (float(n) ** (1.0 / 3.0))


def _fd_quartiles(a: np.ndarray):
    """Q1, Q3 of the sorted array as prEstimateBinSizeFD picks them (1-based
    indexes as in the reference)."""
    n = a.shape[0]
    at = lambda i: float(a[i - 1])      # noqa: E731
    if n % 2 == 0:
        if math.fmod(float(n) / 2.0, 2.0) == 0.0:
            q1 = (at(n // 4) + at(n // 4 + 1)) / 2.0
            q3 = (at(n // 2 + n // 4) + at(n // 2 + n // 4 + 1)) / 2.0
        else:
            q1 = at(n // 4 + 1)
            q3 = at(n // 2 + n // 4 + 1)
    else:
        if math.fmod(float(n - 1) / 2.0, 2.0) == 0.0:
            q1 = (at((n - 1) // 4) + at((n - 1) // 4 + 1)) / 2.0
            q3 = (at(n // 2 + 1 + (n - 1) // 4) + at(n // 2 + 1 + (n - 1) // 4 + 1)) / 2.0
        else:
            q1 = at((n - 1) // 4 + 1)
            q3 = at(n // 2 + 1 + (n - 1) // 4 + 1)
    return q1, q3


def bin_size_fd(x: np.ndarray) -> float:
    """prEstimateBinSizeFD (Freedman-Diaconis).  One point would index
    element 0 in the reference; it is rejected here."""
    n = x.shape[0]
    if n < 2:
        raise SeriesError("Freedman-Diaconis bin size needs at least two points")
    q1, q3 = _fd_quartiles(np.sort(x, kind="stable"))
    return 2.0 * (q3 - q1) / (float(n) ** (1.0 / 3.0))


def histogram_series(x, w, origin, b, nb, exact_point, eff_format):
    """The weighted histogram of the formats 0-3.  Returns counts, wcounts
    (None for formats 0/1) and the effective mass."""
    idx = np.floor((x - origin) / b).astype(np.int64) + (0 if exact_point else 1)
    inside = (idx >= 1) & (idx <= nb)
    k = idx[inside] - 1
    wi = w[inside]
    counts = np.zeros(nb)
    wcounts = None
    if eff_format in (2, 3):
        wcounts = np.zeros(nb)
        np.add.at(wcounts, k, wi)
        if eff_format == 2:
            np.add.at(counts, k, np.ones_like(wi))
        else:
            np.add.at(counts, k, wi ** 2)
            nz = counts != 0.0
            counts[nz] = wcounts[nz] ** 2 / counts[nz]
        return counts, wcounts, 1.0
    np.add.at(counts, k, wi)
    total = _seqsum(w)
    if eff_format == 1:
        eff = total / float(w.shape[0])
    else:
        neff = total ** 2 / _seqsum(w ** 2)
        eff = total / neff
    return counts / eff, None, eff


def gpkde_series(times, weights, *, origin=0.0, domain_size=0.0, bin_size=0.0, bin_format=2,
                 bin_size_fraction=1.0, adapt_grid=False, exact_point=False, eff_format=0,
                 init_selection=0, init_factor=DEFAULT_INITIAL_FACTOR, apply_init_factor=False, n_opt_loops=10,
                 rel_err=0.02, skip_error=False, only_histogram=False, raw_density=False, unit_volume=False):
    """ComputeDensity of a 1-D series (data points (t, 0, 0), weights).

    Returns a dict: counts, wcounts (formats 2/3), density (None for a
    histogram only), n_bins, delta_bins_origin, bin_size, grid_origin,
    coordinates, loops, smoothing."""
    x = np.asarray(times, np.float64)
    w = np.asarray(weights, np.float64)
    n = x.shape[0]
    if n < 1 or w.shape[0] != n:
        raise SeriesError("data points empty, or weights of another length")
    ds = float(domain_size)
    if not adapt_grid and ds <= 0.0:
        raise SeriesError("domain size zero and grid not adapted to the data")
    if ds < 0.0:
        raise SeriesError("negative domain size")
    mx, mn = float(x.max()), float(x.min())
    delta = abs(mx - mn)
    if adapt_grid and ds == 0.0 and delta != 0.0:
        ds = (mx + 1.0 * BORDER_FRACTION * delta) - origin
    # bin size and domain grid size
    b = float(bin_size)
    if bin_format in (0, 1):
        if not (0.0 < bin_size_fraction <= 2.0):
            raise SeriesError("bin size fraction outside (0, 2]")
        b = bin_size_scott(x) if bin_format == 0 else bin_size_fd(x)
        b = bin_size_fraction * b
    if b <= 0.0:
        raise SeriesError("bin size not positive")
    if ds == 0.0:
        raise SeriesError("domain size zero")
    gs = int(ds / b + 0.5)
    if gs < 2:
        raise SeriesError("a time grid of fewer than two bins")
    # the grid (a sub-grid around the data when adapted)
    nb, dbo, gorigin = gs, 0, float(origin)
    if adapt_grid:
        lo = max(mn - 0.5 * BORDER_FRACTION * delta, origin)
        hi = min(mx + 0.5 * BORDER_FRACTION * delta, ds + origin)
        dbo = int((lo - origin) / b)
        nb = math.ceil((hi - origin) / b) - dbo
        gorigin = dbo * b + origin
        if nb > gs:
            raise SeriesError("sub-grid larger than the domain grid")
        if nb < 1:
            raise SeriesError("empty sub-grid")
    coords = (np.arange(1, nb + 1, dtype=np.float64) + dbo - 0.5) * b + origin
    counts, wcounts, eff = histogram_series(x, w, gorigin, b, nb, exact_point, eff_format)
    out = dict(n_bins=nb, delta_bins_origin=dbo, bin_size=b, grid_origin=gorigin, coordinates=coords,
               loops=0, smoothing=None, density=None)
    if only_histogram:
        counts = counts * eff
        if raw_density:
            counts = counts / b
            if wcounts is not None:
                wcounts = wcounts / b
        out.update(counts=counts, wcounts=wcounts)
        return out
    act1 = np.nonzero(counts != 0.0)[0]
    if act1.size == 0:
        out.update(counts=counts, wcounts=wcounts, density=np.zeros(nb))
        return out
    # data statistics and the initial smoothing (Silverman)
    mean = _seqsum(x) / n
    std = math.sqrt(_seqsum((x - mean) ** 2.0) / n)
    hsig = std * (4.0 / ((1.0 + 2.0) * n)) ** (1.0 / (1.0 + 4.0))
    apply = apply_init_factor
    if std == 0.0:
        hsig = DEFAULT_INITIAL_FACTOR * b
        apply = False
    if init_selection == 0:
        init = hsig * init_factor if (apply and init_factor > 0.0 and init_factor != 1.0) else hsig
    elif init_selection == 1:
        init = init_factor * b
    elif init_selection == 2:
        init = DEFAULT_INITIAL_FACTOR * b
    else:
        raise SeriesError("initial smoothing selection not in 0..2")
    g = GPKDE((ds, 0.0, 0.0), (b, 0.0, 0.0), origin=(gorigin, 0.0, 0.0), n_opt_loops=n_opt_loops, rel_err=rel_err,
              skip_error=skip_error, database=False, n_bins=(nb, 1, 1))
    c3 = counts.reshape(nb, 1, 1)
    act = np.stack([act1 + 1, np.ones_like(act1), np.ones_like(act1)], 1)
    dens, ks = g._optimize(c3, act, np.array([init, 0.0, 0.0]), n)
    dens = dens.reshape(nb)
    if eff_format in (0, 1):
        counts = counts * eff
        dens = dens * eff
    else:
        dens = g._density(wcounts.reshape(nb, 1, 1), act, ks).reshape(nb)
    if raw_density:
        counts = counts / b
        if wcounts is not None:
            wcounts = wcounts / b
    if unit_volume:
        dens = dens * b
    out.update(counts=counts, wcounts=wcounts, density=dens, loops=g.loops, smoothing=ks[0].copy())
    return out
