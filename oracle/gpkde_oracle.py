"""numpy restatement of the GPKDE histogram (TEST INFRASTRUCTURE ONLY).

Follows lib/gpkde/Histogram.F90:276-350 (prComputeCountsWeighted):
  gridIndex(d) = floor((x_d - origin_d)/binSize_d) + 1 on the active
  dimensions, points outside [1, nBins] skipped, counts(ix,iy,iz) += w in
  particle order; totalMass = sum(w); Kish nEffective = totalMass**2 /
  sum(w**2); counts /= totalMass/nEffective.
``np.add.at`` accumulates repeated indices sequentially in array order, the
same rounding as the reference's loop.
"""
from __future__ import annotations

import numpy as np


def histogram_weighted(coords: np.ndarray, weights: np.ndarray, origin, bin_size, n_bins):
    """coords (N,3) model coordinates of the active particles in particle order.
    Returns (counts shaped (nz, ny, nx), n_binned, effective_mass)."""
    origin = np.asarray(origin, np.float64)
    bin_size = np.asarray(bin_size, np.float64)
    n_bins = np.asarray(n_bins, np.int64)
    n = coords.shape[0]
    idx = np.zeros((n, 3), np.int64)
    inside = np.ones(n, bool)
    for d in range(3):
        if bin_size[d] == 0.0:
            continue
        q = np.floor((coords[:, d] - origin[d]) / bin_size[d])
        ok = (q >= 0) & (q < n_bins[d])
        inside &= ok
        idx[:, d] = np.where(ok, q, 0).astype(np.int64)
    lin = idx[:, 0] + n_bins[0] * (idx[:, 1] + n_bins[1] * idx[:, 2])
    counts = np.zeros(int(np.prod(n_bins)), np.float64)
    np.add.at(counts, lin[inside], weights[inside])
    total = 0.0
    sw2 = 0.0
    for w in weights:          # sequential sums, as gfortran's sum()
        total = total + float(w)
        sw2 = sw2 + float(w) * float(w)
    eff = 1.0
    if total != 0.0:
        neff = total * total / sw2
        eff = total / neff
        counts = counts / eff
    return counts.reshape(int(n_bins[2]), int(n_bins[1]), int(n_bins[0])), int(inside.sum()), eff
