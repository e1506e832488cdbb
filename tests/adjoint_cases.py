"""Cases of the differentiable walk shared by its CPU and GPU tests: the
lognormal-field generator at reduced sizes (ln K variance sigma2), zones as
2 x 2 x 2 blocks of the grid (8 zones, 25 parameters: alphaL, alphaT and
porosity per zone and a velocity scale), and a base parameter vector."""
from __future__ import annotations

import numpy as np

from mprw import workloads as W
from mprw.model import ACTIVE, EULERIAN, MIN_ADV_DISP, Options


def block_zones(g):
    """Zone of every cell (0-based): 2 x 2 x 2 blocks, x fastest."""
    k, i, j = np.unravel_index(np.arange(g.ncell), (g.nlay, g.nrow, g.ncol))
    return ((j >= g.ncol // 2).astype(np.int32) + 2 * (i >= g.nrow // 2) + 4 * (k >= g.nlay // 2)).astype(np.int32)


def base_theta(nz=8, seed=0):
    """alphaL 0.5, alphaT 0.05, porosity 0.25 per zone (each perturbed by a few
    percent so the zones differ) and velocity scale 1."""
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.95, 1.05, 3 * nz)
    return np.concatenate([0.5 * f[:nz], 0.05 * f[nz:2 * nz], 0.25 * f[2 * nz:], [1.0]])


def field(nlay, nrow, ncol, n_particles, seed, x_release, sigma2=1.0, x0=0.0):
    g, f, _ = W.heterogeneous_flow(nlay, nrow, ncol, sigma2=sigma2, kg=10.0, lh=10.0, lv=2.0, porosity=0.25,
                                   alpha_l=0.5, alpha_t=0.05, dm=1e-4, seed=seed, use_torch=False)
    p = W.release_in_box(g, n_particles, x0, x_release, 0.0, float(nrow), float(g.botm[-1]), float(g.top[0]),
                         seed=77 + seed, status=ACTIVE)
    opt = Options(time_step_kind=MIN_ADV_DISP, ts_param=(0.1, 0.1), advection_kind=EULERIAN, stop_weak_sinks=True)
    return g, f, p, opt
