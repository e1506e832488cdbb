"""GPU against the oracle for the tracking options that the configurations
leave at their defaults: backward tracking, a stop zone, ICBOUND mass
boundaries, stops at weak sources, 2-D and 1-D random walks, the DISP and
FIXED time-step rules, distributed dispersivities, non-uniform porosity and
retardation with interpolated corner porosity, and a convertible top layer
with heads below its top.  Each on the small heterogeneous field (MODFLOW 6
files of the golden fixtures), shared Philox stream: step counts, cells,
statuses and random counters identical, positions within 1e-6, for >= 99 %
of the particles; every stop status with the oracle's count (+-1 %)."""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from golden_cases import hetero_flow
from mprw import workloads as W
from mprw.model import EULERIAN, MIN_ADV_DISP, Options
from oracle import oracle as O


def _variant(name):
    g, f = hetero_flow()
    f = copy.copy(f)
    n = g.ncell
    opt = Options(time_step_kind=MIN_ADV_DISP, ts_param=(0.1, 0.1), advection_kind=EULERIAN, stop_weak_sinks=True)
    rng = np.random.default_rng(17)
    k, i, j = np.unravel_index(np.arange(n), (g.nlay, g.nrow, g.ncol))
    box = ((0.0, 10.0), (0.0, 12.0), (0.0, 4.0))
    if name == "backward":
        opt.backward = True
        box = ((12.0, 22.0), (0.0, 12.0), (0.0, 4.0))
    elif name == "stop_zone":
        f.zones = np.where(j >= 15, 2, 1).astype(np.int32)
        opt.stop_zone = 2
    elif name == "icbound":
        f.icboundts = np.where(k == 0, 1, 0).astype(np.int32)
        f.default_icbound = 0
    elif name == "weak_sources":
        opt.stop_weak_sources = True
        opt.backward = True
        box = ((0.0, 6.0), (0.0, 12.0), (0.0, 4.0))
    elif name == "walk_2d":
        opt.dim_mask = (1, 1, 0)
    elif name == "walk_1d":
        opt.dim_mask = (1, 0, 0)
    elif name == "disp_step":
        opt.time_step_kind = 2
    elif name == "fixed_step":
        opt.time_step_kind = 4
        opt.ts_param = (0.05, 0.0)
    elif name == "distributed":
        f.uniform_dispersion = False
        f.alpha_l = rng.uniform(0.1, 1.0, n)
        f.alpha_t = f.alpha_l * rng.uniform(0.05, 0.2, n)
        f.dm_eff = np.full(n, 1e-4)
    elif name == "porosity":
        f.porosity = rng.uniform(0.15, 0.35, n)
        f.retardation = np.where(j % 5 == 0, 2.0, 1.0)
        opt.uniform_porosity = False
    elif name == "unconfined":
        f.celltype = np.where(k == 0, 1, 0).astype(np.int32)
        top = g.top[(i * g.ncol + j)]
        f.heads = np.where(k == 0, top - 0.3, f.heads)
    else:
        raise KeyError(name)
    p = W.release_in_box(g, 3000, *box[0], *box[1], *box[2], seed=23)
    return g, f, opt, p


VARIANTS = ["backward", "stop_zone", "icbound", "weak_sources", "walk_2d", "walk_1d", "disp_step", "fixed_step",
            "distributed", "porosity", "unconfined"]


@pytest.mark.parametrize("name", VARIANTS)
def test_option_parity(gpu_lib, name):
    g, f, opt, p = _variant(name)
    iv = [(0.0, 12.0), (12.0, 30.0)]
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    gs = sum(tr.advance(a, b) for a, b in iv)
    gp = tr.get_particles()
    tr.close()
    q, os_ = p, 0
    for a, b in iv:
        q, s = O.advance(g, f, opt, q, a, b, rng_kind=O.RNG_PHILOX, nthreads=8)
        os_ += s
    same = (gp["status"] == q.status) & (gp["cell"] == q.cell) & (gp["rng_ctr"] == q.rng_ctr)
    for k in ("lx", "ly", "lz"):
        same &= np.abs(gp[k] - getattr(q, k)) <= 1e-6
    assert same.mean() >= 0.99, f"{name}: {same.mean():.4f}"
    assert abs(gs - os_) <= 0.01 * os_
    for st in range(10):
        a, b = int((gp["status"] == st).sum()), int((q.status == st).sum())
        assert abs(a - b) <= max(3, 0.01 * p.n), (name, st, a, b)
