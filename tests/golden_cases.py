"""The golden fixtures of tests/golden/ (made by tests/golden/make_golden.py
from the oracle): their inputs rebuilt as the library's containers."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from mprw import mf6io
from mprw import workloads as W
from mprw.model import EULERIAN, EXPONENTIAL, MIN_ADV_DISP, Options, Particles

GOLDEN = Path(__file__).resolve().parent / "golden"
STATE = ("cell", "lx", "ly", "lz", "t", "status", "rng_ctr")


def load(name):
    return np.load(GOLDEN / f"{name}.npz")


def particles_in(d) -> Particles:
    n = d["in_cell"].shape[0]
    return Particles(cell=d["in_cell"].copy(), lx=d["in_lx"].copy(), ly=d["in_ly"].copy(), lz=d["in_lz"].copy(),
                     t=d["in_t"].copy(), status=d["in_status"].copy(), mass=d["in_mass"].copy(),
                     id=d["in_id"].copy(), rng_ctr=np.zeros(n, np.uint64))


def particles_out(d) -> Particles:
    n = d["out_cell"].shape[0]
    return Particles(cell=d["out_cell"].copy(), lx=d["out_lx"].copy(), ly=d["out_ly"].copy(),
                     lz=d["out_lz"].copy(), t=d["out_t"].copy(), status=d["out_status"].copy(), mass=np.ones(n),
                     id=np.arange(n, dtype=np.uint64), rng_ctr=d["out_rng_ctr"].copy())


def hetero_flow():
    grb = mf6io.read_grb(GOLDEN / "hetero_small.grb")
    f = mf6io.flow_from_mf6(grb, mf6io.read_heads(GOLDEN / "hetero_small.hds"),
                            mf6io.read_budget(GOLDEN / "hetero_small.bud"), 1, 1, porosity=0.25, retardation=1.0,
                            alpha_l=0.5, alpha_t=0.05, dm_eff=1e-4)
    return grb.grid, f


def case(name):
    """(grid, flow, options, particles, intervals, fixture) of a tracking case."""
    d = load(name)
    iv = [tuple(r) for r in d["intervals"]]
    if name == "uniform_advection":
        g, f, _, opt = W.uniform_pulse(n_particles=1, pure_advection=True)
    elif name == "uniform_dispersion":
        g, f, _, opt = W.uniform_pulse(n_particles=1)
    elif name == "hetero_small":
        g, f = hetero_flow()
        opt = Options(time_step_kind=MIN_ADV_DISP, ts_param=(0.1, 0.1), advection_kind=EULERIAN,
                      stop_weak_sinks=True)
    elif name == "graded_exponential":
        g, f, _ = W.graded_flow()
        opt = Options(time_step_kind=1, ts_param=(0.1, 0.1), advection_kind=EXPONENTIAL)
    else:
        raise KeyError(name)
    return g, f, opt, particles_in(d), iv, d


TRACKING_CASES = ("uniform_advection", "uniform_dispersion", "hetero_small", "graded_exponential")
