"""Regenerate the golden fixtures of this directory from the oracle.

The reference is Fortran and cannot be built here, so these fixtures are the
outputs of the oracle (oracle/: the C restatement of the tracking path and
the numpy restatement of GPKDE) on small seeded inputs.  The CPU tests check
that the oracle still reproduces them bit for bit; the GPU tests check the
CUDA library against them with the parity tolerances.  Inputs that come from
a floating-point solve are stored too (the heterogeneous flow as MODFLOW 6
binary files), so the fixtures do not depend on the solver's rounding on
another machine.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (str(ROOT / "modpath-rw_gb300"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)

from mprw import mf6io  # noqa: E402
from mprw import workloads as W  # noqa: E402
from mprw.model import EXPONENTIAL, Options, Particles  # noqa: E402
from oracle import gpkde_oracle as GO  # noqa: E402
from oracle import oracle as O  # noqa: E402

STATE = ("cell", "lx", "ly", "lz", "t", "status", "rng_ctr")


def spread(p, lo, hi, seed):
    rng = np.random.default_rng(seed)
    n = p.n
    p.cell = (1 + rng.integers(lo, hi, n)).astype(np.int32)
    p.lx, p.ly, p.lz = rng.uniform(0, 1, n), rng.uniform(0, 1, n), rng.uniform(0, 1, n)
    return p


def run(g, f, opt, p, intervals):
    q, steps = p, 0
    for t0, t1 in intervals:
        q, s = O.advance(g, f, opt, q, t0, t1, rng_kind=O.RNG_PHILOX, nthreads=1)
        steps += s
    return q, steps


def save_case(name, p, q, steps, intervals, **extra):
    out = {f"in_{k}": np.asarray(getattr(p, k)) for k in ("cell", "lx", "ly", "lz", "t", "status", "mass", "id")}
    out.update({f"out_{k}": np.asarray(getattr(q, k)) for k in STATE})
    out["steps"] = np.int64(steps)
    out["intervals"] = np.asarray(intervals, np.float64)
    out.update(extra)
    np.savez_compressed(HERE / f"{name}.npz", **out)


def flow_case():
    """The lognormal-field flow of the small heterogeneous cases, as MODFLOW 6 files."""
    g, f, p, opt, info = W.lognormal_slab(n_particles=400, nlay=4, nrow=12, ncol=30, seed=0, use_torch=False)
    mf6io.write_flow_files(HERE / "hetero_small", g, f, spdis=False)
    return opt


def load_flow_case():
    grb = mf6io.read_grb(HERE / "hetero_small.grb")
    f = mf6io.flow_from_mf6(grb, mf6io.read_heads(HERE / "hetero_small.hds"),
                            mf6io.read_budget(HERE / "hetero_small.bud"), 1, 1, porosity=0.25, retardation=1.0,
                            alpha_l=0.5, alpha_t=0.05, dm_eff=1e-4)
    return grb.grid, f


def main():
    # 1. the uniform column pulse, pure advection: trajectories
    g, f, p, opt = W.uniform_pulse(n_particles=300, pure_advection=True)
    p = spread(p, 5, 40, 3)
    iv = [(0.0, 25.0), (25.0, 50.0)]
    q, s = run(g, f, opt, p, iv)
    save_case("uniform_advection", p, q, s, iv)
    # 2. the same with dispersion on the shared Philox stream
    g, f, p, opt = W.uniform_pulse(n_particles=300)
    p = spread(p, 5, 40, 5)
    iv = [(0.0, 10.0), (10.0, 25.0)]
    q, s = run(g, f, opt, p, iv)
    save_case("uniform_dispersion", p, q, s, iv)
    # 3. heterogeneous field from MODFLOW 6 files, weak-sink stops
    opt = flow_case()
    g, f = load_flow_case()
    p = W.release_in_box(g, 400, 0.0, 10.0, 0.0, 12.0, 0.0, 4.0, seed=1000)
    iv = [(0.0, 20.0), (20.0, 40.0)]
    q, s = run(g, f, opt, p, iv)
    save_case("hetero_small", p, q, s, iv)
    # 4. EXPONENTIAL advection in the graded column (no dispersion)
    g, f, Q = W.graded_flow()
    n = 200
    rng = np.random.default_rng(11)
    p = Particles(cell=(1 + rng.integers(0, 10, n)).astype(np.int32), lx=rng.uniform(0, 1, n),
                  ly=np.full(n, 0.5), lz=np.full(n, 0.5), t=np.zeros(n), status=np.zeros(n, np.int32),
                  mass=np.ones(n), id=np.arange(n, dtype=np.uint64), rng_ctr=np.zeros(n, np.uint64))
    opt = Options(time_step_kind=1, ts_param=(0.1, 0.1), advection_kind=EXPONENTIAL)
    iv = [(0.0, 30.0)]
    q, s = run(g, f, opt, p, iv)
    save_case("graded_exponential", p, q, s, iv)
    # 5. GPKDE, 1-D: the uniform column's plume after 50 days
    g, f, p, opt = W.uniform_pulse(n_particles=5000)
    q, _ = run(g, f, opt, p, [(0.0, 50.0)])
    gx, gy, gz = O.global_xyz(g, f, q)
    act = q.status == 1
    co = np.stack([gx, gy, gz], 1)[act]
    G = GO.GPKDE((200.0, 1.0, 1.0), (1.0, 1.0, 1.0))
    dens, _ = G.compute_density(co, np.ones(co.shape[0]))
    hist, nb, eff = GO.histogram_weighted(co, np.ones(co.shape[0]), (0, 0, 0), (1, 1, 1), (200, 1, 1))
    np.savez_compressed(HERE / "gpkde_1d.npz", coords=co, density=dens, histogram=hist, loops=np.int64(G.loops),
                        domain=np.array([200.0, 1.0, 1.0]), bins=np.ones(3),
                        **{f"out_{k}": np.asarray(getattr(q, k)) for k in STATE})
    # 6. GPKDE, 3-D: the heterogeneous case's plume
    g, f = load_flow_case()
    q = np.load(HERE / "hetero_small.npz")
    qq = Particles(cell=q["out_cell"], lx=q["out_lx"], ly=q["out_ly"], lz=q["out_lz"], t=q["out_t"],
                   status=q["out_status"])
    gx, gy, gz = O.global_xyz(g, f, qq)
    act = qq.status == 1
    co = np.stack([gx, gy, gz], 1)[act]
    G = GO.GPKDE((30.0, 12.0, 4.0), (1.0, 1.0, 1.0), n_opt_loops=5)
    dens, _ = G.compute_density(co, np.ones(co.shape[0]))
    np.savez_compressed(HERE / "gpkde_3d.npz", coords=co, density=dens, loops=np.int64(G.loops),
                        domain=np.array([30.0, 12.0, 4.0]), bins=np.ones(3), n_opt_loops=np.int64(5),
                        **{f"out_{k}": q[f"out_{k}"] for k in STATE})
    for f_ in sorted(HERE.glob("*")):
        if f_.suffix != ".py":
            print(f"{f_.name:28s} {f_.stat().st_size:8d} B")


if __name__ == "__main__":
    main()
