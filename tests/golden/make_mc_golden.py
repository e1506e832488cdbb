"""Monte-Carlo fixtures of the reference's own random-walk statistics.

The oracle (oracle/: the C restatement of the reference's tracking path)
runs here on the reference's RNG path -- xoroshiro128+ streams seeded once
per run from the reference's base seed, Irwin-Hall(12) normals
(rng_par_zig.f90:156-335, TrackSubCell.F90:553-555, 613-620, 3631-3663) --
single-threaded, the one setting in which the reference is deterministic.
Each fixture keeps the plume summaries of tests/mc_stats.py after every
tracking interval (status counts, moments, histograms, control-plane and
breakthrough counts), not the particles.  The GPU tests track an
independent sample with the library's Philox stream and compare the two as
samples of one random-walk process (tests/test_gpu_statistics.py).

* mc_uniform_pulse.npz: the uniform-column pulse (200x1x1 cells, v = 1 m/d,
  alphaL 0.1 m, alphaT 0.01 m, Courant 0.1), 1,000,000 particles at x = 10 m,
  summaries at 25, 50 and 100 days on 1 m bins.  At this size the scheme's
  drift bias against the analytic Gaussian (interface forcing at the cell
  faces) is measured to a few millimetres.
* mc_hetero_small.npz: the small lognormal field of hetero_small.* (the
  lognormal-slab generator at 30x12x4 cells, MIN_ADV_DISP 0.1/0.1, stops at
  the weak sinks of the constant-head outlet), 200,000 particles released in
  the 0-6 m inlet box, summaries at 10, 20, 30, 45 and 60 days: 0.5 m
  x-histogram, particles past the control plane x = 20 m, and the outlet
  breakthrough (stop times of the weak-sink stops, 1-day bins).

    python tests/golden/make_mc_golden.py          # about 8 minutes on one core
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (str(ROOT / "modpath-rw_gb300"), str(ROOT), str(HERE.parent)):
    if p not in sys.path:
        sys.path.insert(0, p)

import mc_stats as S  # noqa: E402
from golden_cases import hetero_flow  # noqa: E402
from mprw import workloads as W  # noqa: E402
from mprw.model import EULERIAN, MIN_ADV_DISP, Options  # noqa: E402
from oracle import oracle as O  # noqa: E402

PULSE_INTERVALS = [(0.0, 25.0), (25.0, 50.0), (50.0, 100.0)]
PULSE_N = 1_000_000
PULSE_X_EDGES = np.arange(201, dtype=np.float64)

HETERO_INTERVALS = [(0.0, 10.0), (10.0, 20.0), (20.0, 30.0), (30.0, 45.0), (45.0, 60.0)]
HETERO_N = 200_000
HETERO_X_EDGES = np.arange(0.0, 30.0 + 1e-9, 0.5)
HETERO_T_EDGES = np.arange(0.0, 60.0 + 1e-9, 1.0)
HETERO_PLANE = 20.0
HETERO_BOX = (0.0, 6.0, 0.0, 12.0, 0.0, 4.0)


def hetero_case(n, seed):
    g, f = hetero_flow()
    opt = Options(time_step_kind=MIN_ADV_DISP, ts_param=(0.1, 0.1), advection_kind=EULERIAN, stop_weak_sinks=True)
    p = W.release_in_box(g, n, *HETERO_BOX, seed=seed)
    return g, f, opt, p


def run_oracle(g, f, opt, p, intervals, summ):
    O.reset_xoroshiro()
    out, q, steps = {}, p, 0
    for k, (a, b) in enumerate(intervals):
        q, s = O.advance(g, f, opt, q, a, b, rng_kind=O.RNG_XOROSHIRO, nthreads=1)
        steps += s
        gx, gy, gz = O.global_xyz(g, f, q)
        out.update(S.to_npz(f"t{k}_", summ(q.status, gx, gy, gz, q.t)))
    out["intervals"] = np.asarray(intervals)
    out["particle_steps"] = np.int64(steps)
    return out


def main():
    t0 = time.time()
    g, f, p, opt = W.uniform_pulse(n_particles=PULSE_N)
    out = run_oracle(g, f, opt, p, PULSE_INTERVALS, lambda st, x, y, z, t: S.summarize(st, x, y, z, t, PULSE_X_EDGES))
    np.savez_compressed(HERE / "mc_uniform_pulse.npz", **out)
    print(f"mc_uniform_pulse: {out['particle_steps']} particle-steps, {time.time() - t0:.0f} s")
    t0 = time.time()
    g, f, opt, p = hetero_case(HETERO_N, seed=4242)
    out = run_oracle(g, f, opt, p, HETERO_INTERVALS,
                     lambda st, x, y, z, t: S.summarize(st, x, y, z, t, HETERO_X_EDGES, HETERO_PLANE, HETERO_T_EDGES))
    np.savez_compressed(HERE / "mc_hetero_small.npz", **out)
    print(f"mc_hetero_small: {out['particle_steps']} particle-steps, {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
