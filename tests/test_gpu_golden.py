"""The CUDA library against the committed golden fixtures (oracle outputs on
small seeded inputs; tests/golden/make_golden.py), through the C ABI:

* pure advection: identical cells, statuses and step counts, positions and
  times to 1e-10 relative;
* dispersion on the shared Philox stream (uniform and heterogeneous fields,
  the latter read from MODFLOW 6 files): identical step counts per particle
  (RNG counters) and positions within 1e-6 for >= 99.5 % of the particles;
* EXPONENTIAL advection in a graded field: positions to 1e-9 m;
* GPKDE from the fixtures' particle states: identical histograms and loop
  counts, densities within 1e-10 (1-D) / 1e-9 (3-D) of their maximum."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from golden_cases import STATE, TRACKING_CASES, case, hetero_flow, load, particles_out
from mprw import workloads as W


def _track(g, f, opt, p, iv):
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    steps = sum(tr.advance(t0, t1) for t0, t1 in iv)
    out = tr.get_particles()
    tr.close()
    return out, steps


@pytest.mark.parametrize("name", TRACKING_CASES)
def test_tracking_against_golden(gpu_lib, name):
    g, f, opt, p, iv, d = case(name)
    out, steps = _track(g, f, opt, p, iv)
    if name in ("uniform_advection", "graded_exponential"):
        assert steps == int(d["steps"])
        np.testing.assert_array_equal(out["cell"], d["out_cell"])
        np.testing.assert_array_equal(out["status"], d["out_status"])
        np.testing.assert_allclose(out["t"], d["out_t"], rtol=1e-12, atol=0)
        tol = 1e-10 if name == "uniform_advection" else 1e-9
        for k in ("lx", "ly", "lz"):
            np.testing.assert_allclose(out[k], d[f"out_{k}"], rtol=tol, atol=tol)
    else:
        same = (out["cell"] == d["out_cell"]) & (out["status"] == d["out_status"]) & \
               (out["rng_ctr"] == d["out_rng_ctr"])
        for k in ("lx", "ly", "lz"):
            same &= np.abs(out[k] - d[f"out_{k}"]) <= 1e-6
        assert same.mean() >= 0.995, f"{same.mean():.4f}"
        assert abs(steps - int(d["steps"])) <= 1e-3 * int(d["steps"])


@pytest.mark.parametrize("name", ["gpkde_1d", "gpkde_3d"])
def test_gpkde_against_golden(gpu_lib, name):
    d = load(name)
    if name == "gpkde_1d":
        g, f, _, opt = W.uniform_pulse(n_particles=1)
        kw, tol = {}, 1e-10
    else:
        g, f = hetero_flow()
        _, _, opt, _, _, _ = case("hetero_small")
        kw, tol = {"n_opt_loops": int(d["n_opt_loops"])}, 1e-9
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(particles_out(d))
    dens, hist, loops = tr.gpkde(tuple(d["domain"]), tuple(d["bins"]), **kw)
    assert loops == int(d["loops"])
    ref = d["density"].transpose(2, 1, 0)
    np.testing.assert_allclose(dens, ref, rtol=0, atol=tol * ref.max())
    if "histogram" in d:
        np.testing.assert_array_equal(hist.reshape(-1), d["histogram"].reshape(-1))
    tr.close()
