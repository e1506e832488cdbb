"""Faults made on the host, and what the library does with them: release and
status rules equal the oracle's (pending, unreleased, inactive cell);
non-finite flows and malformed calls are rejected at the C ABI with
MPRW_E_INVAL / MPRW_E_STATE before any device work, and the handle keeps
working."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from mprw import workloads as W
from mprw.model import ACTIVE, INACTIVE, PENDING, UNRELEASED
from oracle import oracle as O


def _gpu(g, f, opt, p, t0, t1):
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    s = tr.advance(t0, t1)
    out = tr.get_particles()
    tr.close()
    return out, s


def test_release_and_status_rules_match_the_oracle(gpu_lib):
    g, f, p, opt = W.uniform_pulse(n_particles=6, pure_advection=True)
    p.t[:] = [0.0, 5.0, 50.0, -1.0, 0.0, 3.0]
    p.status[:] = PENDING
    f.iboundts = f.iboundts.copy()
    p.cell[4:] = 31
    f.iboundts[30] = 0                    # particles 4 and 5 start in an inactive cell
    out, s = _gpu(g, f, opt, p, 0.0, 10.0)
    q, so = O.advance(g, f, opt, p, 0.0, 10.0)
    assert list(q.status) == [ACTIVE, ACTIVE, PENDING, UNRELEASED, INACTIVE, INACTIVE]
    np.testing.assert_array_equal(out["status"], q.status)
    np.testing.assert_array_equal(out["cell"], q.cell)
    np.testing.assert_allclose(out["lx"], q.lx, rtol=1e-12, atol=1e-12)
    assert s == so


def test_non_finite_inputs_are_rejected(gpu_lib):
    """The reference runs with -ffpe-trap=invalid and stops at the first NaN;
    the library rejects non-finite flows at mprw_load_flow, and the handle's
    previous flow stays in use."""
    g, f, p, opt = W.uniform_pulse(n_particles=200)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    rows = np.repeat(np.arange(g.ncell), np.diff(f.ia))
    for field, val in (("flowja", np.nan), ("flowja", np.inf), ("boundary_flows", np.nan), ("alpha_l", np.nan)):
        bad = W.uniform_pulse(n_particles=1)[1]
        arr = getattr(bad, field).copy()
        if field == "flowja":
            arr[rows == 29] = val
        else:
            arr[0] = val
        setattr(bad, field, arr)
        with pytest.raises(mprw.MprwError, match="non-finite"):
            tr.load_flow(bad)
    out0 = O.advance(g, f, opt, p, 0.0, 20.0, rng_kind=O.RNG_PHILOX, nthreads=4)[0]
    assert tr.advance(0.0, 20.0) > 0
    out = tr.get_particles()
    assert (out["cell"] == out0.cell).mean() > 0.99 and np.isfinite(out["lx"]).all()
    tr.close()


def test_malformed_calls_are_rejected(gpu_lib):
    g, f, p, opt = W.uniform_pulse(n_particles=10)
    tr = mprw.Tracker(g, opt)
    with pytest.raises(mprw.MprwError, match="rc=-4"):        # advance before any flow
        tr.advance(0.0, 1.0)
    bad = f.porosity.copy()
    bad[3] = 0.0
    f2 = W.uniform_pulse(n_particles=1)[1]
    f2.porosity = bad
    with pytest.raises(mprw.MprwError, match="porosity"):
        tr.load_flow(f2)
    f3 = W.uniform_pulse(n_particles=1)[1]
    f3.ja = f3.ja.copy()
    f3.ja[5] = g.ncell + 7
    with pytest.raises(mprw.MprwError, match="JA entry"):
        tr.load_flow(f3)
    tr.load_flow(f)
    q = p.copy()
    q.cell = q.cell.copy()
    q.cell[0] = 0
    with pytest.raises(mprw.MprwError, match="cell number"):
        tr.set_particles(q)
    tr.set_particles(p)
    with pytest.raises(mprw.MprwError, match="t_end < t_begin"):
        tr.advance(5.0, 1.0)
    lib = tr.lib
    o = mprw.GpkdeOptions()
    assert lib.mprw_gpkde(tr.h, C.byref(o), None, None, None, None) == -1   # null density
    assert lib.mprw_histogram(tr.h, None, None, None, None, None, None) == -1
    assert tr.advance(0.0, 1.0) >= 0                                       # still usable
    tr.close()
