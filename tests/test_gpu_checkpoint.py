"""Checkpoint / resume of the particle state: a run stopped after its first
interval, written to disk and restored into a new handle, continues bit for
bit as the uninterrupted run (counter-based random numbers keyed by particle
id and draw count), in FP64 and MIXED."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from mprw import workloads as W
from mprw.model import FP64, MIXED


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_resume_is_bit_exact(gpu_lib, tmp_path, precision):
    g, f, p, opt, info = W.lognormal_slab(n_particles=20000, nlay=4, nrow=12, ncol=30, seed=3, precision=precision,
                                   use_torch=False)
    a = mprw.Tracker(g, opt)
    a.load_flow(f)
    a.set_particles(p)
    a.advance(0.0, 15.0)
    a.checkpoint(tmp_path / "state.npz")
    a.advance(15.0, 40.0)
    ref = a.get_particles()
    a.close()
    b = mprw.Tracker(g, opt)
    b.load_flow(f)
    b.restore(tmp_path / "state.npz")
    b.advance(15.0, 40.0)
    out = b.get_particles()
    b.close()
    for k in ("cell", "status", "lx", "ly", "lz", "t", "rng_ctr", "gx"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    assert np.isfinite(out["gx"]).all()
