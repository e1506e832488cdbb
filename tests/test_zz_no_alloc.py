"""The allocation-free histogram entry point, mprw_histogram_noalloc.

It serves callers that cannot allocate device memory when they bin (a host
code that owns a fixed device-memory budget, or one running where cudaMalloc
would synchronise the device or is forbidden): its only scratch is a fixed
array inside the library.  These tests call it through the C ABI on device
buffers and check that it gives exactly the counts of mprw_histogram, the
handle-based entry point, with unit masses, and exactly the counts of the
oracle's restatement of the reference's histogram -- on consecutive calls, so
that a call never sees what the previous one left in the shared array.  The file is
named so that pytest collects it last; it passes both alone in a fresh process
(where its first call does the once-per-device set-up) and after every other
test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from mprw import workloads as W
from mprw.model import ACTIVE
from oracle import gpkde_oracle as GO

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def _bind(lib):
    fn = lib.mprw_histogram_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, _dp, _dp, _ip, C.c_void_p,
                   C.c_void_p, C.c_void_p]
    return fn


def _noalloc(fn, dev, origin, bins, nb):
    """One call on the default stream; returns (counts shaped (nz, ny, nx), n_binned)."""
    import torch
    o = np.ascontiguousarray(origin, np.float64)
    b = np.ascontiguousarray(bins, np.float64)
    n_bins = np.ascontiguousarray(nb, np.int32)
    # fill the output with garbage so that a bin the call failed to write shows up
    counts = torch.full((int(np.prod(n_bins)),), -7.0, dtype=torch.float64, device="cuda")
    nbinned = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    rc = fn(dev["gx"].data_ptr(), dev["gy"].data_ptr(), dev["gz"].data_ptr(), dev["status"].data_ptr(),
            dev["n"], o.ctypes.data_as(_dp), b.ctypes.data_as(_dp), n_bins.ctypes.data_as(_ip), counts.data_ptr(),
            nbinned.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    return counts.cpu().numpy().reshape(int(nb[2]), int(nb[1]), int(nb[0])), int(nbinned.item())


def _device_particles(out):
    import torch
    return dict(gx=torch.from_numpy(out["gx"]).cuda(), gy=torch.from_numpy(out["gy"]).cuda(),
                gz=torch.from_numpy(out["gz"]).cuda(), status=torch.from_numpy(out["status"]).cuda(),
                n=int(out["status"].shape[0]))


def test_noalloc_histogram_matches_histogram(gpu_lib):
    fn = _bind(gpu_lib)
    g, f, p, opt = W.uniform_pulse(n_particles=20000)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    grids = (((0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (200, 1, 1)),      # 1-D, x only
             ((30.0, 0.0, 0.0), (0.25, 0.5, 0.5), (160, 2, 2)),    # 3-D, smaller in x
             ((0.0, 0.0, 0.0), (0.125, 0.25, 0.25), (1600, 4, 4)))  # 3-D, 25 600 bins
    try:
        for t0, t1 in ((0.0, 30.0), (30.0, 60.0)):
            tr.advance(t0, t1)
            out = tr.get_particles()
            dev = _device_particles(out)
            act = out["status"] == ACTIVE
            coords = np.stack([out["gx"], out["gy"], out["gz"]], 1)[act]
            # the same grids twice in a row, then a larger grid after a smaller one
            for origin, bins, nb in grids + grids[:1]:
                ref, ref_binned, _ = tr.histogram(origin, bins, nb)
                got, got_binned = _noalloc(fn, dev, origin, bins, nb)
                np.testing.assert_array_equal(got, ref)
                assert got_binned == ref_binned
                assert ref_binned > 0
                # and against the oracle's histogram of the same active particles
                orc, orc_binned, _ = GO.histogram_weighted(coords, np.ones(coords.shape[0]), origin, bins, nb)
                np.testing.assert_array_equal(got, orc)
                assert got_binned == orc_binned
    finally:
        tr.close()


def test_noalloc_histogram_rejects_oversized_grid(gpu_lib):
    fn = _bind(gpu_lib)
    o = np.zeros(3)
    b = np.ones(3)
    limit = 1 << 20
    import torch
    for nb in ((limit + 1, 1, 1), (1024, 1024, 2), (-1, 1, 1)):
        n_bins = np.asarray(nb, np.int32)
        # an output large enough for the requested grid, so that nothing could be
        # written out of bounds even if the size check were missing
        counts = torch.zeros(max(1, int(np.prod(np.maximum(n_bins, 1)))), dtype=torch.float64, device="cuda")
        rc = fn(None, None, None, None, 0, o.ctypes.data_as(_dp), b.ctypes.data_as(_dp),
                n_bins.ctypes.data_as(_ip), counts.data_ptr(), None, None)
        assert rc == -1
        torch.cuda.synchronize()
        assert float(counts.abs().sum()) == 0.0
