"""GPKDE reconstruction: the device implementation (through the C ABI)
against the numpy restatement of the reference, on identical particle
positions (the GPU's own tracked particles)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import mprw
from mprw import workloads as W
from mprw.model import ACTIVE
from oracle import gpkde_oracle as GO


def _positions(tr):
    out = tr.get_particles()
    act = out["status"] == ACTIVE
    return np.stack([out["gx"], out["gy"], out["gz"]], 1)[act]


def test_gpkde_1d_uniform_pulse(gpu_lib):
    g, f, p, opt = W.uniform_pulse(n_particles=20000)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, 50.0)
    co = _positions(tr)
    dens, hist, loops = tr.gpkde((200.0, 1.0, 1.0), (1.0, 1.0, 1.0))
    G = GO.GPKDE((200.0, 1.0, 1.0), (1.0, 1.0, 1.0))
    ref, _ = G.compute_density(co, np.ones(co.shape[0]))
    assert loops == G.loops
    ref_zyx = ref.transpose(2, 1, 0)
    np.testing.assert_allclose(dens, ref_zyx, rtol=0, atol=1e-10 * ref.max())
    assert abs(dens.sum() - co.shape[0]) < 1e-8 * co.shape[0]   # unit volume: mass is conserved
    h, _, _ = GO.histogram_weighted(co, np.ones(co.shape[0]), (0, 0, 0), (1, 1, 1), (200, 1, 1))
    np.testing.assert_array_equal(hist, h)
    tr.close()


def test_gpkde_3d_heterogeneous(gpu_lib):
    g, f, p, opt, info = W.lognormal_slab(n_particles=4000, nlay=4, nrow=12, ncol=30, seed=0, use_torch=False)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, 20.0)
    co = _positions(tr)
    dens, hist, loops = tr.gpkde((30.0, 12.0, 4.0), (1.0, 1.0, 1.0), n_opt_loops=5)
    G = GO.GPKDE((30.0, 12.0, 4.0), (1.0, 1.0, 1.0), n_opt_loops=5)
    ref, _ = G.compute_density(co, np.ones(co.shape[0]))
    assert loops == G.loops
    np.testing.assert_allclose(dens, ref.transpose(2, 1, 0), rtol=0, atol=1e-9 * ref.max())
    assert abs(dens.sum() - co.shape[0]) < 1e-8 * co.shape[0]
    tr.close()


@pytest.mark.parametrize("case", ["1d", "3d"])
def test_gpkde_work_model_matches_the_restatement(gpu_lib, case):
    """mprw_last_gpkde_work -- the multiply-adds direct 3-D kernels would take,
    summed over the optimisation loops -- against the same model counted by
    the numpy restatement from the database kernels each of its loops used
    (the same loops, so the same levels; within 1e-3 for a level taken on
    the other side of a boundary by rounding)."""
    if case == "1d":
        g, f, p, opt = W.uniform_pulse(n_particles=20000)
        t1, dom = 50.0, (200.0, 1.0, 1.0)
        kw = {}
    else:
        g, f, p, opt, info = W.lognormal_slab(n_particles=4000, nlay=4, nrow=12, ncol=30, seed=0, use_torch=False)
        t1, dom = 20.0, (30.0, 12.0, 4.0)
        kw = dict(n_opt_loops=5)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, t1)
    co = _positions(tr)
    dens, hist, loops = tr.gpkde(dom, (1.0, 1.0, 1.0), **kw)
    work = tr.timings()["gpkde_madds"]
    tr.close()
    G = GO.GPKDE(dom, (1.0, 1.0, 1.0), **kw)
    G.compute_density(co, np.ones(co.shape[0]))
    assert loops == G.loops
    assert G.work > 0
    assert abs(work - G.work) <= 1e-3 * G.work, (work, G.work)


def test_gpkde_without_optimisation_loops(gpu_lib):
    """n_opt_loops = 0: the density of the initial smoothing, no loop run --
    the device-driven loop (a while node, whose body would run at least once)
    is not used then -- as the numpy restatement gives it."""
    g, f, p, opt = W.uniform_pulse(n_particles=20000)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, 50.0)
    co = _positions(tr)
    dens, hist, loops = tr.gpkde((200.0, 1.0, 1.0), (1.0, 1.0, 1.0), n_opt_loops=0)
    work = tr.timings()["gpkde_madds"]
    tr.close()
    G = GO.GPKDE((200.0, 1.0, 1.0), (1.0, 1.0, 1.0), n_opt_loops=0)
    ref, _ = G.compute_density(co, np.ones(co.shape[0]))
    assert loops == 0 == G.loops and work == 0
    np.testing.assert_allclose(dens, ref.transpose(2, 1, 0), rtol=0, atol=1e-10 * ref.max())


def test_gpkde_scaling_and_empty(gpu_lib):
    g, f, p, opt = W.uniform_pulse(n_particles=2000)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, 20.0)
    d1, _, _ = tr.gpkde((200.0, 1.0, 1.0), (1.0, 1.0, 1.0), scaling_factor=1.0)
    d2, _, _ = tr.gpkde((200.0, 1.0, 1.0), (1.0, 1.0, 1.0), scaling_factor=0.25)
    np.testing.assert_allclose(d2, 0.25 * d1, rtol=1e-15)
    # a grid outside the plume has no active bins: zero density, no error
    d3, h3, loops = tr.gpkde((10.0, 1.0, 1.0), (1.0, 1.0, 1.0), origin=(150.0, 0.0, 0.0))
    assert np.all(d3 == 0) and np.all(h3 == 0) and loops == 0
    tr.close()


@pytest.mark.parametrize("case", ["1d", "2d", "3d", "3d_isotropic"])
def test_gpkde_fp32_against_fp64(gpu_lib, case):
    """The mixed-precision reconstruction (FP32 passes and per-bin updates,
    FP64 convergence sums) against the FP64 one on the same particles: the
    same number of optimisation loops, the density within 1e-3 of its
    maximum, the mass conserved to FP32 rounding -- in 1-D, 2-D (the
    reference example's 250 x 50 grid) and 3-D, anisotropic and isotropic."""
    from mprw.model import MIXED
    iso = case == "3d_isotropic"
    if case == "1d":
        g, f, p, opt = W.uniform_pulse(n_particles=20000)
        t1, dom, lo = 50.0, (200.0, 1.0, 1.0), 10
    elif case == "2d":
        g, f, p, opt, info = W.lognormal_slab(n_particles=20000, nlay=1, nrow=50, ncol=250, seed=3, use_torch=False)
        t1, dom, lo = 40.0, (250.0, 50.0, 1.0), 10
    else:
        g, f, p, opt, info = W.lognormal_slab(n_particles=20000, nlay=6, nrow=20, ncol=40, seed=1, use_torch=False)
        t1, dom, lo = 30.0, (40.0, 20.0, 6.0), 10
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, t1)
    n = _positions(tr).shape[0]
    d64, h64, l64 = tr.gpkde(dom, (1.0, 1.0, 1.0), n_opt_loops=lo, isotropic=iso)
    d32, h32, l32 = tr.gpkde(dom, (1.0, 1.0, 1.0), n_opt_loops=lo, precision=MIXED, isotropic=iso)
    tr.close()
    np.testing.assert_array_equal(h32, h64)
    assert l32 == l64
    assert np.abs(d32 - d64).max() <= 1e-3 * d64.max()
    assert abs(d32.sum() - n) < 1e-4 * n


@pytest.mark.parametrize("case", ["uniform_pulse", "lognormal_field"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpkde_is_bitwise_repeatable(gpu_lib, case, precision):
    """The same reconstruction of the same particles, run three times, gives
    the same density to the last bit and the same number of optimisation
    loops: the density scatter adds fixed-point integers, so the order in
    which its atomics land does not matter.  The uniform pulse at 50 days
    (1e5 particles, 1-D) and the lognormal slab (200x100x20 cells, 1e6
    particles) after 20 days (3-D)."""
    from mprw.model import MIXED
    prec = MIXED if precision == "mixed" else 0
    if case == "uniform_pulse":
        g, f, p, opt = W.uniform_pulse(n_particles=100_000)
        t1, dom = 50.0, (200.0, 1.0, 1.0)
    else:
        g, f, p, opt, info = W.lognormal_slab(n_particles=1_000_000, seed=0, use_torch=True)
        t1, dom = 20.0, (200.0, 100.0, 20.0)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, t1)
    runs = [tr.gpkde(dom, (1.0, 1.0, 1.0), precision=prec) for _ in range(3)]
    tr.close()
    d0, h0, l0 = runs[0]
    assert d0.max() > 0 and l0 > 0
    for d, h, lo in runs[1:]:
        assert lo == l0
        np.testing.assert_array_equal(h, h0)
        assert np.array_equal(d.view(np.uint64), d0.view(np.uint64))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_host_driven_loop_matches_the_device_loop(gpu_lib, precision):
    """On a stream that can be captured the optimisation loop runs on the
    device (a while node of a CUDA graph whose last kernel takes the
    convergence decision); on the legacy default stream, which cannot be
    captured, the host drives it, reading the convergence scalars after every
    loop.  Both take the same decisions from the same FP64 scalars: the same
    loop count and the same density to the last bit (lognormal slab, 10^6
    particles after 20 days)."""
    from mprw.model import MIXED
    prec = MIXED if precision == "mixed" else 0
    g, f, p, opt, info = W.lognormal_slab(n_particles=1_000_000, seed=0, use_torch=True)
    dom = (200.0, 100.0, 20.0)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, 20.0)
    d_dev, h_dev, l_dev = tr.gpkde(dom, (1.0, 1.0, 1.0), precision=prec)
    launches_dev = tr.timings()["launches"]
    tr.set_stream(1)  # cudaStreamLegacy
    d_host, h_host, l_host = tr.gpkde(dom, (1.0, 1.0, 1.0), precision=prec)
    launches_host = tr.timings()["launches"]
    tr.set_stream(0)
    tr.close()
    assert l_dev == l_host > 0
    np.testing.assert_array_equal(h_dev, h_host)
    assert np.array_equal(d_dev.view(np.uint64), d_host.view(np.uint64))
    # the device loop adds its decision kernel per loop
    assert launches_dev > launches_host


@pytest.mark.parametrize("isotropic", [False, True], ids=["anisotropic", "isotropic"])
def test_gpkde_2d_on_the_reference_example_grid(gpu_lib, isotropic):
    """2-D reconstruction on the grid of the reference's GPKDE example
    (examples/ex07_mf6/ex07a_mf6.gpkde: 250 x 50 x 1 bins of 1 m), on a 2-D
    lognormal field of that shape (the lognormal-slab generator with one
    layer) after 40 days: the same loop count as the numpy restatement
    (prComputeNetRoughness2D, the 2-D isotropy correction and shapes), the
    density within 1e-10 of its maximum, mass conserved."""
    g, f, p, opt, info = W.lognormal_slab(n_particles=20000, nlay=1, nrow=50, ncol=250, seed=3, use_torch=False)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, 40.0)
    co = _positions(tr)
    dens, hist, loops = tr.gpkde((250.0, 50.0, 1.0), (1.0, 1.0, 1.0), isotropic=isotropic)
    tr.close()
    G = GO.GPKDE((250.0, 50.0, 1.0), (1.0, 1.0, 1.0), isotropic=isotropic)
    assert G.ndim == 2
    ref, _ = G.compute_density(co, np.ones(co.shape[0]))
    assert loops == G.loops
    np.testing.assert_allclose(dens, ref.transpose(2, 1, 0), rtol=0, atol=1e-10 * ref.max())
    assert abs(dens.sum() - co.shape[0]) < 1e-8 * co.shape[0]


def test_gpkde_2d_xz_and_3d_isotropic(gpu_lib):
    """The other 2-D orientation (x-z: one row) and the isotropic option in
    3-D, against the numpy restatement."""
    g, f, p, opt, info = W.lognormal_slab(n_particles=6000, nlay=8, nrow=1, ncol=60, seed=4, use_torch=False)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, 30.0)
    co = _positions(tr)
    dens, _, loops = tr.gpkde((60.0, 1.0, 8.0), (1.0, 1.0, 1.0))
    tr.close()
    G = GO.GPKDE((60.0, 1.0, 8.0), (1.0, 1.0, 1.0))
    assert G.dims == [0, 2]
    ref, _ = G.compute_density(co, np.ones(co.shape[0]))
    assert loops == G.loops
    np.testing.assert_allclose(dens, ref.transpose(2, 1, 0), rtol=0, atol=1e-10 * ref.max())

    g, f, p, opt, info = W.lognormal_slab(n_particles=4000, nlay=4, nrow=12, ncol=30, seed=0, use_torch=False)
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.advance(0.0, 20.0)
    co = _positions(tr)
    dens, _, loops = tr.gpkde((30.0, 12.0, 4.0), (1.0, 1.0, 1.0), n_opt_loops=5, isotropic=True)
    tr.close()
    G = GO.GPKDE((30.0, 12.0, 4.0), (1.0, 1.0, 1.0), n_opt_loops=5, isotropic=True)
    ref, _ = G.compute_density(co, np.ones(co.shape[0]))
    assert loops == G.loops
    np.testing.assert_allclose(dens, ref.transpose(2, 1, 0), rtol=0, atol=1e-9 * ref.max())
