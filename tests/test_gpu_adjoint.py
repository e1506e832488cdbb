"""The differentiable walk and its hand-written adjoint on the GPU
(mprw_adj_setup / mprw_adj_forward / mprw_adj_backward).

The adjoint is reached through the C ABI and wrapped here, in the test
harness only, in a torch.autograd.Function, so that a density misfit
L = sum (rho(theta) - rho*)^2 is differentiated by loss.backward() as any
torch model would be.  Checked:

* against an independent reference gradient: the torch restatement of the
  same walk (oracle/adjoint_oracle.py, FP64, the same Philox normals)
  differentiated by torch's autograd, on a small lognormal field -- the
  density to 1e-12 and the gradient to 1e-9 of their maxima;
* against central finite differences of the library's own forward run
  (relative step 1e-5, common random numbers) on a reduced version of the
  adjoint workload: the lognormal field generator (sigma2 lnK 1) at
  40 x 20 x 8 cells, 8 zones (2 x 2 x 2 blocks) -- 25 parameters: alphaL,
  alphaT, porosity per zone and a velocity scale -- 20,000 particles
  released at 4-10 m, 120 steps of 0.02 d stored every 30 steps (the plume
  travels about three cells), target made by the same run with every
  parameter +10 %: agreement to 1e-3 relative (norm of the difference over
  the norm of the finite-difference gradient, and each component within
  1e-3 of the largest).  The step is 1e-5 because the differences' own
  truncation error is the larger one at 1e-4: on the torch restatement of
  this case (3,000 particles) central differences agree with autograd to
  7.7e-4 of the largest component at 1e-4 and to 1.7e-5 at 1e-5;
* the checkpoint interval changes nothing (stored every step, every 30
  steps, or once);
* a small step along the negative gradient lowers the misfit.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import mprw
from adjoint_cases import base_theta, block_zones, field
from oracle import adjoint_oracle as A

EPS = 0.05  # velocity floor of the dispersion tensor (m/d)


class WalkDensity(torch.autograd.Function):
    """rho(theta) of the library's differentiable walk; backward = mprw_adj_backward."""

    @staticmethod
    def forward(ctx, theta, tracker):
        ctx.tracker = tracker
        return torch.from_numpy(tracker.adj_forward(theta.detach().numpy()).copy())

    @staticmethod
    def backward(ctx, grad_rho):
        g = ctx.tracker.adj_backward(grad_rho.detach().contiguous().numpy())
        return torch.from_numpy(g), None


def misfit(tracker, theta, target):
    rho = WalkDensity.apply(theta, tracker)
    return ((rho - target) ** 2).sum()


def _tracker(g, f, opt, p, zones, nsteps, checkpoint, dt, grid, seed=11):
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    tr.set_particles(p)
    tr.adj_setup(zones, 8, dt, nsteps, checkpoint, grid["origin"], grid["bin_size"], grid["n_bins"], grid["h"], EPS,
                 seed=seed)
    return tr


def test_adjoint_matches_autograd_of_the_restatement(gpu_lib):
    g, f, p, opt = field(nlay=4, nrow=6, ncol=12, n_particles=150, seed=2, x_release=3.0)
    zones = block_zones(g)
    lo = (0.0, 0.0, float(g.botm[-1]))
    grid = dict(origin=lo, bin_size=(1.0, 1.0, 1.0), n_bins=(12, 6, 4), h=(1.5, 1.5, 1.0))
    nsteps, dt = 40, 0.1
    tr = _tracker(g, f, opt, p, zones, nsteps, 10, dt, grid)
    th0 = base_theta()
    target = torch.from_numpy(tr.adj_forward(th0 * 1.1).copy())
    theta = torch.tensor(th0, requires_grad=True)
    L = misfit(tr, theta, target)
    L.backward()
    g_gpu = theta.grad.numpy().copy()
    rho_gpu = tr.adj_forward(th0)
    q = tr.get_particles()
    tr.close()
    # the restatement, from the same start positions and normals
    ns = A.node_setup(g, f, opt, zones, 8)
    x0 = torch.tensor(np.stack([q["gx"], q["gy"], q["gz"]], 1))
    normals = A.philox_walk_normals(11, p.id, nsteps)
    th = torch.tensor(th0, requires_grad=True)
    nodes = A.node_fields(ns, th, 8, (1.0, 1.0, 1.0), EPS)
    rho_t = A.deposit(A.walk(ns, nodes, x0, normals, dt, lo, (1.0, 1.0, 1.0), EPS),
                      torch.ones(p.n, dtype=torch.float64), **grid)
    np.testing.assert_allclose(rho_gpu, rho_t.detach().numpy(), rtol=0, atol=1e-12 * rho_gpu.max())
    Lt = ((rho_t - target) ** 2).sum()
    Lt.backward()
    g_ref = th.grad.numpy()
    assert np.abs(g_ref).max() > 0
    np.testing.assert_allclose(g_gpu, g_ref, rtol=0, atol=1e-9 * np.abs(g_ref).max())


def _config4_small():
    g, f, p, opt = field(nlay=8, nrow=20, ncol=40, n_particles=20_000, seed=1, x_release=10.0, x0=4.0)
    zones = block_zones(g)
    lo = (0.0, 0.0, float(g.botm[-1]))
    grid = dict(origin=lo, bin_size=(1.0, 1.0, 1.0), n_bins=(40, 20, 8), h=(2.0, 2.0, 1.5))
    return g, f, opt, p, zones, grid


def test_adjoint_matches_central_differences(gpu_lib):
    g, f, opt, p, zones, grid = _config4_small()
    nsteps, dt = 120, 0.02
    tr = _tracker(g, f, opt, p, zones, nsteps, 30, dt, grid)
    th0 = base_theta(seed=3)
    target = torch.from_numpy(tr.adj_forward(th0 * 1.1).copy())
    theta = torch.tensor(th0, requires_grad=True)
    L0 = misfit(tr, theta, target)
    L0.backward()
    grad = theta.grad.numpy().copy()
    fd = np.empty_like(th0)
    for k in range(th0.size):
        h = 1e-5 * abs(th0[k])
        e = np.zeros_like(th0)
        e[k] = h
        lp = float(((torch.from_numpy(tr.adj_forward(th0 + e).copy()) - target) ** 2).sum())
        lm = float(((torch.from_numpy(tr.adj_forward(th0 - e).copy()) - target) ** 2).sum())
        fd[k] = (lp - lm) / (2 * h)
    assert np.abs(fd).max() > 0
    assert np.linalg.norm(grad - fd) <= 1e-3 * np.linalg.norm(fd), (grad, fd)
    assert np.abs(grad - fd).max() <= 1e-3 * np.abs(fd).max(), (grad, fd)
    # a small step down the gradient lowers the misfit
    step = 1e-2 * np.abs(th0).min() / np.abs(grad).max()
    l1 = float(((torch.from_numpy(tr.adj_forward(th0 - step * grad).copy()) - target) ** 2).sum())
    assert l1 < float(L0)
    tr.close()


def test_checkpoint_interval_changes_nothing(gpu_lib):
    g, f, opt, p, zones, grid = _config4_small()
    nsteps, dt = 120, 0.02
    th0 = base_theta(seed=4)
    out = []
    for ck in (1, 30, 120):
        tr = _tracker(g, f, opt, p, zones, nsteps, ck, dt, grid)
        rho = tr.adj_forward(th0)
        gr = tr.adj_backward(2.0 * (rho - 0.9 * rho))
        out.append((rho, gr))
        tr.close()
    for rho, gr in out[1:]:
        assert np.array_equal(rho, out[0][0])
        np.testing.assert_allclose(gr, out[0][1], rtol=0, atol=1e-12 * np.abs(out[0][1]).max())
