"""The torch restatement of the differentiable walk (oracle/adjoint_oracle.py)
on the CPU: its automatic gradient of a density misfit against central
differences of its own forward model (relative step 1e-5, the same normals),
on a small lognormal field with 8 zones (25 parameters).  This pins the
reference gradient that the GPU adjoint is checked against."""
import numpy as np
import torch

from adjoint_cases import base_theta, block_zones, field
from oracle import adjoint_oracle as A
from oracle import oracle as O

EPS = 0.05  # velocity floor of the dispersion tensor (m/d)


def test_restatement_gradient_matches_central_differences():
    g, f, p, opt = field(nlay=4, nrow=6, ncol=12, n_particles=40, seed=2, x_release=3.0)
    zones = block_zones(g)
    ns = A.node_setup(g, f, opt, zones, 8)
    gx, gy, gz = O.global_xyz(g, f, p)
    x0 = torch.tensor(np.stack([gx, gy, gz], 1))
    d = (1.0, 1.0, 1.0)
    lo = (0.0, 0.0, float(g.botm[-1]))
    normals = A.philox_walk_normals(11, p.id, 15)
    mass = torch.ones(p.n, dtype=torch.float64)
    grid = dict(origin=(0.0, 0.0, lo[2]), bin_size=(1.0, 1.0, 1.0), n_bins=(12, 6, 4), h=(1.5, 1.5, 1.0))

    def loss(theta, target=None):
        nodes = A.node_fields(ns, theta, 8, d, EPS)
        rho = A.deposit(A.walk(ns, nodes, x0, normals, 0.1, lo, d, EPS), mass, **grid)
        return rho if target is None else ((rho - target) ** 2).sum()

    th0 = base_theta()
    target = loss(torch.tensor(th0 * 1.1)).detach()
    th = torch.tensor(th0, requires_grad=True)
    L = loss(th, target)
    L.backward()
    grad = th.grad.numpy()
    fd = np.empty_like(th0)
    for k in range(th0.size):
        h = 1e-5 * abs(th0[k])
        e = np.zeros_like(th0)
        e[k] = h
        fd[k] = (loss(torch.tensor(th0 + e), target).item() - loss(torch.tensor(th0 - e), target).item()) / (2 * h)
    assert np.abs(fd).max() > 0
    assert np.linalg.norm(grad - fd) <= 1e-4 * np.linalg.norm(fd)
