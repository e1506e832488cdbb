"""torch restatement of the differentiable random walk (TEST INFRASTRUCTURE ONLY).

The library's differentiable walk (mprw_adj_setup / _forward / _backward,
adjoint.cu) has no counterpart in the reference; this module restates its
forward model independently, in FP64 torch operations, so that torch's
automatic differentiation gives a reference gradient for the hand-written
adjoint.  The model:

* node lattice of cell corners; per node the Darcy flux averaged over the
  adjacent active cells' faces that meet at the node (face velocities of
  the oracle's cell record times porosity and retardation), the zone shares
  of those cells, and their mean Dm / R;
* theta = (alphaL per zone, alphaT per zone, porosity per zone, velocity
  scale s): node porosity and dispersivities are share-weighted sums, u = s q
  / (phi R), r = sqrt(|u|^2 + eps^2) (eps the velocity floor), phi D = phi
  ((alphaT r + Dm/R) I + (alphaL - alphaT) u u^T / r), G = div(phi D) / phi by
  central differences (one-sided at the ends);
* a step: trilinear interpolation of u, G, alphaL, alphaT, Dm/R at the
  position, x' = fold(x + (u + G) dt + B xi sqrt(dt)), B xi = a xi + kappa
  (u . xi) u with a = sqrt(2 (alphaT r + Dm/R)), b = sqrt(2 (alphaT r + Dm/R
  + (alphaL - alphaT) |u|^2 / r)), kappa = 2 (alphaL - alphaT) / (r (a + b)),
  so that B B^T = 2 D; fold the reflection at both walls of every axis;
* xi: the Philox Irwin-Hall normals of the oracle (oracle.philox_normals)
  keyed by (seed, particle id) at counter 9 * step;
* density: sum over particles of mass times the product over dimensions with
  several bins of the biweight (15/16h)(1 - (r/h)^2)^2 at the bin centres.

It is written for small cases (every particle against every bin).
"""
from __future__ import annotations

import numpy as np
import torch

from oracle import oracle as O


def node_setup(grid, flow, opt, zones, nzones):
    """Node Darcy flux (nn, 3), zone shares (nn, nzones), Dm / R (nn) and the
    lattice shape (n0, n1, n2) cells along model x, y, z."""
    n0, n1, n2 = grid.ncol, grid.nrow, grid.nlay
    shp = (n2 + 1, n1 + 1, n0 + 1)
    q = np.zeros(shp + (3,))
    beta = np.zeros(shp + (nzones,))
    dm = np.zeros(shp)
    cnt = np.zeros(shp)
    dm_cell = np.asarray(flow.dm_eff, np.float64)
    R = float(np.asarray(flow.retardation)[0])
    for k in range(n2):
        for i in range(n1):
            for j in range(n0):
                c = k * n1 * n0 + i * n0 + j
                if flow.iboundts[c] == 0:
                    continue
                rec = O.cell_record(grid, flow, opt, c + 1)
                v = rec["vface"] * float(flow.porosity[c]) * float(flow.retardation[c])
                cx, cy, cz = j, n1 - 1 - i, n2 - 1 - k
                for oz in (0, 1):
                    for oy in (0, 1):
                        for ox in (0, 1):
                            nd = (cz + oz, cy + oy, cx + ox)
                            q[nd] += (v[0] if ox == 0 else v[1], v[2] if oy == 0 else v[3],
                                      v[4] if oz == 0 else v[5])
                            beta[nd + (int(zones[c]),)] += 1.0
                            dm[nd] += dm_cell[0] if dm_cell.size == 1 else dm_cell[c]
                            cnt[nd] += 1.0
    inv = np.where(cnt > 0, 1.0 / np.maximum(cnt, 1.0), 0.0)
    q *= inv[..., None]
    beta *= inv[..., None]
    dm *= inv / R
    return dict(q=torch.tensor(q.reshape(-1, 3)), beta=torch.tensor(beta.reshape(-1, nzones)),
                dmr=torch.tensor(dm.reshape(-1)), n=(n0, n1, n2), R=R)


def _fd(f, axis, h):
    """Difference quotient of f (shaped (n2+1, n1+1, n0+1)) along a lattice axis
    (0 = z, 1 = y, 2 = x): central inside, one-sided at the ends."""
    m = f.shape[axis] - 1
    fm = torch.movedim(f, axis, 0)
    out = torch.empty_like(fm)
    out[0] = (fm[1] - fm[0]) / h
    out[m] = (fm[m] - fm[m - 1]) / h
    if m > 1:
        out[1:m] = (fm[2:] - fm[:-2]) * (0.5 / h)
    return torch.movedim(out, 0, axis)


def node_fields(ns, theta, nz, d, eps):
    """Node records (nn, 9): u (3), G (3), alphaL, alphaT, Dm / R."""
    n0, n1, n2 = ns["n"]
    aL = ns["beta"] @ theta[:nz]
    aT = ns["beta"] @ theta[nz:2 * nz]
    phi = ns["beta"] @ theta[2 * nz:3 * nz]
    s = theta[3 * nz]
    u = s * ns["q"] / (phi * ns["R"])[:, None]
    r = torch.sqrt((u * u).sum(1) + eps * eps)
    iso = aT * r + ns["dmr"]
    an = (aL - aT) / r
    P = [phi * (iso + an * u[:, 0] * u[:, 0]), phi * (iso + an * u[:, 1] * u[:, 1]),
         phi * (iso + an * u[:, 2] * u[:, 2]), phi * an * u[:, 0] * u[:, 1], phi * an * u[:, 0] * u[:, 2],
         phi * an * u[:, 1] * u[:, 2]]
    shp = (n2 + 1, n1 + 1, n0 + 1)
    comp = {(0, 0): 0, (1, 1): 1, (2, 2): 2, (0, 1): 3, (1, 0): 3, (0, 2): 4, (2, 0): 4, (1, 2): 5, (2, 1): 5}
    lat = {0: 2, 1: 1, 2: 0}  # model axis -> lattice axis
    G = []
    for i in range(3):
        g = 0.0
        for j in range(3):
            g = g + _fd(P[comp[(i, j)]].reshape(shp), lat[j], d[j])
        G.append(g.reshape(-1) / phi)
    return torch.stack([u[:, 0], u[:, 1], u[:, 2], G[0], G[1], G[2], aL, aT, ns["dmr"]], 1)


def _fold(y, lo, L):
    P = 2.0 * L
    t = y - lo
    t = t - torch.floor((t / P).detach()) * P
    return lo + torch.where(t > L, P - t, t)


def walk(ns, nodes, x0, normals, dt, lo, d, eps):
    """Positions after len(normals) steps; normals shaped (nsteps, np, 3)."""
    n0, n1, n2 = ns["n"]
    nmax = torch.tensor([n0 - 1, n1 - 1, n2 - 1], dtype=torch.float64)
    lo_t = torch.tensor(lo, dtype=torch.float64)
    d_t = torch.tensor(d, dtype=torch.float64)
    x = x0
    sdt = float(np.sqrt(dt))
    corners = [(ox, oy, oz) for oz in (0, 1) for oy in (0, 1) for ox in (0, 1)]
    for k in range(normals.shape[0]):
        t = (x - lo_t) / d_t
        c = torch.minimum(torch.clamp(torch.floor(t.detach()), min=0.0), nmax)
        f = torch.clamp(t - c, 0.0, 1.0)
        ci = c.long()
        val = 0.0
        for ox, oy, oz in corners:
            w = (f[:, 0] if ox else 1 - f[:, 0]) * (f[:, 1] if oy else 1 - f[:, 1]) * (f[:, 2] if oz else 1 - f[:, 2])
            nid = (ci[:, 0] + ox) + (n0 + 1) * ((ci[:, 1] + oy) + (n1 + 1) * (ci[:, 2] + oz))
            val = val + w[:, None] * nodes[nid]
        u, G, aL, aT, dm = val[:, 0:3], val[:, 3:6], val[:, 6], val[:, 7], val[:, 8]
        s2 = (u * u).sum(1)
        r = torch.sqrt(s2 + eps * eps)
        lt = aT * r + dm
        ll = lt + (aL - aT) * s2 / r
        a = torch.sqrt(2.0 * lt)
        b = torch.sqrt(2.0 * ll)
        kappa = 2.0 * (aL - aT) / (r * (a + b))
        xi = normals[k]
        P = (u * xi).sum(1)
        bxi = a[:, None] * xi + (kappa * P)[:, None] * u
        y = x + (u + G) * dt + bxi * sdt
        x = torch.stack([_fold(y[:, dd], lo[dd], ns["n"][dd] * d[dd]) for dd in range(3)], 1)
    return x


def deposit(x, mass, origin, bin_size, n_bins, h):
    """Density on the grid, shaped (nz, ny, nx)."""
    fac = []
    for dd in range(3):
        if n_bins[dd] == 1:
            fac.append(torch.ones(x.shape[0], 1, dtype=torch.float64))
            continue
        centre = origin[dd] + (torch.arange(n_bins[dd], dtype=torch.float64) + 0.5) * bin_size[dd]
        r = (centre[None, :] - x[:, dd:dd + 1]) / h[dd]
        k = torch.where(r.abs() < 1.0, (15.0 / (16.0 * h[dd])) * (1.0 - r * r) ** 2, torch.zeros_like(r))
        fac.append(k)
    return torch.einsum("p,pk,pj,pi->kji", mass, fac[2], fac[1], fac[0])


def philox_walk_normals(seed, ids, nsteps):
    """(nsteps, np, 3) normals: particle id, counter 9 * step (three Irwin-Hall normals per step)."""
    out = np.empty((nsteps, len(ids), 3))
    for p, pid in enumerate(ids):
        v, _ = O.philox_normals(seed, int(pid), 3 * nsteps, 0)
        out[:, p, :] = v.reshape(nsteps, 3)
    return torch.tensor(out)
