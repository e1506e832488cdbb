"""Synthetic inputs for the tracking path (no external data is used).

* ``uniform_flow``: a structured grid with uniform specific discharge along
  +x, the inflow/outflow carried by face-assigned boundary flows (IFACE 1/2)
  so that every cell has the same face flows.
* ``lognormal_field``: a seeded Gaussian log-conductivity field with
  exponential covariance, drawn by circulant embedding (FFT) on a periodic
  grid twice the model size and cropped.
* ``steady_heads``: the 7-point finite-volume steady head solve (harmonic
  inter-cell conductance) with fixed heads at the two x-ends and no flow
  elsewhere, solved in FP64 by Jacobi-preconditioned conjugate gradients to a
  relative residual of 1e-12; returns MODFLOW 6 FLOW-JA-FACE in IA/JA form and
  the constant-head budget as per-cell source/sink flows.

The particle releases are seeded uniform local coordinates in the release
cells, unit mass.
"""
from __future__ import annotations

import numpy as np

from .model import ADV, EULERIAN, FP64, MIN_ADV_DISP, MIXED, PENDING, Flow, Grid, Options, Particles


def structured_grid(nlay, nrow, ncol, dx=1.0, dy=1.0, dz=1.0, top=None) -> Grid:
    delr = np.full(ncol, float(dx))
    delc = np.full(nrow, float(dy))
    ztop = float(nlay * dz) if top is None else float(top)
    topa = np.full(nrow * ncol, ztop)
    botm = np.concatenate([np.full(nrow * ncol, ztop - (k + 1) * dz) for k in range(nlay)])
    return Grid(nlay, nrow, ncol, delr, delc, topa, botm)


def dis_connectivity(grid: Grid):
    """IA/JA (1-based, diagonal first, ascending neighbours) of a full DIS grid,
    plus for every off-diagonal entry the 0-based neighbour and its face."""
    nl, nr, nc = grid.nlay, grid.nrow, grid.ncol
    n = grid.ncell
    idx = np.arange(n)
    k, rem = np.divmod(idx, nr * nc)
    i, j = np.divmod(rem, nc)
    # candidate neighbours in ascending node order: top(k-1), back(i-1), left(j-1), right, front, bottom
    cand = [(idx - nr * nc, k > 0), (idx - nc, i > 0), (idx - 1, j > 0), (idx + 1, j < nc - 1),
            (idx + nc, i < nr - 1), (idx + nr * nc, k < nl - 1)]
    counts = 1 + sum(m.astype(np.int64) for _, m in cand)
    ia = np.zeros(n + 1, np.int64)
    ia[1:] = np.cumsum(counts)
    ja = np.empty(ia[-1], np.int64)
    pos = ia[:-1].copy()
    ja[pos] = idx
    pos += 1
    for nb, m in cand:
        ja[pos[m]] = nb[m]
        pos[m] += 1
    return (ia + 1).astype(np.int32), (ja + 1).astype(np.int32)


def uniform_flow(ncol=200, nrow=1, nlay=1, q=0.3, porosity=0.3, dx=1.0, dy=1.0, dz=1.0, alpha_l=0.1,
                 alpha_t=0.01, dm=0.0):
    """Uniform specific discharge q along +x (seepage velocity q/porosity)."""
    g = structured_grid(nlay, nrow, ncol, dx, dy, dz)
    ia, ja = dis_connectivity(g)
    n = g.ncell
    area = dy * dz
    Q = q * area
    flowja = np.zeros(ja.shape[0])
    rows = np.repeat(np.arange(n), np.diff(ia))
    m = ja - 1
    flowja[m == rows - 1] = Q    # from the left neighbour into the cell
    flowja[m == rows + 1] = -Q   # out to the right neighbour
    bflow = np.zeros(6 * n)
    col = np.arange(n) % ncol
    bflow[6 * np.where(col == 0)[0] + 0] = Q            # IFACE 1 inflow
    bflow[6 * np.where(col == ncol - 1)[0] + 1] = -Q    # IFACE 2 outflow
    flow = Flow(ia=ia, ja=ja, flowja=flowja, porosity=np.full(n, porosity), retardation=np.ones(n),
                iboundts=np.ones(n, np.int32), alpha_l=np.array([alpha_l]), alpha_t=np.array([alpha_t]),
                dm_eff=np.array([dm]), uniform_dispersion=True, steady_state=True, default_icbound=1,
                boundary_flows=bflow)
    return g, flow


def graded_flow(ncol=40, q0=0.3, ratio=1.05, porosity=0.3):
    """1-D column whose face flux grows geometrically, Q_i = q0 * ratio**i through
    the left face of cell i (0-based), balanced by a source in every cell: the
    velocity is linear inside each cell with v2 = ratio * v1, the field in which
    exponential advection is exact.  No dispersion."""
    g, f = uniform_flow(ncol=ncol, q=q0, porosity=porosity, alpha_l=0.0, alpha_t=0.0, dm=0.0)
    n = g.ncell
    Q = q0 * ratio ** np.arange(n + 1)
    rows = np.repeat(np.arange(n), np.diff(f.ia))
    m = f.ja - 1
    flowja = np.zeros(f.ja.shape[0])
    flowja[m == rows - 1] = Q[rows[m == rows - 1]]           # in through the left face
    flowja[m == rows + 1] = -Q[rows[m == rows + 1] + 1]      # out through the right face
    f.flowja = flowja
    bflow = np.zeros(6 * n)
    bflow[0] = Q[0]
    bflow[6 * (n - 1) + 1] = -Q[n]
    f.boundary_flows = bflow
    f.source_flow = Q[1:] - Q[:-1]
    return g, f, Q


def graded_flow_exact(x0, t, Q, porosity=0.3, dx=1.0):
    """Exact position at time t of a particle starting at x0 (m) in graded_flow:
    within a cell v(p) = v1 + g p, p(t) = (v(p0)/g)(e^{g t} - 1) + p0, and the
    travel time to the right face is ln(v2/v(p0))/g."""
    x, rem = float(x0), float(t)
    n = Q.shape[0] - 1
    while True:
        i = min(int(np.floor(x / dx)), n - 1)
        p0 = x - i * dx
        v1, v2 = Q[i] / (porosity * dx * dx), Q[i + 1] / (porosity * dx * dx)
        gr = (v2 - v1) / dx
        vp = v1 + gr * p0
        tau = np.log(v2 / vp) / gr
        if tau >= rem or i == n - 1:
            return i * dx + p0 + (vp / gr) * np.expm1(gr * rem)
        rem -= tau
        x = (i + 1) * dx


def lognormal_field(nlay, nrow, ncol, sigma2=1.0, kg=10.0, lh=10.0, lv=2.0, d=1.0, seed=0) -> np.ndarray:
    """ln K ~ N(ln kg, sigma2), exponential covariance; shape (nlay, nrow, ncol)."""
    rng = np.random.default_rng(seed)
    shp = (2 * nlay, 2 * nrow, 2 * ncol)
    ax = [np.minimum(np.arange(s), s - np.arange(s)) * d for s in shp]
    z, y, x = np.meshgrid(ax[0], ax[1], ax[2], indexing="ij")
    r = np.sqrt((x / lh) ** 2 + (y / lh) ** 2 + (z / lv) ** 2)
    cov = sigma2 * np.exp(-r)
    lam = np.fft.fftn(cov).real
    lam[lam < 0] = 0.0
    w = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
    f = np.fft.ifftn(np.sqrt(lam) * w) * np.sqrt(np.prod(shp))
    field = f.real[:nlay, :nrow, :ncol]
    return kg * np.exp(field)


def _cg(apply, b, diag, rtol=1e-12, maxiter=200000, xp=np):
    x = xp.zeros_like(b)
    r = b - apply(x)
    z = r / diag
    p = z.clone() if hasattr(z, "clone") else z.copy()
    rz = float((r * z).sum())
    bn = float(xp.sqrt((b * b).sum()))
    if bn == 0:
        return x, 0
    for it in range(1, maxiter + 1):
        Ap = apply(p)
        alpha = rz / float((p * Ap).sum())
        x += alpha * p
        r -= alpha * Ap
        if float(xp.sqrt((r * r).sum())) <= rtol * bn:
            return x, it
        z = r / diag
        rz_new = float((r * z).sum())
        p = z + (rz_new / rz) * p
        rz = rz_new
    raise RuntimeError("CG did not converge")


def steady_heads(grid: Grid, K: np.ndarray, h_left=1.0, h_right=0.0, rtol=1e-12, use_torch=None):
    """Steady heads, FLOW-JA-FACE, CHD source/sink flows for fixed-head x-ends."""
    nl, nr, nc = grid.nlay, grid.nrow, grid.ncol
    n = grid.ncell
    dx, dy = float(grid.delr[0]), float(grid.delc[0])
    dz = float(grid.top[0] - grid.botm[0])
    Kf = K.reshape(-1).astype(np.float64)
    ia, ja = dis_connectivity(grid)
    rows = np.repeat(np.arange(n), np.diff(ia))
    m = ja.astype(np.int64) - 1
    off = m != rows
    r_o, m_o = rows[off], m[off]
    kh = 2.0 * Kf[r_o] * Kf[m_o] / (Kf[r_o] + Kf[m_o])
    dn = m_o - r_o
    area_len = np.where(np.abs(dn) == 1, dy * dz / dx, np.where(np.abs(dn) == nc, dx * dz / dy, dx * dy / dz))
    cond = kh * area_len
    col = np.arange(n) % nc
    fixed = (col == 0) | (col == nc - 1)
    hfix = np.where(col == 0, h_left, h_right)
    free = ~fixed
    fidx = -np.ones(n, np.int64)
    fidx[free] = np.arange(free.sum())
    diag = np.zeros(n)
    np.add.at(diag, r_o, cond)
    # A h_free = b on free cells: diag*h_i - sum_j c_ij h_j (free j); b = sum_j c_ij hfix_j (fixed j)
    sel = free[r_o]
    rr, mm, cc = r_o[sel], m_o[sel], cond[sel]
    ff = free[mm]
    b = np.zeros(free.sum())
    np.add.at(b, fidx[rr[~ff]], cc[~ff] * hfix[mm[~ff]])
    dg = diag[free]
    if use_torch is None:
        use_torch = n > 200_000
    if use_torch:
        import torch
        dev = "cuda" if torch.cuda.is_available() else "cpu"
        ri = torch.as_tensor(fidx[rr[ff]], device=dev)
        ci = torch.as_tensor(fidx[mm[ff]], device=dev)
        vals = torch.as_tensor(-cc[ff], device=dev, dtype=torch.float64)
        nf = int(free.sum())
        A = torch.sparse_coo_tensor(torch.stack([ri, ci]), vals, (nf, nf)).coalesce().to_sparse_csr()
        dgt = torch.as_tensor(dg, device=dev)
        bt = torch.as_tensor(b, device=dev)
        apply = lambda v: dgt * v + (A @ v.unsqueeze(1)).squeeze(1)
        x, it = _cg(apply, bt, dgt, rtol=rtol, xp=torch)
        hf = x.cpu().numpy()
    else:
        import scipy.sparse as sp
        nf = int(free.sum())
        A = sp.csr_matrix((-cc[ff], (fidx[rr[ff]], fidx[mm[ff]])), shape=(nf, nf))
        apply = lambda v: dg * v + A @ v
        hf, it = _cg(apply, b, dg, rtol=rtol)
    h = hfix.copy().astype(np.float64)
    h[free] = hf
    flowja = np.zeros(ja.shape[0])
    flowja[np.where(off)[0]] = cond * (h[m_o] - h[r_o])
    net = np.zeros(n)
    np.add.at(net, r_o, cond * (h[m_o] - h[r_o]))   # net flow into the cell from neighbours
    chd = np.where(fixed, -net, 0.0)                 # constant-head budget (+ into the model)
    source = np.where(chd > 0, chd, 0.0)
    sink = np.where(chd < 0, chd, 0.0)
    return dict(heads=h, ia=ia, ja=ja, flowja=flowja, source_flow=source, sink_flow=sink, cg_iterations=it)


def heterogeneous_flow(nlay=20, nrow=100, ncol=200, sigma2=1.0, kg=10.0, lh=10.0, lv=2.0, porosity=0.25,
                       alpha_l=0.5, alpha_t=0.05, dm=1e-4, seed=0, use_torch=None):
    g = structured_grid(nlay, nrow, ncol)
    K = lognormal_field(nlay, nrow, ncol, sigma2, kg, lh, lv, seed=seed)
    s = steady_heads(g, K, use_torch=use_torch)
    n = g.ncell
    flow = Flow(ia=s["ia"], ja=s["ja"], flowja=s["flowja"], porosity=np.full(n, porosity), retardation=np.ones(n),
                iboundts=np.ones(n, np.int32), alpha_l=np.array([alpha_l]), alpha_t=np.array([alpha_t]),
                dm_eff=np.array([dm]), uniform_dispersion=True, steady_state=True, default_icbound=1,
                heads=s["heads"], source_flow=s["source_flow"], sink_flow=s["sink_flow"])
    return g, flow, dict(K=K, cg_iterations=s["cg_iterations"])


def release_in_box(grid: Grid, n: int, x0, x1, y0, y1, z0, z1, seed=1000, t0=0.0, status=PENDING) -> Particles:
    """n unit-mass particles uniform in the box [x0,x1]x[y0,y1]x[z0,z1] (model coordinates,
    y measured from the front edge, z from the grid bottom), located by cell + local coords."""
    rng = np.random.default_rng(seed)
    X = rng.uniform(x0, x1, n)
    Y = rng.uniform(y0, y1, n)
    Z = rng.uniform(z0, z1, n)
    xe = np.concatenate([[0.0], np.cumsum(grid.delr)])
    ytot = float(np.sum(grid.delc))
    ye = ytot - np.concatenate([[0.0], np.cumsum(grid.delc)])     # row i spans [ye[i+1], ye[i]]
    j = np.clip(np.searchsorted(xe, X, side="right") - 1, 0, grid.ncol - 1)
    i = np.clip(np.searchsorted(-ye, -Y, side="left") - 1, 0, grid.nrow - 1)
    ztop = grid.top[0]
    zb = np.concatenate([[ztop], grid.botm[:: grid.nrow * grid.ncol]])
    k = np.clip(np.searchsorted(-zb, -Z, side="left") - 1, 0, grid.nlay - 1)
    lx = (X - xe[j]) / grid.delr[j]
    ly = (Y - ye[i + 1]) / grid.delc[i]
    lz = (Z - zb[k + 1]) / (zb[k] - zb[k + 1])
    cell = grid.node(k, i, j).astype(np.int32)
    return Particles(cell=cell, lx=np.clip(lx, 0, 1), ly=np.clip(ly, 0, 1), lz=np.clip(lz, 0, 1),
                     t=np.full(n, float(t0)), status=np.full(n, status, np.int32), mass=np.ones(n),
                     id=np.arange(n, dtype=np.uint64), rng_ctr=np.zeros(n, np.uint64))


def uniform_pulse(n_particles=100_000, pure_advection=False, precision=FP64):
    """200x1x1 uniform flow, v = 1 m/d, pulse at x = 10 m, Courant 0.1 (ADV)."""
    aL, aT = (0.0, 0.0) if pure_advection else (0.1, 0.01)
    g, f = uniform_flow(ncol=200, q=0.3, porosity=0.3, alpha_l=aL, alpha_t=aT, dm=0.0)
    n = n_particles
    p = Particles(cell=np.full(n, 11, np.int32), lx=np.zeros(n), ly=np.full(n, 0.5), lz=np.full(n, 0.5),
                  t=np.zeros(n), status=np.full(n, PENDING, np.int32), mass=np.ones(n),
                  id=np.arange(n, dtype=np.uint64), rng_ctr=np.zeros(n, np.uint64))
    opt = Options(time_step_kind=ADV, ts_param=(0.1, 0.1), advection_kind=EULERIAN, dim_mask=(1, 1, 1),
                  precision=precision)
    return g, f, p, opt


def lognormal_slab(n_particles=1_000_000, nlay=20, nrow=100, ncol=200, seed=0, precision=FP64, use_torch=None,
            mf6_dir=None):
    """200x100x20 lognormal K (sigma2 1, 10 m / 2 m), 1e6 particles in the 10 m inlet slab.

    With ``mf6_dir`` the solved flow is written there as MODFLOW 6 binary files
    (``lognormal_slab.grb/.hds/.bud``: FLOW-JA-FACE and a CHD list) and the flow
    returned is the one read back from them, as a MODFLOW 6 run would feed
    the tracker; ``info["mf6_files"]`` names the files."""
    g, f, info = heterogeneous_flow(nlay, nrow, ncol, sigma2=1.0, kg=10.0, lh=10.0, lv=2.0, porosity=0.25,
                                    alpha_l=0.5, alpha_t=0.05, dm=1e-4, seed=seed, use_torch=use_torch)
    if mf6_dir is not None:
        import os
        from . import mf6io
        files = mf6io.write_flow_files(os.path.join(os.fspath(mf6_dir), "lognormal_slab"), g, f, spdis=False)
        f = mf6io.flow_from_mf6(mf6io.read_grb(files[0]), mf6io.read_heads(files[1]), mf6io.read_budget(files[2]),
                                1, 1, porosity=f.porosity, retardation=f.retardation, alpha_l=f.alpha_l,
                                alpha_t=f.alpha_t, dm_eff=f.dm_eff, uniform_dispersion=f.uniform_dispersion)
        info = dict(info, mf6_files=files)
    p = release_in_box(g, n_particles, 0.0, min(10.0, ncol), 0.0, float(nrow), float(g.botm[-1]),
                       float(g.top[0]), seed=1000 + seed)
    opt = Options(time_step_kind=MIN_ADV_DISP, ts_param=(0.1, 0.1), advection_kind=EULERIAN, dim_mask=(1, 1, 1),
                  stop_weak_sinks=True, precision=precision)
    return g, f, p, opt, info


def ensemble_params(n_real=64, scale=1.0):
    """Per-realization draws of the ensemble: realization r draws, from
    numpy's default_rng(r), the grid (ncol in [100, 400], nrow in [50, 200],
    nlay in [10, 20], each uniform), sigma2 lnK in U[0.5, 2], alphaL in
    U[0.1, 1] m (alphaT = alphaL / 10) and a particle count log-uniform in
    [1e5, 4e6] (times ``scale``)."""
    out = []
    for r in range(n_real):
        rng = np.random.default_rng(r)
        ncol, nrow, nlay = int(rng.integers(100, 401)), int(rng.integers(50, 201)), int(rng.integers(10, 21))
        sigma2 = float(rng.uniform(0.5, 2.0))
        aL = float(rng.uniform(0.1, 1.0))
        n = int(round(np.exp(rng.uniform(np.log(1e5), np.log(4e6))) * scale))
        out.append(dict(r=r, ncol=ncol, nrow=nrow, nlay=nlay, sigma2=sigma2, alpha_l=aL, alpha_t=aL / 10.0,
                        n_particles=max(n, 1)))
    return out


def lognormal_ensemble(n_real=64, scale=1.0, precision=MIXED, use_torch=None, members=None):
    """Ensemble of lognormal-slab-generator realizations (ensemble_params): per member
    (grid, flow, particles); field seed r, placement seed 1000 + r; particle
    ids (r << 40) + index, so every member has its own random streams and a
    separate run of the member with the same ids draws the same ones.
    ``members`` overrides the parameter list (for smaller ensembles)."""
    params = ensemble_params(n_real, scale) if members is None else members
    ens = []
    for prm in params:
        g, f, info = heterogeneous_flow(prm["nlay"], prm["nrow"], prm["ncol"], sigma2=prm["sigma2"], kg=10.0, lh=10.0,
                                        lv=2.0, porosity=0.25, alpha_l=prm["alpha_l"], alpha_t=prm["alpha_t"],
                                        dm=1e-4, seed=prm["r"], use_torch=use_torch)
        p = release_in_box(g, prm["n_particles"], 0.0, min(10.0, float(prm["ncol"])), 0.0, float(prm["nrow"]),
                           float(g.botm[-1]), float(g.top[0]), seed=1000 + prm["r"])
        p.id = (np.uint64(prm["r"]) << np.uint64(40)) + np.arange(p.n, dtype=np.uint64)
        ens.append((g, f, p))
    opt = Options(time_step_kind=MIN_ADV_DISP, ts_param=(0.1, 0.1), advection_kind=EULERIAN, dim_mask=(1, 1, 1),
                  stop_weak_sinks=True, precision=precision)
    return ens, opt, params


def lognormal_injection(n_particles=100_000_000, nlay=50, nrow=500, ncol=500, seed=5, precision=FP64, use_torch=None,
            source=((10.0, 30.0), (240.0, 260.0), (20.0, 30.0)), release_days=50.0):
    """Large single run with continuous injection: 500x500x50 cells of 1 m,
    ln K as the lognormal slab with sigma2 2 and correlation lengths 20 m / 2 m, heads
    1 m / 0 m at the x ends; n_particles released at a constant rate over
    release_days (pending particles with uniform release times) from a
    20x20x10 m source (x, y, z ranges of ``source``, model coordinates)."""
    g, f, info = heterogeneous_flow(nlay, nrow, ncol, sigma2=2.0, kg=10.0, lh=20.0, lv=2.0, porosity=0.25,
                                    alpha_l=0.5, alpha_t=0.05, dm=1e-4, seed=seed, use_torch=use_torch)
    (x0, x1), (y0, y1), (z0, z1) = source
    p = release_in_box(g, n_particles, x0, x1, y0, y1, z0, z1, seed=1000 + seed)
    rng = np.random.default_rng(2000 + seed)
    p.t = rng.uniform(0.0, release_days, n_particles)
    opt = Options(time_step_kind=MIN_ADV_DISP, ts_param=(0.1, 0.1), advection_kind=EULERIAN, dim_mask=(1, 1, 1),
                  stop_weak_sinks=True, precision=precision)
    return g, f, p, opt, info
