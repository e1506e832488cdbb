"""Synthetic inputs: head solve, flows, release geometry (CPU)."""
import numpy as np

from mprw import workloads as W
from oracle import oracle as O


def test_dis_connectivity_counts():
    g = W.structured_grid(3, 4, 5)
    ia, ja = W.dis_connectivity(g)
    assert ia[0] == 1 and ia[-1] - 1 == ja.shape[0]
    # interior cell of a 3x4x5 grid has 6 neighbours + diagonal
    n = g.node(1, 1, 1)
    assert ia[n] - ia[n - 1] == 7
    assert ja[ia[n - 1] - 1] == n  # diagonal first


def test_head_solve_mass_balance_and_residual():
    g, f, info = W.heterogeneous_flow(nlay=3, nrow=6, ncol=15, seed=3, use_torch=False)
    assert f.source_flow.sum() > 0
    np.testing.assert_allclose(f.source_flow.sum(), -f.sink_flow.sum(), rtol=1e-9)
    # every free cell balances: sum of FLOW-JA-FACE into the cell is ~0
    n = g.ncell
    rows = np.repeat(np.arange(n), np.diff(f.ia))
    net = np.zeros(n)
    np.add.at(net, rows, f.flowja)
    col = np.arange(n) % g.ncol
    free = (col != 0) & (col != g.ncol - 1)
    scale = np.abs(f.flowja).max()
    assert np.abs(net[free]).max() < 1e-9 * scale
    # heads decrease from 1 to 0 along x on average
    h = f.heads.reshape(g.nlay, g.nrow, g.ncol)
    assert h[:, :, 0].min() == 1.0 and h[:, :, -1].max() == 0.0
    assert np.all(np.diff(h.mean(axis=(0, 1))) < 0)


def test_lognormal_field_statistics():
    K = W.lognormal_field(10, 30, 60, sigma2=1.0, kg=10.0, lh=5.0, lv=2.0, seed=4)
    lnk = np.log(K)
    assert abs(lnk.mean() - np.log(10.0)) < 0.35
    assert 0.5 < lnk.var() < 1.5


def test_release_box_maps_to_model_coordinates():
    g, f, p, opt, info = W.lognormal_slab(n_particles=2000, nlay=4, nrow=12, ncol=30, seed=0, use_torch=False)
    gx, gy, gz = O.global_xyz(g, f, p)
    assert gx.min() >= 0.0 and gx.max() <= 10.0
    assert gy.min() >= 0.0 and gy.max() <= 12.0
    assert gz.min() >= 0.0 and gz.max() <= 4.0
    # uniform in the box
    assert abs(gx.mean() - 5.0) < 0.3 and abs(gy.mean() - 6.0) < 0.4 and abs(gz.mean() - 2.0) < 0.15
