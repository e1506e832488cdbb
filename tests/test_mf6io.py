"""MODFLOW 6 binary files: grid, heads and budget readers and writers, and the
assignment of budget terms to the flow arrays of one time step
(FlowModelData.f90:225-625).  CPU only."""
import numpy as np
import pytest

from mprw import mf6io as M
from mprw import workloads as W
from mprw.model import Options
from oracle import oracle as O


@pytest.fixture(scope="module")
def hetero():
    g, f, _ = W.heterogeneous_flow(nlay=3, nrow=6, ncol=12, seed=4, use_torch=False)
    return g, f


def test_grb_round_trip(tmp_path, hetero):
    g, f = hetero
    icell = np.zeros(g.ncell, np.int32)
    icell[: g.nrow * g.ncol] = 1
    idom = np.ones(g.ncell, np.int32)
    idom[5] = 0
    p = tmp_path / "m.grb"
    M.write_grb(p, g, f.ia, f.ja, idomain=idom, icelltype=icell, xorigin=10.0, yorigin=-2.5, angrot=30.0)
    r = M.read_grb(p)
    assert (r.grid.nlay, r.grid.nrow, r.grid.ncol) == (g.nlay, g.nrow, g.ncol)
    for a, b in ((r.grid.delr, g.delr), (r.grid.delc, g.delc), (r.grid.top, g.top), (r.grid.botm, g.botm),
                 (r.ia, f.ia), (r.ja, f.ja), (r.idomain, idom), (r.icelltype, icell)):
        np.testing.assert_array_equal(a, b)
    assert (r.xorigin, r.yorigin, r.angrot) == (10.0, -2.5, 30.0)
    assert r.ibound[5] == 0 and r.ibound.sum() == g.ncell - 1
    raw = p.read_bytes()
    assert raw[:50].split() == [b"GRID", b"DIS"] and len(raw[:50]) == 50
    assert raw[200:300].split()[0] == b"NCELLS"


def test_grb_rejects_other_grids(tmp_path, hetero):
    g, f = hetero
    p = tmp_path / "m.grb"
    M.write_grb(p, g, f.ia, f.ja)
    raw = bytearray(p.read_bytes())
    raw[5:9] = b"DISV"
    (tmp_path / "v.grb").write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="GRID DIS"):
        M.read_grb(tmp_path / "v.grb")
    raw = bytearray(p.read_bytes())
    raw[200:206] = b"NCELLX"      # unknown definition: item count no longer matches NTXT
    (tmp_path / "u.grb").write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="unknown item"):
        M.read_grb(tmp_path / "u.grb")


@pytest.mark.parametrize("prec", [1, 2])
def test_heads_round_trip_and_precision_detection(tmp_path, prec):
    rng = np.random.default_rng(0)
    h1 = rng.normal(size=(3, 4, 5))
    h2 = rng.normal(size=(3, 4, 5))
    p = tmp_path / "m.hds"
    M.write_heads(p, [(1, 1, 1.0, 1.0, h1), (2, 1, 1.0, 2.0, h2)], precision=prec)
    hf = M.read_heads(p)
    assert hf.precision == prec and not hf.unstructured
    assert hf.layer_count == 3 and len(hf.records) == 6
    assert hf.times() == [1.0, 2.0]
    want = h2.reshape(-1) if prec == 2 else h2.reshape(-1).astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(hf.get(1, 2), want)
    with pytest.raises(KeyError):
        hf.get(2, 1)


def _records(n, with_spdis=True):
    rng = np.random.default_rng(1)
    ja_like = rng.normal(size=37)
    recs = [M.BudgetRecord(1, 1, "FLOW-JA-FACE", 1, (37, 1, 1), 1.0, 1.0, 1.0, array=ja_like),
            M.BudgetRecord(1, 1, "WEL", 6, (n, 1, 1), 1.0, 1.0, 1.0, id1=np.array([2, 5, 5], np.int32),
                           id2=np.array([1, 2, 3], np.int32), q=np.array([-3.0, 1.5, 0.25]),
                           aux=np.array([[0.0, 7.0], [2.0, 8.0], [0.0, 9.0]]), aux_names=["IFACE", "CONC"],
                           txt_ids=("GWF", "GWF", "GWF", "WEL-1")),
            M.BudgetRecord(1, 1, "RCH", 6, (n, 1, 1), 1.0, 1.0, 1.0, id1=np.array([1, 3], np.int32),
                           id2=np.array([1, 2], np.int32), q=np.array([0.5, 0.75]), aux=np.zeros((2, 0)),
                           aux_names=[], txt_ids=("GWF", "GWF", "GWF", "RCH-1")),
            M.BudgetRecord(1, 1, "DRN", 2, (n, 1, 1), 1.0, 1.0, 1.0, id1=np.array([4], np.int32),
                           q=np.array([-0.125])),
            M.BudgetRecord(1, 1, "EVT", 5, (n, 1, 1), 1.0, 1.0, 1.0, id1=np.array([6], np.int32),
                           q=np.array([-0.5]), aux=np.array([[3.0]]), aux_names=["IFACE"]),
            M.BudgetRecord(1, 1, "STO-SS", 1, (n, 1, 1), 1.0, 1.0, 1.0, array=np.zeros(n))]
    if with_spdis:
        recs.append(M.BudgetRecord(1, 1, "DATA-SPDIS", 6, (n, 1, 1), 1.0, 1.0, 1.0,
                                   id1=np.arange(1, n + 1, dtype=np.int32), id2=np.arange(1, n + 1, dtype=np.int32),
                                   q=np.zeros(n), aux=np.ones((n, 3)), aux_names=["QX", "QY", "QZ"],
                                   txt_ids=("GWF", "GWF", "GWF", "NPF")))
    return recs


@pytest.mark.parametrize("prec", [1, 2])
def test_budget_round_trip_every_list_method(tmp_path, prec):
    n = 8
    recs = _records(n)
    p = tmp_path / "m.bud"
    M.write_budget(p, recs, precision=prec)
    bf = M.read_budget(p)
    assert bf.precision == prec and bf.budget_type == 2 and bf.file_format == 2 and bf.flow_array_size == 37
    assert list(bf.record_range(1, 1)) == list(range(len(recs)))
    assert bf.time_steps() == [(1, 1)]
    cast = (lambda a: a) if prec == 2 else (lambda a: np.asarray(a, np.float32).astype(np.float64))
    for i, r in enumerate(recs):
        b = bf.read(i)
        assert b.text == r.text and b.imeth == r.imeth
        if r.imeth == 1:
            np.testing.assert_array_equal(b.array, cast(r.array))
            continue
        np.testing.assert_array_equal(b.id1, r.id1)
        np.testing.assert_array_equal(b.q, cast(r.q))
        if r.imeth == 6:
            np.testing.assert_array_equal(b.id2, r.id2)
            assert b.txt_ids == r.txt_ids
        if r.imeth in (5, 6):
            assert b.aux_names == r.aux_names
            np.testing.assert_array_equal(b.aux, cast(r.aux))


def test_budget_standard_form_and_mixed_forms_rejected(tmp_path):
    std = [M.BudgetRecord(1, 1, "FLOW-JA-FACE", 0, (10, 1, 1), array=np.arange(10.0)),
           M.BudgetRecord(1, 1, "CHD", 0, (2, 1, 1), array=np.array([1.0, -1.0]))]
    M.write_budget(tmp_path / "s.bud", std)
    bf = M.read_budget(tmp_path / "s.bud")
    assert bf.file_format == 1 and bf.budget_type == 2
    np.testing.assert_array_equal(bf.read(0).array, np.arange(10.0))
    mixed = std[:1] + [M.BudgetRecord(1, 1, "CHD", 2, (2, 1, 1), id1=np.array([1], np.int32), q=np.array([1.0]))]
    M.write_budget(tmp_path / "x.bud", mixed)
    with pytest.raises(ValueError):
        M.read_budget(tmp_path / "x.bud")
    no_flow = [M.BudgetRecord(1, 1, "CHD", 0, (2, 1, 1), array=np.array([1.0, -1.0]))]
    M.write_budget(tmp_path / "n.bud", no_flow)
    with pytest.raises(ValueError):
        M.read_budget(tmp_path / "n.bud")


def test_budget_term_assignment(tmp_path):
    """Every branch of the term assignment on one hand-made time step: IFACE
    auxiliaries, a default IFACE for a label, sources and sinks by sign,
    storage, and the skipped DATA-SPDIS."""
    g = W.structured_grid(1, 2, 4)
    ia, ja = W.dis_connectivity(g)
    n = g.ncell
    recs = _records(n)
    recs[0] = M.BudgetRecord(1, 1, "FLOW-JA-FACE", 1, (ja.shape[0], 1, 1), array=np.linspace(-1, 1, ja.shape[0]))
    recs[-2] = M.BudgetRecord(1, 1, "STO-SS", 1, (n, 1, 1), array=np.where(np.arange(n) == 3, 0.5, 0.0))
    M.write_grb(tmp_path / "a.grb", g, ia, ja)
    M.write_heads(tmp_path / "a.hds", [(1, 1, 1.0, 1.0, np.zeros((1, 2, 4)))])
    M.write_budget(tmp_path / "a.bud", recs)
    grb, hf, bf = M.read_grb(tmp_path / "a.grb"), M.read_heads(tmp_path / "a.hds"), M.read_budget(tmp_path / "a.bud")
    ts = M.load_time_step(grb, hf, bf, 1, 1, default_iface={"rch": 6})
    src, snk, bnd = np.zeros(n), np.zeros(n), np.zeros((n, 6))
    # WEL: cell 2 IFACE 0 -> sink; cell 5 IFACE 2 (+1.5) -> face 2; cell 5 IFACE 0 -> source
    snk[1] += -3.0
    bnd[4, 1] += 1.5
    src[4] += 0.25
    # RCH: default IFACE 6 (the label is compared in upper case)
    bnd[0, 5] += 0.5
    bnd[2, 5] += 0.75
    # DRN (imeth 2, no default) -> sink; EVT (imeth 5, IFACE 3) -> face 3
    snk[3] += -0.125
    bnd[5, 2] += -0.5
    np.testing.assert_array_equal(ts.source_flow, src)
    np.testing.assert_array_equal(ts.sink_flow, snk)
    np.testing.assert_array_equal(ts.boundary_flows.reshape(n, 6), bnd)
    np.testing.assert_array_equal(ts.flowja, recs[0].array)
    assert not ts.steady_state and ts.storage_flow[3] == 0.5
    with pytest.raises(ValueError, match="every time step"):
        M.load_time_step(grb, hf, bf, 2, 1)


def test_dry_cells_leave_iboundts(tmp_path):
    g = W.structured_grid(2, 2, 3)
    ia, ja = W.dis_connectivity(g)
    n = g.ncell
    h = np.full((2, 2, 3), 1.5)
    h[0, 0, 1] = -1.0e30        # dry, convertible layer: leaves IBOUNDTS
    h[1, 1, 2] = -1.0e30        # same head in a confined cell: stays active
    h[0, 1, 0] = -1.0e30 * (1 + 1e-9)   # within the single-precision tolerance: dry
    ict = np.zeros(n, np.int32)
    ict[:6] = 1
    M.write_grb(tmp_path / "d.grb", g, ia, ja, icelltype=ict)
    M.write_heads(tmp_path / "d.hds", [(1, 1, 1.0, 1.0, h)])
    M.write_budget(tmp_path / "d.bud", [M.BudgetRecord(1, 1, "FLOW-JA-FACE", 1, (ja.shape[0], 1, 1),
                                                       array=np.zeros(ja.shape[0]))])
    ts = M.load_time_step(M.read_grb(tmp_path / "d.grb"), M.read_heads(tmp_path / "d.hds"),
                          M.read_budget(tmp_path / "d.bud"), 1, 1)
    want = np.ones(n, np.int32)
    want[g.node(0, 0, 1) - 1] = 0
    want[g.node(0, 1, 0) - 1] = 0
    np.testing.assert_array_equal(ts.iboundts, want)


def test_flow_files_round_trip_heterogeneous(tmp_path, hetero):
    """The lognormal-field flow (FLOW-JA-FACE + CHD) written in MODFLOW 6 form
    and read back gives identical arrays, and the oracle tracks identically
    through both."""
    g, f = hetero
    M.write_flow_files(tmp_path / "h", g, f)
    r = M.flow_from_mf6(M.read_grb(tmp_path / "h.grb"), M.read_heads(tmp_path / "h.hds"),
                        M.read_budget(tmp_path / "h.bud"), 1, 1, porosity=f.porosity, retardation=f.retardation,
                        alpha_l=f.alpha_l, alpha_t=f.alpha_t, dm_eff=f.dm_eff)
    for name in ("ia", "ja", "flowja", "heads", "source_flow", "sink_flow", "porosity", "iboundts"):
        np.testing.assert_array_equal(getattr(r, name), getattr(f, name), err_msg=name)
    np.testing.assert_array_equal(r.boundary_flows, np.zeros(6 * g.ncell))
    opt = Options(time_step_kind=3, ts_param=(0.1, 0.1), stop_weak_sinks=True)
    p = W.release_in_box(g, 500, 0.5, 2.5, 0.5, 5.5, 0.5, 2.5, seed=7)
    a, sa = O.advance(g, f, opt, p.copy(), 0.0, 40.0, rng_kind=O.RNG_PHILOX, nthreads=4)
    b, sb = O.advance(g, r, opt, p.copy(), 0.0, 40.0, rng_kind=O.RNG_PHILOX, nthreads=4)
    assert sa == sb
    for name in ("cell", "lx", "ly", "lz", "t", "status"):
        np.testing.assert_array_equal(getattr(a, name), getattr(b, name), err_msg=name)


def test_flow_files_round_trip_iface_boundaries(tmp_path):
    """Uniform flow whose inflow and outflow are boundary face flows: written
    as a list with an IFACE auxiliary and assigned back to the same faces."""
    g, f = W.uniform_flow(ncol=30, nrow=2, nlay=2, q=0.3)
    M.write_flow_files(tmp_path / "u", g, f, precision=2, spdis=True)
    r = M.flow_from_mf6(M.read_grb(tmp_path / "u.grb"), M.read_heads(tmp_path / "u.hds"),
                        M.read_budget(tmp_path / "u.bud"), 1, 1, porosity=0.3, retardation=1.0,
                        alpha_l=f.alpha_l, alpha_t=f.alpha_t, dm_eff=f.dm_eff)
    np.testing.assert_array_equal(r.boundary_flows, f.boundary_flows)
    np.testing.assert_array_equal(r.flowja, f.flowja)
    assert not r.source_flow.any() and not r.sink_flow.any()


def test_truncated_and_corrupt_files_are_rejected(tmp_path, hetero):
    g, f = hetero
    M.write_flow_files(tmp_path / "t", g, f)
    raw = (tmp_path / "t.bud").read_bytes()
    (tmp_path / "cut.bud").write_bytes(raw[: len(raw) - 100])
    with pytest.raises(ValueError):
        M.read_budget(tmp_path / "cut.bud")
    raw = (tmp_path / "t.hds").read_bytes()
    (tmp_path / "cut.hds").write_bytes(raw[: len(raw) // 2 + 3])
    with pytest.raises(ValueError):
        M.read_heads(tmp_path / "cut.hds")
    raw = (tmp_path / "t.grb").read_bytes()
    (tmp_path / "cut.grb").write_bytes(raw[: len(raw) - 8])
    with pytest.raises(ValueError):
        M.read_grb(tmp_path / "cut.grb")
    (tmp_path / "junk.bud").write_bytes(b"\x07" * 4096)
    with pytest.raises(ValueError):
        M.read_budget(tmp_path / "junk.bud")
