"""The oracle reproduces the committed golden fixtures bit for bit (tracking
through the C restatement, GPKDE through the numpy restatement), so a change
of the oracle cannot silently move the reference the GPU is checked against.
CPU only."""
import numpy as np
import pytest

from golden_cases import STATE, TRACKING_CASES, case, load
from oracle import gpkde_oracle as GO
from oracle import oracle as O


@pytest.mark.parametrize("name", TRACKING_CASES)
def test_oracle_reproduces_tracking_fixture(name):
    g, f, opt, p, iv, d = case(name)
    q, steps = p, 0
    for t0, t1 in iv:
        q, s = O.advance(g, f, opt, q, t0, t1, rng_kind=O.RNG_PHILOX, nthreads=4)
        steps += s
    assert steps == int(d["steps"])
    for k in STATE:
        np.testing.assert_array_equal(getattr(q, k), d[f"out_{k}"], err_msg=k)


@pytest.mark.parametrize("name", ["gpkde_1d", "gpkde_3d"])
def test_oracle_reproduces_gpkde_fixture(name):
    d = load(name)
    kw = {"n_opt_loops": int(d["n_opt_loops"])} if "n_opt_loops" in d else {}
    G = GO.GPKDE(tuple(d["domain"]), tuple(d["bins"]), **kw)
    dens, _ = G.compute_density(d["coords"], np.ones(d["coords"].shape[0]))
    assert G.loops == int(d["loops"])
    np.testing.assert_allclose(dens, d["density"], rtol=1e-13, atol=0)
    if "histogram" in d:
        h, _, _ = GO.histogram_weighted(d["coords"], np.ones(d["coords"].shape[0]), (0, 0, 0), tuple(d["bins"]),
                                        tuple(int(v) for v in d["domain"] / d["bins"]))
        np.testing.assert_array_equal(h, d["histogram"])


def test_fixture_flow_files_read_back():
    """The heterogeneous fixture's MODFLOW 6 files: FLOW-JA-FACE balanced by
    the CHD sources and sinks, every cell active."""
    from golden_cases import hetero_flow
    g, f = hetero_flow()
    n = g.ncell
    rows = np.repeat(np.arange(n), np.diff(f.ia))
    net = np.zeros(n)
    np.add.at(net, rows, f.flowja)
    bal = net + f.source_flow + f.sink_flow
    assert np.abs(bal).max() < 1e-9 * np.abs(f.flowja).max()
    assert (f.iboundts == 1).all() and g.ncell == 4 * 12 * 30
