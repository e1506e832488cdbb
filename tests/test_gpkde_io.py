"""GPKDE output records (GridProjectedKDE.F90:6504-7025): Fortran edit
descriptors, record selection (density > 0, x fastest) and the three column
formats, text and binary.  CPU only."""
import io

import numpy as np
import pytest

from mprw import gpkde_io as G


def test_es18_9e3_matches_fortran_edit_descriptor():
    assert G.es18_9e3(1.0) == "  1.000000000E+000"
    assert G.es18_9e3(-2.5e-7) == " -2.500000000E-007"
    assert G.es18_9e3(123456.789) == "  1.234567890E+005"
    assert G.es18_9e3(9.9999999999) == "  1.000000000E+001"   # rounding carries into the exponent
    assert G.es18_9e3(0.0) == "  0.000000000E+000"
    assert G.es18_9e3(1.5e-300) == "  1.500000000E-300"
    assert G.i8(42) == "      42"


def _grids():
    d = np.zeros((2, 3, 4))
    d[0, 0, 1] = 0.5
    d[1, 2, 3] = 2.0e-3
    d[0, 1, 0] = -1.0        # not exported (<= 0)
    h = np.arange(24, dtype=float).reshape(2, 3, 4)
    return d, h


@pytest.mark.parametrize("fmt", [0, 1, 2])
def test_text_records(tmp_path, fmt):
    d, h = _grids()
    p = tmp_path / "gpkde.txt"
    with open(p, "w") as fh:
        n = G.write_density_text(fh, d, h, 3, 25.0, 1, column_format=fmt, bin_size=(1.0, 0.5, 2.0),
                                 origin=(10.0, 0.0, -4.0))
    assert n == 2
    lines = p.read_text().splitlines()
    width = {0: 8 + 18 + 8 + 24 + 36, 1: 8 + 18 + 8 + 24 + 54 + 36, 2: 8 + 18 + 8 + 54 + 36}[fmt]
    assert all(len(ln) == width for ln in lines)
    r = G.read_density_text(p, fmt)
    # x fastest: (ix=2, iy=1, iz=1) before (ix=4, iy=3, iz=2)
    np.testing.assert_array_equal(r["density"], [0.5, 2.0e-3])
    np.testing.assert_array_equal(r["histogram"], [h[0, 0, 1], h[1, 2, 3]])
    assert (r["t_index"] == 3).all() and (r["time"] == 25.0).all() and (r["solute"] == 1).all()
    if fmt in (0, 1):
        np.testing.assert_array_equal(np.stack([r["ix"], r["iy"], r["iz"]], 1), [[2, 1, 1], [4, 3, 2]])
    if fmt in (1, 2):
        np.testing.assert_allclose(np.stack([r["x"], r["y"], r["z"]], 1), [[11.5, 0.25, -3.0], [13.5, 1.25, -1.0]])


def test_binary_records():
    d, h = _grids()
    buf = io.BytesIO()
    assert G.write_density_binary(buf, d, h, 7, 50.0, 2) == 2
    dt = np.dtype([("t", "<i4"), ("time", "<f8"), ("s", "<i4"), ("ix", "<i4"), ("iy", "<i4"), ("iz", "<i4"),
                   ("d", "<f8"), ("h", "<f8")])
    r = np.frombuffer(buf.getvalue(), dt)
    assert r.shape == (2,) and dt.itemsize == 44
    np.testing.assert_array_equal(r["d"], [0.5, 2.0e-3])
    np.testing.assert_array_equal(r["ix"], [2, 4])
    assert (r["t"] == 7).all() and (r["time"] == 50.0).all() and (r["s"] == 2).all()


def test_one_dimensional_grid():
    dens = np.array([0.0, 1.0, 3.0, 0.0])
    out = io.StringIO()
    assert G.write_density_text(out, dens, dens * 2, 1, 1.0, 1) == 2
    first = out.getvalue().splitlines()[0]
    assert first.split()[3:6] == ["2", "1", "1"]
