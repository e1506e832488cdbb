"""GPKDE reconstruction output records, as the reference writes them.

Restates ``prExportDensityUnit`` (text) and ``prExportDensityUnitBinary``
(stream binary) of GridProjectedKDE.F90:6504-7025 for the call the driver
makes (MPathRW.F90:1626-1642: time index, time, solute id present): one
record per bin whose density is > 0, bins in column-major order (x fastest),
with the columns of the output column format

  0: time index, time, solute id, ix, iy, iz, density, histogram
  1: as 0 plus the bin centre x, y, z after iz
  2: time index, time, solute id, bin centre x, y, z, density, histogram

Text records use the Fortran edit descriptors I8 and ES18.9E3
(``(I8,es18.9e3,4I8,2es18.9e3)`` for format 0); binary records are the same
values unformatted (int32 / float64, little endian), no record markers.

``histogram`` is what the reference's histogram holds at export: the counts
divided by the Kish effective mass (``Histogram.F90:336-343``, effective
weight format 0), which for unit particle masses is the particle count per
bin; bin indexes are 1-based on the reconstruction grid (the grid is not
adapted to the particles, so the reference's deltaBinsOrigin is 0).
"""
from __future__ import annotations

import numpy as np


def es18_9e3(v: float) -> str:
    """Fortran ES18.9E3: one non-zero digit before the point, nine after, a
    signed three-digit exponent, right-justified in 18 columns."""
    v = float(v)
    if v == 0.0:
        return "0.000000000E+000".rjust(18)
    mant, exp = f"{v:.9E}".split("E")
    return f"{mant}E{int(exp):+04d}".rjust(18)


def i8(k: int) -> str:
    return f"{int(k):8d}"


def _records(density, histogram, bin_size, origin):
    d = np.asarray(density, np.float64)
    h = np.asarray(histogram, np.float64)
    if d.ndim == 1:
        d = d.reshape(1, 1, -1)
        h = h.reshape(1, 1, -1)
    if d.shape != h.shape or d.ndim != 3:
        raise ValueError("density and histogram must share the (nz, ny, nx) shape")
    iz, iy, ix = np.nonzero(d > 0.0)        # C order over (z, y, x): x fastest, as the Fortran loops
    bs = np.zeros(3) if bin_size is None else np.asarray(bin_size, np.float64)
    og = np.zeros(3) if origin is None else np.asarray(origin, np.float64)
    idx = np.stack([ix + 1, iy + 1, iz + 1], 1)
    centres = (idx.astype(np.float64) - 0.5) * bs + og
    return idx, centres, d[iz, iy, ix], h[iz, iy, ix]


def write_density_text(fh, density, histogram, time_index: int, time: float, solute_id: int, column_format=0,
                       bin_size=None, origin=None) -> int:
    """Append the text records of one reconstruction to the open text file
    ``fh``; returns how many were written."""
    if column_format not in (0, 1, 2):
        column_format = 0
    if column_format in (1, 2) and bin_size is None:
        raise ValueError("column formats 1 and 2 need bin_size (and origin)")
    idx, cen, dv, hv = _records(density, histogram, bin_size, origin)
    head = i8(time_index) + es18_9e3(time) + i8(solute_id)
    lines = []
    for k in range(dv.shape[0]):
        s = head
        if column_format in (0, 1):
            s += "".join(i8(v) for v in idx[k])
        if column_format in (1, 2):
            s += "".join(es18_9e3(v) for v in cen[k])
        s += es18_9e3(dv[k]) + es18_9e3(hv[k])
        lines.append(s + "\n")
    fh.write("".join(lines))
    return len(lines)


def write_density_binary(fh, density, histogram, time_index: int, time: float, solute_id: int, column_format=0,
                         bin_size=None, origin=None) -> int:
    """Append the unformatted stream records of one reconstruction to the
    binary file ``fh``; returns how many were written."""
    if column_format not in (0, 1, 2):
        column_format = 0
    if column_format in (1, 2) and bin_size is None:
        raise ValueError("column formats 1 and 2 need bin_size (and origin)")
    idx, cen, dv, hv = _records(density, histogram, bin_size, origin)
    fields = [("t_index", "<i4"), ("time", "<f8"), ("solute", "<i4")]
    if column_format in (0, 1):
        fields += [("ix", "<i4"), ("iy", "<i4"), ("iz", "<i4")]
    if column_format in (1, 2):
        fields += [("x", "<f8"), ("y", "<f8"), ("z", "<f8")]
    fields += [("density", "<f8"), ("histogram", "<f8")]
    rec = np.zeros(dv.shape[0], np.dtype(fields))
    rec["t_index"], rec["time"], rec["solute"] = time_index, time, solute_id
    if column_format in (0, 1):
        rec["ix"], rec["iy"], rec["iz"] = idx[:, 0], idx[:, 1], idx[:, 2]
    if column_format in (1, 2):
        rec["x"], rec["y"], rec["z"] = cen[:, 0], cen[:, 1], cen[:, 2]
    rec["density"], rec["histogram"] = dv, hv
    fh.write(rec.tobytes())
    return int(dv.shape[0])


def read_density_text(path, column_format=0) -> np.ndarray:
    """The records of a text output file as a structured array (tests, tools)."""
    names = ["t_index", "time", "solute"]
    if column_format in (0, 1):
        names += ["ix", "iy", "iz"]
    if column_format in (1, 2):
        names += ["x", "y", "z"]
    names += ["density", "histogram"]
    rows = [ln.split() for ln in open(path) if ln.strip()]
    out = np.zeros(len(rows), np.dtype([(n, "<f8") for n in names]))
    for k, r in enumerate(rows):
        out[k] = tuple(float(v) for v in r)
    return out
