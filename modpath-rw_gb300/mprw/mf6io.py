"""MODFLOW 6 binary files for the tracking path: grid (.grb), heads (.hds) and
cell-by-cell budget (.bud / .cbc), read into the ``Grid`` / ``Flow`` containers
that ``Tracker.load_flow`` takes, and written back (for synthetic flows and for
round-trip tests).

Readers restate the reference's:
  * ``read_grb``     -- RectangularGridDisMf6.f90:122-360 (ReadGRB): four
    50-character header lines (GRID DIS / VERSION 1 / NTXT 16 / LENTXT 100),
    NTXT 100-character definition lines, then the data in definition order,
    each item's type fixed by its name;
  * ``read_heads``   -- HeadReader.f90:270-353 (OpenFile: unstructured headers
    tried first, then structured; single precision before double) and
    560-640 (record header: kstp, kper, pertim, totim, text, ncol, nrow, ilay;
    the text must be HEAD);
  * ``read_budget``  -- BudgetReader.f90:563-710 (record header, methods 0-6)
    and 713-850 (header scan: precision detection, file format, budget type),
    381-449 (list records of methods 2, 5, 6);
  * ``flow_from_mf6`` -- FlowModelData.f90:225-625 (LoadTimeStep): dry cells of
    convertible layers leave IBOUNDTS, FLOW-JA-FACE fills the face flows,
    storage terms clear the steady-state flag, every other term goes to the
    source / sink flows by sign or, when its label has a default IFACE or its
    list carries an IFACE auxiliary, to the boundary face flows of that IFACE.

Layout of the files (MODFLOW 6 stream-access binary, little endian):
  budget record:  kstp i4, kper i4, text 16s, ndim1 i4, ndim2 i4, ndim3 i4;
                  ndim3 < 0 ("compact"): imeth i4, delt, pertim, totim (real);
                  imeth 0/1: ndim1*ndim2*|ndim3| reals;
                  imeth 2: nlist i4, nlist x (id i4, q real);
                  imeth 5: ndat i4, (ndat-1) x aux name 16s, nlist i4,
                           nlist x (id i4, q, aux... real);
                  imeth 6: 4 x 16s (model/package names), then as imeth 5 with
                           (id1 i4, id2 i4) per list item;
  head record:    kstp i4, kper i4, pertim, totim (real), text 16s,
                  ncol i4, nrow i4, ilay i4, ncol*nrow reals.
"Real" is f4 or f8 for the whole file.  Methods 3 and 4 (layer-indicator
records of MODFLOW-2005) are parsed as headers but their data are rejected:
MODFLOW 6 never writes them.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

from .model import Flow, Grid

_I4 = np.dtype("<i4")


# --------------------------------------------------------------------------- grid


@dataclass
class Mf6Grid:
    """Contents of a DIS binary grid file.  ``ia``/``ja`` are 1-based with the
    diagonal first in every row (MODFLOW 6 convention)."""
    grid: Grid
    ia: np.ndarray
    ja: np.ndarray
    idomain: np.ndarray
    icelltype: np.ndarray
    xorigin: float = 0.0
    yorigin: float = 0.0
    angrot: float = 0.0

    @property
    def ibound(self) -> np.ndarray:
        """IBOUND of the tracking model: 1 where IDOMAIN >= 1, else 0
        (ModpathBasicData.f90:177-185)."""
        return (self.idomain >= 1).astype(np.int32)


# name -> (kind, length); kind 'i' int32, 'd' float64; length as a function of the
# scalars read so far (ReadGRB reads every item with a fixed type and size).
_GRB_ITEMS = {
    "NCELLS": ("i", lambda s: 1), "NLAY": ("i", lambda s: 1), "NROW": ("i", lambda s: 1),
    "NCOL": ("i", lambda s: 1), "NJA": ("i", lambda s: 1),
    "XORIGIN": ("d", lambda s: 1), "YORIGIN": ("d", lambda s: 1), "ANGROT": ("d", lambda s: 1),
    "DELR": ("d", lambda s: s["NCOL"]), "DELC": ("d", lambda s: s["NROW"]),
    "TOP": ("d", lambda s: s["NROW"] * s["NCOL"]), "BOTM": ("d", lambda s: s["NCELLS"]),
    "IA": ("i", lambda s: s["NCELLS"] + 1), "JA": ("i", lambda s: s["NJA"]),
    "IDOMAIN": ("i", lambda s: s["NCELLS"]), "ICELLTYPE": ("i", lambda s: s["NCELLS"]),
}
_GRB_SCALARS = ("NCELLS", "NLAY", "NROW", "NCOL", "NJA", "XORIGIN", "YORIGIN", "ANGROT")
_GRB_ORDER = ["NCELLS", "NLAY", "NROW", "NCOL", "NJA", "XORIGIN", "YORIGIN", "ANGROT", "DELR", "DELC", "TOP",
              "BOTM", "IA", "JA", "IDOMAIN", "ICELLTYPE"]


def _line(text: str, width: int) -> bytes:
    b = text.encode("ascii")
    if len(b) >= width:
        raise ValueError(f"line longer than {width - 1} characters: {text!r}")
    return b.ljust(width - 1) + b"\n"


def write_grb(path, grid: Grid, ia, ja, idomain=None, icelltype=None, xorigin=0.0, yorigin=0.0, angrot=0.0):
    """Write a DIS binary grid file (VERSION 1, 16 definition lines)."""
    n = grid.ncell
    ia = np.asarray(ia, _I4)
    ja = np.asarray(ja, _I4)
    if ia.shape != (n + 1,) or ja.shape != (int(ia[-1]) - 1,):
        raise ValueError("ia must have ncell+1 entries and ja ia[-1]-1 entries (1-based)")
    idomain = np.ones(n, _I4) if idomain is None else np.asarray(idomain, _I4)
    icelltype = np.zeros(n, _I4) if icelltype is None else np.asarray(icelltype, _I4)
    vals = {"NCELLS": n, "NLAY": grid.nlay, "NROW": grid.nrow, "NCOL": grid.ncol, "NJA": ja.shape[0],
            "XORIGIN": xorigin, "YORIGIN": yorigin, "ANGROT": angrot, "DELR": grid.delr, "DELC": grid.delc,
            "TOP": grid.top, "BOTM": grid.botm, "IA": ia, "JA": ja, "IDOMAIN": idomain, "ICELLTYPE": icelltype}
    with open(path, "wb") as fh:
        for h in ("GRID DIS", "VERSION 1", "NTXT 16", "LENTXT 100"):
            fh.write(_line(h, 50))
        sizes = {k: vals[k] for k in ("NCELLS", "NLAY", "NROW", "NCOL", "NJA")}
        for name in _GRB_ORDER:
            kind, ln = _GRB_ITEMS[name]
            cnt = ln(sizes)
            typ = "INTEGER" if kind == "i" else "DOUBLE"
            dims = "NDIM 0" if name in _GRB_SCALARS else f"NDIM 1 {cnt}"
            fh.write(_line(f"{name} {typ} {dims}", 100))
        for name in _GRB_ORDER:
            kind, ln = _GRB_ITEMS[name]
            cnt = ln(sizes)
            a = np.asarray(vals[name], _I4 if kind == "i" else np.float64).reshape(-1)
            if a.shape[0] != cnt:
                raise ValueError(f"{name}: {a.shape[0]} values, expected {cnt}")
            fh.write(a.astype(a.dtype.newbyteorder("<")).tobytes())


def _words(b: bytes) -> List[str]:
    return b.decode("ascii", errors="replace").split()


def read_grb(path) -> Mf6Grid:
    """Read a DIS binary grid file (RectangularGridDisMf6.f90:122-360)."""
    with open(path, "rb") as fh:
        buf = fh.read()
    pos = 0

    def header(key):
        nonlocal pos
        w = _words(buf[pos:pos + 50])
        pos += 50
        if not w or w[0] != key:
            raise ValueError(f"invalid binary grid file: expected {key}")
        return w

    w = header("GRID")
    if len(w) < 2 or w[1] != "DIS":
        raise ValueError("invalid binary grid type: only GRID DIS is supported")
    if int(header("VERSION")[1]) != 1:
        raise ValueError("unsupported binary grid file version")
    ntxt = int(header("NTXT")[1])
    if ntxt != 16:
        raise ValueError("invalid binary grid file data (NTXT)")
    lentxt = int(header("LENTXT")[1])
    if lentxt != 100:
        raise ValueError("invalid binary grid file data (LENTXT)")
    names = []
    for _ in range(ntxt):
        line = buf[pos:pos + lentxt]
        pos += lentxt
        if line[:1] == b"#":
            names.append("#")
        else:
            w = _words(line)
            names.append(w[0] if w else "")
    vals: Dict[str, object] = {}
    for name in names:
        if name == "#":
            continue
        if name not in _GRB_ITEMS:
            raise ValueError(f"error reading binary grid file: unknown item {name!r}")
        kind, ln = _GRB_ITEMS[name]
        cnt = ln(vals)
        dt = _I4 if kind == "i" else np.dtype("<f8")
        nbytes = cnt * dt.itemsize
        if pos + nbytes > len(buf):
            raise ValueError(f"binary grid file ends inside {name}")
        a = np.frombuffer(buf, dt, cnt, pos).copy()
        pos += nbytes
        if name in _GRB_SCALARS:
            vals[name] = int(a[0]) if kind == "i" else float(a[0])
        else:
            vals[name] = a
    for req in ("NCELLS", "NLAY", "NROW", "NCOL", "NJA", "DELR", "DELC", "TOP", "BOTM", "IA", "JA"):
        if req not in vals:
            raise ValueError(f"binary grid file has no {req}")
    n = vals["NCELLS"]
    if n != vals["NLAY"] * vals["NROW"] * vals["NCOL"]:
        raise ValueError("NCELLS differs from NLAY*NROW*NCOL")
    grid = Grid(vals["NLAY"], vals["NROW"], vals["NCOL"], np.asarray(vals["DELR"], np.float64),
                np.asarray(vals["DELC"], np.float64), np.asarray(vals["TOP"], np.float64),
                np.asarray(vals["BOTM"], np.float64))
    return Mf6Grid(grid=grid, ia=vals["IA"].astype(np.int32), ja=vals["JA"].astype(np.int32),
                   idomain=np.asarray(vals.get("IDOMAIN", np.ones(n, _I4)), np.int32),
                   icelltype=np.asarray(vals.get("ICELLTYPE", np.zeros(n, _I4)), np.int32),
                   xorigin=vals.get("XORIGIN", 0.0), yorigin=vals.get("YORIGIN", 0.0),
                   angrot=vals.get("ANGROT", 0.0))


# --------------------------------------------------------------------------- heads


@dataclass
class HeadRecord:
    kstp: int
    kper: int
    pertim: float
    totim: float
    text: str
    ncol: int
    nrow: int
    ilay: int
    data_pos: int


@dataclass
class HeadFile:
    path: str
    precision: int            # 1 single, 2 double
    records: List[HeadRecord]
    unstructured: bool = False

    @property
    def layer_count(self) -> int:
        return max((r.ilay for r in self.records), default=0)

    def times(self) -> List[float]:
        """Total time of every time step present, in file order."""
        out, last = [], None
        for r in self.records:
            if (r.kper, r.kstp) != last:
                out.append(r.totim)
                last = (r.kper, r.kstp)
        return out

    def get(self, kper: int, kstp: int) -> np.ndarray:
        """Heads of every cell at (stress period, time step), FP64
        (HeadReader.f90:80-112: the layer-1 record and the LayerCount records
        after it)."""
        first = next((i for i, r in enumerate(self.records) if r.kper == kper and r.kstp == kstp and r.ilay == 1),
                     None)
        if first is None:
            raise KeyError(f"no heads for period {kper} step {kstp}")
        dt = np.dtype("<f4") if self.precision == 1 else np.dtype("<f8")
        parts = []
        with open(self.path, "rb") as fh:
            for r in self.records[first:first + self.layer_count]:
                cnt = r.ncol * r.nrow if not self.unstructured else (r.nrow - r.ncol + 1)
                fh.seek(r.data_pos)
                parts.append(np.frombuffer(fh.read(cnt * dt.itemsize), dt, cnt).astype(np.float64))
        return np.concatenate(parts)


def write_heads(path, records, precision: int = 2, text: str = "HEAD"):
    """Write a structured head file.  ``records``: iterable of
    (kstp, kper, pertim, totim, heads) with heads shaped (nlay, nrow, ncol)."""
    rdt = np.dtype("<f4") if precision == 1 else np.dtype("<f8")
    with open(path, "wb") as fh:
        for kstp, kper, pertim, totim, h in records:
            h = np.asarray(h, np.float64)
            if h.ndim != 3:
                raise ValueError("heads must be (nlay, nrow, ncol)")
            nl, nr, nc = h.shape
            for k in range(nl):
                fh.write(np.array([kstp, kper], _I4).tobytes())
                fh.write(np.array([pertim, totim], rdt).tobytes())
                fh.write(text.rjust(16).encode("ascii"))
                fh.write(np.array([nc, nr, k + 1], _I4).tobytes())
                fh.write(h[k].astype(rdt).tobytes())


def _scan_heads(buf: bytes, precision: int, unstructured: bool) -> Optional[List[HeadRecord]]:
    rb = 4 if precision == 1 else 8
    rdt = np.dtype("<f4") if precision == 1 else np.dtype("<f8")
    hsize = 16 + 5 * 4 + 2 * rb
    pos, out = 0, []
    want = "HEADU" if unstructured else "HEAD"
    while pos < len(buf):
        if pos + hsize > len(buf):
            return None
        kstp, kper = np.frombuffer(buf, _I4, 2, pos)
        pertim, totim = np.frombuffer(buf, rdt, 2, pos + 8)
        text = buf[pos + 8 + 2 * rb:pos + 24 + 2 * rb].decode("ascii", errors="replace")
        a, b, ilay = (int(v) for v in np.frombuffer(buf, _I4, 3, pos + 24 + 2 * rb))
        if text.strip() != want:
            return None
        if unstructured:
            cnt = b - a + 1      # first and last node of the layer
        else:
            if a < 1 or b < 1:
                return None
            cnt = a * b
        if cnt < 1:
            return None
        out.append(HeadRecord(int(kstp), int(kper), float(pertim), float(totim), text.strip(), a, b, ilay,
                              pos + hsize))
        pos += hsize + cnt * rb
        if pos > len(buf):
            return None
    return out


def read_heads(path) -> HeadFile:
    """Open a head file, detecting its layout and precision (unstructured
    before structured, single before double: HeadReader.f90:270-300)."""
    with open(path, "rb") as fh:
        buf = fh.read()
    for unstructured in (True, False):
        for prec in (1, 2):
            recs = _scan_heads(buf, prec, unstructured)
            if recs:
                return HeadFile(str(path), prec, recs, unstructured)
    raise ValueError(f"{path}: not a head file")


# --------------------------------------------------------------------------- budget


@dataclass
class BudgetRecord:
    """One budget record.  Array records (imeth 0/1) carry ``array``; list
    records (imeth 2/5/6) carry ``id1`` (cell numbers, 1-based), ``id2``
    (imeth 6), ``q`` and ``aux`` (nlist x naux) with ``aux_names``."""
    kstp: int
    kper: int
    text: str
    imeth: int
    ndim: tuple                       # (ndim1, ndim2, ndim3) as written, ndim3 > 0
    delt: float = 0.0
    pertim: float = 0.0
    totim: float = 0.0
    array: Optional[np.ndarray] = None
    id1: Optional[np.ndarray] = None
    id2: Optional[np.ndarray] = None
    q: Optional[np.ndarray] = None
    aux: Optional[np.ndarray] = None
    aux_names: List[str] = field(default_factory=list)
    txt_ids: tuple = ("", "", "", "")  # imeth 6: model / package names

    def aux_index(self, name: str) -> int:
        """0-based index of an auxiliary column by name, -1 if absent
        (BudgetRecordHeader FindAuxiliaryNameIndex)."""
        for i, a in enumerate(self.aux_names):
            if a.strip() == name:
                return i
        return -1


@dataclass
class BudgetHeader:
    kstp: int
    kper: int
    text: str
    ncol: int
    nrow: int
    nlay: int
    imeth: int
    delt: float
    pertim: float
    totim: float
    nval: int                 # list: values per item (q + aux)
    nlist: int
    aux_names: List[str]
    txt_ids: tuple
    data_pos: int
    data_bytes: int

    @property
    def label(self) -> str:
        return self.text.strip()

    @property
    def array_count(self) -> int:
        if self.imeth in (2, 5, 6):
            return 0
        if self.imeth in (3, 4):
            return self.ncol * self.nrow
        return self.ncol * self.nrow * self.nlay


def _s16(b: bytes) -> str:
    return b.decode("ascii", errors="replace")


def write_budget(path, records: Sequence[BudgetRecord], precision: int = 2):
    """Write a cell-by-cell budget file (compact form for imeth >= 1)."""
    rdt = np.dtype("<f4") if precision == 1 else np.dtype("<f8")
    with open(path, "wb") as fh:
        for r in records:
            n1, n2, n3 = (int(v) for v in r.ndim)
            fh.write(np.array([r.kstp, r.kper], _I4).tobytes())
            fh.write(r.text.rjust(16).encode("ascii")[:16])
            fh.write(np.array([n1, n2, -n3 if r.imeth > 0 else n3], _I4).tobytes())
            if r.imeth > 0:
                fh.write(np.array([r.imeth], _I4).tobytes())
                fh.write(np.array([r.delt, r.pertim, r.totim], rdt).tobytes())
            if r.imeth in (0, 1):
                a = np.asarray(r.array, np.float64).reshape(-1)
                if a.shape[0] != n1 * n2 * n3:
                    raise ValueError(f"{r.text}: array of {a.shape[0]}, expected {n1 * n2 * n3}")
                fh.write(a.astype(rdt).tobytes())
                continue
            if r.imeth not in (2, 5, 6):
                raise ValueError(f"imeth {r.imeth} not supported")
            id1 = np.asarray(r.id1, _I4)
            nl = id1.shape[0]
            q = np.asarray(r.q, np.float64).reshape(nl)
            naux = len(r.aux_names) if r.imeth != 2 else 0
            aux = np.zeros((nl, 0)) if naux == 0 else np.asarray(r.aux, np.float64).reshape(nl, naux)
            if r.imeth == 6:
                for t in r.txt_ids:
                    fh.write(t.rjust(16).encode("ascii")[:16])
            if r.imeth in (5, 6):
                fh.write(np.array([naux + 1], _I4).tobytes())
                for a in r.aux_names:
                    fh.write(a.ljust(16).encode("ascii")[:16])
            fh.write(np.array([nl], _I4).tobytes())
            if r.imeth == 6:
                id2 = np.zeros(nl, _I4) if r.id2 is None else np.asarray(r.id2, _I4)
                rec = np.dtype([("i", "<i4"), ("j", "<i4"), ("v", rdt, (naux + 1,))])
                arr = np.empty(nl, rec)
                arr["j"] = id2
            else:
                rec = np.dtype([("i", "<i4"), ("v", rdt, (naux + 1,))])
                arr = np.empty(nl, rec)
            arr["i"] = id1
            arr["v"][:, 0] = q
            if naux:
                arr["v"][:, 1:] = aux
            fh.write(arr.tobytes())


def _read_header(buf: bytes, pos: int, precision: int) -> Optional[BudgetHeader]:
    """BudgetReader.f90:563-710 at byte offset ``pos``; None where the
    reference's header read fails."""
    rb = 4 if precision == 1 else 8
    rdt = np.dtype("<f4") if precision == 1 else np.dtype("<f8")
    L = len(buf)

    def i4(p):
        if p + 4 > L:
            raise EOFError
        return int(np.frombuffer(buf, _I4, 1, p)[0])

    try:
        kstp, kper = i4(pos), i4(pos + 4)
        if pos + 24 > L:
            raise EOFError
        text = _s16(buf[pos + 8:pos + 24])
        ncol, nrow, nlay = i4(pos + 24), i4(pos + 28), i4(pos + 32)
        p = pos + 36
        imeth, delt, pertim, totim = 0, 0.0, 0.0, 0.0
        nval, nlist, aux, txt = 0, 0, [], ("", "", "", "")
        if nlay < 0:
            nlay = -nlay
            imeth = i4(p)
            if p + 4 + 3 * rb > L:
                raise EOFError
            delt, pertim, totim = (float(v) for v in np.frombuffer(buf, rdt, 3, p + 4))
            if imeth < 1 or imeth > 6:
                return None
            p += 4 + 3 * rb
            if imeth == 2:
                nval = 1
                nlist = i4(p)
                p += 4
                if nlist < 0:
                    return None
            elif imeth in (5, 6):
                if imeth == 6:
                    if p + 64 > L:
                        raise EOFError
                    txt = tuple(_s16(buf[p + 16 * k:p + 16 * (k + 1)]).strip() for k in range(4))
                    p += 64
                nval = i4(p)
                p += 4
                if nval < 0:
                    return None
                for _ in range(nval - 1):
                    if p + 16 > L:
                        raise EOFError
                    aux.append(_s16(buf[p:p + 16]).strip())
                    p += 16
                nlist = i4(p)
                p += 4
                if nlist < 0:
                    return None
    except EOFError:
        return None
    if imeth in (0, 1):
        nbytes = rb * ncol * nrow * nlay
    elif imeth in (2, 5):
        nbytes = nlist * (rb * nval + 4)
    elif imeth == 6:
        nbytes = nlist * (rb * nval + 8)
    elif imeth == 3:
        nbytes = (rb + 4) * nrow * ncol
    else:
        nbytes = rb * nrow * ncol
    return BudgetHeader(kstp, kper, text, ncol, nrow, nlay, imeth, delt, pertim, totim, nval, nlist, aux, txt,
                        p, nbytes)


@dataclass
class BudgetFile:
    path: str
    precision: int              # 1 single, 2 double
    headers: List[BudgetHeader]
    budget_type: int            # 2: FLOW-JA-FACE (unstructured / MODFLOW 6); 1: right/front/lower face
    file_format: int            # 1: all records method 0; 2: all compact
    flow_array_size: int

    def record_range(self, kper: int, kstp: int) -> range:
        """Indexes of the records of one time step (BudgetReader.f90:107-140)."""
        idx = [i for i, h in enumerate(self.headers) if h.kper == kper and h.kstp == kstp]
        if not idx:
            return range(0)
        first = idx[0]
        last = first
        while last + 1 < len(self.headers) and self.headers[last + 1].kper == kper and \
                self.headers[last + 1].kstp == kstp:
            last += 1
        return range(first, last + 1)

    def time_steps(self) -> List[tuple]:
        out = []
        for h in self.headers:
            if not out or out[-1] != (h.kper, h.kstp):
                out.append((h.kper, h.kstp))
        return out

    def read(self, i: int) -> BudgetRecord:
        h = self.headers[i]
        rdt = np.dtype("<f4") if self.precision == 1 else np.dtype("<f8")
        with open(self.path, "rb") as fh:
            fh.seek(h.data_pos)
            raw = fh.read(h.data_bytes)
        if len(raw) != h.data_bytes:
            raise ValueError(f"{self.path}: record {i} ends early")
        rec = BudgetRecord(h.kstp, h.kper, h.label, h.imeth, (h.ncol, h.nrow, h.nlay), h.delt, h.pertim, h.totim,
                           aux_names=list(h.aux_names), txt_ids=h.txt_ids)
        if h.imeth in (0, 1):
            rec.array = np.frombuffer(raw, rdt).astype(np.float64)
            return rec
        if h.imeth in (3, 4):
            raise NotImplementedError("layer-indicator budget records (MODFLOW-2005 methods 3 and 4)")
        nv = h.nval
        if h.imeth == 2 or h.imeth == 5:
            if nv < 1:
                raise ValueError(f"{self.path}: list record {h.label} has no values")
            dt = np.dtype([("i", "<i4"), ("v", rdt, (nv,))])
        else:
            if nv < 1:
                raise ValueError(f"{self.path}: list record {h.label} has no values")
            dt = np.dtype([("i", "<i4"), ("j", "<i4"), ("v", rdt, (nv,))])
        arr = np.frombuffer(raw, dt, h.nlist)
        rec.id1 = arr["i"].astype(np.int32)
        rec.id2 = arr["j"].astype(np.int32) if h.imeth == 6 else np.zeros(h.nlist, np.int32)
        v = arr["v"].reshape(h.nlist, nv).astype(np.float64)
        rec.q = v[:, 0].copy()
        rec.aux = v[:, 1:].copy()
        return rec


def _scan_budget(buf: bytes, precision: int) -> Optional[BudgetFile]:
    """BudgetReader.f90:713-850 for one precision; None where it fails."""
    L = len(buf)
    pos, headers = 0, []
    has_ja = has_face = False
    flow_size = 0
    while pos < L:
        h = _read_header(buf, pos, precision)
        if h is None:
            return None
        headers.append(h)
        lab = h.label
        if lab in ("FLOW JA FACE", "FLOW-JA-FACE") and h.imeth in (0, 1):
            has_ja = True
            flow_size = h.ncol
        if lab in ("FLOW FRONT FACE", "FLOW RIGHT FACE"):
            has_face = True
            flow_size = h.ncol * h.nrow * h.nlay
        nxt = h.data_pos + h.data_bytes
        if nxt <= pos or nxt > L:
            # (1-based, the reference accepts a next position of file size + 1: the end)
            return None
        pos = nxt
    eq0 = sum(1 for h in headers if h.imeth == 0)
    gt0 = len(headers) - eq0
    fmt = 1 if (headers and eq0 == len(headers)) else (2 if (headers and gt0 == len(headers)) else 0)
    btype = 2 if has_ja else (1 if has_face else 0)
    if fmt == 0 or btype == 0:
        return None
    return BudgetFile("", precision, headers, btype, fmt, flow_size)


def read_budget(path) -> BudgetFile:
    """Open a budget file: single precision tried first, then double
    (BudgetReader.f90:452-508); the file must hold FLOW-JA-FACE (MODFLOW 6)
    or right/front face flows, and be all-standard or all-compact."""
    with open(path, "rb") as fh:
        buf = fh.read()
    for prec in (1, 2):
        bf = _scan_budget(buf, prec)
        if bf is not None:
            bf.path = str(path)
            return bf
    raise ValueError(f"{path}: not a budget file this reader accepts")


# --------------------------------------------------------------------------- flow


@dataclass
class TimeStepFlow:
    """The per-time-step budget arrays of FlowModelData after LoadTimeStep."""
    flowja: np.ndarray
    source_flow: np.ndarray
    sink_flow: np.ndarray
    storage_flow: np.ndarray
    boundary_flows: np.ndarray      # 6 per cell, IFACE 1..6
    heads: np.ndarray
    iboundts: np.ndarray
    steady_state: bool


def _by_sign(cells0, vals, src, snk):
    pos = vals > 0
    neg = vals < 0
    np.add.at(src, cells0[pos], vals[pos])
    np.add.at(snk, cells0[neg], vals[neg])


def load_time_step(grb: Mf6Grid, heads: HeadFile, budget: BudgetFile, kper: int, kstp: int,
                   hdry: float = -1.0e30, default_iface: Optional[Dict[str, int]] = None,
                   ibound: Optional[np.ndarray] = None) -> TimeStepFlow:
    """FlowModelData.f90:225-625 (LoadTimeStep) for a MODFLOW 6 DIS grid."""
    if budget.budget_type != 2:
        raise ValueError("a MODFLOW 6 DIS grid needs FLOW-JA-FACE in the budget file")
    g = grb.grid
    n = g.ncell
    rng = budget.record_range(kper, kstp)
    if len(rng) == 0:
        raise ValueError(f"missing budget information for period {kper} step {kstp}: the budget file must have "
                         "output for every time step")
    ib = grb.ibound if ibound is None else np.asarray(ibound, np.int32)
    dflt = {k.strip().upper(): int(v) for k, v in (default_iface or {}).items()}
    h = heads.get(kper, kstp)
    if h.shape[0] != n:
        raise ValueError(f"head record holds {h.shape[0]} cells, the grid {n}")
    # dry cells of convertible layers (FlowModelData.f90:255-273), compared in single precision
    ibts = ib.astype(np.int32).copy()
    tol = np.float32(abs(np.float32(np.finfo(np.float32).eps) * np.float32(hdry)))
    with np.errstate(over="ignore", invalid="ignore"):
        diff = h.astype(np.float32) - np.float32(hdry)
        dry = (grb.icelltype == 1) & (np.abs(diff) < tol)
    ibts[dry] = 0

    flowja = np.zeros(grb.ja.shape[0])
    src, snk, sto = np.zeros(n), np.zeros(n), np.zeros(n)
    bnd = np.zeros(6 * n)
    steady = True
    for i in rng:
        hd = budget.headers[i]
        lab = hd.label
        if lab in ("DATA-SPDIS", "DATA-SAT"):
            continue
        if hd.imeth in (3, 4):
            raise NotImplementedError(f"{lab}: layer-indicator budget records (MODFLOW-2005 methods 3 and 4)")
        rec = budget.read(i)
        if lab in ("CONSTANT HEAD", "CHD"):
            if hd.imeth == 0:
                if hd.array_count == n:
                    _by_sign(np.arange(n), rec.array, src, snk)
            elif hd.imeth == 2:
                _by_sign(rec.id1 - 1, rec.q, src, snk)
            elif hd.imeth in (5, 6):
                _list_iface(rec, dflt.get(lab, 0), src, snk, bnd)
        elif lab in ("FLOW RIGHT FACE", "FLOW FRONT FACE", "FLOW LOWER FACE"):
            raise ValueError(f"{lab}: structured face-flow records belong to MODFLOW-2005 grids")
        elif lab in ("STORAGE", "STO-SS", "STO-SY"):
            if hd.imeth in (0, 1) and hd.array_count == n:
                sto += rec.array
                if np.any(rec.array != 0.0):
                    steady = False
        elif lab in ("FLOW JA FACE", "FLOW-JA-FACE"):
            if hd.imeth in (0, 1):
                if hd.array_count == budget.flow_array_size:
                    if rec.array.shape[0] != flowja.shape[0]:
                        raise ValueError("FLOW-JA-FACE size differs from the grid's NJA")
                    flowja[:] = rec.array
            elif hd.imeth == 6:
                # flows to / from another model: distributed sources and sinks
                _by_sign(rec.id1 - 1, rec.q, src, snk)
        else:
            iface = dflt.get(lab, 0)
            if hd.imeth in (0, 1):
                if hd.array_count == n:
                    if iface > 0:
                        bnd[6 * np.arange(n) + iface - 1] += rec.array
                    else:
                        _by_sign(np.arange(n), rec.array, src, snk)
            elif hd.imeth == 2:
                if iface > 0:
                    np.add.at(bnd, 6 * (rec.id1 - 1) + iface - 1, rec.q)
                else:
                    _by_sign(rec.id1 - 1, rec.q, src, snk)
            elif hd.imeth in (5, 6):
                _list_iface(rec, iface, src, snk, bnd)
    return TimeStepFlow(flowja, src, snk, sto, bnd, h, ibts, steady)


def _list_iface(rec: BudgetRecord, default: int, src, snk, bnd):
    """Per list item: the label's default IFACE, replaced by the item's IFACE
    auxiliary where the list has one; IFACE > 0 adds to that boundary face,
    otherwise the value is a source or sink by sign (FlowModelData.f90:581-605)."""
    k = rec.aux_index("IFACE")
    iface = np.full(rec.q.shape[0], default, np.int64)
    if k >= 0:
        iface = rec.aux[:, k].astype(np.int64)     # Fortran int(): truncation toward zero
    cells0 = (rec.id1 - 1).astype(np.int64)
    b = iface > 0
    np.add.at(bnd, 6 * cells0[b] + iface[b] - 1, rec.q[b])
    _by_sign(cells0[~b], rec.q[~b], src, snk)


def flow_from_mf6(grb: Mf6Grid, heads: HeadFile, budget: BudgetFile, kper: int, kstp: int, porosity, retardation,
                  alpha_l, alpha_t, dm_eff, uniform_dispersion: bool = True, hdry: float = -1.0e30,
                  default_iface: Optional[Dict[str, int]] = None, ibound=None, default_icbound: int = 1,
                  icboundts=None, zones=None, alpha_lv=None, alpha_tv=None) -> Flow:
    """A ``Flow`` for one MODFLOW 6 time step.  Porosity, retardation and the
    dispersion parameters come from the tracking inputs (MPBAS / RWOPTS / DSP),
    the rest from the binary files."""
    ts = load_time_step(grb, heads, budget, kper, kstp, hdry=hdry, default_iface=default_iface, ibound=ibound)
    n = grb.grid.ncell

    def per_cell(v, dt=np.float64):
        a = np.asarray(v, dt).reshape(-1)
        return np.full(n, a[0], dt) if a.shape[0] == 1 else a

    return Flow(ia=grb.ia.copy(), ja=grb.ja.copy(), flowja=ts.flowja, porosity=per_cell(porosity),
                retardation=per_cell(retardation), iboundts=ts.iboundts,
                alpha_l=np.asarray(alpha_l, np.float64).reshape(-1), alpha_t=np.asarray(alpha_t, np.float64).reshape(-1),
                dm_eff=np.asarray(dm_eff, np.float64).reshape(-1), uniform_dispersion=uniform_dispersion,
                steady_state=ts.steady_state, default_icbound=default_icbound, icboundts=icboundts,
                boundary_flows=ts.boundary_flows, heads=ts.heads, celltype=grb.icelltype.copy(),
                source_flow=ts.source_flow, sink_flow=ts.sink_flow, zones=zones, alpha_lv=alpha_lv,
                alpha_tv=alpha_tv)


def write_flow_files(prefix, grid: Grid, flow: Flow, kper: int = 1, kstp: int = 1, delt: float = 1.0,
                     totim: Optional[float] = None, precision: int = 2, chd_cells=None, icelltype=None,
                     idomain=None, boundary_label: str = "WEL", spdis: bool = True):
    """Write ``prefix.grb``, ``prefix.hds`` and ``prefix.bud`` for one steady
    time step of ``flow`` in MODFLOW 6 form: FLOW-JA-FACE (imeth 1), the
    source / sink flows as a CHD list (imeth 6, one item per cell and sign),
    the boundary face flows as a ``boundary_label`` list with an IFACE
    auxiliary, and (optionally) a DATA-SPDIS record that readers skip.
    Returns the three paths."""
    prefix = os.fspath(prefix)
    n = grid.ncell
    totim = delt if totim is None else totim
    write_grb(prefix + ".grb", grid, flow.ia, flow.ja, idomain=idomain,
              icelltype=flow.celltype if icelltype is None and flow.celltype is not None else icelltype)
    hd = flow.heads if flow.heads is not None else np.zeros(n)
    write_heads(prefix + ".hds", [(kstp, kper, delt, totim, np.asarray(hd).reshape(grid.nlay, grid.nrow, grid.ncol))],
                precision=precision)
    recs = [BudgetRecord(kstp, kper, "FLOW-JA-FACE", 1, (flow.ja.shape[0], 1, 1), delt, delt, totim,
                         array=np.asarray(flow.flowja, np.float64))]
    ids, qs = [], []
    for arr in (flow.source_flow, flow.sink_flow):
        if arr is None:
            continue
        a = np.asarray(arr, np.float64)
        c = np.nonzero(a)[0]
        ids.append(c + 1)
        qs.append(a[c])
    if ids:
        id1 = np.concatenate(ids).astype(np.int32)
        recs.append(BudgetRecord(kstp, kper, "CHD", 6, (n, 1, 1), delt, delt, totim, id1=id1, id2=id1.copy(),
                                 q=np.concatenate(qs), aux=np.zeros((id1.shape[0], 0)), aux_names=[],
                                 txt_ids=("GWF", "GWF", "GWF", "CHD-1")))
    if flow.boundary_flows is not None:
        bf = np.asarray(flow.boundary_flows, np.float64).reshape(n, 6)
        c, f = np.nonzero(bf)
        id1 = (c + 1).astype(np.int32)
        recs.append(BudgetRecord(kstp, kper, boundary_label, 6, (n, 1, 1), delt, delt, totim, id1=id1,
                                 id2=np.arange(1, id1.shape[0] + 1, dtype=np.int32), q=bf[c, f],
                                 aux=(f + 1).astype(np.float64).reshape(-1, 1), aux_names=["IFACE"],
                                 txt_ids=("GWF", "GWF", "GWF", boundary_label + "-1")))
    if spdis:
        cells = np.arange(1, n + 1, dtype=np.int32)
        recs.append(BudgetRecord(kstp, kper, "DATA-SPDIS", 6, (n, 1, 1), delt, delt, totim, id1=cells,
                                 id2=cells.copy(), q=np.zeros(n), aux=np.zeros((n, 3)), aux_names=["QX", "QY", "QZ"],
                                 txt_ids=("GWF", "GWF", "GWF", "NPF")))
    write_budget(prefix + ".bud", recs, precision=precision)
    return prefix + ".grb", prefix + ".hds", prefix + ".bud"
