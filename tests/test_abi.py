"""The C-ABI library: builds, loads without a GPU, and exports every entry
point declared in include/mprw_gpu.h (no compute calls); the struct layouts
of the header, of the Python ctypes mirror and of the Fortran bind(C) module
include/mprw_gpu.f90 agree field by field."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "mprw_gpu.h"
FMODULE = ROOT / "include" / "mprw_gpu.f90"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mprw_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib_path():
    from mprw import build as B
    return B.build()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("mprw_create", "mprw_load_flow", "mprw_set_particles", "mprw_advance", "mprw_get_particles",
              "mprw_histogram", "mprw_destroy", "mprw_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT\s+(mprw_[a-z0-9_]+)\b", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing


def test_library_loads_and_binds(lib_path):
    import mprw
    lib = mprw.load_library()
    for s in declared_symbols():
        assert hasattr(lib, s)
    # null-handle calls are rejected without touching the device
    assert lib.mprw_advance(None, 0.0, 1.0, None) == -1
    assert lib.mprw_destroy(None) == 0
    assert lib.mprw_last_error(None) == b"null handle"


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    """Field offsets and sizes of every struct, from a C program compiled against the header."""
    exe = tmp_path_factory.mktemp("abi") / "abi_layout"
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", str(HEADER.parent),
                    str(ROOT / "tests" / "abi_layout.c"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    lay = {}
    for line in out.splitlines():
        struct, field, off, size = line.split()
        d = lay.setdefault(struct, {"fields": [], "sizeof": None})
        if field == "-":
            d["sizeof"] = int(size)
        else:
            d["fields"].append((field, int(off), int(size)))
    return lay


def _ctypes_mirrors():
    import mprw
    return {"mprw_grid_desc": mprw.GridDesc, "mprw_options": mprw.OptionsDesc, "mprw_flow_desc": mprw.FlowDesc,
            "mprw_gpkde_options": mprw.GpkdeOptions, "mprw_series_options": mprw.SeriesOptions,
            "mprw_series_result": mprw.SeriesResult, "mprw_gpkde_sums": mprw.GpkdeSums,
            "mprw_adj_options": mprw.AdjOptions}


def test_header_structs_are_all_probed(c_layout):
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    typedefs = set(re.findall(r"}\s*(mprw_[a-z_]+)\s*;", text))
    assert typedefs == set(c_layout), typedefs ^ set(c_layout)


def test_ctypes_mirror_matches_header(c_layout):
    for name, cls in _ctypes_mirrors().items():
        lay = c_layout[name]
        assert C.sizeof(cls) == lay["sizeof"], name
        names = [f[0] for f in cls._fields_]
        assert names == [f[0] for f in lay["fields"]], name
        for field, off, size in lay["fields"]:
            assert getattr(cls, field).offset == off, (name, field)
            assert getattr(cls, field).size == size, (name, field)


# C sizes of the ISO_C_BINDING kinds used by the module
_FKIND = {"integer(c_int32_t)": 4, "integer(c_int64_t)": 8, "integer(c_int)": 4, "real(c_double)": 8,
          "type(c_ptr)": 8}


def _fortran_types():
    """Fields (name, element size, count) of every bind(C) type of the Fortran module, in order."""
    text = FMODULE.read_text()
    types = {}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)[^\n]*\n(.*?)\n\s*end type", text, flags=re.S):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            kind, names = (x.strip() for x in line.split("::"))
            esize = _FKIND[kind.replace(" ", "")]
            for item in re.findall(r"(\w+)(?:\((\d+)\))?", names):
                fields.append((item[0], esize, int(item[1]) if item[1] else 1))
        types[m.group(1)] = fields
    return types


def test_fortran_bind_c_types_match_header(c_layout):
    ftypes = _fortran_types()
    assert set(ftypes) == set(c_layout), set(ftypes) ^ set(c_layout)
    for name, fields in ftypes.items():
        lay = c_layout[name]
        off = 0
        maxal = 1
        got = []
        for fname, esize, count in fields:
            off = (off + esize - 1) // esize * esize   # C alignment of a scalar / array element
            maxal = max(maxal, esize)
            got.append((fname, off, esize * count))
            off += esize * count
        size = (off + maxal - 1) // maxal * maxal
        assert got == lay["fields"], (name, got, lay["fields"])
        assert size == lay["sizeof"], name


def test_fortran_module_binds_every_entry_point():
    bound = set(re.findall(r'bind\(C, name="(mprw_[a-z0-9_]+)"\)', FMODULE.read_text()))
    missing = [s for s in declared_symbols() if s not in bound]
    assert not missing, missing
    assert bound <= set(declared_symbols()), bound - set(declared_symbols())
