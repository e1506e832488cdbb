"""The C-ABI library: builds, loads without a GPU, and exports every entry
point declared in include/mprw_gpu.h (no compute calls)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "mprw_gpu.h"


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


def test_struct_layouts_match_header():
    import mprw
    # offsets the Fortran bind(C) types rely on
    assert C.sizeof(mprw.GridDesc) == 3 * 4 + 4 + 4 * 8
    assert mprw.OptionsDesc.rng_seed.offset % 8 == 0
    assert mprw.FlowDesc.nja.offset == 16
