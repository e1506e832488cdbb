"""The FP64 step kernel's compares on the integer pipe (csrc/fpbits.cuh).

The header compiles as plain C++ for the host; tests/fpbits_check.cpp checks
every bit-pattern test and compare against the IEEE-754 compare it replaces
(special values, values next to each boundary, random bit patterns, pairs
including signed zeros and NaN) and the bit-assembled Irwin-Hall normal
against the FP64 subtraction it replaces.  The device build compiles the same
functions; only the bit casts and the leading-zero count are intrinsics there.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_fpbits_match_ieee_compares(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "fpbits_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(ROOT / "modpath-rw_gb300" / "csrc"),
                    str(ROOT / "tests" / "fpbits_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok "), r.stdout
    assert int(r.stdout.split()[1]) > 5_000_000
