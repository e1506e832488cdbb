"""Build the CUDA library (sm_103a) in-tree.

Each translation unit under ``csrc/`` is compiled by nvcc in parallel, then
linked into ``mprw/libmprw_gpu.so``.  No CMake, no torch extension machinery:
the library is a plain C-ABI shared object loaded with ctypes.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
SRC_DIR = PKG_DIR.parent / "csrc"
BUILD_DIR = PKG_DIR.parent / "build"
LIB_PATH = PKG_DIR / "libmprw_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "prep.cu", "step.cu", "hist.cu", "sort.cu", "gpkde.cu", "noalloc.cu", "obs.cu", "series.cu",
           "adjoint.cu"]
# The per-cell records and model coordinates follow the reference's operation
# order exactly, so these units are compiled without multiply-add contraction.
NO_FMAD = {"prep.cu", "hist.cu", "noalloc.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile every .cu to an object and link libmprw_gpu.so; returns its path."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    headers = list(SRC_DIR.glob("*.cuh")) + [PKG_DIR.parent.parent / "include" / "mprw_gpu.h"]
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
    flags += extra_flags or []
    cc = nvcc()
    jobs = []
    for src in SOURCES:
        s = SRC_DIR / src
        o = BUILD_DIR / (src + ".o")
        if _stale(o, [s] + headers) or extra_flags:
            fl = flags + (["-fmad=false"] if src in NO_FMAD else [])
            jobs.append([cc, *fl, "-c", str(s), "-o", str(o)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}")

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    objs = [str(BUILD_DIR / (s + ".o")) for s in SOURCES]
    if jobs or not LIB_PATH.exists():
        run([cc, *ARCH, "-shared", "-o", str(LIB_PATH), *objs, "-lcudart"])
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
