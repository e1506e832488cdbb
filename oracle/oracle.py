"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a C restatement of MODPATH-RW's tracking path
(``mprw_oracle.c``) and GPKDE histogram; tests use it as the parity checker
and ``bench.py`` times it as the CPU baseline.  The shipped library never
imports this module.  Parity with the Fortran reference is unpinned by
reference golden vectors (none exist); see ``mprw_oracle.c``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "libmprw_oracle.so"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint64)

RNG_XOROSHIRO = 0  # reference streams (rng_par_zig) + Irwin-Hall(12)
RNG_PHILOX = 1     # the GPU library's counter-based stream


class OrcFlow(C.Structure):
    _fields_ = [("nlay", C.c_int), ("nrow", C.c_int), ("ncol", C.c_int), ("delr", _dp), ("delc", _dp),
                ("top", _dp), ("botm", _dp), ("ia", _ip), ("ja", _ip), ("nja", C.c_int), ("flowja", _dp),
                ("bflow", _dp), ("porosity", _dp), ("retardation", _dp), ("ibound", _ip), ("iboundts", _ip),
                ("icboundts", _ip), ("default_icbound", C.c_int), ("heads", _dp), ("celltype", _ip),
                ("source_flow", _dp), ("sink_flow", _dp), ("zones", _ip), ("alpha_l", _dp), ("alpha_t", _dp),
                ("dm_eff", _dp), ("uniform_dispersion", C.c_int), ("steady_state", C.c_int),
                ("alpha_lv", _dp), ("alpha_tv", _dp)]


class OrcOptions(C.Structure):
    _fields_ = [("time_step_kind", C.c_int), ("ts_param", C.c_double * 2), ("advection_kind", C.c_int),
                ("dim_mask", C.c_int * 3), ("stop_weak_sinks", C.c_int), ("stop_weak_sources", C.c_int),
                ("backward", C.c_int), ("stop_zone", C.c_int), ("uniform_porosity", C.c_int),
                ("rng_kind", C.c_int), ("seed", C.c_uint64), ("nthreads", C.c_int), ("dispersion_model", C.c_int)]


_lib = None


def build() -> Path:
    """Compile the oracle with its Makefile (gcc)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    srcs = list(HERE.glob("*.c")) + list(HERE.glob("*.h"))
    if not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in srcs):
        build()
    L = C.CDLL(str(LIB))
    L.orc_advance.restype = C.c_int
    L.orc_advance.argtypes = [C.POINTER(OrcFlow), C.POINTER(OrcOptions), C.c_int64, _ip, _dp, _dp, _dp, _dp, _ip,
                              _up, _up, C.c_double, C.c_double, C.POINTER(C.c_int64)]
    L.orc_global_xyz.restype = None
    L.orc_global_xyz.argtypes = [C.POINTER(OrcFlow), C.c_int64, _ip, _dp, _dp, _dp, _dp, _dp, _dp]
    L.orc_cell_record.restype = C.c_int
    L.orc_cell_record.argtypes = [C.POINTER(OrcFlow), C.POINTER(OrcOptions), C.c_int, _dp, _dp, _dp, _dp, _dp,
                                  _ip, _ip]
    L.orc_xoro_seed_stream.argtypes = [C.c_int, _up]
    L.orc_xoro_reset.restype = None
    L.orc_xoro_reset.argtypes = []
    L.orc_xoro_next.restype = C.c_uint64
    L.orc_xoro_next.argtypes = [_up]
    L.orc_xoro_uniform.restype = C.c_double
    L.orc_xoro_uniform.argtypes = [_up]
    L.orc_xoro_normal_ih12.restype = C.c_double
    L.orc_xoro_normal_ih12.argtypes = [_up]
    L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    L.orc_philox_normal_ih12.restype = C.c_double
    L.orc_philox_normal_ih12.argtypes = [C.c_uint64, C.c_uint64, _up]
    _lib = L
    return L


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


class _Inputs:
    """Holds contiguous copies so the pointers stay valid for one call."""

    def __init__(self, grid, flow, opt, rng_kind, nthreads):
        f64 = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
        i32 = lambda a: None if a is None else np.ascontiguousarray(a, np.int32)
        self.k = dict(delr=f64(grid.delr), delc=f64(grid.delc), top=f64(grid.top), botm=f64(grid.botm),
                      ia=i32(flow.ia), ja=i32(flow.ja), flowja=f64(flow.flowja), bflow=f64(flow.boundary_flows),
                      por=f64(flow.porosity), ret=f64(flow.retardation), ibts=i32(flow.iboundts),
                      icb=i32(flow.icboundts), heads=f64(flow.heads), ct=i32(flow.celltype),
                      src=f64(flow.source_flow), snk=f64(flow.sink_flow), zn=i32(flow.zones),
                      aL=f64(flow.alpha_l), aT=f64(flow.alpha_t), dm=f64(flow.dm_eff),
                      aLV=f64(getattr(flow, "alpha_lv", None)), aTV=f64(getattr(flow, "alpha_tv", None)))
        k = self.k
        self.f = OrcFlow(grid.nlay, grid.nrow, grid.ncol, _p(k["delr"], _dp), _p(k["delc"], _dp),
                         _p(k["top"], _dp), _p(k["botm"], _dp), _p(k["ia"], _ip), _p(k["ja"], _ip),
                         int(k["ja"].shape[0]), _p(k["flowja"], _dp), _p(k["bflow"], _dp), _p(k["por"], _dp),
                         _p(k["ret"], _dp), _p(k["ibts"], _ip), _p(k["ibts"], _ip), _p(k["icb"], _ip),
                         int(flow.default_icbound), _p(k["heads"], _dp), _p(k["ct"], _ip), _p(k["src"], _dp),
                         _p(k["snk"], _dp), _p(k["zn"], _ip), _p(k["aL"], _dp), _p(k["aT"], _dp),
                         _p(k["dm"], _dp), int(flow.uniform_dispersion), int(flow.steady_state),
                         _p(k["aLV"], _dp), _p(k["aTV"], _dp))
        o = OrcOptions()
        o.time_step_kind = opt.time_step_kind
        o.ts_param[0], o.ts_param[1] = float(opt.ts_param[0]), float(opt.ts_param[1])
        o.advection_kind = opt.advection_kind
        for d in range(3):
            o.dim_mask[d] = int(opt.dim_mask[d])
        o.stop_weak_sinks = int(opt.stop_weak_sinks)
        o.stop_weak_sources = int(opt.stop_weak_sources)
        o.backward = int(opt.backward)
        o.stop_zone = int(opt.stop_zone)
        o.uniform_porosity = int(opt.uniform_porosity)
        o.rng_kind = rng_kind
        o.seed = int(opt.rng_seed) & 0xFFFFFFFFFFFFFFFF
        o.nthreads = nthreads
        o.dispersion_model = int(getattr(opt, "dispersion_model", 0))
        self.o = o


def reset_xoroshiro():
    """Start a new run of the reference's RNG: the xoroshiro128+ thread streams
    (rng_kind RNG_XOROSHIRO) are seeded again on their next use.  Otherwise
    they continue across advance() calls, as the reference seeds them once per
    run (TrackSubCell.F90:613-620) and every tracking interval draws on."""
    lib().orc_xoro_reset()


def advance(grid, flow, opt, particles, t_begin, t_end, rng_kind=RNG_PHILOX, nthreads=1):
    """Advance a copy of ``particles``; returns (particles, particle_steps).
    With RNG_XOROSHIRO the thread streams continue from the previous call
    (reset_xoroshiro() starts a new run); with nthreads=1 the result is the
    reference's single-threaded run, deterministic."""
    L = lib()
    inp = _Inputs(grid, flow, opt, rng_kind, nthreads)
    p = particles.copy()
    n = p.n
    cell = np.ascontiguousarray(p.cell, np.int32)
    lx, ly, lz, t = (np.ascontiguousarray(a, np.float64) for a in (p.lx, p.ly, p.lz, p.t))
    st = np.ascontiguousarray(p.status, np.int32)
    ids = np.arange(n, dtype=np.uint64) if p.id is None else np.ascontiguousarray(p.id, np.uint64)
    ctr = np.zeros(n, np.uint64) if p.rng_ctr is None else np.ascontiguousarray(p.rng_ctr, np.uint64)
    steps = C.c_int64(0)
    rc = L.orc_advance(C.byref(inp.f), C.byref(inp.o), n, _p(cell, _ip), _p(lx, _dp), _p(ly, _dp), _p(lz, _dp),
                       _p(t, _dp), _p(st, _ip), _p(ids, _up), _p(ctr, _up), float(t_begin), float(t_end),
                       C.byref(steps))
    if rc != 0:
        raise RuntimeError(f"orc_advance rc={rc}")
    p.cell, p.lx, p.ly, p.lz, p.t, p.status, p.rng_ctr = cell, lx, ly, lz, t, st, ctr
    if p.id is None:
        p.id = ids
    return p, steps.value


def global_xyz(grid, flow, p):
    L = lib()
    inp = _Inputs(grid, flow, _default_opt(), 1, 1)
    n = p.n
    out = [np.empty(n) for _ in range(3)]
    cell = np.ascontiguousarray(p.cell, np.int32)
    lx, ly, lz = (np.ascontiguousarray(a, np.float64) for a in (p.lx, p.ly, p.lz))
    L.orc_global_xyz(C.byref(inp.f), n, _p(cell, _ip), _p(lx, _dp), _p(ly, _dp), _p(lz, _dp), _p(out[0], _dp),
                     _p(out[1], _dp), _p(out[2], _dp))
    return out


def cell_record(grid, flow, opt, cell):
    L = lib()
    inp = _Inputs(grid, flow, opt, 1, 1)
    v6, q32, p8, d72 = np.empty(6), np.empty(32), np.empty(8), np.empty(72)
    mb6, c6 = np.empty(6, np.int32), np.empty(6, np.int32)
    dt = C.c_double()
    rc = L.orc_cell_record(C.byref(inp.f), C.byref(inp.o), int(cell), _p(v6, _dp), C.byref(dt), _p(q32, _dp),
                           _p(p8, _dp), _p(d72, _dp), _p(mb6, _ip), _p(c6, _ip))
    if rc != 0:
        raise RuntimeError("orc_cell_record failed")
    return dict(vface=v6, dtcell=dt.value, qcorner=q32.reshape(8, 4), phicorner=p8, D=d72.reshape(9, 8),
                massb=mb6, conn=c6)


def _default_opt():
    import types
    return types.SimpleNamespace(time_step_kind=1, ts_param=(0.1, 0.1), advection_kind=2, dim_mask=(1, 1, 1),
                                 stop_weak_sinks=0, stop_weak_sources=0, backward=0, stop_zone=0,
                                 uniform_porosity=1, rng_seed=0)


def xoro_stream(k: int) -> np.ndarray:
    s = np.zeros(2, np.uint64)
    lib().orc_xoro_seed_stream(k, _p(s, _up))
    return s


def xoro_uniforms(state: np.ndarray, n: int) -> np.ndarray:
    L = lib()
    return np.array([L.orc_xoro_uniform(_p(state, _up)) for _ in range(n)])


def xoro_next(state: np.ndarray, n: int) -> np.ndarray:
    L = lib()
    return np.array([L.orc_xoro_next(_p(state, _up)) for _ in range(n)], dtype=np.uint64)


def philox(ctr4, key2):
    c = (C.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr4])
    k = (C.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key2])
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return [o[i] for i in range(4)]


def philox_normals(seed: int, pid: int, n: int, ctr0: int = 0):
    L = lib()
    ctr = np.array([ctr0], np.uint64)
    vals = [L.orc_philox_normal_ih12(seed, pid, _p(ctr, _up)) for _ in range(n)]
    return np.array(vals), int(ctr[0])


def cpu_count() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1
