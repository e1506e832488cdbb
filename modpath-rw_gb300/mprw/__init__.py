"""GB300 random-walk particle tracking (host side).

``Tracker`` wraps the C ABI of ``libmprw_gpu.so`` (include/mprw_gpu.h) with
ctypes, mirroring the reference's calls on the tracking path:

=====================  ==========================================================
``Tracker(grid, opt)``  trackingEngine%Initialize (ParticleTrackingEngine.f90:393)
``load_flow(flow)``     FlowModelData%LoadTimeStep + per-cell buffers
``set_particles(p)``    particle group arrays (Particle.f90:7-17)
``advance(t0, t1)``     the OpenMP particle loop of MPathRW.F90:1207-1539
``get_particles()``     particle state + ConvertToModelXYZ
``histogram(...)``      Histogram%ComputeCountsWeighted (Histogram.F90:276-350)
=====================  ==========================================================

There is no CPU fallback: constructing a Tracker without the built library
or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .model import (ACTIVE, ADV, BOUNDARY, DISP, EULERIAN, EXPONENTIAL, FIXED, FP64, INACTIVE, MIN_ADV_DISP,
                    MIXED, NO_EXIT, PENDING, STOP_ZONE, UNDEFINED, UNRELEASED, WEAK_SINK, WEAK_SOURCE, Flow,
                    Grid, Options, Particles)

LIB_PATH = Path(__file__).resolve().parent / "libmprw_gpu.so"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint64)


class MprwError(RuntimeError):
    pass


class MprwAborted(MprwError):
    """An advance stopped by its timeout or by cancel() (MPRW_E_ABORTED)."""


class GridDesc(C.Structure):
    _fields_ = [("nlay", C.c_int32), ("nrow", C.c_int32), ("ncol", C.c_int32),
                ("delr", _dp), ("delc", _dp), ("top", _dp), ("botm", _dp)]


class OptionsDesc(C.Structure):
    _fields_ = [("time_step_kind", C.c_int32), ("ts_param", C.c_double * 2), ("advection_kind", C.c_int32),
                ("dim_mask", C.c_int32 * 3), ("dispersion_model", C.c_int32), ("stop_weak_sinks", C.c_int32),
                ("stop_weak_sources", C.c_int32), ("backward", C.c_int32), ("stop_zone", C.c_int32),
                ("uniform_porosity", C.c_int32), ("rng_seed", C.c_uint64), ("precision", C.c_int32)]


class GpkdeOptions(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("domain_size", C.c_double * 3), ("bin_size", C.c_double * 3),
                ("n_opt_loops", C.c_int32), ("min_hover_delta", C.c_double), ("delta_hover_delta", C.c_double),
                ("max_hover_delta", C.c_double), ("rel_err_convergence", C.c_double),
                ("skip_error_convergence", C.c_int32), ("unit_volume", C.c_int32), ("scaling_factor", C.c_double),
                ("precision", C.c_int32), ("isotropic", C.c_int32)]


class GpkdeSums(C.Structure):
    _fields_ = [("n_active", C.c_double), ("sum_w", C.c_double), ("sum_w2", C.c_double),
                ("sum_dx", C.c_double * 3), ("sum_dx2", C.c_double * 3)]


class AdjOptions(C.Structure):
    _fields_ = [("nzones", C.c_int32), ("nsteps", C.c_int32), ("checkpoint", C.c_int32), ("dt", C.c_double),
                ("velocity_floor", C.c_double), ("seed", C.c_uint64), ("origin", C.c_double * 3),
                ("bin_size", C.c_double * 3), ("n_bins", C.c_int32 * 3), ("bandwidth", C.c_double * 3)]


class SeriesOptions(C.Structure):
    _fields_ = [("origin", C.c_double), ("domain_size", C.c_double), ("bin_size", C.c_double),
                ("bin_format", C.c_int32), ("bin_size_fraction", C.c_double), ("adapt_grid", C.c_int32),
                ("exact_point", C.c_int32), ("effective_weight_format", C.c_int32),
                ("initial_smoothing_selection", C.c_int32), ("initial_smoothing_factor", C.c_double),
                ("apply_initial_factor", C.c_int32), ("n_opt_loops", C.c_int32), ("rel_err_convergence", C.c_double),
                ("skip_error_convergence", C.c_int32), ("only_histogram", C.c_int32),
                ("compute_raw_density", C.c_int32), ("unit_volume", C.c_int32)]


class SeriesResult(C.Structure):
    _fields_ = [("n_bins", C.c_int32), ("delta_bins_origin", C.c_int32), ("bin_size", C.c_double),
                ("grid_origin", C.c_double), ("loops_done", C.c_int32), ("active_bins", C.c_int32)]


class FlowDesc(C.Structure):
    _fields_ = [("ia", _ip), ("ja", _ip), ("nja", C.c_int64), ("flowja", _dp), ("boundary_flows", _dp),
                ("porosity", _dp), ("retardation", _dp), ("iboundts", _ip), ("icboundts", _ip),
                ("default_icbound", C.c_int32), ("heads", _dp), ("celltype", _ip), ("source_flow", _dp),
                ("sink_flow", _dp), ("zones", _ip), ("alpha_l", _dp), ("alpha_t", _dp), ("dm_eff", _dp),
                ("uniform_dispersion", C.c_int32), ("steady_state", C.c_int32), ("alpha_lv", _dp),
                ("alpha_tv", _dp)]


_lib = None


def load_library() -> C.CDLL:
    """Load libmprw_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise MprwError(f"{LIB_PATH} is missing: build it with mprw.build.build()")
    lib = C.CDLL(str(LIB_PATH))
    H = C.c_void_p
    sig = {
        "mprw_create": (C.c_int, [C.POINTER(H), C.POINTER(GridDesc), C.POINTER(OptionsDesc)]),
        "mprw_load_flow": (C.c_int, [H, C.POINTER(FlowDesc)]),
        "mprw_set_particles": (C.c_int, [H, C.c_int64, _ip, _dp, _dp, _dp, _dp, _ip, _dp, _up, _up]),
        "mprw_advance": (C.c_int, [H, C.c_double, C.c_double, C.POINTER(C.c_int64)]),
        "mprw_get_particles": (C.c_int, [H, _ip, _dp, _dp, _dp, _dp, _ip, _up, _dp, _dp, _dp]),
        "mprw_histogram": (C.c_int, [H, _dp, _dp, _ip, _dp, C.POINTER(C.c_int64), _dp]),
        "mprw_gpkde": (C.c_int, [H, C.POINTER(GpkdeOptions), _dp, _dp, _ip, _ip]),
        "mprw_gpkde_partial": (C.c_int, [H, C.POINTER(GpkdeOptions), _dp, C.POINTER(GpkdeSums)]),
        "mprw_adj_setup": (C.c_int, [H, _ip, C.POINTER(AdjOptions)]),
        "mprw_adj_forward": (C.c_int, [H, _dp, _dp]),
        "mprw_adj_backward": (C.c_int, [H, _dp, _dp]),
        "mprw_gpkde_from_counts": (C.c_int, [H, C.POINTER(GpkdeOptions), _dp, C.POINTER(GpkdeSums), _dp, _dp, _ip,
                                             _ip]),
        "mprw_set_observations": (C.c_int, [H, C.c_int32, _ip, _ip, C.c_int32, _ip]),
        "mprw_observe_resident": (C.c_int, [H, C.POINTER(C.c_int64), _dp]),
        "mprw_observe_sinks": (C.c_int, [H, C.c_int64, _ip, _up, _dp, _dp, C.POINTER(C.c_int64)]),
        "mprw_set_stream": (C.c_int, [H, C.c_void_p]),
        "mprw_last_timings": (C.c_int, [H, _dp, _dp, _dp, _dp, C.POINTER(C.c_int64)]),
        "mprw_last_gpkde_work": (C.c_int, [H, _dp]),
        "mprw_destroy": (C.c_int, [H]),
        "mprw_create_batch": (C.c_int, [C.POINTER(H), C.c_int32, C.POINTER(GridDesc), C.POINTER(OptionsDesc)]),
        "mprw_batch_member": (C.c_int, [H, C.c_int32, C.POINTER(H)]),
        "mprw_set_particles_batch": (C.c_int, [H, C.POINTER(C.c_int64), _ip, _dp, _dp, _dp, _dp, _ip, _dp, _up,
                                               _up]),
        "mprw_gpkde_batch": (C.c_int, [H, C.POINTER(GpkdeOptions), C.POINTER(_dp), C.POINTER(_dp), _ip,
                                       C.c_int32]),
        "mprw_set_tuning": (C.c_int, [H, C.c_int32, C.c_int32]),
        "mprw_set_timeout": (C.c_int, [H, C.c_double]),
        "mprw_cancel": (C.c_int, [H]),
        "mprw_get_tuning": (C.c_int, [H, _ip, _ip, _ip]),
        "mprw_autotune": (C.c_int, [H, C.c_double, C.c_double, _ip, _ip, _dp]),
        "mprw_last_error": (C.c_char_p, [H]),
        "mprw_gpkde_series": (C.c_int, [_dp, _dp, C.c_int64, C.POINTER(SeriesOptions), C.c_int32, _dp, _dp, _dp,
                                        C.POINTER(SeriesResult), C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def _p(a, ptype):
    return None if a is None else a.ctypes.data_as(ptype)


def _grid_desc(grid: Grid, keep: list) -> GridDesc:
    g = dict(delr=_f64(grid.delr), delc=_f64(grid.delc), top=_f64(grid.top), botm=_f64(grid.botm))
    keep.append(g)
    return GridDesc(grid.nlay, grid.nrow, grid.ncol, _p(g["delr"], _dp), _p(g["delc"], _dp), _p(g["top"], _dp),
                    _p(g["botm"], _dp))


def _options_desc(opt: Options) -> OptionsDesc:
    od = OptionsDesc()
    od.time_step_kind = opt.time_step_kind
    od.ts_param[0], od.ts_param[1] = float(opt.ts_param[0]), float(opt.ts_param[1])
    od.advection_kind = opt.advection_kind
    for d in range(3):
        od.dim_mask[d] = int(opt.dim_mask[d])
    od.dispersion_model = opt.dispersion_model
    od.stop_weak_sinks = int(opt.stop_weak_sinks)
    od.stop_weak_sources = int(opt.stop_weak_sources)
    od.backward = int(opt.backward)
    od.stop_zone = int(opt.stop_zone)
    od.uniform_porosity = int(opt.uniform_porosity)
    od.rng_seed = int(opt.rng_seed) & 0xFFFFFFFFFFFFFFFF
    od.precision = int(opt.precision)
    return od


class Tracker:
    """One device-resident tracking engine (one C-ABI handle)."""

    def __init__(self, grid: Grid, opt: Options):
        self.lib = load_library()
        self.grid = grid
        self.opt = opt
        self._keep = []
        gd = _grid_desc(grid, self._keep)
        od = _options_desc(opt)
        self.h = C.c_void_p()
        rc = self.lib.mprw_create(C.byref(self.h), C.byref(gd), C.byref(od))
        if rc != 0:
            msg = self.lib.mprw_last_error(self.h).decode() if self.h.value else "mprw_create failed"
            if self.h.value:
                self.lib.mprw_destroy(self.h)
                self.h = C.c_void_p()
            raise MprwError(f"mprw_create: rc={rc}: {msg}")
        self.n = 0

    def _check(self, rc, what):
        if rc != 0:
            cls = MprwAborted if rc == -5 else MprwError
            raise cls(f"{what}: rc={rc}: {self.lib.mprw_last_error(self.h).decode()}")

    def load_flow(self, f: Flow):
        keep = dict(ia=_i32(f.ia), ja=_i32(f.ja), flowja=_f64(f.flowja), por=_f64(f.porosity),
                    ret=_f64(f.retardation), ibts=_i32(f.iboundts), aL=_f64(f.alpha_l), aT=_f64(f.alpha_t),
                    dm=_f64(f.dm_eff))
        opt = dict(icb=(f.icboundts, _i32, _ip), bf=(f.boundary_flows, _f64, _dp), hd=(f.heads, _f64, _dp),
                   ct=(f.celltype, _i32, _ip), src=(f.source_flow, _f64, _dp), snk=(f.sink_flow, _f64, _dp),
                   zn=(f.zones, _i32, _ip), aLV=(f.alpha_lv, _f64, _dp), aTV=(f.alpha_tv, _f64, _dp))
        ptrs = {}
        for k, (arr, conv, pt) in opt.items():
            keep[k] = None if arr is None else conv(arr)
            ptrs[k] = _p(keep[k], pt)
        fd = FlowDesc()
        fd.ia = _p(keep["ia"], _ip)
        fd.ja = _p(keep["ja"], _ip)
        fd.nja = keep["ja"].shape[0]
        fd.flowja = _p(keep["flowja"], _dp)
        fd.boundary_flows = ptrs["bf"]
        fd.porosity = _p(keep["por"], _dp)
        fd.retardation = _p(keep["ret"], _dp)
        fd.iboundts = _p(keep["ibts"], _ip)
        fd.icboundts = ptrs["icb"]
        fd.default_icbound = int(f.default_icbound)
        fd.heads = ptrs["hd"]
        fd.celltype = ptrs["ct"]
        fd.source_flow = ptrs["src"]
        fd.sink_flow = ptrs["snk"]
        fd.zones = ptrs["zn"]
        fd.alpha_l = _p(keep["aL"], _dp)
        fd.alpha_t = _p(keep["aT"], _dp)
        fd.dm_eff = _p(keep["dm"], _dp)
        fd.uniform_dispersion = int(f.uniform_dispersion)
        fd.steady_state = int(f.steady_state)
        fd.alpha_lv = ptrs["aLV"]
        fd.alpha_tv = ptrs["aTV"]
        self._check(self.lib.mprw_load_flow(self.h, C.byref(fd)), "mprw_load_flow")

    def set_particles(self, p: Particles):
        arrs = dict(cell=_i32(p.cell), lx=_f64(p.lx), ly=_f64(p.ly), lz=_f64(p.lz), t=_f64(p.t),
                    st=_i32(p.status), m=None if p.mass is None else _f64(p.mass),
                    id=None if p.id is None else _u64(p.id), rc=None if p.rng_ctr is None else _u64(p.rng_ctr))
        self._check(self.lib.mprw_set_particles(
            self.h, p.n, _p(arrs["cell"], _ip), _p(arrs["lx"], _dp), _p(arrs["ly"], _dp), _p(arrs["lz"], _dp),
            _p(arrs["t"], _dp), _p(arrs["st"], _ip), _p(arrs["m"], _dp), _p(arrs["id"], _up),
            _p(arrs["rc"], _up)), "mprw_set_particles")
        self.n = p.n
        self._ids, self._mass = arrs["id"], arrs["m"]   # host copies for checkpoints

    def checkpoint(self, path):
        """Write the particle state (cell, local x/y/z, time, status, random
        counter, id, mass) to ``path`` (.npz).  With counter-based random
        numbers, restore() + the remaining advances reproduce an
        uninterrupted run bit for bit."""
        o = self.get_particles(global_xyz=False)
        n = self.n
        np.savez(path, cell=o["cell"], lx=o["lx"], ly=o["ly"], lz=o["lz"], t=o["t"], status=o["status"],
                 rng_ctr=o["rng_ctr"], id=np.arange(n, dtype=np.uint64) if self._ids is None else self._ids,
                 mass=np.ones(n) if self._mass is None else self._mass, has_id=self._ids is not None)

    def restore(self, path):
        """Set the particles from a checkpoint() file."""
        d = np.load(path)
        self.set_particles(Particles(cell=d["cell"], lx=d["lx"], ly=d["ly"], lz=d["lz"], t=d["t"],
                                     status=d["status"], mass=d["mass"],
                                     id=d["id"] if bool(d["has_id"]) else None, rng_ctr=d["rng_ctr"]))

    def advance(self, t_begin: float, t_end: float) -> int:
        steps = C.c_int64(0)
        self._check(self.lib.mprw_advance(self.h, float(t_begin), float(t_end), C.byref(steps)), "mprw_advance")
        return steps.value

    def get_particles(self, global_xyz: bool = True) -> dict:
        n = self.n
        out = dict(cell=np.empty(n, np.int32), lx=np.empty(n), ly=np.empty(n), lz=np.empty(n), t=np.empty(n),
                   status=np.empty(n, np.int32), rng_ctr=np.empty(n, np.uint64))
        g = [np.empty(n) for _ in range(3)] if global_xyz else [None] * 3
        self._check(self.lib.mprw_get_particles(
            self.h, _p(out["cell"], _ip), _p(out["lx"], _dp), _p(out["ly"], _dp), _p(out["lz"], _dp),
            _p(out["t"], _dp), _p(out["status"], _ip), _p(out["rng_ctr"], _up), _p(g[0], _dp), _p(g[1], _dp),
            _p(g[2], _dp)), "mprw_get_particles")
        if global_xyz:
            out["gx"], out["gy"], out["gz"] = g
        return out

    def histogram(self, origin, bin_size, n_bins):
        """Weighted counts of the active particles, shape (nz, ny, nx), plus (n_binned, eff_mass)."""
        o, b = _f64(origin), _f64(bin_size)
        nb = _i32(n_bins)
        counts = np.empty(int(np.prod(nb)), np.float64)
        nbinned = C.c_int64(0)
        eff = C.c_double(0)
        self._check(self.lib.mprw_histogram(self.h, _p(o, _dp), _p(b, _dp), _p(nb, _ip), _p(counts, _dp),
                                            C.byref(nbinned), C.byref(eff)), "mprw_histogram")
        return counts.reshape(int(nb[2]), int(nb[1]), int(nb[0])), nbinned.value, eff.value

    @staticmethod
    def gpkde_options(domain_size, bin_size, origin=(0.0, 0.0, 0.0), n_opt_loops=10, kdb=(0.3, 0.3, 15.0),
                      rel_err=0.02, skip_error=False, unit_volume=True, scaling_factor=1.0,
                      precision=FP64, isotropic=False) -> "GpkdeOptions":
        """The mprw_gpkde_options of a reconstruction grid (defaults: the reference's GPKDE input
        defaults, anisotropic kernels, FP64 arithmetic)."""
        o = GpkdeOptions()
        for d in range(3):
            o.origin[d], o.domain_size[d], o.bin_size[d] = float(origin[d]), float(domain_size[d]), float(bin_size[d])
        o.n_opt_loops = int(n_opt_loops)
        o.min_hover_delta, o.delta_hover_delta, o.max_hover_delta = (float(v) for v in kdb)
        o.rel_err_convergence = float(rel_err)
        o.skip_error_convergence = int(skip_error)
        o.unit_volume = int(unit_volume)
        o.scaling_factor = float(scaling_factor)
        o.precision = int(precision)
        o.isotropic = int(bool(isotropic))
        return o

    def gpkde(self, domain_size, bin_size, origin=(0.0, 0.0, 0.0), n_opt_loops=10, kdb=(0.3, 0.3, 15.0),
              rel_err=0.02, skip_error=False, unit_volume=True, scaling_factor=1.0, precision=FP64,
              isotropic=False):
        """GPKDE reconstruction of the active particles.  Returns (density, histogram,
        loops) with the grids shaped (nz, ny, nx)."""
        o = self.gpkde_options(domain_size, bin_size, origin, n_opt_loops, kdb, rel_err, skip_error, unit_volume,
                               scaling_factor, precision, isotropic)
        nb = [int(domain_size[d] / bin_size[d] + 0.5) if bin_size[d] != 0 else 1 for d in range(3)]
        dens = np.empty(int(np.prod(nb)))
        hist = np.empty(int(np.prod(nb)))
        nbo = np.zeros(3, np.int32)
        loops = C.c_int32(0)
        self._check(self.lib.mprw_gpkde(self.h, C.byref(o), _p(dens, _dp), _p(hist, _dp), _p(nbo, _ip),
                                        C.byref(loops)), "mprw_gpkde")
        shp = (nb[2], nb[1], nb[0])
        return dens.reshape(shp), hist.reshape(shp), loops.value

    def gpkde_partial(self, domain_size, bin_size, origin=(0.0, 0.0, 0.0), **kw):
        """This tracker's summable part of a reconstruction (mprw_gpkde_partial):
        (mass per bin shaped (nz, ny, nx), GpkdeSums)."""
        o = self.gpkde_options(domain_size, bin_size, origin, **kw)
        nb = [int(domain_size[d] / bin_size[d] + 0.5) if bin_size[d] != 0 else 1 for d in range(3)]
        mass = np.empty(int(np.prod(nb)))
        sums = GpkdeSums()
        self._check(self.lib.mprw_gpkde_partial(self.h, C.byref(o), _p(mass, _dp), C.byref(sums)),
                    "mprw_gpkde_partial")
        return mass.reshape(nb[2], nb[1], nb[0]), sums

    def gpkde_from_counts(self, domain_size, bin_size, mass, sums, origin=(0.0, 0.0, 0.0), **kw):
        """The reconstruction of summed parts (mprw_gpkde_from_counts): (density, histogram, loops)."""
        o = self.gpkde_options(domain_size, bin_size, origin, **kw)
        nb = [int(domain_size[d] / bin_size[d] + 0.5) if bin_size[d] != 0 else 1 for d in range(3)]
        m = np.ascontiguousarray(mass, np.float64).reshape(-1)
        if m.shape[0] != int(np.prod(nb)):
            raise ValueError("mass per bin does not match the grid")
        dens = np.empty(int(np.prod(nb)))
        hist = np.empty(int(np.prod(nb)))
        nbo = np.zeros(3, np.int32)
        loops = C.c_int32(0)
        self._check(self.lib.mprw_gpkde_from_counts(self.h, C.byref(o), _p(m, _dp), C.byref(sums), _p(dens, _dp),
                                                    _p(hist, _dp), _p(nbo, _ip), C.byref(loops)),
                    "mprw_gpkde_from_counts")
        shp = (nb[2], nb[1], nb[0])
        return dens.reshape(shp), hist.reshape(shp), loops.value

    def adj_setup(self, zones, nzones, dt, nsteps, checkpoint, origin, bin_size, n_bins, bandwidth, velocity_floor,
                  seed=0):
        """The differentiable walk of this handle's particles (mprw_adj_setup)."""
        z = _i32(zones)
        if z.shape[0] != self.grid.ncell:
            raise ValueError("one zone per cell")
        o = AdjOptions()
        o.nzones, o.nsteps, o.checkpoint, o.dt, o.seed = int(nzones), int(nsteps), int(checkpoint), float(dt), int(seed)
        o.velocity_floor = float(velocity_floor)
        for d in range(3):
            o.origin[d], o.bin_size[d], o.n_bins[d], o.bandwidth[d] = (float(origin[d]), float(bin_size[d]),
                                                                      int(n_bins[d]), float(bandwidth[d]))
        self._adj = dict(nz=int(nzones), nb=tuple(int(v) for v in n_bins))
        self._check(self.lib.mprw_adj_setup(self.h, _p(z, _ip), C.byref(o)), "mprw_adj_setup")

    def adj_forward(self, theta):
        """Density (shaped (nz, ny, nx)) of the walk for theta = (alphaL per zone, alphaT per zone,
        porosity per zone, velocity scale)."""
        th = _f64(theta)
        if th.shape[0] != 3 * self._adj["nz"] + 1:
            raise ValueError("theta: 3 nzones + 1 values")
        nb = self._adj["nb"]
        dens = np.empty(int(np.prod(nb)))
        self._check(self.lib.mprw_adj_forward(self.h, _p(th, _dp), _p(dens, _dp)), "mprw_adj_forward")
        return dens.reshape(nb[2], nb[1], nb[0])

    def adj_backward(self, grad_density):
        """dL/dtheta from dL/d(density) of the last adj_forward."""
        g = _f64(np.asarray(grad_density).reshape(-1))
        out = np.empty(3 * self._adj["nz"] + 1)
        self._check(self.lib.mprw_adj_backward(self.h, _p(g, _dp), _p(out, _dp)), "mprw_adj_backward")
        return out

    def set_observations(self, cells, obs, style):
        """Observation cells: cells (1-based) belong to observations obs (0-based);
        style[k] = 1 resident, 2 sink."""
        c, o, st = _i32(cells), _i32(obs), _i32(style)
        self._obs = (c, o, st)
        self.nobs = int(st.shape[0])
        self._check(self.lib.mprw_set_observations(self.h, int(c.shape[0]), _p(c, _ip), _p(o, _ip), self.nobs,
                                                   _p(st, _ip)), "mprw_set_observations")

    def observe_resident(self):
        """(count, mass) of the ACTIVE particles in each resident observation."""
        cnt = np.zeros(self.nobs, np.int64)
        mass = np.zeros(self.nobs)
        self._check(self.lib.mprw_observe_resident(self.h, cnt.ctypes.data_as(C.POINTER(C.c_int64)),
                                                   _p(mass, _dp)), "mprw_observe_resident")
        return cnt, mass

    def observe_sinks(self):
        """Sink-observation records of the last advance: dict of obs, id, time, mass."""
        nrec = C.c_int64(0)
        cap = int(self.n)
        out = dict(obs=np.empty(cap, np.int32), id=np.empty(cap, np.uint64), time=np.empty(cap),
                   mass=np.empty(cap))
        self._check(self.lib.mprw_observe_sinks(self.h, cap, _p(out["obs"], _ip), _p(out["id"], _up),
                                                _p(out["time"], _dp), _p(out["mass"], _dp), C.byref(nrec)),
                    "mprw_observe_sinks")
        m = nrec.value
        return {k: v[:m] for k, v in out.items()}

    def set_stream(self, stream_ptr: int):
        self._check(self.lib.mprw_set_stream(self.h, C.c_void_p(stream_ptr)), "mprw_set_stream")

    def set_timeout(self, timeout_ms: float):
        """Stop an advance still running after timeout_ms (0: no limit); it then
        raises MprwAborted with every particle at a valid location."""
        self._check(self.lib.mprw_set_timeout(self.h, float(timeout_ms)), "mprw_set_timeout")

    def cancel(self):
        """Stop the running (or else the next) advance; safe from another thread."""
        self.lib.mprw_cancel(self.h)

    def set_tuning(self, blocks_per_sm: int = 0, sort_interval: int = 1):
        self._check(self.lib.mprw_set_tuning(self.h, int(blocks_per_sm), int(sort_interval)), "mprw_set_tuning")

    def tuning(self) -> dict:
        b, si, mx = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self.lib.mprw_get_tuning(self.h, C.byref(b), C.byref(si), C.byref(mx)), "mprw_get_tuning")
        return dict(blocks_per_sm=b.value, sort_interval=si.value, max_blocks_per_sm=mx.value)

    def autotune(self, t_begin: float, t_end: float) -> dict:
        """Pick blocks per SM and the sort interval by timing trial advances
        over [t_begin, t_end] from the current state (left unchanged)."""
        b, si = C.c_int32(), C.c_int32()
        rates = np.zeros(5)
        self._check(self.lib.mprw_autotune(self.h, float(t_begin), float(t_end), C.byref(b), C.byref(si),
                                           _p(rates, _dp)), "mprw_autotune")
        return dict(blocks_per_sm=b.value, sort_interval=si.value, trial_rates_per_ms=rates.tolist())

    def timings(self) -> dict:
        s, p, h, k = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        n = C.c_int64()
        self._check(self.lib.mprw_last_timings(self.h, C.byref(s), C.byref(p), C.byref(h), C.byref(k), C.byref(n)),
                    "mprw_last_timings")
        w = C.c_double()
        self._check(self.lib.mprw_last_gpkde_work(self.h, C.byref(w)), "mprw_last_gpkde_work")
        return dict(step_ms=s.value, prep_ms=p.value, hist_ms=h.value, gpkde_ms=k.value, launches=n.value,
                    gpkde_madds=w.value)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.mprw_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class _MemberView(Tracker):
    """Tracker interface on one member of a Batch (mprw_batch_member): its
    flow, particles, histogram, GPKDE and observations.  The batch owns the
    handle; advancing is done on the batch."""

    def __init__(self, batch: "Batch", k: int, grid: Grid):
        self.lib = batch.lib
        self.grid = grid
        self.opt = batch.opt
        self._keep = []
        self._batch = batch
        self.h = C.c_void_p()
        rc = self.lib.mprw_batch_member(batch.h, int(k), C.byref(self.h))
        if rc != 0:
            raise MprwError(f"mprw_batch_member: rc={rc}: {self.lib.mprw_last_error(batch.h).decode()}")
        self.n = 0

    def advance(self, t_begin, t_end):
        raise MprwError("a batch member is advanced by its batch")

    def close(self):
        self.h = C.c_void_p()


class Batch:
    """Several realizations (grids of any sizes, shared options) tracked in one
    persistent launch per advance (mprw_create_batch).  ``member(k)`` is the
    Tracker interface of realization k."""

    def __init__(self, grids, opt: Options):
        self.lib = load_library()
        self.grids = list(grids)
        self.opt = opt
        self._keep = []
        arr = (GridDesc * len(self.grids))(*[_grid_desc(g, self._keep) for g in self.grids])
        od = _options_desc(opt)
        self.h = C.c_void_p()
        rc = self.lib.mprw_create_batch(C.byref(self.h), len(self.grids), arr, C.byref(od))
        if rc != 0:
            msg = self.lib.mprw_last_error(self.h).decode() if self.h.value else "mprw_create_batch failed"
            if self.h.value:
                self.lib.mprw_destroy(self.h)
                self.h = C.c_void_p()
            raise MprwError(f"mprw_create_batch: rc={rc}: {msg}")
        self.members = [_MemberView(self, k, g) for k, g in enumerate(self.grids)]
        self.counts = np.zeros(len(self.grids), np.int64)

    _check = Tracker._check
    set_timeout = Tracker.set_timeout
    cancel = Tracker.cancel

    def member(self, k: int) -> Tracker:
        return self.members[k]

    def load_flow(self, k: int, f: Flow):
        self.members[k].load_flow(f)

    def set_particles(self, parts):
        """One Particles per member (cells 1-based in the member's grid)."""
        parts = list(parts)
        if len(parts) != len(self.members):
            raise MprwError("set_particles: one particle set per member")
        counts = np.array([p.n for p in parts], np.int64)

        def cat(name, conv):
            vals = [getattr(p, name) for p in parts]
            if any(v is None for v in vals):
                if all(v is None for v in vals):
                    return None
                if name == "mass":
                    vals = [np.ones(p.n) if v is None else v for p, v in zip(parts, vals)]
                else:
                    raise MprwError(f"set_particles: {name} given for some members only")
            return conv(np.concatenate([np.asarray(v) for v in vals]))

        a = dict(cell=cat("cell", _i32), lx=cat("lx", _f64), ly=cat("ly", _f64), lz=cat("lz", _f64),
                 t=cat("t", _f64), st=cat("status", _i32), m=cat("mass", _f64), id=cat("id", _u64),
                 rc=cat("rng_ctr", _u64))
        self._check(self.lib.mprw_set_particles_batch(
            self.h, counts.ctypes.data_as(C.POINTER(C.c_int64)), _p(a["cell"], _ip), _p(a["lx"], _dp),
            _p(a["ly"], _dp), _p(a["lz"], _dp), _p(a["t"], _dp), _p(a["st"], _ip), _p(a["m"], _dp),
            _p(a["id"], _up), _p(a["rc"], _up)), "mprw_set_particles_batch")
        self.counts = counts
        for m, c in zip(self.members, counts):
            m.n = int(c)

    def advance(self, t_begin: float, t_end: float) -> int:
        """Advance every member's particles in one launch; returns the total particle-steps."""
        steps = C.c_int64(0)
        self._check(self.lib.mprw_advance(self.h, float(t_begin), float(t_end), C.byref(steps)), "mprw_advance")
        return steps.value

    def get_particles(self, global_xyz: bool = True) -> list:
        return [m.get_particles(global_xyz) for m in self.members]

    def gpkde(self, domains, bin_size, origin=(0.0, 0.0, 0.0), n_opt_loops=10, kdb=(0.3, 0.3, 15.0), rel_err=0.02,
              skip_error=False, unit_volume=True, scaling_factor=1.0, precision=FP64, concurrency=4,
              histograms=False):
        """GPKDE of every member (mprw_gpkde_batch), ``domains[k]`` the domain
        size of member k's reconstruction grid.  Returns a list of densities
        (and histograms) shaped (nz, ny, nx), and the loops run per member."""
        nm = len(self.members)
        opts = (GpkdeOptions * nm)()
        dens, hists, shapes = [], [], []
        for k in range(nm):
            o = Tracker.gpkde_options(domains[k], bin_size, origin, n_opt_loops, kdb, rel_err, skip_error,
                                      unit_volume, scaling_factor, precision)
            C.memmove(C.byref(opts, k * C.sizeof(GpkdeOptions)), C.byref(o), C.sizeof(GpkdeOptions))
            nb = [int(domains[k][d] / bin_size[d] + 0.5) if bin_size[d] != 0 else 1 for d in range(3)]
            shapes.append((nb[2], nb[1], nb[0]))
            dens.append(np.empty(int(np.prod(nb))))
            hists.append(np.empty(int(np.prod(nb))) if histograms else None)
        dp = (_dp * nm)(*[_p(d, _dp) for d in dens])
        hp = (_dp * nm)(*[_p(h, _dp) for h in hists]) if histograms else None
        loops = np.zeros(nm, np.int32)
        self._check(self.lib.mprw_gpkde_batch(self.h, opts, dp, hp, _p(loops, _ip), int(concurrency)),
                    "mprw_gpkde_batch")
        dens = [d.reshape(s) for d, s in zip(dens, shapes)]
        if histograms:
            return dens, [h.reshape(s) for h, s in zip(hists, shapes)], loops
        return dens, loops

    def set_stream(self, stream_ptr: int):
        self._check(self.lib.mprw_set_stream(self.h, C.c_void_p(stream_ptr)), "mprw_set_stream")

    set_tuning = Tracker.set_tuning
    tuning = Tracker.tuning
    autotune = Tracker.autotune

    def timings(self) -> dict:
        s, p, h, k = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        n = C.c_int64()
        self._check(self.lib.mprw_last_timings(self.h, C.byref(s), C.byref(p), C.byref(h), C.byref(k), C.byref(n)),
                    "mprw_last_timings")
        return dict(step_ms=s.value, gpkde_ms=k.value, launches=n.value)

    def close(self):
        for m in getattr(self, "members", []):
            m.close()
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.mprw_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def gpkde_series(times, weights, *, origin=0.0, domain_size=0.0, bin_size=0.0, bin_format=2, bin_size_fraction=1.0,
                 adapt_grid=False, exact_point=False, eff_format=0, init_selection=0, init_factor=2.0,
                 apply_init_factor=False, n_opt_loops=10, rel_err=0.02, skip_error=False, only_histogram=False,
                 raw_density=False, unit_volume=False, stream=None) -> dict:
    """1-D GPKDE of a weighted time series on the GPU (``mprw_gpkde_series``):
    GridProjectedKDE with a 1-D domain and the kernel database off, as the
    observation post-process runs it (MPathRW.F90:1773-2840).

    Returns a dict with ``counts``, ``wcounts`` (effective-weight formats 2
    and 3, else None), ``density`` (None for a histogram only), ``n_bins``,
    ``delta_bins_origin``, ``bin_size``, ``grid_origin``, ``coordinates``
    (bin centres), ``loops`` and ``active_bins``."""
    lib = load_library()
    t = _f64(times).ravel()
    w = _f64(weights).ravel()
    if t.shape != w.shape:
        raise ValueError("times and weights differ in length")
    o = SeriesOptions(origin=float(origin), domain_size=float(domain_size), bin_size=float(bin_size),
                      bin_format=int(bin_format), bin_size_fraction=float(bin_size_fraction),
                      adapt_grid=int(bool(adapt_grid)), exact_point=int(bool(exact_point)),
                      effective_weight_format=int(eff_format), initial_smoothing_selection=int(init_selection),
                      initial_smoothing_factor=float(init_factor), apply_initial_factor=int(bool(apply_init_factor)),
                      n_opt_loops=int(n_opt_loops), rel_err_convergence=float(rel_err),
                      skip_error_convergence=int(bool(skip_error)), only_histogram=int(bool(only_histogram)),
                      compute_raw_density=int(bool(raw_density)), unit_volume=int(bool(unit_volume)))
    res = SeriesResult()
    cap = 1024
    while True:
        counts = np.zeros(cap)
        wcounts = np.zeros(cap)
        dens = np.zeros(cap)
        rc = lib.mprw_gpkde_series(_p(t, _dp), _p(w, _dp), t.shape[0], C.byref(o), cap, _p(counts, _dp),
                                   _p(wcounts, _dp), _p(dens, _dp), C.byref(res), stream)
        if rc == -6 and res.n_bins > cap:
            cap = int(res.n_bins)
            continue
        if rc != 0:
            raise MprwError(f"mprw_gpkde_series: rc={rc}")
        break
    nb = int(res.n_bins)
    coords = (np.arange(1, nb + 1, dtype=np.float64) + res.delta_bins_origin - 0.5) * res.bin_size + float(origin)
    return dict(counts=counts[:nb].copy(), wcounts=wcounts[:nb].copy() if eff_format in (2, 3) else None,
                density=None if only_histogram else dens[:nb].copy(), n_bins=nb,
                delta_bins_origin=int(res.delta_bins_origin), bin_size=float(res.bin_size),
                grid_origin=float(res.grid_origin), coordinates=coords, loops=int(res.loops_done),
                active_bins=int(res.active_bins))
