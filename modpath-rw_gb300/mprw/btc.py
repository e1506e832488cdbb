"""Breakthrough curves of observation cells (host side).

Restates the observation post-process of MPathRW.F90:1759-2840 for one
observation: the records of each solute's particle groups are reduced to a
time series by a 1-D GPKDE with the kernel database off, which runs on the
GPU (``mprw.gpkde_series``, the C ABI's ``mprw_gpkde_series``):

* ``resident_btc`` -- resident observations (style 1, :1773-2000): record
  times lie on the simulation's time points (``exactPoint``), weights are
  particle mass / retardation, concentrations are the histogram and the
  reconstruction divided by the water volume of the observation cells.
* ``sink_btc`` -- sink observations (style 2, :2002-2840): arrival times at
  the sink, weights mass / |Q|, the bin size from the time points, given, or
  estimated (Scott, Freedman-Diaconis), the grid optionally adapted to the
  data (steady state tracked to the end), series optionally interpolated to
  a regular output step, the cumulative sink flow interpolated to the
  series times.
* ``write_resident`` / ``write_sink`` -- the output records with the
  reference's edit descriptors (``I8`` and ``ES18.9E3``).

Interpolation follows ``linear_interp_1d`` of the reference's vendored
finterp library (src/lib/finterp/linear_interpolation_module.F90:446-757,
1184-1318; J. Williams, BSD): the knot interval holding x (the last one
beyond the end, the first one before the start), then (1-q) f_i + q f_i+1
with q = (x - x_i)/(x_i+1 - x_i) -- linear extrapolation outside.

The record files themselves (their reading and the mass lookups) stay with
the host code that writes them; these functions take the columns the driver
builds from them.  ``series`` selects the reconstruction: the GPU by default.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .gpkde_io import es18_9e3, i8


@dataclass
class ObservationOptions:
    """Post-process options of one observation (Observation.f90:25-48,
    ModpathSimulationData.f90:1420-1590), with the reference's defaults."""
    postprocess: int = 1               # postprocessOption: 0 histogram, 1 histogram + GPKDE
    effective_weight_format: int = 0
    bin_size_factor: float = 3.0       # GPKDE initialSmoothingFactor
    initial_smoothing_format: int = 0
    n_opt_loops: int = 10
    error_convergence: float = 0.01
    histogram_bin_format: int = 1      # 0 Scott, 1 Freedman-Diaconis, 2 given, 3 from the time points
    histogram_bin: float = 0.0
    time_step_out: float = 0.0         # > 0: interpolate to this output step
    bin_size_fraction: float = 0.75


def linear_interp(xk, fk, x):
    """linear_interp_1d%initialize + evaluate for each x."""
    xk = np.asarray(xk, np.float64)
    fk = np.asarray(fk, np.float64)
    if xk.shape[0] < 2 or xk.shape != fk.shape or np.any(np.diff(xk) <= 0.0):
        raise ValueError("interpolation knots must be at least two, strictly increasing")
    x = np.asarray(x, np.float64)
    il = np.clip(np.searchsorted(xk, x, side="right") - 1, 0, xk.shape[0] - 2)
    q = (x - xk[il]) / (xk[il + 1] - xk[il])
    p = 1.0 - q
    return p * fk[il] + q * fk[il + 1]


def sink_flow_knots(total_times, cumm_flow, reference_time, kfirst, klast, backward=False):
    """The knots of the cumulative sink flow against tracking time
    (MPathRW.F90:2588-2610): forward (0, T(kfirst..klast) - t_ref) against
    (q(1), q(:)); backward t_ref - T(kfirst..klast step -1) closed by
    t_ref - T(klast-1) (or t_ref when klast = 1) against (q(:), q(kcount)).
    ``total_times`` is TotalTimes (1-based time-step numbers index it as
    total_times[k-1]); returns None when one time step is tracked (the flow
    is then constant)."""
    tt = np.asarray(total_times, np.float64)
    q = np.asarray(cumm_flow, np.float64)
    if kfirst == klast:
        return None
    if not backward:
        x = np.concatenate([[0.0], tt[kfirst - 1:klast] - reference_time])
        f = np.concatenate([[q[0]], q])
        return x, f
    ks = np.arange(kfirst, klast - 1, -1)
    x = reference_time - tt[ks - 1]
    x = np.concatenate([x, [reference_time - tt[klast - 2] if klast != 1 else reference_time]])
    f = np.concatenate([q, [q[-1]]])
    return x, f


def _series_fn(series):
    if series is not None:
        return series
    from . import gpkde_series
    return gpkde_series


def _solute_rows(groups, solute_groups):
    g = np.asarray(groups)
    return [np.isin(g, np.asarray(sg)) if len(sg) else None for sg in solute_groups]


def resident_btc(times, weights, groups, solute_groups, time_points, water_volume, opt: ObservationOptions,
                 series=None) -> dict:
    """One resident observation (MPathRW.F90:1773-2000).

    ``times``/``weights``/``groups`` are the record columns (record time,
    mass / retardation, particle group); ``solute_groups[s]`` the particle
    groups of solute s; ``water_volume`` the water volume of the observation
    per auxiliary record (n_aux,) or per record and cell (n_aux, ncells).
    Returns ``time``, ``water_volume`` and per solute the histogram and
    (postprocess 1) the reconstruction as concentrations (n_aux, nsolutes),
    zero where the water volume is zero, plus the raw per-solute results."""
    fn = _series_fn(series)
    tp = np.asarray(time_points, np.float64)
    vw = np.asarray(water_volume, np.float64)
    if vw.ndim == 2:
        vw = vw.sum(axis=1)
    n_aux = vw.shape[0]
    if tp.shape[0] < 2 or n_aux < 1 or n_aux > tp.shape[0]:
        raise ValueError("resident observations need two time points and one auxiliary record per time point")
    dt = tp[1] - tp[0]
    t = np.asarray(times, np.float64)
    w = np.asarray(weights, np.float64)
    ns = len(solute_groups)
    hist = np.zeros((n_aux, ns))
    dens = np.zeros((n_aux, ns)) if opt.postprocess == 1 else None
    raw = []
    base = dict(origin=0.0, domain_size=tp[n_aux - 1], bin_size=dt, bin_format=2, exact_point=True,
                eff_format=opt.effective_weight_format, init_selection=opt.initial_smoothing_format,
                init_factor=opt.bin_size_factor, apply_init_factor=True, n_opt_loops=opt.n_opt_loops)
    for s, rows in enumerate(_solute_rows(groups, solute_groups)):
        if rows is None or not rows.any():
            raw.append(None)
            continue
        if opt.postprocess == 0:
            r = fn(t[rows], w[rows], only_histogram=True, **base)
        else:
            r = fn(t[rows], w[rows], unit_volume=True, rel_err=opt.error_convergence, **base)
        h = r["wcounts"] if opt.effective_weight_format in (2, 3) else r["counts"]
        if h.shape[0] != n_aux:
            raise ValueError(f"time grid of {h.shape[0]} bins for {n_aux} auxiliary records")
        hist[:, s] = h
        if dens is not None:
            dens[:, s] = r["density"]
        raw.append(r)
    pos = vw > 0.0
    conc_h = np.where(pos[:, None], hist / np.where(pos, vw, 1.0)[:, None], 0.0)
    out = dict(time=tp[:n_aux].copy(), water_volume=np.where(pos, vw, 0.0), hist=conc_h, raw=raw)
    if dens is not None:
        out["gpkde"] = np.where(pos[:, None], dens / np.where(pos, vw, 1.0)[:, None], 0.0)
    return out


def sink_btc(times, weights, groups, solute_groups, opt: ObservationOptions, *, stoptime, adapt_grid=False,
             time_points=None, flow_knots=None, flow_constant=0.0, apply_initial_factor=None,
             series=None) -> dict:
    """One sink observation (MPathRW.F90:2002-2840).

    ``times``/``weights``/``groups`` are the record columns (arrival time,
    mass / |Q|, particle group).  ``adapt_grid`` is the reference's
    steady-state-to-the-end case (stoptime option 2).  ``flow_knots`` (from
    ``sink_flow_knots``) or ``flow_constant`` (one tracked time step) give
    the cumulative sink flow column.  ``apply_initial_factor`` is whether the
    GPKDE object scales Silverman's initial smoothing by the bin-size factor:
    the reference decides it when it initializes the object with a bin size
    and a domain (formats 2 and 3 on a fixed grid) and otherwise keeps the
    object's previous setting (None: as a fresh object, off).

    Returns ``per_solute`` (True: one series per solute, each with its own
    times) and the series: ``time``, ``flow``, ``hist``, ``gpkde`` (arrays,
    or lists of arrays per solute), plus the raw per-solute results."""
    fn = _series_fn(series)
    fmt = opt.histogram_bin_format
    if fmt not in (0, 1, 2, 3):
        fmt = 1
    do_interp = opt.time_step_out > 0.0
    if fmt == 3:
        tp = np.asarray(time_points, np.float64) if time_points is not None else np.zeros(0)
        if tp.shape[0] < 2:
            raise ValueError("bin format 3 needs at least two time points")
        dt_obs = tp[1] - tp[0]
    elif fmt == 2:
        dt_obs = opt.histogram_bin
    else:
        dt_obs = 0.0
    max_t = 0.0 if adapt_grid else float(stoptime)
    if apply_initial_factor is None:
        apply_initial_factor = (fmt in (2, 3)) and not adapt_grid
    t = np.asarray(times, np.float64)
    w = np.asarray(weights, np.float64)
    base = dict(origin=0.0, domain_size=max_t, bin_size=dt_obs, bin_format=fmt,
                bin_size_fraction=opt.bin_size_fraction, adapt_grid=adapt_grid,
                eff_format=opt.effective_weight_format, init_selection=opt.initial_smoothing_format,
                init_factor=opt.bin_size_factor, apply_init_factor=apply_initial_factor,
                n_opt_loops=opt.n_opt_loops, raw_density=True)

    def flow_at(x):
        x = np.asarray(x, np.float64)
        if flow_knots is None:
            return np.full(x.shape, float(flow_constant))
        return linear_interp(flow_knots[0], flow_knots[1], x)

    # the common output times of fixed grids (:2176-2290)
    common = None
    if not adapt_grid:
        if do_interp:
            count = int(np.ceil(max_t / opt.time_step_out))
            common = opt.time_step_out * np.ones(count)
            for k in range(1, count):
                common[k] = common[k - 1] + opt.time_step_out
            # the reference meant the last output time to be the stop time;
            # its loop leaves that element unassigned
            common[-1] = float(stoptime)
    ns = len(solute_groups)
    per_solute = (fmt in (0, 1) and not do_interp) or adapt_grid
    res = dict(per_solute=per_solute, raw=[])
    if per_solute:
        res.update(time=[], flow=[], hist=[], gpkde=[])
    for s, rows in enumerate(_solute_rows(groups, solute_groups)):
        r = None
        if rows is not None and rows.any():
            if opt.postprocess == 0:
                r = fn(t[rows], w[rows], only_histogram=True, **base)
            else:
                r = fn(t[rows], w[rows], rel_err=opt.error_convergence, **base)
        res["raw"].append(r)
        if r is None:
            if per_solute:
                for k in ("time", "flow", "hist", "gpkde"):
                    res[k].append(None)
            continue
        coords = r["coordinates"]
        h = r["wcounts"] if opt.effective_weight_format in (2, 3) else r["counts"]
        d = r["density"]
        if per_solute:
            if do_interp:
                # adapted grid, interpolated to the output step (:2424-2500)
                count = int(coords.max() / opt.time_step_out)
                if count < 2:
                    for k in ("time", "flow", "hist", "gpkde"):
                        res[k].append(None)
                    continue
                ts = opt.time_step_out * np.ones(count)
                for k in range(1, count):
                    ts[k] = ts[k - 1] + opt.time_step_out
                keep = ts >= coords[0]
                hs = np.where(keep, linear_interp(coords, h, ts), 0.0)
                ds = np.where(keep, linear_interp(coords, d, ts), 0.0) if d is not None else None
            else:
                ts, hs, ds = coords.copy(), h.copy(), (d.copy() if d is not None else None)
            res["time"].append(ts)
            res["flow"].append(flow_at(ts))
            res["hist"].append(hs)
            res["gpkde"].append(ds)
        else:
            if common is None:
                common = coords.copy()
                res["time"] = common
                res["hist"] = np.zeros((common.shape[0], ns))
                res["gpkde"] = np.zeros((common.shape[0], ns)) if opt.postprocess == 1 else None
                res["coordinates"] = coords.copy()
            elif "hist" not in res:
                res["time"] = common
                res["hist"] = np.zeros((common.shape[0], ns))
                res["gpkde"] = np.zeros((common.shape[0], ns)) if opt.postprocess == 1 else None
                res["coordinates"] = coords.copy()
            if do_interp:
                keep = common >= coords[0]
                res["hist"][:, s] = np.where(keep, linear_interp(coords, h, common), 0.0)
                if d is not None:
                    res["gpkde"][:, s] = np.where(keep, linear_interp(coords, d, common), 0.0)
            else:
                if h.shape[0] != common.shape[0]:
                    raise ValueError("solutes reconstructed on grids of different sizes")
                res["hist"][:, s] = h
                if d is not None:
                    res["gpkde"][:, s] = d
    if not per_solute and "hist" in res:
        res["flow"] = flow_at(res["time"])
    return res


def write_resident(fh, btc: dict) -> int:
    """Resident observation output (MPathRW.F90:1968-2000): time index,
    time, water volume, concentrations of the histogram (and of the
    reconstruction) per solute; rows without water hold zeros."""
    n = btc["time"].shape[0]
    lines = []
    for k in range(n):
        vals = [btc["time"][k], btc["water_volume"][k]]
        if btc["water_volume"][k] > 0.0:
            vals += list(btc["hist"][k])
            if "gpkde" in btc:
                vals += list(btc["gpkde"][k])
        else:
            vals += [0.0] * (btc["hist"].shape[1] * (2 if "gpkde" in btc else 1))
        lines.append(i8(k + 1) + "".join(es18_9e3(v) for v in vals) + "\n")
    fh.write("".join(lines))
    return n


def write_sink(fh, btc: dict, solute_ids=None, skip_before=None) -> int:
    """Sink observation output (MPathRW.F90:2616-2790).  Per-solute series:
    solute id, index, time, flow, histogram (, reconstruction); a common
    series: index, time, flow, histogram per solute (, reconstruction per
    solute).  With interpolation on a fixed grid, rows before the first bin
    centre are left out and rows after the last end the table
    (``skip_before`` = the bin centres)."""
    lines = []
    if btc["per_solute"]:
        for s, ts in enumerate(btc["time"]):
            if ts is None:
                continue
            sid = solute_ids[s] if solute_ids is not None else s + 1
            for k in range(ts.shape[0]):
                vals = [ts[k], btc["flow"][s][k], btc["hist"][s][k]]
                if btc["gpkde"][s] is not None:
                    vals.append(btc["gpkde"][s][k])
                lines.append(i8(sid) + i8(k + 1) + "".join(es18_9e3(v) for v in vals) + "\n")
    else:
        ts = btc["time"]
        for k in range(ts.shape[0]):
            if skip_before is not None:
                if ts[k] < skip_before[0]:
                    continue
                if ts[k] > skip_before[-1]:
                    break
            vals = [ts[k], btc["flow"][k]] + list(btc["hist"][k])
            if btc["gpkde"] is not None:
                vals += list(btc["gpkde"][k])
            lines.append(i8(k + 1) + "".join(es18_9e3(v) for v in vals) + "\n")
    fh.write("".join(lines))
    return len(lines)
