"""Benchmark of the random-walk particle-tracking hot path on one GB300.

Workload (the lognormal slab): 200x100x20 cells of 1 m, lognormal K
(sigma2 lnK = 1, geometric mean 10 m/d, exponential covariance 10 m / 2 m,
seeded FFT field), FP64 steady heads by CG to 1e-12, porosity 0.25,
alphaL 0.5 m, alphaT 0.05 m, Dm 1e-4 m2/d, 1,000,000 unit-mass particles
released uniformly in the 10 x 100 x 20 m inlet slab, MIN_ADV_DISP 0.1/0.1,
EULERIAN, stop at weak sinks (constant-head outlet).  Synthetic inputs with
the config's shapes and distributions.

One step = one 10-day tracking interval of the config's pipeline: advance
every particle to the next GPKDE time point, then the GPKDE reconstruction
(histogram + kernel-density optimisation, 1 m bins over the 200 x 100 x 20 m
domain, the reference's default database and convergence settings) of the
active particles, density and histogram returned to the host.  The rate is
particle-steps / time of the whole advance + GPKDE step, measured with CUDA
events on the library's stream (the host-side convergence decisions inside a
reconstruction are inside the span).  W warm-up intervals are run first; the
K timed intervals continue the same simulation.  L2 (129 MB) is flushed
between timed steps by writing a 256 MiB buffer outside the timed events.

Reported: ``value`` = particle-steps/s of the plain FP64 pipeline with the
state resident in HBM; ``e2e`` = the same through the C ABI with pinned host
buffers (particle state host->device, advance, state device->host, GPKDE
density + histogram device->host, every step); ``mixed`` = the MIXED-precision
pipeline (FP32 positions and arithmetic, FP64 time; FP32 reconstruction with
FP64 convergence sums) on the same workload with its plume-moment errors and
density errors against the FP64 run; ``roofline`` of the step kernel (the dominant kernel); ``cpu_baseline`` =
the C restatement of the reference's advance (OpenMP, all host threads) on a
bounded sample -- without the GPKDE reconstruction, whose CPU restatement is
numpy test code and not representative, so the CPU figure is an upper bound
on the reference's pipeline rate.

Also in the line: ``lognormal_slab_btc_150m`` = the breakthrough counts at
the x = 150 m control plane after every advance; ``uniform_pulse`` = the
uniform-column pulse (1e5 particles, 100 days, FP64 and MIXED) with its
plume against the analytic Gaussian; ``batched`` = the ensemble as one batch
in MIXED, the same batch in FP64, and the plain FP64 path (every
realization on its own handle, one after another): the ratio of the batched
mixed-precision rate to that plain FP64 rate, ``speedup_vs_plain_fp64`` (the
target is at least 5 at 0.5 % moment error), and per realization the moment errors and the
L1 error of the breakthrough curve at x = 30 m of the MIXED batch against
the plain FP64 run of the same seed; ``adjoint`` = the differentiable walk
and its adjoint on the lognormal slab in 8 zones (25 parameters, 5e5
particles, 2,000 steps) with a central-difference check of five gradient
components.

``--impl reference`` times the reference's CPU algorithm (the C restatement:
the Fortran reference cannot be compiled on these machines) instead.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (str(ROOT / "modpath-rw_gb300"), str(ROOT)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "particle-steps/s: plain FP64 vs batched mixed-precision at stated moment error"
UNIT = "particle-steps/s"
B_STEP_FP64 = 1008.0   # algorithmic bytes per particle-step, FP64 (state r+w 96 B + cell record 912 B)
B_STEP_MIXED = 544.0   # MIXED (72 B + 472 B)
INTERVAL_D = 10.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--particles", type=int, default=1_000_000)
    ap.add_argument("--cpu-sample", type=int, default=400_000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-pulse", action="store_true", help="skip the uniform-pulse leg (1e5 particles, 100 days)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint leg (8 zones, 5e5 particles, 2000 steps)")
    ap.add_argument("--no-btc", action="store_true",
                    help="skip the breakthrough-curve leg (1-D GPKDE of 10^6 sink records)")
    ap.add_argument("--realizations", type=int, default=64,
                    help="ensemble size of the batched leg (realizations 0..R-1 of the 64-member ensemble; "
                         "64 = the whole ensemble)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default launch tuning instead of mprw_autotune before the warm-up")
    ap.add_argument("--workload", default="lognormal_slab", choices=["lognormal_slab", "lognormal_injection"],
                    help="lognormal_injection: the large continuous-injection run, whole (20 x 25 days), FP64 then MIXED; "
                         "prints its own line")
    ap.add_argument("--injection-particles", type=int, default=100_000_000)
    ap.add_argument("--legacy-stream", action="store_true",
                    help="run the FP64 and MIXED legs on the legacy default stream: the library then drives the "
                         "GPKDE optimisation loop from the host, one launch per kernel (the same kernels and "
                         "results as the device-driven loop), which a per-kernel profile of the loop needs")
    ap.add_argument("--kde-streams", type=int, default=4,
                    help="batched leg: reconstructions run concurrently (mprw_gpkde_batch concurrency)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="precision of the headline run (mixed: for profiling the MIXED kernel alone)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_figure(key):
    """A figure of the step kernel's committed ncu summary (per particle-step or percent)."""
    f = ROOT / "profiles" / "rwpt_advance_kernel_lognormal_slab.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([s.strip() for s in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 7 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 7 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) > 7 for k in range(4) if r[4 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def build_workload(n_particles, rank=0, use_torch=True):
    import tempfile
    from mprw import workloads as W
    # the flow reaches the tracker the way a MODFLOW 6 run delivers it: written as
    # .grb/.hds/.bud and read back through the binary readers
    with tempfile.TemporaryDirectory() as d:
        g, f, p, opt, info = W.lognormal_slab(n_particles=n_particles, seed=0, use_torch=use_torch, mf6_dir=d)
        info = dict(info, mf6_bytes=sum(os.path.getsize(x) for x in info["mf6_files"]))
    if rank:
        # weak scaling: every rank tracks its own particle set on the same field
        q = W.release_in_box(g, n_particles, 0.0, 10.0, 0.0, 100.0, float(g.botm[-1]), float(g.top[0]),
                             seed=1000 + 7919 * rank)
        q.id = q.id + np.uint64(rank * n_particles)
        p = q
    return g, f, p, opt, info


def moments(out):
    act = out["status"] == 1
    m = {}
    for k in ("gx", "gy", "gz"):
        v = out[k][act]
        m[k] = (float(v.mean()), float(v.var()))
    return m, int(act.sum())


def plane_observations(g, x_plane):
    """Observations of a control plane at x = x_plane: observation 0 (resident)
    = the cells of the columns at or beyond the plane except the last column,
    observation 1 (sink) = the last column, the constant-head outlet whose
    weak-sink stops end the particles that reach it."""
    xe = np.concatenate([[0.0], np.cumsum(g.delr)])
    cols = np.nonzero(xe[:-1] >= x_plane - 1e-9)[0]
    cols = cols[cols < g.ncol - 1]
    k, i, j = np.meshgrid(np.arange(g.nlay), np.arange(g.nrow), cols, indexing="ij")
    res = g.node(k.ravel(), i.ravel(), j.ravel())
    k, i = np.meshgrid(np.arange(g.nlay), np.arange(g.nrow), indexing="ij")
    out = g.node(k.ravel(), i.ravel(), np.full(k.size, g.ncol - 1))
    cells = np.concatenate([res, out]).astype(np.int32)
    obs = np.concatenate([np.zeros(res.size, np.int32), np.ones(out.size, np.int32)])
    return cells, obs, np.array([1, 2], np.int32)


def sink_count(tr):
    """Number of sink-observation records of the tracker's last advance (none copied)."""
    import ctypes as C
    n = C.c_int64(0)
    rc = tr.lib.mprw_observe_sinks(tr.h, 0, None, None, None, None, C.byref(n))
    if rc != 0:
        raise RuntimeError(tr.lib.mprw_last_error(tr.h).decode())
    return int(n.value)


class PlaneCounter:
    """Breakthrough at a control plane: after every advance, the ACTIVE particles
    beyond the plane plus every particle stopped so far at the outlet."""

    def __init__(self, tr, g, x_plane):
        tr.set_observations(*plane_observations(g, x_plane))
        self.tr, self.arrived, self.curve = tr, 0, []

    def after_advance(self, t):
        self.arrived += sink_count(self.tr)
        cnt, _ = self.tr.observe_resident()
        self.curve.append((float(t), int(cnt[0]) + self.arrived))


def btc_l1(a, b):
    """L1 distance of two breakthrough curves sampled at the same times, relative to b's."""
    ca = np.array([c for _, c in a], np.float64)
    cb = np.array([c for _, c in b], np.float64)
    den = cb.sum()
    return float(np.abs(ca - cb).sum() / den) if den > 0 else (0.0 if ca.sum() == 0 else float("inf"))


def barrier():
    """Align the ranks around a timed region (no-op for one process)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def run_gpu_arm(args, rank, world, local):
    import torch
    import mprw
    from mprw import shard
    from mprw.model import MIXED

    torch.cuda.set_device(local)
    g, f, p, opt, info = build_workload(args.particles, rank)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    origin, bins, nb = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (g.ncol, g.nrow, g.nlay)
    domain = (float(np.sum(g.delr)), float(np.sum(g.delc)), float(g.top[0] - g.botm[-1]))

    # the legacy default stream is torch's default stream
    stream = torch.cuda.default_stream() if args.legacy_stream else torch.cuda.Stream()

    def timed_run(precision, steps, warmup):
        # the MIXED pipeline reconstructs in FP32 too; FP64 is the reference's arithmetic
        kde_prec = precision
        opt.precision = precision
        tr = mprw.Tracker(g, opt)
        # launch on a stream the events below can see (1: cudaStreamLegacy)
        tr.set_stream(1 if args.legacy_stream else stream.cuda_stream)
        tr.load_flow(f)
        tr.set_particles(p)
        tuning = tr.autotune(0.0, INTERVAL_D) if args.autotune else tr.tuning()
        # breakthrough at the x = 150 m control plane, counted after every advance
        # outside the timed events (two small device reductions)
        plane = PlaneCounter(tr, g, 150.0)
        t = 0.0
        for _ in range(warmup):
            tr.advance(t, t + INTERVAL_D)
            plane.after_advance(t + INTERVAL_D)
            if world > 1:
                shard.gpkde_allreduce(tr, domain, bins, origin, precision=kde_prec)
            else:
                tr.gpkde(domain, bins, origin, precision=kde_prec)
            t += INTERVAL_D
        torch.cuda.synchronize()
        barrier()
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
        kern_ms, kde_ms, wall_ms, steps_done, launches, loops, madds = [], [], [], 0, 0, [], []
        for k in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ev[k][0].record(stream)
            s = tr.advance(t, t + INTERVAL_D)
            tm = tr.timings()
            ev[k][1].record(stream)
            if world > 1:
                # one reconstruction of every rank's particles: the per-rank
                # parts summed by an all-reduce, then smoothed on every rank
                dens, _, nl = shard.gpkde_allreduce(tr, domain, bins, origin, precision=kde_prec)
            else:
                dens, _, nl = tr.gpkde(domain, bins, origin, precision=kde_prec)
            tk = tr.timings()
            ev[k][2].record(stream)
            torch.cuda.synchronize()
            wall_ms.append((time.perf_counter() - t0) * 1e3)
            plane.after_advance(t + INTERVAL_D)
            kern_ms.append(tm["step_ms"])
            kde_ms.append(tk["gpkde_ms"])
            madds.append(tk["gpkde_madds"])
            loops.append(nl)
            launches += tm["launches"] + tk["launches"]
            steps_done += s
            t += INTERVAL_D
        torch.cuda.synchronize()
        barrier()
        ms = [a.elapsed_time(c) for a, _, c in ev]
        adv_ms = [a.elapsed_time(b) for a, b, _ in ev]
        out = tr.get_particles()
        kde_err = None
        if kde_prec != 0:
            # the FP32 reconstruction against an FP64 one on the same particles (untimed)
            d64, _, _ = tr.gpkde(domain, bins, origin)
            kde_err = {"l2_rel": float(np.linalg.norm(dens - d64) / np.linalg.norm(d64)),
                       "max_rel": float(np.abs(dens - d64).max() / d64.max())}
        tr.close()
        return dict(ms=ms, adv_ms=adv_ms, kern_ms=kern_ms, kde_ms=kde_ms, madds=madds, wall_ms=wall_ms, steps=steps_done,
                    launches=launches, out=out, t_end=t, loops=loops, dens=dens, kde_err=kde_err, tuning=tuning,
                    btc150=plane.curve)

    with ClockSampler(local) as clk:
        fp64 = timed_run(MIXED if args.precision == "mixed" else 0, args.steps, args.warmup)
    res = dict(fp64=fp64, clocks=clk.summary())
    if not args.no_mixed:
        res["mixed"] = timed_run(MIXED, args.steps, args.warmup)
    if not args.no_e2e:
        res["e2e"] = e2e_run(args, g, f, p, opt, origin, bins, domain, flush)
    res["geom"] = (g, f, p, opt)
    res["flush"] = flush
    res["mf6_bytes"] = info["mf6_bytes"]
    if not args.no_batched and rank == 0:
        res["batched"] = batched_run(args, flush)
    return res


BATCH_PLANE_X = 30.0   # control plane of the ensemble's breakthrough curves (20 m past the inlet slab)


def batched_run(args, flush):
    """The ensemble (mprw.workloads.lognormal_ensemble, the first R realizations) as ONE
    batch: each step advances every realization's particles in one persistent
    launch and reconstructs every realization with GPKDE.  Timed in MIXED
    precision (FP32 advance + FP32 reconstruction), in FP64 as the same batch,
    and in FP64 as the plain path -- every realization on its own handle, one
    after another -- with the same particles and random streams.  Per
    realization, the plume moments and the breakthrough curve at the control
    plane x = 30 m (ACTIVE particles beyond the plane plus those stopped at the
    outlet, after every step) of the MIXED batch are compared with the plain
    FP64 run, the separate FP64 run of the same seed."""
    import torch
    import mprw
    from mprw import workloads as W
    from mprw.model import MIXED
    t_setup = time.perf_counter()
    prm = W.ensemble_params(64)[: args.realizations]
    ens, opt, _ = W.lognormal_ensemble(members=prm, use_torch=True)
    t_setup = time.perf_counter() - t_setup
    stream = torch.cuda.Stream()
    bins = (1.0, 1.0, 1.0)
    doms = [(float(g.ncol), float(g.nrow), float(g.top[0] - g.botm[-1])) for g, _, _ in ens]

    def run(precision):
        opt.precision = precision
        b = mprw.Batch([e[0] for e in ens], opt)
        b.set_stream(stream.cuda_stream)
        for k, (g, f, p) in enumerate(ens):
            b.load_flow(k, f)
        b.set_particles([e[2] for e in ens])
        tuning = b.autotune(0.0, INTERVAL_D) if args.autotune else b.tuning()
        planes = [PlaneCounter(b.member(k), g, BATCH_PLANE_X) for k, (g, _, _) in enumerate(ens)]
        t = 0.0

        def one_step(t):
            s = b.advance(t, t + INTERVAL_D)
            for pc in planes:
                pc.after_advance(t + INTERVAL_D)
            b.gpkde(doms, bins, precision=precision, concurrency=args.kde_streams)
            return s
        for _ in range(args.warmup):
            one_step(t)
            t += INTERVAL_D
        torch.cuda.synchronize()
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
        steps, launches, adv_kern = 0, 0, []
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ev[k][0].record(stream)
            s = b.advance(t, t + INTERVAL_D)
            adv_kern.append(b.timings()["step_ms"])
            launches += b.timings()["launches"]
            ev[k][1].record(stream)
            b.gpkde(doms, bins, precision=precision, concurrency=args.kde_streams)
            launches += b.timings()["launches"]
            ev[k][2].record(stream)
            torch.cuda.synchronize()
            for pc in planes:          # outside the timed events
                pc.after_advance(t + INTERVAL_D)
            steps += s
            t += INTERVAL_D
        ms = sum(a.elapsed_time(c) for a, _, c in ev)
        adv = sum(a.elapsed_time(bb) for a, bb, _ in ev)
        outs = b.get_particles()
        b.close()
        return dict(steps=steps, ms=ms, adv_ms=adv, kern_ms=float(np.sum(adv_kern)), launches=launches, outs=outs,
                    t_end=t, tuning=tuning, btc=[pc.curve for pc in planes])

    def run_plain():
        """Plain FP64: each realization on its own handle, one after another, the
        same steps (warm-up untimed), advance + GPKDE per step timed with events."""
        opt.precision = 0
        steps, ms, adv_ms, launches, outs, btc = 0, 0.0, 0.0, 0, [], []
        for k, (g, f, p) in enumerate(ens):
            tr = mprw.Tracker(g, opt)
            tr.set_stream(stream.cuda_stream)
            tr.load_flow(f)
            tr.set_particles(p)
            pc = PlaneCounter(tr, g, BATCH_PLANE_X)
            t = 0.0
            for _ in range(args.warmup):
                tr.advance(t, t + INTERVAL_D)
                pc.after_advance(t + INTERVAL_D)
                tr.gpkde(doms[k], bins)
                t += INTERVAL_D
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
                e[0].record(stream)
                steps += tr.advance(t, t + INTERVAL_D)
                launches += tr.timings()["launches"]
                e[1].record(stream)
                tr.gpkde(doms[k], bins)
                launches += tr.timings()["launches"]
                e[2].record(stream)
                torch.cuda.synchronize()
                pc.after_advance(t + INTERVAL_D)
                ms += e[0].elapsed_time(e[2])
                adv_ms += e[0].elapsed_time(e[1])
                t += INTERVAL_D
            outs.append(tr.get_particles())
            btc.append(pc.curve)
            tr.close()
        return dict(steps=steps, ms=ms, adv_ms=adv_ms, launches=launches, outs=outs, btc=btc)

    mx = run(MIXED)
    fp = run(0)
    pl = run_plain()
    errs = []
    for k, (g, f, p) in enumerate(ens):
        m32, n32 = moments(mx["outs"][k])
        m64, n64 = moments(pl["outs"][k])
        x0 = 5.0  # centre of the 10 m inlet slab: first moments are taken as displacement from it
        e = {"mean_disp_x_rel": abs(m32["gx"][0] - m64["gx"][0]) / max(abs(m64["gx"][0] - x0), 1e-30)}
        for ax in ("gx", "gy", "gz"):
            e[f"var_{ax[1]}_rel"] = abs(m32[ax][1] - m64[ax][1]) / max(m64[ax][1], 1e-30)
        # Monte-Carlo standard error of a variance estimate, relative: sqrt(2 / n)
        e["mc_var_rel_se"] = float(np.sqrt(2.0 / max(n64, 1)))
        e["btc_l1_rel"] = btc_l1(mx["btc"][k], pl["btc"][k])
        e["btc_final"] = [mx["btc"][k][-1][1], pl["btc"][k][-1][1]]
        e["active"] = [n32, n64]
        errs.append(e)
    worst = {key: max(e[key] for e in errs)
             for key in ("mean_disp_x_rel", "var_x_rel", "var_y_rel", "var_z_rel", "btc_l1_rel")}
    # the batch in FP64 reproduces the separate FP64 runs particle for particle
    same = all(np.array_equal(a["cell"], b_["cell"]) and np.array_equal(a["lx"], b_["lx"]) and
               np.array_equal(a["status"], b_["status"]) for a, b_ in zip(fp["outs"], pl["outs"]))
    v32 = mx["steps"] / (mx["ms"] / 1e3)
    v64 = fp["steps"] / (fp["ms"] / 1e3)
    vpl = pl["steps"] / (pl["ms"] / 1e3)
    return {"workload": f"realizations 0..{len(ens) - 1} of the 64-member ensemble (the lognormal-slab generator; grids "
                        "U[100..400]x[50..200]x[10..20], sigma2 lnK U[0.5,2], alphaL U[0.1,1], alphaT = alphaL/10, "
                        "particles log-U[1e5,4e6]), one batch: one advance launch for all realizations + one "
                        f"GPKDE per realization per 10-day step ({args.kde_streams} reconstructions at a time)",
            "realizations": len(ens), "particles": int(sum(p.n for _, _, p in ens)),
            "cells": int(sum(g.ncell for g, _, _ in ens)), "setup_s": t_setup,
            "value": v32, "unit": UNIT, "ms_per_step": mx["ms"] / args.steps,
            "advance_ms_per_step": mx["adv_ms"] / args.steps, "advance_kernel_ms_per_step": mx["kern_ms"] / args.steps,
            "gpkde_ms_per_step": (mx["ms"] - mx["adv_ms"]) / args.steps, "gpu_launches": mx["launches"],
            "fp64_plain": {"value": vpl, "ms_per_step": pl["ms"] / args.steps,
                           "advance_ms_per_step": pl["adv_ms"] / args.steps, "gpu_launches": pl["launches"],
                           "path": "every realization on its own handle (FP64 advance + FP64 GPKDE), one after "
                                   "another, default launch tuning"},
            "fp64_batched": {"value": v64, "ms_per_step": fp["ms"] / args.steps,
                             "advance_ms_per_step": fp["adv_ms"] / args.steps, "tuning": fp["tuning"],
                             "identical_to_plain": bool(same)},
            "tuning": mx["tuning"],
            "speedup_vs_plain_fp64": v32 / vpl,
            "speedup_vs_fp64_batched": v32 / v64,
            "control_plane_x_m": BATCH_PLANE_X,
            "error_vs_plain_fp64": {"worst_over_realizations": worst, "per_realization": errs},
            "t_end_days": mx["t_end"]}


def pulse_run(args, flush):
    """The uniform-column pulse (200x1x1 cells of 1 m, v = 1 m/d, alphaL 0.1 m,
    alphaT 0.01 m, Courant 0.1, 1e5 particles at x = 10 m): advance to 25, 50
    and 100 days, each followed by GPKDE on the 1 m grid, FP64 and MIXED,
    timed with CUDA events; the plume against the analytic Gaussian (mean
    10 + t, variance 0.2 t)."""
    import torch
    import mprw
    from mprw import workloads as W
    from mprw.model import MIXED
    out = {"workload": "uniform pulse: 200x1x1 cells, v 1 m/d, alphaL 0.1 m, 1e5 particles at x = 10 m, "
                       "intervals to 25, 50, 100 d, GPKDE on the 1 m grid after each"}
    stream = torch.cuda.Stream()
    for name, prec in (("fp64", 0), ("mixed", MIXED)):
        g, f, p, opt = W.uniform_pulse(n_particles=100_000, precision=prec)
        tr = mprw.Tracker(g, opt)
        tr.set_stream(stream.cuda_stream)
        tr.load_flow(f)
        tr.set_particles(p)
        flush.zero_()
        torch.cuda.synchronize()
        steps, ms, t, plume = 0, 0.0, 0.0, []
        for t_out in (25.0, 50.0, 100.0):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            e[0].record(stream)
            steps += tr.advance(t, t_out)
            tr.gpkde((200.0, 1.0, 1.0), (1.0, 1.0, 1.0), precision=prec)
            e[1].record(stream)
            torch.cuda.synchronize()
            ms += e[0].elapsed_time(e[1])
            x = tr.get_particles()["gx"]
            plume.append({"t": t_out, "mean_minus_analytic_m": float(x.mean() - (10.0 + t_out)),
                          "var_rel_to_analytic": float(x.var() / (0.2 * t_out) - 1.0)})
            t = t_out
        tr.close()
        out[name] = {"value": steps / (ms / 1e3), "unit": UNIT, "particle_steps": steps, "ms": ms, "plume": plume}
    out["mixed_speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["note"] = ("one small launch per interval with few particles per SM: this configuration is launch- and "
                   "latency-bound on one GB300; the scheme's own bias against the analytic Gaussian (interface "
                   "forcing at the cell faces) is -0.25 m on the mean and -4.3 % on the variance at 100 d, "
                   "measured on the reference's RNG path at 1e6 particles")
    return out


def adjoint_run(args, g, f, flush):
    """The adjoint workload: the lognormal-slab field split into 8 zones (2 x 2
    x 2 blocks), 25 parameters (alphaL, alphaT, porosity per zone and a
    velocity scale), 500,000 particles from the inlet slab, 2,000 steps of
    0.05 d (100 days) stored every 100 steps; the misfit is the squared
    difference of the walk's density on the 1 m grid from the density of the
    same run with every parameter +10 %.  Forward and adjoint (the reverse
    sweep with every segment recomputed from its checkpoint) timed with CUDA
    events; five gradient components checked against central differences
    (relative steps 1e-4 and 1e-5, common random numbers) on this run and on
    a short run of the same particles (120 steps of 0.02 d)."""
    import mprw
    from mprw import workloads as W
    from mprw.model import ACTIVE, EULERIAN, MIN_ADV_DISP, Options
    n, nz = 500_000, 8
    k, i, j = np.unravel_index(np.arange(g.ncell), (g.nlay, g.nrow, g.ncol))
    zones = ((j >= g.ncol // 2).astype(np.int32) + 2 * (i >= g.nrow // 2) + 4 * (k >= g.nlay // 2)).astype(np.int32)
    p = W.release_in_box(g, n, 0.0, 10.0, 0.0, float(g.nrow), float(g.botm[-1]), float(g.top[0]), seed=4242,
                         status=ACTIVE)
    opt = Options(time_step_kind=MIN_ADV_DISP, ts_param=(0.1, 0.1), advection_kind=EULERIAN, stop_weak_sinks=True)
    theta = np.concatenate([np.full(nz, 0.5), np.full(nz, 0.05), np.full(nz, 0.25), [1.0]])
    eps = 0.01   # velocity floor of the dispersion tensor, m/d (mean pore velocity ~0.2 m/d)

    def run(nsteps, dt, ck, timed):
        tr = mprw.Tracker(g, opt)
        tr.load_flow(f)
        tr.set_particles(p)
        tr.adj_setup(zones, nz, dt, nsteps, ck, (0.0, 0.0, float(g.botm[-1])), (1.0, 1.0, 1.0),
                     (g.ncol, g.nrow, g.nlay), (2.0, 2.0, 1.0), eps, seed=4242)
        target = tr.adj_forward(theta * 1.1)
        fwd_ms, bwd_ms = [], []
        for _ in range(3 if timed else 1):
            flush.zero_()
            rho = tr.adj_forward(theta)
            fwd_ms.append(tr.timings()["step_ms"])
            gr = tr.adj_backward(2.0 * (rho - target))
            bwd_ms.append(tr.timings()["step_ms"])
        loss = lambda th: float(((tr.adj_forward(th) - target) ** 2).sum())
        check = {}
        for kk, name in ((0, "alphaL_zone0"), (nz, "alphaT_zone0"), (2 * nz, "porosity_zone0"),
                         (3 * nz - 1, "porosity_zone7"), (3 * nz, "velocity_scale")):
            c = {"adjoint": float(gr[kk])}
            for rel in (1e-4, 1e-5):
                h = rel * abs(theta[kk])
                e = np.zeros_like(theta)
                e[kk] = h
                fd = (loss(theta + e) - loss(theta - e)) / (2 * h)
                c[f"central_difference_{rel:g}"] = fd
                c[f"rel_error_{rel:g}"] = abs(gr[kk] - fd) / max(abs(fd), 1e-300)
            check[name] = c
        tr.close()
        return dict(fwd=float(np.median(fwd_ms[-2:] if timed else fwd_ms)),
                    bwd=float(np.median(bwd_ms[-2:] if timed else bwd_ms)), check=check,
                    loss=float(((rho - target) ** 2).sum()), grad_norm=float(np.linalg.norm(gr)))

    full = run(2000, 0.05, 100, True)
    short = run(120, 0.02, 30, False)
    steps = n * 2000
    return {"workload": "lognormal slab (200x100x20), 8 zones (2x2x2 blocks), 25 parameters, 500,000 particles, "
                        "2,000 steps of 0.05 d stored every 100, density on the 1 m grid (biweight 2/2/1 m), misfit "
                        "against the +10 % run; FP64; velocity floor 0.01 m/d",
            "particle_steps": steps, "forward_ms": full["fwd"], "adjoint_ms": full["bwd"],
            "forward_rate": steps / (full["fwd"] / 1e3), "forward_plus_adjoint_rate":
                steps / ((full["fwd"] + full["bwd"]) / 1e3),
            "unit": UNIT, "loss": full["loss"], "grad_norm": full["grad_norm"],
            "gradient_check_100d": full["check"],
            "gradient_check_2.4d": short["check"],
            "note": "the adjoint is the exact derivative of the discrete walk (tests: torch autograd of an "
                    "independent restatement to 1e-9); the walk is piecewise smooth (trilinear fields are only "
                    "continuous across cell faces), so central differences reach it only with a step below the "
                    "spacing of the kinks the perturbed paths cross -- on the restatement at this velocity floor "
                    "(3,000 particles, 120 steps) they differ from autograd by 4e-4 at relative steps 1e-5 and "
                    "1e-6, 2.7e-4 at 1e-7 and 1.8e-7 at 1e-8; with 500,000 particles the kinks are denser and "
                    "the steps here (1e-4, 1e-5) resolve the gradient to ~1e-3 at 2.4 days; over 100 days "
                    "(about 20 cells) the paths' sensitivities grow and the differences are coarser"}


def gpkde_roofline(madds, kde_ms, sm_mhz, fp32):
    """The reconstruction against the issue rate of its arithmetic type: the
    work model (multiply-adds of the reference's direct 3-D kernels, summed
    over the optimisation loops; mprw_last_gpkde_work) per second of the
    reconstructions' CUDA-event time, against 152 SMs x FP64 2 (FP32 128)
    multiply-add lanes per clock at the sampled SM clock."""
    lanes = 128 if fp32 else 2
    peak = 152 * lanes * sm_mhz * 1e6
    achieved = float(np.sum(madds)) / (float(np.sum(kde_ms)) / 1e3)
    return {"bound": "fp32 issue" if fp32 else "fp64 issue", "achieved": achieved, "peak": peak,
            "unit": "multiply-adds/s", "frac": achieved / peak,
            "model": "per loop and active bin |K_W| + 8 |K_sigma| + 3 |K_SD| multiply-adds, |K| = prod_d "
                     "(2 ceil(r hOverDelta_d) + 1) at the bin's database levels (r = 3; 4 for second derivatives); "
                     "the separable passes do a fraction of it, so frac > 1 means fewer operations than direct "
                     "kernels, not more than the hardware issues",
            "peak_source": "nominal lanes per SM per clock at the sampled SM clock",
            "madds_per_reconstruction": float(np.mean(madds)), "ms_per_reconstruction": float(np.mean(kde_ms))}


def e2e_run(args, g, f, p, opt, origin, bins, domain, flush):
    """Through the C ABI with pinned host buffers; copies inside the timed region."""
    import ctypes as C

    import torch
    import mprw
    opt.precision = 0
    tr = mprw.Tracker(g, opt)
    tr.load_flow(f)
    n = p.n
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    st = dict(cell=pin(p.cell.astype(np.int32)), lx=pin(p.lx), ly=pin(p.ly), lz=pin(p.lz), t=pin(p.t),
              status=pin(p.status.astype(np.int32)), mass=pin(p.mass), id=pin(p.id.astype(np.uint64)),
              ctr=pin(np.zeros(n, np.uint64)))
    kopt = mprw.Tracker.gpkde_options(domain, bins, origin)
    ngrid = g.ncell
    dens, hist = pin(np.zeros(ngrid)), pin(np.zeros(ngrid))
    L = tr.lib
    dp, ip, up = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_uint64)
    P = lambda a, t_: a.ctypes.data_as(t_)
    nbo = (C.c_int32 * 3)()
    h2d = n * (4 + 8 * 3 + 8 + 4 + 8 + 8 + 8)
    d2h = n * (4 + 8 * 3 + 8 + 4 + 8) + 2 * 8 * ngrid
    t = 0.0
    tot_ms, steps = 0.0, 0
    steps_i = C.c_int64()
    loops = C.c_int32()
    for it in range(args.warmup + args.steps):
        if it >= args.warmup:
            flush.zero_()
            torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = L.mprw_set_particles(tr.h, n, P(st["cell"], ip), P(st["lx"], dp), P(st["ly"], dp), P(st["lz"], dp),
                                  P(st["t"], dp), P(st["status"], ip), P(st["mass"], dp), P(st["id"], up),
                                  P(st["ctr"], up))
        rc |= L.mprw_advance(tr.h, t, t + INTERVAL_D, C.byref(steps_i))
        rc |= L.mprw_get_particles(tr.h, P(st["cell"], ip), P(st["lx"], dp), P(st["ly"], dp), P(st["lz"], dp),
                                   P(st["t"], dp), P(st["status"], ip), P(st["ctr"], up), None, None, None)
        rc |= L.mprw_gpkde(tr.h, C.byref(kopt), P(dens, dp), P(hist, dp), nbo, C.byref(loops))
        t1 = time.perf_counter()
        if rc != 0:
            raise RuntimeError("e2e C-ABI call failed: " + L.mprw_last_error(tr.h).decode())
        if it >= args.warmup:
            tot_ms += (t1 - t0) * 1e3
            steps += steps_i.value
        t += INTERVAL_D
    tr.close()
    return dict(value=steps / (tot_ms / 1e3), ms_per_step=tot_ms / args.steps, h2d=h2d, d2h=d2h, steps=steps,
                tot_ms=tot_ms)


def btc_run(args, n_records=1_000_000, repeats=5):
    """Breakthrough-curve leg: the observation post-process's 1-D GPKDE
    (Freedman-Diaconis bins at fraction 0.75, raw density, kernel database
    off) of n_records seeded sink arrivals (lognormal times, median 100 d,
    over a 400-day run), timed end to end through mprw_gpkde_series (host
    arrays in and out); the numpy restatement on the host times one call on
    the same records."""
    import time as _t
    import mprw
    rng = np.random.default_rng(2024)
    t = rng.lognormal(np.log(100.0), 0.35, n_records)
    w = rng.uniform(0.5, 1.5, n_records) / 3.0
    kw = dict(domain_size=400.0, bin_format=1, bin_size_fraction=0.75, init_factor=3.0, raw_density=True,
              rel_err=0.01)
    for _ in range(2):
        r = mprw.gpkde_series(t, w, **kw)
    ms = []
    for _ in range(repeats):
        t0 = _t.perf_counter()
        r = mprw.gpkde_series(t, w, **kw)
        ms.append((_t.perf_counter() - t0) * 1e3)
    out = {"records": n_records, "ms": float(np.median(ms)), "records_per_s": n_records / (np.median(ms) / 1e3),
           "n_bins": r["n_bins"], "active_bins": r["active_bins"], "loops": r["loops"], "bin_size_d": r["bin_size"],
           "timing": "median of %d calls, host arrays in and out (H2D of 16 B per record inside)" % repeats}
    if not args.no_cpu:
        from oracle import series_oracle as SO
        t0 = _t.perf_counter()
        ref = SO.gpkde_series(t, w, **kw)
        cpu_ms = (_t.perf_counter() - t0) * 1e3
        out["cpu_baseline"] = {"ms": cpu_ms, "records_per_s": n_records / (cpu_ms / 1e3), "kind": "port",
                               "cores": 1, "sample": "one reconstruction of the same 10^6 records (numpy restatement)"}
        d = ref["density"]
        out["max_abs_diff_vs_port"] = float(np.abs(r["density"] - d).max() / np.abs(d).max())
        out["loops_port"] = ref["loops"]
    return out


def cpu_baseline(g, f, p, opt, n_sample, t_begin_steps, steps):
    """The oracle (C restatement of the reference, OpenMP on all host threads)
    on the first n_sample particles, from t=0 over warmup+steps intervals."""
    from oracle import oracle as O
    from mprw.model import Particles
    idx = slice(0, n_sample)
    q = Particles(cell=p.cell[idx].copy(), lx=p.lx[idx].copy(), ly=p.ly[idx].copy(), lz=p.lz[idx].copy(),
                  t=p.t[idx].copy(), status=p.status[idx].copy(), mass=p.mass[idx].copy(), id=p.id[idx].copy(),
                  rng_ctr=np.zeros(n_sample, np.uint64))
    opt.precision = 0
    th = O.cpu_count()
    O.reset_xoroshiro()   # one run: the thread streams are seeded once and continue across intervals
    t = 0.0
    tot, nsteps = 0.0, 0
    for it in range(t_begin_steps + steps):
        t0 = time.perf_counter()
        q, s = O.advance(g, f, opt, q, t, t + INTERVAL_D, rng_kind=O.RNG_XOROSHIRO, nthreads=th)
        t1 = time.perf_counter()
        if it >= t_begin_steps:
            tot += t1 - t0
            nsteps += s
        t += INTERVAL_D
    return dict(value=nsteps / tot, unit=UNIT, cores=th, kind="port",
                sample=f"first {n_sample} of the {p.n} particles, {steps} x {INTERVAL_D:g}-day intervals "
                       f"after {t_begin_steps} untimed, advance only (no GPKDE); xoroshiro128+ thread streams as "
                       "the reference",
                seconds=tot)


def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        return main_reference(args, rank, world)
    if args.workload == "lognormal_injection":
        return main_injection(args)
    import torch
    res = run_gpu_arm(args, rank, world, local)
    fp = res["fp64"]
    t_kern = sum(fp["ms"])
    ms_step = t_kern / args.steps
    value_rank = fp["steps"] / (t_kern / 1e3)
    # whole-job: all ranks' steps over the slowest rank's time
    tot_steps, max_t = fp["steps"], t_kern
    if world > 1:
        import torch.distributed as dist
        v = torch.tensor([float(fp["steps"]), t_kern], dtype=torch.float64)
        allv = [torch.zeros_like(v) for _ in range(world)]
        dist.all_gather(allv, v)
        tot_steps = sum(float(a[0]) for a in allv)
        max_t = max(float(a[1]) for a in allv)
    value = tot_steps / (max_t / 1e3)
    # the end-to-end rate aggregated the same way (all ranks' steps over the slowest rank)
    e2e_value, e2e_max_ms = None, None
    if "e2e" in res:
        e_steps, e2e_max_ms = float(res["e2e"]["steps"]), float(res["e2e"]["tot_ms"])
        if world > 1:
            v = torch.tensor([e_steps, e2e_max_ms], dtype=torch.float64)
            allv = [torch.zeros_like(v) for _ in range(world)]
            dist.all_gather(allv, v)
            e_steps = sum(float(a[0]) for a in allv)
            e2e_max_ms = max(float(a[1]) for a in allv)
        e2e_value = e_steps / (e2e_max_ms / 1e3)
    if rank != 0:
        return
    hbm, peak_kind = peaks()
    kern_avg_ms = float(np.mean(fp["kern_ms"]))
    steps_per_launch = fp["steps"] / args.steps
    achieved = steps_per_launch * B_STEP_FP64 / (kern_avg_ms / 1e3) / 1e9
    tr_ps = ncu_figure("dram_bytes_per_particle_step")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": max_t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "lognormal_slab: 200x100x20 lognormal-K field (sigma2 lnK 1, 10 m/2 m), FP64 CG heads, "
                               f"{args.particles} particles from the inlet slab, step = one 10-day interval "
                               "(advance + GPKDE reconstruction on the 1 m grid, density and histogram to host)",
                   "particles_per_gpu": args.particles, "interval_days": INTERVAL_D,
                   "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"particles x{world}" + (
                       ", one GPKDE of all ranks' particles per step (per-rank parts all-reduced)" if world > 1 else ""),
                   "flow_input": f"MODFLOW 6 binary .grb/.hds/.bud ({res['mf6_bytes']} B: FLOW-JA-FACE imeth 1, "
                                 "CHD imeth 6) written from the CG solve and read back by mprw.mf6io"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_source": f"{peak_kind} hbm_gbs",
                     "traffic": None if tr_ps is None else tr_ps * steps_per_launch,
                     "kernel": "rwpt_advance_kernel<double>", "kernel_ms": kern_avg_ms,
                     "bytes_model": "1008 B per particle-step (state 96 B + cell record 912 B)",
                     "fp64_pipe_active_pct_ncu": ncu_figure("fp64_pipe_active_pct"),
                     "traffic_source": "not measured in this run: the ncu DRAM bytes per particle-step of the "
                                       "committed 200,000-particle capture (profiles/rwpt_advance_kernel_"
                                       "lognormal_slab.md) times this run's particle-steps per launch; "
                                       "fp64_pipe_active_pct_ncu is read from the same capture",
                     "note": "the step kernel is bound by the FP64 pipe (GB300: 2 FP64 lane-operations per clock "
                             "per SM), not HBM: the records stay in L2; traffic is ncu DRAM bytes"},
        "clocks": res["clocks"],
        "gpu_launches": int(fp["launches"]),
        "tuning": fp["tuning"],
        "kernel_time_share": {"advance_kernel_ms": float(np.sum(fp["kern_ms"])),
                              "advance_event_ms": float(np.sum(fp["adv_ms"])),
                              "gpkde_ms": float(np.sum(fp["kde_ms"])), "step_event_ms": float(np.sum(fp["ms"])),
                              "step_wall_ms": float(np.sum(fp["wall_ms"])), "gpkde_loops": fp["loops"]},
        "gpkde_roofline": gpkde_roofline(fp["madds"], fp["kde_ms"], res["clocks"]["sm_mhz"] or 2070.0,
                                         args.precision == "mixed"),
    }
    if "e2e" in res:
        e = res["e2e"]
        line["e2e"] = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": e["h2d"] * world,
                       "d2h_bytes_per_step": e["d2h"] * world, "ms_per_step": e2e_max_ms / args.steps}
    if "mixed" in res:
        mx = res["mixed"]
        tm = sum(mx["ms"])
        m64, n64 = moments(fp["out"])
        m32, n32 = moments(mx["out"])
        err = {k: {"mean_rel": abs(m32[k][0] - m64[k][0]) / max(abs(m64[k][0]), 1e-30),
                   "var_rel": abs(m32[k][1] - m64[k][1]) / max(abs(m64[k][1]), 1e-30)} for k in m64}
        adv64, adv32 = sum(fp["adv_ms"]), sum(mx["adv_ms"])
        line["mixed"] = {"value": mx["steps"] / (tm / 1e3), "unit": UNIT, "speedup_vs_fp64": (mx["steps"] / tm) /
                         (fp["steps"] / t_kern),
                         "advance_only": {"value": mx["steps"] / (adv32 / 1e3),
                                          "speedup_vs_fp64": (mx["steps"] / adv32) / (fp["steps"] / adv64)},
                         "moment_error_vs_fp64": err, "active_fp64": n64,
                         "active_mixed": n32, "kernel_ms": float(np.mean(mx["kern_ms"])),
                         "gpkde_ms": float(np.mean(mx["kde_ms"])), "gpkde_precision": "fp32", "tuning": mx["tuning"],
                         "gpkde_fp32_vs_fp64_same_particles": mx["kde_err"],
                         "gpkde_roofline": gpkde_roofline(mx["madds"], mx["kde_ms"],
                                                          res["clocks"]["sm_mhz"] or 2070.0, True)}
    line["lognormal_slab_btc_150m"] = {
        "curve": fp["btc150"], "control_plane_x_m": 150.0,
        "counts": "after every 10-day advance (warm-up included): ACTIVE particles at or beyond x = 150 m plus "
                  "those stopped at the outlet; the mean plume (v ~ 0.2 m/d) does not reach the plane in this "
                  "run, only fast-channel early arrivals do"}
    if not args.no_pulse:
        line["uniform_pulse"] = pulse_run(args, res["flush"])
    if not args.no_adjoint:
        g_, f_, _, _ = res["geom"]
        line["adjoint"] = adjoint_run(args, g_, f_, res["flush"])
    if "batched" in res:
        line["batched"] = res["batched"]
        line["batched"]["headline_fp64_value"] = value_rank
    if not args.no_cpu:
        g, f, p, opt = res["geom"]
        line["cpu_baseline"] = cpu_baseline(g, f, p, opt, args.cpu_sample, args.warmup, min(args.steps, 5))
    if not args.no_btc:
        line["btc"] = btc_run(args)
    print(json.dumps(line))


def main_injection(args):
    """The large single run (workloads.lognormal_injection): 12.5e6 cells, particles
    released over 50 days, tracked to 500 days in 25-day intervals, each
    followed by a GPKDE reconstruction on the 250x250x25 grid with 5
    optimisation loops.  Run whole in FP64, then in MIXED on the same
    particles and random streams; every interval is timed with CUDA events."""
    import torch
    import mprw
    from mprw import workloads as W
    from mprw.model import MIXED
    t_setup = time.perf_counter()
    g, f, p, opt, info = W.lognormal_injection(n_particles=args.injection_particles, use_torch=True)
    t_setup = time.perf_counter() - t_setup
    stream = torch.cuda.Stream()
    hbm, peak_kind = peaks()
    domain, bins = (500.0, 500.0, 50.0), (2.0, 2.0, 2.0)
    res = {}
    for name, prec in (("fp64", 0), ("mixed", MIXED)):
        opt.precision = prec
        tr = mprw.Tracker(g, opt)
        tr.set_stream(stream.cuda_stream)
        tr.load_flow(f)
        tr.set_particles(p)
        tuning = tr.autotune(0.0, 25.0)
        torch.cuda.synchronize()
        steps, adv_ms, kern_ms, kde_ms, tot_ms = 0, 0.0, 0.0, 0.0, 0.0
        t = 0.0
        for k in range(20):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            e[0].record(stream)
            steps += tr.advance(t, t + 25.0)
            kern_ms += tr.timings()["step_ms"]
            e[1].record(stream)
            tr.gpkde(domain, bins, n_opt_loops=5, precision=prec)
            e[2].record(stream)
            torch.cuda.synchronize()
            adv_ms += e[0].elapsed_time(e[1])
            kde_ms += e[1].elapsed_time(e[2])
            tot_ms += e[0].elapsed_time(e[2])
            t += 25.0
        out = tr.get_particles()
        tr.close()
        b_step = 1008 if prec == 0 else 544
        res[name] = {"value": steps / (tot_ms / 1e3), "particle_steps": steps, "ms_total": tot_ms,
                     "advance_ms": adv_ms, "gpkde_ms": kde_ms,
                     "advance_rate": steps / (kern_ms / 1e3),
                     "roofline": {"bound": "hbm", "achieved": steps * b_step / (kern_ms / 1e3) / 1e9, "peak": hbm,
                                  "unit": "GB/s", "frac": steps * b_step / (kern_ms / 1e3) / 1e9 / hbm,
                                  "peak_source": f"{peak_kind} hbm_gbs",
                                  "bytes_model": f"{b_step} B per particle-step"},
                     "tuning": tuning, "moments": moments(out)[0], "active": moments(out)[1],
                     "statuses": np.bincount(out["status"], minlength=10).tolist()}
    m64, m32 = res["fp64"]["moments"], res["mixed"]["moments"]
    err = {k: {"mean_rel": abs(m32[k][0] - m64[k][0]) / max(abs(m64[k][0]), 1e-30),
               "var_rel": abs(m32[k][1] - m64[k][1]) / max(m64[k][1], 1e-30)} for k in m64}
    line = {"metric": METRIC, "value": res["fp64"]["value"], "unit": UNIT, "n_gpus": 1, "steps": 20, "warmup": 0,
            "ms_per_step": res["fp64"]["ms_total"] / 20, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "lognormal_injection: 500x500x50 lognormal-K field (sigma2 lnK 2, 20 m / 2 m), "
                                   f"{p.n} particles released over 50 d from a 20x20x10 m source, tracked to "
                                   "500 d in 20 intervals of 25 d, each followed by GPKDE on 250x250x25 (5 loops); "
                                   "the whole run is timed (no warm-up interval)",
                       "cells": g.ncell, "setup_s": t_setup},
            "fp64": res["fp64"], "mixed": res["mixed"],
            "mixed_speedup_vs_fp64": res["mixed"]["value"] / res["fp64"]["value"],
            "moment_error_mixed_vs_fp64": err}
    print(json.dumps(line))


def main_reference(args, rank, world):
    if rank != 0:
        return
    g, f, p, opt, info = build_workload(args.particles, 0, use_torch=False)
    cb = cpu_baseline(g, f, p, opt, args.cpu_sample, args.warmup, args.steps)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "ms_per_step": cb["seconds"] * 1e3 / args.steps,
            "config": {"workload": "lognormal_slab (same field and release), bounded particle sample",
                       "particles": args.cpu_sample, "interval_days": INTERVAL_D},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference is Fortran and no Fortran compiler exists on these machines; the timed CPU "
                    "implementation is the C restatement of its advance (oracle/), OpenMP on all host threads; "
                    "the GPKDE reconstruction is not timed on the CPU, so this rate is an upper bound on the "
                    "reference's advance + GPKDE pipeline"}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
