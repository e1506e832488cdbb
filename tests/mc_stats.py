"""Monte-Carlo summaries of a particle plume and their two-sample comparison.

The GPU tracks with counter-based Philox normals and the reference with
xoroshiro128+ thread streams (rng_par_zig.f90:156-335; normals
TrackSubCell.F90:3631-3663), so the two cannot agree particle by particle:
they are compared as two samples of the same random-walk process.  A summary
holds what characterises a plume -- the stop-status counts (mass leaving
through weak sinks, MPathRW.F90:1337-1403), the first, second and fourth
central moments of the ACTIVE particles' model coordinates, their
histogram along x, the particles past a control plane, and the
breakthrough (stop-time) histogram of the particles that stopped at a weak
sink.  ``compare`` tests each statistic with a two-sample z or chi-square
test at a fixed threshold; it returns the failures as text.
"""
from __future__ import annotations

import math

import numpy as np

ACTIVE, WEAK_SINK = 1, 3
Z_MAX = 4.5          # two-sided; with ~40 statistics per comparison a false alarm has p ~ 3e-4
CHI2_P_MIN = 1e-5


def summarize(status, gx, gy, gz, t, x_edges, x_plane=None, t_edges=None):
    status = np.asarray(status)
    act = status == ACTIVE
    d = {"n": np.int64(status.shape[0]), "status_counts": np.bincount(status, minlength=10).astype(np.int64)}
    for ax, v in (("x", gx), ("y", gy), ("z", gz)):
        a = np.asarray(v, np.float64)[act]
        m = a.mean() if a.size else 0.0
        c = a - m
        d[f"mean_{ax}"] = np.float64(m)
        d[f"var_{ax}"] = np.float64((c * c).mean() if a.size else 0.0)
        d[f"m4_{ax}"] = np.float64((c ** 4).mean() if a.size else 0.0)
    d["hist_x"] = np.histogram(np.asarray(gx)[act], x_edges)[0].astype(np.int64)
    if x_plane is not None:
        gxa = np.asarray(gx)
        d["past_plane"] = np.int64(((act | (status == WEAK_SINK)) & (gxa > x_plane)).sum())
    if t_edges is not None:
        ts = np.asarray(t, np.float64)[status == WEAK_SINK]
        d["hist_stop_t"] = np.histogram(ts, t_edges)[0].astype(np.int64)
        d["mean_stop_t"] = np.float64(ts.mean() if ts.size else 0.0)
        d["var_stop_t"] = np.float64(ts.var() if ts.size else 0.0)
        d["m4_stop_t"] = np.float64(((ts - ts.mean()) ** 4).mean() if ts.size else 0.0)
    return d


def _z_prop(k1, n1, k2, n2):
    p = (k1 + k2) / (n1 + n2)
    se = math.sqrt(max(p * (1 - p) * (1.0 / n1 + 1.0 / n2), 1e-300))
    return (k1 / n1 - k2 / n2) / se


def _chi2_two_sample(r, s, min_count=10):
    """Two-sample chi-square of histograms r, s (different totals); sparse bins merged
    left to right until their pooled count reaches min_count.  Returns (chi2, dof, p)."""
    from scipy import stats
    r, s = np.asarray(r, np.float64), np.asarray(s, np.float64)
    rr, ss, ar, as_ = [], [], 0.0, 0.0
    for a, b in zip(r, s):
        ar += a
        as_ += b
        if ar + as_ >= min_count:
            rr.append(ar)
            ss.append(as_)
            ar = as_ = 0.0
    if ar + as_ > 0:
        if rr:
            rr[-1] += ar
            ss[-1] += as_
        else:
            rr.append(ar)
            ss.append(as_)
    rr, ss = np.array(rr), np.array(ss)
    n1, n2 = rr.sum(), ss.sum()
    if len(rr) < 2 or n1 == 0 or n2 == 0:
        return 0.0, 0, 1.0
    k1, k2 = math.sqrt(n2 / n1), math.sqrt(n1 / n2)
    chi2 = float((((k1 * rr - k2 * ss) ** 2) / (rr + ss)).sum())
    dof = len(rr) - 1
    return chi2, dof, float(stats.chi2.sf(chi2, dof))


def compare(a, b, label=""):
    """Failures (list of str) of summary a against summary b."""
    bad = []
    n1, n2 = int(a["n"]), int(b["n"])
    for st in range(10):
        k1, k2 = int(a["status_counts"][st]), int(b["status_counts"][st])
        if k1 + k2 == 0:
            continue
        if k1 + k2 == n1 + n2:      # every particle in this status on both sides
            continue
        z = _z_prop(k1, n1, k2, n2)
        if abs(z) > Z_MAX:
            bad.append(f"{label} status {st}: {k1}/{n1} vs {k2}/{n2} (z {z:.2f})")
    m1, m2 = int(a["status_counts"][ACTIVE]), int(b["status_counts"][ACTIVE])
    for ax in ("x", "y", "z"):
        v1, v2 = float(a[f"var_{ax}"]), float(b[f"var_{ax}"])
        if m1 > 1 and m2 > 1:
            se = math.sqrt(v1 / m1 + v2 / m2)
            z = (float(a[f"mean_{ax}"]) - float(b[f"mean_{ax}"])) / max(se, 1e-300)
            if abs(z) > Z_MAX:
                bad.append(f"{label} mean_{ax}: {float(a[f'mean_{ax}']):.6g} vs {float(b[f'mean_{ax}']):.6g} "
                           f"(z {z:.2f})")
            se = math.sqrt(max(float(a[f"m4_{ax}"]) - v1 * v1, 0.0) / m1 + max(float(b[f"m4_{ax}"]) - v2 * v2, 0.0) / m2)
            z = (v1 - v2) / max(se, 1e-300)
            if abs(z) > Z_MAX:
                bad.append(f"{label} var_{ax}: {v1:.6g} vs {v2:.6g} (z {z:.2f})")
    chi2, dof, p = _chi2_two_sample(a["hist_x"], b["hist_x"])
    if p < CHI2_P_MIN:
        bad.append(f"{label} hist_x: chi2 {chi2:.1f} dof {dof} p {p:.2e}")
    if "past_plane" in a and "past_plane" in b:
        z = _z_prop(int(a["past_plane"]), n1, int(b["past_plane"]), n2)
        if abs(z) > Z_MAX:
            bad.append(f"{label} past_plane: {int(a['past_plane'])} vs {int(b['past_plane'])} (z {z:.2f})")
    if "hist_stop_t" in a and "hist_stop_t" in b:
        chi2, dof, p = _chi2_two_sample(a["hist_stop_t"], b["hist_stop_t"])
        if p < CHI2_P_MIN:
            bad.append(f"{label} hist_stop_t: chi2 {chi2:.1f} dof {dof} p {p:.2e}")
        s1, s2 = int(a["status_counts"][WEAK_SINK]), int(b["status_counts"][WEAK_SINK])
        if s1 > 1 and s2 > 1:
            v1, v2 = float(a["var_stop_t"]), float(b["var_stop_t"])
            se = math.sqrt(v1 / s1 + v2 / s2)
            z = (float(a["mean_stop_t"]) - float(b["mean_stop_t"])) / max(se, 1e-300)
            if abs(z) > Z_MAX:
                bad.append(f"{label} mean_stop_t: {float(a['mean_stop_t']):.6g} vs {float(b['mean_stop_t']):.6g} "
                           f"(z {z:.2f})")
    return bad


def to_npz(prefix, d):
    return {f"{prefix}{k}": np.asarray(v) for k, v in d.items()}


def from_npz(z, prefix):
    return {k[len(prefix):]: z[k] for k in z.files if k.startswith(prefix)}
