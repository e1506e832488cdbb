"""numpy restatement of GPKDE (TEST INFRASTRUCTURE ONLY).

Follows lib/gpkde of the reference (paths relative to its src/ directory):

* histogram_weighted -- Histogram.F90:276-350 (prComputeCountsWeighted);
* GPKDE              -- GridProjectedKDE.F90 prInitialize (354-998),
  prComputeDensity (3598-4392), prComputeDensityOptimization (4396-5160),
  smoothing scale (5164-5203), curvature bandwidth (5207-5275), net
  roughness 1-D (1666-1903), 2-D (1905-2289) and 3-D (2295-2709), optimal
  smoothing and shape (5404-5724), kernel database and indexes (3138-3528,
  5727-5962, 6467-6500), the isotropic-kernel option (gpkdeIsotropicKernels,
  passed at MPathRW.F90:1639: no isotropy correction, unit shapes, and the
  isotropic net-roughness sums 2182-2228, 2660-2676);
* kernels            -- KernelMultiGaussian.f90: W matrix (720-790), second
  derivative matrices (794-1110), spans and boundary reflection (209-390),
  unfold (516-546), SetupMatrix (549-590).

Reference quirks kept: the second-derivative kernels are never rescaled
(their balance coefficient needs a positive sum of negative entries, and the
`if (...) matrix = 0; return` line returns unconditionally before the scaling,
KernelMultiGaussian.f90:865-887, 969-993, 1071-1097); the 3-D shape
normalisation uses the single-precision exponent 0.333 (GridProjectedKDE.F90:5654);
the 2-D net roughness multiplies the two curvatures before squaring them
(2134-2138) where the 3-D one squares them first (2463-2468).
The options MODPATH-RW uses are restated: for the spatial reconstruction the
kernel database on (logarithmic), bounded kernel sizes (format 0),
minimum-roughness format 3, effective-weight format 0 (Kish), anisotropic
or isotropic kernels, no sliced reconstruction, grid fixed to the domain; for the observation time
series (``series_oracle.py``) the database off and the grid optionally
adapted to the data.  ``np.add.at`` accumulates repeated indices in
array order, the reference's loop order.
"""
from __future__ import annotations

import math
from functools import lru_cache

import numpy as np

SQRT2 = math.sqrt(2.0)
PI = 4.0 * math.atan(1.0)
SQRTPI = math.sqrt(4.0 * math.atan(1.0))
SQRT8PI = math.sqrt(8.0 * PI)
F32_0333 = float(np.float32(0.333))


def histogram_weighted(coords: np.ndarray, weights: np.ndarray, origin, bin_size, n_bins):
    """coords (N,3) model coordinates of the active particles in particle order.
    Returns (counts shaped (nz, ny, nx), n_binned, effective_mass)."""
    origin = np.asarray(origin, np.float64)
    bin_size = np.asarray(bin_size, np.float64)
    n_bins = np.asarray(n_bins, np.int64)
    n = coords.shape[0]
    idx = np.zeros((n, 3), np.int64)
    inside = np.ones(n, bool)
    for d in range(3):
        if bin_size[d] == 0.0:
            continue
        q = np.floor((coords[:, d] - origin[d]) / bin_size[d])
        ok = (q >= 0) & (q < n_bins[d])
        inside &= ok
        idx[:, d] = np.where(ok, q, 0).astype(np.int64)
    lin = idx[:, 0] + n_bins[0] * (idx[:, 1] + n_bins[1] * idx[:, 2])
    counts = np.zeros(int(np.prod(n_bins)), np.float64)
    np.add.at(counts, lin[inside], weights[inside])
    total = 0.0
    sw2 = 0.0
    for w in weights:          # sequential sums, as gfortran's sum()
        total = total + float(w)
        sw2 = sw2 + float(w) * float(w)
    eff = 1.0
    if total != 0.0:
        neff = total * total / sw2
        eff = total / neff
        counts = counts / eff
    return counts.reshape(int(n_bins[2]), int(n_bins[1]), int(n_bins[0])), int(inside.sum()), eff


# --------------------------------------------------------------------------
# kernels (arrays indexed [x, y, z], the Fortran layout)
# --------------------------------------------------------------------------
def _positive_shape(matrix_range, bandwidth, bin_size):
    out = np.zeros(3, np.int64)
    for d in range(3):
        if bin_size[d] != 0.0:
            out[d] = math.ceil(matrix_range * bandwidth[d] / bin_size[d])
    return out


def _hdelta(bandwidth, bin_size):
    return np.array([bandwidth[d] / bin_size[d] if bin_size[d] != 0.0 else 0.0 for d in range(3)])


def _unfold(zp, m):
    """prUnfoldZeroPositiveMatrix: mirror the (m+1)^3 octant to (2m+1)^3."""
    full = np.zeros(tuple(2 * m + 1))
    sx = [slice(m[0], 2 * m[0] + 1), slice(0, m[0])]
    sy = [slice(m[1], 2 * m[1] + 1), slice(0, m[1])]
    sz = [slice(m[2], 2 * m[2] + 1), slice(0, m[2])]
    rx = [slice(None), slice(m[0], 0, -1)]
    ry = [slice(None), slice(m[1], 0, -1)]
    rz = [slice(None), slice(m[2], 0, -1)]
    for a in range(2):
        for b in range(2):
            for c in range(2):
                full[sx[a], sy[b], sz[c]] = zp[rx[a], ry[b], rz[c]]
    return full


def _erf_diff(i, hd):
    e = np.vectorize(math.erf)
    return e((i + 0.5) / (hd * SQRT2)) - e((i - 0.5) / (hd * SQRT2))


def w_matrix(bandwidth, bin_size, ndim, matrix_range=3):
    """prSetupMatrix + prComputeKernelWMatrix."""
    m = _positive_shape(matrix_range, bandwidth, bin_size)
    if np.all(np.asarray(bandwidth) == 0.0):
        return np.zeros(tuple(2 * m + 1)), m
    hd = _hdelta(bandwidth, bin_size)
    grids = np.meshgrid(*[np.arange(m[d] + 1, dtype=np.float64) for d in range(3)], indexing="ij")
    zp = np.full(tuple(m + 1), 0.5 ** float(ndim))
    for d in range(3):
        if hd[d] <= 0.0:
            continue
        zp = zp * _erf_diff(grids[d], hd[d])
    full = _unfold(zp, m)
    s = full.sum()
    if s != 0.0:
        full = full / s
    return full, m


def sd_matrix(axis, bandwidth, bin_size, ndim, matrix_range=4):
    """prComputeKernelV{X,Y,Z}Matrix, with the reference's early return."""
    m = _positive_shape(matrix_range, bandwidth, bin_size)
    if np.all(np.asarray(bandwidth) == 0.0):
        return np.zeros(tuple(2 * m + 1)), m
    hd = _hdelta(bandwidth, bin_size)
    grids = np.meshgrid(*[np.arange(m[d] + 1, dtype=np.float64) for d in range(3)], indexing="ij")
    zp = np.ones(tuple(m + 1))
    for d in range(3):
        if hd[d] <= 0.0:
            continue
        g = grids[d]
        if d == axis:
            h = hd[d]
            c = -1.0 / ((2.0 ** (float(ndim) - 0.5)) * SQRTPI * (h ** 3.0))
            zp = zp * c * ((g + 0.5) * np.exp(-1.0 * ((g + 0.5) * (g + 0.5)) / (2.0 * (h * h)))
                           - (g - 0.5) * np.exp(-1.0 * ((g - 0.5) * (g - 0.5)) / (2.0 * (h * h))))
        else:
            zp = zp * _erf_diff(g, hd[d])
    full = _unfold(zp, m)
    # balance coefficient: the sum of negative entries is never > 0, so it stays 1
    ssq = float((full * full).sum())
    if ssq <= 0.0:
        return np.zeros_like(full), m
    for d in range(3):
        if hd[d] <= 0.0:
            continue
        if d == axis:
            break  # `if (normprod <= 0) matrix = 0; return` returns unconditionally
        full = full / math.sqrt(hd[d])
    return full, m


def spans_and_reflect(matrix, m, gid, nbins, dims):
    """prComputeSpansBounded + prKernelReflection; gid 1-based bin index.
    Returns (grid slices (0-based), reflected matrix restricted to the span)."""
    mat = matrix.copy()
    shape = mat.shape
    gspan, kspan = [], []
    for d in range(3):
        g0 = max(gid[d] - m[d], 1)
        g1 = min(gid[d] + m[d], nbins[d])
        gspan.append((g0, g1))
        kspan.append((g0 + m[d] - gid[d] + 1, g1 + m[d] - gid[d] + 1))
    for d in dims:
        lo = (gid[d] - m[d]) < 1
        hi = (gid[d] + m[d]) > nbins[d]
        if not (lo or hi):
            continue
        ax = [slice(None)] * 3
        if lo:
            b = 1 - gid[d] + m[d]
            dst = list(ax); dst[d] = slice(b, 2 * b)
            src = list(ax); src[d] = _rev(b - 1, 0)
            mat[tuple(dst)] = mat[tuple(dst)] + mat[tuple(src)]
            z = list(ax); z[d] = slice(0, b)
            mat[tuple(z)] = 0.0
        if hi:
            b = 2 * m[d] + 1 - (gid[d] + m[d] - nbins[d]) + 1
            lenb = shape[d] - b + 1
            dst = list(ax); dst[d] = slice(b - lenb - 1, b - 1)
            src = list(ax); src[d] = _rev(shape[d] - 1, b - 1)
            mat[tuple(dst)] = mat[tuple(dst)] + mat[tuple(src)]
            z = list(ax); z[d] = slice(b - 1, None)
            mat[tuple(z)] = 0.0
    gsl = tuple(slice(g0 - 1, g1) for g0, g1 in gspan)
    ksl = tuple(slice(k0 - 1, k1) for k0, k1 in kspan)
    return gsl, mat[ksl]


def _rev(start, stop):
    """0-based indices start, start-1, ..., stop (inclusive) as a slice."""
    return slice(start, stop - 1 if stop - 1 >= 0 else None, -1)


# --------------------------------------------------------------------------
class GPKDE:
    def __init__(self, domain_size, bin_size, origin=(0.0, 0.0, 0.0), n_opt_loops=10, min_hod=0.3,
                 delta_hod=0.3, max_hod=15.0, rel_err=0.02, skip_error=False, isotropic=False, database=True,
                 n_bins=None):
        """``database=False`` sets every kernel up from its exact smoothing
        (prSetKernelBrute / prSetKernelSigmaBrute / prSetKernelSD1DBrute,
        GridProjectedKDE.F90:6224-6317) instead of the database entry.
        ``n_bins`` overrides the reconstruction grid (a sub-grid adapted to the
        data, :3903-3960); the kernel-size bounds keep following the domain
        grid size (:1296-1310)."""
        self.domain_size = np.asarray(domain_size, np.float64)
        self.bin_size = np.asarray(bin_size, np.float64)
        self.origin = np.asarray(origin, np.float64)
        gs = np.ones(3, np.int64)
        for d in range(3):
            if self.bin_size[d] != 0.0:
                gs[d] = int(self.domain_size[d] / self.bin_size[d] + 0.5)
        self.nbins = gs if n_bins is None else np.asarray(n_bins, np.int64)
        self.database = database
        self.mask = np.array([0 if gs[d] == 1 else 1 for d in range(3)])
        self.ndim = int(self.mask.sum())
        self.dims = [d for d in range(3) if self.mask[d]]
        nd = float(self.ndim)
        self.support_c = ((nd + 2.0) * (8.0 * PI) ** (0.5 * nd)) ** 0.25
        self.alpha_c = ((1.0 + 2.0 ** (0.5 * nd + 2.0)) / (3.0 * 2.0 ** (4.0 / (nd + 4.0)))) ** (1.0 / (nd + 6.0)) \
            * (nd + 2.0) ** (1.0 / (nd + 4.0)) / ((nd + 4.0) ** (1.0 / (nd + 6.0)))
        self.beta_c = 2.0 / (nd + 4.0) / (nd + 6.0)
        self.one_over_nd4 = 1.0 / (nd + 4.0)
        self.minus_one_over_nd6 = -1.0 / (nd + 6.0)
        self.one_plus_nd_quarter = 1.0 + 0.25 * nd
        self.n_opt_loops = n_opt_loops
        self.rel_err = rel_err
        self.skip_error = skip_error
        self.isotropic = isotropic
        # histogram geometry (active histogram dimensions: bin size > 0)
        hd = [d for d in range(3) if self.bin_size[d] > 0.0]
        self.bin_volume = float(np.prod(self.bin_size[hd]))
        self.bin_distance = self.bin_volume ** (1.0 / float(len(hd)))
        # kernel database (logarithmic)
        n = math.ceil(math.log10(max_hod / min_hod) / math.log10(1 + delta_hod)) + 1
        li, le = math.log10(min_hod), math.log10(max_hod)
        de = (le - li) / (n - 1)
        acc = 0.0
        hod = []
        for _ in range(n):
            hod.append(10.0 ** (li + acc))
            acc = acc + de
        self.hod = np.array(hod)
        self.n_delta = n
        self.min_hod = min_hod
        self.delta_log = math.log(self.hod[1] / self.hod[0])
        # kernel size bounds (boundKernelSizeFormat 0)
        self.max_k = np.zeros(3)
        self.max_sd = np.zeros(3)
        self.min_k = np.zeros(3)
        self.min_sd = np.zeros(3)
        for d in range(3):
            if not self.mask[d]:
                continue
            self.max_k[d] = self.bin_size[d] * (0.9 * gs[d] - 1) / 3.0
            self.max_sd[d] = self.bin_size[d] * (0.9 * gs[d] - 1) / 4.0
            self.min_k[d] = 1.2 * self.bin_size[d] / 3.0
            self.min_sd[d] = 1.2 * self.bin_size[d] / 4.0
        pos = [d for d in range(3) if self.max_k[d] > 0]
        self.max_dim = min(pos, key=lambda d: (self.max_k[d], d))
        pos = [d for d in range(3) if self.min_k[d] > 0]
        self.min_dim = max(pos, key=lambda d: (self.min_k[d], -d))
        self.max_sigma_growth = 1.5
        self.iso_threshold = 0.85

    # -- database lookups ---------------------------------------------------
    def _log_index(self, h, d):
        if h <= 0.0:
            return 1
        return min(max(math.floor(math.log(h / self.bin_size[d] / self.min_hod) / self.delta_log) + 1, 1),
                   self.n_delta)

    def _w_indexes(self, smoothing):
        idx = [1, 1, 1]
        for d in self.dims:
            if smoothing[d] <= 0.0:
                continue
            idx[d] = self._log_index(smoothing[d], d)
        return tuple(idx)

    @lru_cache(maxsize=None)
    def _w_db(self, idx):
        inp = np.zeros(3)
        for d in self.dims:
            inp[d] = self.hod[idx[d] - 1]
        return w_matrix(inp * self.bin_size, self.bin_size, self.ndim, 3)

    @lru_cache(maxsize=None)
    def _sd_db(self, axis, n):
        inp = np.zeros(3)
        if self.ndim == 3:
            inp[:] = self.hod[n - 1]
        else:
            for d in self.dims:
                inp[d] = self.hod[n - 1]
        return sd_matrix(axis, inp * self.bin_size, self.bin_size, self.ndim, 4)

    def _kernel_span(self, mat_m, gid):
        mat, m = mat_m
        return spans_and_reflect(mat, m, gid, self.nbins, self.dims)

    # -- the reconstruction ---------------------------------------------------
    def compute_density(self, coords, weights, unit_volume=True, scaling_factor=1.0):
        """Returns the density grid shaped (nx, ny, nz) and the smoothing per active bin.
        Afterwards ``self.work`` holds the work model of its optimisation loops
        (per loop and active bin |K_W| + 8 |K_sigma| + 3 |K_SD| cells)."""
        self.work = 0
        counts_zyx, _, eff_mass = histogram_weighted(coords, weights, self.origin, self.bin_size, self.nbins)
        counts = np.ascontiguousarray(counts_zyx.transpose(2, 1, 0))   # [x, y, z]
        npts = coords.shape[0]
        total = float(np.sum(weights))
        dens = np.zeros(tuple(self.nbins))
        act = np.argwhere(counts.transpose(2, 1, 0) != 0.0)[:, ::-1] + 1   # x fastest order, 1-based
        nb = act.shape[0]
        if nb == 0:
            return dens, None
        mean = coords.sum(axis=0) / npts
        std = np.zeros(3)
        for d in range(3):
            if self.mask[d]:
                std[d] = math.sqrt(float(((coords[:, d] - mean[d]) ** 2.0).sum()) / npts)
        ss = float(np.prod(std[self.mask == 1])) ** (1.0 / float(self.ndim))
        hs = ss * (4.0 / ((float(self.ndim) + 2.0) * npts)) ** (1.0 / (float(self.ndim) + 4.0))
        if ss == 0.0:
            hs = 2.0 * self.bin_distance
        init = np.where(self.mask == 1, hs, 0.0)
        d_out, smooth = self._optimize(counts, act, init, npts)
        d_out = d_out * eff_mass
        if unit_volume:
            d_out = d_out * self.bin_volume
        if scaling_factor != 0.0:
            d_out = d_out * scaling_factor
        return d_out, smooth

    def _smoothing_scale(self, ks):
        out = np.ones(ks.shape[1])
        dimc = np.full(ks.shape[1], self.ndim)
        for d in range(3):
            if self.mask[d]:
                nz = ks[d] != 0.0
                out = np.where(nz, out * ks[d], out)
                dimc = np.where(nz, dimc, dimc - 1)
        return np.where(dimc != 0, out ** (1.0 / float(self.ndim)), 0.0)

    def _density(self, counts, act, ks, check_negative=False):
        dens = np.zeros(tuple(self.nbins))
        for n in range(act.shape[0]):
            s = ks[:, n]
            if check_negative and np.any(s < 0.0):
                continue
            gid = act[n]
            gsl, k = self._kernel_span(self._w_kernel(s), gid)
            dens[gsl] = dens[gsl] + counts[gid[0] - 1, gid[1] - 1, gid[2] - 1] * k
        return dens / self.bin_volume

    def _w_kernel(self, smoothing):
        """The W kernel (range 3) of a bin's smoothing: the database entry, or
        set up from the exact values (inactive dimensions have no extent)."""
        if self.database:
            return self._w_db(self._w_indexes(smoothing))
        return w_matrix(np.asarray(smoothing, np.float64), self.bin_size, self.ndim, 3)

    def _sd_kernel(self, axis, h):
        if self.database:
            return self._sd_db(axis, self._log_index(h, axis))
        inp = np.zeros(3)
        inp[axis] = h
        return sd_matrix(axis, inp, self.bin_size, self.ndim, 4)

    def _sigma_gather(self, field, gid, scale):
        gsl, k = self._kernel_span(self._w_kernel(np.full(3, scale)), gid)
        return float((field[gsl] * k).sum())

    def _optimize(self, counts, act, init, npts):
        nb = act.shape[0]
        raw = np.array([counts[g[0] - 1, g[1] - 1, g[2] - 1] for g in act]) / self.bin_volume
        ks = np.repeat(init[:, None], nb, axis=1)
        scale = self._smoothing_scale(ks)
        support = 2.0 * scale
        shape = np.zeros((3, nb))
        for d in range(3):
            if self.mask[d]:
                shape[d] = np.where(scale > 0.0, ks[d] / scale, shape[d])
            else:
                ks[d] = 0.0
        scale_old = scale.copy()
        dens = self._density(counts, act, ks, check_negative=True)
        darr = np.array([dens[g[0] - 1, g[1] - 1, g[2] - 1] for g in act])
        nest = np.zeros(nb)
        netr = np.zeros(nb)
        nd = float(self.ndim)
        err = np.where(scale != 0.0, (nest / ((scale ** nd) * (4.0 * PI) ** (0.5 * nd))
                                      + 0.25 * netr * scale ** 4.0) / (float(npts) ** 2.0), 0.0)
        almise = math.sqrt(float((err ** 2.0).sum()) / nb)
        cum = almise
        almise_old, cum_old = almise, cum
        darr_old = darr.copy()
        loops = 0
        self.work = 0
        for m in range(1, self.n_opt_loops + 1):
            loops = m
            for n in range(nb):
                gid = act[n]
                dn = dens[gid[0] - 1, gid[1] - 1, gid[2] - 1]
                ssc = support[n]
                kscale = scale[n]
                ne = self._sigma_gather(dens, gid, ssc)
                ssc = ne ** 0.5 * kscale ** self.one_plus_nd_quarter / ((4.0 * dn) ** 0.25) * self.support_c
                if ssc > self.max_sigma_growth * support[n]:
                    ssc = self.max_sigma_growth * support[n]
                ssc = min(ssc, self.max_k[self.max_dim])
                if ssc < self.min_k[self.min_dim]:
                    ssc = self.min_k[self.min_dim]
                ne = self._sigma_gather(dens, gid, ssc)
                nest[n] = ne
                support[n] = ssc
            cb = self._curvature_bandwidth(darr, nest, scale, shape, support)
            rxx, ryy, rzz, netr = self._net_roughness(counts, act, cb, support)
            # the isotropy correction changes netRoughnessArray in place (intent(inout),
            # GridProjectedKDE.F90:5420, 5496-5518): the ALMISE below reads the corrected values
            ks, scale, shape, netr = self._optimal_smoothing(nest, netr, rxx, ryy, rzz)
            self.work += self._loop_work(ks, support, cb)
            dens = self._density(counts, act, ks)
            darr = np.array([dens[g[0] - 1, g[1] - 1, g[2] - 1] for g in act])
            e = np.where(darr_old != 0.0, np.abs(darr / darr.max() - darr_old / darr_old.max())
                         / (darr_old / darr_old.max()), 0.0)
            err_dens = math.sqrt(float((e ** 2.0).sum()) / nb)
            e = np.where(scale_old != 0.0, np.abs(scale - scale_old) / scale_old, 0.0)
            err_smooth = math.sqrt(float((e ** 2.0).sum()) / nb)
            e = np.where(scale != 0.0, (nest / ((scale ** nd) * (4.0 * PI) ** (0.5 * nd))
                                        + 0.25 * netr * scale ** 4.0) / (float(npts) ** 2.0), 0.0)
            almise = math.sqrt(float((e ** 2.0).sum()) / nb)
            cum = cum + almise
            if not self.skip_error:
                if almise_old > 0.0 and abs(almise - almise_old) / almise_old < self.rel_err:
                    break
                if err_dens < self.rel_err:
                    break
                if err_smooth < self.rel_err:
                    break
                if m > 7 and abs(cum_old / (m - 1) - cum / m) / cum_old / (m - 1) < self.rel_err:
                    break
            almise_old, cum_old = almise, cum
            darr_old = darr.copy()
            scale_old = scale.copy()
        self.loops = loops
        return dens, ks

    def _loop_work(self, ks, support, cb):
        """The work model of one loop: per active bin the cells of its W kernel,
        eight smoothing-kernel gathers and the second-derivative kernel of each
        active axis, at the database kernels this loop used."""
        w = 0
        for n in range(ks.shape[1]):
            kw = np.prod(2 * np.asarray(self._w_kernel(ks[:, n])[1]) + 1)
            ksg = np.prod(2 * np.asarray(self._w_kernel(np.full(3, support[n]))[1]) + 1)
            ksd = 0
            for a in self.dims:
                h = cb[a, n]
                if h != h:
                    continue
                ksd += np.prod(2 * np.asarray(self._sd_kernel(a, h)[1]) + 1)
            w += int(kw) + 8 * int(ksg) + int(ksd)
        return w

    def _curvature_bandwidth(self, darr, nest, scale, shape, support):
        nb = darr.shape[0]
        nvpb = np.zeros(nb)
        pos = darr > 0.0
        p = (SQRT8PI * support[pos]) ** self.ndim
        nvpb[pos] = (p * nest[pos] ** 2.0 / darr[pos]) ** self.beta_c
        cb = np.zeros((3, nb))
        for d in range(3):
            if not self.mask[d]:
                continue
            nums = np.ones(3)
            nums[d] = 5.0
            tsum = np.zeros(nb)
            for k in range(3):
                if self.mask[k]:
                    nz = shape[k] != 0.0
                    tsum = np.where(nz, tsum + nums[k] / (shape[k] ** 2), tsum)
            nz = shape[d] != 0.0
            term = np.where(nz, ((self.one_over_nd4 / np.where(nz, shape[d], 1.0) ** 4.0) * tsum)
                            ** self.minus_one_over_nd6, 0.0)
            cb[d] = self.alpha_c * nvpb * term * scale
            cb[d] = np.where(cb[d] > self.max_sd[d], self.max_sd[d], cb[d])
            cb[d] = np.where(cb[d] < self.min_sd[d], self.min_sd[d], cb[d])
        return cb

    def _net_roughness(self, counts, act, cb, support):
        """prComputeNetRoughness1D/2D/3D (GridProjectedKDE.F90:1666-1904,
        1905-2289, 2295-2709), local (not global) smoothing."""
        nb = act.shape[0]
        curv = {}
        axes = self.dims if self.ndim != 3 else [0, 1, 2]
        for d in axes:
            c = np.zeros(tuple(self.nbins))
            for n in range(nb):
                h = cb[d, n]
                if self.ndim == 1 and (h < 0.0 or h != h):
                    continue
                # 2-D: a bin with any negative or NaN bandwidth adds to neither curvature (:1967-1968)
                if self.ndim == 2 and (np.any(cb[:, n] < 0.0) or np.any(cb[:, n] != cb[:, n])):
                    continue
                gid = act[n]
                gsl, k = self._kernel_span(self._sd_kernel(d, h), gid)
                c[gsl] = c[gsl] + counts[gid[0] - 1, gid[1] - 1, gid[2] - 1] * k
            c = c / self.bin_volume
            c = c / (self.bin_size[d] ** 2.0)
            curv[d] = c
        rxx = np.zeros(nb); ryy = np.zeros(nb); rzz = np.zeros(nb); net = np.zeros(nb)
        r = {0: rxx, 1: ryy, 2: rzz}
        if self.ndim == 1:
            d = self.dims[0]
            c2 = curv[d] * curv[d]
            for n in range(nb):
                r[d][n] = self._sigma_gather(c2, act[n], support[n])
            net[:] = r[d]
            return rxx, ryy, rzz, net
        if self.ndim == 2:
            # the 2-D form multiplies the curvatures before squaring them (:2134-2138)
            d1, d2 = self.dims
            c12 = curv[d1] * curv[d2]
            c1, c2 = curv[d1] * curv[d1], curv[d2] * curv[d2]
            for n in range(nb):
                gsl, k = self._kernel_span(self._w_kernel(np.full(3, support[n])), act[n])
                r1 = float((c1[gsl] * k).sum())
                r2 = float((c2[gsl] * k).sum())
                r12 = float((c12[gsl] * k).sum())
                r[d1][n], r[d2][n] = r1, r2
                if self.isotropic:
                    net[n] = 2.0 * r12 + r1 + r2
                else:
                    net[n] = 2.0 * r12 + 2.0 * math.sqrt(r1 * r2)
            return rxx, ryy, rzz, net
        # the 3-D form squares the curvatures, then multiplies the squares (:2463-2468)
        for d in (0, 1, 2):
            curv[d] = curv[d] * curv[d]
        cxy, cxz, cyz = curv[0] * curv[1], curv[0] * curv[2], curv[1] * curv[2]
        for n in range(nb):
            gid = act[n]
            gsl, k = self._kernel_span(self._w_kernel(np.full(3, support[n])), gid)
            rxx[n] = float((curv[0][gsl] * k).sum())
            ryy[n] = float((curv[1][gsl] * k).sum())
            rzz[n] = float((curv[2][gsl] * k).sum())
            rxy = float((cxy[gsl] * k).sum())
            rxz = float((cxz[gsl] * k).sum())
            ryz = float((cyz[gsl] * k).sum())
            if self.isotropic:
                # :2675-2676
                net[n] = rxx[n] + 2.0 * rxy + 2.0 * rxz + ryy[n] + 2.0 * ryz + rzz[n]
                continue
            v = 3.0 * (rxx[n] * ryy[n] * rzz[n]) ** (1.0 / 3.0)
            if ryz > 0.0:
                v = v + 2.0 * ryz * (rxx[n] ** 2.0 / ryy[n] / rzz[n]) ** (1.0 / 6.0)
            if rxz > 0.0:
                v = v + 2.0 * rxz * (ryy[n] ** 2.0 / rxx[n] / rzz[n]) ** (1.0 / 6.0)
            if rxy > 0.0:
                v = v + 2.0 * rxy * (rzz[n] ** 2.0 / rxx[n] / ryy[n]) ** (1.0 / 6.0)
            net[n] = v
        return rxx, ryy, rzz, net

    def _optimal_smoothing(self, nest, netr, rxx, ryy, rzz):
        nb = nest.shape[0]
        nd = float(self.ndim)
        if netr.max() == 0.0:
            raise RuntimeError("net roughness is zero everywhere")
        netr = netr.copy()
        r = {0: rxx, 1: ryy, 2: rzz}
        if self.ndim == 2 and not self.isotropic:
            # :5476-5500
            r1, r2 = r[self.dims[0]], r[self.dims[1]]
            sm = r1 + r2
            sm = np.where(sm == 0.0, netr[netr > 0.0].min(), sm)
            iso = (r1 / sm > self.iso_threshold) | (r2 / sm > self.iso_threshold)
            netr = np.where(iso, (1.0 - 0.5) * netr + 0.5 * sm, netr)
        if self.ndim == 3 and not self.isotropic:
            sm = rxx + ryy + rzz
            sm = np.where(sm == 0.0, netr[netr > 0.0].min(), sm)
            iso = (rxx / sm > self.iso_threshold) | (ryy / sm > self.iso_threshold) | (rzz / sm > self.iso_threshold)
            netr = np.where(iso, (1.0 - 0.5) * netr + 0.5 * sm, netr)
        scale = np.zeros(nb)
        pos = netr > 0.0
        scale[pos] = (nd * nest[pos] / ((4.0 * PI) ** (0.5 * nd) * netr[pos])) ** self.one_over_nd4
        zero = netr == 0.0
        if zero.any():
            scale[zero] = scale[scale > 0.0].max()
        shape = np.ones((3, nb))
        if self.ndim == 2 and not self.isotropic:
            # bounded kernels (:5557-5578)
            d1, d2 = self.dims
            r1, r2 = r[d1], r[d2]
            for n in range(nb):
                if r1[n] == 0.0 or r2[n] == 0.0:
                    continue
                s1 = max((netr[n] / r1[n]) ** (1.0 / 8.0), self.min_k[d1] / scale[n])
                s2 = 1.0 / s1
                ns = math.sqrt(s1 * s2)
                if ns == 0.0:
                    continue
                shape[d1, n], shape[d2, n] = s1 / ns, s2 / ns
        if self.ndim == 3 and not self.isotropic:
            for n in range(nb):
                if rxx[n] == 0.0 or ryy[n] == 0.0 or rzz[n] == 0.0:
                    shape[:, n] = 1.0
                    continue
                s1 = max((netr[n] / rxx[n]) ** (1.0 / 12.0), self.min_k[0] / scale[n])
                s2 = max((netr[n] / ryy[n]) ** (1.0 / 12.0), self.min_k[1] / scale[n])
                s3 = 1.0 / s1 / s2
                ns = (s1 * s2 * s3) ** F32_0333
                if ns == 0.0:
                    shape[:, n] = 1.0
                    continue
                shape[:, n] = (s1 / ns, s2 / ns, s3 / ns)
        ks = np.zeros((3, nb))
        update = False
        for d in range(3):
            if not self.mask[d]:
                continue
            ks[d] = shape[d] * scale
            if np.any(ks[d] > self.max_k[d]):
                update = True
                ks[d] = np.where(ks[d] > self.max_k[d], self.max_k[d], ks[d])
            if np.any(ks[d] < self.min_k[d]):
                update = True
                ks[d] = np.where(ks[d] < self.min_k[d], self.min_k[d], ks[d])
        if update:
            scale = self._smoothing_scale(ks)
        return ks, scale, shape, netr
