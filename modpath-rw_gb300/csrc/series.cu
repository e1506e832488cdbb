// series.cu -- the 1-D GPKDE of observation time series (breakthrough curves).
//
// The observation post-process (MPathRW.F90:1759-2840) reconstructs every
// observation's breakthrough curve from the record times of its particles
// with a one-dimensional GridProjectedKDE whose kernel database is off
// (databaseOptimization = .false.): every bin's kernels are set up from its
// exact smoothing (prSetKernelBrute / prSetKernelSigmaBrute /
// prSetKernelSD1DBrute, GridProjectedKDE.F90:6224-6317) instead of being
// looked up.  The time grid is small (10^2..10^5 bins), so the kernels are
// evaluated on the fly: one warp per active bin computes its taps (erf
// differences for W, the Gaussian-derivative differences for the second
// derivative), folds them at the grid ends exactly as prKernelReflection
// does, and gathers from or scatters into the grid.  Reductions run in one
// block in a fixed order; the host takes the per-loop convergence decision
// from a few scalars, as for the spatial reconstruction.
//
// Host-side scalar arithmetic (bin sizes, grid sizes, the initial smoothing,
// effective masses) is done in double precision on the host from sums and
// order statistics the device computes, in the reference's order of
// operations (Histogram.F90:603-720, GridProjectedKDE.F90:3794-4110).
#include <cub/block/block_reduce.cuh>
#include <cub/block/block_scan.cuh>
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/mprw_gpu.h"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRed = 1024;                   // single-block reductions
// Time grids of at most 2^20 bins: a loop costs up to (active bins) x
// (kernel width) tap evaluations, and kernels may grow to 0.9 of the grid.
constexpr int64_t kMaxSeriesBins = 1 << 20;
constexpr double kBorderFraction = 0.05;     // defaultBorderFraction
constexpr double kDefaultInitialFactor = 2.0;
constexpr double kSqrt2 = 1.4142135623730951;

enum {
  S_SUMX, S_MINX, S_MAXX, S_SUMW, S_SUMW2, S_BAD, S_SUMDX2,
  S_MAXD, S_MAXD_OLD, S_ERRD, S_ERRS, S_ALMISE, S_NETMAX, S_MAXSCALE, S_NA, S_SUMABSW,
  S_COUNT
};

// Constants of one reconstruction (1-D, nd = 1).
struct SerParams {
  int G;             // bins of the grid
  double b;          // bin size (= bin volume = bin distance in 1-D)
  double max_k, min_k, max_sd, min_sd;
  double support_c, alpha_c, beta_c, one_over_nd4, minus_one_over_nd6, one_plus_nd_quarter;
  double sqrt8pi, fourpi_half, max_sigma_growth, npts2;
  double sd_c0;      // 2^(nd - 1/2) * sqrt(pi)
};

struct SerBins {
  int na;
  const int *act;    // 0-based grid index of each active bin, ascending
  double *cnt, *wcnt, *ks, *scale, *scale_old, *support, *nest, *netr, *cb, *darr, *darr_old;
};

// ---------------------------------------------------------------------------
// kernel taps
// ---------------------------------------------------------------------------
// W taps of bandwidth h (range 3): zp(k) = 0.5 (erf((k+1/2)/(hd sqrt2)) -
// erf((k-1/2)/(hd sqrt2))), unfolded to 2m+1 entries and divided by their sum
// (KernelMultiGaussian.f90:549-590, 720-790).
struct WTap {
  int m;
  double hs2;   // hd * sqrt(2)
  double sum;
  __device__ double zp(int k) const { return 0.5 * (erf((k + 0.5) / hs2) - erf((k - 0.5) / hs2)); }
};

// Second-derivative taps of bandwidth h (range 4) along the only dimension:
// zp(k) = c ((k+1/2) e^{-(k+1/2)^2/(2 hd^2)} - (k-1/2) e^{-(k-1/2)^2/(2 hd^2)}),
// c = -1/(2^(1/2) sqrt(pi) hd^3); never rescaled (KernelMultiGaussian.f90:794-887).
struct SdTap {
  int m;
  double hd, c;
  __device__ double zp(int k) const {
    const double a = k + 0.5, d = k - 0.5;
    return c * (a * exp(-1.0 * (a * a) / (2.0 * (hd * hd))) - d * exp(-1.0 * (d * d) / (2.0 * (hd * hd))));
  }
};

// The value at grid position p (1-based) of the unfolded kernel centred on
// g, zero outside [g-m, g+m].
template <typename Tap>
__device__ inline double tap_at(const Tap &t, int p, int g, double norm) {
  const int j = p - g;
  if (j < -t.m || j > t.m) return 0.0;
  const double v = t.zp(j < 0 ? -j : j);
  return norm != 0.0 ? v / norm : v;
}

// prKernelReflection in 1-D: taps below position 1 are added onto 1-p
// (low fold first), then taps above G (including folded ones) onto 2G+1-p.
// Every fold target lies inside the (2m+1) matrix, so the value at q in
// [max(g-m,1), min(g+m,G)] is (w(q) + w(1-q)) + (w(2G+1-q) + w(q-2G)) in the
// reference's order of additions (a missing term is an exact zero).
template <typename Tap>
__device__ inline double folded(const Tap &t, int q, int g, int G, double norm) {
  return (tap_at(t, q, g, norm) + tap_at(t, 1 - q, g, norm)) +
         (tap_at(t, 2 * G + 1 - q, g, norm) + tap_at(t, q - 2 * G, g, norm));
}

struct MinOp {
  __device__ double operator()(double a, double b) const { return fmin(a, b); }
};
struct MaxOp {
  __device__ double operator()(double a, double b) const { return fmax(a, b); }
};

__device__ inline double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// W taps of smoothing h for this warp; sum over the unfolded matrix.
__device__ inline WTap make_w(double h, double b, int lane) {
  WTap t;
  t.m = (int)ceil(3.0 * h / b);
  t.hs2 = (h / b) * kSqrt2;
  double s = 0.0;
  for (int j = -t.m + lane; j <= t.m; j += 32) s += t.zp(j < 0 ? -j : j);
  t.sum = warp_sum(s);
  return t;
}

__device__ inline SdTap make_sd(double h, double b, double c0) {
  SdTap t;
  t.m = (int)ceil(4.0 * h / b);
  t.hd = h / b;
  t.c = -1.0 / (c0 * pow(t.hd, 3.0));
  return t;
}

// sum over the kernel's span of field * folded W taps
__device__ inline double w_gather(const double *field, double h, int g, const SerParams &P, int lane) {
  if (h == 0.0) return 0.0;
  const WTap t = make_w(h, P.b, lane);
  const int q0 = max(g - t.m, 1), q1 = min(g + t.m, P.G);
  double acc = 0.0;
  for (int q = q0 + lane; q <= q1; q += 32) acc += field[q - 1] * folded(t, q, g, P.G, t.sum);
  return warp_sum(acc);
}

// ---------------------------------------------------------------------------
// statistics, histogram, active bins
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kRed) ser_stats_kernel(const double *x, const double *w, int64_t n, double *S) {
  using BR = cub::BlockReduce<double, kRed>;
  __shared__ typename BR::TempStorage tmp;
  double sx = 0.0, mn = INFINITY, mx = -INFINITY, sw = 0.0, sw2 = 0.0, bad = 0.0, swa = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += kRed) {
    const double xi = x[i], wi = w[i];
    if (!isfinite(xi) || !isfinite(wi)) bad += 1.0;
    sx += xi;
    mn = fmin(mn, xi);
    mx = fmax(mx, xi);
    sw += wi;
    sw2 += wi * wi;
    swa += fabs(wi);
  }
  double r;
  r = BR(tmp).Sum(sx);
  if (threadIdx.x == 0) S[S_SUMX] = r;
  __syncthreads();
  r = BR(tmp).Reduce(mn, MinOp());
  if (threadIdx.x == 0) S[S_MINX] = r;
  __syncthreads();
  r = BR(tmp).Reduce(mx, MaxOp());
  if (threadIdx.x == 0) S[S_MAXX] = r;
  __syncthreads();
  r = BR(tmp).Sum(sw);
  if (threadIdx.x == 0) S[S_SUMW] = r;
  __syncthreads();
  r = BR(tmp).Sum(sw2);
  if (threadIdx.x == 0) S[S_SUMW2] = r;
  __syncthreads();
  r = BR(tmp).Sum(bad);
  if (threadIdx.x == 0) S[S_BAD] = r;
  __syncthreads();
  r = BR(tmp).Sum(swa);
  if (threadIdx.x == 0) S[S_SUMABSW] = r;
}

__global__ void __launch_bounds__(kRed) ser_var_kernel(const double *x, int64_t n, double mean, double *S) {
  using BR = cub::BlockReduce<double, kRed>;
  __shared__ typename BR::TempStorage tmp;
  double v = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += kRed) {
    const double d = x[i] - mean;
    v += d * d;
  }
  const double r = BR(tmp).Sum(v);
  if (threadIdx.x == 0) S[S_SUMDX2] = r;
}

// Histogram%ComputeCounts{Weighted,AndWeights} / ComputeEffectiveCountsAndWeights
// (Histogram.F90:276-490): bin = floor((t - origin)/binSize) + 1 (+ 0 for an
// exact point), points outside [1, G] skipped.  The sums are 64-bit
// fixed-point integers (scale 2^shift_c for counts, 2^shift_w for wcounts,
// chosen by the host from the totals so that no sum overflows): integer
// additions do not depend on the order of the atomics, so the histogram is
// bit-for-bit repeatable; ser_fixed_kernel turns them into doubles.
__global__ void ser_hist_kernel(const double *x, const double *w, int64_t n, double origin, double b, int G,
                                int exact, int fmt, double sc, double sw, unsigned long long *counts,
                                unsigned long long *wcounts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double q = floor((x[i] - origin) / b) + (exact ? 0.0 : 1.0);
    if (!(q >= 1.0 && q <= (double)G)) continue;
    const int k = (int)q - 1;
    const double wi = w[i];
    const double c = fmt == 2 ? 1.0 : (fmt == 3 ? wi * wi : wi);
    atomicAdd(counts + k, (unsigned long long)__double2ll_rn(c * sc));
    if (fmt >= 2) atomicAdd(wcounts + k, (unsigned long long)__double2ll_rn(wi * sw));
  }
}

__global__ void ser_fixed_kernel(const unsigned long long *a, double inv, double *out, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = (double)(long long)a[i] * inv;
}

// mode 0: a /= f; mode 1: a *= f; mode 2: format 3's effective counts
// (counts = wcounts^2 / counts where counts != 0)
__global__ void ser_grid_op_kernel(double *a, const double *bw, int G, int mode, double f) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < G; i += gridDim.x * blockDim.x) {
    if (mode == 0) a[i] = a[i] / f;
    else if (mode == 1) a[i] = a[i] * f;
    else if (a[i] != 0.0) a[i] = bw[i] * bw[i] / a[i];
  }
}

// active bins (counts != 0) in ascending order (Histogram.F90:493-527)
__global__ void __launch_bounds__(kRed) ser_active_kernel(const double *counts, const double *wcounts, int G,
                                                          int *act, double *cnt, double *wcnt, double *S) {
  using BS = cub::BlockScan<int, kRed>;
  __shared__ typename BS::TempStorage tmp;
  __shared__ int base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  for (int c0 = 0; c0 < G; c0 += kRed) {
    const int i = c0 + threadIdx.x;
    const int flag = (i < G && counts[i] != 0.0) ? 1 : 0;
    int ofs, total;
    BS(tmp).ExclusiveSum(flag, ofs, total);
    if (flag) {
      const int k = base + ofs;
      act[k] = i;
      cnt[k] = counts[i];
      wcnt[k] = wcounts ? wcounts[i] : 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) S[S_NA] = (double)base;
}

// ---------------------------------------------------------------------------
// the optimisation loop (GridProjectedKDE.F90:4396-5160, nd = 1)
// ---------------------------------------------------------------------------
// kernelSmoothing = initial smoothing; scale = its geometric mean (itself in
// 1-D, zero for a zero smoothing); support = 2 scale; shape = 1.
__global__ void ser_init_kernel(SerBins B, double hs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B.na) return;
  B.ks[i] = hs;
  const double sc = (hs != 0.0) ? pow(hs, 1.0) : 0.0;
  B.scale[i] = sc;
  B.scale_old[i] = sc;
  B.support[i] = 2.0 * sc;
  B.nest[i] = 0.0;
  B.netr[i] = 0.0;
}

// density: the sum of (w)counts times the folded W taps of kernelSmoothing
// (check_negative skips a negative smoothing, the first estimate, :4640).
// The reference scatters bin by bin in ascending order; here each grid
// position gathers the bins whose folded kernel reaches it, in the same
// ascending order, so the sums are the reference's and repeatable.  First the
// taps of every bin (one warp per bin; m = -1 for a bin that adds nothing)
// and the largest half-width, then the gather.
__global__ void __launch_bounds__(kThreads) ser_wtap_kernel(SerParams P, SerBins B, int check_negative, WTap *taps,
                                                            int *mmax) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * kWarps + (threadIdx.x >> 5);
  if (i >= B.na) return;
  const double h = B.ks[i];
  if ((check_negative && h < 0.0) || h == 0.0) {
    if (lane == 0) taps[i].m = -1;
    return;
  }
  const WTap t = make_w(h, P.b, lane);
  if (lane == 0) {
    taps[i] = t;
    atomicMax(mmax, t.m);
  }
}

// the first active bin index whose grid position (1-based) is >= g
__device__ inline int first_bin_at(const SerBins &B, int g) {
  int lo = 0, hi = B.na;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (B.act[mid] + 1 < g) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// out[q-1] = sum over the bins i reaching q of val[i] * folded taps: one warp
// per grid position, lane l taking the candidate bins l, l+32, ... in
// ascending order, then a fixed shuffle tree -- a fixed order, so the sum is
// the same on every run.
template <typename Tap, bool NORM>
__global__ void __launch_bounds__(kThreads) ser_gather_kernel(SerParams P, SerBins B, const Tap *taps,
                                                              const int *mmax, const double *val, double *out) {
  const int M = *mmax;
  const int lane = threadIdx.x & 31;
  const int q = blockIdx.x * kWarps + (threadIdx.x >> 5) + 1;
  if (q > P.G) return;  // warp-uniform
  double acc = 0.0;
  if (M >= 0) {
    for (int i = first_bin_at(B, q - M) + lane; i < B.na && B.act[i] + 1 <= q + M; i += 32) {
      const Tap t = taps[i];
      const int g = B.act[i] + 1;
      if (t.m < 0 || q < g - t.m || q > g + t.m) continue;
      double norm = 0.0;
      if constexpr (NORM) norm = t.sum;
      acc += val[i] * folded(t, q, g, P.G, norm);
    }
  }
  acc = warp_sum(acc);
  if (lane == 0) out[q - 1] = acc;
}

// nEstimate with the current support, the support update, nEstimate again
// (GridProjectedKDE.F90:4826-4880)
__global__ void __launch_bounds__(kThreads) ser_nest_kernel(SerParams P, SerBins B, const double *dens) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * kWarps + (threadIdx.x >> 5);
  if (i >= B.na) return;
  const int g = B.act[i] + 1;
  const double dn = dens[g - 1];
  double ssc = B.support[i];
  const double kscale = B.scale[i];
  double ne = w_gather(dens, ssc, g, P, lane);
  ssc = pow(ne, 0.5) * pow(kscale, P.one_plus_nd_quarter) / pow(4.0 * dn, 0.25) * P.support_c;
  if (ssc > P.max_sigma_growth * B.support[i]) ssc = P.max_sigma_growth * B.support[i];
  ssc = fmin(ssc, P.max_k);
  if (ssc < P.min_k) ssc = P.min_k;
  ne = w_gather(dens, ssc, g, P, lane);
  if (lane == 0) {
    B.nest[i] = ne;
    B.support[i] = ssc;
  }
}

// curvature bandwidth (GridProjectedKDE.F90:5207-5275), shape = 1
__global__ void ser_cb_kernel(SerParams P, SerBins B) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B.na) return;
  const double d = B.darr[i];
  double nvpb = 0.0;
  if (d > 0.0) {
    const double p = pow(P.sqrt8pi * B.support[i], 1.0);
    nvpb = pow(p * (B.nest[i] * B.nest[i]) / d, P.beta_c);
  }
  const double shape = 1.0;
  const double tsum = 0.0 + 5.0 / (shape * shape);
  const double term = pow((P.one_over_nd4 / pow(shape, 4.0)) * tsum, P.minus_one_over_nd6);
  double cb = P.alpha_c * nvpb * term * B.scale[i];
  if (cb > P.max_sd) cb = P.max_sd;
  if (cb < P.min_sd) cb = P.min_sd;
  B.cb[i] = cb;
}

// curvature: the sum of counts times the second-derivative taps of the
// curvature bandwidth (prComputeNetRoughness1D, GridProjectedKDE.F90:1666-1760),
// as a gather like the density: the taps of every bin (m = -1 where the
// reference skips the bin: a negative, NaN or zero bandwidth, or a kernel
// whose sum of squares is zero), then ser_gather_kernel<SdTap, false>.
__global__ void __launch_bounds__(kThreads) ser_sdtap_kernel(SerParams P, SerBins B, SdTap *taps, int *mmax) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * kWarps + (threadIdx.x >> 5);
  if (i >= B.na) return;
  const double h = B.cb[i];
  if (h < 0.0 || h != h || h == 0.0) {
    if (lane == 0) taps[i].m = -1;
    return;
  }
  const SdTap t = make_sd(h, P.b, P.sd_c0);
  double s = 0.0;  // the sum of squares decides a zero kernel
  for (int j = -t.m + lane; j <= t.m; j += 32) {
    const double v = t.zp(j < 0 ? -j : j);
    s += v * v;
  }
  const double ss = warp_sum(s);
  if (lane == 0) {
    if (ss <= 0.0) {
      taps[i].m = -1;
    } else {
      taps[i] = t;
      atomicMax(mmax, t.m);
    }
  }
}

// curvature / binVolume / binSize^2, squared
__global__ void ser_curv_square_kernel(double *curv, int G, double b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < G; i += gridDim.x * blockDim.x) {
    double c = curv[i] / b;
    c = c / (b * b);
    curv[i] = c * c;
  }
}

// roughness: W gather of the squared curvature with the support; the raw
// optimal scale where the roughness is positive (GridProjectedKDE.F90:5404-5440)
__global__ void __launch_bounds__(kThreads) ser_rough_kernel(SerParams P, SerBins B, const double *curv) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * kWarps + (threadIdx.x >> 5);
  if (i >= B.na) return;
  const int g = B.act[i] + 1;
  const double r = w_gather(curv, B.support[i], g, P, lane);
  if (lane == 0) {
    B.netr[i] = r;
    B.scale[i] = (r > 0.0) ? pow(1.0 * B.nest[i] / (P.fourpi_half * r), P.one_over_nd4) : 0.0;
  }
}

// max net roughness and max positive scale
__global__ void __launch_bounds__(kRed) ser_rough_reduce_kernel(SerBins B, double *S) {
  using BR = cub::BlockReduce<double, kRed>;
  __shared__ typename BR::TempStorage tmp;
  double mr = -INFINITY, ms = 0.0;
  for (int i = threadIdx.x; i < B.na; i += kRed) {
    mr = fmax(mr, B.netr[i]);
    if (B.scale[i] > 0.0) ms = fmax(ms, B.scale[i]);
  }
  double r = BR(tmp).Reduce(mr, MaxOp());
  if (threadIdx.x == 0) S[S_NETMAX] = r;
  __syncthreads();
  r = BR(tmp).Reduce(ms, MaxOp());
  if (threadIdx.x == 0) S[S_MAXSCALE] = r;
}

// zero roughness takes the largest scale; kernelSmoothing = scale bounded to
// [minKernelSize, maxKernelSize]; the scale of a 1-D kernel is the kernel
// itself (GridProjectedKDE.F90:5440-5724)
__global__ void ser_optimal_kernel(SerParams P, SerBins B, const double *S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B.na) return;
  double sc = B.scale[i];
  if (B.netr[i] == 0.0) sc = S[S_MAXSCALE];
  double k = 1.0 * sc;
  if (k > P.max_k) k = P.max_k;
  if (k < P.min_k) k = P.min_k;
  B.ks[i] = k;
  B.scale[i] = (k != 0.0) ? pow(k, 1.0) : 0.0;
}

// previous density and scale (saved at the start of each loop)
__global__ void ser_loop_init_kernel(SerBins B, double *S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) S[S_MAXD_OLD] = S[S_MAXD];
  if (i >= B.na) return;
  B.darr_old[i] = B.darr[i];
  B.scale_old[i] = B.scale[i];
}

// density grid / binVolume; density at the active bins; the convergence
// measures (GridProjectedKDE.F90:4960-5040)
__global__ void ser_dens_finish_kernel(double *dens, int G, double b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < G; i += gridDim.x * blockDim.x) dens[i] = dens[i] / b;
}

__global__ void __launch_bounds__(kRed) ser_measures_kernel(SerParams P, SerBins B, const double *dens, double *S) {
  using BR = cub::BlockReduce<double, kRed>;
  __shared__ typename BR::TempStorage tmp;
  __shared__ double smax;
  double mx = -INFINITY;
  for (int i = threadIdx.x; i < B.na; i += kRed) {
    const double d = dens[B.act[i]];
    B.darr[i] = d;
    mx = fmax(mx, d);
  }
  const double r = BR(tmp).Reduce(mx, MaxOp());
  if (threadIdx.x == 0) {
    smax = r;
    S[S_MAXD] = r;
  }
  __syncthreads();
  const double mo = S[S_MAXD_OLD];
  double ed = 0.0, es = 0.0, ea = 0.0;
  for (int i = threadIdx.x; i < B.na; i += kRed) {
    const double d = B.darr[i], o = B.darr_old[i];
    if (o != 0.0) {
      const double e = fabs(d / smax - o / mo) / (o / mo);
      ed += e * e;
    }
    const double sc = B.scale[i], so = B.scale_old[i];
    if (so != 0.0) {
      const double e = fabs(sc - so) / so;
      es += e * e;
    }
    if (sc != 0.0) {
      const double e = (B.nest[i] / (pow(sc, 1.0) * P.fourpi_half) + 0.25 * B.netr[i] * pow(sc, 4.0)) / P.npts2;
      ea += e * e;
    }
  }
  double v = BR(tmp).Sum(ed);
  if (threadIdx.x == 0) S[S_ERRD] = v;
  __syncthreads();
  v = BR(tmp).Sum(es);
  if (threadIdx.x == 0) S[S_ERRS] = v;
  __syncthreads();
  v = BR(tmp).Sum(ea);
  if (threadIdx.x == 0) S[S_ALMISE] = v;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct DevMem {
  std::vector<void *> ptrs;
  ~DevMem() {
    for (void *p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T **p, int64_t n) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * (size_t)std::max<int64_t>(n, 1));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

int rc_of(cudaError_t e) { return e == cudaErrorMemoryAllocation ? MPRW_E_OOM : MPRW_E_CUDA; }

#define SCK(x)                          \
  do {                                  \
    cudaError_t e_ = (x);               \
    if (e_ != cudaSuccess) {            \
      (void)cudaGetLastError();         \
      return rc_of(e_);                 \
    }                                   \
  } while (0)

int blocks_of(int64_t n, int threads) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 16));
}

// Q1 and Q3 as prEstimateBinSizeFD picks them from the sorted points
// (Histogram.F90:680-712); `at` reads the 1-based element i.
template <typename F>
cudaError_t fd_quartiles(int64_t n, F at, double *q1, double *q3) {
  double a = 0, b = 0, c = 0, d = 0;
  cudaError_t e = cudaSuccess;
  if (n % 2 == 0) {
    if (std::fmod((double)n / 2.0, 2.0) == 0.0) {
      if ((e = at(n / 4, &a)) || (e = at(n / 4 + 1, &b)) || (e = at(n / 2 + n / 4, &c)) ||
          (e = at(n / 2 + n / 4 + 1, &d)))
        return e;
      *q1 = (a + b) / 2.0;
      *q3 = (c + d) / 2.0;
    } else {
      if ((e = at(n / 4 + 1, &a)) || (e = at(n / 2 + n / 4 + 1, &c))) return e;
      *q1 = a;
      *q3 = c;
    }
  } else {
    if (std::fmod((double)(n - 1) / 2.0, 2.0) == 0.0) {
      if ((e = at((n - 1) / 4, &a)) || (e = at((n - 1) / 4 + 1, &b)) || (e = at(n / 2 + 1 + (n - 1) / 4, &c)) ||
          (e = at(n / 2 + 1 + (n - 1) / 4 + 1, &d)))
        return e;
      *q1 = (a + b) / 2.0;
      *q3 = (c + d) / 2.0;
    } else {
      if ((e = at((n - 1) / 4 + 1, &a)) || (e = at(n / 2 + 1 + (n - 1) / 4 + 1, &c))) return e;
      *q1 = a;
      *q3 = c;
    }
  }
  return cudaSuccess;
}

}  // namespace

extern "C" int mprw_gpkde_series(const double *times, const double *weights, int64_t n,
                                 const mprw_series_options *o, int32_t capacity, double *counts_out,
                                 double *wcounts_out, double *density_out, mprw_series_result *res, void *stream) {
  if (!times || !weights || !o || !res || !counts_out || n < 1 || n > (int64_t)INT32_MAX) return MPRW_E_INVAL;
  *res = mprw_series_result{};
  const int fmt = o->effective_weight_format;
  if (o->bin_format < 0 || o->bin_format > 3 || fmt < 0 || fmt > 3 || o->initial_smoothing_selection < 0 ||
      o->initial_smoothing_selection > 2 || o->n_opt_loops < 0 || !std::isfinite(o->rel_err_convergence) ||
      !std::isfinite(o->origin) || !std::isfinite(o->domain_size) || !std::isfinite(o->bin_size) ||
      !std::isfinite(o->initial_smoothing_factor) || o->domain_size < 0.0 || (!o->adapt_grid && o->domain_size <= 0.0))
    return MPRW_E_INVAL;
  if (o->bin_format <= 1 && !(o->bin_size_fraction > 0.0 && o->bin_size_fraction <= 2.0)) return MPRW_E_INVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DevMem mem;
  double *dx, *dw, *S;
  SCK(mem.alloc(&dx, n));
  SCK(mem.alloc(&dw, n));
  SCK(mem.alloc(&S, S_COUNT));
  SCK(cudaMemcpyAsync(dx, times, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(dw, weights, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  SCK(cudaMemsetAsync(S, 0, sizeof(double) * S_COUNT, s));
  double h[S_COUNT];
  auto fetch = [&](void) -> cudaError_t {
    cudaError_t e = cudaMemcpyAsync(h, S, sizeof(h), cudaMemcpyDeviceToHost, s);
    return e != cudaSuccess ? e : cudaStreamSynchronize(s);
  };
  ser_stats_kernel<<<1, kRed, 0, s>>>(dx, dw, n, S);
  SCK(cudaGetLastError());
  SCK(fetch());
  if (h[S_BAD] != 0.0) return MPRW_E_INVAL;
  const double nd_n = (double)n;
  const double mean = h[S_SUMX] / nd_n;
  ser_var_kernel<<<1, kRed, 0, s>>>(dx, n, mean, S);
  SCK(cudaGetLastError());
  SCK(fetch());
  const double var = h[S_SUMDX2] / nd_n;
  const double mn = h[S_MINX], mx = h[S_MAXX], delta = std::fabs(mx - mn);
  const double origin = o->origin;
  // domain adapted to the data (GridProjectedKDE.F90:3794-3800)
  double ds = o->domain_size;
  if (o->adapt_grid && ds == 0.0 && delta != 0.0) ds = (mx + 1.0 * kBorderFraction * delta) - origin;
  // bin size (Histogram.F90:603-720; GridProjectedKDE.F90:3806-3890)
  double b = o->bin_size;
  if (o->bin_format == 0) {
    b = (var == 0.0) ? 0.0 : (double)3.49f * std::sqrt(var) / std::pow(nd_n, 1.0 / 3.0);
    b = o->bin_size_fraction * b;
  } else if (o->bin_format == 1) {
    if (n < 2) return MPRW_E_INVAL;
    double *sorted;
    SCK(mem.alloc(&sorted, n));
    size_t tb = 0;
    SCK(cub::DeviceRadixSort::SortKeys(nullptr, tb, dx, sorted, (int)n, 0, 64, s));
    void *tmp;
    SCK(mem.alloc(reinterpret_cast<char **>(&tmp), (int64_t)tb));
    SCK(cub::DeviceRadixSort::SortKeys(tmp, tb, dx, sorted, (int)n, 0, 64, s));
    auto at = [&](int64_t i, double *v) -> cudaError_t {
      cudaError_t e = cudaMemcpyAsync(v, sorted + (i - 1), sizeof(double), cudaMemcpyDeviceToHost, s);
      return e != cudaSuccess ? e : cudaStreamSynchronize(s);
    };
    double q1 = 0.0, q3 = 0.0;
    SCK(fd_quartiles(n, at, &q1, &q3));
    b = 2.0 * (q3 - q1) / std::pow(nd_n, 1.0 / 3.0);
    b = o->bin_size_fraction * b;
  }
  if (!(b > 0.0) || !std::isfinite(b) || ds == 0.0) return MPRW_E_INVAL;
  const double gsd = ds / b + 0.5;
  if (!(gsd < (double)kMaxSeriesBins)) return MPRW_E_INVAL;
  const int gs = (int)gsd;
  if (gs < 2) return MPRW_E_INVAL;
  // the grid: a sub-grid around the data when adapted (:3903-3960)
  int nb = gs, dbo = 0;
  double gorigin = origin;
  if (o->adapt_grid) {
    const double lo = std::max(mn - 0.5 * kBorderFraction * delta, origin);
    const double hi = std::min(mx + 0.5 * kBorderFraction * delta, ds + origin);
    const double od = (lo - origin) / b, ld = std::ceil((hi - origin) / b);
    if (!(od < (double)kMaxSeriesBins) || !(ld < (double)kMaxSeriesBins)) return MPRW_E_INVAL;
    dbo = (int)od;
    nb = (int)ld - dbo;
    gorigin = dbo * b + origin;
    if (nb > gs || nb < 1) return MPRW_E_INVAL;
  }
  res->n_bins = nb;
  res->delta_bins_origin = dbo;
  res->bin_size = b;
  res->grid_origin = gorigin;
  if (nb > capacity) return MPRW_E_SIZE;

  // weighted histogram (Histogram.F90:276-490), fixed-point sums: a bin's
  // sum is at most the total over all records (weights are >= 0), and
  // 2^shift times that stays below 2^62
  const bool wfmt = (fmt >= 2);
  double *counts, *wcounts = nullptr;
  SCK(mem.alloc(&counts, nb));
  if (wfmt) SCK(mem.alloc(&wcounts, nb));
  unsigned long long *fc, *fw = nullptr;
  SCK(mem.alloc(&fc, nb));
  SCK(cudaMemsetAsync(fc, 0, sizeof(unsigned long long) * nb, s));
  if (wfmt) {
    SCK(mem.alloc(&fw, nb));
    SCK(cudaMemsetAsync(fw, 0, sizeof(unsigned long long) * nb, s));
  }
  auto shift_for = [](double bound) {
    int e = 0;
    std::frexp(std::max(bound, 1e-300), &e);
    return 61 - e;
  };
  {
    // totals of the statistics pass (with a margin for their rounding)
    const double tw = 1.0001 * h[S_SUMABSW], tw2 = 1.0001 * h[S_SUMW2];
    const double cb = fmt == 2 ? (double)n : (fmt == 3 ? tw2 : tw);
    const int shc = shift_for(cb), shw = shift_for(tw);
    ser_hist_kernel<<<blocks_of(n, kThreads), kThreads, 0, s>>>(dx, dw, n, gorigin, b, nb, o->exact_point ? 1 : 0,
                                                                 fmt, std::ldexp(1.0, shc), std::ldexp(1.0, shw), fc,
                                                                 fw);
    ser_fixed_kernel<<<blocks_of(nb, kThreads), kThreads, 0, s>>>(fc, std::ldexp(1.0, -shc), counts, nb);
    if (wfmt) ser_fixed_kernel<<<blocks_of(nb, kThreads), kThreads, 0, s>>>(fw, std::ldexp(1.0, -shw), wcounts, nb);
  }
  double eff = 1.0;
  if (!wfmt) {
    const double total = h[S_SUMW];
    if (fmt == 1) {
      eff = total / nd_n;
    } else {
      const double neff = total * total / h[S_SUMW2];
      eff = total / neff;
    }
    ser_grid_op_kernel<<<blocks_of(nb, kThreads), kThreads, 0, s>>>(counts, nullptr, nb, 0, eff);
  } else if (fmt == 3) {
    ser_grid_op_kernel<<<blocks_of(nb, kThreads), kThreads, 0, s>>>(counts, wcounts, nb, 2, 0.0);
  }
  SCK(cudaGetLastError());
  auto scale_grid = [&](double *a, int mode, double f) {
    ser_grid_op_kernel<<<blocks_of(nb, kThreads), kThreads, 0, s>>>(a, nullptr, nb, mode, f);
  };
  auto copy_out = [&](double *dens) -> cudaError_t {
    cudaError_t e = cudaMemcpyAsync(counts_out, counts, sizeof(double) * nb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && wcounts_out) {
      e = wfmt ? cudaMemcpyAsync(wcounts_out, wcounts, sizeof(double) * nb, cudaMemcpyDeviceToHost, s)
               : cudaSuccess;
      if (!wfmt) std::fill(wcounts_out, wcounts_out + nb, 0.0);
    }
    if (e == cudaSuccess && density_out) {
      if (dens) e = cudaMemcpyAsync(density_out, dens, sizeof(double) * nb, cudaMemcpyDeviceToHost, s);
      else std::fill(density_out, density_out + nb, 0.0);
    }
    return e != cudaSuccess ? e : cudaStreamSynchronize(s);
  };
  if (o->only_histogram) {
    // counts * effective mass, raw density (GridProjectedKDE.F90:3987-4005)
    scale_grid(counts, 1, eff);
    if (o->compute_raw_density) {
      scale_grid(counts, 0, b);
      if (wfmt) scale_grid(wcounts, 0, b);
    }
    SCK(cudaGetLastError());
    SCK(copy_out(nullptr));
    return MPRW_OK;
  }

  // active bins
  int *act;
  SerBins B{};
  SCK(mem.alloc(&act, nb));
  SCK(mem.alloc(&B.cnt, nb));
  SCK(mem.alloc(&B.wcnt, nb));
  ser_active_kernel<<<1, kRed, 0, s>>>(counts, wcounts, nb, act, B.cnt, B.wcnt, S);
  SCK(cudaGetLastError());
  SCK(fetch());
  const int na = (int)h[S_NA];
  res->active_bins = na;
  if (na == 0) {
    SCK(copy_out(nullptr));
    return MPRW_OK;
  }
  B.na = na;
  B.act = act;
  SCK(mem.alloc(&B.ks, na));
  SCK(mem.alloc(&B.scale, na));
  SCK(mem.alloc(&B.scale_old, na));
  SCK(mem.alloc(&B.support, na));
  SCK(mem.alloc(&B.nest, na));
  SCK(mem.alloc(&B.netr, na));
  SCK(mem.alloc(&B.cb, na));
  SCK(mem.alloc(&B.darr, na));
  SCK(mem.alloc(&B.darr_old, na));
  SCK(cudaMemsetAsync(B.darr_old, 0, sizeof(double) * na, s));
  double *dens, *curv;
  SCK(mem.alloc(&dens, nb));
  SCK(mem.alloc(&curv, nb));
  WTap *wtaps;
  SdTap *sdtaps;
  int *mmax;
  SCK(mem.alloc(&wtaps, na));
  SCK(mem.alloc(&sdtaps, na));
  SCK(mem.alloc(&mmax, 2));

  // data statistics and the initial smoothing (GridProjectedKDE.F90:4020-4110)
  const double std_x = std::sqrt(var);
  double hsig = std_x * std::pow(4.0 / ((1.0 + 2.0) * nd_n), 1.0 / (1.0 + 4.0));
  bool apply = o->apply_initial_factor != 0;
  if (std_x == 0.0) {
    hsig = kDefaultInitialFactor * b;
    apply = false;
  }
  const double fac = o->initial_smoothing_factor;
  double init;
  if (o->initial_smoothing_selection == 0)
    init = (apply && fac > 0.0 && fac != 1.0) ? hsig * fac : hsig;
  else if (o->initial_smoothing_selection == 1)
    init = fac * b;
  else
    init = kDefaultInitialFactor * b;
  // the first support (twice the initial smoothing) is not bounded by the
  // kernel-size limits: refuse one wider than the grid limit
  if (!(init >= 0.0) || !(6.0 * init / b <= (double)kMaxSeriesBins)) return MPRW_E_INVAL;

  // constants of the 1-D reconstruction (prInitializeModuleConstants and
  // the kernel-size bounds of the domain grid, GridProjectedKDE.F90:1296-1310)
  const double nd = 1.0, pi = 4.0 * std::atan(1.0);
  SerParams P{};
  P.G = nb;
  P.b = b;
  P.max_k = b * (0.9 * gs - 1) / 3.0;
  P.max_sd = b * (0.9 * gs - 1) / 4.0;
  P.min_k = 1.2 * b / 3.0;
  P.min_sd = 1.2 * b / 4.0;
  P.support_c = std::pow((nd + 2.0) * std::pow(8.0 * pi, 0.5 * nd), 0.25);
  P.alpha_c = std::pow((1.0 + std::pow(2.0, 0.5 * nd + 2.0)) / (3.0 * std::pow(2.0, 4.0 / (nd + 4.0))),
                       1.0 / (nd + 6.0)) *
              std::pow(nd + 2.0, 1.0 / (nd + 4.0)) / std::pow(nd + 4.0, 1.0 / (nd + 6.0));
  P.beta_c = 2.0 / (nd + 4.0) / (nd + 6.0);
  P.one_over_nd4 = 1.0 / (nd + 4.0);
  P.minus_one_over_nd6 = -1.0 / (nd + 6.0);
  P.one_plus_nd_quarter = 1.0 + 0.25 * nd;
  P.sqrt8pi = std::sqrt(8.0 * pi);
  P.fourpi_half = std::pow(4.0 * pi, 0.5 * nd);
  P.max_sigma_growth = 1.5;
  P.npts2 = std::pow(nd_n, 2.0);
  P.sd_c0 = std::pow(2.0, nd - 0.5) * std::sqrt(4.0 * std::atan(1.0));

  const int eb = blocks_of(na, kThreads);      // one thread per bin
  const int wb = (na + kWarps - 1) / kWarps;   // one warp per bin
  auto density = [&](const double *val, int check_negative) -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(mmax, 0xff, sizeof(int), s);  // -1
    if (e != cudaSuccess) return e;
    ser_wtap_kernel<<<wb, kThreads, 0, s>>>(P, B, check_negative, wtaps, mmax);
    ser_gather_kernel<WTap, true><<<(nb + kWarps - 1) / kWarps, kThreads, 0, s>>>(P, B, wtaps, mmax, val, dens);
    ser_dens_finish_kernel<<<blocks_of(nb, kThreads), kThreads, 0, s>>>(dens, nb, b);
    return cudaGetLastError();
  };
  ser_init_kernel<<<eb, kThreads, 0, s>>>(B, init);
  SCK(density(B.cnt, 1));
  ser_measures_kernel<<<1, kRed, 0, s>>>(P, B, dens, S);
  SCK(cudaGetLastError());
  SCK(fetch());
  double alm = std::sqrt(h[S_ALMISE] / na);
  double alm_old = alm, cum = alm, cum_old = alm;
  const double rel_err = o->rel_err_convergence;
  int m = 0;
  for (m = 1; m <= o->n_opt_loops; ++m) {
    ser_loop_init_kernel<<<eb, kThreads, 0, s>>>(B, S);
    ser_nest_kernel<<<wb, kThreads, 0, s>>>(P, B, dens);
    ser_cb_kernel<<<eb, kThreads, 0, s>>>(P, B);
    SCK(cudaMemsetAsync(mmax + 1, 0xff, sizeof(int), s));
    ser_sdtap_kernel<<<wb, kThreads, 0, s>>>(P, B, sdtaps, mmax + 1);
    ser_gather_kernel<SdTap, false><<<(nb + kWarps - 1) / kWarps, kThreads, 0, s>>>(P, B, sdtaps, mmax + 1, B.cnt,
                                                                                   curv);
    ser_curv_square_kernel<<<blocks_of(nb, kThreads), kThreads, 0, s>>>(curv, nb, b);
    ser_rough_kernel<<<wb, kThreads, 0, s>>>(P, B, curv);
    ser_rough_reduce_kernel<<<1, kRed, 0, s>>>(B, S);
    ser_optimal_kernel<<<eb, kThreads, 0, s>>>(P, B, S);
    SCK(density(B.cnt, 0));
    ser_measures_kernel<<<1, kRed, 0, s>>>(P, B, dens, S);
    SCK(cudaGetLastError());
    SCK(fetch());
    // maxval(netRoughness) == 0: the reference stops (GridProjectedKDE.F90:5443-5446)
    if (h[S_NETMAX] == 0.0) return MPRW_E_INVAL;
    const double err_dens = std::sqrt(h[S_ERRD] / na), err_smooth = std::sqrt(h[S_ERRS] / na);
    alm = std::sqrt(h[S_ALMISE] / na);
    cum = cum + alm;
    if (!o->skip_error_convergence) {
      if (alm_old > 0.0 && std::fabs(alm - alm_old) / alm_old < rel_err) break;
      if (err_dens < rel_err) break;
      if (err_smooth < rel_err) break;
      if (m > 7 && std::fabs(cum_old / (double)(m - 1) - cum / (double)m) / cum_old / (double)(m - 1) < rel_err)
        break;
    }
    alm_old = alm;
    cum_old = cum;
  }
  res->loops_done = (m > o->n_opt_loops) ? o->n_opt_loops : m;

  // closing weights (GridProjectedKDE.F90:5070-5120) and scalings (:4286-4306)
  if (!wfmt) {
    scale_grid(counts, 1, eff);
    scale_grid(dens, 1, eff);
  } else {
    SCK(density(B.wcnt, 0));
  }
  if (o->compute_raw_density) {
    scale_grid(counts, 0, b);
    if (wfmt) scale_grid(wcounts, 0, b);
  }
  if (o->unit_volume) scale_grid(dens, 1, b);
  SCK(cudaGetLastError());
  SCK(copy_out(dens));
  return MPRW_OK;
}
