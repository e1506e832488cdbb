// gpkde.cu -- GPKDE concentration reconstruction on the device.
//
// Restates GridProjectedKDE%ComputeDensity with the options MODPATH-RW uses
// (lib/gpkde/GridProjectedKDE.F90:3598-4392, optimisation loop 4396-5160):
// kernel database on (logarithmic h/delta, 3138-3528), bounded kernel sizes,
// minimum-roughness format 3, Kish effective weights, not isotropic, grid
// fixed to the domain; 1-D and 3-D reconstructions.
//
// GB300 design.  Every GPKDE kernel matrix is a product of one-dimensional
// factors (erf differences for W and the smoothing kernel, the Gaussian
// derivative term for the second-derivative kernels,
// KernelMultiGaussian.f90:720-1110), and the reflection at the grid edges
// (209-390) folds each dimension independently.  So the database is a small
// table of 1-D factors per dimension and h/delta index, each active bin is one
// thread block that folds its three factors in shared memory and then
//   * scatters count * fx fy fz into a grid (FP64 atomics), or
//   * gathers grid * fx fy fz (block reduction),
// and the per-bin smoothing updates are elementwise kernels.  Reductions over
// bins are two-stage with a fixed order, so runs are repeatable; the host
// takes the per-loop convergence decision from four scalars.
#include <cfloat>
#include <cmath>
#include <vector>

#include "gpkde.cuh"

namespace mprw {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int log_index(const KdeParams &P, double h, int d) {
  if (h <= 0.0) return 1;
  int i = (int)floor(log(h / P.bin[d] / P.min_hod) / P.dlog) + 1;
  if (i < 1) i = 1;
  if (i > P.ndelta) i = P.ndelta;
  return i;
}

// Fold one dimension's factor in place (prKernelReflection, one axis).
__device__ void fold_factor(double *v, int m, int gid, int nb) {
  const int len = 2 * m + 1;
  if (gid - m < 1) {
    const int b = 1 - gid + m;
    for (int j = 0; j < b; ++j) v[b + j] = v[b + j] + v[b - 1 - j];
    for (int j = 0; j < b; ++j) v[j] = 0.0;
  }
  if (gid + m > nb) {
    const int B = 2 * m + 1 - (gid + m - nb) + 1;  // 1-based
    const int lenb = len - B + 1;
    for (int j = 0; j < lenb; ++j) v[B - lenb - 1 + j] = v[B - lenb - 1 + j] + v[2 * m - j];
    for (int j = B - 1; j < len; ++j) v[j] = 0.0;
  }
}

struct Span {
  int g0[3], n[3], k0[3];
};

// Load the three factors of one kernel (table `tab`, per-dimension indexes
// idx[d] 1-based) for bin `gid`, fold them, and return the grid span.
__device__ void load_kernel(const KdeParams &P, const KdeTable &tab, const int idx[3], const int gid[3],
                            double *sv, Span &S) {
  __shared__ int s_m[3], s_ofs[3];
  if (threadIdx.x < 3) {
    const int d = threadIdx.x;
    s_m[d] = tab.m[d * KDE_MAXDB + idx[d] - 1];
    s_ofs[d] = tab.ofs[d * KDE_MAXDB + idx[d] - 1];
  }
  __syncthreads();
  for (int d = 0; d < 3; ++d) {
    const int m = s_m[d];
    for (int k = threadIdx.x; k < 2 * m + 1; k += blockDim.x) sv[d * KDE_MAXLEN + k] = tab.val[s_ofs[d] + k];
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int d = threadIdx.x;
    if (P.mask[d]) fold_factor(sv + d * KDE_MAXLEN, s_m[d], gid[d], P.nb[d]);
  }
  __syncthreads();
  for (int d = 0; d < 3; ++d) {
    const int m = s_m[d];
    const int g0 = max(gid[d] - m, 1), g1 = min(gid[d] + m, P.nb[d]);
    S.g0[d] = g0;
    S.n[d] = g1 - g0 + 1;
    S.k0[d] = g0 - gid[d] + m;
  }
}

__device__ __forceinline__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  return s;  // valid in thread 0
}

// kind: 0 = W kernel from ks (3 per-dim smoothings), 1 = isotropic kernel
// from a per-bin scale (sigma support), 2 = second-derivative kernel of
// axis `axis` from cb[axis]
__device__ void bin_indexes(const KdeParams &P, const KdeBins &B, int b, int kind, int axis, int idx[3]) {
  idx[0] = idx[1] = idx[2] = 1;
  if (kind == 0) {
    for (int d = 0; d < 3; ++d)
      if (P.mask[d]) idx[d] = log_index(P, B.ks[d * B.n + b], d);
  } else if (kind == 1) {
    const double s = B.support[b];
    for (int d = 0; d < 3; ++d)
      if (P.mask[d]) idx[d] = log_index(P, s, d);
  } else {
    const int n = log_index(P, B.cb[axis * B.n + b], axis);
    for (int d = 0; d < 3; ++d) idx[d] = n;  // the second-derivative database is isotropic
  }
}

__global__ void scatter_kernel(KdeParams P, KdeBins B, KdeTable tab, int kind, int axis, double *grid) {
  __shared__ double sv[3 * KDE_MAXLEN];
  const int b = blockIdx.x;
  if (b >= B.n) return;
  int idx[3], gid[3] = {B.gx[b], B.gy[b], B.gz[b]};
  bin_indexes(P, B, b, kind, axis, idx);
  Span S;
  load_kernel(P, tab, idx, gid, sv, S);
  const double cnt = B.count[b];
  const int tot = S.n[0] * S.n[1] * S.n[2];
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int ix = t % S.n[0], r = t / S.n[0], iy = r % S.n[1], iz = r / S.n[1];
    const double w = sv[S.k0[0] + ix] * sv[KDE_MAXLEN + S.k0[1] + iy] * sv[2 * KDE_MAXLEN + S.k0[2] + iz];
    const int64_t g = (int64_t)(S.g0[0] - 1 + ix) +
                      (int64_t)P.nb[0] * ((S.g0[1] - 1 + iy) + (int64_t)P.nb[1] * (S.g0[2] - 1 + iz));
    atomicAdd(&grid[g], cnt * w);
  }
}

// nEstimate-type gather with the isotropic kernel of scale `support` (kind 1)
__global__ void gather_kernel(KdeParams P, KdeBins B, KdeTable tab, const double *grid, double *out) {
  __shared__ double sv[3 * KDE_MAXLEN];
  __shared__ double red[32];
  const int b = blockIdx.x;
  if (b >= B.n) return;
  int idx[3], gid[3] = {B.gx[b], B.gy[b], B.gz[b]};
  bin_indexes(P, B, b, 1, 0, idx);
  Span S;
  load_kernel(P, tab, idx, gid, sv, S);
  const int tot = S.n[0] * S.n[1] * S.n[2];
  double acc = 0.0;
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int ix = t % S.n[0], r = t / S.n[0], iy = r % S.n[1], iz = r / S.n[1];
    const double w = sv[S.k0[0] + ix] * sv[KDE_MAXLEN + S.k0[1] + iy] * sv[2 * KDE_MAXLEN + S.k0[2] + iz];
    const int64_t g = (int64_t)(S.g0[0] - 1 + ix) +
                      (int64_t)P.nb[0] * ((S.g0[1] - 1 + iy) + (int64_t)P.nb[1] * (S.g0[2] - 1 + iz));
    acc += grid[g] * w;
  }
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) out[b] = s;
}

// roughness gathers of the squared curvatures (3-D: XX, YY, ZZ and the
// cross products of squares, GridProjectedKDE.F90:2470-2600)
__global__ void gather_roughness3_kernel(KdeParams P, KdeBins B, KdeTable tab, const double *cx, const double *cy,
                                         const double *cz) {
  __shared__ double sv[3 * KDE_MAXLEN];
  __shared__ double red[32];
  const int b = blockIdx.x;
  if (b >= B.n) return;
  int idx[3], gid[3] = {B.gx[b], B.gy[b], B.gz[b]};
  bin_indexes(P, B, b, 1, 0, idx);
  Span S;
  load_kernel(P, tab, idx, gid, sv, S);
  const int tot = S.n[0] * S.n[1] * S.n[2];
  double a[6] = {0, 0, 0, 0, 0, 0};
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int ix = t % S.n[0], r = t / S.n[0], iy = r % S.n[1], iz = r / S.n[1];
    const double w = sv[S.k0[0] + ix] * sv[KDE_MAXLEN + S.k0[1] + iy] * sv[2 * KDE_MAXLEN + S.k0[2] + iz];
    const int64_t g = (int64_t)(S.g0[0] - 1 + ix) +
                      (int64_t)P.nb[0] * ((S.g0[1] - 1 + iy) + (int64_t)P.nb[1] * (S.g0[2] - 1 + iz));
    const double x = cx[g], y = cy[g], z = cz[g];
    a[0] += x * w;
    a[1] += y * w;
    a[2] += z * w;
    a[3] += (x * y) * w;
    a[4] += (x * z) * w;
    a[5] += (y * z) * w;
  }
  double s[6];
  for (int k = 0; k < 6; ++k) s[k] = block_sum(a[k], red);
  if (threadIdx.x == 0) {
    const double rxx = s[0], ryy = s[1], rzz = s[2], rxy = s[3], rxz = s[4], ryz = s[5];
    B.rxx[b] = rxx;
    B.ryy[b] = ryy;
    B.rzz[b] = rzz;
    double v = 3.0 * pow(rxx * ryy * rzz, 1.0 / 3.0);
    if (ryz > 0.0) v = v + 2.0 * ryz * pow(rxx * rxx / ryy / rzz, 1.0 / 6.0);
    if (rxz > 0.0) v = v + 2.0 * rxz * pow(ryy * ryy / rxx / rzz, 1.0 / 6.0);
    if (rxy > 0.0) v = v + 2.0 * rxy * pow(rzz * rzz / rxx / ryy, 1.0 / 6.0);
    B.net[b] = v;
  }
}

__device__ __forceinline__ double smoothing_scale(const KdeParams &P, const double ks[3]) {
  double out = 1.0;
  int dimc = P.ndim;
  for (int d = 0; d < 3; ++d) {
    if (!P.mask[d]) continue;
    if (ks[d] != 0.0) out = out * ks[d];
    else dimc = dimc - 1;
  }
  return (dimc != 0) ? pow(out, 1.0 / (double)P.ndim) : 0.0;
}

__global__ void init_bins_kernel(KdeParams P, KdeBins B, double hs) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B.n) return;
  double ks[3];
  for (int d = 0; d < 3; ++d) ks[d] = P.mask[d] ? hs : 0.0;
  const double sc = smoothing_scale(P, ks);
  B.scale[b] = sc;
  B.support[b] = 2.0 * sc;
  for (int d = 0; d < 3; ++d) {
    B.ks[d * B.n + b] = ks[d];
    B.shape[d * B.n + b] = (P.mask[d] && sc > 0.0) ? ks[d] / sc : 0.0;
  }
  B.nest[b] = 0.0;
  B.net[b] = 0.0;
}

__global__ void grid_scale_kernel(double *g, int64_t n, double div) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    g[i] = g[i] / div;
}

// curvature normalisation: c = ((c / binVolume) / binSize^2)^2
__global__ void curvature_square_kernel(double *g, int64_t n, double binvol, double bs2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double c = g[i] / binvol;
    c = c / bs2;
    g[i] = c * c;
  }
}

__global__ void pick_kernel(KdeParams P, KdeBins B, const double *grid, double *out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B.n) return;
  const int64_t g = (int64_t)(B.gx[b] - 1) + (int64_t)P.nb[0] * ((B.gy[b] - 1) + (int64_t)P.nb[1] * (B.gz[b] - 1));
  out[b] = grid[g];
}

// second-half of the sigma-support update (GridProjectedKDE.F90:4836-4860)
__global__ void support_update_kernel(KdeParams P, KdeBins B, const double *ne1) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B.n) return;
  const double dn = B.dens[b];
  double ssc = pow(ne1[b], 0.5) * pow(B.scale[b], P.one_plus_nd_q) / pow(4.0 * dn, 0.25) * P.support_c;
  if (ssc > P.max_sigma_growth * B.support[b]) ssc = P.max_sigma_growth * B.support[b];
  ssc = fmin(ssc, P.max_k[P.max_dim]);
  if (ssc < P.min_k[P.min_dim]) ssc = P.min_k[P.min_dim];
  B.support[b] = ssc;
}

// prComputeCurvatureKernelBandwidth (GridProjectedKDE.F90:5207-5275)
__global__ void curvature_bandwidth_kernel(KdeParams P, KdeBins B) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B.n) return;
  double nvpb = 0.0;
  const double dn = B.dens[b];
  if (dn > 0.0) {
    const double base = SQRT8PI_D * B.support[b];
    double p = 1.0;
    for (int k = 0; k < P.ndim; ++k) p = (k == 0) ? base : p * base;  // integer power, left to right
    if (P.ndim == 3) p = base * (base * base);
    nvpb = pow(p * pow(B.nest[b], 2.0) / dn, P.beta_c);
  }
  for (int d = 0; d < 3; ++d) {
    if (!P.mask[d]) continue;
    double tsum = 0.0;
    for (int k = 0; k < 3; ++k) {
      if (!P.mask[k]) continue;
      const double sh = B.shape[k * B.n + b];
      if (sh != 0.0) tsum = tsum + (k == d ? 5.0 : 1.0) / (sh * sh);
    }
    const double shd = B.shape[d * B.n + b];
    double term = 0.0;
    if (shd != 0.0) term = pow((P.one_over_nd4 / pow(shd, 4.0)) * tsum, P.minus_one_over_nd6);
    double c = P.alpha_c * nvpb * term * B.scale[b];
    if (c > P.max_sd[d]) c = P.max_sd[d];
    if (c < P.min_sd[d]) c = P.min_sd[d];
    B.cb[d * B.n + b] = c;
  }
}

// deterministic two-stage reductions: stage 1 writes per-block partials
__global__ void reduce_stage1_kernel(KdeBins B, int what, double aux0, double aux1, double *partial) {
  __shared__ double red[32];
  double v0 = 0.0, v1 = 0.0, v2 = 0.0;
  bool isMax = (what == 0 || what == 2);
  double mx0 = -DBL_MAX, mx1 = -DBL_MAX, mn0 = DBL_MAX;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B.n; b += gridDim.x * blockDim.x) {
    if (what == 0) {  // max(net), min(net > 0)
      const double r = B.net[b];
      mx0 = fmax(mx0, r);
      if (r > 0.0) mn0 = fmin(mn0, r);
    } else if (what == 1) {  // error sums: density, smoothing, ALMISE
      const double dn = B.dens[b], dold = B.dens_old[b];
      if (dold != 0.0) {
        const double e = fabs(dn / aux0 - dold / aux1) / (dold / aux1);
        v0 += e * e;
      }
      const double so = B.scale_old[b], sc = B.scale[b];
      if (so != 0.0) {
        const double e = fabs(sc - so) / so;
        v1 += e * e;
      }
    } else if (what == 2) {  // max(dens), max(dens_old), max(scale > 0)
      mx0 = fmax(mx0, B.dens[b]);
      mx1 = fmax(mx1, B.dens_old[b]);
      if (B.scale[b] > 0.0) mn0 = fmin(mn0, -B.scale[b]);  // -max(scale)
    }
  }
  (void)isMax;
  // write per-thread values through a block reduction in fixed order
  if (what == 1) {
    const double s0 = block_sum(v0, red);
    const double s1 = block_sum(v1, red);
    const double s2 = block_sum(v2, red);
    if (threadIdx.x == 0) {
      partial[3 * blockIdx.x + 0] = s0;
      partial[3 * blockIdx.x + 1] = s1;
      partial[3 * blockIdx.x + 2] = s2;
    }
  } else {
    __shared__ double a[kThreads], c[kThreads], e[kThreads];
    a[threadIdx.x] = mx0;
    c[threadIdx.x] = mx1;
    e[threadIdx.x] = mn0;
    __syncthreads();
    if (threadIdx.x == 0) {
      double A = -DBL_MAX, Cc = -DBL_MAX, E = DBL_MAX;
      for (int i = 0; i < (int)blockDim.x; ++i) {
        A = fmax(A, a[i]);
        Cc = fmax(Cc, c[i]);
        E = fmin(E, e[i]);
      }
      partial[3 * blockIdx.x + 0] = A;
      partial[3 * blockIdx.x + 1] = Cc;
      partial[3 * blockIdx.x + 2] = E;
    }
  }
}

__global__ void reduce_stage2_kernel(int what, int nblk, const double *partial, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (what == 1) {
    double s0 = 0, s1 = 0, s2 = 0;
    for (int i = 0; i < nblk; ++i) {
      s0 += partial[3 * i];
      s1 += partial[3 * i + 1];
      s2 += partial[3 * i + 2];
    }
    out[0] = s0;
    out[1] = s1;
    out[2] = s2;
  } else {
    double A = -DBL_MAX, Cc = -DBL_MAX, E = DBL_MAX;
    for (int i = 0; i < nblk; ++i) {
      A = fmax(A, partial[3 * i]);
      Cc = fmax(Cc, partial[3 * i + 1]);
      E = fmin(E, partial[3 * i + 2]);
    }
    out[0] = A;
    out[1] = Cc;
    out[2] = E;
  }
}

// ALMISE per-bin term sum (GridProjectedKDE.F90:4966-4972)
__global__ void almise_stage1_kernel(KdeParams P, KdeBins B, double npts, double *partial) {
  __shared__ double red[32];
  double v = 0.0;
  const double nd = (double)P.ndim;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B.n; b += gridDim.x * blockDim.x) {
    const double sc = B.scale[b];
    if (sc != 0.0) {
      const double e = (B.nest[b] / (pow(sc, nd) * pow(4.0 * PI_D, 0.5 * nd)) + 0.25 * B.net[b] * pow(sc, 4.0)) /
                       pow(npts, 2.0);
      v += e * e;
    }
  }
  const double s = block_sum(v, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void sum_stage2_kernel(int nblk, const double *partial, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0;
  for (int i = 0; i < nblk; ++i) s += partial[i];
  out[0] = s;
}

// prComputeOptimalSmoothingAndShape, per bin (GridProjectedKDE.F90:5404-5724).
// phase 0: isotropy correction of the net roughness + scale where net > 0.
__global__ void optimal_phase0_kernel(KdeParams P, KdeBins B, double min_pos_net) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B.n) return;
  const double nd = (double)P.ndim;
  double net = B.net[b];
  if (P.ndim == 3) {
    double sm = B.rxx[b] + B.ryy[b] + B.rzz[b];
    if (sm == 0.0) sm = min_pos_net;
    if ((B.rxx[b] / sm > P.iso_threshold) || (B.ryy[b] / sm > P.iso_threshold) || (B.rzz[b] / sm > P.iso_threshold))
      net = (1.0 - 0.5) * net + 0.5 * sm;
    B.net[b] = net;
  }
  double sc = 0.0;
  if (net > 0.0) sc = pow(nd * B.nest[b] / (pow(4.0 * PI_D, 0.5 * nd) * net), P.one_over_nd4);
  B.scale[b] = sc;
}

// phase 1: scale for zero net roughness, shapes, bounded smoothing
__global__ void optimal_phase1_kernel(KdeParams P, KdeBins B, double max_pos_scale, int *update_flag) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B.n) return;
  double sc = B.scale[b];
  if (B.net[b] == 0.0) {
    sc = max_pos_scale;
    B.scale[b] = sc;
  }
  double sh[3] = {1.0, 1.0, 1.0};
  if (P.ndim == 3) {
    const double rxx = B.rxx[b], ryy = B.ryy[b], rzz = B.rzz[b], net = B.net[b];
    if (!(rxx == 0.0 || ryy == 0.0 || rzz == 0.0)) {
      const double s1 = fmax(pow(net / rxx, 1.0 / 12.0), P.min_k[0] / sc);
      const double s2 = fmax(pow(net / ryy, 1.0 / 12.0), P.min_k[1] / sc);
      const double s3 = 1.0 / s1 / s2;
      const double ns = pow(s1 * s2 * s3, (double)0.333f);
      if (ns != 0.0) {
        sh[0] = s1 / ns;
        sh[1] = s2 / ns;
        sh[2] = s3 / ns;
      }
    }
  }
  bool upd = false;
  for (int d = 0; d < 3; ++d) {
    B.shape[d * B.n + b] = sh[d];
    if (!P.mask[d]) {
      B.ks[d * B.n + b] = 0.0;
      continue;
    }
    double k = sh[d] * sc;
    if (k > P.max_k[d]) {
      k = P.max_k[d];
      upd = true;
    }
    if (k < P.min_k[d]) {
      k = P.min_k[d];
      upd = true;
    }
    B.ks[d * B.n + b] = k;
  }
  if (upd) atomicOr(update_flag, 1);
}

// phase 2: smoothing scale from the bounded smoothing (all bins)
__global__ void rescale_kernel(KdeParams P, KdeBins B) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B.n) return;
  double ks[3] = {B.ks[b], B.ks[B.n + b], B.ks[2 * B.n + b]};
  B.scale[b] = smoothing_scale(P, ks);
}

__global__ void copy_kernel(double *dst, const double *src, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

// active-bin compaction (x fastest order, Histogram.F90:493-527): count
// per block, then an ordered write.
__global__ void active_count_kernel(const double *counts, int64_t nbins, int chunk, int *blockcnt) {
  __shared__ int s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  const int64_t beg = (int64_t)blockIdx.x * chunk;
  const int64_t end = min(beg + chunk, nbins);
  int c = 0;
  for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) c += (counts[i] != 0.0);
  atomicAdd(&s, c);
  __syncthreads();
  if (threadIdx.x == 0) blockcnt[blockIdx.x] = s;
}

__global__ void active_write_kernel(const double *counts, int64_t nbins, int chunk, const int *blockofs,
                                    KdeParams P, KdeBins B) {
  if (threadIdx.x != 0) return;
  const int64_t beg = (int64_t)blockIdx.x * chunk;
  const int64_t end = min(beg + chunk, nbins);
  int o = blockofs[blockIdx.x];
  for (int64_t i = beg; i < end; ++i) {
    const double c = counts[i];
    if (c == 0.0) continue;
    const int ix = (int)(i % P.nb[0]);
    const int64_t r = i / P.nb[0];
    const int iy = (int)(r % P.nb[1]);
    const int iz = (int)(r / P.nb[1]);
    B.gx[o] = ix + 1;
    B.gy[o] = iy + 1;
    B.gz[o] = iz + 1;
    B.count[o] = c;
    ++o;
  }
}

int blocks_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b > 152 * 8) b = 152 * 8;
  return b < 1 ? 1 : (int)b;
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
cudaError_t KdeState::ensure_bins(int n) {
  if (n <= cap) {
    bins.n = n;
    return cudaSuccess;
  }
  void *old[] = {bins.gx, bins.gy, bins.gz, bins.count, bins.ks, bins.scale, bins.shape, bins.support, bins.nest,
                 bins.dens, bins.cb, bins.rxx, bins.ryy, bins.rzz, bins.net, bins.dens_old, bins.scale_old, tmp,
                 partial};
  for (void *p : old)
    if (p) cudaFree(p);
  const size_t c = (size_t)n;
  cudaError_t e = cudaSuccess;
  auto I = [&](int **p, size_t k) {
    if (e == cudaSuccess) e = cudaMalloc((void **)p, sizeof(int) * k);
  };
  auto D = [&](double **p, size_t k) {
    if (e == cudaSuccess) e = cudaMalloc((void **)p, sizeof(double) * k);
  };
  I(&bins.gx, c); I(&bins.gy, c); I(&bins.gz, c);
  D(&bins.count, c); D(&bins.ks, 3 * c); D(&bins.scale, c); D(&bins.shape, 3 * c); D(&bins.support, c);
  D(&bins.nest, c); D(&bins.dens, c); D(&bins.cb, 3 * c); D(&bins.rxx, c); D(&bins.ryy, c); D(&bins.rzz, c);
  D(&bins.net, c); D(&bins.dens_old, c); D(&bins.scale_old, c); D(&tmp, c);
  D(&partial, 3 * 152 * 8 + 16);
  if (e != cudaSuccess) return e;
  cap = n;
  bins.n = n;
  return cudaSuccess;
}

cudaError_t KdeState::ensure_grid(int64_t ngrid) {
  if (!d_scalars) {
    cudaError_t e = cudaMalloc((void **)&d_scalars, 8 * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&h_scalars, 8 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_flag, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&h_flag, sizeof(int));
    if (e != cudaSuccess) return e;
  }
  if (ngrid <= grid_cap) return cudaSuccess;
  double *old[] = {dens_grid, cx, cy, cz};
  for (double *p : old)
    if (p) cudaFree(p);
  if (d_blockcnt) cudaFree(d_blockcnt);
  cudaError_t e = cudaMalloc((void **)&dens_grid, sizeof(double) * ngrid);
  if (e == cudaSuccess) e = cudaMalloc((void **)&cx, sizeof(double) * ngrid);
  if (e == cudaSuccess) e = cudaMalloc((void **)&cy, sizeof(double) * ngrid);
  if (e == cudaSuccess) e = cudaMalloc((void **)&cz, sizeof(double) * ngrid);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_blockcnt, sizeof(int) * ((ngrid + 4095) / 4096 + 1));
  if (e != cudaSuccess) return e;
  grid_cap = ngrid;
  return cudaSuccess;
}

void KdeState::release() {
  void *ptrs[] = {bins.gx, bins.gy, bins.gz, bins.count, bins.ks, bins.scale, bins.shape, bins.support, bins.nest,
                  bins.dens, bins.cb, bins.rxx, bins.ryy, bins.rzz, bins.net, bins.dens_old, bins.scale_old, tmp,
                  partial, dens_grid, cx, cy, cz, d_scalars, d_flag, d_blockcnt, d_val, d_meta};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (h_scalars) cudaFreeHost(h_scalars);
  if (h_flag) cudaFreeHost(h_flag);
  *this = KdeState();
}
static double erf_diff(double i, double hd) {
  const double s2 = std::sqrt(2.0);
  return std::erf((i + 0.5) / (hd * s2)) - std::erf((i - 0.5) / (hd * s2));
}

void kde_build_tables(const KdeParams &P, std::vector<double> &val, std::vector<int> &wm, std::vector<int> &wofs,
                      std::vector<int> (&sm)[3], std::vector<int> (&sofs)[3]) {
  val.clear();
  wm.assign(3 * KDE_MAXDB, 0);
  wofs.assign(3 * KDE_MAXDB, 0);
  for (int a = 0; a < 3; ++a) {
    sm[a].assign(3 * KDE_MAXDB, 0);
    sofs[a].assign(3 * KDE_MAXDB, 0);
  }
  auto push = [&](const std::vector<double> &v) {
    int o = (int)val.size();
    val.insert(val.end(), v.begin(), v.end());
    return o;
  };
  const double nd = (double)P.ndim;
  for (int n = 0; n < P.ndelta; ++n) {
    const double hod = P.hod[n];
    // W / sigma factor per dimension: prSetupMatrix with bandwidth hod*binSize
    for (int d = 0; d < 3; ++d) {
      std::vector<double> f;
      int m = 0;
      if (P.mask[d]) {
        const double bw = hod * P.bin[d];
        m = (int)std::ceil(3 * bw / P.bin[d]);
        const double hd = bw / P.bin[d];
        std::vector<double> half(m + 1);
        for (int i = 0; i <= m; ++i) half[i] = erf_diff((double)i, hd);
        double s = half[0];
        for (int i = 1; i <= m; ++i) s += 2.0 * half[i];
        f.resize(2 * m + 1);
        for (int i = -m; i <= m; ++i) f[i + m] = half[std::abs(i)] / s;
      } else {
        f.assign(1, 1.0);
      }
      wm[d * KDE_MAXDB + n] = m;
      wofs[d * KDE_MAXDB + n] = push(f);
    }
    // second-derivative kernels of axis a: the 3-D database is isotropic;
    // 1-D uses the active dimension only (prInitializeKernelDatabaseFlat)
    for (int a = 0; a < 3; ++a) {
      if (!P.mask[a]) {
        for (int d = 0; d < 3; ++d) {
          sm[a][d * KDE_MAXDB + n] = 0;
          sofs[a][d * KDE_MAXDB + n] = push(std::vector<double>(1, 0.0));
        }
        continue;
      }
      double hdv[3] = {0, 0, 0};
      int mv[3] = {0, 0, 0};
      for (int d = 0; d < 3; ++d) {
        const bool on = (P.ndim == 3) ? (P.bin[d] != 0.0) : (P.mask[d] != 0);
        if (!on) continue;
        const double bw = hod * P.bin[d];
        mv[d] = (int)std::ceil(4 * bw / P.bin[d]);
        hdv[d] = bw / P.bin[d];
      }
      // the unconditional `return` before the normalisation: scale by
      // 1/sqrt(hdelta) of the active dimensions before the axis only
      double scal = 1.0;
      for (int d = 0; d < 3; ++d) {
        if (hdv[d] <= 0.0) continue;
        if (d == a) break;
        scal = scal / std::sqrt(hdv[d]);
      }
      for (int d = 0; d < 3; ++d) {
        const int m = mv[d];
        std::vector<double> half(m + 1), f(2 * m + 1);
        if (hdv[d] <= 0.0) {
          half.assign(m + 1, 1.0);
        } else if (d == a) {
          const double h = hdv[d];
          const double c = -1.0 / (std::pow(2.0, nd - 0.5) * std::sqrt(4.0 * std::atan(1.0)) * std::pow(h, 3.0));
          for (int i = 0; i <= m; ++i) {
            const double xp = i + 0.5, xm = i - 0.5;
            half[i] = c * (xp * std::exp(-1.0 * (xp * xp) / (2.0 * (h * h))) -
                           xm * std::exp(-1.0 * (xm * xm) / (2.0 * (h * h))));
          }
          for (int i = 0; i <= m; ++i) half[i] *= scal;
        } else {
          for (int i = 0; i <= m; ++i) half[i] = erf_diff((double)i, hdv[d]);
        }
        for (int i = -m; i <= m; ++i) f[i + m] = half[std::abs(i)];
        sm[a][d * KDE_MAXDB + n] = m;
        sofs[a][d * KDE_MAXDB + n] = push(f);
      }
    }
  }
}

#define KCK(x)                            \
  do {                                    \
    cudaError_t e_ = (x);                 \
    if (e_ != cudaSuccess) return e_;     \
  } while (0)

cudaError_t kde_run(KdeState &st, const KdeParams &P, double hs, double npts, int n_opt_loops, double rel_err,
                    bool skip_error, cudaStream_t s, int *loops_done) {
  KdeBins &B = st.bins;
  const int nb = B.n;
  const int64_t ngrid = (int64_t)P.nb[0] * P.nb[1] * P.nb[2];
  const int bb = (nb + kThreads - 1) / kThreads;
  const int gb = blocks_for(ngrid);
  const int rb = blocks_for(nb);
  double *h = st.h_scalars;
  auto density = [&](void) -> cudaError_t {
    KCK(cudaMemsetAsync(st.dens_grid, 0, sizeof(double) * ngrid, s));
    scatter_kernel<<<nb, kThreads, 0, s>>>(P, B, st.wtab, 0, 0, st.dens_grid);
    grid_scale_kernel<<<gb, kThreads, 0, s>>>(st.dens_grid, ngrid, P.binvol);
    pick_kernel<<<bb, kThreads, 0, s>>>(P, B, st.dens_grid, B.dens);
    st.launches += 3;
    return cudaGetLastError();
  };
  auto reduce = [&](int what, double a0, double a1) -> cudaError_t {
    reduce_stage1_kernel<<<rb, kThreads, 0, s>>>(B, what, a0, a1, st.partial);
    reduce_stage2_kernel<<<1, 1, 0, s>>>(what, rb, st.partial, st.d_scalars);
    KCK(cudaMemcpyAsync(h, st.d_scalars, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    st.launches += 2;
    return cudaStreamSynchronize(s);
  };
  auto almise = [&](double &out) -> cudaError_t {
    almise_stage1_kernel<<<rb, kThreads, 0, s>>>(P, B, npts, st.partial);
    sum_stage2_kernel<<<1, 1, 0, s>>>(rb, st.partial, st.d_scalars);
    KCK(cudaMemcpyAsync(h, st.d_scalars, sizeof(double), cudaMemcpyDeviceToHost, s));
    KCK(cudaStreamSynchronize(s));
    st.launches += 2;
    out = std::sqrt(h[0] / nb);
    return cudaSuccess;
  };
  init_bins_kernel<<<bb, kThreads, 0, s>>>(P, B, hs);
  st.launches += 1;
  KCK(density());
  double alm = 0.0;
  KCK(almise(alm));  // nEstimate and net roughness are zero: 0
  double alm_old = alm, cum = alm, cum_old = alm;
  copy_kernel<<<bb, kThreads, 0, s>>>(B.dens_old, B.dens, nb);
  copy_kernel<<<bb, kThreads, 0, s>>>(B.scale_old, B.scale, nb);
  st.launches += 2;
  int m = 0;
  for (m = 1; m <= n_opt_loops; ++m) {
    // nEstimate with the current support, support update, nEstimate again
    gather_kernel<<<nb, kThreads, 0, s>>>(P, B, st.wtab, st.dens_grid, st.tmp);
    support_update_kernel<<<bb, kThreads, 0, s>>>(P, B, st.tmp);
    gather_kernel<<<nb, kThreads, 0, s>>>(P, B, st.wtab, st.dens_grid, B.nest);
    curvature_bandwidth_kernel<<<bb, kThreads, 0, s>>>(P, B);
    st.launches += 4;
    // net roughness
    double *cg[3] = {st.cx, st.cy, st.cz};
    for (int a = 0; a < 3; ++a) {
      if (P.ndim == 1 && !P.mask[a]) continue;
      KCK(cudaMemsetAsync(cg[a], 0, sizeof(double) * ngrid, s));
      scatter_kernel<<<nb, kThreads, 0, s>>>(P, B, st.sdtab[a], 2, a, cg[a]);
      curvature_square_kernel<<<gb, kThreads, 0, s>>>(cg[a], ngrid, P.binvol, P.bin[a] * P.bin[a]);
      st.launches += 2;
    }
    if (P.ndim == 3) {
      gather_roughness3_kernel<<<nb, kThreads, 0, s>>>(P, B, st.wtab, st.cx, st.cy, st.cz);
      st.launches += 1;
    } else {
      int a = 0;
      while (!P.mask[a]) ++a;
      double *r1 = (a == 0) ? B.rxx : (a == 1 ? B.ryy : B.rzz);
      gather_kernel<<<nb, kThreads, 0, s>>>(P, B, st.wtab, cg[a], r1);
      copy_kernel<<<bb, kThreads, 0, s>>>(B.net, r1, nb);
      st.launches += 2;
    }
    KCK(cudaGetLastError());
    // optimal smoothing and shape
    KCK(reduce(0, 0.0, 0.0));
    if (h[0] == 0.0) return cudaErrorInvalidValue;  // maxval(netRoughness) == 0: the reference stops
    const double min_pos_net = h[2];
    optimal_phase0_kernel<<<bb, kThreads, 0, s>>>(P, B, min_pos_net);
    st.launches += 1;
    KCK(reduce(2, 0.0, 0.0));
    const double max_pos_scale = -h[2];
    KCK(cudaMemsetAsync(st.d_flag, 0, sizeof(int), s));
    optimal_phase1_kernel<<<bb, kThreads, 0, s>>>(P, B, max_pos_scale, st.d_flag);
    KCK(cudaMemcpyAsync(st.h_flag, st.d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    KCK(cudaStreamSynchronize(s));
    st.launches += 1;
    if (*st.h_flag) {
      rescale_kernel<<<bb, kThreads, 0, s>>>(P, B);
      st.launches += 1;
    }
    // density with the new smoothing
    KCK(density());
    // errors (GridProjectedKDE.F90:4962-5038)
    KCK(reduce(2, 0.0, 0.0));
    const double mx = h[0], mx_old = h[1];
    KCK(reduce(1, mx, mx_old));
    const double err_dens = std::sqrt(h[0] / nb), err_smooth = std::sqrt(h[1] / nb);
    KCK(almise(alm));
    cum = cum + alm;
    if (!skip_error) {
      if (alm_old > 0.0 && std::fabs(alm - alm_old) / alm_old < rel_err) break;
      if (err_dens < rel_err) break;
      if (err_smooth < rel_err) break;
      if (m > 7 && std::fabs(cum_old / (double)(m - 1) - cum / (double)m) / cum_old / (double)(m - 1) < rel_err)
        break;
    }
    alm_old = alm;
    cum_old = cum;
    copy_kernel<<<bb, kThreads, 0, s>>>(B.dens_old, B.dens, nb);
    copy_kernel<<<bb, kThreads, 0, s>>>(B.scale_old, B.scale, nb);
    st.launches += 2;
  }
  if (loops_done) *loops_done = (m > n_opt_loops) ? n_opt_loops : m;
  return cudaGetLastError();
}

cudaError_t kde_collect_active(KdeState &st, const KdeParams &P, const double *counts, cudaStream_t s, int *nactive) {
  const int64_t ngrid = (int64_t)P.nb[0] * P.nb[1] * P.nb[2];
  const int chunk = 4096;
  const int nblk = (int)((ngrid + chunk - 1) / chunk);
  std::vector<int> cnt(nblk), ofs(nblk);
  int *d_cnt = st.d_blockcnt;
  active_count_kernel<<<nblk, kThreads, 0, s>>>(counts, ngrid, chunk, d_cnt);
  KCK(cudaGetLastError());
  KCK(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int) * nblk, cudaMemcpyDeviceToHost, s));
  KCK(cudaStreamSynchronize(s));
  int tot = 0;
  for (int i = 0; i < nblk; ++i) {
    ofs[i] = tot;
    tot += cnt[i];
  }
  *nactive = tot;
  if (tot == 0) return cudaSuccess;
  KCK(st.ensure_bins(tot));
  KCK(cudaMemcpyAsync(d_cnt, ofs.data(), sizeof(int) * nblk, cudaMemcpyHostToDevice, s));
  active_write_kernel<<<nblk, 32, 0, s>>>(counts, ngrid, chunk, d_cnt, P, st.bins);
  st.launches += 2;
  return cudaGetLastError();
}

}  // namespace mprw
