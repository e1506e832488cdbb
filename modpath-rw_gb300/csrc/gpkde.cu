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
// (209-390) folds each dimension independently.  So the database is a table
// of 1-D factors per dimension and h/delta level:
//   * the density scatter (anisotropic W kernel per bin) runs one warp per
//     bin with FP64/FP32 atomics;
//   * the smoothing-kernel gathers and the second-derivative scatters, whose
//     kernels come from one scalar per bin, run as three 1-D passes per
//     database level over the bounding box of that level's bins (no atomics);
//   * per-bin updates are elementwise kernels; reductions over bins are
//     two-stage with a fixed order, in FP64.
// The host takes the per-loop convergence decision from a few scalars; one
// loop is a captured CUDA graph.  The arithmetic type T is double (the
// reference's arithmetic) or float (the mixed-precision pipeline).
#include <cfloat>
#include <algorithm>
#include <climits>
#include <cmath>
#include <numeric>
#include <type_traits>
#include <vector>

#include "gpkde.cuh"

namespace mprw {

namespace {

constexpr int kThreads = 256;
constexpr int kBinThreads = 64;   // per-bin elementwise kernels: spread few bins over all SMs
constexpr int kPassBlocks = 2432; // most blocks of a separable pass: 16 per SM (measured best of 4-48), grid-stride over all keys' regions

// The database level of a kernel size h along dimension d:
// floor(log(h / bin / minHOverDelta) / dlog) + 1, clamped to the database.
// GB300 issues two FP64 lane-operations per clock per SM, and a double
// logarithm is a few dozen of them, so in FP64 the quotient is first
// estimated in FP32 (within 1e-4 of the FP64 value: the FP32 rounding of h
// and the FP32 logarithm); the FP64 expression runs only when the estimate
// lies within 1e-3 of an integer or is not finite.  The level is the FP64
// expression's in every case.
template <typename T>
__device__ __forceinline__ int log_index(const KdeParams &P, T h, int d) {
  if (h <= T(0)) return 1;
  int i;
  if constexpr (sizeof(T) == 8) {
    const float v = logf((float)h * P.lscale[d]) * P.linv;
    if (isfinite(v) && fabsf(v - rintf(v)) > 1e-3f) i = (int)floorf(v) + 1;
    else i = (int)floor(log(h / T(P.bin[d]) / T(P.min_hod)) / T(P.dlog)) + 1;
  } else {
    i = (int)floor(log(h / T(P.bin[d]) / T(P.min_hod)) / T(P.dlog)) + 1;
  }
  if (i < 1) i = 1;
  if (i > P.ndelta) i = P.ndelta;
  return i;
}

// Powers of the optimisation loop.  The reference raises to real exponents
// (x**0.25, x**(1/(nDim+4)), ...), which its compiler evaluates with the C
// library's pow.  Here each is its identity in square and cube roots where
// the exponent allows (x^0.25 = sqrt(sqrt(x)), x^(1/6) = cbrt(sqrt(x)),
// x^-(1/9) = 1/cbrt(cbrt(x)), ...) and exp(y log x) otherwise: a few
// rounding errors (1e-15 relative for the exponents and arguments here)
// instead of a pow that costs several times as many FP64 operations.  Every
// argument is >= 0 (products and quotients of smoothed squares, densities
// and kernel sizes); for x < 0 the forms give NaN as pow does, and x = 0
// gives 0 (positive exponents) or +inf (negative ones) as pow does.
template <typename T>
__device__ __forceinline__ T root4(T x) { return sqrt(sqrt(x)); }
template <typename T>
__device__ __forceinline__ T pow_general(T x, T y) { return exp(y * log(x)); }
// x^(1/nd)
template <typename T>
__device__ __forceinline__ T pow_inv_nd(T x, int nd) { return nd == 3 ? cbrt(x) : (nd == 2 ? sqrt(x) : x); }
// x^(1 + nd/4)
template <typename T>
__device__ __forceinline__ T pow_one_plus_nd_q(T x, int nd) {
  const T r = sqrt(x);
  return nd == 3 ? x * r * sqrt(r) : (nd == 2 ? x * r : x * sqrt(r));
}
// x^(1/(nd+4))
template <typename T>
__device__ __forceinline__ T pow_one_over_nd4(T x, int nd, double y) {
  return nd == 2 ? cbrt(sqrt(x)) : pow_general(x, T(y));
}
// x^(-1/(nd+6))
template <typename T>
__device__ __forceinline__ T pow_minus_one_over_nd6(T x, int nd, double y) {
  return nd == 3 ? T(1) / cbrt(cbrt(x)) : (nd == 2 ? T(1) / sqrt(sqrt(sqrt(x))) : pow_general(x, T(y)));
}
// x^(2/((nd+4)(nd+6)))
template <typename T>
__device__ __forceinline__ T pow_beta(T x, int nd, double y) {
  return nd == 2 ? cbrt(sqrt(sqrt(sqrt(x)))) : pow_general(x, T(y));
}

// Device scalars of one reconstruction (S, FP64): slot meanings
//   S_NETMAX  max net roughness           S_NETMINPOS  min positive net roughness
//   S_DMAX    max density                 S_DMAXOLD    max previous density
//   S_ERRD    sum of squared density changes   S_ERRS  ... smoothing changes
//   S_ALMISE  sum of squared ALMISE terms S_SCMAX      max positive smoothing scale
//   S_WORK    the reconstruction's work model, summed over its loops (below)
enum { S_NETMAX = 0, S_NETMINPOS = 2, S_DMAX = 3, S_DMAXOLD = 4, S_ERRD = 6, S_ERRS = 7, S_ALMISE = 9,
       S_SCMAX = 11, S_WORK = 12, S_COUNT = 13 };

// The work model of one optimisation loop (the multiply-adds of direct 3-D
// kernels, GridProjectedKDE.F90:4620-4667, 4808-5065): per active bin its W
// kernel, eight smoothing-kernel gathers (support update, nEstimate, six
// roughness terms) and the three second-derivative kernels, each of
// prod_d (2 m_d + 1) cells at the bin's database kernels.  It is counted
// where the kernels' half widths are already at hand -- per level in the
// plans (bins per level times the level's kernel), per bin in the density
// scatter -- as 64-bit integers in S[S_WORK] (exact, in any order), and reset
// before the first loop.  The separable passes do a fraction of it; divided
// by the time it is the rate a direct evaluation would need.
__device__ __forceinline__ unsigned long long *work_counter(double *S) {
  return reinterpret_cast<unsigned long long *>(S + S_WORK);
}

// Extremes of positive values by integer atomics on the IEEE bit patterns
// (their order is the numeric order for positive doubles): order-independent,
// so as repeatable as the fixed-order sums.  One atomic per warp.
__device__ __forceinline__ void warp_max_pos(double *addr, double v) {
  v = (v > 0.0) ? v : 0.0;
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0 && v > 0.0)
    atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void warp_min_pos(double *addr, double v) {
  v = (v > 0.0) ? v : DBL_MAX;
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0 && v < DBL_MAX)
    atomicMin(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

// Fold one dimension's factor in place (prKernelReflection, one axis), the
// lanes of a warp splitting each loop: the part below cell 1 is added onto its
// mirror image and cleared, then the part above cell nb likewise (targets and
// sources of each step are disjoint).  m, gid and nb are warp-uniform.
template <typename T>
__device__ void fold_factor_warp(T *v, int m, int gid, int nb, int lane) {
  const int len = 2 * m + 1;
  if (gid - m < 1) {
    const int b = 1 - gid + m;
    for (int j = lane; j < b; j += 32) v[b + j] = v[b + j] + v[b - 1 - j];
    __syncwarp();
    for (int j = lane; j < b; j += 32) v[j] = T(0);
    __syncwarp();
  }
  if (gid + m > nb) {
    const int B = 2 * m + 1 - (gid + m - nb) + 1;  // 1-based
    const int lenb = len - B + 1;
    for (int j = lane; j < lenb; j += 32) v[B - lenb - 1 + j] = v[B - lenb - 1 + j] + v[2 * m - j];
    __syncwarp();
    for (int j = B - 1 + lane; j < len; j += 32) v[j] = T(0);
    __syncwarp();
  }
}

struct Span {
  int g0[3], n[3], k0[3];
};

// ---- density scatter: one warp per bin --------------------------------------
// The W kernel of a bin is anisotropic (one database level per dimension), so
// bins share no kernel and each warp folds its bin's three factors in shared
// memory and adds count * fy fz * fx over the span (atomics, one multiply per
// cell with the row products cached).
//
// The atomics add 64-bit fixed-point integers, not floating-point values:
// each contribution is scaled by 2^shift and rounded to an integer once, and
// integer sums do not depend on the order in which the warps' atomics land,
// so the density is bit-for-bit repeatable (FP64 atomicAdd is not).  Every
// bin's folded kernel sums to at most one, so the grid's total is at most the
// total count, which the host bounds by the active particles; shift is chosen
// so that this bound times 2^shift stays below 2^62 (no overflow), and the
// rounding error of one contribution is 2^-(shift+1) -- about 2e-13 counts
// for a million particles.
constexpr int kWarpsW = 4;
constexpr int kRowCache = 256;

__device__ __forceinline__ unsigned long long to_fixed(double v, double scale) {
  return (unsigned long long)__double2ll_rn(v * scale);
}
__device__ __forceinline__ unsigned long long to_fixed(float v, float scale) {
  return (unsigned long long)__float2ll_rn(v * scale);
}

// round(a * b / 2^63) for a < 2^63, b <= 2^63 (the 128-bit product, rounded
// to nearest), on the integer pipe
__device__ __forceinline__ unsigned long long mulq63(unsigned long long a, unsigned long long b) {
  const unsigned long long lo = a * b, lo2 = lo + (1ull << 62);
  const unsigned long long hi = __umul64hi(a, b) + (lo2 < lo ? 1ull : 0ull);
  return (hi << 1) | (lo2 >> 63);
}

// FP64 path of the density scatter on the integer pipe.  GB300 issues two FP64
// lane-operations per clock per SM against 64 integer ones, and the scatter's
// per-cell work is a product and a conversion to fixed point, so the folded
// factors are converted once per bin to 63-bit fixed point (fx, fy, fz <= 1)
// and the count to the grid's fixed point (|count| 2^shift < 2^62), and every
// cell's contribution is the rounded integer product |count| fz fy fx:
// three roundings of at most half a unit of 2^-shift, where the FP64 product
// carried a relative 2^-53 -- the same density to far below the tolerance of
// its FP64 reference.
__device__ __forceinline__ unsigned long long fixed63(double f) {
  return __double2ull_rn(f * 9223372036854775808.0);  // 2^63
}

template <typename T>
__global__ void __launch_bounds__(32 * kWarpsW) wscatter_kernel(KdeParams P, KdeBinsT<T> B, KdeTableT<T> tab,
                                                                int stride, T fscale,
                                                                unsigned long long *grid,
                                                                unsigned long long *wcnt) {
  __shared__ T sv_all[kWarpsW][3 * KDE_MAXLEN];
  __shared__ int sm_all[kWarpsW][3], sofs_all[kWarpsW][3];
  __shared__ T crow_all[kWarpsW][kRowCache];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int wi = blockIdx.x * kWarpsW + w;
  if (wi >= B.n) return;  // warp-uniform
  // bins are stored x fastest, so neighbouring warps would add into nearly the
  // same cells at once; warp wi takes bin (wi * stride) mod n instead
  // (gcd(stride, n) = 1: a permutation), spreading the atomics over the grid
  const int b = (int)(((long long)wi * stride) % B.n);
  T *sv = sv_all[w];
  const int gid[3] = {B.gx[b], B.gy[b], B.gz[b]};
  if (lane < 3) {
    const int d = lane;
    // the W kernel's database level along d (lanes 0-2, one dimension each)
    const int idx = P.mask[d] ? log_index<T>(P, B.ks[d * B.n + b], d) : 1;
    sm_all[w][d] = tab.m[d * KDE_MAXDB + idx - 1];
    sofs_all[w][d] = tab.ofs[d * KDE_MAXDB + idx - 1];
  }
  __syncwarp();
  if (lane == 0)  // the work model: the W kernel's cells (64 counters: one address would serialise)
    atomicAdd(wcnt + (wi & 63), (unsigned long long)((2 * sm_all[w][0] + 1) * (2 * sm_all[w][1] + 1) *
                                                     (2 * sm_all[w][2] + 1)));
  for (int d = 0; d < 3; ++d) {
    const int m = sm_all[w][d], o = sofs_all[w][d];
    for (int k = lane; k < 2 * m + 1; k += 32) sv[d * KDE_MAXLEN + k] = tab.val[o + k];
  }
  __syncwarp();
  for (int d = 0; d < 3; ++d)
    if (P.mask[d]) fold_factor_warp<T>(sv + d * KDE_MAXLEN, sm_all[w][d], gid[d], P.nb[d], lane);
  Span S;
  for (int d = 0; d < 3; ++d) {
    const int m = sm_all[w][d];
    const int g0 = max(gid[d] - m, 1), g1 = min(gid[d] + m, P.nb[d]);
    S.g0[d] = g0;
    S.n[d] = g1 - g0 + 1;
    S.k0[d] = g0 - gid[d] + m;
  }
  const T cnt = (T)B.count[b];
  const int n0 = S.n[0], n1 = S.n[1], rows = S.n[1] * S.n[2];
  const T *fx = sv + S.k0[0], *fy = sv + KDE_MAXLEN + S.k0[1], *fz = sv + 2 * KDE_MAXLEN + S.k0[2];
  const int64_t sy = P.nb[0], sz = (int64_t)P.nb[0] * P.nb[1];
  unsigned long long *gbase = grid + (S.g0[0] - 1) + sy * (S.g0[1] - 1) + sz * (S.g0[2] - 1);
  if constexpr (sizeof(T) == 8) {
    // the factors to fixed point in place (each lane converts the entries it
    // owns, then the warp reads them as integers)
    unsigned long long *q = reinterpret_cast<unsigned long long *>(sv);
    for (int d = 0; d < 3; ++d) {
      const int len = 2 * sm_all[w][d] + 1;
      for (int k = lane; k < len; k += 32) q[d * KDE_MAXLEN + k] = fixed63((double)sv[d * KDE_MAXLEN + k]);
    }
    __syncwarp();
    const unsigned long long *qx = q + S.k0[0], *qy = q + KDE_MAXLEN + S.k0[1], *qz = q + 2 * KDE_MAXLEN + S.k0[2];
    const long long ci = __double2ll_rn((double)cnt * (double)fscale);
    const unsigned long long cm = (unsigned long long)(ci < 0 ? -ci : ci);
    const bool neg = ci < 0;
    auto row_val = [&](int iy, int iz) { return mulq63(mulq63(cm, qz[iz]), qy[iy]); };
    auto emit = [&](unsigned long long *dst, unsigned long long r, int ix) {
      const unsigned long long v = mulq63(r, qx[ix]);
      if (v) atomicAdd(dst, neg ? (unsigned long long)(-(long long)v) : v);
    };
    unsigned long long *crq = reinterpret_cast<unsigned long long *>(crow_all[w]);
    const bool cached = rows <= kRowCache;
    if (cached) {
      for (int r = lane; r < rows; r += 32) {
        const int iz = r / n1, iy = r - iz * n1;
        crq[r] = row_val(iy, iz);
      }
      __syncwarp();
    }
    if (n0 <= 32) {
      const int rpi = 32 / n0, ix = lane % n0, r0 = lane / n0;
      if (r0 >= rpi) return;
      int iz = r0 / n1, iy = r0 - iz * n1;
      for (int r = r0; r < rows; r += rpi) {
        emit(gbase + ix + sy * iy + sz * iz, cached ? crq[r] : row_val(iy, iz), ix);
        iy += rpi;
        while (iy >= n1) {
          iy -= n1;
          ++iz;
        }
      }
    } else {
      for (int r = 0; r < rows; ++r) {
        const int iz = r / n1, iy = r - iz * n1;
        const unsigned long long rv = cached ? crq[r] : row_val(iy, iz);
        for (int ix = lane; ix < n0; ix += 32) emit(gbase + ix + sy * iy + sz * iz, rv, ix);
      }
    }
    return;
  }
  // count * fy * fz per row (y fastest), cached when the span has few rows
  T *crow = crow_all[w];
  const bool cached = rows <= kRowCache;
  if (cached) {
    for (int r = lane; r < rows; r += 32) {
      const int iz = r / n1, iy = r - iz * n1;
      crow[r] = cnt * (fy[iy] * fz[iz]);
    }
    __syncwarp();
  }
  if (n0 <= 32) {
    // 32 / n0 rows per pass, lane -> (row offset, x)
    const int rpi = 32 / n0, ix = lane % n0, r0 = lane / n0;
    if (r0 >= rpi) return;
    const T fxv = fx[ix];
    int iz = r0 / n1, iy = r0 - iz * n1;
    for (int r = r0; r < rows; r += rpi) {
      const T c = cached ? crow[r] : cnt * (fy[iy] * fz[iz]);
      atomicAdd(gbase + ix + sy * iy + sz * iz, to_fixed(c * fxv, fscale));
      iy += rpi;
      while (iy >= n1) {
        iy -= n1;
        ++iz;
      }
    }
  } else {
    for (int r = 0; r < rows; ++r) {
      const int iz = r / n1, iy = r - iz * n1;
      const T c = cached ? crow[r] : cnt * (fy[iy] * fz[iz]);
      for (int ix = lane; ix < n0; ix += 32) atomicAdd(gbase + ix + sy * iy + sz * iz, to_fixed(c * fx[ix], fscale));
    }
  }
}

// density grid = raw scatter / binVolume, and the density at every bin
// (GridProjectedKDE.F90:4662-4667), both from the raw grid
// (and S[S_DMAX] = max density, zeroed before)
// (the raw grid is the fixed-point scatter; inv_scale = 2^-shift)
template <typename T>
__global__ void scale_pick_kernel(KdeParams P, KdeBinsT<T> B, const unsigned long long *raw, double inv_scale,
                                  T *grid, int64_t ngrid, double *S) {
  const int64_t n = ngrid > B.n ? ngrid : (int64_t)B.n;
  const T bv = T(P.binvol);
  // x / binVolume; a power-of-two volume (1 m^3, 0.5 m^3, ...) divides
  // exactly as a product with its reciprocal, which costs one FP64 operation
  // instead of a division's dozen (the host sets inv_binvol only then)
  const bool pow2 = P.inv_binvol != 0.0;
  const T ibv = T(P.inv_binvol);
  auto per_vol = [&](T x) { return pow2 ? x * ibv : x / bv; };
  double dmax = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (i < ngrid) grid[i] = per_vol(T((double)(long long)raw[i] * inv_scale));
    if (i < B.n) {
      const int64_t g = (int64_t)(B.gx[i] - 1) + (int64_t)P.nb[0] * ((B.gy[i] - 1) + (int64_t)P.nb[1] * (B.gz[i] - 1));
      const T d = per_vol(T((double)(long long)raw[g] * inv_scale));
      B.dens[i] = d;
      dmax = fmax(dmax, (double)d);
    }
  }
  warp_max_pos(S + S_DMAX, dmax);
}

template <typename T>
__device__ void support_update(const KdeParams &P, const KdeBinsT<T> &B, int b, T ne1);
template <typename T>
__device__ void curvature_bandwidth(const KdeParams &P, const KdeBinsT<T> &B, int b);

// ---- separable passes -------------------------------------------------------
// The reference folds a kernel that crosses a grid edge back into the grid:
// first the part below cell 1 (mirrored about the lower face), then the part
// above cell n (mirrored about the upper face), and drops what still lies
// outside.  Unfolded kernel position p (1-based) therefore lands on
// reflect_pos(p, n), or nowhere when that is < 1; for kernels narrower than
// the grid this is the plain mirror image.
__device__ __forceinline__ int reflect_pos(int p, int n) {
  if (p < 1) p = 1 - p;
  if (p > n) p = 2 * n + 1 - p;
  return p;
}

__global__ void key_init_kernel(KeyAcc *K) {
  if (threadIdx.x == 0) K->done = 0u;
  for (int k = threadIdx.x; k < KDE_KMAX; k += blockDim.x) {
    K->box[k][0] = K->box[k][2] = K->box[k][4] = INT_MAX;
    K->box[k][1] = K->box[k][3] = K->box[k][5] = INT_MIN;
    K->cnt[k] = 0;
  }
}

// kind 1: the smoothing (sigma) kernel of scale support[b]; its level per
// dimension is non-decreasing in the scale, so the sum of the three levels
// (minus 3, each level is >= 1) identifies the triple.  kind 2: the
// second-derivative kernel of each active axis a from cb[a] (the database is
// isotropic: one level), key a*KDE_MAXDB + level-1; a NaN bandwidth has no
// kernel and is skipped, as the reference's 1-D path does
// (GridProjectedKDE.F90:1723-1724; its 3-D path has no such test and no
// defined kernel for NaN).  Boxes and counts are accumulated per
// block in shared memory and merged into K once per block and key.
__device__ void plan_body(const KdeParams &P, KeyAcc *K, const KdeTable &t0, const KdeTable &t1,
                          const KdeTable &t2, int scatter, SepPlan *pl, int nc, long long cap1, long long cap2,
                          long long *need, double *S, int work_weight);

template <typename T>
__global__ void __launch_bounds__(kThreads) key_assign_kernel(KdeParams P, KdeBinsT<T> B, int kind, int *bin_key,
                                                              KeyAcc *K, KdeTable t0, KdeTable t1, KdeTable t2,
                                                              SepPlan *pl, int nc, long long cap1, long long cap2,
                                                              long long *need, double *S, int work_weight) {
  __shared__ int sb[KDE_KMAX][6];
  __shared__ int sl[KDE_KMAX][3];
  __shared__ int sc[KDE_KMAX];
  for (int k = threadIdx.x; k < KDE_KMAX; k += blockDim.x) {
    sb[k][0] = sb[k][2] = sb[k][4] = INT_MAX;
    sb[k][1] = sb[k][3] = sb[k][5] = INT_MIN;
    sc[k] = 0;
  }
  __syncthreads();
  // Neighbouring bins mostly share a key, so the lanes of a warp with the
  // same key first reduce their bounding box and count among themselves
  // (min, max and count do not depend on the order) and one lane of each
  // group updates the block's shared accumulators.  key < 0: nothing to record.
  auto record = [&](unsigned act, int key, const int lev[3], const int g[3]) {
    const unsigned grp = __match_any_sync(act, key);
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      lo[d] = __reduce_min_sync(grp, g[d]);
      hi[d] = __reduce_max_sync(grp, g[d]);
    }
    if (key < 0 || (int)(threadIdx.x & 31) != __ffs(grp) - 1) return;
    for (int d = 0; d < 3; ++d) {
      atomicMin(&sb[key][2 * d], lo[d]);
      atomicMax(&sb[key][2 * d + 1], hi[d]);
      sl[key][d] = lev[d];  // every bin of the key writes the same levels
    }
    atomicAdd(&sc[key], __popc(grp));
  };
  // The loop runs the same number of times on every lane of a warp (its
  // bound depends on the block, not the lane; blockDim is a multiple of 32),
  // so every lane reaches each record() and the full mask is exact; lanes
  // past the last bin take part with key -1.
  for (int base = blockIdx.x * blockDim.x; base < B.n; base += gridDim.x * blockDim.x) {
    const int b = base + threadIdx.x;
    const bool in = b < B.n;
    const unsigned act = 0xffffffffu;
    const int g[3] = {in ? B.gx[b] : 0, in ? B.gy[b] : 0, in ? B.gz[b] : 0};
    if (kind == 1) {
      int lev[3] = {1, 1, 1};
      int key = -1;
      if (in) {
        const T s = B.support[b];
        for (int d = 0; d < 3; ++d)
          if (P.mask[d]) lev[d] = log_index<T>(P, s, d);
        key = lev[0] + lev[1] + lev[2] - 3;
        bin_key[b] = key;
      }
      record(act, key, lev, g);
    } else {
      // 2-D: a bin with a NaN bandwidth adds to neither curvature
      // (GridProjectedKDE.F90:1967-1968; negative bandwidths are clipped to
      // the minimum before this point)
      // (only the active axes' bandwidths are defined)
      bool skip2 = false;
      if (in && P.ndim == 2)
        for (int a = 0; a < 3; ++a)
          if (P.mask[a]) skip2 = skip2 || !(B.cb[a * B.n + b] == B.cb[a * B.n + b]);
      for (int a = 0; a < 3; ++a) {
        int key = -1;
        int n = 1;
        if (in) {
          const T h = B.cb[a * B.n + b];
          if (P.mask[a] && h == h && !skip2) {
            n = log_index<T>(P, h, a);
            key = a * KDE_MAXDB + n - 1;
          }
          bin_key[a * B.n + b] = key;
        }
        const int lev[3] = {n, n, n};
        record(act, key, lev, g);
      }
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < KDE_KMAX; k += blockDim.x) {
    if (sc[k] == 0) continue;
    for (int d = 0; d < 3; ++d) {
      atomicMin(&K->box[k][2 * d], sb[k][2 * d]);
      atomicMax(&K->box[k][2 * d + 1], sb[k][2 * d + 1]);
      K->lev[k][d] = sl[k][d];
    }
    atomicAdd(&K->cnt[k], sc[k]);
  }
  // The last block to merge lays out the plan (one launch fewer per plan):
  // every thread's merges are made visible device-wide before its block
  // takes a ticket, and the block that takes the last ticket then sees all
  // of them.
  __shared__ unsigned int ticket;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(&K->done, 1u);
  __syncthreads();
  if (ticket != gridDim.x - 1) return;
  __threadfence();
  if (threadIdx.x == 0) K->done = 0u;  // for the next assignment (kernel boundaries order it)
  plan_body(P, K, t0, t1, t2, kind == 2, pl, nc, cap1, cap2, need, S, work_weight);
}

// Compact the keys present and lay out the pass regions, one thread per
// key (a block of kPlanThreads >= KDE_KMAX threads), offsets by a block
// prefix sum in key order.  Gather: pass 1 (x) covers the bins' x range and
// the y, z ranges widened by the half widths; pass 2 (y) the bins' x, y
// ranges and the widened z range; the z pass runs per bin.  Scatter: pass 1
// widens x, pass 2 widens y, the z pass writes the grid over the union
// region of each axis's keys.
constexpr int kPlanThreads = 256;
static_assert(kPlanThreads >= KDE_KMAX, "one plan thread per key");
static_assert(kThreads == kPlanThreads, "the key assignment's last block runs the plan");

// Pass-buffer capacity is checked here, on the device: a plan that needs
// more than cap1 / cap2 elements (nc per region cell) records the sizes it
// needs in need[0..1], sets need[2] and presents no key, so the passes do
// nothing and the host reruns the reconstruction with larger buffers.
// Run by the last block of the key assignment; the accumulators the other
// blocks merged are read through L2.
__device__ void plan_body(const KdeParams &P, KeyAcc *K, const KdeTable &t0, const KdeTable &t1,
                          const KdeTable &t2, int scatter, SepPlan *pl, int nc, long long cap1, long long cap2,
                          long long *need, double *S, int work_weight) {
  __shared__ long long sv1[kPlanThreads], sv2[kPlanThreads];
  __shared__ int sp[kPlanThreads];
  __shared__ int su[3][6];
  const int k = threadIdx.x;
  if (k < 3) {
    su[k][0] = su[k][2] = su[k][4] = INT_MAX;
    su[k][1] = su[k][3] = su[k][5] = INT_MIN;
  }
  const int cntk = k < KDE_KMAX ? __ldcg(&K->cnt[k]) : 0;
  const bool present = cntk > 0;
  int m[3] = {0, 0, 0}, fo[3] = {0, 0, 0}, bx[6], r1[6], r2[6];
  long long v1 = 0, v2 = 0;
  if (present) {
    const int axis = k / KDE_MAXDB;
    const KdeTable T = !scatter ? t0 : (axis == 0 ? t0 : (axis == 1 ? t1 : t2));
    for (int d = 0; d < 3; ++d) {
      const int li = d * KDE_MAXDB + __ldcg(&K->lev[k][d]) - 1;
      m[d] = T.m[li];
      fo[d] = T.ofs[li];
    }
    for (int i = 0; i < 6; ++i) bx[i] = r1[i] = r2[i] = __ldcg(&K->box[k][i]);
    if (!scatter) {
      r1[2] = max(1, bx[2] - m[1]);
      r1[3] = min(P.nb[1], bx[3] + m[1]);
      r1[4] = r2[4] = max(1, bx[4] - m[2]);
      r1[5] = r2[5] = min(P.nb[2], bx[5] + m[2]);
    } else {
      r1[0] = r2[0] = max(1, bx[0] - m[0]);
      r1[1] = r2[1] = min(P.nb[0], bx[1] + m[0]);
      r2[2] = max(1, bx[2] - m[1]);
      r2[3] = min(P.nb[1], bx[3] + m[1]);
    }
    v1 = (long long)(r1[1] - r1[0] + 1) * (r1[3] - r1[2] + 1) * (r1[5] - r1[4] + 1);
    v2 = (long long)(r2[1] - r2[0] + 1) * (r2[3] - r2[2] + 1) * (r2[5] - r2[4] + 1);
    // the work model: this level's bins times its kernel's cells
    if (work_weight > 0)
      atomicAdd(work_counter(S), (unsigned long long)cntk * (unsigned long long)work_weight *
                                     (unsigned long long)((2 * m[0] + 1) * (2 * m[1] + 1) * (2 * m[2] + 1)));
  }
  sp[k] = present ? 1 : 0;
  sv1[k] = v1;
  sv2[k] = v2;
  __syncthreads();
  // inclusive Hillis-Steele scans
  for (int o = 1; o < kPlanThreads; o <<= 1) {
    const int a = (k >= o) ? sp[k - o] : 0;
    const long long b1 = (k >= o) ? sv1[k - o] : 0, b2 = (k >= o) ? sv2[k - o] : 0;
    __syncthreads();
    sp[k] += a;
    sv1[k] += b1;
    sv2[k] += b2;
    __syncthreads();
  }
  if (k < KDE_KMAX) pl->slot_of[k] = present ? sp[k] - 1 : -1;
  if (present) {
    const int j = sp[k] - 1;
    for (int d = 0; d < 3; ++d) {
      pl->m[j][d] = m[d];
      pl->fofs[j][d] = fo[d];
    }
    for (int i = 0; i < 6; ++i) {
      pl->box[j][i] = bx[i];
      pl->r1[j][i] = r1[i];
      pl->r2[j][i] = r2[i];
    }
    pl->o1[j] = sv1[k] - v1;
    pl->o2[j] = sv2[k] - v2;
    pl->key[j] = k;
    if (scatter) {
      const int axis = k / KDE_MAXDB;
      atomicMin(&su[axis][0], r2[0]);
      atomicMax(&su[axis][1], r2[1]);
      atomicMin(&su[axis][2], r2[2]);
      atomicMax(&su[axis][3], r2[3]);
      atomicMin(&su[axis][4], max(1, bx[4] - m[2]));
      atomicMax(&su[axis][5], min(P.nb[2], bx[5] + m[2]));
    }
  }
  // the accumulators of key k were read by thread k only: reset them for the
  // next key_assign (key_init runs once per reconstruction attempt)
  if (k < KDE_KMAX) {
    K->box[k][0] = K->box[k][2] = K->box[k][4] = INT_MAX;
    K->box[k][1] = K->box[k][3] = K->box[k][5] = INT_MIN;
    K->cnt[k] = 0;
  }
  // totals: the inclusive scans end at the last key
  const int np = sp[kPlanThreads - 1];
  const long long tot1 = sv1[kPlanThreads - 1], tot2 = sv2[kPlanThreads - 1];
  __syncthreads();  // su complete
  const bool fits = tot1 * nc <= cap1 && tot2 * nc <= cap2;
  if (k < 3)
    for (int i = 0; i < 6; ++i) pl->ur[k][i] = fits ? su[k][i] : (i & 1 ? INT_MIN : INT_MAX);
  if (k == 0) {
    pl->np = fits ? np : 0;
    pl->tot1 = fits ? tot1 : 0;
    pl->tot2 = fits ? tot2 : 0;
    if (!fits) {
      atomicMax(&need[0], tot1 * nc);
      atomicMax(&need[1], tot2 * nc);
      need[2] = 1;
    }
  }
}

// A 64-bit integer division is a long software sequence on the GPU (longer
// than a pass element's whole tap loop); pass elements and grid cells are
// numbered below 2^31 in practice, where two 32-bit divisions do.
__device__ __forceinline__ void split3(long long i, int nx, int ny, int &a, int &b, int &c) {
  if (i <= 0x7fffffffLL) {
    const unsigned ui = (unsigned)i, q = ui / (unsigned)nx, z = q / (unsigned)ny;
    a = (int)(ui - q * (unsigned)nx);
    b = (int)(q - z * (unsigned)ny);
    c = (int)z;
  } else {
    const long long q = i / nx, z = q / ny;
    a = (int)(i - q * nx);
    b = (int)(q - z * ny);
    c = (int)z;
  }
}

__device__ __forceinline__ void region_xyz(const int r[6], long long i, int &x, int &y, int &z) {
  split3(i, r[1] - r[0] + 1, r[3] - r[2] + 1, x, y, z);
  x += r[0];
  y += r[2];
  z += r[4];
}

__device__ __forceinline__ long long region_vol(const int r[6]) {
  return (long long)(r[1] - r[0] + 1) * (r[3] - r[2] + 1) * (r[5] - r[4] + 1);
}

__device__ __forceinline__ long long region_loc(const int r[6], int x, int y, int z) {
  return (long long)(x - r[0]) + (long long)(r[1] - r[0] + 1) * ((y - r[2]) + (long long)(r[3] - r[2] + 1) * (z - r[4]));
}

// The separable passes index every key's region of one pass buffer with one
// flat index g (the buffer's element): the regions are consecutive in key
// order, region j starting at o[j].  A block copies the offsets to shared
// memory once; each element finds its key by binary search.  All keys share
// the grid, so a key with a large region gets the whole GPU, not a fixed
// number of blocks.
__device__ __forceinline__ int load_offsets(const SepPlan *pl, const long long *o, long long *so) {
  const int np = pl->np;
  for (int j = threadIdx.x; j < np; j += blockDim.x) so[j] = o[j];
  __syncthreads();
  return np;
}

__device__ __forceinline__ int flat_slot(const long long *so, int np, long long g) {
  int lo = 0, hi = np - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (so[mid] <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Gather pass 1: T1 = sum_t fx[t] F(reflect(x - m + t), y, z) over region 1.
// NC = 1: one field; NC = 6: the squared curvatures cx, cy, cz and their
// pairwise products cx*cy, cx*cz, cy*cz (the roughness terms,
// GridProjectedKDE.F90:2470-2600).
template <typename T>
struct Fields {
  const T *f[6];
};

// one element g of pass buffer 1 (the slot offsets in shared memory)
template <typename T, int NC>
__device__ __forceinline__ void gx_element(const KdeParams &P, const SepPlan *pl, const T *val, const Fields<T> &F,
                                           T *T1, const long long *so, int np, long long g) {
  const int n = P.nb[0];
  const int j = flat_slot(so, np, g);
  const long long i = g - so[j];
  const int *r = pl->r1[j];
  const int m = pl->m[j][0];
  const T *f = val + pl->fofs[j][0];
  T *out = T1 + so[j] * NC;
  int x, y, z;
  region_xyz(r, i, x, y, z);
  const long long row = (long long)P.nb[0] * ((y - 1) + (long long)P.nb[1] * (z - 1)) - 1;
  T acc[NC];
  for (int c = 0; c < NC; ++c) acc[c] = T(0);
  if (x - m >= 1 && x + m <= n) {
    // the window misses both edges: a straight loop, two partial sums per
    // field so that the loads run ahead of the multiply-adds
    T acc2[NC];
    for (int c = 0; c < NC; ++c) acc2[c] = T(0);
    const long long base = row + x - m;
    int t = 0;
#pragma unroll 2
    for (; t + 1 <= 2 * m; t += 2) {
      const T w0 = f[t], w1 = f[t + 1];
      for (int c = 0; c < NC; ++c) {
        acc[c] += w0 * F.f[c][base + t];
        acc2[c] += w1 * F.f[c][base + t + 1];
      }
    }
    if (t <= 2 * m)
      for (int c = 0; c < NC; ++c) acc[c] += f[t] * F.f[c][base + t];
    for (int c = 0; c < NC; ++c) acc[c] += acc2[c];
  } else {
    for (int t = 0; t <= 2 * m; ++t) {
      const int p = reflect_pos(x - m + t, n);
      if (p < 1) continue;
      const T w = f[t];
      for (int c = 0; c < NC; ++c) acc[c] += w * F.f[c][row + p];
    }
  }
  for (int c = 0; c < NC; ++c) out[i * NC + c] = acc[c];
}

template <typename T, int NC>
__global__ void gather_x_kernel(KdeParams P, const SepPlan *pl, const T *val, Fields<T> F, T *T1) {
  __shared__ long long so[KDE_KMAX];
  const int np = load_offsets(pl, pl->o1, so);
  const long long tot = pl->tot1;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < tot; g += (long long)gridDim.x * blockDim.x)
    gx_element<T, NC>(P, pl, val, F, T1, so, np, g);
}

// Needed elements only (FP64).  Every key's pass regions are bounding boxes,
// and with many database levels interleaved through a plume each box spans
// the plume, while the z pass reads pass 2 only at the bins' columns within
// mz of the bins (their z windows, folded or not, stay inside them) and the
// y pass reads pass 1 only within my of those elements.  mark_needed_kernel
// and dilate_needed_kernel flag these elements (byte masks over the pass
// buffers' layout), and the masked passes compute only them: each warp
// gathers the flagged elements of its chunks into a shared queue and runs
// them 32 at a time, so the FP64 multiply-adds run on full warps.  Elements
// left unflagged are never read.  On the bench workload the flagged
// elements are ~30 % of pass 1's and ~17 % of pass 2's.
template <typename F>
__device__ __forceinline__ void for_needed(long long tot, const unsigned char *mask, int (*q)[64], F &&visit) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  int cnt = 0;
  for (long long base = ((long long)blockIdx.x * (blockDim.x >> 5) + w) * 32; base < tot; base += nwarps * 32) {
    const long long e = base + lane;
    const bool need = e < tot && mask[e] != 0;
    const unsigned bal = __ballot_sync(0xffffffffu, need);
    if (need) q[w][cnt + __popc(bal & ((1u << lane) - 1u))] = (int)e;
    cnt += __popc(bal);
    __syncwarp();
    if (cnt >= 32) {
      visit((long long)q[w][lane]);
      __syncwarp();
      if (lane < cnt - 32) q[w][lane] = q[w][lane + 32];
      cnt -= 32;
      __syncwarp();
    }
  }
  if (lane < cnt) visit((long long)q[w][lane]);
}

template <typename T, int NC>
__global__ void __launch_bounds__(kThreads) gather_x_masked_kernel(KdeParams P, const SepPlan *pl, const T *val,
                                                                  Fields<T> F, const unsigned char *mask, T *T1) {
  __shared__ long long so[KDE_KMAX];
  __shared__ int q[kThreads / 32][64];
  const int np = load_offsets(pl, pl->o1, so);
  for_needed(pl->tot1, mask, q, [&](long long g) { gx_element<T, NC>(P, pl, val, F, T1, so, np, g); });
}

// flag pass 2's elements at the bins' columns within mz of each bin
template <typename T>
__global__ void mark_needed_kernel(KdeBinsT<T> B, const SepPlan *pl, const int *bin_key, unsigned char *m2) {
  if (pl->np == 0) return;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B.n; b += gridDim.x * blockDim.x) {
    const int j = pl->slot_of[bin_key[b]];
    const int *r2 = pl->r2[j];
    const int mz = pl->m[j][2], bz = B.gz[b];
    const int z0 = max(r2[4], bz - mz), z1 = min(r2[5], bz + mz);
    unsigned char *m = m2 + pl->o2[j];
    for (int z = z0; z <= z1; ++z) m[region_loc(r2, B.gx[b], B.gy[b], z)] = 1;
  }
}

// flag pass 1's elements within my of every flagged element of pass 2
__global__ void dilate_needed_kernel(const SepPlan *pl, const unsigned char *m2, unsigned char *m1) {
  __shared__ long long so[KDE_KMAX];
  const int np = load_offsets(pl, pl->o2, so);
  const long long tot = pl->tot2;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < tot; g += (long long)gridDim.x * blockDim.x) {
    if (!m2[g]) continue;
    const int j = flat_slot(so, np, g);
    const int *r1 = pl->r1[j], *r2 = pl->r2[j];
    int x, y, z;
    region_xyz(r2, g - so[j], x, y, z);
    const int my = pl->m[j][1];
    const int y0 = max(r1[2], y - my), y1 = min(r1[3], y + my);
    unsigned char *m = m1 + pl->o1[j];
    for (int yy = y0; yy <= y1; ++yy) m[region_loc(r1, x, yy, z)] = 1;
  }
}

__global__ void clear_needed_kernel(const SepPlan *pl, unsigned char *m1, unsigned char *m2) {
  const long long t1 = pl->tot1, t2 = pl->tot2;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < t1 || g < t2;
       g += (long long)gridDim.x * blockDim.x) {
    if (g < t1) m1[g] = 0;
    if (g < t2) m2[g] = 0;
  }
}

// 2-D: the product of the two curvatures, then their squares
// (GridProjectedKDE.F90:2134-2138; the 3-D form below squares first)
template <typename T>
__global__ void products2d_kernel(T *c1, T *c2, T *c12, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T a = c1[i], b = c2[i];
    c12[i] = a * b;
    c1[i] = a * a;
    c2[i] = b * b;
  }
}

// pairwise products of the squared curvatures (GridProjectedKDE.F90:2466-2468)
template <typename T>
__global__ void products_kernel(const T *cx, const T *cy, const T *cz, T *cxy, T *cxz, T *cyz, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T a = cx[i], b = cy[i], c = cz[i];
    cxy[i] = a * b;
    cxz[i] = a * c;
    cyz[i] = b * c;
  }
}

// Gather pass 2: T2 = sum_t fy[t] T1(x, reflect(y - m + t), z) over region 2.
template <typename T, int NC>
__device__ __forceinline__ void gy_element(const KdeParams &P, const SepPlan *pl, const T *val, const T *T1, T *T2,
                                           const long long *so, int np, long long g) {
  const int n = P.nb[1];
  const int j = flat_slot(so, np, g);
  const long long i = g - so[j];
  const int *r1 = pl->r1[j], *r2 = pl->r2[j];
  const int m = pl->m[j][1];
  const T *f = val + pl->fofs[j][1];
  const T *in = T1 + pl->o1[j] * NC;
  T *out = T2 + so[j] * NC;
  int x, y, z;
  region_xyz(r2, i, x, y, z);
  T acc[NC];
  for (int c = 0; c < NC; ++c) acc[c] = T(0);
  if (y - m >= 1 && y + m <= n) {
    // interior window (inside region 1 by construction): straight loop
    T acc2[NC];
    for (int c = 0; c < NC; ++c) acc2[c] = T(0);
    const T *src = in + region_loc(r1, x, y - m, z) * NC;
    const long long st = (long long)(r1[1] - r1[0] + 1) * NC;
    int t = 0;
#pragma unroll 2
    for (; t + 1 <= 2 * m; t += 2) {
      const T w0 = f[t], w1 = f[t + 1];
      for (int c = 0; c < NC; ++c) {
        acc[c] += w0 * src[t * st + c];
        acc2[c] += w1 * src[(t + 1) * st + c];
      }
    }
    if (t <= 2 * m)
      for (int c = 0; c < NC; ++c) acc[c] += f[t] * src[t * st + c];
    for (int c = 0; c < NC; ++c) acc[c] += acc2[c];
  } else {
    for (int t = 0; t <= 2 * m; ++t) {
      const int p = reflect_pos(y - m + t, n);
      if (p < 1) continue;
      const T w = f[t];
      const long long l = region_loc(r1, x, p, z) * NC;
      for (int c = 0; c < NC; ++c) acc[c] += w * in[l + c];
    }
  }
  for (int c = 0; c < NC; ++c) out[i * NC + c] = acc[c];
}

template <typename T, int NC>
__global__ void gather_y_kernel(KdeParams P, const SepPlan *pl, const T *val, const T *T1, T *T2) {
  __shared__ long long so[KDE_KMAX];
  const int np = load_offsets(pl, pl->o2, so);
  const long long tot = pl->tot2;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < tot; g += (long long)gridDim.x * blockDim.x)
    gy_element<T, NC>(P, pl, val, T1, T2, so, np, g);
}

template <typename T, int NC>
__global__ void __launch_bounds__(kThreads) gather_y_masked_kernel(KdeParams P, const SepPlan *pl, const T *val,
                                                                  const T *T1, const unsigned char *mask, T *T2) {
  __shared__ long long so[KDE_KMAX];
  __shared__ int q[kThreads / 32][64];
  const int np = load_offsets(pl, pl->o2, so);
  for_needed(pl->tot2, mask, q, [&](long long g) { gy_element<T, NC>(P, pl, val, T1, T2, so, np, g); });
}

// Gather pass 3 at every bin: sum_t fz[t] T2(bx, by, reflect(bz - m + t)).
// NC = 1, mode GZ_OUT: out[b] (and out2[b] when given); GZ_SUPPORT: the
// sigma-support update from this first nEstimate; GZ_NEST: nEstimate, then
// the curvature bandwidths.  NC = 6: the roughness terms and the net
// roughness (GridProjectedKDE.F90:2594-2600).
enum { GZ_OUT = 0, GZ_SUPPORT = 1, GZ_NEST = 2, GZ_NET = 3 };

// GZ_NET (1-D): out[b] = out2[b] = the roughness, which is the net roughness;
// NC = 6 and GZ_NET also fold max(net) and min(net > 0) into S.
// FP32: LPB = 4 lanes per bin split the taps (lane s of the group takes t =
// s, s + 4, ...) and a fixed shuffle tree adds their sums (the same order on
// every run): four times the warps of one thread per bin, whose tap loops
// wait on L2 loads.  FP64: one thread per bin -- the bin's finish (roots and
// quotients) is FP64-pipe work, which must run on full warps.
template <typename T>
constexpr int gz_lanes() { return sizeof(T) == 4 ? 4 : 1; }

template <typename T, int NC>
__global__ void gather_z_kernel(KdeParams P, KdeBinsT<T> B, const SepPlan *pl, const T *val, const int *bin_key,
                                const T *T2, int mode, T *out, T *out2, double *S) {
  constexpr int LPB = gz_lanes<T>();
  const int b = (blockIdx.x * blockDim.x + threadIdx.x) / LPB, sub = threadIdx.x % LPB;
  // np == 0: the plan did not fit, the attempt is discarded
  const bool inb = b < B.n && pl->np != 0;
  double net = 0.0;
  T acc[NC];
  for (int c = 0; c < NC; ++c) acc[c] = T(0);
  if (inb) {
    const int j = pl->slot_of[bin_key[b]];
    const int m = pl->m[j][2], n = P.nb[2];
    const T *f = val + pl->fofs[j][2];
    const int bx = B.gx[b], by = B.gy[b], bz = B.gz[b];
    const int *r2 = pl->r2[j];
    const T *in = T2 + pl->o2[j] * NC;
    for (int t = sub; t <= 2 * m; t += LPB) {
      const int p = reflect_pos(bz - m + t, n);
      if (p < 1) continue;
      const T w = f[t];
      const long long l = region_loc(r2, bx, by, p) * NC;
      for (int c = 0; c < NC; ++c) acc[c] += w * in[l + c];
    }
  }
  if constexpr (LPB > 1) {
    // every lane of the warp takes part (lanes past the last bin add zeros)
    for (int o = 1; o < LPB; o <<= 1)
      for (int c = 0; c < NC; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  }
  const bool valid = inb && sub == 0;
  if (valid) {
    if constexpr (NC == 1) {
      if (mode == GZ_SUPPORT) {
        support_update<T>(P, B, b, acc[0]);
      } else if (mode == GZ_NEST) {
        B.nest[b] = acc[0];
        curvature_bandwidth<T>(P, B, b);
      } else {
        out[b] = acc[0];
        if (out2) out2[b] = acc[0];
        net = (double)acc[0];
      }
    } else if constexpr (NC == 3) {
      // 2-D (GridProjectedKDE.F90:2168-2228): roughness of the two active
      // dimensions and the gathered product of their curvatures
      const T r1 = acc[0], r2 = acc[1], r12 = acc[2];
      T *rr[3] = {B.rxx, B.ryy, B.rzz};
      for (int d = 0; d < 3; ++d) rr[d][b] = T(0);
      rr[P.d1][b] = r1;
      rr[P.d2][b] = r2;
      const T v = P.isotropic ? T(2) * r12 + r1 + r2 : T(2) * r12 + T(2) * sqrt(r1 * r2);
      B.net[b] = v;
      net = (double)v;
    } else {
      const T rxx = acc[0], ryy = acc[1], rzz = acc[2], rxy = acc[3], rxz = acc[4], ryz = acc[5];
      B.rxx[b] = rxx;
      B.ryy[b] = ryy;
      B.rzz[b] = rzz;
      T v;
      if (P.isotropic) {
        // GridProjectedKDE.F90:2675-2676
        v = rxx + T(2) * rxy + T(2) * rxz + ryy + T(2) * ryz + rzz;
      } else {
        // x^(1/3) = cbrt(x), x^(1/6) = cbrt(sqrt(x))
        v = T(3) * cbrt(rxx * ryy * rzz);
        if (ryz > T(0)) v = v + T(2) * ryz * cbrt(sqrt(rxx * rxx / ryy / rzz));
        if (rxz > T(0)) v = v + T(2) * rxz * cbrt(sqrt(ryy * ryy / rxx / rzz));
        if (rxy > T(0)) v = v + T(2) * rxy * cbrt(sqrt(rzz * rzz / rxx / ryy));
      }
      B.net[b] = v;
      net = (double)v;
    }
  }
  if (NC != 1 || mode == GZ_NET) {  // block-uniform: every lane takes part
    warp_max_pos(S + S_NETMAX, net);
    warp_min_pos(S + S_NETMINPOS, net);
  }
}

// Scatter = transpose of the folded gather.  Cell x (1-based, 1..n) receives
// the kernel positions whose fold lands on it: x itself, 1-x (mirrored at the
// lower face), x-2n (mirrored at the lower, then the upper face) and
// 2n+1-x (mirrored at the upper face).  acc += f[t] * V(q + m - t) for each
// such q, V read where it is non-zero: source positions in [lo, hi].
template <typename T>
__device__ __forceinline__ T scatter_taps(const T *f, int m, int x, int n, int lo, int hi, const T *V,
                                          long long stride, long long base, const int *cell_bin, const int *keys,
                                          int key, const double *cnt) {
  const int q4[4] = {x, 1 - x, x - 2 * n, 2 * n + 1 - x};
  T acc = T(0);
  for (int k = 0; k < 4; ++k) {
    const int q = q4[k];
    const int t0 = max(0, q + m - hi), t1 = min(2 * m, q + m - lo);
    for (int t = t0; t <= t1; ++t) {
      const int src = q + m - t;
      const long long l = base + (long long)src * stride;
      T v;
      if (cell_bin) {
        const int cb = cell_bin[l];
        if (cb < 0 || keys[cb] != key) continue;
        v = (T)cnt[cb];
      } else {
        v = V[l];
      }
      acc += f[t] * v;
    }
  }
  return acc;
}

// Scatter pass 1 (x) from the bins of each key (count per bin) over region 1.
template <typename T>
__global__ void scatter_x_kernel(KdeParams P, KdeBinsT<T> B, const SepPlan *pl, const T *val, const int *cell_bin,
                                 const int *bin_key, T *V1) {
  __shared__ long long so[KDE_KMAX];
  const int np = load_offsets(pl, pl->o1, so);
  const long long tot = pl->tot1;
  const int n = P.nb[0];
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < tot; g += (long long)gridDim.x * blockDim.x) {
    const int j = flat_slot(so, np, g);
    const long long i = g - so[j];
    const int *r = pl->r1[j], *bx = pl->box[j];
    const int key = pl->key[j], axis = key / KDE_MAXDB;
    const int *keys = bin_key + (long long)axis * B.n;
    const int m = pl->m[j][0];
    const T *f = val + pl->fofs[j][0];
    int x, y, z;
    region_xyz(r, i, x, y, z);
    const long long row = (long long)P.nb[0] * ((y - 1) + (long long)P.nb[1] * (z - 1)) - 1;
    V1[g] = scatter_taps<T>(f, m, x, n, bx[0], bx[1], nullptr, 1, row, cell_bin, keys, key, B.count);
  }
}

// Scatter pass 2 (y) over region 2.
template <typename T>
__global__ void scatter_y_kernel(KdeParams P, const SepPlan *pl, const T *val, const T *V1, T *V2) {
  __shared__ long long so[KDE_KMAX];
  const int np = load_offsets(pl, pl->o2, so);
  const long long tot = pl->tot2;
  const int n = P.nb[1];
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < tot; g += (long long)gridDim.x * blockDim.x) {
    const int j = flat_slot(so, np, g);
    const long long i = g - so[j];
    const int *r1 = pl->r1[j], *r2 = pl->r2[j];
    const int m = pl->m[j][1];
    const T *f = val + pl->fofs[j][1];
    const T *in = V1 + pl->o1[j];
    const long long sy = r1[1] - r1[0] + 1;
    int x, y, z;
    region_xyz(r2, i, x, y, z);
    const long long base = region_loc(r1, x, r1[2], z) - (long long)r1[2] * sy;
    V2[g] = scatter_taps<T>(f, m, y, n, r1[2], r1[3], in, sy, base, nullptr, nullptr, 0, nullptr);
  }
}

// Scatter pass 3 (z) of every key of one axis into that axis's curvature
// grid (zeroed before; only the union of the keys' output regions is
// written), keys in increasing order, then the normalisation
// (c / binVolume) / binSize^2 (GridProjectedKDE.F90:2366-2461), squared
// when `square` (1-D and 3-D; the 2-D form multiplies the curvatures first).
template <typename T>
__global__ void scatter_z_kernel(KdeParams P, const SepPlan *pl, const T *val, const T *V2, T *c0, T *c1, T *c2,
                                 int square) {
  const int axis = blockIdx.y;
  T *out = axis == 0 ? c0 : (axis == 1 ? c1 : c2);
  const T bs2 = T(P.bin[axis] * P.bin[axis]), bv = T(P.binvol);
  int u[6];
  for (int i = 0; i < 6; ++i) u[i] = pl->ur[axis][i];
  // an inactive axis, or one without keys, keeps a zero grid
  const bool any = P.mask[axis] && u[0] <= u[1];
  const long long ngrid = (long long)P.nb[0] * P.nb[1] * P.nb[2];
  const int np = pl->np, n = P.nb[2];
  // this axis's keys (consecutive slots: a key is axis * KDE_MAXDB + level
  // and the slots are in key order) staged in shared memory once per block
  __shared__ int s_r2[KDE_MAXDB][6], s_m[KDE_MAXDB], s_f[KDE_MAXDB];
  __shared__ long long s_o2[KDE_MAXDB];
  __shared__ int s_j0, s_nk;
  if (threadIdx.x == 0) {
    int j0 = 0;
    while (j0 < np && pl->key[j0] < axis * KDE_MAXDB) ++j0;
    int j1 = j0;
    while (j1 < np && pl->key[j1] < (axis + 1) * KDE_MAXDB) ++j1;
    s_j0 = j0;
    s_nk = j1 - j0;
  }
  __syncthreads();
  const int nk = s_nk;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) {
    const int j = s_j0 + k;
    for (int i = 0; i < 6; ++i) s_r2[k][i] = pl->r2[j][i];
    s_m[k] = pl->m[j][2];
    s_f[k] = pl->fofs[j][2];
    s_o2[k] = pl->o2[j];
  }
  __syncthreads();
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ngrid; g += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    split3(g, P.nb[0], P.nb[1], x, y, z);
    ++x;
    ++y;
    ++z;
    if (!any || x < u[0] || x > u[1] || y < u[2] || y > u[3] || z < u[4] || z > u[5]) {
      out[g] = T(0);
      continue;
    }
    T acc = T(0);
    for (int k = 0; k < nk; ++k) {
      const int *r2 = s_r2[k];
      if (x < r2[0] || x > r2[1] || y < r2[2] || y > r2[3]) continue;
      const int m = s_m[k];
      if (z < r2[4] - m || z > r2[5] + m) continue;
      const long long sz = (long long)(r2[1] - r2[0] + 1) * (r2[3] - r2[2] + 1);
      const long long base = region_loc(r2, x, y, r2[4]) - (long long)r2[4] * sz;
      acc += scatter_taps<T>(val + s_f[k], m, z, n, r2[4], r2[5], V2 + s_o2[k], sz, base, nullptr, nullptr, 0,
                             nullptr);
    }
    T c = acc / bv;
    c = c / bs2;
    out[g] = square ? c * c : c;
  }
}

template <typename T>
__device__ __forceinline__ T smoothing_scale(const KdeParams &P, const T ks[3]) {
  T out = T(1);
  int dimc = P.ndim;
  for (int d = 0; d < 3; ++d) {
    if (!P.mask[d]) continue;
    if (ks[d] != T(0)) out = out * ks[d];
    else dimc = dimc - 1;
  }
  return (dimc != 0) ? pow_inv_nd<T>(out, P.ndim) : T(0);
}

template <typename T>
__global__ void init_bins_kernel(KdeParams P, KdeBinsT<T> B, double hs, double *S) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b == 0) {
    S[S_DMAX] = 0.0;
    S[S_WORK] = 0.0;
  }
  if (b >= B.n) return;
  T ks[3];
  for (int d = 0; d < 3; ++d) ks[d] = P.mask[d] ? T(hs) : T(0);
  const T sc = smoothing_scale<T>(P, ks);
  B.scale[b] = sc;
  B.support[b] = T(2) * sc;
  for (int d = 0; d < 3; ++d) {
    B.ks[d * B.n + b] = ks[d];
    B.shape[d * B.n + b] = (P.mask[d] && sc > T(0)) ? ks[d] / sc : T(0);
  }
  B.nest[b] = T(0);
  B.net[b] = T(0);
}

// second-half of the sigma-support update (GridProjectedKDE.F90:4836-4860)
template <typename T>
__device__ void support_update(const KdeParams &P, const KdeBinsT<T> &B, int b, T ne1) {
  const T dn = B.dens[b];
  // nEstimate**0.5: the correctly rounded square root (as the C library's pow)
  T ssc = sqrt(ne1) * pow_one_plus_nd_q<T>(B.scale[b], P.ndim) / root4<T>(T(4) * dn) * T(P.support_c);
  const T grow = T(P.max_sigma_growth) * B.support[b];
  if (ssc > grow) ssc = grow;
  ssc = fmin(ssc, T(P.max_k[P.max_dim]));
  if (ssc < T(P.min_k[P.min_dim])) ssc = T(P.min_k[P.min_dim]);
  B.support[b] = ssc;
}

// prComputeCurvatureKernelBandwidth (GridProjectedKDE.F90:5207-5275);
// nEstimate**fTWO is the product nEstimate*nEstimate, as Fortran compiles it
template <typename T>
__device__ void curvature_bandwidth(const KdeParams &P, const KdeBinsT<T> &B, int b) {
  T nvpb = T(0);
  const T dn = B.dens[b];
  if (dn > T(0)) {
    const T base = T(SQRT8PI_D) * B.support[b];
    T p = T(1);
    for (int k = 0; k < P.ndim; ++k) p = (k == 0) ? base : p * base;  // integer power, left to right
    if (P.ndim == 3) p = base * (base * base);
    const T ne = B.nest[b];
    nvpb = pow_beta<T>(p * (ne * ne) / dn, P.ndim, P.beta_c);
  }
  for (int d = 0; d < 3; ++d) {
    if (!P.mask[d]) continue;
    T tsum = T(0);
    for (int k = 0; k < 3; ++k) {
      if (!P.mask[k]) continue;
      const T sh = B.shape[k * B.n + b];
      if (sh != T(0)) tsum = tsum + (k == d ? T(5) : T(1)) / (sh * sh);
    }
    const T shd = B.shape[d * B.n + b];
    T term = T(0);
    const T sh2 = shd * shd;
    if (shd != T(0)) term = pow_minus_one_over_nd6<T>((T(P.one_over_nd4) / (sh2 * sh2)) * tsum, P.ndim,
                                                      P.minus_one_over_nd6);
    T c = T(P.alpha_c) * nvpb * term * B.scale[b];
    if (c > T(P.max_sd[d])) c = T(P.max_sd[d]);
    if (c < T(P.min_sd[d])) c = T(P.min_sd[d]);
    B.cb[d * B.n + b] = c;
  }
}

// Per-bin sums of the optimisation loop, in FP64 and in two stages with a
// fixed order (per-block partials, then one warp), results in the device
// scalars S:
//   RED_END:    S[S_ERRD], S[S_ERRS] = sums of the squared relative density
//               and smoothing changes (GridProjectedKDE.F90:4976-5000, with
//               S[S_DMAX], S[S_DMAXOLD]), and S[S_ALMISE]
//   RED_ALMISE: S[S_ALMISE] = sum of the squared ALMISE terms (4966-4972)
// (the maxima and minima are folded into the kernels that produce them)
constexpr int kRedBlocks = 152;
enum { RED_END = 1, RED_ALMISE = 3 };

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// npts2: nPoints**fTWO, which Fortran evaluates as the product nPoints*nPoints

template <typename T>
__global__ void __launch_bounds__(kThreads) bin_reduce_kernel(KdeParams P, KdeBinsT<T> B, int what, double npts2,
                                                              const double *S, double *partial) {
  __shared__ double red[kThreads / 32][3];
  double a[3] = {0.0, 0.0, 0.0};
  const double mx = S[S_DMAX], mx_old = S[S_DMAXOLD];
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B.n; b += gridDim.x * blockDim.x) {
    if (what == RED_END) {
      const double dn = (double)B.dens[b], dold = (double)B.dens_old[b];
      if (dold != 0.0) {
        const double e = fabs(dn / mx - dold / mx_old) / (dold / mx_old);
        a[0] += e * e;
      }
      const double so = (double)B.scale_old[b], sc = (double)B.scale[b];
      if (so != 0.0) {
        const double e = fabs(sc - so) / so;
        a[1] += e * e;
      }
    }
    const T sc = B.scale[b];
    if (sc != T(0)) {
      const T sc2 = sc * sc;
      const T scn = P.ndim == 3 ? sc2 * sc : (P.ndim == 2 ? sc2 : sc);
      const T e = (B.nest[b] / (scn * T(P.four_pi_half_nd)) + T(0.25) * B.net[b] * (sc2 * sc2)) / T(npts2);
      a[2] += (double)e * (double)e;
    }
  }
  for (int k = 0; k < 3; ++k) a[k] = warp_sum(a[k]);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 3; ++k) red[w][k] = a[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 3; ++k) {
      double v = red[0][k];
      for (int i = 1; i < kThreads / 32; ++i) v = v + red[i][k];
      partial[3 * blockIdx.x + k] = v;
    }
  }
}

// one warp: lane l folds partials l, l+32, ... then a shuffle tree
__global__ void bin_reduce_final_kernel(int what, int nblk, const double *partial, double *S) {
  const int l = threadIdx.x;
  double a[3] = {0.0, 0.0, 0.0};
  for (int i = l; i < nblk; i += 32)
    for (int k = 0; k < 3; ++k) a[k] = a[k] + partial[3 * i + k];
  for (int k = 0; k < 3; ++k) a[k] = warp_sum(a[k]);
  if (l != 0) return;
  if (what == RED_END) {
    S[S_ERRD] = a[0];
    S[S_ERRS] = a[1];
  }
  S[S_ALMISE] = a[2];
}

// prComputeOptimalSmoothingAndShape, per bin (GridProjectedKDE.F90:5404-5724).
// phase 0: isotropy correction of the net roughness + scale where net > 0.
// (and S[S_SCMAX] = max positive scale, for the bins with zero net roughness)
template <typename T>
__global__ void optimal_phase0_kernel(KdeParams P, KdeBinsT<T> B, double *S, int *flag) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b == 0) *flag = 0;  // read by optimal_phase1 / rescale, which run after this kernel
  double scv = 0.0;
  if (b < B.n) {
    const T min_pos_net = T(S[S_NETMINPOS]);
    const T nd = T(P.ndim), iso = T(P.iso_threshold);
    T net = B.net[b];
    if (P.ndim == 3 && !P.isotropic) {
      T sm = B.rxx[b] + B.ryy[b] + B.rzz[b];
      if (sm == T(0)) sm = min_pos_net;
      if ((B.rxx[b] / sm > iso) || (B.ryy[b] / sm > iso) || (B.rzz[b] / sm > iso))
        net = (T(1) - T(0.5)) * net + T(0.5) * sm;
      B.net[b] = net;
    } else if (P.ndim == 2 && !P.isotropic) {
      const T *rr[3] = {B.rxx, B.ryy, B.rzz};
      const T r1 = rr[P.d1][b], r2 = rr[P.d2][b];
      T sm = r1 + r2;
      if (sm == T(0)) sm = min_pos_net;
      if ((r1 / sm > iso) || (r2 / sm > iso)) net = (T(1) - T(0.5)) * net + T(0.5) * sm;
      B.net[b] = net;
    }
    T sc = T(0);
    if (net > T(0)) sc = pow_one_over_nd4<T>(nd * B.nest[b] / (T(P.four_pi_half_nd) * net), P.ndim, P.one_over_nd4);
    B.scale[b] = sc;
    scv = (double)sc;
  }
  warp_max_pos(S + S_SCMAX, scv);
}

// phase 1: scale for zero net roughness, shapes, bounded smoothing
template <typename T>
__global__ void optimal_phase1_kernel(KdeParams P, KdeBinsT<T> B, const double *S, int *update_flag) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B.n) return;
  const T max_pos_scale = T(S[S_SCMAX]);
  T sc = B.scale[b];
  if (B.net[b] == T(0)) {
    sc = max_pos_scale;
    B.scale[b] = sc;
  }
  T sh[3] = {T(1), T(1), T(1)};
  if (P.ndim == 2 && !P.isotropic) {
    // bounded kernels (GridProjectedKDE.F90:5557-5578)
    const T *rr[3] = {B.rxx, B.ryy, B.rzz};
    const T r1 = rr[P.d1][b], r2 = rr[P.d2][b], net = B.net[b];
    if (!(r1 == T(0) || r2 == T(0))) {
      const T s1 = fmax(sqrt(sqrt(sqrt(net / r1))), T(P.min_k[P.d1]) / sc);  // ^(1/8)
      const T s2 = T(1) / s1;
      const T ns = sqrt(s1 * s2);
      if (ns != T(0)) {
        sh[P.d1] = s1 / ns;
        sh[P.d2] = s2 / ns;
      }
    }
  }
  if (P.ndim == 3 && !P.isotropic) {
    const T rxx = B.rxx[b], ryy = B.ryy[b], rzz = B.rzz[b], net = B.net[b];
    if (!(rxx == T(0) || ryy == T(0) || rzz == T(0))) {
      // ^(1/12) = cbrt(sqrt(sqrt()))
      const T s1 = fmax(cbrt(root4<T>(net / rxx)), T(P.min_k[0]) / sc);
      const T s2 = fmax(cbrt(root4<T>(net / ryy)), T(P.min_k[1]) / sc);
      const T s3 = T(1) / s1 / s2;
      // the reference's exponent is the single-precision literal 0.333
      const T ns = pow_general<T>(s1 * s2 * s3, T(0.333f));
      if (ns != T(0)) {
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
      B.ks[d * B.n + b] = T(0);
      continue;
    }
    T k = sh[d] * sc;
    if (k > T(P.max_k[d])) {
      k = T(P.max_k[d]);
      upd = true;
    }
    if (k < T(P.min_k[d])) {
      k = T(P.min_k[d]);
      upd = true;
    }
    B.ks[d * B.n + b] = k;
  }
  if (upd) atomicOr(update_flag, 1);
}

// phase 2: smoothing scale from the bounded smoothing (all bins)
template <typename T>
__global__ void rescale_kernel(KdeParams P, KdeBinsT<T> B, const int *update_flag) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B.n || *update_flag == 0) return;
  T ks[3] = {B.ks[b], B.ks[B.n + b], B.ks[2 * B.n + b]};
  B.scale[b] = smoothing_scale<T>(P, ks);
}

// start of an optimisation loop: previous density and smoothing scale, the
// previous maximum density, and the extremes the loop accumulates reset
template <typename T>
__global__ void loop_init_kernel(KdeBinsT<T> B, double *S) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < B.n) {
    B.dens_old[b] = B.dens[b];
    B.scale_old[b] = B.scale[b];
  }
  if (b == 0) {
    S[S_DMAXOLD] = S[S_DMAX];
    S[S_DMAX] = 0.0;
    S[S_NETMAX] = 0.0;
    S[S_NETMINPOS] = DBL_MAX;
    S[S_SCMAX] = 0.0;
  }
}

// the exported density: grid * effective-mass factor * (binVolume, scaling
// factor) in FP64 (GridProjectedKDE.F90:4292-4306)
template <typename T>
__global__ void output_kernel(const T *grid, double *out, int64_t n, double f, double scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = ((double)grid[i] * f) * scale;
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

constexpr int kCompactChunk = 4096;  // cells per block of kThreads threads, 16 per thread

__global__ void active_write_kernel(const double *counts, int64_t nbins, const int *blockofs, KdeParams P, KdeBins B,
                                    int *cell_bin) {
  __shared__ int sc[kThreads];
  constexpr int per = kCompactChunk / kThreads;
  const int t = threadIdx.x;
  const int64_t beg = (int64_t)blockIdx.x * kCompactChunk + (int64_t)t * per;
  int c = 0;
  for (int i = 0; i < per; ++i) {
    const int64_t g = beg + i;
    c += (g < nbins && counts[g] != 0.0);
  }
  sc[t] = c;
  __syncthreads();
  for (int o = 1; o < kThreads; o <<= 1) {
    const int a = (t >= o) ? sc[t - o] : 0;
    __syncthreads();
    sc[t] += a;
    __syncthreads();
  }
  int o = blockofs[blockIdx.x] + sc[t] - c;
  for (int i = 0; i < per; ++i) {
    const int64_t g = beg + i;
    if (g >= nbins) break;
    const double v = counts[g];
    if (v == 0.0) continue;
    int ix, iy, iz;
    split3(g, P.nb[0], P.nb[1], ix, iy, iz);
    B.gx[o] = ix + 1;
    B.gy[o] = iy + 1;
    B.gz[o] = iz + 1;
    B.count[o] = v;
    cell_bin[g] = o;
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
                 bins.dens, bins.cb, bins.rxx, bins.ryy, bins.rzz, bins.net, bins.dens_old, bins.scale_old,
                 partial, bin_key};
  for (void *p : old)
    if (p) cudaFree(p);
  bins = KdeBins{};
  partial = nullptr;
  bin_key = nullptr;
  cap = 0;
  // a quarter of headroom: a spreading plume activates more bins at almost
  // every reconstruction, and each regrowth frees and allocates ~20 arrays
  // (cudaFree synchronises the device)
  const size_t c = (size_t)n + (size_t)n / 4;
  cudaError_t e = cudaSuccess;
  auto I = [&](int **p, size_t k) {
    if (e == cudaSuccess) e = cudaMalloc((void **)p, sizeof(int) * k);
  };
  auto D = [&](double **p, size_t k) {
    if (e == cudaSuccess) e = cudaMalloc((void **)p, sizeof(double) * k);
  };
  I(&bins.gx, c); I(&bins.gy, c); I(&bins.gz, c); I(&bin_key, 4 * c);
  D(&bins.count, c); D(&bins.ks, 3 * c); D(&bins.scale, c); D(&bins.shape, 3 * c); D(&bins.support, c);
  D(&bins.nest, c); D(&bins.dens, c); D(&bins.cb, 3 * c); D(&bins.rxx, c); D(&bins.ryy, c); D(&bins.rzz, c);
  D(&bins.net, c); D(&bins.dens_old, c); D(&bins.scale_old, c);
  D(&partial, 3 * 152 * 8 + 16);
  if (e != cudaSuccess) return e;
  cap = (int)std::min<size_t>(c, (size_t)INT_MAX);
  bins.n = n;
  return cudaSuccess;
}

cudaError_t KdeState::ensure_grid(int64_t ngrid) {
  if (!d_scalars) {
    cudaError_t e = cudaMalloc((void **)&d_scalars, 32 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_wcnt, 64 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&h_scalars, 96 * sizeof(double));  // + the 64 counters
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_flag, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_keys, sizeof(KeyAcc));
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_plan, 2 * sizeof(SepPlan));
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_need, 4 * sizeof(long long));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&h_need, 4 * sizeof(long long));
    if (e != cudaSuccess) return e;
  }
  if (ngrid <= grid_cap) return cudaSuccess;
  double **grids[] = {&dens_grid, &dens_raw, &cx, &cy, &cz, &cxy, &cxz, &cyz, &dens_out};
  for (double **p : grids) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  if (d_blockcnt) cudaFree(d_blockcnt);
  if (cell_bin) cudaFree(cell_bin);
  d_blockcnt = cell_bin = nullptr;
  grid_cap = 0;
  cudaError_t e = cudaSuccess;
  for (double **p : grids)
    if (e == cudaSuccess) e = cudaMalloc((void **)p, sizeof(double) * ngrid);
  if (e == cudaSuccess) e = cudaMalloc((void **)&cell_bin, sizeof(int) * ngrid);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_blockcnt, sizeof(int) * ((ngrid + 4095) / 4096 + 1));
  if (e != cudaSuccess) return e;
  grid_cap = ngrid;
  return cudaSuccess;
}

cudaError_t KdeState::ensure_pass(int64_t n1, int64_t n2) {
  if (n1 > t1_cap) {
    if (t1) cudaFree(t1);
    if (need1) cudaFree(need1);
    t1 = nullptr;
    need1 = nullptr;
    t1_cap = 0;
    const int64_t c = n1 + n1 / 4;
    cudaError_t e = cudaMalloc((void **)&t1, sizeof(double) * c);
    if (e == cudaSuccess) e = cudaMalloc((void **)&need1, c);
    if (e != cudaSuccess) return e;
    t1_cap = c;
  }
  if (n2 > t2_cap) {
    if (t2) cudaFree(t2);
    if (need2) cudaFree(need2);
    t2 = nullptr;
    need2 = nullptr;
    t2_cap = 0;
    const int64_t c = n2 + n2 / 4;
    cudaError_t e = cudaMalloc((void **)&t2, sizeof(double) * c);
    if (e == cudaSuccess) e = cudaMalloc((void **)&need2, c);
    if (e != cudaSuccess) return e;
    t2_cap = c;
  }
  return cudaSuccess;
}

void KdeState::release() {
  void *ptrs[] = {bins.gx, bins.gy, bins.gz, bins.count, bins.ks, bins.scale, bins.shape, bins.support, bins.nest,
                  bins.dens, bins.cb, bins.rxx, bins.ryy, bins.rzz, bins.net, bins.dens_old, bins.scale_old,
                  partial, dens_grid, cx, cy, cz, d_scalars, d_flag, d_blockcnt, d_val, d_valf, d_meta, cell_bin,
                  bin_key, d_keys, d_plan, t1, t2, need1, need2, d_wcnt, dens_raw, d_need, cxy, cxz, cyz, dens_out};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (h_scalars) cudaFreeHost(h_scalars);
  if (h_need) cudaFreeHost(h_need);
  if (h_out) cudaFreeHost(h_out);
  if (body_exec) cudaGraphExecDestroy(body_exec);
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

// The optimisation loop on the device.  The loop body is the body of a
// while node of a CUDA graph; its last kernel (one thread) takes the host
// loop's convergence decision from the device scalars -- the same FP64
// operations in the same order, each correctly rounded, so the same decision
// -- and sets the node's condition.  The host reads the outcome once, after
// the last loop, instead of synchronising on every loop.  Control slots of
// the device scalars (after S_COUNT):
enum { C_ALMOLD = 16, C_CUM = 17, C_CUMOLD = 18, C_LOOPS = 19, C_STATUS = 20 };
// C_STATUS: 0 ran to convergence or to the loop limit, 1 a plan did not fit
// its pass buffers (the attempt is discarded), 2 the net roughness is zero
// everywhere (the reference stops, GridProjectedKDE.F90:5443-5446)

__global__ void loop_ctl_init_kernel(double *S, unsigned long long *wcnt, int nb) {
  *work_counter(S) = 0ull;
  for (int k = 0; k < 64; ++k) wcnt[k] = 0ull;
  const double alm = sqrt(S[S_ALMISE] / nb);
  S[C_ALMOLD] = alm;
  S[C_CUM] = alm;
  S[C_CUMOLD] = alm;
  S[C_LOOPS] = 0.0;
  S[C_STATUS] = 0.0;
}

// GridProjectedKDE.F90:5000-5040: the convergence tests after a loop
__global__ void loop_ctl_kernel(double *S, const long long *need, int nb, int n_opt_loops, double rel_err,
                                int skip_error, cudaGraphConditionalHandle cond) {
  const int m = (int)S[C_LOOPS] + 1;
  S[C_LOOPS] = (double)m;
  unsigned cont = 1;
  if (need[2] != 0) {
    S[C_STATUS] = 1.0;
    cont = 0;
  } else if (S[S_NETMAX] == 0.0) {
    S[C_STATUS] = 2.0;
    cont = 0;
  } else {
    const double err_dens = sqrt(S[S_ERRD] / nb), err_smooth = sqrt(S[S_ERRS] / nb);
    const double alm = sqrt(S[S_ALMISE] / nb);
    const double cum = S[C_CUM] + alm;
    const double alm_old = S[C_ALMOLD], cum_old = S[C_CUMOLD];
    S[C_CUM] = cum;
    bool stop = false;
    if (!skip_error) {
      if (alm_old > 0.0 && fabs(alm - alm_old) / alm_old < rel_err) stop = true;
      else if (err_dens < rel_err) stop = true;
      else if (err_smooth < rel_err) stop = true;
      else if (m > 7 && fabs(cum_old / (double)(m - 1) - cum / (double)m) / cum_old / (double)(m - 1) < rel_err)
        stop = true;
    }
    if (stop || m >= n_opt_loops) {
      cont = 0;
    } else {
      S[C_ALMOLD] = alm;
      S[C_CUMOLD] = cum;
    }
  }
  cudaGraphSetConditional(cond, cont);
}

__global__ void zero_u64_kernel(unsigned long long *a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = 0ull;
}

// the work model after the loops: the plans' count plus the scatters' 64
// counters (copied to h + 32 with the last read of the scalars, or here)
static cudaError_t read_work(KdeState &st, double *h, cudaStream_t s, bool copied) {
  if (!copied) {
    KCK(cudaMemcpyAsync(h + 32, st.d_wcnt, 64 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    KCK(cudaStreamSynchronize(s));
  }
  unsigned long long t = *reinterpret_cast<const unsigned long long *>(h + S_WORK);
  const unsigned long long *w = reinterpret_cast<const unsigned long long *>(h + 32);
  for (int k = 0; k < 64; ++k) t += w[k];
  st.work_madds = (double)t;
  return cudaSuccess;
}

// The executable graph of the host-driven loop's body.  A batch's workers
// run one reconstruction after another, each capturing the same kernels in
// the same order (the same options) with new pointers, sizes and grids: the
// executable graph kept from the previous one is updated in place, which
// skips the instantiation, the costly step.  A capture of another topology
// (another precision or dimension) is instantiated afresh.  No launch of the
// kept graph is in flight here: every reconstruction ends with a stream
// synchronisation.  (The device loop's graph is instantiated every time: its
// loop-control kernel sets the conditional handle of its own capture.)
static cudaGraphExec_t body_exec_for(KdeState &st, cudaGraph_t g) {
  if (st.body_exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(st.body_exec, g, &info) == cudaSuccess) return st.body_exec;
    (void)cudaGetLastError();
    cudaGraphExecDestroy(st.body_exec);
    st.body_exec = nullptr;
  }
  if (cudaGraphInstantiate(&st.body_exec, g, 0) != cudaSuccess) {
    (void)cudaGetLastError();
    st.body_exec = nullptr;
  }
  return st.body_exec;
}

// One reconstruction attempt in arithmetic type T; *overflow is set when a
// plan found the pass buffers too small (the sizes it needed are in st.h_need).
template <typename T>
static cudaError_t kde_attempt(KdeState &st, const KdeParams &P, double hs, double npts, int n_opt_loops,
                               double rel_err, bool skip_error, cudaStream_t s, int *loops_done, bool *overflow) {
  const KdeBinsT<T> B = st.view<T>();
  const int nb = B.n;
  const int64_t ngrid = (int64_t)P.nb[0] * P.nb[1] * P.nb[2];
  const int bb = (nb + kBinThreads - 1) / kBinThreads;
  const int gzb = (int)(((long long)nb * gz_lanes<T>() + kBinThreads - 1) / kBinThreads);
  const int gb = blocks_for(ngrid);
  const int rb = std::min(blocks_for(nb), kRedBlocks);
  const int kb = std::min((nb + kThreads - 1) / kThreads, 2 * kRedBlocks);
  const int64_t npick = ngrid > nb ? ngrid : nb;
  double *S = st.d_scalars, *h = st.h_scalars;
  *overflow = false;
  // typed views of the grids and pass buffers, the factor values
  T *dens_grid = reinterpret_cast<T *>(st.dens_grid);
  T *cx = reinterpret_cast<T *>(st.cx), *cy = reinterpret_cast<T *>(st.cy), *cz = reinterpret_cast<T *>(st.cz);
  T *cxy = reinterpret_cast<T *>(st.cxy), *cxz = reinterpret_cast<T *>(st.cxz), *cyz = reinterpret_cast<T *>(st.cyz);
  T *t1 = reinterpret_cast<T *>(st.t1), *t2 = reinterpret_cast<T *>(st.t2);
  const T *val = std::is_same<T, double>::value ? reinterpret_cast<const T *>(st.d_val)
                                                : reinterpret_cast<const T *>(st.d_valf);
  const KdeTableT<T> wtab{val, st.wtab.m, st.wtab.ofs};
  // a stride near n/61 coprime with n (a permutation of the bins)
  int wstride = nb / 61 + 1;
  while (std::gcd(wstride, nb) != 1) ++wstride;
  // fixed-point scale of the density scatter: the total count is at most
  // npts (the active particles), and npts * 2^shift < 2^62
  int shift = 61;
  {
    int e = 0;
    std::frexp(std::max(npts, 1.0), &e);  // npts < 2^e
    shift = 61 - e;
  }
  const double fscale = std::ldexp(1.0, shift), inv_fscale = std::ldexp(1.0, -shift);
  unsigned long long *raw_fixed = reinterpret_cast<unsigned long long *>(st.dens_raw);
  auto density = [&](void) -> cudaError_t {
    zero_u64_kernel<<<blocks_for(ngrid), kThreads, 0, s>>>(raw_fixed, ngrid);
    wscatter_kernel<T><<<(nb + kWarpsW - 1) / kWarpsW, 32 * kWarpsW, 0, s>>>(P, B, wtab, wstride, T(fscale),
                                                                            raw_fixed, st.d_wcnt);
    scale_pick_kernel<T><<<blocks_for(npick), kThreads, 0, s>>>(P, B, raw_fixed, inv_fscale, dens_grid, ngrid, S);
    st.launches += 3;
    return cudaGetLastError();
  };
  // plans: [0] smoothing kernels (kind 1), [1] second-derivative kernels (kind 2)
  SepPlan *plan1 = st.d_plan, *plan2 = st.d_plan + 1;
  int *key1 = st.bin_key, *key2 = st.bin_key + nb;
  // about one block per 20 active bins (a pass covers ~10-25 elements per
  // bin), a multiple of the SM count: a small reconstruction (a batch's
  // small members) does not pay for the prologue of blocks that find no work
  const dim3 pgrid(std::min(kPassBlocks, std::max(152, (nb / 20 + 151) / 152 * 152)));
  // work_weight: the smoothing kernels of the nEstimate plan count eight
  // times (support update, nEstimate, six roughness terms), the second
  // derivatives once, the support plan's not at all
  auto plan = [&](int kind, int nc, int work_weight) -> cudaError_t {
    if (kind == 1)
      key_assign_kernel<T><<<kb, kThreads, 0, s>>>(P, B, kind, key1, st.d_keys, st.wtab, st.wtab, st.wtab, plan1, nc,
                                                   st.t1_cap, st.t2_cap, st.d_need, S, work_weight);
    else
      key_assign_kernel<T><<<kb, kThreads, 0, s>>>(P, B, kind, key2, st.d_keys, st.sdtab[0], st.sdtab[1],
                                                   st.sdtab[2], plan2, nc, st.t1_cap, st.t2_cap, st.d_need, S,
                                                   work_weight);
    st.launches += 1;
    return cudaGetLastError();
  };
  // FP64: the gathers compute only the pass elements that are read (the
  // masks follow each smoothing-kernel plan); their element numbers must fit
  // an int (the pass capacity bounds them)
  const bool masked = sizeof(T) == 8 && st.t1_cap < (int64_t)INT_MAX && st.t2_cap < (int64_t)INT_MAX;
  auto needed = [&](void) -> cudaError_t {
    if (!masked) return cudaSuccess;
    clear_needed_kernel<<<pgrid, kThreads, 0, s>>>(plan1, st.need1, st.need2);
    mark_needed_kernel<T><<<bb, kBinThreads, 0, s>>>(B, plan1, key1, st.need2);
    dilate_needed_kernel<<<pgrid, kThreads, 0, s>>>(plan1, st.need2, st.need1);
    st.launches += 3;
    return cudaGetLastError();
  };
  auto gather_xy = [&](auto nc_tag, Fields<T> F) -> cudaError_t {
    constexpr int NC = decltype(nc_tag)::value;
    if (masked) {
      gather_x_masked_kernel<T, NC><<<pgrid, kThreads, 0, s>>>(P, plan1, val, F, st.need1, t1);
      gather_y_masked_kernel<T, NC><<<pgrid, kThreads, 0, s>>>(P, plan1, val, t1, st.need2, t2);
    } else {
      gather_x_kernel<T, NC><<<pgrid, kThreads, 0, s>>>(P, plan1, val, F, t1);
      gather_y_kernel<T, NC><<<pgrid, kThreads, 0, s>>>(P, plan1, val, t1, t2);
    }
    return cudaGetLastError();
  };
  // sum over every bin's smoothing kernel of `field`, at the bins
  auto gather1 = [&](const T *field, int mode, T *out, T *out2) -> cudaError_t {
    KCK(gather_xy(std::integral_constant<int, 1>{}, Fields<T>{{field}}));
    gather_z_kernel<T, 1><<<gzb, kBinThreads, 0, s>>>(P, B, plan1, val, key1, t2, mode, out, out2, S);
    st.launches += 3;
    return cudaGetLastError();
  };
  auto reduce = [&](int what) -> cudaError_t {
    bin_reduce_kernel<T><<<rb, kThreads, 0, s>>>(P, B, what, npts * npts, S, st.partial);
    bin_reduce_final_kernel<<<1, 32, 0, s>>>(what, rb, st.partial, S);
    st.launches += 2;
    return cudaGetLastError();
  };
  auto fetch_async = [&](void) -> cudaError_t {
    KCK(cudaMemcpyAsync(h, S, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
    return cudaMemcpyAsync(st.h_need, st.d_need, 3 * sizeof(long long), cudaMemcpyDeviceToHost, s);
  };
  auto fetch_wait = [&](void) -> cudaError_t {
    KCK(cudaStreamSynchronize(s));
    *overflow = st.h_need[2] != 0;
    return cudaSuccess;
  };
  // One optimisation loop (GridProjectedKDE.F90:4700-5040) up to the
  // convergence measures, which it copies to the host.  It starts by saving
  // the previous density and smoothing scale (the reference does that at the
  // end of a loop that did not converge; nothing runs in between).  Every
  // data-dependent choice inside is taken on the device, so one captured
  // graph replays every loop.
  auto body_core = [&](void) -> cudaError_t {
    loop_init_kernel<T><<<bb, kBinThreads, 0, s>>>(B, S);
    st.launches += 1;
    // nEstimate with the current support, support update, nEstimate again
    // and the curvature bandwidths
    KCK(plan(1, 1, 0));
    KCK(needed());
    KCK(gather1(dens_grid, GZ_SUPPORT, nullptr, nullptr));
    KCK(plan(1, P.ndim == 3 ? 6 : (P.ndim == 2 ? 3 : 1), 8));
    KCK(needed());
    KCK(gather1(dens_grid, GZ_NEST, nullptr, nullptr));
    // curvatures: second-derivative scatters of the counts, squared (every
    // cell of the three grids is written, zero outside the keys' regions)
    KCK(plan(2, 1, 1));
    scatter_x_kernel<T><<<pgrid, kThreads, 0, s>>>(P, B, plan2, val, st.cell_bin, key2, t1);
    scatter_y_kernel<T><<<pgrid, kThreads, 0, s>>>(P, plan2, val, t1, t2);
    scatter_z_kernel<T><<<dim3(gb, 3), kThreads, 0, s>>>(P, plan2, val, t2, cx, cy, cz, P.ndim != 2);
    st.launches += 3;
    // net roughness: smoothing-kernel gathers of the squared curvatures
    if (P.ndim == 2) {
      T *cg[3] = {cx, cy, cz};
      T *c1 = cg[P.d1], *c2 = cg[P.d2];
      products2d_kernel<T><<<gb, kThreads, 0, s>>>(c1, c2, cxy, ngrid);
      KCK(gather_xy(std::integral_constant<int, 3>{}, Fields<T>{{c1, c2, cxy}}));
      gather_z_kernel<T, 3><<<gzb, kBinThreads, 0, s>>>(P, B, plan1, val, key1, t2, GZ_OUT, nullptr, nullptr, S);
      st.launches += 4;
    } else if (P.ndim == 3) {
      products_kernel<T><<<gb, kThreads, 0, s>>>(cx, cy, cz, cxy, cxz, cyz, ngrid);
      KCK(gather_xy(std::integral_constant<int, 6>{}, Fields<T>{{cx, cy, cz, cxy, cxz, cyz}}));
      gather_z_kernel<T, 6><<<gzb, kBinThreads, 0, s>>>(P, B, plan1, val, key1, t2, GZ_OUT, nullptr, nullptr, S);
      st.launches += 4;
    } else {
      int a = 0;
      while (!P.mask[a]) ++a;
      T *cg[3] = {cx, cy, cz};
      T *r1 = (a == 0) ? B.rxx : (a == 1 ? B.ryy : B.rzz);
      KCK(gather1(cg[a], GZ_NET, r1, B.net));
    }
    // optimal smoothing and shape; the extremes stay on the device
    optimal_phase0_kernel<T><<<bb, kBinThreads, 0, s>>>(P, B, S, st.d_flag);
    optimal_phase1_kernel<T><<<bb, kBinThreads, 0, s>>>(P, B, S, st.d_flag);
    rescale_kernel<T><<<bb, kBinThreads, 0, s>>>(P, B, st.d_flag);
    st.launches += 3;
    // density with the new smoothing, then the convergence measures
    KCK(density());
    return reduce(RED_END);
  };
  auto body = [&](void) -> cudaError_t {
    KCK(body_core());
    return fetch_async();
  };
  KCK(cudaMemsetAsync(st.d_need, 0, 3 * sizeof(long long), s));
  key_init_kernel<<<1, kThreads, 0, s>>>(st.d_keys);
  init_bins_kernel<T><<<bb, kBinThreads, 0, s>>>(P, B, hs, S);
  st.launches += 2;
  KCK(density());
  KCK(reduce(RED_ALMISE));  // nEstimate and net roughness are zero: 0
  if (n_opt_loops > 0 && st.device_loop) {
    // the whole loop as one graph: a while node around the captured body (a
    // while node runs its body at least once: no loops are the host path's)
    cudaGraphExec_t dexec = nullptr;
    int64_t dbody = 0;
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) == cudaSuccess) {
      cudaGraphConditionalHandle cond;
      cudaGraphNode_t node;
      cudaGraphNodeParams cp{};
      cp.type = cudaGraphNodeTypeConditional;
      if (cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) == cudaSuccess) {
        cp.conditional.handle = cond;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) == cudaSuccess &&
            cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
          const int64_t l0 = st.launches;
          cudaError_t eb = body_core();
          if (eb == cudaSuccess) {
            loop_ctl_kernel<<<1, 1, 0, s>>>(S, st.d_need, nb, n_opt_loops, rel_err, skip_error ? 1 : 0, cond);
            eb = cudaGetLastError();
          }
          cudaGraph_t out = nullptr;
          const cudaError_t ee = cudaStreamEndCapture(s, &out);
          dbody = st.launches - l0 + 1;
          st.launches = l0;
          if (eb == cudaSuccess && ee == cudaSuccess && cudaGraphInstantiate(&dexec, g, 0) != cudaSuccess)
            dexec = nullptr;
        }
      }
      cudaGraphDestroy(g);
    }
    (void)cudaGetLastError();  // a failed construction leaves no sticky error
    if (dexec) {
      struct ExecGuard {
        cudaGraphExec_t e;
        ~ExecGuard() { cudaGraphExecDestroy(e); }
      } guard{dexec};
      loop_ctl_init_kernel<<<1, 1, 0, s>>>(S, st.d_wcnt, nb);
      KCK(cudaGetLastError());
      KCK(cudaGraphLaunch(dexec, s));
      KCK(cudaMemcpyAsync(h, S, 32 * sizeof(double), cudaMemcpyDeviceToHost, s));
      KCK(cudaMemcpyAsync(st.h_need, st.d_need, 3 * sizeof(long long), cudaMemcpyDeviceToHost, s));
      KCK(cudaMemcpyAsync(h + 32, st.d_wcnt, 64 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
      KCK(cudaStreamSynchronize(s));
      const int loops = (int)h[C_LOOPS];
      st.launches += 1 + dbody * loops;
      if (h[C_STATUS] == 1.0) {
        *overflow = true;
        return cudaSuccess;
      }
      if (h[C_STATUS] == 2.0) return cudaErrorInvalidValue;
      if (loops_done) *loops_done = loops;
      KCK(read_work(st, h, s, true));
      return cudaGetLastError();
    }
  }
  // the loop driven from the host (a stream that cannot be captured)
  KCK(cudaMemsetAsync(S + S_WORK, 0, sizeof(double), s));
  KCK(cudaMemsetAsync(st.d_wcnt, 0, 64 * sizeof(unsigned long long), s));
  KCK(fetch_async());
  KCK(fetch_wait());
  double alm = std::sqrt(h[S_ALMISE] / nb);
  double alm_old = alm, cum = alm, cum_old = alm;
  // capture the loop body once; a stream that cannot be captured (the legacy
  // default stream) runs it directly
  cudaGraphExec_t exec = nullptr;
  int64_t body_launches = 0;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    const int64_t l0 = st.launches;
    const cudaError_t eb = body();
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(s, &g);
    body_launches = st.launches - l0;
    st.launches = l0;
    if (eb == cudaSuccess && ee == cudaSuccess && g) exec = body_exec_for(st, g);
    if (g) cudaGraphDestroy(g);
    (void)cudaGetLastError();  // a failed capture leaves no sticky error
  } else {
    (void)cudaGetLastError();  // the stream cannot be captured: run the body directly
  }
  int m = 0;
  for (m = 1; m <= n_opt_loops; ++m) {
    if (exec) {
      KCK(cudaGraphLaunch(exec, s));
      st.launches += body_launches;
    } else {
      KCK(body());
    }
    KCK(fetch_wait());
    if (*overflow) return cudaSuccess;
    // maxval(netRoughness) == 0: the reference stops (GridProjectedKDE.F90:5443-5446)
    if (h[S_NETMAX] == 0.0) return cudaErrorInvalidValue;
    const double err_dens = std::sqrt(h[S_ERRD] / nb), err_smooth = std::sqrt(h[S_ERRS] / nb);
    alm = std::sqrt(h[S_ALMISE] / nb);
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
  }
  if (loops_done) *loops_done = (m > n_opt_loops) ? n_opt_loops : m;
  KCK(read_work(st, h, s, false));
  return cudaGetLastError();
}

// The pass buffers start small and grow: an attempt whose plans did not fit
// is discarded and the reconstruction restarts from the histogram with the
// buffers the plans asked for (every attempt re-derives all per-bin state,
// so the result does not depend on how many attempts ran).
cudaError_t kde_run(KdeState &st, const KdeParams &P, double hs, double npts, int n_opt_loops, double rel_err,
                    bool skip_error, int fp32, cudaStream_t s, int *loops_done) {
  const int64_t ngrid = (int64_t)P.nb[0] * P.nb[1] * P.nb[2];
  // eight grid volumes of the six roughness fields: enough for most plumes
  KCK(st.ensure_pass(48 * ngrid, 48 * ngrid));
  for (int attempt = 0; attempt < 8; ++attempt) {
    bool overflow = false;
    if (fp32)
      KCK(kde_attempt<float>(st, P, hs, npts, n_opt_loops, rel_err, skip_error, s, loops_done, &overflow));
    else
      KCK(kde_attempt<double>(st, P, hs, npts, n_opt_loops, rel_err, skip_error, s, loops_done, &overflow));
    if (!overflow) return cudaSuccess;
    // what a discarded attempt asked for is a lower bound: grow geometrically
    KCK(st.ensure_pass(std::max<int64_t>(st.h_need[0], 2 * st.t1_cap), std::max<int64_t>(st.h_need[1], 2 * st.t2_cap)));
  }
  return cudaErrorMemoryAllocation;
}

cudaError_t kde_output(KdeState &st, const KdeParams &P, int fp32, double f, double scale, cudaStream_t s) {
  const int64_t ngrid = (int64_t)P.nb[0] * P.nb[1] * P.nb[2];
  if (fp32)
    output_kernel<float><<<blocks_for(ngrid), kThreads, 0, s>>>(reinterpret_cast<const float *>(st.dens_grid),
                                                                 st.dens_out, ngrid, f, scale);
  else
    output_kernel<double><<<blocks_for(ngrid), kThreads, 0, s>>>(st.dens_grid, st.dens_out, ngrid, f, scale);
  st.launches += 1;
  return cudaGetLastError();
}

cudaError_t kde_collect_active(KdeState &st, const KdeParams &P, const double *counts, cudaStream_t s, int *nactive) {
  const int64_t ngrid = (int64_t)P.nb[0] * P.nb[1] * P.nb[2];
  const int chunk = kCompactChunk;
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
  KCK(cudaMemsetAsync(st.cell_bin, 0xff, sizeof(int) * ngrid, s));  // -1: no active bin
  active_write_kernel<<<nblk, kThreads, 0, s>>>(counts, ngrid, d_cnt, P, st.bins, st.cell_bin);
  st.launches += 2;
  KCK(cudaGetLastError());
  return cudaStreamSynchronize(s);  // the offsets vector goes out of scope
}

}  // namespace mprw
