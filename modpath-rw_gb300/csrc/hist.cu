// hist.cu -- model coordinates of particles and the GPKDE histogram.
//
// global_xyz restates ConvertToModelXYZ (ModflowRectangularGrid.f90:524-548).
// The histogram restates Histogram%ComputeCountsWeighted
// (lib/gpkde/Histogram.F90:276-350): bin = floor((x - origin)/binSize) + 1 on
// every active dimension (bin size non-zero), points outside [1, nBins] are
// dropped, counts accumulate the particle weights.  With unit weights the
// counts are integers, accumulated here with 32-bit integer atomics
// (privatised in shared memory when the grid is small), so the result is
// bit-identical to the reference's sequential floating-point sum.
#include "mprw_kernels.cuh"

namespace mprw {

template <typename R>
__device__ __forceinline__ void model_xyz(const Geometry &geo, int32_t c, R lx, R ly, R lz, double &X,
                                          double &Y, double &Z) {
  const GridDims g = geo.g;
  c -= geo.cell0;
  int k = c / g.ncpl;
  int r = c - k * g.ncpl;
  int i = r / g.ncol;
  int j = r - i * g.ncol;
  (void)k;
  double x = (double)lx, y = (double)ly, z = (double)lz;
  double left = geo.col_left[j], right = geo.col_right[j];
  double front = geo.row_front[i], back = geo.row_back[i];
  double bottom = geo.botm[c], top = geo.sattop[c];
  X = ((1.0 - x) * left) + (x * right);
  if (X < left) X = left;
  if (X > right) X = right;
  Y = ((1.0 - y) * front) + (y * back);
  if (Y < front) Y = front;
  if (Y > back) Y = back;
  Z = ((1.0 - z) * bottom) + (z * top);
  if (Z < bottom) Z = bottom;
  if (Z > top) Z = top;
}

template <typename R>
__global__ void global_xyz_kernel(Geometry geo, int64_t n, const int32_t *cell, const R *x, const R *y,
                                  const R *z, double *gx, double *gy, double *gz) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    double X, Y, Z;
    model_xyz<R>(geo, cell[p], x[p], y[p], z[p], X, Y, Z);
    gx[p] = X;
    gy[p] = Y;
    gz[p] = Z;
  }
}

template <typename R>
cudaError_t launch_global_xyz(const Geometry &geo, int64_t n, const int32_t *cell, const R *x, const R *y,
                              const R *z, double *gx, double *gy, double *gz, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int threads = 256;
  int64_t blocks = (n + threads - 1) / threads;
  if (blocks > 152 * 32) blocks = 152 * 32;
  global_xyz_kernel<R><<<(int)blocks, threads, 0, s>>>(geo, n, cell, x, y, z, gx, gy, gz);
  return cudaGetLastError();
}
template cudaError_t launch_global_xyz<double>(const Geometry &, int64_t, const int32_t *, const double *,
                                               const double *, const double *, double *, double *, double *,
                                               cudaStream_t);
template cudaError_t launch_global_xyz<float>(const Geometry &, int64_t, const int32_t *, const float *,
                                              const float *, const float *, double *, double *, double *,
                                              cudaStream_t);

// Per-block sums over the active particles of the model coordinates
// (pass 0: x, y, z, count) or of squared deviations from `mean` (pass 1);
// the host adds the block partials in order.
template <typename R>
__global__ void coord_sums_kernel(Geometry geo, int64_t n, const int32_t *cell, const int32_t *status, const R *x,
                                  const R *y, const R *z, int pass, double m0, double m1, double m2, double *partial) {
  __shared__ double red[4][32];
  double a[4] = {0, 0, 0, 0};
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    if (status[p] != ST_ACTIVE) continue;
    double X, Y, Z;
    model_xyz<R>(geo, cell[p], x[p], y[p], z[p], X, Y, Z);
    if (pass == 0) {
      a[0] += X; a[1] += Y; a[2] += Z; a[3] += 1.0;
    } else if (pass == 2) {  // centred on (m0, m1, m2)
      a[0] += X - m0; a[1] += Y - m1; a[2] += Z - m2; a[3] += 1.0;
    } else {
      a[0] += (X - m0) * (X - m0); a[1] += (Y - m1) * (Y - m1); a[2] += (Z - m2) * (Z - m2);
    }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int k = 0; k < 4; ++k) {
    double v = a[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (l == 0) red[k][w] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 4; ++k) {
      double s = 0.0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[k][i];
      partial[4 * blockIdx.x + k] = s;
    }
  }
}

cudaError_t launch_coord_sums(const Geometry &geo, int64_t n, const int32_t *cell, const int32_t *status,
                              const void *x, const void *y, const void *z, int mixed, int pass, const double mean[3],
                              double *partial, int *nblocks, cudaStream_t s) {
  const int threads = 256;
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 4) b = 152 * 4;
  if (b < 1) b = 1;
  *nblocks = (int)b;
  if (mixed)
    coord_sums_kernel<float><<<(int)b, threads, 0, s>>>(geo, n, cell, status, (const float *)x, (const float *)y,
                                                         (const float *)z, pass, mean[0], mean[1], mean[2], partial);
  else
    coord_sums_kernel<double><<<(int)b, threads, 0, s>>>(geo, n, cell, status, (const double *)x, (const double *)y,
                                                          (const double *)z, pass, mean[0], mean[1], mean[2], partial);
  return cudaGetLastError();
}

// bin index (0-based linear, x fastest) of an active particle, or -1
template <typename R>
__device__ __forceinline__ int64_t bin_index(const HistArgs &a, int64_t p) {
  if (a.status[p] != ST_ACTIVE) return -2;
  double X[3];
  model_xyz<R>(a.geo, a.cell[p], ((const R *)a.x)[p], ((const R *)a.y)[p], ((const R *)a.z)[p], X[0], X[1], X[2]);
  int64_t idx[3] = {0, 0, 0};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (!a.active_dim[d]) continue;
    double q = floor((X[d] - a.origin[d]) / a.bin[d]);
    if (!(q >= 0.0 && q < (double)a.nb[d])) return -1;
    idx[d] = (int64_t)q;
  }
  return idx[0] + (int64_t)a.nb[0] * (idx[1] + (int64_t)a.nb[1] * idx[2]);
}

template <typename R, bool SMEM>
__global__ void hist_unit_kernel(HistArgs a, int64_t nbins) {
  extern __shared__ unsigned int sh[];
  if (SMEM) {
    for (int64_t b = threadIdx.x; b < nbins; b += blockDim.x) sh[b] = 0;
    __syncthreads();
  }
  unsigned long long mine = 0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.n; p += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = bin_index<R>(a, p);
    if (b < 0) continue;
    ++mine;
    if (SMEM) atomicAdd(&sh[b], 1u);
    else atomicAdd(&a.counts32[b], 1u);
  }
  // warp-reduce the binned count
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(a.nbinned, mine);
  if (SMEM) {
    __syncthreads();
    for (int64_t b = threadIdx.x; b < nbins; b += blockDim.x)
      if (sh[b]) atomicAdd(&a.counts32[b], sh[b]);
  }
}

template <typename R>
__global__ void hist_bins_kernel(HistArgs a) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.n; p += (int64_t)gridDim.x * blockDim.x)
    a.bin_of[p] = bin_index<R>(a, p);
}

static int hist_blocks(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 8) b = 152 * 8;
  if (b < 1) b = 1;
  return (int)b;
}

cudaError_t launch_hist_unit(const HistArgs &a, cudaStream_t s) {
  int64_t nbins = (int64_t)a.nb[0] * a.nb[1] * a.nb[2];
  const int threads = 512;
  int blocks = hist_blocks(a.n, threads);
  bool smem = nbins * 4 <= 48 * 1024;
  size_t sb = smem ? (size_t)nbins * 4 : 0;
  if (a.mixed) {
    if (smem) hist_unit_kernel<float, true><<<blocks, threads, sb, s>>>(a, nbins);
    else hist_unit_kernel<float, false><<<blocks, threads, 0, s>>>(a, nbins);
  } else {
    if (smem) hist_unit_kernel<double, true><<<blocks, threads, sb, s>>>(a, nbins);
    else hist_unit_kernel<double, false><<<blocks, threads, 0, s>>>(a, nbins);
  }
  return cudaGetLastError();
}

cudaError_t launch_hist_bins(const HistArgs &a, cudaStream_t s) {
  const int threads = 256;
  int blocks = hist_blocks(a.n, threads);
  if (a.mixed) hist_bins_kernel<float><<<blocks, threads, 0, s>>>(a);
  else hist_bins_kernel<double><<<blocks, threads, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void u32_to_f64_kernel(const unsigned int *in, double *out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}

cudaError_t launch_u32_to_f64(const unsigned int *in, double *out, int64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  u32_to_f64_kernel<<<hist_blocks(n, 256), 256, 0, s>>>(in, out, n);
  return cudaGetLastError();
}

}  // namespace mprw
