// sort.cu -- radix sorts used around the hot path (CUB, header-only part of
// the CUDA toolkit):
//   * sort_cells: particle processing order by cell, so the warps of the step
//     kernel read neighbouring cell records; with the passes of the previous
//     interval known, heaviest first in buckets of kPassBucket passes (cell
//     order within a bucket), so the persistent kernel's queue does not end on
//     a few long particles;
//   * ordered_bin_sums: per-bin sums of non-unit particle weights in particle
//     order, bit-identical to the reference's sequential loop
//     (Histogram.F90:302-325) together with the sequential totals
//     sum(weights) and sum(weights**2) (Histogram.F90:328-340).
#include <cub/device/device_radix_sort.cuh>

#include "mprw_kernels.cuh"

namespace mprw {

static cudaError_t ensure(void **buf, size_t *have, size_t need) {
  if (*have >= need) return cudaSuccess;
  if (*buf) cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  size_t grow = need + need / 4 + 1024;
  cudaError_t e = cudaMalloc(buf, grow);
  if (e == cudaSuccess) *have = grow;
  return e;
}

__global__ void iota_keys_kernel(const int32_t *cell, uint32_t *keys, uint32_t *vals, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    keys[i] = (uint32_t)cell[i];
    vals[i] = (uint32_t)i;
  }
}

// keys (15 - bucket of the previous interval's passes, cell): passes are the
// random-counter increments over `unit` (counter blocks per pass times the
// bucket width)
__global__ void lpt_keys_kernel(const int32_t *cell, const uint64_t *ctr, const uint64_t *ctr_prev, uint64_t unit,
                                int ncell_bits, uint32_t *keys, uint32_t *vals, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t d = (ctr[i] >= ctr_prev[i]) ? ctr[i] - ctr_prev[i] : 0;
    const uint64_t b = d / unit;
    const uint32_t bucket = (b > (uint64_t)kPassBuckets - 1) ? (uint32_t)kPassBuckets - 1 : (uint32_t)b;
    keys[i] = (((uint32_t)kPassBuckets - 1 - bucket) << ncell_bits) | (uint32_t)cell[i];
    vals[i] = (uint32_t)i;
  }
}

static int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return b < 1 ? 1 : (int)b;
}

cudaError_t sort_cells(const int32_t *cell, const uint64_t *ctr, const uint64_t *ctr_prev, uint64_t ctr_per_pass,
                       uint32_t *perm, int64_t n, int ncell_bits, void **scratch, size_t *scratch_bytes,
                       cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  // pass buckets only when the key still fits 32 bits
  const bool lpt = ctr && ctr_prev && ctr_per_pass > 0 && ncell_bits + kPassBucketBits <= 32;
  const int bits = lpt ? ncell_bits + kPassBucketBits : ncell_bits;
  size_t temp = 0;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, temp, (const uint32_t *)nullptr, (uint32_t *)nullptr,
                                                  (const uint32_t *)nullptr, (uint32_t *)nullptr, (int)n, 0,
                                                  bits, s);
  if (e != cudaSuccess) return e;
  size_t arr = ((size_t)n * 4 + 255) / 256 * 256;
  e = ensure(scratch, scratch_bytes, 3 * arr + temp);
  if (e != cudaSuccess) return e;
  char *b = (char *)*scratch;
  uint32_t *kin = (uint32_t *)b, *kout = (uint32_t *)(b + arr), *vin = (uint32_t *)(b + 2 * arr);
  void *tmp = b + 3 * arr;
  if (lpt)
    lpt_keys_kernel<<<grid_for(n), 256, 0, s>>>(cell, ctr, ctr_prev, ctr_per_pass * (uint64_t)kPassBucket,
                                                ncell_bits, kin, vin, n);
  else
    iota_keys_kernel<<<grid_for(n), 256, 0, s>>>(cell, kin, vin, n);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cub::DeviceRadixSort::SortPairs(tmp, temp, kin, kout, vin, perm, (int)n, 0, bits, s);
}

__global__ void ordered_keys_kernel(const int64_t *bin_of, int64_t n, unsigned long long *keys) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = bin_of[i];
    keys[i] = (b >= 0) ? (((unsigned long long)b << 32) | (unsigned long long)i) : ~0ULL;
  }
}

// each segment head sums its bin's weights in particle order
__global__ void segment_sum_kernel(const unsigned long long *keys, int64_t n, const double *mass, double *counts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long k = keys[i];
    if (k == ~0ULL) continue;
    unsigned long long bin = k >> 32;
    if (i > 0 && (keys[i - 1] >> 32) == bin && keys[i - 1] != ~0ULL) continue;
    double acc = 0.0;
    for (int64_t j = i; j < n; ++j) {
      unsigned long long kj = keys[j];
      if (kj == ~0ULL || (kj >> 32) != bin) break;
      acc = acc + mass[kj & 0xffffffffULL];
    }
    counts[bin] = acc;
  }
}

// sequential totals over the active particles, in particle order
__global__ void sequential_totals_kernel(const double *mass, const int32_t *status, int64_t n, double *out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double tot = 0.0, sw2 = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    if (status[i] != ST_ACTIVE) continue;
    double w = mass[i];
    tot = tot + w;
    sw2 = sw2 + w * w;
  }
  out[0] = tot;
  out[1] = sw2;
}

cudaError_t ordered_bin_sums(const int64_t *bin_of, const double *mass, const int32_t *status, int64_t n,
                             int64_t nbins, double *counts, double *total_mass, double *sum_w2, void **scratch,
                             size_t *scratch_bytes, cudaStream_t s) {
  size_t temp = 0;
  cudaError_t e = cub::DeviceRadixSort::SortKeys(nullptr, temp, (const unsigned long long *)nullptr,
                                                 (unsigned long long *)nullptr, (int)n, 0, 64, s);
  if (e != cudaSuccess) return e;
  size_t arr = ((size_t)n * 8 + 255) / 256 * 256;
  e = ensure(scratch, scratch_bytes, 2 * arr + temp + 256);
  if (e != cudaSuccess) return e;
  char *b = (char *)*scratch;
  unsigned long long *kin = (unsigned long long *)b, *kout = (unsigned long long *)(b + arr);
  double *tot = (double *)(b + 2 * arr);
  void *tmp = b + 2 * arr + 256;
  e = cudaMemsetAsync(counts, 0, sizeof(double) * (size_t)nbins, s);
  if (e != cudaSuccess) return e;
  if (n > 0) {
    ordered_keys_kernel<<<grid_for(n), 256, 0, s>>>(bin_of, n, kin);
    e = cub::DeviceRadixSort::SortKeys(tmp, temp, kin, kout, (int)n, 0, 64, s);
    if (e != cudaSuccess) return e;
    segment_sum_kernel<<<grid_for(n), 256, 0, s>>>(kout, n, mass, counts);
  }
  sequential_totals_kernel<<<1, 1, 0, s>>>(mass, status, n, tot);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(total_mass, tot, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(sum_w2, tot + 1, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

}  // namespace mprw
