// noalloc.cu -- an allocation-free histogram entry point.
//
// Some callers cannot allocate device memory at the point where they need a
// histogram: a host code that owns a fixed device-memory budget and hands out
// only pre-sized buffers, a caller running inside a memory-pool or real-time
// section where cudaMalloc would synchronise the device or fail, or an
// embedding that forbids library-side allocations altogether.  For them,
// mprw_histogram_noalloc takes device pointers to its inputs and output and
// keeps its only scratch -- 32-bit bin counters plus the binned-particle
// counter -- in a file-scope device array of fixed size, so it never calls
// cudaMalloc, cudaFree or an allocating library routine.
//
// The array (MPRW_NOALLOC_MAX_BINS + 2 words, 4 MiB + 8 B) is part of the
// library image: every GPU that loads the library holds it until the process
// exits.  All calls share it and it keeps the last call's contents, so each
// call clears what it uses before counting, and calls that overlap on the GPU
// (different streams, or host threads, without ordering) race on it.
#include <mutex>

#include "../../include/mprw_gpu.h"
#include "mprw_common.cuh"

namespace {

constexpr int64_t kMaxBins = MPRW_NOALLOC_MAX_BINS;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned int g_noalloc_scratch[kMaxBins + 2];

// Device address of g_noalloc_scratch per device.  The host-side name is a
// stand-in, not a device address, so it is looked up once per device with that
// device current (the first call on each device does this set-up).
unsigned int *g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

cudaError_t scratch_for_current_device(unsigned int **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<unsigned int *>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

struct Bins {
  double origin[3], bin[3];
  int32_t nb[3];
  int active[3];
};

// Histogram%ComputeCounts on model coordinates (Histogram.F90:213-273):
// bin = floor((x - origin)/binSize) on every dimension with a non-zero bin
// size, points outside the grid skipped; only ACTIVE particles count.
__global__ void noalloc_count_kernel(const double *gx, const double *gy, const double *gz, const int32_t *status,
                                     int64_t n, Bins B, unsigned int *counts, unsigned int *nbinned) {
  unsigned int mine = 0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    if (status[p] != mprw::ST_ACTIVE) continue;
    const double X[3] = {gx[p], gy[p], gz[p]};
    int64_t idx[3] = {0, 0, 0};
    bool inside = true;
    for (int d = 0; d < 3; ++d) {
      if (!B.active[d]) continue;
      const double q = floor((X[d] - B.origin[d]) / B.bin[d]);
      if (!(q >= 0.0 && q < (double)B.nb[d])) {
        inside = false;
        break;
      }
      idx[d] = (int64_t)q;
    }
    if (!inside) continue;
    atomicAdd(&counts[idx[0] + (int64_t)B.nb[0] * (idx[1] + (int64_t)B.nb[1] * idx[2])], 1u);
    ++mine;
  }
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(nbinned, mine);
}

__global__ void noalloc_clear_kernel(unsigned int *s, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s[i] = 0u;
}

__global__ void noalloc_out_kernel(const unsigned int *counts, int64_t nbins, const unsigned int *nbinned,
                                   double *out, int64_t *nbinned_out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nbins; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)counts[i];
  if (nbinned_out && blockIdx.x == 0 && threadIdx.x == 0) *nbinned_out = (int64_t)*nbinned;
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  return b < 1 ? 1 : (int)b;
}

}  // namespace

extern "C" int mprw_histogram_noalloc(const double *gx, const double *gy, const double *gz, const int32_t *status,
                                      int64_t n, const double origin[3], const double bin_size[3],
                                      const int32_t n_bins[3], double *counts, int64_t *n_binned,
                                      void *stream) {
  if (n < 0 || !origin || !bin_size || !n_bins || !counts) return MPRW_E_INVAL;
  if (n > 0 && (!gx || !gy || !gz || !status)) return MPRW_E_INVAL;
  Bins B;
  int64_t nbins = 1;
  for (int d = 0; d < 3; ++d) {
    if (n_bins[d] < 1 || bin_size[d] < 0.0) return MPRW_E_INVAL;
    nbins *= n_bins[d];
    if (nbins > kMaxBins) return MPRW_E_INVAL;  // beyond the fixed scratch: prod(n_bins) <= MPRW_NOALLOC_MAX_BINS
    B.origin[d] = origin[d];
    B.bin[d] = bin_size[d];
    B.nb[d] = n_bins[d];
    B.active[d] = bin_size[d] != 0.0;
  }
  unsigned int *scratch = nullptr;
  if (scratch_for_current_device(&scratch) != cudaSuccess) return MPRW_E_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned int *nb_counter = scratch + kMaxBins;
  noalloc_clear_kernel<<<grid_for(nbins), 256, 0, s>>>(scratch, nbins);
  noalloc_clear_kernel<<<1, 32, 0, s>>>(nb_counter, 1);
  if (n > 0) noalloc_count_kernel<<<grid_for(n), 256, 0, s>>>(gx, gy, gz, status, n, B, scratch, nb_counter);
  noalloc_out_kernel<<<grid_for(nbins), 256, 0, s>>>(scratch, nbins, nb_counter, counts, n_binned);
  return cudaGetLastError() == cudaSuccess ? MPRW_OK : MPRW_E_CUDA;
}
