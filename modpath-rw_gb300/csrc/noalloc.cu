// noalloc.cu -- an allocation-free histogram entry point.
//
// Some callers cannot allocate device memory at the point where they need a
// histogram: a host code that owns a fixed device-memory budget and hands out
// only pre-sized buffers, a caller running inside a memory-pool or real-time
// section where cudaMalloc would synchronise the device or fail, or an
// embedding that forbids library-side allocations altogether.  For them,
// mprw_histogram_noalloc takes device pointers to its inputs and output and
// keeps its only scratch -- 32-bit bin counters plus a 64-bit binned-particle
// counter -- in a file-scope device array of fixed size, so it never calls
// cudaMalloc, cudaFree or an allocating library routine.
//
// The array (MPRW_NOALLOC_MAX_BINS + 2 32-bit words, 4 MiB + 8 B; the last
// two words are the 8-byte-aligned binned-particle counter) is part of the
// library image: every GPU that loads the library holds it until the process
// exits.  All calls share it and it keeps the last call's contents, so each
// call clears what it uses before counting, and calls that overlap on the GPU
// (different streams, or host threads, without ordering) race on it.  The
// bin counters are 32-bit, so a call takes fewer than 2^32 particles.
#include <cuda.h>

#include <mutex>

#include "../../include/mprw_gpu.h"
#include "mprw_common.cuh"

namespace {

constexpr int64_t kMaxBins = MPRW_NOALLOC_MAX_BINS;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned int g_noalloc_scratch[kMaxBins + 2];

// Device address of g_noalloc_scratch per device, with the CUDA context it
// was looked up in.  The host-side name is a stand-in, not a device address,
// so it is looked up with the device current (the first call on each device
// does this set-up).  A device reset (cudaDeviceReset) or a new primary
// context reloads the module and may move the array, so the address is looked
// up again whenever the current context is not the one it was found in.
struct ScratchSlot {
  CUcontext ctx;
  unsigned int *ptr;
};
ScratchSlot g_scratch[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// cuCtxGetCurrent through the runtime's driver entry point (the library links
// only the runtime).
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);

cudaError_t current_context(CUcontext *ctx) {
  static CtxGetCurrentFn fn = nullptr;
  if (!fn) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !f) return e != cudaSuccess ? e : cudaErrorUnknown;
    fn = reinterpret_cast<CtxGetCurrentFn>(f);
  }
  return fn(ctx) == CUDA_SUCCESS ? cudaSuccess : cudaErrorUnknown;
}

cudaError_t scratch_for_current_device(unsigned int **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  CUcontext ctx = nullptr;
  e = current_context(&ctx);
  if (e != cudaSuccess) return e;
  if (!ctx) {
    // no context current on this thread yet: cudaSetDevice initialises the
    // device's primary context and makes it current
    e = cudaSetDevice(dev);
    if (e == cudaSuccess) e = current_context(&ctx);
    if (e != cudaSuccess) return e;
  }
  if (!g_scratch[dev].ptr || g_scratch[dev].ctx != ctx) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch[dev].ptr = static_cast<unsigned int *>(p);
    g_scratch[dev].ctx = ctx;
  }
  *out = g_scratch[dev].ptr;
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
                                     int64_t n, Bins B, unsigned int *counts, unsigned long long *nbinned) {
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
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(nbinned, (unsigned long long)mine);
}

__global__ void noalloc_clear_kernel(unsigned int *s, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s[i] = 0u;
}

__global__ void noalloc_out_kernel(const unsigned int *counts, int64_t nbins, const unsigned long long *nbinned,
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
  // 32-bit bin counters: fewer than 2^32 particles per call
  if (n < 0 || n > (int64_t)0xFFFFFFFFu || !origin || !bin_size || !n_bins || !counts) return MPRW_E_INVAL;
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
  // the two words after the bins (byte offset 4 MiB, 8-byte aligned) hold the
  // 64-bit binned-particle counter
  static_assert((kMaxBins * sizeof(unsigned int)) % 8 == 0, "binned counter alignment");
  unsigned long long *nb_counter = reinterpret_cast<unsigned long long *>(scratch + kMaxBins);
  noalloc_clear_kernel<<<grid_for(nbins), 256, 0, s>>>(scratch, nbins);
  noalloc_clear_kernel<<<1, 32, 0, s>>>(scratch + kMaxBins, 2);
  if (n > 0) noalloc_count_kernel<<<grid_for(n), 256, 0, s>>>(gx, gy, gz, status, n, B, scratch, nb_counter);
  noalloc_out_kernel<<<grid_for(nbins), 256, 0, s>>>(scratch, nbins, nb_counter, counts, n_binned);
  return cudaGetLastError() == cudaSuccess ? MPRW_OK : MPRW_E_CUDA;
}
