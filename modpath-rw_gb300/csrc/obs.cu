// obs.cu -- observation cells on the device.
//
// Restates the driver's observation records (Observation.f90:7-60 for the
// cell sets; MPathRW.F90:1337-1392 sink records, 1460-1535 resident
// records):
//   * sink observations (style 2): a record for every particle that stops at
//     a weak sink (status 3) or weak source (status 4) in a cell of the
//     observation, with the stop time -- collected after an advance by an
//     order-preserving compaction over the particles;
//   * resident observations (style 1): at a time point, the ACTIVE
//     particles in the observation's cells -- reduced per observation to a
//     count and a mass (the record's concentration is mass / (water volume *
//     retardation) of the cell, MPathRW.F90:1466-1471).
#include <cub/device/device_select.cuh>
#include <thrust/iterator/counting_iterator.h>

#include "mprw_kernels.cuh"

namespace mprw {

namespace {

int obs_grid(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return b < 1 ? 1 : (int)b;
}

cudaError_t ensure_bytes(void **buf, size_t *have, size_t need) {
  if (*have >= need) return cudaSuccess;
  if (*buf) cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  const size_t grow = need + need / 4 + 1024;
  cudaError_t e = cudaMalloc(buf, grow);
  if (e == cudaSuccess) *have = grow;
  return e;
}

__global__ void sink_flags_kernel(ObsArgs a, uint8_t *flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t st = a.status[i];
    bool f = false;
    if ((st == ST_WEAK_SINK || st == ST_WEAK_SOURCE) && a.t[i] > a.t_begin && a.t[i] <= a.t_end) {
      const int32_t k = a.obs_of_cell[a.cell[i] - a.cell0];
      f = k >= 0 && a.obs_style[k] == 2;
    }
    flag[i] = f ? 1 : 0;
  }
}

__global__ void sink_records_kernel(ObsArgs a, const int64_t *sel, const int64_t *nsel, int32_t *obs, uint64_t *id,
                                    double *time, double *mass) {
  const int64_t m = *nsel;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = sel[r];
    obs[r] = a.obs_of_cell[a.cell[i] - a.cell0];
    id[r] = a.id ? a.id[i] : (uint64_t)i;
    time[r] = a.t[i];
    mass[r] = a.mass ? a.mass[i] : 1.0;
  }
}

__global__ void resident_kernel(ObsArgs a, unsigned long long *count, double *msum) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
    if (a.status[i] != ST_ACTIVE) continue;
    const int32_t k = a.obs_of_cell[a.cell[i] - a.cell0];
    if (k < 0 || a.obs_style[k] != 1) continue;
    atomicAdd(&count[k], 1ull);
    atomicAdd(&msum[k], a.mass ? a.mass[i] : 1.0);
  }
}

}  // namespace

cudaError_t collect_sink_records(const ObsArgs &a, void **scratch, size_t *scratch_bytes, int64_t *n_records,
                                 cudaStream_t s) {
  *n_records = 0;
  if (a.n == 0) return cudaSuccess;
  // layout: flags (n B) | selected indices (n int64) | count | records (obs, id, time, mass)
  size_t temp = 0;
  thrust::counting_iterator<int64_t> it(0);
  cudaError_t e = cub::DeviceSelect::Flagged(nullptr, temp, it, (const uint8_t *)nullptr, (int64_t *)nullptr,
                                             (int64_t *)nullptr, a.n, s);
  if (e != cudaSuccess) return e;
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t nb = (size_t)a.n;
  const size_t o_sel = up(nb), o_cnt = o_sel + up(8 * nb), o_obs = o_cnt + 256, o_id = o_obs + up(4 * nb),
               o_t = o_id + up(8 * nb), o_m = o_t + up(8 * nb), o_tmp = o_m + up(8 * nb);
  e = ensure_bytes(scratch, scratch_bytes, o_tmp + temp);
  if (e != cudaSuccess) return e;
  char *b = (char *)*scratch;
  uint8_t *flag = (uint8_t *)b;
  int64_t *sel = (int64_t *)(b + o_sel), *cnt = (int64_t *)(b + o_cnt);
  sink_flags_kernel<<<obs_grid(a.n), 256, 0, s>>>(a, flag);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cub::DeviceSelect::Flagged(b + o_tmp, temp, it, flag, sel, cnt, a.n, s);
  if (e != cudaSuccess) return e;
  sink_records_kernel<<<obs_grid(a.n), 256, 0, s>>>(a, sel, cnt, (int32_t *)(b + o_obs), (uint64_t *)(b + o_id),
                                                     (double *)(b + o_t), (double *)(b + o_m));
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(n_records, cnt, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

cudaError_t sink_record_arrays(void *scratch, int64_t n, int32_t **obs, uint64_t **id, double **time,
                               double **mass) {
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t nb = (size_t)n;
  const size_t o_sel = up(nb), o_cnt = o_sel + up(8 * nb), o_obs = o_cnt + 256, o_id = o_obs + up(4 * nb),
               o_t = o_id + up(8 * nb), o_m = o_t + up(8 * nb);
  char *b = (char *)scratch;
  *obs = (int32_t *)(b + o_obs);
  *id = (uint64_t *)(b + o_id);
  *time = (double *)(b + o_t);
  *mass = (double *)(b + o_m);
  return cudaSuccess;
}

cudaError_t launch_resident(const ObsArgs &a, unsigned long long *count, double *msum, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  resident_kernel<<<obs_grid(a.n), 256, 0, s>>>(a, count, msum);
  return cudaGetLastError();
}

}  // namespace mprw
