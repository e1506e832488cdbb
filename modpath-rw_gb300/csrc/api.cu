// api.cu -- the C ABI declared in include/mprw_gpu.h.
//
// The handle owns the device copy of the grid, one flow time step (raw
// arrays + per-cell records), the particle state and a CUDA stream.  All
// work is issued on that stream; calls that return data synchronise it.
//
// A batch handle (mprw_create_batch) concatenates the cell records,
// IBOUNDTS, cell flags and particle arrays of several realizations: member m
// owns cells [cell0, cell0 + ncell_m) and particles [p0, p0 + n_m) of the
// batch, its records link only to its own cells (connections offset by
// cell0), so one persistent advance launch over the batch tracks every
// realization at once.  Member views (mprw_batch_member) are ordinary
// handles whose record, IBOUNDTS, flag and particle pointers alias their
// slices of the batch; per-realization calls (load_flow, get_particles,
// histogram, gpkde, observations) go through them.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/mprw_gpu.h"
#include "adjoint.cuh"
#include "gpkde.cuh"
#include "mprw_kernels.cuh"

using namespace mprw;

// One concurrent reconstruction slot of a batch (mprw_gpkde_batch): a
// non-blocking stream and the GPKDE state that reconstructions on it use.
struct KdeWorker {
  cudaStream_t stream = nullptr;
  KdeState kde;
};

struct mprw_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  GridDims g{};
  mprw_options opt{};
  int ndim = 3, d1 = 0, d2 = 1;
  int ncell_bits = 1;
  // grid
  double *d_delr = nullptr, *d_delc = nullptr, *d_top = nullptr, *d_botm = nullptr;
  double *d_colL = nullptr, *d_colR = nullptr, *d_rowF = nullptr, *d_rowB = nullptr, *d_sattop = nullptr;
  std::vector<double> h_top_cell;  // Top(n) after layer propagation
  // flow time step
  int32_t *d_ia = nullptr, *d_ja = nullptr;
  int64_t nja_cap = 0;
  double *d_flowja = nullptr, *d_bflow = nullptr, *d_por = nullptr, *d_ret = nullptr, *d_heads = nullptr;
  double *d_src = nullptr, *d_snk = nullptr, *d_aL = nullptr, *d_aT = nullptr, *d_dm = nullptr;
  double *d_aLV = nullptr, *d_aTV = nullptr;
  int32_t *d_ibts = nullptr, *d_icb = nullptr, *d_ctype = nullptr, *d_zones = nullptr;
  CellBase base{};
  uint8_t *d_massb = nullptr;
  CellRec<double> *d_rec64 = nullptr;
  CellRec<float> *d_rec32 = nullptr;
  bool flow_loaded = false;
  bool dm_uniform = true;             // dm_eff of the loaded flow holds one value
  AdjState *adj = nullptr;            // differentiable walk (mprw_adj_*), made on first set-up
  // particles
  int64_t n = 0, cap = 0;
  int32_t *d_cell = nullptr, *d_status = nullptr;
  void *d_x = nullptr, *d_y = nullptr, *d_z = nullptr;
  double *d_t = nullptr, *d_mass = nullptr, *d_stage = nullptr;
  uint64_t *d_ctr = nullptr, *d_id = nullptr;
  // random counters at the start of the last advance (their increments are
  // the passes each particle took: the next sort puts the heaviest first)
  uint64_t *d_ctr_prev = nullptr;
  bool ctr_prev_valid = false;
  uint32_t *d_perm = nullptr;
  bool unit_mass = true;
  bool has_id = false;
  unsigned long long *d_counters = nullptr;  // [0] queue, [1] steps, [2] nbinned
  int *d_pflags = nullptr;            // particle upload checks: [0] a cell out of range, [1] a mass other than 1
  unsigned long long *h_counters = nullptr;  // pinned
  void *scratch = nullptr;
  size_t scratch_bytes = 0;
  void *hscratch = nullptr;
  size_t hscratch_bytes = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
  double step_ms = 0, prep_ms = 0, hist_ms = 0, kde_ms = 0;
  double kde_work = 0;  // work model of the last reconstruction (multiply-adds of direct kernels)
  KdeState kde;
  // observation cells
  int32_t *d_obs_of_cell = nullptr, *d_obs_style = nullptr;
  int32_t nobs = 0;
  unsigned long long *d_obs_count = nullptr;
  double *d_obs_mass = nullptr;
  double last_t_begin = 0.0, last_t_end = 0.0;
  bool advanced = false;
  double *d_kpart = nullptr;          // coordinate-statistics partials
  double *d_counts = nullptr;
  int64_t counts_cap = 0;
  int64_t launches = 0;
  int sms = 152;
  // launch tuning (mprw_set_tuning / mprw_autotune)
  int blocks_per_sm = 0;     // 0: the variant's default
  int sort_interval = 1;     // sort by cell every k-th advance (0 never)
  int64_t advance_count = 0;
  bool perm_valid = false;   // d_perm holds a permutation of the current n particles
  // cancel flag of the step kernel: pinned, mapped host memory
  volatile int *h_abort = nullptr;
  int *d_abort = nullptr;
  double timeout_ms = 0.0;   // mprw_set_timeout: 0 = wait as long as the advance takes
  std::string err;
  // batched realizations
  mprw_handle *parent = nullptr;        // member view: the batch it belongs to
  std::vector<mprw_handle *> members;   // batch: member views, in cell / particle order
  int32_t cell0 = 0;                    // member: first cell in the batch's cell numbering
  int64_t p0 = 0;                       // member: first particle in the batch's particle arrays
  KdeState *kdep = &kde;                // GPKDE state (a member uses the batch's)
  std::vector<KdeWorker *> kde_workers; // batch: concurrent reconstruction slots
};

namespace {

// NVTX ranges around the library's calls, for a profiler's timeline, when
// the environment sets MPRW_NVTX (NVTX is header-only: without a tool
// attached a range costs a branch).
bool nvtx_on() {
  static const bool on = std::getenv("MPRW_NVTX") != nullptr;
  return on;
}
struct NvtxRange {
  bool on;
  explicit NvtxRange(const char *name) : on(nvtx_on()) {
    if (on) nvtxRangePushA(name);
  }
  ~NvtxRange() {
    if (on) nvtxRangePop();
  }
};

int fail(mprw_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

#define CK(call)                                                                            \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return fail(h, e_ == cudaErrorMemoryAllocation ? MPRW_E_OOM : MPRW_E_CUDA,            \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                      \
  } while (0)

template <typename T>
cudaError_t dalloc(T **p, size_t count) {
  if (*p) cudaFree(*p);
  *p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void **)p, sizeof(T) * count);
}

template <typename T>
cudaError_t upload(mprw_handle *h, T **p, const T *src, size_t count) {
  cudaError_t e = dalloc(p, count);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(*p, src, sizeof(T) * count, cudaMemcpyHostToDevice, h->stream);
}

void free_all(mprw_handle *h) {
  if (h->adj) {
    h->adj->release();
    delete h->adj;
    h->adj = nullptr;
  }
  if (h->parent) {
    // slices of the batch's arrays
    h->d_rec64 = nullptr;
    h->d_rec32 = nullptr;
    h->d_ibts = nullptr;
    h->base.flags = nullptr;
    h->d_cell = h->d_status = nullptr;
    h->d_x = h->d_y = h->d_z = nullptr;
    h->d_t = h->d_mass = h->d_stage = nullptr;
    h->d_ctr = h->d_id = nullptr;
    h->d_ctr_prev = nullptr;
    h->d_perm = nullptr;
  }
  for (mprw_handle *m : h->members) {
    free_all(m);
    delete m;
  }
  h->members.clear();
  for (KdeWorker *w : h->kde_workers) {
    w->kde.release();
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
  }
  h->kde_workers.clear();
  void *ptrs[] = {h->d_delr, h->d_delc, h->d_top, h->d_botm, h->d_colL, h->d_colR, h->d_rowF, h->d_rowB,
                  h->d_sattop, h->d_ia, h->d_ja, h->d_flowja, h->d_bflow, h->d_por, h->d_ret, h->d_heads,
                  h->d_src, h->d_snk, h->d_aL, h->d_aT, h->d_dm, h->d_aLV, h->d_aTV, h->d_ibts, h->d_icb, h->d_ctype,
                  h->d_zones, h->base.q, h->base.dz, h->base.conn, h->base.flags, h->d_massb, h->d_rec64,
                  h->d_rec32, h->d_cell, h->d_status, h->d_x, h->d_y, h->d_z, h->d_t, h->d_mass,
                  h->d_stage, h->d_ctr, h->d_ctr_prev, h->d_id, h->d_perm, h->d_counters, h->scratch,
                  h->d_pflags};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (h->h_counters) cudaFreeHost(h->h_counters);
  if (h->h_abort) cudaFreeHost((void *)h->h_abort);
  if (h->d_counts) cudaFree(h->d_counts);
  if (h->d_kpart) cudaFree(h->d_kpart);
  for (void *p : {(void *)h->d_obs_of_cell, (void *)h->d_obs_style, (void *)h->d_obs_count, (void *)h->d_obs_mass})
    if (p) cudaFree(p);
  h->kde.release();  // (a member view's own state is empty)
  if (h->hscratch) cudaFreeHost(h->hscratch);
  cudaEvent_t evs[] = {h->ev0, h->ev1, h->ev2, h->ev3};
  for (auto e : evs)
    if (e) cudaEventDestroy(e);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
}

__global__ void f64_to_f32_kernel(const double *in, float *out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}
__global__ void f32_to_f64_kernel(const float *in, double *out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}
__global__ void cell_shift_kernel(int32_t *cell, int64_t n, int32_t delta) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    cell[i] += delta;
}
// The uploaded cells (1-based) checked against 1..ncell and shifted to the
// stored numbering; flag[0] is set when any is out of range.  One warp vote
// and at most one atomic per warp.
__global__ void cell_check_shift_kernel(int32_t *cell, int64_t n, int32_t ncell, int32_t delta, int *flag) {
  bool bad = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = cell[i];
    bad = bad || c < 1 || c > ncell;
    cell[i] = c + delta;
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}
// flag set when any mass differs from 1
__global__ void unit_mass_kernel(const double *m, int64_t n, int *flag) {
  bool other = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    other = other || m[i] != 1.0;
  if (__any_sync(0xffffffffu, other) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}
// stored cells back to the caller's 1-based numbering
__global__ void cell_out_kernel(const int32_t *cell, int64_t n, int32_t delta, int32_t *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = cell[i] + delta;
}
__global__ void mul2_kernel(double *x, int64_t n, double a, double b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = (x[i] * a) * b;
}
__global__ void div_kernel(double *x, int64_t n, double d) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = x[i] / d;
}

int grid1d(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return b < 1 ? 1 : (int)b;
}

Geometry geometry(mprw_handle *h) {
  Geometry geo;
  geo.col_left = h->d_colL;
  geo.col_right = h->d_colR;
  geo.row_front = h->d_rowF;
  geo.row_back = h->d_rowB;
  geo.botm = h->d_botm;
  geo.sattop = h->d_sattop;
  geo.g = h->g;
  geo.cell0 = h->cell0;
  return geo;
}

bool grid_ok(const mprw_grid_desc *gd) {
  if (gd->nlay <= 0 || gd->nrow <= 0 || gd->ncol <= 0 || !gd->delr || !gd->delc || !gd->top || !gd->botm)
    return false;
  return (int64_t)gd->nlay * gd->nrow * gd->ncol < ((int64_t)1 << 31);
}

// Options, device attributes, events and counters of a handle.
int init_common(mprw_handle *h, const mprw_options *o) {
  if (o->advection_kind != 1 && o->advection_kind != 2)
    return fail(h, MPRW_E_INVAL, "advection_kind: 1 (EXPONENTIAL) or 2 (EULERIAN)");
  if (o->dispersion_model != 0 && o->dispersion_model != 1)
    return fail(h, MPRW_E_INVAL, "dispersion_model: 0 (linear isotropic) or 1 (linear axisymmetric)");
  if (o->time_step_kind < 1 || o->time_step_kind > 4) return fail(h, MPRW_E_INVAL, "time_step_kind");
  if (o->precision != MPRW_FP64 && o->precision != MPRW_MIXED) return fail(h, MPRW_E_INVAL, "precision");
  h->opt = *o;
  int dims[3], nd = 0;
  for (int d = 0; d < 3; ++d)
    if (o->dim_mask[d]) dims[nd++] = d;
  if (nd == 0) return fail(h, MPRW_E_INVAL, "dim_mask selects no dimension");
  h->ndim = nd;
  h->d1 = dims[0];
  h->d2 = nd > 1 ? dims[1] : 0;
  CK(cudaGetDevice(&h->device));
  CK(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device));
  CK(cudaEventCreate(&h->ev0));
  CK(cudaEventCreate(&h->ev1));
  CK(cudaEventCreate(&h->ev2));
  CK(cudaEventCreate(&h->ev3));
  CK(cudaMallocHost(&h->h_counters, 4 * sizeof(unsigned long long)));
  CK(dalloc(&h->d_counters, 4));
  void *ab = nullptr;
  CK(cudaHostAlloc(&ab, sizeof(int), cudaHostAllocMapped));
  h->h_abort = (volatile int *)ab;
  *h->h_abort = 0;
  CK(cudaHostGetDevicePointer((void **)&h->d_abort, ab, 0));
  return MPRW_OK;
}

// Grid dimensions and the geometry arrays, built as the binary-grid reader
// builds them (RectangularGridDisMf6.f90:301-340).
int init_grid(mprw_handle *h, const mprw_grid_desc *gd) {
  const int64_t ncell = (int64_t)gd->nlay * gd->nrow * gd->ncol;
  h->g.nlay = gd->nlay;
  h->g.nrow = gd->nrow;
  h->g.ncol = gd->ncol;
  h->g.ncpl = gd->nrow * gd->ncol;
  h->g.ncell = (int32_t)ncell;
  while (((int64_t)1 << h->ncell_bits) < ncell) ++h->ncell_bits;
  const int ncol = gd->ncol, nrow = gd->nrow, ncpl = h->g.ncpl;
  std::vector<double> colL(ncol), colR(ncol), rowF(nrow), rowB(nrow);
  double X = 0.0;
  for (int c = 0; c < ncol; ++c) {
    double Xn = X + gd->delr[c];
    double cx = (X + Xn) / 2.0;
    colL[c] = cx - (gd->delr[c] / 2.0);
    colR[c] = cx + (gd->delr[c] / 2.0);
    X = Xn;
  }
  double Y = 0.0;
  for (int r = 0; r < nrow; ++r) Y = Y + gd->delc[r];
  for (int r = 0; r < nrow; ++r) {
    double Yn = Y - gd->delc[r];
    double cy = (Y + Yn) / 2.0;
    rowF[r] = cy - (gd->delc[r] / 2.0);
    rowB[r] = cy + (gd->delc[r] / 2.0);
    Y = Yn;
  }
  h->h_top_cell.resize(ncell);
  for (int64_t c = 0; c < ncell; ++c) h->h_top_cell[c] = (c < ncpl) ? gd->top[c] : gd->botm[c - ncpl];
  CK(upload(h, &h->d_delr, gd->delr, ncol));
  CK(upload(h, &h->d_delc, gd->delc, nrow));
  CK(upload(h, &h->d_top, gd->top, ncpl));
  CK(upload(h, &h->d_botm, gd->botm, ncell));
  CK(upload(h, &h->d_colL, colL.data(), ncol));
  CK(upload(h, &h->d_colR, colR.data(), ncol));
  CK(upload(h, &h->d_rowF, rowF.data(), nrow));
  CK(upload(h, &h->d_rowB, rowB.data(), nrow));
  CK(upload(h, &h->d_sattop, h->h_top_cell.data(), ncell));
  CK(cudaStreamSynchronize(h->stream));
  return MPRW_OK;
}

// Member records link to member-local cells; in the batch's numbering the
// connections move by cell0.
template <typename R>
__global__ void offset_conn_kernel(CellRec<R> *rec, int64_t n, int32_t cell0) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
    for (int f = 0; f < 6; ++f)
      if (rec[i].conn[f] >= 0) rec[i].conn[f] += cell0;
}

cudaError_t ensure_host(mprw_handle *h, size_t bytes) {
  if (h->hscratch_bytes >= bytes) return cudaSuccess;
  if (h->hscratch) cudaFreeHost(h->hscratch);
  h->hscratch = nullptr;
  h->hscratch_bytes = 0;
  cudaError_t e = cudaMallocHost(&h->hscratch, bytes);
  if (e == cudaSuccess) h->hscratch_bytes = bytes;
  return e;
}

}  // namespace

extern "C" {

int mprw_create(mprw_handle **out, const mprw_grid_desc *gd, const mprw_options *o) {
  if (!out || !gd || !o) return MPRW_E_INVAL;
  *out = nullptr;
  if (!grid_ok(gd)) return MPRW_E_INVAL;
  mprw_handle *h = new mprw_handle();
  *out = h;
  int rc = init_common(h, o);
  if (rc != MPRW_OK) return rc;
  CK(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
  h->stream = h->own_stream;
  return init_grid(h, gd);
}

int mprw_create_batch(mprw_handle **out, int32_t nmembers, const mprw_grid_desc *grids, const mprw_options *o) {
  if (!out || !grids || !o || nmembers < 1) return MPRW_E_INVAL;
  *out = nullptr;
  int64_t total = 0;
  for (int32_t m = 0; m < nmembers; ++m) {
    if (!grid_ok(&grids[m])) return MPRW_E_INVAL;
    total += (int64_t)grids[m].nlay * grids[m].nrow * grids[m].ncol;
  }
  if (total >= (int64_t)1 << 31) return MPRW_E_INVAL;
  mprw_handle *h = new mprw_handle();
  *out = h;
  int rc = init_common(h, o);
  if (rc != MPRW_OK) return rc;
  CK(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
  h->stream = h->own_stream;
  h->g.ncell = (int32_t)total;
  while (((int64_t)1 << h->ncell_bits) < total) ++h->ncell_bits;
  // the concatenated arrays the advance kernel reads
  if (h->opt.precision == MPRW_FP64) CK(dalloc(&h->d_rec64, total));
  else CK(dalloc(&h->d_rec32, total));
  CK(dalloc(&h->d_ibts, total));
  CK(dalloc(&h->base.flags, total));
  CK(cudaMemsetAsync(h->d_ibts, 0, sizeof(int32_t) * total, h->stream));
  CK(cudaMemsetAsync(h->base.flags, 0, total, h->stream));
  int64_t cell0 = 0;
  for (int32_t k = 0; k < nmembers; ++k) {
    mprw_handle *m = new mprw_handle();
    h->members.push_back(m);
    m->parent = h;
    m->kdep = &h->kde;
    m->cell0 = (int32_t)cell0;
    rc = init_common(m, o);
    if (rc != MPRW_OK) return fail(h, rc, "member " + std::to_string(k) + ": " + m->err);
    m->stream = h->stream;
    rc = init_grid(m, &grids[k]);
    if (rc != MPRW_OK) return fail(h, rc, "member " + std::to_string(k) + ": " + m->err);
    if (h->d_rec64) m->d_rec64 = h->d_rec64 + cell0;
    if (h->d_rec32) m->d_rec32 = h->d_rec32 + cell0;
    m->d_ibts = h->d_ibts + cell0;
    m->base.flags = h->base.flags + cell0;
    cell0 += m->g.ncell;
  }
  CK(cudaStreamSynchronize(h->stream));
  return MPRW_OK;
}

int mprw_batch_member(mprw_handle *h, int32_t member, mprw_handle **view) {
  if (!h || !view) return MPRW_E_INVAL;
  *view = nullptr;
  if (h->members.empty()) return fail(h, MPRW_E_STATE, "mprw_batch_member: not a batch handle");
  if (member < 0 || member >= (int32_t)h->members.size())
    return fail(h, MPRW_E_INVAL, "mprw_batch_member: member index out of range");
  *view = h->members[member];
  return MPRW_OK;
}

int mprw_load_flow(mprw_handle *h, const mprw_flow_desc *f) {
  NvtxRange nvtx_("mprw_load_flow");
  if (!h) return MPRW_E_INVAL;
  if (!h->members.empty()) return fail(h, MPRW_E_STATE, "mprw_load_flow on a batch: load each member's flow");
  if (!f || !f->ia || !f->ja || !f->flowja || !f->porosity || !f->retardation || !f->iboundts || !f->alpha_l ||
      !f->alpha_t || !f->dm_eff)
    return fail(h, MPRW_E_INVAL, "mprw_load_flow: missing required array");
  const int64_t nc = h->g.ncell;
  if (f->nja < nc || f->ia[0] != 1 || f->ia[nc] - 1 != f->nja)
    return fail(h, MPRW_E_INVAL, "mprw_load_flow: IA/JA inconsistent with the grid");
  for (int64_t c = 0; c < nc; ++c) {
    if (!(f->porosity[c] > 0.0) || !(f->retardation[c] > 0.0) || !std::isfinite(f->porosity[c]) ||
        !std::isfinite(f->retardation[c]))
      return fail(h, MPRW_E_INVAL, "mprw_load_flow: porosity and retardation must be finite and > 0");
  }
  // non-finite inputs: the reference runs with -ffpe-trap=invalid and stops on
  // the first NaN; a library call rejects them before any device work
  {
    auto finite = [](const double *a, int64_t n) {
      if (!a) return true;
      for (int64_t i = 0; i < n; ++i)
        if (!std::isfinite(a[i])) return false;
      return true;
    };
    const int64_t nd = f->uniform_dispersion ? 1 : nc;
    if (!finite(f->flowja, f->nja) || !finite(f->boundary_flows, 6 * nc) || !finite(f->source_flow, nc) ||
        !finite(f->sink_flow, nc) || !finite(f->alpha_l, nd) || !finite(f->alpha_t, nd) ||
        !finite(f->dm_eff, nd) || !finite(f->alpha_lv, nd) || !finite(f->alpha_tv, nd))
      return fail(h, MPRW_E_INVAL, "mprw_load_flow: non-finite face flow, boundary flow, source/sink or dispersion value");
    if (f->heads)
      for (int64_t c = 0; c < nc; ++c)
        if (std::isnan(f->heads[c])) return fail(h, MPRW_E_INVAL, "mprw_load_flow: NaN head");
  }
  for (int64_t p = 0; p < f->nja; ++p)
    if (f->ja[p] < 1 || f->ja[p] > nc) return fail(h, MPRW_E_INVAL, "mprw_load_flow: JA entry out of range");
  const size_t nd = f->uniform_dispersion ? 1 : (size_t)nc;
  CK(upload(h, &h->d_ia, f->ia, nc + 1));
  CK(upload(h, &h->d_ja, f->ja, f->nja));
  CK(upload(h, &h->d_flowja, f->flowja, f->nja));
  if (f->boundary_flows) CK(upload(h, &h->d_bflow, f->boundary_flows, 6 * nc));
  CK(upload(h, &h->d_por, f->porosity, nc));
  CK(upload(h, &h->d_ret, f->retardation, nc));
  h->dm_uniform = f->uniform_dispersion != 0;
  if (h->parent)
    CK(cudaMemcpyAsync(h->d_ibts, f->iboundts, sizeof(int32_t) * nc, cudaMemcpyHostToDevice, h->stream));
  else
    CK(upload(h, &h->d_ibts, f->iboundts, nc));
  if (f->icboundts) CK(upload(h, &h->d_icb, f->icboundts, nc));
  if (f->heads) CK(upload(h, &h->d_heads, f->heads, nc));
  if (f->celltype) CK(upload(h, &h->d_ctype, f->celltype, nc));
  if (f->source_flow) CK(upload(h, &h->d_src, f->source_flow, nc));
  if (f->sink_flow) CK(upload(h, &h->d_snk, f->sink_flow, nc));
  if (f->zones) CK(upload(h, &h->d_zones, f->zones, nc));
  CK(upload(h, &h->d_aL, f->alpha_l, nd));
  CK(upload(h, &h->d_aT, f->alpha_t, nd));
  CK(upload(h, &h->d_dm, f->dm_eff, nd));
  if (f->alpha_lv) CK(upload(h, &h->d_aLV, f->alpha_lv, nd));
  if (f->alpha_tv) CK(upload(h, &h->d_aTV, f->alpha_tv, nd));
  // SaturatedTop (FlowModelData.f90:258-279) for ConvertToModelXYZ
  std::vector<double> sat(h->h_top_cell);
  {
    std::vector<double> botm(nc);
    CK(cudaMemcpyAsync(botm.data(), h->d_botm, sizeof(double) * nc, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (f->celltype && f->heads)
      for (int64_t c = 0; c < nc; ++c)
        if (f->celltype[c] == 1 && f->iboundts[c] != 0 && f->heads[c] <= h->h_top_cell[c] && f->heads[c] >= botm[c])
          sat[c] = f->heads[c];
  }
  CK(cudaMemcpyAsync(h->d_sattop, sat.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, h->stream));
  if (!h->base.q) {
    CK(dalloc(&h->base.q, 6 * nc));
    CK(dalloc(&h->base.dz, nc));
    CK(dalloc(&h->base.conn, 6 * nc));
    CK(dalloc(&h->d_massb, nc));
    if (!h->parent) {  // a member's flags and records are slices of the batch's
      CK(dalloc(&h->base.flags, nc));
      if (h->opt.precision == MPRW_FP64) CK(dalloc(&h->d_rec64, nc));
      else CK(dalloc(&h->d_rec32, nc));
    }
  }
  PrepInputs in{};
  in.g = h->g;
  in.delr = h->d_delr;
  in.delc = h->d_delc;
  in.top = h->d_top;
  in.botm = h->d_botm;
  in.ia = h->d_ia;
  in.ja = h->d_ja;
  in.flowja = h->d_flowja;
  in.bflow = f->boundary_flows ? h->d_bflow : nullptr;
  in.porosity = h->d_por;
  in.retardation = h->d_ret;
  in.iboundts = h->d_ibts;
  in.icboundts = f->icboundts ? h->d_icb : nullptr;
  in.default_icbound = f->default_icbound;
  in.heads = f->heads ? h->d_heads : nullptr;
  in.celltype = f->celltype ? h->d_ctype : nullptr;
  in.source_flow = f->source_flow ? h->d_src : nullptr;
  in.sink_flow = f->sink_flow ? h->d_snk : nullptr;
  in.zones = f->zones ? h->d_zones : nullptr;
  in.alpha_l = h->d_aL;
  in.alpha_t = h->d_aT;
  in.dm_eff = h->d_dm;
  in.alpha_lv = f->alpha_lv ? h->d_aLV : nullptr;
  in.alpha_tv = f->alpha_tv ? h->d_aTV : nullptr;
  in.dispersion_model = h->opt.dispersion_model;
  in.uniform_dispersion = f->uniform_dispersion;
  in.steady_state = f->steady_state;
  in.time_step_kind = h->opt.time_step_kind;
  in.ts_param0 = h->opt.ts_param[0];
  in.ts_param1 = h->opt.ts_param[1];
  in.backward = h->opt.backward;
  in.stop_weak_sinks = h->opt.stop_weak_sinks;
  in.stop_weak_sources = h->opt.stop_weak_sources;
  in.stop_zone = h->opt.stop_zone;
  in.uniform_porosity = h->opt.uniform_porosity;
  CK(cudaEventRecord(h->ev2, h->stream));
  CK(launch_prep(in, h->base, h->d_massb, h->d_rec64, h->d_rec32, h->stream));
  if (h->cell0 != 0) {
    if (h->d_rec64) offset_conn_kernel<double><<<grid1d(nc), 256, 0, h->stream>>>(h->d_rec64, nc, h->cell0);
    else offset_conn_kernel<float><<<grid1d(nc), 256, 0, h->stream>>>(h->d_rec32, nc, h->cell0);
    CK(cudaGetLastError());
  }
  CK(cudaEventRecord(h->ev3, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, h->ev2, h->ev3));
  h->prep_ms = ms;
  h->flow_loaded = true;
  return MPRW_OK;
}

}  // extern "C"

namespace {

// Copies n particles into h's arrays (allocating them when h owns them and
// they are too small).  Cells arrive 1-based and are stored 0-based + shift.
int upload_particles(mprw_handle *h, int64_t n, const int32_t *cell, const double *lx, const double *ly,
                     const double *lz, const double *t, const int32_t *status, const double *mass,
                     const uint64_t *id, const uint64_t *rng_ctr, int32_t shift, int32_t ncell_check) {
  const bool mixed = h->opt.precision == MPRW_MIXED;
  const size_t rs = mixed ? sizeof(float) : sizeof(double);
  if (n > h->cap) {
    if (h->parent) return fail(h, MPRW_E_STATE, "batch member particle slice too small");
    size_t c = (size_t)n;
    CK(dalloc(&h->d_cell, c));
    CK(dalloc(&h->d_status, c));
    CK(dalloc((char **)&h->d_x, c * rs));
    CK(dalloc((char **)&h->d_y, c * rs));
    CK(dalloc((char **)&h->d_z, c * rs));
    CK(dalloc(&h->d_t, c));
    CK(dalloc(&h->d_mass, c));
    CK(dalloc(&h->d_ctr, c));
    CK(dalloc(&h->d_ctr_prev, c));
    CK(dalloc(&h->d_id, c));
    CK(dalloc(&h->d_perm, c));
    if (mixed) CK(dalloc(&h->d_stage, c));
    h->cap = n;
  }
  // the pass counts of the last advance (counter increments) still order the
  // next one when the host hands the same particles back; for other
  // particles of the same count they only give a poorer order
  if (n != h->n) h->ctr_prev_valid = false;
  h->n = n;
  h->perm_valid = false;
  h->advance_count = 0;
  if (n == 0) return MPRW_OK;
  cudaStream_t s = h->stream;
  if (!h->d_pflags) CK(cudaMalloc(&h->d_pflags, 2 * sizeof(int)));
  CK(cudaMemsetAsync(h->d_pflags, 0, 2 * sizeof(int), s));
  CK(cudaMemcpyAsync(h->d_cell, cell, 4 * n, cudaMemcpyHostToDevice, s));
  if (ncell_check > 0)
    cell_check_shift_kernel<<<grid1d(n), 256, 0, s>>>(h->d_cell, n, ncell_check, shift, h->d_pflags);
  else
    cell_shift_kernel<<<grid1d(n), 256, 0, s>>>(h->d_cell, n, shift);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(h->d_status, status, 4 * n, cudaMemcpyHostToDevice, s));
  const double *src[3] = {lx, ly, lz};
  void *dst[3] = {h->d_x, h->d_y, h->d_z};
  for (int a = 0; a < 3; ++a) {
    if (mixed) {
      CK(cudaMemcpyAsync(h->d_stage, src[a], 8 * n, cudaMemcpyHostToDevice, s));
      f64_to_f32_kernel<<<grid1d(n), 256, 0, s>>>(h->d_stage, (float *)dst[a], n);
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(s));  // staging buffer reused
    } else {
      CK(cudaMemcpyAsync(dst[a], src[a], 8 * n, cudaMemcpyHostToDevice, s));
    }
  }
  CK(cudaMemcpyAsync(h->d_t, t, 8 * n, cudaMemcpyHostToDevice, s));
  h->unit_mass = true;
  if (mass) {
    CK(cudaMemcpyAsync(h->d_mass, mass, 8 * n, cudaMemcpyHostToDevice, s));
    unit_mass_kernel<<<grid1d(n), 256, 0, s>>>(h->d_mass, n, h->d_pflags + 1);
    CK(cudaGetLastError());
  }
  h->has_id = id != nullptr;
  if (id) CK(cudaMemcpyAsync(h->d_id, id, 8 * n, cudaMemcpyHostToDevice, s));
  if (rng_ctr) CK(cudaMemcpyAsync(h->d_ctr, rng_ctr, 8 * n, cudaMemcpyHostToDevice, s));
  else CK(cudaMemsetAsync(h->d_ctr, 0, 8 * n, s));
  int flags[2] = {0, 0};
  CK(cudaMemcpyAsync(flags, h->d_pflags, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (flags[0]) {
    // the device arrays were overwritten: the handle holds no particles
    h->n = 0;
    return fail(h, MPRW_E_INVAL, "particle cell number out of range");
  }
  h->unit_mass = (mass == nullptr) || flags[1] == 0;
  return MPRW_OK;
}

}  // namespace

extern "C" {

int mprw_set_particles(mprw_handle *h, int64_t n, const int32_t *cell, const double *lx, const double *ly,
                       const double *lz, const double *t, const int32_t *status, const double *mass,
                       const uint64_t *id, const uint64_t *rng_ctr) {
  if (!h) return MPRW_E_INVAL;
  if (!h->members.empty())
    return fail(h, MPRW_E_STATE, "mprw_set_particles on a batch: use mprw_set_particles_batch");
  if (n < 0 || n >= ((int64_t)1 << 32)) return fail(h, MPRW_E_INVAL, "particle count out of range");
  if (n > 0 && (!cell || !lx || !ly || !lz || !t || !status))
    return fail(h, MPRW_E_INVAL, "mprw_set_particles: missing required array");
  if (h->parent) {
    if (n != h->n) return fail(h, MPRW_E_STATE, "a batch member's particle count is set by mprw_set_particles_batch");
    if ((id != nullptr) != h->parent->has_id)
      return fail(h, MPRW_E_INVAL, "a batch member's particles carry ids exactly when the batch's do");
  }
  // the cells are checked against 1..ncell on the device (the upload fails,
  // and the handle then holds no particles, when one is out of range)
  return upload_particles(h, n, cell, lx, ly, lz, t, status, mass, id, rng_ctr, h->cell0 - 1, h->g.ncell);
}

int mprw_set_particles_batch(mprw_handle *h, const int64_t *counts, const int32_t *cell, const double *lx,
                             const double *ly, const double *lz, const double *t, const int32_t *status,
                             const double *mass, const uint64_t *id, const uint64_t *rng_ctr) {
  if (!h) return MPRW_E_INVAL;
  if (h->members.empty()) return fail(h, MPRW_E_STATE, "mprw_set_particles_batch: not a batch handle");
  if (!counts) return fail(h, MPRW_E_INVAL, "mprw_set_particles_batch: null counts");
  const int32_t nm = (int32_t)h->members.size();
  int64_t n = 0;
  for (int32_t k = 0; k < nm; ++k) {
    if (counts[k] < 0) return fail(h, MPRW_E_INVAL, "mprw_set_particles_batch: negative count");
    n += counts[k];
    if (n >= ((int64_t)1 << 32)) return fail(h, MPRW_E_INVAL, "particle count out of range");
  }
  if (n > 0 && (!cell || !lx || !ly || !lz || !t || !status))
    return fail(h, MPRW_E_INVAL, "mprw_set_particles_batch: missing required array");
  {
    int64_t p = 0;
    for (int32_t k = 0; k < nm; ++k)
      for (int64_t e = p + counts[k]; p < e; ++p)
        if (cell[p] < 1 || cell[p] > h->members[k]->g.ncell)
          return fail(h, MPRW_E_INVAL, "member " + std::to_string(k) + ": particle cell number out of range");
  }
  int rc = upload_particles(h, n, cell, lx, ly, lz, t, status, mass, id, rng_ctr, -1, 0);
  if (rc != MPRW_OK) return rc;
  const size_t rs = h->opt.precision == MPRW_MIXED ? sizeof(float) : sizeof(double);
  int64_t p0 = 0;
  for (int32_t k = 0; k < nm; ++k) {
    mprw_handle *m = h->members[k];
    const int64_t nk = counts[k];
    m->p0 = p0;
    m->n = m->cap = nk;
    m->d_cell = h->d_cell + p0;
    m->d_status = h->d_status + p0;
    m->d_x = (char *)h->d_x + rs * p0;
    m->d_y = (char *)h->d_y + rs * p0;
    m->d_z = (char *)h->d_z + rs * p0;
    m->d_t = h->d_t + p0;
    m->d_mass = h->d_mass + p0;
    m->d_ctr = h->d_ctr + p0;
    m->d_id = h->d_id + p0;
    m->d_stage = h->d_stage ? h->d_stage + p0 : nullptr;
    m->d_perm = nullptr;
    m->has_id = h->has_id;
    m->unit_mass = true;
    if (mass)
      for (int64_t q = p0; q < p0 + nk && m->unit_mass; ++q) m->unit_mass = (mass[q] == 1.0);
    m->advanced = false;
    if (nk > 0 && m->cell0 != 0) {
      cell_shift_kernel<<<grid1d(nk), 256, 0, h->stream>>>(m->d_cell, nk, m->cell0);
      CK(cudaGetLastError());
    }
    p0 += nk;
  }
  CK(cudaStreamSynchronize(h->stream));
  return MPRW_OK;
}

}  // extern "C"

namespace {

// Resident blocks per SM of the step kernel variant a handle launches: the
// tuned value, capped by what the variant's registers and shared memory allow.
int max_blocks_per_sm(mprw_handle *h) {
  const bool mixed = h->opt.precision == MPRW_MIXED;
  const bool exp_adv = h->opt.advection_kind == 1, axi = h->opt.dispersion_model == 1;
  int nb = 0;
  const int threads = step_threads(!mixed, exp_adv != 0);
  cudaError_t e = mixed ? advance_occupancy<float>(exp_adv, axi, threads, &nb)
                        : advance_occupancy<double>(exp_adv, axi, threads, &nb);
  if (e != cudaSuccess || nb < 1) nb = 1;
  return nb;
}

int default_blocks_per_sm(mprw_handle *h) {
  // EULERIAN MIXED is compiled for 3 resident blocks per SM (80 registers)
  return (h->opt.precision == MPRW_MIXED && h->opt.advection_kind != 1) ? 3 : 1;
}

// One launch of the persistent step kernel over every particle, processing
// them in the order of d_perm when use_perm; *ms the event-timed duration.
int launch_step(mprw_handle *h, double t_begin, double t_end, int bps, bool use_perm, float *ms, int64_t *steps) {
  cudaStream_t s = h->stream;
  CK(cudaMemsetAsync(h->d_counters, 0, 4 * sizeof(unsigned long long), s));
  const int threads = step_threads(h->opt.precision != MPRW_MIXED, h->opt.advection_kind == 1);
  int64_t need = (h->n + threads - 1) / threads;
  int64_t blocks = (int64_t)h->sms * bps;
  if (need < blocks) blocks = need;
  CK(cudaEventRecord(h->ev0, s));
  if (h->opt.precision == MPRW_MIXED) {
    AdvanceArgs<float> a{};
    a.recs = h->d_rec32;
    a.iboundts = h->d_ibts;
    a.cellflags = h->base.flags;
    a.cell = h->d_cell;
    a.status = h->d_status;
    a.x = (float *)h->d_x;
    a.y = (float *)h->d_y;
    a.z = (float *)h->d_z;
    a.t = h->d_t;
    a.ctr = h->d_ctr;
    a.id = h->has_id ? h->d_id : nullptr;
    a.perm = use_perm ? h->d_perm : nullptr;
    a.queue = h->d_counters;
    a.steps = h->d_counters + 1;
    a.abort = h->d_abort;
    a.n = h->n;
    a.t_begin = t_begin;
    a.t_end = t_end;
    a.ndim = h->ndim;
    a.d1 = h->d1;
    a.d2 = h->d2;
    a.seed = h->opt.rng_seed;
    a.exp_adv = h->opt.advection_kind == 1;
    a.axi = h->opt.dispersion_model == 1;
    CK(launch_advance<float>(a, (int)blocks, threads, s));
  } else {
    AdvanceArgs<double> a{};
    a.recs = h->d_rec64;
    a.iboundts = h->d_ibts;
    a.cellflags = h->base.flags;
    a.cell = h->d_cell;
    a.status = h->d_status;
    a.x = (double *)h->d_x;
    a.y = (double *)h->d_y;
    a.z = (double *)h->d_z;
    a.t = h->d_t;
    a.ctr = h->d_ctr;
    a.id = h->has_id ? h->d_id : nullptr;
    a.perm = use_perm ? h->d_perm : nullptr;
    a.queue = h->d_counters;
    a.steps = h->d_counters + 1;
    a.abort = h->d_abort;
    a.n = h->n;
    a.t_begin = t_begin;
    a.t_end = t_end;
    a.ndim = h->ndim;
    a.d1 = h->d1;
    a.d2 = h->d2;
    a.seed = h->opt.rng_seed;
    a.exp_adv = h->opt.advection_kind == 1;
    a.axi = h->opt.dispersion_model == 1;
    CK(launch_advance<double>(a, (int)blocks, threads, s));
  }
  h->launches += 1;
  CK(cudaEventRecord(h->ev1, s));
  CK(cudaMemcpyAsync(h->h_counters, h->d_counters, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  // wait; past the timeout, raise the cancel flag (the kernel reads it every
  // kAbortPoll iterations of each warp and returns)
  bool timed_out = false;
  if (h->timeout_ms > 0.0) {
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
      const cudaError_t q = cudaEventQuery(h->ev1);
      if (q == cudaSuccess) break;
      if (q != cudaErrorNotReady) CK(q);
      if (std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count() > h->timeout_ms) {
        *h->h_abort = 1;
        timed_out = true;
        break;
      }
      std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
  }
  CK(cudaStreamSynchronize(s));
  const bool cancelled = *h->h_abort != 0;
  *h->h_abort = 0;
  CK(cudaEventElapsedTime(ms, h->ev0, h->ev1));
  *steps = (int64_t)h->h_counters[1];
  if (cancelled)
    return fail(h, MPRW_E_ABORTED,
                timed_out ? "advance stopped at its timeout; the particles hold their last completed pass"
                          : "advance cancelled; the particles hold their last completed pass");
  return MPRW_OK;
}

int sort_particles(mprw_handle *h) {
  const uint64_t per_pass = 3ull * (uint64_t)h->ndim;  // Philox blocks per pass: 3 per normal, ndim normals
  CK(sort_cells(h->d_cell, h->d_ctr, h->ctr_prev_valid ? h->d_ctr_prev : nullptr, per_pass, h->d_perm, h->n,
                h->ncell_bits, &h->scratch, &h->scratch_bytes, h->stream));
  h->launches += 2;
  h->perm_valid = true;
  return MPRW_OK;
}

}  // namespace

extern "C" {

int mprw_advance(mprw_handle *h, double t_begin, double t_end, int64_t *steps_done) {
  NvtxRange nvtx_("mprw_advance");
  if (!h) return MPRW_E_INVAL;
  if (h->parent) return fail(h, MPRW_E_STATE, "mprw_advance on a batch member: advance the batch");
  if (!h->members.empty()) {
    h->flow_loaded = true;
    for (size_t k = 0; k < h->members.size(); ++k)
      if (!h->members[k]->flow_loaded)
        return fail(h, MPRW_E_STATE, "mprw_advance before member " + std::to_string(k) + "'s mprw_load_flow");
  }
  if (!h->flow_loaded) return fail(h, MPRW_E_STATE, "mprw_advance before mprw_load_flow");
  if (!(t_end >= t_begin)) return fail(h, MPRW_E_INVAL, "t_end < t_begin");
  h->launches = 0;
  h->last_t_begin = t_begin;
  h->last_t_end = t_end;
  h->advanced = true;
  for (mprw_handle *m : h->members) {
    m->last_t_begin = t_begin;
    m->last_t_end = t_end;
    m->advanced = true;
  }
  if (h->n == 0) {
    if (steps_done) *steps_done = 0;
    return MPRW_OK;
  }
  // sort the particles by cell every sort_interval-th advance; in between the
  // last order is reused (the permutation stays valid while n is unchanged)
  if (h->sort_interval > 0 && (h->advance_count % h->sort_interval == 0 || !h->perm_valid)) {
    int rc = sort_particles(h);
    if (rc != MPRW_OK) return rc;
  }
  ++h->advance_count;
  if (h->d_ctr_prev) {
    CK(cudaMemcpyAsync(h->d_ctr_prev, h->d_ctr, 8 * (size_t)h->n, cudaMemcpyDeviceToDevice, h->stream));
    h->ctr_prev_valid = true;
  }
  const int bps = h->blocks_per_sm > 0 ? h->blocks_per_sm : default_blocks_per_sm(h);
  float ms = 0;
  int64_t steps = 0;
  int rc = launch_step(h, t_begin, t_end, bps, h->sort_interval > 0 && h->perm_valid, &ms, &steps);
  if (rc != MPRW_OK) return rc;
  h->step_ms = ms;
  if (steps_done) *steps_done = steps;
  return MPRW_OK;
}

int mprw_set_timeout(mprw_handle *h, double timeout_ms) {
  if (!h) return MPRW_E_INVAL;
  if (h->parent) return fail(h, MPRW_E_STATE, "mprw_set_timeout on a batch member: set the batch's");
  if (!(timeout_ms >= 0.0)) return fail(h, MPRW_E_INVAL, "mprw_set_timeout: negative or NaN timeout");
  h->timeout_ms = timeout_ms;
  return MPRW_OK;
}

int mprw_cancel(mprw_handle *h) {
  if (!h) return MPRW_E_INVAL;
  mprw_handle *t = h->parent ? h->parent : h;
  if (t->h_abort) *t->h_abort = 1;
  return MPRW_OK;
}

int mprw_set_tuning(mprw_handle *h, int32_t blocks_per_sm, int32_t sort_interval) {
  if (!h) return MPRW_E_INVAL;
  if (h->parent) return fail(h, MPRW_E_STATE, "mprw_set_tuning on a batch member: tune the batch");
  if (blocks_per_sm < 0 || sort_interval < 0) return fail(h, MPRW_E_INVAL, "mprw_set_tuning: negative value");
  if (blocks_per_sm > max_blocks_per_sm(h))
    return fail(h, MPRW_E_INVAL, "mprw_set_tuning: more blocks per SM than the step kernel can keep resident");
  h->blocks_per_sm = blocks_per_sm;
  h->sort_interval = sort_interval;
  h->advance_count = 0;
  return MPRW_OK;
}

int mprw_get_tuning(mprw_handle *h, int32_t *blocks_per_sm, int32_t *sort_interval, int32_t *max_blocks) {
  if (!h) return MPRW_E_INVAL;
  if (blocks_per_sm) *blocks_per_sm = h->blocks_per_sm > 0 ? h->blocks_per_sm : default_blocks_per_sm(h);
  if (sort_interval) *sort_interval = h->sort_interval;
  if (max_blocks) *max_blocks = max_blocks_per_sm(h);
  return MPRW_OK;
}

int mprw_autotune(mprw_handle *h, double t_begin, double t_end, int32_t *blocks_per_sm, int32_t *sort_interval,
                  double *rates) {
  NvtxRange nvtx_("mprw_autotune");
  if (!h) return MPRW_E_INVAL;
  if (h->parent) return fail(h, MPRW_E_STATE, "mprw_autotune on a batch member: tune the batch");
  if (!h->members.empty()) {
    h->flow_loaded = true;
    for (size_t k = 0; k < h->members.size(); ++k)
      if (!h->members[k]->flow_loaded) return fail(h, MPRW_E_STATE, "mprw_autotune before every member's flow");
  }
  if (!h->flow_loaded) return fail(h, MPRW_E_STATE, "mprw_autotune before mprw_load_flow");
  if (!(t_end > t_begin)) return fail(h, MPRW_E_INVAL, "mprw_autotune: t_end <= t_begin");
  if (h->n == 0) return fail(h, MPRW_E_STATE, "mprw_autotune without particles");
  cudaStream_t s = h->stream;
  const int64_t n = h->n;
  const size_t rs = h->opt.precision == MPRW_MIXED ? sizeof(float) : sizeof(double);
  // the trials run on the real arrays from a saved copy of the state they change
  struct Field {
    void *p;
    size_t bytes;
  } fields[] = {{h->d_cell, 4 * (size_t)n}, {h->d_status, 4 * (size_t)n}, {h->d_x, rs * n}, {h->d_y, rs * n},
                {h->d_z, rs * n},         {h->d_t, 8 * (size_t)n},      {h->d_ctr, 8 * (size_t)n}};
  size_t total = 0;
  for (const Field &f : fields) total += (f.bytes + 255) / 256 * 256;
  char *save = nullptr;
  CK(cudaMalloc(&save, total));
  struct Free {
    char *p;
    ~Free() { cudaFree(p); }
  } guard{save};
  auto snapshot = [&](bool restore) -> cudaError_t {
    size_t o = 0;
    for (const Field &f : fields) {
      cudaError_t e = restore ? cudaMemcpyAsync(f.p, save + o, f.bytes, cudaMemcpyDeviceToDevice, s)
                              : cudaMemcpyAsync(save + o, f.p, f.bytes, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return e;
      o += (f.bytes + 255) / 256 * 256;
    }
    return cudaSuccess;
  };
  CK(snapshot(false));
  const int maxb = std::min(max_blocks_per_sm(h), 4);
  double best_rate = -1.0, rate_sorted = 0.0;
  int best_b = default_blocks_per_sm(h);
  int k = 0;
  // blocks per SM: every resident count, each from the same state, sorted first
  for (int b = 1; b <= maxb; ++b) {
    CK(snapshot(true));
    CK(cudaEventRecord(h->ev2, s));
    int rc = sort_particles(h);
    if (rc != MPRW_OK) return rc;
    float ms = 0, sort_ms = 0;
    int64_t st = 0;
    CK(cudaEventRecord(h->ev3, s));
    rc = launch_step(h, t_begin, t_end, b, true, &ms, &st);
    if (rc != MPRW_OK) return rc;
    CK(cudaEventElapsedTime(&sort_ms, h->ev2, h->ev3));
    const double r = st / (double)(ms + sort_ms);
    if (rates) rates[k++] = r;
    if (r > best_rate) {
      best_rate = r;
      best_b = b;
      rate_sorted = r;
    }
  }
  // the same without sorting: the particles in the order the caller gave
  CK(snapshot(true));
  float ms_u = 0;
  int64_t st_u = 0;
  int rc = launch_step(h, t_begin, t_end, best_b, false, &ms_u, &st_u);
  if (rc != MPRW_OK) return rc;
  const double rate_unsorted = st_u / (double)ms_u;
  if (rates) rates[k++] = rate_unsorted;
  // sorting pays when a sorted advance (sort included) is faster; when it is
  // close, sort every 4th advance to keep most of the locality for less
  int si = 1;
  if (rate_unsorted > rate_sorted * 1.05) si = 0;
  else if (rate_unsorted > rate_sorted * 0.97) si = 4;
  CK(snapshot(true));
  CK(cudaStreamSynchronize(s));
  h->perm_valid = false;
  h->blocks_per_sm = best_b;
  h->sort_interval = si;
  h->advance_count = 0;
  if (blocks_per_sm) *blocks_per_sm = best_b;
  if (sort_interval) *sort_interval = si;
  return MPRW_OK;
}

int mprw_get_particles(mprw_handle *h, int32_t *cell, double *lx, double *ly, double *lz, double *t,
                       int32_t *status, uint64_t *rng_ctr, double *gx, double *gy, double *gz) {
  if (!h) return MPRW_E_INVAL;
  if (!h->members.empty()) {
    // a batch: every member's particles in batch order, member-local cells
    for (mprw_handle *m : h->members) {
      const int64_t o = m->p0;
      int rc = mprw_get_particles(m, cell ? cell + o : nullptr, lx ? lx + o : nullptr, ly ? ly + o : nullptr,
                                  lz ? lz + o : nullptr, t ? t + o : nullptr, status ? status + o : nullptr,
                                  rng_ctr ? rng_ctr + o : nullptr, gx ? gx + o : nullptr, gy ? gy + o : nullptr,
                                  gz ? gz + o : nullptr);
      if (rc != MPRW_OK) return fail(h, rc, m->err);
    }
    return MPRW_OK;
  }
  const int64_t n = h->n;
  if (n == 0) return MPRW_OK;
  cudaStream_t s = h->stream;
  const bool mixed = h->opt.precision == MPRW_MIXED;
  if (cell) {
    // back to 1-based cells on the device, through the scratch buffer
    const size_t need = (size_t)4 * n;
    if (h->scratch_bytes < need) {
      if (h->scratch) cudaFree(h->scratch);
      h->scratch = nullptr;
      h->scratch_bytes = 0;
      CK(cudaMalloc(&h->scratch, need));
      h->scratch_bytes = need;
    }
    cell_out_kernel<<<grid1d(n), 256, 0, s>>>(h->d_cell, n, 1 - h->cell0, (int32_t *)h->scratch);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(cell, h->scratch, 4 * n, cudaMemcpyDeviceToHost, s));
    // the scratch buffer is reused for the model coordinates below
    if (gx || gy || gz) CK(cudaStreamSynchronize(s));
  }
  double *outs[3] = {lx, ly, lz};
  void *srcs[3] = {h->d_x, h->d_y, h->d_z};
  for (int a = 0; a < 3; ++a) {
    if (!outs[a]) continue;
    if (mixed) {
      if (!h->d_stage) CK(dalloc(&h->d_stage, h->cap));
      f32_to_f64_kernel<<<grid1d(n), 256, 0, s>>>((const float *)srcs[a], h->d_stage, n);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(outs[a], h->d_stage, 8 * n, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    } else {
      CK(cudaMemcpyAsync(outs[a], srcs[a], 8 * n, cudaMemcpyDeviceToHost, s));
    }
  }
  if (t) CK(cudaMemcpyAsync(t, h->d_t, 8 * n, cudaMemcpyDeviceToHost, s));
  if (status) CK(cudaMemcpyAsync(status, h->d_status, 4 * n, cudaMemcpyDeviceToHost, s));
  if (rng_ctr) CK(cudaMemcpyAsync(rng_ctr, h->d_ctr, 8 * n, cudaMemcpyDeviceToHost, s));
  if (gx || gy || gz) {
    size_t arr = ((size_t)n * 8 + 255) / 256 * 256;
    if (h->scratch_bytes < 3 * arr) {
      if (h->scratch) cudaFree(h->scratch);
      h->scratch = nullptr;
      h->scratch_bytes = 0;
      CK(cudaMalloc(&h->scratch, 3 * arr));
      h->scratch_bytes = 3 * arr;
    }
    double *g0 = (double *)h->scratch, *g1 = (double *)((char *)h->scratch + arr),
           *g2 = (double *)((char *)h->scratch + 2 * arr);
    Geometry geo = geometry(h);
    if (mixed)
      CK(launch_global_xyz<float>(geo, n, h->d_cell, (const float *)h->d_x, (const float *)h->d_y,
                                  (const float *)h->d_z, g0, g1, g2, s));
    else
      CK(launch_global_xyz<double>(geo, n, h->d_cell, (const double *)h->d_x, (const double *)h->d_y,
                                   (const double *)h->d_z, g0, g1, g2, s));
    if (gx) CK(cudaMemcpyAsync(gx, g0, 8 * n, cudaMemcpyDeviceToHost, s));
    if (gy) CK(cudaMemcpyAsync(gy, g1, 8 * n, cudaMemcpyDeviceToHost, s));
    if (gz) CK(cudaMemcpyAsync(gz, g2, 8 * n, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  return MPRW_OK;
}

}  // extern "C"

namespace {

// h->d_counts holds at least nbins doubles (and nbins 32-bit counters after them)
int ensure_counts(mprw_handle *h, int64_t nbins) {
  if (nbins > h->counts_cap) {
    if (h->d_counts) cudaFree(h->d_counts);
    h->d_counts = nullptr;
    h->counts_cap = 0;
    CK(cudaMalloc(&h->d_counts, sizeof(double) * nbins + sizeof(unsigned int) * nbins));
    h->counts_cap = nbins;
  }
  return MPRW_OK;
}

// Histogram of the active particles into h->d_counts (counts / effMass, the
// reference's histogram%counts after ComputeCountsWeighted; with raw, the
// mass per bin, not divided).  wsums (may be NULL) receives the sum of the
// weights and of their squares that the effective mass comes from (NaN for
// unit masses, whose effective mass is 1).
int histogram_device(mprw_handle *h, const double origin[3], const double bin_size[3], const int32_t n_bins[3],
                     int64_t *n_binned, double *eff_mass, double *wsums, bool raw = false) {
  int64_t nbins = 1;
  HistArgs a{};
  for (int d = 0; d < 3; ++d) {
    if (n_bins[d] < 1) return fail(h, MPRW_E_INVAL, "histogram: n_bins must be >= 1");
    if (bin_size[d] < 0.0) return fail(h, MPRW_E_INVAL, "histogram: bin_size must be >= 0");
    nbins *= n_bins[d];
    a.origin[d] = origin[d];
    a.bin[d] = bin_size[d];
    a.inv_bin[d] = bin_size[d] > 0 ? 1.0 / bin_size[d] : 0.0;
    a.nb[d] = n_bins[d];
    a.active_dim[d] = bin_size[d] != 0.0;
  }
  if (nbins > ((int64_t)1 << 31)) return fail(h, MPRW_E_INVAL, "histogram: too many bins");
  cudaStream_t s = h->stream;
  const int64_t n = h->n;
  if (ensure_counts(h, nbins) != MPRW_OK) return MPRW_E_OOM;
  a.geo = geometry(h);
  a.n = n;
  a.cell = h->d_cell;
  a.status = h->d_status;
  a.x = h->d_x;
  a.y = h->d_y;
  a.z = h->d_z;
  a.mixed = h->opt.precision == MPRW_MIXED;
  a.nbinned = h->d_counters + 2;
  double total = 0, sw2 = 0, eff = 1.0;
  int64_t nb_out = 0;
  if (h->unit_mass) {
    unsigned int *c32 = (unsigned int *)(h->d_counts + nbins);
    CK(cudaMemsetAsync(c32, 0, (size_t)nbins * 4, s));
    CK(cudaMemsetAsync(h->d_counters + 2, 0, 2 * sizeof(unsigned long long), s));
    a.counts32 = c32;
    CK(launch_hist_unit(a, s));
    CK(launch_u32_to_f64(c32, h->d_counts, nbins, s));
    h->launches += 2;
    CK(cudaMemcpyAsync(h->h_counters + 2, h->d_counters + 2, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    nb_out = (int64_t)h->h_counters[2];
    eff = 1.0;  // unit weights: Kish nEffective = totalMass, effective mass 1
  } else {
    size_t arr = ((size_t)n * 8 + 255) / 256 * 256;
    void *tmp = nullptr;
    CK(cudaMalloc(&tmp, arr));
    int64_t *bin_of = (int64_t *)tmp;
    a.bin_of = bin_of;
    cudaError_t e = launch_hist_bins(a, s);
    if (e == cudaSuccess)
      e = ordered_bin_sums(bin_of, h->d_mass, h->d_status, n, nbins, h->d_counts, &total, &sw2, &h->scratch,
                           &h->scratch_bytes, s);
    if (e == cudaSuccess && total != 0.0) {
      double neff = total * total / sw2;  // Kish (Histogram.F90:338-340)
      eff = total / neff;
      if (!raw) {
        div_kernel<<<grid1d(nbins), 256, 0, s>>>(h->d_counts, nbins, eff);
        e = cudaGetLastError();
      }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(tmp);
    CK(e);
    h->launches += 5;
    nb_out = -1;
  }
  if (n_binned) *n_binned = nb_out;
  if (eff_mass) *eff_mass = eff;
  if (wsums) {
    wsums[0] = h->unit_mass ? NAN : total;
    wsums[1] = h->unit_mass ? NAN : sw2;
  }
  return MPRW_OK;
}

}  // namespace

extern "C" {

int mprw_histogram(mprw_handle *h, const double origin[3], const double bin_size[3], const int32_t n_bins[3],
                   double *counts, int64_t *n_binned, double *eff_mass) {
  NvtxRange nvtx_("mprw_histogram");
  if (!h) return MPRW_E_INVAL;
  if (!h->members.empty()) return fail(h, MPRW_E_STATE, "mprw_histogram on a batch: use a member view");
  if (!origin || !bin_size || !n_bins || !counts) return fail(h, MPRW_E_INVAL, "mprw_histogram: null argument");
  h->launches = 0;
  cudaStream_t s = h->stream;
  CK(cudaEventRecord(h->ev2, s));
  int rc = histogram_device(h, origin, bin_size, n_bins, n_binned, eff_mass, nullptr);
  if (rc != MPRW_OK) return rc;
  const int64_t nbins = (int64_t)n_bins[0] * n_bins[1] * n_bins[2];
  CK(cudaMemcpyAsync(counts, h->d_counts, 8 * (size_t)nbins, cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(h->ev3, s));
  CK(cudaStreamSynchronize(s));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, h->ev2, h->ev3));
  h->hist_ms = ms;
  return MPRW_OK;
}

}  // extern "C"

namespace {

// The constants of a reconstruction grid from its options: prInitialize
// (GridProjectedKDE.F90:354-998), the kernel database (prInitializeKernel-
// DatabaseFlat, prGenerateLogSpaceData) and the kernel-size bounds.  Returns
// MPRW_OK, or the failure recorded on h.
int gpkde_params(mprw_handle *h, const mprw_gpkde_options *o, const char *who, KdeParams &P, int32_t nb[3]) {
  P = KdeParams{};
  for (int d = 0; d < 3; ++d) {
    if (o->bin_size[d] < 0.0 || o->domain_size[d] < 0.0) return fail(h, MPRW_E_INVAL, std::string(who) + ": negative size");
    nb[d] = (o->bin_size[d] != 0.0) ? (int32_t)(o->domain_size[d] / o->bin_size[d] + 0.5) : 1;
    if (nb[d] < 1) return fail(h, MPRW_E_INVAL, std::string(who) + ": grid size < 1");
    P.nb[d] = nb[d];
    P.bin[d] = o->bin_size[d];
    P.mask[d] = (nb[d] != 1) ? 1 : 0;
  }
  P.ndim = P.mask[0] + P.mask[1] + P.mask[2];
  if (P.ndim < 1) return fail(h, MPRW_E_INVAL, std::string(who) + ": the grid has no dimension with more than one bin");
  // idDim1 < idDim2: the active dimensions of a 2-D grid (GridProjectedKDE.F90 prInitialize)
  P.d1 = P.d2 = -1;
  for (int d = 0; d < 3; ++d)
    if (P.mask[d]) {
      if (P.d1 < 0) P.d1 = d;
      else if (P.d2 < 0) P.d2 = d;
    }
  if (o->isotropic != 0 && o->isotropic != 1) return fail(h, MPRW_E_INVAL, std::string(who) + ": isotropic must be 0 or 1");
  P.isotropic = o->isotropic;
  if (!(o->min_hover_delta > 0.0) || !(o->max_hover_delta > o->min_hover_delta) || !(o->delta_hover_delta > 0.0))
    return fail(h, MPRW_E_INVAL, std::string(who) + ": invalid kernel database parameters");
  if (o->precision != MPRW_FP64 && o->precision != MPRW_MIXED)
    return fail(h, MPRW_E_INVAL, std::string(who) + ": precision");
  double binvol = 1.0;
  int hd = 0;
  for (int d = 0; d < 3; ++d)
    if (P.bin[d] > 0.0) {
      binvol *= P.bin[d];
      ++hd;
    }
  P.binvol = binvol;
  {
    int e = 0;
    P.inv_binvol = (binvol > 0.0 && std::frexp(binvol, &e) == 0.5) ? 1.0 / binvol : 0.0;
  }
  P.bin_distance = std::pow(binvol, 1.0 / (double)hd);
  const double nd = (double)P.ndim;
  P.support_c = std::pow((nd + 2.0) * std::pow(8.0 * PI_D, 0.5 * nd), 0.25);
  P.alpha_c = std::pow((1.0 + std::pow(2.0, 0.5 * nd + 2.0)) / (3.0 * std::pow(2.0, 4.0 / (nd + 4.0))),
                       1.0 / (nd + 6.0)) *
              std::pow(nd + 2.0, 1.0 / (nd + 4.0)) / (std::pow(nd + 4.0, 1.0 / (nd + 6.0)));
  P.beta_c = 2.0 / (nd + 4.0) / (nd + 6.0);
  P.one_over_nd4 = 1.0 / (nd + 4.0);
  P.minus_one_over_nd6 = -1.0 / (nd + 6.0);
  P.one_plus_nd_q = 1.0 + 0.25 * nd;
  P.four_pi_half_nd = std::pow(4.0 * PI_D, 0.5 * nd);
  P.max_sigma_growth = 1.5;
  P.iso_threshold = 0.85;
  // logarithmic database (prInitializeKernelDatabaseFlat, prGenerateLogSpaceData)
  const int ndelta = (int)std::ceil(std::log10(o->max_hover_delta / o->min_hover_delta) /
                                    std::log10(1 + o->delta_hover_delta)) + 1;
  if (ndelta > KDE_MAXDB || ndelta < 2) return fail(h, MPRW_E_INVAL, std::string(who) + ": kernel database too large");
  P.ndelta = ndelta;
  {
    const double li = std::log10(o->min_hover_delta), le = std::log10(o->max_hover_delta);
    const double de = (le - li) / (ndelta - 1);
    double acc = 0.0;
    for (int n = 0; n < ndelta; ++n) {
      P.hod[n] = std::pow(10.0, li + acc);
      acc = acc + de;
    }
  }
  if (o->max_hover_delta * 4 * 2 + 1 > KDE_MAXLEN) return fail(h, MPRW_E_INVAL, std::string(who) + ": maxHOverDelta too large");
  P.min_hod = o->min_hover_delta;
  P.dlog = std::log(P.hod[1] / P.hod[0]);
  for (int d = 0; d < 3; ++d) P.lscale[d] = P.bin[d] > 0.0 ? (float)(1.0 / (P.bin[d] * P.min_hod)) : 0.0f;
  P.linv = (float)(1.0 / P.dlog);
  // bounded kernel sizes (boundKernelSizeFormat 0)
  int maxd = -1, mind = -1;
  for (int d = 0; d < 3; ++d) {
    if (!P.mask[d]) continue;
    P.max_k[d] = P.bin[d] * (0.9 * nb[d] - 1) / 3.0;
    P.max_sd[d] = P.bin[d] * (0.9 * nb[d] - 1) / 4.0;
    P.min_k[d] = 1.2 * P.bin[d] / 3.0;
    P.min_sd[d] = 1.2 * P.bin[d] / 4.0;
  }
  for (int d = 0; d < 3; ++d)
    if (P.max_k[d] > 0.0 && (maxd < 0 || P.max_k[d] < P.max_k[maxd])) maxd = d;
  for (int d = 0; d < 3; ++d)
    if (P.min_k[d] > 0.0 && (mind < 0 || P.min_k[d] > P.min_k[mind])) mind = d;
  if (maxd < 0 || mind < 0) return fail(h, MPRW_E_INVAL, std::string(who) + ": grid too small for bounded kernels");
  P.max_dim = maxd;
  P.min_dim = mind;
  return MPRW_OK;
}

// Sums over the ACTIVE particles' model coordinates, fixed-order per block
// and summed on the host in block order: pass 0 the coordinates and the
// count, pass 2 the coordinates minus m and the count, pass 1 the squares of
// the coordinates minus m (acc[3] unused).
int coord_sums(mprw_handle *h, int pass, const double m[3], double acc[4]) {
  cudaStream_t s = h->stream;
  if (!h->d_kpart) CK(cudaMalloc(&h->d_kpart, sizeof(double) * 4 * 152 * 4));
  int nblk = 0;
  const double zero[3] = {0, 0, 0};
  CK(launch_coord_sums(geometry(h), h->n, h->d_cell, h->d_status, h->d_x, h->d_y, h->d_z,
                       h->opt.precision == MPRW_MIXED, pass, m ? m : zero, h->d_kpart, &nblk, s));
  std::vector<double> part(4 * (size_t)nblk);
  CK(cudaMemcpyAsync(part.data(), h->d_kpart, sizeof(double) * 4 * nblk, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int k = 0; k < 4; ++k) acc[k] = 0.0;
  for (int i = 0; i < nblk; ++i)
    for (int k = 0; k < 4; ++k) acc[k] += part[4 * i + k];
  h->launches += 1;
  return MPRW_OK;
}

// The reconstruction from the histogram in h->d_counts (counts / effMass,
// the grid of P) and the statistics of the reconstructed points (standard
// deviation per dimension, their number npts): active bins, factor tables,
// the optimisation loop, the exported density and, when asked, the
// histogram (mass per bin) to the host.  The caller has recorded h->ev2.
int gpkde_reconstruct(mprw_handle *h, const mprw_gpkde_options *o, KdeParams &P, const int32_t nb[3], double eff,
                      const double sd[3], double npts, double *density, double *histogram, int32_t *loops_done) {
  cudaStream_t s = h->stream;
  const int fp32 = o->precision == MPRW_MIXED;
  const int64_t ngrid = (int64_t)nb[0] * nb[1] * nb[2];
  const double nd = (double)P.ndim;
  double binvol = P.binvol;
  // active bins
  int nactive = 0;
  CK(kde_collect_active(*h->kdep, P, h->d_counts, s, &nactive));
  int loops = 0;
  h->kde_work = 0.0;
  if (nactive > 0) {
    // initial smoothing (initialSmoothingSelection 0: Silverman-type scale)
    double prod = 1.0;
    for (int d = 0; d < 3; ++d)
      if (P.mask[d]) prod *= sd[d];
    const double ss = std::pow(prod, 1.0 / nd);
    double hs = ss * std::pow(4.0 / ((nd + 2.0) * npts), 1.0 / (nd + 4.0));
    if (ss == 0.0) hs = 2.0 * P.bin_distance;
    // factor tables, rebuilt only when the database or the bins change
    std::vector<double> key = {(double)P.ndim, (double)P.ndelta, P.bin[0], P.bin[1], P.bin[2],
                               (double)P.mask[0], (double)P.mask[1], (double)P.mask[2]};
    key.insert(key.end(), P.hod, P.hod + P.ndelta);
    if (!h->kdep->d_val || key != h->kdep->table_key) {
      std::vector<double> val;
      std::vector<int> wm, wofs, sm[3], sofs[3];
      kde_build_tables(P, val, wm, wofs, sm, sofs);
      CK(cudaStreamSynchronize(s));
      if (h->kdep->d_val) cudaFree(h->kdep->d_val);
      if (h->kdep->d_meta) cudaFree(h->kdep->d_meta);
      h->kdep->d_val = nullptr;
      h->kdep->d_meta = nullptr;
      h->kdep->table_key.clear();
      CK(cudaMalloc(&h->kdep->d_val, sizeof(double) * val.size()));
      CK(cudaMalloc(&h->kdep->d_meta, sizeof(int) * 8 * 3 * KDE_MAXDB));
      std::vector<int> meta;
      meta.insert(meta.end(), wm.begin(), wm.end());
      meta.insert(meta.end(), wofs.begin(), wofs.end());
      for (int a = 0; a < 3; ++a) {
        meta.insert(meta.end(), sm[a].begin(), sm[a].end());
        meta.insert(meta.end(), sofs[a].begin(), sofs[a].end());
      }
      std::vector<float> valf(val.begin(), val.end());
      if (h->kdep->d_valf) cudaFree(h->kdep->d_valf);
      h->kdep->d_valf = nullptr;
      CK(cudaMalloc(&h->kdep->d_valf, sizeof(float) * valf.size()));
      CK(cudaMemcpyAsync(h->kdep->d_val, val.data(), sizeof(double) * val.size(), cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(h->kdep->d_valf, valf.data(), sizeof(float) * valf.size(), cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(h->kdep->d_meta, meta.data(), sizeof(int) * meta.size(), cudaMemcpyHostToDevice, s));
      CK(cudaStreamSynchronize(s));  // the host vectors go out of scope
      h->kdep->table_key = key;
    }
    const int L = 3 * KDE_MAXDB;
    h->kdep->wtab = KdeTable{h->kdep->d_val, h->kdep->d_meta, h->kdep->d_meta + L};
    for (int a = 0; a < 3; ++a)
      h->kdep->sdtab[a] = KdeTable{h->kdep->d_val, h->kdep->d_meta + (2 + 2 * a) * L, h->kdep->d_meta + (3 + 2 * a) * L};
    cudaError_t e = kde_run(*h->kdep, P, hs, npts, o->n_opt_loops, o->rel_err_convergence,
                            o->skip_error_convergence != 0, fp32, s, &loops);
    if (e == cudaErrorInvalidValue) return fail(h, MPRW_E_INVAL, "mprw_gpkde: net roughness is zero everywhere");
    CK(e);
    h->kde_work = h->kdep->work_madds;
    // effective mass, unit volume, scaling (GridProjectedKDE.F90:4292-4306, 5080-5084)
    double f = eff;
    double scale = 1.0;
    if (o->unit_volume) scale *= binvol;
    if (o->scaling_factor != 0.0) scale *= o->scaling_factor;
    CK(kde_output(*h->kdep, P, fp32, f, scale, s));
  } else {
    CK(cudaMemsetAsync(h->kdep->dens_out, 0, sizeof(double) * ngrid, s));
  }
  // outputs through pinned staging (density, then histogram)
  const int64_t nout = histogram ? 2 * ngrid : ngrid;
  if (nout > h->kdep->h_out_cap) {
    CK(cudaStreamSynchronize(s));
    if (h->kdep->h_out) cudaFreeHost(h->kdep->h_out);
    h->kdep->h_out = nullptr;
    h->kdep->h_out_cap = 0;
    CK(cudaMallocHost(&h->kdep->h_out, sizeof(double) * nout));
    h->kdep->h_out_cap = nout;
  }
  CK(cudaMemcpyAsync(h->kdep->h_out, h->kdep->dens_out, sizeof(double) * ngrid, cudaMemcpyDeviceToHost, s));
  if (histogram) {
    mul2_kernel<<<grid1d(ngrid), 256, 0, s>>>(h->d_counts, ngrid, eff, 1.0);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->kdep->h_out + ngrid, h->d_counts, sizeof(double) * ngrid, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaEventRecord(h->ev3, s));
  CK(cudaStreamSynchronize(s));
  std::memcpy(density, h->kdep->h_out, sizeof(double) * ngrid);
  if (histogram) std::memcpy(histogram, h->kdep->h_out + ngrid, sizeof(double) * ngrid);
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, h->ev2, h->ev3));
  h->kde_ms = ms;
  h->launches += h->kdep->launches + 2;
  if (loops_done) *loops_done = loops;
  return MPRW_OK;
}

}  // namespace

extern "C" {


int mprw_gpkde(mprw_handle *h, const mprw_gpkde_options *o, double *density, double *histogram,
               int32_t n_bins_out[3], int32_t *loops_done) {
  NvtxRange nvtx_("mprw_gpkde");
  if (!h) return MPRW_E_INVAL;
  if (!h->members.empty()) return fail(h, MPRW_E_STATE, "mprw_gpkde on a batch: use a member view");
  if (!o || !density) return fail(h, MPRW_E_INVAL, "mprw_gpkde: null argument");
  KdeParams P;
  int32_t nb[3];
  int rc = gpkde_params(h, o, "mprw_gpkde", P, nb);
  if (rc != MPRW_OK) return rc;
  if (n_bins_out)
    for (int d = 0; d < 3; ++d) n_bins_out[d] = nb[d];
  cudaStream_t s = h->stream;
  h->launches = 0;
  h->kdep->launches = 0;
  CK(cudaEventRecord(h->ev2, s));
  // histogram (counts / effective mass)
  int64_t nbinned = 0;
  double eff = 1.0;
  rc = histogram_device(h, o->origin, o->bin_size, nb, &nbinned, &eff, nullptr);
  if (rc != MPRW_OK) return rc;
  const int64_t ngrid = (int64_t)nb[0] * nb[1] * nb[2];
  // statistics of the active particles' coordinates (GridProjectedKDE.F90:4023-4030)
  CK(h->kdep->ensure_grid(ngrid));
  double mean[3] = {0, 0, 0}, sd[3] = {0, 0, 0}, acc[4];
  rc = coord_sums(h, 0, nullptr, acc);
  if (rc != MPRW_OK) return rc;
  const double npts = acc[3];
  if (npts > 0)
    for (int d = 0; d < 3; ++d) mean[d] = acc[d] / npts;
  rc = coord_sums(h, 1, mean, acc);
  if (rc != MPRW_OK) return rc;
  for (int d = 0; d < 3; ++d) sd[d] = (P.mask[d] && npts > 0) ? std::sqrt(acc[d] / npts) : 0.0;
  return gpkde_reconstruct(h, o, P, nb, eff, sd, npts, density, histogram, loops_done);
}

int mprw_gpkde_partial(mprw_handle *h, const mprw_gpkde_options *o, double *mass_per_bin, mprw_gpkde_sums *sums) {
  NvtxRange nvtx_("mprw_gpkde_partial");
  if (!h) return MPRW_E_INVAL;
  if (!h->members.empty()) return fail(h, MPRW_E_STATE, "mprw_gpkde_partial on a batch: use a member view");
  if (!o || !mass_per_bin || !sums) return fail(h, MPRW_E_INVAL, "mprw_gpkde_partial: null argument");
  KdeParams P;
  int32_t nb[3];
  int rc = gpkde_params(h, o, "mprw_gpkde_partial", P, nb);
  if (rc != MPRW_OK) return rc;
  cudaStream_t s = h->stream;
  h->launches = 0;
  double wsums[2];
  rc = histogram_device(h, o->origin, o->bin_size, nb, nullptr, nullptr, wsums, true);
  if (rc != MPRW_OK) return rc;
  const int64_t ngrid = (int64_t)nb[0] * nb[1] * nb[2];
  CK(cudaMemcpyAsync(mass_per_bin, h->d_counts, sizeof(double) * ngrid, cudaMemcpyDeviceToHost, s));
  double c[3], acc[4];
  for (int d = 0; d < 3; ++d) c[d] = o->origin[d] + 0.5 * o->domain_size[d];
  rc = coord_sums(h, 2, c, acc);
  if (rc != MPRW_OK) return rc;
  sums->n_active = acc[3];
  for (int d = 0; d < 3; ++d) sums->sum_dx[d] = acc[d];
  rc = coord_sums(h, 1, c, acc);
  if (rc != MPRW_OK) return rc;
  for (int d = 0; d < 3; ++d) sums->sum_dx2[d] = acc[d];
  // unit masses: the weights are the particles themselves
  sums->sum_w = h->unit_mass ? sums->n_active : wsums[0];
  sums->sum_w2 = h->unit_mass ? sums->n_active : wsums[1];
  CK(cudaStreamSynchronize(s));
  return MPRW_OK;
}

int mprw_gpkde_from_counts(mprw_handle *h, const mprw_gpkde_options *o, const double *mass_per_bin,
                           const mprw_gpkde_sums *sums, double *density, double *histogram, int32_t n_bins_out[3],
                           int32_t *loops_done) {
  NvtxRange nvtx_("mprw_gpkde_from_counts");
  if (!h) return MPRW_E_INVAL;
  if (!h->members.empty()) return fail(h, MPRW_E_STATE, "mprw_gpkde_from_counts on a batch: use a member view");
  if (!o || !mass_per_bin || !sums || !density) return fail(h, MPRW_E_INVAL, "mprw_gpkde_from_counts: null argument");
  KdeParams P;
  int32_t nb[3];
  int rc = gpkde_params(h, o, "mprw_gpkde_from_counts", P, nb);
  if (rc != MPRW_OK) return rc;
  const double n = sums->n_active;
  if (!(n >= 0.0) || !std::isfinite(n) || !(sums->sum_w2 >= 0.0) || !std::isfinite(sums->sum_w) ||
      !std::isfinite(sums->sum_w2))
    return fail(h, MPRW_E_INVAL, "mprw_gpkde_from_counts: invalid sums");
  for (int d = 0; d < 3; ++d)
    if (!std::isfinite(sums->sum_dx[d]) || !std::isfinite(sums->sum_dx2[d]))
      return fail(h, MPRW_E_INVAL, "mprw_gpkde_from_counts: invalid sums");
  if (n_bins_out)
    for (int d = 0; d < 3; ++d) n_bins_out[d] = nb[d];
  cudaStream_t s = h->stream;
  h->launches = 0;
  h->kdep->launches = 0;
  CK(cudaEventRecord(h->ev2, s));
  const int64_t ngrid = (int64_t)nb[0] * nb[1] * nb[2];
  if (ensure_counts(h, ngrid) != MPRW_OK) return fail(h, MPRW_E_OOM, "mprw_gpkde_from_counts: device memory");
  CK(h->kdep->ensure_grid(ngrid));
  CK(cudaMemcpyAsync(h->d_counts, mass_per_bin, sizeof(double) * ngrid, cudaMemcpyHostToDevice, s));
  // Kish effective mass of the summed weights (Histogram.F90:338-340); the
  // mass per bin becomes histogram%counts
  double eff = 1.0;
  if (sums->sum_w != 0.0 && sums->sum_w2 != sums->sum_w) {
    const double neff = sums->sum_w * sums->sum_w / sums->sum_w2;
    eff = sums->sum_w / neff;
    div_kernel<<<grid1d(ngrid), 256, 0, s>>>(h->d_counts, ngrid, eff);
    CK(cudaGetLastError());
    h->launches += 1;
  }
  // mean and standard deviation from the sums about the domain centre
  double sd[3] = {0, 0, 0};
  for (int d = 0; d < 3; ++d) {
    if (!P.mask[d] || n <= 0.0) continue;
    const double m = sums->sum_dx[d] / n;
    const double v = sums->sum_dx2[d] / n - m * m;
    sd[d] = v > 0.0 ? std::sqrt(v) : 0.0;
  }
  return gpkde_reconstruct(h, o, P, nb, eff, sd, n, density, histogram, loops_done);
}

int mprw_gpkde_batch(mprw_handle *h, const mprw_gpkde_options *opts, double *const *density,
                     double *const *histogram, int32_t *loops_done, int32_t concurrency) {
  NvtxRange nvtx_("mprw_gpkde_batch");
  if (!h) return MPRW_E_INVAL;
  if (h->members.empty()) return fail(h, MPRW_E_STATE, "mprw_gpkde_batch: not a batch handle");
  if (!opts || !density) return fail(h, MPRW_E_INVAL, "mprw_gpkde_batch: null argument");
  const int nm = (int)h->members.size();
  for (int k = 0; k < nm; ++k)
    if (!density[k]) return fail(h, MPRW_E_INVAL, "mprw_gpkde_batch: null density for member " + std::to_string(k));
  int nw = concurrency > 0 ? concurrency : 4;
  if (nw > 16) nw = 16;
  if (nw > nm) nw = nm;
  while ((int)h->kde_workers.size() < nw) {
    KdeWorker *w = new KdeWorker();
    w->kde.device_loop = false;
    h->kde_workers.push_back(w);
    CK(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
  }
  const auto t0 = std::chrono::steady_clock::now();
  // the reconstructions read what the batch's stream last wrote
  CK(cudaEventRecord(h->ev2, h->stream));
  for (int i = 0; i < nw; ++i) CK(cudaStreamWaitEvent(h->kde_workers[i]->stream, h->ev2, 0));
  std::atomic<int> next{0};
  std::vector<int> rcs(nw, MPRW_OK);
  std::vector<std::string> errs(nw);
  std::vector<int64_t> launches(nw, 0);
  auto work = [&](int i) {
    KdeWorker *w = h->kde_workers[i];
    for (;;) {
      const int k = next.fetch_add(1);
      if (k >= nm) break;
      mprw_handle *m = h->members[k];
      cudaStream_t s0 = m->stream;
      KdeState *k0 = m->kdep;
      m->stream = w->stream;
      m->kdep = &w->kde;
      const int rc = mprw_gpkde(m, &opts[k], density[k], histogram ? histogram[k] : nullptr, nullptr,
                                loops_done ? &loops_done[k] : nullptr);
      m->stream = s0;
      m->kdep = k0;
      launches[i] += m->launches;
      if (rc != MPRW_OK) {
        rcs[i] = rc;
        errs[i] = "member " + std::to_string(k) + ": " + m->err;
        next.store(nm);
        break;
      }
    }
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < nw; ++i) pool.emplace_back(work, i);
  work(0);
  for (auto &t : pool) t.join();
  for (int i = 0; i < nw; ++i)
    if (rcs[i] != MPRW_OK) return fail(h, rcs[i], errs[i]);
  h->launches = 0;
  for (int i = 0; i < nw; ++i) h->launches += launches[i];
  h->kde_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return MPRW_OK;
}

// ---- observation cells (Observation.f90; MPathRW.F90:1337-1392, 1460-1535) ----
static ObsArgs obs_args(const mprw_handle *h) {
  ObsArgs a{};
  a.n = h->n;
  a.cell = h->d_cell;
  a.status = h->d_status;
  a.t = h->d_t;
  a.mass = h->unit_mass ? nullptr : h->d_mass;
  a.id = h->has_id ? h->d_id : nullptr;
  a.obs_of_cell = h->d_obs_of_cell;
  a.obs_style = h->d_obs_style;
  a.t_begin = h->last_t_begin;
  a.t_end = h->last_t_end;
  a.cell0 = h->cell0;
  return a;
}

int mprw_set_observations(mprw_handle *h, int32_t ncells, const int32_t *cells, const int32_t *obs, int32_t nobs,
                          const int32_t *style) {
  if (!h) return MPRW_E_INVAL;
  if (!h->members.empty()) return fail(h, MPRW_E_STATE, "mprw_set_observations on a batch: use a member view");
  if (ncells < 0 || nobs < 0 || (ncells > 0 && (!cells || !obs)) || (nobs > 0 && !style))
    return fail(h, MPRW_E_INVAL, "mprw_set_observations: null argument or negative size");
  const int32_t ncell = h->g.ncell;
  std::vector<int32_t> of(ncell, -1);
  for (int32_t i = 0; i < ncells; ++i) {
    if (cells[i] < 1 || cells[i] > ncell) return fail(h, MPRW_E_INVAL, "mprw_set_observations: cell out of range");
    if (obs[i] < 0 || obs[i] >= nobs) return fail(h, MPRW_E_INVAL, "mprw_set_observations: observation index");
    int32_t &o = of[cells[i] - 1];
    if (o >= 0 && o != obs[i]) return fail(h, MPRW_E_INVAL, "mprw_set_observations: cell in two observations");
    o = obs[i];
  }
  for (int32_t k = 0; k < nobs; ++k)
    if (style[k] != 1 && style[k] != 2) return fail(h, MPRW_E_INVAL, "mprw_set_observations: style (1 or 2)");
  cudaStream_t s = h->stream;
  CK(cudaStreamSynchronize(s));
  for (void *p : {(void *)h->d_obs_of_cell, (void *)h->d_obs_style, (void *)h->d_obs_count, (void *)h->d_obs_mass})
    if (p) cudaFree(p);
  h->d_obs_of_cell = h->d_obs_style = nullptr;
  h->d_obs_count = nullptr;
  h->d_obs_mass = nullptr;
  h->nobs = 0;
  const size_t k = nobs > 0 ? (size_t)nobs : 1;
  CK(cudaMalloc(&h->d_obs_of_cell, sizeof(int32_t) * ncell));
  CK(cudaMalloc(&h->d_obs_style, sizeof(int32_t) * k));
  CK(cudaMalloc(&h->d_obs_count, sizeof(unsigned long long) * k));
  CK(cudaMalloc(&h->d_obs_mass, sizeof(double) * k));
  CK(cudaMemcpyAsync(h->d_obs_of_cell, of.data(), sizeof(int32_t) * ncell, cudaMemcpyHostToDevice, s));
  if (nobs > 0) CK(cudaMemcpyAsync(h->d_obs_style, style, sizeof(int32_t) * nobs, cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  h->nobs = nobs;
  return MPRW_OK;
}

int mprw_observe_resident(mprw_handle *h, int64_t *count, double *mass) {
  if (!h) return MPRW_E_INVAL;
  if (!h->d_obs_of_cell) return fail(h, MPRW_E_STATE, "mprw_observe_resident before mprw_set_observations");
  if (h->nobs > 0 && (!count || !mass)) return fail(h, MPRW_E_INVAL, "mprw_observe_resident: null argument");
  if (h->nobs == 0) return MPRW_OK;
  cudaStream_t s = h->stream;
  CK(cudaMemsetAsync(h->d_obs_count, 0, sizeof(unsigned long long) * h->nobs, s));
  CK(cudaMemsetAsync(h->d_obs_mass, 0, sizeof(double) * h->nobs, s));
  CK(launch_resident(obs_args(h), h->d_obs_count, h->d_obs_mass, s));
  std::vector<unsigned long long> c(h->nobs);
  CK(cudaMemcpyAsync(c.data(), h->d_obs_count, sizeof(unsigned long long) * h->nobs, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(mass, h->d_obs_mass, sizeof(double) * h->nobs, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int32_t k = 0; k < h->nobs; ++k) count[k] = (int64_t)c[k];
  h->launches = 1;
  return MPRW_OK;
}

int mprw_observe_sinks(mprw_handle *h, int64_t capacity, int32_t *obs, uint64_t *id, double *time, double *mass,
                       int64_t *n_records) {
  if (!h) return MPRW_E_INVAL;
  if (!h->d_obs_of_cell) return fail(h, MPRW_E_STATE, "mprw_observe_sinks before mprw_set_observations");
  if (!n_records || capacity < 0 || (capacity > 0 && (!obs || !id || !time || !mass)))
    return fail(h, MPRW_E_INVAL, "mprw_observe_sinks: null argument or negative capacity");
  *n_records = 0;
  if (!h->advanced || h->n == 0 || h->nobs == 0) return MPRW_OK;
  cudaStream_t s = h->stream;
  int64_t m = 0;
  CK(collect_sink_records(obs_args(h), &h->scratch, &h->scratch_bytes, &m, s));
  *n_records = m;
  const int64_t w = m < capacity ? m : capacity;
  if (w > 0) {
    int32_t *d_obs;
    uint64_t *d_id;
    double *d_t, *d_m;
    CK(sink_record_arrays(h->scratch, h->n, &d_obs, &d_id, &d_t, &d_m));
    CK(cudaMemcpyAsync(obs, d_obs, sizeof(int32_t) * w, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(id, d_id, sizeof(uint64_t) * w, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(time, d_t, sizeof(double) * w, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(mass, d_m, sizeof(double) * w, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  h->launches = 3;
  return MPRW_OK;
}

int mprw_set_stream(mprw_handle *h, void *stream) {
  if (!h) return MPRW_E_INVAL;
  if (h->parent) return fail(h, MPRW_E_STATE, "mprw_set_stream on a batch member: set the batch's stream");
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  for (mprw_handle *m : h->members) m->stream = h->stream;
  return MPRW_OK;
}

int mprw_last_timings(mprw_handle *h, double *step_ms, double *prep_ms, double *hist_ms, double *gpkde_ms,
                      int64_t *launches) {
  if (!h) return MPRW_E_INVAL;
  if (step_ms) *step_ms = h->step_ms;
  if (prep_ms) *prep_ms = h->prep_ms;
  if (hist_ms) *hist_ms = h->hist_ms;
  if (gpkde_ms) *gpkde_ms = h->kde_ms;
  if (launches) *launches = h->launches;
  return MPRW_OK;
}

int mprw_last_gpkde_work(mprw_handle *h, double *madds) {
  if (!h || !madds) return MPRW_E_INVAL;
  *madds = h->kde_work;
  return MPRW_OK;
}

int mprw_destroy(mprw_handle *h) {
  if (!h) return MPRW_OK;
  if (h->parent) return MPRW_E_STATE;  // member views go with their batch
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
  return MPRW_OK;
}

// ---- differentiable walk and its adjoint (adjoint.cu) ----
int mprw_adj_setup(mprw_handle *h, const int32_t *zones, const mprw_adj_options *o) {
  NvtxRange nvtx_("mprw_adj_setup");
  if (!h) return MPRW_E_INVAL;
  if (h->parent || !h->members.empty()) return fail(h, MPRW_E_STATE, "mprw_adj_setup: not on a batch or member");
  if (!zones || !o) return fail(h, MPRW_E_INVAL, "mprw_adj_setup: null argument");
  if (!h->flow_loaded) return fail(h, MPRW_E_STATE, "mprw_adj_setup before mprw_load_flow");
  const GridDims g = h->g;
  const int64_t ncell = g.ncell;
  // a uniform grid: equal column widths, row widths and cell thicknesses
  std::vector<double> delr(g.ncol), delc(g.nrow), botm(ncell), ret(ncell);
  CK(cudaMemcpy(delr.data(), h->d_delr, sizeof(double) * g.ncol, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(delc.data(), h->d_delc, sizeof(double) * g.nrow, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(botm.data(), h->d_botm, sizeof(double) * ncell, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(ret.data(), h->d_ret, sizeof(double) * ncell, cudaMemcpyDeviceToHost));
  const double dx = delr[0], dy = delc[0], dz = h->h_top_cell[0] - botm[0];
  bool uniform = dx > 0.0 && dy > 0.0 && dz > 0.0;
  for (double v : delr) uniform = uniform && v == dx;
  for (double v : delc) uniform = uniform && v == dy;
  for (int64_t c = 0; c < ncell && uniform; ++c)
    uniform = std::fabs((h->h_top_cell[c] - botm[c]) - dz) <= 1e-12 * dz && botm[c] == botm[(c / g.ncpl) * g.ncpl];
  if (!uniform) return fail(h, MPRW_E_INVAL, "mprw_adj_setup: the walk needs a uniform grid (equal cell sizes)");
  for (int64_t c = 0; c < ncell; ++c)
    if (ret[c] != ret[0]) return fail(h, MPRW_E_INVAL, "mprw_adj_setup: the walk needs a uniform retardation");
  AdjInputs in{};
  in.g = g;
  in.geo = geometry(h);
  in.base = h->base;
  in.iboundts = h->d_ibts;
  in.dm = h->d_dm;
  in.dm_uniform = h->dm_uniform ? 1 : 0;
  in.R = ret[0];
  in.lo[0] = 0.0;
  in.lo[1] = 0.0;
  in.lo[2] = botm[(int64_t)(g.nlay - 1) * g.ncpl];
  in.d[0] = dx;
  in.d[1] = dy;
  in.d[2] = dz;
  in.n = h->n;
  in.cell = h->d_cell;
  in.status = h->d_status;
  in.x = h->d_x;
  in.y = h->d_y;
  in.z = h->d_z;
  in.mixed = h->opt.precision == MPRW_MIXED;
  in.mass = h->unit_mass ? nullptr : h->d_mass;
  in.id = h->has_id ? h->d_id : nullptr;
  AdjOptions ao{};
  ao.nzones = o->nzones;
  ao.dt = o->dt;
  ao.eps = o->velocity_floor;
  ao.nsteps = o->nsteps;
  ao.checkpoint = o->checkpoint;
  ao.seed = o->seed;
  for (int d = 0; d < 3; ++d) {
    ao.origin[d] = o->origin[d];
    ao.bin[d] = o->bin_size[d];
    ao.h[d] = o->bandwidth[d];
    ao.nb[d] = o->n_bins[d];
  }
  CK(cudaStreamSynchronize(h->stream));
  if (!h->adj) h->adj = new AdjState();
  std::vector<char> err;
  const cudaError_t e = h->adj->setup(in, ao, zones, err);
  if (e == cudaErrorInvalidValue && !err.empty()) return fail(h, MPRW_E_INVAL, std::string("mprw_adj_setup: ") + err.data());
  if (e == cudaErrorMemoryAllocation) return fail(h, MPRW_E_OOM, "mprw_adj_setup: device memory");
  CK(e);
  return MPRW_OK;
}

int mprw_adj_forward(mprw_handle *h, const double *theta, double *density) {
  NvtxRange nvtx_("mprw_adj_forward");
  if (!h) return MPRW_E_INVAL;
  if (!h->adj) return fail(h, MPRW_E_STATE, "mprw_adj_forward before mprw_adj_setup");
  if (!theta || !density) return fail(h, MPRW_E_INVAL, "mprw_adj_forward: null argument");
  const int nz = h->adj->o.nzones;
  for (int k = 0; k < 3 * nz + 1; ++k)
    if (!std::isfinite(theta[k])) return fail(h, MPRW_E_INVAL, "mprw_adj_forward: non-finite parameter");
  for (int z = 0; z < nz; ++z)
    if (!(theta[2 * nz + z] > 0.0) || theta[z] < 0.0 || theta[nz + z] < 0.0)
      return fail(h, MPRW_E_INVAL, "mprw_adj_forward: porosity must be > 0 and dispersivities >= 0");
  CK(cudaEventRecord(h->ev0, h->stream));
  CK(h->adj->forward(theta, density, h->stream));
  CK(cudaEventRecord(h->ev1, h->stream));
  CK(cudaEventSynchronize(h->ev1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  h->step_ms = ms;
  h->launches = h->adj->launches;
  return MPRW_OK;
}

int mprw_adj_backward(mprw_handle *h, const double *grad_density, double *grad_theta) {
  NvtxRange nvtx_("mprw_adj_backward");
  if (!h) return MPRW_E_INVAL;
  if (!h->adj || !h->adj->forward_done) return fail(h, MPRW_E_STATE, "mprw_adj_backward before mprw_adj_forward");
  if (!grad_density || !grad_theta) return fail(h, MPRW_E_INVAL, "mprw_adj_backward: null argument");
  CK(cudaEventRecord(h->ev0, h->stream));
  CK(h->adj->backward(grad_density, grad_theta, h->stream));
  CK(cudaEventRecord(h->ev1, h->stream));
  CK(cudaEventSynchronize(h->ev1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  h->step_ms = ms;
  h->launches = h->adj->launches;
  return MPRW_OK;
}

const char *mprw_last_error(const mprw_handle *h) { return h ? h->err.c_str() : "null handle"; }

}  // extern "C"
