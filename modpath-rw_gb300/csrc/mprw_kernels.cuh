// mprw_kernels.cuh -- kernel argument blocks and launch wrappers.
#pragma once
#include "mprw_common.cuh"

namespace mprw {

constexpr int kStepThreads = 256;
// FP64 EULERIAN step kernel: 384 threads per block (12 warps per SM fit in
// 168 registers; the FP64 pipe is fuller than with 8 warps at 236)
constexpr int kStepThreadsF64 = 384;
constexpr int step_threads(bool fp64, bool exp_adv) { return (fp64 && !exp_adv) ? kStepThreadsF64 : kStepThreads; }
constexpr int kAbortPoll = 256;  // main-loop iterations between two reads of the cancel flag

template <typename R>
struct AdvanceArgs {
  const CellRec<R> *recs;
  const int32_t *iboundts;
  const uint8_t *cellflags;  // CellBase::flags
  int32_t *cell;             // 0-based
  int32_t *status;
  R *x, *y, *z;
  double *t;
  uint64_t *ctr;
  const uint64_t *id;        // may be null: id = index
  const uint32_t *perm;      // processing order (cell-sorted) or null
  unsigned long long *queue; // work counter, zeroed before launch
  unsigned long long *steps; // particle-step counter
  const volatile int *abort; // host-mapped cancel flag (may be null): polled every kAbortPoll iterations
  int64_t n;
  double t_begin, t_end;
  int ndim, d1, d2;
  uint64_t seed;
  int exp_adv;  // EXPONENTIAL advection with the Newton exit time (else EULERIAN)
  int axi;      // linear axisymmetric dispersion (else linear isotropic)
};

template <typename R>
cudaError_t launch_advance(const AdvanceArgs<R> &a, int blocks, int threads, cudaStream_t s);
template <typename R>
size_t advance_smem_bytes(int threads);
// resident blocks per SM of the step kernel variant (cudaOccupancyMaxActiveBlocksPerMultiprocessor)
template <typename R>
cudaError_t advance_occupancy(int exp_adv, int axi, int threads, int *blocks_per_sm);

// ---- prep (prep.cu) -------------------------------------------------------
struct PrepInputs {
  GridDims g;
  const double *delr, *delc, *top, *botm;
  const int32_t *ia, *ja;
  const double *flowja, *bflow;
  const double *porosity, *retardation;
  const int32_t *iboundts, *icboundts;
  int32_t default_icbound;
  const double *heads;
  const int32_t *celltype;
  const double *source_flow, *sink_flow;
  const int32_t *zones;
  const double *alpha_l, *alpha_t, *dm_eff;
  const double *alpha_lv, *alpha_tv;  // axisymmetric model (null: = alpha_l, alpha_t)
  int32_t uniform_dispersion, steady_state;
  int32_t dispersion_model;           // 0 linear isotropic, 1 linear axisymmetric
  // options
  int32_t time_step_kind;
  double ts_param0, ts_param1;
  int32_t backward, stop_weak_sinks, stop_weak_sources, stop_zone, uniform_porosity;
};

cudaError_t launch_prep(const PrepInputs &in, CellBase base, uint8_t *massb, CellRec<double> *rec64,
                        CellRec<float> *rec32, cudaStream_t s);

// ---- geometry / histogram (hist.cu) --------------------------------------
struct Geometry {
  const double *col_left, *col_right;   // ncol  (GetLeft / GetRight)
  const double *row_front, *row_back;   // nrow  (GetFront / GetBack)
  const double *botm, *sattop;          // ncell
  GridDims g;
  int32_t cell0;                        // particle cells are numbered from cell0 (batch member)
};

template <typename R>
cudaError_t launch_global_xyz(const Geometry &geo, int64_t n, const int32_t *cell, const R *x, const R *y,
                              const R *z, double *gx, double *gy, double *gz, cudaStream_t s);

struct HistArgs {
  Geometry geo;
  int64_t n;
  const int32_t *cell, *status;
  const void *x, *y, *z;  // R per precision
  int mixed;
  double origin[3], bin[3], inv_bin[3];
  int32_t nb[3];
  int active_dim[3];
  unsigned int *counts32;  // unit-mass path (zeroed)
  int64_t *bin_of;         // ordered path: per particle bin (or -1), may be null
  unsigned long long *nbinned;
};

cudaError_t launch_hist_unit(const HistArgs &a, cudaStream_t s);
cudaError_t launch_hist_bins(const HistArgs &a, cudaStream_t s);
cudaError_t launch_u32_to_f64(const unsigned int *in, double *out, int64_t n, cudaStream_t s);
cudaError_t launch_coord_sums(const Geometry &geo, int64_t n, const int32_t *cell, const int32_t *status,
                              const void *x, const void *y, const void *z, int mixed, int pass, const double mean[3],
                              double *partial, int *nblocks, cudaStream_t s);

// ---- observation cells (obs.cu) -------------------------------------------
struct ObsArgs {
  int64_t n;
  const int32_t *cell, *status;  // cell 0-based
  const double *t, *mass;        // mass may be null (unit mass)
  const uint64_t *id;            // may be null: id = index
  const int32_t *obs_of_cell;    // per cell: observation index or -1
  const int32_t *obs_style;      // per observation: 1 resident, 2 sink
  double t_begin, t_end;         // interval of the last advance
  int32_t cell0;                 // particle cells are numbered from cell0 (batch member)
};

// Sink records of the last advance into the scratch buffer; *n_records = how many.
cudaError_t collect_sink_records(const ObsArgs &a, void **scratch, size_t *scratch_bytes, int64_t *n_records,
                                 cudaStream_t s);
// Device addresses of the record arrays collect_sink_records left in scratch (same n).
cudaError_t sink_record_arrays(void *scratch, int64_t n, int32_t **obs, uint64_t **id, double **time,
                               double **mass);
// count[k] += 1, msum[k] += mass for every ACTIVE particle in a style-1 observation cell.
cudaError_t launch_resident(const ObsArgs &a, unsigned long long *count, double *msum, cudaStream_t s);

// Ordered (order-preserving) weighted sums: sort.cu
cudaError_t ordered_bin_sums(const int64_t *bin_of, const double *mass, const int32_t *status, int64_t n,
                             int64_t nbins, double *counts, double *total_mass, double *sum_w2,
                             void **scratch, size_t *scratch_bytes, cudaStream_t s);
// processing order: by cell, or -- given the random counters at the start of
// the previous advance -- heaviest first in buckets of kPassBucket passes
// of that advance, by cell within a bucket
constexpr int kPassBucket = 8;
constexpr int kPassBucketBits = 4;
constexpr int kPassBuckets = 1 << kPassBucketBits;
cudaError_t sort_cells(const int32_t *cell, const uint64_t *ctr, const uint64_t *ctr_prev, uint64_t ctr_per_pass,
                       uint32_t *perm, int64_t n, int ncell_bits, void **scratch, size_t *scratch_bytes,
                       cudaStream_t s);

}  // namespace mprw
