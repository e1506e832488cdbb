/*
 * mprw_gpu.h -- C ABI of the GB300 random-walk particle tracking library.
 *
 * Drop-in replacement for the tracking part of MODPATH-RW's OpenMP particle
 * loop and for its GPKDE histogram.  Every entry point takes plain pointers
 * and sizes, is callable from Fortran through ISO_C_BINDING, and returns an
 * int status (0 = ok, < 0 = error; mprw_last_error() gives the message).
 *
 * Reference interfaces replaced (paths relative to the reference's src/):
 *   mprw_advance        <- the per-particle TrackPath call inside the
 *                          `!$omp parallel do` particle loop, MPathRW.F90:1207-1539
 *                          (trackingEngine%TrackPath at MPathRW.F90:1320-1322,
 *                          ParticleTrackingEngine.f90:1051-1254, release checks
 *                          MPathRW.F90:1256-1302, status map 1337-1403)
 *   mprw_load_flow      <- FillCellBuffer / FillNeighborCellData / corner
 *                          variables rebuilt on every cell entry
 *                          (ParticleTrackingEngine.f90:711-825, 2009-2126;
 *                          ModpathCellData.f90:674-1098, 2522-2684;
 *                          TrackSubCell.F90:3667-4363)
 *   mprw_get_particles  <- ConvertToModelXYZ of the last pathline point
 *                          (ParticleTrackingEngine.f90:1226-1251,
 *                          ModflowRectangularGrid.f90:524-548)
 *   mprw_histogram      <- Histogram%ComputeCountsWeighted / ComputeCounts
 *                          (lib/gpkde/Histogram.F90:213-350), called from
 *                          GridProjectedKDE.F90:3964-3987 on the active
 *                          particles gathered at MPathRW.F90:1568-1624
 *
 * Conventions (the reference's): cell numbers are 1-based MODFLOW 6 DIS
 * node numbers, node = (k-1)*nrow*ncol + (i-1)*ncol + j; IA/JA are the
 * 1-based CSR arrays of the MODFLOW 6 binary grid file; FLOW-JA-FACE is
 * positive into the cell; faces 1..6 are -x, +x, -y (front), +y (back),
 * bottom, top; particle statuses are the driver codes 0..9
 * (0 pending, 1 active, 2 boundary face, 3 weak sink, 4 weak source,
 * 5 no exit possible, 6 stop zone, 7 inactive cell, 8 unreleased,
 * 9 undefined).
 *
 * Threading: one handle per host thread.  Calls on one handle are
 * serialised; the handle owns its device memory and its CUDA stream.
 */
#ifndef MPRW_GPU_H
#define MPRW_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPRW_OK 0
#define MPRW_E_INVAL -1   /* invalid argument or unsupported option          */
#define MPRW_E_CUDA -2    /* CUDA runtime error                              */
#define MPRW_E_OOM -3     /* device allocation failed                        */
#define MPRW_E_STATE -4   /* call out of order (e.g. advance before flow)    */
#define MPRW_E_ABORTED -5 /* a kernel hit its iteration cap and set an error */
#define MPRW_E_SIZE -6    /* an output buffer is too small; the size needed is returned */

#define MPRW_FP64 0  /* positions, velocities, dispersion all in FP64        */
#define MPRW_MIXED 1 /* int32 cell + FP32 local coordinates and arithmetic,  */
                     /* FP64 tracking time                                   */

typedef struct mprw_handle mprw_handle;

/* Structured MODFLOW 6 DIS grid (RectangularGridDisMf6.f90:122-360). */
typedef struct {
  int32_t nlay, nrow, ncol;
  const double *delr; /* ncol                                               */
  const double *delc; /* nrow                                               */
  const double *top;  /* nrow*ncol, top of layer 1                          */
  const double *botm; /* nlay*nrow*ncol                                     */
} mprw_grid_desc;

/* Tracking options as the reference parses them (ParticleTrackingOptions.f90,
 * RWOPTS ModpathSimulationData.f90:1770-2021, DSP TransportModelData.f90). */
typedef struct {
  int32_t time_step_kind;     /* 1 ADV, 2 DISP, 3 MIN_ADV_DISP, 4 FIXED      */
  double ts_param[2];         /* timeStepParameters(1:2)                     */
  int32_t advection_kind;     /* 1 EXPONENTIAL (Newton exit time), 2 EULERIAN */
  int32_t dim_mask[3];        /* random-walk dimension mask                  */
  int32_t dispersion_model;   /* 0 linear isotropic, 1 linear axisymmetric   */
  int32_t stop_weak_sinks;
  int32_t stop_weak_sources;
  int32_t backward;
  int32_t stop_zone;          /* 0 = none                                    */
  int32_t uniform_porosity;   /* isUniformPorosity (ModpathBasicData.f90:208)*/
  uint64_t rng_seed;          /* Philox key                                  */
  int32_t precision;          /* MPRW_FP64 or MPRW_MIXED                     */
} mprw_options;

/* One flow time step (FlowModelData + TransportModelData arrays). */
typedef struct {
  const int32_t *ia;          /* ncell+1, 1-based                            */
  const int32_t *ja;          /* nja, 1-based, diagonal first in each row    */
  int64_t nja;
  const double *flowja;       /* nja FLOW-JA-FACE                            */
  const double *boundary_flows; /* 6*ncell face-assigned boundary flows, or NULL */
  const double *porosity;     /* ncell                                       */
  const double *retardation;  /* ncell                                       */
  const int32_t *iboundts;    /* ncell IBoundTS                              */
  const int32_t *icboundts;   /* ncell ICBoundTS, or NULL (all 0)            */
  int32_t default_icbound;    /* 1 when no IMP file (TransportModelData.f90:202) */
  const double *heads;        /* ncell, or NULL                              */
  const int32_t *celltype;    /* ncell ICELLTYPE, or NULL (all confined)     */
  const double *source_flow;  /* ncell, or NULL                              */
  const double *sink_flow;    /* ncell, or NULL                              */
  const int32_t *zones;       /* ncell, or NULL                              */
  const double *alpha_l;      /* ncell, or 1 value when uniform_dispersion   */
  const double *alpha_t;
  const double *dm_eff;
  int32_t uniform_dispersion;
  int32_t steady_state;
  const double *alpha_lv;     /* axisymmetric model: vertical longitudinal and */
  const double *alpha_tv;     /* transverse dispersivities (layout of alpha_l), */
                              /* or NULL: equal to alpha_l / alpha_t           */
} mprw_flow_desc;

/* Create a handle on the current CUDA device.
 * Replaces trackingEngine%Initialize (ParticleTrackingEngine.f90:393-532)
 * and InitializeRandomWalk (TrackSubCell.F90:542-631). */
int mprw_create(mprw_handle **h, const mprw_grid_desc *grid, const mprw_options *opt);

/* Upload one flow time step and build the per-cell records on the device.
 * Replaces the per-cell-entry buffer fills listed in the header comment. */
int mprw_load_flow(mprw_handle *h, const mprw_flow_desc *flow);

/* Copy n particles (host arrays) to the device.  cell is 1-based; t is the
 * TrackingTime (the release time for pending particles); mass may be NULL
 * (unit mass); id may be NULL (id = index); rng_ctr may be NULL (zeros).
 * Replaces the particle arrays of ParticleGroups (Particle.f90:7-17).
 * The next advance processes the particles heaviest first by the passes each
 * took in the previous advance (their rng_ctr increments) when n is
 * unchanged -- a host that hands back the particles mprw_get_particles gave
 * it keeps that order; results never depend on the order.  A cell outside
 * 1..ncell fails with MPRW_E_INVAL (checked on the device after the copy; the
 * handle then holds no particles until the next successful call). */
int mprw_set_particles(mprw_handle *h, int64_t n, const int32_t *cell, const double *lx,
                       const double *ly, const double *lz, const double *t,
                       const int32_t *status, const double *mass, const uint64_t *id,
                       const uint64_t *rng_ctr);

/* Advance every particle from tracking-interval start t_begin (the driver's
 * `time`) to t_end (the driver's `maxTime`), including the release checks.
 * steps_done (may be NULL) receives the particle-steps taken.
 * Replaces the tracking part of MPathRW.F90:1207-1539. */
int mprw_advance(mprw_handle *h, double t_begin, double t_end, int64_t *steps_done);

/* Copy particle state back (any pointer may be NULL).  gx/gy/gz are the
 * model coordinates of ConvertToModelXYZ. */
int mprw_get_particles(mprw_handle *h, int32_t *cell, double *lx, double *ly, double *lz,
                       double *t, int32_t *status, uint64_t *rng_ctr, double *gx,
                       double *gy, double *gz);

/* Weighted histogram of the ACTIVE particles' model coordinates on the grid
 * origin[3] + bin_size[3] * (n_bins[3]) (Histogram.F90:276-350), column-major
 * counts (x fastest).  counts (prod n_bins doubles) receives the sum of the
 * particle masses per bin, identical to the reference's sequential sum;
 * n_active and eff_mass (Kish effective count (sum w)^2 / sum w^2, computed
 * over the binned particles) may be NULL.  ordered != 0 forces the
 * order-preserving sum for arbitrary masses; with unit or equal
 * power-of-two masses the integer path is exact either way. */
int mprw_histogram(mprw_handle *h, const double origin[3], const double bin_size[3],
                   const int32_t n_bins[3], double *counts, int64_t *n_binned,
                   double *eff_mass);

/* GPKDE reconstruction options (the GPKDE input file, read at
 * ModpathSimulationData.f90:772-1289, passed to gpkde%Initialize at
 * MPathRW.F90:556-574 and to ComputeDensity at MPathRW.F90:1626-1642). */
typedef struct {
  double origin[3];            /* gpkdeDomainOrigin                            */
  double domain_size[3];       /* gpkdeDomainSize                              */
  double bin_size[3];          /* gpkdeBinSize                                 */
  int32_t n_opt_loops;         /* gpkdeNOptLoops (10)                          */
  double min_hover_delta;      /* kernel database: minHOverDelta (0.3)         */
  double delta_hover_delta;    /*                  deltaHOverDelta (0.3)       */
  double max_hover_delta;      /*                  maxHOverDelta (15)          */
  double rel_err_convergence;  /* gpkdeRelErrorConvergence (0.02)              */
  int32_t skip_error_convergence;
  int32_t unit_volume;         /* ComputeDensity(unitVolume=.true.)            */
  double scaling_factor;       /* gpkdeScalingFactor, e.g. 1/binVolume         */
  int32_t precision;           /* MPRW_FP64 (the reference's arithmetic) or    */
                               /* MPRW_MIXED (FP32 smoothing passes and        */
                               /* per-bin updates, FP64 convergence sums)      */
  int32_t isotropic;           /* gpkdeIsotropicKernels (0 = anisotropic, the  */
                               /* default; ModpathSimulationData.f90:1065-1075)*/
} mprw_gpkde_options;

/* GPKDE reconstruction of the ACTIVE particles (weights = particle masses).
 * Replaces gpkde%ComputeDensity (GridProjectedKDE.F90:3598-4392) with the
 * kernel database on, bounded kernel sizes, Kish effective weights and
 * anisotropic (or, with isotropic != 0, isotropic) kernels, for 1-D, 2-D
 * and 3-D grids (the dimensions with more than one bin are active).
 * density: nx*ny*nz doubles, x fastest (nx = int(domain/bin + 0.5)),
 * scaled as the reference exports it (x binVolume if unit_volume, x
 * scaling_factor); histogram (may be NULL): mass per bin; n_bins_out (may be
 * NULL): the grid; loops_done (may be NULL): optimisation loops run. */
int mprw_gpkde(mprw_handle *h, const mprw_gpkde_options *opt, double *density, double *histogram,
               int32_t n_bins_out[3], int32_t *loops_done);

/* Reconstruction from histograms summed over several trackers: the
 * collective of a multi-GPU run.  The reference reconstructs from all
 * particles at once (ComputeDensity on the active particles gathered at
 * MPathRW.F90:1568-1624); when the particles are split over trackers (one per
 * GPU), each bins its own particles and the reconstruction needs only
 * summable quantities: the mass per bin and the sums below.  Summed over the
 * trackers (an all-reduce) they give exactly the histogram, effective mass
 * (Histogram.F90:276-350) and coordinate statistics (GridProjectedKDE.F90:
 * 4023-4030) that mprw_gpkde computes from all particles, up to the rounding
 * of the sums.
 *   mprw_gpkde_partial      this tracker's part on the options' grid:
 *                           mass_per_bin (prod n_bins doubles, host, x
 *                           fastest: the summed masses of its ACTIVE
 *                           particles per bin) and sums
 *   mprw_gpkde_from_counts  the reconstruction of mprw_gpkde from summed
 *                           parts (host arrays): the same outputs; it uses
 *                           the handle's device memory and stream, not its
 *                           particles (any handle of the run may do it)
 * The coordinate sums are taken about the domain centre origin +
 * domain_size/2 of the options, so every tracker must use the same options. */
typedef struct {
  double n_active;   /* ACTIVE particles                                   */
  double sum_w;      /* sum of their masses                                */
  double sum_w2;     /* sum of their squared masses                        */
  double sum_dx[3];  /* sum of (model coordinate - domain centre)          */
  double sum_dx2[3]; /* sum of (model coordinate - domain centre)^2        */
} mprw_gpkde_sums;

int mprw_gpkde_partial(mprw_handle *h, const mprw_gpkde_options *opt, double *mass_per_bin, mprw_gpkde_sums *sums);
int mprw_gpkde_from_counts(mprw_handle *h, const mprw_gpkde_options *opt, const double *mass_per_bin,
                           const mprw_gpkde_sums *sums, double *density, double *histogram, int32_t n_bins_out[3],
                           int32_t *loops_done);

/* Observation cells (TrackingOptions%isObservation / idObservation;
 * Observation.f90:7-60).  cells[i] (1-based) belongs to observation obs[i]
 * (0-based, < nobs); style[k] of observation k is 1 (resident) or 2 (sink).
 * A cell belongs to at most one observation.  Replaces the observation
 * bookkeeping of the particle loop, MPathRW.F90:1337-1392 and 1460-1535. */
int mprw_set_observations(mprw_handle *h, int32_t ncells, const int32_t *cells, const int32_t *obs,
                          int32_t nobs, const int32_t *style);

/* Resident observations at the current time (MPathRW.F90:1460-1535): for
 * every style-1 observation k, count[k] ACTIVE particles lie in its cells
 * with total mass mass[k] (nobs entries each). */
int mprw_observe_resident(mprw_handle *h, int64_t *count, double *mass);

/* Sink observations of the last mprw_advance (MPathRW.F90:1337-1392): the
 * particles that stopped at a weak sink or weak source (status 3 or 4)
 * during that interval in a cell of a style-2 observation, as records
 * (observation, particle id, stop time, mass) in particle order.  At most
 * capacity records are copied; n_records receives how many there are. */
int mprw_observe_sinks(mprw_handle *h, int64_t capacity, int32_t *obs, uint64_t *id, double *time,
                       double *mass, int64_t *n_records);

/* 1-D GPKDE of an observation time series (breakthrough curve): the
 * reconstruction the observation post-process runs on the record times of
 * one solute (MPathRW.F90:1773-2000 resident, 2000-2840 sink observations),
 * i.e. GridProjectedKDE%Initialize with a 1-D domain and
 * databaseOptimization = .false. followed by ComputeDensity with weights
 * (GridProjectedKDE.F90:354-998, 3598-4392; Histogram.F90:276-720).  Every
 * kernel is set up from its bin's exact smoothing.
 *
 * times[n], weights[n] are HOST arrays (the record times and the weights the
 * driver gives them: mass / retardation for resident records, mass / |Q| for
 * sink records).  counts[capacity] receives the histogram the driver reads
 * (Histogram%counts), wcounts[capacity] (may be NULL) the weighted counts of
 * effective-weight formats 2 and 3 (zeros otherwise), density[capacity] (may
 * be NULL) the reconstruction (densityEstimateGrid; zeros for a histogram
 * only), all after the reference's closing scalings.  res receives the grid
 * actually used: n_bins, the first bin's offset in the domain grid
 * (deltaBinsOrigin; bin m's centre is (m + delta_bins_origin - 1/2) *
 * bin_size + origin), the bin size (estimated for bin formats 0 and 1), the
 * histogram origin, the optimisation loops run and the active bins.  When
 * n_bins > capacity nothing is reconstructed and MPRW_E_SIZE is returned
 * with res filled: call again with a larger buffer.
 *
 * Inputs the reference stops on return MPRW_E_INVAL: no points, non-finite
 * times or weights, a bin size that is not positive (a Scott or
 * Freedman-Diaconis estimate of identical times), a grid of fewer than two
 * bins, a sub-grid larger than the domain grid, a net roughness that is zero
 * everywhere.  Freedman-Diaconis needs two points (the reference reads
 * element 0 of the sorted array for one).  Grids of more than 2^20 bins and
 * an initial smoothing whose support spans more than 2^20 bins are refused.
 * The work runs on `stream` (a cudaStream_t, NULL = the default stream); the
 * call returns when the results are on the host. */
typedef struct {
  double origin;               /* domainOrigin(1), 0 for times                  */
  double domain_size;          /* domainSize(1); 0 with adapt_grid: from data  */
  double bin_size;             /* binSize(1) for bin_format 2 and 3            */
  int32_t bin_format;          /* histogramBinFormat: 0 Scott, 1 Freedman-     */
                               /* Diaconis, 2/3 the given bin_size             */
  double bin_size_fraction;    /* binSizeFraction (formats 0, 1), in (0, 2]    */
  int32_t adapt_grid;          /* adaptGridToCoords                            */
  int32_t exact_point;         /* exactPoint (resident records: a time on a    */
                               /* bin boundary opens that bin)                 */
  int32_t effective_weight_format; /* 0 Kish, 1 mean weight, 2 counts and     */
                               /* weights, 3 effective counts and weights      */
  int32_t initial_smoothing_selection; /* 0 Silverman, 1 factor * bin size, */
                               /* 2 twice the bin size                         */
  double initial_smoothing_factor; /* initialSmoothingFactor                   */
  int32_t apply_initial_factor; /* selection 0: the factor scales Silverman's  */
                               /* estimate (applyInitialSmoothingFactor)       */
  int32_t n_opt_loops;         /* nOptimizationLoops                           */
  double rel_err_convergence;  /* relativeErrorConvergence                     */
  int32_t skip_error_convergence;
  int32_t only_histogram;      /* onlyHistogram                                */
  int32_t compute_raw_density; /* computeRawDensity: histogram / bin size      */
  int32_t unit_volume;         /* unitVolume: density * bin size               */
} mprw_series_options;

typedef struct {
  int32_t n_bins;
  int32_t delta_bins_origin;
  double bin_size;
  double grid_origin;
  int32_t loops_done;
  int32_t active_bins;
} mprw_series_result;

int mprw_gpkde_series(const double *times, const double *weights, int64_t n, const mprw_series_options *opt,
                      int32_t capacity, double *counts, double *wcounts, double *density,
                      mprw_series_result *res, void *stream);

/* Allocation-free unit-mass histogram.  No counterpart in the reference: it
 * exists for callers that cannot allocate device memory when they bin -- a
 * host code that owns a fixed device-memory budget and hands the library only
 * pre-sized buffers, or one running where cudaMalloc would synchronise the
 * device or is forbidden.  It needs no handle and calls no cudaMalloc,
 * cudaFree or allocating library routine.
 *
 * gx, gy, gz, status, counts and n_binned are DEVICE pointers: gx/gy/gz are
 * model coordinates (as mprw_get_particles returns them), status the particle
 * statuses; only ACTIVE (1) particles are counted.  counts (prod n_bins
 * doubles, x fastest) receives the particle count per bin, identical to
 * mprw_histogram's with unit masses; n_binned (one int64, may be NULL) the
 * particles binned.  origin, bin_size and n_bins are HOST arrays of 3, read
 * during the call.  The work is queued on `stream` (a cudaStream_t, NULL =
 * the default stream) and the call returns without waiting for it.
 *
 * Limits: prod(n_bins) <= MPRW_NOALLOC_MAX_BINS and n < 2^32 (the bin
 * counters are 32-bit), else MPRW_E_INVAL.  The scratch
 * (MPRW_NOALLOC_MAX_BINS 32-bit bin counters plus a 64-bit binned-particle
 * counter, about 4 MiB) is a fixed array in the library's device image that
 * every GPU loading the library holds until the process exits.  The first
 * call on each device (and the first after a device reset) looks up the
 * array's device address in the current context, so make that first call
 * before any stream capture.  All calls share the array and each clears it
 * before counting; calls that overlap on the GPU race on it. */
#define MPRW_NOALLOC_MAX_BINS (1 << 20)
int mprw_histogram_noalloc(const double *gx, const double *gy, const double *gz, const int32_t *status,
                           int64_t n, const double origin[3], const double bin_size[3],
                           const int32_t n_bins[3], double *counts, int64_t *n_binned, void *stream);

/* Batched realizations.  No counterpart in the reference, which tracks one
 * realization per run (one mpathrw process per flow model): a batch holds
 * nmembers grids of any sizes that share the tracking options, one flow time
 * step and one particle set per member, and mprw_advance on the batch tracks
 * every member's particles in ONE persistent launch over the concatenated
 * cell records and particle arrays (each member's cells link only to its own
 * cells).
 *   mprw_create_batch      grids[nmembers]; the batch is destroyed with
 *                          mprw_destroy, which also ends its member views
 *   mprw_batch_member      a view handle of member k: mprw_load_flow,
 *                          mprw_get_particles (its particles, its cell
 *                          numbers), mprw_histogram, mprw_gpkde and the
 *                          observation calls work on it as on a single
 *                          handle; mprw_set_particles on it overwrites its
 *                          particles but cannot change their count;
 *                          mprw_advance, mprw_set_stream and mprw_destroy on
 *                          it return MPRW_E_STATE
 *   mprw_set_particles_batch  counts[nmembers] particles per member, the
 *                          arrays concatenated in member order, cell numbers
 *                          1-based within each member's grid
 * On the batch handle itself, mprw_advance advances every member (all member
 * flows loaded first); mprw_get_particles returns every member's particles
 * in batch order with member cell numbers; mprw_load_flow, mprw_histogram,
 * mprw_gpkde and the observation calls return MPRW_E_STATE.  Particle ids
 * select the random streams: without ids the id is the particle's index in
 * the batch, so members draw independent streams; a member reproduces a
 * separate single-handle run when both use the same ids. */
int mprw_create_batch(mprw_handle **batch, int32_t nmembers, const mprw_grid_desc *grids,
                      const mprw_options *opt);
int mprw_batch_member(mprw_handle *batch, int32_t member, mprw_handle **view);
int mprw_set_particles_batch(mprw_handle *batch, const int64_t *counts, const int32_t *cell,
                             const double *lx, const double *ly, const double *lz, const double *t,
                             const int32_t *status, const double *mass, const uint64_t *id,
                             const uint64_t *rng_ctr);

/* GPKDE of every member of a batch (as mprw_gpkde on each member view), up to
 * `concurrency` members at a time (<= 0: 4; at most 16), each on its own
 * non-blocking stream driven by its own host thread, so that one member's
 * host round trips and small launches overlap another's kernels.  opts,
 * density and loops_done (may be NULL) have one entry per member; histogram
 * may be NULL or hold one pointer (NULL allowed) per member.  The
 * reconstructions see the particles after the batch's last advance.  Each
 * concurrency slot keeps its own reconstruction state (pass buffers sized
 * for the largest grid it has reconstructed). */
int mprw_gpkde_batch(mprw_handle *batch, const mprw_gpkde_options *opts, double *const *density,
                     double *const *histogram, int32_t *loops_done, int32_t concurrency);

/* Launch tuning of mprw_advance.  No counterpart in the reference (its loop
 * is `!$omp parallel do schedule(dynamic,1)`).  blocks_per_sm: resident
 * blocks per SM of the persistent step kernel (0 = the variant's default: 3
 * for EULERIAN MIXED, else 1; at most what its registers allow, which
 * mprw_get_tuning reports as max_blocks; blocks of 384 threads for the FP64
 * EULERIAN kernel, 256 otherwise); sort_interval: the particles are sorted
 * -- by the passes each took in the previous advance, heaviest first in
 * buckets of 8, then by cell -- before every k-th advance and processed in
 * that order until the next sort (1 = every advance, the default; 0 =
 * never).  Results do not depend on the tuning: each particle's steps use
 * only its own state and its own counter-based random numbers.
 *
 * mprw_autotune picks both on the handle's real work: from the current
 * particle state it runs one advance over [t_begin, t_end] per candidate
 * (sorted first, with 1 .. min(max_blocks, 4) blocks per SM, then the best
 * block count unsorted), restoring the state before each trial and at the
 * end, so the particles are unchanged on return.  The fastest block count
 * (particle-steps per ms, sort included) is kept; sorting is kept every
 * advance if it pays, every 4th if unsorted is within 3 %, never if unsorted
 * is more than 5 % faster.  rates (may be NULL; room for 5 doubles) receives
 * the particle-steps per ms of each trial in that order.  Costs one extra
 * copy of the particle state on the device. */
int mprw_set_tuning(mprw_handle *h, int32_t blocks_per_sm, int32_t sort_interval);
int mprw_get_tuning(mprw_handle *h, int32_t *blocks_per_sm, int32_t *sort_interval, int32_t *max_blocks);
int mprw_autotune(mprw_handle *h, double t_begin, double t_end, int32_t *blocks_per_sm, int32_t *sort_interval,
                  double *rates);

/* Differentiable random walk and its adjoint.  No counterpart in the
 * reference: its step is not differentiable in the parameters (a step cut at
 * a cell face shifts every later normal to another step, TrackSubCell.F90:
 * 956-1368, and the histogram deposit, Histogram.F90:276-350, is piecewise
 * constant), so a gradient of a concentration misfit needs a walk whose path
 * is continuous in the parameters.  This variant sits beside the tracking
 * path and leaves it unchanged:
 *   - fields on the lattice of cell corners, interpolated trilinearly: pore
 *     velocity u = s q / (phi R) from the Darcy flux of the loaded flow
 *     (averaged over the faces that meet at a corner), the drift correction
 *     div(phi D) / phi by central differences of the corner values of phi D
 *     (the reference's div D term, TrackSubCell.F90:2695-2818), alphaL,
 *     alphaT and Dm of each corner's share of the zones;
 *   - D = (alphaT r + Dm/R) I + (alphaL - alphaT) u u^T / r with r =
 *     sqrt(|u|^2 + velocity_floor^2): the reference's tensor where the
 *     velocity is well above the floor, smooth where it vanishes;
 *   - a fixed time step dt: x' = x + (u + div term) dt + B xi sqrt(dt), with
 *     B B^T = 2 D (TrackSubCell.F90:2821-2928) and B smooth in u;
 *     reflection at every domain wall;
 *   - xi: normals keyed by (seed, particle id, step): a perturbed run draws
 *     the same numbers (common random numbers);
 *   - the density on a grid: a deposit of a product biweight kernel of
 *     half-width bandwidth[d] per dimension (dimensions with one bin are
 *     integrated over), per unit length / area / volume.
 * Parameters theta (3 nzones + 1 doubles): alphaL of each zone, alphaT of
 * each zone, porosity of each zone, then a velocity scale s (1 = the loaded
 * flow).  The grid must be uniform (equal cell sizes) with one retardation.
 * The pathwise gradient is exact for this discrete model; it is a useful
 * estimate of the gradient of the expected misfit while the particles travel
 * a few correlation lengths of the velocity field at most -- over longer
 * runs in a heterogeneous field the paths' sensitivities grow fast.
 *   mprw_adj_setup     zones (one 0-based zone per cell, < nzones), the walk
 *                      and density grid; the walkers are the handle's
 *                      particles that are ACTIVE or PENDING (pending ones
 *                      start at the first step), from their positions now
 *   mprw_adj_forward   runs nsteps steps for theta, storing the positions
 *                      every `checkpoint` steps, and returns the density
 *                      (prod n_bins doubles, x fastest); repeatable to the
 *                      last bit
 *   mprw_adj_backward  given dL/d density of the last forward run, the
 *                      gradient dL/d theta (3 nzones + 1 doubles): the
 *                      hand-written reverse sweep of every step, each
 *                      segment recomputed from its checkpoint */
typedef struct {
  int32_t nzones;        /* 1..64                                          */
  int32_t nsteps;        /* steps of a run                                 */
  int32_t checkpoint;    /* steps between stored positions (1..nsteps)     */
  double dt;             /* time step                                      */
  double velocity_floor; /* > 0, in the velocity's units                   */
  uint64_t seed;         /* Philox key of the normals                      */
  double origin[3];      /* density grid                                   */
  double bin_size[3];
  int32_t n_bins[3];
  double bandwidth[3];   /* biweight half-width per dimension              */
} mprw_adj_options;

int mprw_adj_setup(mprw_handle *h, const int32_t *zones, const mprw_adj_options *opt);
int mprw_adj_forward(mprw_handle *h, const double *theta, double *density);
int mprw_adj_backward(mprw_handle *h, const double *grad_density, double *grad_theta);

/* Cancellation of mprw_advance (the reference has none: its loops end by
 * their own caps).  The step kernel reads a cancel flag in mapped host memory
 * every few hundred iterations of each warp.  mprw_set_timeout: an advance
 * that is still running after timeout_ms (0 = no limit, the default) raises
 * the flag.  mprw_cancel raises it from any host thread and stops the advance
 * that is running, or else the next one.  A cancelled advance returns
 * MPRW_E_ABORTED after the kernel has returned (the context stays usable):
 * every particle then holds a valid location -- its last completed step, or
 * the start of the cell it was entering -- with status ACTIVE and its random
 * counter; particles not reached keep their previous state.  The next
 * mprw_advance continues from there (it starts new cell visits, so the
 * result is a valid trajectory but not bit-identical to an uninterrupted
 * one).  On a batch member both apply to the batch. */
int mprw_set_timeout(mprw_handle *h, double timeout_ms);
int mprw_cancel(mprw_handle *h);

/* Optional: launch on a caller-provided cudaStream_t (NULL = the handle's). */
int mprw_set_stream(mprw_handle *h, void *stream);

/* Device time (ms) of the last launch of each kernel family, of the last
 * whole mprw_gpkde call (stream time from its first to its last operation,
 * host-side waits included), and the number of kernel launches issued by the
 * last mprw_advance / mprw_histogram / mprw_gpkde call.  Any pointer may be
 * NULL. */
int mprw_last_timings(mprw_handle *h, double *step_ms, double *prep_ms, double *hist_ms,
                      double *gpkde_ms, int64_t *launches);

/* Work model of the last mprw_gpkde (0 when it had no active bins): the
 * multiply-adds of the reference's direct 3-D kernels, summed over its
 * optimisation loops -- per loop and active bin |K_W| + 8 |K_sigma| + 3 |K_SD|
 * with |K| = prod_d (2 ceil(r hOverDelta_d) + 1) at the bin's database levels
 * (r = 3 for W and the smoothing kernel, 4 for the second derivatives).
 * Divided by the reconstruction's time it is the rate a direct evaluation
 * would need; the library's separable passes do a fraction of it. */
int mprw_last_gpkde_work(mprw_handle *h, double *madds);

int mprw_destroy(mprw_handle *h);

const char *mprw_last_error(const mprw_handle *h);

#ifdef __cplusplus
}
#endif
#endif
