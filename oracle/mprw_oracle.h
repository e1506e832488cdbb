/*
 * mprw_oracle.h -- CPU restatement of MODPATH-RW's random-walk particle
 * tracking path (TEST INFRASTRUCTURE ONLY).
 *
 * This is the oracle: a serial (optionally OpenMP) C restatement of the
 * Fortran reference, used by the tests to check the CUDA library and by the
 * benchmark as the timed CPU baseline.  Nothing in the shipped library links
 * or calls it.  Parity of this restatement with the Fortran reference is
 * UNPINNED by any reference golden vector (the reference ships no tests or
 * expected outputs); it is pinned by the analytic Gaussian ADE solution and by
 * an independent Python restatement of the RNG.
 *
 * Conventions follow the reference: 1-based cell numbers, MODFLOW 6 DIS
 * node numbering node = (k-1)*nrow*ncol + (i-1)*ncol + j, CSR IA/JA 1-based
 * (binary grid file convention), faces 1..6 = -x,+x,-y(front),+y(back),
 * bottom,top.
 */
#ifndef MPRW_ORACLE_H
#define MPRW_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int nlay, nrow, ncol;
  const double *delr;        /* ncol */
  const double *delc;        /* nrow */
  const double *top;         /* nrow*ncol  (top of layer 1)            */
  const double *botm;        /* ncell                                   */
  const int    *ia;          /* ncell+1, 1-based                        */
  const int    *ja;          /* nja, 1-based, diagonal first per row    */
  int           nja;
  const double *flowja;      /* nja  (MF6 FLOW-JA-FACE, + into cell)    */
  const double *bflow;       /* 6*ncell face-assigned boundary flows or NULL */
  const double *porosity;    /* ncell */
  const double *retardation; /* ncell */
  const int    *ibound;      /* ncell (IBound)                          */
  const int    *iboundts;    /* ncell (IBoundTS)                        */
  const int    *icboundts;   /* ncell (ICBoundTS) or NULL => all 0      */
  int           default_icbound;
  const double *heads;       /* ncell or NULL */
  const int    *celltype;    /* ncell or NULL => all confined */
  const double *source_flow; /* ncell or NULL */
  const double *sink_flow;   /* ncell or NULL */
  const int    *zones;       /* ncell or NULL */
  const double *alpha_l;     /* ncell, or 1 value if uniform_dispersion */
  const double *alpha_t;
  const double *dm_eff;
  int           uniform_dispersion;
  int           steady_state;
  const double *alpha_lv;    /* vertical dispersivities of the axisymmetric  */
  const double *alpha_tv;    /* model (layout of alpha_l), or NULL: = alpha_l / alpha_t */
} orc_flow;

typedef struct {
  int    time_step_kind;     /* 1 ADV, 2 DISP, 3 MIN_ADV_DISP, 4 FIXED   */
  double ts_param[2];        /* timeStepParameters(1:2)                 */
  int    advection_kind;     /* 1 EXPONENTIAL, 2 EULERIAN               */
  int    dim_mask[3];
  int    stop_weak_sinks, stop_weak_sources, backward, stop_zone;
  int    uniform_porosity;   /* isUniformPorosity                       */
  int    rng_kind;           /* 0 = xoroshiro128+ thread streams + Irwin-Hall(12)
                                1 = Philox4x32-10 per-particle counters + Irwin-Hall(12) */
  uint64_t seed;             /* Philox key (rng_kind 1)                 */
  int    nthreads;           /* >1: OpenMP particle loop (rng_kind 0 uses one stream per thread) */
  int    dispersion_model;   /* 0 linear isotropic, 1 linear axisymmetric  */
} orc_options;

/* Particle status codes of the driver (MPathRW.F90:1337-1403). */
enum { ORC_PENDING = 0, ORC_ACTIVE = 1, ORC_BOUNDARY = 2, ORC_WEAK_SINK = 3,
       ORC_WEAK_SOURCE = 4, ORC_NO_EXIT = 5, ORC_STOP_ZONE = 6, ORC_INACTIVE = 7,
       ORC_UNRELEASED = 8, ORC_UNDEFINED = 9 };

/* Advance every particle from tracking interval start t_begin to t_end.
 * cell[] is 1-based.  t[] holds TrackingTime (for pending particles: the
 * release time).  rng_ctr[] (rng_kind 1) is the per-particle Philox block
 * counter.  id[] is the particle key.  Returns 0 on success. */
int orc_advance(const orc_flow *f, const orc_options *o, int64_t n,
                int *cell, double *lx, double *ly, double *lz, double *t,
                int *status, const uint64_t *id, uint64_t *rng_ctr,
                double t_begin, double t_end, int64_t *steps_out);

/* ConvertToModelXYZ (ModflowRectangularGrid.f90:524-548) for n particles. */
void orc_global_xyz(const orc_flow *f, int64_t n, const int *cell,
                    const double *lx, const double *ly, const double *lz,
                    double *gx, double *gy, double *gz);

/* Per-cell quantities the tracking engine builds on cell entry, exported for
 * the tests: face velocities (6), dtcell, corner discharge (8x4), corner
 * porosity (8), corner dispersion (9x8), mass boundary (6), connection (6). */
int orc_cell_record(const orc_flow *f, const orc_options *o, int cell,
                    double *vface6, double *dtcell, double *qcorner32,
                    double *phicorner8, double *d72, int *massb6, int *conn6);

/* RNG restatements (rng_par_zig.f90, TrackSubCell.F90:3631-3663). */
void     orc_xoro_seed_stream(int k, uint64_t s[2]);      /* base seed jumped k times */
void     orc_xoro_reset(void);  /* rng_kind 0: start a new run; the thread streams otherwise
                                   continue across orc_advance calls, as rng_init seeds them
                                   once per run in the reference (TrackSubCell.F90:613-620) */
uint64_t orc_xoro_next(uint64_t s[2]);
double   orc_xoro_uniform(uint64_t s[2]);
double   orc_xoro_normal_ih12(uint64_t s[2]);
void     orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double   orc_philox_normal_ih12(uint64_t seed, uint64_t id, uint64_t *ctr);

#ifdef __cplusplus
}
#endif
#endif
