// gpkde.cuh -- types of the device GPKDE reconstruction (gpkde.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace mprw {

constexpr int KDE_MAXDB = 64;    // h/delta database entries (16 at the defaults)
constexpr int KDE_MAXLEN = 256;  // longest 1-D factor, 2*ceil(4*maxHOverDelta)+1
constexpr double PI_D = 3.14159265358979323846;
constexpr double SQRT8PI_D = 5.01325654926724104;  // sqrt(8*pi)

// Constants of one reconstruction grid (GridProjectedKDE.F90 prInitialize,
// prInitializeModuleConstants 1582-1611).
struct KdeParams {
  int ndim, mask[3], nb[3];
  double bin[3], binvol, bin_distance;
  int ndelta;
  double hod[KDE_MAXDB];
  double min_hod, dlog;  // log database: index = floor(log(h/bin/min)/dlog)+1
  double max_k[3], min_k[3], max_sd[3], min_sd[3];
  int max_dim, min_dim;
  double support_c, alpha_c, beta_c, one_over_nd4, minus_one_over_nd6, one_plus_nd_q;
  double four_pi_half_nd;  // (4 pi)**(0.5 nDim)
  double max_sigma_growth, iso_threshold;
};

// 1-D factor table: for dimension d and database index n (0-based),
// m[d*KDE_MAXDB+n] is the half width and val[ofs[...] + k], k = 0..2m, the
// full symmetric factor.
struct KdeTable {
  const double *val;
  const int *m, *ofs;
};

// Separable passes.  The smoothing (sigma) and second-derivative kernels of
// a bin are chosen from the database by one scalar, so the bins fall into at
// most KDE_KMAX groups ("keys") that share one kernel; a gather or scatter
// over all bins is then, per key, three one-dimensional passes over the key's
// bounding box.
constexpr int KDE_KMAX = 3 * KDE_MAXDB;

// Bounding box (1-based, inclusive: x0,x1,y0,y1,z0,z1), database levels and
// bin count of every key, accumulated with atomics.
struct KeyAcc {
  int box[KDE_KMAX][6];
  int lev[KDE_KMAX][3];
  int cnt[KDE_KMAX];
};

// The keys present, compacted: per key its half widths and factors per
// dimension, the regions of the two intermediate passes and their offsets
// (in elements) into the pass buffers.
struct SepPlan {
  int np;
  int slot_of[KDE_KMAX];
  int key[KDE_KMAX];
  int m[KDE_KMAX][3];
  const double *f[KDE_KMAX][3];
  int box[KDE_KMAX][6], r1[KDE_KMAX][6], r2[KDE_KMAX][6];
  long long o1[KDE_KMAX], o2[KDE_KMAX];
  int ur[3][6];  // scatter: union of the output regions of each axis's keys
};

// Per active bin state (SoA).  3-vectors are stored dimension-major: v[d*n + b].
struct KdeBins {
  int n;
  int *gx, *gy, *gz;  // 1-based bin indexes
  double *count;
  double *ks, *scale, *shape, *support, *nest, *dens, *cb, *rxx, *ryy, *rzz, *net, *dens_old, *scale_old;
};

struct KdeState {
  KdeBins bins{};
  int cap = 0;
  double *dens_grid = nullptr, *dens_raw = nullptr, *cx = nullptr, *cy = nullptr, *cz = nullptr;
  double *cxy = nullptr, *cxz = nullptr, *cyz = nullptr;  // products of the squared curvatures
  int64_t grid_cap = 0;
  double *tmp = nullptr, *partial = nullptr, *d_scalars = nullptr, *h_scalars = nullptr;
  int *d_flag = nullptr, *h_flag = nullptr, *d_blockcnt = nullptr;
  int *cell_bin = nullptr;          // per grid cell: active bin index or -1
  int *bin_key = nullptr;           // per bin: smoothing key (n) and SD keys per axis (3n)
  int *wlev = nullptr;              // per bin: W kernel database level per dimension (3n)
  KeyAcc *d_keys = nullptr;
  SepPlan *d_plan = nullptr;
  double *t1 = nullptr, *t2 = nullptr;
  int64_t t1_cap = 0, t2_cap = 0;
  long long *d_need = nullptr, *h_need = nullptr;  // pass-buffer sizes a plan needed, overflow flag
  KdeTable wtab{}, sdtab[3]{};
  double *d_val = nullptr;
  int *d_meta = nullptr;  // wm, wofs, sm[3], sofs[3]
  int64_t launches = 0;

  cudaError_t ensure_bins(int n);
  cudaError_t ensure_pass(int64_t n1, int64_t n2);
  cudaError_t ensure_grid(int64_t ngrid);
  void release();
};

void kde_build_tables(const KdeParams &P, std::vector<double> &val, std::vector<int> &wm, std::vector<int> &wofs,
                      std::vector<int> (&sm)[3], std::vector<int> (&sofs)[3]);
cudaError_t kde_collect_active(KdeState &st, const KdeParams &P, const double *counts, cudaStream_t s,
                               int *nactive);
cudaError_t kde_run(KdeState &st, const KdeParams &P, double hs, double npts, int n_opt_loops, double rel_err,
                    bool skip_error, cudaStream_t s, int *loops_done);

}  // namespace mprw
