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
  double inv_binvol;  // 1 / binvol when binvol is a power of two (exact), else 0
  int ndelta;
  double hod[KDE_MAXDB];
  double min_hod, dlog;  // log database: index = floor(log(h/bin/min)/dlog)+1
  float lscale[3], linv;  // FP32 estimate of the index: 1/(bin*min_hod), 1/dlog
  double max_k[3], min_k[3], max_sd[3], min_sd[3];
  int max_dim, min_dim;
  double support_c, alpha_c, beta_c, one_over_nd4, minus_one_over_nd6, one_plus_nd_q;
  double four_pi_half_nd;  // (4 pi)**(0.5 nDim)
  double max_sigma_growth, iso_threshold;
  int isotropic;  // isotropic kernels (gpkdeIsotropicKernels): no shapes, isotropic net roughness
  int d1, d2;     // 2-D grids: the two active dimensions (idDim1 < idDim2)
};

// 1-D factor table: for dimension d and database index n (0-based),
// m[d*KDE_MAXDB+n] is the half width and val[ofs[...] + k], k = 0..2m, the
// full symmetric factor.  Every table of a reconstruction indexes the same
// value array (one copy per arithmetic type).
template <typename T>
struct KdeTableT {
  const T *val;
  const int *m, *ofs;
};
using KdeTable = KdeTableT<double>;

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
  unsigned int done;  // blocks of the key assignment that have merged (the last one plans)
};

// The keys present, compacted: per key its half widths and the offsets of its
// factors in the value array per dimension, the regions of the two
// intermediate passes and their offsets (in elements) into the pass buffers.
struct SepPlan {
  int np;
  long long tot1, tot2;  // elements (region cells) of the two pass buffers, all keys
  int slot_of[KDE_KMAX];
  int key[KDE_KMAX];
  int m[KDE_KMAX][3];
  int fofs[KDE_KMAX][3];
  int box[KDE_KMAX][6], r1[KDE_KMAX][6], r2[KDE_KMAX][6];
  long long o1[KDE_KMAX], o2[KDE_KMAX];
  int ur[3][6];  // scatter: union of the output regions of each axis's keys
};

// Per active bin state (SoA) in the reconstruction's arithmetic type T; the
// histogram count stays FP64.  3-vectors are stored dimension-major: v[d*n + b].
template <typename T>
struct KdeBinsT {
  int n;
  int *gx, *gy, *gz;  // 1-based bin indexes
  double *count;
  T *ks, *scale, *shape, *support, *nest, *dens, *cb, *rxx, *ryy, *rzz, *net, *dens_old, *scale_old;
};
using KdeBins = KdeBinsT<double>;

// Device state of the reconstructions of one handle.  Every array is
// allocated with FP64 elements; an FP32 reconstruction uses the same memory
// through float views (view<float>()).
struct KdeState {
  KdeBins bins{};
  int cap = 0;
  double *dens_grid = nullptr, *dens_raw = nullptr, *cx = nullptr, *cy = nullptr, *cz = nullptr;
  double *cxy = nullptr, *cxz = nullptr, *cyz = nullptr;  // products of the squared curvatures
  double *dens_out = nullptr;                             // FP64 output grid
  int64_t grid_cap = 0;
  double *partial = nullptr, *d_scalars = nullptr, *h_scalars = nullptr;
  int *d_flag = nullptr, *d_blockcnt = nullptr;
  int *cell_bin = nullptr;          // per grid cell: active bin index or -1
  int *bin_key = nullptr;           // per bin: smoothing key (n) and SD keys per axis (3n)
  KeyAcc *d_keys = nullptr;
  SepPlan *d_plan = nullptr;
  double *t1 = nullptr, *t2 = nullptr;
  int64_t t1_cap = 0, t2_cap = 0;
  unsigned char *need1 = nullptr, *need2 = nullptr;  // FP64 gathers: the elements of the passes that are read
  double work_madds = 0;  // the last reconstruction's work model (multiply-adds of direct kernels)
  // run the optimisation loop as a device-side graph loop when the stream can
  // be captured; a batch's workers drive it from the host (several small
  // reconstructions in flight: building each one's conditional graph cost
  // more than the host's per-loop reads)
  bool device_loop = true;
  // the host-driven loop's body as an executable graph, kept across
  // reconstructions and updated in place when a new capture has its topology
  cudaGraphExec_t body_exec = nullptr;
  unsigned long long *d_wcnt = nullptr;  // the density scatters' part of it, spread over 64 counters
  long long *d_need = nullptr, *h_need = nullptr;  // pass-buffer sizes a plan needed, overflow flag
  KdeTable wtab{}, sdtab[3]{};
  double *d_val = nullptr;
  float *d_valf = nullptr;  // the factor values in FP32
  int *d_meta = nullptr;    // wm, wofs, sm[3], sofs[3]
  std::vector<double> table_key;  // database parameters of the uploaded factor tables
  double *h_out = nullptr;  // pinned staging of the density / histogram grids
  int64_t h_out_cap = 0;
  int64_t launches = 0;

  template <typename T>
  KdeBinsT<T> view() const {
    KdeBinsT<T> v;
    v.n = bins.n;
    v.gx = bins.gx;
    v.gy = bins.gy;
    v.gz = bins.gz;
    v.count = bins.count;
    double *const src[] = {bins.ks,  bins.scale, bins.shape, bins.support, bins.nest, bins.dens,     bins.cb,
                           bins.rxx, bins.ryy,   bins.rzz,   bins.net,     bins.dens_old, bins.scale_old};
    T **dst[] = {&v.ks,  &v.scale, &v.shape, &v.support, &v.nest, &v.dens,     &v.cb,
                 &v.rxx, &v.ryy,   &v.rzz,   &v.net,     &v.dens_old, &v.scale_old};
    for (int i = 0; i < 13; ++i) *dst[i] = reinterpret_cast<T *>(src[i]);
    return v;
  }

  cudaError_t ensure_bins(int n);
  cudaError_t ensure_pass(int64_t n1, int64_t n2);
  cudaError_t ensure_grid(int64_t ngrid);
  void release();
};

void kde_build_tables(const KdeParams &P, std::vector<double> &val, std::vector<int> &wm, std::vector<int> &wofs,
                      std::vector<int> (&sm)[3], std::vector<int> (&sofs)[3]);
cudaError_t kde_collect_active(KdeState &st, const KdeParams &P, const double *counts, cudaStream_t s,
                               int *nactive);
// fp32 != 0: the reconstruction runs in FP32 (convergence sums in FP64)
cudaError_t kde_run(KdeState &st, const KdeParams &P, double hs, double npts, int n_opt_loops, double rel_err,
                    bool skip_error, int fp32, cudaStream_t s, int *loops_done);
// st.dens_out = density grid * f * scale (FP64), from the last reconstruction
cudaError_t kde_output(KdeState &st, const KdeParams &P, int fp32, double f, double scale, cudaStream_t s);

}  // namespace mprw
