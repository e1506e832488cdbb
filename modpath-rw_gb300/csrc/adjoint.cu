// adjoint.cu -- the differentiable random walk, its density deposit and the
// hand-written adjoint of both (the model is described in adjoint.cuh).
//
// Kernels:
//   adj_node_setup_kernel  per node: Darcy flux averaged over the faces that
//                          meet at the node, zone shares, Dm / R (once per set-up)
//   adj_node_fields_kernel per node, per theta: phi, alphaL, alphaT, u, phi D
//   adj_node_div_kernel    per node: G = div(phi D) / phi, central differences
//   adj_walk_kernel        one thread per particle: steps of one segment from a
//                          checkpoint (optionally storing every position)
//   adj_deposit_kernel     biweight deposit, 64-bit fixed-point atomics (the
//                          density is repeatable to the last bit)
//   adj_deposit_adj_kernel adjoint of the deposit: per particle, a gather of
//                          the density gradient over the kernel's support
//   adj_reverse_kernel     one thread per particle: the reverse sweep of one
//                          segment; node adjoints accumulated per cell visit
//                          in local memory and flushed with atomics
//   adj_phid_bar_kernel    per node: adjoint of phi D from the adjoint of G
//                          (the transpose of the central differences, as a gather)
//   adj_theta_kernel       per node: adjoint of u, phi, alphaL, alphaT mapped to
//                          the zone parameters and the velocity scale,
//                          fixed-order per-block partial sums
// Everything is FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "adjoint.cuh"

namespace mprw {

namespace {

constexpr int kAdjThreads = 128;

__host__ __device__ __forceinline__ int64_t node_id(const AdjGrid &G, int a, int b, int c) {
  return (int64_t)a + (int64_t)(G.n[0] + 1) * ((int64_t)b + (int64_t)(G.n[1] + 1) * c);
}

// cell (model indexes cx, cy, cz; y from the front, z from the bottom) ->
// 0-based MODFLOW node (layer 0 on top, row 0 at the back)
__device__ __forceinline__ int32_t cell_of(const GridDims &g, int cx, int cy, int cz) {
  const int i = g.nrow - 1 - cy, k = g.nlay - 1 - cz;
  return k * g.ncpl + i * g.ncol + cx;
}

__global__ void adj_node_setup_kernel(AdjGrid G, GridDims g, CellBase base, const int32_t *ibound,
                                      const int32_t *zones, int nz, const double *dm, int dm_uniform, double R,
                                      double *q, double *beta, double *dmr) {
  const int64_t nn = G.nnode;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nn; v += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(v % (G.n[0] + 1));
    const int64_t r = v / (G.n[0] + 1);
    const int b = (int)(r % (G.n[1] + 1)), c = (int)(r / (G.n[1] + 1));
    double qs[3] = {0, 0, 0}, dms = 0.0;
    int cnt = 0;
    for (int z = 0; z < nz; ++z) beta[v * nz + z] = 0.0;
    for (int oz = -1; oz <= 0; ++oz)
      for (int oy = -1; oy <= 0; ++oy)
        for (int ox = -1; ox <= 0; ++ox) {
          const int cx = a + ox, cy = b + oy, cz = c + oz;
          if (cx < 0 || cx >= G.n[0] || cy < 0 || cy >= G.n[1] || cz < 0 || cz >= G.n[2]) continue;
          const int32_t cell = cell_of(g, cx, cy, cz);
          if (ibound[cell] == 0) continue;
          const double *Q = base.q + 6 * (int64_t)cell;  // Q1..Q6: flows along +x, +y, +z
          // the face of this cell that the node lies on, per axis
          qs[0] += (ox == 0 ? Q[0] : Q[1]) / (G.d[1] * G.d[2]);
          qs[1] += (oy == 0 ? Q[2] : Q[3]) / (G.d[0] * G.d[2]);
          qs[2] += (oz == 0 ? Q[4] : Q[5]) / (G.d[0] * G.d[1]);
          dms += dm_uniform ? dm[0] : dm[cell];
          beta[v * nz + zones[cell]] += 1.0;
          ++cnt;
        }
    const double inv = cnt ? 1.0 / cnt : 0.0;
    for (int d = 0; d < 3; ++d) q[3 * v + d] = qs[d] * inv;
    for (int z = 0; z < nz; ++z) beta[v * nz + z] *= inv;
    dmr[v] = dms * inv / R;
  }
}

// the dispersion tensor D = (aT r + dmr) I + (aL - aT) u u^T / r, r =
// sqrt(|u|^2 + eps^2), times phi; components xx, yy, zz, xy, xz, yz
__device__ __forceinline__ void phi_d(double phi, const double u[3], double aL, double aT, double dmr, double eps2,
                                      double out[6]) {
  const double r = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2] + eps2);
  const double iso = aT * r + dmr;
  const double an = (aL - aT) / r;
  out[0] = phi * (iso + an * u[0] * u[0]);
  out[1] = phi * (iso + an * u[1] * u[1]);
  out[2] = phi * (iso + an * u[2] * u[2]);
  out[3] = phi * (an * u[0] * u[1]);
  out[4] = phi * (an * u[0] * u[2]);
  out[5] = phi * (an * u[1] * u[2]);
}

__global__ void adj_node_fields_kernel(AdjGrid G, int nz, const double *theta, const double *q, const double *beta,
                                       const double *dmr, double R, double *phi_out, double *phid, double *nodes) {
  const int64_t nn = G.nnode;
  const double s = theta[3 * nz];
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nn; v += (int64_t)gridDim.x * blockDim.x) {
    double aL = 0.0, aT = 0.0, phi = 0.0;
    for (int z = 0; z < nz; ++z) {
      const double w = beta[v * nz + z];
      aL += w * theta[z];
      aT += w * theta[nz + z];
      phi += w * theta[2 * nz + z];
    }
    double u[3];
    for (int d = 0; d < 3; ++d) u[d] = phi > 0.0 ? s * q[3 * v + d] / (phi * R) : 0.0;
    double pd[6];
    phi_d(phi, u, aL, aT, dmr[v], G.eps2, pd);
    phi_out[v] = phi;
    for (int k = 0; k < 6; ++k) phid[6 * v + k] = pd[k];
    double *nd = nodes + ADJ_NV * v;
    nd[0] = u[0];
    nd[1] = u[1];
    nd[2] = u[2];
    nd[6] = aL;
    nd[7] = aT;
    nd[8] = dmr[v];
  }
}

// coefficient of f[ap] in the difference quotient at node index a along an
// axis of n cells (n + 1 nodes): central inside, one-sided at the ends
__host__ __device__ __forceinline__ double fd_coef(int a, int ap, int n, double h) {
  if (a == 0) return ap == 1 ? 1.0 / h : (ap == 0 ? -1.0 / h : 0.0);
  if (a == n) return ap == n ? 1.0 / h : (ap == n - 1 ? -1.0 / h : 0.0);
  return ap == a + 1 ? 0.5 / h : (ap == a - 1 ? -0.5 / h : 0.0);
}

// index of the phi D component (i, j) in the 6-vector
__host__ __device__ __forceinline__ int pd_index(int i, int j) {
  if (i == j) return i;
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  return lo == 0 ? (hi == 1 ? 3 : 4) : 5;
}

__global__ void adj_node_div_kernel(AdjGrid G, const double *phi, const double *phid, double *nodes) {
  const int64_t nn = G.nnode;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nn; v += (int64_t)gridDim.x * blockDim.x) {
    int idx[3];
    idx[0] = (int)(v % (G.n[0] + 1));
    const int64_t r = v / (G.n[0] + 1);
    idx[1] = (int)(r % (G.n[1] + 1));
    idx[2] = (int)(r / (G.n[1] + 1));
    double g[3] = {0, 0, 0};
    for (int j = 0; j < 3; ++j) {
      for (int ap = idx[j] - 1; ap <= idx[j] + 1; ++ap) {
        if (ap < 0 || ap > G.n[j]) continue;
        const double cf = fd_coef(idx[j], ap, G.n[j], G.d[j]);
        if (cf == 0.0) continue;
        int o[3] = {idx[0], idx[1], idx[2]};
        o[j] = ap;
        const double *pd = phid + 6 * node_id(G, o[0], o[1], o[2]);
        for (int i = 0; i < 3; ++i) g[i] += cf * pd[pd_index(i, j)];
      }
    }
    const double p = phi[v];
    double *nd = nodes + ADJ_NV * v;
    for (int i = 0; i < 3; ++i) nd[3 + i] = p > 0.0 ? g[i] / p : 0.0;
  }
}

// ---- one step ----------------------------------------------------------------
// The cell of a position and its local coordinates (the position is inside
// the domain after the fold; the last cell takes the upper face).
__device__ __forceinline__ void locate(const AdjGrid &G, const double x[3], int c[3], double f[3]) {
  for (int d = 0; d < 3; ++d) {
    const double t = (x[d] - G.lo[d]) / G.d[d];
    int i = (int)floor(t);
    if (i < 0) i = 0;
    if (i > G.n[d] - 1) i = G.n[d] - 1;
    double fr = t - (double)i;
    fr = fr < 0.0 ? 0.0 : (fr > 1.0 ? 1.0 : fr);
    c[d] = i;
    f[d] = fr;
  }
}

// reflection at both walls of [lo, lo + L] (a triangle wave: continuous,
// slope +1 or -1, returned in sgn)
__device__ __forceinline__ double fold(double y, double lo, double L, double &sgn) {
  const double P = 2.0 * L;
  double t = y - lo;
  t -= floor(t / P) * P;
  if (t > L) {
    sgn = -1.0;
    return lo + (P - t);
  }
  sgn = 1.0;
  return lo + t;
}

struct Interp {
  int64_t base;
  double w[8];       // trilinear weights of the corners, corner o = ox + 2 oy + 4 oz
  double u[3], g[3], aL, aT, dm;
};

__device__ __forceinline__ int64_t corner_node(const AdjGrid &G, int64_t base, int o) {
  return base + (o & 1) + (int64_t)(G.n[0] + 1) * (((o >> 1) & 1) + (int64_t)(G.n[1] + 1) * ((o >> 2) & 1));
}

__device__ __forceinline__ void interp(const AdjGrid &G, const double *nodes, const int c[3], const double f[3],
                                       Interp &I) {
  I.base = node_id(G, c[0], c[1], c[2]);
  for (int d = 0; d < 3; ++d) I.u[d] = I.g[d] = 0.0;
  I.aL = I.aT = I.dm = 0.0;
#pragma unroll
  for (int o = 0; o < 8; ++o) {
    const double w = ((o & 1) ? f[0] : 1.0 - f[0]) * (((o >> 1) & 1) ? f[1] : 1.0 - f[1]) *
                     (((o >> 2) & 1) ? f[2] : 1.0 - f[2]);
    I.w[o] = w;
    const double *nd = nodes + ADJ_NV * corner_node(G, I.base, o);
    for (int d = 0; d < 3; ++d) {
      I.u[d] += w * nd[d];
      I.g[d] += w * nd[3 + d];
    }
    I.aL += w * nd[6];
    I.aT += w * nd[7];
    I.dm += w * nd[8];
  }
}

// gradient of corner o's weight
__device__ __forceinline__ void weight_grad(const AdjGrid &G, const double f[3], int o, double gw[3]) {
  const double fx = (o & 1) ? f[0] : 1.0 - f[0], fy = ((o >> 1) & 1) ? f[1] : 1.0 - f[1],
               fz = ((o >> 2) & 1) ? f[2] : 1.0 - f[2];
  const double sx = (o & 1) ? 1.0 : -1.0, sy = ((o >> 1) & 1) ? 1.0 : -1.0, sz = ((o >> 2) & 1) ? 1.0 : -1.0;
  gw[0] = sx / G.d[0] * fy * fz;
  gw[1] = sy / G.d[1] * fx * fz;
  gw[2] = sz / G.d[2] * fx * fy;
}

struct Disp {
  double s2, r, a, b, kappa, P, bxi[3];
};

// B xi = a xi + kappa (u . xi) u
__device__ __forceinline__ void displacement(const AdjGrid &G, const Interp &I, const double xi[3], Disp &D) {
  D.s2 = I.u[0] * I.u[0] + I.u[1] * I.u[1] + I.u[2] * I.u[2];
  D.r = sqrt(D.s2 + G.eps2);
  const double lt = I.aT * D.r + I.dm;
  const double ll = lt + (I.aL - I.aT) * D.s2 / D.r;
  D.a = sqrt(2.0 * lt);
  D.b = sqrt(2.0 * ll);
  D.kappa = 2.0 * (I.aL - I.aT) / (D.r * (D.a + D.b));
  D.P = I.u[0] * xi[0] + I.u[1] * xi[1] + I.u[2] * xi[2];
  for (int d = 0; d < 3; ++d) D.bxi[d] = D.a * xi[d] + D.kappa * D.P * I.u[d];
}

__device__ __forceinline__ void normals(uint64_t seed, uint64_t id, int64_t step, double xi[3]) {
  uint64_t ctr = 9ull * (uint64_t)step;
  for (int d = 0; d < 3; ++d) xi[d] = normal_ih12(seed, id, ctr);
}

__device__ __forceinline__ void step_forward(const AdjGrid &G, const double *nodes, double x[3], const double xi[3],
                                             double dt, double sdt) {
  int c[3];
  double f[3];
  locate(G, x, c, f);
  Interp I;
  interp(G, nodes, c, f, I);
  Disp D;
  displacement(G, I, xi, D);
  for (int d = 0; d < 3; ++d) {
    const double y = x[d] + (I.u[d] + I.g[d]) * dt + D.bxi[d] * sdt;
    double sg;
    x[d] = fold(y, G.lo[d], G.n[d] * G.d[d], sg);
  }
}

__global__ void __launch_bounds__(kAdjThreads) adj_walk_kernel(AdjGrid G, const double *nodes, int64_t np,
                                                               const uint64_t *id, uint64_t seed, int64_t step0,
                                                               int nst, double dt, const double *xin, double *xout,
                                                               double *seg) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= np) return;
  double x[3] = {xin[p], xin[np + p], xin[2 * np + p]};
  const double sdt = sqrt(dt);
  const uint64_t pid = id[p];
  for (int k = 0; k < nst; ++k) {
    if (seg)
      for (int d = 0; d < 3; ++d) seg[((int64_t)k * 3 + d) * np + p] = x[d];
    double xi[3];
    normals(seed, pid, step0 + k, xi);
    step_forward(G, nodes, x, xi, dt, sdt);
  }
  if (xout)
    for (int d = 0; d < 3; ++d) xout[d * np + p] = x[d];
}

// ---- deposit -------------------------------------------------------------------
struct DepGrid {
  double origin[3], bin[3], h[3];
  int nb[3];
};

// the biweight factor of one dimension and its derivative in r
__device__ __forceinline__ double biweight(double r, double h, double &dk) {
  const double t = r / h;
  if (fabs(t) >= 1.0) {
    dk = 0.0;
    return 0.0;
  }
  const double s = 1.0 - t * t;
  const double c = 15.0 / (16.0 * h);
  dk = c * 2.0 * s * (-2.0 * t / h);
  return c * s * s;
}

// range of bins whose centres lie within h of x (empty when lo > hi)
__device__ __forceinline__ void support(const DepGrid &Q, int d, double x, int &lo, int &hi) {
  if (Q.nb[d] == 1) {
    lo = hi = 0;
    return;
  }
  const double a = (x - Q.h[d] - Q.origin[d]) / Q.bin[d] - 0.5, b = (x + Q.h[d] - Q.origin[d]) / Q.bin[d] - 0.5;
  lo = (int)ceil(a);
  hi = (int)floor(b);
  if (lo < 0) lo = 0;
  if (hi > Q.nb[d] - 1) hi = Q.nb[d] - 1;
}

__global__ void adj_deposit_kernel(DepGrid Q, int64_t np, const double *x, const double *mass, double fscale,
                                   unsigned long long *grid) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    const double m = mass[p];
    if (m == 0.0) continue;
    const double X[3] = {x[p], x[np + p], x[2 * np + p]};
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) support(Q, d, X[d], lo[d], hi[d]);
    for (int k = lo[2]; k <= hi[2]; ++k) {
      double dk;
      const double kz = Q.nb[2] == 1 ? 1.0 : biweight(Q.origin[2] + (k + 0.5) * Q.bin[2] - X[2], Q.h[2], dk);
      if (kz == 0.0) continue;
      for (int j = lo[1]; j <= hi[1]; ++j) {
        const double ky = Q.nb[1] == 1 ? 1.0 : biweight(Q.origin[1] + (j + 0.5) * Q.bin[1] - X[1], Q.h[1], dk);
        if (ky == 0.0) continue;
        for (int i = lo[0]; i <= hi[0]; ++i) {
          const double kx = Q.nb[0] == 1 ? 1.0 : biweight(Q.origin[0] + (i + 0.5) * Q.bin[0] - X[0], Q.h[0], dk);
          if (kx == 0.0) continue;
          const double v = m * (kx * (ky * kz));
          const int64_t g = i + (int64_t)Q.nb[0] * (j + (int64_t)Q.nb[1] * k);
          atomicAdd(grid + g, (unsigned long long)__double2ll_rn(v * fscale));
        }
      }
    }
  }
}

__global__ void adj_fixed_to_double_kernel(const unsigned long long *a, double inv, double *out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)(long long)a[i] * inv;
}

// lambda = d(sum_c gdens_c rho_c) / dx_p
__global__ void adj_deposit_adj_kernel(DepGrid Q, int64_t np, const double *x, const double *mass,
                                       const double *gdens, double *lam) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    const double m = mass[p];
    double l[3] = {0, 0, 0};
    if (m != 0.0) {
      const double X[3] = {x[p], x[np + p], x[2 * np + p]};
      int lo[3], hi[3];
      for (int d = 0; d < 3; ++d) support(Q, d, X[d], lo[d], hi[d]);
      for (int k = lo[2]; k <= hi[2]; ++k) {
        double dz = 0.0;
        const double kz = Q.nb[2] == 1 ? 1.0 : biweight(Q.origin[2] + (k + 0.5) * Q.bin[2] - X[2], Q.h[2], dz);
        for (int j = lo[1]; j <= hi[1]; ++j) {
          double dy = 0.0;
          const double ky = Q.nb[1] == 1 ? 1.0 : biweight(Q.origin[1] + (j + 0.5) * Q.bin[1] - X[1], Q.h[1], dy);
          for (int i = lo[0]; i <= hi[0]; ++i) {
            double dx = 0.0;
            const double kx = Q.nb[0] == 1 ? 1.0 : biweight(Q.origin[0] + (i + 0.5) * Q.bin[0] - X[0], Q.h[0], dx);
            const double gg = gdens[i + (int64_t)Q.nb[0] * (j + (int64_t)Q.nb[1] * k)] * m;
            // d/dX of K(centre - X) = -K'
            l[0] -= gg * dx * ky * kz;
            l[1] -= gg * kx * dy * kz;
            l[2] -= gg * kx * ky * dz;
          }
        }
      }
    }
    for (int d = 0; d < 3; ++d) lam[d * np + p] = l[d];
  }
}

// ---- the reverse sweep -------------------------------------------------------------
// Adjoint of x' = fold(x + (u + G) dt + B xi sqrt(dt)) at one step, given
// lam' = dL/dx'.  Returns lam = dL/dx in lam and adds w_o * (du, dG, daL,
// daT) of every corner o to acc (8 values per corner; acc belongs to the
// particle's current cell: the caller flushes it on a cell change).
__device__ __forceinline__ void step_reverse(const AdjGrid &G, const double *nodes, const double x[3],
                                             const double xi[3], double dt, double sdt, double lam[3],
                                             double acc[64]) {
  int c[3];
  double f[3];
  locate(G, x, c, f);
  Interp I;
  interp(G, nodes, c, f, I);
  Disp D;
  displacement(G, I, xi, D);
  double lt[3];
  for (int d = 0; d < 3; ++d) {
    const double y = x[d] + (I.u[d] + I.g[d]) * dt + D.bxi[d] * sdt;
    double sg;
    (void)fold(y, G.lo[d], G.n[d] * G.d[d], sg);
    lt[d] = sg * lam[d];
  }
  // B xi = a xi + kappa P u as a function of u, aL, aT, dm: the transposed
  // derivatives applied to lt.  With r = sqrt(|u|^2 + eps^2): da = (aT / a)
  // dr, dr = (u . du) / r, db = d(ll) / b, dkappa = -kappa (dr / r + (da + db)
  // / (a + b)).
  const double ul = I.u[0] * lt[0] + I.u[1] * lt[1] + I.u[2] * lt[2];
  const double xl = xi[0] * lt[0] + xi[1] * lt[1] + xi[2] * lt[2];
  const double r = D.r, a = D.a, b = D.b, k = D.kappa, P = D.P, s2 = D.s2, ab = a + b;
  const double dA = I.aL - I.aT;
  const double ca = (I.aT / a) / r;                                          // da = ca (u . du)
  const double cb = (I.aT / r + dA * (2.0 / r - s2 / (r * r * r))) / b;      // db = cb (u . du)
  const double ck = -k * (1.0 / (r * r) + (ca + cb) / ab);                   // dkappa = ck (u . du)
  double jv[3];
  for (int d = 0; d < 3; ++d) jv[d] = ca * xl * I.u[d] + ck * P * ul * I.u[d] + k * ul * xi[d] + k * P * lt[d];
  const double dk_daL = 2.0 / (r * ab) - k * (s2 / (r * b)) / ab;
  const double da_daT = r / a, db_daT = (r - s2 / r) / b;
  const double dk_daT = -2.0 / (r * ab) - k * (da_daT + db_daT) / ab;
  const double dk_ddm = -k * (1.0 / a + 1.0 / b) / ab;
  const double cL = dk_daL * P * ul;
  const double cT = da_daT * xl + dk_daT * P * ul;
  const double cD = xl / a + dk_ddm * P * ul;
  double ln[3] = {lt[0], lt[1], lt[2]};
#pragma unroll
  for (int o = 0; o < 8; ++o) {
    const double w = I.w[o];
    double *A = acc + 8 * o;
    for (int d = 0; d < 3; ++d) {
      A[d] += w * (dt * lt[d] + sdt * jv[d]);
      A[3 + d] += w * (dt * lt[d]);
    }
    A[6] += w * sdt * cL;
    A[7] += w * sdt * cT;
    const double *nd = nodes + ADJ_NV * corner_node(G, I.base, o);
    const double s = dt * ((nd[0] + nd[3]) * lt[0] + (nd[1] + nd[4]) * lt[1] + (nd[2] + nd[5]) * lt[2]) +
                     sdt * (nd[0] * jv[0] + nd[1] * jv[1] + nd[2] * jv[2] + nd[6] * cL + nd[7] * cT + nd[8] * cD);
    double gw[3];
    weight_grad(G, f, o, gw);
    for (int d = 0; d < 3; ++d) ln[d] += s * gw[d];
  }
  for (int d = 0; d < 3; ++d) lam[d] = ln[d];
}

__device__ __forceinline__ void flush_acc(const AdjGrid &G, int64_t base, double acc[64], double *nadj) {
  if (base < 0) return;
#pragma unroll
  for (int o = 0; o < 8; ++o) {
    double *dst = nadj + 8 * corner_node(G, base, o);
    for (int k = 0; k < 8; ++k) {
      const double v = acc[8 * o + k];
      if (v != 0.0) atomicAdd(dst + k, v);
      acc[8 * o + k] = 0.0;
    }
  }
}

__global__ void __launch_bounds__(kAdjThreads) adj_reverse_kernel(AdjGrid G, const double *nodes, int64_t np,
                                                                  const uint64_t *id, uint64_t seed, int64_t step0,
                                                                  int nst, double dt, const double *seg,
                                                                  double *lam_io, double *nadj) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= np) return;
  double lam[3] = {lam_io[p], lam_io[np + p], lam_io[2 * np + p]};
  const double sdt = sqrt(dt);
  const uint64_t pid = id[p];
  double acc[64];
  for (int k = 0; k < 64; ++k) acc[k] = 0.0;
  int64_t base = -1;
  for (int k = nst - 1; k >= 0; --k) {
    const double x[3] = {seg[((int64_t)k * 3 + 0) * np + p], seg[((int64_t)k * 3 + 1) * np + p],
                         seg[((int64_t)k * 3 + 2) * np + p]};
    int c[3];
    double f[3];
    locate(G, x, c, f);
    const int64_t b = node_id(G, c[0], c[1], c[2]);
    if (b != base) {
      flush_acc(G, base, acc, nadj);
      base = b;
    }
    double xi[3];
    normals(seed, pid, step0 + k, xi);
    step_reverse(G, nodes, x, xi, dt, sdt, lam, acc);
  }
  flush_acc(G, base, acc, nadj);
  for (int d = 0; d < 3; ++d) lam_io[d * np + p] = lam[d];
}

// ---- node adjoints to the parameters ----------------------------------------------
// adjoint of phi D (6 per node) from the adjoint of G (nadj[3..5]): G_i =
// (1/phi) sum_j D_j (phi D)_ij, the transpose of the differences as a gather
// over the neighbours along each axis; and the part of phi's adjoint that G
// carries directly (-G . Gbar / phi).
__global__ void adj_phid_bar_kernel(AdjGrid G, const double *phi, const double *nodes, const double *nadj,
                                    double *phidbar, double *phibar) {
  const int64_t nn = G.nnode;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nn; v += (int64_t)gridDim.x * blockDim.x) {
    int idx[3];
    idx[0] = (int)(v % (G.n[0] + 1));
    const int64_t r = v / (G.n[0] + 1);
    idx[1] = (int)(r % (G.n[1] + 1));
    idx[2] = (int)(r / (G.n[1] + 1));
    double pb[6] = {0, 0, 0, 0, 0, 0};
    for (int j = 0; j < 3; ++j) {
      for (int a = idx[j] - 1; a <= idx[j] + 1; ++a) {
        if (a < 0 || a > G.n[j]) continue;
        const double cf = fd_coef(a, idx[j], G.n[j], G.d[j]);
        if (cf == 0.0) continue;
        int o[3] = {idx[0], idx[1], idx[2]};
        o[j] = a;
        const int64_t c = node_id(G, o[0], o[1], o[2]);
        const double pc = phi[c];
        if (!(pc > 0.0)) continue;
        const double *gb = nadj + 8 * c + 3;
        for (int i = 0; i < 3; ++i) pb[pd_index(i, j)] += cf * gb[i] / pc;
      }
    }
    for (int k = 0; k < 6; ++k) phidbar[6 * v + k] = pb[k];
    const double p = phi[v];
    const double *g = nodes + ADJ_NV * v + 3;
    const double *gb = nadj + 8 * v + 3;
    phibar[v] = p > 0.0 ? -(g[0] * gb[0] + g[1] * gb[1] + g[2] * gb[2]) / p : 0.0;
  }
}

// per node: phi D -> (u, alphaL, alphaT, phi); u = s q / (phi R) -> (s, phi);
// node values -> zone parameters; per-block partial sums (fixed order)
__global__ void __launch_bounds__(kAdjThreads) adj_theta_kernel(AdjGrid G, int nz, const double *theta,
                                                                const double *beta, const double *phi,
                                                                const double *nodes, const double *nadj,
                                                                const double *phidbar, const double *phibar0,
                                                                double *part) {
  __shared__ double red[3 * ADJ_MAXZONES + 1][kAdjThreads / 32];
  const int nth = 3 * nz + 1;
  double loc[3 * ADJ_MAXZONES + 1];
  for (int k = 0; k < nth; ++k) loc[k] = 0.0;
  const double s = theta[3 * nz];
  const int64_t nn = G.nnode;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nn; v += (int64_t)gridDim.x * blockDim.x) {
    const double *nd = nodes + ADJ_NV * v;
    const double u[3] = {nd[0], nd[1], nd[2]};
    const double aL = nd[6], aT = nd[7], dmr = nd[8], p = phi[v];
    const double *A = nadj + 8 * v;
    double ub[3] = {A[0], A[1], A[2]};
    double aLb = A[6], aTb = A[7];
    double pbar = phibar0[v];
    // phi D = phi * D(u, aL, aT), D = (aT r + dmr) I + (aL - aT) u u^T / r
    const double *PB = phidbar + 6 * v;
    double Dm[6];
    phi_d(1.0, u, aL, aT, dmr, G.eps2, Dm);
    for (int k = 0; k < 6; ++k) pbar += PB[k] * Dm[k];
    double Db[6];
    for (int k = 0; k < 6; ++k) Db[k] = p * PB[k];
    const double r = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2] + G.eps2);
    const double an = (aL - aT) / r;
    // dD_ii/du_k = aT u_k / r + (aL - aT)(2 u_i d_ik / r - u_i^2 u_k / r^3)
    // dD_ij/du_k = (aL - aT)((d_ik u_j + u_i d_jk) / r - u_i u_j u_k / r^3), i != j
    double sum_uDu = 0.0, tr = 0.0;
    for (int i = 0; i < 3; ++i) {
      tr += Db[i];
      sum_uDu += Db[i] * u[i] * u[i];
    }
    sum_uDu += Db[3] * u[0] * u[1] + Db[4] * u[0] * u[2] + Db[5] * u[1] * u[2];
    double lin[3];  // sum over the components of Db * d(u_i u_j)/du_k
    lin[0] = 2.0 * Db[0] * u[0] + Db[3] * u[1] + Db[4] * u[2];
    lin[1] = 2.0 * Db[1] * u[1] + Db[3] * u[0] + Db[5] * u[2];
    lin[2] = 2.0 * Db[2] * u[2] + Db[4] * u[0] + Db[5] * u[1];
    for (int k = 0; k < 3; ++k) ub[k] += aT * tr * u[k] / r + an * lin[k] - (aL - aT) * sum_uDu * u[k] / (r * r * r);
    aLb += sum_uDu / r;
    aTb += tr * r - sum_uDu / r;
    // u = s q / (phi R)
    const double su = ub[0] * u[0] + ub[1] * u[1] + ub[2] * u[2];
    if (p > 0.0) pbar -= su / p;
    const double sbar = s != 0.0 ? su / s : 0.0;
    for (int z = 0; z < nz; ++z) {
      const double w = beta[v * nz + z];
      if (w == 0.0) continue;
      loc[z] += w * aLb;
      loc[nz + z] += w * aTb;
      loc[2 * nz + z] += w * pbar;
    }
    loc[3 * nz] += sbar;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < nth; ++k) {
    double v = loc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[k][wid] = v;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nth; k += blockDim.x) {
    double v = 0.0;
    for (int w = 0; w < kAdjThreads / 32; ++w) v += red[k][w];
    part[(int64_t)blockIdx.x * nth + k] = v;
  }
}

__global__ void adj_init_particles_kernel(int64_t n, const int32_t *status, const double *mass, const uint64_t *id,
                                          double *m_out, uint64_t *id_out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int32_t st = status[p];
    const bool walk = st == ST_ACTIVE || st == ST_PENDING;
    m_out[p] = walk ? (mass ? mass[p] : 1.0) : 0.0;
    id_out[p] = id ? id[p] : (uint64_t)p;
  }
}

int blocks_for_adj(int64_t n) {
  int64_t b = (n + kAdjThreads - 1) / kAdjThreads;
  if (b > 152 * 32) b = 152 * 32;
  return b < 1 ? 1 : (int)b;
}

#define ACK(x)                        \
  do {                                \
    cudaError_t e_ = (x);             \
    if (e_ != cudaSuccess) return e_; \
  } while (0)

template <typename T>
cudaError_t alloc(T **p, size_t n) {
  if (*p) cudaFree(*p);
  *p = nullptr;
  return cudaMalloc(p, sizeof(T) * (n ? n : 1));
}

DepGrid dep_grid(const AdjOptions &o) {
  DepGrid Q;
  for (int d = 0; d < 3; ++d) {
    Q.origin[d] = o.origin[d];
    Q.bin[d] = o.bin[d];
    Q.h[d] = o.h[d];
    Q.nb[d] = o.nb[d];
  }
  return Q;
}

}  // namespace

void AdjState::release() {
  void *ptrs[] = {d_q,   d_beta, d_dmr, d_theta, d_phi,     d_phid,   d_nodes, d_ckpt, d_seg, d_mass,
                  d_id,  d_lam,  d_nadj, d_phidbar, d_phibar, d_part, d_dens,  d_densf, d_gdens};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  d_q = d_beta = d_dmr = d_theta = d_phi = d_phid = d_nodes = d_ckpt = d_seg = d_mass = d_lam = d_nadj = nullptr;
  d_phidbar = d_phibar = d_part = d_densf = d_gdens = nullptr;
  d_id = nullptr;
  d_dens = nullptr;
  forward_done = false;
}

cudaError_t AdjState::setup(const AdjInputs &in, const AdjOptions &opt, const int32_t *zones_host,
                            std::vector<char> &err) {
  auto bad = [&](const char *m) {
    err.assign(m, m + std::strlen(m) + 1);
    return cudaErrorInvalidValue;
  };
  if (opt.nzones < 1 || opt.nzones > ADJ_MAXZONES) return bad("nzones must be in 1..64");
  if (!(opt.dt > 0.0) || opt.nsteps < 1 || opt.checkpoint < 1 || opt.checkpoint > opt.nsteps)
    return bad("dt > 0, nsteps >= 1 and 1 <= checkpoint <= nsteps are required");
  if (!(opt.eps > 0.0) || !std::isfinite(opt.eps)) return bad("the velocity floor must be > 0");
  for (int d = 0; d < 3; ++d) {
    if (opt.nb[d] < 1) return bad("density grid: n_bins >= 1");
    if (opt.nb[d] > 1 && (!(opt.bin[d] > 0.0) || !(opt.h[d] > 0.0)))
      return bad("density grid: bin size and kernel half-width > 0 along every dimension with several bins");
  }
  const int64_t ncell = in.g.ncell;
  for (int64_t c = 0; c < ncell; ++c)
    if (zones_host[c] < 0 || zones_host[c] >= opt.nzones) return bad("zone index out of range");
  release();
  o = opt;
  R = in.R;
  G.n[0] = in.g.ncol;
  G.n[1] = in.g.nrow;
  G.n[2] = in.g.nlay;
  for (int d = 0; d < 3; ++d) {
    G.lo[d] = in.lo[d];
    G.d[d] = in.d[d];
  }
  G.nnode = (int64_t)(G.n[0] + 1) * (G.n[1] + 1) * (G.n[2] + 1);
  G.eps2 = opt.eps * opt.eps;
  const int nz = opt.nzones;
  ACK(alloc(&d_q, 3 * G.nnode));
  ACK(alloc(&d_beta, (size_t)nz * G.nnode));
  ACK(alloc(&d_dmr, G.nnode));
  int32_t *d_zones = nullptr;
  ACK(cudaMalloc(&d_zones, sizeof(int32_t) * ncell));
  cudaError_t e = cudaMemcpy(d_zones, zones_host, sizeof(int32_t) * ncell, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    adj_node_setup_kernel<<<blocks_for_adj(G.nnode), kAdjThreads>>>(G, in.g, in.base, in.iboundts, d_zones, nz, in.dm,
                                                                     in.dm_uniform, R, d_q, d_beta, d_dmr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  cudaFree(d_zones);
  ACK(e);
  // particles: model coordinates, masses (zero for particles that are not walked), ids
  np = in.n;
  const int nseg = (opt.nsteps + opt.checkpoint - 1) / opt.checkpoint;
  ACK(alloc(&d_ckpt, (size_t)(nseg + 1) * 3 * np));
  ACK(alloc(&d_seg, (size_t)opt.checkpoint * 3 * np));
  ACK(alloc(&d_mass, np));
  ACK(alloc(&d_id, np));
  ACK(alloc(&d_lam, 3 * np));
  mass_total = 0.0;
  if (np > 0) {
    if (in.mixed)
      ACK(launch_global_xyz<float>(in.geo, np, in.cell, (const float *)in.x, (const float *)in.y,
                                   (const float *)in.z, d_ckpt, d_ckpt + np, d_ckpt + 2 * np, 0));
    else
      ACK(launch_global_xyz<double>(in.geo, np, in.cell, (const double *)in.x, (const double *)in.y,
                                    (const double *)in.z, d_ckpt, d_ckpt + np, d_ckpt + 2 * np, 0));
    adj_init_particles_kernel<<<blocks_for_adj(np), kAdjThreads>>>(np, in.status, in.mass, in.id, d_mass, d_id);
    ACK(cudaGetLastError());
    std::vector<double> hm(np);
    ACK(cudaMemcpy(hm.data(), d_mass, sizeof(double) * np, cudaMemcpyDeviceToHost));
    for (double m : hm) mass_total += std::fabs(m);
  }
  // per-theta buffers
  ACK(alloc(&d_theta, 3 * nz + 1));
  ACK(alloc(&d_phi, G.nnode));
  ACK(alloc(&d_phid, 6 * G.nnode));
  ACK(alloc(&d_nodes, ADJ_NV * G.nnode));
  ACK(alloc(&d_nadj, 8 * G.nnode));
  ACK(alloc(&d_phidbar, 6 * G.nnode));
  ACK(alloc(&d_phibar, G.nnode));
  part_blocks = blocks_for_adj(G.nnode);
  if (part_blocks > 152 * 4) part_blocks = 152 * 4;
  ACK(alloc(&d_part, (size_t)part_blocks * (3 * nz + 1)));
  ngrid = (int64_t)opt.nb[0] * opt.nb[1] * opt.nb[2];
  ACK(alloc(&d_dens, ngrid));
  ACK(alloc(&d_densf, ngrid));
  ACK(alloc(&d_gdens, ngrid));
  forward_done = false;
  return cudaDeviceSynchronize();
}

cudaError_t AdjState::forward(const double *theta_host, double *density_host, cudaStream_t s) {
  const int nz = o.nzones;
  ACK(cudaMemcpyAsync(d_theta, theta_host, sizeof(double) * (3 * nz + 1), cudaMemcpyHostToDevice, s));
  const int nb = blocks_for_adj(G.nnode);
  adj_node_fields_kernel<<<nb, kAdjThreads, 0, s>>>(G, nz, d_theta, d_q, d_beta, d_dmr, R, d_phi, d_phid, d_nodes);
  adj_node_div_kernel<<<nb, kAdjThreads, 0, s>>>(G, d_phi, d_phid, d_nodes);
  launches = 2;
  const int nseg = (o.nsteps + o.checkpoint - 1) / o.checkpoint;
  const int pb = (int)((np + kAdjThreads - 1) / kAdjThreads);
  for (int j = 0; j < nseg && np > 0; ++j) {
    const int64_t step0 = (int64_t)j * o.checkpoint;
    const int nst = (int)std::min<int64_t>(o.checkpoint, o.nsteps - step0);
    adj_walk_kernel<<<pb, kAdjThreads, 0, s>>>(G, d_nodes, np, d_id, o.seed, step0, nst, o.dt,
                                                d_ckpt + (size_t)j * 3 * np, d_ckpt + (size_t)(j + 1) * 3 * np,
                                                nullptr);
    ++launches;
  }
  ACK(cudaGetLastError());
  // deposit: the density of every cell is at most the total mass times the
  // kernel's peak; 2^shift times that stays below 2^62
  double bound = mass_total;
  for (int d = 0; d < 3; ++d)
    if (o.nb[d] > 1) bound *= 15.0 / (16.0 * o.h[d]);
  int ex = 0;
  std::frexp(std::max(bound, 1e-300), &ex);
  const int shift = 61 - ex;
  const DepGrid Q = dep_grid(o);
  ACK(cudaMemsetAsync(d_dens, 0, sizeof(unsigned long long) * ngrid, s));
  adj_deposit_kernel<<<blocks_for_adj(np), kAdjThreads, 0, s>>>(Q, np, d_ckpt + (size_t)nseg * 3 * np, d_mass,
                                                                 std::ldexp(1.0, shift), d_dens);
  adj_fixed_to_double_kernel<<<blocks_for_adj(ngrid), kAdjThreads, 0, s>>>(d_dens, std::ldexp(1.0, -shift), d_densf,
                                                                           ngrid);
  launches += 2;
  ACK(cudaGetLastError());
  ACK(cudaMemcpyAsync(density_host, d_densf, sizeof(double) * ngrid, cudaMemcpyDeviceToHost, s));
  ACK(cudaStreamSynchronize(s));
  forward_done = true;
  return cudaSuccess;
}

cudaError_t AdjState::backward(const double *gdens_host, double *grad_host, cudaStream_t s) {
  const int nz = o.nzones, nth = 3 * nz + 1;
  const int nseg = (o.nsteps + o.checkpoint - 1) / o.checkpoint;
  const DepGrid Q = dep_grid(o);
  ACK(cudaMemcpyAsync(d_gdens, gdens_host, sizeof(double) * ngrid, cudaMemcpyHostToDevice, s));
  launches = 0;
  if (np > 0) {
    adj_deposit_adj_kernel<<<blocks_for_adj(np), kAdjThreads, 0, s>>>(Q, np, d_ckpt + (size_t)nseg * 3 * np, d_mass,
                                                                     d_gdens, d_lam);
    ++launches;
  }
  ACK(cudaMemsetAsync(d_nadj, 0, sizeof(double) * 8 * G.nnode, s));
  const int pb = (int)((np + kAdjThreads - 1) / kAdjThreads);
  for (int j = nseg - 1; j >= 0 && np > 0; --j) {
    const int64_t step0 = (int64_t)j * o.checkpoint;
    const int nst = (int)std::min<int64_t>(o.checkpoint, o.nsteps - step0);
    // recompute the segment from its checkpoint, storing the position before every step
    adj_walk_kernel<<<pb, kAdjThreads, 0, s>>>(G, d_nodes, np, d_id, o.seed, step0, nst, o.dt,
                                                d_ckpt + (size_t)j * 3 * np, nullptr, d_seg);
    adj_reverse_kernel<<<pb, kAdjThreads, 0, s>>>(G, d_nodes, np, d_id, o.seed, step0, nst, o.dt, d_seg, d_lam,
                                                   d_nadj);
    launches += 2;
  }
  ACK(cudaGetLastError());
  const int nb = blocks_for_adj(G.nnode);
  adj_phid_bar_kernel<<<nb, kAdjThreads, 0, s>>>(G, d_phi, d_nodes, d_nadj, d_phidbar, d_phibar);
  adj_theta_kernel<<<part_blocks, kAdjThreads, 0, s>>>(G, nz, d_theta, d_beta, d_phi, d_nodes, d_nadj, d_phidbar,
                                                       d_phibar, d_part);
  launches += 2;
  ACK(cudaGetLastError());
  std::vector<double> part((size_t)part_blocks * nth);
  ACK(cudaMemcpyAsync(part.data(), d_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, s));
  ACK(cudaStreamSynchronize(s));
  for (int k = 0; k < nth; ++k) {
    double v = 0.0;
    for (int b = 0; b < part_blocks; ++b) v += part[(size_t)b * nth + k];
    grad_host[k] = v;
  }
  return cudaSuccess;
}

}  // namespace mprw
