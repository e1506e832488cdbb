// adjoint.cuh -- the differentiable random walk and its adjoint (adjoint.cu).
//
// A variant of the random walk that sits beside the reference's scheme: the
// reference's step is not differentiable in its parameters (a step cut at a
// cell face shifts every later normal to another step, and the histogram
// deposit is piecewise constant), so gradients of a concentration misfit
// need a walk whose path is a continuous function of the parameters.  Here:
//   * every field lives on the lattice of cell corners ("nodes") and is
//     interpolated trilinearly: pore velocity u = s q / (phi R) (q the Darcy
//     flux averaged over the faces that meet at the node, s a velocity scale),
//     the drift correction G = div(phi D) / phi from central differences of
//     the node values of phi D (the reference's (div D) term,
//     TrackSubCell.F90:2695-2818, on nodes instead of cell corners), and the
//     dispersivities alphaL, alphaT and Dm;
//   * D = (alphaT r + Dm/R) I + (alphaL - alphaT) u u^T / r with r =
//     sqrt(|u|^2 + eps^2): the reference's tensor where |u| >> eps (the
//     velocity floor eps), smooth where u vanishes -- without it the tensor's
//     axis turns arbitrarily fast near stagnation and the path's sensitivity
//     to the parameters grows without bound;
//   * a fixed time step dt, x' = fold(x + (u + G) dt + B xi sqrt(dt)) with
//     B xi = a xi + kappa (u . xi) u, a = sqrt(2 (alphaT r + Dm/R)),
//     b = sqrt(2 (alphaT r + Dm/R + (alphaL - alphaT) |u|^2 / r)),
//     kappa = 2 (alphaL - alphaT) / (r (a + b)), so that B B^T = 2 D as the
//     reference's B matrix gives (TrackSubCell.F90:2821-2928) but smooth in
//     u; fold reflects at the domain walls (continuous, piecewise linear);
//   * xi: Irwin-Hall(12) normals from Philox keyed by (seed, particle id,
//     step), so a perturbed run draws the same numbers (common random
//     numbers) whatever its path does;
//   * the density on a grid is a deposit of a product biweight kernel
//     (15/16)(1 - r^2)^2 / h per dimension, continuously differentiable in
//     the particle position.
// Parameters theta: alphaL, alphaT and porosity per zone (a zone per cell,
// nodes take the share of their adjacent cells in each zone) and the
// velocity scale s.  The adjoint sweeps the steps backwards from the density
// gradient; the particle positions are stored every `checkpoint` steps and
// each segment is recomputed before its reverse sweep.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "mprw_kernels.cuh"

namespace mprw {

constexpr int ADJ_MAXZONES = 64;
constexpr int ADJ_NV = 9;  // node record: u[3], g[3], alphaL, alphaT, Dm/R

struct AdjGrid {
  int n[3];       // cells along model x, y, z
  double lo[3];   // domain corner (model coordinates)
  double d[3];    // cell size
  int64_t nnode;  // (n0+1)(n1+1)(n2+1)
  double eps2;    // velocity floor squared
};

// What the walk needs from a tracker handle.
struct AdjInputs {
  GridDims g;
  Geometry geo;
  CellBase base;             // face flows Q1..Q6 per cell
  const int32_t *iboundts;   // cell active flags
  const double *dm;          // Dm per cell, or one value
  int dm_uniform;
  double R;                  // retardation (uniform)
  double lo[3], d[3];        // domain corner and cell sizes (uniform grid)
  int64_t n;                 // particles
  const int32_t *cell, *status;
  const void *x, *y, *z;
  int mixed;
  const double *mass;        // may be null: unit mass
  const uint64_t *id;        // may be null: index
};

struct AdjOptions {
  int nzones;
  double dt, eps;
  int nsteps, checkpoint;
  uint64_t seed;
  double origin[3], bin[3], h[3];
  int nb[3];
};

struct AdjState {
  AdjGrid G{};
  AdjOptions o{};
  double R = 1.0;
  int64_t np = 0;              // particles (those not ACTIVE or PENDING at set-up carry zero mass)
  double mass_total = 0.0;
  // node data fixed per set-up: Darcy flux (3 per node), zone shares (nzones per node), Dm / R
  double *d_q = nullptr, *d_beta = nullptr, *d_dmr = nullptr;
  // per theta
  double *d_theta = nullptr;   // 3 nz + 1
  double *d_phi = nullptr, *d_phid = nullptr, *d_nodes = nullptr;  // phi, phi D (6), node records
  // particles
  double *d_ckpt = nullptr;    // (nseg + 1) * 3 * np positions, SoA per checkpoint
  double *d_seg = nullptr;     // checkpoint * 3 * np positions of one segment
  double *d_mass = nullptr;
  uint64_t *d_id = nullptr;
  double *d_lam = nullptr;     // 3 * np adjoint of the positions
  // adjoint accumulators
  double *d_nadj = nullptr;    // nnode * 8: u[3], g[3], alphaL, alphaT
  double *d_phidbar = nullptr; // nnode * 6
  double *d_phibar = nullptr;  // nnode
  double *d_part = nullptr;    // per-block partial sums of the theta gradient
  int part_blocks = 0;
  unsigned long long *d_dens = nullptr;  // fixed-point density accumulator
  double *d_densf = nullptr, *d_gdens = nullptr;
  int64_t ngrid = 0;
  bool forward_done = false;
  int64_t launches = 0;

  cudaError_t setup(const AdjInputs &in, const AdjOptions &opt, const int32_t *zones_host, std::vector<char> &err);
  cudaError_t forward(const double *theta_host, double *density_host, cudaStream_t s);
  cudaError_t backward(const double *gdens_host, double *grad_host, cudaStream_t s);
  void release();
};

}  // namespace mprw
