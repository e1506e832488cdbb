// prep.cu -- builds the per-cell records the step kernel reads.
//
// Stage 1 (one thread per cell): face connections from the IA/JA CSR, face
// flows Q1..Q6 with boundary flows, mass-boundary flags and GetDZRW
// (SetMassTransportDataUnstructured, ModpathCellData.f90:674-1098;
//  pr_GetDZRW :3208-3256; pr_VerifyDryCell :3161-3205).
// Stage 2 (one thread per cell): the 18-neighbour stencil, corner discharge,
// corner porosity, corner dispersion and the derived interpolation
// coefficients (pr_ComputeCornerVariables, TrackSubCell.F90:3667-4363;
// pr_CornerDispersionLinearIsotropic :2557-2691), the face velocities of
// FillMassSubCellDataBuffer (ModpathCellData.f90:2557-2564), the random-walk
// time step (TrackSubCell.F90:1376-1458) and the cell-entry checks of
// TrackCell (TrackCell.f90:405-497) and TrackSubCell (:866-935).
//
// This work is done once per flow time step instead of on every cell entry
// of every particle; its arithmetic follows the reference's order so the
// corner quantities are bit-identical to the reference's.
#include <cfloat>

#include "mprw_kernels.cuh"

namespace mprw {

__device__ __forceinline__ void klj(const GridDims &g, int n, int &k, int &i, int &j) {
  k = n / g.ncpl;
  int r = n - k * g.ncpl;
  i = r / g.ncol;
  j = r - i * g.ncol;
}

__global__ void prep_base_kernel(PrepInputs in, CellBase base, uint8_t *massb_out) {
  const GridDims g = in.g;
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.ncell) return;
  int k, i, j;
  klj(g, n, k, i, j);
  int conn[6] = {-1, -1, -1, -1, -1, -1};
  int64_t fidx[6] = {-1, -1, -1, -1, -1, -1};
  // rows of the 1-based CSR; the first entry is the diagonal
  int64_t beg = in.ia[n] - 1, end = in.ia[n + 1] - 1;
  for (int64_t p = beg + 1; p < end; ++p) {
    int m = in.ja[p] - 1;
    int km, im, jm;
    klj(g, m, km, im, jm);
    int face = -1;
    if (km == k && im == i && jm == j - 1) face = 0;
    else if (km == k && im == i && jm == j + 1) face = 1;
    else if (km == k && jm == j && im == i + 1) face = 2;
    else if (km == k && jm == j && im == i - 1) face = 3;
    else if (im == i && jm == j && km == k + 1) face = 4;
    else if (im == i && jm == j && km == k - 1) face = 5;
    if (face >= 0) {
      conn[face] = m;
      fidx[face] = p;
    }
  }
  double q[6];
  int sbc[6];
  uint8_t mb = 0;
  double src = in.source_flow ? in.source_flow[n] : 0.0;
  double snk = in.sink_flow ? in.sink_flow[n] : 0.0;
  for (int f = 0; f < 6; ++f) {
    q[f] = 0.0;
    sbc[f] = 1;
    int mbv;
    if (conn[f] >= 0) {
      sbc[f] = (in.iboundts[conn[f]] == 0) ? 1 : 0;
      mbv = in.icboundts ? in.icboundts[conn[f]] : 0;
      double fj = in.flowja[fidx[f]];
      q[f] = (f % 2 == 0) ? fj : -fj;
    } else {
      mbv = in.default_icbound;
    }
    if (mbv == 1) mb |= (uint8_t)(1u << f);
  }
  if (in.bflow) {
    for (int f = 0; f < 6; ++f) {
      double bf = in.bflow[6 * (int64_t)n + f];
      if (bf != 0.0) {
        if (sbc[f] > 0) {
          double flow = bf / sbc[f];
          if (conn[f] < 0 || in.iboundts[conn[f]] == 0) q[f] = (f % 2 == 0) ? flow : -flow;
        } else {
          if (bf > 0.0) src = src + bf;
          else snk = snk + bf;
        }
      }
    }
  }
  // GetDZRW
  double top = (n < g.ncpl) ? in.top[n] : in.botm[n - g.ncpl];
  double bot = in.botm[n];
  int ltype = in.celltype ? in.celltype[n] : 0;
  double head = in.heads ? in.heads[n] : 0.0;
  double dz = top - bot, dzc = top - bot;
  bool dry = false, pdry = false;
  bool anyflow = false;
  for (int f = 0; f < 6; ++f) anyflow |= (q[f] != 0.0);
  if (ltype == 1 && head < top) {
    dz = head - bot;
    pdry = true;
    if ((dz <= 0.0) || ((head - bot) / dzc < 0.01)) {
      dz = top - bot;
      dry = true;
      pdry = false;
      if (anyflow) {
        dry = false;
        pdry = true;
      }
    }
  }
  // VerifyDryCell's partiallyDry (used by the status-7 recheck, MPathRW.F90:1295-1302)
  bool vpdry = (ltype == 1 && head < top) && ((head - bot > 0.0) || anyflow);
  double sgn = in.backward ? -1.0 : 1.0;
  bool hasExit = (sgn * q[0] < 0.0) || (sgn * q[1] > 0.0) || (sgn * q[2] < 0.0) || (sgn * q[3] > 0.0) ||
                 (sgn * q[4] < 0.0) || (sgn * q[5] > 0.0);
  for (int f = 0; f < 6; ++f) {
    base.q[6 * (int64_t)n + f] = q[f];
    base.conn[6 * (int64_t)n + f] = conn[f];
  }
  base.dz[n] = dz;
  base.flags[n] = (uint8_t)((dry ? 1u : 0u) | (vpdry ? 2u : 0u) | (hasExit ? 4u : 0u) |
                            (snk != 0.0 ? 8u : 0u) | (src != 0.0 ? 16u : 0u) | (pdry ? 32u : 0u));
  massb_out[n] = mb;
}

// Monomial coefficients of the trilinear interpolant of corner values
// v[0..7] (corner index = ix + 2 iy + 4 iz).
__device__ __forceinline__ void monomials(const double v[8], double a[8]) {
  a[0] = v[0];
  a[1] = v[1] - v[0];
  a[2] = v[2] - v[0];
  a[3] = v[4] - v[0];
  a[4] = v[3] - v[1] - v[2] + v[0];
  a[5] = v[5] - v[1] - v[4] + v[0];
  a[6] = v[6] - v[2] - v[4] + v[0];
  a[7] = v[7] - v[3] - v[5] - v[6] + v[1] + v[2] + v[4] - v[0];
}

// sum of d/dx trilinear(A) + d/dy trilinear(B) + d/dz trilinear(C), scaled
__device__ __forceinline__ void divergence_coeffs(const double A[8], const double B[8], const double C[8],
                                                  double DX, double DY, double DZ, double scale,
                                                  double out[7]) {
  double a[8], b[8], c[8];
  monomials(A, a);
  monomials(B, b);
  monomials(C, c);
  out[0] = (a[1] / DX + b[2] / DY + c[3] / DZ) * scale;
  out[1] = (b[4] / DY + c[5] / DZ) * scale;  // x
  out[2] = (a[4] / DX + c[6] / DZ) * scale;  // y
  out[3] = (a[5] / DX + b[6] / DY) * scale;  // z
  out[4] = (c[7] / DZ) * scale;              // xy
  out[5] = (b[7] / DY) * scale;              // xz
  out[6] = (a[7] / DX) * scale;              // yz
}

// corner-component neighbour tables (TrackSubCell.F90:4142-4224, 4329-4363), 1-based
__constant__ int8_t kCXI[8][4] = {{7, 8, 13, 1}, {7, 8, 13, 2}, {10, 11, 13, 1}, {10, 11, 13, 2},
                                  {7, 9, 16, 1}, {7, 9, 16, 2}, {10, 12, 16, 1}, {10, 12, 16, 2}};
__constant__ int8_t kCYI[8][4] = {{1, 13, 14, 3}, {4, 13, 15, 3}, {1, 13, 14, 4}, {4, 13, 15, 4},
                                  {1, 16, 17, 3}, {4, 16, 18, 3}, {1, 16, 17, 4}, {4, 16, 18, 4}};
__constant__ int8_t kCZI[8][4] = {{1, 2, 7, 5}, {4, 5, 7, 5}, {1, 3, 10, 5}, {4, 6, 10, 5},
                                  {1, 2, 7, 6}, {4, 5, 7, 6}, {1, 3, 10, 6}, {4, 6, 10, 6}};
__constant__ int8_t kCPI[8][6] = {{1, 2, 7, 8, 13, 14},   {4, 5, 7, 8, 13, 15},  {1, 3, 10, 11, 13, 14},
                                  {4, 6, 10, 12, 16, 18}, {1, 2, 7, 9, 16, 17},  {4, 5, 7, 9, 16, 18},
                                  {1, 3, 10, 12, 16, 17}, {4, 6, 10, 11, 13, 15}};
// second-level neighbours of the six direct neighbours (ParticleTrackingEngine.f90:2033-2115)
__constant__ int8_t kSub[6][2] = {{2, 3}, {2, 3}, {4, 5}, {4, 5}, {0, 1}, {0, 1}};

template <typename R>
__device__ void store_record(CellRec<R> *dst, const double v1[3], const double v2[3], const double d[3],
                             const double div[3][7], const double vb[3][8], double aL, double aT, double aLV,
                             double aTV, double dm, double tr, double dtcell, const int32_t conn[6], int32_t es,
                             uint32_t mb) {
  CellRec<R> r;
  for (int m = 0; m < 3; ++m) {
    r.v1[m] = (R)v1[m];
    r.dv[m] = (R)(v2[m] - v1[m]);
    r.d[m] = (R)d[m];
    r.inv_d[m] = (R)(1.0 / d[m]);
    r.v2[m] = (R)v2[m];
    for (int q = 0; q < 7; ++q) r.div[m][q] = (R)div[m][q];
    for (int q = 0; q < 8; ++q) r.vb[m][q] = (R)vb[m][q];
  }
  r.aL = (R)aL;
  r.aT = (R)aT;
  r.aLV = (R)aLV;
  r.aTV = (R)aTV;
  r.dm = (R)dm;
  r.two_over_r = (R)tr;
  r.dtcell = dtcell;
  r.sqrt_dtcell = sqrt(dtcell);
  for (int f = 0; f < 6; ++f) r.conn[f] = conn[f];
  r.entry_status = es;
  r.massb = mb;
  *dst = r;
}

__global__ void prep_rec_kernel(PrepInputs in, CellBase base, const uint8_t *massb, CellRec<double> *rec64,
                                CellRec<float> *rec32) {
  const GridDims g = in.g;
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.ncell) return;
  int k, i, j;
  klj(g, n, k, i, j);
  const double DX = in.delr[j] / 1.0, DY = in.delc[i] / 1.0, DZ = base.dz[n];
  const double phi = in.porosity[n], R = in.retardation[n];
  const double *Q = base.q + 6 * (int64_t)n;
  const uint8_t fl = base.flags[n];
  const bool dry = fl & 1u;
  double sign = 1.0;
  if (in.backward) sign = -sign;
  // FillMassSubCellDataBuffer face velocities (ModpathCellData.f90:2559-2564)
  double v[6];
  v[0] = sign * Q[0] / DY / DZ / phi / R;
  v[1] = sign * Q[1] / DY / DZ / phi / R;
  v[2] = sign * Q[2] / DX / DZ / phi / R;
  v[3] = sign * Q[3] / DX / DZ / phi / R;
  v[4] = sign * Q[4] / DX / DY / phi / R;
  v[5] = sign * Q[5] / DX / DY / phi / R;
  int di = in.uniform_dispersion ? 0 : n;
  double aL = in.alpha_l[di], aT = in.alpha_t[di], dm = in.dm_eff[di];
  double aLV = in.alpha_lv ? in.alpha_lv[di] : aL, aTV = in.alpha_tv ? in.alpha_tv[di] : aT;
  // ComputeRandomWalkTimeStep
  double mx = fmax(fabs(v[0]), fabs(v[1])), my = fmax(fabs(v[2]), fabs(v[3])), mz = fmax(fabs(v[4]), fabs(v[5]));
  double dtcell = 0.0;
  {
    double adv = in.ts_param0 / (mx / DX + my / DY + mz / DZ);
    double dsp = in.ts_param1 / (aL * mx / (DX * DX) + aT * my / (DY * DY) + aT * mz / (DZ * DZ));
    switch (in.time_step_kind) {
      case 1: dtcell = adv; break;
      case 2: dtcell = in.ts_param1 / (aL * mx / (DX * DX) + aT * my / (DY * DY) + aT * mz / (DZ * DZ)); break;
      case 3: {
        double t = DBL_MAX;
        if (adv > 0.0 && adv < t) t = adv;
        if (dsp > 0.0 && dsp < t) t = dsp;
        dtcell = t;
        break;
      }
      case 4: dtcell = in.ts_param0; break;
    }
  }
  // 18-neighbour stencil
  int nb[18];
  for (int f = 0; f < 6; ++f) {
    int d0 = base.conn[6 * (int64_t)n + f];
    nb[3 * f] = d0;
    nb[3 * f + 1] = (d0 >= 0) ? base.conn[6 * (int64_t)d0 + kSub[f][0]] : -1;
    nb[3 * f + 2] = (d0 >= 0) ? base.conn[6 * (int64_t)d0 + kSub[f][1]] : -1;
  }
  double narea[18][3], nvol[18], nphi[18];
  for (int q = 0; q < 18; ++q) {
    narea[q][0] = narea[q][1] = narea[q][2] = 0.0;
    nvol[q] = 0.0;
    nphi[q] = 0.0;
    int m = nb[q];
    if (m < 0) continue;
    int km, im, jm;
    klj(g, m, km, im, jm);
    double mdx = in.delr[jm], mdy = in.delc[im], mdz = base.dz[m];
    narea[q][0] = mdy * mdz;
    narea[q][1] = mdx * mdz;
    narea[q][2] = mdx * mdy;
    nvol[q] = mdx * mdy * mdz;
    nphi[q] = in.porosity[m];
  }
  auto nflow = [&](int q1, int face1) -> double {
    int m = nb[q1 - 1];
    return (m < 0) ? 0.0 : base.q[6 * (int64_t)m + face1 - 1];
  };
  double qc[8][4];
  for (int c = 0; c < 8; ++c) {
    double sa = DY * DZ, sf = Q[kCXI[c][3] - 1];
    for (int m = 0; m < 3; ++m) {
      sa = sa + narea[kCXI[c][m] - 1][0];
      sf = sf + nflow(kCXI[c][m], kCXI[c][3]);
    }
    qc[c][0] = sf / sa;
    sa = DX * DZ;
    sf = Q[kCYI[c][3] - 1];
    for (int m = 0; m < 3; ++m) {
      sa = sa + narea[kCYI[c][m] - 1][1];
      sf = sf + nflow(kCYI[c][m], kCYI[c][3]);
    }
    qc[c][1] = sf / sa;
    sa = DX * DY;
    sf = Q[kCZI[c][3] - 1];
    for (int m = 0; m < 3; ++m) {
      sa = sa + narea[kCZI[c][m] - 1][2];
      sf = sf + nflow(kCZI[c][m], kCZI[c][3]);
    }
    qc[c][2] = sf / sa;
    qc[c][3] = sqrt(qc[c][0] * qc[c][0] + qc[c][1] * qc[c][1] + qc[c][2] * qc[c][2]);
  }
  double phic[8];
  for (int c = 0; c < 8; ++c) {
    if (in.uniform_porosity) {
      phic[c] = phi;
    } else {
      double sv = DX * DY * DZ, sw = phi * sv;
      for (int m = 0; m < 6; ++m) {
        int q = kCPI[c][m] - 1;
        sv = sv + nvol[q];
        sw = sw + nvol[q] * nphi[q];
      }
      phic[c] = sw / sv;
    }
  }
  // qprod and isotropic corner dispersion (quirk: corners 3..8 use |q| of corner 100)
  double D[9][8];
  const double aLmT = aL - aT;
  for (int c = 0; c < 8; ++c) {
    double qp[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (qc[c][3] > 0.0) {
      qp[0] = qc[c][0] * qc[c][0];
      qp[1] = qc[c][0] * qc[c][1];
      qp[2] = qc[c][0] * qc[c][2];
      qp[3] = qc[c][1] * qc[c][1];
      qp[4] = qc[c][1] * qc[c][2];
      qp[5] = qc[c][2] * qc[c][2];
      qp[6] = qp[0] + qp[3];
      for (int m = 0; m < 7; ++m) qp[m] = qp[m] / qc[c][3];
    }
    if (in.dispersion_model == 1) {
      // pr_CornerDispersionAxisymmetric (TrackSubCell.F90:3117-3303): per
      // corner alphaL/alphaT blended with cosinesq = qz**2/|q| (as written),
      // Dxyx from the xx product (as written)
      if (qc[c][3] > 0.0 && qp[6] > 0.0) qp[7] = (qc[c][2] * qc[c][2]) / (qc[c][0] * qc[c][0] + qc[c][1] * qc[c][1]);
      const double pD = phic[c] * dm;
      double cosinesq = 0.0;
      if (qc[c][3] > 0.0) cosinesq = qc[c][2] * qc[c][2] / qc[c][3];
      const double aLc = aL + cosinesq * (aLV - aL);
      const double aTc = aTV + cosinesq * (aT - aTV);
      const double aLmTc = aLc - aTc;
      D[0][c] = pD + (aLc + aTc * qp[7]) * qp[0] + aT * qp[3] * (1.0 + qp[7]);
      D[1][c] = pD + aT * qp[0] * (1.0 + qp[7]) + qp[3] * (aLc + aTc * qp[7]);
      D[3][c] = (aLc - aT * (1.0 + qp[7]) + aTc * qp[7]) * qp[0];
      D[5][c] = D[3][c];
      D[2][c] = pD + aTc * qp[6] + aLc * qp[5];
      D[4][c] = aLmTc * qp[2];
      D[6][c] = aLmTc * qp[4];
      D[7][c] = D[4][c];
      D[8][c] = D[6][c];
      continue;
    }
    double qn = (c == 0) ? qc[0][3] : qc[1][3];
    double aTQ = aT * qn + phic[c] * dm;
    D[0][c] = aTQ + aLmT * qp[0];
    D[1][c] = aTQ + aLmT * qp[3];
    D[2][c] = aTQ + aLmT * qp[5];
    D[3][c] = aLmT * qp[1];
    D[4][c] = aLmT * qp[2];
    D[5][c] = D[3][c];
    D[6][c] = aLmT * qp[4];
    D[7][c] = D[4][c];
    D[8][c] = D[6][c];
  }
  // divergence coefficients, (sum)/porosity/retardation folded into one scale
  double scale = 1.0 / (phi * R);
  double div[3][7];
  divergence_coeffs(D[0], D[5], D[7], DX, DY, DZ, scale, div[0]);  // Dxxx, Dxyy, Dxzz
  divergence_coeffs(D[3], D[1], D[8], DX, DY, DZ, scale, div[1]);  // Dxyx, Dyyy, Dyzz
  divergence_coeffs(D[4], D[6], D[2], DX, DY, DZ, scale, div[2]);  // Dxzx, Dyzy, Dzzz
  // corner velocities for the displacement matrix (TrackSubCell.F90:2869-2876)
  double vb[3][8];
  for (int m = 0; m < 3; ++m) {
    double cv[8];
    for (int c = 0; c < 8; ++c) cv[c] = qc[c][m] / phic[c];
    monomials(cv, vb[m]);
  }
  // entry checks
  int32_t es = 0;
  const bool hasExitQ = fl & 4u, sinkNZ = fl & 8u, srcNZ = fl & 16u;
  int zone = in.zones ? in.zones[n] : 0;
  if (in.iboundts[n] == 0) es = ST_INACTIVE;
  else if (in.stop_zone > 0 && zone == in.stop_zone) es = ST_STOP_ZONE;
  bool stopIfNoExit = true;
  if (es == 0) {
    if (in.backward) {
      if (in.stop_weak_sources) {
        if (srcNZ) es = ST_WEAK_SOURCE;
        else if (!in.steady_state) stopIfNoExit = false;
      }
    } else {
      if (in.stop_weak_sinks) {
        if (sinkNZ) es = ST_WEAK_SINK;
        else if (!in.steady_state) stopIfNoExit = false;
      }
    }
  }
  if (es == 0 && !hasExitQ) {
    if (in.steady_state) es = ST_NO_EXIT;
    else if (in.backward && srcNZ) es = ST_NO_EXIT;
    else if (!in.backward && sinkNZ) es = ST_NO_EXIT;
  }
  if (es == 0 && stopIfNoExit) {
    bool sub = (v[0] < 0.0) || (v[1] > 0.0) || (v[2] < 0.0) || (v[3] > 0.0) || (v[4] < 0.0) || (v[5] > 0.0);
    if (!sub) es = ST_NO_EXIT;
  }
  if (es == 0 && dry) es = ST_INACTIVE;
  if (es == 0 && !(dtcell > 0.0 && dtcell <= DBL_MAX)) es = ST_UNDEFINED;
  int32_t conn[6];
  for (int f = 0; f < 6; ++f) {
    int m = base.conn[6 * (int64_t)n + f];
    conn[f] = (m >= 0 && in.iboundts[m] != 0) ? m : -1;
  }
  double v1[3] = {v[0], v[2], v[4]}, v2[3] = {v[1], v[3], v[5]}, d[3] = {DX, DY, DZ};
  double tr = 2.0 / R;
  if (rec64)
    store_record<double>(rec64 + n, v1, v2, d, div, vb, aL, aT, aLV, aTV, dm, tr, dtcell, conn, es, massb[n]);
  if (rec32)
    store_record<float>(rec32 + n, v1, v2, d, div, vb, aL, aT, aLV, aTV, dm, tr, dtcell, conn, es, massb[n]);
}

cudaError_t launch_prep(const PrepInputs &in, CellBase base, uint8_t *massb, CellRec<double> *rec64,
                        CellRec<float> *rec32, cudaStream_t s) {
  int threads = 128;
  int blocks = (in.g.ncell + threads - 1) / threads;
  prep_base_kernel<<<blocks, threads, 0, s>>>(in, base, massb);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  prep_rec_kernel<<<blocks, threads, 0, s>>>(in, base, massb, rec64, rec32);
  return cudaGetLastError();
}

}  // namespace mprw
