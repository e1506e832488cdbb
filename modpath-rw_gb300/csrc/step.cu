// step.cu -- the random-walk particle-tracking step kernel.
//
// One persistent kernel advances every particle to the end of the tracking
// interval.  Each lane runs a flat state machine, one time-loop pass per
// iteration of its main loop:
//   fetch particle -> release checks -> enter cell (stage the cell record in
//   shared memory, entry checks) -> time-loop passes -> exit / stop / store
// so lanes of a warp stay on the common step body no matter which particle,
// cell or phase each one is in.  Particles are taken from an atomic queue in
// cell-sorted order (perm[]), which keeps the records a warp reads in cache.
//
// Per-pass logic restates pr_ExecuteRandomWalkParticleTracking
// (TrackSubCell.F90:812-1373) with the quadratic exit-face solver of the
// EULERIAN advection model (TrackSubCell.F90:1576-1892); the cell-to-cell
// logic restates pr_RWPTrackPath (ParticleTrackingEngine.f90:1051-1254),
// TrackCell (TrackCell.f90:375-669) and ConvertFromNeighbor
// (RectangularGridDisMf6.f90:50-108).  Interpolants are evaluated from the
// monomial coefficients the prep kernel stores, with fused multiply-adds.
#include "mprw_common.cuh"
#include "mprw_kernels.cuh"

namespace mprw {

// Shared-memory view of one lane's record: field f at sm[f*stride + lane],
// conflict-free for a warp reading the same field.
enum : int {
  F_V1 = 0, F_DV = 3, F_D = 6, F_INVD = 9, F_DIV = 12, F_VB = 33,
  F_AL = 57, F_AT = 58, F_DM = 59, F_2R = 60, F_V2 = 61, F_ALV = 64, F_ATV = 65, NFIELDS = 66
};

template <typename R>
struct Lane {
  R *p;
  int stride;
  __device__ __forceinline__ R operator()(int f) const { return p[f * stride]; }
};

// Tests against the constants 0, 1/2 and 1 and the time compares: native in
// the FP32 kernel, from the IEEE-754 bit patterns in the FP64 kernel (the
// same decisions for every input; fpbits.cuh).  Where a site reads
// `sizeof(R) == 8 ? <bit-pattern form> : <compare>`, the FP32 kernel keeps
// its compare written as before: it is latency-bound at 80 registers, and
// every reshaping of its compares measured slower.
template <typename R>
__device__ __forceinline__ bool above1(R v) { return v > R(1); }
template <>
__device__ __forceinline__ bool above1<double>(double v) { return fb::above1(v); }
template <typename R>
__device__ __forceinline__ bool below0(R v) { return v < R(0); }
template <>
__device__ __forceinline__ bool below0<double>(double v) { return fb::below0(v); }
template <typename R>
__device__ __forceinline__ bool above0(R v) { return v > R(0); }
template <>
__device__ __forceinline__ bool above0<double>(double v) { return fb::above0(v); }
template <typename R>
__device__ __forceinline__ bool is0(R v) { return v == R(0); }
template <>
__device__ __forceinline__ bool is0<double>(double v) { return fb::is0(v); }
template <typename R>
__device__ __forceinline__ bool nonneg(R v) { return v >= R(0); }
template <>
__device__ __forceinline__ bool nonneg<double>(double v) { return fb::nonneg(v); }
template <typename R>
__device__ __forceinline__ bool abs_above_half(R v) { return fabs(v) > R(0.5); }
template <>
__device__ __forceinline__ bool abs_above_half<double>(double v) { return fb::abs_above_half(v); }
template <typename R>
__device__ __forceinline__ bool out01(R v) { return v > R(1) || v < R(0); }
template <>
__device__ __forceinline__ bool out01<double>(double v) { return fb::out01(v); }
template <typename R>
__device__ __forceinline__ bool is1(R v) { return v == R(1); }
template <>
__device__ __forceinline__ bool is1<double>(double v) { return fb::is1(v); }
// a < b for a, b > 0 (not NaN)
template <typename R>
__device__ __forceinline__ bool pos_lt(R a, R b) { return a < b; }
template <>
__device__ __forceinline__ bool pos_lt<double>(double a, double b) { return fb::pos_lt(a, b); }
using fb::eq_any;
using fb::lt_any;
using fb::past_end;

// The staged fields are the record's first NFIELDS values and records are
// 16-byte aligned, so they are read with 16-byte loads (FP32: 16 float4 and
// one float2; FP64: 33 double2) and scattered to the lane's SoA slots.
static_assert(NFIELDS == 66, "stage_record reads 66 leading fields");
template <typename R>
__device__ __forceinline__ void stage_record(const CellRec<R> *__restrict__ recs, int32_t c, R *sm, int stride);

template <>
__device__ __forceinline__ void stage_record<float>(const CellRec<float> *__restrict__ recs, int32_t c, float *sm,
                                                    int stride) {
  const float4 *src = reinterpret_cast<const float4 *>(recs + c);
#pragma unroll 4
  for (int q = 0; q < 16; ++q) {
    const float4 v = __ldg(src + q);
    sm[(4 * q + 0) * stride] = v.x;
    sm[(4 * q + 1) * stride] = v.y;
    sm[(4 * q + 2) * stride] = v.z;
    sm[(4 * q + 3) * stride] = v.w;
  }
  const float2 t = __ldg(reinterpret_cast<const float2 *>(src + 16));
  sm[64 * stride] = t.x;
  sm[65 * stride] = t.y;
}

template <>
__device__ __forceinline__ void stage_record<double>(const CellRec<double> *__restrict__ recs, int32_t c,
                                                     double *sm, int stride) {
  const double2 *src = reinterpret_cast<const double2 *>(recs + c);
#pragma unroll 4
  for (int q = 0; q < 33; ++q) {
    const double2 v = __ldg(src + q);
    sm[(2 * q + 0) * stride] = v.x;
    sm[(2 * q + 1) * stride] = v.y;
  }
}

template <typename R>
__device__ __forceinline__ R tril(const Lane<R> &F, int base, R x, R y, R z, R xy, R xz, R yz, R xyz) {
  R a = F(base + 0);
  a = fma(F(base + 1), x, a);
  a = fma(F(base + 2), y, a);
  a = fma(F(base + 3), z, a);
  a = fma(F(base + 4), xy, a);
  a = fma(F(base + 5), xz, a);
  a = fma(F(base + 6), yz, a);
  a = fma(F(base + 7), xyz, a);
  return a;
}

template <typename R>
__device__ __forceinline__ R divc(const Lane<R> &F, int base, R x, R y, R z, R xy, R xz, R yz) {
  R a = F(base + 0);
  a = fma(F(base + 1), x, a);
  a = fma(F(base + 2), y, a);
  a = fma(F(base + 3), z, a);
  a = fma(F(base + 4), xy, a);
  a = fma(F(base + 5), xz, a);
  a = fma(F(base + 6), yz, a);
  return a;
}

// The step's standard normals, the reference's Irwin-Hall(12) distribution
// in both paths, from the same 3 Philox blocks per normal: FP64 exact, MIXED
// rounded to FP32 (the two precisions share their random numbers).
template <typename R>
struct Normals;
template <>
struct Normals<double> {
  __device__ __forceinline__ static void draw(int ndim, uint64_t seed, uint64_t id, uint64_t &ctr, double &r0,
                                              double &r1, double &r2) {
    r0 = normal_ih12(seed, id, ctr);
    r1 = (ndim > 1) ? normal_ih12(seed, id, ctr) : 0.0;
    r2 = (ndim > 2) ? normal_ih12(seed, id, ctr) : 0.0;
  }
};
template <>
struct Normals<float> {
  __device__ __forceinline__ static void draw(int ndim, uint64_t seed, uint64_t id, uint64_t &ctr, float &r0,
                                              float &r1, float &r2) {
    r0 = normal_ih12_f32(seed, id, ctr);
    r1 = (ndim > 1) ? normal_ih12_f32(seed, id, ctr) : 0.0f;
    r2 = (ndim > 2) ? normal_ih12_f32(seed, id, ctr) : 0.0f;
  }
};

// pr_DisplacementRandomDischarge (3-D :2821-2928, 2-D :2931-3028, 1-D :3031-3113).
// AXI (linear axisymmetric model): alphaL, alphaT are blended with the
// particle's velocity (vpx, vpy, vpz) as pr_RWPTDisplacementsAxisymmetric
// does (:750-806, cosinesq = vz**2/|v| as written), and the horizontal
// transverse terms use alphaTH (pr_DisplacementRandomDischargeAxisymmetric
// {,2D,1D}, :3306-3604).
template <typename R, bool AXI>
__device__ __forceinline__ void random_displacement(const Lane<R> &F, int ndim, int d1, int d2, R x, R y,
                                                    R z, R vpx, R vpy, R vpz, uint64_t seed, uint64_t id,
                                                    uint64_t &ctr, R &bx, R &by, R &bz) {
  const R zero = R(0);
  R xy = x * y, xz = x * z, yz = y * z, xyz = xy * z;
  R aL = F(F_AL), aT = F(F_AT), dm = F(F_DM), tr = F(F_2R);
  R aTH = aT;
  if constexpr (AXI) {
    const R vnorm = sqrt(vpx * vpx + vpy * vpy + vpz * vpz);
    R cosinesq = zero;
    if (vnorm > zero) cosinesq = vpz * vpz / vnorm;
    aL = aL + cosinesq * (F(F_ALV) - aL);
    aT = F(F_ATV) + cosinesq * (aTH - F(F_ATV));
  }
  if (ndim == 3) {
    R vx = tril(F, F_VB + 0, x, y, z, xy, xz, yz, xyz);
    R vy = tril(F, F_VB + 8, x, y, z, xy, xz, yz, xyz);
    R vz = tril(F, F_VB + 16, x, y, z, xy, xz, yz, xyz);
    R nxy2 = fma(vx, vx, vy * vy);
    R n2 = fma(vz, vz, nxy2);
    R B11 = zero, B12 = zero, B13 = zero, B21 = zero, B22 = zero, B23 = zero, B31 = zero, B32 = zero;
    if (sizeof(R) == 8 ? above0(n2) : n2 > zero) {
      R inv = rsqrt(n2);
      R nrm = n2 * inv;
      R sL = sqrt(tr * fma(aL, nrm, dm));
      R sT = sqrt(tr * fma(aT, nrm, dm));
      R sTH = AXI ? sqrt(tr * fma(aTH, nrm, dm)) : sT;
      R sLi = sL * inv;
      B11 = vx * sLi;
      B21 = vy * sLi;
      B31 = vz * sLi;
      if (sizeof(R) == 8 ? above0(nxy2) : nxy2 > zero) {
        R invxy = rsqrt(nxy2);
        R nxy = nxy2 * invxy;
        R sTi = sT * inv;
        B32 = nxy * sTi;
        R sTixy = sTi * invxy;
        B12 = -(vx * vz) * sTixy;
        B22 = -(vy * vz) * sTixy;
        R sTxy = sTH * invxy;
        B13 = -vy * sTxy;
        B23 = vx * sTxy;
      }
    }
    R rx, ry, rz;
    Normals<R>::draw(3, seed, id, ctr, rx, ry, rz);
    bx = fma(B13, rz, fma(B12, ry, B11 * rx));
    by = fma(B23, rz, fma(B22, ry, B21 * rx));
    bz = fma(B32, ry, B31 * rx);
  } else if (ndim == 2) {
    R v1 = tril(F, F_VB + 8 * d1, x, y, z, xy, xz, yz, xyz);
    R v2 = tril(F, F_VB + 8 * d2, x, y, z, xy, xz, yz, xyz);
    R n2 = fma(v1, v1, v2 * v2);
    R B11 = zero, B12 = zero, B21 = zero, B22 = zero;
    if (n2 > zero) {
      R inv = rsqrt(n2);
      R nrm = n2 * inv;
      R sLi = sqrt(tr * fma(aL, nrm, dm)) * inv;
      R sTi = sqrt(tr * fma(aTH, nrm, dm)) * inv;
      B11 = v1 * sLi;
      B21 = v2 * sLi;
      B12 = -v2 * sTi;
      B22 = v1 * sTi;
    }
    R r1, r2, r3;
    Normals<R>::draw(2, seed, id, ctr, r1, r2, r3);
    R o1 = fma(B12, r2, B11 * r1), o2 = fma(B22, r2, B21 * r1);
    bx = zero; by = zero; bz = zero;
    if (d1 == 0) bx = o1; else if (d1 == 1) by = o1; else bz = o1;
    if (d2 == 0) bx = o2; else if (d2 == 1) by = o2; else bz = o2;
  } else {
    R v1 = tril(F, F_VB + 8 * d1, x, y, z, xy, xz, yz, xyz);
    R nrm = fabs(v1);
    R B11 = zero;
    if (nrm > zero) B11 = sqrt(tr * fma(aL, nrm, dm));
    R r1, r2, r3;
    Normals<R>::draw(1, seed, id, ctr, r1, r2, r3);
    bx = zero; by = zero; bz = zero;
    R o1 = B11 * r1;
    if (d1 == 0) bx = o1; else if (d1 == 1) by = o1; else bz = o1;
  }
}

// One axis of pr_DetectExitFaceAndUpdateTimeStepQuadratic (:1622-1710).
// Returns true when the routine must return at once (exitFace, dt set).
// The step length dt comes in the type T of its comparison: FP64 compares in
// double as the reference; MIXED passes the FP32 copy of dt (no FP64 op).
template <typename R, typename T>
__device__ __forceinline__ bool quad_axis(R npos, R pos, R d, R v, R divD, R dB, int faceLo, int faceHi,
                                          T dt, R &dtaxis, int &exitAxis, int &exitFace,
                                          double &dtout) {
  const R zero = R(0), one = R(1);
  R dI;
  if (npos > one) {
    dI = d * (one - pos);
    exitAxis = faceHi;
  } else {
    dI = -d * pos;
    exitAxis = faceLo;
  }
  if (dI == zero) {
    exitFace = exitAxis;
    dtout = 0.0;
    return true;
  }
  R A = v + divD, B = dB;
  R arg = B * B + R(4) * dI * A;
  if ((arg >= zero) && (A != zero)) {
    R zs = sqrt(arg);
    R z1, z2;
    if constexpr (sizeof(R) == 4) {
      // the same two roots without cancellation: q = -(B + sign(B) sqrt(arg))/2,
      // roots q/A and -dI/q
      R q = (B >= zero) ? -(B + zs) * R(0.5) : (zs - B) * R(0.5);
      z1 = q / A;
      z2 = (q != zero) ? -dI / q : zero;
    } else {
      z1 = (-B + zs) / (R(2) * A);
      z2 = (-B - zs) / (R(2) * A);
    }
    if (z1 > zero || z2 > zero) {
      R zm = (z1 > zero && z2 > zero) ? (z1 < z2 ? z1 : z2) : (z1 > zero ? z1 : z2);
      dtaxis = zm * zm;
      if (dtaxis == zero) {
        exitFace = exitAxis;
        dtout = 0.0;
        return true;
      }
    } else if (z1 == zero || z2 == zero) {
      exitFace = exitAxis;
      dtout = 0.0;
      return true;
    }
  } else if (A == zero) {
    if (B != zero) {
      R q = dI / B;
      dtaxis = q * q;
      if (dtaxis == zero) {
        exitFace = exitAxis;
        dtout = 0.0;
        return true;
      }
    }
  }
  if ((T)dtaxis > dt) dtaxis = zero;
  return false;
}

// quad_axis in FP64 with its tests against 0 and 1 and its step compare on
// the integer pipe (the same decisions, see above).
__device__ __forceinline__ bool quad_axis_f64(double npos, double pos, double d, double v, double divD, double dB,
                                              int faceLo, int faceHi, double dt, double &dtaxis, int &exitAxis,
                                              int &exitFace, double &dtout) {
  using R = double;
  const R zero = R(0), one = R(1);
  R dI;
  if (above1(npos)) {
    dI = d * (one - pos);
    exitAxis = faceHi;
  } else {
    dI = -d * pos;
    exitAxis = faceLo;
  }
  if (is0(dI)) {
    exitFace = exitAxis;
    dtout = 0.0;
    return true;
  }
  R A = v + divD, B = dB;
  R arg = B * B + R(4) * dI * A;
  if (nonneg(arg) && !is0(A)) {
    R zs = sqrt(arg);
    R z1, z2;
    z1 = (-B + zs) / (R(2) * A);
    z2 = (-B - zs) / (R(2) * A);
    const bool p1 = above0(z1), p2 = above0(z2);
    if (p1 || p2) {
      R zm = (p1 && p2) ? (pos_lt(z1, z2) ? z1 : z2) : (p1 ? z1 : z2);
      dtaxis = zm * zm;
      if (is0(dtaxis)) {
        exitFace = exitAxis;
        dtout = 0.0;
        return true;
      }
    } else if (is0(z1) || is0(z2)) {
      exitFace = exitAxis;
      dtout = 0.0;
      return true;
    }
  } else if (is0(A)) {
    if (!is0(B)) {
      R q = dI / B;
      dtaxis = q * q;
      if (is0(dtaxis)) {
        exitFace = exitAxis;
        dtout = 0.0;
        return true;
      }
    }
  }
  if (lt_any(dt, dtaxis)) dtaxis = zero;
  return false;
}

// ---- EXPONENTIAL advection (TrackSubCell.F90:1487-1538) and its exit time by
// Newton-Raphson (:1895-2554).  Both run in FP64 whatever the particle
// precision: the displacement v (e^{dv dt} - 1)/dv and the exit-time solve
// lose their digits to cancellation at small velocity gradients.
__device__ __forceinline__ double adv_exponential(double v, double dvdx, double dt) {
  const double dvtol = 1.0e-10;
  return (fabs(dvdx) > dvtol) ? v * (exp(dvdx * dt) - 1.0) / dvdx : v * dt;
}

// pr_NewtonRaphsonVariablesExponentialAdvection (:2082-2120)
__device__ void nr_vars(double dt, double v, double dvdx, double dI, double divD, double dB, double &f0, double &f1,
                        double &f2, double &f3) {
  if (dt == 0.0) return;
  f0 = adv_exponential(v, dvdx, dt) + divD * dt + dB * sqrt(dt) - dI;
  const double e = exp(dvdx * dt);
  f1 = v * e + divD + 0.5 * dB / sqrt(dt);
  f2 = dvdx * v * e - 0.25 * dB * pow(dt, -1.5);
  f3 = dvdx * dvdx * v * e + 0.375 * dB * pow(dt, -2.5);
}
__device__ __forceinline__ double nr_conv_g(double f0, double f1, double f2) { return fabs(f2 * f0 / (f1 * f1)); }
__device__ __forceinline__ double nr_conv_gder(double f0, double f1, double f2, double f3) {
  const double gna = f2 * f0 / (f1 * f1);
  const double gpp = -2.0 * (f0 * (f2 * f2)) / (f1 * f1 * f1) + (f1 * f2 + f0 * f3) / (f1 * f1);
  return gna / fabs(gna) * gpp;
}
__device__ __forceinline__ double nr_p10(int e) {  // 10d0**e, exact for |e| <= 22
  double r = 1.0;
  for (int i = 0; i < (e < 0 ? -e : e); ++i) r *= 10.0;
  return e < 0 ? 1.0 / r : r;
}

// pr_SetInitialGuess (:2162-2448); every loop is bounded (7, 50 and 8 passes)
__device__ double nr_initial_guess(double dt, double v, double dvdx, double dI, double divD, double dB) {
  const double gdtol = (double)1e-6f;
  const int maxter = 50;
  double f0 = 0, f1 = 0, f2 = 0, f3 = 0;
  double dtnew = 0.0, dtold, dt0, gprimdernew, gprimnew, gprimder, gprim, gprimmin, gamman;
  double dtfraction = 0, dtoldfraction, mindtfrac = 0;
  int counter, ccount, bcount, zcount, rcount, gcount;
  if (dt == 0.0) return dtnew;
  gprimmin = (double)1e10f;
  gprim = (double)1e10f;
  gcount = 0;
  while ((gprim > 1) && (gcount < 7)) {
    gcount = gcount + 1;
    dtfraction = nr_p10(-8 + gcount);
    dt0 = dt * dtfraction;
    nr_vars(dt0, v, dvdx, dI, divD, dB, f0, f1, f2, f3);
    gprim = nr_conv_g(f0, f1, f2);
    if (gprim < gprimmin) {
      gprimmin = gprim;
      mindtfrac = dtfraction;
    }
  }
  if ((gprim < 1) && (gcount == 1)) dtoldfraction = 1e-8;
  else if (gprim < 1) dtoldfraction = nr_p10(-8 + gcount - 1);
  else {
    dtfraction = mindtfrac;
    dtoldfraction = 0.5 * dtfraction / 10.0;
  }
  dtnew = dtfraction * dt;
  dtold = dtoldfraction * dt;
  nr_vars(dtnew, v, dvdx, dI, divD, dB, f0, f1, f2, f3);
  gprim = nr_conv_g(f0, f1, f2);
  if (gprim < 0.5) return dtnew;
  gprimnew = 10.0;
  gprim = 10.0;
  ccount = bcount = zcount = rcount = counter = 0;
  while (counter < maxter) {
    counter = counter + 1;
    nr_vars(dtold, v, dvdx, dI, divD, dB, f0, f1, f2, f3);
    gprimder = nr_conv_gder(f0, f1, f2, f3);
    nr_vars(dtnew, v, dvdx, dI, divD, dB, f0, f1, f2, f3);
    gprimdernew = nr_conv_gder(f0, f1, f2, f3);
    gprim = nr_conv_g(f0, f1, f2);
    if ((gprimdernew - gprimder) > 0.0)
      gamman = fabs((dtnew - dtold) * (gprimdernew - gprimder)) /
               ((gprimdernew - gprimder) * (gprimdernew - gprimder));
    else
      gamman = 0.0;
    dtold = dtnew;
    dtnew = dtnew - gamman * gprimdernew;
    if (isnan(dtnew)) {
      dtnew = 0.0;
      break;
    }
    if ((gprim < 1) && (dtnew / dt > 1)) {
      dtnew = dtold;
      return dtnew;
    } else if (dtnew / dt > 1) {
      dtnew = (double)0.99f * dt;
    }
    if ((gprim < 1) && (dtnew < 0) && (dtold > 0)) {
      dtnew = dtold;
      return dtnew;
    } else if (dtnew < 0) {
      dtnew = (double)1e-8f * dt;
      zcount = zcount + 1;
      if (zcount > 1) {
        dtnew = 0.0;
        break;
      }
    }
    nr_vars(dtnew, v, dvdx, dI, divD, dB, f0, f1, f2, f3);
    gprimnew = nr_conv_g(f0, f1, f2);
    if ((gprimnew < 1) && (dtnew > 0) && (dtnew / dt < 1)) {
      rcount = rcount + 1;
      if (rcount > 1) return dtnew;
    } else {
      rcount = 0;
    }
    if ((gprim < 1) && (gprimnew > gprim)) {
      dtnew = dtold;
      return dtnew;
    }
    if ((fabs((dtold - dtnew) / dtold) < gdtol) && (gprim < 1)) {
      ccount = ccount + 1;
      if (ccount > 1) return dtnew;
    } else {
      ccount = 0;
    }
    if ((fabs((dtold - dtnew) / dtold) < gdtol) && (gprim > 1)) {
      bcount = bcount + 1;
      if (bcount > 1) break;
    } else {
      bcount = 0;
    }
  }
  if (gprim < 1) return dtnew;
  gprim = (double)1e10f;
  gprimmin = (double)1e10f;
  mindtfrac = 0.0;
  gcount = 1;
  while ((gprim > 1) && (gcount < 9)) {
    gcount = gcount + 1;
    dtfraction = (double)(0.1f * (float)gcount);
    dt0 = dt * dtfraction;
    nr_vars(dt0, v, dvdx, dI, divD, dB, f0, f1, f2, f3);
    gprim = nr_conv_g(f0, f1, f2);
    if (gprim < gprimmin) {
      gprimmin = gprim;
      mindtfrac = dtfraction;
    }
  }
  if (gprimmin < 1) dtnew = dt * mindtfrac;
  if ((dtnew <= 0.0) && (fabs(v) > 0.0)) dtnew = fabs(dI / v);
  return dtnew;
}

// NewtonRaphsonTimeStepExponentialAdvection (:2451-2554), at most 50 iterations
__device__ double nr_time_step(double dt, double v, double dvdx, double dI, double divD, double dB) {
  const double nrtol = (double)1e-6f;
  const int maxIter = 50;
  double nrerror = 1e6;
  double dt0 = nr_initial_guess(dt, v, dvdx, dI, divD, dB);
  if (dt0 == 0.0) return 0.0;
  int countIter = 0;
  while ((fabs(nrerror / dt0) > nrtol) && (countIter < maxIter)) {
    countIter = countIter + 1;
    const double f0 = adv_exponential(v, dvdx, dt0) + divD * dt0 + dB * sqrt(dt0) - dI;
    const double f1 = v * exp(dvdx * dt0) + divD + 0.5 * dB / sqrt(dt0);
    nrerror = -f0 / f1;
    dt0 = dt0 + nrerror;
    if (dt0 < 0.0) dt0 = -(double)0.9f * dt0;
  }
  if (dt0 > dt) return dt;
  if ((countIter == maxIter) && (fabs(nrerror / dt0) > nrtol)) return 0.0;
  return dt0;
}

// One axis of pr_DetectExitFaceAndUpdateTimeStepNewton (:1895-2079).
// Returns true when the routine must return at once (exitFace, dt set).
__device__ bool newton_axis(double npos, double pos, double d, double v, double dvdx, double divD, double dB,
                            int faceLo, int faceHi, double dt, double &dtaxis, int &exitAxis, int &exitFace,
                            double &dtout) {
  double dI;
  if (npos > 1.0) {
    dI = d * (1.0 - pos);
    exitAxis = faceHi;
  } else {
    dI = -d * pos;
    exitAxis = faceLo;
  }
  if (dI == 0.0) {
    exitFace = exitAxis;
    dtout = 0.0;
    return true;
  }
  dtaxis = nr_time_step(dt, v, dvdx, dI, divD, dB);
  if (dtaxis > dt) dtaxis = 0.0;
  return false;
}

template <typename R>
struct Visit {
  R x, y, z;     // current local position (TrackSubCell x,y,z)
  R ix, iy, iz;  // cell-entry location (initialLocation)
  double t, tinit, dtcell;
  R sqrt_dtcell, rdt_cell;
  int exitFace, posRestart;
  bool reachedMax;
  int64_t passes;
};

enum : int { PASS_CONTINUE = 0, PASS_MAXTIME = 1, PASS_EXIT = 2, PASS_UNDEFINED = 3 };

// component k (0, 1, 2) of three values, by selects (no local-memory array)
template <typename T>
__device__ __forceinline__ T pick3(int k, T a, T b, T c) {
  return (k == 0) ? a : ((k == 1) ? b : c);
}

// bit k set when component k of the proposed position is outside [0, 1]
template <typename R>
__device__ __forceinline__ unsigned axes_outside(R nx, R ny, R nz) {
  if constexpr (sizeof(R) == 8) {
    return (out01(nx) ? 1u : 0u) | (out01(ny) ? 2u : 0u) | (out01(nz) ? 4u : 0u);
  } else {
    const R zero = R(0), one = R(1);
    return ((nx > one || nx < zero) ? 1u : 0u) | ((ny > one || ny < zero) ? 2u : 0u) |
           ((nz > one || nz < zero) ? 4u : 0u);
  }
}

template <typename R>
__device__ __forceinline__ bool outside3(R a, R b, R c) {
  if constexpr (sizeof(R) == 8) {
    return out01(a) | out01(b) | out01(c);
  } else {
    const R zero = R(0), one = R(1);
    return (a > one) || (a < zero) || (b > one) || (b < zero) || (c > one) || (c < zero);
  }
}
#define MPRW_OUTSIDE(a, b, c) outside3(a, b, c)

// The first interface iteration's exit-face solves of the leaving lanes of
// `grp`, dealt out to every lane of `grp` (FP64).  Each (leaving lane,
// leaving axis) pair is a task; tasks in axis-major order go to the group's
// lanes by rank (a second round only past one task per lane), every lane
// solves one with its owner's values (quad_axis is a pure function of them),
// and each owner gets back, per leaving axis, whether the solve returned at
// once (bit k of rbits), its exit face and its time.  Without this, a warp
// solves its lanes' first leaving axes together and then their second axes
// (corner crossings) in a second round of one or two lanes.  Every lane of
// grp calls it together.
__device__ __forceinline__ void warp_exit_solves(unsigned grp, unsigned need, double nx, double ny, double nz,
                                                 double x, double y, double z, double dX, double dY, double dZ,
                                                 double vx, double vy, double vz, double ddx, double ddy,
                                                 double ddz, double bx, double by, double bz, double dt,
                                                 unsigned &rbits, double &tx, double &ty, double &tz, int &fx,
                                                 int &fy, int &fz) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const unsigned m0 = __ballot_sync(grp, need & 1u), m1 = __ballot_sync(grp, need & 2u);
  const unsigned m2 = __ballot_sync(grp, need & 4u);
  const int c0 = __popc(m0), c1 = __popc(m1), total = c0 + c1 + __popc(m2);
  const int nw = __popc(grp), rank = __popc(grp & below);
  // this lane's own tasks, one per leaving axis
  const int t0 = __popc(m0 & below), t1 = c0 + __popc(m1 & below), t2 = c0 + c1 + __popc(m2 & below);
  rbits = 0u;
  tx = ty = tz = 0.0;
  fx = fy = fz = 0;
  for (int base = 0; base < total; base += nw) {
    const int t = base + rank;
    int a = 0, owner = lane;
    if (t < total) {
      if (t < c0) {
        owner = __fns(m0, 0, t + 1);
      } else if (t < c0 + c1) {
        a = 1;
        owner = __fns(m1, 0, t - c0 + 1);
      } else {
        a = 2;
        owner = __fns(m2, 0, t - c0 - c1 + 1);
      }
    }
    // the owner's values on all three axes, the task's axis picked after
    const double onx = __shfl_sync(grp, nx, owner), ony = __shfl_sync(grp, ny, owner);
    const double onz = __shfl_sync(grp, nz, owner);
    const double ox = __shfl_sync(grp, x, owner), oy = __shfl_sync(grp, y, owner), oz = __shfl_sync(grp, z, owner);
    const double odX = __shfl_sync(grp, dX, owner), odY = __shfl_sync(grp, dY, owner);
    const double odZ = __shfl_sync(grp, dZ, owner);
    const double ovx = __shfl_sync(grp, vx, owner), ovy = __shfl_sync(grp, vy, owner);
    const double ovz = __shfl_sync(grp, vz, owner);
    const double oddx = __shfl_sync(grp, ddx, owner), oddy = __shfl_sync(grp, ddy, owner);
    const double oddz = __shfl_sync(grp, ddz, owner);
    const double obx = __shfl_sync(grp, bx, owner), oby = __shfl_sync(grp, by, owner);
    const double obz = __shfl_sync(grp, bz, owner);
    const double odt = __shfl_sync(grp, dt, owner);
    bool r = false;
    double dta = 0.0;
    int efa = 0;
    if (t < total) {
      int ef_unused = 0;
      double dt_unused = 0.0;
      r = quad_axis_f64(pick3(a, onx, ony, onz), pick3(a, ox, oy, oz), pick3(a, odX, odY, odZ),
                            pick3(a, ovx, ovy, ovz), pick3(a, oddx, oddy, oddz), pick3(a, obx, oby, obz),
                            2 * a + 1, 2 * a + 2, odt, dta, efa, ef_unused, dt_unused);
    }
    // results back to their owners, one axis at a time
    const unsigned packed = (r ? 8u : 0u) | (unsigned)efa;
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const int tb = (b == 0) ? t0 : ((b == 1) ? t1 : t2);
      const bool mine = ((need >> b) & 1u) && tb >= base && tb < base + nw;
      const int wl = mine ? (int)__fns(grp, 0, tb - base + 1) : lane;
      const unsigned pk = __shfl_sync(grp, packed, wl);
      const double dv = __shfl_sync(grp, dta, wl);
      if (mine) {
        if (pk & 8u) rbits |= 1u << b;
        if (b == 0) { tx = dv; fx = (int)(pk & 7u); }
        else if (b == 1) { ty = dv; fy = (int)(pk & 7u); }
        else { tz = dv; fz = (int)(pk & 7u); }
      }
    }
  }
}

// One pass of the `do while (continueTimeLoop)` body, TrackSubCell.F90:956-1368.
// On PASS_MAXTIME / PASS_EXIT the final location is (ox,oy,oz,V.t); on
// PASS_UNDEFINED the caller uses the last recorded point.
template <typename R, bool EXP, bool AXI>
__device__ int rw_pass(Visit<R> &V, const Lane<R> &F, uint32_t massb, double maxTime, int ndim, int d1, int d2,
                       uint64_t seed, uint64_t id, uint64_t &ctr, R &ox, R &oy, R &oz) {
  const R zero = R(0), one = R(1), half = R(0.5);
  const unsigned grp = __activemask();  // the lanes running this pass together
  const double dtRed = (double)0.1f;  // dtReductionFactor, a single-precision literal (:850)
  double dt = V.dtcell;
  R rdt = V.rdt_cell, sdt = V.sqrt_dtcell;  // FP32 copies: no conversion on the common pass
  V.t = V.t + dt;
  if (sizeof(R) == 8 ? past_end(maxTime, V.t) : maxTime < V.t) {
    V.t = V.t - dt;
    dt = fmax(maxTime - V.t, 0.0);
    V.t = maxTime;
    V.reachedMax = true;
    rdt = (R)dt;
    sdt = sqrt(rdt);
  }
  R x = V.x, y = V.y, z = V.z;
  R dX = F(F_D + 0), dY = F(F_D + 1), dZ = F(F_D + 2);
  R iX = F(F_INVD + 0), iY = F(F_INVD + 1), iZ = F(F_INVD + 2);
  // pr_RWPTDisplacementsLinear (:673-706)
  R vx = fma(x, F(F_DV + 0), F(F_V1 + 0));
  R vy = fma(y, F(F_DV + 1), F(F_V1 + 1));
  R vz = fma(z, F(F_DV + 2), F(F_V1 + 2));
  R xy = x * y, xz = x * z, yz = y * z;
  R ddx = divc(F, F_DIV + 0, x, y, z, xy, xz, yz);
  R ddy = divc(F, F_DIV + 7, x, y, z, xy, xz, yz);
  R ddz = divc(F, F_DIV + 14, x, y, z, xy, xz, yz);
  R bx, by, bz;
  random_displacement<R, AXI>(F, ndim, d1, d2, x, y, z, vx, vy, vz, seed, id, ctr, bx, by, bz);
  // advection displacement: EULERIAN v dt, EXPONENTIAL (FP64) v (e^{dv dt}-1)/dv
  // with dv = (V2 - V1)/D of the cell (pr_AdvectionDisplacement*, :1487-1573)
  double dvx = 0.0, dvy = 0.0, dvz = 0.0;
  if constexpr (EXP) {
    dvx = (double)F(F_DV + 0) / (double)dX;
    dvy = (double)F(F_DV + 1) / (double)dY;
    dvz = (double)F(F_DV + 2) / (double)dZ;
  }
  R ax, ay, az;
  auto advect = [&]() {
    if constexpr (EXP) {
      ax = (R)adv_exponential((double)vx, dvx, dt);
      ay = (R)adv_exponential((double)vy, dvy, dt);
      az = (R)adv_exponential((double)vz, dvz, dt);
    } else {
      ax = vx * rdt;
      ay = vy * rdt;
      az = vz * rdt;
    }
  };
  advect();
  R dxrw = ax + ddx * rdt + bx * sdt;
  R dyrw = ay + ddy * rdt + by * sdt;
  R dzrw = az + ddz * rdt + bz * sdt;
  // jump limiter (:989-1013)
  if constexpr (sizeof(R) == 4 && !EXP) {
    // MIXED: the cut step stays in FP32 (rdt = 0.1 rdt) and the simulation
    // time is corrected once after the loop.  The loop runs with a few
    // lanes, and every FP64 operation in it would cost a whole warp
    // instruction on the narrow FP64 pipe.
    const double dt0 = dt;
    bool cut = false;
    while ((fabs(dxrw * iX) > half) || (fabs(dyrw * iY) > half) || (fabs(dzrw * iZ) > half)) {
      rdt = R(0.1f) * rdt;
      sdt = sqrt(rdt);
      advect();
      dxrw = ax + ddx * rdt + bx * sdt;
      dyrw = ay + ddy * rdt + by * sdt;
      dzrw = az + ddz * rdt + bz * sdt;
      cut = true;
    }
    if (cut) {
      dt = (double)rdt;
      V.t = (V.t - dt0) + dt;
      V.reachedMax = false;
    }
  } else
  while (sizeof(R) == 8 ? abs_above_half(dxrw * iX) | abs_above_half(dyrw * iY) | abs_above_half(dzrw * iZ)
                        : (fabs(dxrw * iX) > half) || (fabs(dyrw * iY) > half) || (fabs(dzrw * iZ) > half)) {
    V.t = V.t - dt;
    dt = dtRed * dt;
    rdt = (R)dt;
    sdt = sqrt(rdt);
    advect();
    dxrw = ax + ddx * rdt + bx * sdt;
    dyrw = ay + ddy * rdt + by * sdt;
    dzrw = az + ddz * rdt + bz * sdt;
    V.t = V.t + dt;
    V.reachedMax = false;
  }
  R nx = x + dxrw * iX, ny = y + dyrw * iY, nz = z + dzrw * iZ;
  // FP64 EULERIAN: the first interface iteration's exit-face solves of the
  // leaving lanes, spread over every lane of the pass
  unsigned pre_r = 0u;
  double pre_tx = 0.0, pre_ty = 0.0, pre_tz = 0.0;
  int pre_fx = 0, pre_fy = 0, pre_fz = 0;
  if constexpr (sizeof(R) == 8 && !EXP) {
    __syncwarp(grp);
    warp_exit_solves(grp, MPRW_OUTSIDE(nx, ny, nz) ? axes_outside(nx, ny, nz) : 0u, nx, ny, nz, x, y, z, dX, dY,
                     dZ, vx, vy, vz, ddx, ddy, ddz, bx, by, bz, dt, pre_r, pre_tx, pre_ty, pre_tz, pre_fx, pre_fy,
                     pre_fz);
  }
  // particleLeavingCell (:1025-1316)
  int intLoop = 0;
  while (MPRW_OUTSIDE(nx, ny, nz)) {
    ++intLoop;
    if constexpr (EXP) {
      // ExitFaceAndUpdateTimeStep (Newton, :1895-2079), FP64
      double dtx = 0.0, dty = 0.0, dtz = 0.0;
      int efx = 0, efy = 0, efz = 0;
      bool ret = false;
      V.t = V.t - dt;
      // the axes the step leaves through, x then y then z, solved in one
      // shared block: the first axis of every leaving lane together, then
      // the second (a warp's leaving lanes mostly leave through different
      // axes; three per-axis branches would each run with a few lanes)
      unsigned need = axes_outside(nx, ny, nz);
      while (!ret && need) {
        const int k = __ffs(need) - 1;
        need &= need - 1;
        double dta = 0.0;
        int efa = 0;
        ret = newton_axis((double)pick3(k, nx, ny, nz), (double)pick3(k, x, y, z), (double)pick3(k, dX, dY, dZ),
                          (double)pick3(k, vx, vy, vz), pick3(k, dvx, dvy, dvz), (double)pick3(k, ddx, ddy, ddz),
                          (double)pick3(k, bx, by, bz), 2 * k + 1, 2 * k + 2, dt, dta, efa, V.exitFace, dt);
        if (k == 0) { dtx = dta; efx = efa; }
        else if (k == 1) { dty = dta; efy = efa; }
        else { dtz = dta; efz = efa; }
      }
      if (!ret) {
        if (dtx == 0.0 && dty == 0.0 && dtz == 0.0) {
          V.t = V.t + dt;
        } else {
          int im = -1;
          double best = 0.0;
          if (dtx > 0.0) { im = 0; best = dtx; }
          if (dty > 0.0 && (im < 0 || dty < best)) { im = 1; best = dty; }
          if (dtz > 0.0 && (im < 0 || dtz < best)) { im = 2; best = dtz; }
          dt = best;
          V.exitFace = (im == 0) ? efx : (im == 1 ? efy : efz);
          V.t = V.t + dt;
        }
      }
    } else {
      R dtx = zero, dty = zero, dtz = zero;
      // ExitFaceAndUpdateTimeStep (quadratic, :1576-1892)
      int efx = 0, efy = 0, efz = 0;
      bool ret = false;
      // MIXED takes the time back only when the step changes (below)
      const double dt_in = dt;
      if constexpr (sizeof(R) == 8) V.t = V.t - dt;
      if constexpr (sizeof(R) == 8) {
        // FP64: the first iteration takes the warp-wide solves (the same
        // inputs: nothing has moved yet); later ones solve the leaving axes
        // in one shared block (as for EXPONENTIAL).  The FP32 solve is cheap
        // enough that the extra registers of either cost more than the
        // divergence.
        unsigned need = axes_outside(nx, ny, nz);
        if (intLoop == 1) {
          while (!ret && need) {
            const int k = __ffs(need) - 1;
            need &= need - 1;
            if ((pre_r >> k) & 1u) {
              V.exitFace = pick3(k, pre_fx, pre_fy, pre_fz);
              dt = 0.0;
              ret = true;
            } else if (k == 0) { dtx = pre_tx; efx = pre_fx; }
            else if (k == 1) { dty = pre_ty; efy = pre_fy; }
            else { dtz = pre_tz; efz = pre_fz; }
          }
        }
        while (!ret && need) {
          const int k = __ffs(need) - 1;
          need &= need - 1;
          R dta = zero;
          int efa = 0;
          ret = quad_axis_f64(pick3(k, nx, ny, nz), pick3(k, x, y, z), pick3(k, dX, dY, dZ), pick3(k, vx, vy, vz),
                          pick3(k, ddx, ddy, ddz), pick3(k, bx, by, bz), 2 * k + 1, 2 * k + 2, dt, dta, efa,
                          V.exitFace, dt);
          if (k == 0) { dtx = dta; efx = efa; }
          else if (k == 1) { dty = dta; efy = efa; }
          else { dtz = dta; efz = efa; }
        }
      } else {
        if (!ret && ((nx > one) || (nx < zero)))
          ret = quad_axis(nx, x, dX, vx, ddx, bx, 1, 2, rdt, dtx, efx, V.exitFace, dt);
        if (!ret && ((ny > one) || (ny < zero)))
          ret = quad_axis(ny, y, dY, vy, ddy, by, 3, 4, rdt, dty, efy, V.exitFace, dt);
        if (!ret && ((nz > one) || (nz < zero)))
          ret = quad_axis(nz, z, dZ, vz, ddz, bz, 5, 6, rdt, dtz, efz, V.exitFace, dt);
      }
      if (!ret) {
        if (sizeof(R) == 8 ? is0(dtx) && is0(dty) && is0(dtz) : dtx == zero && dty == zero && dtz == zero) {
          if constexpr (sizeof(R) == 8) V.t = V.t + dt;
        } else {
          int im = -1;
          R best = zero;
          if constexpr (sizeof(R) == 8) {
            // (best > 0 once im >= 0)
            if (above0(dtx)) { im = 0; best = dtx; }
            if (above0(dty) && (im < 0 || pos_lt(dty, best))) { im = 1; best = dty; }
            if (above0(dtz) && (im < 0 || pos_lt(dtz, best))) { im = 2; best = dtz; }
          } else {
            if (dtx > zero) { im = 0; best = dtx; }
            if (dty > zero && (im < 0 || dty < best)) { im = 1; best = dty; }
            if (dtz > zero && (im < 0 || dtz < best)) { im = 2; best = dtz; }
          }
          dt = (double)best;
          V.exitFace = (im == 0) ? efx : (im == 1 ? efy : efz);
          if constexpr (sizeof(R) == 8) {
            V.t = V.t + dt;
          } else {
            V.t = (V.t - dt_in) + dt;
            rdt = best;
          }
        }
      } else if constexpr (sizeof(R) == 4) {
        V.t = V.t - dt_in;
        rdt = zero;
      }
    }
    if (intLoop > 5) {
      nx = V.ix; ny = V.iy; nz = V.iz;
      V.t = V.tinit;
      dt = V.dtcell;
      if (++V.posRestart > 10) {
        V.x = x; V.y = y; V.z = z;
        return PASS_UNDEFINED;
      }
      break;
    }
    if constexpr (sizeof(R) == 8 || EXP) rdt = (R)dt;  // MIXED EULERIAN: rdt set above
    sdt = sqrt(rdt);
    advect();
    V.reachedMax = false;
    int ef = V.exitFace;
    if (ef >= 1 && ef <= 6 && sizeof(R) == 8) {
      // FP64: the step of the truncated time on every axis (one shared
      // block), then the exit axis pinned to its face
      const R dxc = ax + ddx * rdt + bx * sdt;
      const R dyc = ay + ddy * rdt + by * sdt;
      const R dzc = az + ddz * rdt + bz * sdt;
      const R nxc = x + dxc * iX, nyc = y + dyc * iY, nzc = z + dzc * iZ;
      const int fa = (ef - 1) >> 1;
      const R pin = (ef & 1) ? zero : one;
      if (fa != 0) { dxrw = dxc; nx = nxc; } else { nx = pin; }
      if (fa != 1) { dyrw = dyc; ny = nyc; } else { ny = pin; }
      if (fa != 2) { dzrw = dzc; nz = nzc; } else { nz = pin; }
    } else if (ef == 1 || ef == 2) {
      nx = (ef == 1) ? zero : one;
      dyrw = ay + ddy * rdt + by * sdt;
      ny = y + dyrw * iY;
      dzrw = az + ddz * rdt + bz * sdt;
      nz = z + dzrw * iZ;
    } else if (ef == 3 || ef == 4) {
      dxrw = ax + ddx * rdt + bx * sdt;
      nx = x + dxrw * iX;
      ny = (ef == 3) ? zero : one;
      dzrw = az + ddz * rdt + bz * sdt;
      nz = z + dzrw * iZ;
    } else if (ef == 5 || ef == 6) {
      dxrw = ax + ddx * rdt + bx * sdt;
      nx = x + dxrw * iX;
      dyrw = ay + ddy * rdt + by * sdt;
      ny = y + dyrw * iY;
      nz = (ef == 5) ? zero : one;
    } else {
      nx = V.ix; ny = V.iy; nz = V.iz;
      V.t = V.tinit;
      dt = V.dtcell;
      if (++V.posRestart > 10) {
        V.x = x; V.y = y; V.z = z;
        return PASS_UNDEFINED;
      }
      break;
    }
    if (MPRW_OUTSIDE(nx, ny, nz)) continue;
    // elasticRebound (:1157-1312)
    int rebound = 0;
    while (V.exitFace > 0) {
      if (!((massb >> (V.exitFace - 1)) & 1u)) break;
      if (++rebound > 10) {
        V.x = x; V.y = y; V.z = z;
        return PASS_UNDEFINED;
      }
      R xi = nx, yi = ny, zi = nz;
      if (sizeof(R) == 8 ? is0(dt) : dt == 0.0) {
        nx = V.ix; ny = V.iy; nz = V.iz;
        V.t = V.t - dt;
        dt = V.dtcell;
        V.exitFace = 0;
        ++V.posRestart;
        break;
      }
      V.t = V.t + dt;
      if (sizeof(R) == 8 ? past_end(maxTime, V.t) : maxTime < V.t) {
        V.t = V.t - dt;
        dt = fmax(maxTime - V.t, 0.0);
        V.t = maxTime;
        V.reachedMax = true;
        rdt = (R)dt;
        sdt = sqrt(rdt);
        advect();
        dxrw = ax + ddx * rdt + bx * sdt;
        dyrw = ay + ddy * rdt + by * sdt;
        dzrw = az + ddz * rdt + bz * sdt;
      }
      ef = V.exitFace;
      if (ef == 1 || ef == 2) {
        nx = nx - dxrw * iX; ny = ny + dyrw * iY; nz = nz + dzrw * iZ;
      } else if (ef == 3 || ef == 4) {
        nx = nx + dxrw * iX; ny = ny - dyrw * iY; nz = nz + dzrw * iZ;
      } else {
        nx = nx + dxrw * iX; ny = ny + dyrw * iY; nz = nz - dzrw * iZ;
      }
      if (MPRW_OUTSIDE(nx, ny, nz)) {
        x = xi; y = yi; z = zi;
        if (ef == 1 || ef == 2) { vx = -vx; ddx = -ddx; bx = -bx; }
        else if (ef == 3 || ef == 4) { vy = -vy; ddy = -ddy; by = -by; }
        else { vz = -vz; ddz = -ddz; bz = -bz; }
        V.exitFace = 0;
      } else {
        dt = V.dtcell;
        V.exitFace = 0;
        if constexpr (sizeof(R) == 8) {
          if (is0(nx)) V.exitFace = 1;
          if (is1(nx)) V.exitFace = 2;
          if (is0(ny)) V.exitFace = 3;
          if (is1(ny)) V.exitFace = 4;
          if (is0(nz)) V.exitFace = 5;
          if (is1(nz)) V.exitFace = 6;
        } else {
          if (nx == zero) V.exitFace = 1;
          if (nx == one) V.exitFace = 2;
          if (ny == zero) V.exitFace = 3;
          if (ny == one) V.exitFace = 4;
          if (nz == zero) V.exitFace = 5;
          if (nz == one) V.exitFace = 6;
        }
      }
    }
  }
  if (V.reachedMax) {
    ox = nx; oy = ny; oz = nz;
    return PASS_MAXTIME;
  }
  if (V.exitFace > 0) {
    ox = nx; oy = ny; oz = nz;
    return PASS_EXIT;
  }
  V.x = nx; V.y = ny; V.z = nz;
  return PASS_CONTINUE;
}

// Persistent kernel: every lane owns one particle at a time.  Each iteration of
// the main loop (a) refills lanes without a particle from the atomic queue
// (one atomic per warp), (b) runs the cell-entry phase for lanes that changed
// cell, (c) runs one time-loop pass for every tracking lane.  All phases are
// structured and the loop head re-converges the warp, so the common pass body
// runs with every tracking lane active; the loop ends when no lane of the warp
// has work.
template <typename R, bool EXP, bool AXI>
__global__ void __launch_bounds__(step_threads(sizeof(R) == 8, EXP), (sizeof(R) == 4 && !EXP) ? 3 : 1) rwpt_advance_kernel(AdvanceArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  R *sm = reinterpret_cast<R *>(smraw) + threadIdx.x;
  const int stride = blockDim.x;
  Lane<R> F{sm, stride};
  const R zero = R(0), one = R(1);
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;

  int64_t my_passes = 0;
  int64_t p = -1;        // particle being tracked (index into the state arrays)
  bool open = true;      // the queue may still have particles for this lane
  int32_t c = 0;         // current cell (0-based)
  bool need_cell = false;
  uint64_t id = 0, ctr = 0;
  // last point of the pathline (cell, local coords, time)
  int32_t lc = 0;
  R lx = zero, ly = zero, lz = zero;
  double lt = 0.0;
  // location at cell entry
  R ex = zero, ey = zero, ez = zero;
  double et = 0.0;
  Visit<R> V;
  V.x = V.y = V.z = V.ix = V.iy = V.iz = zero;
  V.t = V.tinit = V.dtcell = 0.0;
  V.sqrt_dtcell = zero;
  V.rdt_cell = zero;
  V.exitFace = V.posRestart = 0;
  V.reachedMax = false;
  V.passes = 0;
  uint32_t massb = 0;
  // cell exits of the current particle in this launch (bits 0-19) and how
  // many of the last ones took no time (bits 20-30): one register for both caps
  static_assert(kMaxVisitsPerAdvance < (1 << 20) - 1 && kMaxZeroTimeExits < (1 << 11) - 1, "exit counter bits");
  uint32_t exits = 0;

  unsigned iter = 0;
  for (;;) {
    __syncwarp(FULL);
    // cancel: the host set the flag (timeout or mprw_cancel).  Each lane keeps
    // its particle where it is -- the start of the cell it is entering, or the
    // last completed pass of its visit -- as ACTIVE, and the queue is not
    // drained further, so every particle holds a valid location.
    if (a.abort && (++iter % kAbortPoll) == 0) {
      int ab = (lane == 0) ? *a.abort : 0;
      ab = __shfl_sync(FULL, ab, 0);
      if (ab) {
        if (p >= 0) {
          a.cell[p] = c;
          if (need_cell) {
            a.x[p] = ex; a.y[p] = ey; a.z[p] = ez; a.t[p] = et;
          } else {
            a.x[p] = V.x; a.y[p] = V.y; a.z[p] = V.z; a.t[p] = V.t;
          }
          a.status[p] = ST_ACTIVE;
          a.ctr[p] = ctr;
        }
        break;
      }
    }
    // (a) refill
    const bool want = (p < 0) && open;
    const unsigned m = __ballot_sync(FULL, want);
    if (m) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader)
        base = atomicAdd(reinterpret_cast<unsigned long long *>(a.queue), (unsigned long long)__popc(m));
      base = __shfl_sync(FULL, base, leader);
      if (want) {
        const int64_t q = (int64_t)base + __popc(m & ((1u << lane) - 1u));
        if (q >= a.n) {
          open = false;
        } else {
          p = a.perm ? (int64_t)a.perm[q] : q;
          int32_t status = a.status[p];
          c = a.cell[p];
          ex = a.x[p]; ey = a.y[p]; ez = a.z[p];
          et = a.t[p];
          // release checks, MPathRW.F90:1256-1302
          if (status == ST_PENDING) {
            if (et < a.t_begin) status = ST_UNRELEASED;
            else if (et <= a.t_end) {
              status = ST_ACTIVE;
              if (a.iboundts[c] == 0) status = ST_INACTIVE;
            }
          }
          if (status == ST_INACTIVE && (a.cellflags[c] & 2u)) status = ST_ACTIVE;  // partially dry
          if (status != ST_ACTIVE) {
            a.status[p] = status;
            p = -1;
          } else {
            id = a.id ? a.id[p] : (uint64_t)p;
            ctr = a.ctr[p];
            lc = c; lx = ex; ly = ey; lz = ez; lt = et;
            need_cell = true;
            exits = 0;
          }
        }
      }
    }
    if (!__any_sync(FULL, (p >= 0) || open)) break;

    // (b) cell entry (TrackCell checks + sub-cell set-up)
    if (p >= 0 && need_cell) {
      need_cell = false;
      int32_t fin = 0;  // 0 track, else final status
      bool use_last = false;
      if (sizeof(R) == 8 ? outside3(ex, ey, ez)
                         : ex < zero || ex > one || ey < zero || ey > one || ez < zero || ez > one) {
        fin = ST_UNDEFINED;  // InvalidLocation (TrackCell.f90:410-413)
        use_last = true;
      } else {
        const CellRec<R> *rec = a.recs + c;
        const int32_t es = rec->entry_status;
        if (es != 0) {
          fin = es;
          use_last = (es == ST_UNDEFINED);
        } else {
          stage_record(a.recs, c, sm, stride);
          massb = rec->massb;
          V.x = ex; V.y = ey; V.z = ez;
          V.ix = ex; V.iy = ey; V.iz = ez;
          V.t = et; V.tinit = et;
          V.dtcell = rec->dtcell;
          V.sqrt_dtcell = (R)rec->sqrt_dtcell;
          V.rdt_cell = (R)rec->dtcell;
          V.exitFace = 0;
          V.posRestart = 0;
          V.reachedMax = false;
          V.passes = 0;
        }
      }
      if (fin != 0) {
        if (use_last) {
          a.cell[p] = lc; a.x[p] = lx; a.y[p] = ly; a.z[p] = lz; a.t[p] = lt;
        } else {
          a.cell[p] = c; a.x[p] = ex; a.y[p] = ey; a.z[p] = ez; a.t[p] = et;
        }
        a.status[p] = fin;
        a.ctr[p] = ctr;
        p = -1;
      }
    }

    // (c) one time-loop pass (with the per-visit safety cap)
    if (p >= 0 && !need_cell) {
      R ox = zero, oy = zero, oz = zero;
      int r;
      if (++V.passes > kMaxStepsPerVisit) {
        r = PASS_UNDEFINED;
      } else {
        r = rw_pass<R, EXP, AXI>(V, F, massb, a.t_end, a.ndim, a.d1, a.d2, a.seed, id, ctr, ox, oy, oz);
        ++my_passes;
      }
      if (r == PASS_MAXTIME) {
        a.cell[p] = c; a.x[p] = ox; a.y[p] = oy; a.z[p] = oz; a.t[p] = V.t;
        a.status[p] = ST_ACTIVE;
        a.ctr[p] = ctr;
        p = -1;
      } else if (r == PASS_UNDEFINED) {
        a.cell[p] = lc; a.x[p] = lx; a.y[p] = ly; a.z[p] = lz; a.t[p] = lt;
        a.status[p] = ST_UNDEFINED;
        a.ctr[p] = ctr;
        p = -1;
      } else if (r == PASS_EXIT &&
                 ((exits = ((exits & 0xFFFFFu) + 1u) | ((sizeof(R) == 8 ? eq_any(V.t, V.tinit) : V.t == V.tinit) ? ((exits >> 20) + 1u) << 20 : 0u)) >> 20 >
                      (uint32_t)kMaxZeroTimeExits ||
                  (exits & 0xFFFFFu) > (uint32_t)kMaxVisitsPerAdvance)) {
        a.cell[p] = lc; a.x[p] = lx; a.y[p] = ly; a.z[p] = lz; a.t[p] = lt;
        a.status[p] = ST_UNDEFINED;
        a.ctr[p] = ctr;
        p = -1;
      } else if (r == PASS_EXIT) {
        // the exit point becomes the last pathline point
        const int face = V.exitFace;
        lc = c; lx = ox; ly = oy; lz = oz; lt = V.t;
        // the neighbour through the exit face, read from the cell's record
        // (not held in registers through the visit)
        const int32_t nc = __ldg(&a.recs[c].conn[face - 1]);
        // ConvertFromNeighbor: the exit coordinate must sit exactly on the face
        const bool bad = sizeof(R) == 8
                             ? (face == 2 && !is1(ox)) || (face == 1 && !is0(ox)) || (face == 4 && !is1(oy)) ||
                                   (face == 3 && !is0(oy)) || (face == 6 && !is1(oz)) || (face == 5 && !is0(oz))
                             : (face == 2 && ox != one) || (face == 1 && ox != zero) || (face == 4 && oy != one) ||
                                   (face == 3 && oy != zero) || (face == 6 && oz != one) || (face == 5 && oz != zero);
        if (nc < 0 || bad) {
          a.cell[p] = lc; a.x[p] = lx; a.y[p] = ly; a.z[p] = lz; a.t[p] = lt;
          a.status[p] = (nc < 0) ? ST_BOUNDARY : ST_UNDEFINED;
          a.ctr[p] = ctr;
          p = -1;
        } else {
          ex = ox; ey = oy; ez = oz; et = V.t;
          if (face == 2) ex = zero;
          if (face == 1) ex = one;
          if (face == 4) ey = zero;
          if (face == 3) ey = one;
          if (face == 6) ez = zero;
          if (face == 5) ez = one;
          c = nc;
          need_cell = true;
        }
      }
    }
  }
  // block-level sum of passes, one atomic per block
  __shared__ unsigned long long blk;
  if (threadIdx.x == 0) blk = 0;
  __syncthreads();
  atomicAdd(&blk, (unsigned long long)my_passes);
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(reinterpret_cast<unsigned long long *>(a.steps), blk);
}

template <typename R>
size_t advance_smem_bytes(int threads) {
  return (size_t)NFIELDS * sizeof(R) * threads;
}

template <typename R>
cudaError_t launch_advance(const AdvanceArgs<R> &a, int blocks, int threads, cudaStream_t s) {
  size_t smem = advance_smem_bytes<R>(threads);
  auto kern = a.exp_adv ? (a.axi ? rwpt_advance_kernel<R, true, true> : rwpt_advance_kernel<R, true, false>)
                        : (a.axi ? rwpt_advance_kernel<R, false, true> : rwpt_advance_kernel<R, false, false>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<blocks, threads, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename R>
cudaError_t advance_occupancy(int exp_adv, int axi, int threads, int *blocks_per_sm) {
  size_t smem = advance_smem_bytes<R>(threads);
  auto kern = exp_adv ? (axi ? rwpt_advance_kernel<R, true, true> : rwpt_advance_kernel<R, true, false>)
                      : (axi ? rwpt_advance_kernel<R, false, true> : rwpt_advance_kernel<R, false, false>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kern, threads, smem);
}

template cudaError_t launch_advance<double>(const AdvanceArgs<double> &, int, int, cudaStream_t);
template cudaError_t advance_occupancy<double>(int, int, int, int *);
template cudaError_t advance_occupancy<float>(int, int, int, int *);
template cudaError_t launch_advance<float>(const AdvanceArgs<float> &, int, int, cudaStream_t);
template size_t advance_smem_bytes<double>(int);
template size_t advance_smem_bytes<float>(int);

}  // namespace mprw
