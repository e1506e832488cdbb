// mprw_common.cuh -- device data layout and helpers shared by the kernels.
//
// HBM layout (one flow time step resident on the device):
//   CellBase  (SoA, per cell)  : face flows Q1..Q6, saturated thickness, links
//   CellRec<R>(AoS, per cell)  : everything one random-walk step needs, built
//                                once per flow time step by the prep kernels;
//                                R = double (FP64 path) or float (MIXED path)
//   particles (SoA)            : cell (int32, 0-based), status (int32),
//                                local x/y/z (R), tracking time (double),
//                                Philox block counter (uint64), id (uint64)
//
// The record replaces the 19 cell buffers + corner variables that the
// reference rebuilds on every cell entry (ParticleTrackingEngine.f90:1093-1108,
// TrackCell.f90:511-518, TrackSubCell.F90:3667-4363).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "fpbits.cuh"

namespace mprw {

// Trilinear interpolants are stored as monomial coefficients
//   f(x,y,z) = a0 + a1 x + a2 y + a3 z + a4 xy + a5 xz + a6 yz + a7 xyz
// and the dispersion divergence (TrackSubCell.F90:2695-2818, a sum of three
// trilinear derivatives per component, divided by porosity*retardation) as
//   g(x,y,z) = c0 + c1 x + c2 y + c3 z + c4 xy + c5 xz + c6 yz.
template <typename R>
struct __align__(16) CellRec {
  R v1[3];       // VX1, VY1, VZ1 (TrackSubCell.F90:1461-1484)
  R dv[3];       // VX2-VX1, VY2-VY1, VZ2-VZ1
  R d[3];        // DX, DY, DZ (DZ = GetDZRW)
  R inv_d[3];    // 1/DX, 1/DY, 1/DZ
  R div[3][7];   // dispersion divergence coefficients
  R vb[3][8];    // corner velocity q_c/phi_c, trilinear monomials
  R aL, aT, dm, two_over_r;
  R v2[3];       // VX2, VY2, VZ2 (exit-face solver needs face values)
  R aLV, aTV;    // vertical dispersivities (axisymmetric model; = aL, aT otherwise)
  double dtcell; // ComputeRandomWalkTimeStep (TrackSubCell.F90:1376-1458)
  double sqrt_dtcell;
  int32_t conn[6];     // 0-based neighbour, -1 = boundary face or inactive neighbour
  int32_t entry_status;// 0 = track; else the driver status assigned on entry
  uint32_t massb;      // bit f set: MassBoundary(f+1) == 1 (reflecting face)
};

// Per-cell intermediate of the prep stage (ModpathCellData buffer fields that
// the corner interpolation reads from the 18 neighbours).
struct CellBase {
  double *q;        // 6*ncell face flows Q1..Q6 (boundary flows applied)
  double *dz;       // GetDZRW thickness
  int32_t *conn;    // 6*ncell, 0-based connected cell or -1
  uint8_t *flags;   // bit0 dry, bit1 partiallyDry, bit2 hasExit(Q), bit3 sink!=0, bit4 source!=0
};

// Problem constants passed by value to the kernels.
struct GridDims {
  int32_t nlay, nrow, ncol, ncpl, ncell;
};

// ---------------------------------------------------------------------------
// Counter-based normal variates: Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), key = seed,
// counter = (block index lo, hi, particle id lo, hi).  One normal is the
// Irwin-Hall sum of the twelve 32-bit words of three blocks, scaled by 2^-32,
// minus 6 -- the same distribution as the reference's
// GenerateStandardNormalRandomZig (TrackSubCell.F90:3631-3663), with streams
// that depend only on (seed, particle id, draw index).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t lo0 = 0xD2511F53u * c0;
    uint32_t hi0 = __umulhi(0xD2511F53u, c0);
    uint32_t lo1 = 0xCD9E8D57u * c2;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

// Exact Irwin-Hall(12) normal from three Philox blocks; advances ctr by 3.
// The normal is S*2^-32 - 6 for the 36-bit sum S of the twelve words.
__device__ __forceinline__ double normal_ih12(uint64_t seed, uint64_t id, uint64_t &ctr) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  uint32_t i0 = (uint32_t)id, i1 = (uint32_t)(id >> 32);
  uint64_t sum = 0;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    uint64_t n = ctr++;
    uint32_t o[4];
    philox4x32_10((uint32_t)n, (uint32_t)(n >> 32), i0, i1, k0, k1, o);
    sum += (uint64_t)o[0] + o[1] + o[2] + o[3];
  }
  // assembled from its bits on the integer pipe (GB300's FP64 pipe is the
  // step kernel's limit)
  return fb::ih12_normal(sum);
}

// MIXED-precision normals: the same three Philox blocks (twelve 32-bit
// words) as normal_ih12, so both precisions draw the same normal from the
// same counter (common random numbers); only the final value is rounded to
// FP32.  With S = hi*2^32 + lo the normal is (hi - 6) + lo*2^-32: hi - 6 is an
// exact small integer, lo*2^-32 < 1 carries one FP32 rounding, and the FMA
// adds a second, so the result is within 2^-23 of the FP64 normal.
__device__ __forceinline__ float normal_ih12_f32(uint64_t seed, uint64_t id, uint64_t &ctr) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  uint32_t i0 = (uint32_t)id, i1 = (uint32_t)(id >> 32);
  uint64_t sum = 0;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    uint64_t n = ctr++;
    uint32_t o[4];
    philox4x32_10((uint32_t)n, (uint32_t)(n >> 32), i0, i1, k0, k1, o);
    sum += (uint64_t)o[0] + o[1] + o[2] + o[3];
  }
  const int hi = (int)(sum >> 32);
  return fmaf(__uint2float_rn((uint32_t)sum), 2.3283064365386963e-10f, (float)(hi - 6));  // 2^-32
}

// Driver status codes (MPathRW.F90:1337-1403).
enum : int32_t {
  ST_PENDING = 0, ST_ACTIVE = 1, ST_BOUNDARY = 2, ST_WEAK_SINK = 3, ST_WEAK_SOURCE = 4,
  ST_NO_EXIT = 5, ST_STOP_ZONE = 6, ST_INACTIVE = 7, ST_UNRELEASED = 8, ST_UNDEFINED = 9
};

// Safety cap on time-loop passes in one cell visit: a pathological record
// (for example a NaN time step) ends as status 9 instead of spinning.
constexpr int64_t kMaxStepsPerVisit = 1000000;
// Safety cap on consecutive cell exits that take no time: a particle sitting
// on a face where the flow turns back (possible when the random walk is
// restricted to fewer dimensions than the flow) can cross back and forth at
// the same instant forever -- the reference's cell loop has no cap.  Past this
// many such exits the particle ends as status 9.
constexpr int kMaxZeroTimeExits = 1000;
// ... and on the cell visits of one particle in one advance call, so that no
// lane can keep crossing faces for ever (a particle crosses about one cell
// per Courant-limited handful of steps; a million visits in one tracking
// interval is far beyond any physical path).
constexpr int kMaxVisitsPerAdvance = 1000000;

}  // namespace mprw
