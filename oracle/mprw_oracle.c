/*
 * mprw_oracle.c -- CPU restatement of MODPATH-RW's random-walk particle
 * tracking (RWPT) hot path.  TEST INFRASTRUCTURE ONLY: the tests use it as
 * the parity checker and bench.py times it as the CPU baseline; the CUDA
 * library never links or calls it.
 *
 * Parity status: UNPINNED by reference golden vectors (the reference ships
 * no tests or outputs and its Fortran cannot be compiled here).  Pinned by:
 * the analytic 1-D Gaussian ADE solution (uniform flow), an independent
 * Python restatement of the RNG, and the known-answer properties listed in
 * the tests.
 *
 * Every function follows the reference line by line, including its quirks:
 *   - the "normal" variate is an Irwin-Hall sum of 12 uniforms minus 6
 *     (TrackSubCell.F90:3631-3663);
 *   - corners 010..111 use the |q| of corner 100 in the isotropic corner
 *     dispersion (TrackSubCell.F90:2622-2677);
 *   - reflection at faces with MassBoundary == 1 (TrackSubCell.F90:1157-1312);
 *   - the single-precision literals 0.1 (dtReductionFactor, :850) and those
 *     of the Newton initial-guess search (:2178-2179, :2451-2554).
 * Paths are relative to the reference project's src/ directory.
 *
 * Build: -O2 -ffp-contract=off (no fused multiply-add, matching gfortran's
 * default x86-64 code), optional -fopenmp.
 */
#include "mprw_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* RNG: xoroshiro128+ streams (lib/rngzig/rng_par_zig.f90)                   */
/* ------------------------------------------------------------------------ */
static const uint64_t XORO_BASE[2] = {0x1DADBEEFBAADD0D0ULL, 0x5BADD0D0DEADBEEFULL};

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* rng_xoroshiro128plus, rng_par_zig.f90:253-281 */
uint64_t orc_xoro_next(uint64_t s[2]) {
  uint64_t s1 = s[0], s2 = s[1];
  uint64_t ival = s1 + s2;
  s2 ^= s1;
  s1 = rotl64(s1, 24) ^ s2 ^ (s2 << 16);
  s2 = rotl64(s2, 37);
  s[0] = s1;
  s[1] = s2;
  return ival;
}

/* rng_jump, rng_par_zig.f90:284-307 (jump by 2^64 calls) */
static void xoro_jump(uint64_t s[2]) {
  static const uint64_t jmp[2] = {0xdf900294d8f554a5ULL, 0x170865df4b3201fcULL};
  uint64_t s1 = 0, s2 = 0;
  for (int i = 0; i < 2; ++i)
    for (int b = 0; b < 64; ++b) {
      if (jmp[i] & (1ULL << b)) {
        s1 ^= s[0];
        s2 ^= s[1];
      }
      (void)orc_xoro_next(s);
    }
  s[0] = s1;
  s[1] = s2;
}

/* rng_zigset seeding, rng_par_zig.f90:175-191: stream k = base jumped k times */
void orc_xoro_seed_stream(int k, uint64_t s[2]) {
  s[0] = XORO_BASE[0];
  s[1] = XORO_BASE[1];
  for (int i = 0; i < k; ++i) xoro_jump(s);
}

/* The streams live for the whole run, as the reference's module state does:
 * rng_init seeds one stream per OpenMP thread once, in
 * pr_InitializeRandomWalk (TrackSubCell.F90:613-620, called from
 * trackingEngine%Initialize), and every tracking interval continues them.
 * orc_xoro_reset() starts a new run (stream k = base jumped k times again). */
#define ORC_MAX_THREADS 512
static uint64_t g_xoro_state[ORC_MAX_THREADS][2];
static int g_xoro_seeded[ORC_MAX_THREADS];

void orc_xoro_reset(void) { memset(g_xoro_seeded, 0, sizeof g_xoro_seeded); }

/* rng_int64_to_real64, rng_par_zig.f90:67-74 */
double orc_xoro_uniform(uint64_t s[2]) {
  uint64_t x = orc_xoro_next(s);
  uint64_t bits = 0x3FF0000000000000ULL | (x >> 12);
  double d;
  memcpy(&d, &bits, 8);
  return d - 1.0;
}

/* pr_GenerateStandardNormalRandomZig, TrackSubCell.F90:3631-3663 */
double orc_xoro_normal_ih12(uint64_t s[2]) {
  double r = 0.0;
  for (int m = 0; m < 12; ++m) r = r + orc_xoro_uniform(s);
  return r - 6.0;
}

/* ------------------------------------------------------------------------ */
/* RNG: Philox4x32-10 (Salmon et al., SC'11), Irwin-Hall(12) on 32-bit words */
/* This is the counter-based stream the GPU library uses; the oracle restates */
/* it independently so trajectories can be compared with identical normals.  */
/* ------------------------------------------------------------------------ */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* One standard "normal" = Irwin-Hall sum of the 12 words of three Philox
 * blocks, scaled by 2^-32, minus 6.  Computed exactly in double:
 * (sum - 6*2^32) * 2^-32 has at most 36 significant bits. */
double orc_philox_normal_ih12(uint64_t seed, uint64_t id, uint64_t *ctr) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint64_t sum = 0;
  for (int b = 0; b < 3; ++b) {
    uint64_t n = (*ctr)++;
    uint32_t c[4] = {(uint32_t)n, (uint32_t)(n >> 32), (uint32_t)id, (uint32_t)(id >> 32)};
    uint32_t o[4];
    orc_philox4x32_10(c, key, o);
    sum += (uint64_t)o[0] + o[1] + o[2] + o[3];
  }
  int64_t centred = (int64_t)sum - (int64_t)25769803776LL; /* 6 * 2^32 */
  return (double)centred * 0x1p-32;
}

typedef struct {
  int kind;
  uint64_t xs[2];   /* kind 0: the thread's xoroshiro stream */
  uint64_t seed, id, *ctr;
} rng_t;

static inline double rng_normal(rng_t *r) {
  if (r->kind == 0) return orc_xoro_normal_ih12(r->xs);
  return orc_philox_normal_ih12(r->seed, r->id, r->ctr);
}

/* ------------------------------------------------------------------------ */
/* Grid helpers (MF6 DIS, RectangularGridDisMf6.f90:122-360)                 */
/* ------------------------------------------------------------------------ */
typedef struct {
  const orc_flow *f;
  int ncpl, ncell;
  int *faceconn;   /* 6*ncell, 1-based neighbour or 0 */
  int *faceidx;    /* 6*ncell, 0-based JA position of the connection or -1 */
  double *cellx, *celly; /* centres as ReadGRB computes them */
  double *celltop;       /* Top(n) after ReadGRB's layer propagation */
  double *sattop;        /* SaturatedTop (FlowModelData.f90:258-279) */
} grid_t;

static void cell_klj(const grid_t *g, int n, int *k, int *i, int *j) {
  int n0 = n - 1;
  *k = n0 / g->ncpl;
  int r = n0 % g->ncpl;
  *i = r / g->f->ncol;
  *j = r % g->f->ncol;
}

static int grid_init(grid_t *g, const orc_flow *f) {
  g->f = f;
  g->ncpl = f->nrow * f->ncol;
  g->ncell = g->ncpl * f->nlay;
  int nc = g->ncell;
  g->faceconn = (int *)calloc((size_t)6 * nc, sizeof(int));
  g->faceidx = (int *)malloc(sizeof(int) * 6 * (size_t)nc);
  g->cellx = (double *)malloc(sizeof(double) * f->ncol);
  g->celly = (double *)malloc(sizeof(double) * f->nrow);
  g->celltop = (double *)malloc(sizeof(double) * nc);
  g->sattop = (double *)malloc(sizeof(double) * nc);
  if (!g->faceconn || !g->faceidx || !g->cellx || !g->celly || !g->celltop || !g->sattop) return -1;
  for (int q = 0; q < 6 * nc; ++q) g->faceidx[q] = -1;
  /* Face assignment from the JA connection list: the diagonal entry comes
   * first, GetPotentialFaceConnectionCount scans entries 2..count
   * (ModflowRectangularGrid.f90:321-343). */
  for (int n = 1; n <= nc; ++n) {
    int k, i, j;
    cell_klj(g, n, &k, &i, &j);
    for (int p = f->ia[n - 1] - 1 + 1; p < f->ia[n] - 1; ++p) {
      int m = f->ja[p];
      int km, im, jm;
      cell_klj(g, m, &km, &im, &jm);
      int face = 0;
      if (km == k && im == i && jm == j - 1) face = 1;
      else if (km == k && im == i && jm == j + 1) face = 2;
      else if (km == k && jm == j && im == i + 1) face = 3;
      else if (km == k && jm == j && im == i - 1) face = 4;
      else if (im == i && jm == j && km == k + 1) face = 5;
      else if (im == i && jm == j && km == k - 1) face = 6;
      if (face) {
        g->faceconn[6 * (n - 1) + face - 1] = m;
        g->faceidx[6 * (n - 1) + face - 1] = p;
      }
    }
  }
  /* X(1)=0, X(n+1)=X(n)+DX(n); Y(1)=sum DY, Y(n+1)=Y(n)-DY(n);
   * CellX=(X(c)+X(c+1))/2 (RectangularGridDisMf6.f90:301-340). */
  double X = 0.0;
  for (int c = 0; c < f->ncol; ++c) {
    double Xn = X + f->delr[c];
    g->cellx[c] = (X + Xn) / 2.0;
    X = Xn;
  }
  double Y = 0.0;
  for (int r = 0; r < f->nrow; ++r) Y = Y + f->delc[r];
  for (int r = 0; r < f->nrow; ++r) {
    double Yn = Y - f->delc[r];
    g->celly[r] = (Y + Yn) / 2.0;
    Y = Yn;
  }
  for (int n = 0; n < nc; ++n) g->celltop[n] = (n < g->ncpl) ? f->top[n] : f->botm[n - g->ncpl];
  for (int n = 0; n < nc; ++n) {
    double st = g->celltop[n];
    int ct = f->celltype ? f->celltype[n] : 0;
    if (ct == 1 && f->heads && f->iboundts[n] != 0) {
      if (f->heads[n] <= g->celltop[n] && f->heads[n] >= f->botm[n]) st = f->heads[n];
    }
    g->sattop[n] = st;
  }
  return 0;
}

static void grid_free(grid_t *g) {
  free(g->faceconn); free(g->faceidx); free(g->cellx); free(g->celly);
  free(g->celltop); free(g->sattop);
}

/* ------------------------------------------------------------------------ */
/* Cell buffer: SetMassTransportDataUnstructured (ModpathCellData.f90:674-1098) */
/* ------------------------------------------------------------------------ */
typedef struct {
  int CellNumber;           /* 0 => reset buffer */
  double DX, DY, Top, Bottom, Head;
  int LayerType, IboundTS, Zone;
  double Porosity, Retardation, SourceFlow, SinkFlow;
  double Q[6];
  int SubFaceConn[6], MassBoundary[6];
  double alphaLH, alphaTH, alphaLV, alphaTV, dMEff;
  int dry, partiallyDry;
} cdata;

static void fill_cell(const grid_t *g, int n, cdata *c) {
  const orc_flow *f = g->f;
  int k, i, j;
  cell_klj(g, n, &k, &i, &j);
  memset(c, 0, sizeof(*c));
  int n0 = n - 1;
  c->CellNumber = n;
  c->DX = f->delr[j];
  c->DY = f->delc[i];
  c->Bottom = f->botm[n0];
  c->Top = g->celltop[n0];
  c->Zone = f->zones ? f->zones[n0] : 0;
  c->LayerType = f->celltype ? f->celltype[n0] : 0;
  c->Head = f->heads ? f->heads[n0] : 0.0;
  c->IboundTS = f->iboundts[n0];
  c->Porosity = f->porosity[n0];
  c->Retardation = f->retardation[n0];
  c->SourceFlow = f->source_flow ? f->source_flow[n0] : 0.0;
  c->SinkFlow = f->sink_flow ? f->sink_flow[n0] : 0.0;
  int sbc[6];
  for (int face = 0; face < 6; ++face) {
    int conn = g->faceconn[6 * n0 + face];
    c->Q[face] = 0.0;
    c->SubFaceConn[face] = 0;
    sbc[face] = 1; /* SubFaceBoundaryCounts reset value (ModpathCellData.f90:439) */
    if (conn > 0) {
      c->SubFaceConn[face] = conn;
      sbc[face] = (f->iboundts[conn - 1] == 0) ? 1 : 0;
      c->MassBoundary[face] = f->icboundts ? f->icboundts[conn - 1] : 0;
      double fj = f->flowja[g->faceidx[6 * n0 + face]];
      /* Q1=+, Q2=-, Q3=+, Q4=-, Q5=+, Q6=- (ModpathCellData.f90:899-949) */
      c->Q[face] = (face % 2 == 0) ? fj : -fj;
    } else {
      c->MassBoundary[face] = f->default_icbound;
    }
  }
  /* boundary flows (ModpathCellData.f90:951-1077) */
  if (f->bflow) {
    for (int face = 0; face < 6; ++face) {
      double bf = f->bflow[6 * n0 + face];
      if (bf != 0.0) {
        if (sbc[face] > 0) {
          double flow = bf / sbc[face];
          int conn = c->SubFaceConn[face];
          if (conn == 0 || f->iboundts[conn - 1] == 0) c->Q[face] = (face % 2 == 0) ? flow : -flow;
        } else {
          if (bf > 0.0) c->SourceFlow = c->SourceFlow + bf;
          else c->SinkFlow = c->SinkFlow + bf;
        }
      }
    }
  }
  /* FillDispersionParameters{Uniform,Distributed} (ParticleTrackingEngine.f90:535-570) */
  int di = f->uniform_dispersion ? 0 : n0;
  c->alphaLH = f->alpha_l[di];
  c->alphaTH = f->alpha_t[di];
  c->alphaLV = f->alpha_lv ? f->alpha_lv[di] : c->alphaLH;
  c->alphaTV = f->alpha_tv ? f->alpha_tv[di] : c->alphaTH;
  c->dMEff = f->dm_eff[di];
}

/* pr_GetDZRW, ModpathCellData.f90:3208-3256 (sets dry / partiallyDry) */
static double get_dzrw(cdata *c) {
  double dz = c->Top - c->Bottom;
  double dzc = c->Top - c->Bottom;
  c->dry = 0;
  c->partiallyDry = 0;
  if (c->LayerType == 1) {
    if (c->Head < c->Top) {
      dz = c->Head - c->Bottom;
      c->dry = 0;
      c->partiallyDry = 1;
      if ((dz <= 0.0) || ((c->Head - c->Bottom) / dzc < 0.01)) {
        dz = c->Top - c->Bottom;
        c->dry = 1;
        c->partiallyDry = 0;
        int anyflow = 0;
        for (int q = 0; q < 6; ++q) anyflow |= (c->Q[q] != 0.0);
        if (anyflow) {
          c->dry = 0;
          c->partiallyDry = 1;
        }
      }
    }
  }
  return dz;
}

/* pr_VerifyDryCell, ModpathCellData.f90:3161-3205: returns partiallyDry */
static int verify_dry_partial(const cdata *c) {
  int pd = 0;
  if (c->LayerType == 1 && c->Head < c->Top) {
    pd = 1;
    if (c->Head - c->Bottom <= 0.0) {
      int anyflow = 0;
      for (int q = 0; q < 6; ++q) anyflow |= (c->Q[q] != 0.0);
      pd = anyflow;
    }
  }
  return pd;
}

/* ------------------------------------------------------------------------ */
/* Sub-cell buffer + corner variables                                         */
/* ------------------------------------------------------------------------ */
typedef struct {
  double DX, DY, DZ;
  double VX1, VX2, VY1, VY2, VZ1, VZ2;
  int Connection[6], MassBoundary[6];
  double Porosity, Retardation, alphaLH, alphaTH, alphaLV, alphaTV, dMEff;
  int dry, partiallyDry;
  double qC[8][4];   /* qCorner000..111 (qx,qy,qz,|q|) */
  double phiC[8];    /* porosity000..111 */
  double D[9][8];    /* Dxxx,Dyyy,Dzzz,Dxyx,Dxzx,Dxyy,Dyzy,Dxzz,Dyzz */
} subcell_t;

/* pr_FillMassSubCellDataBuffer, ModpathCellData.f90:2522-2684 */
static void fill_subcell(cdata *c, int backward, subcell_t *s) {
  memset(s, 0, sizeof(*s));
  s->DX = c->DX / 1.0;
  s->DY = c->DY / 1.0;
  s->DZ = get_dzrw(c);
  s->dry = c->dry;
  s->partiallyDry = c->partiallyDry;
  double sign = 1.0;
  if (backward) sign = -sign;
  s->VX1 = sign * c->Q[0] / s->DY / s->DZ / c->Porosity / c->Retardation;
  s->VX2 = sign * c->Q[1] / s->DY / s->DZ / c->Porosity / c->Retardation;
  s->VY1 = sign * c->Q[2] / s->DX / s->DZ / c->Porosity / c->Retardation;
  s->VY2 = sign * c->Q[3] / s->DX / s->DZ / c->Porosity / c->Retardation;
  s->VZ1 = sign * c->Q[4] / s->DX / s->DY / c->Porosity / c->Retardation;
  s->VZ2 = sign * c->Q[5] / s->DX / s->DY / c->Porosity / c->Retardation;
  for (int q = 0; q < 6; ++q) {
    s->Connection[q] = c->SubFaceConn[q];
    s->MassBoundary[q] = c->MassBoundary[q];
  }
  s->Porosity = c->Porosity;
  s->Retardation = c->Retardation;
  s->alphaLH = c->alphaLH;
  s->alphaTH = c->alphaTH;
  s->alphaLV = c->alphaLV;
  s->alphaTV = c->alphaTV;
  s->dMEff = c->dMEff;
}

/* Neighbour buffer order (ModpathCellData.f90:2877-2895):
 * 1 dc1, 2 ic13, 3 ic14, 4 dc2, 5 ic23, 6 ic24, 7 dc3, 8 ic35, 9 ic36,
 * 10 dc4, 11 ic45, 12 ic46, 13 dc5, 14 ic51, 15 ic52, 16 dc6, 17 ic61, 18 ic62.
 * pr_FillNeighborCellDataStructured, ParticleTrackingEngine.f90:2009-2126. */
static void fill_neighbours(const grid_t *g, int n, cdata nb[18]) {
  static const int sub[6][2] = {{3, 4}, {3, 4}, {5, 6}, {5, 6}, {1, 2}, {1, 2}};
  int counter = 0;
  for (int face = 1; face <= 6; ++face) {
    int conn = g->faceconn[6 * (n - 1) + face - 1];
    if (conn > 0) {
      fill_cell(g, conn, &nb[counter]);
      for (int s = 0; s < 2; ++s) {
        int c2 = g->faceconn[6 * (conn - 1) + sub[face - 1][s] - 1];
        if (c2 > 0) fill_cell(g, c2, &nb[counter + 1 + s]);
        else nb[counter + 1 + s].CellNumber = 0;
      }
    } else {
      nb[counter].CellNumber = 0;
      nb[counter + 1].CellNumber = 0;
      nb[counter + 2].CellNumber = 0;
    }
    counter += 3;
  }
}

/* pr_SetCornerComponentsIndexes, TrackSubCell.F90:4142-4224 */
static const int CXI[8][4] = {{7, 8, 13, 1}, {7, 8, 13, 2}, {10, 11, 13, 1}, {10, 11, 13, 2},
                              {7, 9, 16, 1}, {7, 9, 16, 2}, {10, 12, 16, 1}, {10, 12, 16, 2}};
static const int CYI[8][4] = {{1, 13, 14, 3}, {4, 13, 15, 3}, {1, 13, 14, 4}, {4, 13, 15, 4},
                              {1, 16, 17, 3}, {4, 16, 18, 3}, {1, 16, 17, 4}, {4, 16, 18, 4}};
static const int CZI[8][4] = {{1, 2, 7, 5}, {4, 5, 7, 5}, {1, 3, 10, 5}, {4, 6, 10, 5},
                              {1, 2, 7, 6}, {4, 5, 7, 6}, {1, 3, 10, 6}, {4, 6, 10, 6}};
/* pr_SetCornerPorosityIndexes, TrackSubCell.F90:4329-4363 (kept as written) */
static const int CPI[8][6] = {{1, 2, 7, 8, 13, 14}, {4, 5, 7, 8, 13, 15}, {1, 3, 10, 11, 13, 14},
                              {4, 6, 10, 12, 16, 18}, {1, 2, 7, 9, 16, 17}, {4, 5, 7, 9, 16, 18},
                              {1, 3, 10, 12, 16, 17}, {4, 6, 10, 11, 13, 15}};

/* pr_ComputeCornerVariables, TrackSubCell.F90:3667-3850 */
static void corner_variables(const grid_t *g, int n, cdata *center, subcell_t *s, int uniform_porosity,
                             int dispersion_model) {
  cdata nb[18];
  fill_neighbours(g, n, nb);
  double nflow[18][6], narea[18][3], nvol[18], nphi[18];
  memset(nflow, 0, sizeof(nflow));
  memset(narea, 0, sizeof(narea));
  memset(nvol, 0, sizeof(nvol));
  memset(nphi, 0, sizeof(nphi));
  /* pr_FillNeighborSubCellVariables, unrefined branch, TrackSubCell.F90:3886-3906 */
  for (int q = 0; q < 18; ++q) {
    if (nb[q].CellNumber == 0) continue;
    for (int fc = 0; fc < 6; ++fc) nflow[q][fc] = nb[q].Q[fc];
    double dz = get_dzrw(&nb[q]);
    narea[q][0] = nb[q].DY * dz;
    narea[q][1] = nb[q].DX * dz;
    narea[q][2] = nb[q].DX * nb[q].DY;
    nvol[q] = nb[q].DX * nb[q].DY * get_dzrw(&nb[q]);
    nphi[q] = nb[q].Porosity;
  }
  /* pr_ComputeCornerDischarge / GetInterpolatedCornerDischarge, :4016-4138 */
  const double *cf = center->Q;
  for (int corner = 0; corner < 8; ++corner) {
    double sumArea, sumFlow;
    sumArea = s->DY * s->DZ;
    sumFlow = cf[CXI[corner][3] - 1];
    for (int m = 0; m < 3; ++m) {
      sumArea = sumArea + narea[CXI[corner][m] - 1][0];
      sumFlow = sumFlow + nflow[CXI[corner][m] - 1][CXI[corner][3] - 1];
    }
    s->qC[corner][0] = sumFlow / sumArea;
    sumArea = s->DX * s->DZ;
    sumFlow = cf[CYI[corner][3] - 1];
    for (int m = 0; m < 3; ++m) {
      sumArea = sumArea + narea[CYI[corner][m] - 1][1];
      sumFlow = sumFlow + nflow[CYI[corner][m] - 1][CYI[corner][3] - 1];
    }
    s->qC[corner][1] = sumFlow / sumArea;
    sumArea = s->DX * s->DY;
    sumFlow = cf[CZI[corner][3] - 1];
    for (int m = 0; m < 3; ++m) {
      sumArea = sumArea + narea[CZI[corner][m] - 1][2];
      sumFlow = sumFlow + nflow[CZI[corner][m] - 1][CZI[corner][3] - 1];
    }
    s->qC[corner][2] = sumFlow / sumArea;
  }
  for (int corner = 0; corner < 8; ++corner) {
    double *q = s->qC[corner];
    q[3] = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
  }
  /* corner porosity, :4227-4326 */
  for (int corner = 0; corner < 8; ++corner) {
    if (uniform_porosity) {
      s->phiC[corner] = s->Porosity;
    } else {
      double sumVolume = s->DX * s->DY * s->DZ;
      double sumWP = s->Porosity * sumVolume;
      for (int m = 0; m < 6; ++m) {
        int q = CPI[corner][m] - 1;
        sumVolume = sumVolume + nvol[q];
        sumWP = sumWP + nvol[q] * nphi[q];
      }
      s->phiC[corner] = sumWP / sumVolume;
    }
  }
  /* qprod, :3720-3823 */
  double qprod[8][8];
  for (int corner = 0; corner < 8; ++corner) {
    double *qp = qprod[corner];
    const double *q = s->qC[corner];
    for (int m = 0; m < 8; ++m) qp[m] = 0.0;
    if (q[3] > 0.0) {
      qp[0] = q[0] * q[0];
      qp[1] = q[0] * q[1];
      qp[2] = q[0] * q[2];
      qp[3] = q[1] * q[1];
      qp[4] = q[1] * q[2];
      qp[5] = q[2] * q[2];
      qp[6] = qp[0] + qp[3];
      if (qp[6] > 0.0) qp[7] = qp[5] / qp[6];
      for (int m = 0; m < 7; ++m) qp[m] = qp[m] / q[3];
    }
  }
  if (dispersion_model == 1) {
    /* pr_CornerDispersionAxisymmetric, :3117-3303: per corner, alphaL/alphaT
     * blended with cosinesq = qz**2/|q| (as written: over |q|, not |q|**2);
     * Dxyx uses the xx product (as written) */
    const double aLH = s->alphaLH, aLV = s->alphaLV, aTH = s->alphaTH, aTV = s->alphaTV, dm = s->dMEff;
    for (int corner = 0; corner < 8; ++corner) {
      const double *q = s->qC[corner], *qp = qprod[corner];
      const double pD = s->phiC[corner] * dm;
      double cosinesq = 0.0;
      if (q[3] > 0.0) cosinesq = q[2] * q[2] / q[3];
      const double aL = aLH + cosinesq * (aLV - aLH);
      const double aT = aTV + cosinesq * (aTH - aTV);
      const double aLmT = aL - aT;
      s->D[0][corner] = pD + (aL + aT * qp[7]) * qp[0] + aTH * qp[3] * (1.0 + qp[7]);
      s->D[1][corner] = pD + aTH * qp[0] * (1.0 + qp[7]) + qp[3] * (aL + aT * qp[7]);
      s->D[3][corner] = (aL - aTH * (1.0 + qp[7]) + aT * qp[7]) * qp[0];
      s->D[5][corner] = s->D[3][corner];
      s->D[2][corner] = pD + aT * qp[6] + aL * qp[5];
      s->D[4][corner] = aLmT * qp[2];
      s->D[6][corner] = aLmT * qp[4];
      s->D[7][corner] = s->D[4][corner];
      s->D[8][corner] = s->D[6][corner];
    }
    return;
  }
  /* pr_CornerDispersionLinearIsotropic, :2557-2691 (quirk: corners 3..8 use
   * qCorner100(4)) */
  double dMEff = s->dMEff, aL = s->alphaLH, aT = s->alphaTH;
  double aLmT = aL - aT;
  for (int corner = 0; corner < 8; ++corner) {
    double qn = (corner == 0) ? s->qC[0][3] : s->qC[1][3];
    double aTQ = aT * qn + s->phiC[corner] * dMEff;
    const double *qp = qprod[corner];
    s->D[0][corner] = aTQ + aLmT * qp[0];
    s->D[1][corner] = aTQ + aLmT * qp[3];
    s->D[2][corner] = aTQ + aLmT * qp[5];
    s->D[3][corner] = aLmT * qp[1];
    s->D[4][corner] = aLmT * qp[2];
    s->D[5][corner] = s->D[3][corner];
    s->D[6][corner] = aLmT * qp[4];
    s->D[7][corner] = s->D[4][corner];
    s->D[8][corner] = s->D[6][corner];
  }
}

/* ------------------------------------------------------------------------ */
/* Per-step helpers (TrackSubCell.F90)                                        */
/* ------------------------------------------------------------------------ */
/* corner order: 0=000 1=100 2=010 3=110 4=001 5=101 6=011 7=111 */
static double tri_dx(const subcell_t *s, double x, double y, double z, const double *v) {
  (void)x;
  double v00 = (v[1] - v[0]) / s->DX, v01 = (v[5] - v[4]) / s->DX;
  double v10 = (v[3] - v[2]) / s->DX, v11 = (v[7] - v[6]) / s->DX;
  double v0 = (1.0 - y) * v00 + y * v10;
  double v1 = (1.0 - y) * v01 + y * v11;
  return (1.0 - z) * v0 + z * v1;
}
static double tri_dy(const subcell_t *s, double x, double y, double z, const double *v) {
  (void)y;
  double v00 = (v[2] - v[0]) / s->DY, v01 = (v[6] - v[4]) / s->DY;
  double v10 = (v[3] - v[1]) / s->DY, v11 = (v[7] - v[5]) / s->DY;
  double v0 = (1.0 - x) * v00 + x * v10;
  double v1 = (1.0 - x) * v01 + x * v11;
  return (1.0 - z) * v0 + z * v1;
}
static double tri_dz(const subcell_t *s, double x, double y, double z, const double *v) {
  (void)z;
  double v00 = (v[4] - v[0]) / s->DZ, v01 = (v[6] - v[2]) / s->DZ;
  double v10 = (v[5] - v[1]) / s->DZ, v11 = (v[7] - v[3]) / s->DZ;
  double v0 = (1.0 - x) * v00 + x * v10;
  double v1 = (1.0 - x) * v01 + x * v11;
  return (1.0 - y) * v0 + y * v1;
}
/* pr_Trilinear, :4546-4580 */
static double trilinear(double x, double y, double z, const double v[8]) {
  double v00 = (1.0 - x) * v[0] + x * v[1];
  double v01 = (1.0 - x) * v[4] + x * v[5];
  double v10 = (1.0 - x) * v[2] + x * v[3];
  double v11 = (1.0 - x) * v[6] + x * v[7];
  double v0 = (1.0 - y) * v00 + y * v10;
  double v1 = (1.0 - y) * v01 + y * v11;
  return (1.0 - z) * v0 + z * v1;
}

/* pr_DispersionDivergence, :2695-2818 */
static void divergence(const subcell_t *s, double x, double y, double z, double *dx, double *dy, double *dz) {
  double dDxxdx = tri_dx(s, x, y, z, s->D[0]);
  double dDyydy = tri_dy(s, x, y, z, s->D[1]);
  double dDzzdz = tri_dz(s, x, y, z, s->D[2]);
  double dDxydx = tri_dx(s, x, y, z, s->D[3]);
  double dDxzdx = tri_dx(s, x, y, z, s->D[4]);
  double dDxydy = tri_dy(s, x, y, z, s->D[5]);
  double dDyzdy = tri_dy(s, x, y, z, s->D[6]);
  double dDxzdz = tri_dz(s, x, y, z, s->D[7]);
  double dDyzdz = tri_dz(s, x, y, z, s->D[8]);
  *dx = (dDxxdx + dDxydy + dDxzdz) / s->Porosity / s->Retardation;
  *dy = (dDxydx + dDyydy + dDyzdz) / s->Porosity / s->Retardation;
  *dz = (dDxzdx + dDyzdy + dDzzdz) / s->Porosity / s->Retardation;
}

/* pr_DisplacementRandomDischarge{,2D,1D}, :2821-3113; axisymmetric model:
 * pr_RWPTDisplacementsAxisymmetric :750-806 blends alphaL/alphaT with the
 * particle's velocity (cosinesq = vz**2/|v|, as written) and
 * pr_DisplacementRandomDischargeAxisymmetric{,2D,1D} :3306-3604 use alphaTH
 * for the horizontal transverse terms */
static void random_displacement(const subcell_t *s, const orc_options *o, const int *dims, int ndim,
                                double x, double y, double z, double vx, double vy, double vz, rng_t *rng,
                                double *dBx, double *dBy, double *dBz) {
  double aL = s->alphaLH, aT = s->alphaTH, dm = s->dMEff, R = s->Retardation;
  double aTH = aT;  /* horizontal transverse term of the axisymmetric model */
  if (o->dispersion_model == 1) {
    const double vnorm = sqrt(pow(vx, 2.0) + pow(vy, 2.0) + pow(vz, 2.0));
    double cosinesq = 0.0;
    if (vnorm > 0.0) cosinesq = pow(vz, 2.0) / vnorm;
    aL = s->alphaLH + cosinesq * (s->alphaLV - s->alphaLH);
    aT = s->alphaTV + cosinesq * (s->alphaTH - s->alphaTV);
    aTH = s->alphaTH;
  }
  double vc[3][8];
  for (int c = 0; c < 8; ++c)
    for (int m = 0; m < 3; ++m) vc[m][c] = s->qC[c][m] / s->phiC[c];
  (void)o;
  if (ndim == 3) {
    double vBx = trilinear(x, y, z, vc[0]);
    double vBy = trilinear(x, y, z, vc[1]);
    double vBz = trilinear(x, y, z, vc[2]);
    double vBnorm = sqrt(vBx * vBx + vBy * vBy + vBz * vBz);
    double vBnormxy = sqrt(vBx * vBx + vBy * vBy);
    double B11 = 0, B12 = 0, B13 = 0, B21 = 0, B22 = 0, B23 = 0, B31 = 0, B32 = 0;
    if (vBnorm > 0.0) {
      B11 = vBx * sqrt(2 * (aL * vBnorm + dm) / R) / vBnorm;
      B21 = vBy * sqrt(2 * (aL * vBnorm + dm) / R) / vBnorm;
      B31 = vBz * sqrt(2 * (aL * vBnorm + dm) / R) / vBnorm;
      B32 = vBnormxy * sqrt(2 * (aT * vBnorm + dm) / R) / vBnorm;
      if (vBnormxy > 0.0) {
        B12 = -(vBx * vBz * sqrt(2 * (aT * vBnorm + dm) / R) / vBnorm / vBnormxy);
        B13 = -(vBy * sqrt(2 * (aTH * vBnorm + dm) / R) / vBnormxy);
        B22 = -(vBy * vBz * sqrt(2 * (aT * vBnorm + dm) / R) / vBnorm / vBnormxy);
        B23 = vBx * sqrt(2 * (aTH * vBnorm + dm) / R) / vBnormxy;
      }
    }
    double rx = rng_normal(rng), ry = rng_normal(rng), rz = rng_normal(rng);
    *dBx = B11 * rx + B12 * ry + B13 * rz;
    *dBy = B21 * rx + B22 * ry + B23 * rz;
    *dBz = B31 * rx + B32 * ry;
  } else if (ndim == 2) {
    int d1 = dims[0], d2 = dims[1];
    double vB1 = trilinear(x, y, z, vc[d1]);
    double vB2 = trilinear(x, y, z, vc[d2]);
    double vBnorm = sqrt(vB1 * vB1 + vB2 * vB2);
    double B11 = 0, B12 = 0, B21 = 0, B22 = 0;
    if (vBnorm > 0.0) {
      B11 = vB1 * sqrt(2 * (aL * vBnorm + dm) / R) / vBnorm;
      B21 = vB2 * sqrt(2 * (aL * vBnorm + dm) / R) / vBnorm;
      B12 = -(vB2 * sqrt(2 * (aTH * vBnorm + dm) / R) / vBnorm);
      B22 = vB1 * sqrt(2 * (aTH * vBnorm + dm) / R) / vBnorm;
    }
    double r1 = rng_normal(rng), r2 = rng_normal(rng);
    double dB[3] = {0, 0, 0};
    dB[d1] = B11 * r1 + B12 * r2;
    dB[d2] = B21 * r1 + B22 * r2;
    *dBx = dB[0]; *dBy = dB[1]; *dBz = dB[2];
  } else {
    int d1 = dims[0];
    double vB1 = trilinear(x, y, z, vc[d1]);
    double vBnorm = sqrt(vB1 * vB1);
    double B11 = 0;
    if (vBnorm > 0.0) B11 = sqrt(2 * (aL * vBnorm + dm) / R);
    double r1 = rng_normal(rng);
    double dB[3] = {0, 0, 0};
    dB[d1] = B11 * r1;
    *dBx = dB[0]; *dBy = dB[1]; *dBz = dB[2];
  }
}

/* pr_AdvectionDisplacementEulerian / Exponential, :1487-1573 */
static void advection(const subcell_t *s, int kind, double dt, double vx, double vy, double vz,
                      double *ax, double *ay, double *az) {
  if (kind == 2) {
    *ax = vx * dt;
    *ay = vy * dt;
    *az = vz * dt;
    return;
  }
  const double dvtol = 1.0e-10;
  double dvxdx = (s->VX2 - s->VX1) / s->DX;
  *ax = (fabs(dvxdx) > dvtol) ? vx * (exp(dvxdx * dt) - 1.0) / dvxdx : vx * dt;
  double dvydy = (s->VY2 - s->VY1) / s->DY;
  *ay = (fabs(dvydy) > dvtol) ? vy * (exp(dvydy * dt) - 1.0) / dvydy : vy * dt;
  double dvzdz = (s->VZ2 - s->VZ1) / s->DZ;
  *az = (fabs(dvzdz) > dvtol) ? vz * (exp(dvzdz * dt) - 1.0) / dvzdz : vz * dt;
}

/* pr_DetectExitFaceAndUpdateTimeStepQuadratic, one axis (:1622-1710) */
/* returns 1 if the routine must return immediately (exitFace/dt already set) */
static int quad_axis(double npos, double pos, double d, double v, double divD, double dB,
                     int faceLo, int faceHi, double dt, double *dtaxis, int *exitAxis,
                     int *exitFace, double *dtout) {
  double dInterface;
  if (npos > 1.0) {
    dInterface = d * (1.0 - pos);
    *exitAxis = faceHi;
  } else {
    dInterface = -d * pos;
    *exitAxis = faceLo;
  }
  if (dInterface == 0.0) {
    *exitFace = *exitAxis;
    *dtout = 0.0;
    return 1;
  }
  double A = v + divD, B = dB;
  double arg = B * B + 4 * dInterface * A;
  if ((arg >= 0.0) && (A != 0.0)) {
    double zs = sqrt(arg);
    double z1 = (-B + zs) / (2 * A);
    double z2 = (-B - zs) / (2 * A);
    if (z1 > 0.0 || z2 > 0.0) {
      double zm;
      if (z1 > 0.0 && z2 > 0.0) zm = (z1 < z2) ? z1 : z2;
      else zm = (z1 > 0.0) ? z1 : z2;
      *dtaxis = zm * zm;
      if (*dtaxis == 0.0) {
        *exitFace = *exitAxis;
        *dtout = 0.0;
        return 1;
      }
    } else if (z1 == 0.0 || z2 == 0.0) {
      *exitFace = *exitAxis;
      *dtout = 0.0;
      return 1;
    }
  } else if (A == 0.0) {
    if (B != 0.0) {
      double q = dInterface / B;
      *dtaxis = q * q;
      if (*dtaxis == 0.0) {
        *exitFace = *exitAxis;
        *dtout = 0.0;
        return 1;
      }
    }
  }
  if (*dtaxis > dt) *dtaxis = 0.0;
  return 0;
}

/* ---- EXPONENTIAL advection: Newton-Raphson exit time (:1895-2554) ---- */
static void nr_vars(double dt, double v, double v1, double v2, double dx, double dI, double divD, double dB,
                    double *f0, double *f1, double *f2, double *f3) {
  if (dt == 0.0) return;
  const double dvtol = 1.0e-10;
  *f0 = 0; *f1 = 0; *f2 = 0; *f3 = 0;
  double dvdx = (v2 - v1) / dx, dAdv;
  if (fabs(dvdx) > dvtol) dAdv = v * (exp(dvdx * dt) - 1.0) / dvdx;
  else dAdv = v * dt;
  *f0 = dAdv + divD * dt + dB * sqrt(dt) - dI;
  *f1 = v * exp(dvdx * dt) + divD + 0.5 * dB / sqrt(dt);
  *f2 = dvdx * v * exp(dvdx * dt) - 0.25 * dB * pow(dt, -1.5);
  *f3 = dvdx * dvdx * v * exp(dvdx * dt) + 0.375 * dB * pow(dt, -2.5);
}
static double conv_g(double f0, double f1, double f2) { return fabs(f2 * f0 / (f1 * f1)); }
static double conv_gder(double f0, double f1, double f2, double f3) {
  double gna = f2 * f0 / (f1 * f1);
  double gpp = -2.0 * (f0 * (f2 * f2)) / (f1 * f1 * f1) + (f1 * f2 + f0 * f3) / (f1 * f1);
  return gna / fabs(gna) * gpp;
}
static double p10(int e) { /* 10d0**e for integer e (exact for |e| <= 22) */
  double r = 1.0;
  for (int i = 0; i < (e < 0 ? -e : e); ++i) r *= 10.0;
  return e < 0 ? 1.0 / r : r;
}
/* pr_SetInitialGuess, :2162-2448 */
static double nr_initial_guess(double dt, double v, double v1, double v2, double dx, double dI, double divD,
                               double dB) {
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
    dtfraction = p10(-8 + gcount);
    dt0 = dt * dtfraction;
    nr_vars(dt0, v, v1, v2, dx, dI, divD, dB, &f0, &f1, &f2, &f3);
    gprim = conv_g(f0, f1, f2);
    if (gprim < gprimmin) {
      gprimmin = gprim;
      mindtfrac = dtfraction;
    }
  }
  if ((gprim < 1) && (gcount == 1)) dtoldfraction = 1e-8;
  else if (gprim < 1) dtoldfraction = p10(-8 + gcount - 1);
  else {
    dtfraction = mindtfrac;
    dtoldfraction = 0.5 * dtfraction / 10.0;
  }
  dtnew = dtfraction * dt;
  dtold = dtoldfraction * dt;
  nr_vars(dtnew, v, v1, v2, dx, dI, divD, dB, &f0, &f1, &f2, &f3);
  gprim = conv_g(f0, f1, f2);
  if (gprim < 0.5) return dtnew;
  gprimnew = 10.0;
  gprim = 10.0;
  ccount = bcount = zcount = rcount = counter = 0;
  while (counter < maxter) {
    counter = counter + 1;
    nr_vars(dtold, v, v1, v2, dx, dI, divD, dB, &f0, &f1, &f2, &f3);
    gprimder = conv_gder(f0, f1, f2, f3);
    nr_vars(dtnew, v, v1, v2, dx, dI, divD, dB, &f0, &f1, &f2, &f3);
    gprimdernew = conv_gder(f0, f1, f2, f3);
    gprim = conv_g(f0, f1, f2);
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
    nr_vars(dtnew, v, v1, v2, dx, dI, divD, dB, &f0, &f1, &f2, &f3);
    gprimnew = conv_g(f0, f1, f2);
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
    if (counter > maxter) break;
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
    nr_vars(dt0, v, v1, v2, dx, dI, divD, dB, &f0, &f1, &f2, &f3);
    gprim = conv_g(f0, f1, f2);
    if (gprim < gprimmin) {
      gprimmin = gprim;
      mindtfrac = dtfraction;
    }
  }
  if (gprimmin < 1) dtnew = dt * mindtfrac;
  if ((dtnew <= 0.0) && (fabs(v) > 0.0)) dtnew = fabs(dI / v);
  return dtnew;
}
/* NewtonRaphsonTimeStepExponentialAdvection, :2451-2554 */
static double nr_time_step(double dt, double v, double v1, double v2, double dx, double dI, double divD,
                           double dB) {
  const double dvtol = 1.0e-10;
  const double nrtol = (double)1e-6f;
  const int maxIter = 50;
  double nrerror = 1e6, dvdx = (v2 - v1) / dx, dAdv, f0, f1;
  double dt0 = nr_initial_guess(dt, v, v1, v2, dx, dI, divD, dB);
  if (dt0 == 0.0) return 0.0;
  int countIter = 0;
  while ((fabs(nrerror / dt0) > nrtol) && (countIter < maxIter)) {
    countIter = countIter + 1;
    if (fabs(dvdx) > dvtol) dAdv = v * (exp(dvdx * dt0) - 1.0) / dvdx;
    else dAdv = v * dt0;
    f0 = dAdv + divD * dt0 + dB * sqrt(dt0) - dI;
    f1 = v * exp(dvdx * dt0) + divD + 0.5 * dB / sqrt(dt0);
    nrerror = -f0 / f1;
    dt0 = dt0 + nrerror;
    if (dt0 < 0.0) dt0 = -(double)0.9f * dt0;
  }
  if (dt0 > dt) return dt;
  if ((countIter == maxIter) && (fabs(nrerror / dt0) > nrtol)) return 0.0;
  return dt0;
}
static int newton_axis(double npos, double pos, double d, double v, double v1, double v2, double divD, double dB,
                       int faceLo, int faceHi, double dt, double *dtaxis, int *exitAxis, int *exitFace,
                       double *dtout) {
  double dInterface;
  if (npos > 1.0) {
    dInterface = d * (1.0 - pos);
    *exitAxis = faceHi;
  } else {
    dInterface = -d * pos;
    *exitAxis = faceLo;
  }
  if (dInterface == 0.0) {
    *exitFace = *exitAxis;
    *dtout = 0.0;
    return 1;
  }
  *dtaxis = nr_time_step(dt, v, v1, v2, d, dInterface, divD, dB);
  if (*dtaxis > dt) *dtaxis = 0.0;
  return 0;
}

/* ExitFaceAndUpdateTimeStep (Quadratic :1576-1892, Newton :1895-2079) */
static void exit_face_update(const subcell_t *s, int kind, double x, double y, double z, double nx, double ny,
                             double nz, double vx, double vy, double vz, double ddx, double ddy, double ddz,
                             double bx, double by, double bz, double *t, double *dt, double dtxyz[3],
                             int *exitFace) {
  int efx = 0, efy = 0, efz = 0;
  *t = *t - *dt;
  if ((nx > 1.0) || (nx < 0.0)) {
    int r = (kind == 2) ? quad_axis(nx, x, s->DX, vx, ddx, bx, 1, 2, *dt, &dtxyz[0], &efx, exitFace, dt)
                        : newton_axis(nx, x, s->DX, vx, s->VX1, s->VX2, ddx, bx, 1, 2, *dt, &dtxyz[0], &efx,
                                      exitFace, dt);
    if (r) return;
  }
  if ((ny > 1.0) || (ny < 0.0)) {
    int r = (kind == 2) ? quad_axis(ny, y, s->DY, vy, ddy, by, 3, 4, *dt, &dtxyz[1], &efy, exitFace, dt)
                        : newton_axis(ny, y, s->DY, vy, s->VY1, s->VY2, ddy, by, 3, 4, *dt, &dtxyz[1], &efy,
                                      exitFace, dt);
    if (r) return;
  }
  if ((nz > 1.0) || (nz < 0.0)) {
    int r = (kind == 2) ? quad_axis(nz, z, s->DZ, vz, ddz, bz, 5, 6, *dt, &dtxyz[2], &efz, exitFace, dt)
                        : newton_axis(nz, z, s->DZ, vz, s->VZ1, s->VZ2, ddz, bz, 5, 6, *dt, &dtxyz[2], &efz,
                                      exitFace, dt);
    if (r) return;
  }
  if (dtxyz[0] == 0.0 && dtxyz[1] == 0.0 && dtxyz[2] == 0.0) {
    *t = *t + *dt;
    return;
  }
  int imin = -1;
  for (int a = 0; a < 3; ++a)
    if (dtxyz[a] > 0.0 && (imin < 0 || dtxyz[a] < dtxyz[imin])) imin = a;
  *dt = dtxyz[imin];
  if (imin == 0) *exitFace = efx;
  else if (imin == 1) *exitFace = efy;
  else *exitFace = efz;
  *t = *t + *dt;
}

/* pr_ComputeRandomWalkTimeStep, :1376-1458 */
static double rw_time_step(const subcell_t *s, const orc_options *o) {
  double dts[2] = {0.0, 0.0}, dt = 0.0;
  double mx = fmax(fabs(s->VX1), fabs(s->VX2)), my = fmax(fabs(s->VY1), fabs(s->VY2)),
         mz = fmax(fabs(s->VZ1), fabs(s->VZ2));
  double aL = s->alphaLH, aT = s->alphaTH;
  switch (o->time_step_kind) {
    case 1:
      dt = o->ts_param[0] / (mx / s->DX + my / s->DY + mz / s->DZ);
      break;
    case 2:
      dt = o->ts_param[1] / (aL * mx / (s->DX * s->DX) + aT * my / (s->DY * s->DY) + aT * mz / (s->DZ * s->DZ));
      break;
    case 3:
      dts[0] = o->ts_param[0] / (mx / s->DX + my / s->DY + mz / s->DZ);
      dts[1] = o->ts_param[1] / (aL * mx / (s->DX * s->DX) + aT * my / (s->DY * s->DY) + aT * mz / (s->DZ * s->DZ));
      dt = DBL_MAX; /* minval over an empty mask is +huge */
      if (dts[0] > 0.0 && dts[0] < dt) dt = dts[0];
      if (dts[1] > 0.0 && dts[1] < dt) dt = dts[1];
      break;
    case 4:
      dt = o->ts_param[0];
      break;
  }
  return dt;
}

/* ------------------------------------------------------------------------ */
/* pr_ExecuteRandomWalkParticleTracking (TrackSubCell.F90:812-1373)          */
/* ------------------------------------------------------------------------ */
enum { SC_UNDEFINED = 0, SC_EXIT_CELL_FACE, SC_EXIT_INTERNAL, SC_MAXTIME, SC_NO_EXIT, SC_INACTIVE };

#define ORC_MAX_PASSES_PER_VISIT 1000000
#define ORC_MAX_ZERO_TIME_EXITS 1000 /* the GPU kernel's kMaxZeroTimeExits */
#define ORC_MAX_VISITS 1000000        /* the GPU kernel's kMaxVisitsPerAdvance */

typedef struct {
  int status, exitFace, conn;
  double x, y, z, t;
} scres_t;

static int subcell_has_exit(const subcell_t *s) {
  return (s->VX1 < 0.0) || (s->VX2 > 0.0) || (s->VY1 < 0.0) || (s->VY2 > 0.0) || (s->VZ1 < 0.0) || (s->VZ2 > 0.0);
}

#define OUTSIDE(a, b, c) (((a) > 1.0) || ((a) < 0.0) || ((b) > 1.0) || ((b) < 0.0) || ((c) > 1.0) || ((c) < 0.0))

static void track_subcell(const subcell_t *s, const orc_options *o, const int *dims, int ndim, int stopIfNoExit,
                          double ix, double iy, double iz, double initialTime, double maximumTime, rng_t *rng,
                          scres_t *res, int64_t *steps) {
  const double maxRelativeJump = 0.5;
  const double dtReductionFactor = (double)0.1f; /* single-precision literal 0.1 */
  const int kind = o->advection_kind;
  res->status = SC_UNDEFINED;
  res->exitFace = 0;
  res->conn = 0;
  res->x = ix; res->y = iy; res->z = iz; res->t = initialTime;
  if (stopIfNoExit && !subcell_has_exit(s)) {
    res->status = SC_NO_EXIT;
    return;
  }
  double dx = s->DX, dy = s->DY, dz = s->DZ;
  double x = ix, y = iy, z = iz, nx = ix, ny = iy, nz = iz;
  if (s->dry) {
    res->status = SC_INACTIVE;
    return;
  }
  double dtcell = rw_time_step(s, o);
  double t = initialTime, tinit = initialTime, dt;
  /* the reference tests dtcell .le. 0; a non-finite step would loop forever
   * (or trap under -ffpe-trap), so it is treated as undefined here too */
  if (!(dtcell > 0.0 && dtcell <= DBL_MAX)) {
    res->status = SC_UNDEFINED;
    return;
  }
  int intLoopCounter = 0, posRestartCounter = 0, reboundCounter;
  int exitFace = 0, reachedMax = 0;
  double vx, vy, vz, ddx, ddy, ddz, bx, by, bz, ax, ay, az, dxrw, dyrw, dzrw, xi, yi, zi;
  double dtxyz[3];
  int64_t passes = 0;
  for (;;) {
    if (++passes > ORC_MAX_PASSES_PER_VISIT) { /* safety cap shared with the GPU kernel */
      res->status = SC_UNDEFINED;
      return;
    }
    ++*steps;
    dt = dtcell;
    t = t + dt;
    if (maximumTime < t) {
      t = t - dt;
      dt = fmax(maximumTime - t, 0.0);
      t = maximumTime;
      reachedMax = 1;
    }
    /* pr_RWPTDisplacementsLinear, :673-706 */
    vx = (1.0 - x) * s->VX1 + x * s->VX2;
    vy = (1.0 - y) * s->VY1 + y * s->VY2;
    vz = (1.0 - z) * s->VZ1 + z * s->VZ2;
    divergence(s, x, y, z, &ddx, &ddy, &ddz);
    random_displacement(s, o, dims, ndim, x, y, z, vx, vy, vz, rng, &bx, &by, &bz);
    advection(s, kind, dt, vx, vy, vz, &ax, &ay, &az);
    dxrw = ax + ddx * dt + bx * sqrt(dt);
    dyrw = ay + ddy * dt + by * sqrt(dt);
    dzrw = az + ddz * dt + bz * sqrt(dt);
    while ((fabs(dxrw / dx) > maxRelativeJump) || (fabs(dyrw / dy) > maxRelativeJump) ||
           (fabs(dzrw / dz) > maxRelativeJump)) {
      t = t - dt;
      dt = dtReductionFactor * dt;
      advection(s, kind, dt, vx, vy, vz, &ax, &ay, &az);
      dxrw = ax + ddx * dt + bx * sqrt(dt);
      dyrw = ay + ddy * dt + by * sqrt(dt);
      dzrw = az + ddz * dt + bz * sqrt(dt);
      t = t + dt;
      if (reachedMax) reachedMax = 0;
    }
    nx = x + dxrw / dx;
    ny = y + dyrw / dy;
    nz = z + dzrw / dz;
    intLoopCounter = 0;
    while (OUTSIDE(nx, ny, nz)) {
      intLoopCounter = intLoopCounter + 1;
      dtxyz[0] = dtxyz[1] = dtxyz[2] = 0.0;
      exit_face_update(s, kind, x, y, z, nx, ny, nz, vx, vy, vz, ddx, ddy, ddz, bx, by, bz, &t, &dt, dtxyz,
                       &exitFace);
      if (intLoopCounter > 5) {
        nx = ix; ny = iy; nz = iz;
        t = tinit;
        dt = dtcell;
        posRestartCounter = posRestartCounter + 1;
        if (posRestartCounter > 10) {
          res->exitFace = 0;
          res->status = SC_UNDEFINED;
          res->x = x; res->y = y; res->z = z; res->t = t;
          return;
        }
        break;
      }
      advection(s, kind, dt, vx, vy, vz, &ax, &ay, &az);
      if (reachedMax) reachedMax = 0;
      int restart = 0;
      switch (exitFace) {
        case 1: case 2:
          nx = (exitFace == 1) ? 0.0 : 1.0;
          dyrw = ay + ddy * dt + by * sqrt(dt);
          ny = y + dyrw / dy;
          dzrw = az + ddz * dt + bz * sqrt(dt);
          nz = z + dzrw / dz;
          break;
        case 3: case 4:
          dxrw = ax + ddx * dt + bx * sqrt(dt);
          nx = x + dxrw / dx;
          ny = (exitFace == 3) ? 0.0 : 1.0;
          dzrw = az + ddz * dt + bz * sqrt(dt);
          nz = z + dzrw / dz;
          break;
        case 5: case 6:
          dxrw = ax + ddx * dt + bx * sqrt(dt);
          nx = x + dxrw / dx;
          dyrw = ay + ddy * dt + by * sqrt(dt);
          ny = y + dyrw / dy;
          nz = (exitFace == 5) ? 0.0 : 1.0;
          break;
        case 0:
          nx = ix; ny = iy; nz = iz;
          t = tinit;
          dt = dtcell;
          posRestartCounter = posRestartCounter + 1;
          if (posRestartCounter > 10) {
            res->exitFace = 0;
            res->status = SC_UNDEFINED;
            res->x = x; res->y = y; res->z = z; res->t = t;
            return;
          }
          restart = 1;
          break;
      }
      if (restart) break;
      if (OUTSIDE(nx, ny, nz)) continue;
      /* elastic rebound, :1157-1312 */
      reboundCounter = 0;
      while (exitFace > 0) {
        if (s->MassBoundary[exitFace - 1] != 1) break;
        reboundCounter = reboundCounter + 1;
        if (reboundCounter > 10) {
          res->exitFace = 0;
          res->status = SC_UNDEFINED;
          res->x = x; res->y = y; res->z = z; res->t = t;
          return;
        }
        xi = nx; yi = ny; zi = nz;
        if (dt == 0.0) {
          nx = ix; ny = iy; nz = iz;
          t = t - dt;
          dt = dtcell;
          exitFace = 0;
          posRestartCounter = posRestartCounter + 1;
          break;
        }
        t = t + dt;
        if (maximumTime < t) {
          t = t - dt;
          dt = fmax(maximumTime - t, 0.0);
          t = maximumTime;
          reachedMax = 1;
          advection(s, kind, dt, vx, vy, vz, &ax, &ay, &az);
          dxrw = ax + ddx * dt + bx * sqrt(dt);
          dyrw = ay + ddy * dt + by * sqrt(dt);
          dzrw = az + ddz * dt + bz * sqrt(dt);
        }
        switch (exitFace) {
          case 1: case 2:
            nx = nx - dxrw / dx; ny = ny + dyrw / dy; nz = nz + dzrw / dz;
            break;
          case 3: case 4:
            nx = nx + dxrw / dx; ny = ny - dyrw / dy; nz = nz + dzrw / dz;
            break;
          case 5: case 6:
            nx = nx + dxrw / dx; ny = ny + dyrw / dy; nz = nz - dzrw / dz;
            break;
        }
        if (OUTSIDE(nx, ny, nz)) {
          x = xi; y = yi; z = zi;
          switch (exitFace) {
            case 1: case 2: vx = -vx; ddx = -ddx; bx = -bx; break;
            case 3: case 4: vy = -vy; ddy = -ddy; by = -by; break;
            case 5: case 6: vz = -vz; ddz = -ddz; bz = -bz; break;
          }
          exitFace = 0;
        } else {
          dt = dtcell;
          exitFace = 0;
          if ((nx == 0.0) || (nx == 1.0) || (ny == 0.0) || (ny == 1.0) || (nz == 0.0) || (nz == 1.0)) {
            if (nx == 0.0) exitFace = 1;
            if (nx == 1.0) exitFace = 2;
            if (ny == 0.0) exitFace = 3;
            if (ny == 1.0) exitFace = 4;
            if (nz == 0.0) exitFace = 5;
            if (nz == 1.0) exitFace = 6;
          }
        }
      }
    }
    if (reachedMax) {
      res->status = SC_MAXTIME;
      res->exitFace = exitFace;
      res->x = nx; res->y = ny; res->z = nz; res->t = t;
      return;
    }
    if (exitFace > 0) {
      res->conn = s->Connection[exitFace - 1];
      res->status = (res->conn < 0) ? SC_EXIT_INTERNAL : SC_EXIT_CELL_FACE;
      res->exitFace = exitFace;
      res->x = nx; res->y = ny; res->z = nz; res->t = t;
      return;
    }
    x = nx;
    y = ny;
    z = nz;
  }
}

/* ------------------------------------------------------------------------ */
/* TrackCell (TrackCell.f90:375-669) + TrackPath (ParticleTrackingEngine.f90:1051-1254) */
/* ------------------------------------------------------------------------ */
static int cell_has_exit(const cdata *c, int backward) {
  double sign = backward ? -1.0 : 1.0;
  if (sign * c->Q[0] < 0.0) return 1;
  if (sign * c->Q[1] > 0.0) return 1;
  if (sign * c->Q[2] < 0.0) return 1;
  if (sign * c->Q[3] > 0.0) return 1;
  if (sign * c->Q[4] < 0.0) return 1;
  if (sign * c->Q[5] > 0.0) return 1;
  return 0;
}

typedef struct {
  int cell;
  double x, y, z, t;
} loc_t;

/* Track one particle from loc to maximumTime; returns the driver status and
 * writes the particle's final location (the last point of its pathline). */
static int track_path(const grid_t *g, const orc_options *o, const int *dims, int ndim, loc_t loc,
                      double maximumTime, rng_t *rng, loc_t *out, int64_t *steps) {
  const orc_flow *f = g->f;
  loc_t last = loc; /* last point in LocBuffP */
  int zero_time_exits = 0; /* consecutive cell exits that took no time (shared cap with the GPU kernel) */
  int64_t visits = 0;      /* cell exits in this call (shared cap with the GPU kernel) */
  for (;;) {
    int n = loc.cell;
    cdata c;
    fill_cell(g, n, &c);
    /* TrackCell checks, TrackCell.f90:405-497 */
    int stopIfNoSubCellExit = 1;
    if (loc.x < 0.0 || loc.x > 1.0 || loc.y < 0.0 || loc.y > 1.0 || loc.z < 0.0 || loc.z > 1.0) {
      *out = last;
      return ORC_UNDEFINED; /* InvalidLocation maps to Undefined in the driver */
    }
    if (c.IboundTS == 0) { *out = loc; return ORC_INACTIVE; }
    if (o->stop_zone > 0 && c.Zone == o->stop_zone) { *out = loc; return ORC_STOP_ZONE; }
    if (o->backward) {
      if (o->stop_weak_sources) {
        if (c.SourceFlow != 0.0) { *out = loc; return ORC_WEAK_SOURCE; }
        else if (!f->steady_state) stopIfNoSubCellExit = 0;
      }
    } else {
      if (o->stop_weak_sinks) {
        if (c.SinkFlow != 0.0) { *out = loc; return ORC_WEAK_SINK; }
        else if (!f->steady_state) stopIfNoSubCellExit = 0;
      }
    }
    if (!cell_has_exit(&c, o->backward)) {
      if (f->steady_state) { *out = loc; return ORC_NO_EXIT; }
      if (o->backward && c.SourceFlow != 0.0) { *out = loc; return ORC_NO_EXIT; }
      if (!o->backward && c.SinkFlow != 0.0) { *out = loc; return ORC_NO_EXIT; }
    }
    subcell_t s;
    fill_subcell(&c, o->backward, &s);
    corner_variables(g, n, &c, &s, o->uniform_porosity, o->dispersion_model);
    scres_t r;
    track_subcell(&s, o, dims, ndim, stopIfNoSubCellExit, loc.x, loc.y, loc.z, loc.t, maximumTime, rng, &r, steps);
    switch (r.status) {
      case SC_UNDEFINED:
        *out = last;
        return ORC_UNDEFINED;
      case SC_EXIT_INTERNAL:
        *out = last; /* refined cells only; not reachable on structured grids */
        return ORC_UNDEFINED;
      case SC_MAXTIME:
        out->cell = n; out->x = r.x; out->y = r.y; out->z = r.z; out->t = r.t;
        return ORC_ACTIVE;
      case SC_INACTIVE: *out = loc; return ORC_INACTIVE;
      case SC_NO_EXIT: *out = loc; return ORC_NO_EXIT;
      case SC_EXIT_CELL_FACE: {
        /* a particle that keeps crossing faces without time advancing would loop
         * forever (the reference has no cap on its cell loop): end it as undefined */
        zero_time_exits = (r.t == loc.t) ? zero_time_exits + 1 : 0;
        if (zero_time_exits > ORC_MAX_ZERO_TIME_EXITS || ++visits > ORC_MAX_VISITS) { *out = last; return ORC_UNDEFINED; }
        last.cell = n; last.x = r.x; last.y = r.y; last.z = r.z; last.t = r.t;
        int next = r.conn;
        if (next > 0 && f->iboundts[next - 1] != 0) {
          /* ConvertFromNeighbor, RectangularGridDisMf6.f90:50-108 */
          int face = r.exitFace; /* exit face of n; entry face of next is its opposite */
          int bad = 0;
          if (face == 2 && r.x != 1.0) bad = 1;
          if (face == 1 && r.x != 0.0) bad = 1;
          if (face == 4 && r.y != 1.0) bad = 1;
          if (face == 3 && r.y != 0.0) bad = 1;
          if (face == 6 && r.z != 1.0) bad = 1;
          if (face == 5 && r.z != 0.0) bad = 1;
          if (bad) { *out = last; return ORC_UNDEFINED; }
          loc.cell = next; loc.x = r.x; loc.y = r.y; loc.z = r.z; loc.t = r.t;
          if (face == 2) loc.x = 0.0;
          if (face == 1) loc.x = 1.0;
          if (face == 4) loc.y = 0.0;
          if (face == 3) loc.y = 1.0;
          if (face == 6) loc.z = 0.0;
          if (face == 5) loc.z = 1.0;
        } else {
          *out = last;
          return ORC_BOUNDARY;
        }
        break;
      }
    }
  }
}

static int dims_from_mask(const int mask[3], int dims[3]) {
  int nd = 0;
  for (int d = 0; d < 3; ++d)
    if (mask[d]) dims[nd++] = d;
  return nd;
}

int orc_advance(const orc_flow *f, const orc_options *o, int64_t n, int *cell, double *lx, double *ly, double *lz,
                double *t, int *status, const uint64_t *id, uint64_t *rng_ctr, double t_begin, double t_end,
                int64_t *steps_out) {
  grid_t g;
  if (grid_init(&g, f)) { grid_free(&g); return -1; }
  int dims[3];
  int ndim = dims_from_mask(o->dim_mask, dims);
  if (ndim == 0) { grid_free(&g); return -2; }
  int64_t steps_total = 0;
  int nthreads = o->nthreads > 0 ? o->nthreads : 1;
  if (nthreads > ORC_MAX_THREADS) { grid_free(&g); return -3; }
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) reduction(+ : steps_total)
#endif
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    rng_t rng;
    rng.kind = o->rng_kind;
    rng.seed = o->seed;
    if (o->rng_kind == 0) {
      /* continue this thread's stream of the run (seeded on first use) */
      if (!g_xoro_seeded[tid]) {
        orc_xoro_seed_stream(tid, g_xoro_state[tid]);
        g_xoro_seeded[tid] = 1;
      }
      rng.xs[0] = g_xoro_state[tid][0];
      rng.xs[1] = g_xoro_state[tid][1];
    }
    /* the reference's particle loop: schedule(dynamic,1) (MPathRW.F90:1207) */
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for (int64_t p = 0; p < n; ++p) {
      /* release logic, MPathRW.F90:1256-1302 */
      if (status[p] == ORC_PENDING) {
        if (t[p] < t_begin) status[p] = ORC_UNRELEASED;
        else if (t[p] <= t_end) {
          status[p] = ORC_ACTIVE;
          if (f->iboundts[cell[p] - 1] == 0) status[p] = ORC_INACTIVE;
        }
      }
      if (status[p] == ORC_INACTIVE) {
        cdata c;
        fill_cell(&g, cell[p], &c);
        if (verify_dry_partial(&c)) status[p] = ORC_ACTIVE;
      }
      if (status[p] != ORC_ACTIVE) continue;
      loc_t loc = {cell[p], lx[p], ly[p], lz[p], t[p]}, out;
      rng.id = id ? id[p] : (uint64_t)p;
      rng.ctr = rng_ctr ? &rng_ctr[p] : NULL;
      int64_t st = 0;
      int s = track_path(&g, o, dims, ndim, loc, t_end, &rng, &out, &st);
      steps_total += st;
      cell[p] = out.cell; lx[p] = out.x; ly[p] = out.y; lz[p] = out.z; t[p] = out.t;
      status[p] = s;
    }
    if (o->rng_kind == 0) {
      g_xoro_state[tid][0] = rng.xs[0];
      g_xoro_state[tid][1] = rng.xs[1];
    }
  }
  if (steps_out) *steps_out = steps_total;
  grid_free(&g);
  return 0;
}

void orc_global_xyz(const orc_flow *f, int64_t n, const int *cell, const double *lx, const double *ly,
                    const double *lz, double *gx, double *gy, double *gz) {
  grid_t g;
  if (grid_init(&g, f)) { grid_free(&g); return; }
  for (int64_t p = 0; p < n; ++p) {
    int k, i, j;
    cell_klj(&g, cell[p], &k, &i, &j);
    double left = g.cellx[j] - (f->delr[j] / 2.0), right = g.cellx[j] + (f->delr[j] / 2.0);
    double front = g.celly[i] - (f->delc[i] / 2.0), back = g.celly[i] + (f->delc[i] / 2.0);
    double bottom = f->botm[cell[p] - 1], top = g.sattop[cell[p] - 1];
    double X = ((1.0 - lx[p]) * left) + (lx[p] * right);
    if (X < left) X = left;
    if (X > right) X = right;
    double Y = ((1.0 - ly[p]) * front) + (ly[p] * back);
    if (Y < front) Y = front;
    if (Y > back) Y = back;
    double Z = ((1.0 - lz[p]) * bottom) + (lz[p] * top);
    if (Z < bottom) Z = bottom;
    if (Z > top) Z = top;
    gx[p] = X; gy[p] = Y; gz[p] = Z;
  }
  grid_free(&g);
}

int orc_cell_record(const orc_flow *f, const orc_options *o, int cell, double *vface6, double *dtcell,
                    double *qcorner32, double *phicorner8, double *d72, int *massb6, int *conn6) {
  grid_t g;
  if (grid_init(&g, f)) { grid_free(&g); return -1; }
  cdata c;
  subcell_t s;
  fill_cell(&g, cell, &c);
  fill_subcell(&c, o->backward, &s);
  corner_variables(&g, cell, &c, &s, o->uniform_porosity, o->dispersion_model);
  double v[6] = {s.VX1, s.VX2, s.VY1, s.VY2, s.VZ1, s.VZ2};
  for (int q = 0; q < 6; ++q) {
    vface6[q] = v[q];
    massb6[q] = s.MassBoundary[q];
    conn6[q] = s.Connection[q];
  }
  *dtcell = rw_time_step(&s, o);
  for (int cc = 0; cc < 8; ++cc) {
    for (int m = 0; m < 4; ++m) qcorner32[4 * cc + m] = s.qC[cc][m];
    phicorner8[cc] = s.phiC[cc];
  }
  for (int a = 0; a < 9; ++a)
    for (int cc = 0; cc < 8; ++cc) d72[8 * a + cc] = s.D[a][cc];
  grid_free(&g);
  return 0;
}
