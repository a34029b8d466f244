// Tetrahedron polarization weights w_nm(k,q,iω) on sm_103a, FP64.
//
// Drop-in for PyGW's bz_calcqdepw_par2 (for_tetrahedra.f90:390-464) and its
// callees (for_tetrahedra3.f90:3-743, for_tetrahedra2.f90:1688-2773).
//
// Structure (GPU-first, deterministic):
//   1. k_kcsr_*       : for every mesh point k, the ascending list of
//                       (tetrahedron, corner) slots that touch it (CSR).
//   Then per chunk of tetrahedra (items = (tetrahedron, occupied band ib,
//   unoccupied band jb)):
//   2. k_tet_geometry : one thread per item.  It builds the integration
//                       polyhedron {e ≤ EF ≤ f} (surfnodes → unrepnodes →
//                       relnodes → sortnodes), splits it into sub-tetrahedra
//                       and sets each one up (volume, sorteq grouping,
//                       closed-form coefficients): frequency-independent work,
//                       done once and stored as records, with the item's
//                       class (node count, first grouping).
//   3. k_class_offsets / k_class_scatter: the chunk's items in class order.
//   4. k_tet_eval     : one thread per (item, frequency) in class order: the
//                       closed-form corner weights of the item's records at
//                       that frequency.  atan/log are evaluated once per
//                       distinct corner value (4 + 4 in the generic case, where
//                       the reference evaluates 16 + 16) and shared by the four
//                       vertex formulas.  Lanes of a warp share one item (and
//                       its code path); the kernel has no stack frame.  Results
//                       go to a scratch array laid out [tet][corner][ω][pair].
//   5. k_gather       : kcw[pair, k, ω] = Σ over k's CSR slots in ascending
//                       tetrahedron order of (w·6)·(1/ntet) — the reference's
//                       accumulation order, without atomics.
//
// Arithmetic matches the oracle bit for bit: this file is compiled with
// -fmad=false, atan/log come from fp64_math.h, and every expression keeps the
// reference's left-to-right order.  The reference's case-4 closed form
// assigns the weights of small-tetrahedron vertices 2 and 4 to each other
// (verified against quadrature); this is kept, since the product must return
// the reference's results.
#include <cuda_runtime.h>
#include <atomic>
#include <stdint.h>
#include "fp64_math.h"
#include "pygw_status.h"
#include "launches.h"

namespace pgw {

// Default-real literals of the reference, widened to double.
#define ZTOL_VOL ((double)1.e-10f)
#define ZTOL_SORTEQ ((double)1.e-2f)
#define RDIST_TINY ((double)1.0e-10f)
#define OMEG_TINY ((double)1.0e-20f)
#define CHECK_OMEG ((double)1.e-6f)
#define TOL_UNPHYS 1.0e4
#define TOL_TAYLOR 10.0

struct SubTet;

struct Params {
  const double* enk;   // [nbnd][nkp] column-major: enk[b + nbnd*k]
  const int* kqid;     // [nkp]
  const double* omega; // [nom]
  const int* tetc;     // [ntet][4]: tetc[i + 4*t]
  double* scratch;     // [ntet][4][nomc][P]
  const int* order;    // items of the chunk sorted by polyhedron class
  SubTet* recs;        // set-up sub-tetrahedra of the chunk's items (≤ 6 per item)
  int* recoff;         // [chunk items] first record of each contributing item
  unsigned* nrec;      // records claimed so far in the chunk
  unsigned* status;    // device status word (may be null)
  unsigned long long* counters;  // PG_NCOUNTERS (may be null)
  double ef;
  int nbnd, nkp, ncg, numin, nb1, nb2, ntet, om0, nomc;
  int tet0;            // first tetrahedron of the chunk
  int ref_layout;      // reproduce the reference's wtemp addressing (7- and 8-node polyhedra)
};

struct Ctx {
  unsigned status;
  unsigned long long cnt[PG_NCOUNTERS];
};

__device__ __forceinline__ double sq(double x) { return x * x; }
__device__ __forceinline__ double cube(double x) { return (x * x) * x; }
__device__ __forceinline__ double pow4(double x) { double t = x * x; return t * t; }

// ------------------------------------------------------------------ sorteq
__device__ double f_rdist(double v1, double v2) {
  if ((fabs(v1) + fabs(v2)) < RDIST_TINY) return 0.0;
  return 2.0 * fabs(v1 - v2) / (fabs(v1) + fabs(v2));
}

__device__ int sorteq(double v[4], int index[4], Ctx& cx) {
  int sig[4] = {0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (f_rdist(v[i], v[j]) < ZTOL_SORTEQ) sig[i] += 1;
  int s5 = sig[0] + sig[1] + sig[2] + sig[3];
  int mx = max(max(sig[0], sig[1]), max(sig[2], sig[3]));
  if (s5 == 8 && mx == 3) {
#pragma unroll
    for (int i = 0; i < 4; i++) if (sig[i] == 2) sig[i] += 1;
    s5 = sig[0] + sig[1] + sig[2] + sig[3];
  }
  int mn = min(min(sig[0], sig[1]), min(sig[2], sig[3]));
  if (s5 == 10 && mn == 2) {
#pragma unroll
    for (int i = 0; i < 4; i++) sig[i] = 4;
    s5 = 16;
  }
  if (s5 == 12 || s5 == 14) s5 = 16;
#pragma unroll
  for (int i = 0; i < 4; i++) index[i] = i + 1;
  double vt; int it;
  if (s5 == 10) {
    for (int i = 0; i < 3; i++) {
      if (sig[i] == 1) {
        vt = v[i]; v[i] = v[3]; v[3] = vt;
        it = index[i]; index[i] = index[3]; index[3] = it;
        it = sig[3]; sig[3] = sig[i]; sig[i] = it;
      }
    }
  } else if (s5 == 8) {
    for (int i = 2; i < 4; i++) {
      if (f_rdist(v[i], v[0]) < f_rdist(v[1], v[0])) {
        vt = v[i]; v[i] = v[1]; v[1] = vt;
        it = index[i]; index[i] = index[1]; index[1] = it;
        it = sig[i]; sig[i] = sig[1]; sig[1] = it;
      }
    }
  } else if (s5 == 6) {
    int j = 0;
    for (int i = 0; i < 4; i++) {
      if (sig[i] == 2) {
        vt = v[j]; v[j] = v[i]; v[i] = vt;
        it = index[j]; index[j] = index[i]; index[i] = it;
        it = sig[j]; sig[j] = sig[i]; sig[i] = it;
        j++;
      }
    }
  } else if (s5 != 4 && s5 != 16) {
    cx.status |= PG_ERR_SORTEQ;
  }
  return s5;
}

// ------------------------------------------------------- one sub-tetrahedron
// Everything about a sub-tetrahedron that does not depend on ω.
struct SubTet {
  double corner[4][3];     // corners in the big-tetrahedron frame
  double vol;
  double ds[4];            // Δe at the corners (unsorted; Taylor uses these)
  double taylor_omega;
  int flag;                // sorteq grouping 4/6/8/10/16
  int ind[4];              // sorteq permutation (1-based)
  double val[5];           // distinct corner values whose atan/log are needed
  int nval;
  // Per-vertex closed-form coefficients (vertex-major).  Slot layout by case:
  //  case 4 : evt[1..9], evw[1..9], cc; node map m[1..4]
  //  case 6 : evt[1..7], evw[1..7], cc; node map for slots 1,3,4
  //  case 8 : evt/evw as in the reference, cc
  //  case 10: evt/evw, cc1, cc2
  //  case 16: ev
  double cf[4][20];
  int map[4][4];
};

__device__ void stweight_itaylor(const double dv[4], double omeg, double wv[4]) {
  double omt2 = omeg * omeg;
  double omt4 = omt2 * omt2;
  double denom1 = 6.0e+1 * omt2;
  double denom3 = 4.2e+2 * omt4;
#pragma unroll
  for (int ivert = 1; ivert <= 4; ivert++) {
    double ev[5];
#pragma unroll
    for (int j = 1; j <= 4; j++) ev[j] = dv[(j + ivert - 2) % 4];
    double w01 = -(2.0 * ev[1] + ev[2] + ev[3] + ev[4]) / denom1;
    double n03 = 4.0 * (ev[1] * ev[1] * ev[1]) + 3.0 * (ev[1] * ev[1]) * (ev[2] + ev[3] + ev[4]);
    n03 = n03 + 2.0 * ev[1] * (ev[2] * ev[2] + ev[3] * ev[3] + ev[4] * ev[4] + ev[2] * ev[3] + ev[2] * ev[4] + ev[3] * ev[4]);
    n03 = n03 + (ev[2] * ev[2] * ev[2]) + (ev[3] * ev[3] * ev[3]) + (ev[4] * ev[4] * ev[4]) + (ev[2] * ev[2]) * ev[3] +
          (ev[2] * ev[2]) * ev[4] + (ev[3] * ev[3]) * ev[4] + ev[2] * (ev[3] * ev[3]) + ev[2] * (ev[4] * ev[4]) +
          ev[3] * (ev[4] * ev[4]) + ev[2] * ev[3] * ev[4];
    double w03 = n03 / denom3;
    wv[ivert - 1] = w01 + w03;
  }
}

// Case-4 coefficients for one vertex (for_tetrahedra3.f90:485-519).
__device__ void coef_case4(const double ev[5], double* c) {
  double vdif[5][5];
#pragma unroll
  for (int i = 1; i <= 4; i++)
#pragma unroll
    for (int j = 1; j <= 4; j++) vdif[i][j] = ev[i] - ev[j];
  double ev3t4 = ev[3] * ev[4];
  double ev1_2 = ev[1] * ev[1];
  double ev_2[5];
  ev_2[1] = 3.0 * ev1_2;
  ev_2[2] = 3.0 * sq(ev[2]);
  ev_2[3] = 3.0 * sq(ev[3]);
  ev_2[4] = 3.0 * sq(ev[4]);
  double vdf24 = vdif[2][3] * vdif[2][4] * vdif[3][4];
  double* evt = c;        // evt[1..9] at c[1..9]
  double* evw = c + 9;    // evw[1..9] at c[10..18]
  evw[1] = 2.0 * vdif[1][2] * (vdif[1][3] * vdif[1][4]) * vdf24;
  evt[1] = -ev1_2 * evw[1];
  evw[2] = vdf24 * 2.0 * ((2.0 * ev[1] - ev[2]) * (ev[3] + ev[4]) + ev[1] * (2.0 * ev[2] - 3.0 * ev[1]) - ev[3] * ev[4]);
  evt[2] = vdf24 * 6.0 * ev[1] * (2.0 * ev[2] * ev3t4 + ev[1] * (ev1_2 - ev3t4 - ev[2] * (ev[3] + ev[4])));
  evw[3] = 2.0 * sq(vdif[1][3] * vdif[1][4]) * vdif[3][4];
  evt[3] = -ev_2[2] * evw[3];
  evw[4] = -2.0 * sq(vdif[1][2] * vdif[1][4]) * vdif[2][4];
  evt[4] = -ev_2[3] * evw[4];
  evw[5] = 2.0 * sq(vdif[1][2] * vdif[1][3]) * vdif[2][3];
  evt[5] = -ev_2[4] * evw[5];
  evt[6] = vdf24 * ev1_2 * (3.0 * ev[2] * ev3t4 + ev[1] * (ev[2] * (ev[1] - 2.0 * ev[3]) + ev[4] * (ev[1] - 2.0 * ev[2]) + ev[3] * (ev[1] - 2.0 * ev[4])));
  evw[6] = -3.0 * vdf24 * (ev[2] * ev[3] * ev[4] + ev1_2 * (2.0 * ev[1] - ev[2] - ev[3] - ev[4]));
  double evdf2 = ev[2] * sq(vdif[1][3] * vdif[1][4]) * vdif[3][4] / 3.0;
  double evdf3 = ev[3] * sq(vdif[1][2] * vdif[1][4]) * vdif[2][4] / 3.0;
  double evdf4 = ev[4] * sq(vdif[1][2] * vdif[1][3]) * vdif[2][3] / 3.0;
  evt[7] = -ev_2[2] * evdf2;
  evw[7] = 9.0 * evdf2;
  evw[8] = -9.0 * evdf3;
  evt[8] = ev_2[3] * evdf3;
  evw[9] = 9.0 * evdf4;
  evt[9] = -ev_2[4] * evdf4;
  c[19] = 6.0 * sq(vdif[1][2] * vdif[1][3] * vdif[1][4]) * vdif[2][3] * vdif[2][4] * vdif[3][4];
}

// Case-6 coefficients, vertices 1-2 (for_tetrahedra3.f90:539-563).
__device__ void coef_case6a(const double ev[5], double* c) {
  double vdif[5][5];
#pragma unroll
  for (int i = 1; i <= 4; i++)
#pragma unroll
    for (int j = 1; j <= 4; j++) vdif[i][j] = ev[i] - ev[j];
  double* evt = c;       // evt[1..7] at c[1..7]
  double* evw = c + 7;   // evw[1..7] at c[8..14]
  double evf = vdif[3][1] * vdif[1][4] * vdif[3][4];
  evw[1] = (2.0 * ev[1] - ev[3] - ev[4]) * evf * 2.0;
  evt[1] = ev[1] * (5.0 * ev[3] * ev[4] + ev[1] * (ev[1] - 3.0 * ev[3] - 3.0 * ev[4])) * evf;
  evt[2] = -6.0 * (sq(ev[1]) * (ev[1] * ev[3] + ev[1] * ev[4] - 3.0 * ev[3] * ev[4]) + sq(ev[3] * ev[4])) * vdif[3][4];
  evw[2] = 2.0 * (3.0 * ev[1] * (ev[1] - ev[3] - ev[4]) + sq(ev[3]) + ev[3] * ev[4] + sq(ev[4])) * vdif[3][4];
  evw[3] = -2.0 * cube(vdif[1][4]);
  evt[3] = -3.0 * sq(ev[3]) * evw[3];
  evw[4] = 2.0 * cube(vdif[1][3]);
  evt[4] = -3.0 * sq(ev[4]) * evw[4];
  evt[5] = -vdif[3][4] * ev[1] * (3.0 * ev[3] * ev[4] * (ev[1] * (ev[1] - ev[3] - ev[4]) + ev[3] * ev[4]) + sq(ev[1]) * sq(ev[3] - ev[4]));
  evw[5] = -3.0 * vdif[3][4] * (ev[3] * ev[4] * (3.0 * ev[1] - ev[3] - ev[4]) - cube(ev[1]));
  evf = ev[3] * cube(vdif[1][4]);
  evw[6] = -3.0 * evf;
  evt[6] = sq(ev[3]) * evf;
  evf = ev[4] * cube(vdif[1][3]);
  evw[7] = 3.0 * evf;
  evt[7] = -sq(ev[4]) * evf;
  c[19] = 6.0 * cube(vdif[1][3]) * cube(vdif[1][4]) * vdif[3][4];
}

// Case-6 coefficients, vertices 3-4 (for_tetrahedra3.f90:578-600).
__device__ void coef_case6b(const double ev[5], double* c) {
  double vdif[5][5];
#pragma unroll
  for (int i = 1; i <= 4; i++)
#pragma unroll
    for (int j = 1; j <= 4; j++) vdif[i][j] = ev[i] - ev[j];
  double* evt = c;
  double* evw = c + 7;
  evt[1] = (sq(ev[3]) * ev[4] + sq(ev[1]) * vdif[4][3] - ev[1] * sq(ev[3])) * 2.0 * vdif[1][3] * vdif[1][4] * vdif[3][4];
  evw[1] = ((ev[1] + ev[3] - 2.0 * ev[4])) * 2.0 * vdif[1][3] * vdif[1][4] * vdif[3][4];
  evt[2] = (3.0 * ev[1] * (ev[1] * (ev[3] + ev[1]) - 2.0 * ev[3] * ev[4])) * 2.0 * sq(vdif[3][4]);
  evw[2] = (ev[3] + 2.0 * ev[4] - 3.0 * ev[1]) * 2.0 * sq(vdif[3][4]);
  evt[3] = -3.0 * ev[3] * (sq(ev[3]) + ev[1] * (ev[3] - 2.0 * ev[4])) * 2.0 * sq(vdif[1][4]);
  evw[3] = -(ev[1] - 3.0 * ev[3] + 2.0 * ev[4]) * 2.0 * sq(vdif[1][4]);
  evw[4] = 2.0 * cube(vdif[1][3]);
  evt[4] = (-3.0 * sq(ev[4])) * evw[4];
  evt[5] = sq(ev[1]) * (-3.0 * ev[3] * ev[4] + ev[1] * (2.0 * ev[3] + ev[4])) * sq(vdif[3][4]);
  evw[5] = (-6.0 * sq(ev[1]) + 3.0 * ev[1] * ev[4] + 3.0 * ev[3] * ev[4]) * sq(vdif[3][4]);
  evt[6] = -sq(ev[3]) * (2.0 * ev[1] * ev[3] - 3.0 * ev[1] * ev[4] + ev[3] * ev[4]) * sq(vdif[1][4]);
  evw[6] = -3.0 * (-2.0 * sq(ev[3]) + (ev[1] + ev[3]) * ev[4]) * sq(vdif[1][4]);
  evt[7] = -ev[4] * cube(vdif[1][3]) * sq(ev[4]);
  evw[7] = ev[4] * cube(vdif[1][3]) * 3.0;
  c[19] = 6.0 * cube(vdif[1][3]) * sq(vdif[1][4]) * sq(vdif[3][4]);
}

__device__ void setup_subtet(SubTet& s, const double e[4], const double f[4], Ctx& cx) {
  double dbig[4];
#pragma unroll
  for (int i = 0; i < 4; i++) dbig[i] = f[i] - e[i];
  double vec[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) vec[i][j] = s.corner[i + 1][j] - s.corner[0][j];
  double vol = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    vol = vol + vec[0][i] * (vec[1][j] * vec[2][k] - vec[1][k] * vec[2][j]);
  }
  s.vol = fabs(vol);
  if (s.vol < ZTOL_VOL) return;
  double max_de = 0.0;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    s.ds[i] = (dbig[1] - dbig[0]) * s.corner[i][0] + (dbig[2] - dbig[0]) * s.corner[i][1] +
              (dbig[3] - dbig[0]) * s.corner[i][2] + dbig[0];
    if (fabs(s.ds[i]) > max_de) max_de = fabs(s.ds[i]);
  }
  s.taylor_omega = TOL_TAYLOR * max_de;
  double v[4] = {s.ds[0], s.ds[1], s.ds[2], s.ds[3]};
  s.flag = sorteq(v, s.ind, cx);
  double ev[5];
  switch (s.flag) {
    case 4:
      s.nval = 4;
#pragma unroll
      for (int j = 0; j < 4; j++) s.val[j] = v[j];
      for (int ivert = 1; ivert <= 4; ivert++) {
        for (int j = 1; j <= 4; j++) {
          const int k = (j + ivert - 2) % 4 + 1;
          ev[k] = v[j - 1];
          s.map[ivert - 1][k - 1] = j - 1;
        }
        coef_case4(ev, s.cf[ivert - 1]);
      }
      break;
    case 6:
      s.nval = 5;
#pragma unroll
      for (int j = 0; j < 4; j++) s.val[j] = v[j];
      s.val[4] = (v[0] + v[1]) * 0.5;
      for (int ivert = 1; ivert <= 2; ivert++) {
        ev[1] = v[ivert - 1]; ev[2] = ev[1]; ev[3] = v[2]; ev[4] = v[3];
        s.map[ivert - 1][0] = ivert - 1; s.map[ivert - 1][2] = 2; s.map[ivert - 1][3] = 3;
        coef_case6a(ev, s.cf[ivert - 1]);
      }
      for (int ivert = 3; ivert <= 4; ivert++) {
        ev[1] = s.val[4]; ev[2] = ev[1];
        s.map[ivert - 1][0] = 4;
        for (int j = 3; j <= 4; j++) {
          const int k = (j + ivert) % 2 + 3;
          ev[k] = v[j - 1];
          s.map[ivert - 1][k - 1] = j - 1;
        }
        coef_case6b(ev, s.cf[ivert - 1]);
      }
      break;
    case 8: {
      s.nval = 2;
      ev[1] = (v[0] + v[1]) / 2.0; ev[2] = ev[1];
      ev[3] = (v[2] + v[3]) / 2.0; ev[4] = ev[3];
      s.val[0] = ev[1]; s.val[1] = ev[3];
      const double v13 = ev[1] - ev[3], v31 = ev[3] - ev[1];
      double* c = s.cf[0];
      c[1] = 6.0 * v31;                                                       // evw(1)
      c[2] = (sq(ev[1]) - 5.0 * ev[1] * ev[3] - 2.0 * sq(ev[3])) * v31;       // evt(1)
      c[3] = -6.0 * (sq(ev[3]) + 2.0 * ev[1] * ev[3]);                        // evt(2)
      c[4] = 3.0 * (ev[1] + 2.0 * ev[3]);                                     // evw(3)
      c[5] = -3.0 * ev[1] * sq(ev[3]);                                        // evt(3)
      c[6] = 6.0 * v13;                                                       // evw(4)
      c[7] = -(2.0 * sq(ev[1]) + 5.0 * ev[1] * ev[3] - sq(ev[3])) * v13;      // evt(4)
      c[8] = 6.0 * (sq(ev[1]) + 2.0 * ev[1] * ev[3]);                         // evt(5)
      c[9] = -3.0 * (2.0 * ev[1] + ev[3]);                                    // evw(6)
      c[10] = 3.0 * sq(ev[1]) * ev[3];                                        // evt(6)
      c[19] = 6.0 * pow4(v13);                                                // cc
    } break;
    case 10: {
      s.nval = 2;
      const double a = ((v[0] + v[1]) + v[2]) / 3.0;
      ev[1] = ev[2] = ev[3] = a;
      ev[4] = v[3];
      s.val[0] = a; s.val[1] = ev[4];
      const double v14 = ev[1] - ev[4], v41 = ev[4] - ev[1];
      double* c = s.cf[0];
      c[1] = 6.0 * v14;                                                            // evw(1)
      c[2] = -v14 * (2.0 * sq(ev[1]) - 7.0 * ev[1] * ev[4] + 11.0 * sq(ev[4]));  // evt(1)
      c[3] = 18.0 * sq(ev[4]);                                                     // evt(2)
      c[4] = -9.0 * ev[4];                                                         // evw(3)
      c[5] = 3.0 * cube(ev[4]);                                                    // evt(3)
      c[6] = 6.0 * v41;                                                            // evw(4)
      c[7] = v41 * (sq(ev[1]) - 5.0 * ev[1] * ev[4] - 2.0 * sq(ev[4]));           // evt(4)
      c[8] = -6.0 * ev[4] * (ev[4] + 2.0 * ev[1]);                                 // evt(5)
      c[9] = -3.0 * ev[1] * sq(ev[4]);                                             // evt(6)
      c[10] = 3.0 * (ev[1] + 2.0 * ev[4]);                                         // evw(6)
      c[18] = 18.0 * pow4(v14);                                                    // cc1
      c[19] = 6.0 * pow4(v14);                                                     // cc2
    } break;
    case 16:
      s.nval = 0;
      s.cf[0][1] = (((v[0] + v[1]) + v[2]) + v[3]) / 4.0;
      break;
    default:
      s.nval = 0;
      break;
  }
}

__device__ __forceinline__ void check_weight(double& w, double omeg, Ctx& cx) {
  if (fabs(w) > TOL_UNPHYS) {
    if (fabs(omeg) < CHECK_OMEG) { w = 0.0; cx.cnt[PG_CNT_BIGW_ZEROED]++; }
    else cx.cnt[PG_CNT_BIGW_WARN]++;
  }
}

__device__ __forceinline__ double pick5(const double (&a)[5], int i) {
  return i == 0 ? a[0] : i == 1 ? a[1] : i == 2 ? a[2] : i == 3 ? a[3] : a[4];
}

// Weights of one sub-tetrahedron at one frequency, already mapped to the
// big-tetrahedron corners and multiplied by the sub-tetrahedron volume
// (generictetra_par's epilogue, for_tetrahedra3.f90:392-403).
__device__ void eval_subtet(const SubTet& s, double omeg, double wout[4], Ctx& cx) {
  double ws[4] = {0.0, 0.0, 0.0, 0.0};
  if (omeg > s.taylor_omega) {
    stweight_itaylor(s.ds, omeg, ws);
  } else {
    // T, L of the distinct corner values, kept in registers (the vertex
    // formulas pick them by the record's node map through pick5); one copy
    // of the atan/log code in a loop, its results moved into place by selects
    double T[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, L[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const int nval = s.nval;
#pragma unroll 1
    for (int q = 0; q < nval; q++) {
      const double x = s.val[q];
      const double t = (omeg > OMEG_TINY) ? pg_atan(x / omeg) : copysign(1.0, x) * 2.0 * pg_atan(1.0);
      const double l = ((omeg * omeg + x * x) > 1.0e-10) ? pg_log(x * x + omeg * omeg) : 0.0;
#pragma unroll
      for (int i = 0; i < 5; i++) {
        T[i] = (q == i) ? t : T[i];
        L[i] = (q == i) ? l : L[i];
      }
    }
    const double omeg2 = omeg * omeg;
    double wt[4];
    switch (s.flag) {
      case 4:
#pragma unroll
        for (int v = 0; v < 4; v++) {
          const double* c = s.cf[v];
          const double* evt = c;
          const double* evw = c + 9;
          const int* m = s.map[v];
          const double t1 = pick5(T, m[0]), t2 = pick5(T, m[1]), t3 = pick5(T, m[2]), t4 = pick5(T, m[3]);
          const double l1 = pick5(L, m[0]), l2 = pick5(L, m[1]), l3 = pick5(L, m[2]), l4 = pick5(L, m[3]);
          double aa = evt[1] + omeg2 * evw[1] + omeg * (t1 * evt[2] + t2 * evt[3] + t3 * evt[4] + t4 * evt[5] +
                                                        omeg2 * (t1 * evw[2] + t2 * evw[3] + t3 * evw[4] + t4 * evw[5]));
          double bb = l1 * evt[6] + l2 * evt[7] + l3 * evt[8] + l4 * evt[9] +
                      omeg2 * (l1 * evw[6] + l2 * evw[7] + l3 * evw[8] + l4 * evw[9]);
          wt[v] = (aa + bb) / c[19];
          check_weight(wt[v], omeg, cx);
        }
        break;
      case 6:
#pragma unroll
        for (int v = 0; v < 4; v++) {
          const double* c = s.cf[v];
          const double* evt = c;
          const double* evw = c + 7;
          const int* m = s.map[v];
          const double t1 = pick5(T, m[0]), t3 = pick5(T, m[2]), t4 = pick5(T, m[3]);
          const double l1 = pick5(L, m[0]), l3 = pick5(L, m[2]), l4 = pick5(L, m[3]);
          double aa = evt[1] + omeg2 * evw[1] + omeg * (t1 * evt[2] + t3 * evt[3] + t4 * evt[4] +
                                                        omeg2 * (t1 * evw[2] + t3 * evw[3] + t4 * evw[4]));
          double bb = l1 * evt[5] + l3 * evt[6] + l4 * evt[7] + omeg2 * (l1 * evw[5] + l3 * evw[6] + l4 * evw[7]);
          wt[v] = (aa + bb) / c[19];
          check_weight(wt[v], omeg, cx);
        }
        break;
      case 8: {
        const double* c = s.cf[0];
        const double dt = T[0] - T[1], dl = L[0] - L[1];
        double aa = c[2] + c[1] * omeg2 + omeg * dt * (6.0 * omeg2 + c[3]);
        double bb = dl * (c[5] + c[4] * omeg2);
        wt[0] = (aa + bb) / c[19];
        check_weight(wt[0], omeg, cx);
        wt[1] = wt[0];
        aa = c[7] + c[6] * omeg2 + omeg * dt * (-6.0 * omeg2 + c[8]);
        bb = dl * (c[10] + c[9] * omeg2);
        wt[2] = (aa + bb) / c[19];
        check_weight(wt[2], omeg, cx);
        wt[3] = wt[2];
      } break;
      case 10: {
        const double* c = s.cf[0];
        const double dt = T[0] - T[1], dl = L[0] - L[1];
        double aa = c[2] + omeg2 * c[1] + omeg * dt * (-6.0 * omeg2 + c[3]);
        double bb = dl * (c[5] + c[4] * omeg2);
        wt[0] = (aa + bb) / c[18];
        check_weight(wt[0], omeg, cx);
        wt[1] = wt[0]; wt[2] = wt[0];
        aa = c[7] + c[6] * omeg2 + omeg * dt * (6.0 * omeg2 + c[8]);
        bb = dl * (c[9] + c[10] * omeg2);
        wt[3] = (aa + bb) / c[19];
        check_weight(wt[3], omeg, cx);
      } break;
      case 16: {
        const double e1 = s.cf[0][1];
        wt[0] = -e1 / (12.0 * (sq(omeg) + sq(e1)));
        check_weight(wt[0], omeg, cx);
        wt[1] = wt[0]; wt[2] = wt[0]; wt[3] = wt[0];
      } break;
      default:
        wt[0] = wt[1] = wt[2] = wt[3] = 0.0;
        cx.status |= PG_ERR_EQUIV;
        break;
    }
    // ws[ind[i] − 1] = wt[i] in i order, as register selects (the last
    // write to a slot wins, slots never written keep 0)
    int ind[4];
#pragma unroll
    for (int i = 0; i < 4; i++) ind[i] = s.ind[i] - 1;
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int i = 0; i < 4; i++)
        if (ind[i] == j) ws[j] = wt[i];
  }
  double sm = ws[0];
  sm = sm + ws[1];
  sm = sm + ws[2];
  sm = sm + ws[3];
  double w[4] = {sm, 0.0, 0.0, 0.0};
#pragma unroll
  for (int i = 1; i <= 3; i++) {
#pragma unroll
    for (int j = 0; j < 4; j++) w[i] = w[i] + ws[j] * s.corner[j][i - 1];
    w[0] = w[0] - w[i];
  }
#pragma unroll
  for (int i = 0; i < 4; i++) wout[i] = w[i] * s.vol;
}

// ------------------------------------------------------- polyhedron nodes
struct Nodes {
  double x[21][3];   // node 1..20, coordinates 0..2
  int ntype[21];
  int nnod;
};

__device__ void surfnodes(Nodes& N, const double e[4], const double f[4], double ef) {
  const double zerotol = 1.0e-12;
  const int types[20] = {7, 11, 13, 14, 19, 21, 22, 25, 26, 28, 35, 37, 38, 41, 42, 44, 49, 50, 52, 56};
  for (int n = 1; n <= 20; n++) { N.x[n][0] = N.x[n][1] = N.x[n][2] = 0.0; N.ntype[n] = types[n - 1]; }
  N.x[2][2] = 1.0; N.x[3][1] = 1.0; N.x[4][0] = 1.0;
  int inod = 4, iint = 4;
  double nt[3];
#define PG_ADD()                                              \
  {                                                           \
    inod++;                                                   \
    N.x[inod][0] = nt[0]; N.x[inod][1] = nt[1]; N.x[inod][2] = nt[2]; \
    N.ntype[inod] = N.ntype[iint];                            \
  }
  for (int j = 2; j <= 4; j++) {
    const int i = 6 - j; iint++;
    const double denom = e[i - 1] - e[0];
    nt[0] = nt[1] = nt[2] = 0.0;
    if (fabs(denom) > zerotol) {
      nt[i - 2] = (ef - e[0]) / denom;
      if ((nt[i - 2] > 0.0) && (nt[i - 2] <= 1.0)) PG_ADD();
    }
  }
  for (int k = 1; k <= 3; k++) {
    const int i = k % 3 + 1, j = i % 3 + 1; iint++;
    const double denom = e[i] - e[j];
    nt[0] = nt[1] = nt[2] = 0.0;
    if (fabs(denom) > zerotol) {
      nt[i - 1] = (ef - e[j]) / denom;
      nt[j - 1] = (e[i] - ef) / denom;
      if ((nt[i - 1] >= 0.0) && (nt[j - 1] >= 0.0)) PG_ADD();
    }
  }
  for (int j = 2; j <= 4; j++) {
    const int i = 6 - j; iint++;
    const double denom = f[i - 1] - f[0];
    nt[0] = nt[1] = nt[2] = 0.0;
    if (fabs(denom) > zerotol) {
      nt[i - 2] = (ef - f[0]) / denom;
      if ((nt[i - 2] >= 0.0) && (nt[i - 2] <= 1.0)) PG_ADD();
    }
  }
  for (int k = 1; k <= 3; k++) {
    const int i = k % 3 + 1; iint++; const int j = i % 3 + 1;
    const double denom = f[i] - f[j];
    nt[0] = nt[1] = nt[2] = 0.0;
    if (fabs(denom) > zerotol) {
      nt[i - 1] = (ef - f[j]) / denom;
      nt[j - 1] = (f[i] - ef) / denom;
      if ((nt[i - 1] >= 0.0) && (nt[j - 1] >= 0.0)) PG_ADD();
    }
  }
  // efdif(i,j,k) = (e_i−e_j)(f_k−f_j) − (e_k−e_j)(f_i−f_j); efef(i,j) = (ef−e_i)(f_j−f_i) − (ef−f_i)(e_j−e_i)
#define EFDIF(i, j, k) ((e[(i)-1] - e[(j)-1]) * (f[(k)-1] - f[(j)-1]) - (e[(k)-1] - e[(j)-1]) * (f[(i)-1] - f[(j)-1]))
#define EFEF(i, j) ((ef - e[(i)-1]) * (f[(j)-1] - f[(i)-1]) - (ef - f[(i)-1]) * (e[(j)-1] - e[(i)-1]))
  for (int k = 1; k <= 3; k++) {
    const int i = k % 3 + 1; iint++; const int j = i % 3 + 1;
    const double denom1 = EFDIF(i + 1, 1, j + 1);
    const double denom2 = EFDIF(j + 1, 1, i + 1);
    nt[0] = nt[1] = nt[2] = 0.0;
    if ((fabs(denom1) > zerotol) && (fabs(denom2) > zerotol)) {
      nt[i - 1] = EFEF(1, j + 1) / denom1;
      nt[j - 1] = EFEF(1, i + 1) / denom2;
      const double sumnt = nt[i - 1] + nt[j - 1];
      if ((nt[i - 1] > 0.0) && (nt[j - 1] > 0.0) && (sumnt <= 1.0)) PG_ADD();
    }
  }
  {
    const double denom1 = EFDIF(2, 4, 3), denom2 = EFDIF(3, 4, 2), denom3 = EFDIF(4, 2, 3);
    iint++;
    if ((fabs(denom1) > zerotol) && (fabs(denom2) > zerotol) && (fabs(denom3) > zerotol)) {
      nt[0] = EFEF(4, 3) / denom1;
      nt[1] = EFEF(4, 2) / denom2;
      nt[2] = EFEF(2, 3) / denom3;
      if ((nt[0] > 0.0) && (nt[1] > 0.0) && (nt[2] > 0.0)) PG_ADD();
    }
  }
#undef EFDIF
#undef EFEF
#undef PG_ADD
  N.nnod = inod;
}

__device__ void unrepnodes(Nodes& N) {
  const double zerotol = 1.0e-8;
  int i = 1;
  while (i < N.nnod) {
    const double xi0 = N.x[i][0], xi1 = N.x[i][1], xi2 = N.x[i][2];
    int j = i + 1;
    while (j <= N.nnod) {
      double sumnt = 0.0;
      sumnt = sumnt + fabs(xi0 - N.x[j][0]);
      sumnt = sumnt + fabs(xi1 - N.x[j][1]);
      sumnt = sumnt + fabs(xi2 - N.x[j][2]);
      if (sumnt < zerotol) {
        N.ntype[i] |= (N.ntype[j] & 63);
        for (int k = j + 1; k <= N.nnod; k++) {
          N.x[k - 1][0] = N.x[k][0]; N.x[k - 1][1] = N.x[k][1]; N.x[k - 1][2] = N.x[k][2];
          N.ntype[k - 1] = N.ntype[k];
        }
        N.x[N.nnod][0] = N.x[N.nnod][1] = N.x[N.nnod][2] = 0.0;
        N.ntype[N.nnod] = 0;
        N.nnod = N.nnod - 1;
      } else {
        j = j + 1;
      }
    }
    i = i + 1;
  }
}

__device__ __forceinline__ double tlinap(const double* x, const double* fv) {
  double fx = fv[0];
  fx = fx + (fv[1] - fv[0]) * x[0];
  fx = fx + (fv[2] - fv[0]) * x[1];
  fx = fx + (fv[3] - fv[0]) * x[2];
  return fx;
}

__device__ int relnodes(Nodes& N, const double e[4], const double f[4], double ef) {
  const double zerotol = 1.00e-12;
  int info = 0, inod = 1, maxnod = N.nnod;
  bool keep = false;
  while (inod <= maxnod) {
    const double e1 = tlinap(N.x[inod], e) - ef;
    const double e2 = tlinap(N.x[inod], f) - ef;
    const int t = N.ntype[inod];
    if (t >= 7 && t <= 15) {
      keep = ((e1 < 0.0) || (fabs(e1) <= zerotol)) && ((e2 > 0.0) || (fabs(e2) <= zerotol));
    } else if (t >= 16 && t <= 31) {
      keep = (e2 > 0.0) || (fabs(e2) <= zerotol);
    } else if (t >= 32 && t <= 47) {
      keep = (e1 < 0.0) || (fabs(e1) <= zerotol);
    } else if (t >= 48 && t <= 63) {
      keep = true;
    } else {
      info = 1;
    }
    if (keep) {
      inod = inod + 1;
    } else {
      for (int jn = inod + 1; jn <= maxnod; jn++) {
        N.x[jn - 1][0] = N.x[jn][0]; N.x[jn - 1][1] = N.x[jn][1]; N.x[jn - 1][2] = N.x[jn][2];
        N.ntype[jn - 1] = N.ntype[jn];
      }
      maxnod = maxnod - 1;
    }
  }
  for (int in = maxnod + 1; in <= N.nnod; in++) {
    N.x[in][0] = N.x[in][1] = N.x[in][2] = 0.0;
    N.ntype[in] = 0;
  }
  N.nnod = maxnod;
  return info;
}

// Bit test that treats the reference's undefined bit positions (an unset
// plane slot) as "not set" and records them.
__device__ __forceinline__ bool bt(int nt, int pos, Ctx& cx) {
  if (pos < 0 || pos > 7) { cx.status |= PG_ERR_UNDEFINED; return false; }
  return (nt >> pos) & 1;
}

// sortnodes (for_tetrahedra2.f90:2306-2773).  index[inod][isub] 1-based, 0 = unset.
__device__ int sortnodes(const Nodes& N, int index[9][2], Ctx& cx) {
  const int nnod = N.nnod;
  const int UNSET = -1;
  int spl[6] = {0, 0, 0, 0, 0, 0};
  int it = 0, is = 0, ip = 0, info = 0;
  int triangle[7], square[7], penta[3], ibt[4];
  for (int i = 0; i < 7; i++) triangle[i] = square[i] = UNSET;
  penta[0] = penta[1] = penta[2] = UNSET;
  ibt[0] = ibt[1] = ibt[2] = ibt[3] = UNSET;
  int signbit = UNSET, signbita = UNSET, signbitb = UNSET;
  int signnod = 0, signnodb = 0, iind = 0;
  for (int a = 0; a < 9; a++) index[a][0] = index[a][1] = 0;
  auto nty = [&](int inod) -> int {
    if (inod < 1 || inod > nnod) { cx.status |= PG_ERR_UNDEFINED; return 0; }
    return N.ntype[inod];
  };
  auto tri = [&](int k) -> int {
    if (k < 1 || k > 6) { cx.status |= PG_ERR_UNDEFINED; return UNSET; }
    return triangle[k];
  };
  if (nnod == 5) {
    for (int ibit = 0; ibit <= 5; ibit++) {
      for (int inod = 1; inod <= 5; inod++) if (bt(N.ntype[inod], ibit, cx)) spl[ibit]++;
      if (spl[ibit] == 3) { it++; triangle[it] = ibit; }
      else if (spl[ibit] == 4) { is++; square[is] = ibit; signbit = ibit; }
    }
    if (is != 0) {
      int is1 = 1;
      for (int inod = 1; inod <= 5; inod++) {
        if (bt(N.ntype[inod], tri(1), cx)) {
          if (!bt(N.ntype[inod], signbit, cx)) {
            index[inod][0] = 2;
          } else {
            index[inod][0] = is1;
            is1 = is1 + 2;
            signnod = inod;
          }
        }
      }
      for (int i = 2; i <= 4; i++) if (bt(nty(signnod), tri(i), cx)) signbit = triangle[i];
      for (int inod = 1; inod <= 5; inod++)
        if (index[inod][0] == 0) index[inod][0] = bt(N.ntype[inod], signbit, cx) ? 5 : 4;
    } else {
      for (int inod = 1; inod <= 5; inod++) {
        int nb = 0;
        for (int ibit = 0; ibit <= 5; ibit++) if (bt(N.ntype[inod], ibit, cx)) nb++;
        index[inod][0] = (nb == 3) ? 1 : 2;   // the reference's counters restart per node
      }
    }
  } else if (nnod == 6) {
    for (int ibit = 0; ibit <= 5; ibit++) {
      for (int inod = 1; inod <= 6; inod++) if (bt(N.ntype[inod], ibit, cx)) spl[ibit]++;
      if (spl[ibit] == 3) { it++; triangle[it] = ibit; }
      else if (spl[ibit] == 4) { is++; square[is] = ibit; }
    }
    if (is == 2) {
      int cnt = 1;
      for (int inod = 1; inod <= 6; inod++) {
        if (bt(N.ntype[inod], square[1], cx) && bt(N.ntype[inod], square[2], cx)) {
          index[inod][0] = 2 + (cnt - 1) * 3;
          if (cnt == 1) signnod = inod;
          if (cnt == 2) signnodb = inod;
          cnt++;
        }
      }
      int sigtri[7] = {0, 0, 0, 0, 0, 0, 0};
      for (int inod = 1; inod <= 6; inod++)
        for (int k = 1; k <= 4; k++) if (bt(N.ntype[inod], tri(k), cx)) sigtri[inod]++;
      for (int k = 1; k <= 4; k++) {
        if (bt(nty(signnod), tri(k), cx)) signbita = k;
        if (bt(nty(signnodb), tri(k), cx)) signbitb = k;
      }
      for (int inod = 1; inod <= 6; inod++) {
        if (index[inod][0] == 0) {
          const int ta = tri(signbita == UNSET ? 0 : signbita), tb = tri(signbitb == UNSET ? 0 : signbitb);
          if (sigtri[inod] == 3 && bt(N.ntype[inod], ta, cx)) index[inod][0] = 4;
          if (sigtri[inod] == 2 && bt(N.ntype[inod], ta, cx)) index[inod][0] = 1;
          if (sigtri[inod] == 3 && bt(N.ntype[inod], tb, cx)) index[inod][0] = 3;
          if (sigtri[inod] == 2 && bt(N.ntype[inod], tb, cx)) index[inod][0] = 6;
        }
      }
    } else if (is == 3) {
      for (int inod = 1; inod <= 6; inod++) {
        for (int k = 1; k <= 2; k++) {
          if (bt(N.ntype[inod], tri(k), cx)) {
            if (bt(N.ntype[inod], square[1], cx) && bt(N.ntype[inod], square[2], cx)) index[inod][0] = 1 + 3 * (k - 1);
            else if (bt(N.ntype[inod], square[1], cx)) index[inod][0] = 2 + 3 * (k - 1);
            else if (bt(N.ntype[inod], square[2], cx)) index[inod][0] = 3 + 3 * (k - 1);
            else { cx.status |= PG_ERR_SORTNODES; info = 61; }
          }
        }
      }
    }
  } else if (nnod == 7 || nnod == 8) {
    for (int ibit = 0; ibit <= 5; ibit++) {
      for (int inod = 1; inod <= nnod; inod++) if (bt(N.ntype[inod], ibit, cx)) spl[ibit]++;
      if (spl[ibit] == 3) { it++; triangle[it] = ibit; }
      else if (spl[ibit] == 4) { is++; square[is] = ibit; }
      else if (spl[ibit] == 5) { ip++; if (ip <= 2) penta[ip] = ibit; else cx.status |= PG_ERR_UNDEFINED; }
    }
    if (nnod == 7) {
      if (it == 2) {
        if (is == 4) {
          for (int inod = 1; inod <= 7; inod++) {
            if (bt(N.ntype[inod], triangle[1], cx) && bt(N.ntype[inod], triangle[2], cx)) {
              index[inod][0] = index[inod][1] = 2;
              signnod = inod;
            }
          }
          int is1 = 0;
          for (int ibit = 0; ibit <= 5; ibit++) {
            if (bt(nty(signnod), ibit, cx) && (spl[ibit] == 4) && (is1 == 0)) { signbita = ibit; is1++; }
            else if (bt(nty(signnod), ibit, cx) && (spl[ibit] == 4)) signbitb = ibit;
          }
          for (int inod = 1; inod <= 7; inod++) {
            if (inod != signnod) {
              const int t = N.ntype[inod];
              if (bt(t, triangle[1], cx) && bt(t, signbita, cx)) index[inod][0] = 1;
              else if (bt(t, triangle[1], cx) && bt(t, signbitb, cx)) index[inod][0] = 3;
              else if (bt(t, triangle[2], cx) && bt(t, signbita, cx)) index[inod][1] = 1;
              else if (bt(t, triangle[2], cx) && bt(t, signbitb, cx)) index[inod][1] = 3;
              else if (bt(t, signbita, cx)) index[inod][0] = index[inod][1] = 4;
              else index[inod][0] = index[inod][1] = 5;
            }
          }
        } else {
          info = 72; cx.status |= PG_ERR_SORTNODES;
        }
      } else if (it == 3) {
        for (int inod = 1; inod <= 7; inod++) {
          int nb = 0;
          for (int k = 1; k <= 3; k++) if (bt(N.ntype[inod], triangle[k], cx)) nb++;
          if (bt(N.ntype[inod], penta[1], cx)) {
            if (nb == 2) index[inod][0] = 1;
          } else {
            if (nb == 2) { index[inod][0] = 2; index[inod][1] = 1; }
            else { index[inod][1] = 4; iind = inod; }
          }
        }
        for (int k = 1; k <= 3; k++) if (bt(nty(iind), triangle[k], cx)) signbita = triangle[k];
        for (int inod = 1; inod <= 7; inod++) {
          if (index[inod][0] == 0 && index[inod][1] == 0) {
            const int t = N.ntype[inod];
            if (bt(t, signbita, cx) && bt(t, square[1], cx)) index[inod][1] = 5;
            else if (bt(t, signbita, cx) && bt(t, square[2], cx)) { index[inod][0] = 5; index[inod][1] = 2; }
            else if (bt(t, square[1], cx)) { index[inod][0] = 4; index[inod][1] = 3; }
            else index[inod][0] = 3;
          }
        }
      } else {
        info = 73; cx.status |= PG_ERR_SORTNODES;
      }
    } else {  // nnod == 8
      if (is == 2) {
        for (int inod = 1; inod <= 8; inod++) {
          const int t = N.ntype[inod];
          for (int it1 = 1; it1 <= 2; it1++) {
            if (bt(t, triangle[it1], cx)) {
              if (bt(t, penta[1], cx) && bt(t, penta[2], cx)) index[inod][0] = 1 + (it1 - 1) * 3;
              else if (bt(t, penta[1], cx)) index[inod][0] = 2 + (it1 - 1) * 3;
              else if (bt(t, penta[2], cx)) index[inod][0] = 3 + (it1 - 1) * 3;
            }
          }
          for (int iq1 = 1; iq1 <= 2; iq1++) {
            if (bt(t, penta[iq1], cx)) {
              if (bt(t, square[1], cx) && bt(t, square[2], cx)) index[inod][1] = 1 + (iq1 - 1) * 3;
              else if (bt(t, square[1], cx)) index[inod][1] = 2 + (iq1 - 1) * 3;
              else if (bt(t, square[2], cx)) index[inod][1] = 3 + (iq1 - 1) * 3;
            }
          }
        }
      } else if (is == 6) {
        int is1 = 0;
        index[1][0] = 1;
        index[1][1] = 0;
        for (int ibit = 0; ibit <= 5; ibit++) {
          if (bt(N.ntype[1], ibit, cx)) { is1++; if (is1 <= 3) ibt[is1] = ibit; else cx.status |= PG_ERR_UNDEFINED; }
        }
        for (int inod = 2; inod <= 8; inod++) {
          const int t = N.ntype[inod];
          if (bt(t, ibt[1], cx)) {
            if (bt(t, ibt[2], cx)) index[inod][0] = index[inod][1] = 2;
            else if (bt(t, ibt[3], cx)) index[inod][0] = index[inod][1] = 3;
            else { index[inod][0] = 0; index[inod][1] = 1; }
          } else if (bt(t, ibt[2], cx)) {
            if (bt(t, ibt[3], cx)) { index[inod][0] = 4; index[inod][1] = 0; }
            else index[inod][0] = index[inod][1] = 5;
          } else {
            if (bt(t, ibt[3], cx)) index[inod][0] = index[inod][1] = 6;
            else { index[inod][0] = 0; index[inod][1] = 4; }
          }
        }
      } else {
        info = 81; cx.status |= PG_ERR_SORTNODES;
      }
    }
  }
  return info;
}

// Corner energies of item (tetrahedron, band pair) and its integration
// polyhedron: surfnodes → unrepnodes → relnodes → sortnodes
// (for_tetrahedra3.f90:3-136 up to the nnod dispatch).  Returns true when
// the item contributes zero (skipped by the reference's tests at
// for_tetrahedra.f90:447/452, fewer than 4 nodes, or a geometry error).
struct Item {
  int tet, pair;
  double e[4], f[4];
};
__device__ bool item_geometry(const Params& p, long long item, Item& it, Nodes& N, int index[9][2], Ctx& cx) {
  const int P = p.nb1 * p.nb2;
  it.tet = (int)(item / P);
  it.pair = (int)(item - (long long)it.tet * P);
  const int ib = it.pair % p.nb1;
  const int jb = it.pair / p.nb1;
  const int lt = 6 * p.kqid[it.tet / 6] + it.tet % 6;   // linked k−q tetrahedron (for_tetrahedra.f90:426-432)
#pragma unroll
  for (int i = 0; i < 4; i++) {
    it.e[i] = p.enk[(size_t)ib + (size_t)p.nbnd * p.tetc[i + 4 * it.tet]];
    it.f[i] = p.enk[(size_t)(jb + p.ncg + p.numin) + (size_t)p.nbnd * p.tetc[i + 4 * lt]];
  }
  const double fhi = fmax(fmax(it.f[0], it.f[1]), fmax(it.f[2], it.f[3]));
  const double emin = fmin(fmin(it.e[0], it.e[1]), fmin(it.e[2], it.e[3]));
  bool zero = (fhi <= p.ef) || (emin > p.ef);   // for_tetrahedra.f90:447, 452
  if (!zero) {
    cx.cnt[PG_CNT_CALLS]++;
    surfnodes(N, it.e, it.f, p.ef);
    unrepnodes(N);
    if (relnodes(N, it.e, it.f, p.ef) != 0) { cx.status |= PG_ERR_RELNODES; zero = true; }
    else if (N.nnod > 8) { cx.status |= PG_ERR_NNOD; zero = true; }
    else if (sortnodes(N, index, cx) != 0) { zero = true; }
    else {
      cx.cnt[PG_CNT_NNOD0 + N.nnod]++;
      if (N.nnod < 4) zero = true;
    }
  }
  return zero;
}

// Corners of the pentahedron (5) / prism (6) — two of them for 7 and 8 nodes —
// from the node order sortnodes produced (genericfunf_par / genericprism_par
// inputs, for_tetrahedra3.f90:60-131).
__device__ void place_nodes(const Nodes& N, const int index[9][2], double tc[2][6][3], Ctx& cx) {
  const int nnod = N.nnod;
  const int cap = (nnod == 5 || nnod == 7) ? 5 : 6;
  const int ngroup = (nnod >= 7) ? 2 : 1;
  bool written[6] = {false, false, false, false, false, false};
  for (int a = 0; a < 6; a++) for (int c = 0; c < 3; c++) tc[0][a][c] = tc[1][a][c] = 0.0;
  for (int g = 0; g < ngroup; g++) {
    if (g == 1) for (int a = 0; a < 6; a++) for (int c = 0; c < 3; c++) tc[1][a][c] = tc[0][a][c];
    for (int inod = 1; inod <= nnod; inod++) {
      const int pos = index[inod][g];
      if (ngroup == 2 && pos == 0) continue;
      if (pos < 1 || pos > cap) { cx.status |= PG_ERR_UNDEFINED; continue; }
      for (int c = 0; c < 3; c++) tc[g][pos - 1][c] = N.x[inod][c];
      written[pos - 1] = true;
    }
    for (int a = 0; a < cap; a++) if (!written[a]) cx.status |= PG_ERR_UNDEFINED;
  }
}

// Class of an item for the work sort: 0 = contributes zero; otherwise
// 1 + 6·(nnod − 4) + grouping of its first sub-tetrahedron (0: below the
// volume tolerance, 1..5: sorteq case 4/6/8/10/16).  Items of one class run
// the same code path, so sorting by class keeps warps converged.
constexpr int NCLASS = 32;
__host__ __device__ constexpr int class_nnod(int c) { return (c - 1) / 6 + 4; }
// Sub-tetrahedra per polyhedron half: 1 (4 nodes), 2 (pentahedron: 5 or 7
// nodes), 3 (prism: 6 or 8); 7 and 8 nodes have two halves.
__host__ __device__ constexpr int nodes_nsub(int nnod) { return nnod == 4 ? 1 : (nnod == 5 || nnod == 7) ? 2 : 3; }
__host__ __device__ constexpr int nodes_ngroup(int nnod) { return nnod >= 7 ? 2 : 1; }
constexpr int MAX_SUBTET = 6;   // sub-tetrahedra of one item at most (8 nodes: 2 × 3)

// Geometry pass over the items of one tetrahedron chunk (frequency-
// independent): builds the integration polyhedron of each item
// (item_geometry), splits it into sub-tetrahedra (place_nodes, the
// genericfunf_par / genericprism_par corner order), sets each one up
// (setup_subtet: volume, sorteq grouping, closed-form coefficients) and
// stores the set-up sub-tetrahedra as records for k_tet_eval, the item's
// first record index in recoff and its class in cls.  Records are
// claimed with one atomic per item; their order in the array does not matter
// (each item reads back only its own, in its own order).  The per-item and
// per-sub-tetrahedron counters (calls, node counts, groupings, zero volumes)
// are counted here, once.
__global__ void __launch_bounds__(128) k_tet_geometry(Params p, long long nitems, unsigned char* cls,
                                                      unsigned* hist) {
  __shared__ unsigned h[NCLASS];
  if (threadIdx.x < NCLASS) h[threadIdx.x] = 0;
  __syncthreads();
  const long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (li < nitems) {
    Ctx cx;
    cx.status = 0;
    for (int i = 0; i < PG_NCOUNTERS; i++) cx.cnt[i] = 0;
    const int P = p.nb1 * p.nb2;
    const long long item = (long long)p.tet0 * P + li;
    Item it;
    Nodes N;
    int index[9][2];
    int cl = 0;
    if (!item_geometry(p, item, it, N, index, cx)) {
      const int nnod = N.nnod;
      const int nsub = nodes_nsub(nnod), ngroup = nodes_ngroup(nnod);
      const unsigned r0 = atomicAdd(p.nrec, (unsigned)(nsub * ngroup));
      p.recoff[li] = (int)r0;
      double tc[2][6][3];
      if (nnod > 4) place_nodes(N, index, tc, cx);
      int g0 = 0;
      for (int g = 0; g < ngroup; g++) {
        for (int st = 0; st < nsub; st++) {
          SubTet& s = p.recs[r0 + g * nsub + st];
          for (int n = 0; n < 4; n++)
            for (int c = 0; c < 3; c++) s.corner[n][c] = (nnod == 4) ? N.x[n + 1][c] : tc[g][st + n][c];
          setup_subtet(s, it.e, it.f, cx);
          int grp = 0;
          if (s.vol < ZTOL_VOL) {
            cx.cnt[PG_CNT_ZERO_VOL]++;
          } else {
            grp = s.flag == 4 ? 1 : s.flag == 6 ? 2 : s.flag == 8 ? 3 : s.flag == 10 ? 4 : 5;
            cx.cnt[PG_CNT_EQ4 + grp - 1]++;
          }
          if (g == 0 && st == 0) g0 = grp;
        }
      }
      cl = 1 + 6 * (nnod - 4) + g0;
    }
    cls[li] = (unsigned char)cl;
    atomicAdd(&h[cl], 1u);
    if (p.status && cx.status) atomicOr(p.status, cx.status);
    if (p.counters) {
      for (int i = 0; i < PG_NCOUNTERS; i++)
        if (cx.cnt[i]) atomicAdd(p.counters + i, cx.cnt[i]);
    }
  }
  __syncthreads();
  if (threadIdx.x < NCLASS && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

// Exclusive prefix of the class histogram → per-class write cursors, the
// classes in descending order: the largest polyhedra (the most sub-tetrahedra
// per item) run first and the items that contribute zero last, so the last
// wave of blocks is short (ascending order left most SMs idle behind a tail
// of 8-node items).
__global__ void k_class_offsets(const unsigned* hist, unsigned* cursor) {
  if (threadIdx.x == 0) {
    unsigned acc = 0;
    for (int c = NCLASS - 1; c >= 0; c--) { cursor[c] = acc; acc += hist[c]; }
  }
}

// order[cursor[class]++] = item, one atomic per (warp, class).  The order
// within a class is arbitrary; results do not depend on it (every item
// writes only its own slots, counters are integer sums).
__global__ void k_class_scatter(const unsigned char* cls, long long nitems, unsigned* cursor, int* order) {
  const long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = item < nitems;
  const int c = in ? cls[item] : -1;
  const unsigned lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(0xffffffffu, c);
  const unsigned leader = __ffs(peers) - 1;
  const unsigned rank = __popc(peers & ((1u << lane) - 1u));
  unsigned base = 0;
  if (in && lane == leader) base = atomicAdd(&cursor[c], (unsigned)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  if (in) order[base + rank] = (int)item;
}

// Evaluation pass: one thread per (item of the chunk in class order,
// frequency), the frequency fastest, so a warp covers one or two items and
// follows one code path.  Each thread evaluates its item's sub-tetrahedra at
// its frequency from the records (read through L1; the lanes of an item read
// the same addresses) and writes the four corner weights into the scratch
// slots, summing exactly as the reference does: the first polyhedron's
// sub-tetrahedra in order (generictetra_par results added one by one), the
// second polyhedron of a 7- or 8-node item summed separately from 0 and then
// added (for_tetrahedra3.f90:60-131).
__global__ void __launch_bounds__(128, 4) k_tet_eval(Params p, long long nitems, const unsigned char* __restrict__ cls) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = t < nitems * p.nomc;
  Ctx cx;
  cx.status = 0;
  cx.cnt[PG_CNT_BIGW_WARN] = 0;
  cx.cnt[PG_CNT_BIGW_ZEROED] = 0;
  unsigned n_exact = 0, n_taylor = 0;
  if (in) {
    const int P = p.nb1 * p.nb2;
    const long long pos = t / p.nomc;
    const int w = (int)(t - pos * p.nomc);
    const int li = p.order[pos];
    const long long item = (long long)p.tet0 * P + li;
    const int tet = (int)(item / P), pair = (int)(item - (long long)tet * P);
    const size_t cstride = (size_t)p.nomc * P;
    double* out = p.scratch + (size_t)tet * 4 * cstride + (size_t)w * P + pair;
    const int cl = cls[li];
    double o[4] = {0.0, 0.0, 0.0, 0.0};
    if (cl != 0) {
      const double omeg = p.omega[p.om0 + w];
      const int nnod = class_nnod(cl);
      const int nsub = nodes_nsub(nnod);
      const SubTet* r = p.recs + p.recoff[li];
      // records in order: the first polyhedron's nsub sub-tetrahedra, then
      // (7, 8 nodes) the second's; one evaluation site keeps the code small.
      // With the reference's wtemp addressing (ref_layout) a 7- or 8-node
      // item's first half is replaced, from the third frequency on, by its
      // second half two frequencies earlier (for_tetrahedra3.f90:36, 100-120):
      // the second half's records are evaluated once more at that frequency
      // (not counted: the reference evaluates each (sub-tetrahedron, ω) once).
      const int nrec = nsub * nodes_ngroup(nnod);
      const int jg = p.om0 + w;
      const int nextra = (p.ref_layout && nrec > nsub && jg >= 2) ? nsub : 0;
      const double omeg_b = nextra ? p.omega[jg - 2] : omeg;
      double acc[4] = {0.0, 0.0, 0.0, 0.0}, acc_b[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll 1
      for (int i = 0; i < nrec + nextra; i++) {
        const bool extra = i >= nrec;
        const int ri = extra ? i - nsub : i;
        const SubTet& s = r[ri];
        const bool second = ri >= nsub;
        const int st = second ? ri - nsub : ri;
        const double om_i = extra ? omeg_b : omeg;
        double wo[4] = {0.0, 0.0, 0.0, 0.0};
        const bool live = s.vol >= ZTOL_VOL;
        if (live) {
          const unsigned long long bw = cx.cnt[PG_CNT_BIGW_WARN], bz = cx.cnt[PG_CNT_BIGW_ZEROED];
          eval_subtet(s, om_i, wo, cx);
          if (extra) {
            cx.cnt[PG_CNT_BIGW_WARN] = bw;
            cx.cnt[PG_CNT_BIGW_ZEROED] = bz;
          } else if (om_i > s.taylor_omega) {
            n_taylor++;
          } else {
            n_exact++;
          }
        }
        if (!second) {
          // the first one sets the slots (0.0 below the volume tolerance),
          // later ones below the tolerance add nothing
#pragma unroll
          for (int c = 0; c < 4; c++) o[c] = (st == 0) ? wo[c] : (live ? o[c] + wo[c] : o[c]);
        } else if (!extra) {
          // the second polyhedron sums from 0 on its own, then adds in
#pragma unroll
          for (int c = 0; c < 4; c++) acc[c] = (st == 0) ? (0.0 + wo[c]) : (acc[c] + wo[c]);
        } else {
#pragma unroll
          for (int c = 0; c < 4; c++) acc_b[c] = (st == 0) ? (0.0 + wo[c]) : (acc_b[c] + wo[c]);
        }
      }
      if (nrec > nsub) {
#pragma unroll
        for (int c = 0; c < 4; c++) o[c] = (nextra ? acc_b[c] : o[c]) + acc[c];
      }
#pragma unroll
      for (int c = 0; c < 4; c++)
        if (!isfinite(o[c])) cx.status |= PG_ERR_NONFINITE;
    }
#pragma unroll
    for (int c = 0; c < 4; c++) out[c * cstride] = o[c];
  }
  // status and counters: one atomic per warp
  const unsigned st_w = __reduce_or_sync(0xffffffffu, cx.status);
  const unsigned ex_w = __reduce_add_sync(0xffffffffu, n_exact);
  const unsigned ty_w = __reduce_add_sync(0xffffffffu, n_taylor);
  const unsigned bw_w = __reduce_add_sync(0xffffffffu, (unsigned)cx.cnt[PG_CNT_BIGW_WARN]);
  const unsigned bz_w = __reduce_add_sync(0xffffffffu, (unsigned)cx.cnt[PG_CNT_BIGW_ZEROED]);
  if ((threadIdx.x & 31) == 0) {
    if (p.status && st_w) atomicOr(p.status, st_w);
    if (p.counters) {
      if (ex_w) atomicAdd(p.counters + PG_CNT_EXACT, (unsigned long long)ex_w);
      if (ty_w) atomicAdd(p.counters + PG_CNT_TAYLOR, (unsigned long long)ty_w);
      if (bw_w) atomicAdd(p.counters + PG_CNT_BIGW_WARN, (unsigned long long)bw_w);
      if (bz_w) atomicAdd(p.counters + PG_CNT_BIGW_ZEROED, (unsigned long long)bz_w);
    }
  }
}

// ------------------------------------------------------------------- CSR
// Slot s = 4*tet + corner.  kptr[k]..kptr[k+1] lists the slots of point k in
// ascending s (= ascending tetrahedron, then corner), the reference's
// accumulation order (for_tetrahedra.f90:439, 455-458).
__global__ void k_kcsr_count(const int* tetc, int ntet, int nkp, int* kcount) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nkp) return;
  int c = 0;
  for (int s = 0; s < 4 * ntet; s++) c += (tetc[s] == k);
  kcount[k] = c;
}

__global__ void k_kcsr_scan(const int* kcount, int nkp, int* kptr) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int acc = 0;
    for (int k = 0; k < nkp; k++) { kptr[k] = acc; acc += kcount[k]; }
    kptr[nkp] = acc;
  }
}

__global__ void k_kcsr_fill(const int* tetc, int ntet, int nkp, const int* kptr, int* kslot) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nkp) return;
  int o = kptr[k];
  for (int s = 0; s < 4 * ntet; s++)
    if (tetc[s] == k) kslot[o++] = s;
}

// ---------------------------------------------------------------- gather
// kcw[pair + P*(k + nkp*ω)] for the ω chunk.
__global__ void k_gather(const double* scratch, const int* kptr, const int* kslot, int P, int nkp, int nomc,
                         int om0, double wtet, double* kcw) {
  const int pair = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  const int w = blockIdx.z;
  if (pair >= P) return;
  double acc = 0.0;
  const int b = kptr[k], e = kptr[k + 1];
  for (int i = b; i < e; i++) {
    const int s = kslot[i];
    const int tet = s >> 2, c = s & 3;
    const double v = scratch[(((size_t)tet * 4 + c) * nomc + w) * P + pair];
    acc = acc + v * 6.0 * wtet;
  }
  kcw[(size_t)pair + (size_t)P * ((size_t)k + (size_t)nkp * (om0 + w))] = acc;
}

// ------------------------------------------------------ SVD projection
// par3 (for_tetrahedra.f90:505-513): every (tetrahedron, corner, pair) weight
// vector over ω projected on the SVD basis, w2(l) = Σ_ω w1(ω)·dUl(ω,l), ω
// ascending (the oracle's matmul order; no contraction: -fmad=false).
// dUl (nom, nl) Fortran order is staged in shared memory.
__global__ void k_svd_project(const double* __restrict__ scratch, const double* __restrict__ dUl, int nom, int nl,
                              int P, long long nslot, double* __restrict__ scratch2) {
  extern __shared__ double du[];
  for (int i = threadIdx.x; i < nom * nl; i += blockDim.x) du[i] = dUl[i];
  __syncthreads();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // (slot, pair), slot = 4·tet + corner
  if (t >= nslot * P) return;
  const long long slot = t / P;
  const int pair = (int)(t - slot * P);
  const double* src = scratch + (size_t)slot * nom * P + pair;
  for (int l = 0; l < nl; l++) {
    double acc = 0.0;
    for (int w = 0; w < nom; w++) acc = acc + src[(size_t)w * P] * du[w + nom * l];
    scratch2[((size_t)slot * nl + l) * P + pair] = acc;
  }
}

}  // namespace pgw

// -------------------------------------------------------------- C-ABI part
using namespace pgw;

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Workspace of the weight passes: the k → slot lists (CSR), the per-chunk
// item arrays (class, class order, first record), the class histogram and
// record counter, the sub-tetrahedron records of one tetrahedron chunk, and
// the scratch weights [ntet][4][nomc][P] (plus the SVD-projected copy for
// par3).  The chunk is the most tetrahedra whose records fit in rec_budget
// even when every item yields the maximum of six sub-tetrahedra.
constexpr size_t REC_BUDGET = 1ull << 30;
struct WLayout {
  int tpc;   // tetrahedra per chunk
  size_t kptr, kcount, kslot, cls, order, recoff, hist, cursor, recs, scratch, scratch2, total;
};
static WLayout weights_layout(int nkp, int ntet, long long P, int nomc, int nl, size_t rec_budget) {
  WLayout L;
  long long tpc = (long long)(rec_budget / ((size_t)P * MAX_SUBTET * sizeof(SubTet)));
  if (tpc < 1) tpc = 1;
  if (tpc > ntet) tpc = ntet;
  L.tpc = (int)tpc;
  const size_t ci = (size_t)tpc * P;
  size_t o = 0;
  L.kptr = o; o += align256(sizeof(int) * (size_t)(nkp + 1));
  L.kcount = o; o += align256(sizeof(int) * (size_t)nkp);
  L.kslot = o; o += align256(sizeof(int) * (size_t)4 * ntet);
  L.cls = o; o += align256(ci);
  L.order = o; o += align256(sizeof(int) * ci);
  L.recoff = o; o += align256(sizeof(int) * ci);
  L.hist = o; o += align256(sizeof(unsigned) * (NCLASS + 1));
  L.cursor = o; o += align256(sizeof(unsigned) * NCLASS);
  L.recs = o; o += align256(ci * MAX_SUBTET * sizeof(SubTet));
  L.scratch = o; o += align256(sizeof(double) * (size_t)4 * ntet * nomc * P);
  L.scratch2 = o; o += nl > 0 ? align256(sizeof(double) * (size_t)4 * ntet * nl * P) : 0;
  L.total = o;
  return L;
}

// k → (tetrahedron, corner) slot lists.
static void enqueue_kcsr(const WLayout& L, char* w, const int* tetc, int ntet, int nkp, cudaStream_t s) {
  int* kptr = (int*)(w + L.kptr);
  int* kcount = (int*)(w + L.kcount);
  int* kslot = (int*)(w + L.kslot);
  k_kcsr_count<<<(nkp + 127) / 128, 128, 0, s>>>(tetc, ntet, nkp, kcount);
  k_kcsr_scan<<<1, 1, 0, s>>>(kcount, nkp, kptr);
  k_kcsr_fill<<<(nkp + 127) / 128, 128, 0, s>>>(tetc, ntet, nkp, kptr, kslot);
  pg_count_launches(3);
}

// Scratch weights of frequencies om0 … om0+nomc−1 (p.om0, p.nomc) for every
// tetrahedron, chunk by chunk: geometry and records, class order, evaluation.
static int enqueue_tet_weights(Params p, const WLayout& L, char* w, cudaStream_t s) {
  unsigned char* cls = (unsigned char*)(w + L.cls);
  unsigned* hist = (unsigned*)(w + L.hist);
  unsigned* cursor = (unsigned*)(w + L.cursor);
  int* order = (int*)(w + L.order);
  p.order = order;
  p.recoff = (int*)(w + L.recoff);
  p.recs = (SubTet*)(w + L.recs);
  p.nrec = hist + NCLASS;
  const long long P = (long long)p.nb1 * p.nb2;
  for (int t0 = 0; t0 < p.ntet; t0 += L.tpc) {
    const int ntc = (t0 + L.tpc <= p.ntet) ? L.tpc : p.ntet - t0;
    const long long ni = (long long)ntc * P;
    const unsigned nblk = (unsigned)((ni + 127) / 128);
    p.tet0 = t0;
    if (cudaMemsetAsync(hist, 0, sizeof(unsigned) * (NCLASS + 1), s) != cudaSuccess) return PG_ECUDA;
    k_tet_geometry<<<nblk, 128, 0, s>>>(p, ni, cls, hist);
    k_class_offsets<<<1, 32, 0, s>>>(hist, cursor);
    k_class_scatter<<<nblk, 128, 0, s>>>(cls, ni, cursor, order);
    const long long nt = ni * p.nomc;
    k_tet_eval<<<(unsigned)((nt + 127) / 128), 128, 0, s>>>(p, ni, cls);
    pg_count_launches(4);
  }
  return PG_OK;
}

// Reproduce the reference's addressing of wtemp(4,2,nom) for 7- and 8-node
// polyhedra (process-wide; read by every later call): off = add the two halves
// at every frequency.
static std::atomic<int> g_ref_layout{0};
extern "C" int pg_set_weights_reference_layout(int on) {
  g_ref_layout.store(on ? 1 : 0);
  return PG_OK;
}
extern "C" int pg_weights_reference_layout(void) { return g_ref_layout.load(); }

static Params make_params(const double* enk, int nbnd, int nkp, double ef, const int* kqid, int ncg, int numin,
                          int nb1, int nb2, const double* omega, const int* tetc, int ntet, double* scratch,
                          unsigned* d_status, unsigned long long* d_counters) {
  Params p;
  memset(&p, 0, sizeof(p));
  p.enk = enk; p.kqid = kqid; p.omega = omega; p.tetc = tetc; p.scratch = scratch;
  p.status = d_status; p.counters = d_counters; p.ef = ef;
  p.nbnd = nbnd; p.nkp = nkp; p.ncg = ncg; p.numin = numin; p.nb1 = nb1; p.nb2 = nb2; p.ntet = ntet;
  p.ref_layout = g_ref_layout.load();
  return p;
}

extern "C" size_t pg_bz_calcqdepw_par2_workspace(int nbnd, int nkp, int ncg, int nomx, int numin, int nom, int ntet,
                                                  int nom_chunk) {
  const long long nb1 = ncg + nomx + 1, nb2 = nbnd - ncg - numin;
  if (nb1 <= 0 || nb2 <= 0 || nkp <= 0 || ntet <= 0 || nom <= 0) return 0;
  const int nomc = (nom_chunk > 0 && nom_chunk < nom) ? nom_chunk : nom;
  return weights_layout(nkp, ntet, nb1 * nb2, nomc, 0, REC_BUDGET).total;
}

static int par2_impl(const double* enk, int nbnd, int nkp, double ef, const int* kqid, int ncg, int nomx, int numin,
                     const double* omega, int nom, const int* tetc, int ntet, double* kcw, void* work,
                     size_t work_bytes, int nom_chunk, size_t rec_budget, unsigned* d_status,
                     unsigned long long* d_counters, void* stream) {
  const int nb1 = ncg + nomx + 1, nb2 = nbnd - ncg - numin;
  if (!enk || !kqid || !omega || !tetc || !kcw || !work) return PG_EARG;
  if (nb1 <= 0 || nb2 <= 0 || nkp <= 0 || ntet <= 0 || nom <= 0 || ncg < 0 || numin < 0) return PG_EARG;
  if (ntet != 6 * nkp) return PG_EARG;   // tetln = 6*kqid(ik)+it needs six tetrahedra per point
  const long long items = (long long)nb1 * nb2 * ntet;
  if (items >= (1ll << 31)) return PG_ETOOBIG;   // item indices are int
  const int nomc = (nom_chunk > 0 && nom_chunk < nom) ? nom_chunk : nom;
  const WLayout L = weights_layout(nkp, ntet, (long long)nb1 * nb2, nomc, 0, rec_budget);
  if (work_bytes < L.total) return PG_EWORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  char* w = (char*)work;
  double* scratch = (double*)(w + L.scratch);
  enqueue_kcsr(L, w, tetc, ntet, nkp, s);
  const int P = nb1 * nb2;
  Params p = make_params(enk, nbnd, nkp, ef, kqid, ncg, numin, nb1, nb2, omega, tetc, ntet, scratch, d_status,
                         d_counters);
  for (int om0 = 0; om0 < nom; om0 += nomc) {
    p.om0 = om0;
    p.nomc = (om0 + nomc <= nom) ? nomc : (nom - om0);
    const int rc = enqueue_tet_weights(p, L, w, s);
    if (rc != PG_OK) return rc;
    dim3 g((P + 127) / 128, nkp, p.nomc);
    k_gather<<<g, 128, 0, s>>>(scratch, (const int*)(w + L.kptr), (const int*)(w + L.kslot), P, nkp, p.nomc, om0,
                               1.0 / ntet, kcw);
    pg_count_launches(1);
  }
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? PG_OK : PG_ECUDA;
}

extern "C" int pg_bz_calcqdepw_par2(const double* enk, int nbnd, int nkp, double ef, const int* kqid, int ncg,
                                    int nomx, int numin, const double* omega, int nom, const int* tetc, int ntet,
                                    double* kcw, void* work, size_t work_bytes, int nom_chunk, unsigned* d_status,
                                    unsigned long long* d_counters, void* stream) {
  return par2_impl(enk, nbnd, nkp, ef, kqid, ncg, nomx, numin, omega, nom, tetc, ntet, kcw, work, work_bytes,
                   nom_chunk, REC_BUDGET, d_status, d_counters, stream);
}

// ---------------------------------------------------------------------------
// SVD-basis weights (bz_calcqdepw_par3, for_tetrahedra.f90:466-542).
extern "C" size_t pg_bz_calcqdepw_par3_workspace(int nbnd, int nkp, int ncg, int nomx, int numin, int nom, int ntet,
                                                  int nl) {
  const long long nb1 = ncg + nomx + 1, nb2 = nbnd - ncg - numin;
  if (nb1 <= 0 || nb2 <= 0 || nkp <= 0 || ntet <= 0 || nom <= 0 || nl <= 0) return 0;
  return weights_layout(nkp, ntet, nb1 * nb2, nom, nl, REC_BUDGET).total;
}

// kcw (nb1, nb2, nkp, nl) = the par2 corner weights of every (tetrahedron,
// pair) projected on dUl (device, (nom, nl) Fortran order) and accumulated
// like par2.  All frequencies are evaluated in one pass.
extern "C" int pg_bz_calcqdepw_par3(const double* enk, int nbnd, int nkp, double ef, const int* kqid, int ncg,
                                    int nomx, int numin, const double* dUl, int nl, const double* omega, int nom,
                                    const int* tetc, int ntet, double* kcw, void* work, size_t work_bytes,
                                    unsigned* d_status, unsigned long long* d_counters, void* stream) {
  const int nb1 = ncg + nomx + 1, nb2 = nbnd - ncg - numin;
  if (!enk || !kqid || !omega || !tetc || !kcw || !work || !dUl) return PG_EARG;
  if (nb1 <= 0 || nb2 <= 0 || nkp <= 0 || ntet <= 0 || nom <= 0 || nl <= 0 || ncg < 0 || numin < 0) return PG_EARG;
  if (ntet != 6 * nkp) return PG_EARG;
  if ((size_t)nom * nl * sizeof(double) > 48 * 1024) return PG_ETOOBIG;   // dUl staged in shared memory
  const long long items = (long long)nb1 * nb2 * ntet;
  if (items >= (1ll << 31)) return PG_ETOOBIG;
  const int P = nb1 * nb2;
  const WLayout L = weights_layout(nkp, ntet, P, nom, nl, REC_BUDGET);
  if (work_bytes < L.total) return PG_EWORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  char* w = (char*)work;
  double* scratch = (double*)(w + L.scratch);
  double* scratch2 = (double*)(w + L.scratch2);
  enqueue_kcsr(L, w, tetc, ntet, nkp, s);
  Params p = make_params(enk, nbnd, nkp, ef, kqid, ncg, numin, nb1, nb2, omega, tetc, ntet, scratch, d_status,
                         d_counters);
  p.om0 = 0;
  p.nomc = nom;
  const int rc = enqueue_tet_weights(p, L, w, s);
  if (rc != PG_OK) return rc;
  const long long nthr = (long long)4 * ntet * P;
  k_svd_project<<<(unsigned)((nthr + 127) / 128), 128, (size_t)nom * nl * sizeof(double), s>>>(
      scratch, dUl, nom, nl, P, (long long)4 * ntet, scratch2);
  dim3 g((P + 127) / 128, nkp, nl);
  k_gather<<<g, 128, 0, s>>>(scratch2, (const int*)(w + L.kptr), (const int*)(w + L.kslot), P, nkp, nl, 0,
                             1.0 / ntet, kcw);
  pg_count_launches(2);
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? PG_OK : PG_ECUDA;
}

// ---------------------------------------------------------------------------
// Weights without any device allocation by the caller.
//
// Some callers cannot allocate device memory: host code that reaches this
// library through a thin foreign-function layer (a Fortran program over
// ISO_C_BINDING, an f2py wrapper) has no device allocator of its own, and
// services that run under a fixed device-memory budget may not allocate per
// call.  pg_bz_calcqdepw_par2_noalloc takes only the inputs and the output
// kcw; its scratch (the k → tetrahedron lists and the per-tetrahedron weights
// of one frequency chunk) lives in a file-scope device array of
// PG_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds until
// the process exits.  Frequencies are processed in chunks that fit; a problem
// whose k lists plus ONE frequency of scratch exceed the array is rejected
// with PG_ETOOBIG.  The array keeps the previous call's contents; nothing in
// it has to start at zero, because every call rewrites each entry it reads.
// All calls share the one array, so calls whose work overlaps on the GPU
// (different streams, or other threads) race: serialise them.
// The first call in a device context looks up the array's device address
// (with that device current) and caches it under the context's unique id, so
// a new context (after cudaDeviceReset, or another context made current)
// gets a fresh lookup instead of a stale address; make that first call
// before any stream capture.
namespace pgw {
static __device__ __align__(256) unsigned char g_noalloc_scratch[PG_NOALLOC_SCRATCH_BYTES];
}

#include <mutex>
#include <cuda.h>
static std::mutex g_noalloc_mutex;
static void* g_noalloc_ptr[64] = {nullptr};
static unsigned long long g_noalloc_ctx[64] = {0};

// Unique id of the current context (0 if the driver cannot say; the address
// is then looked up on every call).
static unsigned long long current_context_id() {
  typedef CUresult (*get_cur_t)(CUcontext*);
  typedef CUresult (*get_id_t)(CUcontext, unsigned long long*);
  static get_cur_t get_cur = nullptr;
  static get_id_t get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess)
      get_cur = (get_cur_t)a;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
        qb == cudaDriverEntryPointSuccess)
      get_id = (get_id_t)b;
    looked_up = true;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_cur || !get_id || get_cur(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

extern "C" size_t pg_bz_calcqdepw_par2_noalloc_capacity(void) { return (size_t)PG_NOALLOC_SCRATCH_BYTES; }

extern "C" int pg_bz_calcqdepw_par2_noalloc(const double* enk, int nbnd, int nkp, double ef, const int* kqid,
                                            int ncg, int nomx, int numin, const double* omega, int nom,
                                            const int* tetc, int ntet, double* kcw, unsigned* d_status,
                                            unsigned long long* d_counters, void* stream) {
  const int nb1 = ncg + nomx + 1, nb2 = nbnd - ncg - numin;
  if (!enk || !kqid || !omega || !tetc || !kcw) return PG_EARG;
  if (nb1 <= 0 || nb2 <= 0 || nkp <= 0 || ntet <= 0 || nom <= 0 || ncg < 0 || numin < 0) return PG_EARG;
  if (ntet != 6 * nkp) return PG_EARG;
  // A quarter of the array for the sub-tetrahedron records of one
  // tetrahedron chunk, and the largest frequency chunk whose scratch fits in
  // the rest next to the k lists and the item arrays.
  const long long P = (long long)nb1 * nb2;
  const size_t cap = (size_t)PG_NOALLOC_SCRATCH_BYTES, rec_budget = cap / 4;
  if ((long long)P * ntet >= (1ll << 31)) return PG_ETOOBIG;
  const size_t fixed = weights_layout(nkp, ntet, P, 0, 0, rec_budget).total;
  const size_t per_omega = sizeof(double) * (size_t)4 * ntet * (size_t)P;
  if (fixed + per_omega + 256 > cap) return PG_ETOOBIG;
  const size_t fit = (cap - fixed - 256) / per_omega;
  const int nomc = (int)((fit < (size_t)nom) ? fit : (size_t)nom);
  // Lookup of the array's device address once per device context: in host
  // code the symbol names a host-side stand-in, not device memory.
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return PG_ECUDA;
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    const unsigned long long ctx = current_context_id();
    if (!g_noalloc_ptr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, pgw::g_noalloc_scratch) != cudaSuccess || !p) return PG_ECUDA;
      g_noalloc_ptr[dev] = p;
      g_noalloc_ctx[dev] = ctx;
    }
    base = g_noalloc_ptr[dev];
  }
  return par2_impl(enk, nbnd, nkp, ef, kqid, ncg, nomx, numin, omega, nom, tetc, ntet, kcw, base, cap, nomc,
                   rec_budget, d_status, d_counters, stream);
}
