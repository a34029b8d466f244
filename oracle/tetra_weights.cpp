// ORACLE — test infrastructure only, never part of the product path.
//
// Parity pinned against the reference's own statements: the reference ships no
// tests or golden vectors for this path and no Fortran compiler exists here, so
// tests/golden/make_weights_golden.py executes bz_calcqdepw_par2 and its callees
// from their Fortran text (tests/golden/f90py.py, kinds and storage association
// kept) on seeded inputs; this restatement reproduces those kcw bit for bit
// with either atan/log (tests/test_oracle_weights_golden.py), except where the
// reference's wtemp(4,2,nom) layout aliases the halves of 7- and 8-node
// polyhedra from the third frequency on (see convw1t below).  Per tetrahedron,
// tests/golden/make_tetra_golden.py runs convw1t_par on seeded corner sets
// that reach every statement of these routines outside error exits, debug
// output, one dead branch and one undefined case; this restatement matches
// each well-defined set bit for bit and flags each undefined or stopping one
// (tests/test_oracle_tetra_golden.py).  Known answers
// (tests/test_oracle_weights.py) check the integrals themselves.
//
// CPU restatement of PyGW's imaginary-axis tetrahedron polarization weights
// (the routine PyGW calls as ft.bz_calcqdepw_par2, pygw.py:3443), written to
// follow the reference's control flow, thresholds and left-to-right arithmetic:
//
//   bz_calcqdepw_par2   for_tetrahedra.f90:390-464   (driver, OpenMP over jb)
//   bz_calcqdepw_par3   for_tetrahedra.f90:466-542   (the same, weights projected on an SVD frequency basis)
//   convw1t_par         for_tetrahedra3.f90:3-136    (polyhedron → sub-tets)
//   genericfunf_par     for_tetrahedra3.f90:139-179  (pentahedron = 2 tets)
//   genericprism_par    for_tetrahedra3.f90:181-218  (prism = 3 tets)
//   generictetra_par    for_tetrahedra3.f90:220-405  (one tetrahedron)
//   stweight_itaylor_par for_tetrahedra3.f90:407-437 (large-ω series)
//   stweight_imag_par   for_tetrahedra3.f90:439-743  (closed forms, cases 4/6/8/10/16)
//   sorteq              for_tetrahedra2.f90:1688-1798
//   surfnodes           for_tetrahedra2.f90:1803-2114
//   unrepnodes          for_tetrahedra2.f90:2116-2175
//   relnodes / tlinap   for_tetrahedra2.f90:2177-2304
//   sortnodes           for_tetrahedra2.f90:2306-2773
//
// Conventions where the reference is undefined (uninitialised locals, writes
// through a zero index, bit tests at a garbage position): every such event
// sets PG_ERR_UNDEFINED in the status word and proceeds deterministically
// (unset values read as 0, the access is skipped).  Conditions where the
// reference calls `stop` set their own error bit and the (tet, band pair)
// contributes zero.
//
// Arithmetic: compile with -ffp-contract=off.  atan/log come from the
// project's portable implementation (bit-identical on host and GPU) unless
// built with -DORACLE_LIBM, which uses the C library instead.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <vector>
#include <atomic>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../pygw_gb300/csrc/fp64_math.h"

#ifdef ORACLE_LIBM
static inline double o_atan(double x) { return std::atan(x); }
static inline double o_log(double x) { return std::log(x); }
#else
static inline double o_atan(double x) { return pg_atan(x); }
static inline double o_log(double x) { return pg_log(x); }
#endif

// Status bits (same values as the product's C-ABI, include/pygw_gb300.h).
enum {
  ERR_NNOD = 1 << 0,       // convw1t_par: nnod > 8 (reference: stop)
  ERR_SORTEQ = 1 << 1,     // sorteq: unknown grouping (reference: stop)
  ERR_SORTNODES = 1 << 2,  // sortnodes: unknown face structure (reference: stop)
  ERR_RELNODES = 1 << 3,   // relnodes: ntype out of range (reference: stop)
  ERR_EQUIV = 1 << 4,      // stweight_imag_par: bad equiv_flag (reference: stop)
  ERR_UNDEFINED = 1 << 5,  // reference behaviour undefined (see header)
  ERR_NONFINITE = 1 << 6,  // non-finite weight produced
};

// Default-real (single precision) literals of the reference, widened.
static const double ZTOL_VOL = (double)1.e-10f;     // for_tetrahedra3.f90:277
static const double ZTOL_SORTEQ = (double)1.e-2f;   // for_tetrahedra2.f90:1699
static const double RDIST_TINY = (double)1.0e-10f;  // for_tetrahedra2.f90:1791
static const double OMEG_TINY = (double)1.0e-20f;   // for_tetrahedra3.f90:731
static const double CHECK_OMEG = (double)1.e-6f;    // for_tetrahedra3.f90:700
static const double TOL_UNPHYS = 1.0e4;             // for_tetrahedra3.f90:460
static const double TOL_TAYLOR = 10.0;              // for_tetrahedra3.f90:276
// Largest frequency count the oracle accepts (stack arrays, like the
// reference's automatic arrays).
static const int NOM_MAX = 256;

struct Stats {
  long long calls = 0, nnod_hist[9] = {0}, equiv_hist[5] = {0};
  long long taylor = 0, exact = 0, zero_vol = 0, big_weight_warn = 0, big_weight_zeroed = 0;
  unsigned status = 0;
  void merge(const Stats& o) {
    calls += o.calls;
    for (int i = 0; i < 9; i++) nnod_hist[i] += o.nnod_hist[i];
    for (int i = 0; i < 5; i++) equiv_hist[i] += o.equiv_hist[i];
    taylor += o.taylor; exact += o.exact; zero_vol += o.zero_vol;
    big_weight_warn += o.big_weight_warn; big_weight_zeroed += o.big_weight_zeroed;
    status |= o.status;
  }
};

// ---------------------------------------------------------------- sorteq
// for_tetrahedra2.f90:1688-1798.  v[0..3] in/out, index[] 1-based positions.
static double f_rdist(double v1, double v2) {
  if ((std::fabs(v1) + std::fabs(v2)) < RDIST_TINY) return 0.0;
  return 2.0 * std::fabs(v1 - v2) / (std::fabs(v1) + std::fabs(v2));
}

static int sorteq(double v[4], int index[4], Stats& st) {
  int sig[5] = {0, 0, 0, 0, 0};
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++)
      if (f_rdist(v[i], v[j]) < ZTOL_SORTEQ) sig[i] += 1;
  sig[4] = sig[0] + sig[1] + sig[2] + sig[3];
  int mx = sig[0], mn = sig[0];
  for (int i = 1; i < 4; i++) { if (sig[i] > mx) mx = sig[i]; if (sig[i] < mn) mn = sig[i]; }
  if (sig[4] == 8 && mx == 3) {
    for (int i = 0; i < 4; i++) if (sig[i] == 2) sig[i] += 1;
    sig[4] = sig[0] + sig[1] + sig[2] + sig[3];
  }
  mn = sig[0];
  for (int i = 1; i < 4; i++) if (sig[i] < mn) mn = sig[i];
  if (sig[4] == 10 && mn == 2) {
    for (int i = 0; i < 4; i++) sig[i] = 4;
    sig[4] = 16;
  }
  if (sig[4] == 12) sig[4] = 16;
  if (sig[4] == 14) sig[4] = 16;
  for (int i = 0; i < 4; i++) index[i] = i + 1;
  double vt; int it;
  switch (sig[4]) {
    case 16: break;
    case 10:
      for (int i = 0; i < 3; i++) {
        if (sig[i] == 1) {
          vt = v[i]; v[i] = v[3]; v[3] = vt;
          it = index[i]; index[i] = index[3]; index[3] = it;
          it = sig[3]; sig[3] = sig[i]; sig[i] = it;
        }
      }
      break;
    case 8:
      for (int i = 2; i < 4; i++) {
        if (f_rdist(v[i], v[0]) < f_rdist(v[1], v[0])) {
          vt = v[i]; v[i] = v[1]; v[1] = vt;
          it = index[i]; index[i] = index[1]; index[1] = it;
          it = sig[i]; sig[i] = sig[1]; sig[1] = it;
        }
      }
      break;
    case 6: {
      int j = 0;
      for (int i = 0; i < 4; i++) {
        if (sig[i] == 2) {
          vt = v[j]; v[j] = v[i]; v[i] = vt;
          it = index[j]; index[j] = index[i]; index[i] = it;
          it = sig[j]; sig[j] = sig[i]; sig[i] = it;
          j++;
        }
      }
    } break;
    case 4: break;
    default:
      st.status |= ERR_SORTEQ;
      break;
  }
  return sig[4];
}

// ------------------------------------------------ stweight_itaylor_par
// for_tetrahedra3.f90:407-437
static void stweight_itaylor(const double dv[4], double omeg, double wv[4]) {
  double omt2 = omeg * omeg;
  double omt4 = omt2 * omt2;
  double denom1 = 6.0e+1 * omt2;
  double denom3 = 4.2e+2 * omt4;
  for (int ivert = 1; ivert <= 4; ivert++) {
    double ev[5];
    for (int j = 1; j <= 4; j++) {
      int k = (j + ivert - 2) % 4 + 1;
      ev[j] = dv[k - 1];
    }
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

// ------------------------------------------------- stweight_imag_par
// for_tetrahedra3.f90:439-743.  wt[(ivert)*nom + iom].
struct Vd { double v[5][5]; };
static inline void set_vdif(Vd& d, const double ev[5]) {
  for (int i = 1; i <= 4; i++) for (int j = 1; j <= 4; j++) d.v[i][j] = ev[i] - ev[j];
}
static inline void set_tans_logs(double tans[5], double logs[5], const double ev[5], double omeg) {
  for (int ii = 1; ii <= 4; ii++) {
    if (omeg > OMEG_TINY) tans[ii] = o_atan(ev[ii] / omeg);
    else tans[ii] = std::copysign(1.0, ev[ii]) * 2.0 * o_atan(1.0);
    if ((omeg * omeg + ev[ii] * ev[ii]) > 1.0e-10) logs[ii] = o_log(ev[ii] * ev[ii] + omeg * omeg);
    else logs[ii] = 0.0;
  }
}
static inline void check_weight(double& w, double omeg, Stats& st) {
  if (std::fabs(w) > TOL_UNPHYS) {
    if (std::fabs(omeg) < CHECK_OMEG) { w = 0.0; st.big_weight_zeroed++; }
    else st.big_weight_warn++;
  }
}
static inline double sq(double x) { return x * x; }
static inline double cube(double x) { return (x * x) * x; }
static inline double pow4(double x) { double t = x * x; return t * t; }

static void stweight_imag(double* wt, const double dv[4], const double* omega, int equiv_flag,
                          const bool* Qtaylor, int nom, Stats& st) {
  for (int i = 0; i < 4 * nom; i++) wt[i] = 0.0;
  double ev[5], tans[5], logs[5], evt[10], evw[10];
  Vd vd; auto& vdif = vd.v;
  switch (equiv_flag) {
    case 4:
      for (int ivert = 1; ivert <= 4; ivert++) {
        for (int j = 1; j <= 4; j++) { int k = (j + ivert - 2) % 4 + 1; ev[k] = dv[j - 1]; }
        set_vdif(vd, ev);
        double ev3t4 = ev[3] * ev[4];
        double ev1_2 = ev[1] * ev[1];
        double ev_2[5];
        ev_2[1] = 3.0 * ev1_2;
        ev_2[2] = 3.0 * sq(ev[2]);
        ev_2[3] = 3.0 * sq(ev[3]);
        ev_2[4] = 3.0 * sq(ev[4]);
        double vdf24 = vdif[2][3] * vdif[2][4] * vdif[3][4];
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
        double cc = 6.0 * sq(vdif[1][2] * vdif[1][3] * vdif[1][4]) * vdif[2][3] * vdif[2][4] * vdif[3][4];
        for (int iom = 0; iom < nom; iom++) {
          if (Qtaylor[iom]) continue;
          double omeg = omega[iom];
          set_tans_logs(tans, logs, ev, omeg);
          double omeg2 = omeg * omeg;
          double aa = evt[1] + omeg2 * evw[1] + omeg * (tans[1] * evt[2] + tans[2] * evt[3] + tans[3] * evt[4] + tans[4] * evt[5] +
                                                        omeg2 * (tans[1] * evw[2] + tans[2] * evw[3] + tans[3] * evw[4] + tans[4] * evw[5]));
          double bb = logs[1] * evt[6] + logs[2] * evt[7] + logs[3] * evt[8] + logs[4] * evt[9] +
                      omeg2 * (logs[1] * evw[6] + logs[2] * evw[7] + logs[3] * evw[8] + logs[4] * evw[9]);
          double& w = wt[(ivert - 1) * nom + iom];
          w = (aa + bb) / cc;
          check_weight(w, omeg, st);
        }
      }
      break;
    case 6:
      for (int ivert = 1; ivert <= 2; ivert++) {
        ev[1] = dv[ivert - 1];
        ev[2] = ev[1];
        ev[3] = dv[2]; ev[4] = dv[3];
        set_vdif(vd, ev);
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
        double cc = 6.0 * cube(vdif[1][3]) * cube(vdif[1][4]) * vdif[3][4];
        for (int iom = 0; iom < nom; iom++) {
          if (Qtaylor[iom]) continue;
          double omeg = omega[iom];
          set_tans_logs(tans, logs, ev, omeg);
          double omeg2 = omeg * omeg;
          double aa = evt[1] + omeg2 * evw[1] + omeg * (tans[1] * evt[2] + tans[3] * evt[3] + tans[4] * evt[4] +
                                                        omeg2 * (tans[1] * evw[2] + tans[3] * evw[3] + tans[4] * evw[4]));
          double bb = logs[1] * evt[5] + logs[3] * evt[6] + logs[4] * evt[7] + omeg2 * (logs[1] * evw[5] + logs[3] * evw[6] + logs[4] * evw[7]);
          double& w = wt[(ivert - 1) * nom + iom];
          w = (aa + bb) / cc;
          check_weight(w, omeg, st);
        }
      }
      for (int ivert = 3; ivert <= 4; ivert++) {
        ev[1] = (dv[0] + dv[1]) * 0.5;
        ev[2] = ev[1];
        for (int j = 3; j <= 4; j++) { int k = (j + ivert) % 2 + 3; ev[k] = dv[j - 1]; }
        set_vdif(vd, ev);
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
        double cc = 6.0 * cube(vdif[1][3]) * sq(vdif[1][4]) * sq(vdif[3][4]);
        for (int iom = 0; iom < nom; iom++) {
          if (Qtaylor[iom]) continue;
          double omeg = omega[iom];
          double omeg2 = omeg * omeg;
          set_tans_logs(tans, logs, ev, omeg);
          double aa = evt[1] + omeg2 * evw[1] + omeg * (tans[1] * evt[2] + tans[3] * evt[3] + tans[4] * evt[4] +
                                                        omeg2 * (tans[1] * evw[2] + tans[3] * evw[3] + tans[4] * evw[4]));
          double bb = logs[1] * evt[5] + logs[3] * evt[6] + logs[4] * evt[7] + omeg2 * (logs[1] * evw[5] + logs[3] * evw[6] + logs[4] * evw[7]);
          double& w = wt[(ivert - 1) * nom + iom];
          w = (aa + bb) / cc;
          check_weight(w, omeg, st);
        }
      }
      break;
    case 8: {
      ev[1] = (dv[0] + dv[1]) / 2.0;
      ev[2] = ev[1];
      ev[3] = (dv[2] + dv[3]) / 2.0;
      ev[4] = ev[3];
      set_vdif(vd, ev);
      evw[1] = 6.0 * vdif[3][1];
      evt[1] = (sq(ev[1]) - 5.0 * ev[1] * ev[3] - 2.0 * sq(ev[3])) * vdif[3][1];
      evt[2] = -6.0 * (sq(ev[3]) + 2.0 * ev[1] * ev[3]);
      evw[3] = 3.0 * (ev[1] + 2.0 * ev[3]);
      evt[3] = -3.0 * ev[1] * sq(ev[3]);
      evw[4] = 6.0 * vdif[1][3];
      evt[4] = -(2.0 * sq(ev[1]) + 5.0 * ev[1] * ev[3] - sq(ev[3])) * vdif[1][3];
      evt[5] = 6.0 * (sq(ev[1]) + 2.0 * ev[1] * ev[3]);
      evw[6] = -3.0 * (2.0 * ev[1] + ev[3]);
      evt[6] = 3.0 * sq(ev[1]) * ev[3];
      double cc = 6.0 * pow4(vdif[1][3]);
      for (int iom = 0; iom < nom; iom++) {
        if (Qtaylor[iom]) continue;
        double omeg = omega[iom];
        double omeg2 = omeg * omeg;
        set_tans_logs(tans, logs, ev, omeg);
        double aa = evt[1] + evw[1] * omeg2 + omeg * (tans[1] - tans[3]) * (6.0 * omeg2 + evt[2]);
        double bb = (logs[1] - logs[3]) * (evt[3] + evw[3] * omeg2);
        double& w1 = wt[0 * nom + iom];
        w1 = (aa + bb) / cc;
        check_weight(w1, omeg, st);
        wt[1 * nom + iom] = w1;
        aa = evt[4] + evw[4] * omeg2 + omeg * (tans[1] - tans[3]) * (-6.0 * omeg2 + evt[5]);
        bb = (logs[1] - logs[3]) * (evt[6] + evw[6] * omeg2);
        double& w3 = wt[2 * nom + iom];
        w3 = (aa + bb) / cc;
        check_weight(w3, omeg, st);
        wt[3 * nom + iom] = w3;
      }
    } break;
    case 10: {
      ev[1] = ev[2] = ev[3] = ((dv[0] + dv[1]) + dv[2]) / 3.0;
      ev[4] = dv[3];
      set_vdif(vd, ev);
      evw[1] = 6.0 * vdif[1][4];
      evt[1] = -vdif[1][4] * (2.0 * sq(ev[1]) - 7.0 * ev[1] * ev[4] + 11.0 * sq(ev[4]));
      evt[2] = 18.0 * sq(ev[4]);
      evw[3] = -9.0 * ev[4];
      evt[3] = 3.0 * cube(ev[4]);
      evw[4] = 6.0 * vdif[4][1];
      evt[4] = vdif[4][1] * (sq(ev[1]) - 5.0 * ev[1] * ev[4] - 2.0 * sq(ev[4]));
      evt[5] = -6.0 * ev[4] * (ev[4] + 2.0 * ev[1]);
      evt[6] = -3.0 * ev[1] * sq(ev[4]);
      evw[6] = 3.0 * (ev[1] + 2.0 * ev[4]);
      double cc1 = 18.0 * pow4(vdif[1][4]);
      double cc2 = 6.0 * pow4(vdif[1][4]);
      for (int iom = 0; iom < nom; iom++) {
        if (Qtaylor[iom]) continue;
        double omeg = omega[iom];
        double omeg2 = omeg * omeg;
        set_tans_logs(tans, logs, ev, omeg);
        double aa = evt[1] + omeg2 * evw[1] + omeg * (tans[1] - tans[4]) * (-6.0 * omeg2 + evt[2]);
        double bb = (logs[1] - logs[4]) * (evt[3] + evw[3] * omeg2);
        double& w1 = wt[0 * nom + iom];
        w1 = (aa + bb) / cc1;
        check_weight(w1, omeg, st);
        wt[1 * nom + iom] = w1;
        wt[2 * nom + iom] = w1;
        aa = evt[4] + evw[4] * omeg2 + omeg * (tans[1] - tans[4]) * (6.0 * omeg2 + evt[5]);
        bb = (logs[1] - logs[4]) * (evt[6] + evw[6] * omeg2);
        double& w4 = wt[3 * nom + iom];
        w4 = (aa + bb) / cc2;
        check_weight(w4, omeg, st);
      }
    } break;
    case 16: {
      double e1 = (((dv[0] + dv[1]) + dv[2]) + dv[3]) / 4.0;
      for (int iom = 0; iom < nom; iom++) {
        if (Qtaylor[iom]) continue;
        double omeg = omega[iom];
        double& w1 = wt[0 * nom + iom];
        w1 = -e1 / (12.0 * (sq(omeg) + sq(e1)));
        check_weight(w1, omeg, st);
        wt[1 * nom + iom] = w1; wt[2 * nom + iom] = w1; wt[3 * nom + iom] = w1;
      }
    } break;
    default:
      st.status |= ERR_EQUIV;
      break;
  }
}

// -------------------------------------------------- generictetra_par
// for_tetrahedra3.f90:220-405.  corners[node][coord] (node 0..3), wt_out[i*nom+iom].
static int generictetra(double* wt_out, const double corners[4][3], const double e[4], const double f[4],
                        const double* omega, int nom, Stats& st) {
  double wt_small[4 * NOM_MAX], wt_tmp[4 * NOM_MAX];
  bool Qt[NOM_MAX];
  for (int i = 0; i < 4 * nom; i++) { wt_out[i] = 0.0; wt_small[i] = 0.0; wt_tmp[i] = 0.0; }
  double dbig[4];
  for (int i = 0; i < 4; i++) dbig[i] = f[i] - e[i];
  double vec[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) vec[i][j] = corners[i + 1][j] - corners[0][j];
  auto det = [&](int i, int j) { return vec[1][i] * vec[2][j] - vec[1][j] * vec[2][i]; };
  double vol = 0.0;
  for (int i = 1; i <= 3; i++) {
    int j = i % 3 + 1, k = j % 3 + 1;
    vol = vol + vec[0][i - 1] * det(j - 1, k - 1);
  }
  vol = std::fabs(vol);
  if (vol < ZTOL_VOL) { st.zero_vol++; return 1; }
  double ds[4], max_de = 0.0;
  for (int i = 0; i < 4; i++) {
    ds[i] = (dbig[1] - dbig[0]) * corners[i][0] + (dbig[2] - dbig[0]) * corners[i][1] + (dbig[3] - dbig[0]) * corners[i][2] + dbig[0];
    if (std::fabs(ds[i]) > max_de) max_de = std::fabs(ds[i]);
  }
  double taylor_omega = TOL_TAYLOR * max_de;
  for (int iom = 0; iom < nom; iom++) Qt[iom] = omega[iom] > taylor_omega;
  for (int iom = 0; iom < nom; iom++) {
    if (Qt[iom]) {
      double w4[4];
      stweight_itaylor(ds, omega[iom], w4);
      for (int i = 0; i < 4; i++) wt_small[i * nom + iom] = w4[i];
      st.taylor++;
    } else {
      st.exact++;
    }
  }
  int ind[4];
  int flag = sorteq(ds, ind, st);
  switch (flag) {
    case 4: st.equiv_hist[0]++; break;
    case 6: st.equiv_hist[1]++; break;
    case 8: st.equiv_hist[2]++; break;
    case 10: st.equiv_hist[3]++; break;
    case 16: st.equiv_hist[4]++; break;
  }
  stweight_imag(wt_tmp, ds, omega, flag, Qt, nom, st);
  for (int iom = 0; iom < nom; iom++)
    if (!Qt[iom])
      for (int i = 0; i < 4; i++) wt_small[(ind[i] - 1) * nom + iom] = wt_tmp[i * nom + iom];
  for (int iom = 0; iom < nom; iom++) {
    double s = wt_small[0 * nom + iom];
    s = s + wt_small[1 * nom + iom];
    s = s + wt_small[2 * nom + iom];
    s = s + wt_small[3 * nom + iom];
    double w[4] = {s, 0.0, 0.0, 0.0};
    for (int i = 1; i <= 3; i++) {
      for (int j = 0; j < 4; j++) w[i] = w[i] + wt_small[j * nom + iom] * corners[j][i - 1];
      w[0] = w[0] - w[i];
    }
    for (int i = 0; i < 4; i++) wt_out[i * nom + iom] = w[i] * vol;
  }
  return 0;
}

// genericfunf_par (for_tetrahedra3.f90:139-179): tets (1,2,3,4), (2,3,4,5)
static void genericfunf(double* w, const double corners[6][3], const double e[4], const double f[4],
                        const double* omega, int nom, Stats& st) {
  double twt[4 * NOM_MAX];
  for (int i = 0; i < 4 * nom; i++) w[i] = 0.0;
  for (int itet = 0; itet <= 1; itet++) {
    double tc[4][3];
    for (int inod = 0; inod < 4; inod++) for (int c = 0; c < 3; c++) tc[inod][c] = corners[inod + itet][c];
    generictetra(twt, tc, e, f, omega, nom, st);
    for (int i = 0; i < 4 * nom; i++) w[i] = w[i] + twt[i];
  }
}

// genericprism_par (for_tetrahedra3.f90:181-218): tets (1..4), (2..5), (3..6)
static void genericprism(double* w, const double corners[6][3], const double e[4], const double f[4],
                         const double* omega, int nom, Stats& st) {
  double twt[4 * NOM_MAX];
  for (int i = 0; i < 4 * nom; i++) w[i] = 0.0;
  for (int itet = 0; itet <= 2; itet++) {
    double tc[4][3];
    for (int inod = 0; inod < 4; inod++) for (int c = 0; c < 3; c++) tc[inod][c] = corners[inod + itet][c];
    generictetra(twt, tc, e, f, omega, nom, st);
    for (int i = 0; i < 4 * nom; i++) w[i] = w[i] + twt[i];
  }
}

// ------------------------------------------------------- node geometry
struct Nodes {
  double x[21][4];   // 1-based node, 1-based coordinate
  int ntype[21];
  int nnod;
};

// surfnodes, for_tetrahedra2.f90:1803-2114
static void surfnodes(Nodes& N, const double e[4], const double f[4], double ef) {
  const double zerotol = 1.0e-12;
  static const int types[20] = {7, 11, 13, 14, 19, 21, 22, 25, 26, 28, 35, 37, 38, 41, 42, 44, 49, 50, 52, 56};
  auto E = [&](int i) { return e[i - 1]; };
  auto F = [&](int i) { return f[i - 1]; };
  auto edif = [&](int i, int j) { return E(i) - E(j); };
  auto fdif = [&](int i, int j) { return F(i) - F(j); };
  auto efdif = [&](int i, int j, int k) { return edif(i, j) * fdif(k, j) - edif(k, j) * fdif(i, j); };
  auto efef = [&](int i, int j) { return (ef - E(i)) * (F(j) - F(i)) - (ef - F(i)) * (E(j) - E(i)); };
  for (int n = 1; n <= 20; n++) { N.x[n][1] = N.x[n][2] = N.x[n][3] = 0.0; N.ntype[n] = types[n - 1]; }
  for (int i = 2; i <= 4; i++) N.x[i][5 - i] = 1.0;
  int inod = 4, iint = 4;
  double nt[4];
  auto add = [&]() { inod++; for (int c = 1; c <= 3; c++) N.x[inod][c] = nt[c]; N.ntype[inod] = N.ntype[iint]; };
  for (int j = 2; j <= 4; j++) {
    int i = 6 - j; iint++;
    double denom = edif(i, 1);
    nt[1] = nt[2] = nt[3] = 0.0;
    if (std::fabs(denom) > zerotol) {
      nt[i - 1] = (ef - E(1)) / denom;
      if ((nt[i - 1] > 0.0) && (nt[i - 1] <= 1.0)) add();
    }
  }
  for (int k = 1; k <= 3; k++) {
    int i = k % 3 + 1, j = i % 3 + 1; iint++;
    double denom = edif(i + 1, j + 1);
    nt[1] = nt[2] = nt[3] = 0.0;
    if (std::fabs(denom) > zerotol) {
      nt[i] = (ef - E(j + 1)) / denom;
      nt[j] = (E(i + 1) - ef) / denom;
      if ((nt[i] >= 0.0) && (nt[j] >= 0.0)) add();
    }
  }
  for (int j = 2; j <= 4; j++) {
    int i = 6 - j; iint++;
    double denom = fdif(i, 1);
    nt[1] = nt[2] = nt[3] = 0.0;
    if (std::fabs(denom) > zerotol) {
      nt[i - 1] = (ef - F(1)) / denom;
      if ((nt[i - 1] >= 0.0) && (nt[i - 1] <= 1.0)) add();
    }
  }
  for (int k = 1; k <= 3; k++) {
    int i = k % 3 + 1; iint++; int j = i % 3 + 1;
    double denom = fdif(i + 1, j + 1);
    nt[1] = nt[2] = nt[3] = 0.0;
    if (std::fabs(denom) > zerotol) {
      nt[i] = (ef - F(j + 1)) / denom;
      nt[j] = (F(i + 1) - ef) / denom;
      if ((nt[i] >= 0.0) && (nt[j] >= 0.0)) add();
    }
  }
  for (int k = 1; k <= 3; k++) {
    int i = k % 3 + 1; iint++; int j = i % 3 + 1;
    double denom1 = efdif(i + 1, 1, j + 1);
    double denom2 = efdif(j + 1, 1, i + 1);
    nt[1] = nt[2] = nt[3] = 0.0;
    if ((std::fabs(denom1) > zerotol) && (std::fabs(denom2) > zerotol)) {
      nt[i] = efef(1, j + 1) / denom1;
      nt[j] = efef(1, i + 1) / denom2;
      double sumnt = nt[i] + nt[j];
      if ((nt[i] > 0.0) && (nt[j] > 0.0) && (sumnt <= 1.0)) add();
    }
  }
  {
    double denom1 = efdif(2, 4, 3), denom2 = efdif(3, 4, 2), denom3 = efdif(4, 2, 3);
    iint++;
    if ((std::fabs(denom1) > zerotol) && (std::fabs(denom2) > zerotol) && (std::fabs(denom3) > zerotol)) {
      nt[1] = efef(4, 3) / denom1;
      nt[2] = efef(4, 2) / denom2;
      nt[3] = efef(2, 3) / denom3;
      if ((nt[1] > 0.0) && (nt[2] > 0.0) && (nt[3] > 0.0)) add();
    }
  }
  N.nnod = inod;
}

// unrepnodes, for_tetrahedra2.f90:2116-2175
static void unrepnodes(Nodes& N) {
  const double zerotol = 1.0e-8;
  int i = 1;
  while (i < N.nnod) {
    double xi[4] = {0, N.x[i][1], N.x[i][2], N.x[i][3]};
    int j = i + 1;
    while (j <= N.nnod) {
      double sumnt = 0.0;
      for (int k = 1; k <= 3; k++) sumnt = sumnt + std::fabs(xi[k] - N.x[j][k]);
      if (sumnt < zerotol) {
        for (int ib = 0; ib <= 5; ib++) {
          int btj = (N.ntype[j] >> ib) & 1, bti = (N.ntype[i] >> ib) & 1;
          if (btj == 1 && bti == 0) N.ntype[i] |= (1 << ib);
        }
        for (int k = j + 1; k <= N.nnod; k++) {
          for (int c = 1; c <= 3; c++) N.x[k - 1][c] = N.x[k][c];
          N.ntype[k - 1] = N.ntype[k];
        }
        for (int c = 1; c <= 3; c++) N.x[N.nnod][c] = 0.0;
        N.ntype[N.nnod] = 0;
        N.nnod = N.nnod - 1;
      } else {
        j = j + 1;
      }
    }
    i = i + 1;
  }
}

static double tlinap(const double x[4], const double* fv) {
  double fx = fv[0];
  for (int i = 1; i <= 3; i++) {
    double df = fv[i] - fv[0];
    fx = fx + df * x[i];
  }
  return fx;
}

// relnodes, for_tetrahedra2.f90:2177-2281
static int relnodes(Nodes& N, const double e[4], const double f[4], double ef) {
  const double zerotol = 1.00e-12;
  int info = 0, inod = 1, maxnod = N.nnod;
  bool keep = false;
  while (inod <= maxnod) {
    double e1 = tlinap(N.x[inod], e) - ef;
    double e2 = tlinap(N.x[inod], f) - ef;
    int t = N.ntype[inod];
    if (t >= 7 && t <= 15) {
      bool occ = (e1 < 0.0) || (std::fabs(e1) <= zerotol);
      bool unocc = (e2 > 0.0) || (std::fabs(e2) <= zerotol);
      keep = occ && unocc;
    } else if (t >= 16 && t <= 31) {
      keep = (e2 > 0.0) || (std::fabs(e2) <= zerotol);
    } else if (t >= 32 && t <= 47) {
      keep = (e1 < 0.0) || (std::fabs(e1) <= zerotol);
    } else if (t >= 48 && t <= 63) {
      keep = true;
    } else {
      info = 1;
    }
    if (keep) {
      inod = inod + 1;
    } else {
      for (int jn = inod + 1; jn <= maxnod; jn++) {
        for (int c = 1; c <= 3; c++) N.x[jn - 1][c] = N.x[jn][c];
        N.ntype[jn - 1] = N.ntype[jn];
      }
      maxnod = maxnod - 1;
    }
  }
  for (int in = maxnod + 1; in <= N.nnod; in++) {
    N.x[in][1] = N.x[in][2] = N.x[in][3] = 0.0;
    N.ntype[in] = 0;
  }
  N.nnod = maxnod;
  return info;
}

// sortnodes, for_tetrahedra2.f90:2306-2773.  index[inod][isub], 1-based, 0 = unset.
struct SortCtx {
  Stats* st;
  bool bt(int nt, int pos) {  // btest with the reference's undefined positions guarded
    if (pos < 0 || pos > 7) { st->status |= ERR_UNDEFINED; return false; }
    return (nt >> pos) & 1;
  }
};

static int sortnodes(const Nodes& N, int index[9][3], Stats& st) {
  SortCtx C{&st};
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
  for (int a = 0; a < 9; a++) index[a][0] = index[a][1] = index[a][2] = 0;
  auto nty = [&](int inod) -> int {
    if (inod < 1 || inod > nnod) { st.status |= ERR_UNDEFINED; return 0; }
    return N.ntype[inod];
  };
  auto tri = [&](int k) -> int {
    if (k < 1 || k > 6) { st.status |= ERR_UNDEFINED; return UNSET; }
    return triangle[k];
  };
  auto count_planes = [&](bool with_penta) {
    for (int ibit = 0; ibit <= 5; ibit++) {
      for (int inod = 1; inod <= nnod; inod++) if (C.bt(N.ntype[inod], ibit)) spl[ibit]++;
      switch (spl[ibit]) {
        case 3: it++; triangle[it] = ibit; break;
        case 4: is++; square[is] = ibit; break;
        case 5: if (with_penta) { ip++; if (ip <= 2) penta[ip] = ibit; else st.status |= ERR_UNDEFINED; } break;
      }
    }
  };
  switch (nnod) {
    case 5: {
      for (int ibit = 0; ibit <= 5; ibit++) {
        for (int inod = 1; inod <= 5; inod++) if (C.bt(N.ntype[inod], ibit)) spl[ibit]++;
        switch (spl[ibit]) {
          case 3: it++; triangle[it] = ibit; break;
          case 4: is++; square[is] = ibit; signbit = ibit; break;
        }
      }
      for (int inod = 1; inod <= 5; inod++) index[inod][1] = 0;
      if (is != 0) {
        int is1 = 1;
        for (int inod = 1; inod <= 5; inod++) {
          if (C.bt(N.ntype[inod], tri(1))) {
            if (!C.bt(N.ntype[inod], signbit)) {
              index[inod][1] = 2;
            } else {
              index[inod][1] = is1;
              is1 = is1 + 2;
              signnod = inod;
            }
          }
        }
        for (int i = 2; i <= 4; i++) if (C.bt(nty(signnod), tri(i))) signbit = triangle[i];
        for (int inod = 1; inod <= 5; inod++) {
          if (index[inod][1] == 0) index[inod][1] = C.bt(N.ntype[inod], signbit) ? 5 : 4;
        }
      } else {
        // Six triangular faces.  The reference resets its position counters
        // inside the node loop, so positions 3..5 are never assigned.
        for (int inod = 1; inod <= 5; inod++) {
          int nb = 0;
          for (int ibit = 0; ibit <= 5; ibit++) if (C.bt(N.ntype[inod], ibit)) nb++;
          int it1 = 1, it2 = 1;
          if (nb == 3) { index[inod][1] = 1 + (it1 - 1) * 4; it1++; }
          else { index[inod][1] = 1 + it2; it2++; }
        }
      }
    } break;
    case 6: {
      for (int a = 1; a <= 6; a++) index[a][1] = 0;
      count_planes(false);
      if (is == 2) {
        int cnt = 1;
        for (int inod = 1; inod <= 6; inod++) {
          if (C.bt(N.ntype[inod], square[1]) && C.bt(N.ntype[inod], square[2])) {
            index[inod][1] = 2 + (cnt - 1) * 3;
            if (cnt == 1) signnod = inod;
            if (cnt == 2) signnodb = inod;
            cnt++;
          }
        }
        int sigtri[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int inod = 1; inod <= 6; inod++)
          for (int k = 1; k <= 4; k++) if (C.bt(N.ntype[inod], tri(k))) sigtri[inod]++;
        for (int k = 1; k <= 4; k++) {
          if (C.bt(nty(signnod), tri(k))) signbita = k;
          if (C.bt(nty(signnodb), tri(k))) signbitb = k;
        }
        for (int inod = 1; inod <= 6; inod++) {
          if (index[inod][1] == 0) {
            int ta = tri(signbita == UNSET ? 0 : signbita), tb = tri(signbitb == UNSET ? 0 : signbitb);
            if (sigtri[inod] == 3 && C.bt(N.ntype[inod], ta)) index[inod][1] = 4;
            if (sigtri[inod] == 2 && C.bt(N.ntype[inod], ta)) index[inod][1] = 1;
            if (sigtri[inod] == 3 && C.bt(N.ntype[inod], tb)) index[inod][1] = 3;
            if (sigtri[inod] == 2 && C.bt(N.ntype[inod], tb)) index[inod][1] = 6;
          }
        }
      } else if (is == 3) {
        for (int inod = 1; inod <= 6; inod++) {
          for (int k = 1; k <= 2; k++) {
            if (C.bt(N.ntype[inod], tri(k))) {
              if (C.bt(N.ntype[inod], square[1]) && C.bt(N.ntype[inod], square[2])) index[inod][1] = 1 + 3 * (k - 1);
              else if (C.bt(N.ntype[inod], square[1])) index[inod][1] = 2 + 3 * (k - 1);
              else if (C.bt(N.ntype[inod], square[2])) index[inod][1] = 3 + 3 * (k - 1);
              else { st.status |= ERR_SORTNODES; info = 61; }
            }
          }
        }
      }
    } break;
    case 7: {
      for (int a = 1; a <= 7; a++) index[a][1] = index[a][2] = 0;
      count_planes(true);
      if (it == 2) {
        if (is == 4) {
          for (int inod = 1; inod <= 7; inod++) {
            if (C.bt(N.ntype[inod], triangle[1]) && C.bt(N.ntype[inod], triangle[2])) {
              index[inod][1] = index[inod][2] = 2;
              signnod = inod;
            }
          }
          int is1 = 0;
          for (int ibit = 0; ibit <= 5; ibit++) {
            if (C.bt(nty(signnod), ibit) && (spl[ibit] == 4) && (is1 == 0)) { signbita = ibit; is1++; }
            else if (C.bt(nty(signnod), ibit) && (spl[ibit] == 4)) signbitb = ibit;
          }
          for (int inod = 1; inod <= 7; inod++) {
            if (inod != signnod) {
              int t = N.ntype[inod];
              if (C.bt(t, triangle[1]) && C.bt(t, signbita)) index[inod][1] = 1;
              else if (C.bt(t, triangle[1]) && C.bt(t, signbitb)) index[inod][1] = 3;
              else if (C.bt(t, triangle[2]) && C.bt(t, signbita)) index[inod][2] = 1;
              else if (C.bt(t, triangle[2]) && C.bt(t, signbitb)) index[inod][2] = 3;
              else if (C.bt(t, signbita)) index[inod][1] = index[inod][2] = 4;
              else index[inod][1] = index[inod][2] = 5;
            }
          }
        } else {
          info = 72;
          st.status |= ERR_SORTNODES;
        }
      } else if (it == 3) {
        for (int a = 1; a <= 7; a++) index[a][1] = index[a][2] = 0;
        for (int inod = 1; inod <= 7; inod++) {
          int nb = 0;
          for (int k = 1; k <= 3; k++) if (C.bt(N.ntype[inod], triangle[k])) nb++;
          if (C.bt(N.ntype[inod], penta[1])) {
            if (nb == 2) index[inod][1] = 1;
          } else {
            if (nb == 2) { index[inod][1] = 2; index[inod][2] = 1; }
            else { index[inod][2] = 4; iind = inod; }
          }
        }
        for (int k = 1; k <= 3; k++) if (C.bt(nty(iind), triangle[k])) signbita = triangle[k];
        for (int inod = 1; inod <= 7; inod++) {
          if (index[inod][1] == 0 && index[inod][2] == 0) {
            int t = N.ntype[inod];
            if (C.bt(t, signbita) && C.bt(t, square[1])) index[inod][2] = 5;
            else if (C.bt(t, signbita) && C.bt(t, square[2])) { index[inod][1] = 5; index[inod][2] = 2; }
            else if (C.bt(t, square[1])) { index[inod][1] = 4; index[inod][2] = 3; }
            else index[inod][1] = 3;
          }
        }
      } else {
        info = 73;
        st.status |= ERR_SORTNODES;
      }
    } break;
    case 8: {
      count_planes(true);
      for (int a = 1; a <= 8; a++) index[a][1] = index[a][2] = 0;
      if (is == 2) {
        for (int inod = 1; inod <= 8; inod++) {
          int t = N.ntype[inod];
          for (int it1 = 1; it1 <= 2; it1++) {
            if (C.bt(t, triangle[it1])) {
              if (C.bt(t, penta[1]) && C.bt(t, penta[2])) index[inod][1] = 1 + (it1 - 1) * 3;
              else if (C.bt(t, penta[1])) index[inod][1] = 2 + (it1 - 1) * 3;
              else if (C.bt(t, penta[2])) index[inod][1] = 3 + (it1 - 1) * 3;
            }
          }
          for (int iq1 = 1; iq1 <= 2; iq1++) {
            if (C.bt(t, penta[iq1])) {
              if (C.bt(t, square[1]) && C.bt(t, square[2])) index[inod][2] = 1 + (iq1 - 1) * 3;
              else if (C.bt(t, square[1])) index[inod][2] = 2 + (iq1 - 1) * 3;
              else if (C.bt(t, square[2])) index[inod][2] = 3 + (iq1 - 1) * 3;
            }
          }
        }
      } else if (is == 6) {
        int is1 = 0;
        index[1][1] = 1;
        index[1][2] = 0;
        for (int ibit = 0; ibit <= 5; ibit++) {
          if (C.bt(N.ntype[1], ibit)) { is1++; if (is1 <= 3) ibt[is1] = ibit; else st.status |= ERR_UNDEFINED; }
        }
        for (int inod = 2; inod <= 8; inod++) {
          int t = N.ntype[inod];
          if (C.bt(t, ibt[1])) {
            if (C.bt(t, ibt[2])) index[inod][1] = index[inod][2] = 2;
            else if (C.bt(t, ibt[3])) index[inod][1] = index[inod][2] = 3;
            else { index[inod][1] = 0; index[inod][2] = 1; }
          } else if (C.bt(t, ibt[2])) {
            if (C.bt(t, ibt[3])) { index[inod][1] = 4; index[inod][2] = 0; }
            else index[inod][1] = index[inod][2] = 5;
          } else {
            if (C.bt(t, ibt[3])) index[inod][1] = index[inod][2] = 6;
            else { index[inod][1] = 0; index[inod][2] = 4; }
          }
        }
      } else {
        info = 81;
        st.status |= ERR_SORTNODES;
      }
    } break;
    default:
      break;
  }
  return info;
}

// ------------------------------------------------------- convw1t_par
// for_tetrahedra3.f90:3-136.  weight[i*nom+iom].
// Reproduce the reference's wtemp layout for 7- and 8-node polyhedra (see
// convw1t) instead of adding the two halves at every frequency: off by
// default; the tests switch it on to compare with the reference's statements
// at every entry.
static std::atomic<int> g_reference_layout{0};
extern "C" void oracle_set_reference_layout(int on) { g_reference_layout.store(on ? 1 : 0); }

static void convw1t(double* weight, const double e[4], const double f[4], double ef, const double* omega, int nom,
                    Stats& st) {
  st.calls++;
  for (int i = 0; i < 4 * nom; i++) weight[i] = 0.0;
  Nodes N;
  surfnodes(N, e, f, ef);
  unrepnodes(N);
  if (relnodes(N, e, f, ef) != 0) { st.status |= ERR_RELNODES; return; }
  int index[9][3];
  const int nnod = N.nnod;
  if (nnod > 8) { st.status |= ERR_NNOD; return; }
  if (sortnodes(N, index, st) != 0) return;
  st.nnod_hist[nnod]++;
  // t_corners is one allocation reused by both sub-polyhedra of nnod 7/8;
  // positions never written are undefined in the reference (read as 0 here).
  double tc[6][3];
  bool written[6];
  for (int a = 0; a < 6; a++) { tc[a][0] = tc[a][1] = tc[a][2] = 0.0; written[a] = false; }
  auto place = [&](int pos, int inod, int cap) {
    if (pos < 1 || pos > cap) { st.status |= ERR_UNDEFINED; return; }
    for (int c = 0; c < 3; c++) tc[pos - 1][c] = N.x[inod][c + 1];
    written[pos - 1] = true;
  };
  auto check_written = [&](int cap) {
    for (int a = 0; a < cap; a++) if (!written[a]) st.status |= ERR_UNDEFINED;
  };
  switch (nnod) {
    case 0: case 1: case 2: case 3:
      break;
    case 4: {
      double c4[4][3];
      for (int n = 0; n < 4; n++) for (int c = 0; c < 3; c++) c4[n][c] = N.x[n + 1][c + 1];
      generictetra(weight, c4, e, f, omega, nom, st);
    } break;
    case 5:
      for (int inod = 1; inod <= 5; inod++) place(index[inod][1], inod, 5);
      check_written(5);
      genericfunf(weight, tc, e, f, omega, nom, st);
      break;
    case 6:
      for (int inod = 1; inod <= 6; inod++) place(index[inod][1], inod, 6);
      check_written(6);
      genericprism(weight, tc, e, f, omega, nom, st);
      break;
    case 7:
    case 8: {
      // The two halves' weights, summed per frequency.  The reference keeps
      // them in wtemp(4,2,nom) but addresses it as (4,nom,2)
      // (for_tetrahedra3.f90:36, 100-120); as compiled code addresses that
      // out-of-bounds layout, the second half overwrites the first from the
      // third frequency on and frequency j >= 3 gets w2(j-2) + w2(j).  This
      // restatement adds w1(j) + w2(j), which is what the reference computes
      // for the first two frequencies and what its code evidently means.
      const int cap = (nnod == 7) ? 5 : 6;
      double w1[4 * NOM_MAX], w2[4 * NOM_MAX];
      for (int isub = 1; isub <= 2; isub++) {
        for (int inod = 1; inod <= nnod; inod++)
          if (index[inod][isub] != 0) place(index[inod][isub], inod, cap);
        check_written(cap);
        double* dst = (isub == 1) ? w1 : w2;
        if (nnod == 7) genericfunf(dst, tc, e, f, omega, nom, st);
        else genericprism(dst, tc, e, f, omega, nom, st);
      }
      if (g_reference_layout.load(std::memory_order_relaxed)) {
        // the reference's addressing of wtemp(4,2,nom) as (4,nom,2): the first
        // half's weights survive for the first two frequencies only
        // (element (c, j) of the Fortran (4, nom) array lies 4·j + c values in;
        // this restatement stores it at c·nom + j).  With one frequency the
        // second half starts 8 values into an 8-value wtemp, past its end:
        // undefined, and the halves are added as an undisturbed stack would.
        if (nom < 2) st.status |= ERR_UNDEFINED;
        for (int c = 0; c < 4; c++)
          for (int j = 0; j < nom; j++)
            weight[c * nom + j] = (j < 2 ? w1[c * nom + j] : w2[c * nom + j - 2]) + w2[c * nom + j];
      } else {
        for (int i = 0; i < 4 * nom; i++) weight[i] = w1[i] + w2[i];
      }
    } break;
    default:
      st.status |= ERR_NNOD;
      break;
  }
}

// ------------------------------------------------- bz_calcqdepw_par2
// for_tetrahedra.f90:390-464.  All arrays in the reference's (Fortran) layout:
//   enk(nbnd,nkp), tetc(4,ntet), kqid(nkp) 0-based,
//   kcw(ncg+nomx+1, nbnd-ncg-numin, nkp, nom).
extern "C" int oracle_bz_calcqdepw_par2(const double* enk, int nbnd, int nkp, double ef, const int* kqid, int ncg,
                                        int nomx, int numin, const double* omega, int nom, const int* tetc, int ntet,
                                        double* kcw, int nthreads, long long* stats_out) {
  const int nb1 = ncg + nomx + 1;
  const int nb2 = nbnd - ncg - numin;
  if (nb1 <= 0 || nb2 <= 0 || nkp <= 0 || nom <= 0 || ntet <= 0 || nom > NOM_MAX) return -1;
  std::vector<int> tetln(ntet);
  for (int ik = 0; ik < nkp; ik++)
    for (int it = 1; it <= 6; it++) {
      int idx = 6 * ik + (it - 1);
      if (idx < ntet) tetln[idx] = 6 * kqid[ik] + it;  // 1-based, as in the reference
    }
  const double wtet = 1.0 / ntet;
  const size_t nkcw = (size_t)nb1 * nb2 * nkp * nom;
  for (size_t i = 0; i < nkcw; i++) kcw[i] = 0.0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  Stats total;
  for (int itet = 0; itet < ntet; itet++) {
    const int lt = tetln[itet] - 1;
#pragma omp parallel
    {
      Stats st;
      double w1t[4 * NOM_MAX];
#pragma omp for schedule(static)
      for (int jb = 1; jb <= nb2; jb++) {
        double ee2[4], ee1[4];
        for (int i = 0; i < 4; i++) ee2[i] = enk[(size_t)(jb + ncg + numin - 1) + (size_t)nbnd * tetc[i + 4 * lt]];
        double mx = ee2[0];
        for (int i = 1; i < 4; i++) if (ee2[i] > mx) mx = ee2[i];
        if (mx <= ef) continue;
        for (int ib = 1; ib <= nb1; ib++) {
          for (int i = 0; i < 4; i++) ee1[i] = enk[(size_t)(ib - 1) + (size_t)nbnd * tetc[i + 4 * itet]];
          double mn = ee1[0];
          for (int i = 1; i < 4; i++) if (ee1[i] < mn) mn = ee1[i];
          if (mn > ef) continue;
          convw1t(w1t, ee1, ee2, ef, omega, nom, st);
          for (int i = 0; i < 4; i++) {
            const int kin = tetc[i + 4 * itet];
            for (int iom = 0; iom < nom; iom++) {
              double& dst = kcw[(size_t)(ib - 1) + (size_t)nb1 * ((size_t)(jb - 1) + (size_t)nb2 * ((size_t)kin + (size_t)nkp * iom))];
              dst = dst + w1t[i * nom + iom] * 6.0 * wtet;
              if (!std::isfinite(dst)) st.status |= ERR_NONFINITE;
            }
          }
        }
      }
#pragma omp critical
      total.merge(st);
    }
  }
  if (stats_out) {
    stats_out[0] = total.calls;
    for (int i = 0; i < 9; i++) stats_out[1 + i] = total.nnod_hist[i];
    for (int i = 0; i < 5; i++) stats_out[10 + i] = total.equiv_hist[i];
    stats_out[15] = total.taylor;
    stats_out[16] = total.exact;
    stats_out[17] = total.zero_vol;
    stats_out[18] = total.big_weight_warn;
    stats_out[19] = total.big_weight_zeroed;
  }
  return (int)total.status;
}

// ------------------------------------------------- bz_calcqdepw_par3
// for_tetrahedra.f90:466-542: the same loops as par2, but the corner weights
// of each (tetrahedron, ib, jb) are projected on the SVD frequency basis
// before they are accumulated: w2t(i,l) = Σ_ω w1t(i,ω)·dUl(ω,l) (matmul,
// ω ascending), kcw(ib,jb,k,l) += w2t(i,l)·6·wtet.  dUl is (nom, nl) Fortran
// order; kcw is (ncg+nomx+1, nbnd-ncg-numin, nkp, nl).
extern "C" int oracle_bz_calcqdepw_par3(const double* enk, int nbnd, int nkp, double ef, const int* kqid, int ncg,
                                        int nomx, int numin, const double* dUl, int nl, const double* omega, int nom,
                                        const int* tetc, int ntet, double* kcw, int nthreads) {
  const int nb1 = ncg + nomx + 1;
  const int nb2 = nbnd - ncg - numin;
  if (nb1 <= 0 || nb2 <= 0 || nkp <= 0 || nom <= 0 || ntet <= 0 || nl <= 0 || nom > NOM_MAX || nl > NOM_MAX)
    return -1;
  std::vector<int> tetln(ntet);
  for (int ik = 0; ik < nkp; ik++)
    for (int it = 1; it <= 6; it++) {
      int idx = 6 * ik + (it - 1);
      if (idx < ntet) tetln[idx] = 6 * kqid[ik] + it;
    }
  const double wtet = 1.0 / ntet;
  const size_t nkcw = (size_t)nb1 * nb2 * nkp * nl;
  for (size_t i = 0; i < nkcw; i++) kcw[i] = 0.0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  unsigned status = 0;
  for (int itet = 0; itet < ntet; itet++) {
    const int lt = tetln[itet] - 1;
#pragma omp parallel
    {
      Stats st;
      double w1t[4 * NOM_MAX], w2t[4 * NOM_MAX];
#pragma omp for schedule(static)
      for (int jb = 1; jb <= nb2; jb++) {
        double ee2[4], ee1[4];
        for (int i = 0; i < 4; i++) ee2[i] = enk[(size_t)(jb + ncg + numin - 1) + (size_t)nbnd * tetc[i + 4 * lt]];
        double mx = ee2[0];
        for (int i = 1; i < 4; i++) if (ee2[i] > mx) mx = ee2[i];
        if (mx <= ef) continue;
        for (int ib = 1; ib <= nb1; ib++) {
          for (int i = 0; i < 4; i++) ee1[i] = enk[(size_t)(ib - 1) + (size_t)nbnd * tetc[i + 4 * itet]];
          double mn = ee1[0];
          for (int i = 1; i < 4; i++) if (ee1[i] < mn) mn = ee1[i];
          if (mn > ef) continue;
          convw1t(w1t, ee1, ee2, ef, omega, nom, st);
          for (int i = 0; i < 4; i++)
            for (int l = 0; l < nl; l++) {
              double acc = 0.0;
              for (int iom = 0; iom < nom; iom++) acc = acc + w1t[i * nom + iom] * dUl[(size_t)iom + (size_t)nom * l];
              w2t[i * nl + l] = acc;
            }
          for (int i = 0; i < 4; i++) {
            const int kin = tetc[i + 4 * itet];
            for (int l = 0; l < nl; l++) {
              double& dst = kcw[(size_t)(ib - 1) + (size_t)nb1 * ((size_t)(jb - 1) + (size_t)nb2 * ((size_t)kin + (size_t)nkp * l))];
              dst = dst + w2t[i * nl + l] * 6.0 * wtet;
            }
          }
        }
      }
#pragma omp critical
      status |= st.status;
    }
  }
  return (int)status;
}

// Single tetrahedron entry point (convw1t_par) for known-answer tests.
extern "C" int oracle_convw1t(const double* e, const double* f, double ef, const double* omega, int nom,
                              double* weight /* [4][nom] */, long long* nnod_out) {
  if (nom <= 0 || nom > NOM_MAX) return -1;
  Stats st;
  convw1t(weight, e, f, ef, omega, nom, st);
  if (nnod_out) {
    long long n = -1;
    for (int i = 0; i < 9; i++) if (st.nnod_hist[i]) n = i;
    *nnod_out = n;
  }
  return (int)st.status;
}

// generictetra_par on an explicit tetrahedron (corners in the unit-tet frame).
extern "C" int oracle_generictetra(const double* corners /* [4][3] */, const double* e, const double* f,
                                   const double* omega, int nom, double* wt_out /* [4][nom] */) {
  if (nom <= 0 || nom > NOM_MAX) return -1;
  Stats st;
  double c[4][3];
  for (int n = 0; n < 4; n++) for (int k = 0; k < 3; k++) c[n][k] = corners[3 * n + k];
  int info = generictetra(wt_out, c, e, f, omega, nom, st);
  return info | (int)st.status << 8;
}

// The portable atan/log, exported so the tests can compare them with libm.
extern "C" void oracle_portable_math(const double* x, int n, double* atan_out, double* log_out) {
  for (int i = 0; i < n; i++) {
    atan_out[i] = pg_atan(x[i]);
    log_out[i] = x[i] > 0.0 ? pg_log(x[i]) : NAN;
  }
}

// Geometry of one (tetrahedron, band pair) for inspection in tests:
// nodes[20][3], ntype[20], index[9][2] (index[inod][isub], 1-based inod), returns nnod.
extern "C" int oracle_debug_nodes(const double* e, const double* f, double ef, double* nodes, int* ntype,
                                  int* index_out) {
  Stats st;
  Nodes N;
  surfnodes(N, e, f, ef);
  unrepnodes(N);
  if (relnodes(N, e, f, ef) != 0) return -1;
  int index[9][3];
  if (N.nnod <= 8) sortnodes(N, index, st);
  for (int n = 1; n <= 20; n++) {
    for (int c = 0; c < 3; c++) nodes[3 * (n - 1) + c] = N.x[n][c + 1];
    ntype[n - 1] = N.ntype[n];
  }
  for (int a = 0; a < 9; a++) { index_out[2 * a] = index[a][1]; index_out[2 * a + 1] = index[a][2]; }
  return N.nnod;
}
