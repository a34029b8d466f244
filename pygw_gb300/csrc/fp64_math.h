// Portable double-precision atan and log, compiled identically for the host
// and for sm_103a so that both produce the same bits.
//
// Why: the tetrahedron weight formulas (closed form of
// 2Re∫ f_i/(iω−Δe) over a tetrahedron) cancel heavily when the corner energy
// differences are close but not grouped (relative spread just above 1%).  A
// one-ulp difference in atan/log between two math libraries is then amplified
// to ~1e-11 relative in the weight.  Using one implementation built only from
// IEEE-754 correctly rounded operations (+ − × ÷ √ and fma) on both sides makes
// the CUDA weights bit-identical to the CPU restatement.
//
// Methods (both textbook, constants derived here with mpmath at 200 bits):
//  * log:  x = 2^k·m with m in [√½, √2); log m = 2·atanh(s), s = (m−1)/(m+1),
//          |s| ≤ 0.1716, atanh series truncated after s^21 (tail < 2^-55
//          relative); k·ln2 with a 42-bit ln2_hi so k·ln2_hi is exact
//          (Cody–Waite splitting).
//  * atan: odd symmetry; |x| > 1 uses π/2 − atan(1/|x|); then the addition
//          formula atan(t) = atan(c) + atan((t−c)/(1+t·c)) with c = j/8,
//          j = round(8t), so the reduced argument is ≤ 1/16 and the Taylor
//          series truncated after u^15 has tail < 2^-59.  atan(j/8) and π/2
//          are double-double constants.
// Accuracy: a few ulp at worst (checked against libm in the tests); what
// matters here is determinism, not correct rounding.
// Build rule: the translation units that include this file must not contract
// a*b+c into fma on their own (nvcc -fmad=false, gcc -ffp-contract=off);
// every fma below is explicit.
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define PG_HD __host__ __device__ __forceinline__
#else
#define PG_HD static inline
#endif

PG_HD uint64_t pg_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u; memcpy(&u, &x, 8); return u;
#endif
}
PG_HD double pg_from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x; memcpy(&x, &u, 8); return x;
#endif
}

// Natural logarithm for finite x > 0 (the only inputs the weight code
// produces: ev^2 + ω^2 > 1e-10).  Non-positive / non-finite inputs give NaN/inf.
PG_HD double pg_log(double x) {
  if (!(x > 0.0)) return (x == 0.0) ? -INFINITY : NAN;
  if (x == INFINITY) return x;
  int k = 0;
  uint64_t u = pg_bits(x);
  int ex = (int)((u >> 52) & 0x7ff);
  if (ex == 0) {                      // subnormal: scale by 2^54 (exact)
    x = x * 18014398509481984.0;
    u = pg_bits(x);
    ex = (int)((u >> 52) & 0x7ff);
    k = -54;
  }
  // m in [1, 2): replace the exponent field by the bias
  k += ex - 1023;
  double m = pg_from_bits((u & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
  if (m > 1.4142135623730951) { m = m * 0.5; k += 1; }   // exact halving
  const double f = m - 1.0;                 // exact (Sterbenz)
  const double s = f / (m + 1.0);           // m+1 exact: m in [0.70,1.42), ulp(m) ≥ 2^-53
  const double z = s * s;
  // R(z) = sum_{n=1..10} 2 z^n/(2n+1), Horner with explicit fma
  double r = 0.09523809523809523;
  r = fma(r, z, 0.10526315789473684);
  r = fma(r, z, 0.11764705882352941);
  r = fma(r, z, 0.13333333333333333);
  r = fma(r, z, 0.15384615384615385);
  r = fma(r, z, 0.18181818181818182);
  r = fma(r, z, 0.2222222222222222);
  r = fma(r, z, 0.2857142857142857);
  r = fma(r, z, 0.4);
  r = fma(r, z, 0.6666666666666666);
  r = r * z;
  const double two_s = s + s;
  const double lm = fma(s, r, two_s);       // log(m) = 2s + s·R
  if (k == 0) return lm;
  const double dk = (double)k;
  const double LN2_HI = 0.6931471805598903;      // 0x1.62e42fefa3800p-1
  const double LN2_LO = 5.497923018708371e-14;   // 0x1.ef35793c76730p-45
  return dk * LN2_HI + fma(dk, LN2_LO, lm);
}

// Arc tangent for any double.
PG_HD double pg_atan(double x) {
  if (x != x) return x;
  const double a = fabs(x);
  const int inv = a > 1.0;
  const double t = inv ? 1.0 / a : a;       // t in [0, 1]
  const int j = (int)(t * 8.0 + 0.5);       // 0..8
  const double c = (double)j * 0.125;       // exact
  double u, th, tl;
  switch (j) {                              // atan(j/8) as double-double
    case 0: th = 0.0; tl = 0.0; break;
    case 1: th = 0.12435499454676144; tl = -3.1253241424539383e-18; break;
    case 2: th = 0.24497866312686414; tl = 1.0698755618734451e-17; break;
    case 3: th = 0.35877067027057225; tl = -2.4623815582638635e-17; break;
    case 4: th = 0.4636476090008061;  tl = 2.2698777452961687e-17; break;
    case 5: th = 0.5585993153435624;  tl = -5.4556305485916264e-18; break;
    case 6: th = 0.6435011087932844;  tl = 1.5834785051444286e-17; break;
    case 7: th = 0.7188299996216245;  tl = -2.1478388444456983e-17; break;
    default: th = 0.7853981633974483; tl = 3.061616997868383e-17; break;
  }
  if (j == 0) {
    u = t;
  } else {
    u = (t - c) / fma(t, c, 1.0);           // t − c exact (Sterbenz)
  }
  const double z = u * u;
  // P(z) = sum_{n=1..7} (−1)^n z^n/(2n+1)
  double p = -0.06666666666666667;
  p = fma(p, z, 0.07692307692307693);
  p = fma(p, z, -0.09090909090909091);
  p = fma(p, z, 0.1111111111111111);
  p = fma(p, z, -0.14285714285714285);
  p = fma(p, z, 0.2);
  p = fma(p, z, -0.3333333333333333);
  p = p * z;
  const double au = fma(u, p, u);           // atan(u) = u + u·P(u²)
  double res;
  if (!inv) {
    res = th + (tl + au);
  } else {
    const double PIO2_HI = 1.5707963267948966;
    const double PIO2_LO = 6.123233995736766e-17;
    res = (PIO2_HI - th) + ((PIO2_LO - tl) - au);
  }
  return copysign(res, x);
}
