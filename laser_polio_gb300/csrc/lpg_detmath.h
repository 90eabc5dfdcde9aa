/*
 * lpg_detmath.h — deterministic double-precision elementary functions.
 *
 * Every function here is built from IEEE-754 operations that are correctly
 * rounded on every target this project compiles for (add, sub, mul, div,
 * sqrt, floor, and exact power-of-two scaling), evaluated in a fixed order.
 * Compiled with contraction disabled (gcc -ffp-contract=off, nvcc
 * --fmad=false) the same input gives the same bits on x86-64, aarch64 and
 * sm_103a.  That is what lets the CUDA engine and the CPU oracle consume one
 * counter-based random stream and agree bit for bit on every integer draw
 * that depends on an exp() or a log() (Poisson counts, gamma variates,
 * probabilities of exposure).
 *
 * Methods (all textbook mathematics, coefficients derived from first
 * principles, not taken from any vendor library):
 *   exp    Cody–Waite reduction x = k ln2 + r with a two-part ln2
 *          (high part with 33 significant bits so k*hi is exact), then the
 *          Taylor series of e^r to degree 14 (|r| <= ln2/2, truncation error
 *          below 1e-18 relative), then exact scaling by 2^k.
 *   Every polynomial is evaluated by Estrin's scheme (short dependency
 *   chains: double-precision latency, not throughput, bounds the
 *   single-thread draws on the GPU).
 *   expm1  the same Taylor series without its constant term when
 *          |x| < ln2/2 (full relative precision for tiny rates), else exp-1.
 *   log    x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s),
 *          s = (m-1)/(m+1), |s| <= 0.1716, atanh series to s^25.
 *   lfact  log(k!) exactly from the double k! for k < 20, else Stirling's
 *          series for log Gamma(k+1) to the x^-7 term.
 * Accuracy is a few ulp; the tests compare against numpy.
 */
#ifndef LPG_DETMATH_H
#define LPG_DETMATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define LPG_HD __host__ __device__ __forceinline__
#else
#define LPG_HD static inline
#endif

#if !defined(__CUDACC__)
#include <math.h>
#include <string.h>
#endif

/* ln 2 split: LN2_HI = ln2 rounded to double with its low 20 mantissa bits
 * cleared; LN2_LO = ln2 - LN2_HI rounded to double. */
#define LPG_LN2_HI 0x1.62e42fef00000p-1
#define LPG_LN2_LO 0x1.473de6af278edp-34
#define LPG_INV_LN2 0x1.71547652b82fep+0
#define LPG_SQRT2 0x1.6a09e667f3bcdp+0
#define LPG_HALF_LOG_2PI 0x1.d67f1c864beb5p-1

LPG_HD uint64_t lpg_dbits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

LPG_HD double lpg_bitsd(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

/* 2^k for -1022 <= k <= 1023, built from the exponent field. */
LPG_HD double lpg_pow2i(int k) { return lpg_bitsd((uint64_t)(k + 1023) << 52); }

/* p * 2^k, exact whenever the result is a normal double. */
LPG_HD double lpg_scale2(double p, int k) {
  if (k > 1023) return (p * lpg_pow2i(1023)) * lpg_pow2i(k - 1023);
  if (k < -1022) return (p * lpg_pow2i(k + 600)) * lpg_pow2i(-600);
  return p * lpg_pow2i(k);
}

/* Polynomials by Estrin's scheme (pairs, then powers r^2, r^4, r^8): the
 * same polynomial as Horner's rule with a dependency depth of about 8
 * operations instead of 2 per coefficient, which matters on a GPU whose
 * double-precision operations have a long latency.  Coefficients are the
 * correctly rounded reciprocals of the exact double factorials.  The series
 * are arranged as r + r^2 P(r) so that the dominant term r is exact and the
 * rounding of P is scaled down by r. */

/* P(r) = sum_{n=0}^{14} r^n / (n+2)! */
LPG_HD double lpg_em1_tail16(double r, double r2, double r4, double r8) {
  const double q0 = 0.5 + (1.0 / 6.0) * r;
  const double q1 = (1.0 / 24.0) + (1.0 / 120.0) * r;
  const double q2 = (1.0 / 720.0) + (1.0 / 5040.0) * r;
  const double q3 = (1.0 / 40320.0) + (1.0 / 362880.0) * r;
  const double q4 = (1.0 / 3628800.0) + (1.0 / 39916800.0) * r;
  const double q5 = (1.0 / 479001600.0) + (1.0 / 6227020800.0) * r;
  const double q6 = (1.0 / 87178291200.0) + (1.0 / 1307674368000.0) * r;
  const double q7 = 1.0 / 20922789888000.0;
  const double s0 = q0 + q1 * r2;
  const double s1 = q2 + q3 * r2;
  const double s2 = q4 + q5 * r2;
  const double s3 = q6 + q7 * r2;
  const double t0 = s0 + s1 * r4;
  const double t1 = s2 + s3 * r4;
  return t0 + t1 * r8;
}

/* P(r) = sum_{n=0}^{12} r^n / (n+2)! */
LPG_HD double lpg_em1_tail14(double r, double r2, double r4, double r8) {
  const double q0 = 0.5 + (1.0 / 6.0) * r;
  const double q1 = (1.0 / 24.0) + (1.0 / 120.0) * r;
  const double q2 = (1.0 / 720.0) + (1.0 / 5040.0) * r;
  const double q3 = (1.0 / 40320.0) + (1.0 / 362880.0) * r;
  const double q4 = (1.0 / 3628800.0) + (1.0 / 39916800.0) * r;
  const double q5 = (1.0 / 479001600.0) + (1.0 / 6227020800.0) * r;
  const double q6 = 1.0 / 87178291200.0;
  const double s0 = q0 + q1 * r2;
  const double s1 = q2 + q3 * r2;
  const double s2 = q4 + q5 * r2;
  const double t0 = s0 + s1 * r4;
  const double t1 = s2 + q6 * r4;
  return t0 + t1 * r8;
}

/* sum_{n=0}^{14} r^n / n! = 1 + (r + r^2 P(r)). */
LPG_HD double lpg_exp_series(double r) {
  const double r2 = r * r;
  const double r4 = r2 * r2;
  const double r8 = r4 * r4;
  return 1.0 + (r + r2 * lpg_em1_tail14(r, r2, r4, r8));
}

/* sum_{n=1}^{16} r^n / n! = r + r^2 P(r) — e^r - 1 without its constant. */
LPG_HD double lpg_expm1_series(double r) {
  const double r2 = r * r;
  const double r4 = r2 * r2;
  const double r8 = r4 * r4;
  return r + r2 * lpg_em1_tail16(r, r2, r4, r8);
}

LPG_HD double lpg_exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return lpg_bitsd(0x7ff0000000000000ULL);
  if (x < -745.2) return 0.0;
  double kd = floor(x * LPG_INV_LN2 + 0.5);
  double r = (x - kd * LPG_LN2_HI) - kd * LPG_LN2_LO;
  return lpg_scale2(lpg_exp_series(r), (int)kd);
}

LPG_HD double lpg_expm1(double x) {
  if (x != x) return x;
  if (x > -0.3465 && x < 0.3465) return lpg_expm1_series(x);
  if (x < -40.0) return -1.0;
  return lpg_exp(x) - 1.0;
}

LPG_HD double lpg_log(double x) {
  if (x != x) return x;
  if (x <= 0.0) return x == 0.0 ? -lpg_bitsd(0x7ff0000000000000ULL) : lpg_bitsd(0x7ff8000000000000ULL);
  if (x == lpg_bitsd(0x7ff0000000000000ULL)) return x;
  int eadj = 0;
  if (x < 0x1.0p-1022) { x = x * 0x1.0p54; eadj = -54; }
  uint64_t b = lpg_dbits(x);
  int e = (int)((b >> 52) & 0x7ff) - 1023 + eadj;
  double m = lpg_bitsd((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL); /* [1,2) */
  if (m > LPG_SQRT2) { m = m * 0.5; e += 1; }
  double s = (m - 1.0) / (m + 1.0);
  /* log m = 2s + 2s z Q(z), z = s^2, Q = sum_{n=0}^{11} z^n / (2n+3) by
   * Estrin's scheme; the leading 2s is exact */
  const double z = s * s;
  const double z2 = z * z;
  const double z4 = z2 * z2;
  const double z8 = z4 * z4;
  const double p0 = (1.0 / 3.0) + (1.0 / 5.0) * z;
  const double p1 = (1.0 / 7.0) + (1.0 / 9.0) * z;
  const double p2 = (1.0 / 11.0) + (1.0 / 13.0) * z;
  const double p3 = (1.0 / 15.0) + (1.0 / 17.0) * z;
  const double p4 = (1.0 / 19.0) + (1.0 / 21.0) * z;
  const double p5 = (1.0 / 23.0) + (1.0 / 25.0) * z;
  const double u0 = p0 + p1 * z2;
  const double u1 = p2 + p3 * z2;
  const double u2 = p4 + p5 * z2;
  const double v0 = u0 + u1 * z4;
  const double q = v0 + u2 * z8;
  const double s2x = 2.0 * s;
  double lm = s2x + (s2x * z) * q;
  double ed = (double)e;
  return ed * LPG_LN2_HI + (ed * LPG_LN2_LO + lm);
}

/* log(k!) for integer k >= 0. */
LPG_HD double lpg_lfact(int64_t k) {
  if (k < 2) return 0.0;
  if (k < 20) {
    double f = 1.0;
    for (int64_t i = 2; i <= k; ++i) f = f * (double)i; /* exact below 2^53 */
    return lpg_log(f);
  }
  double x = (double)(k + 1);
  double ix = 1.0 / x;
  double ix2 = ix * ix;
  double corr = ix * (1.0 / 12.0 - ix2 * (1.0 / 360.0 - ix2 * (1.0 / 1260.0 - ix2 * (1.0 / 1680.0))));
  return (x - 0.5) * lpg_log(x) - x + LPG_HALF_LOG_2PI + corr;
}

/* rint(r * 2^24) as an unsigned integer, clamped to [0, 2^62], for a float
 * r (0 for r <= 0 and NaN) — the fixed-point susceptibility weight — from
 * the bits of r alone, with integer operations only.  r * 2^24 is exact in
 * double, so this equals the double-precision definition
 * (d = (double)r * 2^24; !(d > 0) -> 0; min(d, 2^62); rint(d)) bit for bit:
 * for r = M * 2^(E - 150) (M the 24-bit significand, E the biased exponent)
 * the product is M * 2^(E - 126), a left shift for E >= 126 and otherwise a
 * right shift rounded half to even. */
LPG_HD uint64_t lpg_fix_risk_bits(float r) {
  union {
    float f;
    uint32_t u;
  } c;
  c.f = r;
  const uint32_t u = c.u;
  if (u & 0x80000000u) return 0; /* negative (or -0, negative NaN) */
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t frac = u & 0x7fffffu;
  if (e == 0xffu) return frac ? 0 : ((uint64_t)1 << 62); /* NaN -> 0, +inf -> clamp */
  if (e == 0) return 0;                                   /* zero or subnormal: below 2^-126 * 2^24 < 1/2 */
  const uint64_t m = (uint64_t)(frac | 0x800000u);
  if (e >= 126) {
    const uint32_t sh = e - 126;
    if (sh >= 39) return (uint64_t)1 << 62; /* m * 2^sh >= 2^62 */
    const uint64_t v = m << sh;
    return v > ((uint64_t)1 << 62) ? ((uint64_t)1 << 62) : v;
  }
  const uint32_t s = 126 - e; /* 1 .. 125 */
  if (s > 24) return 0;       /* m * 2^-s < 1/2 */
  const uint64_t q = m >> s;
  const uint64_t rem = m & (((uint64_t)1 << s) - 1);
  const uint64_t half = (uint64_t)1 << (s - 1);
  return q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
}

/* The same weight with single-precision arithmetic: r * 2^24 is exact in
 * float (a power-of-two scaling), and rounding an exact value to the nearest
 * integer, ties to even, gives the same integer in float as in double (below
 * 2^24 the result is representable; above 2^23 the value is already an
 * integer).  One multiply and one rounding conversion, no branches on the
 * bits. */
LPG_HD uint64_t lpg_fix_risk_f32(float r) {
  const float f = r * 16777216.0f;
  if (!(f > 0.0f)) return 0;
  if (f > 0x1.0p62f) return (uint64_t)1 << 62;
#if defined(__CUDA_ARCH__)
  /* the 32-bit conversion (single-precision path) whenever the integer fits:
   * every risk below 256; the 64-bit conversion is far slower on this GPU */
  if (f < 4294967296.0f) return (uint64_t)__float2uint_rn(f);
  return __float2ull_rn(f);
#else
  return (uint64_t)rintf(f);
#endif
}

#endif /* LPG_DETMATH_H */
