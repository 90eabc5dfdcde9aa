/*
 * lpg_init.h — per-slot arithmetic of the model's initialisation, shared by
 * the CUDA kernels (lpg_init.cu) and the C oracle, so that both fill the
 * agent table with the same bits from the same counter-based draws.
 *
 * What each function restates (laser_polio/model.py unless noted):
 *   lpg_init_timers  exposure, infection and paralysis timers of every
 *                    capacity slot (:575-587): a draw stored into int8 the
 *                    way numpy's unsafe cast does (truncation, low byte),
 *                    then clipped to [0, 127]; the paralysis timer is the
 *                    time to paralysis less the exposure timer, clipped to
 *                    [0, min(infection timer, 127)] and truncated.
 *   lpg_init_het     acquisition risk and daily infectivity of every slot
 *                    (populate_heterogeneous_values, :816-866): a pair of
 *                    standard normals correlated through the Cholesky factor
 *                    of [[1, rho], [rho, 1]], rho = 2 sin(pi corr / 6) (the
 *                    Spearman correction); risk lognormal with mean 1, its
 *                    variance risk_mult_var; infectivity the exponential
 *                    (gamma, shape 1) quantile of the second normal's CDF,
 *                    -scale ln(1 - Phi(z)).
 *   lpg_init_age     an initial agent's age in days (:1576-1596): an age bin
 *                    with probability proportional to its weight, then a day
 *                    uniformly in [lo, hi); at least 1.
 *   lpg_km_age_at_death  laser_core's KaplanMeierEstimator.
 *                    predict_age_at_death as this package restates it
 *                    (core.py): the year of death drawn from the cumulative
 *                    deaths behind the agent's age-year, the day uniform in
 *                    that year and not before the current age.
 *   lpg_init_ri      the RI date (:1887-1894): date of birth plus a uniform
 *                    day in [42, 98), truncated to int32 and stored in int16.
 * The draws are this project's own (purposes LPG_P_INIT_* of lpg_rng.h);
 * the reference draws the same distributions from numpy's generator.
 */
#ifndef LPG_INIT_H
#define LPG_INIT_H

#include <stdint.h>

#include "lpg_rng.h"

#define LPG_PI 3.14159265358979323846
#define LPG_SQRT1_2 0.70710678118654752440    /* 1/sqrt(2) */
#define LPG_2_SQRTPI 1.12837916709551257390   /* 2/sqrt(pi) */
#define LPG_1_SQRTPI 0.56418958354775628695   /* 1/sqrt(pi) */

/* erf(x) for 0 <= x < 2 from its Maclaurin series
 * 2/sqrt(pi) sum_n (-1)^n x^(2n+1) / (n! (2n+1)), summed until the term
 * no longer changes the sum (at most 60 terms; the divisions by n and by
 * 2n + 1 through the correctly rounded reciprocal table). */
LPG_HD double lpg_erf_series(double x) {
  const double x2 = x * x;
  double term = x; /* x^(2n+1) / n! */
  double sum = x;
  for (int n = 1; n < 60; ++n) {
    term = -(term * x2) * lpg_recip_small(n);
    const double add = term * lpg_recip_small(2 * n + 1);
    const double next = sum + add;
    if (next == sum) break;
    sum = next;
  }
  return LPG_2_SQRTPI * sum;
}

/* erfc(x) for x >= 2 from Laplace's continued fraction
 * erfc(x) = exp(-x^2)/sqrt(pi) / (x + (1/2)/(x + 1/(x + (3/2)/(x + ...)))),
 * evaluated from depth 64 upward. */
LPG_HD double lpg_erfc_cf(double x) {
  double t = x;
  for (int n = 64; n >= 1; --n) t = x + (0.5 * (double)n) / t;
  return lpg_exp(-(x * x)) * LPG_1_SQRTPI / t;
}

/* 1 - Phi(z), the standard normal's upper tail. */
LPG_HD double lpg_norm_sf(double z) {
  const double x = fabs(z) * LPG_SQRT1_2;
  double half_erfc; /* 0.5 erfc(x) = P(Z > |z|) */
  if (x < 2.0) {
    half_erfc = 0.5 - 0.5 * lpg_erf_series(x);
  } else {
    half_erfc = 0.5 * lpg_erfc_cf(x);
  }
  return z >= 0.0 ? half_erfc : 1.0 - half_erfc;
}

/* Timers of one capacity slot. */
LPG_HD void lpg_init_timers(uint64_t seed, uint64_t slot, int k_exp, double e1, double e2, int k_inf, double i1,
                            double i2, int k_par, double p1, double p2, int8_t* et, int8_t* it, int8_t* pt) {
  lpg_stream s;
  lpg_stream_init(&s, seed, LPG_P_INIT_TIMER, 0, slot, 0);
  int8_t e = lpg_trunc_i8(lpg_dist_sample(&s, k_exp, e1, e2));
  lpg_stream_init(&s, seed, LPG_P_INIT_TIMER, 0, slot, 1);
  int8_t i = lpg_trunc_i8(lpg_dist_sample(&s, k_inf, i1, i2));
  e = e < 0 ? (int8_t)0 : e;
  i = i < 0 ? (int8_t)0 : i;
  lpg_stream_init(&s, seed, LPG_P_INIT_TIMER, 0, slot, 2);
  double raw = lpg_dist_sample(&s, k_par, p1, p2) - (double)e;
  const double upper = (double)i; /* min(infection timer, 127): already <= 127 */
  raw = raw < 0.0 ? 0.0 : raw;
  raw = raw > upper ? upper : raw;
  *et = e;
  *it = i;
  *pt = lpg_trunc_i8(raw);
}

/* Risk and infectivity of one capacity slot: mu, sigma of the risk's
 * normal; rho and sqrt(1 - rho^2); the infectivity's scale (mean); het = 0
 * gives risk 1 and the mean infectivity, as without heterogeneity. */
LPG_HD void lpg_init_het(uint64_t seed, uint64_t slot, int het, double mu, double sigma, double rho, double srho,
                         double scale, float* risk, float* inf) {
  if (!het) {
    *risk = 1.0f;
    *inf = (float)scale;
    return;
  }
  lpg_stream s;
  lpg_stream_init(&s, seed, LPG_P_INIT_HET, 0, slot, 0);
  const double z0 = lpg_std_normal(&s);
  const double z1 = lpg_std_normal(&s);
  const double zc1 = rho * z0 + srho * z1;
  *risk = (float)lpg_exp(mu + sigma * z0);
  *inf = (float)(-scale * lpg_log(lpg_norm_sf(zc1)));
}

/* Age in days of an initial agent: bin b with probability weight[b] / total
 * (cum[b] = weight[0] + ... + weight[b], integers), day uniform in
 * [lo[b], hi[b]); at least 1. */
LPG_HD int32_t lpg_init_age(uint64_t seed, uint64_t slot, int32_t n_bins, const int64_t* cum, const int32_t* lo,
                            const int32_t* hi) {
  const uint64_t total = (uint64_t)cum[n_bins - 1];
  const uint64_t v = lpg_scale_target(lpg_u53(seed, LPG_P_INIT_AGE, 0, slot, 0, 0), total);
  int32_t a = 0, b = n_bins - 1; /* first bin with cum > v */
  while (a < b) {
    const int32_t m = (a + b) >> 1;
    if ((uint64_t)cum[m] > v) b = m; else a = m + 1;
  }
  const double span = (double)(hi[a] - lo[a]);
  int32_t age = lo[a] + (int32_t)floor(lpg_u01(seed, LPG_P_INIT_AGE, 0, slot, 0, 1) * span);
  return age < 1 ? 1 : age;
}

/* Age at death in days of an agent aged age_days, from cumulative deaths by
 * age-year cum[0..len) up to max_year, with uniforms u0, u1. */
LPG_HD int32_t lpg_km_age_at_death(const int64_t* cum, int32_t len, int32_t max_year, int64_t age_days, double u0,
                                   double u1) {
  const int32_t top = max_year < len - 1 ? max_year : len - 1;
  int64_t years = age_days / 365;
  if (years > top) years = top;
  const int64_t lower = years > 0 ? cum[years - 1] : 0;
  const int64_t total = cum[top];
  const int64_t span = total - lower > 0 ? total - lower : 0;
  int64_t y = top;
  if (span > 0) {
    const int64_t draw = lower + (int64_t)floor(u0 * (double)span);
    int32_t a = 0, b = top + 1; /* first index with cum > draw, top + 1 if none */
    while (a < b) {
      const int32_t m = (a + b) >> 1;
      if (cum[m] > draw) b = m; else a = m + 1;
    }
    y = a > years ? a : years;
    if (y > top) y = top;
  }
  const int64_t day_lo = y == years ? age_days : y * 365;
  int64_t day_hi = (y + 1) * 365;
  if (day_hi < day_lo + 1) day_hi = day_lo + 1;
  return (int32_t)(day_lo + (int64_t)floor(u1 * (double)(day_hi - day_lo)));
}

/* RI date of an initial agent born on dob (int16, as the column stores it). */
LPG_HD int16_t lpg_init_ri(uint64_t seed, uint64_t slot, int32_t dob) {
  const double day = 42.0 + 56.0 * lpg_u01(seed, LPG_P_INIT_RI, 0, slot, 0, 0);
  const double v = (double)dob + day;
  return (int16_t)(uint16_t)(uint32_t)(int32_t)v;
}

#endif /* LPG_INIT_H */
