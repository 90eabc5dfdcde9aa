/*
 * lpg_rng.h — the counter-based draw hook shared by the CUDA engine and the
 * CPU oracle.
 *
 * The reference draws from numba's per-thread np.random state
 * (laser_polio/model.py:446, :1712-1716, :1848, :1852, :2047, :1096,
 * :1130, :1388-1405), which cannot be replayed on another machine or thread
 * count.  Here every random number is a pure function of
 *     (seed, purpose, tick, a, b, k)
 * evaluated with Philox4x64-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
 * numbers: as easy as 1, 2, 3", SC'11).  a/b identify the agent slot (in the
 * reference's slot order) or the node, k is the position in that stream.
 * Any thread, in any order, on either machine gets the same value, so the
 * GPU and the oracle agree on every draw without sharing state.
 *
 * Samplers built on it (all published methods):
 *   Poisson   inversion by sequential search for lam < 10; PTRS transformed
 *             rejection (W. Hormann, "The transformed rejection method for
 *             generating Poisson random variables", Insurance: Mathematics
 *             and Economics 12, 1993) for lam >= 10.
 *   normal    Marsaglia polar method.
 *   gamma     Marsaglia & Tsang (ACM TOMS 26(3), 2000) for shape >= 1,
 *             boosted by U^(1/a) for shape < 1.
 *   neg. binomial  Poisson(Gamma(r, (1-p)/p)) — the gamma–Poisson mixture
 *             numpy's negative_binomial uses.
 * Rejection loops are bounded; the bound is never reached in practice and a
 * deterministic fallback keeps both sides identical if it were.
 */
#ifndef LPG_RNG_H
#define LPG_RNG_H

#include "lpg_detmath.h"

/* Purposes: the first counter word's high half. */
enum {
  LPG_P_PARALYSIS = 1,  /* a = slot                       */
  LPG_P_RI = 2,         /* a = slot, k=0 OPV, k=1 IPV     */
  LPG_P_SIA = 3,        /* a = slot, k = event of the day */
  LPG_P_BIRTH = 4,      /* a = node                       */
  LPG_P_KM = 5,         /* a = slot, k = 0,1,...          */
  LPG_P_TXCOUNT = 6,    /* a = node, k = 0,1,...          */
  LPG_P_SELECT = 7,     /* a = node, b = round, k = draw  */
  LPG_P_STRAIN = 8,     /* a = slot                       */
  LPG_P_SEEDPICK = 9,   /* a = slot, b = seed event       */
  LPG_P_SEEDTIMER = 10, /* a = slot, b = seed event, k    */
  /* initialisation (tick 0) */
  LPG_P_INIT_MISSED = 11,  /* a = slot: selection key          */
  LPG_P_INIT_IMMUNE = 12,  /* a = slot: selection key          */
  LPG_P_INIT_PREV = 13,    /* a = slot: selection key          */
  LPG_P_INIT_TIMER = 14,   /* a = slot, b = 0 exposure, 1 infection, 2 paralysis */
  LPG_P_INIT_HET = 15,     /* a = slot: two normals            */
  LPG_P_INIT_AGE = 16,     /* a = slot: age bin, day           */
  LPG_P_INIT_KM = 17,      /* a = slot: year, day of death     */
  LPG_P_INIT_RI = 18,      /* a = slot: day of RI              */
  LPG_P_INIT_MEANINF = 19  /* the 1000 infectious durations whose mean scales infectivity */
};

#define LPG_PHILOX_M0 0xD2E7470EE14C6C93ULL
#define LPG_PHILOX_M1 0xCA5A826395121157ULL
#define LPG_PHILOX_W0 0x9E3779B97F4A7C15ULL
#define LPG_PHILOX_W1 0xBB67AE8584CAA73BULL
/* Second key word: a fixed tag so that streams of this project do not
 * coincide with a plain Philox(seed) stream. */
#define LPG_KEY_TAG 0x6C617365722D706FULL

LPG_HD uint64_t lpg_mulhilo64(uint64_t a, uint64_t b, uint64_t* hi) {
#if defined(__CUDA_ARCH__)
  *hi = __umul64hi(a, b);
  return a * b;
#else
  unsigned __int128 p = (unsigned __int128)a * (unsigned __int128)b;
  *hi = (uint64_t)(p >> 64);
  return (uint64_t)p;
#endif
}

/* Philox4x64 with 10 rounds; ctr is replaced by the output block. */
LPG_HD void lpg_philox4x64_10(uint64_t ctr[4], uint64_t k0, uint64_t k1) {
  uint64_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    uint64_t hi0, hi1;
    uint64_t lo0 = lpg_mulhilo64(LPG_PHILOX_M0, c0, &hi0);
    uint64_t lo1 = lpg_mulhilo64(LPG_PHILOX_M1, c2, &hi1);
    uint64_t n0 = hi1 ^ c1 ^ k0;
    uint64_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += LPG_PHILOX_W0;
    k1 += LPG_PHILOX_W1;
  }
  ctr[0] = c0;
  ctr[1] = c1;
  ctr[2] = c2;
  ctr[3] = c3;
}

/* Raw 64-bit word k of stream (seed, purpose, tick, a, b). */
LPG_HD uint64_t lpg_raw(uint64_t seed, uint32_t purpose, int32_t tick, uint64_t a, uint64_t b, uint64_t k) {
  uint64_t c[4];
  c[0] = a;
  c[1] = b;
  c[2] = ((uint64_t)purpose << 32) | (uint64_t)(uint32_t)tick;
  c[3] = k >> 2;
  lpg_philox4x64_10(c, seed, LPG_KEY_TAG);
  /* word k mod 4 of the block, chosen without indexing the array (an
   * indexed register array would live in local memory on the GPU) */
  const unsigned w = (unsigned)(k & 3);
  return w == 0 ? c[0] : w == 1 ? c[1] : w == 2 ? c[2] : c[3];
}

/* 53-bit integer and the matching uniform on [0, 1). */
LPG_HD uint64_t lpg_u53(uint64_t seed, uint32_t purpose, int32_t tick, uint64_t a, uint64_t b, uint64_t k) {
  return lpg_raw(seed, purpose, tick, a, b, k) >> 11;
}

LPG_HD double lpg_u01(uint64_t seed, uint32_t purpose, int32_t tick, uint64_t a, uint64_t b, uint64_t k) {
  return (double)lpg_u53(seed, purpose, tick, a, b, k) * 0x1.0p-53;
}

/* floor(m * T / 2^53) for a 53-bit m: the CDF target of a uniform draw
 * scaled to an integer total weight T (exact, 128-bit product). */
LPG_HD uint64_t lpg_scale_target(uint64_t m53, uint64_t total) {
  uint64_t hi;
  uint64_t lo = lpg_mulhilo64(m53, total, &hi);
  return (hi << 11) | (lo >> 53);
}

/* A sequential stream: draws k = 0, 1, 2, ... of one (purpose, tick, a, b). */
typedef struct {
  uint64_t seed, a, b;
  uint32_t purpose;
  int32_t tick;
  uint64_t k;
  uint64_t blk[4];
  uint64_t blk_id;
  uint64_t nxt[4]; /* a block generated ahead (lpg_stream_ahead) */
  uint64_t nxt_id;
} lpg_stream;

LPG_HD void lpg_stream_init(lpg_stream* s, uint64_t seed, uint32_t purpose, int32_t tick, uint64_t a, uint64_t b) {
  s->seed = seed;
  s->purpose = purpose;
  s->tick = tick;
  s->a = a;
  s->b = b;
  s->k = 0;
  s->blk_id = ~(uint64_t)0;
  s->nxt_id = ~(uint64_t)0;
}

LPG_HD void lpg_stream_block(const lpg_stream* s, uint64_t id, uint64_t* out) {
  out[0] = s->a;
  out[1] = s->b;
  out[2] = ((uint64_t)s->purpose << 32) | (uint64_t)(uint32_t)s->tick;
  out[3] = id;
  lpg_philox4x64_10(out, s->seed, LPG_KEY_TAG);
}

/* Blocks 0 and 1 of the stream formed now, before any draw needs them (the
 * draws are the same; on the GPU the integer work then overlaps the
 * double-precision chain that precedes the first draw). */
LPG_HD void lpg_stream_ahead(lpg_stream* s) {
  lpg_stream_block(s, 0, s->blk);
  s->blk_id = 0;
  lpg_stream_block(s, 1, s->nxt);
  s->nxt_id = 1;
}

LPG_HD double lpg_next(lpg_stream* s) {
  uint64_t id = s->k >> 2;
  if (id != s->blk_id) {
    if (id == s->nxt_id) {
      for (int j = 0; j < 4; ++j) s->blk[j] = s->nxt[j];
    } else {
      lpg_stream_block(s, id, s->blk);
    }
    s->blk_id = id;
  }
  uint64_t w = s->blk[s->k & 3];
  s->k += 1;
  return (double)(w >> 11) * 0x1.0p-53;
}

#define LPG_MAX_REJECT 1000

/* Standard normal, Marsaglia polar method. */
LPG_HD double lpg_std_normal(lpg_stream* s) {
  for (int it = 0; it < LPG_MAX_REJECT; ++it) {
    double u = 2.0 * lpg_next(s) - 1.0;
    double v = 2.0 * lpg_next(s) - 1.0;
    double q = u * u + v * v;
    if (q >= 1.0 || q == 0.0) continue;
    return u * sqrt(-2.0 * lpg_log(q) / q);
  }
  return 0.0;
}

/* Marsaglia–Tsang's constants for shape a >= 1: d = a - 1/3, c = 1/sqrt(9d). */
LPG_HD void lpg_gamma_consts(double a, double* d, double* c) {
  *d = a - 1.0 / 3.0;
  *c = 1.0 / sqrt(9.0 * *d);
}

/* Marsaglia–Tsang's rejection loop with its constants, times boost. */
LPG_HD double lpg_gamma_mt(lpg_stream* s, double d, double c, double boost) {
  for (int it = 0; it < LPG_MAX_REJECT; ++it) {
    double x = lpg_std_normal(s);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    double u = lpg_next(s);
    double x2 = x * x;
    if (u < 1.0 - 0.0331 * (x2 * x2)) return d * v * boost;
    if (lpg_log(u) < 0.5 * x2 + d * (1.0 - v + lpg_log(v))) return d * v * boost;
  }
  return d * boost;
}

/* Gamma(shape a, scale 1). */
LPG_HD double lpg_std_gamma(lpg_stream* s, double a) {
  if (!(a > 0.0)) return 0.0;
  double boost = 1.0;
  if (a < 1.0) {
    double u = lpg_next(s);
    boost = lpg_exp(lpg_log(u) / a);
    a = a + 1.0;
  }
  double d, c;
  lpg_gamma_consts(a, &d, &c);
  return lpg_gamma_mt(s, d, c, boost);
}

/* 1/x for 1 <= x <= 512, correctly rounded (constant expressions), so that
 * the inversions below multiply instead of dividing. */
#define LPG_RECIP_N 512
#define LPG_R8(b) 1.0 / (b + 1.0), 1.0 / (b + 2.0), 1.0 / (b + 3.0), 1.0 / (b + 4.0), \
                  1.0 / (b + 5.0), 1.0 / (b + 6.0), 1.0 / (b + 7.0), 1.0 / (b + 8.0)
#define LPG_R64(b) LPG_R8(b), LPG_R8(b + 8.0), LPG_R8(b + 16.0), LPG_R8(b + 24.0), LPG_R8(b + 32.0), \
                   LPG_R8(b + 40.0), LPG_R8(b + 48.0), LPG_R8(b + 56.0)
#define LPG_R512 LPG_R64(0.0), LPG_R64(64.0), LPG_R64(128.0), LPG_R64(192.0), LPG_R64(256.0), LPG_R64(320.0), \
                 LPG_R64(384.0), LPG_R64(448.0)
#if defined(__CUDACC__)
__constant__ double lpg_recip_tab_dev[LPG_RECIP_N] = {LPG_R512};
#endif
static const double lpg_recip_tab_host[LPG_RECIP_N] = {LPG_R512};
#undef LPG_R8
#undef LPG_R64
#undef LPG_R512
LPG_HD double lpg_recip_small(int64_t x) {
#if defined(__CUDA_ARCH__)
  return lpg_recip_tab_dev[x - 1];
#else
  return lpg_recip_tab_host[x - 1];
#endif
}

/* ln k! for 0 <= k < 256 (the correctly rounded table). */
LPG_HD double lpg_lfact_small(int64_t k) {
#if defined(__CUDA_ARCH__)
  return lpg_tab_lfact_dev[k];
#else
  return lpg_tab_lfact_host[k];
#endif
}

/* Poisson(lam) for 10 <= lam < 200 by inversion from the mode: P(m) for
 * m = floor(lam) from exp(-lam + m ln lam - ln m!), then the outcomes in the
 * order m, m+1, m-1, m+2, m-2, ..., each probability from its neighbour
 * (P(m+j) = P(m+j-1) lam/(m+j), P(m-j) = P(m-j+1) (m-j+1)/lam); the first
 * whose running sum reaches the uniform.  An exact sampler with no
 * rejection: about 0.8 sqrt(lam) steps after one exp and one log. */
LPG_HD int64_t lpg_poisson_mode(lpg_stream* s, double lam) {
  const int64_t m = (int64_t)lam;
  const double pm = lpg_exp((-lam + (double)m * lpg_log(lam)) - lpg_lfact_small(m));
  const double ilam = 1.0 / lam;
  const double u = lpg_next(s);
  double f = pm;
  if (u <= f) return m;
  double ph = pm, pl = pm;
  int64_t hi = m, lo = m;
  for (int it = 0; it < 4 * LPG_RECIP_N; ++it) {
    hi += 1;
    ph = (ph * lam) * (hi <= LPG_RECIP_N ? lpg_recip_small(hi) : 1.0 / (double)hi);
    f = f + ph;
    if (u <= f) return hi;
    if (lo > 0) {
      pl = (pl * (double)lo) * ilam;
      lo -= 1;
      f = f + pl;
      if (u <= f) return lo;
    }
  }
  return m; /* the running sum fell short of u by rounding: the mode */
}

/* Poisson(lam): inversion below 10 (p_x = p_{x-1} * lam * (1/x)),
 * inversion from the mode below 200, PTRS (Hormann's transformed rejection
 * with squeeze) above. */
LPG_HD int64_t lpg_poisson(lpg_stream* s, double lam) {
  if (!(lam > 0.0)) return 0;
  if (lam < 10.0) {
    double p = lpg_exp(-lam);
    double f = p;
    double u = lpg_next(s);
    int64_t x = 0;
    while (u > f && x < 1000) {
      x += 1;
      p = x <= 64 ? (p * lam) * lpg_recip_small(x) : (p * lam) / (double)x;
      f = f + p;
    }
    return x;
  }
  if (lam < 200.0) return lpg_poisson_mode(s, lam);
  double slam = sqrt(lam);
  double loglam = 0.0, logia = 0.0; /* formed on the first squeeze failure */
  int have_logs = 0;
  double b = 0.931 + 2.53 * slam;
  double a = -0.059 + 0.02483 * b;
  double invalpha = 1.1239 + 1.1328 / (b - 3.4);
  double vr = 0.9277 - 3.6224 / (b - 2.0);
  for (int it = 0; it < LPG_MAX_REJECT; ++it) {
    double u = lpg_next(s) - 0.5;
    double v = lpg_next(s);
    double us = 0.5 - fabs(u);
    double kd = floor((2.0 * a / us + b) * u + lam + 0.43);
    if (us >= 0.07 && v <= vr) return (int64_t)kd;
    if (kd < 0.0 || (us < 0.013 && v > us)) continue;
    if (!have_logs) {
      loglam = lpg_log(lam);
      logia = lpg_log(invalpha);
      have_logs = 1;
    }
    double lhs = lpg_log(v) + logia - lpg_log(a / (us * us) + b);
    double rhs = -lam + kd * loglam - lpg_lfact((int64_t)kd);
    if (lhs <= rhs) return (int64_t)kd;
  }
  return (int64_t)floor(lam);
}

/* Negative binomial (number of failures before r successes, success
 * probability p), as the gamma–Poisson mixture. */
LPG_HD int64_t lpg_negbinom(lpg_stream* s, double r, double p) {
  double y = lpg_std_gamma(s, r) * ((1.0 - p) / p);
  return lpg_poisson(s, y);
}

/* The same for r >= 1 with Marsaglia–Tsang's constants of r formed once
 * (lpg_gamma_consts): equal draws, two fewer dependent operations. */
LPG_HD int64_t lpg_negbinom_dc(lpg_stream* s, double d, double c, double p) {
  double y = lpg_gamma_mt(s, d, c, 1.0) * ((1.0 - p) / p);
  return lpg_poisson(s, y);
}

/* Distribution kinds, mirroring laser_polio/distributions.py:17-102. */
enum {
  LPG_DIST_CONSTANT = 0,
  LPG_DIST_EXPONENTIAL = 1,
  LPG_DIST_GAMMA = 2,
  LPG_DIST_LOGNORMAL = 3,   /* p1 = mean, p2 = sigma of the lognormal itself */
  LPG_DIST_NORMAL = 4,
  LPG_DIST_POISSON = 5,
  LPG_DIST_UNIFORM = 6,     /* integer in [p1, p2) */
  LPG_DIST_LOGNORMAL_INT = 7
};

LPG_HD double lpg_dist_sample(lpg_stream* s, int kind, double p1, double p2) {
  switch (kind) {
    case LPG_DIST_CONSTANT:
      return p1;
    case LPG_DIST_EXPONENTIAL:
      return -p1 * lpg_log(1.0 - lpg_next(s));
    case LPG_DIST_GAMMA:
      return lpg_std_gamma(s, p1) * p2;
    case LPG_DIST_LOGNORMAL:
    case LPG_DIST_LOGNORMAL_INT: {
      if (!(p1 > 0.0)) return 0.0;
      double mu = lpg_log(p1 * p1 / sqrt(p2 * p2 + p1 * p1));
      double sg = sqrt(lpg_log(p2 * p2 / (p1 * p1) + 1.0));
      double v = lpg_exp(mu + sg * lpg_std_normal(s));
      if (kind == LPG_DIST_LOGNORMAL_INT) v = floor(v + 0.5);
      return v;
    }
    case LPG_DIST_NORMAL:
      return p1 + p2 * lpg_std_normal(s);
    case LPG_DIST_POISSON:
      return (double)lpg_poisson(s, p1);
    case LPG_DIST_UNIFORM: {
      double span = p2 - p1;
      return p1 + floor(lpg_next(s) * span);
    }
    default:
      return 0.0;
  }
}

/* Store a float draw into an int8 column the way numpy's unsafe cast does
 * on both of this project's hosts: truncate toward zero, keep the low byte. */
LPG_HD int8_t lpg_trunc_i8(double v) {
  if (v != v) return 0;
  if (v > 9.2e18 || v < -9.2e18) return 0;
  int64_t w = (int64_t)v;
  return (int8_t)(uint8_t)(uint64_t)w;
}

#endif /* LPG_RNG_H */
