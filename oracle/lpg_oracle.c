/*
 * lpg_oracle.c — CPU restatement of laser_polio's per-tick agent step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the CUDA engine is
 * compared against (tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline).  The product never links, loads or calls it.
 *
 * It follows the reference loops one for one, in the reference's slot order,
 * with full per-tick sweeps and per-tick recounts exactly as numba runs
 * them (OpenMP for numba's prange, thread-local node buffers reduced after
 * the loop).  Only two things differ from the reference, both by design:
 *   1. Random numbers come from the counter-based draw hook (lpg_rng.h)
 *      instead of numba's per-thread np.random state, so two runs on any
 *      machine or thread count draw the same numbers.
 *   2. Per-node sums that the reference accumulates in float32 thread-local
 *      buffers (model.py:952-954) are exact fixed-point integers here:
 *      acquisition risk in units of 2^-24, infectivity x strain scalar in
 *      units of 2^-40.  The weighted selection CDF (model.py:1108) is the
 *      integer prefix of the same risk units.  Integer sums do not depend
 *      on summation order.
 * Citations are laser_polio/model.py unless stated.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "lpg.h"
#include "lpg_rng.h"
#include "lpg_init.h"

#define NRES 22
enum {
  R_S, R_E, R_I, R_R, R_EBS, R_IBS, R_POTP, R_P, R_NEWPOTP, R_NEWP, R_POP, R_BIRTHS, R_DEATHS,
  R_NEWEXP, R_NEWEXPBS, R_RIVAC, R_RIPROT, R_RINEWEXPBS, R_IPVVAC, R_SIAVAC, R_SIAPROT, R_SIANEWEXPBS
};
static const int res_by_strain[NRES] = {0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 1};

typedef struct {
  lpg_sim_desc d;
  /* owned copies of the descriptor arrays */
  double *birth_rate, *vx_prob_ri, *vx_prob_ipv, *strain_r0_scalars, *network, *r0_scalars, *seasonality;
  float* vx_prob_sia;
  int64_t* km;
  lpg_seed_event* seeds;
  lpg_sia_event* sia;
  uint8_t* sia_masks;
  /* columns */
  int8_t *ds, *strain, *et, *it, *pt, *pp, *par, *ipv;
  uint8_t* cm;
  int16_t *node, *ri;
  float *risk, *inf;
  int32_t *dob, *dod;
  int64_t count;
  int32_t t;
  int32_t stopped;
  int32_t err;
  int32_t started;
  int32_t* res[NRES];
  /* per transmission tick and node: srisk, pop, the expected new exposures,
   * beta before mixing by strain ([nt][n_nodes][3 + ns]), or NULL */
  double* rec;
  /* the same tick's susceptible risk and infectivity sums straight from the
   * float32 columns in FP64, without the fixed-point units the step uses
   * ([nt][n_nodes][1 + ns]; set with rec) */
  double* rec64;
  char msg[256];
} lpo_sim;

static void* xdup(const void* p, size_t n) {
  if (!p || !n) return NULL;
  void* q = malloc(n);
  memcpy(q, p, n);
  return q;
}

static int nthreads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
static int tid(void) {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

/* Fixed-point conversions shared with the engine's definition. */
static inline uint64_t fix_risk(float r) {
  double d = (double)r * 16777216.0; /* 2^24 */
  if (!(d > 0.0)) return 0;
  if (d > 0x1.0p62) d = 0x1.0p62;
  return (uint64_t)nearbyint(d);
}
static inline uint64_t fix_beta(float inf, double scal) {
  double d = ((double)inf * scal) * 0x1.0p40;
  if (!(d > 0.0)) return 0;
  if (d > 0x1.0p62) d = 0x1.0p62;
  return (uint64_t)nearbyint(d);
}

static inline int8_t dec_i8(int8_t v) { return (int8_t)(uint8_t)((uint8_t)v - 1u); }

#define NN (s->d.n_nodes)
#define NS (s->d.n_strains)
#define RES(k, t) (s->res[k] + (size_t)(t) * (size_t)NN * (res_by_strain[k] ? (size_t)NS : 1))

lpo_sim* lpo_create(const lpg_sim_desc* d) {
  lpo_sim* s = (lpo_sim*)calloc(1, sizeof(lpo_sim));
  s->d = *d;
  size_t n = (size_t)d->n_nodes;
  s->birth_rate = xdup(d->birth_rate, n * sizeof(double));
  s->vx_prob_ri = xdup(d->vx_prob_ri, n * sizeof(double));
  s->vx_prob_ipv = xdup(d->vx_prob_ipv, n * sizeof(double));
  s->strain_r0_scalars = xdup(d->strain_r0_scalars, (size_t)d->n_strains * sizeof(double));
  s->network = xdup(d->network, n * n * sizeof(double));
  s->r0_scalars = xdup(d->r0_scalars, n * sizeof(double));
  s->seasonality = xdup(d->seasonality, (size_t)d->nt * sizeof(double));
  s->vx_prob_sia = xdup(d->vx_prob_sia, n * sizeof(float));
  s->km = xdup(d->km_cumdeaths, (size_t)d->km_len * sizeof(int64_t));
  s->seeds = xdup(d->seeds, (size_t)d->n_seeds * sizeof(lpg_seed_event));
  s->sia = xdup(d->sia, (size_t)d->n_sia * sizeof(lpg_sia_event));
  if (d->n_sia) {
    s->sia_masks = (uint8_t*)malloc((size_t)d->n_sia * n);
    for (int e = 0; e < d->n_sia; ++e) {
      memcpy(s->sia_masks + (size_t)e * n, d->sia[e].node_mask, n);
      s->sia[e].node_mask = s->sia_masks + (size_t)e * n;
    }
  }
  size_t cap = (size_t)d->capacity;
  s->ds = calloc(cap, 1);
  s->strain = calloc(cap, 1);
  s->et = calloc(cap, 1);
  s->it = calloc(cap, 1);
  s->pt = calloc(cap, 1);
  s->pp = calloc(cap, 1);
  s->par = calloc(cap, 1);
  s->ipv = calloc(cap, 1);
  s->cm = calloc(cap, 1);
  s->node = calloc(cap, 2);
  s->ri = calloc(cap, 2);
  s->risk = calloc(cap, 4);
  s->inf = calloc(cap, 4);
  s->dob = calloc(cap, 4);
  s->dod = calloc(cap, 4);
  /* reference defaults (model.py:144-162, 571-573, 1201-1206, 1550, 1603, 1891) */
  memset(s->ds, 0xff, cap);
  memset(s->pp, 0xff, cap);
  memset(s->node, 0xff, cap * 2);
  memset(s->ri, 0xff, cap * 2);
  memset(s->dob, 0xff, cap * 4);
  for (size_t i = 0; i < cap; ++i) { s->risk[i] = 1.0f; s->inf[i] = 1.0f; }
  for (int k = 0; k < NRES; ++k)
    s->res[k] = calloc((size_t)d->nt * n * (res_by_strain[k] ? (size_t)d->n_strains : 1), sizeof(int32_t));
  memcpy(s->res[R_POP], d->pop0, n * sizeof(int32_t));
  if (d->R_preseed) memcpy(s->res[R_R], d->R_preseed, (size_t)d->nt * n * sizeof(int32_t));
  s->count = d->count;
  s->t = 0;
  return s;
}

void lpo_destroy(lpo_sim* s) {
  if (!s) return;
  void* ps[] = {s->birth_rate, s->vx_prob_ri, s->vx_prob_ipv, s->strain_r0_scalars, s->network, s->r0_scalars,
                s->seasonality, s->vx_prob_sia, s->km, s->seeds, s->sia, s->sia_masks, s->ds, s->strain, s->et,
                s->it, s->pt, s->pp, s->par, s->ipv, s->cm, s->node, s->ri, s->risk, s->inf, s->dob, s->dod};
  for (size_t i = 0; i < sizeof ps / sizeof ps[0]; ++i) free(ps[i]);
  for (int k = 0; k < NRES; ++k) free(s->res[k]);
  free(s->rec);
  free(s->rec64);
  free(s);
}

#define CPY(dst, src, esz) \
  if (src) memcpy(dst, src, cap * (esz))

int lpo_bind_columns(lpo_sim* s, const lpg_columns* c) {
  size_t cap = (size_t)s->d.capacity;
  CPY(s->ds, c->disease_state, 1);
  CPY(s->strain, c->strain, 1);
  CPY(s->et, c->exposure_timer, 1);
  CPY(s->it, c->infection_timer, 1);
  CPY(s->pt, c->paralysis_timer, 1);
  CPY(s->pp, c->potentially_paralyzed, 1);
  CPY(s->par, c->paralyzed, 1);
  CPY(s->ipv, c->ipv_protected, 1);
  CPY(s->cm, c->chronically_missed, 1);
  CPY(s->node, c->node_id, 2);
  CPY(s->ri, c->ri_timer, 2);
  CPY(s->risk, c->acq_risk_multiplier, 4);
  CPY(s->inf, c->daily_infectivity, 4);
  CPY(s->dob, c->date_of_birth, 4);
  CPY(s->dod, c->date_of_death, 4);
  return 0;
}

int lpo_read_columns(lpo_sim* s, const lpg_columns* c) {
  size_t cap = (size_t)s->count;
#define OUT(dst, src, esz) \
  if (dst) memcpy(dst, src, cap * (esz))
  OUT(c->disease_state, s->ds, 1);
  OUT(c->strain, s->strain, 1);
  OUT(c->exposure_timer, s->et, 1);
  OUT(c->infection_timer, s->it, 1);
  OUT(c->paralysis_timer, s->pt, 1);
  OUT(c->potentially_paralyzed, s->pp, 1);
  OUT(c->paralyzed, s->par, 1);
  OUT(c->ipv_protected, s->ipv, 1);
  OUT(c->chronically_missed, s->cm, 1);
  OUT(c->node_id, s->node, 2);
  OUT(c->ri_timer, s->ri, 2);
  OUT(c->acq_risk_multiplier, s->risk, 4);
  OUT(c->daily_infectivity, s->inf, 4);
  OUT(c->date_of_birth, s->dob, 4);
  OUT(c->date_of_death, s->dod, 4);
#undef OUT
  return 0;
}

int lpo_read_results(lpo_sim* s, const lpg_results_view* v) {
  int32_t* const* outs = (int32_t* const*)v;
  for (int k = 0; k < NRES; ++k) {
    if (!outs[k]) continue;
    memcpy(outs[k], s->res[k], (size_t)s->d.nt * NN * (res_by_strain[k] ? (size_t)NS : 1) * sizeof(int32_t));
  }
  return 0;
}

int lpo_get_state(lpo_sim* s, lpg_sim_state* st) {
  st->t = s->t;
  st->stopped = s->stopped;
  st->count = s->count;
  st->error = s->err;
  return 0;
}

const char* lpo_last_error(lpo_sim* s) { return s->msg; }

/* ---------------------------------------------------------------------- */
/* Kaplan–Meier age at death for a newborn (age 0 days), restating
 * laser_core's KaplanMeierEstimator.predict_age_at_death as called at
 * model.py:1725: the year of death is drawn from the cumulative deaths table
 * (a uniform integer below its last entry, located with searchsorted
 * side='right'), the day uniformly within that year. */
int32_t lpo_km_newborn(const int64_t* cum, int32_t km_len, int32_t max_year, uint64_t seed, int32_t t, uint64_t slot) {
  int32_t top = max_year < km_len - 1 ? max_year : km_len - 1;
  int64_t total = cum[top];
  int32_t y = top;
  if (total > 0) {
    double u0 = lpg_u01(seed, LPG_P_KM, t, slot, 0, 0);
    int64_t draw = (int64_t)floor(u0 * (double)total);
    int32_t lo = 0, hi = top; /* first y with cum[y] > draw */
    while (lo < hi) {
      int32_t mid = (lo + hi) >> 1;
      if (cum[mid] > draw) hi = mid; else lo = mid + 1;
    }
    y = lo;
  }
  double u1 = lpg_u01(seed, LPG_P_KM, t, slot, 0, 1);
  return y * 365 + (int32_t)floor(u1 * 365.0);
}

/* ---------------------------------------------------------------------- */
/* Transmission_ABM.log / count_SEIRP (model.py:869-929, 1461-1487). */
static void lpo_log_tick(lpo_sim* s, int32_t t) {
  int nth = nthreads();
  int n = NN, ns = NS;
  int32_t* tl = calloc((size_t)nth * (size_t)n * (4 + 2 * (size_t)ns), sizeof(int32_t));
  int64_t count = s->count;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < count; ++i) {
    int8_t st = s->ds[i];
    if (st < 0) continue;
    int nd = s->node[i];
    int32_t* b = tl + (size_t)tid() * (size_t)n * (4 + 2 * (size_t)ns);
    int k = s->strain[i];
    if (st == 0) b[nd] += 1;
    else if (st == 1) b[4 * n + nd * ns + k] += 1;
    else if (st == 2) b[4 * n + n * ns + nd * ns + k] += 1;
    else if (st == 3) b[n + nd] += 1;
    if (s->pp[i] == 1) b[2 * n + nd] += 1;
    if (s->par[i] == 1) b[3 * n + nd] += 1;
  }
  int32_t *S = RES(R_S, t), *E = RES(R_E, t), *I = RES(R_I, t), *R = RES(R_R, t), *EB = RES(R_EBS, t),
          *IB = RES(R_IBS, t), *PP = RES(R_POTP, t), *P = RES(R_P, t);
  for (int nd = 0; nd < n; ++nd) {
    int32_t vs = 0, vr = 0, vpp = 0, vp = 0;
    int32_t es = 0, is = 0;
    for (int th = 0; th < nth; ++th) {
      int32_t* b = tl + (size_t)th * (size_t)n * (4 + 2 * (size_t)ns);
      vs += b[nd];
      vr += b[n + nd];
      vpp += b[2 * n + nd];
      vp += b[3 * n + nd];
    }
    for (int k = 0; k < ns; ++k) {
      int32_t e = 0, i = 0;
      for (int th = 0; th < nth; ++th) {
        int32_t* b = tl + (size_t)th * (size_t)n * (4 + 2 * (size_t)ns);
        e += b[4 * n + nd * ns + k];
        i += b[4 * n + n * ns + nd * ns + k];
      }
      EB[nd * ns + k] = e;
      IB[nd * ns + k] = i;
      es += e;
      is += i;
    }
    S[nd] = vs;
    E[nd] = es;
    I[nd] = is;
    R[nd] += vr;
    PP[nd] = vpp;
    P[nd] = vp;
  }
  free(tl);
}

/* ---------------------------------------------------------------------- */
/* VitalDynamics_ABM.step (model.py:1689-1757) and get_deaths (:1767-1781). */
static int lpo_vd(lpo_sim* s, int32_t t) {
  int n = NN;
  int32_t* pop = RES(R_POP, t);
  int32_t* pop1 = RES(R_POP, t - 1);
  if (t % s->d.vd_step != 0) {
    memcpy(pop, pop1, (size_t)n * sizeof(int32_t));
    return 0;
  }
  int nth = nthreads();
  int32_t* tl = calloc((size_t)nth * n, sizeof(int32_t));
  int64_t count = s->count;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < count; ++i) {
    if (s->ds[i] >= 0 && s->dod[i] <= t) {
      s->ds[i] = -1;
      tl[(size_t)tid() * n + s->node[i]] += 1;
    }
  }
  int32_t* deaths = RES(R_DEATHS, t);
  for (int nd = 0; nd < n; ++nd) {
    int32_t v = 0;
    for (int th = 0; th < nth; ++th) v += tl[(size_t)th * n + nd];
    deaths[nd] = v;
  }
  free(tl);
  /* births: integer part plus a Bernoulli draw on the fraction (:1712-1716) */
  int64_t total = 0;
  int32_t* births = RES(R_BIRTHS, t);
  int32_t* b = malloc((size_t)n * sizeof(int32_t));
  for (int nd = 0; nd < n; ++nd) {
    double expected = ((double)s->d.vd_step * s->birth_rate[nd]) * (double)pop1[nd];
    int32_t bi = (int32_t)expected;
    double frac = expected - (double)bi;
    double u = lpg_u01(s->d.seed, LPG_P_BIRTH, t, (uint64_t)nd, 0, 0);
    b[nd] = bi + (u < frac ? 1 : 0);
    total += b[nd];
  }
  if (total > 0) {
    if (s->count + total > s->d.capacity) {
      snprintf(s->msg, sizeof s->msg, "births at tick %d need %lld slots beyond capacity %lld", t,
               (long long)(s->count + total - s->d.capacity), (long long)s->d.capacity);
      free(b);
      return LPG_ERR_CAPACITY;
    }
    int64_t slot = s->count;
    for (int nd = 0; nd < n; ++nd) {
      for (int32_t j = 0; j < b[nd]; ++j, ++slot) {
        s->dob[slot] = t;
        s->dod[slot] = t + lpo_km_newborn(s->km, s->d.km_len, s->d.km_max_year, s->d.seed, t, (uint64_t)slot);
        s->ds[slot] = 0;
        s->node[slot] = (int16_t)nd;
      }
    }
    s->count += total;
    memcpy(births, b, (size_t)n * sizeof(int32_t));
  }
  free(b);
  for (int nd = 0; nd < n; ++nd) pop[nd] = pop1[nd] + births[nd] - deaths[nd];
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Seed schedule of DiseaseState_ABM.step (model.py:759-786).  The uniform
 * subset (np.random.choice without replacement) is restated as: the n
 * candidates with the smallest counter-based keys, ties broken by slot. */
typedef struct {
  uint64_t key;
  int64_t slot;
} keyslot;
static int cmp_keyslot(const void* a, const void* b) {
  const keyslot* x = a;
  const keyslot* y = b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->slot < y->slot ? -1 : (x->slot > y->slot);
}

static void lpo_seed(lpo_sim* s, int32_t t) {
  for (int e = 0; e < s->d.n_seeds; ++e) {
    const lpg_seed_event* ev = &s->seeds[e];
    if (ev->tick != t) continue;
    int64_t nc = 0;
    for (int64_t i = 0; i < s->count; ++i)
      if (s->node[i] == ev->node && s->ds[i] >= 0) ++nc;
    int64_t nseed = ev->is_count ? (int64_t)ev->value : (int64_t)((double)nc * ev->value);
    if (ev->is_count && nseed > nc) nseed = nc;
    if (nseed <= 0) continue;
    keyslot* ks = malloc((size_t)nc * sizeof(keyslot));
    int64_t m = 0;
    for (int64_t i = 0; i < s->count; ++i)
      if (s->node[i] == ev->node && s->ds[i] >= 0) {
        ks[m].key = lpg_raw(s->d.seed, LPG_P_SEEDPICK, t, (uint64_t)i, (uint64_t)e, 0);
        ks[m].slot = i;
        ++m;
      }
    qsort(ks, (size_t)nc, sizeof(keyslot), cmp_keyslot);
    for (int64_t j = 0; j < nseed; ++j) {
      int64_t i = ks[j].slot;
      s->ds[i] = 2;
      if (s->it[i] <= 0) {
        lpg_stream st;
        lpg_stream_init(&st, s->d.seed, LPG_P_SEEDTIMER, t, (uint64_t)i, (uint64_t)e);
        s->it[i] = lpg_trunc_i8(lpg_dist_sample(&st, s->d.dur_inf.kind, s->d.dur_inf.p1, s->d.dur_inf.p2));
      }
    }
    free(ks);
  }
}

/* DiseaseState_ABM.step (model.py:715-795) with the kernel of :393-454. */
static void lpo_ds(lpo_sim* s, int32_t t) {
  int n = NN;
  int nth = nthreads();
  int32_t* tl = calloc((size_t)nth * 2 * n, sizeof(int32_t));
  int64_t count = s->count;
  double ppar = (double)s->d.p_paralysis;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < count; ++i) {
    int nid = s->node[i];
    if (s->ds[i] == 1) {
      if (s->et[i] <= 0) s->ds[i] = 2;
      s->et[i] = dec_i8(s->et[i]);
    }
    if (s->ds[i] == 2) {
      if (s->it[i] <= 0) s->ds[i] = 3;
      s->it[i] = dec_i8(s->it[i]);
      if (s->strain[i] == 0) {
        if (s->pt[i] <= 0 && s->pp[i] == -1) {
          if (s->ipv[i] == 0) {
            s->pp[i] = 1;
            tl[(size_t)tid() * 2 * n + nid] += 1;
            if (lpg_u01(s->d.seed, LPG_P_PARALYSIS, t, (uint64_t)i, 0, 0) < ppar) {
              s->par[i] = 1;
              tl[(size_t)tid() * 2 * n + n + nid] += 1;
            }
          } else {
            s->pp[i] = 0;
          }
        }
        s->pt[i] = dec_i8(s->pt[i]);
      }
    }
  }
  int32_t *np_ = RES(R_NEWPOTP, t), *npar = RES(R_NEWP, t);
  for (int nd = 0; nd < n; ++nd) {
    int32_t a = 0, b = 0;
    for (int th = 0; th < nth; ++th) {
      a += tl[(size_t)th * 2 * n + nd];
      b += tl[(size_t)th * 2 * n + n + nd];
    }
    np_[nd] = a;
    npar[nd] = b;
  }
  free(tl);
  lpo_seed(s, t);
  if (s->d.stop_if_no_cases) {
    int64_t e = 0, in = 0;
    int32_t *E = RES(R_E, t - 1), *I = RES(R_I, t - 1);
    for (int nd = 0; nd < n; ++nd) {
      e += E[nd];
      in += I[nd];
    }
    int future = 0;
    for (int k = 0; k < s->d.n_seeds; ++k)
      if (s->seeds[k].tick > t) future = 1;
    if (!(e > 0 || in > 0 || future)) s->stopped = 1;
  }
}

/* ---------------------------------------------------------------------- */
/* RI_ABM.step (model.py:1920-1985) with fast_ri (:1784-1855). */
static void lpo_ri(lpo_sim* s, int32_t t) {
  if (!s->d.ri_enabled) return;
  if (t % s->d.ri_step != 0) return;
  int n = NN, ns = NS;
  int nth = nthreads();
  int32_t* tl = calloc((size_t)nth * 3 * n, sizeof(int32_t));
  int64_t count = s->count;
  int32_t step = s->d.ri_step;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < count; ++i) {
    int8_t state = s->ds[i];
    if (state < 0) continue;
    if (s->cm[i] == 1) continue;
    int node = s->node[i];
    int32_t timer = (int32_t)s->ri[i] - step;
    s->ri[i] = (int16_t)(uint16_t)(uint32_t)timer;
    int eligible = 0;
    if (t == step) eligible = timer <= 0 && timer >= -step;
    else if (t > step) eligible = timer <= 0 && timer > -step;
    if (eligible) {
      int32_t* b = tl + (size_t)tid() * 3 * n;
      if (lpg_u01(s->d.seed, LPG_P_RI, t, (uint64_t)i, 0, 0) < s->vx_prob_ri[node]) {
        b[node] += 1;
        if (state == 0) {
          s->ds[i] = 1;
          s->strain[i] = (int8_t)s->d.ri_strain;
          b[n + node] += 1;
        }
      }
      if (lpg_u01(s->d.seed, LPG_P_RI, t, (uint64_t)i, 0, 1) < s->vx_prob_ipv[node]) {
        b[2 * n + node] += 1;
        s->ipv[i] = 1;
      }
    }
  }
  int32_t *vac = RES(R_RIVAC, t), *prot = RES(R_RIPROT, t), *ne = RES(R_NEWEXP, t), *nebs = RES(R_NEWEXPBS, t),
          *rinebs = RES(R_RINEWEXPBS, t), *ipv = RES(R_IPVVAC, t);
  for (int nd = 0; nd < n; ++nd) {
    int32_t a = 0, b = 0, c = 0;
    for (int th = 0; th < nth; ++th) {
      a += tl[(size_t)th * 3 * n + nd];
      b += tl[(size_t)th * 3 * n + n + nd];
      c += tl[(size_t)th * 3 * n + 2 * n + nd];
    }
    vac[nd] = a;
    prot[nd] = b;
    ne[nd] += b;
    nebs[nd * ns + s->d.ri_strain] += b;
    rinebs[nd * ns + s->d.ri_strain] = b;
    ipv[nd] = c;
  }
  free(tl);
}

/* ---------------------------------------------------------------------- */
/* SIA_ABM.step (model.py:2099-2156) with fast_sia (:1994-2060). */
static void lpo_sia(lpo_sim* s, int32_t t) {
  int n = NN, ns = NS;
  int nth = nthreads();
  int k_of_day = 0;
  for (int e = 0; e < s->d.n_sia; ++e) {
    const lpg_sia_event* ev = &s->sia[e];
    if (ev->tick != t) continue;
    int kd = k_of_day++;
    int32_t* tl = calloc((size_t)nth * 2 * n, sizeof(int32_t));
    int64_t count = s->count;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < count; ++i) {
      if (s->ds[i] < 0) continue;
      if (s->cm[i] == 1) continue;
      int64_t age = (int64_t)t - (int64_t)s->dob[i];
      if (!(ev->min_age <= age && age <= ev->max_age)) continue;
      int node = s->node[i];
      if (ev->node_mask[node] == 0) continue;
      double r = lpg_u01(s->d.seed, LPG_P_SIA, t, (uint64_t)i, 0, (uint64_t)kd);
      double p = (double)s->vx_prob_sia[node];
      if (r < p) {
        int32_t* b = tl + (size_t)tid() * 2 * n;
        b[node] += 1;
        if (s->ds[i] == 0) {
          if (r < p * ev->efficacy) {
            s->ds[i] = 1;
            s->strain[i] = (int8_t)ev->strain;
            b[n + node] += 1;
          }
        }
      }
    }
    int32_t *vac = RES(R_SIAVAC, t), *prot = RES(R_SIAPROT, t), *ne = RES(R_NEWEXP, t),
            *nebs = RES(R_NEWEXPBS, t), *snebs = RES(R_SIANEWEXPBS, t);
    for (int nd = 0; nd < n; ++nd) {
      int32_t a = 0, b = 0;
      for (int th = 0; th < nth; ++th) {
        a += tl[(size_t)th * 2 * n + nd];
        b += tl[(size_t)th * 2 * n + n + nd];
      }
      vac[nd] = a;
      prot[nd] = b;
      ne[nd] += b;
      nebs[nd * ns + ev->strain] += b;
      snebs[nd * ns + ev->strain] += b;
    }
    free(tl);
  }
}

/* ---------------------------------------------------------------------- */
/* Three-word accumulator: a += x*y (128-bit product). */
static inline void lpo_acc3_mul(uint64_t a[3], uint64_t x, uint64_t y) {
  unsigned __int128 p = (unsigned __int128)x * y;
  unsigned __int128 lo = ((unsigned __int128)a[1] << 64) | a[0];
  unsigned __int128 sum = lo + p;
  if (sum < lo) a[2] += 1;
  a[0] = (uint64_t)sum;
  a[1] = (uint64_t)(sum >> 64);
}

/* Node-level force of infection and exposure counts
 * (model.py:1327-1407), restated in the order the engine evaluates it. */
void lpo_node_tx(int n, int ns, const uint64_t* B, const uint64_t* SW, const int32_t* Scount, const double* net,
                 const double* r0s, double seas, const int32_t* pop, int use_pop, double zi, int32_t nb_r,
                 uint64_t seed, int32_t t, double* prob_out, int64_t* size_out, double* rec_t) {
  for (int nd = 0; nd < n; ++nd) {
    double p[LPG_MAX_STRAINS];
    double total_p = 0.0;
    int local_zero = 1;
    for (int k = 0; k < ns; ++k) {
      if (B[(size_t)nd * ns + k] != 0) local_zero = 0;
      /* incoming infectivity sum_i beta_i N[i][nd], exact: B (units 2^-40)
       * times the network weight in its two fixed-point parts
       * (lpg_net_split), each product summed in three words, converted once
       * (lpg_mix_value) */
      uint64_t A[3] = {0, 0, 0}, Rr[3] = {0, 0, 0};
      for (int i = 0; i < n; ++i) {
        uint64_t whi, wlo;
        lpg_net_split(net[(size_t)i * n + nd], &whi, &wlo);
        lpo_acc3_mul(A, B[(size_t)i * ns + k], whi);
        lpo_acc3_mul(Rr, B[(size_t)i * ns + k], wlo);
      }
      double inc = lpg_mix_value(A[0], A[1], A[2], Rr[0], Rr[1], Rr[2]);
      double rowsum = 0.0;
      for (int j = 0; j < n; ++j) rowsum = rowsum + net[(size_t)nd * n + j];
      double bpre = (double)B[(size_t)nd * ns + k] * 0x1.0p-40;
      double beta = bpre + (inc - bpre * rowsum);
      beta = (beta * seas) * r0s[nd];
      double denom = use_pop ? (double)(pop[nd] > 1 ? pop[nd] : 1) : 1.0;
      double rate = beta / denom;
      double pk = -lpg_expm1(-rate);
      if (!(pk > 0.0)) pk = 0.0;
      p[k] = pk;
      total_p = total_p + pk;
    }
    for (int k = 0; k < ns; ++k) prob_out[(size_t)nd * ns + k] = p[k];
    double srisk = (double)SW[nd] * 0x1.0p-24;
    double exposure = srisk * total_p;
    if (rec_t) { /* the inputs of the expected-incidence map, and its value */
      double* rr = rec_t + (size_t)nd * (3 + ns);
      rr[0] = srisk;
      rr[1] = (double)pop[nd];
      rr[2] = exposure;
      for (int k = 0; k < ns; ++k) rr[3 + k] = (double)B[(size_t)nd * ns + k] * 0x1.0p-40;
    }
    int64_t total = 0;
    lpg_stream st;
    lpg_stream_init(&st, seed, LPG_P_TXCOUNT, t, (uint64_t)nd, 0);
    if (!(exposure > 0.0)) {
      total = 0;
    } else if (local_zero) {
      if (zi >= 1.0) {
        total = 0;
      } else {
        double mean = exposure / (1.0 - zi);
        double r = (double)nb_r;
        double pp = r / (r + mean);
        double u = lpg_next(&st);
        total = (u < zi) ? 0 : lpg_negbinom(&st, r, pp);
      }
    } else {
      total = lpg_poisson(&st, exposure);
    }
    size_out[nd] = total < (int64_t)Scount[nd] ? total : (int64_t)Scount[nd];
  }
}

/* Strain of a newly exposed agent (model.py:1127-1145). */
static inline int pick_strain(const double* p, int ns, double total_p, double r) {
  double cum = 0.0;
  for (int k = 0; k < ns; ++k) {
    cum = cum + p[k] / total_p;
    if (r < cum) return k;
  }
  return 0;
}

/* Transmission_ABM.step (model.py:1281-1459): tx_step_prep, mixing, draws,
 * tx_infect_nb (:1010-1149). */
static void lpo_tx(lpo_sim* s, int32_t t) {
  int n = NN, ns = NS;
  int nth = nthreads();
  int64_t count = s->count;
  size_t per = (size_t)n * (2 + (size_t)ns);
  uint64_t* tl = calloc((size_t)nth * per, sizeof(uint64_t));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < count; ++i) {
    int8_t st = s->ds[i];
    int nid = s->node[i];
    uint64_t* b = tl + (size_t)tid() * per;
    if (st == 0) {
      b[nid] += fix_risk(s->risk[i]);
      b[n + nid] += 1;
    } else if (st == 2) {
      int k = s->strain[i];
      b[2 * n + (size_t)nid * ns + k] += fix_beta(s->inf[i], s->strain_r0_scalars[k]);
    }
  }
  uint64_t* SW = calloc((size_t)n, sizeof(uint64_t));
  int32_t* Sc = calloc((size_t)n, sizeof(int32_t));
  uint64_t* B = calloc((size_t)n * ns, sizeof(uint64_t));
  for (int th = 0; th < nth; ++th) {
    uint64_t* b = tl + (size_t)th * per;
    for (int nd = 0; nd < n; ++nd) {
      SW[nd] += b[nd];
      Sc[nd] += (int32_t)b[n + nd];
      for (int k = 0; k < ns; ++k) B[(size_t)nd * ns + k] += b[2 * n + (size_t)nd * ns + k];
    }
  }
  free(tl);
  double* prob = calloc((size_t)n * ns, sizeof(double));
  int64_t* size = calloc((size_t)n, sizeof(int64_t));
  int use_pop = 1;
  lpo_node_tx(n, ns, B, SW, Sc, s->network, s->r0_scalars, s->seasonality[t], RES(R_POP, t), use_pop,
              s->d.zero_inflation, s->d.nb_r, s->d.seed, t, prob, size,
              s->rec ? s->rec + (size_t)t * n * (3 + ns) : NULL);
  if (s->rec64) { /* FP64 sums of the unquantised columns (a check of the fixed-point units) */
    double* r64 = s->rec64 + (size_t)t * n * (1 + ns);
    for (int64_t i = 0; i < count; ++i) {
      int8_t st = s->ds[i];
      double* rr = r64 + (size_t)s->node[i] * (1 + ns);
      if (st == 0) rr[0] += (double)s->risk[i];
      else if (st == 2) rr[1 + s->strain[i]] += (double)s->inf[i] * s->strain_r0_scalars[s->strain[i]];
    }
  }

  /* serial gather of susceptible slots per node, index order (:1055-1061) */
  int64_t* off = calloc((size_t)n + 1, sizeof(int64_t));
  for (int nd = 0; nd < n; ++nd) off[nd + 1] = off[nd] + (size[nd] > 0 ? Sc[nd] : 0);
  int64_t* nxt = malloc((size_t)n * sizeof(int64_t));
  memcpy(nxt, off, (size_t)n * sizeof(int64_t));
  int64_t* sus = malloc((size_t)(off[n] > 0 ? off[n] : 1) * sizeof(int64_t));
  for (int64_t i = 0; i < count; ++i) {
    int nid = s->node[i];
    if (size[nid] > 0 && s->ds[i] == 0) sus[nxt[nid]++] = i;
  }
  int32_t* newexp = calloc((size_t)n * ns, sizeof(int32_t));
#pragma omp parallel for schedule(dynamic, 1)
  for (int nd = 0; nd < n; ++nd) {
    int64_t want = size[nd];
    if (want <= 0) continue;
    int64_t m = off[nd + 1] - off[nd];
    const int64_t* idx = sus + off[nd];
    uint64_t* w = malloc((size_t)m * sizeof(uint64_t));
    uint64_t* cdf = malloc((size_t)m * sizeof(uint64_t));
    uint8_t* hit = calloc((size_t)m, 1);
    for (int64_t j = 0; j < m; ++j) w[j] = fix_risk(s->risk[idx[j]]);
    int64_t uniq = 0;
    uint64_t round = 0;
    while (uniq < want) {
      uint64_t acc = 0;
      for (int64_t j = 0; j < m; ++j) {
        acc += w[j];
        cdf[j] = acc;
      }
      if (acc == 0) break;
      int64_t k = want - uniq;
      int64_t got = 0;
      for (int64_t q = 0; q < k; ++q) {
        uint64_t v = lpg_scale_target(lpg_u53(s->d.seed, LPG_P_SELECT, t, (uint64_t)nd, round, (uint64_t)q), acc);
        int64_t lo = 0, hi = m - 1; /* first j with cdf[j] > v */
        while (lo < hi) {
          int64_t mid = (lo + hi) >> 1;
          if (cdf[mid] > v) hi = mid; else lo = mid + 1;
        }
        if (hit[lo] == 0) {
          hit[lo] = 2; /* picked in this round */
          ++got;
        }
      }
      for (int64_t j = 0; j < m; ++j)
        if (hit[j] == 2) {
          hit[j] = 1;
          w[j] = 0;
        }
      uniq += got;
      ++round;
    }
    double totalp = 0.0;
    for (int k = 0; k < ns; ++k) totalp = totalp + prob[(size_t)nd * ns + k];
    for (int64_t j = 0; j < m; ++j) {
      if (!hit[j]) continue;
      int64_t i = idx[j];
      double r = lpg_u01(s->d.seed, LPG_P_STRAIN, t, (uint64_t)i, 0, 0);
      int k = pick_strain(prob + (size_t)nd * ns, ns, totalp, r);
      s->ds[i] = 1;
      s->strain[i] = (int8_t)k;
      newexp[(size_t)nd * ns + k] += 1;
    }
    free(w);
    free(cdf);
    free(hit);
  }
  int32_t *ne = RES(R_NEWEXP, t), *nebs = RES(R_NEWEXPBS, t);
  for (int nd = 0; nd < n; ++nd) {
    int32_t tot = 0;
    for (int k = 0; k < ns; ++k) {
      nebs[(size_t)nd * ns + k] += newexp[(size_t)nd * ns + k];
      tot += newexp[(size_t)nd * ns + k];
    }
    ne[nd] += tot;
  }
  free(newexp);
  free(sus);
  free(nxt);
  free(off);
  free(prob);
  free(size);
  free(SW);
  free(Sc);
  free(B);
}

/* ---------------------------------------------------------------------- */
int lpo_start(lpo_sim* s) {
  if (s->started) return 0;
  s->started = 1;
  if (s->d.components & LPG_COMP_TX) lpo_log_tick(s, 0);
  s->t = 1;
  return 0;
}

/* One tick of SEIR_ABM.run (model.py:257-271). */
static int lpo_tick(lpo_sim* s) {
  int32_t t = s->t;
  uint32_t c = s->d.components;
  int rc = 0;
  if (c & LPG_COMP_VD) {
    rc = lpo_vd(s, t);
    if (rc) return rc;
  }
  if (c & LPG_COMP_DS) lpo_ds(s, t);
  if (c & LPG_COMP_RI) lpo_ri(s, t);
  if (c & LPG_COMP_SIA) lpo_sia(s, t);
  if (c & LPG_COMP_TX) {
    lpo_tx(s, t);
    lpo_log_tick(s, t);
  }
  s->t = t + 1;
  return 0;
}

int lpo_step(lpo_sim* s, int32_t n_ticks) {
  if (!s->started) lpo_start(s);
  for (int32_t k = 0; k < n_ticks; ++k) {
    if (s->t >= s->d.nt || s->stopped || s->err) break;
    int rc = lpo_tick(s);
    if (rc) {
      s->err = rc;
      return rc;
    }
  }
  return 0;
}

int lpo_num_threads(void) { return nthreads(); }

/* Record the expected-incidence map's inputs on every transmission tick
 * (the engine's lpg_record_aggregates); before lpo_start. */
int lpo_record_aggregates(lpo_sim* s, int enable) {
  if (s->started) return LPG_ERR_STATE;
  free(s->rec);
  free(s->rec64);
  s->rec = enable ? calloc((size_t)s->d.nt * NN * (3 + NS), sizeof(double)) : NULL;
  s->rec64 = enable ? calloc((size_t)s->d.nt * NN * (1 + NS), sizeof(double)) : NULL;
  return 0;
}

/* lpg_read_aggregates' layout: srisk, pop, lam [nt][n] and beta [nt][n][ns]. */
int lpo_read_aggregates(lpo_sim* s, double* srisk, double* beta, double* pop, double* lam) {
  if (!s->rec) return LPG_ERR_STATE;
  const int w = 3 + NS;
  const size_t rows = (size_t)s->d.nt * NN;
  for (size_t q = 0; q < rows; ++q) {
    const double* b = s->rec + q * w;
    if (srisk) srisk[q] = b[0];
    if (pop) pop[q] = b[1];
    if (lam) lam[q] = b[2];
    if (beta)
      for (int k = 0; k < NS; ++k) beta[q * NS + k] = b[3 + k];
  }
  return 0;
}

/* The FP64 sums recorded beside the aggregates: srisk [nt][n] and beta
 * [nt][n][ns] from the float32 columns without fixed-point units. */
int lpo_read_aggregates_fp64(lpo_sim* s, double* srisk, double* beta) {
  if (!s->rec64) return LPG_ERR_STATE;
  const int w = 1 + NS;
  const size_t rows = (size_t)s->d.nt * NN;
  for (size_t q = 0; q < rows; ++q) {
    const double* b = s->rec64 + q * w;
    if (srisk) srisk[q] = b[0];
    if (beta)
      for (int k = 0; k < NS; ++k) beta[q * NS + k] = b[1 + k];
  }
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Initialisation (the engine's lpg_init_columns), restated for host columns:
 * the per-slot parts with the arithmetic of lpg_init.h (each citing the
 * reference lines it follows), the choices without replacement by sorting
 * each group's (key, slot) pairs and taking the k smallest, which is the
 * set the engine's radix select finds. */
static void lpo_select(uint64_t seed, uint32_t purpose, const int64_t* start, int G, const int64_t* k, int action,
                       const lpg_columns* c) {
  for (int g = 0; g < G; ++g) {
    const int64_t s0 = start[g], n = start[g + 1] - start[g];
    const int64_t kk = k[g];
    if (kk <= 0 || n <= 0) continue;
    keyslot* ks = malloc((size_t)n * sizeof(keyslot));
    for (int64_t j = 0; j < n; ++j) {
      ks[j].key = lpg_raw(seed, purpose, 0, (uint64_t)(s0 + j), 0, 0);
      ks[j].slot = s0 + j;
    }
    if (kk < n) qsort(ks, (size_t)n, sizeof(keyslot), cmp_keyslot);
    const int64_t take = kk < n ? kk : n;
    for (int64_t j = 0; j < take; ++j) {
      const int64_t i = ks[j].slot;
      if (action == 0) c->chronically_missed[i] = 1;
      else if (action == 1) c->disease_state[i] = 3;
      else c->disease_state[i] = 2;
    }
    free(ks);
  }
}

double lpo_init_mean_infectivity(uint64_t seed, double r0, lpg_dist dur_inf) {
  lpg_stream st;
  lpg_stream_init(&st, seed, LPG_P_INIT_MEANINF, 0, 0, 0);
  double sum = 0.0;
  for (int j = 0; j < 1000; ++j) sum = sum + lpg_dist_sample(&st, dur_inf.kind, dur_inf.p1, dur_inf.p2);
  return r0 / (sum / 1000.0);
}

int lpo_init_columns(const lpg_init_desc* d, uint32_t parts, const lpg_columns* c) {
  const int n = d->n_nodes;
  int64_t* start = malloc(((size_t)n + 1) * sizeof(int64_t));
  start[0] = 0;
  for (int i = 0; i < n; ++i) start[i + 1] = start[i] + d->node_pop[i];
  if (start[n] != d->count) {
    free(start);
    return LPG_ERR_ARG;
  }
  double mu = 0, sigma = 0, rho = 0, srho = 0, scale = 0;
  if (parts & LPG_INIT_HETEROGENEITY) { /* model.py:839-851 */
    const double var = d->risk_mult_var;
    mu = log(1.0 / sqrt(var + 1.0));
    sigma = sqrt(log(var + 1.0));
    rho = 2.0 * sin(LPG_PI * d->corr_risk_inf / 6.0);
    srho = sqrt(1.0 - rho * rho);
    const double mean = lpo_init_mean_infectivity(d->seed, d->r0, d->dur_inf);
    scale = mean > 1e-10 ? mean : 1e-10;
  }
  int64_t* cum = NULL;
  if (parts & LPG_INIT_AGES) {
    cum = malloc((size_t)d->n_age_bins * sizeof(int64_t));
    int64_t acc = 0;
    for (int b = 0; b < d->n_age_bins; ++b) cum[b] = (acc += d->age_weight[b]);
  }
  const int64_t count = d->count;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < d->capacity; ++i) {
    const int live = i < count;
    if (parts & LPG_INIT_BASE) { /* model.py:139-162 */
      int g = 0;
      if (live) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
          int m = (lo + hi + 1) >> 1;
          if (start[m] <= i) lo = m; else hi = m - 1;
        }
        g = lo;
      }
      c->disease_state[i] = live ? 0 : -1;
      c->node_id[i] = live ? (int16_t)g : (int16_t)-1;
      c->strain[i] = 0;
      c->potentially_paralyzed[i] = -1;
      c->paralyzed[i] = 0;
      c->ipv_protected[i] = 0;
      c->chronically_missed[i] = 0;
    }
    if (parts & LPG_INIT_TIMERS)
      lpg_init_timers(d->seed, (uint64_t)i, d->dur_exp.kind, d->dur_exp.p1, d->dur_exp.p2, d->dur_inf.kind,
                      d->dur_inf.p1, d->dur_inf.p2, d->t_to_paralysis.kind, d->t_to_paralysis.p1,
                      d->t_to_paralysis.p2, &c->exposure_timer[i], &c->infection_timer[i], &c->paralysis_timer[i]);
    if (parts & LPG_INIT_HETEROGENEITY)
      lpg_init_het(d->seed, (uint64_t)i, d->heterogeneity != 0, mu, sigma, rho, srho, scale,
                   &c->acq_risk_multiplier[i], &c->daily_infectivity[i]);
    int32_t dob = -1;
    if (parts & LPG_INIT_AGES) {
      dob = live ? -lpg_init_age(d->seed, (uint64_t)i, d->n_age_bins, cum, d->age_lo_days, d->age_hi_days) : -1;
      c->date_of_birth[i] = dob;
    } else if (parts & (LPG_INIT_DEATHS | LPG_INIT_RI)) {
      dob = c->date_of_birth[i];
    }
    if (parts & LPG_INIT_DEATHS) {
      int32_t dod = 0;
      if (live) {
        const int64_t age = -(int64_t)dob;
        const double u0 = lpg_u01(d->seed, LPG_P_INIT_KM, 0, (uint64_t)i, 0, 0);
        const double u1 = lpg_u01(d->seed, LPG_P_INIT_KM, 0, (uint64_t)i, 0, 1);
        dod = (int32_t)(lpg_km_age_at_death(d->km_cumdeaths, d->km_len, d->km_max_year, age, u0, u1) - age);
      }
      c->date_of_death[i] = dod;
    }
    if (parts & LPG_INIT_RI) c->ri_timer[i] = live ? lpg_init_ri(d->seed, (uint64_t)i, dob) : (int16_t)-1;
  }
  const int64_t all[2] = {0, count};
  if (parts & LPG_INIT_MISSED) lpo_select(d->seed, LPG_P_INIT_MISSED, all, 1, &d->missed_k, 0, c);
  if (parts & LPG_INIT_IMMUNITY) lpo_select(d->seed, LPG_P_INIT_IMMUNE, start, n, d->immune_k, 1, c);
  if (parts & LPG_INIT_PREVALENCE) {
    if (d->prev_per_node) lpo_select(d->seed, LPG_P_INIT_PREV, start, n, d->prev_k, 2, c);
    else lpo_select(d->seed, LPG_P_INIT_PREV, all, 1, d->prev_k, 2, c);
  }
  free(cum);
  free(start);
  return 0;
}

/* Single draws of the counter-based hook, for a harness that hands them to
 * another implementation of the same step (the reference's own code run
 * with its random calls redirected): each returns exactly what the oracle
 * and the engine draw for that (purpose, tick, a, b, k). */
double lpo_u01(uint64_t seed, int32_t purpose, int32_t t, uint64_t a, uint64_t b, uint64_t k) {
  return lpg_u01(seed, (uint32_t)purpose, t, a, b, k);
}
uint64_t lpo_u53(uint64_t seed, int32_t purpose, int32_t t, uint64_t a, uint64_t b, uint64_t k) {
  return lpg_u53(seed, (uint32_t)purpose, t, a, b, k);
}
uint64_t lpo_raw(uint64_t seed, int32_t purpose, int32_t t, uint64_t a, uint64_t b, uint64_t k) {
  return lpg_raw(seed, (uint32_t)purpose, t, a, b, k);
}
/* The node's exposure-count stream (lpo_node_tx): its first uniform (the
 * zero-inflation test), the negative binomial drawn after it, or the
 * Poisson count from its start. */
double lpo_tx_u0(uint64_t seed, int32_t t, uint64_t node) {
  lpg_stream st;
  lpg_stream_init(&st, seed, LPG_P_TXCOUNT, t, node, 0);
  return lpg_next(&st);
}
int64_t lpo_tx_negbinom(uint64_t seed, int32_t t, uint64_t node, double r, double p) {
  lpg_stream st;
  lpg_stream_init(&st, seed, LPG_P_TXCOUNT, t, node, 0);
  (void)lpg_next(&st);
  return lpg_negbinom(&st, r, p);
}
int64_t lpo_tx_poisson(uint64_t seed, int32_t t, uint64_t node, double lam) {
  lpg_stream st;
  lpg_stream_init(&st, seed, LPG_P_TXCOUNT, t, node, 0);
  return lpg_poisson(&st, lam);
}
/* The infection timer a seed event e redraws for slot (lpo_seed). */
double lpo_seed_timer(uint64_t seed, int32_t t, uint64_t slot, uint64_t e, int kind, double p1, double p2) {
  lpg_stream st;
  lpg_stream_init(&st, seed, LPG_P_SEEDTIMER, t, slot, e);
  return lpg_dist_sample(&st, kind, p1, p2);
}

/* Building blocks exposed for the unit tests of the draw hook. */
void lpo_philox(uint64_t ctr[4], uint64_t k0, uint64_t k1) { lpg_philox4x64_10(ctr, k0, k1); }
double lpo_exp(double x) { return lpg_exp(x); }
double lpo_expm1(double x) { return lpg_expm1(x); }
double lpo_mlog(double x) { return lpg_log(x); }
double lpo_lfact(int64_t k) { return lpg_lfact(k); }
/* fixed-point weights: the double-precision definition and the integer form
 * the CUDA engine uses, for many inputs at once (test export) */
void lpo_fix_risk_many(const float* r, int64_t n, uint64_t* by_double, uint64_t* by_bits, uint64_t* by_f32) {
  for (int64_t i = 0; i < n; ++i) {
    by_double[i] = fix_risk(r[i]);
    by_bits[i] = lpg_fix_risk_bits(r[i]);
    by_f32[i] = lpg_fix_risk_f32(r[i]);
  }
}
void lpo_poisson_many(uint64_t seed, double lam, int64_t n, int64_t* out) {
  for (int64_t i = 0; i < n; ++i) {
    lpg_stream st;
    lpg_stream_init(&st, seed, LPG_P_TXCOUNT, 0, (uint64_t)i, 7);
    out[i] = lpg_poisson(&st, lam);
  }
}
void lpo_gamma_many(uint64_t seed, double shape, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    lpg_stream st;
    lpg_stream_init(&st, seed, LPG_P_TXCOUNT, 0, (uint64_t)i, 8);
    out[i] = lpg_std_gamma(&st, shape);
  }
}
void lpo_negbinom_many(uint64_t seed, double r, double p, int64_t n, int64_t* out) {
  for (int64_t i = 0; i < n; ++i) {
    lpg_stream st;
    lpg_stream_init(&st, seed, LPG_P_TXCOUNT, 0, (uint64_t)i, 9);
    out[i] = lpg_negbinom(&st, r, p);
  }
}
void lpo_dist_many(uint64_t seed, int kind, double p1, double p2, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    lpg_stream st;
    lpg_stream_init(&st, seed, LPG_P_SEEDTIMER, 0, (uint64_t)i, 10);
    out[i] = lpg_dist_sample(&st, kind, p1, p2);
  }
}
