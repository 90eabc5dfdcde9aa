/*
 * lpg_init.cu — the model's initialisation on the device (lpg_init_columns).
 *
 * The reference builds its agent table on the host with numpy
 * (model.py:101-175, 561-713, 816-866, 1548-1611, 1887-1894), minutes at
 * Nigeria scale.  Here:
 *   - k_init_slots fills every per-slot column in one grid-stride pass over
 *     the capacity (lpg_init.h holds the arithmetic, shared with the oracle);
 *   - the choices without replacement (chronically missed, immune and
 *     initially infected agents) take, in each group, the k agents with the
 *     smallest counter-based 64-bit keys: a radix select on the keys' high
 *     32 bits in four 8-bit passes (a privatised shared-memory histogram per
 *     CTA tile, one thread per group to pick the digit), then one marking
 *     pass; the few agents whose high key bits equal the threshold are
 *     ordered by (full key, slot) on one thread per group.  The keys are
 *     recomputed from Philox in every pass instead of being stored, so the
 *     only scratch is per group.
 * Groups are whole nodes (the initial table is node-contiguous) or the whole
 * population.  Everything is HBM-light integer work: the passes are bound by
 * Philox arithmetic (about 140 integer instructions per key).
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <vector>

#include "lpg.h"
#include "lpg_init.h"

int lpg_ops_fail(int code, const char* fmt, ...);

namespace {

constexpr int kTile = 8192;  /* slots per CTA tile of the histogram passes */
constexpr int kEqCap = 256;  /* keys per group whose high 32 bits may equal the threshold */
constexpr int kThreads = 256;

struct SlotArgs {
  uint64_t seed;
  int64_t count, capacity;
  int32_t n_nodes, n_bins;
  const int64_t* node_start; /* [n_nodes + 1] */
  int32_t k_exp, k_inf, k_par, het;
  double e1, e2, i1, i2, p1, p2;
  double mu, sigma, rho, srho, scale;
  const int64_t* age_cum;
  const int32_t* age_lo;
  const int32_t* age_hi;
  const int64_t* km;
  int32_t km_len, km_max_year;
};

__device__ __forceinline__ int32_t group_of(const int64_t* start, int32_t n, int64_t slot) {
  int32_t a = 0, b = n - 1; /* last group with start <= slot */
  while (a < b) {
    const int32_t m = (a + b + 1) >> 1;
    if (start[m] <= slot) a = m; else b = m - 1;
  }
  return a;
}

__global__ void __launch_bounds__(kThreads) k_init_slots(SlotArgs A, lpg_columns c, uint32_t parts) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.capacity; i += stride) {
    const bool live = i < A.count;
    if (parts & LPG_INIT_BASE) {
      c.disease_state[i] = live ? 0 : -1;
      c.node_id[i] = live ? (int16_t)group_of(A.node_start, A.n_nodes, i) : (int16_t)-1;
      c.strain[i] = 0;
      c.potentially_paralyzed[i] = -1;
      c.paralyzed[i] = 0;
      c.ipv_protected[i] = 0;
      c.chronically_missed[i] = 0;
    }
    if (parts & LPG_INIT_TIMERS)
      lpg_init_timers(A.seed, (uint64_t)i, A.k_exp, A.e1, A.e2, A.k_inf, A.i1, A.i2, A.k_par, A.p1, A.p2,
                      &c.exposure_timer[i], &c.infection_timer[i], &c.paralysis_timer[i]);
    if (parts & LPG_INIT_HETEROGENEITY)
      lpg_init_het(A.seed, (uint64_t)i, A.het, A.mu, A.sigma, A.rho, A.srho, A.scale, &c.acq_risk_multiplier[i],
                   &c.daily_infectivity[i]);
    int32_t dob = -1;
    if (parts & LPG_INIT_AGES) {
      dob = live ? -lpg_init_age(A.seed, (uint64_t)i, A.n_bins, A.age_cum, A.age_lo, A.age_hi) : -1;
      c.date_of_birth[i] = dob;
    } else if (parts & (LPG_INIT_DEATHS | LPG_INIT_RI)) {
      dob = c.date_of_birth[i];
    }
    if (parts & LPG_INIT_DEATHS) {
      int32_t dod = 0;
      if (live) {
        const int64_t age = -(int64_t)dob;
        const double u0 = lpg_u01(A.seed, LPG_P_INIT_KM, 0, (uint64_t)i, 0, 0);
        const double u1 = lpg_u01(A.seed, LPG_P_INIT_KM, 0, (uint64_t)i, 0, 1);
        dod = (int32_t)(lpg_km_age_at_death(A.km, A.km_len, A.km_max_year, age, u0, u1) - age);
      }
      c.date_of_death[i] = dod;
    }
    if (parts & LPG_INIT_RI) c.ri_timer[i] = live ? lpg_init_ri(A.seed, (uint64_t)i, dob) : (int16_t)-1;
  }
}

/* --- selection of k agents per group by their smallest keys ------------- */
struct Sel {
  uint64_t seed;
  uint32_t purpose;
  int32_t n_groups;
  const int64_t* start; /* [n_groups + 1] */
  const int64_t* k;     /* [n_groups] */
  uint32_t* prefix;     /* [n_groups] high key bits fixed so far */
  int64_t* krem;        /* [n_groups] agents still to take among those matching the prefix */
  uint32_t* hist;       /* [n_groups][256] */
  uint32_t* eq_n;       /* [n_groups] */
  int64_t* eq;          /* [n_groups][kEqCap] */
  int* err;
};

__device__ __forceinline__ bool sel_active(const Sel& S, int32_t g) {
  const int64_t n = S.start[g + 1] - S.start[g];
  return S.k[g] > 0 && S.k[g] < n;
}

__device__ __forceinline__ uint32_t key_hi(const Sel& S, int64_t i) {
  return (uint32_t)(lpg_raw(S.seed, S.purpose, 0, (uint64_t)i, 0, 0) >> 32);
}

__global__ void k_rsel_init(Sel S) {
  for (int32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < S.n_groups; g += gridDim.x * blockDim.x) {
    S.prefix[g] = 0;
    S.krem[g] = S.k[g];
    S.eq_n[g] = 0;
    for (int d = 0; d < 256; ++d) S.hist[(int64_t)g * 256 + d] = 0;
  }
}

__global__ void __launch_bounds__(kThreads) k_rsel_hist(Sel S, int pass, int64_t count) {
  __shared__ uint32_t h[256];
  const int shift = 24 - 8 * pass;
  for (int64_t t0 = (int64_t)blockIdx.x * kTile; t0 < count; t0 += (int64_t)gridDim.x * kTile) {
    const int64_t t1 = t0 + kTile < count ? t0 + kTile : count;
    const int32_t g0 = group_of(S.start, S.n_groups, t0), g1 = group_of(S.start, S.n_groups, t1 - 1);
    const bool priv = g0 == g1;
    if (priv && !sel_active(S, g0)) continue; /* uniform over the CTA */
    if (priv) {
      for (int d = threadIdx.x; d < 256; d += blockDim.x) h[d] = 0;
      __syncthreads();
    }
    for (int64_t i = t0 + threadIdx.x; i < t1; i += blockDim.x) {
      const int32_t g = priv ? g0 : group_of(S.start, S.n_groups, i);
      if (!priv && !sel_active(S, g)) continue;
      const uint32_t key = key_hi(S, i);
      if (pass > 0 && (key >> (shift + 8)) != S.prefix[g]) continue;
      const uint32_t d = (key >> shift) & 255u;
      if (priv) atomicAdd(&h[d], 1u); else atomicAdd(&S.hist[(int64_t)g * 256 + d], 1u);
    }
    if (priv) {
      __syncthreads();
      for (int d = threadIdx.x; d < 256; d += blockDim.x)
        if (h[d]) atomicAdd(&S.hist[(int64_t)g0 * 256 + d], h[d]);
      __syncthreads();
    }
  }
}

/* the digit holding the krem-th smallest key of each group */
__global__ void k_rsel_scan(Sel S) {
  for (int32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < S.n_groups; g += gridDim.x * blockDim.x) {
    if (!sel_active(S, g)) continue;
    uint32_t* h = S.hist + (int64_t)g * 256;
    int64_t below = 0;
    int digit = 255;
    for (int d = 0; d < 256; ++d) {
      if (below + (int64_t)h[d] >= S.krem[g]) {
        digit = d;
        break;
      }
      below += h[d];
    }
    S.prefix[g] = (S.prefix[g] << 8) | (uint32_t)digit;
    S.krem[g] -= below;
    for (int d = 0; d < 256; ++d) h[d] = 0;
  }
}

__device__ __forceinline__ void sel_apply(const lpg_columns& c, int action, int64_t i) {
  if (action == 0) c.chronically_missed[i] = 1;
  else if (action == 1) c.disease_state[i] = 3;
  else c.disease_state[i] = 2;
}

__global__ void __launch_bounds__(kThreads) k_rsel_mark(Sel S, lpg_columns c, int action, int64_t count) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const int32_t g = group_of(S.start, S.n_groups, i);
    const int64_t n = S.start[g + 1] - S.start[g], k = S.k[g];
    if (k <= 0) continue;
    if (k >= n) {
      sel_apply(c, action, i);
      continue;
    }
    const uint32_t key = key_hi(S, i);
    if (key < S.prefix[g]) {
      sel_apply(c, action, i);
    } else if (key == S.prefix[g]) {
      const uint32_t q = atomicAdd(&S.eq_n[g], 1u);
      if (q < (uint32_t)kEqCap) S.eq[(int64_t)g * kEqCap + q] = i;
      else atomicOr(S.err, 1);
    }
  }
}

/* among the agents whose high key bits equal the threshold, the krem first
 * by (full key, slot) */
__global__ void k_rsel_ties(Sel S, lpg_columns c, int action) {
  for (int32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < S.n_groups; g += gridDim.x * blockDim.x) {
    if (!sel_active(S, g)) continue;
    const int n = (int)(S.eq_n[g] < (uint32_t)kEqCap ? S.eq_n[g] : (uint32_t)kEqCap);
    int64_t* e = S.eq + (int64_t)g * kEqCap;
    for (int a = 1; a < n; ++a) { /* insertion sort by (key, slot) */
      const int64_t v = e[a];
      const uint64_t kv = lpg_raw(S.seed, S.purpose, 0, (uint64_t)v, 0, 0);
      int b = a - 1;
      while (b >= 0) {
        const uint64_t kb = lpg_raw(S.seed, S.purpose, 0, (uint64_t)e[b], 0, 0);
        if (kb < kv || (kb == kv && e[b] < v)) break;
        e[b + 1] = e[b];
        --b;
      }
      e[b + 1] = v;
    }
    const int64_t take = S.krem[g] < n ? S.krem[g] : n;
    for (int64_t j = 0; j < take; ++j) sel_apply(c, action, e[j]);
  }
}

#define CKI(x)                                                                              \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) return lpg_ops_fail(LPG_ERR_CUDA, "init: %s", cudaGetErrorString(e_)); \
  } while (0)

/* Device scratch freed on the stream when it goes out of scope. */
struct Scratch {
  cudaStream_t st;
  std::vector<void*> ptrs;
  explicit Scratch(cudaStream_t s) : st(s) {}
  ~Scratch() {
    for (void* p : ptrs) cudaFreeAsync(p, st);
  }
  template <class T>
  int alloc(T** out, size_t n) {
    void* p = nullptr;
    if (cudaMallocAsync(&p, (n ? n : 1) * sizeof(T), st) != cudaSuccess) {
      cudaGetLastError();
      return lpg_ops_fail(LPG_ERR_NOMEM, "init: device scratch of %zu bytes", n * sizeof(T));
    }
    ptrs.push_back(p);
    *out = (T*)p;
    return 0;
  }
  template <class T>
  int upload(T** out, const std::vector<T>& v) {
    int rc = alloc(out, v.size());
    if (rc) return rc;
    if (cudaMemcpyAsync(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st) != cudaSuccess)
      return lpg_ops_fail(LPG_ERR_CUDA, "init: upload");
    return 0;
  }
};

int grid_for(int64_t n, int per_block) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t want = (n + per_block - 1) / per_block;
  int64_t cap = (int64_t)(sms > 0 ? sms : 152) * 8;
  if (want > cap) want = cap;
  return (int)(want > 0 ? want : 1);
}

int select_k(Scratch& sc, cudaStream_t st, const lpg_columns& c, uint64_t seed, uint32_t purpose, int action,
             const std::vector<int64_t>& start, const std::vector<int64_t>& k, int64_t count) {
  const int32_t G = (int32_t)k.size();
  Sel S{};
  S.seed = seed;
  S.purpose = purpose;
  S.n_groups = G;
  int64_t *d_start, *d_k, *krem, *eq;
  uint32_t *prefix, *hist, *eq_n;
  int* err;
  int rc = sc.upload(&d_start, start);
  if (!rc) rc = sc.upload(&d_k, k);
  if (!rc) rc = sc.alloc(&prefix, (size_t)G);
  if (!rc) rc = sc.alloc(&krem, (size_t)G);
  if (!rc) rc = sc.alloc(&hist, (size_t)G * 256);
  if (!rc) rc = sc.alloc(&eq_n, (size_t)G);
  if (!rc) rc = sc.alloc(&eq, (size_t)G * kEqCap);
  if (!rc) rc = sc.alloc(&err, 1);
  if (rc) return rc;
  S.start = d_start;
  S.k = d_k;
  S.prefix = prefix;
  S.krem = krem;
  S.hist = hist;
  S.eq_n = eq_n;
  S.eq = eq;
  S.err = err;
  CKI(cudaMemsetAsync(err, 0, sizeof(int), st));
  const int gb = (G + 255) / 256;
  k_rsel_init<<<gb, 256, 0, st>>>(S);
  const int tiles = grid_for(count, kTile);
  for (int pass = 0; pass < 4; ++pass) {
    k_rsel_hist<<<tiles, kThreads, 0, st>>>(S, pass, count);
    k_rsel_scan<<<gb, 256, 0, st>>>(S);
  }
  k_rsel_mark<<<grid_for(count, kThreads * 4), kThreads, 0, st>>>(S, c, action, count);
  k_rsel_ties<<<gb, 256, 0, st>>>(S, c, action);
  CKI(cudaGetLastError());
  int h_err = 0;
  CKI(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKI(cudaStreamSynchronize(st));
  if (h_err) return lpg_ops_fail(LPG_ERR_INTERNAL, "init: more than %d keys tie at a selection threshold", kEqCap);
  return 0;
}

}  // namespace

extern "C" double lpg_init_mean_infectivity(uint64_t seed, double r0, lpg_dist dur_inf) {
  lpg_stream s;
  lpg_stream_init(&s, seed, LPG_P_INIT_MEANINF, 0, 0, 0);
  double sum = 0.0;
  for (int j = 0; j < 1000; ++j) sum = sum + lpg_dist_sample(&s, dur_inf.kind, dur_inf.p1, dur_inf.p2);
  return r0 / (sum / 1000.0);
}

extern "C" int lpg_init_columns(const lpg_init_desc* d, uint32_t parts, const lpg_columns* cols, void* stream) {
  if (!d || !cols) return lpg_ops_fail(LPG_ERR_ARG, "init: null argument");
  const int32_t n = d->n_nodes;
  if (n < 1 || n > 32767) return lpg_ops_fail(LPG_ERR_ARG, "init: n_nodes %d out of range", n);
  if (d->count < 0 || d->capacity < d->count || d->capacity >= (int64_t)0xFFFFFFF0LL)
    return lpg_ops_fail(LPG_ERR_ARG, "init: count %lld / capacity %lld", (long long)d->count, (long long)d->capacity);
  if (!d->node_pop) return lpg_ops_fail(LPG_ERR_ARG, "init: node_pop is required");
  std::vector<int64_t> start(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    if (d->node_pop[i] < 0) return lpg_ops_fail(LPG_ERR_ARG, "init: node_pop[%d] is negative", i);
    start[i + 1] = start[i] + d->node_pop[i];
  }
  if (start[n] != d->count) return lpg_ops_fail(LPG_ERR_ARG, "init: node_pop sums to %lld, count is %lld",
                                                (long long)start[n], (long long)d->count);
  const lpg_columns& c = *cols;
  auto need = [&](uint32_t part, std::initializer_list<const void*> ptrs, const char* what) -> int {
    if (!(parts & part)) return 0;
    for (const void* p : ptrs)
      if (!p) return lpg_ops_fail(LPG_ERR_ARG, "init: %s needs its columns", what);
    return 0;
  };
  int rc = 0;
  if ((rc = need(LPG_INIT_BASE, {c.disease_state, c.node_id, c.strain, c.potentially_paralyzed, c.paralyzed,
                                 c.ipv_protected, c.chronically_missed}, "BASE")) ||
      (rc = need(LPG_INIT_MISSED, {c.chronically_missed}, "MISSED")) ||
      (rc = need(LPG_INIT_TIMERS, {c.exposure_timer, c.infection_timer, c.paralysis_timer}, "TIMERS")) ||
      (rc = need(LPG_INIT_IMMUNITY, {c.disease_state, d->immune_k}, "IMMUNITY")) ||
      (rc = need(LPG_INIT_PREVALENCE, {c.disease_state, d->prev_k}, "PREVALENCE")) ||
      (rc = need(LPG_INIT_HETEROGENEITY, {c.acq_risk_multiplier, c.daily_infectivity}, "HETEROGENEITY")) ||
      (rc = need(LPG_INIT_AGES, {c.date_of_birth, d->age_lo_days, d->age_hi_days, d->age_weight}, "AGES")) ||
      (rc = need(LPG_INIT_DEATHS, {c.date_of_birth, c.date_of_death, d->km_cumdeaths}, "DEATHS")) ||
      (rc = need(LPG_INIT_RI, {c.date_of_birth, c.ri_timer}, "RI")))
    return rc;
  cudaStream_t st = (cudaStream_t)stream;
  Scratch sc(st);
  SlotArgs A{};
  A.seed = d->seed;
  A.count = d->count;
  A.capacity = d->capacity;
  A.n_nodes = n;
  int64_t* d_start;
  if ((rc = sc.upload(&d_start, start))) return rc;
  A.node_start = d_start;
  A.k_exp = d->dur_exp.kind;
  A.e1 = d->dur_exp.p1;
  A.e2 = d->dur_exp.p2;
  A.k_inf = d->dur_inf.kind;
  A.i1 = d->dur_inf.p1;
  A.i2 = d->dur_inf.p2;
  A.k_par = d->t_to_paralysis.kind;
  A.p1 = d->t_to_paralysis.p1;
  A.p2 = d->t_to_paralysis.p2;
  if (parts & LPG_INIT_HETEROGENEITY) {
    /* model.py:839-851: lognormal risk with mean 1 and variance risk_mult_var;
     * infectivity mean r0 / mean(dur_inf(1000)), at least 1e-10 */
    const double var = d->risk_mult_var;
    if (!(var >= 0.0) || !std::isfinite(var)) return lpg_ops_fail(LPG_ERR_ARG, "init: risk_mult_var %g", var);
    A.het = d->heterogeneity != 0;
    A.mu = std::log(1.0 / std::sqrt(var + 1.0));
    A.sigma = std::sqrt(std::log(var + 1.0));
    A.rho = 2.0 * std::sin(LPG_PI * d->corr_risk_inf / 6.0);
    if (!(std::fabs(A.rho) <= 1.0)) return lpg_ops_fail(LPG_ERR_ARG, "init: corr_risk_inf %g", d->corr_risk_inf);
    A.srho = std::sqrt(1.0 - A.rho * A.rho);
    const double mean = lpg_init_mean_infectivity(d->seed, d->r0, d->dur_inf);
    A.scale = mean > 1e-10 ? mean : 1e-10;
  }
  if (parts & LPG_INIT_AGES) {
    const int nb = d->n_age_bins;
    if (nb < 1) return lpg_ops_fail(LPG_ERR_ARG, "init: no age bins");
    std::vector<int64_t> cum(nb);
    std::vector<int32_t> lo(d->age_lo_days, d->age_lo_days + nb), hi(d->age_hi_days, d->age_hi_days + nb);
    int64_t acc = 0;
    for (int b = 0; b < nb; ++b) {
      if (d->age_weight[b] < 0 || hi[b] <= lo[b]) return lpg_ops_fail(LPG_ERR_ARG, "init: age bin %d", b);
      acc += d->age_weight[b];
      cum[b] = acc;
    }
    if (acc <= 0) return lpg_ops_fail(LPG_ERR_ARG, "init: age weights sum to 0");
    A.n_bins = nb;
    int64_t* dc;
    int32_t *dl, *dh;
    if ((rc = sc.upload(&dc, cum)) || (rc = sc.upload(&dl, lo)) || (rc = sc.upload(&dh, hi))) return rc;
    A.age_cum = dc;
    A.age_lo = dl;
    A.age_hi = dh;
  }
  if (parts & LPG_INIT_DEATHS) {
    if (d->km_len < 1) return lpg_ops_fail(LPG_ERR_ARG, "init: empty km table");
    std::vector<int64_t> km(d->km_cumdeaths, d->km_cumdeaths + d->km_len);
    int64_t* dk;
    if ((rc = sc.upload(&dk, km))) return rc;
    A.km = dk;
    A.km_len = d->km_len;
    A.km_max_year = d->km_max_year;
  }
  const uint32_t slot_parts =
      parts & (LPG_INIT_BASE | LPG_INIT_TIMERS | LPG_INIT_HETEROGENEITY | LPG_INIT_AGES | LPG_INIT_DEATHS | LPG_INIT_RI);
  if (slot_parts && d->capacity > 0) {
    k_init_slots<<<grid_for(d->capacity, kThreads * 8), kThreads, 0, st>>>(A, c, slot_parts);
    CKI(cudaGetLastError());
  }
  const std::vector<int64_t> all = {0, d->count};
  if ((parts & LPG_INIT_MISSED) && d->count > 0) {
    if ((rc = select_k(sc, st, c, d->seed, LPG_P_INIT_MISSED, 0, all, {d->missed_k}, d->count))) return rc;
  }
  if ((parts & LPG_INIT_IMMUNITY) && d->count > 0) {
    std::vector<int64_t> k(d->immune_k, d->immune_k + n);
    if ((rc = select_k(sc, st, c, d->seed, LPG_P_INIT_IMMUNE, 1, start, k, d->count))) return rc;
  }
  if ((parts & LPG_INIT_PREVALENCE) && d->count > 0) {
    if (d->prev_per_node) {
      std::vector<int64_t> k(d->prev_k, d->prev_k + n);
      rc = select_k(sc, st, c, d->seed, LPG_P_INIT_PREV, 2, start, k, d->count);
    } else {
      rc = select_k(sc, st, c, d->seed, LPG_P_INIT_PREV, 2, all, {d->prev_k[0]}, d->count);
    }
    if (rc) return rc;
  }
  CKI(cudaStreamSynchronize(st));
  return LPG_OK;
}
