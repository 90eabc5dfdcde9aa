/*
 * lpg_kernels.cuh — device kernels of the per-tick agent step.
 *
 * One tick is this launch sequence (every kernel reads the tick and its
 * flags from device memory, so blocks of ticks are captured in CUDA graphs
 * and replayed; the kernels only some ticks need are launched only then):
 *   k_begin      birth ticks, per simulation: births per node
 *                (model.py:1711-1716) and their chunk placement
 *   k_newborns   birth ticks: newborn rows (model.py:1719-1730)
 *   k_due        the sub-blocks with a disease-state event or a death due,
 *                from the per-sub-block indexes
 *   k_sweep_due  those sub-blocks, evenly over the CTAs: deaths (get_deaths,
 *                model.py:1767-1781), then each CTA's queue of deaths and
 *                of agents in E or I whose event is now: death bookkeeping,
 *                disease progression and paralysis (model.py:393-454)
 *   k_seed       the seed schedule (model.py:759-786)
 *   k_sweep_rs   on RI/SIA ticks: the queue of agents that RI (fast_ri,
 *                :1784-1855; due sub-blocks only) or today's SIA campaigns
 *                (fast_sia, :1994-2060; every slot, staged) reach
 *   k_evb        their draws and exposures
 *   k_node_tx    per node: population (model.py:1751-1755), mixing,
 *                seasonality, probabilities and exposure counts
 *                (model.py:1327-1407)
 *   k_sel_round0, k_sel_rounds               weighted selection rounds
 *                and strain assignment (tx_infect_nb, model.py:1010-1149);
 *                k_sel_rounds then ends the tick (end_tick): results rows
 *                (model.py:1461-1487 and the result writes of every
 *                component), the next tick's flags and stop rule
 */
#ifndef LPG_KERNELS_CUH
#define LPG_KERNELS_CUH

#include <stdint.h>

#include "lpg_engine.cuh"

#define FULLMASK 0xffffffffu
#define LPG_NONE 0xffffffffu
/* State byte of an agent claimed by a round-0 target of this tick while the
 * round is still running: the round's other targets locate on the frozen
 * CDF, so they still count it as susceptible; k_sel_round0 makes it exposed
 * (1) after its grid barrier.  No other kernel sees it. */
#define LPG_DS_CLAIMED 0x40u
/* a state byte that carries selection weight: susceptible, or claimed in the
 * running round 0 */
__device__ __forceinline__ bool sel_open(uint32_t b) { return (b & ~LPG_DS_CLAIMED & 0xffu) == 0; }

/* Programmatic dependent launch: the tick's kernels are launched so that
 * the next one's CTAs may be scheduled while this one finishes.  Every tick
 * kernel first waits until the kernel before it has completed and its
 * writes are visible (griddepcontrol.wait: nothing of the previous kernel is
 * read or written before it), then lets the next one be scheduled
 * (griddepcontrol.launch_dependents).  Both are no-ops for a kernel launched
 * without the attribute or without dependents. */
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
#define LPG_MAX_ROUNDS 1000000

/* ------------------------------------------------------------------------ */
/* fixed-point weights (identical definitions in the oracle)                */
__device__ __forceinline__ uint64_t fix_risk(float r) { return lpg_fix_risk_f32(r); }
__device__ __forceinline__ uint64_t fix_beta(float inf, double scal) {
  double d = ((double)inf * scal) * 0x1.0p40;
  if (!(d > 0.0)) return 0;
  if (d > 0x1.0p62) d = 0x1.0p62;
  return (uint64_t)rint(d);
}
/* Three-word (192-bit) unsigned accumulators with the carry chain in PTX:
 * acc3_mul adds the 128-bit product x*y, acc3_add another accumulator. */
__device__ __forceinline__ void acc3_mul(uint64_t& a0, uint64_t& a1, uint64_t& a2, uint64_t x, uint64_t y) {
  const uint64_t lo = x * y, hi = __umul64hi(x, y);
  asm("add.cc.u64 %0, %0, %3;\n\taddc.cc.u64 %1, %1, %4;\n\taddc.u64 %2, %2, 0;"
      : "+l"(a0), "+l"(a1), "+l"(a2)
      : "l"(lo), "l"(hi));
}
__device__ __forceinline__ void acc3_add(uint64_t& a0, uint64_t& a1, uint64_t& a2, uint64_t b0, uint64_t b1,
                                         uint64_t b2) {
  asm("add.cc.u64 %0, %0, %3;\n\taddc.cc.u64 %1, %1, %4;\n\taddc.u64 %2, %2, %5;"
      : "+l"(a0), "+l"(a1), "+l"(a2)
      : "l"(b0), "l"(b1), "l"(b2));
}
__device__ __forceinline__ int8_t dec_i8(int8_t v) { return (int8_t)(uint8_t)((uint8_t)v - 1u); }
__device__ __forceinline__ int8_t sub_i8(int8_t v, int k) { return (int8_t)(uint8_t)((uint8_t)v - (uint8_t)k); }

/* Disease-state timers on events (disease_state_step_kernel, model.py:393-454).
 * The reference counts every timer of an agent in E or I down by one each
 * tick.  Here an agent keeps its timers as of the last tick tm at which they
 * were brought up to date, plus evt = tm + 1 + K: K = ev_pure(...) is the
 * number of steps that only count down before the next step that is an
 * event (E: exposure timer <= 0, the move to I; I: infection timer <= 0, the
 * move to R, or for strain 0 with potentially_paralyzed still -1 the
 * paralysis check at paralysis timer <= 0).  Only event steps touch the
 * agent; the skipped count-downs are applied (ev_advance, int8 wrap like the
 * reference's stores) when the agent is next touched: at its event, death,
 * a seed, or when the columns are read back.  With tc the last tick whose
 * step has run, the skipped steps are tc - tm = tc - evt + 1 + K. */
__device__ __forceinline__ int ev_pure(int8_t ds, int8_t strain, int8_t et, int8_t it, int8_t pt, int8_t pp) {
  if (ds == 1) return et > 0 ? et : 0;
  int k = it > 0 ? it : 0;
  if (strain == 0 && pp == -1) {
    const int kp = pt > 0 ? pt : 0;
    k = kp < k ? kp : k;
  }
  return k;
}
__device__ __forceinline__ void ev_advance(int8_t ds, int8_t strain, int8_t& et, int8_t& it, int8_t& pt, int k) {
  if (ds == 1) {
    et = sub_i8(et, k);
  } else {
    it = sub_i8(it, k);
    if (strain == 0) pt = sub_i8(pt, k);
  }
}
__device__ __forceinline__ unsigned long long neg64(uint64_t w) { return (unsigned long long)(0ULL - w); }

/* RI runs for the simulation: RI_ABM among the components and vx_prob_ri
 * set (model.py:1920-1923).  Only then do the timers count down. */
__device__ __forceinline__ bool ri_runs(const DevRep* rp) { return (rp->comps & LPG_COMP_RI) && rp->ri_enabled; }
/* RI due tick of an agent from its base timer u, reference index and date
 * of birth (lpg_ri.h). */
__device__ __forceinline__ int32_t ri_due_of(const DevRep* rp, int16_t u, uint32_t ref, int32_t dob) {
  const int32_t s = rp->ri_step;
  return lpg_ri_due_tick(u, lpg_ri_first((int64_t)ref >= rp->count0, dob, s), s);
}
/* The reference's ri_timer of an agent once the RI ticks up to t_last have run. */
__device__ __forceinline__ int16_t ri_now(const DevRep* rp, int16_t u, uint32_t ref, int32_t dob, int32_t t_last) {
  const int32_t s = rp->ri_step;
  return lpg_ri_value(u, lpg_ri_applied(lpg_ri_first((int64_t)ref >= rp->count0, dob, s), t_last, s), s);
}

__device__ __forceinline__ int32_t* RES(const DevRep* rp, int k, int t) {
  int wide = (k == RS_EBS || k == RS_IBS || k == RS_NEWEXPBS || k == RS_RINEWEXPBS || k == RS_SIANEWEXPBS);
  return rp->res + rp->res_off[k] + (int64_t)t * rp->n_nodes * (wide ? rp->ns : 1);
}

/* Newborn lifespan: restates laser_core's KaplanMeierEstimator for age 0
 * (model.py:1725).  Same arithmetic as the oracle's lpo_km_newborn. */
__device__ int32_t km_newborn(const DevRep* rp, int32_t t, uint64_t slot, const int64_t* cum) {
  int32_t top = rp->km_max_year < rp->km_len - 1 ? rp->km_max_year : rp->km_len - 1;
  int64_t total = cum[top];
  int32_t y = top;
  if (total > 0) {
    double u0 = lpg_u01(rp->seed, LPG_P_KM, t, slot, 0, 0);
    int64_t draw = (int64_t)floor(u0 * (double)total);
    int32_t lo = 0, hi = top;
    while (lo < hi) {
      int32_t mid = (lo + hi) >> 1;
      if (cum[mid] > draw) hi = mid; else lo = mid + 1;
    }
    y = lo;
  }
  double u1 = lpg_u01(rp->seed, LPG_P_KM, t, slot, 0, 1);
  return y * 365 + (int32_t)floor(u1 * 365.0);
}

/* Block-wide exclusive scan of one value per thread (blockDim multiple of 32). */
__device__ int64_t block_excl_scan(int64_t v, int64_t* total) {
  __shared__ int64_t ws[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(FULLMASK, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t s = lane < nw ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(FULLMASK, s, o);
      if (lane >= o) s += y;
    }
    ws[lane] = s;
  }
  __syncthreads();
  int64_t incl = x + (wid > 0 ? ws[wid - 1] : 0);
  *total = ws[nw - 1];
  __syncthreads();
  return incl - v;
}

/* ------------------------------------------------------------------------ */
/* The flags of the replicate's next tick (rp->t): which components run and
 * the tick's schedule entries (model.py:246-282 with each component's own
 * step condition), and the per-tick bookkeeping reset.  k_end's last CTA
 * calls it for every replicate, so a tick starts prepared. */
__device__ void rep_prepare(DevRep* rp) {
  /* every field read before the first store (the stores could alias) */
  const int t = rp->t;
  const int started = rp->started, error = rp->error, stopped = rp->stopped, nt = rp->nt;
  const uint32_t comps = rp->comps;
  const int vd_step = rp->vd_step, ri_step = rp->ri_step, ri_enabled = rp->ri_enabled;
  const int64_t count = rp->count;
  const int active = started && !error && !stopped && t >= 1 && t < nt;
  const int tt = active ? t : 0;
  const int sia_cnt = rp->sia_cnt[tt], sia_first = rp->sia_first[tt];
  const int seed_cnt = rp->seed_cnt[tt], seed_first = rp->seed_first[tt];
  rp->cur_t = t;
  rp->active = active;
  rp->vd_tick = active && (comps & LPG_COMP_VD) && (t % vd_step == 0);
  rp->ri_tick = active && (comps & LPG_COMP_RI) && ri_enabled && (t % ri_step == 0);
  rp->sia_n = (active && (comps & LPG_COMP_SIA)) ? sia_cnt : 0;
  rp->sia_i0 = active ? sia_first : 0;
  rp->seed_n = (active && (comps & LPG_COMP_DS)) ? seed_cnt : 0;
  rp->seed_i0 = active ? seed_first : 0;
  rp->nb_total = 0;
  rp->count_before = count;
  rp->any_demand = 0;
  rp->csr_flip = 0;
}

/* VD ticks: births per node and their chunk placement (the tick's flags,
 * the stop rule and the cleared event counters come from the previous
 * tick's k_end). */
__global__ void k_begin(DevWorld W) {
  pdl_begin();
  DevRep* rp = &W.reps[blockIdx.x];
  if (!rp->active || !rp->vd_tick) return;
  const int n = rp->n_nodes, nb = rp->node_base, t = rp->cur_t, G = W.G;

  /* births per node: integer part + Bernoulli on the fraction (model.py:1711-1716) */
  const int32_t* pop1 = RES(rp, RS_POP, t - 1);
  int64_t carry_b = 0, carry_c = 0;
  for (int base = 0; base < n; base += blockDim.x) {
    int i = base + threadIdx.x;
    int64_t b = 0, newch = 0, li0 = 0;
    if (i < n) {
      int g = nb + i;
      double expected = ((double)rp->vd_step * rp->birth_rate[i]) * (double)pop1[i];
      int32_t bi = (int32_t)expected;
      double frac = expected - (double)bi;
      double u = lpg_u01(rp->seed, LPG_P_BIRTH, t, (uint64_t)i, 0, 0);
      b = (int64_t)bi + (u < frac ? 1 : 0);
      li0 = W.node_count[g];
      int64_t c_old = li0 > 0 ? (li0 + LPG_CHUNK - 1) / LPG_CHUNK : 1;
      int64_t c_new = li0 + b > 0 ? (li0 + b + LPG_CHUNK - 1) / LPG_CHUNK : 1;
      newch = c_new - c_old;
    }
    int64_t tb, tc;
    int64_t eb = block_excl_scan(b, &tb);
    int64_t ec = block_excl_scan(newch, &tc);
    if (i < n) {
      int g = nb + i;
      W.nb_end[g] = carry_b + eb + b;
      W.nb_li0[g] = li0;
      W.ev[(int64_t)EV_BIRTHS * G + g] = (int32_t)b;
      W.ksel[g] = carry_c + ec; /* scratch: new chunks before this node */
    }
    carry_b += tb;
    carry_c += tc;
  }
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    s_ok = 1;
    if (rp->count + carry_b > rp->capacity) {
      rp->error = LPG_ERR_CAPACITY;
      rp->active = 0;
      s_ok = 0;
    } else if (rp->used_chunks + carry_c > rp->chunk_cap) {
      rp->error = LPG_ERR_INTERNAL;
      rp->active = 0;
      s_ok = 0;
    }
  }
  __syncthreads();
  if (!s_ok || carry_b == 0) return;

  const int cur = rp->csr_cur;
  const int32_t* so = W.node_chunk_start[cur] + rp->csr_base;
  const int32_t* lo_ = W.node_chunks[cur] + rp->chunk_base;
  const int32_t used0 = rp->used_chunks;
  if (carry_c > 0) {
    /* the new node -> chunk starts, in the other buffer; k_newborns copies
     * the lists (many CTAs) before any later kernel reads them */
    int32_t* sn = W.node_chunk_start[1 - cur] + rp->csr_base;
    for (int i = threadIdx.x; i < n; i += blockDim.x) sn[i] = so[i] + (int32_t)W.ksel[nb + i];
    if (threadIdx.x == 0) sn[n] = so[n] + (int32_t)carry_c;
  }
  /* chunk fills and newborn markers.  Chunk k of node i is entry k of its
   * current list, or its (k - listed)-th new chunk: new chunks are numbered
   * from used0 in node order (W.ksel holds the count before each node). */
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    int g = nb + i;
    int64_t b = W.ev[(int64_t)EV_BIRTHS * G + g];
    if (b == 0) continue;
    int64_t li0 = W.nb_li0[g], newc = li0 + b;
    const int32_t nold = so[i + 1] - so[i];
    for (int64_t k = li0 / LPG_CHUNK; k <= (newc - 1) / LPG_CHUNK; ++k) {
      const bool added = k >= nold;
      const int32_t cid = added ? rp->chunk_base + used0 + (int32_t)W.ksel[g] + (int32_t)(k - nold) : lo_[so[i] + k];
      if (added) {
        W.chunk_w[cid] = 0;
        for (int s = 0; s < LPG_NSUB; ++s) W.sub_w[(int64_t)cid * LPG_NSUB + s] = 0;
      }
      int64_t f = newc - k * LPG_CHUNK;
      W.cmeta[cid] = make_int4(nb + i, (int32_t)(f < LPG_CHUNK ? f : LPG_CHUNK), t,
                               (k == li0 / LPG_CHUNK) ? (int32_t)(li0 % LPG_CHUNK) : 0);
    }
    W.node_count[g] = newc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    rp->csr_cur = carry_c > 0 ? 1 - cur : cur;
    rp->csr_flip = carry_c > 0;
    rp->used_before = used0;
    rp->used_chunks += (int32_t)carry_c;
    rp->count += carry_b;
    rp->nb_total = carry_b;
  }
}

/* ------------------------------------------------------------------------ */
/* Warp reductions over runs of consecutive lanes that hold the same key
 * (equal keys only ever form one contiguous run).  run_merge_bits: bit k set
 * when the lane 2^k above holds the same key; the run_* reductions then
 * leave the run's total on its first lane (run_head).  All 32 lanes call. */
__device__ __forceinline__ uint32_t run_merge_bits(uint64_t key) {
  const int lane = threadIdx.x & 31;
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const uint64_t o = __shfl_down_sync(FULLMASK, key, 1 << k);
    if (lane + (1 << k) < 32 && o == key) m |= 1u << k;
  }
  return m;
}
__device__ __forceinline__ bool run_head(uint64_t key) {
  const uint64_t p = __shfl_up_sync(FULLMASK, key, 1);
  return (threadIdx.x & 31) == 0 || p != key;
}
__device__ __forceinline__ uint64_t run_sum_u64(uint64_t v, uint32_t m) {
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const uint64_t y = __shfl_down_sync(FULLMASK, v, 1 << k);
    if ((m >> k) & 1u) v += y;
  }
  return v;
}
__device__ __forceinline__ int32_t run_sum_i32(int32_t v, uint32_t m) {
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int32_t y = __shfl_down_sync(FULLMASK, v, 1 << k);
    if ((m >> k) & 1u) v += y;
  }
  return v;
}
__device__ __forceinline__ int32_t run_min_i32(int32_t v, uint32_t m) {
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int32_t y = __shfl_down_sync(FULLMASK, v, 1 << k);
    if ((m >> k) & 1u) v = min(v, y);
  }
  return v;
}

/* Newborns of a VD tick (model.py:1719-1733), one thread each, after k_begin
 * placed them: rows from the unborn pool, the Kaplan-Meier date of death,
 * and the running totals and indexes, summed over each warp's runs of
 * newborns that share a node, chunk or sub-block before one atomic per run.
 * On ticks that added chunks it first copies the node -> chunk lists into
 * the buffer k_begin switched to (one warp per node).  Chunk k of a node is
 * entry k of its previous list or its (k - listed)-th new chunk, numbered
 * from used_before in node order (W.ksel: new chunks before each node). */
#define LPG_NB_SMEM 4096
#define LPG_KM_SMEM 256
__global__ void __launch_bounds__(256) k_newborns(DevWorld W) {
  pdl_begin();
  const DevRep* rp = &W.reps[blockIdx.y];
  if (!rp->active || !rp->vd_tick || rp->nb_total == 0) return;
  __shared__ int64_t s_end[LPG_NB_SMEM];
  __shared__ int64_t s_km[LPG_KM_SMEM];
  const int n = rp->n_nodes, nb = rp->node_base, t = rp->cur_t, G = W.G;
  const int lane = threadIdx.x & 31;
  const int64_t total = rp->nb_total;
  const int cur = rp->csr_cur, prev = rp->csr_flip ? 1 - cur : cur;
  const int32_t* so = W.node_chunk_start[prev] + rp->csr_base;
  const int32_t* lo_ = W.node_chunks[prev] + rp->chunk_base;
  const int32_t add0 = rp->chunk_base + rp->used_before;
  if (rp->csr_flip) {
    const int32_t* sn = W.node_chunk_start[cur] + rp->csr_base;
    int32_t* ln = W.node_chunks[cur] + rp->chunk_base;
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = gw; i < n; i += nw) {
      const int32_t a0 = so[i], nold = so[i + 1] - a0, d0 = sn[i], nnew = sn[i + 1] - d0;
      const int32_t c0 = add0 + (int32_t)W.ksel[nb + i];
      for (int32_t k = lane; k < nnew; k += 32) ln[d0 + k] = k < nold ? lo_[a0 + k] : c0 + (k - nold);
    }
  }
  const bool end_sm = n <= LPG_NB_SMEM, km_sm = rp->km_len <= LPG_KM_SMEM;
  if (end_sm)
    for (int i = threadIdx.x; i < n; i += blockDim.x) s_end[i] = W.nb_end[nb + i];
  if (km_sm)
    for (int i = threadIdx.x; i < rp->km_len; i += blockDim.x) s_km[i] = rp->km[i];
  __syncthreads();
  const int64_t* nbe = end_sm ? s_end : W.nb_end + nb;
  const int64_t* km = km_sm ? s_km : rp->km;
  const bool ri_on = ri_runs(rp);
  for (int64_t j0 = (int64_t)blockIdx.x * blockDim.x;; j0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = j0 + threadIdx.x;
    if (__all_sync(FULLMASK, j >= total)) break;
    const bool on = j < total;
    uint64_t kg = ~0ULL - (uint64_t)lane, kc = kg, ks = kg; /* idle lanes: keys of their own */
    uint64_t w = 0;
    int32_t dod = LPG_NO_DOD, rdt = LPG_NO_DOD, one = 0;
    int g = 0;
    int32_t cid = 0;
    if (on) {
      int lo = 0, hi = n - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (nbe[mid] > j) hi = mid; else lo = mid + 1;
      }
      g = nb + lo;
      const int64_t bstart = nbe[lo] - W.ev[(int64_t)EV_BIRTHS * G + g];
      const int64_t li = W.nb_li0[g] + (j - bstart);
      const int64_t k = li / LPG_CHUNK;
      const int32_t nold = so[lo + 1] - so[lo];
      cid = k < nold ? lo_[so[lo] + k] : add0 + (int32_t)W.ksel[g] + (int32_t)(k - nold);
      const int64_t off = li % LPG_CHUNK;
      const int64_t pos = (int64_t)cid * LPG_CHUNK + off;
      const int64_t ref = rp->count_before + j;
      const int64_t q = ref - rp->count0;
      W.et[pos] = rp->pl_et[q];
      W.it[pos] = rp->pl_it[q];
      W.pt[pos] = rp->pl_pt[q];
      W.strain[pos] = rp->pl_strain[q];
      const int8_t pp = rp->pl_pp[q], par = rp->pl_par[q];
      const uint8_t cm = rp->pl_cm[q];
      const int16_t ri = rp->pl_ri[q];
      W.pp[pos] = pp;
      W.par[pos] = par;
      W.ipv[pos] = rp->pl_ipv[q];
      W.cm[pos] = cm;
      W.ri[pos] = ri;
      const float risk = rp->pl_risk[q];
      W.risk[pos] = risk;
      W.inf[pos] = rp->pl_inf[q];
      W.dob[pos] = t;
      dod = t + km_newborn(rp, t, (uint64_t)ref, km);
      W.dod[pos] = dod;
      W.ref[pos] = (uint32_t)ref;
      W.ds[pos] = 0;
      if (ri_on && cm != 1) rdt = ri_due_of(rp, ri, (uint32_t)ref, t);
      W.rdt[pos] = rdt;
      w = fix_risk(risk);
      one = 1;
      if (pp == 1) atomicAdd(&W.tot[(int64_t)TT_POTP * G + g], 1);
      if (par == 1) atomicAdd(&W.tot[(int64_t)TT_P * G + g], 1);
      kg = (uint64_t)g;
      kc = (uint64_t)cid;
      ks = (uint64_t)cid * LPG_NSUB + (uint64_t)(off / LPG_SUB);
    }
    const uint32_t mg = run_merge_bits(kg), mc = run_merge_bits(kc), ms = run_merge_bits(ks);
    const bool hg = run_head(kg), hc = run_head(kc), hs = run_head(ks);
    const uint64_t wg = run_sum_u64(w, mg), wc = run_sum_u64(w, mc), wsb = run_sum_u64(w, ms);
    const int32_t ng = run_sum_i32(one, mg);
    const int32_t dmin = run_min_i32(dod, ms), rmin = run_min_i32(rdt, ms);
    if (on && hg) {
      atomicAdd(&W.tot[(int64_t)TT_S * G + g], ng);
      if (wg) atomicAdd((unsigned long long*)&W.sw[g], (unsigned long long)wg);
    }
    if (on && hc && wc) atomicAdd((unsigned long long*)&W.chunk_w[cid], (unsigned long long)wc);
    if (on && hs) {
      atomicMin(&W.sub_dod[ks], dmin);
      if (rmin != LPG_NO_DOD) atomicMin(&W.sub_rdt[ks], rmin);
      if (wsb) atomicAdd((unsigned long long*)&W.sub_w[ks], (unsigned long long)wsb);
    }
  }
}

/* The sweeps.
 *   k_due, k_sweep_due: deaths (get_deaths, model.py:1767-1781) on VD ticks
 *            and the agents in E or I whose disease-state event is due,
 *            through the sub-block indexes.
 *   k_sweep_rs: routine immunisation (fast_ri, model.py:1784-1855) and SIA
 *            campaigns (fast_sia, :1994-2060), on the ticks that have them,
 *            after progression and the seed schedule as in default_run_order.
 *            RI alone goes through the RI due index (ri_direct); SIA days
 *            stage every slot.
 *
 * The staged path is a warp-specialised pipeline.  Each CTA owns a
 * contiguous range of chunks.  One producer warp stages chunk metadata and
 * the columns every agent needs into shared memory with 1-D bulk copies
 * (cp.async.bulk; completion on a "full" mbarrier), through a ring of
 * LPG_NST stages; eight consumer warps process a stage and release it on an
 * "empty" mbarrier.  A stage holds k consecutive chunks, k = as many as fit
 * in LPG_COL_BYTES given the day's columns: state bytes,
 * chronically_missed and date_of_birth, and the RI due ticks when RI falls
 * on the same day.  Each consumer thread tests 16 slots at a time with SIMD
 * byte compares and appends the agents that need work to its CTA's queue
 * slab.  Each consumer warp releases a stage with one arrival.  There is no
 * CTA-wide barrier in the steady state.  Every mbarrier wait is bounded; on
 * a timeout the kernel raises an error, stops issuing, waits (bounded) for
 * the copies it issued and returns. */
#define LPG_NST 4
#define LPG_META_BYTES 256
#define LPG_COL_BYTES (24 * 1024)
#define LPG_STAGE_BYTES (LPG_META_BYTES + LPG_COL_BYTES)
#define LPG_PLAIN_GROUP (LPG_COL_BYTES / LPG_CHUNK)
#define LPG_SWEEP_SMEM (LPG_NST * LPG_STAGE_BYTES)
#define LPG_MBAR_SPIN (1LL << 24)

/* 16-byte global load that bypasses L1 allocation (streamed once). */
__device__ __forceinline__ uint4 ldg_stream16(const void* p) {
  uint4 v;
  asm volatile("ld.global.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
/* bounded wait; false on timeout */
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = LPG_MBAR_SPIN) {
  for (long long it = 0; it < limit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 64) __nanosleep(32);
  }
  return false;
}

/* per-simulation flags of the launch, cached in shared memory */
enum { SF_WORK = 1, SF_DENSE = 2, SF_RI = 16, SF_SIA = 32 };

struct SweepPlan {
  int32_t total, nreps;
  int32_t off[LPG_MAX_REPS + 1]; /* work-item offsets per simulation */
  int32_t cbase[LPG_MAX_REPS];   /* first chunk id per simulation */
  int32_t tick[LPG_MAX_REPS];
  uint8_t flags[LPG_MAX_REPS];
};

/* Staged bytes per chunk for a simulation's flags. */
__device__ __forceinline__ int chunk_bytes(uint8_t f) {
  return LPG_CHUNK + ((f & SF_RI) ? 4 * LPG_CHUNK : 0) +
         ((f & (SF_RI | SF_SIA)) ? LPG_CHUNK : 0) + ((f & SF_SIA) ? 4 * LPG_CHUNK : 0);
}
/* Chunks per stage (k consecutive chunks: each column is one contiguous copy). */
__device__ __forceinline__ int stage_chunks(uint8_t f) {
  const int k = LPG_COL_BYTES / chunk_bytes(f);
  return k < LPG_PLAIN_GROUP ? k : LPG_PLAIN_GROUP;
}
struct StageLayout {
  int ds, rdt, cm, dob;
};
__device__ __forceinline__ StageLayout stage_layout(uint8_t f, int k) {
  StageLayout L;
  int off = 0;
  L.ds = off;
  off += k * LPG_CHUNK;
  L.rdt = off;
  if (f & SF_RI) off += k * 4 * LPG_CHUNK;
  L.cm = off;
  if (f & (SF_RI | SF_SIA)) off += k * LPG_CHUNK;
  L.dob = off;
  return L;
}

/* End of the stage that starts at work item w (same answer on every thread). */
__device__ __forceinline__ int32_t stage_end(const SweepPlan& P, int32_t w, int32_t w1, int* r_out) {
  int lo = 0, hi = P.nreps - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (P.off[mid] <= w) lo = mid; else hi = mid - 1;
  }
  *r_out = lo;
  const int32_t lim = min(w1, P.off[lo + 1]);
  return min(lim, w + stage_chunks(P.flags[lo]));
}

/* Queue entries of the sweeps (u64): bits 0-31 position, bits 32-47 kind
 * and simulation (k_sweep_due) or event flags (k_sweep_rs), bits 48-55 the
 * state byte before the sweep (deaths). */
#define QA_DS 1u
#define QA_DEATH 2u
#define QB_RI 1u /* bit 0: RI-eligible; bit 1 + k: candidate of SIA event k */

__device__ __forceinline__ uint64_t q_entry(int64_t pos, uint32_t kind, uint32_t old_state) {
  return (uint64_t)(uint32_t)pos | ((uint64_t)(kind & 0xffffu) << 32) | ((uint64_t)(old_state & 0xffu) << 48);
}

/* Reserve n entries of this CTA's slab for each lane (warp scan + one shared
 * atomic per warp); returns the lane's first index.  All 32 lanes call. */
__device__ __forceinline__ uint32_t slab_reserve(uint32_t* s_cnt, uint32_t n) {
  const int lane = threadIdx.x & 31;
  uint32_t x = n;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(FULLMASK, x, o);
    if (lane >= o) x += y;
  }
  const uint32_t tot = __shfl_sync(FULLMASK, x, 31);
  uint32_t base = 0;
  if (lane == 31 && tot) base = atomicAdd(s_cnt, tot);
  base = __shfl_sync(FULLMASK, base, 31);
  return base + x - n;
}

/* Append one thread's queue entries of 16 slots (ei: agents in E or I,
 * dead: deaths with their state before the sweep) of simulation sim: the
 * entry's kind field holds QA_* in bits 0-1 and sim in bits 2-15.  All 32
 * lanes call. */
__device__ __forceinline__ void queue_a16(uint64_t* slab, uint32_t* s_cnt, int64_t pos0, uint32_t ei, uint32_t dead,
                                          uint4 sv, uint32_t sim) {
  if (__ballot_sync(FULLMASK, (ei | dead) != 0) == 0) return;
  uint32_t at = slab_reserve(s_cnt, __popc(ei) + __popc(dead));
  uint32_t m = ei | dead;
  while (m) {
    const int k = __ffs(m) - 1;
    m &= m - 1;
    const bool is_dead = (dead >> k) & 1u;
    const uint32_t word = k < 4 ? sv.x : k < 8 ? sv.y : k < 12 ? sv.z : sv.w;
    slab[at++] = q_entry(pos0 + k, (is_dead ? QA_DEATH : QA_DS) | (sim << 2), is_dead ? (word >> (8 * (k & 3))) : 0u);
  }
}

/* k_sweep_rs on an SIA day, one thread's 16 staged slots: the masks of the
 * agents that RI (due today) or today's SIA campaigns reach, queued with
 * their event flags. */
__device__ __forceinline__ void sweep_b16(uint64_t* slab, uint32_t* s_cnt, DevWorld& W, bool on, const DevRep* rp,
                                          uint8_t fl, int t, int ni, int64_t pos0, int off, uint4 sv,
                                          const uint8_t* scm, const int32_t* srdt, const int32_t* sdob) {
  uint32_t fri = 0;
  uint32_t fsia[LPG_MAX_SIA_PER_DAY] = {0, 0, 0, 0, 0, 0, 0, 0};
  int nsia_used = 0;
  if (on) {
    const uint32_t wv[4] = {sv.x, sv.y, sv.z, sv.w};
    const uint4 cv = *reinterpret_cast<const uint4*>(scm + off);
    const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
    /* per-byte 0xff where the agent is alive (state >= 0) and not chronically missed */
    uint32_t reachw[4];
    uint32_t any_reach = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      /* alive: sign bit clear, i.e. (byte ^ 0x80) >= 0x80 unsigned */
      const uint32_t missed = __vcmpeq4(cw[q], 0x01010101u);
      reachw[q] = __vcmpgeu4(wv[q] ^ 0x80808080u, 0x80808080u) & ~missed;
      any_reach |= reachw[q];
    }
    if (any_reach && (fl & SF_RI)) {
      /* RI on an SIA day (staged): the agents whose RI due tick is today */
      const int4* r4 = reinterpret_cast<const int4*>(srdt + off);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int4 d = r4[q];
        const int32_t dd[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) fri |= (uint32_t)(((reachw[q] >> (8 * j)) & 1u) && dd[j] == t) << (4 * q + j);
      }
    }
    if (any_reach && (fl & SF_SIA)) {
      const int4* d4 = reinterpret_cast<const int4*>(sdob + off);
      int4 dq[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) dq[q] = d4[q];
      nsia_used = rp->sia_n;
      for (int k = 0; k < nsia_used && k < LPG_MAX_SIA_PER_DAY; ++k) {
        const DevSia& ev = rp->sia[rp->sia_i0 + k];
        if (ev.mask[ni] == 0) continue;
        /* age window  min <= t - dob <= max  <=>  t - max <= dob <= t - min */
        const int64_t lo64 = (int64_t)t - ev.max_age, hi64 = (int64_t)t - ev.min_age;
        uint32_t mk = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int32_t dd[4] = {dq[q].x, dq[q].y, dq[q].z, dq[q].w};
#pragma unroll
          for (int j = 0; j < 4; ++j)
            mk |= (uint32_t)(((reachw[q] >> (8 * j)) & 1u) && (int64_t)dd[j] >= lo64 && (int64_t)dd[j] <= hi64) << (4 * q + j);
        }
        fsia[k] = mk;
      }
    }
  }
  uint32_t any = fri;
#pragma unroll
  for (int k = 0; k < LPG_MAX_SIA_PER_DAY; ++k) any |= fsia[k];
  if (__ballot_sync(FULLMASK, any != 0) == 0) return;
  uint32_t at = slab_reserve(s_cnt, __popc(any));
  while (any) {
    const int j = __ffs(any) - 1;
    any &= any - 1;
    uint32_t f = (fri >> j) & 1u;
#pragma unroll
    for (int k = 0; k < LPG_MAX_SIA_PER_DAY; ++k) f |= ((fsia[k] >> j) & 1u) << (1 + k);
    slab[at++] = q_entry(pos0 + j, f, 0);
  }
}

/* Of one thread's 16 slots (state bytes v, event ticks eq):
 * the agents in E or I whose event is at t or before (bit mask), and the
 * earliest later event among the others (LPG_NO_DOD if none).  `dead`
 * slots are left out of both. */
__device__ __forceinline__ uint32_t ev_due16(const int4* eq, uint4 v, uint32_t dead, int t, int32_t& nmin) {
  const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
  uint32_t due = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int32_t ee[4] = {eq[q].x, eq[q].y, eq[q].z, eq[q].w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = 4 * q + j;
      const uint32_t b = (wv[q] >> (8 * j)) & 0xffu;
      if ((b == 1 || b == 2) && !((dead >> k) & 1u)) {
        if (ee[j] <= t) due |= 1u << k;
        else nmin = min(nmin, ee[j]);
      }
    }
  }
  return due;
}

/* Of one thread's 16 slots at pos0 (state bytes v): the alive agents whose
 * RI due tick (rdt: LPG_NO_DOD for the chronically missed and where RI does
 * not run) is t (bit mask), and the earliest due tick after t among the
 * others (nmin, LPG_NO_DOD if none). */
__device__ __forceinline__ uint32_t ri_due16(const DevWorld& W, int64_t pos0, uint4 v, int t, int32_t& nmin) {
  const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
  if ((__vcmpltu4(wv[0], 0x80808080u) | __vcmpltu4(wv[1], 0x80808080u) | __vcmpltu4(wv[2], 0x80808080u) |
       __vcmpltu4(wv[3], 0x80808080u)) == 0)
    return 0;
  uint32_t due = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int4 d = __ldcg(reinterpret_cast<const int4*>(W.rdt + pos0) + q);
    const int32_t dd[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if ((wv[q] >> (8 * j + 7)) & 1u) continue; /* dead */
      if (dd[j] == t) due |= 1u << (4 * q + j);
      else if (dd[j] > t) nmin = min(nmin, dd[j]);
    }
  }
  return due;
}

/* Earliest value over the 8 lanes of a 128-slot sub-block (all 32 lanes call). */
__device__ __forceinline__ int32_t sub8_min(int32_t x) {
  x = min(x, __shfl_xor_sync(FULLMASK, x, 4));
  x = min(x, __shfl_xor_sync(FULLMASK, x, 2));
  return min(x, __shfl_xor_sync(FULLMASK, x, 1));
}

/* Sub-blocks with something due at this tick, the work list of
 * k_sweep_due: the index of earliest events (sub_evt) where the simulation
 * steps disease states, and on VD ticks the index of earliest dates of
 * death (sub_dod), read 4 entries per 16-byte load, four loads in flight per
 * thread over each simulation's sub-blocks.  A due sub-block is appended to
 * W.due as (sub-block | simulation << 32 | what << 48; what: 1 event, 2
 * death), one global atomic per warp. */
#define LPG_DUE_MAX 8192
#define LPG_DUE_FLAT 256 /* replicates whose index entries k_due scans as one range */
/* Due flags of 16 sub-blocks (4 index entries of 4) at tick t: 2 bits each
 * (1 event, 2 death). */
__device__ __forceinline__ uint32_t due_flags16(const int4* e, const int4* d, int t) {
  uint32_t fl = 0;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int32_t ee[4] = {e[u].x, e[u].y, e[u].z, e[u].w}, dd[4] = {d[u].x, d[u].y, d[u].z, d[u].w};
#pragma unroll
    for (int j = 0; j < 4; ++j) fl |= ((ee[j] <= t ? 1u : 0u) | (dd[j] <= t ? 2u : 0u)) << (2 * (4 * u + j));
  }
  return fl;
}
/* FLAT: the instance for a batch of replicates (the host launches it when
 * there are 2 to LPG_DUE_FLAT of them); the other scans one replicate after
 * another, with fewer registers. */
template <bool FLAT>
__global__ void __launch_bounds__(256) k_due(DevWorld W) {
  pdl_begin();
  const int lane = threadIdx.x & 31;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t gsz = (int64_t)gridDim.x * blockDim.x;
  const int4 none = make_int4(LPG_NO_DOD, LPG_NO_DOD, LPG_NO_DOD, LPG_NO_DOD);
  const int R = W.n_reps;
  if constexpr (FLAT) {
    /* the replicates' index entries as one range (a batch of small
     * simulations is one pass, not one pass each): per replicate its first
     * entry in the range, sub-block base, tick and which indexes it reads */
    __shared__ int64_t s_off[LPG_DUE_FLAT + 1], s_sb0[LPG_DUE_FLAT];
    __shared__ int32_t s_t[LPG_DUE_FLAT];
    __shared__ uint32_t s_what[LPG_DUE_FLAT];
    int64_t nq = 0;
    if (threadIdx.x < R) {
      const DevRep* rp = &W.reps[threadIdx.x];
      const uint32_t what = rp->active ? ((rp->comps & LPG_COMP_DS) ? 1u : 0u) | (rp->vd_tick ? 2u : 0u) : 0u;
      if (what) nq = (int64_t)rp->used_chunks * (LPG_NSUB / 4);
      s_sb0[threadIdx.x] = (int64_t)rp->chunk_base * LPG_NSUB;
      s_t[threadIdx.x] = rp->cur_t;
      s_what[threadIdx.x] = what;
      if (blockIdx.x == 0 && nq)
        atomicAdd(&W.ctr[LPG_CTR_SWEEP_INDEX], (unsigned long long)(nq * 4 * ((what & 1u) + (what >> 1))));
    }
    int64_t total;
    const int64_t ex = block_excl_scan(nq, &total);
    if (threadIdx.x < R) s_off[threadIdx.x] = ex;
    if (threadIdx.x == 0) s_off[R] = total;
    __syncthreads();
    const int64_t nall = total;
    for (int64_t q0 = gtid; q0 - lane < nall; q0 += 4 * gsz) {
      int4 e[4], d[4];
      int rr[4];
      int64_t ql[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t q = q0 + u * gsz;
        e[u] = none;
        d[u] = none;
        rr[u] = 0;
        ql[u] = 0;
        if (q < nall) {
          /* the replicate whose entries hold q: the last with s_off <= q */
          int lo = 0, hi = R;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_off[mid] <= q) lo = mid; else hi = mid - 1;
          }
          const int r = lo;
          rr[u] = r;
          ql[u] = q - s_off[r];
          const uint32_t what = s_what[r];
          if (what & 1u) e[u] = __ldcg(reinterpret_cast<const int4*>(W.sub_evt + s_sb0[r]) + ql[u]);
          if (what & 2u) d[u] = __ldcg(reinterpret_cast<const int4*>(W.sub_dod + s_sb0[r]) + ql[u]);
        }
      }
      uint32_t fl = 0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int32_t t = s_t[rr[u]];
        const int32_t ee[4] = {e[u].x, e[u].y, e[u].z, e[u].w}, dd[4] = {d[u].x, d[u].y, d[u].z, d[u].w};
#pragma unroll
        for (int j = 0; j < 4; ++j) fl |= ((ee[j] <= t ? 1u : 0u) | (dd[j] <= t ? 2u : 0u)) << (2 * (4 * u + j));
      }
      const uint32_t nf = __popc((fl | (fl >> 1)) & 0x55555555u);
      uint32_t x = nf;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULLMASK, x, o);
        if (lane >= o) x += y;
      }
      const uint32_t tot = __shfl_sync(FULLMASK, x, 31);
      if (tot == 0) continue;
      uint32_t base = 0;
      if (lane == 31) base = atomicAdd(W.due_n, tot);
      uint32_t at = __shfl_sync(FULLMASK, base, 31) + x - nf;
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const uint32_t f = (fl >> (2 * (4 * u + j))) & 3u;
          if (f)
            W.due[at++] = (uint64_t)(s_sb0[rr[u]] + 4 * ql[u] + j) | ((uint64_t)rr[u] << 32) | ((uint64_t)f << 48);
        }
    }
    return;
  } else {
  for (int r = 0; r < R; ++r) {
    const DevRep* rp = &W.reps[r];
    if (!rp->active) continue;
    const bool dsq = (rp->comps & LPG_COMP_DS) != 0, vd = rp->vd_tick != 0;
    if (!dsq && !vd) continue;
    const int t = rp->cur_t;
    const int64_t sb0 = (int64_t)rp->chunk_base * LPG_NSUB;
    const int64_t nq = (int64_t)rp->used_chunks * (LPG_NSUB / 4);
    if (gtid == 0) atomicAdd(&W.ctr[LPG_CTR_SWEEP_INDEX], (unsigned long long)(nq * 4 * ((dsq ? 1 : 0) + (vd ? 1 : 0))));
    for (int64_t q0 = gtid; q0 - lane < nq; q0 += 4 * gsz) {
      int4 e[4], d[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t q = q0 + u * gsz;
        e[u] = (dsq && q < nq) ? __ldcg(reinterpret_cast<const int4*>(W.sub_evt + sb0) + q) : none;
        d[u] = (vd && q < nq) ? __ldcg(reinterpret_cast<const int4*>(W.sub_dod + sb0) + q) : none;
      }
      const uint32_t fl = due_flags16(e, d, t);
      const uint32_t nf = __popc((fl | (fl >> 1)) & 0x55555555u);
      uint32_t x = nf;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULLMASK, x, o);
        if (lane >= o) x += y;
      }
      const uint32_t tot = __shfl_sync(FULLMASK, x, 31);
      if (tot == 0) continue;
      uint32_t base = 0;
      if (lane == 31) base = atomicAdd(W.due_n, tot);
      uint32_t at = __shfl_sync(FULLMASK, base, 31) + x - nf;
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const uint32_t f = (fl >> (2 * (4 * u + j))) & 3u;
          if (f) W.due[at++] = (uint64_t)(sb0 + 4 * (q0 + u * gsz) + j) | ((uint64_t)r << 32) | ((uint64_t)f << 48);
        }
    }
  }
  }
}


/* k_sweep_rs on an RI tick without SIA, over one simulation's sub-blocks
 * [sb0, sb0 + nsb), in windows of LPG_DUE_MAX sub-blocks: the CTA lists the
 * sub-blocks whose earliest RI due tick (sub_rdt) has come, then 8 lanes
 * per listed sub-block queue the agents due now (fast_ri, model.py:1825-1854:
 * alive, not chronically missed, the subtraction landing in the window) and
 * write the sub-block's next due tick.  No timer is written: the column
 * keeps each agent's base (lpg_ri.h).  All threads of the CTA run it. */
__device__ __noinline__ void ri_direct(DevWorld& W, const DevRep* rp, uint64_t* slab, uint32_t* s_cnt, int64_t sb0,
                                       int64_t nsb, int t, uint32_t* s_due, int* s_ndue) {
  const int lane = threadIdx.x & 31;
  uint32_t n_due = 0;
  for (int64_t wb = 0; wb < nsb; wb += LPG_DUE_MAX) {
    const int nw = (int)min((int64_t)LPG_DUE_MAX, nsb - wb);
    if (threadIdx.x == 0) {
      *s_ndue = 0;
      atomicAdd(&W.ctr[LPG_CTR_RI_INDEX], (unsigned long long)nw);
    }
    __syncthreads();
    for (int q = threadIdx.x * 4; q < nw; q += blockDim.x * 4) {
      const int4 e4 = __ldcg(reinterpret_cast<const int4*>(W.sub_rdt + sb0 + wb + q));
      const int32_t ee[4] = {e4.x, e4.y, e4.z, e4.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (ee[j] <= t && q + j < nw) {
          const int at = atomicAdd(s_ndue, 1);
          s_due[at] = (uint32_t)(q + j);
        }
      }
    }
    __syncthreads();
    const int ndue = *s_ndue;
    const int per_pass = (blockDim.x / 32) * 4;
    for (int base = 0; base < ndue; base += per_pass) {
      const int item = base + (threadIdx.x >> 5) * 4 + (lane >> 3);
      const bool on = item < ndue;
      const int64_t sb = sb0 + wb + (on ? s_due[item] : 0u);
      const int64_t pos0 = sb * LPG_SUB + (int64_t)(lane & 7) * 16;
      int32_t nmin = LPG_NO_DOD;
      uint32_t due = 0;
      if (on) {
        n_due += (lane & 7) == 0 ? 1u : 0u;
        due = ri_due16(W, pos0, ldg_stream16(W.ds + pos0), t, nmin);
      }
      nmin = sub8_min(nmin);
      if (on && (lane & 7) == 0) W.sub_rdt[sb] = nmin;
      if (__ballot_sync(FULLMASK, due != 0)) {
        uint32_t at = slab_reserve(s_cnt, __popc(due));
        while (due) {
          const int k = __ffs(due) - 1;
          due &= due - 1;
          slab[at++] = q_entry(pos0 + k, QB_RI, 0);
        }
      }
    }
    __syncthreads();
  }
  n_due = __reduce_add_sync(FULLMASK, n_due);
  if (lane == 0 && n_due) atomicAdd(&W.ctr[LPG_CTR_RI_DUE], (unsigned long long)n_due);
}

/* The first work item at or after w whose simulation is staged (dense), or w1. */
__device__ __forceinline__ int32_t dense_from(const SweepPlan& P, int32_t w, int32_t w1) {
  while (w < w1) {
    int lo = 0, hi = P.nreps - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (P.off[mid] <= w) lo = mid; else hi = mid - 1;
    }
    if (P.flags[lo] & SF_DENSE) return w;
    w = min(w1, P.off[lo + 1]);
  }
  return w1;
}

__global__ void __launch_bounds__(LPG_SWEEP_BLOCK) k_sweep_rs(DevWorld W) {
  pdl_begin();
  extern __shared__ __align__(128) uint8_t sm_stage[];
  __shared__ SweepPlan P;
  __shared__ __align__(8) uint64_t full[LPG_NST];
  __shared__ __align__(8) uint64_t empty[LPG_NST];
  __shared__ uint32_t s_qcnt;
  __shared__ int32_t s_issued;
  __shared__ int s_ndue;
  __shared__ volatile int s_abort;
  const int R = W.n_reps < LPG_MAX_REPS ? W.n_reps : LPG_MAX_REPS;
  if (threadIdx.x == 0) {
    int32_t acc = 0;
    for (int r = 0; r < R; ++r) {
      P.off[r] = acc;
      const DevRep* rp = &W.reps[r];
      uint8_t f = 0;
      if (rp->active) {
        if (rp->ri_tick) f |= SF_RI;
        if (rp->sia_n > 0) f |= SF_SIA;
        if (f) f |= SF_WORK;
        if (f & SF_SIA) f |= SF_DENSE; /* RI alone: through the due index */
      }
      P.flags[r] = f;
      P.cbase[r] = rp->chunk_base;
      P.tick[r] = rp->cur_t;
      acc += (f & SF_WORK) ? rp->used_chunks : 0;
    }
    P.off[R] = acc;
    P.total = acc;
    P.nreps = R;
    s_qcnt = 0;
    s_issued = 0;
    s_abort = 0;
    for (int b = 0; b < LPG_NST; ++b) {
      mbar_init(&full[b], 1);
      mbar_init(&empty[b], LPG_SWEEP_CONSUMERS / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int32_t total = P.total;
  const int32_t per = (total + gridDim.x - 1) / gridDim.x;
  const int32_t w0 = min((int32_t)blockIdx.x * per, total);
  const int32_t w1 = min(w0 + per, total);
  uint64_t* slab = W.evq + (int64_t)w0 * LPG_CHUNK;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  {
    /* Simulations with RI today and no SIA: the due sub-blocks only
     * (ri_direct), all threads, with the list in the stage buffers before
     * any bulk copy reaches them. */
    int32_t w = w0;
    while (w < w1) {
      int r;
      (void)stage_end(P, w, w1, &r);
      const int32_t we = min(w1, P.off[r + 1]);
      if ((P.flags[r] & (SF_WORK | SF_DENSE)) == SF_WORK) {
        const int64_t sb0 = (P.cbase[r] + (int64_t)(w - P.off[r])) * LPG_NSUB;
        ri_direct(W, &W.reps[r], slab, &s_qcnt, sb0, (int64_t)(we - w) * LPG_NSUB, P.tick[r],
                  reinterpret_cast<uint32_t*>(sm_stage), &s_ndue);
      }
      w = we;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
  }
  if (warp == LPG_SWEEP_CONSUMERS / 32) {
    /* ---- producer warp: one lane issues the stages ---- */
    if (lane == 0 && w0 < w1) {
      int32_t wp = dense_from(P, w0, w1);
      int32_t i = 0;
      for (; wp < w1; ++i) {
        const int b = i % LPG_NST;
        if (i >= LPG_NST && !mbar_wait(&empty[b], (uint32_t)((i / LPG_NST) - 1) & 1u)) {
          s_abort = 1;
          break;
        }
        if (s_abort) break;
        if (W.stall_after >= 0 && i >= W.stall_after) break; /* test hook: withhold the rest */
        int r;
        const int32_t we = stage_end(P, wp, w1, &r);
        const uint8_t f = P.flags[r];
        const int64_t cid = P.cbase[r] + (wp - P.off[r]);
        const int nc = we - wp;
        const StageLayout L = stage_layout(f, nc);
        uint8_t* dst = sm_stage + (size_t)b * LPG_STAGE_BYTES;
        uint8_t* cols = dst + LPG_META_BYTES;
        const uint32_t bytes = (uint32_t)nc * 16u + (uint32_t)nc * (uint32_t)chunk_bytes(f);
        if (i >= LPG_NST) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&full[b], bytes);
        bulk_g2s(dst, W.cmeta + cid, (uint32_t)nc * 16u, &full[b]);
        bulk_g2s(cols + L.ds, W.ds + cid * LPG_CHUNK, (uint32_t)nc * LPG_CHUNK, &full[b]);
        if (f & SF_RI) bulk_g2s(cols + L.rdt, W.rdt + cid * LPG_CHUNK, (uint32_t)nc * 4 * LPG_CHUNK, &full[b]);
        if (f & (SF_RI | SF_SIA)) bulk_g2s(cols + L.cm, W.cm + cid * LPG_CHUNK, (uint32_t)nc * LPG_CHUNK, &full[b]);
        if (f & SF_SIA) bulk_g2s(cols + L.dob, W.dob + cid * LPG_CHUNK, (uint32_t)nc * 4 * LPG_CHUNK, &full[b]);
        wp = dense_from(P, we, w1);
      }
      s_issued = i;
    }
  } else if (w0 < w1) {
    /* ---- consumer warps: 16-slot groups of the stage, 256 groups per pass ---- */
    int32_t wc = dense_from(P, w0, w1);
    for (int32_t i = 0; wc < w1; ++i) {
      const int b = i % LPG_NST;
      const uint32_t parity = (uint32_t)(i / LPG_NST) & 1u;
      int r;
      const int32_t we = stage_end(P, wc, w1, &r);
      bool ok = !s_abort && mbar_wait(&full[b], parity, W.wait_spin);
      ok = __all_sync(FULLMASK, ok);
      if (!ok) {
        s_abort = 1;
        break;
      }
      const DevRep* rp = &W.reps[r];
      const uint8_t fl = P.flags[r];
      const int t = P.tick[r];
      const uint8_t* stg = sm_stage + (size_t)b * LPG_STAGE_BYTES;
      const int4* meta = reinterpret_cast<const int4*>(stg);
      const uint8_t* cols = stg + LPG_META_BYTES;
      const int nc = we - wc;
      const StageLayout L = stage_layout(fl, nc);
      const int ngroups = nc * (LPG_CHUNK / 16);
      for (int gb = 0; gb < ngroups; gb += LPG_SWEEP_CONSUMERS) {
        const int gi = gb + threadIdx.x;
        const bool on = gi < ngroups;
        const int kk = on ? gi / (LPG_CHUNK / 16) : 0;
        const int off = on ? (gi % (LPG_CHUNK / 16)) * 16 : 0;
        const int64_t cid = P.cbase[r] + (wc + kk - P.off[r]);
        const int64_t pos0 = cid * LPG_CHUNK + off;
        /* slots past a chunk's fill hold state -1 (never alive), so they drop
         * out of every test below without a fill check */
        const uint4 sv = on ? *reinterpret_cast<const uint4*>(cols + L.ds + kk * LPG_CHUNK + off)
                            : make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
        const int ni = meta[kk].x - rp->node_base;
        sweep_b16(slab, &s_qcnt, W, on, rp, fl, t, ni, pos0, off, sv, cols + L.cm + kk * LPG_CHUNK,
                  reinterpret_cast<const int32_t*>(cols + L.rdt + kk * 4 * LPG_CHUNK),
                  reinterpret_cast<const int32_t*>(cols + L.dob + kk * 4 * LPG_CHUNK));
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[b]);
      wc = dense_from(P, we, w1);
    }
  }
  __syncthreads();
  if (s_abort && threadIdx.x == LPG_SWEEP_CONSUMERS) {
    /* the error goes to every simulation whose staged chunks this CTA was
     * sweeping (RI-only simulations take the due index, not the stages);
     * then leave no bulk copy in flight into this CTA's shared memory (the
     * drain waits on the normal limit) */
    for (int r = 0; r < P.nreps; ++r)
      if ((P.flags[r] & SF_DENSE) && P.off[r] < w1 && P.off[r + 1] > w0) W.reps[r].error = LPG_ERR_TIMEOUT;
    const int32_t n = s_issued;
    for (int b = 0; b < LPG_NST; ++b) {
      int32_t last = -1;
      for (int32_t j = b; j < n; j += LPG_NST) last = j;
      if (last >= 0) mbar_wait(&full[b], (uint32_t)(last / LPG_NST) & 1u);
    }
  }
  if (threadIdx.x == 0) {
    W.qcnt[1024 + blockIdx.x] = s_qcnt;
    W.qfirst[1024 + blockIdx.x] = (uint32_t)w0 * LPG_CHUNK;
  }
}

/* ------------------------------------------------------------------------ */
/* Queue kernels: one thread per queued agent.  The queue is one slab per CTA
 * of the sweep; entries of a warp mostly belong to one node, so node counters
 * are summed across the lanes that share a node before the global atomics. */
__device__ __forceinline__ void warp_add(int32_t* p, unsigned peers, int32_t v) {
  const int32_t tot = __reduce_add_sync(peers, v);
  if ((threadIdx.x & 31) == __ffs(peers) - 1 && tot) atomicAdd(p, tot);
}
/* Sum of 64-bit values over the lanes of peers, exact modulo 2^64 (four
 * 16-bit parts, each summed in 32 bits without overflow). */
__device__ __forceinline__ uint64_t warp_sum_u64(unsigned peers, uint64_t w) {
  uint64_t tot = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    tot += (uint64_t)__reduce_add_sync(peers, (uint32_t)((w >> (16 * k)) & 0xffffu)) << (16 * k);
  return tot;
}
/* The lowest lane of peers subtracts the peers' total weight from *p. */
__device__ __forceinline__ void warp_sub_w(unsigned long long* p, unsigned peers, uint64_t w) {
  const uint64_t tot = warp_sum_u64(peers, w);
  if ((threadIdx.x & 31) == __ffs(peers) - 1 && tot) atomicAdd(p, neg64(tot));
}

/* Entry q of the queue of k_sweep_rs (prefix of the slab sizes in s_pre). */
__device__ __forceinline__ uint64_t q_get(const DevWorld& W, int phase, const uint32_t* s_pre, int nslabs, uint32_t q) {
  int lo = 0, hi = nslabs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (s_pre[mid] <= q) lo = mid; else hi = mid - 1;
  }
  return W.evq[(int64_t)W.qfirst[phase * 1024 + lo] + (q - s_pre[lo])];
}

__device__ __forceinline__ uint32_t q_prefix(const DevWorld& W, int phase, uint32_t* s_pre, int nslabs) {
  int64_t carry = 0;
  for (int base = 0; base < nslabs; base += blockDim.x) {
    const int b = base + threadIdx.x;
    const int64_t v = b < nslabs ? W.qcnt[phase * 1024 + b] : 0;
    int64_t tot;
    const int64_t ex = block_excl_scan(v, &tot);
    if (b < nslabs) s_pre[b] = (uint32_t)(carry + ex);
    carry += tot;
  }
  if (threadIdx.x == 0) s_pre[nslabs] = (uint32_t)carry;
  __syncthreads();
  return s_pre[nslabs];
}

/* One entry e of k_sweep_due's queue (on: the lane has one; all 32 lanes of
 * the warp call): death bookkeeping (get_deaths, model.py:1767-1781) or the
 * disease-state step of an agent whose event is now
 * (disease_state_step_kernel, model.py:393-454), node totals summed per
 * warp before the atomics. */
__device__ __forceinline__ void ds_queue_step(DevWorld& W, uint64_t e, bool on) {
  const int64_t G = W.G;
  int g = -1, st = 0;
  int32_t dS = 0, dE = 0, dI = 0, dR = 0, dPP = 0, dP = 0, nPP = 0, nP = 0, nDead = 0;
  if (on) {
    const int64_t pos = (int64_t)(uint32_t)e;
    const uint32_t kind = (uint32_t)(e >> 32) & 3u;
    const int64_t cid = pos / LPG_CHUNK;
    g = W.cmeta[cid].x;
    const DevRep* rp = &W.reps[(e >> 34) & 0x3fffu]; /* the simulation, carried by the entry */
    const int t = rp->cur_t;
    if (kind == QA_DEATH) {
      const int8_t s = (int8_t)(uint8_t)(e >> 48);
      nDead = 1;
      if (s == 0) {
        dS = -1;
        const uint64_t w = fix_risk(W.risk[pos]);
        if (w) {
          atomicAdd((unsigned long long*)&W.sw[g], neg64(w));
          atomicAdd((unsigned long long*)&W.chunk_w[cid], neg64(w));
          atomicAdd((unsigned long long*)&W.sub_w[cid * LPG_NSUB + (pos % LPG_CHUNK) / LPG_SUB], neg64(w));
        }
      } else if (s == 1 || s == 2) {
        st = W.strain[pos];
        if (s == 1) {
          dE = -1;
        } else {
          dI = -1;
          const uint64_t bw = fix_beta(W.inf[pos], rp->strain_scal[st]);
          if (bw) atomicAdd((unsigned long long*)&W.bb[(int64_t)st * G + g], neg64(bw));
        }
        /* timers frozen at death: brought up to the step of t - 1 (they
         * count down only where disease states are stepped) */
        int8_t et = W.et[pos], it = W.it[pos], pt = W.pt[pos];
        const int k = (rp->comps & LPG_COMP_DS) ? t - W.evt[pos] + ev_pure(s, (int8_t)st, et, it, pt, W.pp[pos]) : 0;
        if (k > 0) {
          ev_advance(s, (int8_t)st, et, it, pt, k);
          if (s == 1) W.et[pos] = et;
          else {
            W.it[pos] = it;
            if (st == 0) W.pt[pos] = pt;
          }
        }
      } else if (s == 3) {
        dR = -1;
      }
      /* the RI timer stops at death: its value after the RI ticks before t */
      if (ri_runs(rp) && W.cm[pos] != 1) W.ri[pos] = ri_now(rp, W.ri[pos], W.ref[pos], W.dob[pos], t - 1);
      if (W.pp[pos] == 1) dPP -= 1;
      if (W.par[pos] == 1) dP -= 1;
    } else {
      /* an event step of an agent in E or I (its evt is t) */
      const int8_t s0 = W.ds[pos];
      int8_t s = s0;
      st = W.strain[pos];
      int8_t et = W.et[pos], it = W.it[pos], pt = W.pt[pos], pp = W.pp[pos];
      /* the count-downs skipped since the timers were last brought up to date */
      ev_advance(s0, (int8_t)st, et, it, pt, t - W.evt[pos] + ev_pure(s0, (int8_t)st, et, it, pt, pp));
      if (s == 1) {
        if (et <= 0) {
          s = 2;
          dE -= 1;
          dI += 1;
          const uint64_t bw = fix_beta(W.inf[pos], rp->strain_scal[st]);
          if (bw) atomicAdd((unsigned long long*)&W.bb[(int64_t)st * G + g], (unsigned long long)bw);
        }
        et = dec_i8(et);
        W.et[pos] = et;
      }
      if (s == 2) {
        if (it <= 0) {
          s = 3;
          dI -= 1;
          dR += 1;
          const uint64_t bw = fix_beta(W.inf[pos], rp->strain_scal[st]);
          if (bw) atomicAdd((unsigned long long*)&W.bb[(int64_t)st * G + g], neg64(bw));
        }
        it = dec_i8(it);
        W.it[pos] = it;
        if (st == 0) {
          if (pt <= 0 && pp == -1) {
            if (W.ipv[pos] == 0) {
              pp = 1;
              dPP += 1;
              nPP += 1;
              if (lpg_u53(rp->seed, LPG_P_PARALYSIS, t, W.ref[pos], 0, 0) < rp->thr_par) {
                W.par[pos] = 1;
                dP += 1;
                nP += 1;
              }
            } else {
              pp = 0;
            }
            W.pp[pos] = pp;
          }
          pt = dec_i8(pt);
          W.pt[pos] = pt;
        }
      }
      if (s != s0) W.ds[pos] = s;
      if (s == 1 || s == 2) {
        const int32_t e1 = t + 1 + ev_pure(s, (int8_t)st, et, it, pt, pp);
        W.evt[pos] = e1;
        atomicMin(&W.sub_evt[pos >> 7], e1);
      }
    }
  }
  /* nothing to add when every delta of the warp is zero */
  const bool any = on && (dS | dE | dI | dR | dPP | dP | nPP | nP | nDead);
  const unsigned act = __ballot_sync(FULLMASK, any);
  if (!any) return;
  const unsigned by_node = __match_any_sync(act, g);
  warp_add(&W.ev[(int64_t)EV_DEATHS * G + g], by_node, nDead);
  warp_add(&W.tot[(int64_t)TT_S * G + g], by_node, dS);
  warp_add(&W.tot[(int64_t)TT_R * G + g], by_node, dR);
  warp_add(&W.tot[(int64_t)TT_POTP * G + g], by_node, dPP);
  warp_add(&W.tot[(int64_t)TT_P * G + g], by_node, dP);
  warp_add(&W.ev[(int64_t)EV_NEWPOT * G + g], by_node, nPP);
  warp_add(&W.ev[(int64_t)EV_NEWPAR * G + g], by_node, nP);
  const unsigned by_ns = __match_any_sync(act, g * LPG_MAX_STRAINS + st);
  warp_add(&W.tot[(int64_t)(TT_E0 + st) * G + g], by_ns, dE);
  warp_add(&W.tot[(int64_t)(TT_I0 + st) * G + g], by_ns, dI);
}


/* The due sub-blocks of W.due, split evenly over the CTAs (an outbreak makes
 * most sub-blocks of a few nodes due while most others have none), 8 lanes
 * per sub-block (16 slots each): state bytes, the dates of death when a
 * death is due and the event ticks when an event is due.  Deaths
 * (model.py:1767-1781; this tick's newborns are not checked), the queue of
 * the agents whose event is now, and the sub-block's new earliest event
 * and date of death over the rest, with no atomics; then the steps of the
 * queued agents (ds_queue_step).  A CTA's queue slab starts at its first
 * item times 128 entries of evq. */
__global__ void __launch_bounds__(LPG_SWEEP_BLOCK) k_sweep_due(DevWorld W) {
  pdl_begin();
  __shared__ uint32_t s_qcnt;
  const int lane = threadIdx.x & 31;
  const int64_t D = (int64_t)*(volatile uint32_t*)W.due_n;
  const int64_t i0 = D * blockIdx.x / gridDim.x, i1 = D * (blockIdx.x + 1) / gridDim.x;
  uint64_t* slab = W.evq + i0 * LPG_SUB;
  if (threadIdx.x == 0) s_qcnt = 0;
  __syncthreads();
  uint32_t n_due = 0, n_edue = 0, n_ddue = 0; /* work counters, lanes (lane & 7) == 0 */
  const int per_pass = (blockDim.x / 32) * 4;
  for (int64_t base = i0; base < i1; base += per_pass) {
    const int64_t item = base + (threadIdx.x >> 5) * 4 + (lane >> 3);
    const bool on = item < i1;
    const uint64_t rec = on ? __ldcg(W.due + item) : 0ULL;
    const int64_t sb = (int64_t)(uint32_t)rec;
    const uint32_t f = (uint32_t)(rec >> 48);
    const bool edue = (f & 1u) != 0, ddue = (f & 2u) != 0;
    const int t = on ? W.reps[(rec >> 32) & 0xffffu].cur_t : 0;
    if (on && (lane & 7) == 0) {
      n_due += 1;
      n_edue += edue ? 1 : 0;
      n_ddue += ddue ? 1 : 0;
    }
    const int64_t pos0 = sb * LPG_SUB + (int64_t)(lane & 7) * 16;
    const uint4 v = on ? ldg_stream16(W.ds + pos0) : make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
    /* the event ticks requested with the state bytes, before the deaths */
    int4 eq[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) eq[q] = edue ? __ldcg(reinterpret_cast<const int4*>(W.evt + pos0) + q) : make_int4(0, 0, 0, 0);
    uint32_t dead = 0;
    if (__ballot_sync(FULLMASK, ddue)) {
      int32_t nmin = LPG_NO_DOD;
      if (ddue) {
        const int4* d4 = reinterpret_cast<const int4*>(W.dod + pos0);
        int4 dq[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) dq[q] = d4[q];
        const int4 m = W.cmeta[pos0 >> 11];
        const int off = (int)(pos0 & (LPG_CHUNK - 1));
        const int nbo = (m.z == t) ? m.w : LPG_CHUNK; /* this tick's newborns are not checked */
        const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int32_t dd[4] = {dq[q].x, dq[q].y, dq[q].z, dq[q].w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int k = 4 * q + j;
            const bool alive = ((wv[q] >> (8 * j + 7)) & 1u) == 0;
            const bool dies = alive && dd[j] <= t && off + k < nbo;
            dead |= (uint32_t)dies << k;
            if (alive && !dies) nmin = min(nmin, dd[j]);
          }
        }
        if (dead) {
          uint4 out = v;
          uint32_t* ow = reinterpret_cast<uint32_t*>(&out);
#pragma unroll
          for (int k = 0; k < 16; ++k)
            if ((dead >> k) & 1u) ow[k >> 2] |= 0xffu << (8 * (k & 3));
          *reinterpret_cast<uint4*>(W.ds + pos0) = out;
        }
      }
      nmin = sub8_min(nmin);
      if (ddue && (lane & 7) == 0) W.sub_dod[sb] = nmin;
    }
    uint32_t ei = 0;
    if (__ballot_sync(FULLMASK, edue)) {
      int32_t nmin = LPG_NO_DOD;
      if (edue) ei = ev_due16(eq, v, dead, t, nmin);
      nmin = sub8_min(nmin);
      /* the agents due now get their next event in ds_queue_step (atomicMin) */
      if (edue && (lane & 7) == 0) W.sub_evt[sb] = nmin;
    }
    queue_a16(slab, &s_qcnt, pos0, ei, dead, v, (uint32_t)(rec >> 32) & 0x3fffu);
  }
  n_due = __reduce_add_sync(FULLMASK, n_due);
  n_edue = __reduce_add_sync(FULLMASK, n_edue);
  n_ddue = __reduce_add_sync(FULLMASK, n_ddue);
  if (lane == 0 && n_due) {
    atomicAdd(&W.ctr[LPG_CTR_SWEEP_DUE], (unsigned long long)n_due);
    atomicAdd(&W.ctr[LPG_CTR_SWEEP_EVT_DUE], (unsigned long long)n_edue);
    atomicAdd(&W.ctr[LPG_CTR_SWEEP_DOD_DUE], (unsigned long long)n_ddue);
  }
  /* the CTA's own queue: its sub-blocks are its alone, so the steps need
   * no other CTA's sweep (the index entries it wrote above come first) */
  __syncthreads();
  const uint32_t n = s_qcnt;
  if (threadIdx.x == 0 && n) atomicAdd(&W.ctr[LPG_CTR_QUEUE_DS], (unsigned long long)n);
  for (uint32_t b = 0; b < n; b += blockDim.x) {
    const uint32_t q = b + threadIdx.x;
    ds_queue_step(W, q < n ? slab[q] : 0ULL, q < n);
  }
}

/* Queue of k_sweep_rs: the draws of RI (fast_ri, model.py:1845-1854) and of
 * the SIA campaigns of the day (fast_sia, :2047-2059), in that order per
 * agent.  Probability tests are integer compares of the 53-bit draw with
 * precomputed thresholds (same outcome as the double compares). */
__global__ void __launch_bounds__(256) k_evb(DevWorld W, int nslabs) {
  pdl_begin();
  __shared__ uint32_t s_pre[1025];
  {
    /* nothing queued unless some simulation has RI or SIA work today */
    int any = 0;
    for (int r = 0; r < W.n_reps && !any; ++r)
      any = W.reps[r].active && (W.reps[r].ri_tick || W.reps[r].sia_n > 0);
    if (!any) return;
  }
  const uint32_t n = q_prefix(W, 1, s_pre, nslabs);
  if (blockIdx.x == 0 && threadIdx.x == 0 && n) atomicAdd(&W.ctr[LPG_CTR_QUEUE_RS], (unsigned long long)n);
  const int64_t G = W.G;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const uint32_t q = base + threadIdx.x;
    const bool on = q < n;
    int g = -1;
    int32_t rivac = 0, riprot = 0, ipvvac = 0, dS = 0;
    int32_t dE[LPG_MAX_STRAINS] = {0, 0, 0, 0};
    int32_t sv[LPG_MAX_SIA_PER_DAY] = {0, 0, 0, 0, 0, 0, 0, 0};
    int32_t sp[LPG_MAX_SIA_PER_DAY] = {0, 0, 0, 0, 0, 0, 0, 0};
    int nsia = 0;
    /* an exposure's next event tick and weight, summed per sub-block, chunk
     * and node over the warp before the atomics */
    int32_t ex_e1 = LPG_NO_DOD;
    uint64_t ex_w = 0;
    int64_t ex_pos = 0;
    if (on) {
      const uint64_t e = q_get(W, 1, s_pre, nslabs, q);
      const int64_t pos = (int64_t)(uint32_t)e;
      const uint32_t fl = (uint32_t)(e >> 32) & 0xffffu;
      const int64_t cid = pos / LPG_CHUNK;
      g = W.cmeta[cid].x;
      const DevRep* rp = &W.reps[W.node_rep[g]];
      const int t = rp->cur_t, ni = g - rp->node_base;
      const uint32_t ref = W.ref[pos];
      int8_t s = W.ds[pos];
      const int8_t s_in = s;
      bool exposed = false;
      if (fl & QB_RI) {
        if (lpg_u53(rp->seed, LPG_P_RI, t, ref, 0, 0) < rp->thr_ri[ni]) {
          rivac = 1;
          if (s == 0) {
            s = 1;
            W.strain[pos] = (int8_t)rp->ri_strain;
            riprot = 1;
            dE[rp->ri_strain] += 1;
            exposed = true;
          }
        }
        if (lpg_u53(rp->seed, LPG_P_RI, t, ref, 0, 1) < rp->thr_ipv[ni]) {
          ipvvac = 1;
          W.ipv[pos] = 1;
        }
      }
      nsia = rp->sia_n;
#pragma unroll
      for (int k = 0; k < LPG_MAX_SIA_PER_DAY; ++k) {
        if (k >= nsia) break;
        if (!((fl >> (1 + k)) & 1u)) continue;
        const DevSia& ev = rp->sia[rp->sia_i0 + k];
        const uint64_t r = lpg_u53(rp->seed, LPG_P_SIA, t, ref, 0, (uint64_t)k);
        if (r < ev.thr_vac[ni]) {
          sv[k] = 1;
          if (s == 0 && r < ev.thr_pro[ni]) {
            s = 1;
            W.strain[pos] = (int8_t)ev.strain;
            sp[k] = 1;
            dE[ev.strain] += 1;
            exposed = true;
          }
        }
      }
      if (exposed) {
        dS = -1;
        const int8_t et = W.et[pos];
        ex_e1 = t + 1 + (et > 0 ? et : 0);
        W.evt[pos] = ex_e1;
        ex_w = fix_risk(W.risk[pos]);
      }
      if (s != s_in) W.ds[pos] = s;
      ex_pos = pos;
    }
    const unsigned act = __ballot_sync(FULLMASK, on);
    if (!on) continue;
    const unsigned by_node = __match_any_sync(act, g);
    if (__any_sync(act, ex_e1 != LPG_NO_DOD)) {
      const uint32_t sb = (uint32_t)(ex_pos >> 7), ch = (uint32_t)(ex_pos / LPG_CHUNK);
      const unsigned by_sub = __match_any_sync(act, sb);
      const unsigned by_chunk = __match_any_sync(act, ch);
      const int32_t emin = __reduce_min_sync(by_sub, ex_e1);
      if ((int)(threadIdx.x & 31) == __ffs(by_sub) - 1 && emin != LPG_NO_DOD) atomicMin(&W.sub_evt[sb], emin);
      warp_sub_w((unsigned long long*)&W.sub_w[sb], by_sub, ex_w);
      warp_sub_w((unsigned long long*)&W.chunk_w[ch], by_chunk, ex_w);
      warp_sub_w((unsigned long long*)&W.sw[g], by_node, ex_w);
    }
    warp_add(&W.ev[(int64_t)EV_RIVAC * G + g], by_node, rivac);
    warp_add(&W.ev[(int64_t)EV_RIPROT * G + g], by_node, riprot);
    warp_add(&W.ev[(int64_t)EV_IPVVAC * G + g], by_node, ipvvac);
    warp_add(&W.tot[(int64_t)TT_S * G + g], by_node, dS);
#pragma unroll
    for (int k = 0; k < LPG_MAX_STRAINS; ++k) warp_add(&W.tot[(int64_t)(TT_E0 + k) * G + g], by_node, dE[k]);
    const int ns_max = __reduce_max_sync(by_node, nsia);
#pragma unroll
    for (int k = 0; k < LPG_MAX_SIA_PER_DAY; ++k) {
      if (k >= ns_max) break;
      warp_add(&W.ev[(int64_t)(EV_SIAVAC0 + k) * G + g], by_node, sv[k]);
      warp_add(&W.ev[(int64_t)(EV_SIAPROT0 + k) * G + g], by_node, sp[k]);
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Seed schedule: one CTA per simulation, events of the tick in order. */
__global__ void __launch_bounds__(1024) k_seed(DevWorld W) {
  pdl_begin();
  const DevRep* rp = &W.reps[blockIdx.x];
  if (!rp->active || rp->seed_n == 0) return;
  const int t = rp->cur_t, nb = rp->node_base, G = W.G;
  const int32_t* st = W.node_chunk_start[rp->csr_cur] + rp->csr_base;
  const int32_t* ls = W.node_chunks[rp->csr_cur] + rp->chunk_base;
  __shared__ unsigned long long s_cnt;
  __shared__ unsigned int hist[256];
  __shared__ uint64_t s_prefix;
  __shared__ int64_t s_need;
  __shared__ unsigned long long s_ties;
  __shared__ int s_ntie;
  __shared__ uint32_t s_tie_ref[64];
  __shared__ int64_t s_tie_pos[64];
  for (int e = rp->seed_i0; e < rp->seed_i0 + rp->seed_n; ++e) {
    const DevSeed ev = rp->seeds[e];
    const int ni = ev.node;
    if (ni < 0 || ni >= rp->n_nodes) continue;
    const int g = nb + ni;
    const int64_t nslots = W.node_count[g];
    const int32_t c0 = st[ni];
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    unsigned long long local = 0;
    for (int64_t li = threadIdx.x; li < nslots; li += blockDim.x) {
      int64_t pos = (int64_t)ls[c0 + li / LPG_CHUNK] * LPG_CHUNK + li % LPG_CHUNK;
      local += W.ds[pos] >= 0;
    }
    atomicAdd(&s_cnt, local);
    __syncthreads();
    const int64_t N = (int64_t)s_cnt;
    int64_t nseed = ev.is_count ? (int64_t)ev.value : (int64_t)((double)N * ev.value);
    if (ev.is_count && nseed > N) nseed = N;
    if (nseed <= 0) {
      __syncthreads();
      continue;
    }
    /* radix select of the nseed-th smallest key among the candidates */
    if (threadIdx.x == 0) {
      s_prefix = 0;
      s_need = nseed;
    }
    __syncthreads();
    const bool all = nseed >= N;
    if (!all) {
      for (int shift = 56; shift >= 0; shift -= 8) {
        for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
        __syncthreads();
        const uint64_t hmask = shift == 56 ? 0ULL : (~0ULL << (shift + 8));
        const uint64_t pre = s_prefix;
        for (int64_t li = threadIdx.x; li < nslots; li += blockDim.x) {
          int64_t pos = (int64_t)ls[c0 + li / LPG_CHUNK] * LPG_CHUNK + li % LPG_CHUNK;
          if (W.ds[pos] < 0) continue;
          uint64_t key = lpg_raw(rp->seed, LPG_P_SEEDPICK, t, W.ref[pos], (uint64_t)ev.pad, 0);
          if ((key & hmask) == (pre & hmask)) atomicAdd(&hist[(key >> shift) & 255], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          int64_t need = s_need, cum = 0;
          int b = 0;
          for (; b < 256; ++b) {
            if (cum + hist[b] >= need) break;
            cum += hist[b];
          }
          s_prefix = pre | ((uint64_t)b << shift);
          s_need = need - cum;
        }
        __syncthreads();
      }
    }
    const uint64_t kstar = s_prefix;
    const int64_t need_ties = s_need;
    /* ties on the threshold key: keep the lowest reference slots */
    if (threadIdx.x == 0) {
      s_ties = 0;
      s_ntie = 0;
    }
    __syncthreads();
    if (!all) {
      for (int64_t li = threadIdx.x; li < nslots; li += blockDim.x) {
        int64_t pos = (int64_t)ls[c0 + li / LPG_CHUNK] * LPG_CHUNK + li % LPG_CHUNK;
        if (W.ds[pos] < 0) continue;
        uint64_t key = lpg_raw(rp->seed, LPG_P_SEEDPICK, t, W.ref[pos], (uint64_t)ev.pad, 0);
        if (key == kstar) {
          unsigned long long k = atomicAdd(&s_ties, 1ULL);
          if (k < 64) {
            s_tie_ref[k] = W.ref[pos];
            s_tie_pos[k] = pos;
          }
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0 && !all) {
      int nt_ = (int)(s_ties < 64 ? s_ties : 64);
      if (s_ties > 64) W.reps[blockIdx.x].error = LPG_ERR_INTERNAL;
      /* order the ties by reference slot (insertion sort, at most 64) */
      for (int a = 1; a < nt_; ++a) {
        uint32_t rk = s_tie_ref[a];
        int64_t pk = s_tie_pos[a];
        int b = a - 1;
        while (b >= 0 && s_tie_ref[b] > rk) {
          s_tie_ref[b + 1] = s_tie_ref[b];
          s_tie_pos[b + 1] = s_tie_pos[b];
          --b;
        }
        s_tie_ref[b + 1] = rk;
        s_tie_pos[b + 1] = pk;
      }
      s_ntie = (int)(need_ties < nt_ ? need_ties : nt_);
    }
    __syncthreads();
    /* apply: state 2 regardless of state; redraw non-positive infection timers */
    for (int64_t li = threadIdx.x; li < nslots + 64; li += blockDim.x) {
      int64_t pos;
      if (li < nslots) {
        pos = (int64_t)ls[c0 + li / LPG_CHUNK] * LPG_CHUNK + li % LPG_CHUNK;
        int8_t s = W.ds[pos];
        if (s < 0) continue;
        if (!all) {
          uint64_t key = lpg_raw(rp->seed, LPG_P_SEEDPICK, t, W.ref[pos], (uint64_t)ev.pad, 0);
          if (!(key < kstar)) continue;
        }
      } else {
        int k = (int)(li - nslots);
        if (all || k >= s_ntie) continue;
        pos = s_tie_pos[k];
      }
      int8_t s = W.ds[pos];
      int sti = W.strain[pos];
      const int64_t cid = pos / LPG_CHUNK;
      if (s == 1 || s == 2) {
        /* timers up to this tick's step, which has run */
        int8_t et = W.et[pos], it = W.it[pos], pt = W.pt[pos];
        const int k = t - W.evt[pos] + 1 + ev_pure(s, (int8_t)sti, et, it, pt, W.pp[pos]);
        if (k > 0) {
          ev_advance(s, (int8_t)sti, et, it, pt, k);
          W.et[pos] = et;
          W.it[pos] = it;
          W.pt[pos] = pt;
        }
      }
      if (s != 2) {
        uint64_t bw = fix_beta(W.inf[pos], rp->strain_scal[sti]);
        if (s == 0) {
          uint64_t w = fix_risk(W.risk[pos]);
          atomicAdd(&W.tot[(int64_t)TT_S * G + g], -1);
          if (w) {
            atomicAdd((unsigned long long*)&W.sw[g], neg64(w));
            atomicAdd((unsigned long long*)&W.chunk_w[cid], neg64(w));
            atomicAdd((unsigned long long*)&W.sub_w[cid * LPG_NSUB + (pos % LPG_CHUNK) / LPG_SUB], neg64(w));
          }
        } else if (s == 1) {
          atomicAdd(&W.tot[(int64_t)(TT_E0 + sti) * G + g], -1);
        } else if (s == 3) {
          atomicAdd(&W.tot[(int64_t)TT_R * G + g], -1);
        }
        atomicAdd(&W.tot[(int64_t)(TT_I0 + sti) * G + g], 1);
        if (bw) atomicAdd((unsigned long long*)&W.bb[(int64_t)sti * G + g], (unsigned long long)bw);
        W.ds[pos] = 2;
      }
      if (W.it[pos] <= 0) {
        lpg_stream sm;
        lpg_stream_init(&sm, rp->seed, LPG_P_SEEDTIMER, t, W.ref[pos], (uint64_t)ev.pad);
        W.it[pos] = lpg_trunc_i8(lpg_dist_sample(&sm, rp->dur_kind, rp->dur_p1, rp->dur_p2));
      }
      {
        const int32_t e1 = t + 1 + ev_pure(2, (int8_t)sti, W.et[pos], W.it[pos], W.pt[pos], W.pp[pos]);
        W.evt[pos] = e1;
        atomicMin(&W.sub_evt[pos >> 7], e1);
      }
    }
    __syncthreads();
  }
}

/* ------------------------------------------------------------------------ */
/* Per-node record of one selection step, written once per tick so that a
 * target needs one load to find everything about its node. */
#define LPG_SEL_OFFS 2048 /* target offsets kept in shared memory when G < this */
#define LPG_NODE_TX_THREADS 64
/* six CTAs of the node step per SM (at most 170 registers a thread): one
 * wave covers 912 nodes, so a 774-node tick needs no second wave */
#define LPG_NODE_TX_MIN_BLOCKS 6
/* the mixing step: MW warps of products and sums, one warp for the node's
 * chunk prefix.  MW = 4 for a simulation of hundreds of nodes (six CTAs per
 * SM, at most 68 registers a thread: 774 nodes in one wave); MW = 1 for a
 * batch of thousands of small nodes, where more CTAs a wave count more than
 * more warps a node. */
#define LPG_NODE_MIX_WARPS 4
#define LPG_NODE_MIX_THREADS (32 * (LPG_NODE_MIX_WARPS + 1))
#define LPG_NODE_MIX_MIN_BLOCKS 6
/* the node steps switch to their batch forms above this many nodes (six
 * CTAs of the per-node kernels per SM: more would take a second wave); the
 * mixing only when no simulation has more than LPG_NODE_BATCH_MAX_NODES
 * nodes: one warp then sweeps each network row in a few passes, where rows
 * of thousands of sources keep the per-node form's four mixing warps */
#define LPG_NODE_BATCH_MIN_PER_SM 6
#define LPG_NODE_BATCH_MAX_NODES 512

struct SelInfo {
  uint64_t seed;
  uint64_t T;        /* remaining susceptible weight */
  uint64_t thr[LPG_MAX_STRAINS]; /* the cumulative relative FOI (model.py:1127-1135) as 53-bit thresholds */
  int32_t a;         /* first entry of the node's chunk list in the concatenated lists */
  int32_t n;         /* its chunks */
  int32_t i;         /* node index in its simulation */
  int32_t t;         /* tick */
  int32_t ns;
  int32_t csr;       /* which of the two chunk-list buffers holds the node's list */
};

/* A uniform r = m 2^-53 (m a 53-bit integer) is below c exactly when m is
 * below ceil(c 2^53) (the scaling is exact); so the strain draw compares
 * integers, with the same outcome as comparing r with c (NaN or c <= 0:
 * never below; c >= 1: always). */
__device__ __forceinline__ uint64_t strain_threshold(double c) {
  const double x = c * 0x1.0p53;
  if (!(x > 0.0)) return 0;
  if (x >= 0x1.0p53) return (uint64_t)1 << 53;
  return (uint64_t)ceil(x);
}

/* Cumulative relative FOI that the strain draw compares against
 * (model.py:1127-1135), formed with the same operations in the same order. */
__device__ __forceinline__ void sel_strain_cum(const DevWorld& W, const DevRep* rp, int g, uint64_t* thr) {
  double p[LPG_MAX_STRAINS], q[LPG_MAX_STRAINS];
  double totalp = 0.0;
  const int ns = rp->ns;
#pragma unroll
  for (int k = 0; k < LPG_MAX_STRAINS; ++k) {
    p[k] = k < ns ? W.prob[(int64_t)k * W.G + g] : 0.0;
    if (k < ns) totalp = totalp + p[k];
  }
#pragma unroll
  for (int k = 0; k < LPG_MAX_STRAINS; ++k) q[k] = p[k] / totalp; /* independent divisions */
  double c = 0.0;
#pragma unroll
  for (int k = 0; k < LPG_MAX_STRAINS; ++k) {
    if (k < ns) c = c + q[k];
    thr[k] = strain_threshold(c);
  }
}

/* Node-local inclusive prefix of the chunk weights of a chunk list (n
 * entries) into cp, by one warp (8 weights per lane requested at once). */
__device__ __forceinline__ void warp_chunk_prefix(const DevWorld& W, const int32_t* ls, int32_t n, uint64_t* cp) {
  const int lane = threadIdx.x & 31;
  uint64_t carry = 0;
  for (int32_t a0 = 0; a0 < n; a0 += 32 * 8) {
    uint64_t wv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int32_t idx = a0 + u * 32 + lane;
      wv[u] = idx < n ? __ldcg(&W.chunk_w[ls[idx]]) : 0;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      if (a0 + u * 32 >= n) break;
      uint64_t x = wv[u];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(FULLMASK, x, o);
        if (lane >= o) x += y;
      }
      const int32_t idx = a0 + u * 32 + lane;
      if (idx < n) cp[idx] = carry + x;
      carry += __shfl_sync(FULLMASK, x, 31);
    }
  }
}

/* Incoming infectivity of every node and strain (model.py:1327-1363: the
 * network product), and the node's chunk prefix for the selection.  One CTA
 * per node: four warps share the source nodes, exact integer arithmetic: B
 * in units of 2^-40 times the network weight in its two fixed-point parts
 * (lpg_net_split; transposed row, contiguous), the two products summed in
 * three-word accumulators, one conversion (lpg_mix_value) into inck; an
 * exact sum does not depend on how the threads split it.  The fifth warp
 * forms the node-local chunk prefix (exact in integers) meanwhile. */
template <int MW>
__global__ void __launch_bounds__(32 * (MW + 1), MW == 4 ? LPG_NODE_MIX_MIN_BLOCKS : 16) k_node_mix(DevWorld W) {
  pdl_begin();
  const int g = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __shared__ uint64_t s_mix[MW][LPG_MAX_STRAINS][6]; /* per warp: A, R words */
  if (g >= W.G) return;
  const DevRep* rp = &W.reps[W.node_rep[g]];
  if (!rp->active || !(rp->comps & LPG_COMP_TX)) return;
  const int i = g - rp->node_base, n = rp->n_nodes, ns = rp->ns, G = W.G, nb = rp->node_base;
  if (wid == MW) {
    const int32_t* st = W.node_chunk_start[rp->csr_cur] + rp->csr_base;
    const int32_t a = st[i], nch = st[i + 1] - st[i];
    warp_chunk_prefix(W, W.node_chunks[rp->csr_cur] + rp->chunk_base + a, nch, W.cpref + rp->chunk_base + a);
    return;
  }
  /* qrow[ii] = network[ii][i] as (hi 2^-62, lo 2^-120), lpg_net_split */
  const ulonglong2* qrow = reinterpret_cast<const ulonglong2*>(rp->netq_t) + (int64_t)i * n;
  constexpr int NT = 32 * MW;
  constexpr int PER = 6; /* source nodes a thread takes per pass: PER x NT nodes a pass */
  if (lane == 0)
    for (int k = 0; k < ns; ++k)
#pragma unroll
      for (int q = 0; q < 6; ++q) s_mix[wid][k][q] = 0;
  /* per strain: A = sum B hi and R = sum B lo, three words each, exact;
   * one strain at a time (six accumulators live).  Sources without
   * infectivity add nothing to an exact sum, so a network entry is loaded
   * only where some strain's B is nonzero, and a strain whose B is zero
   * across the warp's sources of the pass is skipped: the sums, and so the
   * results, are those of the full product. */
  /* the same number of passes for every thread (the shuffles below need
   * all 32 lanes), loads past the last node predicated off */
  const int npass = (n + PER * NT - 1) / (PER * NT);
  for (int pass = 0; pass < npass; ++pass) {
    const int ii0 = pass * PER * NT + threadIdx.x;
    unsigned need = 0; /* bit u: source ii0 + u NT has infectivity of some strain */
    for (int k = 0; k < ns; ++k) {
#pragma unroll
      for (int u = 0; u < PER; ++u) {
        const int ii = ii0 + u * NT;
        if (ii < n && W.bb[(int64_t)k * G + nb + ii] != 0) need |= 1u << u;
      }
    }
    if (!__any_sync(FULLMASK, need != 0)) continue; /* warp-uniform */
    ulonglong2 w[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) w[u] = (need >> u) & 1 ? qrow[ii0 + u * NT] : make_ulonglong2(0, 0);
#pragma unroll 1
    for (int k = 0; k < ns; ++k) {
      uint64_t b[PER];
      bool any = false;
#pragma unroll
      for (int u = 0; u < PER; ++u) {
        const int ii = ii0 + u * NT;
        b[u] = (need >> u) & 1 ? W.bb[(int64_t)k * G + nb + ii] : 0;
        any |= b[u] != 0;
      }
      if (!__any_sync(FULLMASK, any)) continue; /* warp-uniform */
      uint64_t a0 = 0, a1 = 0, a2 = 0, r0 = 0, r1 = 0, r2 = 0;
#pragma unroll
      for (int u = 0; u < PER; ++u) {
        acc3_mul(a0, a1, a2, b[u], w[u].x);
        acc3_mul(r0, r1, r2, b[u], w[u].y);
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const uint64_t x0 = __shfl_down_sync(FULLMASK, a0, off), x1 = __shfl_down_sync(FULLMASK, a1, off),
                       x2 = __shfl_down_sync(FULLMASK, a2, off);
        acc3_add(a0, a1, a2, x0, x1, x2);
        const uint64_t y0 = __shfl_down_sync(FULLMASK, r0, off), y1 = __shfl_down_sync(FULLMASK, r1, off),
                       y2 = __shfl_down_sync(FULLMASK, r2, off);
        acc3_add(r0, r1, r2, y0, y1, y2);
      }
      if (lane == 0) {
        acc3_add(s_mix[wid][k][0], s_mix[wid][k][1], s_mix[wid][k][2], a0, a1, a2);
        acc3_add(s_mix[wid][k][3], s_mix[wid][k][4], s_mix[wid][k][5], r0, r1, r2);
      }
    }
  }
  /* the four mixing warps only (the fifth may have left) */
  asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory");
  if (threadIdx.x < ns) {
    const int k = threadIdx.x;
    uint64_t x0 = 0, x1 = 0, x2 = 0, y0 = 0, y1 = 0, y2 = 0;
#pragma unroll
    for (int w4 = 0; w4 < MW; ++w4) {
      acc3_add(x0, x1, x2, s_mix[w4][k][0], s_mix[w4][k][1], s_mix[w4][k][2]);
      acc3_add(y0, y1, y2, s_mix[w4][k][3], s_mix[w4][k][4], s_mix[w4][k][5]);
    }
    W.inck[(int64_t)k * G + g] = lpg_mix_value(x0, x1, x2, y0, y1, y2);
  }
}

/* Node-level force of infection and exposure counts (model.py:1327-1407);
 * the same arithmetic, in the same order, as the oracle's lpo_node_tx,
 * from the incoming infectivity k_node_mix formed.  One CTA per node. */
/* Lane k < ns of the second warp: this node's infectivity total of strain k
 * (the first warp's pre_bb). */
__device__ __forceinline__ uint64_t pre_bb_w1(const DevWorld& W, int g, int lane, int ns) {
  return lane < ns ? W.bb[(int64_t)lane * W.G + g] : 0;
}

__global__ void __launch_bounds__(LPG_NODE_TX_THREADS, LPG_NODE_TX_MIN_BLOCKS) k_node_tx(DevWorld W) {
  pdl_begin();
  const int g = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __shared__ double s_gam;   /* the negative binomial's gamma variate, formed ahead by the second warp */
  __shared__ uint64_t s_gamk; /* the exposure stream's position after it */
  if (g >= W.G) return;
  DevRep* rp = &W.reps[W.node_rep[g]];
  if (threadIdx.x == 0) W.ksel[g] = 0;
  if (!rp->active) return;
  const int i = g - rp->node_base, n = rp->n_nodes, ns = rp->ns, t = rp->cur_t, G = W.G;
  int32_t pop_t = 0;
  if (rp->comps & LPG_COMP_VD) {
    const int32_t* pop1 = RES(rp, RS_POP, t - 1);
    pop_t = pop1[i];
    if (rp->vd_tick) pop_t = pop_t + W.ev[(int64_t)EV_BIRTHS * G + g] - W.ev[(int64_t)EV_DEATHS * G + g];
    if (threadIdx.x == 0) RES(rp, RS_POP, t)[i] = pop_t;
  } else {
    pop_t = RES(rp, RS_POP, t)[i];
  }
  if (threadIdx.x == 0) {
    W.size[g] = 0;
    W.uniq[g] = 0;
  }
  if (!(rp->comps & LPG_COMP_TX)) return;
  /* inputs of lane 0's draw, requested now so that they arrive during the
   * mixing */
  double pre_seas = 0.0, pre_r0s = 0.0, pre_rowsum = 0.0, pre_inck = 0.0;
  uint64_t pre_bb = 0;
  uint64_t pre_sw = 0;
  int64_t pre_sc = 0;
  /* lane k < ns of the first warp works on strain k after the mixing */
  if (threadIdx.x < ns) {
    pre_seas = rp->seas[t];
    pre_r0s = rp->r0s[i];
    pre_rowsum = rp->rowsum[i];
    pre_bb = W.bb[(int64_t)threadIdx.x * G + g];
    pre_inck = W.inck[(int64_t)threadIdx.x * G + g];
  }
  if (threadIdx.x == 0) {
    pre_sw = W.sw[g];
    pre_sc = W.tot[(int64_t)TT_S * G + g];
  }
  if (rp->rec) { /* the aggregates the expected-incidence map replays */
    double* rr = rp->rec + ((int64_t)t * n + i) * (3 + ns);
    if (threadIdx.x == 0) {
      rr[0] = (double)pre_sw * 0x1.0p-24;
      rr[1] = (double)pop_t;
    }
    if (threadIdx.x < ns) rr[3 + threadIdx.x] = (double)pre_bb * 0x1.0p-40;
  }
  if (wid == 1) {
    /* the second warp: when the node has no local infectivity (the
     * zero-inflated negative binomial, model.py:1383-1395), its gamma
     * variate first: it uses the exposure stream from its second draw and
     * not the tick's force of infection, so it is formed while the first
     * warp works out the probabilities (a warp's double-precision operations
     * do not overlap, another warp's do) */
    const bool lz = __ballot_sync(FULLMASK, lane < ns && pre_bb_w1(W, g, lane, ns) != 0) == 0;
    if (lane == 0 && lz && rp->zi < 1.0 && rp->nb_r >= 1) {
      lpg_stream sg;
      lpg_stream_init(&sg, rp->seed, LPG_P_TXCOUNT, t, (uint64_t)i, 0);
      sg.k = 1; /* draw 0 is the zero-inflation test */
      s_gam = lpg_gamma_mt(&sg, rp->nb_d, rp->nb_c, 1.0);
      s_gamk = sg.k;
    }
    __syncwarp();
    asm volatile("bar.sync 1, 64;" ::: "memory");
    return;
  }
  if (wid != 0) return;
  /* the first two blocks of lane 0's exposure-count stream, formed while
   * the double-precision work below waits on its latencies */
  lpg_stream sm;
  lpg_stream_init(&sm, rp->seed, LPG_P_TXCOUNT, t, (uint64_t)i, 0);
  lpg_stream_ahead(&sm);
  /* Strain k on lane k (a double-precision warp instruction costs the same
   * for one lane or 32): incoming infectivity, beta, rate, probability
   * (model.py:1327-1363); then the sums over strains in strain order, as
   * the oracle forms them. */
  double pk = 0.0;
  const double denom = (double)(pop_t > 1 ? pop_t : 1);
  if (lane < ns) {
    const double inck = pre_inck;
    const double bpre = (double)pre_bb * 0x1.0p-40;
    double beta = bpre + (inck - bpre * pre_rowsum);
    beta = (beta * pre_seas) * pre_r0s;
    const double rate = beta / denom;
    pk = -lpg_expm1(-rate);
    if (!(pk > 0.0)) pk = 0.0;
    W.prob[(int64_t)lane * G + g] = pk;
  }
  const int local_zero = __ballot_sync(FULLMASK, lane < ns && pre_bb != 0) == 0;
  double p[LPG_MAX_STRAINS];
#pragma unroll
  for (int k = 0; k < LPG_MAX_STRAINS; ++k) p[k] = __shfl_sync(FULLMASK, pk, k);
  double total_p = 0.0;
#pragma unroll
  for (int k = 0; k < LPG_MAX_STRAINS; ++k)
    if (k < ns) total_p = total_p + p[k];
  /* strain thresholds of the selection (sel_strain_cum's values), the
   * divisions on their own lanes */
  const double qk = pk / total_p;
  uint64_t thr[LPG_MAX_STRAINS];
  {
    double c = 0.0;
#pragma unroll
    for (int k = 0; k < LPG_MAX_STRAINS; ++k) {
      const double q = __shfl_sync(FULLMASK, qk, k);
      if (k < ns) c = c + q;
      thr[k] = strain_threshold(c);
    }
  }
  __syncwarp();
  asm volatile("bar.sync 1, 64;" ::: "memory"); /* the second warp's gamma variate is in s_gam */
  if (lane != 0) return;
  const double srisk = (double)pre_sw * 0x1.0p-24;
  const double exposure = srisk * total_p;
  if (rp->rec) rp->rec[((int64_t)t * n + i) * (3 + ns) + 2] = exposure;
  int64_t total = 0;
  if (!(exposure > 0.0)) {
    total = 0;
  } else if (local_zero) {
    if (rp->zi >= 1.0) {
      total = 0;
    } else {
      double mean = exposure / (1.0 - rp->zi);
      double r = (double)rp->nb_r;
      double pp = r / (r + mean);
      double u = lpg_next(&sm);
      if (u < rp->zi) {
        total = 0;
      } else if (rp->nb_r >= 1) {
        /* lpg_negbinom_dc with its gamma variate from the second warp */
        sm.k = s_gamk;
        total = lpg_poisson(&sm, s_gam * ((1.0 - pp) / pp));
      } else {
        total = lpg_negbinom(&sm, r, pp);
      }
    }
  } else {
    total = lpg_poisson(&sm, exposure);
  }
  const int64_t sc = pre_sc;
  const int64_t size = total < sc ? total : sc;
  W.size[g] = size;
  /* the selection record of the node (round 0 targets: all of size) */
  const uint64_t Tw = pre_sw;
  if (size > 0 && Tw > 0) {
    const int32_t* st = W.node_chunk_start[rp->csr_cur] + rp->csr_base;
    SelInfo N;
    N.seed = rp->seed;
    N.T = Tw;
#pragma unroll
    for (int k = 0; k < LPG_MAX_STRAINS; ++k) N.thr[k] = thr[k];
    N.a = rp->chunk_base + st[i];
    N.n = st[i + 1] - st[i];
    N.i = i;
    N.t = t;
    N.ns = ns;
    N.csr = rp->csr_cur;
    reinterpret_cast<SelInfo*>(W.sel_info)[g] = N;
    W.ksel[g] = size;
  }
  if (size > 0) rp->any_demand = 1;
}

/* k_node_tx for a batch of thousands of small nodes: one node a thread,
 * the same operations in the same order (strains one after another; the
 * negative binomial's gamma variate drawn in line, from the same stream
 * positions).  A double-precision warp instruction costs the same for one
 * lane or 32, so here one serves 32 nodes: a batch's nodes take one wave
 * where a CTA a node takes ten. */
__global__ void __launch_bounds__(128) k_node_tx_lanes(DevWorld W) {
  pdl_begin();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= W.G) return;
  DevRep* rp = &W.reps[W.node_rep[g]];
  W.ksel[g] = 0;
  if (!rp->active) return;
  const int i = g - rp->node_base, n = rp->n_nodes, ns = rp->ns, t = rp->cur_t, G = W.G;
  int32_t pop_t = 0;
  if (rp->comps & LPG_COMP_VD) {
    pop_t = RES(rp, RS_POP, t - 1)[i];
    if (rp->vd_tick) pop_t = pop_t + W.ev[(int64_t)EV_BIRTHS * G + g] - W.ev[(int64_t)EV_DEATHS * G + g];
    RES(rp, RS_POP, t)[i] = pop_t;
  } else {
    pop_t = RES(rp, RS_POP, t)[i];
  }
  W.size[g] = 0;
  W.uniq[g] = 0;
  if (!(rp->comps & LPG_COMP_TX)) return;
  const double seas = rp->seas[t], r0s = rp->r0s[i], rowsum = rp->rowsum[i];
  const uint64_t sw = W.sw[g];
  const int64_t sc = W.tot[(int64_t)TT_S * G + g];
  uint64_t bb[LPG_MAX_STRAINS];
  double inc[LPG_MAX_STRAINS];
#pragma unroll
  for (int k = 0; k < LPG_MAX_STRAINS; ++k) {
    bb[k] = k < ns ? W.bb[(int64_t)k * G + g] : 0;
    inc[k] = k < ns ? W.inck[(int64_t)k * G + g] : 0.0;
  }
  double* rr = rp->rec ? rp->rec + ((int64_t)t * n + i) * (3 + ns) : nullptr;
  if (rr) {
    rr[0] = (double)sw * 0x1.0p-24;
    rr[1] = (double)pop_t;
  }
  /* incoming infectivity, beta, rate and probability of each strain
   * (model.py:1327-1363), and their sum in strain order */
  const double denom = (double)(pop_t > 1 ? pop_t : 1);
  double p[LPG_MAX_STRAINS];
  double total_p = 0.0;
  bool local_zero = true;
#pragma unroll
  for (int k = 0; k < LPG_MAX_STRAINS; ++k) {
    p[k] = 0.0;
    if (k < ns) {
      const double bpre = (double)bb[k] * 0x1.0p-40;
      if (rr) rr[3 + k] = bpre;
      if (bb[k] != 0) local_zero = false;
      double beta = bpre + (inc[k] - bpre * rowsum);
      beta = (beta * seas) * r0s;
      const double rate = beta / denom;
      double pk = -lpg_expm1(-rate);
      if (!(pk > 0.0)) pk = 0.0;
      p[k] = pk;
      W.prob[(int64_t)k * G + g] = pk;
      total_p = total_p + pk;
    }
  }
  /* strain thresholds of the selection (sel_strain_cum's values) */
  uint64_t thr[LPG_MAX_STRAINS];
  {
    double c = 0.0;
#pragma unroll
    for (int k = 0; k < LPG_MAX_STRAINS; ++k) {
      if (k < ns) c = c + p[k] / total_p;
      thr[k] = strain_threshold(c);
    }
  }
  lpg_stream sm;
  lpg_stream_init(&sm, rp->seed, LPG_P_TXCOUNT, t, (uint64_t)i, 0);
  const double srisk = (double)sw * 0x1.0p-24;
  const double exposure = srisk * total_p;
  if (rr) rr[2] = exposure;
  int64_t total = 0;
  if (!(exposure > 0.0)) {
    total = 0;
  } else if (local_zero) {
    if (rp->zi >= 1.0) {
      total = 0;
    } else {
      double mean = exposure / (1.0 - rp->zi);
      double r = (double)rp->nb_r;
      double pp = r / (r + mean);
      double u = lpg_next(&sm);
      if (u < rp->zi) {
        total = 0;
      } else if (rp->nb_r >= 1) {
        const double gam = lpg_gamma_mt(&sm, rp->nb_d, rp->nb_c, 1.0); /* lpg_negbinom_dc */
        total = lpg_poisson(&sm, gam * ((1.0 - pp) / pp));
      } else {
        total = lpg_negbinom(&sm, r, pp);
      }
    }
  } else {
    total = lpg_poisson(&sm, exposure);
  }
  const int64_t size = total < sc ? total : sc;
  W.size[g] = size;
  if (size > 0 && sw > 0) {
    const int32_t* st = W.node_chunk_start[rp->csr_cur] + rp->csr_base;
    SelInfo N;
    N.seed = rp->seed;
    N.T = sw;
#pragma unroll
    for (int k = 0; k < LPG_MAX_STRAINS; ++k) N.thr[k] = thr[k];
    N.a = rp->chunk_base + st[i];
    N.n = st[i + 1] - st[i];
    N.i = i;
    N.t = t;
    N.ns = ns;
    N.csr = rp->csr_cur;
    reinterpret_cast<SelInfo*>(W.sel_info)[g] = N;
    W.ksel[g] = size;
  }
  if (size > 0) rp->any_demand = 1;
}

/* ------------------------------------------------------------------------ */

/* Slot of target v inside chunk cid (v < the chunk's remaining weight):
 * sub-block by its 16 totals, slot by the 128 state bytes and risks.
 * LPG_NONE if the weights are inconsistent (an internal error). */
__device__ __forceinline__ uint32_t locate_in_chunk(const DevWorld& W, int64_t cid, uint64_t v) {
  uint64_t swv[LPG_NSUB];
#pragma unroll
  for (int k = 0; k < LPG_NSUB; ++k) swv[k] = __ldcg(&W.sub_w[cid * LPG_NSUB + k]);
  int sb = LPG_NSUB;
#pragma unroll
  for (int k = 0; k < LPG_NSUB; ++k) {
    if (sb == LPG_NSUB) {
      if (swv[k] > v) sb = k;
      else v -= swv[k];
    }
  }
  uint32_t hit = LPG_NONE;
  if (sb < LPG_NSUB) {
    const int64_t p0 = cid * LPG_CHUNK + (int64_t)sb * LPG_SUB;
    uint4 sv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) sv[k] = __ldcg(reinterpret_cast<const uint4*>(W.ds + p0) + k);
    for (int grp = 0; grp < 4 && hit == LPG_NONE; ++grp) {
      float4 rv[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) rv[k] = reinterpret_cast<const float4*>(W.risk + p0 + grp * 32)[k];
      const uint32_t* sw32 = reinterpret_cast<const uint32_t*>(&sv[grp * 2]);
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        if (hit != LPG_NONE) break;
        const uint32_t sbyte = (sw32[k >> 2] >> (8 * (k & 3))) & 0xffu;
        if (!sel_open(sbyte)) continue;
        const uint64_t w = fix_risk(reinterpret_cast<const float*>(rv)[k]);
        if (w > v) hit = (uint32_t)(p0 + grp * 32 + k);
        else v -= w;
      }
    }
  }
  return hit;
}

/* Locate target v (< the node's remaining susceptible weight) in the node's
 * frozen CDF.  cp holds n chunk prefixes of the node's chunk list ls (n
 * entries); the node's own prefix of entry j is cp[j] - base.  First chunk
 * whose prefix exceeds v (searchsorted side='right', model.py:1118), then
 * the slot inside it. */
__device__ __forceinline__ uint32_t locate(const DevWorld& W, const int32_t* ls, const uint64_t* cp, int32_t n,
                                           uint64_t v, uint64_t base) {
  int32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    int32_t mid = (lo + hi) >> 1;
    if (cp[mid] - base > v) hi = mid; else lo = mid + 1;
  }
  if (lo > 0) v -= cp[lo - 1] - base;
  return locate_in_chunk(W, ls[lo], v);
}

/* A team of T lanes (T a power of two <= 32, aligned in its warp) that
 * locates one target together. */
struct Team {
  unsigned mask; /* the team's lanes */
  int T, l, lane0;
};
__device__ __forceinline__ Team make_team(int T) {
  Team t;
  const int lane = threadIdx.x & 31;
  t.T = T;
  t.l = lane & (T - 1);
  t.lane0 = lane & ~(T - 1);
  t.mask = T == 32 ? FULLMASK : (((1u << T) - 1u) << t.lane0);
  return t;
}
__device__ __forceinline__ unsigned team_ballot(const Team& tm, bool p) {
  return tm.T == 32 ? __ballot_sync(tm.mask, p) : (__ballot_sync(tm.mask, p) >> tm.lane0) & ((1u << tm.T) - 1u);
}
__device__ __forceinline__ uint64_t team_incl_scan(const Team& tm, uint64_t x) {
  for (int o = 1; o < tm.T; o <<= 1) {
    const uint64_t y = __shfl_up_sync(tm.mask, x, o, tm.T);
    if (tm.l >= o) x += y;
  }
  return x;
}

/* Probe l of a (T+1)-ary search of [lo, lo + m): lo + (l + 1) m / (T + 1).
 * In 32 bits: m is below 2^21 (chunks of a node, or nodes of a batch) and
 * l + 1 at most 32; with T a constant the division is a multiply. */
template <int T>
__device__ __forceinline__ int32_t team_probe(int32_t lo, int32_t m, int l) {
  return lo + (int32_t)(((uint32_t)(l + 1) * (uint32_t)m) / (uint32_t)(T + 1));
}

/* locate() by a team of T lanes: the same answer, with a (T+1)-ary search
 * of the chunk prefix and, for T >= 4, the sub-block totals and the 128
 * slots split over the lanes (each lane a contiguous run; a team scan finds
 * the lane that holds the target).  Every lane of the team returns the hit.
 * All 32 lanes of the warp call it together (teams without a target pass
 * active = false) so that the warp reconverges between the stages: teams
 * that diverged in the search would otherwise run the later stages one team
 * at a time.  Each probe of the search requests the chunk id beside the
 * prefix, and the team keeps the values at the bounds (the prefix below lo,
 * the chunk at hi), so that the chunk and the target's offset in it are
 * known when the search ends, without further loads.  word_out / risk_out
 * (when given) receive the hit slot's state word (4 state bytes) and risk as
 * read.  T is a template constant, so that every loop below has its exact
 * trip count and no dead iterations (the kernels run once a tick and fetch
 * their instructions cold: code that is not there costs nothing). */
template <int T>
__device__ __forceinline__ uint32_t locate_team_t(const DevWorld& W, const int32_t* ls, const uint64_t* cp,
                                                  int32_t n, uint64_t v, uint64_t base, bool active,
                                                  uint32_t* word_out, float* risk_out) {
  const Team tm = make_team(T);
  int32_t lo = 0, hi = active ? n - 1 : 0;
  uint64_t cp_lo = base;                    /* cp[lo - 1] (base while lo = 0) */
  int32_t ls_hi = active ? ls[hi] : 0;      /* ls[hi] */
  while (lo < hi) {
    const int32_t m = hi - lo;
    const int32_t p = team_probe<T>(lo, m, tm.l);
    const uint64_t cpp = cp[p];
    const int32_t lsp = ls[p];
    const unsigned b = team_ballot(tm, cpp - base > v);
    const int c = __ffs(b) - 1; /* first probe above v; probes ascend with the lane */
    const uint64_t cp_below = __shfl_sync(tm.mask, cpp, c < 0 ? T - 1 : (c > 0 ? c - 1 : 0), T);
    const int32_t ls_c = __shfl_sync(tm.mask, lsp, c < 0 ? 0 : c, T);
    const int32_t lo0 = lo;
    if (c < 0) {
      lo = team_probe<T>(lo0, m, T - 1) + 1;
      cp_lo = cp_below;
    } else {
      if (c > 0) {
        lo = team_probe<T>(lo0, m, c - 1) + 1;
        cp_lo = cp_below;
      }
      hi = team_probe<T>(lo0, m, c);
      ls_hi = ls_c;
    }
  }
  __syncwarp();
  uint32_t hit = LPG_NONE;
  int64_t cid = 0;
  if (active) {
    if (lo > 0) v -= cp_lo - base;
    cid = ls_hi;
  }
  if constexpr (T < 4) {
    if (active && tm.l == 0) hit = locate_in_chunk(W, cid, v);
    __syncwarp();
    hit = active ? __shfl_sync(tm.mask, hit, 0, T) : LPG_NONE;
    if (word_out && hit != LPG_NONE) {
      *word_out = __ldcg(reinterpret_cast<const uint32_t*>(W.ds + ((int64_t)hit & ~3LL)));
      *risk_out = W.risk[hit];
    }
    return hit;
  } else {
    /* sub-block: lanes l < min(T, 16) hold 16 / min(T, 16) consecutive totals */
    constexpr int TS = T < LPG_NSUB ? T : LPG_NSUB;
    constexpr int PER = LPG_NSUB / TS;
    int sb = -1;
    uint64_t vl = 0;
    if (active) {
      uint64_t sw[PER];
      uint64_t sum = 0;
#pragma unroll
      for (int k = 0; k < PER; ++k) {
        sw[k] = tm.l < TS ? __ldcg(&W.sub_w[cid * LPG_NSUB + tm.l * PER + k]) : 0;
        sum += sw[k];
      }
      const uint64_t incl = team_incl_scan(tm, sum);
      const uint64_t excl = incl - sum;
      const unsigned own = team_ballot(tm, sum > 0 && excl <= v && v < incl);
      if (own != 0) {
        const int ol = __ffs(own) - 1;
        vl = v - excl;
        if (tm.l == ol) {
#pragma unroll
          for (int k = 0; k < PER; ++k) {
            if (sb < 0) {
              if (sw[k] > vl) sb = tm.l * PER + k;
              else vl -= sw[k];
            }
          }
        }
        sb = __shfl_sync(tm.mask, sb, ol, T);
        vl = __shfl_sync(tm.mask, vl, ol, T);
      }
    }
    __syncwarp();
    /* slots: lane l holds L = 128 / T consecutive slots (L / 4 state words) */
    constexpr int L = LPG_SUB / T;
    const bool go = active && sb >= 0;
    const int64_t s0 = go ? cid * LPG_CHUNK + (int64_t)sb * LPG_SUB + (int64_t)tm.l * L : 0;
    uint32_t dw[L / 4];
    float4 rv[L / 4];
#pragma unroll
    for (int k = 0; k < L / 4; ++k) {
      if (go) {
        dw[k] = __ldcg(reinterpret_cast<const uint32_t*>(W.ds + s0) + k);
        rv[k] = reinterpret_cast<const float4*>(W.risk + s0)[k];
      } else {
        dw[k] = 0xffffffffu;
        rv[k] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    uint64_t wsum = 0;
#pragma unroll
    for (int k = 0; k < L; ++k)
      if (sel_open((dw[k >> 2] >> (8 * (k & 3))) & 0xffu)) wsum += fix_risk(reinterpret_cast<const float*>(rv)[k]);
    if (go) {
      const uint64_t incl = team_incl_scan(tm, wsum);
      const uint64_t excl = incl - wsum;
      const unsigned own = team_ballot(tm, wsum > 0 && excl <= vl && vl < incl);
      if (own != 0) {
        const int ol = __ffs(own) - 1;
        uint32_t word = 0;
        float rk = 0.f;
        if (tm.l == ol) {
          uint64_t r = vl - excl;
#pragma unroll
          for (int k = 0; k < L; ++k) {
            if (hit == LPG_NONE && sel_open((dw[k >> 2] >> (8 * (k & 3))) & 0xffu)) {
              const uint64_t w = fix_risk(reinterpret_cast<const float*>(rv)[k]);
              if (w > r) {
                hit = (uint32_t)(s0 + k);
                word = dw[k >> 2];
                rk = reinterpret_cast<const float*>(rv)[k];
              } else {
                r -= w;
              }
            }
          }
        }
        hit = __shfl_sync(tm.mask, hit, ol, T);
        if (word_out) {
          *word_out = __shfl_sync(tm.mask, word, ol, T);
          *risk_out = __shfl_sync(tm.mask, rk, ol, T);
        }
      }
    }
    __syncwarp();
    return hit;
  }
}

/* locate_team_t for a team size known only at run time (uniform in the
 * warp). */
__device__ __forceinline__ uint32_t locate_team(const DevWorld& W, const Team& tm, const int32_t* ls,
                                                const uint64_t* cp, int32_t n, uint64_t v, uint64_t base,
                                                bool active = true, uint32_t* word_out = nullptr,
                                                float* risk_out = nullptr) {
  switch (tm.T) {
    case 32: return locate_team_t<32>(W, ls, cp, n, v, base, active, word_out, risk_out);
    case 16: return locate_team_t<16>(W, ls, cp, n, v, base, active, word_out, risk_out);
    case 8: return locate_team_t<8>(W, ls, cp, n, v, base, active, word_out, risk_out);
    case 4: return locate_team_t<4>(W, ls, cp, n, v, base, active, word_out, risk_out);
    case 2: return locate_team_t<2>(W, ls, cp, n, v, base, active, word_out, risk_out);
    default: return locate_team_t<1>(W, ls, cp, n, v, base, active, word_out, risk_out);
  }
}

/* The exposure of an agent that a target has claimed: strain by relative
 * FOI (model.py:1127-1145), its first step in E, and every susceptible total
 * but the sub-block's (sub_now: that one too).  Returns its weight. */
__device__ __forceinline__ uint64_t expose_claimed(DevWorld& W, int64_t pos, int g, const SelInfo& N, uint64_t r53,
                                                   int8_t et, float risk, bool sub_now) {
  const int G = W.G;
  const int64_t cid = pos / LPG_CHUNK;
  int s = 0;
  bool found = false;
#pragma unroll
  for (int k = 0; k < LPG_MAX_STRAINS; ++k)
    if (!found && k < N.ns && r53 < N.thr[k]) {
      s = k;
      found = true;
    }
  W.strain[pos] = (int8_t)s;
  {
    /* first step in E is at t + 1 (model.py:393-454) */
    const int32_t e1 = N.t + 1 + (et > 0 ? et : 0);
    W.evt[pos] = e1;
    atomicMin(&W.sub_evt[pos >> 7], e1);
  }
  const uint64_t w = fix_risk(risk);
  atomicAdd(&W.tot[(int64_t)TT_S * G + g], -1);
  atomicAdd(&W.tot[(int64_t)(TT_E0 + s) * G + g], 1);
  atomicAdd(&W.ev[(int64_t)(EV_TXNEW0 + s) * G + g], 1);
  atomicAdd((unsigned long long*)&W.uniq[g], 1ULL);
  if (w) {
    atomicAdd((unsigned long long*)&W.sw[g], neg64(w));
    atomicAdd((unsigned long long*)&W.chunk_w[cid], neg64(w));
    if (sub_now) atomicAdd((unsigned long long*)&W.sub_w[cid * LPG_NSUB + (pos % LPG_CHUNK) / LPG_SUB], neg64(w));
  }
  return w;
}

/* The first target to claim an agent (state 0 -> 1) exposes it (rounds
 * after the first, whose claims follow all of the round's locates).
 * Returns whether this target claimed it (and the weight it removed in
 * *w_out). */
__device__ __forceinline__ bool claim(DevWorld& W, uint32_t hit, int g, const SelInfo& N, uint64_t* w_out = nullptr) {
  const int64_t pos = hit;
  /* the agent's fixed columns requested first, and its strain draw formed
   * while the claim's atomic is in flight (a lost claim discards them) */
  const uint32_t ref = W.ref[pos];
  const int8_t et = W.et[pos];
  const float risk = W.risk[pos];
  uint32_t* wp = reinterpret_cast<uint32_t*>(W.ds + (pos & ~3LL));
  const int sh = (int)(pos & 3) * 8;
  uint32_t old = *(volatile uint32_t*)wp;
  const uint64_t r53 = lpg_u53(N.seed, LPG_P_STRAIN, N.t, ref, 0, 0);
  bool won = false;
  while (((old >> sh) & 0xffu) == 0) {
    const uint32_t nw = (old & ~(0xffu << sh)) | (1u << sh);
    const uint32_t prev = atomicCAS(wp, old, nw);
    if (prev == old) {
      won = true;
      break;
    }
    old = prev;
  }
  if (!won) return false;
  const uint64_t w = expose_claimed(W, pos, g, N, r53, et, risk, true);
  if (w_out) *w_out = w;
  return true;
}

/* A round-0 claim, made as soon as the target is located: state 0 ->
 * LPG_DS_CLAIMED (the round's other targets still see the agent's weight),
 * the exposure and every total but the sub-block weight, which the claimer
 * removes after the round (claim0_finish).  word and risk are the slot's
 * state word and risk as the locate read them (the word is the first guess
 * of the compare-and-swap). */
__device__ __forceinline__ bool claim0(DevWorld& W, uint32_t hit, uint32_t word, float risk, int g,
                                       const SelInfo& N, uint64_t* w_out) {
  const int64_t pos = hit;
  const uint32_t ref = W.ref[pos];
  const int8_t et = W.et[pos];
  uint32_t* wp = reinterpret_cast<uint32_t*>(W.ds + (pos & ~3LL));
  const int sh = (int)(pos & 3) * 8;
  uint32_t old = word;
  const uint64_t r53 = lpg_u53(N.seed, LPG_P_STRAIN, N.t, ref, 0, 0);
  bool won = false;
  while (((old >> sh) & 0xffu) == 0) {
    const uint32_t nw = (old & ~(0xffu << sh)) | (LPG_DS_CLAIMED << sh);
    const uint32_t prev = atomicCAS(wp, old, nw);
    if (prev == old) {
      won = true;
      break;
    }
    old = prev;
  }
  if (!won) return false;
  *w_out = expose_claimed(W, pos, g, N, r53, et, risk, false);
  return true;
}

/* After round 0: the claimed agent becomes exposed (state 1) and leaves its
 * sub-block's weight. */
__device__ __forceinline__ void claim0_finish(DevWorld& W, uint32_t hit, uint64_t w) {
  if (hit == LPG_NONE) return;
  const int64_t pos = hit;
  W.ds[pos] = 1;
  if (w) {
    const int64_t cid = pos / LPG_CHUNK;
    atomicAdd((unsigned long long*)&W.sub_w[cid * LPG_NSUB + (pos % LPG_CHUNK) / LPG_SUB], neg64(w));
  }
}

/* Grid-wide barrier of a cooperative launch (every CTA resident), on a
 * counter that only grows: thread 0 of each CTA adds 1 and polls until the
 * count reaches the next multiple of the grid size, at most `limit` times.
 * Every barrier adds exactly one per CTA, so the count is a multiple of the
 * grid size whenever none is open (the host clears it when the grid size
 * changes).  Returns false (in every thread of the CTA) when the poll ran
 * out. */
__device__ bool grid_sync(unsigned long long* ctr, long long limit, bool skip_arrive = false) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    if (skip_arrive) {
      ok = 0;
    } else {
      __threadfence();
      const unsigned long long old = atomicAdd(ctr, 1ULL);
      const unsigned long long target = (old / gridDim.x + 1) * gridDim.x;
      const volatile unsigned long long* vc = ctr;
      long long it = 0;
      while (*vc < target) {
        if (++it > limit) {
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

/* First g in [lo, hi] with off[g] > q (the answer is known to be <= hi), by
 * a (T+1)-ary search of the team over off (shared memory). */
template <int T>
__device__ __forceinline__ int team_first_above(const Team& tm, const int64_t* off, int lo, int hi, int64_t q) {
  while (lo < hi) {
    const int m = hi - lo;
    const unsigned b = team_ballot(tm, off[team_probe<T>(lo, m, tm.l)] > q);
    const int c = __ffs(b) - 1;
    const int lo0 = lo;
    if (c < 0) {
      lo = team_probe<T>(lo0, m, T - 1) + 1;
    } else {
      if (c > 0) lo = team_probe<T>(lo0, m, c - 1) + 1;
      hi = team_probe<T>(lo0, m, c);
    }
  }
  return lo;
}

/* Last g in [0, G) with off[g] <= q (off ascending from off[0] = 0, q below
 * off[G]), by one lane. */
__device__ __forceinline__ int node_of_target(const int64_t* off, int G, int64_t q) {
  int lo = 0, hi = G; /* off[lo] <= q < off[hi] */
  while (hi - lo > 1) {
    const int m = (lo + hi) >> 1;
    if (off[m] <= q) lo = m;
    else hi = m;
  }
  return lo;
}

/* Round 0's targets for a team size T.  A team takes its targets T at a
 * time: lane l of the team finds the node and forms the uniform of the
 * batch's l-th target (target q0 + (b T + l) nteams), the team then locates
 * the batch's targets one after another on the frozen CDF, and each lane
 * claims its own target's agent (claim0), so that the per-target work that
 * is not the search (node, uniform, claim, strain draw) runs once per lane
 * rather than once per team.  A lane keeps its first claim in registers and
 * stores later ones' slots in hits[q]; then the grid barrier, after which
 * each lane settles its claims (state 1, sub-block weight).  Returns false
 * when the barrier's wait ran out. */
template <int T>
__device__ __forceinline__ bool round0_targets(DevWorld& W, const int64_t* offs, const SelInfo* info, int64_t K) {
  const int G = W.G;
  const Team tm = make_team(T);
  const int64_t nteams = ((int64_t)gridDim.x * blockDim.x) / T;
  const int64_t q0 = (int64_t)(threadIdx.x / T) * gridDim.x + blockIdx.x;
  uint32_t h0 = LPG_NONE;
  uint64_t w0 = 0;
  /* warp-uniform trip count: every lane stays until no team of its warp has a target */
  int b = 0;
  for (int64_t qb = q0; __any_sync(FULLMASK, qb < K); qb += (int64_t)T * nteams, ++b) {
    /* this lane's target of the batch */
    const int64_t q = qb + (int64_t)tm.l * nteams;
    const bool act = q < K;
    int g = 0;
    uint64_t v = 0;
    int32_t la = 0, ln = 1, lcsr = 0;
    if (act) {
      g = node_of_target(offs, G, q);
      const SelInfo& N = info[g];
      v = lpg_scale_target(lpg_u53(N.seed, LPG_P_SELECT, N.t, (uint64_t)N.i, 0, (uint64_t)(q - offs[g])), N.T);
      la = N.a;
      ln = N.n;
      lcsr = N.csr;
    }
    /* the batch's targets are a prefix of the team's lanes (q ascends with l) */
    const int nk = __reduce_max_sync(FULLMASK, (unsigned)__popc(team_ballot(tm, act)));
    uint32_t my_hit = LPG_NONE, my_word = 0;
    float my_rk = 0.f;
    for (int k = 0; k < nk; ++k) {
      const bool ak = __shfl_sync(FULLMASK, (int)act, k, T) != 0;
      const uint64_t vk = __shfl_sync(FULLMASK, v, k, T);
      const int32_t ak_a = __shfl_sync(FULLMASK, la, k, T);
      const int32_t ak_n = __shfl_sync(FULLMASK, ln, k, T);
      const int32_t ak_c = __shfl_sync(FULLMASK, lcsr, k, T);
      const int32_t* ls = W.node_chunks[ak_c] + ak_a;
      uint32_t word = 0;
      float rk = 0.f;
      const uint32_t hit = locate_team_t<T>(W, ls, W.cpref + ak_a, ak ? ak_n : 1, vk, 0, ak, &word, &rk);
      if (tm.l == k) {
        my_hit = hit;
        my_word = word;
        my_rk = rk;
      }
    }
    if (act) {
      uint32_t won_at = LPG_NONE;
      uint64_t w = 0;
      if (my_hit == LPG_NONE) W.reps[W.node_rep[g]].error = LPG_ERR_INTERNAL;
      else if (claim0(W, my_hit, my_word, my_rk, g, info[g], &w)) won_at = my_hit;
      if (b == 0) {
        h0 = won_at;
        w0 = w;
      } else {
        W.hits[q] = won_at;
      }
    }
  }
  /* every target of the round located and claimed: the claimed agents
   * become exposed and leave their sub-blocks' weights */
  if (!grid_sync(W.grid_bar, W.wait_spin, W.test_bar_skip && blockIdx.x == 0)) return false;
  claim0_finish(W, h0, w0);
  /* this lane's later claims: batches 1, 2, ... */
  for (int64_t q = q0 + ((int64_t)T + tm.l) * nteams; q < K; q += (int64_t)T * nteams) {
    const uint32_t h = W.hits[q];
    if (h != LPG_NONE) claim0_finish(W, h, fix_risk(W.risk[h]));
  }
  return true;
}

/* Weighted selection without replacement (tx_infect_nb, model.py:1066-1147),
 * in two kernels.  k_node_tx has left, per node with demand, its round-0
 * target count (ksel), its selection record and its node-local chunk
 * prefix.  Round 0 runs over all nodes at once in one cooperative launch
 * (k_sel_round0): every CTA forms the target offsets in its shared memory;
 * targets go round-robin over the CTAs, each located by a team of lanes on
 * the round's frozen CDF and claimed at once (claim0: the agent keeps its
 * weight for the round's other targets); after a grid barrier the claimers
 * settle the sub-block weights.  The few collisions left after round 0 are
 * redrawn per node by one CTA in later rounds (k_sel_rounds), with CTA
 * barriers only.  Round r of node n draws the (n, r, j) uniforms of the
 * oracle, so the CDF targets are the same whatever runs them, and which of
 * two targets on one agent claims it changes nothing (its strain draw is
 * keyed by the agent). */
__global__ void __launch_bounds__(256, 3) k_sel_round0(DevWorld W) {
  pdl_begin();
  const int R = W.n_reps, G = W.G;
  int any = 0;
  for (int r = 0; r < R; ++r) any |= (W.reps[r].active && W.reps[r].any_demand);
  if (!any) return; /* the same answer in every CTA: none waits at the barrier */
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t gsz = (int64_t)gridDim.x * blockDim.x;
  const SelInfo* info = reinterpret_cast<const SelInfo*>(W.sel_info);
  __shared__ int64_t s_K;
  __shared__ int64_t s_off[LPG_SEL_OFFS];
  const bool offs_in_smem = G < LPG_SEL_OFFS;

  /* target offsets of all nodes; every CTA computes the same values and
   * keeps them in shared memory when they fit */
  {
    int64_t carry = 0;
    for (int base = 0; base < G; base += 4 * blockDim.x) {
      /* 4 consecutive nodes a thread: one block scan per 4 * blockDim nodes */
      const int g0 = base + 4 * threadIdx.x;
      int64_t k[4], sum = 0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        k[u] = g0 + u < G ? __ldcg(&W.ksel[g0 + u]) : 0;
        sum += k[u];
      }
      int64_t tot;
      int64_t run = carry + block_excl_scan(sum, &tot);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (g0 + u < G) {
          if (offs_in_smem) s_off[g0 + u] = run;
          if (!offs_in_smem || blockIdx.x == 0) W.tgt_off[g0 + u] = run;
        }
        run += k[u];
      }
      carry += tot;
    }
    if (threadIdx.x == 0) {
      if (offs_in_smem) s_off[G] = carry;
      if (!offs_in_smem || blockIdx.x == 0) W.tgt_off[G] = carry;
      s_K = carry;
    }
    __syncthreads();
  }
  const int64_t K = s_K;
  if (K > W.hits_cap) { /* the same in every CTA */
    if (gtid == 0) W.reps[0].error = LPG_ERR_INTERNAL;
    return;
  }
  if (gtid == 0 && K) atomicAdd(&W.ctr[LPG_CTR_SEL_TARGETS], (unsigned long long)K);
  /* (when the offsets do not fit in shared memory, every CTA has written
   * all of them to tgt_off itself, so it reads its own values back) */
  const int64_t* offs = offs_in_smem ? s_off : W.tgt_off;
  /* Targets go round-robin over the CTAs (target q on CTA q mod grid), so
   * that a few thousand of them still use every SM, each located by a team
   * of T lanes: the largest power of two <= 32 with T * K <= threads, and
   * at least 8 (more targets than teams: each team takes several in turn;
   * smaller teams would hold more slots a lane than the registers of two
   * CTAs an SM allow). */
  int T = 8;
  while (T < 32 && (int64_t)(2 * T) * K <= gsz) T *= 2;
  bool ok;
  switch (T) {
    case 32: ok = round0_targets<32>(W, offs, info, K); break;
    case 16: ok = round0_targets<16>(W, offs, info, K); break;
    default: ok = round0_targets<8>(W, offs, info, K); break;
  }
  /* a CTA that never reached the barrier: the round is incomplete, and the
   * barrier's count is no longer to be trusted, so every replicate stops */
  if (!ok && threadIdx.x == 0)
    for (int r = 0; r < R; ++r)
      if (W.reps[r].active) W.reps[r].error = LPG_ERR_TIMEOUT;
}

/* Later rounds (after the round 0 claims): one CTA per node that still
 * lacks agents, rounds of its remaining target count over its current
 * weights until the node is served or has no susceptible weight left; then
 * the end of the tick (end_tick) for the CTA's nodes.  All threads of the
 * CTA run sel_rounds. */
__device__ __noinline__ void sel_rounds(DevWorld& W);
__device__ void end_tick(DevWorld& W, int64_t g0, int64_t gstride);
__global__ void __launch_bounds__(256) k_sel_rounds(DevWorld W) {
  pdl_begin();
  const int R = W.n_reps;
  int any = 0;
  for (int r = 0; r < R; ++r) any |= (W.reps[r].active && W.reps[r].any_demand);
  if (any) sel_rounds(W);
  /* every node of this CTA is served: the tick's rows of its nodes, and the
   * next tick's setup by the last CTA (end_tick) */
  __syncthreads();
  end_tick(W, blockIdx.x + (int64_t)threadIdx.x * gridDim.x, (int64_t)blockDim.x * gridDim.x);
}

__device__ __noinline__ void sel_rounds(DevWorld& W) {
  const int G = W.G;
  __shared__ int64_t s_off[LPG_SEL_OFFS];

  __shared__ int64_t s_k;
  __shared__ uint64_t s_T;
  __shared__ unsigned int s_won;
  __shared__ unsigned long long s_wsum;
  __shared__ SelInfo s_N;
  __shared__ int32_t s_need[256];
  __shared__ int32_t s_nneed;
  uint64_t* s_cp = reinterpret_cast<uint64_t*>(s_off);
  /* this CTA's nodes (g = blockIdx.x + j * grid) checked at once: which
   * still lack agents after round 0 */
  if (threadIdx.x == 0) s_nneed = 0;
  __syncthreads();
  for (int j = threadIdx.x; blockIdx.x + (int64_t)j * gridDim.x < G; j += blockDim.x) {
    const int g = blockIdx.x + j * gridDim.x;
    if (__ldcg(&W.ksel[g]) <= 0) continue;
    const int64_t k = __ldcg(&W.size[g]) - (int64_t)__ldcg((const unsigned long long*)&W.uniq[g]);
    if (k > 0 && __ldcg(&W.sw[g]) > 0) {
      const int at = atomicAdd(&s_nneed, 1);
      if (at < 256) s_need[at] = g;
    }
  }
  __syncthreads();
  const int nneed = s_nneed;
  for (int jn = 0; jn < (nneed < 256 ? nneed : 0) + (nneed >= 256 ? (G + gridDim.x - 1) / gridDim.x : 0); ++jn) {
    /* the listed nodes, or (list overflow) every node of the CTA in order */
    const int g = nneed < 256 ? s_need[jn] : blockIdx.x + jn * gridDim.x;
    if (g >= G) break;
    const DevRep* rp = &W.reps[W.node_rep[g]];
    if (!rp->active || !(rp->comps & LPG_COMP_TX)) continue;
    const int i = g - rp->node_base;
    const int32_t* st = W.node_chunk_start[rp->csr_cur] + rp->csr_base;
    const int32_t a = st[i], n = st[i + 1] - st[i];
    const int32_t* ls = W.node_chunks[rp->csr_cur] + rp->chunk_base + a;
    uint64_t* cp = W.cpref + rp->chunk_base + a;
    const bool local = n <= LPG_SEL_OFFS;
    /* this node's region of the target buffer: its own positions */
    uint32_t* hits = W.hits + (int64_t)(rp->chunk_base + a) * LPG_CHUNK;
    for (int round = 1; round < LPG_MAX_ROUNDS; ++round) {
      if (threadIdx.x == 0) {
        /* round 1 from the node's totals after round 0; later rounds from the
         * previous round's claims, all made by this CTA (the totals equal
         * these values: size - uniq, and sw less the claimed weights) */
        int64_t k;
        uint64_t T;
        if (round == 1) {
          k = __ldcg(&W.size[g]) - (int64_t)__ldcg((const unsigned long long*)&W.uniq[g]);
          T = __ldcg(&W.sw[g]);
        } else {
          k = s_k - (int64_t)s_won;
          T = s_T - s_wsum;
        }
        s_T = T;
        s_k = (k > 0 && T > 0) ? k : 0;
        s_won = 0;
        s_wsum = 0;
        if (s_k > 0) {
          atomicAdd(&W.ctr[LPG_CTR_SEL_TARGETS], (unsigned long long)s_k);
          atomicAdd(&W.ctr[LPG_CTR_SEL_NODE_ROUNDS], 1ULL);
          if (round == 1) { /* the node's strain thresholds are the same every round */
            s_N.seed = rp->seed;
            s_N.t = rp->cur_t;
            s_N.ns = rp->ns;
            sel_strain_cum(W, rp, g, s_N.thr);
          }
        }
      }
      __syncthreads();
      const int64_t k = s_k;
      const uint64_t T = s_T;
      if (k == 0) break;
      /* chunk prefix of the node (8 consecutive chunks a thread, every weight
       * requested at once, one CTA scan per 8 * blockDim chunks), in shared
       * memory when it fits */
      uint64_t carry = 0;
      for (int32_t a0 = 0; a0 < n; a0 += 8 * blockDim.x) {
        const int32_t i0 = a0 + 8 * threadIdx.x;
        uint64_t wv[8], sum = 0;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          wv[u] = i0 + u < n ? __ldcg(&W.chunk_w[ls[i0 + u]]) : 0;
          sum += wv[u];
        }
        int64_t tot;
        uint64_t run = carry + (uint64_t)block_excl_scan((int64_t)sum, &tot);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          run += wv[u];
          if (i0 + u < n) {
            if (local) s_cp[i0 + u] = run;
            else cp[i0 + u] = run;
          }
        }
        carry += (uint64_t)tot;
      }
      __syncthreads();
      int TT = 1;
      while (TT < 32 && (int64_t)(2 * TT) * k <= (int64_t)blockDim.x) TT *= 2;
      const Team tm = make_team(TT);
      for (int64_t j = threadIdx.x / TT; __any_sync(FULLMASK, j < k); j += blockDim.x / TT) {
        const bool act = j < k;
        const uint64_t v = act ? lpg_scale_target(lpg_u53(rp->seed, LPG_P_SELECT, rp->cur_t, (uint64_t)i, (uint64_t)round, (uint64_t)j), T) : 0;
        const uint32_t hit = locate_team(W, tm, ls, local ? s_cp : cp, n, v, 0, act);
        if (act && tm.l == 0) {
          if (hit == LPG_NONE) W.reps[W.node_rep[g]].error = LPG_ERR_INTERNAL;
          hits[j] = hit;
        }
      }
      __syncthreads();
      for (int64_t j = threadIdx.x; j < k; j += blockDim.x) {
        const uint32_t hit = hits[j];
        uint64_t w = 0;
        if (hit != LPG_NONE && claim(W, hit, g, s_N, &w)) {
          atomicAdd(&s_won, 1u);
          if (w) atomicAdd(&s_wsum, (unsigned long long)w);
        }
      }
      __threadfence_block();
      __syncthreads();
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Results rows of the tick and the tick advance. */
/* The tick's node rows (k_end_node), then the next tick's setup by the last
 * CTA: the stop rule (model.py:788-795: no node with E or I at this tick and
 * no seed after the next), the flags of every replicate (rep_prepare), the
 * due list emptied. */
__device__ void k_end_node(DevWorld& W, int g, int* ei_out);
/* The end of a tick for nodes g0, g0 + gstride, ... of this thread; all
 * threads of every CTA of the launch call it. */
__device__ void end_tick(DevWorld& W, int64_t g0, int64_t gstride) {
  __shared__ int s_last;
  for (int64_t g = g0; g < W.G; g += gstride) {
    int ei = 0;
    k_end_node(W, (int)g, &ei);
    /* stop rule input: nodes with E > 0 plus nodes with I > 0, per replicate */
    if (ei) atomicAdd(&W.reps[W.node_rep[g]].ei_sum, ei);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(W.end_done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int r = threadIdx.x; r < W.n_reps; r += blockDim.x) {
    DevRep* rp = &W.reps[r];
    const int ran = rp->active, sum = rp->ei_sum;
    rp->ei_sum = 0;
    const int tn = rp->t;
    if (ran && (rp->comps & LPG_COMP_DS) && rp->stop_if && !rp->stopped && !rp->error && tn < rp->nt && sum == 0 &&
        !rp->future_seed[tn])
      rp->stop_at = tn;
    rep_prepare(rp);
  }
  if (threadIdx.x == 0) {
    *W.due_n = 0; /* the due list of the tick is spent */
    *W.end_done = 0;
  }
}

/* The end of tick 0 (lpg_start); later ticks end in k_sel_rounds. */
__global__ void k_end(DevWorld W) {
  end_tick(W, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

__device__ void k_end_node(DevWorld& W, int g, int* ei_out) {
  DevRep* rp = &W.reps[W.node_rep[g]];
  /* every field of the replicate record this thread needs, read before the
   * first store (stores through int32_t* could otherwise alias them and
   * force a reload after each one) */
  const int active = rp->active;
  if (!active) return;
  const int i = g - rp->node_base, ns = rp->ns, t = rp->cur_t, G = W.G, n = rp->n_nodes;
  const uint32_t comps = rp->comps;
  const int vd_tick = rp->vd_tick, ri_tick = rp->ri_tick, ri_strain = rp->ri_strain;
  const int64_t nb_total = rp->nb_total;
  const int sia_n = rp->sia_n, sia_i0 = rp->sia_i0;
  const DevSia* sia = rp->sia;
  const int stop_at = rp->stop_at;
  int32_t* const res = rp->res;
  int64_t off[RS_N];
#pragma unroll
  for (int k = 0; k < RS_N; ++k) off[k] = rp->res_off[k];
  int32_t ev[EV_N];
#pragma unroll
  for (int k = 0; k < EV_N; ++k) ev[k] = W.ev[(int64_t)k * G + g];
  int32_t tt[TT_N];
#pragma unroll
  for (int k = 0; k < TT_N; ++k) tt[k] = W.tot[(int64_t)k * G + g];
  const int64_t row1 = (int64_t)t * n, rowS = (int64_t)t * n * ns;
#define ROW(k) (res + off[k] + row1)
#define ROWS(k) (res + off[k] + rowS)
  if (comps & LPG_COMP_TX) {
    int32_t e = 0, in = 0;
    for (int k = 0; k < ns; ++k) {
      const int32_t ek = tt[TT_E0 + k], ik = tt[TT_I0 + k];
      ROWS(RS_EBS)[i * ns + k] = ek;
      ROWS(RS_IBS)[i * ns + k] = ik;
      e += ek;
      in += ik;
    }
    ROW(RS_S)[i] = tt[TT_S];
    ROW(RS_E)[i] = e;
    ROW(RS_I)[i] = in;
    *ei_out = (e > 0 ? 1 : 0) + (in > 0 ? 1 : 0);
    ROW(RS_R)[i] += tt[TT_R];
    ROW(RS_POTP)[i] = tt[TT_POTP];
    ROW(RS_P)[i] = tt[TT_P];
  }
  if (t >= 1) {
    if (comps & LPG_COMP_DS) {
      ROW(RS_NEWPOTP)[i] = ev[EV_NEWPOT];
      ROW(RS_NEWP)[i] = ev[EV_NEWPAR];
    }
    if (vd_tick) {
      ROW(RS_DEATHS)[i] = ev[EV_DEATHS];
      if (nb_total > 0) ROW(RS_BIRTHS)[i] = ev[EV_BIRTHS];
    }
    int32_t ne = 0;
    int32_t nebs[LPG_MAX_STRAINS] = {0, 0, 0, 0};
    if (ri_tick) {
      const int32_t prot = ev[EV_RIPROT];
      ROW(RS_RIVAC)[i] = ev[EV_RIVAC];
      ROW(RS_RIPROT)[i] = prot;
      ROWS(RS_RINEWEXPBS)[i * ns + ri_strain] = prot;
      ROW(RS_IPVVAC)[i] = ev[EV_IPVVAC];
      ne += prot;
#pragma unroll
      for (int k = 0; k < LPG_MAX_STRAINS; ++k) nebs[k] += k == ri_strain ? prot : 0;
    }
    for (int k = 0; k < sia_n && k < LPG_MAX_SIA_PER_DAY; ++k) {
      const int sst = sia[sia_i0 + k].strain;
      int32_t vac = 0, prot = 0;
#pragma unroll
      for (int q = 0; q < LPG_MAX_SIA_PER_DAY; ++q)
        if (q == k) {
          vac = ev[EV_SIAVAC0 + q];
          prot = ev[EV_SIAPROT0 + q];
        }
      ROW(RS_SIAVAC)[i] = vac;
      ROW(RS_SIAPROT)[i] = prot;
      ROWS(RS_SIANEWEXPBS)[i * ns + sst] += prot;
      ne += prot;
#pragma unroll
      for (int q = 0; q < LPG_MAX_STRAINS; ++q) nebs[q] += q == sst ? prot : 0;
    }
    if (comps & LPG_COMP_TX) {
#pragma unroll
      for (int k = 0; k < LPG_MAX_STRAINS; ++k)
        if (k < ns) {
          const int32_t v = ev[EV_TXNEW0 + k];
          ne += v;
          nebs[k] += v;
        }
    }
    ROW(RS_NEWEXP)[i] += ne;
#pragma unroll
    for (int k = 0; k < LPG_MAX_STRAINS; ++k)
      if (k < ns) ROWS(RS_NEWEXPBS)[i * ns + k] += nebs[k];
  }
#undef ROW
#undef ROWS
  /* the tick's event counters are spent: cleared for the next */
#pragma unroll
  for (int k = 0; k < EV_N; ++k) W.ev[(int64_t)k * G + g] = 0;
  if (i == 0) {
    rp->t = t + 1;
    if (stop_at == t) rp->stopped = 1;
  }
}

/* ------------------------------------------------------------------------ */
/* Next events of the agents in E or I whose timers are as of tick tm (the
 * start: tm = 0), and their sub-blocks' earliest events (sub_evt cleared to
 * LPG_NO_DOD before). */
__global__ void k_init_events(DevWorld W, int32_t* evt, int32_t* sub_evt, int tm) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < W.n_reps; ++r) {
    const DevRep* rp = &W.reps[r];
    const int64_t n = (int64_t)rp->used_chunks * LPG_CHUNK;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
      const int64_t pos = (int64_t)rp->chunk_base * LPG_CHUNK + q;
      const int8_t ds = W.ds[pos];
      if (ds != 1 && ds != 2) continue;
      const int32_t e = tm + 1 + ev_pure(ds, W.strain[pos], W.et[pos], W.it[pos], W.pt[pos], W.pp[pos]);
      evt[pos] = e;
      atomicMin(&sub_evt[pos >> 7], e);
    }
  }
}

/* RI due ticks from their definition (base timer, reference index, date
 * of birth; lpg_ri.h) for every agent, and per sub-block the earliest due
 * tick after tick tl of its alive agents, written to out (LPG_NO_DOD for
 * none, or where RI does not run).  At the start (tl = 0) it also writes the
 * rdt column; the invariant check recounts with tl = the last tick run and
 * flags (bad) any rdt entry that differs from its definition.  One thread
 * per slot, a warp per 32 slots (4 warps per sub-block). */
__global__ void k_ri_index(DevWorld W, int32_t* out, int at_start, int* bad) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < W.n_reps; ++r) {
    const DevRep* rp = &W.reps[r];
    const bool on_r = ri_runs(rp);
    const int tl = at_start ? 0 : rp->t - 1;
    const int64_t p0 = (int64_t)rp->chunk_base * LPG_CHUNK, np = (int64_t)rp->used_chunks * LPG_CHUNK;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q - lane < np; q += stride) {
      const bool on = q < np;
      const int64_t pos = p0 + q;
      int32_t d = LPG_NO_DOD, m = LPG_NO_DOD;
      if (on && on_r) {
        const int8_t ds = W.ds[pos];
        if (W.cm[pos] != 1) d = ri_due_of(rp, W.ri[pos], W.ref[pos], W.dob[pos]);
        if (ds >= 0) {
          if (at_start) W.rdt[pos] = d;
          else if (W.rdt[pos] != d) atomicOr(bad, 256);
          if (d > tl) m = d;
        } else if (at_start) {
          W.rdt[pos] = d;
        }
      } else if (on && at_start) {
        W.rdt[pos] = LPG_NO_DOD;
      }
      m = __reduce_min_sync(FULLMASK, m);
      if (lane == 0 && q < np) atomicMin(&out[pos >> 7], m);
    }
  }
}

/* Recount of the sub-blocks' earliest events from the evt column (the
 * invariant check: the kept index must not exceed it). */
__global__ void k_count_events(DevWorld W, int32_t* sub_evt_out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < W.n_reps; ++r) {
    const DevRep* rp = &W.reps[r];
    const int64_t n = (int64_t)rp->used_chunks * LPG_CHUNK;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
      const int64_t pos = (int64_t)rp->chunk_base * LPG_CHUNK + q;
      const int8_t ds = W.ds[pos];
      if (ds == 1 || ds == 2) atomicMin(&sub_evt_out[pos >> 7], W.evt[pos]);
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Full recount of the running totals and selection weights (tick 0 and the
 * invariant check).  One CTA per chunk. */
__global__ void __launch_bounds__(LPG_SWEEP_THREADS) k_count(DevWorld W, int32_t* tot_out, uint64_t* sw_out,
                                                             uint64_t* bb_out, uint64_t* chunk_w_out,
                                                             uint64_t* sub_w_out, int32_t* sub_dod_out) {
  __shared__ int32_t s_tot[TT_N], s_dmin[LPG_NSUB];
  __shared__ unsigned long long s_sw, s_bb[LPG_MAX_STRAINS], s_sub[LPG_NSUB];
  for (int r = 0; r < W.n_reps; ++r) {
    const DevRep* rp = &W.reps[r];
    for (int32_t lc = blockIdx.x; lc < rp->used_chunks; lc += gridDim.x) {
      const int64_t cid = rp->chunk_base + lc;
      const int4 meta = W.cmeta[cid];
      const int g = meta.x;
      if (threadIdx.x < TT_N) s_tot[threadIdx.x] = 0;
      if (threadIdx.x < LPG_NSUB) {
        s_sub[threadIdx.x] = 0;
        s_dmin[threadIdx.x] = LPG_NO_DOD;
      }
      if (threadIdx.x < LPG_MAX_STRAINS) s_bb[threadIdx.x] = 0;
      if (threadIdx.x == 0) s_sw = 0;
      __syncthreads();
      const int fill = meta.y;
      /* a warp takes 32 consecutive slots (one sub-block's quarter): its
       * counts by ballot, its sums and minimum by warp reductions, one
       * shared-memory update per warp and quantity */
      const int lane = threadIdx.x & 31;
      for (int o0 = threadIdx.x & ~31; o0 < fill; o0 += blockDim.x) {
        const int o = o0 + lane;
        const int64_t pos = cid * LPG_CHUNK + o;
        const int8_t s = o < fill ? W.ds[pos] : (int8_t)-1;
        const bool alive = s >= 0;
        const int st = alive ? W.strain[pos] : 0;
        const int32_t dod = alive ? W.dod[pos] : LPG_NO_DOD;
        const uint64_t w = s == 0 ? fix_risk(W.risk[pos]) : 0;
        const uint64_t bw = s == 2 ? fix_beta(W.inf[pos], rp->strain_scal[st]) : 0;
        const bool potp = alive && W.pp[pos] == 1, par = alive && W.par[pos] == 1;
        const int32_t dmin = __reduce_min_sync(FULLMASK, dod);
        const int nS = __popc(__ballot_sync(FULLMASK, s == 0)), nR = __popc(__ballot_sync(FULLMASK, s == 3));
        const int nPotp = __popc(__ballot_sync(FULLMASK, potp)), nPar = __popc(__ballot_sync(FULLMASK, par));
        uint64_t ws = w;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) ws += __shfl_xor_sync(FULLMASK, ws, off);
        if (lane == 0) {
          atomicMin(&s_dmin[o0 / LPG_SUB], dmin);
          if (nS) atomicAdd(&s_tot[TT_S], nS);
          if (nR) atomicAdd(&s_tot[TT_R], nR);
          if (nPotp) atomicAdd(&s_tot[TT_POTP], nPotp);
          if (nPar) atomicAdd(&s_tot[TT_P], nPar);
          if (ws) {
            atomicAdd(&s_sw, (unsigned long long)ws);
            atomicAdd(&s_sub[o0 / LPG_SUB], (unsigned long long)ws);
          }
        }
        /* exposed and infectious agents are few: one update each */
        if (s == 1) atomicAdd(&s_tot[TT_E0 + st], 1);
        if (s == 2) {
          atomicAdd(&s_tot[TT_I0 + st], 1);
          if (bw) atomicAdd(&s_bb[st], (unsigned long long)bw);
        }
      }
      __syncthreads();
      if (threadIdx.x < TT_N && s_tot[threadIdx.x]) atomicAdd(&tot_out[(int64_t)threadIdx.x * W.G + g], s_tot[threadIdx.x]);
      if (threadIdx.x < LPG_MAX_STRAINS && s_bb[threadIdx.x])
        atomicAdd((unsigned long long*)&bb_out[(int64_t)threadIdx.x * W.G + g], s_bb[threadIdx.x]);
      if (threadIdx.x < LPG_NSUB) {
        sub_w_out[cid * LPG_NSUB + threadIdx.x] = s_sub[threadIdx.x];
        sub_dod_out[cid * LPG_NSUB + threadIdx.x] = s_dmin[threadIdx.x];
      }
      if (threadIdx.x == 0) {
        if (s_sw) atomicAdd((unsigned long long*)&sw_out[g], s_sw);
        chunk_w_out[cid] = s_sw;
      }
      __syncthreads();
    }
  }
}

#endif
