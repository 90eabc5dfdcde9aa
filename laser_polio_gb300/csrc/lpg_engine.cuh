/*
 * lpg_engine.cuh — device data layout of the GB300 per-tick agent step.
 *
 * Layout.  The reference keeps agents in one append-only table in slot
 * order (LaserFrame, laser_polio/model.py:139); within a node, agents appear
 * in slot order, but nodes interleave once births append new runs
 * (model.py:1730).  On the device the table is re-laid node-major: every
 * node owns an ordered list of CHUNK-slot chunks, and a chunk holds agents of
 * exactly one node, in the reference's slot order.  Births go to the tail of
 * their node's list.  So
 *   - the fused sweep processes whole chunks whose node is known up front
 *     (no per-agent node id read, no segmented reductions: one set of node
 *     counters per chunk);
 *   - a node's susceptible CDF in slot order (model.py:1108) is the
 *     concatenation of its chunks, indexed by per-chunk and per-SUB-slot
 *     susceptible weight totals kept exact in integers;
 *   - every column access is an aligned, coalesced vector access.
 * ref_slot[pos] maps each position back to the reference slot, which keys
 * all per-agent random draws and the copy back to the host.
 *
 * Aggregates.  Node totals the reference recounts every tick (count_SEIRP,
 * model.py:869-929; tx_step_prep, :932-1007) are kept as running integer
 * totals, updated by every transition that changes them (exact, so they
 * equal a recount bit for bit).  Susceptible acquisition risk is summed in
 * units of 2^-24, infectivity x strain scalar in units of 2^-40.
 */
#ifndef LPG_ENGINE_CUH
#define LPG_ENGINE_CUH

#include <stdint.h>

#include "lpg.h"
#include "lpg_rng.h"
#include "lpg_ri.h"

#define LPG_CHUNK 2048
#define LPG_SUB 128
#define LPG_NSUB (LPG_CHUNK / LPG_SUB)
#define LPG_SWEEP_THREADS 256
#define LPG_MAX_REPS 256
#define LPG_NO_DOD 0x7f7f7f7f /* "no alive agent": bytes 0x7f, above every date of death */
#define LPG_SWEEP_CONSUMERS 256
#define LPG_SWEEP_BLOCK (LPG_SWEEP_CONSUMERS + 32)

/* per-tick event counters per node */
enum {
  EV_DEATHS = 0,
  EV_BIRTHS = 1,
  EV_NEWPOT = 2,
  EV_NEWPAR = 3,
  EV_RIVAC = 4,
  EV_RIPROT = 5,
  EV_IPVVAC = 6,
  EV_SIAVAC0 = 7,
  EV_SIAPROT0 = EV_SIAVAC0 + LPG_MAX_SIA_PER_DAY,
  EV_TXNEW0 = EV_SIAPROT0 + LPG_MAX_SIA_PER_DAY,
  EV_N = EV_TXNEW0 + LPG_MAX_STRAINS
};

/* running totals per node */
enum {
  TT_S = 0,
  TT_R = 1,
  TT_POTP = 2,
  TT_P = 3,
  TT_E0 = 4,
  TT_I0 = TT_E0 + LPG_MAX_STRAINS,
  TT_N = TT_I0 + LPG_MAX_STRAINS
};

/* results fields, in the order of lpg_results_view */
enum {
  RS_S, RS_E, RS_I, RS_R, RS_EBS, RS_IBS, RS_POTP, RS_P, RS_NEWPOTP, RS_NEWP, RS_POP, RS_BIRTHS, RS_DEATHS,
  RS_NEWEXP, RS_NEWEXPBS, RS_RIVAC, RS_RIPROT, RS_RINEWEXPBS, RS_IPVVAC, RS_SIAVAC, RS_SIAPROT, RS_SIANEWEXPBS,
  RS_N
};

typedef struct {
  int32_t tick, strain, min_age, max_age;
  double efficacy;
  const uint8_t* mask;     /* device, [n_nodes] */
  const uint64_t* thr_vac; /* [n_nodes] u < p            <=> u53 < thr_vac  */
  const uint64_t* thr_pro; /* [n_nodes] u < p * efficacy <=> u53 < thr_pro  */
} DevSia;

typedef struct {
  int32_t tick, node, is_count, pad;
  double value;
} DevSeed;

/* Per-simulation device record. */
typedef struct {
  /* static */
  int32_t n_nodes, ns, nt, comps;
  int32_t stop_if, vd_step, ri_step, ri_enabled;
  int32_t ri_strain, km_len, km_max_year, nb_r;
  double nb_d, nb_c; /* Marsaglia–Tsang's constants of nb_r (lpg_gamma_consts) when nb_r >= 1 */
  int32_t node_base;  /* first global node id */
  int32_t chunk_base; /* first chunk id */
  int32_t chunk_cap;  /* chunks reserved */
  int32_t csr_base;   /* offset of this sim's node_chunk_start entries (n_nodes + 1) */
  int64_t count0, capacity;
  uint64_t seed;
  float p_par;
  int32_t pad0;
  uint64_t thr_par;        /* u < p_paralysis <=> u53 < thr_par */
  const uint64_t* thr_ri;  /* [n_nodes] */
  const uint64_t* thr_ipv; /* [n_nodes] */
  double zi;
  int32_t dur_kind;
  int32_t pad1;
  double dur_p1, dur_p2;
  const double* birth_rate;
  const double* p_ri;
  const double* p_ipv;
  const double* strain_scal;
  const double* net;   /* network[i][j], row-major */
  const uint64_t* netq_t; /* transposed, in two fixed-point parts: netq_t[j][i][0..1] = network[i][j] (lpg_net_split) */
  const double* rowsum;
  const double* r0s;
  const double* seas;
  const float* p_sia;
  const int64_t* km;
  const int32_t* sia_first; /* [nt] index into sia[] of the first event of the tick */
  const int32_t* sia_cnt;   /* [nt] */
  const DevSia* sia;
  const int32_t* seed_first;
  const int32_t* seed_cnt;
  const DevSeed* seeds;
  const uint8_t* future_seed; /* [nt] 1 if a seed event is scheduled after tick t */
  int32_t* res;               /* results base */
  int64_t res_off[RS_N];
  /* aggregates the expected-incidence map replays, recorded by k_node_tx
   * when lpg_record_aggregates asked for them, else NULL: per tick and
   * node, [0] the susceptibles' summed risk, [1] the population, [2] the
   * expected new exposures, [3 + s] the pre-mixing infectivity of strain s
   * ([nt][n_nodes][3 + ns]) */
  double* rec;
  /* unborn pool columns, indexed by reference slot - count0 */
  int8_t *pl_et, *pl_it, *pl_pt, *pl_strain, *pl_pp, *pl_par, *pl_ipv;
  uint8_t* pl_cm;
  int16_t* pl_ri;
  float *pl_risk, *pl_inf;
  /* dynamic */
  int32_t t;       /* next tick */
  int32_t stopped; /* early stop happened */
  int32_t stop_at; /* tick at which the stop rule fired, or INT32_MAX */
  int32_t error;
  int64_t count;
  int32_t used_chunks;
  int32_t csr_cur; /* which CSR buffer is current */
  int32_t started;
  /* per-tick, written by k_begin */
  int32_t cur_t, active, vd_tick, ri_tick;
  int32_t sia_n, sia_i0, seed_n, seed_i0;
  int64_t nb_total, count_before;
  int32_t any_demand;
  int32_t csr_flip;    /* the node -> chunk lists were rebuilt this tick (k_newborns fills them) */
  int32_t used_before; /* used_chunks before this tick's new chunks */
  int32_t ei_sum;      /* k_end: nodes with E > 0 plus nodes with I > 0 (the next tick's stop rule) */
} DevRep;

/* Global device state shared by the kernels of one handle. */
typedef struct {
  int32_t n_reps, G; /* replicates, global nodes */
  int32_t total_chunks;
  int32_t stall_after; /* test hook (lpg_test_stall_sweep): the staged sweep's producer issues only this many
                          stages (-1: all) */
  int64_t wait_spin;   /* iterations of the staged sweep's consumer waits before they give up */
  DevRep* reps;
  /* per position */
  int8_t *ds, *strain, *et, *it, *pt, *pp, *par, *ipv;
  uint8_t* cm;
  int16_t* ri; /* where RI runs: alive, not chronically-missed agents keep the timer before their
                  first RI tick (lpg_ri.h); the dead keep the value they died with */
  float *risk, *inf;
  int32_t *dob, *dod;
  int32_t* evt; /* agents in E or I: tick of the next disease-state step that is an event */
  int32_t* rdt; /* RI due tick (lpg_ri.h), LPG_NO_DOD for the chronically missed or where RI does not run */
  uint32_t* ref;
  /* per chunk */
  int4* cmeta; /* per chunk: x node, y fill, z tick of the newborns written into it, w offset of the first */
  uint64_t* chunk_w;  /* susceptible weight total */
  uint64_t* sub_w;    /* [chunk][LPG_NSUB] */
  int32_t* sub_evt;   /* [chunk][LPG_NSUB] earliest evt of the sub-block's agents in E or I, a lower
                         bound (LPG_NO_DOD when none): only sub-blocks with an event due are read */
  int32_t* sub_dod;   /* [chunk][LPG_NSUB] earliest date of death of the sub-block's alive agents
                         (LPG_NO_DOD when it has none); deaths on a VD tick need only the
                         sub-blocks whose earliest date has come */
  int32_t* sub_rdt;   /* [chunk][LPG_NSUB] earliest RI due tick of the sub-block's alive, not
                         chronically-missed agents, a lower bound (LPG_NO_DOD when none): RI
                         ticks read only the sub-blocks with an agent due */
  uint64_t* cpref;    /* selection: node-local prefix of chunk weights, CSR order */
  int32_t* node_chunks[2];
  int32_t* node_chunk_start[2]; /* per sim: n_nodes + 1 entries at csr_base */
  /* per global node */
  int32_t* node_rep;
  int64_t* node_count;
  int32_t* ev;  /* [EV_N][G] */
  int32_t* tot; /* [TT_N][G] */
  uint64_t* sw; /* [G] */
  uint64_t* bb; /* [LPG_MAX_STRAINS][G] */
  int64_t* nb_end;
  int64_t* nb_li0;
  double* prob; /* [LPG_MAX_STRAINS][G] */
  double* inck; /* [LPG_MAX_STRAINS][G] incoming infectivity of the tick (k_node_mix) */
  int64_t* size;
  int64_t* uniq;
  int64_t* ksel;
  int64_t* tgt_off; /* [G + 1] */
  void* sel_info;     /* [G] SelInfo: per-node selection record of the tick */
  uint32_t* hits; /* selection targets */
  int64_t hits_cap;
  uint64_t* evq;     /* event queues of the sweeps: one slab per sweep CTA */
  uint32_t* qcnt;    /* [2][1024] entries per slab (k_sweep_due, k_sweep_rs) */
  uint32_t* qfirst;  /* [2][1024] first entry of the slab of each sweep CTA in evq */
  uint64_t* due;     /* sub-blocks with something due this tick: sub-block | sim << 32 | what << 48 */
  uint32_t* due_n;   /* entries of due (k_due appends, k_end clears) */
  unsigned long long* ctr; /* [LPG_NUM_COUNTERS] work counters */
  uint32_t* end_done;      /* CTAs of k_end done with the tick (the last prepares the next) */
  unsigned long long* grid_bar; /* arrivals at k_sel_round0's grid barrier (only grows) */
  int32_t test_bar_skip;   /* test hook: CTA 0 of k_sel_round0 does not arrive at its barrier */
} DevWorld;

#endif
