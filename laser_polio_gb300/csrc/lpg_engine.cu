/*
 * lpg_engine.cu — host side of the C ABI in include/lpg.h.
 *
 * Owns the device state of a handle (one or more simulations on one GPU),
 * lays the reference-ordered agent columns out node-major on the device,
 * and launches the per-tick kernel sequence of lpg_kernels.cuh, captured
 * once in a CUDA graph and replayed per tick.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lpg.h"
#include <utility>

#include "lpg_kernels.cuh"

namespace {

/* Kernels a tick needs only on some ticks (births: k_begin, k_newborns;
 * seeds; RI/SIA); the host knows the schedule, so a tick without them does
 * not launch them. */
enum { NEED_NB = 1, NEED_SEED = 2, NEED_RS = 4 };
static bool kernel_needed(int k, uint8_t need) {
  switch (k) {
    case 0:
    case 1: return (need & NEED_NB) != 0;
    case 4: return (need & NEED_SEED) != 0;
    case 5:
    case 6: return (need & NEED_RS) != 0;
    default: return true;
  }
}

const char* kKernelNames[] = {"k_begin", "k_newborns", "k_due", "k_sweep_a", "k_seed", "k_sweep_b",
                              "k_evb", "k_node_mix", "k_node_tx", "k_sel_round0", "k_sel_rounds"};
constexpr int kNumTickKernels = 11; /* k_sel_rounds ends the tick (results rows, next tick's setup) */
constexpr int kTicksPerGraph = 8;

/* Reference-ordered columns of one simulation on the device. */
struct Staging {
  int8_t *ds = nullptr, *strain = nullptr, *et = nullptr, *it = nullptr, *pt = nullptr, *pp = nullptr, *par = nullptr,
         *ipv = nullptr;
  uint8_t* cm = nullptr;
  int16_t *node = nullptr, *ri = nullptr;
  float *risk = nullptr, *inf = nullptr;
  int32_t *dob = nullptr, *dod = nullptr;
  void* base = nullptr; /* the one allocation the columns are carved from */
  bool bound = false;
};

struct SimHost {
  lpg_sim_desc d;
  std::vector<double> birth_rate, p_ri, p_ipv, strain_scal, net, rowsum, r0s, seas;
  std::vector<uint64_t> netq_t;
  std::vector<float> p_sia;
  std::vector<int64_t> km;
  std::vector<lpg_seed_event> seeds;
  std::vector<lpg_sia_event> sia;
  std::vector<std::vector<uint8_t>> sia_masks;
  std::vector<int32_t> pop0, Rpre;
  Staging stg;
  int64_t res_elems = 0;
  bool record = false; /* lpg_record_aggregates */
};

}  // namespace

struct lpg_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<SimHost> sims;
  std::vector<DevRep> hreps;
  DevWorld W{};
  std::vector<void*> allocs;
  bool started = false;
  std::string err;
  bool use_graphs = true;
  int32_t test_stall_after = -1; /* lpg_test_stall_sweep */
  int64_t test_wait_spin = 0;
  int32_t test_bar_skip = 0;     /* lpg_test_stall_round0 */
  std::map<uint32_t, std::pair<cudaGraphExec_t, int>> graphs; /* by the needs of 8 ticks: graph, launches */
  bool graph_failed = false;
  std::vector<uint8_t> tick_need; /* per tick: the optional kernels some simulation needs (NEED_*) */
  int32_t next_tick = 0;          /* the tick the next launch runs */
  bool profiling = false;
  double prof_ms[16] = {0};
  int64_t prof_n[16] = {0};
  std::vector<cudaEvent_t> ev_pool;
  int64_t launches = 0;
  int sm_count = 0;
  int sweep_blocks = 0;  /* k_sweep_rs (staged through shared memory) */
  int sweep0_blocks = 0; /* k_sweep_due (direct loads, no staging) */
  int due_blocks = 0;    /* k_due */
  int select_blocks = 0; /* k_sel_round0 (cooperative: at most round0_max) */
  int round0_max = 0;    /* CTAs of k_sel_round0 that fit on the GPU at once */
  int rounds_blocks = 0; /* k_sel_rounds */
  int evb_blocks = 0;
  int newborn_blocks = 0; /* per replicate */
  bool node_batch_tx = false;  /* the draws one node a thread (k_node_tx_lanes) */
  bool node_batch_mix = false; /* the mixing one warp a node (k_node_mix<1>) */
};

static int fail(lpg_handle* h, int code, const char* fmt, ...) {
  if (h) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    h->err = buf;
  }
  return code;
}

#define CK(call)                                                                                       \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess) return fail(h, LPG_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                       __FILE__, __LINE__);                                            \
  } while (0)

template <typename T>
static int dalloc(lpg_handle* h, T** p, size_t n) {
  size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) return fail(h, LPG_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
  h->allocs.push_back((void*)*p);
  return 0;
}

template <typename T>
static int dupload(lpg_handle* h, T** p, const std::vector<T>& v) {
  int rc = dalloc(h, p, v.size());
  if (rc) return rc;
  if (!v.empty()) CK(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
  return 0;
}

static void dfree_one(lpg_handle* h, void* p) {
  if (!p) return;
  cudaFree(p);
  auto it = std::find(h->allocs.begin(), h->allocs.end(), p);
  if (it != h->allocs.end()) h->allocs.erase(it);
}

__global__ void k_fill_f32(float* p, int64_t n, float v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

/* Node histogram of slots [0, count), node-id range check and sortedness. */
__global__ void k_hist(const int16_t* node, int64_t count, int n_nodes, unsigned long long* cnt, int* flags) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    int v = node[i];
    const unsigned act = __activemask();
    if (v < 0 || v >= n_nodes) {
      atomicOr(&flags[0], 1);
      v = -1;
    } else if (i + 1 < count && node[i + 1] < v) {
      atomicOr(&flags[1], 1);
    }
    /* one atomic per distinct node id in the warp */
    const unsigned peers = __match_any_sync(act, v);
    if (v >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&cnt[v], (unsigned long long)__popc(peers));
  }
}

struct ScatterArgs {
  Staging s;
  int64_t count;
  const int32_t* node_chunk0; /* first chunk id of each local node */
  const int64_t* node_first;  /* first slot of each node (sorted input) */
  const int32_t* rank;        /* rank within node (unsorted input), or null */
};

/* One agent of the reference order into its slot of the node-major layout. */
__device__ __forceinline__ void scatter_one(const DevWorld& W, const ScatterArgs& a, int64_t i) {
  const int n = a.s.node[i];
  const int64_t rk = a.rank ? (int64_t)a.rank[i] : i - a.node_first[n];
  const int64_t pos = (int64_t)a.node_chunk0[n] * LPG_CHUNK + rk; /* a node's chunks are consecutive */
  W.ds[pos] = a.s.ds[i];
  W.strain[pos] = a.s.strain[i];
  W.et[pos] = a.s.et[i];
  W.it[pos] = a.s.it[i];
  W.pt[pos] = a.s.pt[i];
  W.pp[pos] = a.s.pp[i];
  W.par[pos] = a.s.par[i];
  W.ipv[pos] = a.s.ipv[i];
  W.cm[pos] = a.s.cm[i];
  W.ri[pos] = a.s.ri[i];
  W.risk[pos] = a.s.risk[i];
  W.inf[pos] = a.s.inf[i];
  W.dob[pos] = a.s.dob[i];
  W.dod[pos] = a.s.dod[i];
  W.ref[pos] = (uint32_t)i;
}

/* 16 slots of one column from 16 consecutive agents: element loads (the
 * source run may start anywhere), packed into 16-byte stores (the slots
 * start at a multiple of 16). */
__device__ __forceinline__ void fill16(int8_t* __restrict__ dst, const int8_t* __restrict__ src) {
  uint32_t w[4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
    w[j] = (uint32_t)(uint8_t)__ldg(src + 4 * j) | (uint32_t)(uint8_t)__ldg(src + 4 * j + 1) << 8 |
           (uint32_t)(uint8_t)__ldg(src + 4 * j + 2) << 16 | (uint32_t)(uint8_t)__ldg(src + 4 * j + 3) << 24;
  *reinterpret_cast<uint4*>(dst) = make_uint4(w[0], w[1], w[2], w[3]);
}
__device__ __forceinline__ void fill16(uint8_t* dst, const uint8_t* src) {
  fill16(reinterpret_cast<int8_t*>(dst), reinterpret_cast<const int8_t*>(src));
}
__device__ __forceinline__ void fill16(int16_t* __restrict__ dst, const int16_t* __restrict__ src) {
  uint32_t w[8];
#pragma unroll
  for (int j = 0; j < 8; ++j)
    w[j] = (uint32_t)(uint16_t)__ldg(src + 2 * j) | (uint32_t)(uint16_t)__ldg(src + 2 * j + 1) << 16;
  reinterpret_cast<uint4*>(dst)[0] = make_uint4(w[0], w[1], w[2], w[3]);
  reinterpret_cast<uint4*>(dst)[1] = make_uint4(w[4], w[5], w[6], w[7]);
}
template <typename T>
__device__ __forceinline__ void fill16_32(T* __restrict__ dst, const T* __restrict__ src) {
  static_assert(sizeof(T) == 4, "32-bit columns");
  const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
#pragma unroll
  for (int j = 0; j < 4; ++j)
    reinterpret_cast<uint4*>(dst)[j] = make_uint4(__ldg(s + 4 * j), __ldg(s + 4 * j + 1), __ldg(s + 4 * j + 2),
                                                  __ldg(s + 4 * j + 3));
}

/* The reference-ordered columns of sorted input into the node-major layout,
 * slot-driven: a thread fills 16 slots of a chunk from the agents that go
 * there (a node's agents are a contiguous run of the input and its chunks
 * consecutive), so every store is a full 16-byte vector; the last partial
 * group of a chunk slot by slot. */
__global__ void k_scatter_sorted(DevWorld W, ScatterArgs a, int32_t chunk_base, int32_t used, int32_t node_base) {
  const int64_t groups = (int64_t)used * (LPG_CHUNK / 16);
  for (int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gi < groups; gi += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cid = chunk_base + gi / (LPG_CHUNK / 16);
    const int o0 = (int)(gi % (LPG_CHUNK / 16)) * 16;
    const int4 meta = W.cmeta[cid];
    if (o0 >= meta.y) continue;
    const int nl = meta.x - node_base;
    const int64_t i0 = a.node_first[nl] + (cid - a.node_chunk0[nl]) * LPG_CHUNK + o0;
    const int64_t p0 = cid * LPG_CHUNK + o0;
    if (o0 + 16 <= meta.y) {
      fill16(W.ds + p0, a.s.ds + i0);
      fill16(W.strain + p0, a.s.strain + i0);
      fill16(W.et + p0, a.s.et + i0);
      fill16(W.it + p0, a.s.it + i0);
      fill16(W.pt + p0, a.s.pt + i0);
      fill16(W.pp + p0, a.s.pp + i0);
      fill16(W.par + p0, a.s.par + i0);
      fill16(W.ipv + p0, a.s.ipv + i0);
      fill16(W.cm + p0, a.s.cm + i0);
      fill16(W.ri + p0, a.s.ri + i0);
      fill16_32(W.risk + p0, a.s.risk + i0);
      fill16_32(W.inf + p0, a.s.inf + i0);
      fill16_32(W.dob + p0, a.s.dob + i0);
      fill16_32(W.dod + p0, a.s.dod + i0);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        reinterpret_cast<uint4*>(W.ref + p0)[j] = make_uint4((uint32_t)(i0 + 4 * j), (uint32_t)(i0 + 4 * j + 1),
                                                             (uint32_t)(i0 + 4 * j + 2), (uint32_t)(i0 + 4 * j + 3));
    } else {
      for (int k = 0; k < meta.y - o0; ++k) scatter_one(W, a, i0 + k);
    }
  }
}

/* Unsorted input: agent by agent, each to the slot of its rank in its node. */
__global__ void k_scatter(DevWorld W, ScatterArgs a) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.count; i += (int64_t)gridDim.x * blockDim.x)
    scatter_one(W, a, i);
}

/* Columns of one simulation (rep) back in reference slot order.  Timers of
 * agents in E or I are brought up to the step of tick tc (the last that has
 * run) when the simulation steps disease states (ds_on); RI timers of the
 * alive, not chronically-missed agents to the RI ticks up to tc when RI
 * runs. */
__global__ void k_gather(DevWorld W, Staging s, int32_t chunk_base, int32_t used, int32_t node_base, int32_t tc,
                         int ds_on, int rep) {
  const DevRep* rp = &W.reps[rep];
  const bool ri_on = ri_runs(rp);
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < (int64_t)used * LPG_CHUNK;
       q += (int64_t)gridDim.x * blockDim.x) {
    int64_t cid = chunk_base + q / LPG_CHUNK;
    int o = (int)(q % LPG_CHUNK);
    const int4 meta = W.cmeta[cid];
    if (o >= meta.y) continue;
    int64_t pos = cid * LPG_CHUNK + o;
    uint32_t i = W.ref[pos];
    const int8_t ds = W.ds[pos], st = W.strain[pos], pp = W.pp[pos];
    const uint8_t cm = W.cm[pos];
    int8_t et = W.et[pos], it = W.it[pos], pt = W.pt[pos];
    if (ds_on && (ds == 1 || ds == 2)) /* the count-downs up to the step of tick tc */
      ev_advance(ds, st, et, it, pt, tc - W.evt[pos] + 1 + ev_pure(ds, st, et, it, pt, pp));
    s.ds[i] = ds;
    s.strain[i] = st;
    s.et[i] = et;
    s.it[i] = it;
    s.pt[i] = pt;
    s.pp[i] = pp;
    s.par[i] = W.par[pos];
    s.ipv[i] = W.ipv[pos];
    s.cm[i] = cm;
    s.node[i] = (int16_t)(meta.x - node_base);
    int16_t ri = W.ri[pos];
    if (ri_on && ds >= 0 && cm != 1) ri = ri_now(rp, ri, i, W.dob[pos], tc);
    s.ri[i] = ri;
    s.risk[i] = W.risk[pos];
    s.inf[i] = W.inf[pos];
    s.dob[i] = W.dob[pos];
    s.dod[i] = W.dod[pos];
  }
}

__global__ void k_cmp_counts(DevWorld W, const int32_t* tot, const uint64_t* sw, const uint64_t* bb,
                             const uint64_t* cw, const uint64_t* subw, const int32_t* subd, const int32_t* sube,
                             const int32_t* subr, int* bad) {
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid < W.G) {
    for (int k = 0; k < TT_N; ++k)
      if (tot[(int64_t)k * W.G + gid] != W.tot[(int64_t)k * W.G + gid]) atomicOr(bad, 1);
    if (sw[gid] != W.sw[gid]) atomicOr(bad, 2);
    for (int k = 0; k < LPG_MAX_STRAINS; ++k)
      if (bb[(int64_t)k * W.G + gid] != W.bb[(int64_t)k * W.G + gid]) atomicOr(bad, 4);
  }
  for (int r = 0; r < W.n_reps; ++r) {
    const DevRep* rp = &W.reps[r];
    for (int64_t q = gid; q < rp->used_chunks; q += (int64_t)gridDim.x * blockDim.x) {
      int64_t cid = rp->chunk_base + q;
      if (cw[cid] != W.chunk_w[cid]) atomicOr(bad, 8);
      for (int s = 0; s < LPG_NSUB; ++s) {
        if (subw[cid * LPG_NSUB + s] != W.sub_w[cid * LPG_NSUB + s]) atomicOr(bad, 16);
        if (subd[cid * LPG_NSUB + s] != W.sub_dod[cid * LPG_NSUB + s]) atomicOr(bad, 32);
        if (W.sub_evt[cid * LPG_NSUB + s] > sube[cid * LPG_NSUB + s]) atomicOr(bad, 64);
        if (W.sub_rdt[cid * LPG_NSUB + s] > subr[cid * LPG_NSUB + s]) atomicOr(bad, 128);
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
extern "C" int lpg_version(void) { return LPG_ABI_VERSION; }

extern "C" const char* lpg_last_error(const lpg_handle* h) { return h ? h->err.c_str() : "null handle"; }

extern "C" void* lpg_cuda_stream(lpg_handle* h) { return h ? (void*)h->stream : nullptr; }

extern "C" int64_t lpg_kernel_launches(lpg_handle* h) { return h ? h->launches : 0; }

/* Integer threshold T with  u < p  <=>  m < T  for u = m * 2^-53, m a 53-bit
 * integer: T = ceil(p * 2^53) clamped to [0, 2^53] (p * 2^53 is exact). */
static uint64_t u53_threshold(double p) {
  if (!(p > 0.0)) return 0;
  if (p >= 1.0) return 1ULL << 53;
  return (uint64_t)std::ceil(p * 9007199254740992.0);
}

static const int res_wide[RS_N] = {0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 1};

/* Every check lpg_create makes on one simulation's description: sizes,
 * required arrays, event ranges, and that every parameter array holds finite
 * values in its range (the reference raises ValueError on such inputs, e.g.
 * model.py:169-170, 602, 687, 702, 770, 1256; a NaN here would silently turn
 * into zero probabilities on the device). */
static int validate_desc(const lpg_sim_desc& d, int r, std::string* msg) {
  char buf[256];
  auto bad = [&](int code, const char* fmt, auto... args) {
    snprintf(buf, sizeof buf, fmt, args...);
    *msg = buf;
    return code;
  };
  if (d.n_nodes < 1 || d.n_nodes > 32767) return bad(LPG_ERR_ARG, "sim %d: n_nodes %d out of range", r, d.n_nodes);
  if (d.n_strains < 1 || d.n_strains > LPG_MAX_STRAINS)
    return bad(LPG_ERR_ARG, "sim %d: n_strains %d out of range [1, %d]", r, d.n_strains, LPG_MAX_STRAINS);
  if (d.nt < 1) return bad(LPG_ERR_ARG, "sim %d: nt must be >= 1", r);
  if (d.count < 0 || d.capacity < d.count || d.capacity >= (int64_t)0xFFFFFFF0LL)
    return bad(LPG_ERR_ARG, "sim %d: count %lld / capacity %lld invalid", r, (long long)d.count, (long long)d.capacity);
  if (d.vd_step < 1 || d.ri_step < 1) return bad(LPG_ERR_ARG, "sim %d: step sizes must be >= 1", r);
  /* an agent's RI timer comes back into the window no sooner than 65536 / step - 1 RI ticks
   * after it was there, so no agent is due twice while the last RI tick's index is below
   * 65536 / step; the engine gives each agent one RI due tick a run */
  if ((d.components & LPG_COMP_RI) && d.ri_enabled && (d.nt - 1) / d.ri_step >= 65536 / d.ri_step)
    return bad(LPG_ERR_ARG, "sim %d: RI over %d ticks with step %d: an agent's RI timer would come round twice", r,
               d.nt - 1, d.ri_step);
  if (!d.pop0) return bad(LPG_ERR_ARG, "sim %d: pop0 is required", r);
  if ((d.components & LPG_COMP_TX) && (!d.network || !d.seasonality || !d.strain_r0_scalars || !d.r0_scalars))
    return bad(LPG_ERR_ARG, "sim %d: transmission needs network, seasonality and scalars", r);
  if (d.km_len < 1 || !d.km_cumdeaths) return bad(LPG_ERR_ARG, "sim %d: km table required", r);
  const size_t n = (size_t)d.n_nodes;
  auto check = [&](const double* a, size_t k, double lo, double hi, const char* name) -> int {
    if (!a) return 0;
    for (size_t i = 0; i < k; ++i)
      if (!std::isfinite(a[i]) || a[i] < lo || a[i] > hi)
        return bad(LPG_ERR_ARG, "sim %d: %s[%zu] = %g is not finite or outside [%g, %g]", r, name, i, a[i], lo, hi);
    return 0;
  };
  const double inf = HUGE_VAL;
  int rc = 0;
  if ((rc = check(d.birth_rate, n, 0.0, inf, "birth_rate"))) return rc;
  if ((rc = check(d.vx_prob_ri, n, 0.0, 1.0, "vx_prob_ri"))) return rc;
  if ((rc = check(d.vx_prob_ipv, n, 0.0, 1.0, "vx_prob_ipv"))) return rc;
  if ((rc = check(d.strain_r0_scalars, (size_t)d.n_strains, 0.0, inf, "strain_r0_scalars"))) return rc;
  if ((rc = check(d.network, n * n, 0.0, inf, "network"))) return rc;
  if ((rc = check(d.r0_scalars, n, 0.0, inf, "r0_scalars"))) return rc;
  if ((rc = check(d.seasonality, (size_t)d.nt, -inf, inf, "seasonality"))) return rc;
  if (d.vx_prob_sia)
    for (size_t i = 0; i < n; ++i)
      if (!std::isfinite(d.vx_prob_sia[i]) || d.vx_prob_sia[i] < 0.0f || d.vx_prob_sia[i] > 1.0f)
        return bad(LPG_ERR_ARG, "sim %d: vx_prob_sia[%zu] = %g is not finite or outside [0, 1]", r, i,
                   (double)d.vx_prob_sia[i]);
  if (!std::isfinite(d.p_paralysis) || d.p_paralysis < 0.0f || d.p_paralysis > 1.0f)
    return bad(LPG_ERR_ARG, "sim %d: p_paralysis %g outside [0, 1]", r, (double)d.p_paralysis);
  if (!std::isfinite(d.zero_inflation) || d.zero_inflation < 0.0)
    return bad(LPG_ERR_ARG, "sim %d: zero inflation %g is not finite and >= 0", r, d.zero_inflation);
  for (int i = 0; i < (int)n; ++i)
    if (d.pop0[i] < 0) return bad(LPG_ERR_ARG, "sim %d: pop0[%d] = %d is negative", r, i, d.pop0[i]);
  for (int k = 0; k < d.n_seeds; ++k) {
    const lpg_seed_event& e = d.seeds[k];
    if (e.node < 0 || e.node >= d.n_nodes) return bad(LPG_ERR_NODE, "sim %d: seed event node %d out of range", r, e.node);
    if (!std::isfinite(e.value) || e.value < 0.0) return bad(LPG_ERR_ARG, "sim %d: seed event value %g", r, e.value);
  }
  std::vector<int32_t> per_tick(d.nt, 0);
  for (int k = 0; k < d.n_sia; ++k) {
    const lpg_sia_event& e = d.sia[k];
    if (e.tick < 0 || e.tick >= d.nt) continue;
    if (e.strain < 0 || e.strain >= d.n_strains) return bad(LPG_ERR_ARG, "sim %d: SIA strain out of range", r);
    if (!std::isfinite(e.efficacy)) return bad(LPG_ERR_ARG, "sim %d: SIA efficacy %g is not finite", r, e.efficacy);
    if (++per_tick[e.tick] > LPG_MAX_SIA_PER_DAY)
      return bad(LPG_ERR_ARG, "sim %d: more than %d SIA events on tick %d", r, LPG_MAX_SIA_PER_DAY, e.tick);
  }
  if (d.ri_strain < 0 || d.ri_strain >= d.n_strains) return bad(LPG_ERR_ARG, "sim %d: RI strain out of range", r);
  return LPG_OK;
}

int lpg_ops_fail(int code, const char* fmt, ...);

extern "C" int lpg_check_desc(const lpg_sim_desc* d) {
  if (!d) return lpg_ops_fail(LPG_ERR_ARG, "null description");
  std::string msg;
  const int rc = validate_desc(*d, 0, &msg);
  if (rc) return lpg_ops_fail(rc, "%s", msg.c_str());
  return LPG_OK;
}

extern "C" int lpg_create(const lpg_sim_desc* sims, int32_t n_sims, int32_t device, lpg_handle** out) {
  if (!out) return LPG_ERR_ARG;
  *out = nullptr;
  if (!sims || n_sims < 1 || n_sims > LPG_MAX_REPS) return LPG_ERR_ARG;
  lpg_handle* h = new lpg_handle();
  *out = h;
  h->device = device;
  for (int r = 0; r < n_sims; ++r) {
    const lpg_sim_desc& d = sims[r];
    {
      std::string msg;
      const int rc = validate_desc(d, r, &msg);
      if (rc) return fail(h, rc, "%s", msg.c_str());
    }
    SimHost s;
    s.d = d;
    const size_t n = (size_t)d.n_nodes;
    auto vec = [&](const double* p, size_t k, double dflt) {
      std::vector<double> v(k, dflt);
      if (p) std::copy(p, p + k, v.begin());
      return v;
    };
    s.birth_rate = vec(d.birth_rate, n, 0.0);
    s.p_ri = vec(d.vx_prob_ri, n, 0.0);
    s.p_ipv = vec(d.vx_prob_ipv, n, 0.0);
    s.strain_scal = vec(d.strain_r0_scalars, (size_t)d.n_strains, 1.0);
    s.net = vec(d.network, n * n, 0.0);
    s.r0s = vec(d.r0_scalars, n, 1.0);
    s.seas = vec(d.seasonality, (size_t)d.nt, 1.0);
    s.netq_t.assign(2 * n * n, 0);
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j) {
        uint64_t hi, lo;
        lpg_net_split(s.net[i * n + j], &hi, &lo);
        s.netq_t[2 * (j * n + i)] = hi;
        s.netq_t[2 * (j * n + i) + 1] = lo;
      }
    s.rowsum.assign(n, 0.0);
    for (size_t i = 0; i < n; ++i) {
      double acc = 0.0;
      for (size_t j = 0; j < n; ++j) acc = acc + s.net[i * n + j];
      s.rowsum[i] = acc;
    }
    s.p_sia.assign(n, 0.0f);
    if (d.vx_prob_sia) std::copy(d.vx_prob_sia, d.vx_prob_sia + n, s.p_sia.begin());
    s.km.assign(d.km_cumdeaths, d.km_cumdeaths + d.km_len);
    for (int k = 0; k < d.n_seeds; ++k) {
      lpg_seed_event e = d.seeds[k];
      s.seeds.push_back(e);
    }
    for (int k = 0; k < d.n_sia; ++k) {
      lpg_sia_event e = d.sia[k];
      if (e.tick < 0 || e.tick >= d.nt) continue;
      s.sia.push_back(e);
      s.sia_masks.emplace_back(e.node_mask, e.node_mask + n);
    }
    s.pop0.assign(d.pop0, d.pop0 + n);
    if (d.R_preseed) s.Rpre.assign(d.R_preseed, d.R_preseed + (size_t)d.nt * n);
    h->sims.push_back(std::move(s));
  }
  CK(cudaSetDevice(device));
  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  CK(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device));
  return LPG_OK;
}

static int alloc_staging(lpg_handle* h, Staging& s, int64_t cap) {
  /* one allocation carved into the fifteen columns, each at a 256-byte
   * boundary (one cudaMalloc and one cudaFree instead of fifteen) */
  const size_t n = (size_t)std::max<int64_t>(cap, 1);
  const size_t esz[15] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 4, 4, 4, 4};
  size_t off[15], total = 0;
  for (int k = 0; k < 15; ++k) {
    off[k] = total;
    total += (esz[k] * n + 255) & ~(size_t)255;
  }
  uint8_t* base = nullptr;
  if (dalloc(h, &base, total)) return LPG_ERR_NOMEM;
  s.base = base;
  s.ds = reinterpret_cast<int8_t*>(base + off[0]);
  s.strain = reinterpret_cast<int8_t*>(base + off[1]);
  s.et = reinterpret_cast<int8_t*>(base + off[2]);
  s.it = reinterpret_cast<int8_t*>(base + off[3]);
  s.pt = reinterpret_cast<int8_t*>(base + off[4]);
  s.pp = reinterpret_cast<int8_t*>(base + off[5]);
  s.par = reinterpret_cast<int8_t*>(base + off[6]);
  s.ipv = reinterpret_cast<int8_t*>(base + off[7]);
  s.cm = reinterpret_cast<uint8_t*>(base + off[8]);
  s.node = reinterpret_cast<int16_t*>(base + off[9]);
  s.ri = reinterpret_cast<int16_t*>(base + off[10]);
  s.risk = reinterpret_cast<float*>(base + off[11]);
  s.inf = reinterpret_cast<float*>(base + off[12]);
  s.dob = reinterpret_cast<int32_t*>(base + off[13]);
  s.dod = reinterpret_cast<int32_t*>(base + off[14]);
  return 0;
}

static void free_staging(lpg_handle* h, Staging& s) {
  dfree_one(h, s.base);
  s = Staging();
}

extern "C" int lpg_bind_columns(lpg_handle* h, int32_t sim, const lpg_columns* c) {
  if (!h || !c || sim < 0 || sim >= (int)h->sims.size()) return LPG_ERR_ARG;
  if (h->started) return fail(h, LPG_ERR_STATE, "columns must be bound before lpg_start");
  SimHost& s = h->sims[sim];
  const int64_t cap = s.d.capacity;
  CK(cudaSetDevice(h->device));
  if (!s.stg.bound) {
    int rc = alloc_staging(h, s.stg, cap);
    if (rc) return rc;
  }
  Staging& g = s.stg;
  cudaStream_t st = h->stream;
#define COPY_OR(dst, src, esz, memv)                                                   \
  if (src) {                                                                           \
    CK(cudaMemcpyAsync(dst, src, (size_t)cap * (esz), cudaMemcpyDefault, st));          \
  } else {                                                                             \
    CK(cudaMemsetAsync(dst, memv, (size_t)cap * (esz), st));                            \
  }
  COPY_OR(g.ds, c->disease_state, 1, 0xff);
  COPY_OR(g.strain, c->strain, 1, 0);
  COPY_OR(g.et, c->exposure_timer, 1, 0);
  COPY_OR(g.it, c->infection_timer, 1, 0);
  COPY_OR(g.pt, c->paralysis_timer, 1, 0);
  COPY_OR(g.pp, c->potentially_paralyzed, 1, 0xff);
  COPY_OR(g.par, c->paralyzed, 1, 0);
  COPY_OR(g.ipv, c->ipv_protected, 1, 0);
  COPY_OR(g.cm, c->chronically_missed, 1, 0);
  COPY_OR(g.node, c->node_id, 2, 0xff);
  COPY_OR(g.ri, c->ri_timer, 2, 0xff);
  COPY_OR(g.dob, c->date_of_birth, 4, 0xff);
  COPY_OR(g.dod, c->date_of_death, 4, 0);
#undef COPY_OR
  if (c->acq_risk_multiplier) {
    CK(cudaMemcpyAsync(g.risk, c->acq_risk_multiplier, (size_t)cap * 4, cudaMemcpyDefault, st));
  } else {
    k_fill_f32<<<256, 256, 0, st>>>(g.risk, cap, 1.0f);
  }
  if (c->daily_infectivity) {
    CK(cudaMemcpyAsync(g.inf, c->daily_infectivity, (size_t)cap * 4, cudaMemcpyDefault, st));
  } else {
    k_fill_f32<<<256, 256, 0, st>>>(g.inf, cap, 1.0f);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  g.bound = true;
  return LPG_OK;
}

static int launch_tick(lpg_handle* h, uint8_t need, int* n_launched);

extern "C" int lpg_start(lpg_handle* h) {
  if (!h) return LPG_ERR_ARG;
  if (h->started) return LPG_OK;
  CK(cudaSetDevice(h->device));
  cudaStream_t st = h->stream;
  const int R = (int)h->sims.size();
  for (int r = 0; r < R; ++r)
    if (!h->sims[r].stg.bound) return fail(h, LPG_ERR_STATE, "sim %d has no bound columns", r);

  /* 1. node counts, id range and sortedness per simulation */
  std::vector<std::vector<int64_t>> counts(R);
  std::vector<int> sorted(R, 1);
  unsigned long long* dcnt = nullptr;
  int* dflags = nullptr;
  int maxn = 0;
  for (auto& s : h->sims) maxn = std::max(maxn, s.d.n_nodes);
  if (dalloc(h, &dcnt, maxn) || dalloc(h, &dflags, 2)) return LPG_ERR_NOMEM;
  for (int r = 0; r < R; ++r) {
    SimHost& s = h->sims[r];
    CK(cudaMemsetAsync(dcnt, 0, sizeof(unsigned long long) * maxn, st));
    CK(cudaMemsetAsync(dflags, 0, sizeof(int) * 2, st));
    if (s.d.count > 0) k_hist<<<1024, 256, 0, st>>>(s.stg.node, s.d.count, s.d.n_nodes, dcnt, dflags);
    CK(cudaGetLastError());
    std::vector<unsigned long long> hc(s.d.n_nodes);
    int hf[2];
    CK(cudaMemcpyAsync(hc.data(), dcnt, sizeof(unsigned long long) * s.d.n_nodes, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hf, dflags, sizeof hf, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hf[0]) return fail(h, LPG_ERR_NODE, "sim %d: node_id outside [0, %d) among the first %lld slots", r, s.d.n_nodes,
                           (long long)s.d.count);
    sorted[r] = !hf[1];
    counts[r].assign(hc.begin(), hc.end());
  }
  dfree_one(h, dcnt);
  dfree_one(h, dflags);

  /* 2. chunk layout */
  std::vector<DevRep>& hr = h->hreps;
  hr.assign(R, DevRep{});
  int32_t chunk_total = 0, G = 0, csr_total = 0;
  std::vector<std::vector<int32_t>> node_chunk0(R), csr_start(R), chunk_fill_init(R);
  for (int r = 0; r < R; ++r) {
    SimHost& s = h->sims[r];
    const int n = s.d.n_nodes;
    DevRep& d = hr[r];
    d.node_base = G;
    d.chunk_base = chunk_total;
    d.csr_base = csr_total;
    node_chunk0[r].resize(n);
    csr_start[r].resize(n + 1);
    int32_t used = 0;
    for (int i = 0; i < n; ++i) {
      int64_t cnt = counts[r][i];
      int32_t k = (int32_t)std::max<int64_t>(1, (cnt + LPG_CHUNK - 1) / LPG_CHUNK);
      node_chunk0[r][i] = d.chunk_base + used;
      csr_start[r][i] = used;
      for (int32_t q = 0; q < k; ++q) {
        int64_t f = cnt - (int64_t)q * LPG_CHUNK;
        chunk_fill_init[r].push_back((int32_t)std::max<int64_t>(0, std::min<int64_t>(f, LPG_CHUNK)));
      }
      used += k;
    }
    csr_start[r][n] = used;
    int64_t reserve = (s.d.capacity - s.d.count + LPG_CHUNK - 1) / LPG_CHUNK + n;
    d.used_chunks = used;
    d.chunk_cap = (int32_t)(used + reserve);
    chunk_total += d.chunk_cap;
    G += n;
    csr_total += n + 1;
  }
  if ((int64_t)chunk_total * LPG_CHUNK >= (int64_t)0xFFFFFFF0LL)
    return fail(h, LPG_ERR_ARG, "device layout needs more than 2^32 positions");

  /* 3. allocations */
  DevWorld& W = h->W;
  W.n_reps = R;
  W.G = G;
  h->node_batch_tx = G > LPG_NODE_BATCH_MIN_PER_SM * h->sm_count;
  h->node_batch_mix = h->node_batch_tx && maxn <= LPG_NODE_BATCH_MAX_NODES;
  W.total_chunks = chunk_total;
  W.stall_after = h->test_stall_after;
  W.wait_spin = h->test_wait_spin > 0 ? h->test_wait_spin : LPG_MBAR_SPIN;
  W.test_bar_skip = h->test_bar_skip;
  const int64_t P = (int64_t)chunk_total * LPG_CHUNK;
  int rc = 0;
  rc |= dalloc(h, &W.ds, P);
  rc |= dalloc(h, &W.strain, P);
  rc |= dalloc(h, &W.et, P);
  rc |= dalloc(h, &W.it, P);
  rc |= dalloc(h, &W.pt, P);
  rc |= dalloc(h, &W.pp, P);
  rc |= dalloc(h, &W.par, P);
  rc |= dalloc(h, &W.ipv, P);
  rc |= dalloc(h, &W.cm, P);
  rc |= dalloc(h, &W.ri, P);
  rc |= dalloc(h, &W.risk, P);
  rc |= dalloc(h, &W.inf, P);
  rc |= dalloc(h, &W.dob, P);
  rc |= dalloc(h, &W.dod, P);
  rc |= dalloc(h, &W.evt, P);
  rc |= dalloc(h, &W.rdt, P);
  rc |= dalloc(h, &W.ref, P);
  rc |= dalloc(h, &W.cmeta, chunk_total);
  rc |= dalloc(h, &W.qcnt, 2048);
  rc |= dalloc(h, &W.qfirst, 2048);
  rc |= dalloc(h, &W.due, (size_t)chunk_total * LPG_NSUB);
  rc |= dalloc(h, &W.due_n, 1);
  rc |= dalloc(h, &W.evq, (size_t)chunk_total * LPG_CHUNK);
  rc |= dalloc(h, &W.chunk_w, chunk_total);
  rc |= dalloc(h, &W.sub_w, (size_t)chunk_total * LPG_NSUB);
  rc |= dalloc(h, &W.sub_dod, (size_t)chunk_total * LPG_NSUB);
  rc |= dalloc(h, &W.sub_evt, (size_t)chunk_total * LPG_NSUB);
  rc |= dalloc(h, &W.sub_rdt, (size_t)chunk_total * LPG_NSUB);
  rc |= dalloc(h, &W.cpref, chunk_total);
  rc |= dalloc(h, &W.node_chunks[0], chunk_total);
  rc |= dalloc(h, &W.node_chunks[1], chunk_total);
  rc |= dalloc(h, &W.node_chunk_start[0], csr_total);
  rc |= dalloc(h, &W.node_chunk_start[1], csr_total);
  rc |= dalloc(h, &W.node_rep, G);
  rc |= dalloc(h, &W.node_count, G);
  rc |= dalloc(h, &W.ev, (size_t)EV_N * G);
  rc |= dalloc(h, &W.tot, (size_t)TT_N * G);
  rc |= dalloc(h, &W.sw, G);
  rc |= dalloc(h, &W.bb, (size_t)LPG_MAX_STRAINS * G);
  rc |= dalloc(h, &W.nb_end, G);
  rc |= dalloc(h, &W.nb_li0, G);
  rc |= dalloc(h, &W.prob, (size_t)LPG_MAX_STRAINS * G);
  rc |= dalloc(h, &W.inck, (size_t)LPG_MAX_STRAINS * G);
  rc |= dalloc(h, &W.size, G);
  rc |= dalloc(h, &W.uniq, G);
  rc |= dalloc(h, &W.ksel, G);
  rc |= dalloc(h, &W.tgt_off, G + 1);
  {
    uint8_t* si = nullptr;
    rc |= dalloc(h, &si, (size_t)G * sizeof(SelInfo));
    W.sel_info = si;
  }
  /* selection targets (at most the susceptibles) and the E/I queue slabs
   * (at most one entry per position) share this buffer */
  int64_t hits = (int64_t)chunk_total * LPG_CHUNK;
  W.hits_cap = hits;
  rc |= dalloc(h, &W.hits, hits);
  rc |= dalloc(h, &W.ctr, LPG_NUM_COUNTERS);
  rc |= dalloc(h, &W.end_done, 1);
  rc |= dalloc(h, &W.grid_bar, 1);
  rc |= dalloc(h, &W.reps, R);
  if (rc) return LPG_ERR_NOMEM;
  CK(cudaMemsetAsync(W.ds, 0xff, P, st));
  CK(cudaMemsetAsync(W.ref, 0xff, P * 4, st));
  CK(cudaMemsetAsync(W.qcnt, 0, 4 * 2048, st));
  CK(cudaMemsetAsync(W.qfirst, 0, 4 * 2048, st));
  CK(cudaMemsetAsync(W.due_n, 0, 4, st));
  CK(cudaMemsetAsync(W.ev, 0, sizeof(int32_t) * EV_N * G, st));
  CK(cudaMemsetAsync(W.tot, 0, sizeof(int32_t) * TT_N * G, st));
  CK(cudaMemsetAsync(W.sw, 0, sizeof(uint64_t) * G, st));
  CK(cudaMemsetAsync(W.bb, 0, sizeof(uint64_t) * LPG_MAX_STRAINS * G, st));
  CK(cudaMemsetAsync(W.size, 0, sizeof(int64_t) * G, st));
  CK(cudaMemsetAsync(W.uniq, 0, sizeof(int64_t) * G, st));
  CK(cudaMemsetAsync(W.ctr, 0, sizeof(unsigned long long) * LPG_NUM_COUNTERS, st));
  CK(cudaMemsetAsync(W.end_done, 0, 4, st));
  CK(cudaMemsetAsync(W.grid_bar, 0, 8, st));

  /* 4. per-simulation static data, results, pools, chunk tables */
  std::vector<int4> h_meta(chunk_total, make_int4(-1, 0, -1, 0));
  std::vector<int32_t> h_node_rep(G), h_csr(chunk_total, 0),
      h_start(csr_total, 0);
  std::vector<int64_t> h_node_count(G);
  for (int r = 0; r < R; ++r) {
    SimHost& s = h->sims[r];
    const lpg_sim_desc& d = s.d;
    DevRep& rp = hr[r];
    const int n = d.n_nodes;
    rp.n_nodes = n;
    rp.ns = d.n_strains;
    rp.nt = d.nt;
    rp.comps = (int32_t)d.components;
    rp.stop_if = d.stop_if_no_cases;
    rp.vd_step = d.vd_step;
    rp.ri_step = d.ri_step;
    rp.ri_enabled = d.ri_enabled;
    rp.ri_strain = d.ri_strain;
    rp.km_len = d.km_len;
    rp.km_max_year = d.km_max_year;
    rp.nb_r = d.nb_r;
    if (d.nb_r >= 1) lpg_gamma_consts((double)d.nb_r, &rp.nb_d, &rp.nb_c);
    rp.count0 = d.count;
    rp.capacity = d.capacity;
    rp.seed = d.seed;
    rp.p_par = d.p_paralysis;
    rp.zi = d.zero_inflation;
    rp.dur_kind = d.dur_inf.kind;
    rp.dur_p1 = d.dur_inf.p1;
    rp.dur_p2 = d.dur_inf.p2;
    rp.t = 0;
    rp.stopped = 0;
    rp.stop_at = 0x7fffffff;
    rp.error = 0;
    rp.count = d.count;
    rp.csr_cur = 0;
    rp.started = 0;
    double* dp;
    float* fp;
    int64_t* ip;
    if (dupload(h, &dp, s.birth_rate)) return LPG_ERR_NOMEM;
    rp.birth_rate = dp;
    if (dupload(h, &dp, s.p_ri)) return LPG_ERR_NOMEM;
    rp.p_ri = dp;
    if (dupload(h, &dp, s.p_ipv)) return LPG_ERR_NOMEM;
    rp.p_ipv = dp;
    if (dupload(h, &dp, s.strain_scal)) return LPG_ERR_NOMEM;
    rp.strain_scal = dp;
    if (dupload(h, &dp, s.net)) return LPG_ERR_NOMEM;
    rp.net = dp;
    {
      uint64_t* qp;
      if (dupload(h, &qp, s.netq_t)) return LPG_ERR_NOMEM;
      rp.netq_t = qp;
    }
    if (dupload(h, &dp, s.rowsum)) return LPG_ERR_NOMEM;
    rp.rowsum = dp;
    if (dupload(h, &dp, s.r0s)) return LPG_ERR_NOMEM;
    rp.r0s = dp;
    if (dupload(h, &dp, s.seas)) return LPG_ERR_NOMEM;
    rp.seas = dp;
    if (dupload(h, &fp, s.p_sia)) return LPG_ERR_NOMEM;
    rp.p_sia = fp;
    {
      std::vector<uint64_t> tri(n), tipv(n);
      for (int i = 0; i < n; ++i) {
        tri[i] = u53_threshold(s.p_ri[i]);
        tipv[i] = u53_threshold(s.p_ipv[i]);
      }
      uint64_t* up;
      if (dupload(h, &up, tri)) return LPG_ERR_NOMEM;
      rp.thr_ri = up;
      if (dupload(h, &up, tipv)) return LPG_ERR_NOMEM;
      rp.thr_ipv = up;
      rp.thr_par = u53_threshold((double)d.p_paralysis);
    }
    if (dupload(h, &ip, s.km)) return LPG_ERR_NOMEM;
    rp.km = ip;
    /* per-tick SIA and seed tables, events in schedule order */
    std::vector<int32_t> sfirst(d.nt, 0), scnt(d.nt, 0), dfirst(d.nt, 0), dcnt_(d.nt, 0);
    std::vector<uint8_t> future(d.nt, 0);
    std::vector<DevSia> hsia;
    std::vector<uint8_t*> masks;
    for (int tt = 0; tt < d.nt; ++tt) {
      sfirst[tt] = (int32_t)hsia.size();
      for (size_t k = 0; k < s.sia.size(); ++k) {
        if (s.sia[k].tick != tt) continue;
        uint8_t* m;
        if (dupload(h, &m, s.sia_masks[k])) return LPG_ERR_NOMEM;
        std::vector<uint64_t> tv(n), tp(n);
        for (int i = 0; i < n; ++i) {
          const double pv = (double)s.p_sia[i];
          tv[i] = u53_threshold(pv);
          tp[i] = u53_threshold(pv * s.sia[k].efficacy);
        }
        uint64_t *dtv, *dtp;
        if (dupload(h, &dtv, tv) || dupload(h, &dtp, tp)) return LPG_ERR_NOMEM;
        DevSia e{s.sia[k].tick, s.sia[k].strain, s.sia[k].min_age, s.sia[k].max_age, s.sia[k].efficacy, m, dtv, dtp};
        hsia.push_back(e);
        scnt[tt] += 1;
      }
    }
    std::vector<DevSeed> hseed;
    for (int tt = 0; tt < d.nt; ++tt) {
      dfirst[tt] = (int32_t)hseed.size();
      for (size_t k = 0; k < s.seeds.size(); ++k) {
        if (s.seeds[k].tick != tt) continue;
        DevSeed e{s.seeds[k].tick, s.seeds[k].node, s.seeds[k].is_count, (int32_t)k, s.seeds[k].value};
        hseed.push_back(e);
        dcnt_[tt] += 1;
      }
    }
    for (int tt = 0; tt < d.nt; ++tt)
      for (auto& e : s.seeds)
        if (e.tick > tt) future[tt] = 1;
    /* the ticks that need the optional kernels (the conditions k_begin sets
     * vd_tick, ri_tick, sia_n and seed_n by) */
    if ((int)h->tick_need.size() < d.nt) h->tick_need.resize(d.nt, 0);
    for (int tt = 1; tt < d.nt; ++tt) {
      uint8_t m = 0;
      if ((d.components & LPG_COMP_VD) && tt % rp.vd_step == 0) m |= NEED_NB;
      if ((d.components & LPG_COMP_DS) && dcnt_[tt] > 0) m |= NEED_SEED;
      if ((d.components & LPG_COMP_RI) && rp.ri_enabled && tt % rp.ri_step == 0) m |= NEED_RS;
      if ((d.components & LPG_COMP_SIA) && scnt[tt] > 0) m |= NEED_RS;
      h->tick_need[tt] |= m;
    }
    int32_t* i32;
    uint8_t* u8;
    if (dupload(h, &i32, sfirst)) return LPG_ERR_NOMEM;
    rp.sia_first = i32;
    if (dupload(h, &i32, scnt)) return LPG_ERR_NOMEM;
    rp.sia_cnt = i32;
    if (dupload(h, &i32, dfirst)) return LPG_ERR_NOMEM;
    rp.seed_first = i32;
    if (dupload(h, &i32, dcnt_)) return LPG_ERR_NOMEM;
    rp.seed_cnt = i32;
    if (dupload(h, &u8, future)) return LPG_ERR_NOMEM;
    rp.future_seed = u8;
    DevSia* ds_;
    DevSeed* dd_;
    if (dupload(h, &ds_, hsia)) return LPG_ERR_NOMEM;
    rp.sia = ds_;
    if (dupload(h, &dd_, hseed)) return LPG_ERR_NOMEM;
    rp.seeds = dd_;
    /* results */
    int64_t off = 0;
    for (int k = 0; k < RS_N; ++k) {
      rp.res_off[k] = off;
      off += (int64_t)d.nt * n * (res_wide[k] ? d.n_strains : 1);
    }
    s.res_elems = off;
    if (dalloc(h, &rp.res, off)) return LPG_ERR_NOMEM;
    CK(cudaMemsetAsync(rp.res, 0, sizeof(int32_t) * off, st));
    CK(cudaMemcpyAsync(rp.res + rp.res_off[RS_POP], s.pop0.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    if (!s.Rpre.empty())
      CK(cudaMemcpyAsync(rp.res + rp.res_off[RS_R], s.Rpre.data(), sizeof(int32_t) * s.Rpre.size(), cudaMemcpyHostToDevice, st));
    if (s.record) {
      const size_t nrec = (size_t)d.nt * n * (3 + d.n_strains);
      if (dalloc(h, &rp.rec, nrec)) return LPG_ERR_NOMEM;
      CK(cudaMemsetAsync(rp.rec, 0, sizeof(double) * nrec, st));
    }
    /* unborn pool: reference slots [count, capacity) */
    const int64_t np = std::max<int64_t>(d.capacity - d.count, 1);
    rc = 0;
    rc |= dalloc(h, &rp.pl_et, np);
    rc |= dalloc(h, &rp.pl_it, np);
    rc |= dalloc(h, &rp.pl_pt, np);
    rc |= dalloc(h, &rp.pl_strain, np);
    rc |= dalloc(h, &rp.pl_pp, np);
    rc |= dalloc(h, &rp.pl_par, np);
    rc |= dalloc(h, &rp.pl_ipv, np);
    rc |= dalloc(h, &rp.pl_cm, np);
    rc |= dalloc(h, &rp.pl_ri, np);
    rc |= dalloc(h, &rp.pl_risk, np);
    rc |= dalloc(h, &rp.pl_inf, np);
    if (rc) return LPG_ERR_NOMEM;
    const int64_t pc = d.capacity - d.count;
    if (pc > 0) {
      Staging& g = s.stg;
      const int64_t c0 = d.count;
      CK(cudaMemcpyAsync(rp.pl_et, g.et + c0, pc, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(rp.pl_it, g.it + c0, pc, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(rp.pl_pt, g.pt + c0, pc, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(rp.pl_strain, g.strain + c0, pc, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(rp.pl_pp, g.pp + c0, pc, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(rp.pl_par, g.par + c0, pc, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(rp.pl_ipv, g.ipv + c0, pc, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(rp.pl_cm, g.cm + c0, pc, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(rp.pl_ri, g.ri + c0, pc * 2, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(rp.pl_risk, g.risk + c0, pc * 4, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(rp.pl_inf, g.inf + c0, pc * 4, cudaMemcpyDeviceToDevice, st));
    }
    /* chunk tables */
    int32_t c = 0;
    for (int i = 0; i < n; ++i) {
      h_node_rep[rp.node_base + i] = r;
      h_node_count[rp.node_base + i] = counts[r][i];
      h_start[rp.csr_base + i] = csr_start[r][i];
      for (int32_t k = csr_start[r][i]; k < csr_start[r][i + 1]; ++k, ++c) {
        h_meta[rp.chunk_base + c] = make_int4(rp.node_base + i, chunk_fill_init[r][c], -1, 0);
        h_csr[rp.chunk_base + k] = rp.chunk_base + c;
      }
    }
    h_start[rp.csr_base + n] = csr_start[r][n];
  }
  CK(cudaMemcpyAsync(W.node_rep, h_node_rep.data(), sizeof(int32_t) * G, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(W.node_count, h_node_count.data(), sizeof(int64_t) * G, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(W.cmeta, h_meta.data(), sizeof(int4) * chunk_total, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(W.node_chunks[0], h_csr.data(), sizeof(int32_t) * chunk_total, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(W.node_chunk_start[0], h_start.data(), sizeof(int32_t) * csr_total, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(W.reps, hr.data(), sizeof(DevRep) * R, cudaMemcpyHostToDevice, st));

  /* 5. scatter the reference-ordered columns into the node-major layout */
  for (int r = 0; r < R; ++r) {
    SimHost& s = h->sims[r];
    const int n = s.d.n_nodes;
    int32_t* d_nc0;
    int64_t* d_first;
    std::vector<int64_t> first(n, 0);
    for (int i = 1; i < n; ++i) first[i] = first[i - 1] + counts[r][i - 1];
    if (dupload(h, &d_nc0, node_chunk0[r])) return LPG_ERR_NOMEM;
    if (dupload(h, &d_first, first)) return LPG_ERR_NOMEM;
    int32_t* d_rank = nullptr;
    if (!sorted[r] && s.d.count > 0) {
      /* stable rank of each slot within its node, from the host copy */
      std::vector<int16_t> nodes(s.d.count);
      CK(cudaMemcpyAsync(nodes.data(), s.stg.node, sizeof(int16_t) * s.d.count, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      std::vector<int32_t> rank(s.d.count), next(n, 0);
      for (int64_t i = 0; i < s.d.count; ++i) rank[i] = next[nodes[i]]++;
      if (dupload(h, &d_rank, rank)) return LPG_ERR_NOMEM;
      CK(cudaStreamSynchronize(st));
    }
    ScatterArgs a{s.stg, s.d.count, d_nc0, d_first, d_rank};
    if (s.d.count > 0) {
      if (a.rank) k_scatter<<<2048, 256, 0, st>>>(W, a);
      else k_scatter_sorted<<<h->sm_count * 16, 256, 0, st>>>(W, a, hr[r].chunk_base, hr[r].used_chunks, hr[r].node_base);
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    dfree_one(h, d_nc0);
    dfree_one(h, d_first);
    dfree_one(h, d_rank);
    free_staging(h, s.stg);
  }

  /* 6. running totals and selection weights from a full count, then tick 0 */
  CK(cudaMemsetAsync(W.sub_dod, 0x7f, sizeof(int32_t) * (size_t)W.total_chunks * LPG_NSUB, st));
  k_count<<<std::max(1, h->sm_count * 4), LPG_SWEEP_THREADS, 0, st>>>(W, W.tot, W.sw, W.bb, W.chunk_w, W.sub_w,
                                                                      W.sub_dod);
  /* first events of the agents in E or I at tick 0 */
  CK(cudaMemsetAsync(W.sub_evt, 0x7f, sizeof(int32_t) * (size_t)W.total_chunks * LPG_NSUB, st));
  k_init_events<<<std::max(1, h->sm_count * 4), 256, 0, st>>>(W, W.evt, W.sub_evt, 0);
  /* RI due ticks of the initial population */
  CK(cudaMemsetAsync(W.sub_rdt, 0x7f, sizeof(int32_t) * (size_t)W.total_chunks * LPG_NSUB, st));
  k_ri_index<<<std::max(1, h->sm_count * 8), 256, 0, st>>>(W, W.sub_rdt, 1, nullptr);
  CK(cudaGetLastError());
  for (int r = 0; r < R; ++r) {
    hr[r].started = 1;
    hr[r].cur_t = 0;
    hr[r].active = 1;
    hr[r].vd_tick = hr[r].ri_tick = hr[r].sia_n = hr[r].seed_n = 0;
    hr[r].nb_total = 0;
  }
  CK(cudaMemcpyAsync(W.reps, hr.data(), sizeof(DevRep) * R, cudaMemcpyHostToDevice, st));
  k_end<<<(G + 255) / 256, 256, 0, st>>>(W);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));

  /* launch geometry */
  int occ = 0;
  CK(cudaFuncSetAttribute(k_sweep_rs, cudaFuncAttributeMaxDynamicSharedMemorySize, LPG_SWEEP_SMEM));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sweep_rs, LPG_SWEEP_BLOCK, LPG_SWEEP_SMEM));
  h->sweep_blocks = std::min(1024, std::max(1, occ) * h->sm_count);
  occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sweep_due, LPG_SWEEP_BLOCK, 0));
  h->sweep0_blocks = std::min(1024, std::max(1, occ) * h->sm_count);
  occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, R > 1 && R <= LPG_DUE_FLAT ? k_due<true> : k_due<false>, 256, 0));
  h->due_blocks = std::max(1, occ) * h->sm_count;
  occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sel_round0, 256, 0));
  if (occ < 1) return fail(h, LPG_ERR_CUDA, "k_sel_round0 does not fit on an SM");
  h->round0_max = occ * h->sm_count;
  h->select_blocks = h->round0_max;
  occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sel_rounds, 256, 0));
  h->rounds_blocks = std::min(1024, std::max(1, occ) * h->sm_count);
  h->evb_blocks = h->sm_count * 8;
  h->newborn_blocks = h->sm_count * 8;
  h->next_tick = 1; /* tick 0 ran above (k_end); the components run from tick 1 */
  h->started = true;
  return LPG_OK;
}

/* ------------------------------------------------------------------------ */
/* A tick kernel launched with programmatic stream serialization: its CTAs
 * may be scheduled before the previous kernel on the stream has finished;
 * it waits for that kernel's completion itself (pdl_begin). */
template <typename... Exp, typename... Act>
static cudaError_t launch_pdl(void (*k)(Exp...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Act&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Act>(args)...);
}

static int launch_one(lpg_handle* h, int k, bool timed) {
  cudaStream_t st = h->stream;
  DevWorld& W = h->W;
  const int R = W.n_reps, G = W.G;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (timed) {
    e0 = h->ev_pool[2 * k];
    e1 = h->ev_pool[2 * k + 1];
    CK(cudaEventRecord(e0, st));
  }
  switch (k) {
    case 0: CK(launch_pdl(k_begin, dim3(R), dim3(1024), 0, st, W)); break;
    case 1: CK(launch_pdl(k_newborns, dim3(h->newborn_blocks, R), dim3(256), 0, st, W)); break;
    case 2:
      if (R > 1 && R <= LPG_DUE_FLAT) CK(launch_pdl(k_due<true>, dim3(h->due_blocks), dim3(256), 0, st, W));
      else CK(launch_pdl(k_due<false>, dim3(h->due_blocks), dim3(256), 0, st, W));
      break;
    case 3: CK(launch_pdl(k_sweep_due, dim3(h->sweep0_blocks), dim3(LPG_SWEEP_BLOCK), 0, st, W)); break;
    case 4: CK(launch_pdl(k_seed, dim3(R), dim3(1024), 0, st, W)); break;
    case 5: CK(launch_pdl(k_sweep_rs, dim3(h->sweep_blocks), dim3(LPG_SWEEP_BLOCK), LPG_SWEEP_SMEM, st, W)); break;
    case 6: CK(launch_pdl(k_evb, dim3(h->evb_blocks), dim3(256), 0, st, W, h->sweep_blocks)); break;
    case 7:
      if (h->node_batch_mix) CK(launch_pdl(k_node_mix<1>, dim3(G), dim3(64), 0, st, W));
      else CK(launch_pdl(k_node_mix<LPG_NODE_MIX_WARPS>, dim3(G), dim3(LPG_NODE_MIX_THREADS), 0, st, W));
      break;
    case 8:
      if (h->node_batch_tx) CK(launch_pdl(k_node_tx_lanes, dim3((G + 127) / 128), dim3(128), 0, st, W));
      else CK(launch_pdl(k_node_tx, dim3(G), dim3(LPG_NODE_TX_THREADS), 0, st, W));
      break;
    case 9: {
      /* cooperative: its CTAs meet at a grid barrier, so all must be resident */
      void* args[] = {&W};
      CK(cudaLaunchCooperativeKernel((const void*)k_sel_round0, dim3(h->select_blocks), dim3(256), args, 0, st));
      break;
    }
    case 10: CK(launch_pdl(k_sel_rounds, dim3(h->rounds_blocks), dim3(256), 0, st, W)); break;
  }
  CK(cudaGetLastError());
  if (timed) CK(cudaEventRecord(e1, st));
  return 0;
}

static uint8_t need_of(const lpg_handle* h, int64_t t) {
  return (t >= 0 && t < (int64_t)h->tick_need.size()) ? h->tick_need[(size_t)t] : 0;
}

static int launch_tick(lpg_handle* h, uint8_t need, int* n_launched) {
  for (int k = 0; k < kNumTickKernels; ++k) {
    if (!kernel_needed(k, need)) continue;
    int rc = launch_one(h, k, false);
    if (rc) return rc;
    ++*n_launched;
  }
  return 0;
}

/* The graph of kTicksPerGraph ticks whose needs pack into key (3 bits a
 * tick), captured on first use; null if capture is not available. */
static int get_graph(lpg_handle* h, uint32_t key, cudaGraphExec_t* out, int* n_launched) {
  auto it = h->graphs.find(key);
  if (it != h->graphs.end()) {
    *out = it->second.first;
    *n_launched = it->second.second;
    return 0;
  }
  *out = nullptr;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int rc = 0, n = 0;
  for (int t = 0; t < kTicksPerGraph && !rc; ++t) rc = launch_tick(h, (uint8_t)((key >> (3 * t)) & 7u), &n);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (rc || e != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    h->graph_failed = true;
    return 0;
  }
  cudaGraphExec_t ge = nullptr;
  e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    h->graph_failed = true;
    return 0;
  }
  h->graphs[key] = {ge, n};
  *out = ge;
  *n_launched = n;
  return 0;
}

extern "C" int lpg_step(lpg_handle* h, int32_t n_ticks) {
  if (!h) return LPG_ERR_ARG;
  if (!h->started) return fail(h, LPG_ERR_STATE, "lpg_step before lpg_start");
  if (n_ticks <= 0) return LPG_OK;
  CK(cudaSetDevice(h->device));
  if (h->profiling) {
    if (h->ev_pool.empty()) {
      h->ev_pool.resize(2 * kNumTickKernels);
      for (auto& e : h->ev_pool) CK(cudaEventCreate(&e));
    }
    for (int t = 0; t < n_ticks; ++t) {
      const uint8_t need = need_of(h, h->next_tick);
      for (int k = 0; k < kNumTickKernels; ++k) {
        if (!kernel_needed(k, need)) continue;
        int rc = launch_one(h, k, true);
        if (rc) return rc;
      }
      CK(cudaStreamSynchronize(h->stream));
      for (int k = 0; k < kNumTickKernels; ++k) {
        if (!kernel_needed(k, need)) continue;
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, h->ev_pool[2 * k], h->ev_pool[2 * k + 1]));
        h->prof_ms[k] += ms;
        h->prof_n[k] += 1;
        h->launches += 1;
      }
      h->next_tick += 1;
    }
    return LPG_OK;
  }
  int left = n_ticks;
  while (h->use_graphs && !h->graph_failed && left >= kTicksPerGraph) {
    uint32_t key = 0;
    for (int t = 0; t < kTicksPerGraph; ++t) key |= (uint32_t)need_of(h, (int64_t)h->next_tick + t) << (3 * t);
    cudaGraphExec_t ge = nullptr;
    int n = 0;
    int rc = get_graph(h, key, &ge, &n);
    if (rc) return rc;
    if (!ge) break;
    CK(cudaGraphLaunch(ge, h->stream));
    h->launches += n;
    h->next_tick += kTicksPerGraph;
    left -= kTicksPerGraph;
  }
  for (; left > 0; --left) {
    int n = 0;
    int rc = launch_tick(h, need_of(h, h->next_tick), &n);
    if (rc) return rc;
    h->launches += n;
    h->next_tick += 1;
  }
  return LPG_OK;
}

extern "C" int lpg_sync(lpg_handle* h) {
  if (!h) return LPG_ERR_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  if (!h->started) return LPG_OK;
  std::vector<DevRep> reps(h->W.n_reps);
  CK(cudaMemcpy(reps.data(), h->W.reps, sizeof(DevRep) * reps.size(), cudaMemcpyDeviceToHost));
  for (size_t r = 0; r < reps.size(); ++r) {
    if (reps[r].error == LPG_ERR_CAPACITY)
      return fail(h, LPG_ERR_CAPACITY, "sim %zu: births at tick %d exceed capacity %lld", r, reps[r].cur_t,
                  (long long)reps[r].capacity);
    if (reps[r].error) return fail(h, reps[r].error, "sim %zu: device error %d at tick %d", r, reps[r].error, reps[r].cur_t);
  }
  return LPG_OK;
}

extern "C" int lpg_get_state(lpg_handle* h, int32_t sim, lpg_sim_state* out) {
  if (!h || !out || sim < 0 || sim >= (int)h->sims.size()) return LPG_ERR_ARG;
  if (!h->started) {
    out->t = 0;
    out->stopped = 0;
    out->count = h->sims[sim].d.count;
    out->error = 0;
    return LPG_OK;
  }
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  DevRep r;
  CK(cudaMemcpy(&r, h->W.reps + sim, sizeof(DevRep), cudaMemcpyDeviceToHost));
  out->t = r.t;
  out->stopped = r.stopped;
  out->count = r.count;
  out->error = r.error;
  return LPG_OK;
}

extern "C" int lpg_read_results(lpg_handle* h, int32_t sim, const lpg_results_view* v) {
  if (!h || !v || sim < 0 || sim >= (int)h->sims.size()) return LPG_ERR_ARG;
  if (!h->started) return fail(h, LPG_ERR_STATE, "no results before lpg_start");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  DevRep r;
  CK(cudaMemcpy(&r, h->W.reps + sim, sizeof(DevRep), cudaMemcpyDeviceToHost));
  int32_t* const* outs = (int32_t* const*)v;
  const lpg_sim_desc& d = h->sims[sim].d;
  for (int k = 0; k < RS_N; ++k) {
    if (!outs[k]) continue;
    size_t n = (size_t)d.nt * d.n_nodes * (res_wide[k] ? d.n_strains : 1);
    CK(cudaMemcpy(outs[k], r.res + r.res_off[k], n * sizeof(int32_t), cudaMemcpyDefault));
  }
  return LPG_OK;
}

extern "C" int lpg_record_aggregates(lpg_handle* h, int32_t sim, int32_t enable) {
  if (!h || sim < 0 || sim >= (int)h->sims.size()) return LPG_ERR_ARG;
  if (h->started) return fail(h, LPG_ERR_STATE, "lpg_record_aggregates after lpg_start");
  h->sims[sim].record = enable != 0;
  return LPG_OK;
}

extern "C" int lpg_read_aggregates(lpg_handle* h, int32_t sim, double* srisk, double* beta, double* pop,
                                   double* lam) {
  if (!h || sim < 0 || sim >= (int)h->sims.size()) return LPG_ERR_ARG;
  if (!h->started) return fail(h, LPG_ERR_STATE, "no aggregates before lpg_start");
  if (!h->sims[sim].record) return fail(h, LPG_ERR_STATE, "simulation %d does not record aggregates", sim);
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  DevRep r;
  CK(cudaMemcpy(&r, h->W.reps + sim, sizeof(DevRep), cudaMemcpyDeviceToHost));
  const lpg_sim_desc& d = h->sims[sim].d;
  const int w = 3 + d.n_strains;
  const size_t rows = (size_t)d.nt * d.n_nodes;
  std::vector<double> buf(rows * w);
  CK(cudaMemcpy(buf.data(), r.rec, sizeof(double) * buf.size(), cudaMemcpyDeviceToHost));
  for (size_t q = 0; q < rows; ++q) {
    const double* b = buf.data() + q * w;
    if (srisk) srisk[q] = b[0];
    if (pop) pop[q] = b[1];
    if (lam) lam[q] = b[2];
    if (beta)
      for (int s = 0; s < d.n_strains; ++s) beta[q * d.n_strains + s] = b[3 + s];
  }
  return LPG_OK;
}

extern "C" int lpg_read_columns(lpg_handle* h, int32_t sim, const lpg_columns* c) {
  if (!h || !c || sim < 0 || sim >= (int)h->sims.size()) return LPG_ERR_ARG;
  if (!h->started) return fail(h, LPG_ERR_STATE, "no columns before lpg_start");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  DevRep r;
  CK(cudaMemcpy(&r, h->W.reps + sim, sizeof(DevRep), cudaMemcpyDeviceToHost));
  Staging s;
  int rc = alloc_staging(h, s, std::max<int64_t>(r.count, 1));
  if (rc) return rc;
  k_gather<<<2048, 256, 0, h->stream>>>(h->W, s, r.chunk_base, r.used_chunks, r.node_base, r.t - 1,
                                        (r.comps & LPG_COMP_DS) ? 1 : 0, sim);
  CK(cudaGetLastError());
  const size_t n = (size_t)r.count;
#define OUT(dst, src, esz) \
  if (dst) CK(cudaMemcpyAsync(dst, src, n * (esz), cudaMemcpyDefault, h->stream))
  OUT(c->disease_state, s.ds, 1);
  OUT(c->strain, s.strain, 1);
  OUT(c->exposure_timer, s.et, 1);
  OUT(c->infection_timer, s.it, 1);
  OUT(c->paralysis_timer, s.pt, 1);
  OUT(c->potentially_paralyzed, s.pp, 1);
  OUT(c->paralyzed, s.par, 1);
  OUT(c->ipv_protected, s.ipv, 1);
  OUT(c->chronically_missed, s.cm, 1);
  OUT(c->node_id, s.node, 2);
  OUT(c->ri_timer, s.ri, 2);
  OUT(c->acq_risk_multiplier, s.risk, 4);
  OUT(c->daily_infectivity, s.inf, 4);
  OUT(c->date_of_birth, s.dob, 4);
  OUT(c->date_of_death, s.dod, 4);
#undef OUT
  CK(cudaStreamSynchronize(h->stream));
  free_staging(h, s);
  return LPG_OK;
}

/* Recount everything and compare with the running totals (diagnostic). */
extern "C" int lpg_check_invariants(lpg_handle* h) {
  if (!h || !h->started) return LPG_ERR_STATE;
  CK(cudaSetDevice(h->device));
  DevWorld& W = h->W;
  const int G = W.G;
  int32_t *tot, *subd, *sube, *subr;
  uint64_t *sw, *bb, *cw, *subw;
  int* bad;
  if (dalloc(h, &tot, (size_t)TT_N * G) || dalloc(h, &sw, G) || dalloc(h, &bb, (size_t)LPG_MAX_STRAINS * G) ||
      dalloc(h, &cw, W.total_chunks) || dalloc(h, &subw, (size_t)W.total_chunks * LPG_NSUB) ||
      dalloc(h, &subd, (size_t)W.total_chunks * LPG_NSUB) || dalloc(h, &sube, (size_t)W.total_chunks * LPG_NSUB) ||
      dalloc(h, &subr, (size_t)W.total_chunks * LPG_NSUB) || dalloc(h, &bad, 1))
    return LPG_ERR_NOMEM;
  cudaStream_t st = h->stream;
  CK(cudaMemsetAsync(tot, 0, sizeof(int32_t) * TT_N * G, st));
  CK(cudaMemsetAsync(sw, 0, sizeof(uint64_t) * G, st));
  CK(cudaMemsetAsync(bb, 0, sizeof(uint64_t) * LPG_MAX_STRAINS * G, st));
  CK(cudaMemsetAsync(cw, 0, sizeof(uint64_t) * W.total_chunks, st));
  CK(cudaMemsetAsync(subw, 0, sizeof(uint64_t) * W.total_chunks * LPG_NSUB, st));
  CK(cudaMemsetAsync(bad, 0, 4, st));
  CK(cudaMemsetAsync(subd, 0x7f, sizeof(int32_t) * (size_t)W.total_chunks * LPG_NSUB, st));
  k_count<<<std::max(1, h->sm_count * 4), LPG_SWEEP_THREADS, 0, st>>>(W, tot, sw, bb, cw, subw, subd);
  CK(cudaMemsetAsync(sube, 0x7f, sizeof(int32_t) * (size_t)W.total_chunks * LPG_NSUB, st));
  k_count_events<<<std::max(1, h->sm_count * 4), 256, 0, st>>>(W, sube);
  CK(cudaMemsetAsync(subr, 0x7f, sizeof(int32_t) * (size_t)W.total_chunks * LPG_NSUB, st));
  k_ri_index<<<std::max(1, h->sm_count * 8), 256, 0, st>>>(W, subr, 0, bad);
  k_cmp_counts<<<std::max(1, h->sm_count * 4), 256, 0, st>>>(W, tot, sw, bb, cw, subw, subd, sube, subr, bad);
  CK(cudaGetLastError());
  int hb = 0;
  CK(cudaMemcpyAsync(&hb, bad, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  void* ps[] = {tot, sw, bb, cw, subw, subd, sube, subr, bad};
  for (void* p : ps) dfree_one(h, p);
  if (hb) return fail(h, LPG_ERR_INTERNAL, "running totals differ from a recount (mask 0x%x)", hb);
  return LPG_OK;
}

static int* launch_slot(lpg_handle* h, int32_t which, int* limit) {
  switch (which) {
    case LPG_LAUNCH_DUE: *limit = 8192; return &h->due_blocks;
    case LPG_LAUNCH_SWEEP_DUE: *limit = 1024; return &h->sweep0_blocks;
    case LPG_LAUNCH_SWEEP_RS: *limit = 1024; return &h->sweep_blocks;
    case LPG_LAUNCH_EVB: *limit = 8192; return &h->evb_blocks;
    case LPG_LAUNCH_SELECT: *limit = h->round0_max; return &h->select_blocks;
    case LPG_LAUNCH_ROUNDS: *limit = 1024; return &h->rounds_blocks;
    case LPG_LAUNCH_NEWBORNS: *limit = 8192; return &h->newborn_blocks;
    default: return nullptr;
  }
}

extern "C" int lpg_set_launch(lpg_handle* h, int32_t which, int32_t blocks) {
  if (!h) return LPG_ERR_ARG;
  if (!h->started) return fail(h, LPG_ERR_STATE, "lpg_set_launch before lpg_start");
  int limit = 0;
  int* slot = launch_slot(h, which, &limit);
  if (!slot) return fail(h, LPG_ERR_ARG, "no tick kernel %d", which);
  if (blocks < 1 || blocks > limit) return fail(h, LPG_ERR_ARG, "grid of %d CTAs outside [1, %d]", blocks, limit);
  if (*slot != blocks) {
    *slot = blocks;
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second.first);
    h->graphs.clear();
    /* the grid barrier's count is kept a multiple of the grid size */
    if (which == LPG_LAUNCH_SELECT) {
      CK(cudaSetDevice(h->device));
      CK(cudaMemsetAsync(h->W.grid_bar, 0, sizeof(unsigned long long), h->stream));
    }
  }
  return LPG_OK;
}

extern "C" int lpg_get_launch(lpg_handle* h, int32_t which) {
  if (!h) return LPG_ERR_ARG;
  if (!h->started) return fail(h, LPG_ERR_STATE, "lpg_get_launch before lpg_start");
  int limit = 0;
  int* slot = launch_slot(h, which, &limit);
  if (!slot) return fail(h, LPG_ERR_ARG, "no tick kernel %d", which);
  return *slot;
}

extern "C" int lpg_test_stall_sweep(lpg_handle* h, int32_t stages, int64_t wait_spin) {
  if (!h) return LPG_ERR_ARG;
  if (wait_spin < 0 || wait_spin > LPG_MBAR_SPIN) return fail(h, LPG_ERR_ARG, "wait_spin %lld out of range", (long long)wait_spin);
  h->test_stall_after = stages < 0 ? -1 : stages;
  h->test_wait_spin = wait_spin;
  h->W.stall_after = h->test_stall_after;
  h->W.wait_spin = wait_spin > 0 ? wait_spin : LPG_MBAR_SPIN;
  /* graphs hold the kernels' arguments as captured: capture again */
  for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second.first);
  h->graphs.clear();
  return LPG_OK;
}

extern "C" int lpg_test_stall_round0(lpg_handle* h, int32_t skip, int64_t wait_spin) {
  if (!h) return LPG_ERR_ARG;
  if (wait_spin < 0 || wait_spin > LPG_MBAR_SPIN) return fail(h, LPG_ERR_ARG, "wait_spin %lld out of range", (long long)wait_spin);
  h->test_bar_skip = skip != 0;
  h->test_wait_spin = wait_spin;
  h->W.test_bar_skip = h->test_bar_skip;
  h->W.wait_spin = wait_spin > 0 ? wait_spin : LPG_MBAR_SPIN;
  for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second.first);
  h->graphs.clear();
  return LPG_OK;
}

extern "C" int lpg_set_graphs(lpg_handle* h, int32_t enable) {
  if (!h) return LPG_ERR_ARG;
  h->use_graphs = enable != 0;
  return LPG_OK;
}

extern "C" int lpg_set_profiling(lpg_handle* h, int32_t enable) {
  if (!h) return LPG_ERR_ARG;
  h->profiling = enable != 0;
  if (h->profiling) {
    for (int k = 0; k < kNumTickKernels; ++k) {
      h->prof_ms[k] = 0;
      h->prof_n[k] = 0;
    }
    if (h->W.ctr) CK(cudaMemsetAsync(h->W.ctr, 0, sizeof(unsigned long long) * LPG_NUM_COUNTERS, h->stream));
  }
  return LPG_OK;
}

extern "C" int lpg_read_counters(lpg_handle* h, uint64_t* out, int32_t n) {
  if (!h || !out || n < 0) return LPG_ERR_ARG;
  if (!h->W.ctr) return LPG_ERR_STATE;
  unsigned long long c[LPG_NUM_COUNTERS];
  CK(cudaMemcpyAsync(c, h->W.ctr, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < n && k < LPG_NUM_COUNTERS; ++k) out[k] = (uint64_t)c[k];
  return LPG_OK;
}

extern "C" int lpg_read_profile(lpg_handle* h, lpg_profile* out) {
  if (!h || !out) return LPG_ERR_ARG;
  out->n_kernels = kNumTickKernels;
  for (int k = 0; k < kNumTickKernels; ++k) {
    out->names[k] = kKernelNames[k];
    out->total_ms[k] = h->prof_ms[k];
    out->launches[k] = h->prof_n[k];
  }
  return LPG_OK;
}

extern "C" void lpg_destroy(lpg_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second.first);
  for (auto e : h->ev_pool) cudaEventDestroy(e);
  for (void* p : h->allocs) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}
