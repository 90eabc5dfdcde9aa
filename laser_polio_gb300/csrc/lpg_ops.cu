/*
 * lpg_ops.cu — standalone per-node state counts over plain device columns.
 *
 * lpg_count_seirp restates count_SEIRP (laser_polio/model.py:869-899) and
 * its kernel (:902-929): for every slot with disease_state >= 0, count it
 * into S / E_by_strain / I_by_strain / R of its node by state, and into
 * potentially_paralyzed / paralyzed when those flags equal 1; E and I are
 * the per-node sums over strains.  The reference reduces numba thread-local
 * tables; here every CTA builds a node x field histogram in shared memory
 * from run-length counters (slots of a node are mostly contiguous), writes
 * the whole histogram to a scratch slice, and one reduce kernel sums the
 * slices in a fixed order.  Integer counts, so the result is exact and does
 * not depend on the grid.  No global atomics, and the outputs are written
 * (not accumulated): the caller need not clear them.
 *
 * Two entry points share these kernels:
 *   lpg_count_seirp         scratch from cudaMallocAsync on the caller's stream;
 *   lpg_count_seirp_static  scratch in a file-scope __device__ array, for
 *                           callers that cannot allocate device memory.
 */
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <mutex>

#include "lpg.h"

#define SEIRP_THREADS 256
#define SEIRP_APT 16 /* slots per thread in the vector path */
#define SEIRP_FIELDS_MAX (4 + 2 * LPG_MAX_STRAINS)
#define SEIRP_MAX_DEVICES 64

/* Field layout of one histogram slice: [field][node], then one word holding
 * the number of invalid slots.  Fields: 0 S, 1 R, 2 potentially_paralyzed,
 * 3 paralyzed, 4.. E by strain, 4+ns.. I by strain. */
struct SeirpIn {
  const int16_t* node;
  const int8_t* ds;
  const int8_t* strain;
  const int8_t* pp;
  const int8_t* par;
  int64_t n;
  int32_t G, ns, F, pad;
};

struct SeirpOut {
  int32_t *S, *E, *I, *R, *Ebs, *Ibs, *POTP, *P;
  int64_t* n_invalid;
};

static thread_local char g_err[256] = "";

static int op_fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

/* The same error text for the ops of other translation units (lpg_adjoint.cu). */
int lpg_ops_fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

extern "C" const char* lpg_op_last_error(void) { return g_err; }

/* ------------------------------------------------------------------------ */
/* Run-length counters of one thread: c[0..3] S R POTP P, c[4+k] E of strain
 * k, c[8+k] I of strain k, all for node `cur`. */
__device__ __forceinline__ void seirp_flush(int32_t* h, const SeirpIn& a, int cur, int32_t (&c)[SEIRP_FIELDS_MAX]) {
  if (cur < 0) return;
#pragma unroll
  for (int f = 0; f < 4; ++f)
    if (c[f]) {
      atomicAdd(&h[f * a.G + cur], c[f]);
      c[f] = 0;
    }
#pragma unroll
  for (int k = 0; k < LPG_MAX_STRAINS; ++k) {
    if (c[4 + k]) {
      atomicAdd(&h[(4 + k) * a.G + cur], c[4 + k]);
      c[4 + k] = 0;
    }
    if (c[8 + k]) {
      atomicAdd(&h[(4 + a.ns + k) * a.G + cur], c[8 + k]);
      c[8 + k] = 0;
    }
  }
}

/* count_SEIRP_kernel's body for one slot (model.py:913-929).  Slots whose
 * node id lies outside [0, G), or which are E/I with a strain outside
 * [0, ns), are counted as invalid instead (the reference indexes out of
 * bounds there). */
__device__ __forceinline__ void seirp_slot(int32_t* h, const SeirpIn& a, int8_t s, int nd, int8_t st, int8_t pp,
                                           int8_t pa, int& cur, int32_t (&c)[SEIRP_FIELDS_MAX], int32_t& bad) {
  if (s < 0) return;
  if ((unsigned)nd >= (unsigned)a.G) {
    ++bad;
    return;
  }
  if (nd != cur) {
    seirp_flush(h, a, cur, c);
    cur = nd;
  }
  if (s == 0) {
    ++c[0];
  } else if (s == 1 || s == 2) {
    if ((unsigned)st < (unsigned)a.ns) {
      const int base = s == 1 ? 4 : 8;
#pragma unroll
      for (int k = 0; k < LPG_MAX_STRAINS; ++k) c[base + k] += (st == k);
    } else {
      ++bad;
    }
  } else if (s == 3) {
    ++c[1];
  }
  if (pp == 1) ++c[2];
  if (pa == 1) ++c[3];
}

__device__ __forceinline__ int8_t byte_of(const int4& v, int j) {
  const uint32_t w = j < 4 ? (uint32_t)v.x : j < 8 ? (uint32_t)v.y : j < 12 ? (uint32_t)v.z : (uint32_t)v.w;
  return (int8_t)(uint8_t)(w >> (8 * (j & 3)));
}

__device__ __forceinline__ int16_t half_of(const int4& v, int j) {
  const uint32_t w = j < 2 ? (uint32_t)v.x : j < 4 ? (uint32_t)v.y : j < 6 ? (uint32_t)v.z : (uint32_t)v.w;
  return (int16_t)(uint16_t)(w >> (16 * (j & 1)));
}

/* One CTA: histogram of its slots in shared memory, then the whole slice to
 * part[blockIdx.x].  VEC: 16 consecutive slots per thread with 16-byte loads
 * (every column 16-byte aligned); the tail past the last full group, and the
 * whole range when VEC is false, go slot by slot. */
template <bool VEC>
__global__ void __launch_bounds__(SEIRP_THREADS) k_seirp_partial(SeirpIn a, int32_t* part) {
  extern __shared__ int32_t h[];
  const int64_t slice = (int64_t)a.F * a.G + 1;
  for (int64_t i = threadIdx.x; i < slice; i += blockDim.x) h[i] = 0;
  __syncthreads();
  int32_t c[SEIRP_FIELDS_MAX];
#pragma unroll
  for (int f = 0; f < SEIRP_FIELDS_MAX; ++f) c[f] = 0;
  int cur = -1;
  int32_t bad = 0;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t tail0 = 0;
  if (VEC) {
    const int64_t groups = a.n / SEIRP_APT;
    tail0 = groups * SEIRP_APT;
    for (int64_t g = gtid; g < groups; g += stride) {
      const int64_t i0 = g * SEIRP_APT;
      const int4 vds = __ldg(reinterpret_cast<const int4*>(a.ds + i0));
      const int4 vst = __ldg(reinterpret_cast<const int4*>(a.strain + i0));
      const int4 vpp = __ldg(reinterpret_cast<const int4*>(a.pp + i0));
      const int4 vpa = __ldg(reinterpret_cast<const int4*>(a.par + i0));
      const int4 vn0 = __ldg(reinterpret_cast<const int4*>(a.node + i0));
      const int4 vn1 = __ldg(reinterpret_cast<const int4*>(a.node + i0 + 8));
#pragma unroll
      for (int j = 0; j < SEIRP_APT; ++j) {
        const int nd = j < 8 ? half_of(vn0, j) : half_of(vn1, j - 8);
        seirp_slot(h, a, byte_of(vds, j), nd, byte_of(vst, j), byte_of(vpp, j), byte_of(vpa, j), cur, c, bad);
      }
    }
  }
  for (int64_t i = tail0 + gtid; i < a.n; i += stride)
    seirp_slot(h, a, a.ds[i], a.node[i], a.strain[i], a.pp[i], a.par[i], cur, c, bad);
  seirp_flush(h, a, cur, c);
  if (bad) atomicAdd(&h[slice - 1], bad);
  __syncthreads();
  int32_t* out = part + (int64_t)blockIdx.x * slice;
  for (int64_t i = threadIdx.x; i < slice; i += blockDim.x) out[i] = h[i];
}

/* Sum the nblk slices in block order; one CTA per 32 nodes, 8 warps split
 * the slices.  Writes every output element of its nodes. */
__global__ void __launch_bounds__(SEIRP_THREADS) k_seirp_reduce(SeirpIn a, SeirpOut o, const int32_t* part,
                                                                int32_t nblk) {
  __shared__ int64_t red[SEIRP_THREADS / 32][32];
  __shared__ int32_t vals[SEIRP_FIELDS_MAX][32];
  const int lane = threadIdx.x & 31, y = threadIdx.x >> 5, ny = SEIRP_THREADS / 32;
  const int nd = blockIdx.x * 32 + lane;
  const int64_t slice = (int64_t)a.F * a.G + 1;
  for (int f = 0; f < a.F; ++f) {
    int64_t s = 0;
    if (nd < a.G)
      for (int b = y; b < nblk; b += ny) s += part[(int64_t)b * slice + (int64_t)f * a.G + nd];
    red[y][lane] = s;
    __syncthreads();
    if (y == 0) {
      int64_t t = 0;
      for (int k = 0; k < ny; ++k) t += red[k][lane];
      vals[f][lane] = (int32_t)t;
    }
    __syncthreads();
  }
  if (y == 0 && nd < a.G) {
    o.S[nd] = vals[0][lane];
    o.R[nd] = vals[1][lane];
    o.POTP[nd] = vals[2][lane];
    o.P[nd] = vals[3][lane];
    int32_t e = 0, i = 0;
    for (int k = 0; k < a.ns; ++k) {
      o.Ebs[(int64_t)nd * a.ns + k] = vals[4 + k][lane];
      o.Ibs[(int64_t)nd * a.ns + k] = vals[4 + a.ns + k][lane];
      e += vals[4 + k][lane];
      i += vals[4 + a.ns + k][lane];
    }
    o.E[nd] = e;
    o.I[nd] = i;
  }
  if (blockIdx.x == 0 && o.n_invalid) {
    int64_t s = 0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += part[(int64_t)b * slice + slice - 1];
    red[y][lane] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      int64_t t = 0;
      for (int k = 0; k < ny; ++k)
        for (int l = 0; l < 32; ++l) t += red[k][l];
      *o.n_invalid = t;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Per-device setup shared by both entry points: SM count, and the dynamic
 * shared memory opt-in of the partial kernels (up to SEIRP_FIELDS_MAX x
 * LPG_COUNT_SEIRP_MAX_NODES + 1 words). */
struct SeirpDev {
  bool ready;
  int sms;
  bool static_ready;
  int32_t* static_scratch; /* device address of g_seirp_scratch on this device */
};
static SeirpDev g_dev[SEIRP_MAX_DEVICES];
static std::mutex g_dev_mu;

static const size_t kSmemMax = ((size_t)SEIRP_FIELDS_MAX * LPG_COUNT_SEIRP_MAX_NODES + 1) * sizeof(int32_t);

static int seirp_dev_setup(int dev) {
  std::lock_guard<std::mutex> lk(g_dev_mu);
  SeirpDev& d = g_dev[dev];
  if (d.ready) return LPG_OK;
  cudaError_t e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_seirp_partial<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_seirp_partial<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax);
  if (e != cudaSuccess) return op_fail(LPG_ERR_CUDA, "count_SEIRP setup: %s", cudaGetErrorString(e));
  d.ready = true;
  return LPG_OK;
}

struct SeirpLaunch {
  SeirpIn in;
  SeirpOut out;
  bool vec;
  size_t smem;
  int nblk;
  cudaStream_t st;
  int dev;
};

/* Argument checks shared by both entry points; fills the launch record with
 * the grid the allocating entry point uses. */
static int seirp_prepare(SeirpLaunch& L, const int16_t* node_id, const int8_t* disease_state, const int8_t* strain,
                         const int8_t* potentially_paralyzed, const int8_t* paralyzed, int32_t n_nodes,
                         int32_t n_strains, int64_t n_people, int32_t* S, int32_t* E, int32_t* I, int32_t* R,
                         int32_t* E_by_strain, int32_t* I_by_strain, int32_t* POTP, int32_t* P, int64_t* n_invalid,
                         void* stream) {
  if (n_nodes < 1 || n_nodes > LPG_COUNT_SEIRP_MAX_NODES)
    return op_fail(LPG_ERR_ARG, "count_SEIRP: n_nodes %d outside [1, %d]", n_nodes, LPG_COUNT_SEIRP_MAX_NODES);
  if (n_strains < 1 || n_strains > LPG_MAX_STRAINS)
    return op_fail(LPG_ERR_ARG, "count_SEIRP: n_strains %d outside [1, %d]", n_strains, LPG_MAX_STRAINS);
  if (n_people < 0) return op_fail(LPG_ERR_ARG, "count_SEIRP: n_people %lld < 0", (long long)n_people);
  if (n_people > 0 && (!node_id || !disease_state || !strain || !potentially_paralyzed || !paralyzed))
    return op_fail(LPG_ERR_ARG, "count_SEIRP: a column pointer is NULL");
  if (!S || !E || !I || !R || !E_by_strain || !I_by_strain || !POTP || !P)
    return op_fail(LPG_ERR_ARG, "count_SEIRP: an output pointer is NULL");
  cudaError_t e = cudaGetDevice(&L.dev);
  if (e != cudaSuccess) return op_fail(LPG_ERR_CUDA, "count_SEIRP: %s", cudaGetErrorString(e));
  if (L.dev < 0 || L.dev >= SEIRP_MAX_DEVICES) return op_fail(LPG_ERR_ARG, "count_SEIRP: device %d", L.dev);
  int rc = seirp_dev_setup(L.dev);
  if (rc) return rc;
  L.in = SeirpIn{node_id, disease_state, strain, potentially_paralyzed, paralyzed, n_people,
                 n_nodes, n_strains, 4 + 2 * n_strains, 0};
  L.out = SeirpOut{S, E, I, R, E_by_strain, I_by_strain, POTP, P, n_invalid};
  auto al16 = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
  L.vec = al16(node_id) && al16(disease_state) && al16(strain) && al16(potentially_paralyzed) && al16(paralyzed);
  L.smem = ((size_t)L.in.F * n_nodes + 1) * sizeof(int32_t);
  int per_sm = 0;
  e = L.vec ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_seirp_partial<true>, SEIRP_THREADS, L.smem)
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_seirp_partial<false>, SEIRP_THREADS, L.smem);
  if (e != cudaSuccess) return op_fail(LPG_ERR_CUDA, "count_SEIRP occupancy: %s", cudaGetErrorString(e));
  const int64_t per_block = (int64_t)SEIRP_THREADS * SEIRP_APT;
  const int64_t want = std::max<int64_t>(1, (n_people + per_block - 1) / per_block);
  L.nblk = (int)std::min<int64_t>(want, (int64_t)std::max(1, per_sm) * g_dev[L.dev].sms);
  L.st = (cudaStream_t)stream;
  return LPG_OK;
}

static int seirp_launch(const SeirpLaunch& L, int32_t* part) {
  if (L.vec)
    k_seirp_partial<true><<<L.nblk, SEIRP_THREADS, L.smem, L.st>>>(L.in, part);
  else
    k_seirp_partial<false><<<L.nblk, SEIRP_THREADS, L.smem, L.st>>>(L.in, part);
  k_seirp_reduce<<<(L.in.G + 31) / 32, SEIRP_THREADS, 0, L.st>>>(L.in, L.out, part, L.nblk);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return op_fail(LPG_ERR_CUDA, "count_SEIRP launch: %s", cudaGetErrorString(e));
  return LPG_OK;
}

extern "C" int lpg_count_seirp(const int16_t* node_id, const int8_t* disease_state, const int8_t* strain,
                               const int8_t* potentially_paralyzed, const int8_t* paralyzed, int32_t n_nodes,
                               int32_t n_strains, int64_t n_people, int32_t* S, int32_t* E, int32_t* I, int32_t* R,
                               int32_t* E_by_strain, int32_t* I_by_strain, int32_t* POTP, int32_t* P,
                               int64_t* n_invalid, void* stream) {
  SeirpLaunch L;
  int rc = seirp_prepare(L, node_id, disease_state, strain, potentially_paralyzed, paralyzed, n_nodes, n_strains,
                         n_people, S, E, I, R, E_by_strain, I_by_strain, POTP, P, n_invalid, stream);
  if (rc) return rc;
  int32_t* part = nullptr;
  const size_t bytes = (size_t)L.nblk * ((size_t)L.in.F * n_nodes + 1) * sizeof(int32_t);
  cudaError_t e = cudaMallocAsync((void**)&part, bytes, L.st);
  if (e != cudaSuccess) return op_fail(LPG_ERR_NOMEM, "count_SEIRP scratch: %s", cudaGetErrorString(e));
  rc = seirp_launch(L, part);
  e = cudaFreeAsync(part, L.st);
  if (rc) return rc;
  if (e != cudaSuccess) return op_fail(LPG_ERR_CUDA, "count_SEIRP scratch free: %s", cudaGetErrorString(e));
  return LPG_OK;
}

/* ------------------------------------------------------------------------ */
/* The no-allocation variant.  Its scratch is this file-scope array, one per
 * device that loads the library: LPG_COUNT_SEIRP_STATIC_WORDS int32 words
 * (4 MiB).  It exists for callers that cannot allocate device memory at call
 * time: a host process whose device memory is already claimed by its own
 * caching pool (a framework allocator that reserved the free memory, so a
 * second allocator fails with out-of-memory), and a loop that must not
 * stall the device (cudaFree synchronizes the whole device, and a
 * stream-ordered pool may have to grow).
 *
 * Nothing in the array needs to start at zero: every launch writes each
 * histogram slice in full before the reduce kernel reads it.  The grid is
 * shrunk so that nblk slices fit; the largest slice (4096 nodes, 4 strains)
 * still leaves room for 21 CTAs.
 *
 * All calls on one device share the array, so two calls whose kernels
 * overlap on the GPU (different streams, or different host threads without
 * ordering between their streams) race on it and may return wrong counts.
 * Serialize them, e.g. by issuing them on one stream. */
static __device__ __align__(256) int32_t g_seirp_scratch[LPG_COUNT_SEIRP_STATIC_WORDS];

/* The first call on each device takes the device address of
 * g_seirp_scratch with that device current (the call's current device);
 * later calls reuse it.  That first call per device should come before any
 * stream capture begins. */
static int seirp_static_setup(int dev, int32_t** out) {
  std::lock_guard<std::mutex> lk(g_dev_mu);
  SeirpDev& d = g_dev[dev];
  if (!d.static_ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_seirp_scratch);
    if (e != cudaSuccess || !p)
      return op_fail(LPG_ERR_CUDA, "count_SEIRP static scratch address: %s", cudaGetErrorString(e));
    d.static_scratch = (int32_t*)p;
    d.static_ready = true;
  }
  *out = d.static_scratch;
  return LPG_OK;
}

extern "C" int lpg_count_seirp_static(const int16_t* node_id, const int8_t* disease_state, const int8_t* strain,
                                      const int8_t* potentially_paralyzed, const int8_t* paralyzed, int32_t n_nodes,
                                      int32_t n_strains, int64_t n_people, int32_t* S, int32_t* E, int32_t* I,
                                      int32_t* R, int32_t* E_by_strain, int32_t* I_by_strain, int32_t* POTP,
                                      int32_t* P, int64_t* n_invalid, void* stream) {
  SeirpLaunch L;
  int rc = seirp_prepare(L, node_id, disease_state, strain, potentially_paralyzed, paralyzed, n_nodes, n_strains,
                         n_people, S, E, I, R, E_by_strain, I_by_strain, POTP, P, n_invalid, stream);
  if (rc) return rc;
  const int64_t slice = (int64_t)L.in.F * n_nodes + 1;
  if (slice > LPG_COUNT_SEIRP_STATIC_WORDS)
    return op_fail(LPG_ERR_ARG, "count_SEIRP_static: %lld histogram words exceed the static scratch of %d",
                   (long long)slice, LPG_COUNT_SEIRP_STATIC_WORDS);
  L.nblk = (int)std::min<int64_t>(L.nblk, LPG_COUNT_SEIRP_STATIC_WORDS / slice);
  int32_t* part = nullptr;
  rc = seirp_static_setup(L.dev, &part);
  if (rc) return rc;
  return seirp_launch(L, part);
}
