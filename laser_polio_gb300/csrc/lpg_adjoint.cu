/*
 * lpg_adjoint.cu — expected incidence of a tick range and its
 * vector-Jacobian product (lpg_incidence_plan_* and lpg_expected_incidence
 * in lpg.h).
 *
 * With the agent state held fixed, the transmission step's node-level part
 * (model.py:1315-1363) maps the replayed aggregates of each tick t — the
 * susceptibles' risk sum srisk[t,n], the pre-mixing infectivity
 * beta[t,n,s], the population pop[t,n] — to the expected exposures
 *
 *   N        = rownorm(gravity(p, d, k, a, b, c) / (sum p)^c, m)       (model.py:1250-1258)
 *   u[t,n,s] = beta[t,n,s] (1 - sum_k N[n,k]) + sum_i N[i,n] beta[t,i,s]
 *   seas[t]  = 1 + amp cos(2 pi (doy[t] - peak) / year[t])             (utils.py:589-625)
 *   r        = u seas[t] r0s[n] R / max(pop[t,n], 1)
 *   lam[t,n] = srisk[t,n] sum_s (1 - exp(-r))
 *
 * where R scales every agent's infectivity (R0 over the R0 the aggregates
 * were recorded at).  Given dL/dlam, the reverse pass returns dL/dR, dL/damp,
 * dL/dpeak, dL/dr0s, dL/dN and dL/d(k, a, b, c) through the row
 * normalisation (a row whose sum exceeds m is scaled down to m) and the
 * gravity flows k p_i^a p_j^b / d_ij^c (zero diagonal).  With a target
 * curve the plan also forms the calibration loss
 * L = sum (log1p(lam) - log1p(target))^2 and its dL/dlam on the device.
 *
 * Layout in HBM: a plan keeps the aggregates resident — srisk, pop [T][G];
 * beta as [T][S][G] (strain-major per tick, so that the (t, s) rows of the
 * mixing product and every elementwise pass read G consecutive doubles);
 * u, exp(-r) and dL/du the same way; log(dist) and the network and its
 * gradients [G][G]; log(pops) [G].
 *
 * Arithmetic: double precision throughout, except inside the two
 * contractions, u = beta N per (t, s) row and dL/dN = beta^T dL/du, both
 * (T S) x G x G.  GB300 issues about two FP64 FMAs per clock per SM and 128
 * FP32 FMAs, so the products run in double-float: their operands are held
 * as FP32 pairs hi + lo (beta split once per plan, N and dL/du by the
 * kernels that produce them), each term hi*hi is formed exactly (Dekker's
 * product via FMA) with the cross terms, and the running sum is an FP32
 * pair kept by Knuth's TwoSum — about 2^-44 relative per dot product,
 * twelve FP32 operations per term and no FP64 work inside the products.
 * The FP32 pair cannot hold magnitudes below 2^-126, so products of
 * operands under about 1e-19 each lose relative (not absolute) accuracy.
 * The sums use atomics, so results agree with a sequential FP64 evaluation
 * to rounding, not bit for bit.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "lpg.h"

/* Per-host-thread error text of the standalone ops (lpg_ops.cu). */
int lpg_ops_fail(int code, const char* fmt, ...);

namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;
#define INC_THREADS 256
#define DF_BM 32      /* product tile rows */
#define DF_BN 64      /* product tile columns */
#define DF_BK 32      /* product tile depth */
#define DF_THREADS 128 /* 4 x 4 outputs per thread */
#define DF_MAX_SPLIT 8 /* depth slices of the flows product */

enum { PH_NETWORK, PH_MIX, PH_FORWARD, PH_BACKWARD, PH_FLOWS, PH_NETWORK_GRAD, PH_COUNT };
const char* const kPhaseNames[PH_COUNT] = {"k_inc_network", "k_inc_gemm_mix", "k_inc_forward",
                                           "k_inc_backward", "k_inc_gemm_flows", "k_inc_network_grad"};

struct IncScalars {
  double R, amp, peak;
};

__device__ __forceinline__ double block_sum(double v, double* s_part) {
  s_part[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s_part[threadIdx.x] += s_part[threadIdx.x + o];
    __syncthreads();
  }
  const double r = s_part[0];
  __syncthreads();
  return r;
}

/* An FP64 value as an FP32 pair hi + lo. */
__device__ __forceinline__ float2 df_split(double x) {
  const float hi = __double2float_rn(x);
  return make_float2(hi, __double2float_rn(x - (double)hi));
}

__global__ void __launch_bounds__(INC_THREADS) k_inc_split(size_t n, const double* x, float2* y) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) y[idx] = df_split(x[idx]);
}

/* log(pops) [G] and log(dist) [G][G] (the diagonal is never read), once
 * per plan.  Zero gives -inf. */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_logs(int G, const double* pops, const double* dist, double* logp, double* logd) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < (size_t)G * G) logd[idx] = log(dist[idx]);
  if (idx < (size_t)G) logp[idx] = log(pops[idx]);
}

/* Blocks [0, G): one network row i each — the scaled gravity flows
 * G[i,j] = k p_i^a p_j^b / d_ij^c / P^c (zero diagonal; non-finite
 * values are 0), formed as k p_i^a exp(b log p_j - c log d_ij) / P^c with
 * the 0^0 = 1 convention kept, their sum rs[i], and the normalised row
 * N[i,j] (scaled down to max_frac when rs[i] exceeds it; stored as FP32
 * pairs for the mixing product) with its FP64 sum.
 * Blocks [G, G + ceil(T/256)): the seasonal factor of each tick and its
 * derivatives with respect to amp and peak. */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_network(int G, int T, const double* pops, const double* logp, const double* logd, double k, double a,
                  double b, double c, double Pc, double max_frac, double* Gm, float2* N, double* rs, double* rsN,
                  int* capped, const double* doy, const double* year, IncScalars sc, double* seas) {
  __shared__ double s_part[INC_THREADS];
  if ((int)blockIdx.x >= G) {
    const int t = (blockIdx.x - G) * INC_THREADS + threadIdx.x;
    if (t < T) {
      const double ang = kTwoPi * (doy[t] - sc.peak) / year[t];
      const double ca = cos(ang);
      seas[t] = 1.0 + sc.amp * ca;
      seas[T + t] = ca;                                      /* d seas / d amp */
      seas[2 * T + t] = sc.amp * sin(ang) * kTwoPi / year[t]; /* d seas / d peak */
    }
    return;
  }
  const int i = blockIdx.x;
  const double kpa = k * pow(pops[i], a) / Pc;
  double sum = 0.0;
  for (int j = threadIdx.x; j < G; j += blockDim.x) {
    double v = 0.0;
    if (j != i) {
      const double x = (b == 0.0 ? 0.0 : b * logp[j]) - (c == 0.0 ? 0.0 : c * logd[(size_t)i * G + j]);
      v = kpa * exp(x);
      if (!isfinite(v)) v = 0.0;
    }
    Gm[(size_t)i * G + j] = v;
    sum += v;
  }
  const double r = block_sum(sum, s_part);
  const bool cap = r > max_frac;
  double sumN = 0.0;
  for (int j = threadIdx.x; j < G; j += blockDim.x) {
    const double v = Gm[(size_t)i * G + j]; /* written by this thread above */
    const double nv = cap ? v * (max_frac / r) : v;
    N[(size_t)i * G + j] = df_split(nv);
    sumN += nv;
  }
  const double rn = block_sum(sumN, s_part);
  if (threadIdx.x == 0) {
    rs[i] = r;
    rsN[i] = rn;
    capped[i] = cap ? 1 : 0;
  }
}

/* (sh, sl) += a * b for FP32 pairs a, b: the exact product of the high
 * parts (Dekker, by FMA) plus the cross terms, added by Knuth's TwoSum.
 * The _rn intrinsics are never contracted or reassociated. */
__device__ __forceinline__ void df_fma(float& sh, float& sl, float2 a, float2 b) {
  const float ph = __fmul_rn(a.x, b.x);
  float pl = __fmaf_rn(a.x, b.x, -ph);
  pl = __fmaf_rn(a.x, b.y, pl);
  pl = __fmaf_rn(a.y, b.x, pl);
  const float s = __fadd_rn(sh, ph);
  const float bp = __fsub_rn(s, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bp)), __fsub_rn(ph, bp));
  sl = __fadd_rn(sl, __fadd_rn(err, pl));
  sh = s;
}

/* C_z[M][N] = sum over k in slice z of A(m, k) B[k][n], row-major, in
 * double-float, A and B given as FP32 pairs.  A(m, k) = A[m][k] (M x K) or, with TRANS_A, A[k][m]
 * (K x M).  blockIdx.z picks the depth slice [z kchunk, (z+1) kchunk) and
 * the output C + z M N.  32 x 64 tiles, 128 threads with 4 x 4 outputs
 * each (rows ty + 8i, columns tx + 16j). */
template <bool TRANS_A>
__global__ void __launch_bounds__(DF_THREADS)
    k_inc_gemm(int M, int N, int K, int kchunk, const float2* __restrict__ A, const float2* __restrict__ B,
               double* C) {
  __shared__ float2 sA[DF_BK][DF_BM + 1]; /* [k][m] */
  __shared__ float2 sB[DF_BK][DF_BN];     /* [k][n] */
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * DF_BM, n0 = blockIdx.x * DF_BN;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  float sh[4][4], sl[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) sh[i][j] = sl[i][j] = 0.f;
  for (int k0 = kb; k0 < ke; k0 += DF_BK) {
#pragma unroll
    for (int r = 0; r < (DF_BK * DF_BM) / DF_THREADS; ++r) {
      const int e = tid + r * DF_THREADS;
      const int hi = e >> 5, lo = e & 31;
      float2 v = make_float2(0.f, 0.f);
      if (TRANS_A) { /* hi = k, lo = m: consecutive threads read consecutive m */
        if (k0 + hi < ke && m0 + lo < M) v = A[(size_t)(k0 + hi) * M + m0 + lo];
        sA[hi][lo] = v;
      } else { /* hi = m, lo = k: consecutive threads read consecutive k */
        if (m0 + hi < M && k0 + lo < ke) v = A[(size_t)(m0 + hi) * K + k0 + lo];
        sA[lo][hi] = v;
      }
    }
#pragma unroll
    for (int r = 0; r < (DF_BK * DF_BN) / DF_THREADS; ++r) {
      const int e = tid + r * DF_THREADS;
      const int hi = e >> 6, lo = e & 63;
      float2 v = make_float2(0.f, 0.f);
      if (k0 + hi < ke && n0 + lo < N) v = B[(size_t)(k0 + hi) * N + n0 + lo];
      sB[hi][lo] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int q = 0; q < DF_BK; ++q) {
      float2 av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = sA[q][ty + 8 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = sB[q][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) df_fma(sh[i][j], sl[i][j], av[i], bv[j]);
    }
    /* renormalise each pair (Fast2Sum: |sh| >= |sl|) so that sl stays small */
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float t = __fadd_rn(sh[i][j], sl[i][j]);
        sl[i][j] = __fsub_rn(sl[i][j], __fsub_rn(t, sh[i][j]));
        sh[i][j] = t;
      }
    __syncthreads();
  }
  double* Cz = C + (size_t)blockIdx.z * M * N;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int row = m0 + ty + 8 * i;
    if (row >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = n0 + tx + 16 * j;
      if (col < N) Cz[(size_t)row * N + col] = (double)sh[i][j] + (double)sl[i][j];
    }
  }
}

/* Per (t, n), one tick per blockIdx.y: the mixing's diagonal term, the
 * rates, exp(-r) kept for the reverse pass, lam, and with a target the
 * loss term and dL/dlam. */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_forward(int T, int G, int S, const double* srisk, const double* beta, const double* pop,
                  const double* seas, const double* r0s, const double* rsN, IncScalars sc, double* u, double* e,
                  double* lam, const double* target, double* g, double* loss) {
  __shared__ double s_part[INC_THREADS];
  const int t = blockIdx.y, n = blockIdx.x * blockDim.x + threadIdx.x;
  const size_t idx = (size_t)t * G + n;
  double part = 0.0;
  if (n < G) {
    const double q = seas[t] * r0s[n] * sc.R / fmax(pop[idx], 1.0);
    double l = 0.0;
    for (int s = 0; s < S; ++s) {
      const size_t k = ((size_t)t * S + s) * G + n;
      const double uu = u[k] + beta[k] * (1.0 - rsN[n]);
      u[k] = uu;
      const double ex = exp(-(uu * q));
      e[k] = ex;
      l += 1.0 - ex;
    }
    const double lv = srisk[idx] * l;
    lam[idx] = lv;
    if (target) {
      const double r = log1p(lv) - log1p(target[idx]);
      g[idx] = 2.0 * r / (1.0 + lv);
      part = r * r;
    }
  }
  if (target) { /* uniform over the grid */
    const double tot = block_sum(part, s_part);
    if (threadIdx.x == 0) atomicAdd(loss, tot);
  }
}

/* Per (t, n) of the reverse pass, one tick per blockIdx.y: dL/du (as FP32
 * pairs for the dL/dN product) and the contributions to dL/dseas[t],
 * dL/dr0s[n] and dL/dR (block sums for the per-tick and scalar ones). */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_backward(int T, int G, int S, const double* g, const double* srisk, const double* pop, const double* seas,
                   const double* r0s, IncScalars sc, const double* u, const double* e, float2* gu, double* g_seas,
                   double* g_r0s, double* g_R) {
  __shared__ double s_part[INC_THREADS];
  const int t = blockIdx.y, n = blockIdx.x * blockDim.x + threadIdx.x;
  const size_t idx = (size_t)t * G + n;
  double cR = 0.0, cS = 0.0;
  if (n < G) {
    const double st = seas[t];
    const double popc = fmax(pop[idx], 1.0);
    const double q = st * r0s[n] * sc.R / popc;
    const double gs = g[idx] * srisk[idx];
    double gq = 0.0;
    for (int s = 0; s < S; ++s) {
      const size_t k = ((size_t)t * S + s) * G + n;
      const double gr = gs * e[k];
      gu[k] = df_split(gr * q);
      gq += gr * u[k];
    }
    cS = gq * r0s[n] * sc.R / popc;
    atomicAdd(&g_r0s[n], gq * st * sc.R / popc);
    cR = gq * st * r0s[n] / popc;
  }
  const double tS = block_sum(cS, s_part);
  const double tR = block_sum(cR, s_part);
  if (threadIdx.x == 0) {
    atomicAdd(&g_seas[t], tS);
    atomicAdd(g_R, tR);
  }
}

/* dL/damp and dL/dpeak from dL/dseas[t] (one CTA). */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_seasonal(int T, const double* seas, const double* g_seas, double* out) {
  __shared__ double s_part[INC_THREADS];
  double ga = 0.0, gp = 0.0;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    ga += g_seas[t] * seas[T + t];
    gp += g_seas[t] * seas[2 * T + t];
  }
  ga = block_sum(ga, s_part);
  gp = block_sum(gp, s_part);
  if (threadIdx.x == 0) {
    out[0] = ga;
    out[1] = gp;
  }
}

/* One row a per CTA: C[a][b] = the sum of the flows product's nsplit
 * depth slices, dL/dN[a][b] = C[a][b] - C[a][a] (zero on the diagonal),
 * then dL/dG through the row normalisation and the row's contributions to
 * dL/dk, dL/da, dL/db, dL/dc. */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_network_grad(int G, int nsplit, const double* C, const double* Gm, const double* rs, const int* capped,
                       const double* logp, const double* logd, double k, double logP, double max_frac, double* gN,
                       double* g_theta) {
  __shared__ double s_part[INC_THREADS];
  const int a = blockIdx.x;
  const size_t GG = (size_t)G * G, row = (size_t)a * G;
  double diag = 0.0;
  for (int z = 0; z < nsplit; ++z) diag += C[z * GG + row + a];
  double cpl = 0.0; /* the row's sum of dL/dN * G (the normalisation's coupling term) */
  for (int b = threadIdx.x; b < G; b += blockDim.x) {
    double cab = 0.0;
    for (int z = 0; z < nsplit; ++z) cab += C[z * GG + row + b];
    const double v = b == a ? 0.0 : cab - diag;
    gN[row + b] = v;
    cpl += v * Gm[row + b];
  }
  const double coupling = block_sum(cpl, s_part);
  const bool cap = capped[a] != 0;
  const double ra = rs[a];
  const double lpa = logp[a];
  double wk = 0.0, wa = 0.0, wb = 0.0, wc = 0.0;
  for (int b = threadIdx.x; b < G; b += blockDim.x) {
    if (b == a) continue;
    const double gn = gN[row + b]; /* written by this thread above */
    const double gg = cap ? (max_frac / ra) * (gn - coupling / ra) : gn;
    const double w = gg * Gm[row + b];
    if (w == 0.0) continue; /* a zero flow: its logs may be infinite */
    wk += w;
    wa += w * lpa;
    wb += w * logp[b];
    wc += w * (-logd[row + b] - logP);
  }
  wk = block_sum(wk, s_part);
  wa = block_sum(wa, s_part);
  wb = block_sum(wb, s_part);
  wc = block_sum(wc, s_part);
  if (threadIdx.x == 0) {
    atomicAdd(&g_theta[0], wk / k);
    atomicAdd(&g_theta[1], wa);
    atomicAdd(&g_theta[2], wb);
    atomicAdd(&g_theta[3], wc);
  }
}

}  // namespace

struct lpg_incidence_plan {
  int T = 0, G = 0, S = 0;
  int nsm = 0;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  double P = 0.0, logP = 0.0;
  /* resident inputs */
  double *srisk = nullptr, *beta = nullptr, *pop = nullptr, *doy = nullptr, *year = nullptr, *pops = nullptr,
         *logp = nullptr, *logd = nullptr, *target = nullptr;
  /* per evaluation */
  double *r0s = nullptr, *seas = nullptr, *Gm = nullptr, *rs = nullptr, *rsN = nullptr, *u = nullptr,
         *e = nullptr, *lam = nullptr, *g = nullptr, *gseas = nullptr, *gr0s = nullptr, *scal = nullptr,
         *C = nullptr, *gN = nullptr;
  float2 *beta_hl = nullptr, *N = nullptr, *gu = nullptr; /* the products' operands as FP32 pairs */
  int* cap = nullptr;
  double* h_scal = nullptr; /* pinned: [0] loss, [1] R, [2] amp, [3] peak, [4..7] k, a, b, c */
  /* profiling */
  bool prof = false;
  cudaEvent_t ev[PH_COUNT + 1] = {};
  double ms[PH_COUNT] = {};
  int64_t launches[PH_COUNT] = {};
};

namespace {

int plan_cuda(cudaError_t e, const char* what) {
  return e == cudaSuccess ? LPG_OK : lpg_ops_fail(LPG_ERR_CUDA, "incidence plan: %s: %s", what, cudaGetErrorString(e));
}

#define PCK(call)                             \
  do {                                        \
    const int rc_ = plan_cuda((call), #call); \
    if (rc_ != LPG_OK) return rc_;            \
  } while (0)

template <typename T>
int dalloc(T** p, size_t n) {
  if (cudaMalloc((void**)p, sizeof(T) * (n ? n : 1)) != cudaSuccess) {
    *p = nullptr;
    return lpg_ops_fail(LPG_ERR_NOMEM, "incidence plan: device allocation of %zu bytes failed", sizeof(T) * n);
  }
  return LPG_OK;
}

void plan_free(lpg_incidence_plan* p) {
  void* ps[] = {p->srisk, p->beta, p->pop, p->doy, p->year,  p->pops, p->logp, p->logd, p->target,
                p->r0s,   p->seas, p->Gm,  p->N,   p->rs,    p->rsN,  p->u,    p->e,    p->lam,
                p->g,     p->gu,   p->gseas, p->gr0s, p->scal, p->C,   p->gN,   p->cap,  p->beta_hl};
  for (void* q : ps)
    if (q) cudaFree(q);
  if (p->h_scal) cudaFreeHost(p->h_scal);
  for (auto& ev : p->ev)
    if (ev) cudaEventDestroy(ev);
  if (p->own_stream && p->st) cudaStreamDestroy(p->st);
  delete p;
}

int plan_alloc(lpg_incidence_plan* p) {
  const size_t T = p->T, G = p->G, TG = T * G, TSG = TG * p->S, GG = G * G;
  int rc;
  if ((rc = dalloc(&p->srisk, TG)) || (rc = dalloc(&p->beta, TSG)) || (rc = dalloc(&p->pop, TG)) ||
      (rc = dalloc(&p->doy, T)) || (rc = dalloc(&p->year, T)) || (rc = dalloc(&p->pops, G)) ||
      (rc = dalloc(&p->logp, G)) || (rc = dalloc(&p->logd, GG)) || (rc = dalloc(&p->r0s, G)) ||
      (rc = dalloc(&p->seas, 3 * T)) || (rc = dalloc(&p->Gm, GG)) || (rc = dalloc(&p->N, GG)) ||
      (rc = dalloc(&p->beta_hl, TSG)) ||
      (rc = dalloc(&p->rs, G)) || (rc = dalloc(&p->rsN, G)) || (rc = dalloc(&p->cap, G)) ||
      (rc = dalloc(&p->u, TSG)) || (rc = dalloc(&p->e, TSG)) || (rc = dalloc(&p->lam, TG)) ||
      (rc = dalloc(&p->g, TG)) || (rc = dalloc(&p->gu, TSG)) || (rc = dalloc(&p->gseas, T)) ||
      (rc = dalloc(&p->gr0s, G)) || (rc = dalloc(&p->scal, 8)) || (rc = dalloc(&p->C, DF_MAX_SPLIT * GG)) ||
      (rc = dalloc(&p->gN, GG)))
    return rc;
  PCK(cudaMallocHost((void**)&p->h_scal, 8 * sizeof(double)));
  for (auto& ev : p->ev) PCK(cudaEventCreate(&ev));
  return LPG_OK;
}

/* Marks the start of phase ph (and the end of the previous one). */
inline void mark(lpg_incidence_plan* p, int ph, int n_launch) {
  if (p->prof) cudaEventRecord(p->ev[ph], p->st);
  p->launches[ph] += n_launch;
}

int plan_forward(lpg_incidence_plan* p, const lpg_incidence_params* prm, IncScalars sc, bool with_loss) {
  const int T = p->T, G = p->G, S = p->S;
  const double Pc = pow(p->P, prm->c);
  mark(p, PH_NETWORK, 1);
  k_inc_network<<<G + (T + INC_THREADS - 1) / INC_THREADS, INC_THREADS, 0, p->st>>>(
      G, T, p->pops, p->logp, p->logd, prm->k, prm->a, prm->b, prm->c, Pc, prm->max_frac, p->Gm, p->N, p->rs,
      p->rsN, p->cap, p->doy, p->year, sc, p->seas);
  mark(p, PH_MIX, 1);
  {
    const dim3 grd((G + DF_BN - 1) / DF_BN, (T * S + DF_BM - 1) / DF_BM, 1);
    k_inc_gemm<false><<<grd, DF_THREADS, 0, p->st>>>(T * S, G, G, G, p->beta_hl, p->N, p->u);
  }
  mark(p, PH_FORWARD, 1);
  k_inc_forward<<<dim3((G + INC_THREADS - 1) / INC_THREADS, T), INC_THREADS, 0, p->st>>>(
      T, G, S, p->srisk, p->beta, p->pop, p->seas, p->r0s, p->rsN, sc, p->u, p->e, p->lam,
      with_loss ? p->target : nullptr, p->g, p->scal);
  return plan_cuda(cudaGetLastError(), "forward launch");
}

int plan_backward(lpg_incidence_plan* p, const lpg_incidence_params* prm, IncScalars sc) {
  const int T = p->T, G = p->G, S = p->S;
  mark(p, PH_BACKWARD, 2);
  k_inc_backward<<<dim3((G + INC_THREADS - 1) / INC_THREADS, T), INC_THREADS, 0, p->st>>>(
      T, G, S, p->g, p->srisk, p->pop, p->seas, p->r0s, sc, p->u, p->e, p->gu, p->gseas, p->gr0s, p->scal + 1);
  k_inc_seasonal<<<1, INC_THREADS, 0, p->st>>>(T, p->seas, p->gseas, p->scal + 2);
  mark(p, PH_FLOWS, 1);
  /* depth slices so that the G x G output fills the SMs about four deep */
  const int K = T * S, gx = (G + DF_BN - 1) / DF_BN, gy = (G + DF_BM - 1) / DF_BM;
  const int ktiles = (K + DF_BK - 1) / DF_BK;
  int split = (4 * p->nsm + gx * gy - 1) / (gx * gy);
  split = split < 1 ? 1 : split > DF_MAX_SPLIT ? DF_MAX_SPLIT : split;
  if (split > ktiles) split = ktiles;
  const int kchunk = ((ktiles + split - 1) / split) * DF_BK;
  const int nsplit = (K + kchunk - 1) / kchunk;
  k_inc_gemm<true><<<dim3(gx, gy, nsplit), DF_THREADS, 0, p->st>>>(G, G, K, kchunk, p->beta_hl, p->gu, p->C);
  mark(p, PH_NETWORK_GRAD, 1);
  k_inc_network_grad<<<G, INC_THREADS, 0, p->st>>>(G, nsplit, p->C, p->Gm, p->rs, p->cap, p->logp, p->logd,
                                                   prm->k, p->logP, prm->max_frac, p->gN, p->scal + 4);
  return plan_cuda(cudaGetLastError(), "backward launch");
}

}  // namespace

extern "C" int lpg_incidence_plan_create(const lpg_incidence_in* in, const double* target, void* stream,
                                         lpg_incidence_plan** out) {
  if (!in || !out) return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: null argument");
  *out = nullptr;
  const int T = in->T, G = in->G, S = in->S;
  if (T <= 0 || G <= 0 || S <= 0 || S > LPG_MAX_STRAINS)
    return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: bad sizes T=%d G=%d S=%d", T, G, S);
  if ((int64_t)T * S > 65535LL * DF_BM || T > 65535)
    return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: T=%d or T*S = %lld too large (T <= 65535, T*S <= %d)", T,
                        (long long)T * S, 65535 * DF_BM);
  if (!in->srisk || !in->beta || !in->pop || !in->doy || !in->year || !in->pops || !in->dist)
    return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: null input array");
  double P = 0.0;
  for (int i = 0; i < G; ++i) {
    if (!(in->pops[i] >= 0.0)) return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: pops[%d] is negative", i);
    P += in->pops[i];
  }
  if (!(P > 0.0) || !std::isfinite(P)) return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: total population %g", P);
  for (size_t i = 0; i < (size_t)G * G; ++i)
    if ((int)(i / G) != (int)(i % G) && !(in->dist[i] >= 0.0))
      return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: dist[%zu][%zu] is negative", i / G, i % G);
  lpg_incidence_plan* p = new lpg_incidence_plan;
  p->T = T;
  p->G = G;
  p->S = S;
  p->P = P;
  p->logP = log(P);
  int rc = LPG_OK;
  int dev = 0;
  rc = plan_cuda(cudaGetDevice(&dev), "device");
  if (rc == LPG_OK) rc = plan_cuda(cudaDeviceGetAttribute(&p->nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
  if (rc == LPG_OK) {
    if (stream) {
      p->st = (cudaStream_t)stream;
    } else {
      rc = plan_cuda(cudaStreamCreateWithFlags(&p->st, cudaStreamNonBlocking), "stream");
      p->own_stream = rc == LPG_OK;
    }
  }
  if (rc == LPG_OK) rc = plan_alloc(p);
  double* d_dist = nullptr;
  if (rc == LPG_OK) rc = dalloc(&d_dist, (size_t)G * G);
  if (rc == LPG_OK) {
    const size_t TG = (size_t)T * G, GG = (size_t)G * G;
    std::vector<double> bt(TG * S); /* [T][G][S] -> [T][S][G] */
    for (int t = 0; t < T; ++t)
      for (int n = 0; n < G; ++n)
        for (int s = 0; s < S; ++s) bt[((size_t)t * S + s) * G + n] = in->beta[((size_t)t * G + n) * S + s];
    struct {
      double* dst;
      const double* src;
      size_t n;
    } up[] = {{p->srisk, in->srisk, TG},       {p->beta, bt.data(), TG * S},        {p->pop, in->pop, TG},
              {p->doy, in->doy, (size_t)T},    {p->year, in->year, (size_t)T},      {p->pops, in->pops, (size_t)G},
              {d_dist, in->dist, GG}};
    for (auto& c : up) {
      rc = plan_cuda(cudaMemcpyAsync(c.dst, c.src, sizeof(double) * c.n, cudaMemcpyHostToDevice, p->st), "upload");
      if (rc != LPG_OK) break;
    }
    if (rc == LPG_OK) {
      k_inc_logs<<<(unsigned)((GG + INC_THREADS - 1) / INC_THREADS), INC_THREADS, 0, p->st>>>(G, p->pops, d_dist,
                                                                                             p->logp, p->logd);
      k_inc_split<<<(unsigned)((TG * S + INC_THREADS - 1) / INC_THREADS), INC_THREADS, 0, p->st>>>(TG * S, p->beta,
                                                                                                 p->beta_hl);
      rc = plan_cuda(cudaGetLastError(), "log launch");
    }
    if (rc == LPG_OK && target) {
      rc = dalloc(&p->target, TG);
      if (rc == LPG_OK)
        rc = plan_cuda(cudaMemcpyAsync(p->target, target, sizeof(double) * TG, cudaMemcpyHostToDevice, p->st),
                       "upload target");
    }
    if (rc == LPG_OK) rc = plan_cuda(cudaStreamSynchronize(p->st), "upload sync");
  }
  if (d_dist) cudaFree(d_dist);
  if (rc != LPG_OK) {
    plan_free(p);
    return rc;
  }
  *out = p;
  return LPG_OK;
}

extern "C" int lpg_incidence_plan_eval(lpg_incidence_plan* p, const lpg_incidence_params* prm, const double* g_lam,
                                       double* lam_out, double* loss_out, lpg_incidence_grad* grad) {
  if (!p || !prm || !prm->r0s) return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: null argument");
  if (grad && !g_lam && !p->target)
    return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: a gradient needs g_lam or a target");
  if (loss_out && !p->target) return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: a loss needs a target");
  const int T = p->T, G = p->G;
  const size_t TG = (size_t)T * G, GG = (size_t)G * G;
  const IncScalars sc{prm->R, prm->amp, prm->peak};
  const bool with_loss = p->target != nullptr && (!g_lam || loss_out);
  PCK(cudaMemcpyAsync(p->r0s, prm->r0s, sizeof(double) * G, cudaMemcpyHostToDevice, p->st));
  PCK(cudaMemsetAsync(p->scal, 0, sizeof(double) * 8, p->st));
  int rc = plan_forward(p, prm, sc, with_loss);
  if (rc != LPG_OK) return rc;
  if (grad) {
    if (g_lam) PCK(cudaMemcpyAsync(p->g, g_lam, sizeof(double) * TG, cudaMemcpyHostToDevice, p->st));
    PCK(cudaMemsetAsync(p->gseas, 0, sizeof(double) * T, p->st));
    PCK(cudaMemsetAsync(p->gr0s, 0, sizeof(double) * G, p->st));
    rc = plan_backward(p, prm, sc);
    if (rc != LPG_OK) return rc;
  }
  if (p->prof) PCK(cudaEventRecord(p->ev[PH_COUNT], p->st));
  PCK(cudaMemcpyAsync(p->h_scal, p->scal, sizeof(double) * 8, cudaMemcpyDeviceToHost, p->st));
  if (lam_out) PCK(cudaMemcpyAsync(lam_out, p->lam, sizeof(double) * TG, cudaMemcpyDeviceToHost, p->st));
  if (grad && grad->r0s) PCK(cudaMemcpyAsync(grad->r0s, p->gr0s, sizeof(double) * G, cudaMemcpyDeviceToHost, p->st));
  if (grad && grad->network)
    PCK(cudaMemcpyAsync(grad->network, p->gN, sizeof(double) * GG, cudaMemcpyDeviceToHost, p->st));
  PCK(cudaStreamSynchronize(p->st));
  if (p->prof) {
    const int last = grad ? PH_COUNT : PH_BACKWARD;
    for (int ph = 0; ph < last; ++ph) {
      float ms = 0.f;
      const int nxt = ph + 1 == last ? PH_COUNT : ph + 1;
      PCK(cudaEventElapsedTime(&ms, p->ev[ph], p->ev[nxt]));
      p->ms[ph] += ms;
    }
  }
  if (loss_out) *loss_out = p->h_scal[0];
  if (grad) {
    grad->R = p->h_scal[1];
    grad->amp = p->h_scal[2];
    grad->peak = p->h_scal[3];
    grad->k = p->h_scal[4];
    grad->a = p->h_scal[5];
    grad->b = p->h_scal[6];
    grad->c = p->h_scal[7];
  }
  return LPG_OK;
}

extern "C" void* lpg_incidence_plan_stream(lpg_incidence_plan* p) { return p ? (void*)p->st : nullptr; }

extern "C" int lpg_incidence_plan_set_profiling(lpg_incidence_plan* p, int32_t enable) {
  if (!p) return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: null argument");
  p->prof = enable != 0;
  for (int ph = 0; ph < PH_COUNT; ++ph) {
    p->ms[ph] = 0.0;
    p->launches[ph] = 0;
  }
  return LPG_OK;
}

extern "C" int lpg_incidence_plan_read_profile(lpg_incidence_plan* p, lpg_profile* out) {
  if (!p || !out) return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: null argument");
  *out = lpg_profile{};
  out->n_kernels = PH_COUNT;
  for (int ph = 0; ph < PH_COUNT; ++ph) {
    out->names[ph] = kPhaseNames[ph];
    out->total_ms[ph] = p->ms[ph];
    out->launches[ph] = p->launches[ph];
  }
  return LPG_OK;
}

extern "C" void lpg_incidence_plan_destroy(lpg_incidence_plan* p) {
  if (p) plan_free(p);
}

extern "C" int lpg_expected_incidence(const lpg_incidence_in* in, double* lam_out, const double* g_lam,
                                      lpg_incidence_grad* grad, void* stream) {
  if (!in || !lam_out) return lpg_ops_fail(LPG_ERR_ARG, "expected_incidence: null argument");
  if (g_lam && !grad) return lpg_ops_fail(LPG_ERR_ARG, "expected_incidence: a gradient needs grad");
  if (!in->r0s) return lpg_ops_fail(LPG_ERR_ARG, "expected_incidence: null input array");
  lpg_incidence_plan* p = nullptr;
  int rc = lpg_incidence_plan_create(in, nullptr, stream, &p);
  if (rc != LPG_OK) return rc;
  const lpg_incidence_params prm{in->R, in->amp, in->peak, in->k, in->a, in->b, in->c, in->max_frac, in->r0s};
  rc = lpg_incidence_plan_eval(p, &prm, g_lam, lam_out, nullptr, g_lam ? grad : nullptr);
  lpg_incidence_plan_destroy(p);
  return rc;
}
