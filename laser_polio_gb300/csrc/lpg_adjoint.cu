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
 * u, exp(-r) and dL/du the same way; the network and its gradients [G][G].
 *
 * Everything is double precision.  The two contractions, u = beta N per
 * (t, s) row and dL/dN = beta^T dL/du, are (T S) x G x G products done by
 * one shared-memory tiled kernel; the rest is elementwise work and per-row
 * or per-tick reductions.  The sums use atomics, so results agree with a
 * sequential evaluation to rounding, not bit for bit.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "lpg.h"

/* Per-host-thread error text of the standalone ops (lpg_ops.cu). */
int lpg_ops_fail(int code, const char* fmt, ...);

namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;
#define INC_TILE 32
#define INC_THREADS 256

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

/* One row i per CTA: the scaled gravity flows G[i,j] = k p_i^a p_j^b /
 * d_ij^c / P^c (zero diagonal), their sum rs[i], and the normalised row
 * N[i,j] (scaled down to max_frac when rs[i] exceeds it) with its sum. */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_network(int G, const double* pops, const double* dist, double k, double a, double b, double c, double Pc,
                  double max_frac, double* Gm, double* N, double* rs, double* rsN, int* capped) {
  __shared__ double s_part[INC_THREADS];
  const int i = blockIdx.x;
  const double pa = pow(pops[i], a);
  double sum = 0.0;
  for (int j = threadIdx.x; j < G; j += blockDim.x) {
    double v = 0.0;
    if (j != i) {
      v = k * pa * pow(pops[j], b) / pow(dist[(size_t)i * G + j], c) / Pc;
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
    N[(size_t)i * G + j] = nv;
    sumN += nv;
  }
  const double rn = block_sum(sumN, s_part);
  if (threadIdx.x == 0) {
    rs[i] = r;
    rsN[i] = rn;
    capped[i] = cap ? 1 : 0;
  }
}

/* C[M][N] = sum_k A(m, k) B[k][n], row-major, over 32 x 32 tiles staged in
 * shared memory; 256 threads, each with a 2 x 2 block of outputs (rows
 * ty, ty + 16; columns tx, tx + 16).  A(m, k) = A[m][k] (M x K) or, with
 * TRANS_A, A[k][m] (K x M).  The FP64 pipe bounds it (GB300 issues about
 * two FP64 FMAs per clock per SM; two shared loads per FMA are far inside
 * the shared-memory bandwidth). */
template <bool TRANS_A>
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_gemm(int M, int N, int K, const double* __restrict__ A, const double* __restrict__ B, double* C) {
  __shared__ double sA[INC_TILE][INC_TILE + 1]; /* [k][m] */
  __shared__ double sB[INC_TILE][INC_TILE + 1]; /* [k][n] */
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * INC_TILE, n0 = blockIdx.x * INC_TILE;
  double c00 = 0.0, c01 = 0.0, c10 = 0.0, c11 = 0.0;
  for (int k0 = 0; k0 < K; k0 += INC_TILE) {
#pragma unroll
    for (int r = 0; r < (INC_TILE * INC_TILE) / INC_THREADS; ++r) {
      const int e = tid + r * INC_THREADS;
      const int hi = e >> 5, lo = e & 31;
      double va = 0.0;
      if (TRANS_A) { /* hi = k, lo = m: consecutive threads read consecutive m */
        if (k0 + hi < K && m0 + lo < M) va = A[(size_t)(k0 + hi) * M + m0 + lo];
        sA[hi][lo] = va;
      } else { /* hi = m, lo = k: consecutive threads read consecutive k */
        if (m0 + hi < M && k0 + lo < K) va = A[(size_t)(m0 + hi) * K + k0 + lo];
        sA[lo][hi] = va;
      }
      double vb = 0.0;
      if (k0 + hi < K && n0 + lo < N) vb = B[(size_t)(k0 + hi) * N + n0 + lo];
      sB[hi][lo] = vb;
    }
    __syncthreads();
#pragma unroll 8
    for (int q = 0; q < INC_TILE; ++q) {
      const double a0 = sA[q][ty], a1 = sA[q][ty + 16];
      const double b0 = sB[q][tx], b1 = sB[q][tx + 16];
      c00 = fma(a0, b0, c00); /* fused even under --fmad=false */
      c01 = fma(a0, b1, c01);
      c10 = fma(a1, b0, c10);
      c11 = fma(a1, b1, c11);
    }
    __syncthreads();
  }
  const int r0 = m0 + ty, r1 = m0 + ty + 16, q0 = n0 + tx, q1 = n0 + tx + 16;
  if (r0 < M && q0 < N) C[(size_t)r0 * N + q0] = c00;
  if (r0 < M && q1 < N) C[(size_t)r0 * N + q1] = c01;
  if (r1 < M && q0 < N) C[(size_t)r1 * N + q0] = c10;
  if (r1 < M && q1 < N) C[(size_t)r1 * N + q1] = c11;
}

__device__ __forceinline__ double seasonal(const double* doy, const double* year, int t, const IncScalars& sc) {
  return 1.0 + sc.amp * cos(kTwoPi * (doy[t] - sc.peak) / year[t]);
}

/* Per (t, n): the mixing's diagonal term, the rates, exp(-r) kept for the
 * reverse pass, lam, and with a target the loss term and dL/dlam. */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_forward(int T, int G, int S, const double* srisk, const double* beta, const double* pop, const double* doy,
                  const double* year, const double* r0s, const double* rsN, IncScalars sc, double* u, double* e,
                  double* lam, const double* target, double* g, double* loss) {
  __shared__ double s_part[INC_THREADS];
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double part = 0.0;
  if (idx < (size_t)T * G) {
    const int t = (int)(idx / G), n = (int)(idx % G);
    const double q = seasonal(doy, year, t, sc) * r0s[n] * sc.R / fmax(pop[idx], 1.0);
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

/* Per (t, n) of the reverse pass: dL/du (kept for the dL/dN product) and
 * the contributions to dL/dseas[t], dL/dr0s[n] and dL/dR. */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_backward(int T, int G, int S, const double* g, const double* srisk, const double* pop, const double* doy,
                   const double* year, const double* r0s, IncScalars sc, const double* u, const double* e,
                   double* gu, double* g_seas, double* g_r0s, double* g_R) {
  __shared__ double s_part[INC_THREADS];
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double cR = 0.0;
  if (idx < (size_t)T * G) {
    const int t = (int)(idx / G), n = (int)(idx % G);
    const double seas = seasonal(doy, year, t, sc);
    const double popc = fmax(pop[idx], 1.0);
    const double q = seas * r0s[n] * sc.R / popc;
    const double gs = g[idx] * srisk[idx];
    double gq = 0.0;
    for (int s = 0; s < S; ++s) {
      const size_t k = ((size_t)t * S + s) * G + n;
      const double gr = gs * e[k];
      gu[k] = gr * q;
      gq += gr * u[k];
    }
    atomicAdd(&g_seas[t], gq * r0s[n] * sc.R / popc);
    atomicAdd(&g_r0s[n], gq * seas * sc.R / popc);
    cR = gq * seas * r0s[n] / popc;
  }
  const double tot = block_sum(cR, s_part);
  if (threadIdx.x == 0) atomicAdd(g_R, tot);
}

/* dL/damp and dL/dpeak from dL/dseas[t] (one CTA). */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_seasonal(int T, const double* doy, const double* year, const double* g_seas, IncScalars sc, double* out) {
  __shared__ double s_part[INC_THREADS];
  double ga = 0.0, gp = 0.0;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const double ang = kTwoPi * (doy[t] - sc.peak) / year[t];
    ga += g_seas[t] * cos(ang);
    gp += g_seas[t] * sc.amp * sin(ang) * kTwoPi / year[t];
  }
  ga = block_sum(ga, s_part);
  gp = block_sum(gp, s_part);
  if (threadIdx.x == 0) {
    out[0] = ga;
    out[1] = gp;
  }
}

/* One row a per CTA: dL/dN[a][b] = C[a][b] - C[a][a] (zero on the
 * diagonal), then dL/dG through the row normalisation and the row's
 * contributions to dL/dk, dL/da, dL/db, dL/dc. */
__global__ void __launch_bounds__(INC_THREADS)
    k_inc_network_grad(int G, const double* C, const double* Gm, const double* rs, const int* capped,
                       const double* pops, const double* dist, double k, double logP, double max_frac, double* gN,
                       double* g_theta) {
  __shared__ double s_part[INC_THREADS];
  const int a = blockIdx.x;
  const double diag = C[(size_t)a * G + a];
  double cpl = 0.0; /* the row's sum of dL/dN * G (the normalisation's coupling term) */
  for (int b = threadIdx.x; b < G; b += blockDim.x) {
    const double v = b == a ? 0.0 : C[(size_t)a * G + b] - diag;
    gN[(size_t)a * G + b] = v;
    cpl += v * Gm[(size_t)a * G + b];
  }
  const double coupling = block_sum(cpl, s_part);
  const bool cap = capped[a] != 0;
  const double ra = rs[a];
  const double lpa = log(pops[a]);
  double wk = 0.0, wa = 0.0, wb = 0.0, wc = 0.0;
  for (int b = threadIdx.x; b < G; b += blockDim.x) {
    if (b == a) continue;
    const double gn = gN[(size_t)a * G + b]; /* written by this thread above */
    const double gg = cap ? (max_frac / ra) * (gn - coupling / ra) : gn;
    const double w = gg * Gm[(size_t)a * G + b];
    if (w == 0.0) continue; /* a zero flow: its logs may be infinite */
    wk += w;
    wa += w * lpa;
    wb += w * log(pops[b]);
    wc += w * (-log(dist[(size_t)a * G + b]) - logP);
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
  cudaStream_t st = nullptr;
  bool own_stream = false;
  double P = 0.0, logP = 0.0;
  /* resident inputs */
  double *srisk = nullptr, *beta = nullptr, *pop = nullptr, *doy = nullptr, *year = nullptr, *pops = nullptr,
         *dist = nullptr, *target = nullptr;
  /* per evaluation */
  double *r0s = nullptr, *Gm = nullptr, *N = nullptr, *rs = nullptr, *rsN = nullptr, *u = nullptr, *e = nullptr,
         *lam = nullptr, *g = nullptr, *gu = nullptr, *gseas = nullptr, *gr0s = nullptr, *scal = nullptr,
         *C = nullptr, *gN = nullptr;
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

#define PCK(call)                                \
  do {                                           \
    const int rc_ = plan_cuda((call), #call);    \
    if (rc_ != LPG_OK) return rc_;               \
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
  void* ps[] = {p->srisk, p->beta, p->pop,   p->doy,   p->year, p->pops, p->dist, p->target, p->r0s, p->Gm,
                p->N,     p->rs,   p->rsN,   p->u,     p->e,    p->lam,  p->g,    p->gu,     p->gseas, p->gr0s,
                p->scal,  p->C,    p->gN,    p->cap};
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
      (rc = dalloc(&p->dist, GG)) || (rc = dalloc(&p->r0s, G)) || (rc = dalloc(&p->Gm, GG)) ||
      (rc = dalloc(&p->N, GG)) || (rc = dalloc(&p->rs, G)) || (rc = dalloc(&p->rsN, G)) ||
      (rc = dalloc(&p->cap, G)) || (rc = dalloc(&p->u, TSG)) || (rc = dalloc(&p->e, TSG)) ||
      (rc = dalloc(&p->lam, TG)) || (rc = dalloc(&p->g, TG)) || (rc = dalloc(&p->gu, TSG)) ||
      (rc = dalloc(&p->gseas, T)) || (rc = dalloc(&p->gr0s, G)) || (rc = dalloc(&p->scal, 8)) ||
      (rc = dalloc(&p->C, GG)) || (rc = dalloc(&p->gN, GG)))
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
  const size_t TG = (size_t)T * G;
  const double Pc = pow(p->P, prm->c);
  mark(p, PH_NETWORK, 1);
  k_inc_network<<<G, INC_THREADS, 0, p->st>>>(G, p->pops, p->dist, prm->k, prm->a, prm->b, prm->c, Pc,
                                              prm->max_frac, p->Gm, p->N, p->rs, p->rsN, p->cap);
  mark(p, PH_MIX, 1);
  {
    const dim3 grd((G + INC_TILE - 1) / INC_TILE, (T * S + INC_TILE - 1) / INC_TILE);
    k_inc_gemm<false><<<grd, INC_THREADS, 0, p->st>>>(T * S, G, G, p->beta, p->N, p->u);
  }
  mark(p, PH_FORWARD, 1);
  k_inc_forward<<<(unsigned)((TG + INC_THREADS - 1) / INC_THREADS), INC_THREADS, 0, p->st>>>(
      T, G, S, p->srisk, p->beta, p->pop, p->doy, p->year, p->r0s, p->rsN, sc, p->u, p->e, p->lam,
      with_loss ? p->target : nullptr, p->g, p->scal);
  return plan_cuda(cudaGetLastError(), "forward launch");
}

int plan_backward(lpg_incidence_plan* p, const lpg_incidence_params* prm, IncScalars sc) {
  const int T = p->T, G = p->G, S = p->S;
  const size_t TG = (size_t)T * G;
  mark(p, PH_BACKWARD, 2);
  k_inc_backward<<<(unsigned)((TG + INC_THREADS - 1) / INC_THREADS), INC_THREADS, 0, p->st>>>(
      T, G, S, p->g, p->srisk, p->pop, p->doy, p->year, p->r0s, sc, p->u, p->e, p->gu, p->gseas, p->gr0s,
      p->scal + 1);
  k_inc_seasonal<<<1, INC_THREADS, 0, p->st>>>(T, p->doy, p->year, p->gseas, sc, p->scal + 2);
  mark(p, PH_FLOWS, 1);
  {
    const dim3 grd((G + INC_TILE - 1) / INC_TILE, (G + INC_TILE - 1) / INC_TILE);
    k_inc_gemm<true><<<grd, INC_THREADS, 0, p->st>>>(G, G, T * S, p->beta, p->gu, p->C);
  }
  mark(p, PH_NETWORK_GRAD, 1);
  k_inc_network_grad<<<G, INC_THREADS, 0, p->st>>>(G, p->C, p->Gm, p->rs, p->cap, p->pops, p->dist, prm->k,
                                                   p->logP, prm->max_frac, p->gN, p->scal + 4);
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
  if ((int64_t)T * S > 65535LL * INC_TILE)
    return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: T*S = %lld above %d", (long long)T * S, 65535 * INC_TILE);
  if (!in->srisk || !in->beta || !in->pop || !in->doy || !in->year || !in->pops || !in->dist)
    return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: null input array");
  double P = 0.0;
  for (int i = 0; i < G; ++i) {
    if (!(in->pops[i] >= 0.0)) return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: pops[%d] is negative", i);
    P += in->pops[i];
  }
  if (!(P > 0.0) || !std::isfinite(P)) return lpg_ops_fail(LPG_ERR_ARG, "incidence plan: total population %g", P);
  lpg_incidence_plan* p = new lpg_incidence_plan;
  p->T = T;
  p->G = G;
  p->S = S;
  p->P = P;
  p->logP = log(P);
  int rc = LPG_OK;
  if (stream) {
    p->st = (cudaStream_t)stream;
  } else {
    rc = plan_cuda(cudaStreamCreateWithFlags(&p->st, cudaStreamNonBlocking), "stream");
    p->own_stream = rc == LPG_OK;
  }
  if (rc == LPG_OK) rc = plan_alloc(p);
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
    } up[] = {{p->srisk, in->srisk, TG}, {p->beta, bt.data(), TG * S}, {p->pop, in->pop, TG}, {p->doy, in->doy, (size_t)T},
              {p->year, in->year, (size_t)T}, {p->pops, in->pops, (size_t)G}, {p->dist, in->dist, GG}};
    for (auto& c : up) {
      rc = plan_cuda(cudaMemcpyAsync(c.dst, c.src, sizeof(double) * c.n, cudaMemcpyHostToDevice, p->st), "upload");
      if (rc != LPG_OK) break;
    }
    if (rc == LPG_OK && target) {
      rc = dalloc(&p->target, TG);
      if (rc == LPG_OK)
        rc = plan_cuda(cudaMemcpyAsync(p->target, target, sizeof(double) * TG, cudaMemcpyHostToDevice, p->st),
                       "upload target");
    }
    if (rc == LPG_OK) rc = plan_cuda(cudaStreamSynchronize(p->st), "upload sync");
  }
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
  const bool with_loss = p->target != nullptr && !g_lam;
  PCK(cudaMemcpyAsync(p->r0s, prm->r0s, sizeof(double) * G, cudaMemcpyHostToDevice, p->st));
  PCK(cudaMemsetAsync(p->scal, 0, sizeof(double) * 8, p->st));
  int rc = plan_forward(p, prm, sc, with_loss || (p->target && loss_out));
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
