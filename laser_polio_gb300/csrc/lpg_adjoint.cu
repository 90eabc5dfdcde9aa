/*
 * lpg_adjoint.cu — expected incidence of a tick range and its
 * vector-Jacobian product (the C ABI lpg_expected_incidence in lpg.h).
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
 * gravity flows k p_i^a p_j^b / d_ij^c (zero diagonal).
 *
 * Everything is double precision.  The two contractions, u = N^T beta per
 * (t, s) and dL/dN = beta^T dL/du, are (T S) x G x G products done by one
 * shared-memory tiled kernel; the rest is elementwise work and per-row or
 * per-tick reductions.  The sums use atomics, so results agree with a
 * sequential evaluation to rounding, not bit for bit.
 */
#include <cuda_runtime.h>

#include <cmath>

#include "lpg.h"

/* Per-host-thread error text of the standalone ops (lpg_ops.cu). */
int lpg_ops_fail(int code, const char* fmt, ...);

namespace {

#define ICK(call)                                                                                        \
  do {                                                                                                   \
    cudaError_t e_ = (call);                                                                             \
    if (e_ != cudaSuccess) {                                                                             \
      rc = lpg_ops_fail(LPG_ERR_CUDA, "expected_incidence: %s: %s", #call, cudaGetErrorString(e_)); \
      goto done;                                                                                         \
    }                                                                                                    \
  } while (0)

constexpr double kTwoPi = 6.283185307179586476925286766559;
#define INC_TILE 32

/* One row i per CTA: the scaled gravity flows G[i,j] = k p_i^a p_j^b /
 * d_ij^c / P^c (zero diagonal), their sum rs[i], and the normalised row
 * N[i,j] (scaled down to max_frac when rs[i] exceeds it) with its sum. */
__global__ void k_inc_network(int G, const double* pops, const double* dist, double k, double a, double b, double c,
                              double Pc, double max_frac, double* Gm, double* N, double* rs, double* rsN,
                              int* capped) {
  __shared__ double s_part[256];
  const int i = blockIdx.x;
  if (i >= G) return;
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
  s_part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s_part[threadIdx.x] += s_part[threadIdx.x + o];
    __syncthreads();
  }
  const double r = s_part[0];
  const bool cap = r > max_frac;
  __syncthreads();
  double sumN = 0.0;
  for (int j = threadIdx.x; j < G; j += blockDim.x) {
    const double v = Gm[(size_t)i * G + j];
    const double nv = cap ? v * (max_frac / r) : v;
    N[(size_t)i * G + j] = nv;
    sumN += nv;
  }
  s_part[threadIdx.x] = sumN;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s_part[threadIdx.x] += s_part[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    rs[i] = r;
    rsN[i] = s_part[0];
    capped[i] = cap ? 1 : 0;
  }
}

/* C[m][n] = sum_k A(m, k) B(k, n) over 32 x 32 tiles in shared memory,
 * MODE 0: the mixing, m = (t, s), A(m, i) = beta[t][i][s], B(i, n) = N[i][n],
 *         C = u[t][n][s] (M = T S, K = G, N = G);
 * MODE 1: dL/dN before its diagonal term, C[a][b] = sum_m beta(m, a) gu(m, b)
 *         with m = (t, s) (M = G, K = T S, N = G). */
template <int MODE>
__global__ void k_inc_gemm(int T, int G, int S, const double* beta, const double* B2, double* C) {
  __shared__ double sA[INC_TILE][INC_TILE + 1];
  __shared__ double sB[INC_TILE][INC_TILE + 1];
  const int Mdim = MODE == 0 ? T * S : G, Kdim = MODE == 0 ? G : T * S;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int row = blockIdx.y * INC_TILE + ty, col = blockIdx.x * INC_TILE + tx;
  double acc = 0.0;
  for (int k0 = 0; k0 < Kdim; k0 += INC_TILE) {
    /* A tile: rows blockIdx.y*32 + ty, columns k0 + tx */
    {
      const int m = blockIdx.y * INC_TILE + ty, kk = k0 + tx;
      double v = 0.0;
      if (m < Mdim && kk < Kdim) {
        if (MODE == 0) {
          const int t = m / S, s = m % S;
          v = beta[((size_t)t * G + kk) * S + s];
        } else {
          const int t = kk / S, s = kk % S;
          v = beta[((size_t)t * G + m) * S + s];
        }
      }
      sA[ty][tx] = v;
    }
    /* B tile: rows k0 + ty, columns blockIdx.x*32 + tx */
    {
      const int kk = k0 + ty, n = blockIdx.x * INC_TILE + tx;
      double v = 0.0;
      if (kk < Kdim && n < G) {
        if (MODE == 0) {
          v = B2[(size_t)kk * G + n];
        } else {
          const int t = kk / S, s = kk % S;
          v = B2[((size_t)t * G + n) * S + s];
        }
      }
      sB[ty][tx] = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int q = 0; q < INC_TILE; ++q) acc = fma(sA[ty][q], sB[q][tx], acc); /* fused even under --fmad=false */
    __syncthreads();
  }
  if (row < Mdim && col < G) {
    if (MODE == 0) {
      const int t = row / S, s = row % S;
      C[((size_t)t * G + col) * S + s] = acc;
    } else {
      C[(size_t)row * G + col] = acc;
    }
  }
}

struct IncScalars {
  double R, amp, peak;
};

/* Per (t, n): the mixing's diagonal term, the rates, exp(-r) kept for the
 * reverse pass, and lam. */
__global__ void k_inc_forward(int T, int G, int S, const double* srisk, const double* beta, const double* pop,
                              const double* doy, const double* year, const double* r0s, const double* rsN,
                              IncScalars sc, double* u, double* e, double* lam) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)T * G) return;
  const int t = (int)(idx / G), n = (int)(idx % G);
  const double ang = kTwoPi * (doy[t] - sc.peak) / year[t];
  const double seas = 1.0 + sc.amp * cos(ang);
  const double q = seas * r0s[n] * sc.R / fmax(pop[idx], 1.0);
  double l = 0.0;
  for (int s = 0; s < S; ++s) {
    const size_t k = idx * S + s;
    const double uu = u[k] + beta[k] * (1.0 - rsN[n]);
    u[k] = uu;
    const double ex = exp(-(uu * q));
    e[k] = ex;
    l += 1.0 - ex;
  }
  lam[idx] = srisk[idx] * l;
}

/* Per (t, n) of the reverse pass: dL/du (kept for the dL/dN product) and
 * the contributions to dL/dseas[t], dL/dr0s[n] and dL/dR. */
__global__ void k_inc_backward(int T, int G, int S, const double* g, const double* srisk, const double* pop,
                               const double* doy, const double* year, const double* r0s, IncScalars sc,
                               const double* u, const double* e, double* gu, double* g_seas, double* g_r0s,
                               double* g_R) {
  __shared__ double s_R[256];
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double cR = 0.0;
  if (idx < (size_t)T * G) {
    const int t = (int)(idx / G), n = (int)(idx % G);
    const double ang = kTwoPi * (doy[t] - sc.peak) / year[t];
    const double seas = 1.0 + sc.amp * cos(ang);
    const double popc = fmax(pop[idx], 1.0);
    const double q = seas * r0s[n] * sc.R / popc;
    const double gs = g[idx] * srisk[idx];
    double gq = 0.0;
    for (int s = 0; s < S; ++s) {
      const size_t k = idx * S + s;
      const double gr = gs * e[k];
      gu[k] = gr * q;
      gq += gr * u[k];
    }
    atomicAdd(&g_seas[t], gq * r0s[n] * sc.R / popc);
    atomicAdd(&g_r0s[n], gq * seas * sc.R / popc);
    cR = gq * seas * r0s[n] / popc;
  }
  s_R[threadIdx.x] = cR;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s_R[threadIdx.x] += s_R[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(g_R, s_R[0]);
}

/* dL/damp and dL/dpeak from dL/dseas[t] (one CTA). */
__global__ void k_inc_seasonal(int T, const double* doy, const double* year, const double* g_seas, IncScalars sc,
                               double* out) {
  __shared__ double s_a[256], s_p[256];
  double ga = 0.0, gp = 0.0;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const double ang = kTwoPi * (doy[t] - sc.peak) / year[t];
    ga += g_seas[t] * cos(ang);
    gp += g_seas[t] * sc.amp * sin(ang) * kTwoPi / year[t];
  }
  s_a[threadIdx.x] = ga;
  s_p[threadIdx.x] = gp;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s_a[threadIdx.x] += s_a[threadIdx.x + o];
      s_p[threadIdx.x] += s_p[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s_a[0];
    out[1] = s_p[0];
  }
}

/* One row a per CTA: dL/dN[a][b] = C[a][b] - C[a][a] (zero on the
 * diagonal), then dL/dG through the row normalisation and the row's
 * contributions to dL/dk, dL/da, dL/db, dL/dc. */
__global__ void k_inc_network_grad(int G, const double* C, const double* Gm, const double* rs, const int* capped,
                                   const double* pops, const double* dist, double k, double logP, double max_frac,
                                   double* gN, double* g_theta) {
  __shared__ double s_red[4][256];
  const int a = blockIdx.x;
  if (a >= G) return;
  const double diag = C[(size_t)a * G + a];
  /* the row's sum of dL/dN * G (the normalisation's coupling term) */
  double cpl = 0.0;
  for (int b = threadIdx.x; b < G; b += blockDim.x) {
    const double v = b == a ? 0.0 : C[(size_t)a * G + b] - diag;
    gN[(size_t)a * G + b] = v;
    cpl += v * Gm[(size_t)a * G + b];
  }
  s_red[0][threadIdx.x] = cpl;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s_red[0][threadIdx.x] += s_red[0][threadIdx.x + o];
    __syncthreads();
  }
  const double coupling = s_red[0][0];
  const bool cap = capped[a] != 0;
  const double ra = rs[a];
  __syncthreads();
  const double lpa = log(pops[a]);
  double wk = 0.0, wa = 0.0, wb = 0.0, wc = 0.0;
  for (int b = threadIdx.x; b < G; b += blockDim.x) {
    if (b == a) continue;
    const double gn = gN[(size_t)a * G + b];
    const double gg = cap ? (max_frac / ra) * (gn - coupling / ra) : gn;
    const double w = gg * Gm[(size_t)a * G + b];
    if (w == 0.0) continue; /* a zero flow: its logs may be infinite */
    wk += w;
    wa += w * lpa;
    wb += w * log(pops[b]);
    const double d = dist[(size_t)a * G + b];
    wc += w * (-log(d) - logP);
  }
  s_red[0][threadIdx.x] = wk;
  s_red[1][threadIdx.x] = wa;
  s_red[2][threadIdx.x] = wb;
  s_red[3][threadIdx.x] = wc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int q = 0; q < 4; ++q) s_red[q][threadIdx.x] += s_red[q][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(&g_theta[0], s_red[0][0] / k);
    atomicAdd(&g_theta[1], s_red[1][0]);
    atomicAdd(&g_theta[2], s_red[2][0]);
    atomicAdd(&g_theta[3], s_red[3][0]);
  }
}

template <typename T>
int dmalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, sizeof(T) * (n ? n : 1)) == cudaSuccess ? 0 : 1;
}

}  // namespace

extern "C" int lpg_expected_incidence(const lpg_incidence_in* in, double* lam_out, const double* g_lam,
                                      lpg_incidence_grad* grad_out, void* stream) {
  if (!in || !lam_out) return lpg_ops_fail(LPG_ERR_ARG, "expected_incidence: null argument");
  const int T = in->T, G = in->G, S = in->S;
  if (T <= 0 || G <= 0 || S <= 0 || S > LPG_MAX_STRAINS)
    return lpg_ops_fail(LPG_ERR_ARG, "expected_incidence: bad sizes T=%d G=%d S=%d", T, G, S);
  if ((int64_t)T * S > 65535LL * INC_TILE)
    return lpg_ops_fail(LPG_ERR_ARG, "expected_incidence: T*S = %lld above %d", (long long)T * S, 65535 * INC_TILE);
  if (!in->srisk || !in->beta || !in->pop || !in->doy || !in->year || !in->r0s || !in->pops || !in->dist)
    return lpg_ops_fail(LPG_ERR_ARG, "expected_incidence: null input array");
  if (g_lam && !grad_out) return lpg_ops_fail(LPG_ERR_ARG, "expected_incidence: a gradient needs grad_out");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t TG = (size_t)T * G, TGS = TG * S, GG = (size_t)G * G;
  double P = 0.0;
  for (int i = 0; i < G; ++i) P += in->pops[i];
  const double Pc = pow(P, in->c), logP = log(P);
  IncScalars sc{in->R, in->amp, in->peak};
  double *d_srisk = nullptr, *d_beta = nullptr, *d_pop = nullptr, *d_doy = nullptr, *d_year = nullptr,
         *d_r0s = nullptr, *d_pops = nullptr, *d_dist = nullptr, *d_G = nullptr, *d_N = nullptr, *d_rs = nullptr,
         *d_rsN = nullptr, *d_u = nullptr, *d_e = nullptr, *d_lam = nullptr, *d_g = nullptr, *d_gu = nullptr,
         *d_gseas = nullptr, *d_gr0s = nullptr, *d_scal = nullptr, *d_C = nullptr, *d_gN = nullptr;
  int* d_cap = nullptr;
  int rc = LPG_OK;
  if (dmalloc(&d_srisk, TG) || dmalloc(&d_beta, TGS) || dmalloc(&d_pop, TG) || dmalloc(&d_doy, T) ||
      dmalloc(&d_year, T) || dmalloc(&d_r0s, G) || dmalloc(&d_pops, G) || dmalloc(&d_dist, GG) ||
      dmalloc(&d_G, GG) || dmalloc(&d_N, GG) || dmalloc(&d_rs, G) || dmalloc(&d_rsN, G) || dmalloc(&d_cap, G) ||
      dmalloc(&d_u, TGS) || dmalloc(&d_e, TGS) || dmalloc(&d_lam, TG)) {
    rc = lpg_ops_fail(LPG_ERR_NOMEM, "expected_incidence: device allocation failed");
    goto done;
  }
  ICK(cudaMemcpyAsync(d_srisk, in->srisk, sizeof(double) * TG, cudaMemcpyHostToDevice, st));
  ICK(cudaMemcpyAsync(d_beta, in->beta, sizeof(double) * TGS, cudaMemcpyHostToDevice, st));
  ICK(cudaMemcpyAsync(d_pop, in->pop, sizeof(double) * TG, cudaMemcpyHostToDevice, st));
  ICK(cudaMemcpyAsync(d_doy, in->doy, sizeof(double) * T, cudaMemcpyHostToDevice, st));
  ICK(cudaMemcpyAsync(d_year, in->year, sizeof(double) * T, cudaMemcpyHostToDevice, st));
  ICK(cudaMemcpyAsync(d_r0s, in->r0s, sizeof(double) * G, cudaMemcpyHostToDevice, st));
  ICK(cudaMemcpyAsync(d_pops, in->pops, sizeof(double) * G, cudaMemcpyHostToDevice, st));
  ICK(cudaMemcpyAsync(d_dist, in->dist, sizeof(double) * GG, cudaMemcpyHostToDevice, st));
  k_inc_network<<<G, 256, 0, st>>>(G, d_pops, d_dist, in->k, in->a, in->b, in->c, Pc, in->max_frac, d_G, d_N, d_rs,
                                   d_rsN, d_cap);
  {
    const dim3 blk(INC_TILE, INC_TILE), grd((G + INC_TILE - 1) / INC_TILE, (T * S + INC_TILE - 1) / INC_TILE);
    k_inc_gemm<0><<<grd, blk, 0, st>>>(T, G, S, d_beta, d_N, d_u);
  }
  k_inc_forward<<<(unsigned)((TG + 255) / 256), 256, 0, st>>>(T, G, S, d_srisk, d_beta, d_pop, d_doy, d_year, d_r0s,
                                                              d_rsN, sc, d_u, d_e, d_lam);
  ICK(cudaGetLastError());
  ICK(cudaMemcpyAsync(lam_out, d_lam, sizeof(double) * TG, cudaMemcpyDeviceToHost, st));
  if (g_lam) {
    if (dmalloc(&d_g, TG) || dmalloc(&d_gu, TGS) || dmalloc(&d_gseas, T) || dmalloc(&d_gr0s, G) ||
        dmalloc(&d_scal, 8) || dmalloc(&d_C, GG) || dmalloc(&d_gN, GG)) {
      rc = lpg_ops_fail(LPG_ERR_NOMEM, "expected_incidence: device allocation failed");
      goto done;
    }
    ICK(cudaMemcpyAsync(d_g, g_lam, sizeof(double) * TG, cudaMemcpyHostToDevice, st));
    ICK(cudaMemsetAsync(d_gseas, 0, sizeof(double) * T, st));
    ICK(cudaMemsetAsync(d_gr0s, 0, sizeof(double) * G, st));
    ICK(cudaMemsetAsync(d_scal, 0, sizeof(double) * 8, st));
    /* d_scal: [0] R, [1] amp, [2] peak, [3..6] k, a, b, c */
    k_inc_backward<<<(unsigned)((TG + 255) / 256), 256, 0, st>>>(T, G, S, d_g, d_srisk, d_pop, d_doy, d_year,
                                                                 d_r0s, sc, d_u, d_e, d_gu, d_gseas, d_gr0s,
                                                                 d_scal);
    k_inc_seasonal<<<1, 256, 0, st>>>(T, d_doy, d_year, d_gseas, sc, d_scal + 1);
    {
      const dim3 blk(INC_TILE, INC_TILE), grd((G + INC_TILE - 1) / INC_TILE, (G + INC_TILE - 1) / INC_TILE);
      k_inc_gemm<1><<<grd, blk, 0, st>>>(T, G, S, d_beta, d_gu, d_C);
    }
    k_inc_network_grad<<<G, 256, 0, st>>>(G, d_C, d_G, d_rs, d_cap, d_pops, d_dist, in->k, logP, in->max_frac, d_gN,
                                          d_scal + 3);
    ICK(cudaGetLastError());
    double h_scal[8];
    ICK(cudaMemcpyAsync(h_scal, d_scal, sizeof(h_scal), cudaMemcpyDeviceToHost, st));
    if (grad_out->r0s) ICK(cudaMemcpyAsync(grad_out->r0s, d_gr0s, sizeof(double) * G, cudaMemcpyDeviceToHost, st));
    if (grad_out->network) ICK(cudaMemcpyAsync(grad_out->network, d_gN, sizeof(double) * GG, cudaMemcpyDeviceToHost, st));
    ICK(cudaStreamSynchronize(st));
    grad_out->R = h_scal[0];
    grad_out->amp = h_scal[1];
    grad_out->peak = h_scal[2];
    grad_out->k = h_scal[3];
    grad_out->a = h_scal[4];
    grad_out->b = h_scal[5];
    grad_out->c = h_scal[6];
  }
  ICK(cudaStreamSynchronize(st));
done:
  {
    void* ps[] = {d_srisk, d_beta, d_pop, d_doy, d_year, d_r0s, d_pops, d_dist, d_G, d_N, d_rs, d_rsN, d_cap,
                  d_u, d_e, d_lam, d_g, d_gu, d_gseas, d_gr0s, d_scal, d_C, d_gN};
    for (void* p : ps)
      if (p) cudaFree(p);
  }
  return rc;
}
