// Batched gradient for logistic-likelihood models that share one design
// matrix across all chains (logistic regression, regularised horseshoe).
//
// For C chains with coefficient rows B[c] = (b0, beta_1..K) the likelihood
// part of log_prob_grad is
//     eta[n,c] = b0_c + X[n,:] . beta_c                     (X . B^T)
//     lp_c    += sum_n y_n eta[n,c] - log1p_exp(eta[n,c])
//     r[n,c]   = y_n - inv_logit(eta[n,c])
//     grad_c   = (sum_n r[n,c], X^T r[:,c])                 (R^T . X)
// -- two contractions with an elementwise step between them, which is what
// Stan Math's reverse sweep over the bernoulli_logit / GLM node computes for
// one chain at a time (contract of log_prob_grad, src/cmdstan/
// command_helper.hpp:589-593).  The model-specific parts (coefficients from
// the unconstrained point, priors, Jacobians, chain rule to z / lambda / tau
// for the horseshoe) run per chain in stage_request / reduce_gradient.
//
// Row blocks are split over S CTAs per chain tile; each CTA writes its
// partial sums to [S][C] / [S][C][K+1] buffers which reduce_gradient sums in
// a fixed order, so results are bitwise reproducible run to run.
#pragma once
#include <cuda_bf16.h>
#include "device_models.cuh"

namespace gnuts {

struct GradOut {
  int kind;     // MK_LOGISTIC or MK_HORSESHOE
  int prec;     // GNUTS_PRECISION_*
  int C, K, S;  // chains, predictors, row splits
  int rows_per_split;
  double* coef64;   // [C][K+1]
  float* coef32;    // [C][K+1]
  double* part_lp;  // [S][C]
  double* part_g;   // [S][C][K+1] (SIMT path)
  float* part_g32;  // [S][C][TC_GSTRIDE] (tensor-core path: FP32 accumulators; position k < K is
                    // beta_k, position K the intercept, as the tensor-core columns are ordered)
  const int* done_count;
  int C_total;
  void* tc;           // tensor-core plan (grad_tc.cu), null for the SIMT path
  void* wide;         // tcgen05 plan for wide designs (grad_wide.cu), or null
  uint16_t* coef_bf;  // tensor-core operand: [2][Cpad][128] BF16 hi / lo planes
  int Cpad;
  double* lin;        // [C] tensor-core path: linear likelihood part (hi + lo) . xtc_ym
};

// Sum the S row-split partials of chain c in a fixed order (s = 0, 1, ...):
// FP32 sums for the mixed path, whose partials are FP32 tensor-memory
// accumulators, FP64 otherwise.  Thread l of the team owns coefficients l,
// l + TW, ...; the
// loads of 8 splits x SCH coefficients are issued together.  out[i] receives
// the sum for coefficient i (i <= K).
constexpr int SCH = 4;  // coefficients per lane per pass
template <class Acc, int TW = 32>
__device__ __forceinline__ void sum_splits(const GradOut& G, int c, double* out, int lane) {
  const int K1 = G.K + 1;
  const size_t stride = (size_t)G.C * K1;
  const double* src = G.part_g + (size_t)c * K1;
  for (int base = 0; base < K1; base += TW * SCH) {
    Acc acc[SCH];
#pragma unroll
    for (int j = 0; j < SCH; ++j) acc[j] = 0;
    for (int s0 = 0; s0 < G.S; s0 += 8) {
      double v[8][SCH];
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int j = 0; j < SCH; ++j) {
          const int i = base + lane + TW * j;
          v[u][j] = (s0 + u < G.S && i < K1) ? src[(size_t)(s0 + u) * stride + i] : 0.0;
        }
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int j = 0; j < SCH; ++j)
          if (s0 + u < G.S) acc[j] += (Acc)v[u][j];
    }
#pragma unroll
    for (int j = 0; j < SCH; ++j) {
      const int i = base + lane + TW * j;
      if (i < K1) out[i] = (double)acc[j];
    }
  }
}
// Tensor-core partials: lane l owns positions 4l .. 4l+3 and loads one
// 16-byte vector per split, all splits in flight at once, summed in split
// order in FP32 (the same values and order as the FP64-stored path).
// Position p < K is beta_p (out[1 + p]), position K the intercept (out[0]).
__device__ __forceinline__ void sum_splits_f32(const GradOut& G, int c, double* out, int lane) {
  const float4* src = reinterpret_cast<const float4*>(G.part_g32 + (size_t)c * TC_GSTRIDE) + lane;
  const size_t stride = (size_t)G.C * TC_GSTRIDE / 4;
  constexpr int SB = 16;  // splits loaded together
  float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int s0 = 0; s0 < G.S; s0 += SB) {
    float4 v[SB];
#pragma unroll
    for (int u = 0; u < SB; ++u)
      if (s0 + u < G.S) v[u] = src[(size_t)(s0 + u) * stride];
#pragma unroll
    for (int u = 0; u < SB; ++u)
      if (s0 + u < G.S) {
        a.x += v[u].x;
        a.y += v[u].y;
        a.z += v[u].z;
        a.w += v[u].w;
      }
  }
  const float av[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int p = 4 * lane + j;
    if (p < G.K) out[1 + p] = (double)av[j];
    else if (p == G.K) out[0] = (double)av[j];
  }
}

// lp partials of chain c summed in FP64, same order on every lane
__device__ __forceinline__ double sum_split_lp(const GradOut& G, int c) {
  double t = 0;
  for (int s0 = 0; s0 < G.S; s0 += 8) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = s0 + u < G.S ? G.part_lp[(size_t)(s0 + u) * G.C + c] : 0.0;
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (s0 + u < G.S) t += v[u];
  }
  return t;
}

inline bool batched_supported(const DevModel& M) {
  return M.kind == MK_LOGISTIC || M.kind == MK_HORSESHOE;
}

// ---------------------------------------------------------------- staging
// coefficient row of chain c from its unconstrained position q
template <int TW = 32>
__device__ __forceinline__ void stage_request(const GradOut& G, const DevModel& M, int c, const double* q,
                                              int lane) {
  const int K = M.K;
  double* o64 = G.coef64 + (size_t)c * (K + 1);
  float* o32 = G.coef32 ? G.coef32 + (size_t)c * (K + 1) : nullptr;
  if (M.kind == MK_LOGISTIC) {
    if (G.coef_bf) {
      // tensor-core operand: column k < K -> beta_k, column K -> intercept (it
      // meets the ones column of X), split v = hi + lo in BF16.  The kernel
      // sums only the even part of the likelihood; its linear part
      // sum_n (y_n - 1/2) eta_n = (hi + lo) . Xtc^T (y - 1/2) is formed here,
      // in FP64, for exactly the coefficients the kernel multiplies.
      __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(G.coef_bf) + (size_t)c * 128;
      __nv_bfloat16* lo = reinterpret_cast<__nv_bfloat16*>(G.coef_bf) + ((size_t)G.Cpad + c) * 128;
      double lin = 0;
      for (int i = lane; i < 128; i += TW) {
        double v = i < K ? q[1 + i] : (i == K ? q[0] : 0.0);
        __nv_bfloat16 h = __float2bfloat16_rn((float)v);
        __nv_bfloat16 l = __float2bfloat16_rn((float)(v - (double)__bfloat162float(h)));
        hi[i] = h;
        lo[i] = l;
        if (i < XTC_LD) lin += ((double)__bfloat162float(h) + (double)__bfloat162float(l)) * M.xtc_ym[i];
      }
      lin = tsum<TW>(lin);
      if (lane == 0) G.lin[c] = lin;
      return;
    }
    for (int i = lane; i <= K; i += TW) {
      double v = q[i];
      o64[i] = v;
      if (o32) o32[i] = (float)v;
    }
  } else {  // horseshoe: beta = z .* lambda_tilde * tau
    double tau = exp(q[K + 1]), caux = exp(q[2 * K + 2]);
    double c2 = M.slab_scale * M.slab_scale * caux;
    if (lane == 0) {
      o64[0] = q[0];
      if (o32) o32[0] = (float)q[0];
    }
    if (G.prec == GNUTS_PRECISION_MIXED) {
      // the coefficients feed a BF16 hi + lo split (16 significant bits):
      // FP32 per coefficient, in the overflow-safe form
      // lambda_tilde = sqrt(c2 / (c2 e + tau^2)) with e = 1 / lambda^2
      const float c2f = (float)c2, t2f = (float)(tau * tau), tf = (float)tau;
      for (int d = lane; d < K; d += TW) {
        const float e = expf(-2.0f * (float)q[K + 2 + d]);
        const float lamt = sqrtf(c2f / fmaf(c2f, e, t2f));
        const double b = (double)((float)q[1 + d] * lamt * tf);
        o64[1 + d] = b;
        if (o32) o32[1 + d] = (float)b;
      }
      return;
    }
    for (int d = lane; d < K; d += TW) {
      double lam = exp(q[K + 2 + d]);
      double l2 = lam * lam;
      double lamt = sqrt(c2 * l2 / (c2 + tau * tau * l2));
      double b = q[1 + d] * lamt * tau;
      o64[1 + d] = b;
      if (o32) o32[1 + d] = (float)b;
    }
  }
}

// reduce_gradient for the logistic model on the tensor-core path.  Every
// load of the step -- the split partials, the lp partials, the linear part
// and the chain's coefficients -- is issued before the arithmetic that needs
// them (one memory round trip where the general path below takes seven:
// its loops are ordered by stores the compiler must assume may alias).  The
// results are bitwise those of the general path: the split partials are
// summed in split order in FP32, the lp partials in split order in FP64 (one
// shuffle per split), and each prior term takes its likelihood gradient from
// the owning lane by shuffles instead of a store and reload.
__device__ __forceinline__ double reduce_logistic_tc(const GradOut& G, const DevModel& M, int c, const double* q,
                                                     double* g, int lane) {
  const int K = M.K, S = G.S;
  double qv[4];  // coefficient i = lane + 32 j (K + 1 <= 128)
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int i = lane + 32 * j;
    qv[j] = i <= K ? q[i] : 0.0;
  }
  const double lin = G.lin[c];
  const double lp0 = lane < S ? G.part_lp[(size_t)lane * G.C + c] : 0.0;  // splits 0..31, one per lane
  const float4* src = reinterpret_cast<const float4*>(G.part_g32 + (size_t)c * TC_GSTRIDE) + lane;
  const size_t stride = (size_t)G.C * TC_GSTRIDE / 4;
  constexpr int SB = 16;  // splits loaded together
  float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int s0 = 0; s0 < S; s0 += SB) {
    float4 v[SB];
#pragma unroll
    for (int u = 0; u < SB; ++u)
      if (s0 + u < S) v[u] = src[(size_t)(s0 + u) * stride];
#pragma unroll
    for (int u = 0; u < SB; ++u)
      if (s0 + u < S) {
        a.x += v[u].x;
        a.y += v[u].y;
        a.z += v[u].z;
        a.w += v[u].w;
      }
  }
  double lp = 0;
  for (int b = 0; b < S; b += 32) {
    const double v = b == 0 ? lp0 : (b + lane < S ? G.part_lp[(size_t)(b + lane) * G.C + c] : 0.0);
    const int n = min(32, S - b);
    for (int u = 0; u < n; ++u) lp += __shfl_sync(GN_FULL, v, u);
  }
  lp += lin;
  double pri = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    // coefficient i sits at position p = i - 1 (beta) or K (intercept), held by lane p / 4
    const int i = lane + 32 * j;
    const int pos = i == 0 ? K : i - 1;
    const int own = (pos >> 2) & 31;
    const float x0 = __shfl_sync(GN_FULL, a.x, own), x1 = __shfl_sync(GN_FULL, a.y, own);
    const float x2 = __shfl_sync(GN_FULL, a.z, own), x3 = __shfl_sync(GN_FULL, a.w, own);
    const int e = pos & 3;
    const double t = (double)(e == 0 ? x0 : e == 1 ? x1 : e == 2 ? x2 : x3);
    if (i <= K) {
      const double v = qv[j];
      if (i == 0) {
        g[0] = t - v / 6.25;
        pri += -0.5 * (v / 2.5) * (v / 2.5);
      } else {
        g[i] = t - v;
        pri += -0.5 * v * v;
      }
    }
  }
  return lp + wsum(pri);
}

// sum the partials of chain c, add priors / Jacobian, write grad, return lp
template <int TW = 32>
__device__ __forceinline__ double reduce_gradient(const GradOut& G, const DevModel& M, int c, const double* q,
                                                  double* g, int lane) {
  if constexpr (TW == 32) {
    if (G.part_g32 && G.lin && M.kind == MK_LOGISTIC && M.K + 1 <= 128) return reduce_logistic_tc(G, M, c, q, g, lane);
  }
  const int K = M.K;
  // likelihood gradient wrt (b0, beta) -> g[0..K]; priors added below
  if (G.part_g32) {
    if (TW == 32 || lane < 32) sum_splits_f32(G, c, g, lane);  // 32 lanes x 4 positions
  } else if (G.prec == GNUTS_PRECISION_FP64) {
    sum_splits<double, TW>(G, c, g, lane);
  } else {
    sum_splits<float, TW>(G, c, g, lane);
  }
  double lp = sum_split_lp(G, c);
  if (G.lin) lp += G.lin[c];
  tsync<TW>();
  const double* gs = g;
  if (M.kind == MK_LOGISTIC) {
    double pri = 0;
    for (int i = lane; i <= K; i += TW) {
      const double t = gs[i];
      double v = q[i];
      if (i == 0) {
        g[0] = t - v / 6.25;
        pri += -0.5 * (v / 2.5) * (v / 2.5);
      } else {
        g[i] = t - v;
        pri += -0.5 * v * v;
      }
    }
    return lp + tsum<TW>(pri);
  }
  // horseshoe
  const double nu = M.slab_df, ssl = M.slab_scale, sg = M.scale_global;
  double lt = q[K + 1], tau = exp(lt), lc = q[2 * K + 2], caux = exp(lc);
  double c2 = ssl * ssl * caux;
  double pri = 0, glt = 0, glc = 0;
  if (G.prec == GNUTS_PRECISION_MIXED) {
    // The chain rule through the per-coefficient transform in FP32 (its
    // input, the likelihood gradient, carries BF16 residual error), in forms
    // that stay finite wherever the FP32 exponentials do: with
    // e = 1 / lambda^2 and r = tau^2 lambda^2 / c2,
    //   a = c2 / (c2 + tau^2 lambda^2) = 1 / (1 + r),  bt = 1 - a = r / (1 + r),
    //   lambda_tilde = sqrt(c2 / (c2 e + tau^2)),  lambda^2 / (1 + lambda^2) = 1 / (1 + e),
    //   log1p(lambda^2) = 2 log(lambda) + log1p(e) (log lambda > 0), log1p(1 / e) otherwise.
    // The per-lane sums of the prior and of the tau / c chain-rule terms are FP64.
    const float c2f = (float)c2, t2f = (float)(tau * tau), tf = (float)tau;
    const float lrat = (float)(2.0 * lt - log(c2));
    for (int d = lane; d < K; d += TW) {
      const float t = (float)gs[1 + d];
      const float z = (float)q[1 + d];
      const float ll = (float)q[K + 2 + d];
      const float e = expf(-2.0f * ll);
      const float r = expf(fmaf(2.0f, ll, lrat));
      const float a = 1.0f / (1.0f + r);
      const float bt = r < 1.0f ? r * a : 1.0f - a;
      const float lamt = sqrtf(c2f / fmaf(c2f, e, t2f));
      const float gbd = t * (z * lamt * tf);
      const float l1p = ll > 0.0f ? fmaf(2.0f, ll, log1pf(e)) : log1pf(1.0f / e);
      pri += (double)(fmaf(-0.5f * z, z, ll) - l1p);
      g[1 + d] = (double)fmaf(t * lamt, tf, -z);
      g[K + 2 + d] = (double)(fmaf(gbd, a, 1.0f) - 2.0f / (1.0f + e));
      glt += (double)(gbd * a);  // 1 - bt
      glc += (double)(gbd * 0.5f * bt);
    }
  } else {
    for (int d = lane; d < K; d += TW) {
      const double t = gs[1 + d];
      double z = q[1 + d];
      double ll = q[K + 2 + d];
      double lam = exp(ll);
      double l2 = lam * lam;
      double den = c2 + tau * tau * l2;
      double a = c2 / den, bt = tau * tau * l2 / den;
      double lamt = sqrt(c2 * l2 / den);
      double beta = z * lamt * tau;
      double gbd = t * beta;
      pri += -0.5 * z * z - log1p(l2) + ll;
      g[1 + d] = t * lamt * tau - z;
      g[K + 2 + d] = gbd * a - 2.0 * l2 / (1.0 + l2) + 1.0;
      glt += gbd * (1.0 - bt);
      glc += gbd * 0.5 * bt;
    }
  }
  {
    double v3[3] = {pri, glt, glc};
    tsum_n<TW, 3>(v3);
    pri = v3[0];
    glt = v3[1];
    glc = v3[2];
  }
  double b0 = q[0];
  double ts = tau / sg;
  lp += pri - 0.5 * (b0 / 2.5) * (b0 / 2.5) - log1p(ts * ts) + (-0.5 * nu - 1.0) * lc - 0.5 * nu / caux + lt + lc;
  if (lane == 0) {
    g[0] = gs[0] - b0 / 6.25;
    g[K + 1] = glt - 2.0 * ts * ts / (1.0 + ts * ts) + 1.0;
    g[2 * K + 2] = glc + (-0.5 * nu - 1.0) + 0.5 * nu / caux + 1.0;
  }
  return lp;
}

// ---------------------------------------------------------------- SIMT contraction
// T = double (FP64 reference path) or float (FP32 CUDA-core path); the lp
// sum is always accumulated in FP64.
constexpr int GLM_CT = 16;   // chains per CTA
constexpr int GLM_RB = 16;   // rows per block
constexpr int GLM_KC = 128;  // predictor chunk
constexpr int GLM_THREADS = 256;
// NKC = predictor chunks held in registers: 1 for K <= 128, 8 for K <= 1024
template <class T, int NKC>
__global__ void __launch_bounds__(GLM_THREADS) k_glm_simt(GradOut G, DevModel M) {
  if (G.done_count && *G.done_count >= G.C_total) return;
  const int K = M.K;
  const int c0 = blockIdx.x * GLM_CT;
  const int split = blockIdx.y;
  const int row_begin = split * G.rows_per_split;
  const int row_end = min(M.N, row_begin + G.rows_per_split);
  const int t = threadIdx.x;
  const T* X = nullptr;
  if constexpr (sizeof(T) == 8) X = (const T*)M.X; else X = (const T*)M.Xf;
  const T* coef;
  if constexpr (sizeof(T) == 8) coef = (const T*)G.coef64; else coef = (const T*)G.coef32;

  __shared__ T xs[GLM_RB][GLM_KC + 1];
  __shared__ T cs[GLM_CT][GLM_KC + 1];
  __shared__ T rs[GLM_CT][GLM_RB];
  __shared__ double lps[GLM_THREADS];

  // eta / residual ownership: thread t -> (row t / CT, chain t % CT)
  const int er = t / GLM_CT, ec = t % GLM_CT;
  double lp_acc = 0;
  T gacc[NKC][GLM_CT];
#pragma unroll
  for (int j = 0; j < NKC; ++j)
#pragma unroll
    for (int c = 0; c < GLM_CT; ++c) gacc[j][c] = 0;
  T g0acc = 0;  // intercept gradient (thread ec handles chain ec when t < CT)
  const int nkc = min(NKC, (K + GLM_KC - 1) / GLM_KC);

  for (int r0 = row_begin; r0 < row_end; r0 += GLM_RB) {
    // ---- eta
    T eta = 0;
    for (int kc = 0; kc < nkc; ++kc) {
      const int k0 = kc * GLM_KC;
      __syncthreads();
      for (int i = t; i < GLM_RB * GLM_KC; i += GLM_THREADS) {
        int rr = i / GLM_KC, kk = i % GLM_KC;
        int n = r0 + rr, k = k0 + kk;
        xs[rr][kk] = (n < row_end && k < K) ? X[(size_t)n * K + k] : T(0);
      }
      for (int i = t; i < GLM_CT * GLM_KC; i += GLM_THREADS) {
        int cc = i / GLM_KC, kk = i % GLM_KC;
        int c = c0 + cc, k = k0 + kk;
        cs[cc][kk] = (c < G.C && k < K) ? coef[(size_t)c * (K + 1) + 1 + k] : T(0);
      }
      __syncthreads();
#pragma unroll 8
      for (int kk = 0; kk < GLM_KC; ++kk) eta += xs[er][kk] * cs[ec][kk];
    }
    {
      const int n = r0 + er, c = c0 + ec;
      T r = 0;
      if (n < row_end && c < G.C) {
        const int y = M.yi[n];
        if constexpr (sizeof(T) == 8) {
          double e = eta + coef[(size_t)c * (K + 1)];
          lp_acc += y * e - log1p_exp(e);
          r = y - inv_logit(e);
        } else {
          // FP32 elementwise step (FP64 is scarce on this part); the sum stays FP64
          float e = eta + coef[(size_t)c * (K + 1)];
          float ax = fabsf(e);
          float l1p = log1pf(__expf(-ax));            // log1p(exp(-|e|))
          float term = (y ? fminf(e, 0.f) : -fmaxf(e, 0.f)) - l1p;  // y e - log1p_exp(e)
          lp_acc += (double)term;
          float s = 1.f / (1.f + __expf(-ax));         // inv_logit(|e|)
          float il = e >= 0.f ? s : 1.f - s;
          r = (float)y - il;
        }
      }
      rs[ec][er] = r;
    }
    __syncthreads();
    if (t < GLM_CT) {
#pragma unroll
      for (int rr = 0; rr < GLM_RB; ++rr) g0acc += rs[t][rr];
    }
    // ---- gradient: thread t owns predictor k = kc*KC + t (t < KC)
#pragma unroll
    for (int kc = 0; kc < NKC; ++kc) {
      if (kc >= nkc) break;
      const int k0 = kc * GLM_KC;
      if (nkc > 1) {
        __syncthreads();
        for (int i = t; i < GLM_RB * GLM_KC; i += GLM_THREADS) {
          int rr = i / GLM_KC, kk = i % GLM_KC;
          int n = r0 + rr, k = k0 + kk;
          xs[rr][kk] = (n < row_end && k < K) ? X[(size_t)n * K + k] : T(0);
        }
        __syncthreads();
      }
      if (t < GLM_KC) {
#pragma unroll
        for (int rr = 0; rr < GLM_RB; ++rr) {
          T x = xs[rr][t];
#pragma unroll
          for (int c = 0; c < GLM_CT; ++c) gacc[kc][c] += rs[c][rr] * x;
        }
      }
    }
    __syncthreads();
  }
  // ---- write partials
  lps[t] = lp_acc;
  __syncthreads();
  if (t < GLM_CT) {
    double s = 0;
    for (int rr = 0; rr < GLM_RB; ++rr) s += lps[rr * GLM_CT + t];
    int c = c0 + t;
    if (c < G.C) {
      G.part_lp[(size_t)split * G.C + c] = s;
      G.part_g[((size_t)split * G.C + c) * (K + 1)] = (double)g0acc;
    }
  }
  if (t < GLM_KC) {
    for (int kc = 0; kc < nkc; ++kc) {
      int k = kc * GLM_KC + t;
      if (k >= K) continue;
      for (int cc = 0; cc < GLM_CT; ++cc) {
        int c = c0 + cc;
        if (c < G.C) G.part_g[((size_t)split * G.C + c) * (K + 1) + 1 + k] = (double)gacc[kc][cc];
      }
    }
  }
}

}  // namespace gnuts
