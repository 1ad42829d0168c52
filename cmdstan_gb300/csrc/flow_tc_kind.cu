// The learned sampler's gradient pass on the tensor cores, and the fused
// flow sampler built on it (NUTS in the pulled-back space: the state machine
// of stan::services::sample::hmc_nuts_diag_e_adapt's sampler, reached from
// src/cmdstan/command.hpp:673-688, with the model's log_prob_grad contract,
// command_helper.hpp:589-593, evaluated at x = T(z)).  The map and the
// weight layouts are described in flow.cuh.
//
// This file is compiled once per model kind (-DGNUTS_KIND=k), so that each
// kernel carries only its own model's gradient code; flow.cu dispatches.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "internal.h"
#include "flow.cuh"
#include "nuts_device.cuh"

#ifndef GNUTS_KIND
#error "compile with -DGNUTS_KIND=<model kind>"
#endif

namespace gnuts {

// ---------------------------------------------------------------- tensor-core gradient pass
// The sampler's gradient pass with the flow's four per-layer contractions on
// the tensor cores (mma.sync m16n8k16, BF16 operands, FP32 accumulation):
// the layer's weights are the A operand (rows = outputs, tensor-core layout
// of w16t staged in shared memory), the CTA's T <= 8 points are the columns
// of B.  Each activation is stored as three BF16 parts (hi + mid + lo, 24
// significant bits in all) when it is produced; the three products go to
// three FP32 accumulators, so the contraction carries FP32 accuracy on the
// exact BF16 weights.  The elementwise steps (tanh, clamp, exp, coupling
// update, log-determinant) are FP32 per point; the model at x is FP64.  With
// at most 8 m-tiles and N = 8 these contractions are latency-bound: the
// warp-level mma keeps them in registers with no tensor-memory round trip.
__device__ __forceinline__ void tc_mma(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
// v as hi + mid + lo BF16 parts at p, p + pls, p + 2 pls (|v - sum| <= 2^-24 |v|)
__device__ __forceinline__ void tc_put3(__nv_bfloat16* p, int pls, float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  const float r = v - __bfloat162float(h);
  const __nv_bfloat16 m = __float2bfloat16_rn(r);
  p[0] = h;
  p[pls] = m;
  p[2 * pls] = __float2bfloat16_rn(r - __bfloat162float(m));
}
__device__ __forceinline__ float tc_get3(const __nv_bfloat16* p, int pls) {
  return __bfloat162float(p[0]) + (__bfloat162float(p[pls]) + __bfloat162float(p[2 * pls]));
}

// C[m][n] = sum_k A[m][k] b_n[k] for m < 16 mtiles, n < T, k < 16 ksteps.
// A: BF16 row-major, row stride lda (shared memory).  b_n: the three parts
// of point n's vector at Bp + q * pls + n * ps (q = 0, 1, 2).  Warp w takes
// m-tiles w, w + W, ...; epi(m, n, c) receives every element with n < T.
template <int W, class Epi>
__device__ __forceinline__ void tc_gemm(const __nv_bfloat16* A, int lda, int mtiles, int ksteps,
                                        const __nv_bfloat16* Bp, int ps, int pls, int T, int warp, int lane,
                                        Epi epi) {
  constexpr int MPW = (8 + W - 1) / W;  // at most 8 m-tiles: H <= 128, 2 n_a <= 128, n_b <= 64
  const int g = lane >> 2, t = lane & 3;
  float acc[MPW][3][4];
#pragma unroll
  for (int i = 0; i < MPW; ++i)
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][q][j] = 0.f;
  const bool bon = g < T;
  const __nv_bfloat16* bp = Bp + (size_t)g * ps + 2 * t;
  if (warp < mtiles) {
    for (int ks = 0; ks < ksteps; ++ks) {
      const int k0 = 16 * ks;
      uint32_t b[3][2];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        b[q][0] = bon ? *reinterpret_cast<const uint32_t*>(bp + (size_t)q * pls + k0) : 0u;
        b[q][1] = bon ? *reinterpret_cast<const uint32_t*>(bp + (size_t)q * pls + k0 + 8) : 0u;
      }
#pragma unroll
      for (int i = 0; i < MPW; ++i) {
        const int mt = warp + i * W;
        if (mt < mtiles) {
          const __nv_bfloat16* ap = A + (size_t)(16 * mt + g) * lda + k0 + 2 * t;
          uint32_t a[4];
          a[0] = *reinterpret_cast<const uint32_t*>(ap);
          a[1] = *reinterpret_cast<const uint32_t*>(ap + 8 * (size_t)lda);
          a[2] = *reinterpret_cast<const uint32_t*>(ap + 8);
          a[3] = *reinterpret_cast<const uint32_t*>(ap + 8 * (size_t)lda + 8);
#pragma unroll
          for (int q = 0; q < 3; ++q) tc_mma(acc[i][q], a, b[q][0], b[q][1]);
        }
      }
    }
  }
#pragma unroll
  for (int i = 0; i < MPW; ++i) {
    const int mt = warp + i * W;
    if (mt < mtiles) {
      const int m0 = 16 * mt + g, n0 = 2 * t;
      float c[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) c[j] = acc[i][0][j] + (acc[i][1][j] + acc[i][2][j]);
      if (n0 < T) {
        epi(m0, n0, c[0]);
        epi(m0 + 8, n0, c[2]);
      }
      if (n0 + 1 < T) {
        epi(m0, n0 + 1, c[1]);
        epi(m0 + 8, n0 + 1, c[3]);
      }
    }
  }
}

// stage s < L: forward block of layer s; s >= L: adjoint block of layer 2L-1-s
__device__ __forceinline__ void issue_stage_tc(const FlowDev& F, int s, __nv_bfloat16* buf) {
  const int l = s < F.L ? s : 2 * F.L - 1 - s;
  const long fw = tc_fwd_elems(F.H, F.nb[l], F.na[l]);
  const __nv_bfloat16* src = F.w16t + F.wt_off[l] + (s < F.L ? 0 : fw);
  const long n = s < F.L ? fw : tc_adj_elems(F.H, F.nb[l], F.na[l]);
  const int chunks = (int)(n / 8);
  for (int i = threadIdx.x; i < chunks; i += blockDim.x) fl_cp16(buf + 8 * (size_t)i, src + 8 * (size_t)i);
}

// the pass's shared memory
struct TcSmem {
  int* sidx;
  __nv_bfloat16 *wbuf0, *wbuf1;
  double* sig;      // exp(rho)
  float* regions;   // [T][pr]
  __nv_bfloat16 *ub, *rb, *pb, *hb;
};
__device__ __forceinline__ TcSmem tc_smem(const FlowDev& F, const FlowTcLayout& Lo, unsigned char* fsm) {
  TcSmem t;
  const size_t idx_bytes = flow_align16(sizeof(int) * (size_t)F.L * F.d);
  const size_t wb = flow_align16(2 * (size_t)F.stage_max_tc);
  t.sidx = reinterpret_cast<int*>(fsm);
  t.wbuf0 = reinterpret_cast<__nv_bfloat16*>(fsm + idx_bytes);
  t.wbuf1 = reinterpret_cast<__nv_bfloat16*>(fsm + idx_bytes + wb);
  float* area = reinterpret_cast<float*>(fsm + idx_bytes + 2 * wb);
  __nv_bfloat16* ab = reinterpret_cast<__nv_bfloat16*>(area);
  t.sig = reinterpret_cast<double*>(area + Lo.o_sig);
  t.regions = area + Lo.o_regions;
  t.ub = ab + Lo.o_ub;
  t.rb = ab + Lo.o_rb;
  t.pb = ab + Lo.o_pb;
  t.hb = ab + Lo.o_hb;
  return t;
}

// per-launch setup: index table and exp(rho); returns sum(rho)
__device__ __forceinline__ double tc_setup(const FlowDev& F, const TcSmem S) {
  for (int i = threadIdx.x; i < F.L * F.d; i += blockDim.x) S.sidx[i] = F.idx[i];
  const float* rho = F.theta + F.th_rho;
  double sr = 0;
  for (int i = 0; i < F.d; ++i) sr += (double)rho[i];
  for (int i = threadIdx.x; i < F.d; i += blockDim.x) S.sig[i] = exp((double)rho[i]);
  return sr;
}

// layer l's conditioner inputs u_b of point n as BF16 parts (zero up to kb)
__device__ __forceinline__ void tc_gather_ub(const FlowDev& F, const FlowTcLayout& Lo, const TcSmem S, int l,
                                             const int* bi, const float* y, int n, int lane) {
  const int nb = F.nb[l], kb = tc_pad16(nb), pls = Lo.T * Lo.ub_stride;
  __nv_bfloat16* u = S.ub + (size_t)n * Lo.ub_stride;
  for (int r = lane; r < kb; r += 32) tc_put3(u + r, pls, r < nb ? y[bi[r]] : 0.f);
}

// One gradient pass for the CTA's T points (point n is warp n's; warps
// n >= T and points with live == false only take part in the contractions
// and barriers).  Input z (FP64, d values, the warp's chain), output g (FP64
// gradient in z); returns lp_x(T(z)) + log|det| to the point's warp.
template <int W, int KIND>
__device__ __forceinline__ double flow_grad_pass_tc(const FlowDev& F, const FlowTcLayout& Lo, const DevModel& M,
                                                    const TcSmem S, double sum_rho, bool live, const double* z,
                                                    double* g) {
  const int d = F.d, H = F.H, L = F.L, pr = Lo.pr, T = Lo.T;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool mine = warp < T && live;  // this warp owns live point `warp`
  float* R = S.regions + (size_t)warp * pr;
  float* y = R + Lo.o_y;
  float* yb = R + Lo.o_yb;
  const int pls_rb = T * Lo.rb_stride, pls_pb = T * Lo.pb_stride;
  issue_stage_tc(F, 0, S.wbuf0);
  fl_commit();
  float ld = 0.f;
  double lp = 0;
  if (mine) {
    for (int i = lane; i < d; i += 32) y[i] = (float)z[i];
    __syncwarp();
    tc_gather_ub(F, Lo, S, 0, S.sidx, y, warp, lane);
  }
  const int Sg = 2 * L;
  for (int st = 0; st < Sg; ++st) {
    if (st + 1 < Sg) {
      issue_stage_tc(F, st + 1, (st + 1) & 1 ? S.wbuf1 : S.wbuf0);
      fl_commit();
      fl_wait<1>();
    } else {
      fl_wait<0>();
    }
    const __nv_bfloat16* buf = st & 1 ? S.wbuf1 : S.wbuf0;
    const int l = st < L ? st : 2 * L - 1 - st;
    const int nb = F.nb[l], na = F.na[l], n2 = 2 * na;
    const int kb = tc_pad16(nb), ma = tc_pad16(n2);
    const int* bi = S.sidx + l * d;
    const int* ai = bi + nb;
    float* h_all = S.regions + Lo.o_h + l * Lo.h_stride;  // point n's FP32 h row: + n * pr
    const float* b1 = F.theta + F.th_off[l] + (long)nb * H;
    const float* b2 = b1 + H + (long)H * n2;
    if (st >= L && mine) {
      if (st == L) {
        // x = mu + exp(rho) u_L, the model at x, the adjoint seed
        double* x = reinterpret_cast<double*>(R + Lo.o_x);
        double* gx = reinterpret_cast<double*>(R + Lo.o_gx);
        const float* mu = F.theta + F.th_off[L];
        for (int i = lane; i < d; i += 32) x[i] = (double)mu[i] + S.sig[i] * (double)y[i];
        __syncwarp();
        const double lpx = warp_lpg_k<KIND>(M, x, gx, 1, lane);
        __syncwarp();
        lp = lpx + wsum((double)ld) + sum_rho;
        for (int i = lane; i < d; i += 32) yb[i] = (float)(gx[i] * S.sig[i]);
        __syncwarp();
      }
      // adjoint of the coupling update: output adjoints as BF16 parts (zero to ma)
      const float* ts = R + Lo.o_s + l * Lo.s_stride;
      const float* tua = R + Lo.o_ua + l * Lo.s_stride;
      __nv_bfloat16* rb = S.rb + (size_t)warp * Lo.rb_stride;
      const float cl = F.clamp;
      for (int m = lane; m < na; m += 32) {
        const int a = ai[m];
        const float s = ts[m], es = expf(s), gy = yb[a];
        const float q = s / cl;
        tc_put3(rb + m, pls_rb, fmaf(gy * tua[m], es, 1.0f) * (1.0f - q * q));
        tc_put3(rb + na + m, pls_rb, gy);
        yb[a] = gy * es;
      }
      for (int m = n2 + lane; m < ma; m += 32) tc_put3(rb + m, pls_rb, 0.f);
    }
    __syncthreads();
    if (st < L) {
      // pre = W1^T u_b + b1; h = tanh(pre) onto the FP32 tape and as BF16 parts
      tc_gemm<W>(buf, kb + 8, H / 16, kb / 16, S.ub, Lo.ub_stride, T * Lo.ub_stride, T, warp, lane,
                 [&](int j, int n, float v) {
                   const float h = tanhf(v + b1[j]);
                   h_all[(size_t)n * pr + j] = h;
                   tc_put3(S.hb + (size_t)n * Lo.pb_stride + j, pls_pb, h);
                 });
      __syncthreads();
      // r = W2^T h + b2
      tc_gemm<W>(buf + (size_t)H * (kb + 8), H + 8, ma / 16, H / 16, S.hb, Lo.pb_stride, pls_pb, T, warp, lane,
                 [&](int m, int n, float v) {
                   if (m < n2) S.regions[(size_t)n * pr + Lo.o_r + m] = v + b2[m];
                 });
      __syncthreads();
      if (mine) {
        // coupling update of the a set; tape s and u_a; next layer's inputs
        float* ts = R + Lo.o_s + l * Lo.s_stride;
        float* tua = R + Lo.o_ua + l * Lo.s_stride;
        const float* r = R + Lo.o_r;
        for (int m = lane; m < na; m += 32) {
          const float s = F.clamp * tanhf(r[m] / F.clamp);
          const int a = ai[m];
          const float ua = y[a];
          ts[m] = s;
          tua[m] = ua;
          y[a] = fmaf(ua, expf(s), r[na + m]);
          ld += s;
        }
        __syncwarp();
        if (st + 1 < L) tc_gather_ub(F, Lo, S, st + 1, S.sidx + (st + 1) * d, y, warp, lane);
      }
    } else {
      // hbar = W2 rbar; pbar = hbar (1 - h^2) as BF16 parts
      tc_gemm<W>(buf, ma + 8, H / 16, ma / 16, S.rb, Lo.rb_stride, pls_rb, T, warp, lane,
                 [&](int j, int n, float v) {
                   const float h = h_all[(size_t)n * pr + j];
                   tc_put3(S.pb + (size_t)n * Lo.pb_stride + j, pls_pb, v * (1.0f - h * h));
                 });
      __syncthreads();
      // u_b adjoint += W1 pbar
      tc_gemm<W>(buf + (size_t)H * (ma + 8), H + 8, kb / 16, H / 16, S.pb, Lo.pb_stride, pls_pb, T, warp, lane,
                 [&](int r, int n, float v) {
                   if (r < nb) S.regions[(size_t)n * pr + Lo.o_yb + bi[r]] += v;
                 });
      __syncthreads();
    }
  }
  if (mine)
    for (int i = lane; i < d; i += 32) g[i] = (double)yb[i];
  return lp;
}

// Fused flow sampler on the tensor-core pass: W warps per CTA, the first T
// of them each run one chain's NUTS state machine (chains cached in shared
// memory behind the flow's area when P.cache is set).
template <int W, int KIND>
__global__ void __launch_bounds__(32 * W) k_fused_flow_tc(FlowDev Fp, Params P, Bufs B, DevModel M, int T,
                                                          size_t flow_bytes) {
  extern __shared__ __align__(16) unsigned char fsm[];
  __shared__ FlowDev Fsh;
  __shared__ FlowTcLayout Lsh;
  if (threadIdx.x == 0) {
    Fsh = Fp;
    Lsh = flow_tc_layout(Fp, T);
  }
  __syncthreads();
  const FlowDev& F = Fsh;
  const FlowTcLayout& Lo = Lsh;
  const TcSmem S = tc_smem(F, Lo, fsm);
  const double sum_rho = tc_setup(F, S);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * T + w;
  const bool exists = w < T && c < P.C;
  Scal s;
  if (exists) s = B.sc[c];
  bool live = exists && s.phase < PH_DONE;
  const bool attached = live && P.cache;
  Chain ch(P, B, M, s, exists ? c : 0, lane);
  double* cache = reinterpret_cast<double*>(fsm + flow_bytes) + (size_t)w * P.cache_stride;
  if (attached) ch.cache_attach(cache);
  __syncthreads();
  for (int b = 0; b < P.grad_budget; ++b) {
    if (!__syncthreads_or(live)) break;
    const double lp = flow_grad_pass_tc<W, KIND>(F, Lo, M, S, sum_rho, live, ch.Wq, ch.Wg);
    if (live) {
      s.W_lp = lp;
      __syncwarp();
      live = ch.advance();
    }
  }
  if (attached) ch.cache_detach();
  __syncwarp();
  if (exists && lane == 0) B.sc[c] = s;
}

// the tensor-core pass at given points (parity checks of the sampler's pass)
template <int W, int KIND>
__global__ void __launch_bounds__(32 * W) k_flow_grad_tc(FlowDev Fp, DevModel M, int n, int T, const double* z,
                                                         double* lp, double* g) {
  extern __shared__ __align__(16) unsigned char fsm[];
  __shared__ FlowDev Fsh;
  __shared__ FlowTcLayout Lsh;
  if (threadIdx.x == 0) {
    Fsh = Fp;
    Lsh = flow_tc_layout(Fp, T);
  }
  __syncthreads();
  const FlowDev& F = Fsh;
  const FlowTcLayout& Lo = Lsh;
  const TcSmem S = tc_smem(F, Lo, fsm);
  const double sum_rho = tc_setup(F, S);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int p = blockIdx.x * T + w;
  const bool live = w < T && p < n;
  __syncthreads();
  const size_t off = live ? (size_t)p * F.d : 0;
  const double v = flow_grad_pass_tc<W, KIND>(F, Lo, M, S, sum_rho, live, z + off, g + off);
  if (live && lane == 0) lp[p] = v;
}


template <int KIND>
cudaError_t flow_tc_fused_launch_k(const FlowDev& F, const Params& P, const Bufs& B, const DevModel& M, int T,
                                   size_t flow_bytes, int blocks, size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(k_fused_flow_tc<FLOW_TC_W, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  k_fused_flow_tc<FLOW_TC_W, KIND><<<blocks, 32 * FLOW_TC_W, smem>>>(F, P, B, M, T, flow_bytes);
  return cudaGetLastError();
}

template <int KIND>
cudaError_t flow_tc_grad_launch_k(const FlowDev& F, const DevModel& M, int n, int T, const double* z, double* lp,
                                  double* g, size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(k_flow_grad_tc<FLOW_TC_W, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  k_flow_grad_tc<FLOW_TC_W, KIND><<<(n + T - 1) / T, 32 * FLOW_TC_W, smem>>>(F, M, n, T, z, lp, g);
  return cudaGetLastError();
}

template cudaError_t flow_tc_fused_launch_k<GNUTS_KIND>(const FlowDev&, const Params&, const Bufs&, const DevModel&,
                                                        int, size_t, int, size_t);
template cudaError_t flow_tc_grad_launch_k<GNUTS_KIND>(const FlowDev&, const DevModel&, int, int, const double*,
                                                       double*, double*, size_t);

}  // namespace gnuts
