// tcgen05 tensor-core kernels for the batched logistic-likelihood gradient of
// wide designs: more predictors than k_glm_tc's 128-column tile holds (the
// regularised-horseshoe workload, X 200,000 x 1000 BF16, 256 chains).  Per
// round every live chain c needs, for its coefficients beta_c and intercept
// b0_c,
//     eta[c, n] = b0_c + beta_c . X_n
//     lp_c      = sum_n y_n eta[c, n] - softplus(eta[c, n])
//     r[c, n]   = y_n - inv_logit(eta[c, n])
//     g_c       = (sum_n r[c, n], X^T r_c)
// which is the reverse sweep of stan::model::log_prob_grad for the logistic
// GLM (the gradient contract of src/cmdstan/command_helper.hpp:589-593);
// coefficient transforms and priors stay in stage_request / reduce_gradient.
// With K = 1000 neither the coefficients of a chain tile (1 MB with both
// BF16 parts) nor a chain tile's gradient (128 x 1000 FP32) fits on chip
// next to the other GEMM's operands, so the two contractions are two kernels
// and only the BF16 residuals cross HBM between them:
//
//   k_wide_eta  CTA = 128 chains x interleaved 256-row blocks.  M = chains,
//               N = 256 rows, K = predictors in 64-wide chunks:
//               H = [beta_hi ; beta_lo] . X^T as two BF16 MMAs per k-step
//               accumulated in FP32 TMEM (two 256-column buffers, so the
//               epilogue of block t overlaps the MMAs of block t + 1).  The
//               epilogue (thread = chain, 128 rows) forms eta, the
//               likelihood terms and the residuals, writes the residuals as
//               BF16 rows r[c][n] and keeps per-chain sums of lp and r.
//   k_wide_xtr  CTA = 128 chains x 256 predictors x a row range.  M =
//               chains, N = predictors, K = rows in 64-row chunks:
//               G^T += r . X, A = r (K-major), B = X (MN-major, four 64-column
//               boxes per chunk); one FP32 accumulator per CTA, written as a
//               row-range partial.
//   k_wide_final  fixed-order sums of the partials into the [C][K+1]
//               gradient and [C] lp rows that reduce_gradient consumes.
//
// Precision matches the tcgen05 path of narrow designs: X BF16-exact,
// coefficients split into two BF16 parts (16 significant bits), FP32
// accumulation, residuals BF16 in X^T r and exact (FP32) in the intercept
// sum; lp per thread in FP32 with a compensation term, per CTA and per chain
// in FP64; the row ranges' X^T r partials summed in FP32; every sum in a
// fixed order (bitwise reproducible).
// Every mbarrier wait is bounded; on expiry a kernel records an error, drains
// what it issued and frees its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <string>
#include "internal.h"
#include "batched.cuh"
#include "grad_wide.h"
#include "tc_ptx.cuh"

namespace gnuts {

namespace {
using namespace tcx;

constexpr int NUM_SMS = 152;

// ---- k_wide_eta
constexpr int E_ROWS = 256;                          // rows per block (MMA N)
constexpr int E_NS = 3;                              // pipeline stages
constexpr int E_A_BYTES = 128 * 128;                 // one coefficient plane: 128 chains x 64 predictors
constexpr int E_X_BYTES = E_ROWS * 128;              // 256 rows x 64 predictors
constexpr int E_STAGE = 2 * E_A_BYTES + E_X_BYTES;   // 64 KB
constexpr int E_EPI_WARPS = 8;                       // two per TMEM lane quadrant, 128 rows each
constexpr int E_THREADS = 64 + 32 * E_EPI_WARPS;
constexpr int E_OFF_BAR = E_NS * E_STAGE;
constexpr int E_OFF_MISC = E_OFF_BAR + 16 * 8;       // tmem base, abort flag
constexpr int E_OFF_RED = E_OFF_MISC + 16;           // [2][128] doubles: second half's sums
constexpr int E_SMEM = E_OFF_RED + 2 * 128 * 8 + 1024;
enum { E_FULL = 0, E_EMPTY = E_NS, E_HFULL = 2 * E_NS, E_HFULL1, E_HEMPTY, E_HEMPTY1, E_DRAIN };
static_assert(E_DRAIN < 16, "barrier area");

// ---- k_wide_xtr
constexpr int G_NS = 4;
constexpr int G_A_BYTES = 128 * 128;                 // residuals: 128 chains x 64 rows
constexpr int G_B_BYTES = 4 * 64 * 128;              // X: 64 rows x 256 predictors (four 64-column boxes)
constexpr int G_STAGE = G_A_BYTES + G_B_BYTES;       // 48 KB
constexpr int G_THREADS = 64 + 128;
constexpr int G_OFF_BAR = G_NS * G_STAGE;
constexpr int G_OFF_MISC = G_OFF_BAR + 16 * 8;
constexpr int G_SMEM = G_OFF_MISC + 16 + 1024;
enum { G_FULL = 0, G_EMPTY = G_NS, G_DONE = 2 * G_NS, G_DRAIN };
static_assert(G_DRAIN < 16, "barrier area");

constexpr float LOG2E = 1.4426950408889634f;
constexpr float LN2 = 0.6931471805599453f;

struct WideArgs {
  int N, K, C, Cpad, Npad, Kp;
  int P;          // k_wide_eta: CTAs per chain tile; CTA p takes row blocks p, p + P, ...
  int nblocks;    // 256-row blocks
  int nchunks;    // 64-row chunks (k_wide_xtr)
  int cps;        // k_wide_xtr: chunks per row range
  int S2;         // k_wide_xtr: row ranges
  const double* coef64;   // [C][K+1]: intercept, then beta
  const uint32_t* ybits;  // y packed 32 rows per word
  uint16_t* rt;           // [Cpad][Npad] BF16 residuals
  double* plp;            // [P][C] lp sums of k_wide_eta's CTAs
  double* prs;            // [P][C] residual sums (intercept gradient)
  float* gpart;           // [S2][Cpad][Kp] FP32 partials of X^T r
  const int* done_count;
  int C_total;
  int* error;
};

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return p + ((1024u - (su32(p) & 1023u)) & 1023u);
}

__global__ void __launch_bounds__(E_THREADS, 1)
    k_wide_eta(const __grid_constant__ CUtensorMap cmap, const __grid_constant__ CUtensorMap xmap, WideArgs A) {
  if (A.done_count && *A.done_count >= A.C_total) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  const uint32_t sbase = su32(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c0 = blockIdx.x * 128;
  const int split = blockIdx.y;
  const int T = split < A.nblocks ? (A.nblocks - split + A.P - 1) / A.P : 0;
  const int KC = (A.K + 63) / 64;
  auto bar = [&](int i) { return sbase + E_OFF_BAR + 8u * (uint32_t)i; };
  volatile int* abort = (volatile int*)(smem + E_OFF_MISC + 4);
  uint32_t* tmem_slot = (uint32_t*)(smem + E_OFF_MISC);
  double* red = (double*)(smem + E_OFF_RED);

  if (threadIdx.x == 0) {
    for (int s = 0; s < E_NS; ++s) {
      mbar_init(bar(E_FULL + s), 1);
      mbar_init(bar(E_EMPTY + s), 1);
    }
    mbar_init(bar(E_HFULL), 1);
    mbar_init(bar(E_HFULL1), 1);
    mbar_init(bar(E_HEMPTY), E_EPI_WARPS);
    mbar_init(bar(E_HEMPTY1), E_EPI_WARPS);
    mbar_init(bar(E_DRAIN), 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(tmem_slot, 512);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer: both coefficient planes and the X rows of each chunk
    if (lane == 0) {
      int issued = 0;
      for (int t = 0; t < T; ++t) {
        const int row0 = (split + t * A.P) * E_ROWS;
        bool ok = true;
        for (int kc = 0; kc < KC; ++kc) {
          const int it = t * KC + kc, s = it % E_NS;
          if (it >= E_NS && !mbar_wait(bar(E_EMPTY + s), ((it / E_NS) - 1) & 1, abort)) { ok = false; break; }
          const uint32_t dst = sbase + s * E_STAGE;
          mbar_expect_tx(bar(E_FULL + s), E_STAGE);
          tma_load_2d(dst, &cmap, kc * 64, c0, bar(E_FULL + s));
          tma_load_2d(dst + E_A_BYTES, &cmap, kc * 64, A.Cpad + c0, bar(E_FULL + s));
          tma_load_2d(dst + 2 * E_A_BYTES, &xmap, kc * 64, row0, bar(E_FULL + s));
          ++issued;
        }
        if (!ok) break;
      }
      if (*abort) {
        for (int it = (issued > E_NS ? issued - E_NS : 0); it < issued; ++it) {
          volatile int never = 0;
          mbar_wait(bar(E_FULL + it % E_NS), (it / E_NS) & 1, &never);
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer: H(t) (buffer t & 1) = beta_hi . X^T + beta_lo . X^T
    if (lane == 0) {
      const uint32_t ID = idesc(false, false, E_ROWS);
      const uint64_t d0 = sdesc(sbase, 0, 1024);
      const uint32_t dlo = (uint32_t)d0, dhi = (uint32_t)(d0 >> 32);
      bool ok = true;
      for (int t = 0; ok && t < T; ++t) {
        const int b = t & 1;
        // buffer b holds block t - 2 until its epilogue has read it
        if (t >= 2 && !mbar_wait(bar(E_HEMPTY + b), ((t >> 1) - 1) & 1, abort)) break;
        fence_after();
        const uint32_t tH = tmem + (uint32_t)(b * E_ROWS);
        for (int kc = 0; kc < KC; ++kc) {
          const int it = t * KC + kc, s = it % E_NS;
          if (!mbar_wait(bar(E_FULL + s), (it / E_NS) & 1, abort)) { ok = false; break; }
          fence_after();
          const uint32_t a = dlo + (uint32_t)((s * E_STAGE) >> 4);
          const uint32_t x = a + (uint32_t)((2 * E_A_BYTES) >> 4);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            mma_ss(tH, a + 2 * i, dhi, x + 2 * i, dhi, ID, (kc > 0 || i > 0) ? 1u : 0u);
            mma_ss(tH, a + (uint32_t)(E_A_BYTES >> 4) + 2 * i, dhi, x + 2 * i, dhi, ID, 1u);
          }
          mma_commit(bar(E_EMPTY + s));
        }
        if (ok) mma_commit(bar(E_HFULL + b));
      }
      mma_commit(bar(E_DRAIN));
      volatile int never = 0;
      mbar_wait(bar(E_DRAIN), 0, &never);
    }
  } else {
    // ---------------- epilogue: thread = (chain, 128 rows of each block)
    const int q = warp & 3;              // TMEM lane quadrant (fixed by warp id % 4)
    const int half = (warp - 2) >> 2;    // rows [128 half, 128 half + 128) of a block
    const int cl = q * 32 + lane;
    const int c = c0 + cl;
    const bool cv = c < A.C;
    const float b0 = cv ? (float)A.coef64[(size_t)c * (A.K + 1)] : 0.f;
    uint16_t* rrow = A.rt + (size_t)c * A.Npad;
    double lp_tot = 0.0, rs_tot = 0.0;
    for (int t = 0; t < T; ++t) {
      const int b = t & 1;
      if (!mbar_wait(bar(E_HFULL + b), (t >> 1) & 1, abort)) break;
      fence_after();
      const int n0 = (split + t * A.P) * E_ROWS + half * 128;
      const int nvalid = max(0, min(128, A.N - n0));
      uint32_t yw[4];
#pragma unroll
      for (int w = 0; w < 4; ++w) yw[w] = n0 + 32 * w < A.N ? A.ybits[(n0 >> 5) + w] : 0u;
      const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * E_ROWS + half * 128);
      float lp_acc = 0.f, lp_comp = 0.f, rs = 0.f;
#pragma unroll 1
      for (int g = 0; g < 8; ++g) {
        float v[16];
        tmem_ld16(ta + 16 * g, v);
        tmem_wait_ld();
        const uint32_t ybits16 = (yw[g >> 1] >> ((g & 1) * 16)) & 0xFFFFu;
        float lin = 0.f, prod = 1.f;
        uint32_t pk[8];
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
          float rr[2];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const int jj = j + u;
            const bool valid = 16 * g + jj < nvalid;
            const float h = v[jj] + b0;
            const float yv = (ybits16 >> jj) & 1u ? 1.f : 0.f;
            const float e = ex2a(-fabsf(h) * LOG2E);
            const float d = 1.f + e;
            const float ir = rcpa(d);
            const float sig = h >= 0.f ? ir : e * ir;
            rr[u] = valid ? yv - sig : 0.f;
            lin += valid ? fmaf(yv, h, -fmaxf(h, 0.f)) : 0.f;
            prod *= valid ? d : 1.f;
            rs += rr[u];
          }
          pk[j >> 1] = pack_bf16(rr[0], rr[1]);
        }
        // y h - softplus(h) = y h - max(h, 0) - log(1 + e^-|h|); the sixteen
        // log terms as one lg2 of their product (at most 2^16)
        const float grp = fmaf(-LN2, lg2a(prod), lin);
        const float yk = grp - lp_comp;
        const float tk = lp_acc + yk;
        lp_comp = (tk - lp_acc) - yk;
        lp_acc = tk;
        uint4* dst = reinterpret_cast<uint4*>(rrow + n0 + 16 * g);
        dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(bar(E_HEMPTY + b));
      lp_tot += (double)lp_acc - (double)lp_comp;
      rs_tot += (double)rs;
    }
    if (half == 1) {
      red[cl] = lp_tot;
      red[128 + cl] = rs_tot;
    }
    asm volatile("bar.sync 1, 256;" ::: "memory");
    if (half == 0 && cv) {
      A.plp[(size_t)split * A.C + c] = lp_tot + red[cl];
      A.prs[(size_t)split * A.C + c] = rs_tot + red[128 + cl];
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    tmem_dealloc(tmem, 512);
  }
  if (threadIdx.x == 0 && *abort) atomicExch(A.error, 1);
}

__global__ void __launch_bounds__(G_THREADS, 1)
    k_wide_xtr(const __grid_constant__ CUtensorMap rmap, const __grid_constant__ CUtensorMap xmap, WideArgs A) {
  if (A.done_count && *A.done_count >= A.C_total) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  const uint32_t sbase = su32(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c0 = blockIdx.x * 128;
  const int k0 = blockIdx.y * 256;
  const int split = blockIdx.z;
  const int j0 = split * A.cps, j1 = min(A.nchunks, j0 + A.cps);
  const int T = max(0, j1 - j0);
  auto bar = [&](int i) { return sbase + G_OFF_BAR + 8u * (uint32_t)i; };
  volatile int* abort = (volatile int*)(smem + G_OFF_MISC + 4);
  uint32_t* tmem_slot = (uint32_t*)(smem + G_OFF_MISC);

  if (threadIdx.x == 0) {
    for (int s = 0; s < G_NS; ++s) {
      mbar_init(bar(G_FULL + s), 1);
      mbar_init(bar(G_EMPTY + s), 1);
    }
    mbar_init(bar(G_DONE), 1);
    mbar_init(bar(G_DRAIN), 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(tmem_slot, 256);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int t = 0; t < T; ++t) {
        const int s = t % G_NS, n = (j0 + t) * 64;
        if (t >= G_NS && !mbar_wait(bar(G_EMPTY + s), ((t / G_NS) - 1) & 1, abort)) break;
        const uint32_t dst = sbase + s * G_STAGE;
        mbar_expect_tx(bar(G_FULL + s), G_STAGE);
        tma_load_2d(dst, &rmap, n, c0, bar(G_FULL + s));
#pragma unroll
        for (int g = 0; g < 4; ++g) tma_load_2d(dst + G_A_BYTES + g * 8192, &xmap, k0 + 64 * g, n, bar(G_FULL + s));
        ++issued;
      }
      if (*abort) {
        for (int t = (issued > G_NS ? issued - G_NS : 0); t < issued; ++t) {
          volatile int never = 0;
          mbar_wait(bar(G_FULL + t % G_NS), (t / G_NS) & 1, &never);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // A = r (K-major: a chain's 64 rows in one 128-byte line); B = X
      // (MN-major: four 64-predictor boxes 8 KB apart, 16 rows per k-step)
      const uint32_t ID = idesc(false, true, 256);
      const uint64_t da = sdesc(sbase, 0, 1024), db = sdesc(sbase + G_A_BYTES, 8192, 1024);
      const uint32_t alo = (uint32_t)da, ahi = (uint32_t)(da >> 32);
      const uint32_t blo = (uint32_t)db, bhi = (uint32_t)(db >> 32);
      for (int t = 0; t < T; ++t) {
        const int s = t % G_NS;
        if (!mbar_wait(bar(G_FULL + s), (t / G_NS) & 1, abort)) break;
        fence_after();
        const uint32_t so = (uint32_t)((s * G_STAGE) >> 4);
#pragma unroll
        for (int i = 0; i < 4; ++i)
          mma_ss(tmem, alo + so + 2 * i, ahi, blo + so + (uint32_t)((i * 2048) >> 4), bhi, ID,
                 (t > 0 || i > 0) ? 1u : 0u);
        mma_commit(bar(G_EMPTY + s));
      }
      mma_commit(bar(G_DONE));
      mma_commit(bar(G_DRAIN));
      volatile int never = 0;
      mbar_wait(bar(G_DRAIN), 0, &never);
    }
  } else {
    // ---------------- epilogue: thread = chain, 256 predictor columns
    const int q = warp & 3;
    const int c = c0 + q * 32 + lane;
    const bool ok = mbar_wait(bar(G_DONE), 0, abort);
    fence_after();
    float4* dst = reinterpret_cast<float4*>(A.gpart + ((size_t)split * A.Cpad + c) * A.Kp + k0);
    const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
    for (int g = 0; g < 16; ++g) {
      float v[16];
      tmem_ld16(ta + 16 * g, v);
      tmem_wait_ld();
#pragma unroll
      for (int i = 0; i < 4; ++i)
        dst[4 * g + i] = ok && T > 0 ? make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3])
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    tmem_dealloc(tmem, 256);
  }
  if (threadIdx.x == 0 && *abort) atomicExch(A.error, 1);
}

// coefficient rows -> the two BF16 planes of k_wide_eta's A operand
// ([2][Cpad][K]; rows of padding chains stay zero)
__global__ void k_wide_stage(const double* coef64, int C, int Cpad, int K, uint16_t* planes) {
  const size_t n = (size_t)C * K;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / K), k = (int)(i % K);
    const double v = coef64[(size_t)c * (K + 1) + 1 + k];
    const __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
    const __nv_bfloat16 lo = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
    planes[(size_t)c * K + k] = *reinterpret_cast<const uint16_t*>(&hi);
    planes[((size_t)Cpad + c) * K + k] = *reinterpret_cast<const uint16_t*>(&lo);
  }
}

// partials -> lp [C] and gradient rows [C][K+1] (intercept first).  Blocks
// [0, nb_g): thread per (chain, predictor), the FP32 partials of the row
// ranges summed in FP32 in range order (they are FP32 tensor-memory
// accumulators; eight loads in flight per step); blocks after: warp per
// chain, the eta kernel's FP64 lp and residual sums, lane l taking CTAs l,
// l + 32, ... and a fixed butterfly.
constexpr int F_THREADS = 256;
__global__ void __launch_bounds__(F_THREADS) k_wide_final(WideArgs A, int nb_g, double* part_lp, double* part_g) {
  if (A.done_count && *A.done_count >= A.C_total) return;
  const int K1 = A.K + 1;
  if ((int)blockIdx.x < nb_g) {
    const size_t i = (size_t)blockIdx.x * F_THREADS + threadIdx.x;
    const int c = (int)(i / A.K), k = (int)(i % A.K);
    if (c >= A.C) return;
    const float* src = A.gpart + (size_t)c * A.Kp + k;
    const size_t stride = (size_t)A.Cpad * A.Kp;
    float s = 0.f;
    for (int p0 = 0; p0 < A.S2; p0 += 8) {
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = p0 + u < A.S2 ? src[(size_t)(p0 + u) * stride] : 0.f;
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (p0 + u < A.S2) s += v[u];
    }
    part_g[(size_t)c * K1 + 1 + k] = (double)s;
    return;
  }
  const int c = ((int)blockIdx.x - nb_g) * (F_THREADS / 32) + (int)(threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= A.C) return;
  double l = 0.0, r = 0.0;
  for (int p = lane; p < A.P; p += 32) {
    l += A.plp[(size_t)p * A.C + c];
    r += A.prs[(size_t)p * A.C + c];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    l += __shfl_xor_sync(0xffffffffu, l, o);
    r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  if (lane == 0) {
    part_lp[c] = l;
    part_g[(size_t)c * K1] = r;
  }
}

}  // namespace

struct WidePlan {
  CUtensorMap cmap, xmap_eta, rmap, xmap_xtr;
  WideArgs args{};
  dim3 grid_eta, grid_xtr;
  uint16_t* planes = nullptr;  // [2][Cpad][K] BF16
  uint16_t* rt = nullptr;      // [Cpad][Npad] BF16
  double *plp = nullptr, *prs = nullptr;
  float* gpart = nullptr;
  double* coef64 = nullptr;                      // [C][K+1] coefficient rows (stage_request)
  double *part_lp = nullptr, *part_g = nullptr;  // [1][C], [1][C][K+1] for reduce_gradient
  int* error = nullptr;
};

bool wide_supported(const DevModel& M) {
  return (M.kind == MK_LOGISTIC || M.kind == MK_HORSESHOE) && M.Xb && M.ybits && M.K % 8 == 0 && M.N > 0 &&
         M.K >= 8;
}

void wide_destroy(WidePlan* p) {
  if (!p) return;
  for (void* q : {(void*)p->planes, (void*)p->rt, (void*)p->plp, (void*)p->prs, (void*)p->gpart,
                  (void*)p->coef64, (void*)p->part_lp, (void*)p->part_g, (void*)p->error})
    if (q) cudaFree(q);
  delete p;
}

int wide_create(const DevModel& M, int C, const int* done_count, WidePlan** out, double** coef64,
                double** part_lp, double** part_g, std::string& err) {
  *out = nullptr;
  if (!wide_supported(M)) {
    err = "wide-design gradient needs a logistic or horseshoe model with a multiple of 8 predictors";
    return GNUTS_ERR_ARGUMENT;
  }
  if (C < 1) {
    err = "the wide-design gradient needs at least one chain";
    return GNUTS_ERR_ARGUMENT;
  }
  WidePlan* p = new WidePlan();
  const int N = M.N, K = M.K;
  const int Cpad = (C + 127) / 128 * 128, ctiles = Cpad / 128;
  const int nblocks = (N + E_ROWS - 1) / E_ROWS;
  const int Npad = nblocks * E_ROWS;
  const int kblocks = (K + 255) / 256, Kp = kblocks * 256;
  // k_wide_eta: one CTA per SM over the chain tiles
  const int P = std::max(1, std::min(nblocks, NUM_SMS / ctiles));
  // k_wide_xtr: row ranges so that chain tiles x predictor blocks x ranges fill the SMs
  const int nchunks = Npad / 64;
  int S2 = std::max(1, std::min(nchunks, NUM_SMS / (ctiles * kblocks)));
  const int cps = (nchunks + S2 - 1) / S2;
  S2 = (nchunks + cps - 1) / cps;  // every range non-empty
  auto fail = [&](cudaError_t e) {
    err = std::string("CUDA error: ") + cudaGetErrorString(e);
    wide_destroy(p);
    return GNUTS_ERR_CUDA;
  };
  cudaError_t e;
  if ((e = cudaMalloc(&p->planes, sizeof(uint16_t) * 2 * Cpad * K)) != cudaSuccess) return fail(e);
  if ((e = cudaMemset(p->planes, 0, sizeof(uint16_t) * 2 * Cpad * K)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&p->rt, sizeof(uint16_t) * (size_t)Cpad * Npad)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&p->plp, sizeof(double) * P * C)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&p->prs, sizeof(double) * P * C)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&p->gpart, sizeof(float) * (size_t)S2 * Cpad * Kp)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&p->coef64, sizeof(double) * C * (K + 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMemset(p->coef64, 0, sizeof(double) * C * (K + 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&p->part_lp, sizeof(double) * C)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&p->part_g, sizeof(double) * C * (K + 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&p->error, sizeof(int))) != cudaSuccess) return fail(e);
  if ((e = cudaMemset(p->error, 0, sizeof(int))) != cudaSuccess) return fail(e);
  int rc = make_map_bf16(&p->cmap, p->planes, K, 2 * (uint64_t)Cpad, (uint64_t)K * 2, 128, err);
  if (!rc) rc = make_map_bf16(&p->xmap_eta, M.Xb, K, N, (uint64_t)K * 2, E_ROWS, err);
  if (!rc) rc = make_map_bf16(&p->rmap, p->rt, Npad, Cpad, (uint64_t)Npad * 2, 128, err);
  if (!rc) rc = make_map_bf16(&p->xmap_xtr, M.Xb, K, N, (uint64_t)K * 2, 64, err);
  if (rc) {
    wide_destroy(p);
    return rc;
  }
  p->args = WideArgs{N, K, C, Cpad, Npad, Kp, P, nblocks, nchunks, cps, S2, p->coef64, M.ybits, p->rt,
                     p->plp, p->prs, p->gpart, done_count, C, p->error};
  p->grid_eta = dim3(ctiles, P);
  p->grid_xtr = dim3(ctiles, kblocks, S2);
  if ((e = cudaFuncSetAttribute(k_wide_eta, cudaFuncAttributeMaxDynamicSharedMemorySize, E_SMEM)) != cudaSuccess)
    return fail(e);
  if ((e = cudaFuncSetAttribute(k_wide_xtr, cudaFuncAttributeMaxDynamicSharedMemorySize, G_SMEM)) != cudaSuccess)
    return fail(e);
  *coef64 = p->coef64;
  *part_lp = p->part_lp;
  *part_g = p->part_g;
  *out = p;
  return GNUTS_OK;
}

int wide_launch(const WidePlan* p, const GradOut& G, const DevModel& M, cudaStream_t st) {
  (void)M;
  const WideArgs& A = p->args;
  k_wide_stage<<<std::min(4096, (A.C * A.K + 255) / 256), 256, 0, st>>>(G.coef64, A.C, A.Cpad, A.K, p->planes);
  k_wide_eta<<<p->grid_eta, E_THREADS, E_SMEM, st>>>(p->cmap, p->xmap_eta, A);
  k_wide_xtr<<<p->grid_xtr, G_THREADS, G_SMEM, st>>>(p->rmap, p->xmap_xtr, A);
  const int nb_g = (int)(((size_t)A.C * A.K + F_THREADS - 1) / F_THREADS);
  const int nb_c = (A.C + F_THREADS / 32 - 1) / (F_THREADS / 32);
  k_wide_final<<<nb_g + nb_c, F_THREADS, 0, st>>>(A, nb_g, G.part_lp, G.part_g);
  return cudaGetLastError() == cudaSuccess ? GNUTS_OK : GNUTS_ERR_CUDA;
}

int wide_error(const WidePlan* p) {
  int h = 0;
  cudaMemcpy(&h, p->error, sizeof(int), cudaMemcpyDeviceToHost);
  return h;
}

}  // namespace gnuts
