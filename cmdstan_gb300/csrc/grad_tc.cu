// tcgen05 tensor-core kernel for the batched logistic-regression gradient.
//
// Per round every live chain c needs, for its coefficients B_c (intercept
// folded in through a ones column of X),
//     H[c, n] = B_c . X_n                       GEMM1, M = chains, N = rows, K = predictors
//     lp_c    = sum_n y_n H[c, n] - softplus(H[c, n])
//     R[c, n] = y_n - inv_logit(H[c, n])
//     G[c, k] = sum_n R[c, n] X[n, k]           GEMM2, M = chains, N = predictors, K = rows
// which is the reverse sweep Stan Math performs for one chain's
// bernoulli_logit likelihood (log_prob_grad contract, src/cmdstan/
// command_helper.hpp:589-593), done for 128 chains at once.
//
// The likelihood is split into a linear and an even part,
//     y h - softplus(h) = (y - 1/2) h  -  (|h|/2 + log1p(exp(-|h|))),
// and the linear part summed over rows is B_c . v with v = X^T (y - 1/2), a
// vector fixed by the data: stage_request forms that dot product in FP64 for
// the exact BF16 hi + lo coefficients this kernel multiplies, so the kernel
// only sums the even part.  Per element it then takes one ex2 (e =
// exp(-|h|)); the log1p terms of a thread's 32-row slice are summed as one
// lg2 of the product of their (1 + e) factors (at most 2^32), and the
// inverse-logit shares one reciprocal between four rows (1/d_i from
// 1/(d_0 d_1 d_2 d_3) and the partial products): 1.28 special-function
// operations per element (ex2, a quarter rcp, 1/32 lg2) instead of three.
//
// Precision: X is BF16-exact (the workload's design matrix is defined on
// BF16 values).  Coefficients are split hi + lo in BF16, so GEMM1 is two BF16
// MMAs accumulated in FP32 TMEM (about 16 significant bits of each
// coefficient: this is what keeps lp accurate).  Residuals enter GEMM2 in
// BF16 (relative error 2^-9 per residual, about 1e-3 on a gradient
// component); a gradient error leaves the leapfrog volume preserving and
// reversible and lp is computed separately, so it does not bias the target.
// The even part runs in FP32; each thread's slice sum is added to its total
// with Kahan-compensated FP32 additions; the reduction over the 512 threads'
// totals and over row splits is FP64, and so is the linear part.
//
// X rows carry 104 BF16 columns (K predictors, the ones column, zeros), so
// GEMM1 runs 7 K-steps of 16 (112 columns) and GEMM2 has N = 112.
//
// CTA = one 128-chain tile x one row split, 608 threads:
//   warp 0       TMA producer: X row tiles (6-stage ring, 128 rows x 128
//                predictors, SWIZZLE_128B)
//   warp 1       GEMM1 issuer (one thread) + TMEM owner
//   warps 2..17  epilogue: thread = (chain, 32-row slice of the tile), four
//                warps per TMEM lane quadrant; reads its H slice from TMEM and
//                writes its 32 BF16 residuals back over the first 16 columns
//                of that slice; y - 1/2 of the split is staged as floats
//   warp 18      GEMM2 issuer (one thread)
// TMEM (512 columns): two H buffers (128 each; each also carries the
// residuals of its tile, GEMM2's A operand: lane = chain, two BF16 rows per
// column), G (112, at 256), and the coefficient tile as GEMM1's A operand
// (hi and lo planes, 56 columns each), written once per launch by the
// epilogue warps with tcgen05.st.  Both A operands live in TMEM, so shared
// memory holds only the X ring: an X tile is held from its load until GEMM2
// of that tile retires (across GEMM1, the epilogue and GEMM2), and six stages
// keep the next loads in flight behind the L2 latency (with two, the loads
// sat on the critical path).  The two GEMMs are issued by two threads on
// different warp schedulers: the epilogue's FP32 work takes most issue slots,
// and one thread issuing both GEMMs plus their waits and commits left the
// tensor pipe idle between tiles (6% slower).  GEMM1 of tile t + 2 overwrites
// the buffer GEMM2 of tile t reads, so the GEMM1 thread waits on a commit
// barrier of that GEMM2 (MMAs of different threads are not ordered).  No
// barrier is needed between the epilogue's reads of H and its residual
// writes (the slice's own columns, after tcgen05.wait::ld).  GEMM1 of tile
// t+1 and GEMM2 of tile t-1 run while the epilogue works on tile t.
// Every mbarrier wait is bounded; on expiry the kernel records an error,
// drains what it issued and frees TMEM.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstring>
#include <string>
#include "grad_tc.h"
#include "tc_ptx.cuh"

namespace gnuts {
namespace {

using namespace tcx;

constexpr int TILE_BYTES = 128 * 128 * 2;   // [2 k-halves][128 rows][64] BF16
constexpr int HALF_BYTES = TILE_BYTES / 2;  // one k-half: 128 rows x 128 B
constexpr int NS = 6;
constexpr int EPI_WARPS = 16;                 // 4 per TMEM lane quadrant, 32 rows each
constexpr int G2_WARP = 2 + EPI_WARPS;  // GEMM2 issuer
constexpr int NUM_THREADS = 64 + 32 * EPI_WARPS + 32;
constexpr int MAX_SPLIT_ROWS = 6144;          // y of a whole row split staged as floats
constexpr int OFF_X = 0;
constexpr int OFF_BAR = OFF_X + NS * TILE_BYTES;  // 24 barriers
constexpr int OFF_MISC = OFF_BAR + 24 * 8;     // tmem base, abort flag
constexpr int OFF_LP = OFF_MISC + 16;          // [4][128] doubles
constexpr int OFF_Y = OFF_LP + 4 * 128 * 8;    // [MAX_SPLIT_ROWS] floats
constexpr int SMEM_USED = OFF_Y + MAX_SPLIT_ROWS * 4;
constexpr int SMEM_BYTES = SMEM_USED + 1024;   // alignment slack
constexpr uint32_t TMEM_COLS = 512;
// K-steps of 16 columns that cover an X row of XTC_LD columns, and GEMM2's N
constexpr int KSTEPS = (XTC_LD + 15) / 16;
constexpr uint32_t GN = 16u * KSTEPS;
static_assert(KSTEPS <= 8 && GN % 16 == 0, "X rows fit the 128-column tile");
// TMEM columns: H buffers at 0 and 128, G at 256, coefficient planes after
constexpr uint32_t TM_G = 256;
constexpr uint32_t ACOLS = 8 * KSTEPS;        // one plane of A: GN BF16 per lane
constexpr uint32_t TM_AHI = 384, TM_ALO = TM_AHI + ACOLS;
static_assert(TM_ALO + ACOLS <= TMEM_COLS && TM_G + 128 <= TM_AHI, "TMEM column map");
static_assert(ACOLS / 2 == 28, "each half-plane is written as x16 + x8 + x4 columns");

// barrier indices
enum { B_XFULL = 0, B_XEMPTY = NS, B_HFULL = 2 * NS, B_HFULL1, B_RFULL, B_RFULL1, B_GDONE, B_DRAIN, B_AREADY,
       B_G2DONE, B_G2DONE1, B_DRAIN2 };
static_assert(B_DRAIN2 < 24, "barrier area holds 24 barriers");

struct TcArgs {
  int N, K, C, Cpad, rows_per_split, S, C_total;
  const uint16_t* coef;  // [2][Cpad][128] BF16 hi / lo planes (stage_request)
  const uint32_t* ybits;
  double* part_lp;
  float* part_g;  // [S][C][TC_GSTRIDE]: position k < K = beta_k, K = intercept, zeros after
  const int* done_count;
  int* error;
};

__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_glm_tc(const __grid_constant__ CUtensorMap xmap, TcArgs A) {
  if (A.done_count && *A.done_count >= A.C_total) return;
  extern __shared__ uint8_t smem_raw[];
  // SWIZZLE_128B tiles need 1024-byte alignment in the shared address space
  uint8_t* smem = smem_raw + ((1024u - (su32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sbase = su32(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c0 = blockIdx.x * 128;
  const int split = blockIdx.y;
  const int row_begin = split * A.rows_per_split;
  const int row_end = min(A.N, row_begin + A.rows_per_split);
  const int T = row_end > row_begin ? (row_end - row_begin + 127) / 128 : 0;
  auto bar = [&](int i) { return sbase + OFF_BAR + 8u * (uint32_t)i; };
  volatile int* abort = (volatile int*)(smem + OFF_MISC + 4);
  uint32_t* tmem_slot = (uint32_t*)(smem + OFF_MISC);
  double* lpx = (double*)(smem + OFF_LP);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(bar(B_XFULL + s), 1);
      mbar_init(bar(B_XEMPTY + s), 1);
    }
    mbar_init(bar(B_HFULL), 1);
    mbar_init(bar(B_HFULL1), 1);
    mbar_init(bar(B_RFULL), EPI_WARPS);
    mbar_init(bar(B_RFULL1), EPI_WARPS);
    mbar_init(bar(B_GDONE), 1);
    mbar_init(bar(B_DRAIN), 1);
    mbar_init(bar(B_AREADY), EPI_WARPS);
    mbar_init(bar(B_G2DONE), 1);
    mbar_init(bar(B_G2DONE1), 1);
    mbar_init(bar(B_DRAIN2), 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;
  if (warp >= 2 && warp < G2_WARP) {
    // GEMM1's A operand into TMEM: warp (quadrant q, sub) writes lanes 32q..32q+31
    // (chains c0 + 32q + lane), plane sub >> 1 (hi, lo), columns of half sub & 1
    const int q = warp & 3, sub = (warp - 2) >> 2;
    const int plane = sub >> 1, half = sub & 1;
    const uint4* src = reinterpret_cast<const uint4*>(
        A.coef + ((size_t)(plane ? A.Cpad : 0) + c0 + q * 32 + lane) * 128 + half * (ACOLS / 2) * 2);
    uint32_t r[ACOLS / 2];
#pragma unroll
    for (int i = 0; i < (int)ACOLS / 8; ++i) {
      const uint4 u = src[i];
      r[4 * i] = u.x;
      r[4 * i + 1] = u.y;
      r[4 * i + 2] = u.z;
      r[4 * i + 3] = u.w;
    }
    const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (plane ? TM_ALO : TM_AHI) + half * (ACOLS / 2);
    tmem_st16(ta, r);
    tmem_st8(ta + 16, r + 16);
    tmem_st4(ta + 24, r + 24);
    tmem_wait_st();
    fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(bar(B_AREADY));  // the GEMM1 thread waits for all 16
  }

  if (warp == 0) {
    // ---------------- TMA producer
    if (lane == 0) {
      int issued = 0;
      for (int t = 0; t < T; ++t) {
        const int s = t % NS;
        if (t >= NS && !mbar_wait(bar(B_XEMPTY + s), ((t / NS) - 1) & 1, abort)) break;
        const uint32_t dst = sbase + OFF_X + s * TILE_BYTES;
        mbar_expect_tx(bar(B_XFULL + s), TILE_BYTES);
        tma_load_2d(dst, &xmap, 0, row_begin + t * 128, bar(B_XFULL + s));
        tma_load_2d(dst + HALF_BYTES, &xmap, 64, row_begin + t * 128, bar(B_XFULL + s));
        ++issued;
      }
      if (*abort) {
        // drain: wait (bounded) for every load issued into the ring
        for (int t = (issued > NS ? issued - NS : 0); t < issued; ++t) {
          volatile int never = 0;
          mbar_wait(bar(B_XFULL + t % NS), (t / NS) & 1, &never);
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- GEMM1 issuer: H(t) = coef . X(t)
    if (lane == 0) {
      const uint32_t ID1 = idesc(false, false, 128);  // A coef (TMEM), B = X K-major (N = 128 rows)
      bool ok = mbar_wait(bar(B_AREADY), 0, abort);
      const uint64_t d1 = sdesc(sbase + OFF_X, 0, 1024);  // X stage 0, K-major
      const uint32_t d1lo = (uint32_t)d1, d1hi = (uint32_t)(d1 >> 32);
      for (int t = 0; ok && t < T; ++t) {
        const int s = t % NS, b = t & 1;
        if (!mbar_wait(bar(B_XFULL + s), (t / NS) & 1, abort)) break;
        // buffer b still holds the residuals of tile t - 2 until its GEMM2 retires
        if (t >= 2 && !mbar_wait(bar(B_G2DONE + b), ((t >> 1) - 1) & 1, abort)) break;
        fence_after();
        const uint32_t xlo = d1lo + (uint32_t)((s * TILE_BYTES) >> 4);
        const uint32_t tH = tmem + b * 128;
#pragma unroll
        for (int part = 0; part < 2; ++part) {
          const uint32_t ta = tmem + (part ? TM_ALO : TM_AHI);
#pragma unroll
          for (int i = 0; i < KSTEPS; ++i) {
            const uint32_t koff = (i >> 2) * HALF_BYTES + (i & 3) * 32;
            mma_ta(tH, ta + 8 * i, xlo + (koff >> 4), d1hi, ID1, (part > 0 || i > 0) ? 1u : 0u);
          }
        }
        mma_commit(bar(B_HFULL + b));
      }
      // drain every MMA this thread issued before TMEM is released
      mma_commit(bar(B_DRAIN));
      volatile int never = 0;
      mbar_wait(bar(B_DRAIN), 0, &never);
    }
  } else if (warp == G2_WARP) {
    // ---------------- GEMM2 issuer: G += R(u) . X(u); rows 16i .. 16i + 15 of
    // R sit in columns 8i .. 8i + 7 of slice i / 2 (slice j starts at column 32 j)
    if (lane == 0) {
      const uint32_t ID2 = idesc(false, true, GN);  // A = R (TMEM), B = X MN-major (N = GN predictors)
      const uint32_t tG = tmem + TM_G;
      const uint64_t d2 = sdesc(sbase + OFF_X, HALF_BYTES, 1024);
      const uint32_t d2lo = (uint32_t)d2, d2hi = (uint32_t)(d2 >> 32);
      for (int u = 0; u < T; ++u) {
        const int rb = u & 1;
        if (!mbar_wait(bar(B_RFULL + rb), (u >> 1) & 1, abort)) break;
        fence_after();
        const uint32_t xlo = d2lo + (uint32_t)(((u % NS) * TILE_BYTES) >> 4);
        const uint32_t tR = tmem + rb * 128;
        const uint32_t acc0 = u > 0 ? 1u : 0u;
#pragma unroll
        for (int i = 0; i < 8; ++i)
          mma_ta(tG, tR + (i >> 1) * 32 + (i & 1) * 8, xlo + (uint32_t)((i * 2048) >> 4), d2hi, ID2, i > 0 ? 1u : acc0);
        mma_commit(bar(B_XEMPTY + u % NS));
        mma_commit(bar(B_G2DONE + rb));
      }
      mma_commit(bar(B_GDONE));
      mma_commit(bar(B_DRAIN2));
      volatile int never = 0;
      mbar_wait(bar(B_DRAIN2), 0, &never);
    }
  } else {
    // ---------------- epilogue: 16 warps, thread = (chain, 32-row slice of the tile)
    const int q = warp & 3;             // TMEM lane quadrant (fixed by warp id % 4)
    const int sub = (warp - 2) >> 2;    // rows [32 sub, 32 sub + 32) of each tile
    const int cl = q * 32 + lane;       // chain within the tile
    const int c = c0 + cl;
    const int et = threadIdx.x - 64;    // 0 .. 511
    float* ys = (float*)(smem + OFF_Y);
    // stage y - 1/2 of this row split as floats (read back as warp-wide
    // broadcasts), each group of four rows in the order (0, 2, 1, 3) that the
    // epilogue pairs them in.  Thread et writes float4 number f = et + 512 k
    // (rows 4f .. 4f + 3, from packed word f / 8: row_begin is a multiple of 128); the
    // loads of a thread's four float4 are issued together.  Rows past the data
    // have zero bits (the packed words are zero-padded), i.e. y - 1/2 = -1/2.
    {
      const uint32_t* yw = A.ybits + (row_begin >> 5);
      const int nf = T * 32;  // float4 count: 128 rows per tile
      for (int f0 = et; f0 < nf; f0 += 4 * 32 * EPI_WARPS) {
        uint32_t w[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int f = f0 + k * 32 * EPI_WARPS;
          w[k] = f < nf ? yw[f >> 3] : 0u;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int f = f0 + k * 32 * EPI_WARPS;
          const uint32_t bb = w[k] >> (4 * (f & 7));
          if (f < nf)
            reinterpret_cast<float4*>(ys)[f] = make_float4((bb & 1u) ? 0.5f : -0.5f, (bb & 4u) ? 0.5f : -0.5f,
                                                           (bb & 2u) ? 0.5f : -0.5f, (bb & 8u) ? 0.5f : -0.5f);
        }
      }
    }
    asm volatile("bar.sync 1, 512;" ::: "memory");
    // the slice sums of successive tiles are added in FP32 with Kahan
    // compensation (no FP64 instruction per tile on this part's narrow FP64
    // pipe); the thread's total becomes FP64 once, at the end
    float lp_acc = 0.f, lp_comp = 0.f;
    bool ok = true;
    for (int t = 0; t < T && ok; ++t) {
      const int b = t & 1;
      if (!mbar_wait(bar(B_HFULL + b), (t >> 1) & 1, abort)) { ok = false; break; }
      fence_after();
      float v[32];
      const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + b * 128 + sub * 32;
      tmem_ld16(ta, v);
      tmem_ld16(ta + 16, v + 16);
      tmem_wait_ld();
      const int r0 = row_begin + t * 128 + sub * 32;
      const float4* y4 = reinterpret_cast<const float4*>(ys + t * 128 + sub * 32);
      const int nvalid = row_end - r0;  // >= 32 on every tile but the last
      if (nvalid < 32) {
        // rows past the data: their X rows are TMA zero fill, so h = 0 there;
        // with h set to +0 each contributes a factor 1 + 2^0 = 2 to the
        // product and nothing to the |h| sum (R there meets a zero X row)
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = j < nvalid ? v[j] : 0.f;
      }
      // per quad of rows 0..3, pairs A = (0, 2) and B = (1, 3); products of
      // (1 + e) over alternate quads (each at most 2^16); sums of
      // t = -log2(e) |h| in pairs (|h| = -t ln 2)
      const f2 ONE2 = f2pack(1.f, 1.f), MHALF2 = f2pack(-0.5f, -0.5f);
      float pr0 = 1.f, pr1 = 1.f;
      f2 tsA = f2pack(0.f, 0.f), tsB = f2pack(0.f, 0.f);
      uint32_t hi[16];
#pragma unroll
      for (int j4 = 0; j4 < 8; ++j4) {
        const float4 yv = y4[j4];  // y - 1/2 of rows 0, 2, 1, 3
        const float x0 = v[4 * j4], x1 = v[4 * j4 + 1], x2 = v[4 * j4 + 2], x3 = v[4 * j4 + 3];
        const float t0 = -1.4426950408889634f * fabsf(x0), t1 = -1.4426950408889634f * fabsf(x1);
        const float t2 = -1.4426950408889634f * fabsf(x2), t3 = -1.4426950408889634f * fabsf(x3);
        const f2 tA = f2pack(t0, t2), tB = f2pack(t1, t3);
        const f2 dA = f2add(f2pack(ex2a(t0), ex2a(t2)), ONE2);  // (d0, d2), d = 1 + e
        const f2 dB = f2add(f2pack(ex2a(t1), ex2a(t3)), ONE2);  // (d1, d3)
        const f2 P = f2mul(dA, dB);                              // (d0 d1, d2 d3)
        float p01, p23;
        f2unpack(P, p01, p23);
        const float pq = p01 * p23;
        const float rq = rcpa(pq);
        const f2 S = f2mul(f2pack(p23, p01), f2pack(rq, rq));   // (1 / (d0 d1), 1 / (d2 d3))
        // inv_logit(|h|) - 1/2 = 1/d - 1/2, and
        // y - inv_logit(h) = (y - 1/2) - sign(h) (inv_logit(|h|) - 1/2)
        float w0, w1, w2, w3;
        f2unpack(f2fma(dB, S, MHALF2), w0, w2);
        f2unpack(f2fma(dA, S, MHALF2), w1, w3);
        float R0, R1, R2, R3;
        f2unpack(f2add(f2pack(yv.x, yv.y), f2pack(copysignf(w0, -x0), copysignf(w2, -x2))), R0, R2);
        f2unpack(f2add(f2pack(yv.z, yv.w), f2pack(copysignf(w1, -x1), copysignf(w3, -x3))), R1, R3);
        if (j4 & 1) pr1 *= pq;
        else pr0 *= pq;
        tsA = f2add(tsA, tA);
        tsB = f2add(tsB, tB);
        hi[2 * j4] = pack_bf16(R0, R1);
        hi[2 * j4 + 1] = pack_bf16(R2, R3);
      }
      {
        // this slice's even part: sum |h|/2 + ln(prod (1 + e)); each row past
        // the data contributed exactly one factor 2 and nothing to |h|
        float l2 = lg2a(pr0 * pr1);
        if (nvalid < 32) l2 -= (float)(32 - max(nvalid, 0));
        float ta0, ta1, tb0, tb1;
        f2unpack(tsA, ta0, ta1);
        f2unpack(tsB, tb0, tb1);
        const float tsum = (ta0 + ta1) + (tb0 + tb1);  // -log2(e) sum |h|
        const float yk = -fmaf(l2, 0.69314718055994531f, -0.34657359027997264f * tsum) - lp_comp;
        const float tk = lp_acc + yk;
        lp_comp = (tk - lp_acc) - yk;
        lp_acc = tk;
      }
      // the slice's residuals, two BF16 rows per column, over its first 16 columns
      tmem_st16(ta, hi);
      tmem_wait_st();
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(bar(B_RFULL + b));
    }
    // G readout: 32 columns per thread, stored in TMEM column order (position
    // k < K: beta_k, position K: intercept, zeros after) as 16-byte vectors, so
    // each thread writes 128 contiguous bytes of its chain's row
    {
      float g[32];
      const bool have = ok && T > 0 && mbar_wait(bar(B_GDONE), 0, abort);
      if (have) {
        fence_after();
        const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + TM_G + sub * 32;
        tmem_ld16(ta, g);
        tmem_ld16(ta + 16, g + 16);
        tmem_wait_ld();
      }
#pragma unroll
      for (int j = 0; j < 32; ++j) g[j] = (have && sub * 32 + j <= A.K) ? g[j] : 0.f;
      if (c < A.C && (have || T == 0)) {
        float4* pg = reinterpret_cast<float4*>(A.part_g + ((size_t)split * A.C + c) * TC_GSTRIDE + sub * 32);
#pragma unroll
        for (int j = 0; j < 8; ++j) pg[j] = make_float4(g[4 * j], g[4 * j + 1], g[4 * j + 2], g[4 * j + 3]);
      }
    }
    lpx[sub * 128 + cl] = (double)lp_acc - (double)lp_comp;
    asm volatile("bar.sync 1, 512;" ::: "memory");
    if (sub == 0 && c < A.C)
      A.part_lp[(size_t)split * A.C + c] = (lpx[cl] + lpx[128 + cl]) + (lpx[256 + cl] + lpx[384 + cl]);
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
  if (threadIdx.x == 0 && *abort) atomicExch(A.error, 1);
}

}  // namespace

struct TcPlan {
  CUtensorMap xmap;
  TcArgs args;
  dim3 grid;
  uint16_t* coef = nullptr;
  int* error = nullptr;
  double* part_lp = nullptr;
  float* part_g = nullptr;
  double* lin = nullptr;
};

bool tc_supported(const DevModel& M) {
  return M.kind == MK_LOGISTIC && M.Xtc && M.xtc_ym && M.K + 1 <= XTC_LD;
}

int tc_create(const DevModel& M, int C, const int* done_count, TcPlan** out, uint16_t** coef_bf, int* S_out,
              double** part_lp, float** part_g, double** lin, std::string& err) {
  if (!tc_supported(M)) {
    err = "tensor-core gradient needs a logistic model with at most 103 predictors";
    return GNUTS_ERR_ARGUMENT;
  }
  TcPlan* p = new TcPlan();
  const int Cpad = (C + 127) / 128 * 128;
  const int ctiles = Cpad / 128;
  // row splits: fill the 152 SMs with one CTA each
  const int ntiles = (M.N + 127) / 128;
  int S = std::max(1, 152 / ctiles);
  S = std::min(S, ntiles);
  // a split's y values are staged in shared memory: at most MAX_SPLIT_ROWS rows
  const int tiles_per_split = std::min((ntiles + S - 1) / S, MAX_SPLIT_ROWS / 128);
  S = (ntiles + tiles_per_split - 1) / tiles_per_split;
  auto fail = [&](cudaError_t e) {
    err = std::string("CUDA error: ") + cudaGetErrorString(e);
    tc_destroy(p);
    return GNUTS_ERR_CUDA;
  };
  cudaError_t e;
  if ((e = cudaMalloc(&p->coef, sizeof(uint16_t) * 2 * Cpad * 128)) != cudaSuccess) return fail(e);
  cudaMemset(p->coef, 0, sizeof(uint16_t) * 2 * Cpad * 128);
  if ((e = cudaMalloc(&p->error, sizeof(int))) != cudaSuccess) return fail(e);
  cudaMemset(p->error, 0, sizeof(int));
  if ((e = cudaMalloc(&p->part_lp, sizeof(double) * S * C)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&p->lin, sizeof(double) * C)) != cudaSuccess) return fail(e);
  cudaMemset(p->lin, 0, sizeof(double) * C);
  // padded to TC_GSTRIDE floats per chain (entries past K stay zero) so the
  // consumer sums whole 16-byte vectors
  if ((e = cudaMalloc(&p->part_g, sizeof(float) * S * C * TC_GSTRIDE)) != cudaSuccess) return fail(e);
  cudaMemset(p->part_g, 0, sizeof(float) * S * C * TC_GSTRIDE);
  int rc = make_map_bf16(&p->xmap, M.Xtc, XTC_LD, (uint64_t)M.N, XTC_LD * 2, 128, err);
  if (rc) {
    tc_destroy(p);
    return rc;
  }
  p->args = TcArgs{M.N, M.K, C, Cpad, tiles_per_split * 128, S, C, p->coef, M.ybits, p->part_lp, p->part_g,
                   done_count, p->error};
  p->grid = dim3(ctiles, S);
  if ((e = cudaFuncSetAttribute(k_glm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES)) != cudaSuccess)
    return fail(e);
  *out = p;
  *coef_bf = p->coef;
  *S_out = S;
  *part_lp = p->part_lp;
  *part_g = p->part_g;
  *lin = p->lin;
  return GNUTS_OK;
}

void tc_destroy(TcPlan* p) {
  if (!p) return;
  cudaFree(p->coef);
  cudaFree(p->error);
  cudaFree(p->part_lp);
  cudaFree(p->part_g);
  cudaFree(p->lin);
  delete p;
}

void tc_launch(const TcPlan* p, cudaStream_t stream) {
  k_glm_tc<<<p->grid, NUM_THREADS, SMEM_BYTES, stream>>>(p->xmap, p->args);
}

int tc_error(const TcPlan* p) {
  int h = 0;
  cudaMemcpy(&h, p->error, sizeof(int), cudaMemcpyDeviceToHost);
  return h;
}

}  // namespace gnuts
