// tcgen05 tensor-core kernel for the batched logistic-regression gradient.
//
// Per round every live chain c needs, for its coefficients B_c (intercept
// folded in through a ones column of X),
//     H[c, n] = B_c . X_n                       GEMM1, M = chains, N = rows, K = predictors
//     lp_c    = -sum_n softplus(s_n H[c, n]),   s_n = 1 - 2 y_n
//     R[c, n] = -s_n inv_logit(s_n H[c, n])     (= y_n - inv_logit(H[c, n]))
//     G[c, k] = sum_n R[c, n] X[n, k]           GEMM2, M = chains, N = predictors, K = rows
// which is the reverse sweep Stan Math performs for one chain's
// bernoulli_logit likelihood (log_prob_grad contract, src/cmdstan/
// command_helper.hpp:589-593), done for 128 chains at once.
//
// Precision: X is BF16-exact (the workload's design matrix is defined on
// BF16 values).  Coefficients are split hi + lo in BF16, so GEMM1 is two BF16
// MMAs accumulated in FP32 TMEM (about 16 significant bits of each
// coefficient: this is what keeps lp accurate).  Residuals enter GEMM2 in
// BF16 (relative error 2^-9 per residual, about 1e-3 on a gradient
// component); a gradient error leaves the leapfrog volume preserving and
// reversible and lp is computed separately, so it does not bias the target.
// softplus / inv_logit run in FP32; each thread sums its 32-row slice of lp
// in FP32 (four interleaved partial sums) and the slices of successive tiles
// with Kahan-compensated FP32 additions; the reduction over the 512 threads'
// totals and over row splits is FP64.
//
// CTA = one 128-chain tile x one row split, 576 threads:
//   warp 0       TMA producer: coefficient hi/lo tiles once, X row tiles
//                (2-stage ring, 128 rows x 128 predictors, SWIZZLE_128B)
//   warp 1       MMA issuer (one thread) + TMEM owner
//   warps 2..17  epilogue: thread = (chain, 32-row slice of the tile), four
//                warps per TMEM lane quadrant; reads its H slice from TMEM,
//                writes R into one of two shared-memory buffers in the SW128
//                K-major layout GEMM2 reads; y of the split is staged as floats
// TMEM: H double buffer (2 x 128 columns) + G (128 columns).  With H and R
// double-buffered, GEMM1 of tile t+1 and GEMM2 of tile t-1 run while the
// epilogue works on tile t.
// Every mbarrier wait is bounded; on expiry the kernel records an error,
// drains what it issued and frees TMEM.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstring>
#include <string>
#include "grad_tc.h"

namespace gnuts {
namespace {

constexpr int TILE_BYTES = 128 * 128 * 2;   // [2 k-halves][128 rows][64] BF16
constexpr int HALF_BYTES = TILE_BYTES / 2;  // one k-half: 128 rows x 128 B
constexpr int NS = 2;
constexpr int EPI_WARPS = 16;                 // 4 per TMEM lane quadrant, 32 rows each
constexpr int NUM_THREADS = 64 + 32 * EPI_WARPS;
constexpr int MAX_SPLIT_ROWS = 6144;          // y of a whole row split staged as floats
constexpr int OFF_CHI = 0;
constexpr int OFF_CLO = OFF_CHI + TILE_BYTES;
constexpr int OFF_X = OFF_CLO + TILE_BYTES;
constexpr int OFF_R = OFF_X + NS * TILE_BYTES;  // 2 residual buffers (BF16)
constexpr int OFF_BAR = OFF_R + 2 * TILE_BYTES;  // 16 barriers
constexpr int OFF_MISC = OFF_BAR + 16 * 8;     // tmem base, abort flag
constexpr int OFF_LP = OFF_MISC + 16;          // [4][128] doubles
constexpr int OFF_Y = OFF_LP + 4 * 128 * 8;    // [MAX_SPLIT_ROWS] floats
constexpr int SMEM_USED = OFF_Y + MAX_SPLIT_ROWS * 4;
constexpr int SMEM_BYTES = SMEM_USED + 1024;   // alignment slack
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t SPIN_LIMIT = 1u << 22;

// barrier indices
enum { B_XFULL = 0, B_XEMPTY = NS, B_CFULL = 2 * NS, B_HFULL, B_HFULL1, B_HEMPTY, B_HEMPTY1, B_RFULL, B_RFULL1,
       B_REMPTY, B_REMPTY1, B_GDONE, B_DRAIN };
static_assert(B_DRAIN < 16, "barrier area holds 16 barriers");

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// bounded wait for the phase with the given parity; false on timeout / abort
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort) {
  for (uint32_t i = 0; i < SPIN_LIMIT; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if ((i & 255u) == 255u && *abort) return false;
  }
  *abort = 1;
  return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: SWIZZLE_128B, descriptor version 1
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// instruction descriptor, kind::f16: D FP32, A/B BF16, M = 128, N = 128
__host__ __device__ constexpr uint32_t idesc(bool a_mn, bool b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
         ((128u >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// single-instruction approximations (SFU): 2^x, log2(x), 1/x
__device__ __forceinline__ float ex2a(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2a(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcpa(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

struct TcArgs {
  int N, K, C, Cpad, rows_per_split, S, C_total;
  const uint32_t* ybits;
  double* part_lp;
  float* part_g;  // [S][C][TC_GSTRIDE]: coefficient 0 = intercept, 1 + k = beta_k
  const int* done_count;
  int* error;
};

__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_glm_tc(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap cmap, TcArgs A) {
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
    mbar_init(bar(B_CFULL), 1);
    mbar_init(bar(B_HFULL), 1);
    mbar_init(bar(B_HFULL1), 1);
    mbar_init(bar(B_HEMPTY), EPI_WARPS);
    mbar_init(bar(B_HEMPTY1), EPI_WARPS);
    mbar_init(bar(B_RFULL), EPI_WARPS);
    mbar_init(bar(B_RFULL1), EPI_WARPS);
    mbar_init(bar(B_REMPTY), 1);
    mbar_init(bar(B_REMPTY1), 1);
    mbar_init(bar(B_GDONE), 1);
    mbar_init(bar(B_DRAIN), 1);
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

  if (warp == 0) {
    // ---------------- TMA producer
    if (lane == 0) {
      int issued = 0;
      mbar_expect_tx(bar(B_CFULL), 2 * TILE_BYTES);
      tma_load_2d(sbase + OFF_CHI, &cmap, 0, c0, bar(B_CFULL));
      tma_load_2d(sbase + OFF_CHI + HALF_BYTES, &cmap, 64, c0, bar(B_CFULL));
      tma_load_2d(sbase + OFF_CLO, &cmap, 0, A.Cpad + c0, bar(B_CFULL));
      tma_load_2d(sbase + OFF_CLO + HALF_BYTES, &cmap, 64, A.Cpad + c0, bar(B_CFULL));
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
        volatile int never = 0;
        mbar_wait(bar(B_CFULL), 0, &never);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t ID1 = idesc(false, false);  // A coef K-major, B = X K-major
      const uint32_t ID2 = idesc(false, true);   // A = R K-major, B = X MN-major
      const uint32_t tG = tmem + 256;
      bool ok = mbar_wait(bar(B_CFULL), 0, abort);
      // GEMM2 of tile u: G += R(u) . X(u), R in residual buffer u & 1
      auto gemm2 = [&](int u) -> bool {
        const int rb = u & 1;
        if (!mbar_wait(bar(B_RFULL + rb), (u >> 1) & 1, abort)) return false;
        fence_after();
        const uint32_t xs = sbase + OFF_X + (u % NS) * TILE_BYTES;
        const uint32_t rs = sbase + OFF_R + rb * TILE_BYTES;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          uint64_t a = sdesc(rs + (i >> 2) * HALF_BYTES + (i & 3) * 32, 0, 1024);
          uint64_t b = sdesc(xs + i * 2048, HALF_BYTES, 1024);
          mma(tG, a, b, ID2, (u > 0 || i > 0) ? 1u : 0u);
        }
        mma_commit(bar(B_XEMPTY + u % NS));
        mma_commit(bar(B_REMPTY + rb));
        return true;
      };
      int t = 0;
      for (; ok && t < T; ++t) {
        const int s = t % NS, b = t & 1;
        if (!mbar_wait(bar(B_XFULL + s), (t / NS) & 1, abort)) { ok = false; break; }
        if (t >= 2 && !mbar_wait(bar(B_HEMPTY + b), ((t >> 1) - 1) & 1, abort)) { ok = false; break; }
        fence_after();
        const uint32_t xs = sbase + OFF_X + s * TILE_BYTES;
        const uint32_t tH = tmem + b * 128;
#pragma unroll
        for (int part = 0; part < 2; ++part) {
          const uint32_t cs = sbase + (part ? OFF_CLO : OFF_CHI);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const uint32_t koff = (i >> 2) * HALF_BYTES + (i & 3) * 32;
            mma(tH, sdesc(cs + koff, 0, 1024), sdesc(xs + koff, 0, 1024), ID1, (part > 0 || i > 0) ? 1u : 0u);
          }
        }
        mma_commit(bar(B_HFULL + b));
        if (t >= 1 && !gemm2(t - 1)) { ok = false; break; }
      }
      if (ok && T > 0) ok = gemm2(T - 1);
      mma_commit(bar(B_GDONE));
      // drain every MMA this thread issued before TMEM is released
      mma_commit(bar(B_DRAIN));
      volatile int never = 0;
      mbar_wait(bar(B_DRAIN), 0, &never);
    }
  } else {
    // ---------------- epilogue: 16 warps, thread = (chain, 32-row slice of the tile)
    const int q = warp & 3;             // TMEM lane quadrant (fixed by warp id % 4)
    const int sub = (warp - 2) >> 2;    // rows [32 sub, 32 sub + 32) of each tile
    const int cl = q * 32 + lane;       // chain within the tile
    const int c = c0 + cl;
    const int et = threadIdx.x - 64;    // 0 .. 511
    float* ys = (float*)(smem + OFF_Y);
    // stage y of this row split as 0/1 floats (read back as warp-wide broadcasts)
    for (int i = et; i < T * 128; i += 32 * EPI_WARPS) {
      const int n = row_begin + i;
      ys[i] = (n < row_end && ((A.ybits[n >> 5] >> (n & 31)) & 1u)) ? 1.f : 0.f;
    }
    asm volatile("bar.sync 1, 512;" ::: "memory");
    // the slice sums of successive tiles are added in FP32 with Kahan
    // compensation (no FP64 instruction per tile on this part's narrow FP64
    // pipe); the thread's total becomes FP64 once, at the end
    float lp_acc = 0.f, lp_comp = 0.f;
    const int kh = sub >> 1;            // k-half of the R tile this slice lands in
    uint8_t* rrow = smem + OFF_R + kh * HALF_BYTES + cl * 128;
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
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(bar(B_HEMPTY + b));
      const int r0 = row_begin + t * 128 + sub * 32;
      const float4* y4 = reinterpret_cast<const float4*>(ys + t * 128 + sub * 32);
      const int nvalid = row_end - r0;  // >= 32 on every tile but the last
      float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, acc3 = 0.f;
      uint32_t hi[16];
#define GN_EPI_ELEMENT(J, Y, R, ACC)                                               \
      {                                                                            \
        const float eta = v[J];                                                    \
        const float ex = ex2a(-1.4426950408889634f * fabsf(eta));                  \
        const float d = 1.f + ex;                                                  \
        const float sp = fmaf(lg2a(d), 0.69314718055994531f, fmaxf(eta, 0.f));     \
        const float inv = rcpa(d);                                                 \
        const float sig = (eta >= 0.f ? 1.f : ex) * inv;                           \
        ACC += fmaf(Y, eta, -sp);                                                  \
        R = Y - sig;                                                               \
      }
      if (nvalid >= 32) {
#pragma unroll
        for (int j4 = 0; j4 < 8; ++j4) {
          const float4 yv = y4[j4];
          float r0v, r1v, r2v, r3v;
          GN_EPI_ELEMENT(4 * j4 + 0, yv.x, r0v, acc0)
          GN_EPI_ELEMENT(4 * j4 + 1, yv.y, r1v, acc1)
          GN_EPI_ELEMENT(4 * j4 + 2, yv.z, r2v, acc2)
          GN_EPI_ELEMENT(4 * j4 + 3, yv.w, r3v, acc3)
          hi[2 * j4] = pack_bf16(r0v, r1v);
          hi[2 * j4 + 1] = pack_bf16(r2v, r3v);
        }
      } else {
#pragma unroll
        for (int j4 = 0; j4 < 8; ++j4) {
          const float4 yv = y4[j4];
          float rv[4];
          const float yy[4] = {yv.x, yv.y, yv.z, yv.w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            float a = 0.f, r;
            GN_EPI_ELEMENT(4 * j4 + e, yy[e], r, a)
            const bool valid = 4 * j4 + e < nvalid;
            rv[e] = valid ? r : 0.f;
            acc0 += valid ? a : 0.f;
          }
          hi[2 * j4] = pack_bf16(rv[0], rv[1]);
          hi[2 * j4 + 1] = pack_bf16(rv[2], rv[3]);
        }
      }
#undef GN_EPI_ELEMENT
      {
        const float yk = ((acc0 + acc1) + (acc2 + acc3)) - lp_comp;
        const float tk = lp_acc + yk;
        lp_comp = (tk - lp_acc) - yk;
        lp_acc = tk;
      }
      // residual buffer t & 1 is free once GEMM2 of tile t - 2 has completed
      if (t >= 2 && !mbar_wait(bar(B_REMPTY + b), ((t >> 1) - 1) & 1, abort)) { ok = false; break; }
      // row cl of the K-major SW128 residual tile: 4 chunks of 8 rows' values
      uint8_t* rdst = rrow + b * TILE_BYTES;
#pragma unroll
      for (int c4 = 0; c4 < 4; ++c4) {
        const int pc = ((((sub & 1) * 4 + c4) ^ (cl & 7)) * 16);
        *reinterpret_cast<uint4*>(rdst + pc) = make_uint4(hi[4 * c4], hi[4 * c4 + 1], hi[4 * c4 + 2], hi[4 * c4 + 3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(bar(B_RFULL + b));
    }
    // G readout: 32 predictor columns per thread
    if (ok && T > 0 && mbar_wait(bar(B_GDONE), 0, abort)) {
      fence_after();
      float g[32];
      const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + 256 + sub * 32;
      tmem_ld16(ta, g);
      tmem_ld16(ta + 16, g + 16);
      tmem_wait_ld();
      if (c < A.C) {
        float* pg = A.part_g + ((size_t)split * A.C + c) * TC_GSTRIDE;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int k = sub * 32 + j;
          if (k < A.K) pg[1 + k] = g[j];
          else if (k == A.K) pg[0] = g[j];
        }
      }
    } else if (T == 0 && c < A.C) {
      float* pg = A.part_g + ((size_t)split * A.C + c) * TC_GSTRIDE;
      for (int k = sub; k <= A.K; k += 4) pg[k] = 0.f;
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

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled get_encode(std::string& err) {
  static EncodeTiled fn = nullptr;
  if (fn) return fn;
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  // the entry point as introduced (CUDA 12.0)
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
    err = "cuTensorMapEncodeTiled unavailable";
    return nullptr;
  }
  fn = (EncodeTiled)p;
  return fn;
}

int make_map(CUtensorMap* map, const void* base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
             std::string& err) {
  EncodeTiled enc = get_encode(err);
  if (!enc) return GNUTS_ERR_CUDA;
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {row_bytes};
  cuuint32_t box[2] = {64, 128};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    err = "cuTensorMapEncodeTiled failed with code " + std::to_string((int)r);
    return GNUTS_ERR_CUDA;
  }
  return GNUTS_OK;
}

}  // namespace

struct TcPlan {
  CUtensorMap xmap, cmap;
  TcArgs args;
  dim3 grid;
  uint16_t* coef = nullptr;
  int* error = nullptr;
  double* part_lp = nullptr;
  float* part_g = nullptr;
};

bool tc_supported(const DevModel& M) { return M.kind == MK_LOGISTIC && M.Xtc && M.K + 1 <= XTC_LD; }

int tc_create(const DevModel& M, int C, const int* done_count, TcPlan** out, uint16_t** coef_bf, int* S_out,
              double** part_lp, float** part_g, std::string& err) {
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
  // padded to TC_GSTRIDE floats per chain (entries past K stay zero) so the
  // consumer sums whole 16-byte vectors
  if ((e = cudaMalloc(&p->part_g, sizeof(float) * S * C * TC_GSTRIDE)) != cudaSuccess) return fail(e);
  cudaMemset(p->part_g, 0, sizeof(float) * S * C * TC_GSTRIDE);
  int rc = make_map(&p->xmap, M.Xtc, XTC_LD, (uint64_t)M.N, XTC_LD * 2, err);
  if (!rc) rc = make_map(&p->cmap, p->coef, 128, (uint64_t)2 * Cpad, 256, err);
  if (rc) {
    tc_destroy(p);
    return rc;
  }
  p->args = TcArgs{M.N, M.K, C, Cpad, tiles_per_split * 128, S, C, M.ybits, p->part_lp, p->part_g, done_count,
                   p->error};
  p->grid = dim3(ctiles, S);
  if ((e = cudaFuncSetAttribute(k_glm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES)) != cudaSuccess)
    return fail(e);
  *out = p;
  *coef_bf = p->coef;
  *S_out = S;
  *part_lp = p->part_lp;
  *part_g = p->part_g;
  return GNUTS_OK;
}

void tc_destroy(TcPlan* p) {
  if (!p) return;
  cudaFree(p->coef);
  cudaFree(p->error);
  cudaFree(p->part_lp);
  cudaFree(p->part_g);
  delete p;
}

void tc_launch(const TcPlan* p, cudaStream_t stream) {
  k_glm_tc<<<p->grid, NUM_THREADS, SMEM_BYTES, stream>>>(p->xmap, p->cmap, p->args);
}

int tc_error(const TcPlan* p) {
  int h = 0;
  cudaMemcpy(&h, p->error, sizeof(int), cudaMemcpyDeviceToHost);
  return h;
}

}  // namespace gnuts
