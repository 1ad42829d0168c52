// Affine-coupling flow kernels (forward, inverse, log-determinant, adjoint,
// parameter gradient, Adam), reverse-KL training, and the host side of the
// fused NUTS sampler in the pulled-back space (its kernels, on the tensor
// cores, are in flow_tc_kind.cu).  The map and the layouts are described in
// flow.cuh.
//
// No counterpart in the reference: CmdStan's NUTS (reached through
// stan::services::sample::hmc_nuts_diag_e_adapt, src/cmdstan/command.hpp:
// 673-688) samples the model's unconstrained space directly.  Here the same
// state machine samples z with x = T(z), and the model's own log density and
// gradient (the log_prob_grad contract, command_helper.hpp:589-593) are
// evaluated at x inside the flow kernel.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>
#include "internal.h"
#include "flow.cuh"
#include "nuts_device.cuh"

namespace gnuts {

#define FL_CUDA(call)                                                                        \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      err = std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call;            \
      return GNUTS_ERR_CUDA;                                                                 \
    }                                                                                        \
  } while (0)

enum FlowMode : int { FM_FWD = 0, FM_GRAD = 1, FM_TRAIN = 2 };

struct FlowIO {
  int n;
  const double* z;   // [n][ldz] input points; null: Philox base draws (training)
  int ldz;
  const Scal* sc;    // sampling: skip the points of finished chains
  uint32_t seed;     // base draws: Philox(seed, point, stream 2, step * ceil(d/2) + i/2)
  int step;
  float base_scale;  // base draws are base_scale * N(0, 1)
  double beta;       // TRAIN: objective beta * lp_x + log|det| (tempered target while annealing)
  int jac;
  int with_model;    // FM_FWD: evaluate the model at x as well
  double* x;         // [n][d] T(z) (may be null)
  double* logdet;    // [n] (may be null)
  double* lp;        // [n] lp_x + log|det| (GRAD/TRAIN), may be null
  double* g;         // [n][ldg] gradient in z (GRAD/TRAIN), may be null
  int ldg;
  double* lpx;       // [n] lp_x at T(z), may be null
  float* fac;        // TRAIN: per-layer factors of the parameter gradient
  float* loss;       // TRAIN: -(lp_x + log|det|) per point
  int* valid;        // TRAIN: 1 if the point's loss and gradient are finite
  int* nvalid;       // TRAIN: count of valid points
  double* draw_rows; // FM_FWD with model: row p gets lp__ = lp_x and write_array(x) from column 7
  int draw_ncol;
};

// ---------------------------------------------------------------- helpers
template <int HPL>
__device__ __forceinline__ void ld_bf(const __nv_bfloat16* p, float* f) {
  if constexpr (HPL == 4) {
    const uint2 v = *reinterpret_cast<const uint2*>(p);
    f[0] = __uint_as_float(v.x << 16);
    f[1] = __uint_as_float(v.x & 0xffff0000u);
    f[2] = __uint_as_float(v.y << 16);
    f[3] = __uint_as_float(v.y & 0xffff0000u);
  } else if constexpr (HPL == 2) {
    const uint32_t v = *reinterpret_cast<const uint32_t*>(p);
    f[0] = __uint_as_float(v << 16);
    f[1] = __uint_as_float(v & 0xffff0000u);
  } else {
    const uint32_t v = *reinterpret_cast<const uint16_t*>(p);
    f[0] = __uint_as_float(v << 16);
  }
}


// stage s < L: forward layer s -> [W2 | W1]; stage s >= L: adjoint layer 2L-1-s -> [W1 | W2^T]
__device__ __forceinline__ void issue_stage(const FlowDev& F, int s, __nv_bfloat16* buf) {
  const int l = s < F.L ? s : 2 * F.L - 1 - s;
  const long H = F.H, nb = F.nb[l], na = F.na[l];
  const __nv_bfloat16* src = F.w16 + F.w_off[l] + (s < F.L ? 0 : H * 2 * na);
  const long n = H * 2 * na + nb * H;
  const int chunks = (int)(n / 8);
  for (int i = threadIdx.x; i < chunks; i += blockDim.x) fl_cp16(buf + 8 * (size_t)i, src + 8 * (size_t)i);
}

__device__ __forceinline__ int flow_namax(const FlowDev& F) {
  int m = 0;
  for (int l = 0; l < F.L; ++l) m = F.na[l] > m ? F.na[l] : m;
  return m;
}
__device__ __forceinline__ int tape_off(const FlowDev& F, int l) {
  int t = 0;
  for (int k = 0; k < l; ++k) t += F.d + F.H + F.na[k];
  return t;
}
// factor block of layer l (l == L: the final [xbar | u_L] block) for n points
__device__ __forceinline__ size_t fac_off(const FlowDev& F, int l, int n) {
  size_t o = 0;
  for (int k = 0; k < l; ++k) o += (size_t)n * (F.nb[k] + 2 * F.H + 2 * F.na[k]);
  return o;
}

// conditioner of layer l on the current vector y: h (H) into th, raw outputs
// (2 n_a: log-scale pre-activations, then shifts) into sc.  W1 [n_b][H] and
// W2 [H][2 n_a] may be in shared or global memory.
template <int HPL>
__device__ __forceinline__ void conditioner(const FlowDev& F, int l, const __nv_bfloat16* W1,
                                            const __nv_bfloat16* W2, const int* bi, const float* y, float* th,
                                            float* sc, int lane) {
  const int H = F.H, nb = F.nb[l], na = F.na[l];
  const float* b1 = F.theta + F.th_off[l] + (long)nb * H;
  const float* b2 = b1 + H + (long)H * 2 * na;
  const int j0 = HPL * lane;
  float acc[HPL];
#pragma unroll
  for (int k = 0; k < HPL; ++k) acc[k] = b1[j0 + k];
  int r = 0;
  for (; r + 4 <= nb; r += 4) {
    float w[4][HPL], u[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      ld_bf<HPL>(W1 + (size_t)(r + q) * H + j0, w[q]);
      u[q] = y[bi[r + q]];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int k = 0; k < HPL; ++k) acc[k] = fmaf(w[q][k], u[q], acc[k]);
  }
  for (; r < nb; ++r) {
    float w[HPL];
    ld_bf<HPL>(W1 + (size_t)r * H + j0, w);
    const float u = y[bi[r]];
#pragma unroll
    for (int k = 0; k < HPL; ++k) acc[k] = fmaf(w[k], u, acc[k]);
  }
#pragma unroll
  for (int k = 0; k < HPL; ++k) th[j0 + k] = tanhf(acc[k]);
  __syncwarp();
  const int n2 = 2 * na;
  float o[4];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int c = 2 * lane + 64 * q;
    o[2 * q] = c < n2 ? b2[c] : 0.f;
    o[2 * q + 1] = c < n2 ? b2[c + 1] : 0.f;
  }
#pragma unroll 4
  for (int j = 0; j < H; ++j) {
    const float hj = th[j];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int c = 2 * lane + 64 * q;
      if (c < n2) {
        const uint32_t v = *reinterpret_cast<const uint32_t*>(W2 + (size_t)j * n2 + c);
        o[2 * q] = fmaf(__uint_as_float(v << 16), hj, o[2 * q]);
        o[2 * q + 1] = fmaf(__uint_as_float(v & 0xffff0000u), hj, o[2 * q + 1]);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int c = 2 * lane + 64 * q;
    if (c < n2) {
      sc[c] = o[2 * q];
      sc[c + 1] = o[2 * q + 1];
    }
  }
  __syncwarp();
}

// forward layer l: records u (input), h and s on the tape, updates y in place
template <int HPL>
__device__ __forceinline__ void fwd_layer(const FlowDev& F, int l, const __nv_bfloat16* buf, const int* bi,
                                          const int* ai, float* y, float* tu, float* th, float* ts, float* sc,
                                          double& ld, int lane) {
  const int H = F.H, na = F.na[l];
  for (int i = lane; i < F.d; i += 32) tu[i] = y[i];
  conditioner<HPL>(F, l, buf + (size_t)H * 2 * na, buf, bi, y, th, sc, lane);
  for (int m = lane; m < na; m += 32) {
    const float s = F.clamp * tanhf(sc[m] / F.clamp);
    const int a = ai[m];
    ts[m] = s;
    y[a] = fmaf(y[a], expf(s), sc[na + m]);
    ld += (double)s;
  }
  __syncwarp();
}

// adjoint of layer l: yb holds d(objective)/d(u_{l+1}) on entry and
// d(objective)/d(u_l) on exit (objective = lp_x + log|det|).  sc receives the
// output adjoints (log-scale pre-activations, shifts), pb the hidden
// pre-activation adjoints; with TRAIN they are written to the factor row.
template <int HPL, bool TRAIN>
__device__ __forceinline__ void adj_layer(const FlowDev& F, int l, const __nv_bfloat16* buf, const int* bi,
                                          const int* ai, float* yb, const float* tu, const float* th,
                                          const float* ts, float* sc, float* pb, float* frow, int lane) {
  const int H = F.H, nb = F.nb[l], na = F.na[l], n2 = 2 * na;
  const float cl = F.clamp;
  for (int m = lane; m < na; m += 32) {
    const int a = ai[m];
    const float s = ts[m], es = expf(s), g = yb[a], ua = tu[a];
    const float q = s / cl;
    sc[m] = fmaf(g * ua, es, 1.0f) * (1.0f - q * q);
    sc[na + m] = g;
    yb[a] = g * es;
  }
  __syncwarp();
  const __nv_bfloat16* W1 = buf;
  const __nv_bfloat16* W2T = buf + (size_t)nb * H;
  const int j0 = HPL * lane;
  float hb[HPL];
#pragma unroll
  for (int k = 0; k < HPL; ++k) hb[k] = 0.f;
#pragma unroll 4
  for (int m = 0; m < n2; ++m) {
    float w[HPL];
    ld_bf<HPL>(W2T + (size_t)m * H + j0, w);
    const float r = sc[m];
#pragma unroll
    for (int k = 0; k < HPL; ++k) hb[k] = fmaf(w[k], r, hb[k]);
  }
  float pk[HPL];
#pragma unroll
  for (int k = 0; k < HPL; ++k) {
    const float h = th[j0 + k];
    pk[k] = hb[k] * (1.0f - h * h);
    pb[j0 + k] = pk[k];
  }
  // u_b adjoint += W1 pbar: 16 rows per pass; the two half-warps' partials
  // are folded, then a reduce-scatter over 16 lanes leaves the sum of row
  // r0 + (L mod 16) on lane L (31 shuffles per 16 rows, 16 registers)
  for (int r0 = 0; r0 < nb; r0 += 16) {
    float part[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float t = 0.f;
      if (r0 + q < nb) {
        float w[HPL];
        ld_bf<HPL>(W1 + (size_t)(r0 + q) * H + j0, w);
#pragma unroll
        for (int k = 0; k < HPL; ++k) t = fmaf(w[k], pk[k], t);
      }
      part[q] = t;
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) part[q] += __shfl_xor_sync(0xffffffffu, part[q], 16);
#pragma unroll
    for (int off = 8; off >= 1; off >>= 1) {
      const bool up = (lane & off) != 0;
#pragma unroll
      for (int i = 0; i < off; ++i) {
        const float send = up ? part[i] : part[i + off];
        const float keep = up ? part[i + off] : part[i];
        part[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
      }
    }
    if (lane < 16 && r0 + lane < nb) yb[bi[r0 + lane]] += part[0];
  }
  __syncwarp();
  if (TRAIN) {
    float* fu = frow;
    float* fp = fu + nb;
    float* fh = fp + H;
    float* fr = fh + H;
    for (int r = lane; r < nb; r += 32) fu[r] = tu[bi[r]];
    for (int j = lane; j < H; j += 32) {
      fp[j] = pb[j];
      fh[j] = th[j];
    }
    for (int m = lane; m < n2; m += 32) fr[m] = sc[m];
  }
}

// ---------------------------------------------------------------- the flow kernel
template <int HPL, int MODE>
__global__ void __launch_bounds__(128) k_flow(FlowDev Fp, DevModel M, FlowIO io) {
  extern __shared__ __align__(16) unsigned char fsm[];
  // the per-layer tables are indexed by a runtime layer number: from shared
  // memory, not from a local-memory copy of the parameter block
  __shared__ FlowDev Fsh;
  if (threadIdx.x == 0) Fsh = Fp;
  __syncthreads();
  const FlowDev& F = Fsh;
  const int T = blockDim.x >> 5;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int d = F.d, H = F.H, L = F.L;
  const int namax = flow_namax(F);
  const size_t idx_bytes = flow_align16(sizeof(int) * (size_t)L * d);
  const size_t wbuf_bytes = flow_align16(2 * (size_t)F.stage_max);
  const size_t warp_bytes = flow_warp_bytes(F, namax);
  int* sidx = reinterpret_cast<int*>(fsm);
  __nv_bfloat16* wbuf0 = reinterpret_cast<__nv_bfloat16*>(fsm + idx_bytes);
  __nv_bfloat16* wbuf1 = reinterpret_cast<__nv_bfloat16*>(fsm + idx_bytes + wbuf_bytes);
  unsigned char* wr = fsm + idx_bytes + 2 * wbuf_bytes + (size_t)w * warp_bytes;
  double* x = reinterpret_cast<double*>(wr);
  double* gx = x + d;
  float* y = reinterpret_cast<float*>(gx + d);
  float* yb = y + d;
  float* sc = yb + d;
  const int scn = 2 * namax > H ? 2 * namax : H;
  float* pb = sc + scn;
  float* tape = pb + H;
  const int tape_total = tape_off(F, L);
  float* uL = tape + tape_total;

  const int p = blockIdx.x * T + w;
  bool active = p < io.n;
  if (MODE == FM_GRAD && active && io.sc) active = io.sc[p].phase < PH_DONE;

  issue_stage(F, 0, wbuf0);
  fl_commit();
  for (int i = threadIdx.x; i < L * d; i += blockDim.x) sidx[i] = F.idx[i];

  double ld = 0;
  if (active) {
    if (io.z) {
      for (int i = lane; i < d; i += 32) y[i] = (float)io.z[(size_t)p * io.ldz + i];
    } else {
      const uint64_t base = (uint64_t)io.step * (uint64_t)((d + 1) / 2);
      for (int i = lane; i < d; i += 32)
        y[i] = io.base_scale * (float)rng_normal(io.seed, (uint32_t)p, 2u, base + (i >> 1), i & 1);
    }
  }
  __syncwarp();
  const float* mu = F.theta + F.th_off[L];
  const float* rho = F.theta + F.th_rho;
  double lp = 0, lpx = 0;
  const int S = MODE == FM_FWD ? L : 2 * L;
  for (int s = 0; s < S; ++s) {
    if (s + 1 < S) {
      issue_stage(F, s + 1, (s + 1) & 1 ? wbuf1 : wbuf0);
      fl_commit();
      fl_wait<1>();
    } else {
      fl_wait<0>();
    }
    __syncthreads();
    const __nv_bfloat16* buf = s & 1 ? wbuf1 : wbuf0;
    if (active) {
      if (s < L) {
        const int to = tape_off(F, s);
        fwd_layer<HPL>(F, s, buf, sidx + s * d, sidx + s * d + F.nb[s], y, tape + to, tape + to + d,
                       tape + to + d + H, sc, ld, lane);
      } else {
        if (s == L) {
          // x = mu + exp(rho) u_L, the model at x, and the adjoint seed
          for (int i = lane; i < d; i += 32) {
            uL[i] = y[i];
            x[i] = (double)mu[i] + exp((double)rho[i]) * (double)y[i];
            ld += (double)rho[i];
          }
          __syncwarp();
          lpx = warp_log_prob_grad(M, x, gx, io.jac, lane);
          __syncwarp();
          if (MODE == FM_TRAIN && io.beta != 1.0) {
            lpx *= io.beta;
            for (int i = lane; i < d; i += 32) gx[i] *= io.beta;
            __syncwarp();
          }
          lp = lpx + wsum(ld);
          for (int i = lane; i < d; i += 32) yb[i] = (float)(gx[i] * exp((double)rho[i]));
          __syncwarp();
        }
        const int l = 2 * L - 1 - s;
        const int to = tape_off(F, l);
        float* frow = nullptr;
        if (MODE == FM_TRAIN)
          frow = io.fac + fac_off(F, l, io.n) + (size_t)p * (F.nb[l] + 2 * H + 2 * F.na[l]);
        adj_layer<HPL, MODE == FM_TRAIN>(F, l, buf, sidx + l * d, sidx + l * d + F.nb[l], yb, tape + to,
                                         tape + to + d, tape + to + d + H, sc, pb, frow, lane);
      }
    }
    __syncthreads();
  }
  if (!active) return;
  if (MODE == FM_FWD) {
    for (int i = lane; i < d; i += 32) {
      x[i] = (double)mu[i] + exp((double)rho[i]) * (double)y[i];
      ld += (double)rho[i];
    }
    __syncwarp();
    const double ldt = wsum(ld);
    if (io.x)
      for (int i = lane; i < d; i += 32) io.x[(size_t)p * d + i] = x[i];
    if (io.logdet && lane == 0) io.logdet[p] = ldt;
    if (io.with_model) {
      const double lx = warp_log_prob_grad(M, x, gx, io.jac, lane);
      __syncwarp();
      if (io.lpx && lane == 0) io.lpx[p] = lx;
      if (io.draw_rows) {
        double* row = io.draw_rows + (size_t)p * io.draw_ncol;
        if (lane == 0) row[0] = lx;
        warp_write_array(M, x, row + 7, lane);
      }
    }
    return;
  }
  // gradient in z = adjoint of u_0
  bool fin = isfinite(lp);
  for (int i = lane; i < d; i += 32) fin = fin && isfinite(yb[i]);
  fin = wall(fin);
  if (io.g)
    for (int i = lane; i < d; i += 32) io.g[(size_t)p * io.ldg + i] = (double)yb[i];
  if (lane == 0) {
    if (io.lp) io.lp[p] = lp;
    if (io.lpx) io.lpx[p] = lpx;
  }
  if (io.x)
    for (int i = lane; i < d; i += 32) io.x[(size_t)p * d + i] = x[i];
  if (MODE == FM_TRAIN) {
    float* fb = io.fac + fac_off(F, L, io.n) + (size_t)p * 2 * d;
    for (int i = lane; i < d; i += 32) {
      fb[i] = (float)gx[i];
      fb[d + i] = uL[i];
    }
    if (lane == 0) {
      io.loss[p] = (float)(-lp);
      io.valid[p] = fin ? 1 : 0;
      if (fin) atomicAdd(io.nvalid, 1);
    }
  }
}

// ---------------------------------------------------------------- inverse
// x -> z, one warp per point, weights read from global memory (used once per
// chain to map starting points into the pulled-back space)
template <int HPL>
__global__ void __launch_bounds__(128) k_flow_inverse(FlowDev F, int n, const double* x, double* z, double* logdet) {
  extern __shared__ __align__(16) unsigned char fsm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int p = blockIdx.x * (blockDim.x >> 5) + w;
  const int d = F.d, H = F.H, L = F.L;
  const int namax = flow_namax(F);
  const int scn = 2 * namax > H ? 2 * namax : H;
  float* y = reinterpret_cast<float*>(fsm) + (size_t)w * (d + H + scn);
  float* th = y + d;
  float* sc = th + H;
  if (p >= n) return;
  const float* mu = F.theta + F.th_off[L];
  const float* rho = F.theta + F.th_rho;
  double ld = 0;
  for (int i = lane; i < d; i += 32) {
    y[i] = (float)((x[(size_t)p * d + i] - (double)mu[i]) * exp(-(double)rho[i]));
    ld += (double)rho[i];
  }
  __syncwarp();
  for (int l = L - 1; l >= 0; --l) {
    const int na = F.na[l];
    const int* bi = F.idx + l * d;
    const int* ai = bi + F.nb[l];
    const __nv_bfloat16* blk = F.w16 + F.w_off[l];
    conditioner<HPL>(F, l, blk + (size_t)H * 2 * na, blk, bi, y, th, sc, lane);
    for (int m = lane; m < na; m += 32) {
      const float s = F.clamp * tanhf(sc[m] / F.clamp);
      const int a = ai[m];
      y[a] = (y[a] - sc[na + m]) * expf(-s);
      ld += (double)s;
    }
    __syncwarp();
  }
  for (int i = lane; i < d; i += 32) z[(size_t)p * d + i] = (double)y[i];
  ld = wsum(ld);
  if (lane == 0 && logdet) logdet[p] = ld;
}

// ---------------------------------------------------------------- parameters
// parameter i -> (layer, kind, a, b); kind 0 W1[a][b], 1 b1[a], 2 W2[a][b],
// 3 b2[a], 4 mu[a], 5 rho[a]
__device__ __forceinline__ int flow_decode(const FlowDev& F, long i, int& l, int& a, int& b) {
  if (i >= F.th_rho) { a = (int)(i - F.th_rho); l = -1; b = 0; return 5; }
  if (i >= F.th_off[F.L]) { a = (int)(i - F.th_off[F.L]); l = -1; b = 0; return 4; }
  l = 0;
  while (l + 1 < F.L && i >= F.th_off[l + 1]) ++l;
  long o = i - F.th_off[l];
  const long H = F.H, nb = F.nb[l], n2 = 2 * (long)F.na[l];
  if (o < nb * H) { a = (int)(o / H); b = (int)(o % H); return 0; }
  o -= nb * H;
  if (o < H) { a = (int)o; b = 0; return 1; }
  o -= H;
  if (o < H * n2) { a = (int)(o / n2); b = (int)(o % n2); return 2; }
  o -= H * n2;
  a = (int)o;
  b = 0;
  return 3;
}

// BF16 copies of weight parameter i (forward and transposed layouts)
__device__ __forceinline__ void flow_put_w16(const FlowDev& F, int kind, int l, int a, int b, float v,
                                             __nv_bfloat16* w16, __nv_bfloat16* w16t) {
  if (kind != 0 && kind != 2) return;
  const long H = F.H, nb = F.nb[l], n2 = 2 * (long)F.na[l];
  __nv_bfloat16* blk = w16 + F.w_off[l];
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  // tensor-core blocks: F1 [H][kb+8], F2 [ma][H+8], A3 [H][ma+8], A4 [kb][H+8]
  const long sb = tc_pad16((int)nb) + 8, sa = tc_pad16((int)n2) + 8, sh = H + 8;
  __nv_bfloat16* f1 = w16t + F.wt_off[l];
  __nv_bfloat16* f2 = f1 + H * sb;
  __nv_bfloat16* a3 = f2 + (long)tc_pad16((int)n2) * sh;
  __nv_bfloat16* a4 = a3 + H * sa;
  if (kind == 0) {
    blk[H * n2 + (long)a * H + b] = h;  // W1 [r][j]
    f1[(long)b * sb + a] = h;
    a4[(long)a * sh + b] = h;
  } else {
    blk[(long)a * n2 + b] = h;                // W2 [j][m]
    blk[H * n2 + nb * H + (long)b * H + a] = h;  // W2^T [m][j]
    f2[(long)b * sh + a] = h;
    a3[(long)a * sa + b] = h;
  }
}

__global__ void k_flow_sync_w16(FlowDev F, __nv_bfloat16* w16, __nv_bfloat16* w16t) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < F.th_off[F.L]; i += (long)gridDim.x * blockDim.x) {
    int l, a, b;
    const int kind = flow_decode(F, i, l, a, b);
    flow_put_w16(F, kind, l, a, b, F.theta[i], w16, w16t);
  }
}

// sum over valid points of d(lp_x + log|det|)/d(theta_i)
__global__ void k_flow_pgrad(FlowDev F, int n, const float* fac, const int* valid, float* grad) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= F.n_params) return;
  int l, a, b;
  const int kind = flow_decode(F, i, l, a, b);
  float acc = 0.f;
  if (kind >= 4) {
    const float* blk = fac + fac_off(F, F.L, n);
    const int d = F.d;
    const float sig = expf(F.theta[F.th_rho + a]);
    for (int p = 0; p < n; ++p) {
      if (!valid[p]) continue;
      const float* r = blk + (size_t)p * 2 * d;
      acc += kind == 4 ? r[a] : fmaf(r[a] * sig, r[d + a], 1.0f);
    }
  } else {
    const int H = F.H, nb = F.nb[l], n2 = 2 * F.na[l];
    const size_t stride = (size_t)nb + 2 * H + n2;
    const float* blk = fac + fac_off(F, l, n);
    for (int p = 0; p < n; ++p) {
      if (!valid[p]) continue;
      const float* r = blk + (size_t)p * stride;  // [u_b | pbar | h | rbar]
      switch (kind) {
        case 0: acc = fmaf(r[a], r[nb + b], acc); break;
        case 1: acc += r[nb + a]; break;
        case 2: acc = fmaf(r[nb + H + a], r[nb + 2 * H + b], acc); break;
        default: acc += r[nb + 2 * H + a]; break;
      }
    }
  }
  grad[i] = acc;
}

// Adam (Kingma & Ba 2015, bias-corrected) on the FP32 master parameters; the
// step's gradient is grad * scale, scale = -1 / (valid points) when nvalid is
// given (gradient of the mean loss), else 1.  Weight matrices are re-rounded
// into their BF16 copies.
__global__ void k_flow_adam(FlowDev F, float* theta, float* m, float* v, const float* grad, const int* nvalid,
                            int t, float lr, float b1, float b2, float eps, __nv_bfloat16* w16,
                            __nv_bfloat16* w16t) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= F.n_params) return;
  float scale = 1.0f;
  if (nvalid) {
    const int nv = *nvalid;
    if (nv <= 0) return;
    scale = -1.0f / (float)nv;
  }
  const float g = grad[i] * scale;
  const float mi = b1 * m[i] + (1.0f - b1) * g;
  const float vi = b2 * v[i] + (1.0f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
  const float th = theta[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  theta[i] = th;
  int l, a, b;
  const int kind = flow_decode(F, i, l, a, b);
  flow_put_w16(F, kind, l, a, b, th, w16, w16t);
}

__global__ void k_flow_loss_mean(int n, const float* loss, const int* valid, double* out) {
  __shared__ double s[256];
  __shared__ int c[256];
  double t = 0;
  int k = 0;
  for (int p = threadIdx.x; p < n; p += blockDim.x)
    if (valid[p]) {
      t += loss[p];
      ++k;
    }
  s[threadIdx.x] = t;
  c[threadIdx.x] = k;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s[threadIdx.x] += s[threadIdx.x + o];
      c[threadIdx.x] += c[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = c[0] ? s[0] / c[0] : __longlong_as_double(0x7ff8000000000000ll);
}

// ---------------------------------------------------------------- host side
Flow::~Flow() {
  for (void* p : {(void*)theta, (void*)adam_m, (void*)adam_v, (void*)grad, (void*)w16, (void*)w16t, (void*)didx,
                  (void*)nvalid})
    if (p) cudaFree(p);
}

namespace {

FlowDev dev_of(const Flow& f) {
  FlowDev F{};
  F.d = f.d;
  F.L = f.L;
  F.H = f.H;
  F.clamp = f.clamp;
  for (int l = 0; l < f.L; ++l) {
    F.nb[l] = f.nb[l];
    F.na[l] = f.na[l];
    F.idx_off[l] = f.idx_off[l];
    F.th_off[l] = f.th_off[l];
    F.w_off[l] = f.w_off[l];
  }
  F.th_off[f.L] = f.th_off[f.L];
  F.th_rho = f.th_rho;
  F.n_params = f.n_params;
  F.stage_max = f.stage_max;
  for (int l = 0; l < f.L; ++l) F.wt_off[l] = f.wt_off[l];
  F.stage_max_tc = f.stage_max_tc;
  F.idx = f.didx;
  F.theta = f.theta;
  F.w16 = reinterpret_cast<const __nv_bfloat16*>(f.w16);
  F.w16t = reinterpret_cast<const __nv_bfloat16*>(f.w16t);
  return F;
}

int ensure_flow_device(Flow& f, std::string& err) {
  if (f.device >= 0) return GNUTS_OK;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    err = "no CUDA device available (the flow runs on the GPU only)";
    return GNUTS_ERR_CUDA;
  }
  FL_CUDA(cudaMalloc(&f.theta, sizeof(float) * f.n_params));
  FL_CUDA(cudaMalloc(&f.adam_m, sizeof(float) * f.n_params));
  FL_CUDA(cudaMalloc(&f.adam_v, sizeof(float) * f.n_params));
  FL_CUDA(cudaMalloc(&f.grad, sizeof(float) * f.n_params));
  FL_CUDA(cudaMalloc(&f.w16, sizeof(uint16_t) * f.n_w16));
  FL_CUDA(cudaMalloc(&f.w16t, sizeof(uint16_t) * f.n_w16t));
  FL_CUDA(cudaMemset(f.w16t, 0, sizeof(uint16_t) * f.n_w16t));  // padding stays zero
  FL_CUDA(cudaMalloc(&f.didx, sizeof(int) * f.idx.size()));
  FL_CUDA(cudaMalloc(&f.nvalid, sizeof(int) * 2));
  FL_CUDA(cudaMemset(f.theta, 0, sizeof(float) * f.n_params));
  FL_CUDA(cudaMemset(f.adam_m, 0, sizeof(float) * f.n_params));
  FL_CUDA(cudaMemset(f.adam_v, 0, sizeof(float) * f.n_params));
  FL_CUDA(cudaMemset(f.w16, 0, sizeof(uint16_t) * f.n_w16));
  FL_CUDA(cudaMemset(f.nvalid, 0, sizeof(int) * 2));
  FL_CUDA(cudaMemcpy(f.didx, f.idx.data(), sizeof(int) * f.idx.size(), cudaMemcpyHostToDevice));
  cudaGetDevice(&f.device);
  return GNUTS_OK;
}

int configure_flow(const Flow& f, std::string& err);

template <class T>
struct DevBuf {
  T* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)); }
};

constexpr size_t FLOW_SMEM_LIMIT = 220 * 1024;

#define FLOW_KIND_SWITCH(kind, CALL)               \
  switch (kind) {                                  \
    case MK_BERNOULLI: return CALL(MK_BERNOULLI);   \
    case MK_NORMAL: return CALL(MK_NORMAL);         \
    case MK_LOGISTIC: return CALL(MK_LOGISTIC);     \
    case MK_HIER: return CALL(MK_HIER);             \
    case MK_FUNNEL: return CALL(MK_FUNNEL);         \
    case MK_VARINT: return CALL(MK_VARINT);         \
    case MK_HORSESHOE: return CALL(MK_HORSESHOE);   \
  }                                                \
  return cudaErrorInvalidValue

cudaError_t flow_tc_fused_launch(int kind, const FlowDev& F, const Params& P, const Bufs& B, const DevModel& M,
                                 int T, size_t flow_bytes, int blocks, size_t smem) {
#define CALL(K) flow_tc_fused_launch_k<K>(F, P, B, M, T, flow_bytes, blocks, smem)
  FLOW_KIND_SWITCH(kind, CALL);
#undef CALL
}

cudaError_t flow_tc_grad_launch(int kind, const FlowDev& F, const DevModel& M, int n, int T, const double* z,
                                double* lp, double* g, size_t smem) {
#define CALL(K) flow_tc_grad_launch_k<K>(F, M, n, T, z, lp, g, smem)
  FLOW_KIND_SWITCH(kind, CALL);
#undef CALL
}

// shared-memory opt-in of the flow kernels for this flow's plan; called
// before any launch (and outside stream capture)
template <int HPL>
int configure_hpl(size_t bytes, std::string& err) {
  FL_CUDA(cudaFuncSetAttribute(k_flow<HPL, FM_FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  FL_CUDA(cudaFuncSetAttribute(k_flow<HPL, FM_GRAD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  FL_CUDA(cudaFuncSetAttribute(k_flow<HPL, FM_TRAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return GNUTS_OK;
}

int configure_flow(const Flow& f, std::string& err) {
  const FlowPlan plan = flow_plan(dev_of(f), FLOW_SMEM_LIMIT);
  if (plan.T == 0) {
    err = "flow does not fit in shared memory";
    return GNUTS_ERR_ARGUMENT;
  }
  if (f.H == 128) return configure_hpl<4>(plan.total, err);
  if (f.H == 64) return configure_hpl<2>(plan.total, err);
  return configure_hpl<1>(plan.total, err);
}

template <int MODE>
int launch_flow_mode(const Flow& f, const DevModel& M, const FlowIO& io, cudaStream_t st, std::string& err) {
  const FlowDev F = dev_of(f);
  const FlowPlan plan = flow_plan(F, FLOW_SMEM_LIMIT);
  if (plan.T == 0) {
    err = "flow does not fit in shared memory";
    return GNUTS_ERR_ARGUMENT;
  }
  if (io.n <= 0) return GNUTS_OK;
  const int blocks = (io.n + plan.T - 1) / plan.T;
  switch (f.H) {
    case 128: k_flow<4, MODE><<<blocks, 32 * plan.T, plan.total, st>>>(F, M, io); break;
    case 64: k_flow<2, MODE><<<blocks, 32 * plan.T, plan.total, st>>>(F, M, io); break;
    default: k_flow<1, MODE><<<blocks, 32 * plan.T, plan.total, st>>>(F, M, io); break;
  }
  FL_CUDA(cudaGetLastError());
  return GNUTS_OK;
}

// launches one flow kernel; configure_flow must have run for this flow
int launch_flow(const Flow& f, const DevModel& M, int mode, const FlowIO& io, cudaStream_t st, std::string& err) {
  if (mode == FM_FWD) return launch_flow_mode<FM_FWD>(f, M, io, st, err);
  if (mode == FM_GRAD) return launch_flow_mode<FM_GRAD>(f, M, io, st, err);
  return launch_flow_mode<FM_TRAIN>(f, M, io, st, err);
}

}  // namespace

int flow_create(int d, int L, int H, double clamp, Flow** out, std::string& err) {
  if (d < 2 || d > FLOW_MAX_D) {
    err = "flow dimension must be in 2.." + std::to_string(FLOW_MAX_D);
    return GNUTS_ERR_ARGUMENT;
  }
  if (L < 1 || L > FLOW_MAX_L) {
    err = "flow layers must be in 1.." + std::to_string(FLOW_MAX_L);
    return GNUTS_ERR_ARGUMENT;
  }
  if (H != 32 && H != 64 && H != 128) {
    err = "flow hidden width must be 32, 64 or 128";
    return GNUTS_ERR_ARGUMENT;
  }
  if (!(clamp > 0)) {
    err = "flow log-scale clamp must be > 0";
    return GNUTS_ERR_ARGUMENT;
  }
  Flow* f = new Flow();
  f->d = d;
  f->L = L;
  f->H = H;
  f->clamp = (float)clamp;
  int B = 0;
  while ((1 << B) < d) ++B;
  long o = 0, wo = 0;
  for (int l = 0; l < L; ++l) {
    const int k = l % B, pol = (l / B) & 1;
    std::vector<int> b, a;
    for (int i = 0; i < d; ++i) (((i >> k) & 1) == pol ? b : a).push_back(i);
    f->nb.push_back((int)b.size());
    f->na.push_back((int)a.size());
    f->idx_off.push_back((int)f->idx.size());
    f->idx.insert(f->idx.end(), b.begin(), b.end());
    f->idx.insert(f->idx.end(), a.begin(), a.end());
    f->th_off.push_back(o);
    const long nb = (long)b.size(), n2 = 2 * (long)a.size();
    o += nb * H + H + (long)H * n2 + n2;
    f->w_off.push_back(wo);
    wo += (long)H * n2 + nb * H + n2 * H;
    f->stage_max = std::max<int>(f->stage_max, (int)((long)H * n2 + nb * H));
    const long tf = tc_fwd_elems(H, (int)nb, (int)a.size()), ta = tc_adj_elems(H, (int)nb, (int)a.size());
    f->wt_off.push_back(f->n_w16t);
    f->n_w16t += tf + ta;
    f->stage_max_tc = std::max<int>(f->stage_max_tc, (int)std::max(tf, ta));
  }
  f->th_off.push_back(o);
  f->th_rho = o + d;
  f->n_params = o + 2 * (long)d;
  f->n_w16 = wo;
  *out = f;
  return GNUTS_OK;
}

int flow_set_params(Flow& f, const double* theta, std::string& err) {
  int rc = ensure_flow_device(f, err);
  if (rc) return rc;
  std::vector<float> t(f.n_params);
  for (long i = 0; i < f.n_params; ++i) t[i] = (float)theta[i];
  FL_CUDA(cudaMemcpy(f.theta, t.data(), sizeof(float) * f.n_params, cudaMemcpyHostToDevice));
  FL_CUDA(cudaMemset(f.adam_m, 0, sizeof(float) * f.n_params));
  FL_CUDA(cudaMemset(f.adam_v, 0, sizeof(float) * f.n_params));
  const FlowDev F = dev_of(f);
  k_flow_sync_w16<<<256, 256>>>(F, reinterpret_cast<__nv_bfloat16*>(f.w16),
                                reinterpret_cast<__nv_bfloat16*>(f.w16t));
  FL_CUDA(cudaGetLastError());
  FL_CUDA(cudaDeviceSynchronize());
  return GNUTS_OK;
}

int flow_get_params(const Flow& f, double* theta, std::string& err) {
  if (f.device < 0) {
    for (long i = 0; i < f.n_params; ++i) theta[i] = 0.0;
    return GNUTS_OK;
  }
  std::vector<float> t(f.n_params);
  FL_CUDA(cudaMemcpy(t.data(), f.theta, sizeof(float) * f.n_params, cudaMemcpyDeviceToHost));
  for (long i = 0; i < f.n_params; ++i) theta[i] = t[i];
  return GNUTS_OK;
}

int flow_forward(Flow& f, int n, const double* z, double* x, double* logdet, std::string& err) {
  int rc = ensure_flow_device(f, err);
  if (rc || n <= 0) return rc;
  DevBuf<double> dz, dx, dl;
  FL_CUDA(dz.alloc((size_t)n * f.d));
  FL_CUDA(dx.alloc((size_t)n * f.d));
  FL_CUDA(dl.alloc(n));
  FL_CUDA(cudaMemcpy(dz.p, z, sizeof(double) * n * f.d, cudaMemcpyHostToDevice));
  FlowIO io{};
  io.n = n;
  io.z = dz.p;
  io.ldz = f.d;
  io.x = dx.p;
  io.logdet = dl.p;
  DevModel M{};
  if ((rc = configure_flow(f, err)) || (rc = launch_flow(f, M, FM_FWD, io, 0, err))) return rc;
  FL_CUDA(cudaMemcpy(x, dx.p, sizeof(double) * n * f.d, cudaMemcpyDeviceToHost));
  FL_CUDA(cudaMemcpy(logdet, dl.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return GNUTS_OK;
}

namespace {
int launch_inverse(const Flow& f, int n, const double* dx, double* dz, double* dl, std::string& err) {
  if (n <= 0) return GNUTS_OK;
  const FlowDev F = dev_of(f);
  int namax = 0;
  for (int a : f.na) namax = std::max(namax, a);
  const int scn = std::max(2 * namax, f.H);
  const size_t smem = 4 * sizeof(float) * (size_t)(f.d + f.H + scn);
  const int blocks = (n + 3) / 4;
  switch (f.H) {
    case 128: k_flow_inverse<4><<<blocks, 128, smem>>>(F, n, dx, dz, dl); break;
    case 64: k_flow_inverse<2><<<blocks, 128, smem>>>(F, n, dx, dz, dl); break;
    default: k_flow_inverse<1><<<blocks, 128, smem>>>(F, n, dx, dz, dl); break;
  }
  FL_CUDA(cudaGetLastError());
  return GNUTS_OK;
}
}  // namespace

int flow_inverse(Flow& f, int n, const double* x, double* z, double* logdet, std::string& err) {
  int rc = ensure_flow_device(f, err);
  if (rc || n <= 0) return rc;
  DevBuf<double> dz, dx, dl;
  FL_CUDA(dz.alloc((size_t)n * f.d));
  FL_CUDA(dx.alloc((size_t)n * f.d));
  FL_CUDA(dl.alloc(n));
  FL_CUDA(cudaMemcpy(dx.p, x, sizeof(double) * n * f.d, cudaMemcpyHostToDevice));
  if ((rc = launch_inverse(f, n, dx.p, dz.p, dl.p, err))) return rc;
  FL_CUDA(cudaMemcpy(z, dz.p, sizeof(double) * n * f.d, cudaMemcpyDeviceToHost));
  if (logdet) FL_CUDA(cudaMemcpy(logdet, dl.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return GNUTS_OK;
}

namespace {
size_t fac_floats(const Flow& f, int n) {
  size_t o = 0;
  for (int l = 0; l < f.L; ++l) o += (size_t)n * (f.nb[l] + 2 * f.H + 2 * f.na[l]);
  return o + (size_t)n * 2 * f.d;
}
}  // namespace

int flow_log_prob_grad(Model& m, Flow& f, int n, const double* z, int jacobian, double* lp, double* grad_z,
                       double* grad_theta, std::string& err) {
  int rc = upload(m, err);
  if (rc) return rc;
  if (m.dev.D != f.d) {
    err = "flow dimension does not match the model's";
    return GNUTS_ERR_ARGUMENT;
  }
  if ((rc = ensure_flow_device(f, err)) || n <= 0) return rc;
  DevBuf<double> dz, dg, dl;
  DevBuf<float> fac, loss;
  DevBuf<int> valid;
  FL_CUDA(dz.alloc((size_t)n * f.d));
  FL_CUDA(dg.alloc((size_t)n * f.d));
  FL_CUDA(dl.alloc(n));
  FL_CUDA(fac.alloc(fac_floats(f, n)));
  FL_CUDA(loss.alloc(n));
  FL_CUDA(valid.alloc(n));
  FL_CUDA(cudaMemcpy(dz.p, z, sizeof(double) * n * f.d, cudaMemcpyHostToDevice));
  FL_CUDA(cudaMemset(f.nvalid, 0, sizeof(int)));
  FlowIO io{};
  io.n = n;
  io.z = dz.p;
  io.ldz = f.d;
  io.jac = jacobian;
  io.lp = dl.p;
  io.g = dg.p;
  io.ldg = f.d;
  io.fac = fac.p;
  io.loss = loss.p;
  io.valid = valid.p;
  io.nvalid = f.nvalid;
  io.beta = 1.0;
  if ((rc = configure_flow(f, err)) || (rc = launch_flow(f, m.dev, FM_TRAIN, io, 0, err))) return rc;
  if (grad_theta) {
    const FlowDev F = dev_of(f);
    k_flow_pgrad<<<(int)((f.n_params + 255) / 256), 256>>>(F, n, fac.p, valid.p, f.grad);
    FL_CUDA(cudaGetLastError());
    std::vector<float> g(f.n_params);
    FL_CUDA(cudaMemcpy(g.data(), f.grad, sizeof(float) * f.n_params, cudaMemcpyDeviceToHost));
    for (long i = 0; i < f.n_params; ++i) grad_theta[i] = g[i];
  }
  FL_CUDA(cudaMemcpy(lp, dl.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  FL_CUDA(cudaMemcpy(grad_z, dg.p, sizeof(double) * n * f.d, cudaMemcpyDeviceToHost));
  return GNUTS_OK;
}

int flow_log_prob_grad_tc(Model& m, Flow& f, int n, const double* z, double* lp, double* grad_z,
                          std::string& err) {
  int rc = upload(m, err);
  if (rc) return rc;
  if (m.dev.D != f.d) {
    err = "flow dimension does not match the model's";
    return GNUTS_ERR_ARGUMENT;
  }
  if ((rc = ensure_flow_device(f, err)) || n <= 0) return rc;
  const FlowDev F = dev_of(f);
  int T = 8;
  while (T > 1 && flow_tc_bytes(F, T) > FLOW_SMEM_LIMIT) T >>= 1;
  const size_t smem = flow_tc_bytes(F, T);
  if (smem > FLOW_SMEM_LIMIT) {
    err = "flow does not fit in shared memory";
    return GNUTS_ERR_ARGUMENT;
  }
  DevBuf<double> dz, dg, dl;
  FL_CUDA(dz.alloc((size_t)n * f.d));
  FL_CUDA(dg.alloc((size_t)n * f.d));
  FL_CUDA(dl.alloc(n));
  FL_CUDA(cudaMemcpy(dz.p, z, sizeof(double) * n * f.d, cudaMemcpyHostToDevice));
  FL_CUDA(flow_tc_grad_launch(m.dev.kind, F, m.dev, n, T, dz.p, dl.p, dg.p, smem));
  FL_CUDA(cudaMemcpy(lp, dl.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  FL_CUDA(cudaMemcpy(grad_z, dg.p, sizeof(double) * n * f.d, cudaMemcpyDeviceToHost));
  return GNUTS_OK;
}

int flow_adam_step(Flow& f, const double* grad, int t, double lr, double b1, double b2, double eps,
                   std::string& err) {
  int rc = ensure_flow_device(f, err);
  if (rc) return rc;
  std::vector<float> g(f.n_params);
  for (long i = 0; i < f.n_params; ++i) g[i] = (float)grad[i];
  FL_CUDA(cudaMemcpy(f.grad, g.data(), sizeof(float) * f.n_params, cudaMemcpyHostToDevice));
  const FlowDev F = dev_of(f);
  k_flow_adam<<<(int)((f.n_params + 255) / 256), 256>>>(F, f.theta, f.adam_m, f.adam_v, f.grad, nullptr, t,
                                                       (float)lr, (float)b1, (float)b2, (float)eps,
                                                       reinterpret_cast<__nv_bfloat16*>(f.w16),
                                                       reinterpret_cast<__nv_bfloat16*>(f.w16t));
  FL_CUDA(cudaGetLastError());
  FL_CUDA(cudaDeviceSynchronize());
  return GNUTS_OK;
}

int flow_train(Model& m, Flow& f, const gnuts_train_args& ta, double* loss_trace, std::string& err) {
  NvtxRange range("gnuts.flow.train");
  const int steps = ta.steps, batch = ta.batch;
  const double lr = ta.learning_rate;
  int rc = upload(m, err);
  if (rc) return rc;
  if (m.dev.D != f.d) {
    err = "flow dimension does not match the model's";
    return GNUTS_ERR_ARGUMENT;
  }
  if ((rc = ensure_flow_device(f, err))) return rc;
  if (steps <= 0) return GNUTS_OK;
  DevBuf<float> fac, loss;
  DevBuf<int> valid;
  DevBuf<double> trace;
  FL_CUDA(fac.alloc(fac_floats(f, batch)));
  FL_CUDA(loss.alloc(batch));
  FL_CUDA(valid.alloc(batch));
  FL_CUDA(trace.alloc(steps));
  const FlowDev F = dev_of(f);
  FlowIO io{};
  io.n = batch;
  io.seed = ta.seed;
  io.base_scale = (float)ta.base_scale;
  io.jac = 1;
  io.fac = fac.p;
  io.loss = loss.p;
  io.valid = valid.p;
  io.nvalid = f.nvalid;
  const int pblocks = (int)((f.n_params + 255) / 256);
  if ((rc = configure_flow(f, err))) return rc;
  for (int t = 1; t <= steps; ++t) {
    FL_CUDA(cudaMemsetAsync(f.nvalid, 0, sizeof(int)));
    io.step = t - 1;
    // tempered target beta * lp_x, beta rising linearly from beta0 to 1 over
    // the first anneal_fraction of the steps
    const double ramp = ta.anneal_fraction > 0 ? (double)(t - 1) / (ta.anneal_fraction * steps) : 1.0;
    io.beta = ramp >= 1.0 ? 1.0 : ta.beta0 + (1.0 - ta.beta0) * ramp;
    if ((rc = launch_flow(f, m.dev, FM_TRAIN, io, 0, err))) return rc;
    k_flow_pgrad<<<pblocks, 256>>>(F, batch, fac.p, valid.p, f.grad);
    // learning rate decays linearly to a tenth of its start over the run
    const float lr_t = (float)(lr * (1.0 - 0.9 * (double)(t - 1) / (double)steps));
    k_flow_adam<<<pblocks, 256>>>(F, f.theta, f.adam_m, f.adam_v, f.grad, f.nvalid, t, lr_t, 0.9f, 0.999f, 1e-8f,
                                  reinterpret_cast<__nv_bfloat16*>(f.w16),
                                  reinterpret_cast<__nv_bfloat16*>(f.w16t));
    k_flow_loss_mean<<<1, 256>>>(batch, loss.p, valid.p, trace.p + (t - 1));
    FL_CUDA(cudaGetLastError());
  }
  FL_CUDA(cudaDeviceSynchronize());
  if (loss_trace) FL_CUDA(cudaMemcpy(loss_trace, trace.p, sizeof(double) * steps, cudaMemcpyDeviceToHost));
  return GNUTS_OK;
}

// saved z draws -> lp__ and write_array(T(z)) in the draw rows
int flow_finalize_draws(Model& m, const Flow& f, int rows, const double* zdraws, double* draws, int ncol,
                        std::string& err) {
  FlowIO io{};
  io.n = rows;
  io.z = zdraws;
  io.ldz = f.d;
  io.jac = 1;
  io.with_model = 1;
  io.draw_rows = draws;
  io.draw_ncol = ncol;
  int rc = configure_flow(f, err);
  if (!rc) rc = launch_flow(f, m.dev, FM_FWD, io, 0, err);
  if (rc) return rc;
  FL_CUDA(cudaDeviceSynchronize());
  return GNUTS_OK;
}

int flow_inverse_device(const Flow& f, int n, const double* dx, double* dz, std::string& err) {
  int rc = launch_inverse(f, n, dx, dz, nullptr, err);
  if (rc) return rc;
  FL_CUDA(cudaDeviceSynchronize());
  return GNUTS_OK;
}

int run_flow_fused(Model& m, const Flow& f, Params& P, const Bufs& B, double per_chain_max, double* stats,
                   std::string& err) {
  if (P.ld != ((f.d + 3) & ~3) || P.D != f.d) {
    err = "flow / sampler dimension mismatch";
    return GNUTS_ERR_ARGUMENT;
  }
  const FlowDev F = dev_of(f);
  // CTA shape: 8 warps (each contraction has at most 8 m-tiles, one per
  // warp); T chains per CTA, the smallest power of two that keeps the grid
  // within one CTA per SM, reduced while the flow region plus the chains'
  // cached vectors exceed the shared-memory budget (the cache goes first)
  int sms = 0, dev = 0;
  FL_CUDA(cudaGetDevice(&dev));
  FL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int T = 1;
  while (T < 8 && (P.C + T - 1) / T > sms) T <<= 1;
  const size_t chain_bytes = (size_t)P.cache_stride * sizeof(double);
  bool cache = true;
  size_t flow_bytes = flow_tc_bytes(F, T);
  while (flow_bytes + (cache ? (size_t)T * chain_bytes : 0) > FLOW_SMEM_LIMIT) {
    if (cache) {
      cache = false;
    } else if (T > 1) {
      T >>= 1;
      cache = true;
      flow_bytes = flow_tc_bytes(F, T);
    } else {
      err = "flow does not fit in shared memory";
      return GNUTS_ERR_ARGUMENT;
    }
  }
  P.cache = cache ? 1 : 0;
  const size_t smem = flow_bytes + (cache ? (size_t)T * chain_bytes : 0);
  const int blocks = (P.C + T - 1) / T;
  FL_CUDA(cudaDeviceSynchronize());  // k_init done
  int* h_done = nullptr;
  FL_CUDA(cudaMallocHost(&h_done, sizeof(int)));
  struct HG { int* p; ~HG() { cudaFreeHost(p); } } hg{h_done};
  cudaEvent_t e0, e1;
  FL_CUDA(cudaEventCreate(&e0));
  FL_CUDA(cudaEventCreate(&e1));
  struct EG { cudaEvent_t a, b; ~EG() { cudaEventDestroy(a); cudaEventDestroy(b); } } eg{e0, e1};
  const long long max_launches = (long long)(per_chain_max / P.grad_budget) + 16;
  long long launches = 0;
  FL_CUDA(cudaEventRecord(e0));
  for (; launches < max_launches; ++launches) {
    FL_CUDA(flow_tc_fused_launch(m.dev.kind, F, P, B, m.dev, T, flow_bytes, blocks, smem));
    FL_CUDA(cudaMemcpy(h_done, B.done_count, sizeof(int), cudaMemcpyDeviceToHost));
    if (*h_done >= P.C) {
      ++launches;
      break;
    }
    if (interrupt_requested()) {
      err = "sampling interrupted by the caller's interrupt callback (gnuts_set_interrupt)";
      return GNUTS_ERR_INTERRUPTED;
    }
  }
  FL_CUDA(cudaEventRecord(e1));
  FL_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  stats[0] = (double)launches;
  stats[1] = ms;
  stats[2] = (double)launches;
  stats[3] = 0;
  stats[4] = launches ? 1e3 * ms / launches : 0;
  stats[5] = T;
  return GNUTS_OK;
}

}  // namespace gnuts
