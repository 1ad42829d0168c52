// Device sampler: kernels and the host driver behind the hmc_nuts_* entry
// points of the C ABI.
//
// Execution modes
//   fused : one warp per chain runs its whole sampler (state machine +
//           inline warp gradient) for a budget of gradient evaluations per
//           launch; used for models without a large shared design matrix.
//   rounds: the state machine (k_advance) and a batched gradient over all
//           chains (grad_logistic.cu) alternate; each round every live chain
//           needs exactly one gradient, so one contraction serves all chains.
//           Rounds are captured in CUDA graphs.
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "internal.h"
#include "nuts_device.cuh"
#include "batched.cuh"
#include "grad_tc.h"
#include "grad_wide.h"
#include "advance.h"

namespace gnuts {

#define GN_CUDA(call)                                                                        \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      err = std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call;            \
      return GNUTS_ERR_CUDA;                                                                 \
    }                                                                                        \
  } while (0)


// ---------------------------------------------------------------- kernels
__global__ void k_init(Params P, Bufs B, DevModel M, const double* inv_metric, ReplayBufs RB) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= P.C) return;
  Scal s;
  memset(&s, 0, sizeof(Scal));
  Chain ch(P, B, chain_model(M, warp, P.C), s, warp, lane);
  if (RB.chain_ids) ch.chain_id = RB.chain_ids[warp];
  s.t_start = globaltimer();
  const double eps0 = B.init_eps ? B.init_eps[warp] : P.stepsize;
  s.nom_eps = eps0;
  s.eps = eps0;
  s.rng_n = RB.rng_start ? RB.rng_start[warp] : 0ull;
  s.irng_n = 0;
  s.da_mu = log(10.0 * eps0);
  // windowed_adaptation::set_window_params
  {
    unsigned nw = (unsigned)P.num_warmup;
    if (nw < 20) {
      s.w_nw = 0; s.w_ib = 0; s.w_tb = 0; s.w_bw = 0;
    } else if (P.init_buffer + P.window + P.term_buffer > nw) {
      s.w_nw = nw;
      s.w_ib = (unsigned)(0.15 * nw);
      s.w_tb = (unsigned)(0.1 * nw);
      s.w_bw = nw - (s.w_ib + s.w_tb);
    } else {
      s.w_nw = nw; s.w_ib = P.init_buffer; s.w_tb = P.term_buffer; s.w_bw = P.window;
    }
    s.w_counter = 0;
    s.w_size = s.w_bw;
    s.w_next = s.w_ib + s.w_size - 1;
  }
  const int D = P.D;
  if (P.metric == 1) {
    const size_t mo = (size_t)warp * D * P.ld;
    for (int i = 0; i < D; ++i)
      for (int j = lane; j < D; j += 32) {
        double v = inv_metric ? inv_metric[((size_t)warp * D + i) * D + j] : (i == j ? 1.0 : 0.0);
        ch.minv[(size_t)i * P.ld + j] = v;
        ch.wm2[(size_t)i * P.ld + j] = 0.0;
        if (P.dense32) {
          B.minv32[mo + (size_t)i * P.ld + j] = (float)v;
          B.wm2_32[mo + (size_t)i * P.ld + j] = 0.f;
          B.wm2_32lo[mo + (size_t)i * P.ld + j] = 0.f;
        }
      }
    __syncwarp();
    bool pd = true;
    if (inv_metric) {
      pd = ch.cholesky();
    } else {
      // the factor of the identity is the identity (what cholesky() computes, bit for bit)
      for (int i = 0; i < D; ++i)
        for (int j = lane; j < D; j += 32) ch.chol[(size_t)i * P.ld + j] = i == j ? 1.0 : 0.0;
      __syncwarp();
    }
    if (!pd) {
      s.err = CE_NOT_PD;
      s.phase = PH_ERROR;
      if (lane == 0) atomicAdd(B.done_count, 1);
      if (lane == 0) B.sc[warp] = s;
      return;
    }
    if (P.dense32)
      for (int i = 0; i < D; ++i)
        for (int j = lane; j < D; j += 32) B.chol32[mo + (size_t)i * P.ld + j] = (float)ch.chol[(size_t)i * P.ld + j];
  } else {
    for (int d = lane; d < D; d += 32) {
      ch.minv[d] = (P.metric == 0 && inv_metric) ? inv_metric[(size_t)warp * D + d] : 1.0;
      ch.wm2[d] = 0.0;
    }
  }
  for (int d = lane; d < D; d += 32) {
    ch.wm[d] = 0.0;
    ch.Wp[d] = 0.0;
    ch.Wg[d] = 0.0;
  }
  ch.init_candidate();
  if (lane == 0) B.sc[warp] = s;
}

// Round mode: advance every live chain by one gradient.  Instantiated per
// metric (MET), so the diag_e kernel's hot path carries no dense-metric code.
// The Welford samples that this round's k_advance queued for wide dense
// chains (Chain::welford_add): item = (queued chain, 16 rows of its D x D
// float-float sums), spread over every SM.  The last CTA to finish empties
// the queue for the next round.
constexpr int WF_THREADS = 256, WF_ROWS = 16;
__global__ void __launch_bounds__(WF_THREADS) k_welford_dense(Params P, Bufs B) {
  const int n = B.wlist[0];
  const int D = P.D, nrb = (D + WF_ROWS - 1) / WF_ROWS;
  for (int it = blockIdx.x; it < n * nrb; it += gridDim.x) {
    const int c = B.wlist[2 + it / nrb], i0 = (it % nrb) * WF_ROWS;
    const float* bh = B.wpend + (size_t)c * 4 * P.ld;
    const float *bl = bh + P.ld, *ah = bh + 2 * P.ld, *al = bh + 3 * P.ld;
    const size_t mo = (size_t)c * D * P.ld;
    // 16-byte vectors (ld is a multiple of 4; the padding columns of b are
    // zero, so the padding of a row's sums stays zero)
    for (int i = i0; i < min(D, i0 + WF_ROWS); ++i) {
      const float a0 = ah[i], a1 = al[i];
      float4* wr = reinterpret_cast<float4*>(B.wm2_32 + mo + (size_t)i * P.ld);
      float4* wl = reinterpret_cast<float4*>(B.wm2_32lo + mo + (size_t)i * P.ld);
      const float4* b0 = reinterpret_cast<const float4*>(bh);
      const float4* b1 = reinterpret_cast<const float4*>(bl);
      for (int j = threadIdx.x; 4 * j < D; j += WF_THREADS) {
        float4 h = wr[j], l = wl[j];
        const float4 x = b0[j], y = b1[j];
        ff_axpy(h.x, l.x, a0, a1, x.x, y.x);
        ff_axpy(h.y, l.y, a0, a1, x.y, y.y);
        ff_axpy(h.z, l.z, a0, a1, x.z, y.z);
        ff_axpy(h.w, l.w, a0, a1, x.w, y.w);
        wr[j] = h;
        wl[j] = l;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&B.wlist[1], 1) == (int)gridDim.x - 1) {
      B.wlist[0] = 0;
      B.wlist[1] = 0;
      __threadfence();
    }
  }
}

// k_advance (advance_kind.cu, one object per metric and team width):
// chains of at least TEAM_MIN_D parameters advance as CTA teams
static void launch_advance(int blocks, int threads, size_t smem, cudaStream_t st, const Params& P, const Bufs& B,
                           const DevModel& M, const GradOut& G) {
  if (M.D >= TEAM_MIN_D && !P.cache) {
    if (P.metric == 0) advance_launch_k<0, TEAM_TW>(P.C, TEAM_TW, 0, st, P, B, M, G);
    else if (P.metric == 1) advance_launch_k<1, TEAM_TW>(P.C, TEAM_TW, 0, st, P, B, M, G);
    else advance_launch_k<2, TEAM_TW>(P.C, TEAM_TW, 0, st, P, B, M, G);
    return;
  }
  if (P.metric == 0) advance_launch_k<0, 32>(blocks, threads, smem, st, P, B, M, G);
  else if (P.metric == 1) advance_launch_k<1, 32>(blocks, threads, smem, st, P, B, M, G);
  else advance_launch_k<2, 32>(blocks, threads, smem, st, P, B, M, G);
}

__global__ void k_log_prob_grad(DevModel M, int n, const double* q, int jac, double* lp, double* g) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const DevModel& Mc = chain_model(M, warp, n);
  double v = warp_log_prob_grad(Mc, q + (size_t)warp * M.D, g + (size_t)warp * M.D, jac, lane);
  if (lane == 0) lp[warp] = v;
}

// FP32 and BF16 (round to nearest even) copies of the FP64 design matrix
__global__ void k_derive_x(const double* X, size_t n, float* Xf, uint16_t* Xb) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float f = (float)X[i];
    Xf[i] = f;
    const uint32_t u = __float_as_uint(f);
    Xb[i] = (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
  }
}
// tensor-core rows: [x_1..x_K, 1, 0 ...] in BF16, XTC_LD elements per row
__global__ void k_derive_xtc(const uint16_t* Xb, size_t rows, int K, uint16_t* Xtc) {
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < rows; n += (size_t)gridDim.x * blockDim.x) {
    for (int k = 0; k < XTC_LD; ++k)
      Xtc[n * XTC_LD + k] = k < K ? Xb[n * K + k] : (k == K ? (uint16_t)0x3f80 : (uint16_t)0);
  }
}
// column k of Xtc^T (y - 1/2) in FP64, one block per column; fixed
// per-thread row order and a fixed tree, so the result is reproducible
__global__ void k_xtc_ym(const uint16_t* Xtc, const int* y, int rows, double* out) {
  __shared__ double red[256];
  const int k = blockIdx.x;
  double s = 0;
  for (int n = threadIdx.x; n < rows; n += blockDim.x) {
    const float x = __uint_as_float((uint32_t)Xtc[(size_t)n * XTC_LD + k] << 16);
    s += (double)x * (y[n] ? 0.5 : -0.5);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[k] = red[0];
}
// y packed 32 rows per word (words beyond the data are zero)
__global__ void k_pack_y(const int* y, size_t rows, size_t words, uint32_t* out) {
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < words; w += (size_t)gridDim.x * blockDim.x) {
    uint32_t v = 0;
    for (int b = 0; b < 32; ++b) {
      const size_t n = w * 32 + b;
      if (n < rows && y[n]) v |= 1u << b;
    }
    out[w] = v;
  }
}

__global__ void k_write_array(DevModel M, int n, const double* q, double* out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const DevModel& Mc = chain_model(M, warp, n);
  double* o = out + (size_t)warp * M.ncon;
  warp_write_array(Mc, q + (size_t)warp * M.D, o, lane);
  for (int i = Mc.ncon + lane; i < M.ncon; i += 32) o[i] = __longlong_as_double(0x7ff8000000000000ll);
}

// ---------------------------------------------------------------- host side
// dynamic shared memory of k_fused / k_advance (128-thread blocks: 4 chains)
static size_t cache_bytes(const Params& P) { return P.cache ? 4 * (size_t)P.cache_stride * sizeof(double) : 0; }

namespace {

struct Arena {
  std::vector<void*> ptrs;
  ~Arena() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T** p, size_t count) {
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) {
      ptrs.push_back(v);
      cudaMemset(v, 0, std::max<size_t>(count, 1) * sizeof(T));
    }
    *p = (T*)v;
    return e;
  }
};

const char* chain_error_message(int code) {
  switch (code) {
    case CE_INIT: return "Initialization failed: log density or gradient not finite at every attempted initial value";
    case CE_IMPROPER: return "Posterior is improper. Please check your model.";
    case CE_NO_STEPSIZE: return "No acceptably small step size could be found. Perhaps the posterior is not continuous?";
    case CE_METRIC: return "Numerical overflow in metric adaptation. This occurs when the sampler encounters extreme values on the unconstrained space; this may happen when the posterior density function is too wide or improper. There may be problems with your model specification.";
    case CE_NOT_PD: return "Inverse metric is not positive definite";
  }
  return "unknown sampler error";
}

int ensure_device(std::string& err) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    err = "no CUDA device available (the sampler runs on the GPU only)";
    return GNUTS_ERR_CUDA;
  }
  return GNUTS_OK;
}

bool use_rounds(const Model& m) {
  return batched_supported(m.dev) && m.dev.N >= 4096;
}

// the warp (fused) gradients hold a chain's coefficients in registers
int check_warp_limits(const Model& m, std::string& err) {
  if (use_rounds(m)) return GNUTS_OK;
  if (m.dev.kind == MK_LOGISTIC && m.dev.K > 256) {
    err = "logistic models with more than 256 predictors need N >= 4096 (batched gradient)";
    return GNUTS_ERR_ARGUMENT;
  }
  if (m.dev.kind == MK_HORSESHOE && m.dev.K > 1024) {
    err = "horseshoe models support at most 1024 predictors";
    return GNUTS_ERR_ARGUMENT;
  }
  return GNUTS_OK;
}

}  // namespace

int upload(Model& m, std::string& err) {
  // every device entry point passes here: drop a stale non-sticky error left
  // by an earlier runtime call so that launch checks report this call's errors
  (void)cudaGetLastError();
  if (m.device >= 0) {
    // the model's data lives on the device it was uploaded to: refuse a call
    // made with another device current instead of launching on foreign pointers
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) {
      err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
      return GNUTS_ERR_CUDA;
    }
    if (cur != m.device) {
      err = "the model's data is on CUDA device " + std::to_string(m.device) + " but device " + std::to_string(cur) +
            " is current; make device " + std::to_string(m.device) + " current for calls on this model";
      return GNUTS_ERR_ARGUMENT;
    }
    return GNUTS_OK;
  }
  int rc = ensure_device(err);
  if (rc) return rc;
  auto put = [&](const void* src, size_t bytes, void** dst) -> int {
    if (bytes == 0) { *dst = nullptr; return GNUTS_OK; }
    cudaError_t e = cudaMalloc(dst, bytes);
    if (e != cudaSuccess) { err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return GNUTS_ERR_CUDA; }
    m.device_allocs.push_back(*dst);
    e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { err = std::string("cudaMemcpy: ") + cudaGetErrorString(e); return GNUTS_ERR_CUDA; }
    return GNUTS_OK;
  };
  // The host-side Model holds host pointers in dev.*; replace them by device copies.
  DevModel h = m.dev;
  DevModel d = h;
  size_t xcols = (h.kind == MK_VARINT) ? (size_t)h.K : (size_t)h.K;
  size_t xn = (size_t)h.N * xcols;
  if (h.yi && (rc = put(h.yi, sizeof(int) * h.N, (void**)&d.yi))) return rc;
  if (h.yr) {
    size_t n = h.kind == MK_HIER ? (size_t)h.J : (size_t)h.N;
    if ((rc = put(h.yr, sizeof(double) * n, (void**)&d.yr))) return rc;
  }
  if (h.X && xn) {
    // only FP64 X crosses the bus; the FP32, BF16 and tensor-core copies are derived on the device
    if ((rc = put(h.X, sizeof(double) * xn, (void**)&d.X))) return rc;
    auto dev_alloc = [&](size_t bytes, void** dst) -> int {
      cudaError_t e = cudaMalloc(dst, bytes);
      if (e != cudaSuccess) { err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return GNUTS_ERR_CUDA; }
      m.device_allocs.push_back(*dst);
      return GNUTS_OK;
    };
    if ((rc = dev_alloc(sizeof(float) * xn, (void**)&d.Xf))) return rc;
    if ((rc = dev_alloc(sizeof(uint16_t) * xn, (void**)&d.Xb))) return rc;
    const bool tc = h.kind == MK_LOGISTIC && h.K + 1 <= XTC_LD;
    // y packed 32 rows per word for the tensor-core likelihood epilogues
    const bool yb = (h.kind == MK_LOGISTIC || h.kind == MK_HORSESHOE) && h.yi;
    if (tc) {
      if ((rc = dev_alloc(sizeof(uint16_t) * (size_t)h.N * XTC_LD, (void**)&d.Xtc))) return rc;
      if ((rc = dev_alloc(sizeof(double) * XTC_LD, (void**)&d.xtc_ym))) return rc;
    }
    if (yb && (rc = dev_alloc(sizeof(uint32_t) * (((size_t)h.N + 31) / 32 + 4), (void**)&d.ybits))) return rc;
    k_derive_x<<<std::min<size_t>(4096, (xn + 255) / 256), 256>>>(d.X, xn, const_cast<float*>(d.Xf),
                                                                  const_cast<uint16_t*>(d.Xb));
    if (tc) {
      const size_t rows = (size_t)h.N;
      k_derive_xtc<<<std::min<size_t>(4096, (rows + 255) / 256), 256>>>(d.Xb, rows, h.K,
                                                                        const_cast<uint16_t*>(d.Xtc));
      k_xtc_ym<<<XTC_LD, 256>>>(d.Xtc, d.yi, h.N, const_cast<double*>(d.xtc_ym));
    }
    if (yb) {
      const size_t rows = (size_t)h.N, words = (rows + 31) / 32 + 4;
      k_pack_y<<<std::min<size_t>(4096, (words + 255) / 256), 256>>>(d.yi, rows, words,
                                                                     const_cast<uint32_t*>(d.ybits));
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) { err = std::string("deriving X copies: ") + cudaGetErrorString(e); return GNUTS_ERR_CUDA; }
  }
  if (h.group && (rc = put(h.group, sizeof(int) * h.N, (void**)&d.group))) return rc;
  size_t n_gstart = (size_t)h.J + 1;
  if (!m.members.empty()) n_gstart = (size_t)(m.members.back().g_off + m.members.back().J + 1);
  if (h.gstart && (rc = put(h.gstart, sizeof(int) * n_gstart, (void**)&d.gstart))) return rc;
  if (h.sigma && (rc = put(h.sigma, sizeof(double) * h.J, (void**)&d.sigma))) return rc;
  if (h.scales && (rc = put(h.scales, sizeof(double) * h.K, (void**)&d.scales))) return rc;
  if (!m.members.empty()) {
    // one DevModel per posterior, pointing into the shared device arrays
    std::vector<DevModel> mem(m.members.size());
    for (size_t i = 0; i < mem.size(); ++i) {
      const Model::Member& s = m.members[i];
      DevModel e = d;
      e.N = s.N;
      e.J = s.J;
      e.D = s.D;
      e.ncon = s.D;
      e.X = d.X + (size_t)s.row_off * d.K;
      e.Xf = d.Xf + (size_t)s.row_off * d.K;
      e.Xb = d.Xb + (size_t)s.row_off * d.K;
      e.yr = d.yr + s.row_off;
      e.group = d.group + s.row_off;
      e.gstart = d.gstart + s.g_off;
      e.members = nullptr;
      e.n_members = 0;
      mem[i] = e;
    }
    if ((rc = put(mem.data(), sizeof(DevModel) * mem.size(), (void**)&d.members))) return rc;
  }
  m.dev = d;
  cudaGetDevice(&m.device);
  return GNUTS_OK;
}


// ---------------------------------------------------------------- round mode
__global__ void k_stage(GradOut G, Params P, Bufs B, DevModel M) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= P.C) return;
  if (B.sc[warp].phase >= PH_DONE) return;
  stage_request(G, M, warp, B.Wq + (size_t)warp * P.ld, lane);
}

__global__ void k_stage_points(GradOut G, DevModel M, int n, const double* q) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  stage_request(G, M, warp, q + (size_t)warp * M.D, lane);
}

__global__ void k_reduce_points(GradOut G, DevModel M, int n, const double* q, int jac, double* lp, double* g) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  double v = reduce_gradient(G, M, warp, q + (size_t)warp * M.D, g + (size_t)warp * M.D, lane);
  if (!jac && M.kind == MK_HORSESHOE) {
    // remove the Jacobian terms added by reduce_gradient
    const int K = M.K;
    const double* qq = q + (size_t)warp * M.D;
    double* gg = g + (size_t)warp * M.D;
    double jl = 0;
    for (int d = lane; d < K; d += 32) { jl += qq[K + 2 + d]; gg[K + 2 + d] -= 1.0; }
    jl = wsum(jl);
    v -= jl + qq[K + 1] + qq[2 * K + 2];
    __syncwarp();
    if (lane == 0) { gg[K + 1] -= 1.0; gg[2 * K + 2] -= 1.0; }
  }
  if (lane == 0) lp[warp] = v;
}

namespace {

struct GradSetup {
  Arena ar;
  GradOut G{};
  TcPlan* plan = nullptr;
  WidePlan* wide = nullptr;
  ~GradSetup() {
    tc_destroy(plan);
    wide_destroy(wide);
  }
};

int setup_grad(GradSetup& gs, const DevModel& M, int C, int prec, const int* done_count, std::string& err) {
  GradOut& G = gs.G;
  G.kind = M.kind;
  G.prec = prec;
  G.C = C;
  G.C_total = C;
  G.K = M.K;
  G.done_count = done_count;
  if (prec == GNUTS_PRECISION_MIXED && tc_supported(M)) {
    int st = tc_create(M, C, done_count, &gs.plan, &G.coef_bf, &G.S, &G.part_lp, &G.part_g32, &G.lin, err);
    if (st) return st;
    G.tc = gs.plan;
    G.Cpad = (C + 127) / 128 * 128;
    return GNUTS_OK;
  }
  if (prec == GNUTS_PRECISION_MIXED && wide_supported(M)) {
    // wider than k_glm_tc's tile: the two-kernel tcgen05 path
    int st = wide_create(M, C, done_count, &gs.wide, &G.coef64, &G.part_lp, &G.part_g, err);
    if (st) return st;
    G.wide = gs.wide;
    G.S = 1;
    G.rows_per_split = M.N;
    return GNUTS_OK;
  }
  // row splits: enough CTAs to fill 152 SMs a few times over
  const int ctiles = (C + GLM_CT - 1) / GLM_CT;
  int S = std::max(1, (152 * 4 + ctiles - 1) / ctiles);
  S = std::min(S, std::max(1, M.N / 256));
  G.S = S;
  G.rows_per_split = (M.N + S - 1) / S;
  G.rows_per_split = (G.rows_per_split + GLM_RB - 1) / GLM_RB * GLM_RB;
  G.S = (M.N + G.rows_per_split - 1) / G.rows_per_split;
  G.done_count = done_count;
  GN_CUDA(gs.ar.alloc(&G.coef64, (size_t)C * (M.K + 1)));
  GN_CUDA(gs.ar.alloc(&G.coef32, (size_t)C * (M.K + 1)));
  GN_CUDA(gs.ar.alloc(&G.part_lp, (size_t)G.S * C));
  GN_CUDA(gs.ar.alloc(&G.part_g, (size_t)G.S * C * (M.K + 1)));
  return GNUTS_OK;
}

// the batched contraction (tcgen05 narrow or wide design, or SIMT); its
// partials are summed by the consumer (reduce_gradient, inside the
// state-machine kernel).  Returns the launch status of the wide-design path;
// the others report through the stream's launch errors.
int launch_glm(const GradOut& G, const DevModel& M, cudaStream_t st) {
  if (G.tc) {
    tc_launch((const TcPlan*)G.tc, st);
  } else if (G.wide) {
    return wide_launch((const WidePlan*)G.wide, G, M, st);
  } else {
    dim3 grid((G.C + GLM_CT - 1) / GLM_CT, G.S);
    const bool small = M.K <= GLM_KC;
    if (G.prec == GNUTS_PRECISION_FP64) {
      if (small) k_glm_simt<double, 1><<<grid, GLM_THREADS, 0, st>>>(G, M);
      else k_glm_simt<double, 8><<<grid, GLM_THREADS, 0, st>>>(G, M);
    } else {
      if (small) k_glm_simt<float, 1><<<grid, GLM_THREADS, 0, st>>>(G, M);
      else k_glm_simt<float, 8><<<grid, GLM_THREADS, 0, st>>>(G, M);
    }
  }
  return GNUTS_OK;
}

}  // namespace

// a tensor-core kernel whose bounded pipeline wait ran out records it in its
// plan's error flag (after a synchronisation)
static int plan_timeout(const GradSetup& gs, std::string& err) {
  if ((gs.plan && tc_error(gs.plan)) || (gs.wide && wide_error(gs.wide))) {
    err = "tensor-core gradient: a bounded pipeline wait ran out";
    return GNUTS_ERR_TIMEOUT;
  }
  return GNUTS_OK;
}

int batched_log_prob_grad(const DevModel& M, int n, const double* dq, int jac, double* dl, double* dg, int prec,
                          std::string& err) {
  if (M.K > 1024) { err = "batched gradient supports at most 1024 predictors"; return GNUTS_ERR_ARGUMENT; }
  GradSetup gs;
  int st = setup_grad(gs, M, n, prec, nullptr, err);
  if (st) return st;
  const int threads = 128, blocks = (n * 32 + threads - 1) / threads;
  k_stage_points<<<blocks, threads>>>(gs.G, M, n, dq);
  if (launch_glm(gs.G, M, 0)) {
    err = "the batched gradient could not be launched";
    return GNUTS_ERR_CUDA;
  }
  k_reduce_points<<<blocks, threads>>>(gs.G, M, n, dq, jac, dl, dg);
  GN_CUDA(cudaGetLastError());
  GN_CUDA(cudaDeviceSynchronize());
  return plan_timeout(gs, err);
}

// Hands completed draw rows to the caller's sink (gnuts_set_draw_sink) while
// the run proceeds.  Per-chain row counts are read back after launches that
// have completed; once every chain has written rows [delivered, r), a block
// of them (at most 64 MB) is copied with one strided copy on its own stream
// -- those rows are final, so the copy runs beside the kernels -- and passed
// to the sink.  finish() delivers the rest after the run.
class DrawStreamer {
 public:
  DrawStreamer(const Params& P, const Bufs& B, bool enabled) : P_(P), B_(B) {
    const RunHooks& h = run_hooks();
    if (!enabled || !h.sink || P.n_saved == 0) return;
    sink_ = h.sink;
    ctx_ = h.sink_ctx;
    const size_t row_bytes = (size_t)P.C * P.ncol * sizeof(double);
    batch_ = (int)std::max<size_t>(1, std::min<size_t>((size_t)P.n_saved, (64u << 20) / row_bytes));
  }
  ~DrawStreamer() {
    if (h_rows_) cudaFreeHost(h_rows_);
    if (stage_) cudaFreeHost(stage_);
    if (copy_) cudaStreamDestroy(copy_);
  }
  bool active() const { return sink_ != nullptr; }
  // enqueue the read of every chain's row count into slot (0 or 1) on stream s
  int request_rows(cudaStream_t s, int slot, std::string& err) {
    if (!active()) return GNUTS_OK;
    if (!h_rows_) {
      GN_CUDA(cudaMallocHost(&h_rows_, sizeof(int) * 2 * P_.C));
      std::fill(h_rows_, h_rows_ + 2 * P_.C, 0);
    }
    GN_CUDA(cudaMemcpy2DAsync(h_rows_ + slot * P_.C, sizeof(int), &B_.sc[0].row, sizeof(Scal), sizeof(int), P_.C,
                              cudaMemcpyDeviceToHost, s));
    return GNUTS_OK;
  }
  // the row counts in slot are complete (their launch has finished): deliver full blocks
  int deliver(int slot, std::string& err) {
    if (!active() || !h_rows_) return GNUTS_OK;
    int min_row = P_.n_saved;
    for (int c = 0; c < P_.C; ++c) min_row = std::min(min_row, h_rows_[slot * P_.C + c]);
    while (min_row - delivered_ >= batch_) {
      int st = send(batch_, err);
      if (st) return st;
    }
    return GNUTS_OK;
  }
  int finish(std::string& err) {
    while (active() && delivered_ < P_.n_saved) {
      int st = send(std::min(batch_, P_.n_saved - delivered_), err);
      if (st) return st;
    }
    return GNUTS_OK;
  }

 private:
  int send(int k, std::string& err) {
    const size_t rb = (size_t)P_.ncol * sizeof(double);
    if (!stage_) {
      GN_CUDA(cudaMallocHost(&stage_, rb * P_.C * batch_));
      GN_CUDA(cudaStreamCreateWithFlags(&copy_, cudaStreamNonBlocking));
    }
    GN_CUDA(cudaMemcpy2DAsync(stage_, rb * k, B_.draws + (size_t)delivered_ * P_.ncol, rb * P_.n_saved, rb * k,
                              P_.C, cudaMemcpyDeviceToHost, copy_));
    GN_CUDA(cudaStreamSynchronize(copy_));
    sink_(ctx_, delivered_, k, stage_);
    delivered_ += k;
    return GNUTS_OK;
  }
  const Params& P_;
  const Bufs& B_;
  gnuts_draws_fn sink_ = nullptr;
  void* ctx_ = nullptr;
  int batch_ = 1, delivered_ = 0;
  int* h_rows_ = nullptr;
  double* stage_ = nullptr;
  cudaStream_t copy_ = nullptr;
};

static const char* kInterrupted = "sampling interrupted by the caller's interrupt callback (gnuts_set_interrupt)";

struct RunStats {
  double rounds = 0, grad_us = 0, advance_us = 0, device_ms = 0, launches = 0, reduce_us = 0;
  double chains_per_cta = 4;
};

static int run_rounds(Model& m, const Params& P, const Bufs& B, int prec, double per_chain_max, int refresh,
                      gnuts_progress_fn progress, void* ctx, DrawStreamer& streamer, RunStats& stats,
                      std::string& err) {
  const DevModel& M = m.dev;
  if (M.K > 1024) { err = "batched gradient supports at most 1024 predictors"; return GNUTS_ERR_ARGUMENT; }
  GradSetup gs;
  int st = setup_grad(gs, M, P.C, prec, B.done_count, err);
  if (st) return st;
  const GradOut& G = gs.G;
  cudaStream_t stream;
  GN_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{stream};
  const int threads = 128, blocks = (P.C * 32 + threads - 1) / threads;
  GN_CUDA(cudaDeviceSynchronize());  // k_init done
  k_stage<<<blocks, threads, 0, stream>>>(G, P, B, M);
  GN_CUDA(cudaGetLastError());
  // capture ROUNDS x (gradient, advance) as one graph.  Every 64th step of
  // the loop runs one uncaptured round bracketed by events instead, which is
  // where the per-kernel durations come from.
  const int ROUNDS = 16;
  cudaEvent_t tev[6];
  for (auto& e : tev) GN_CUDA(cudaEventCreate(&e));
  struct EvGuard { cudaEvent_t* e; ~EvGuard() { for (int i = 0; i < 6; ++i) cudaEventDestroy(e[i]); } } eg{tev};
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  GN_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
  int glm_rc = GNUTS_OK;
  for (int r = 0; r < ROUNDS; ++r) {
    glm_rc |= launch_glm(G, M, stream);
    launch_advance(blocks, threads, cache_bytes(P), stream, P, B, M, G);
    if (P.dense32) k_welford_dense<<<2 * 152, WF_THREADS, 0, stream>>>(P, B);
  }
  GN_CUDA(cudaStreamEndCapture(stream, &graph));
  if (glm_rc) {
    cudaGraphDestroy(graph);
    err = "the batched gradient could not be captured";
    return GNUTS_ERR_CUDA;
  }
  GN_CUDA(cudaEventRecord(tev[3], stream));
  GN_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  struct GraphGuard { cudaGraph_t g; cudaGraphExec_t e; ~GraphGuard() { cudaGraphExecDestroy(e); cudaGraphDestroy(g); } } gg{graph, exec};
  int* h_done = nullptr;
  GN_CUDA(cudaMallocHost(&h_done, sizeof(int) * 2));
  struct HostGuard { int* p; ~HostGuard() { cudaFreeHost(p); } } hg{h_done};
  h_done[0] = h_done[1] = 0;
  cudaEvent_t ev[2];
  GN_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  GN_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
  const long long max_graphs = (long long)(per_chain_max / ROUNDS) + 16;
  int last_reported = -1;
  long long rounds = 0, launches = 0;
  double gsum = 0, asum = 0;
  int nt = 0;
  bool timed_pending = false;
  for (long long l = 0; l < max_graphs * 2; ++l) {
    const int b = (int)(l & 1);
    const bool timed = (l & 63) == 5;
    if (timed) {
      GN_CUDA(cudaEventRecord(tev[0], stream));
      if (launch_glm(G, M, stream)) {
        err = "the batched gradient could not be launched";
        return GNUTS_ERR_CUDA;
      }
      GN_CUDA(cudaEventRecord(tev[1], stream));
      launch_advance(blocks, threads, cache_bytes(P), stream, P, B, M, G);
      if (P.dense32) k_welford_dense<<<2 * 152, WF_THREADS, 0, stream>>>(P, B);
      GN_CUDA(cudaEventRecord(tev[2], stream));
      rounds += 1;
      launches += P.dense32 ? 3 : 2;
    } else {
      GN_CUDA(cudaGraphLaunch(exec, stream));
      rounds += ROUNDS;
      launches += (P.dense32 ? 3 : 2) * ROUNDS;
    }
    GN_CUDA(cudaMemcpyAsync(&h_done[b], B.done_count, sizeof(int), cudaMemcpyDeviceToHost, stream));
    if ((st = streamer.request_rows(stream, b, err))) return st;
    GN_CUDA(cudaEventRecord(ev[b], stream));
    if (l > 0) {
      GN_CUDA(cudaEventSynchronize(ev[b ^ 1]));
      if ((st = streamer.deliver(b ^ 1, err))) return st;
      if (interrupt_requested()) {
        cudaStreamSynchronize(stream);
        err = kInterrupted;
        return GNUTS_ERR_INTERRUPTED;
      }
      if (timed_pending) {
        // the timed round was enqueued one step earlier and has completed
        float g_ms = 0, a_ms = 0;
        if (h_done[b ^ 1] < P.C && cudaEventElapsedTime(&g_ms, tev[0], tev[1]) == cudaSuccess &&
            cudaEventElapsedTime(&a_ms, tev[1], tev[2]) == cudaSuccess) {
          gsum += g_ms;
          asum += a_ms;
          ++nt;
        }
        timed_pending = false;
      }
      if (h_done[b ^ 1] >= P.C) break;
      if (progress && refresh > 0 && (l & 63) == 0) {
        Scal s0;
        GN_CUDA(cudaMemcpy(&s0, B.sc, sizeof(Scal), cudaMemcpyDeviceToHost));
        if (s0.iter / refresh != last_reported) {
          last_reported = s0.iter / refresh;
          progress(ctx, 0, s0.iter, P.num_warmup + P.num_samples, s0.iter < P.num_warmup);
        }
      }
    }
    if (timed) timed_pending = true;
  }
  GN_CUDA(cudaEventRecord(tev[4], stream));
  GN_CUDA(cudaStreamSynchronize(stream));
  if ((st = plan_timeout(gs, err))) return st;
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  float total_ms = 0;
  cudaEventElapsedTime(&total_ms, tev[3], tev[4]);
  stats.rounds = (double)rounds;
  stats.chains_per_cta = M.D >= TEAM_MIN_D && !P.cache ? 1.0 : 4.0;  // launch_advance's choice
  stats.grad_us = nt ? 1e3 * gsum / nt : 0;
  stats.advance_us = nt ? 1e3 * asum / nt : 0;
  stats.device_ms = total_ms;
  stats.launches = (double)launches + 1;  // + k_stage
  return GNUTS_OK;
}

static int run_nuts_impl(Model& m, const gnuts_sample_args& a, const RunConfig& rc, const double* inits,
                         const double* inv_metric, const double* p0, const unsigned* chain_ids,
                         uint64_t* counters, double* replay_q_out, gnuts_output* out,
                         gnuts_progress_fn progress, void* ctx, std::string& err);
// flow.cu
int run_flow_fused(Model& m, const Flow& f, Params& P, const Bufs& B, double per_chain_max, double* stats,
                   std::string& err);
int flow_finalize_draws(Model& m, const Flow& f, int rows, const double* zdraws, double* draws, int ncol,
                        std::string& err);

int run_nuts(Model& m, const gnuts_sample_args& a, const RunConfig& rc, const double* inits,
             const double* inv_metric, gnuts_output* out, gnuts_progress_fn progress, void* ctx,
             std::string& err) {
  return run_nuts_impl(m, a, rc, inits, inv_metric, nullptr, nullptr, nullptr, nullptr, out, progress, ctx, err);
}

static int run_nuts_impl(Model& m, const gnuts_sample_args& a, const RunConfig& rc, const double* inits,
                         const double* inv_metric, const double* p0, const unsigned* chain_ids,
                         uint64_t* counters, double* replay_q_out, gnuts_output* out,
                         gnuts_progress_fn progress, void* ctx, std::string& err) {
  NvtxRange range(rc.flow ? "gnuts.nuts.flow" : (rc.adapt ? "gnuts.nuts.adapt" : "gnuts.nuts"));
  int st = upload(m, err);
  if (st) return st;
  if ((st = check_warp_limits(m, err))) return st;
  const int C = a.num_chains, D = m.dev.D;
  if (m.dev.n_members && (C % m.dev.n_members != 0 || rc.flow)) {
    err = "a posterior set needs num_chains to be a multiple of its " + std::to_string(m.dev.n_members) +
          " posteriors (and no flow)";
    return GNUTS_ERR_ARGUMENT;
  }
  Params P{};
  P.C = C;
  P.D = D;
  P.ld = (D + 3) & ~3;
  P.ncon = m.dev.ncon;
  P.ncol = 7 + P.ncon;
  P.max_depth = a.max_depth;
  P.R = a.max_depth + 2;
  P.metric = rc.metric;
  P.adapt = rc.adapt;
  P.num_warmup = a.num_warmup;
  P.num_samples = a.num_samples;
  P.thin = a.thin;
  P.save_warmup = a.save_warmup;
  P.stepsize = a.stepsize;
  P.jitter = a.stepsize_jitter;
  P.delta = a.delta;
  P.gamma = a.gamma;
  P.kappa = a.kappa;
  P.t0 = a.t0;
  P.init_buffer = a.init_buffer;
  P.term_buffer = a.term_buffer;
  P.window = a.window;
  P.seed = a.seed;
  P.id_base = a.chain_id;
  P.init_radius = a.init_radius;
  P.has_init = inits != nullptr;
  P.replay = p0 != nullptr;
  P.n_saved = (a.save_warmup ? (a.num_warmup + a.thin - 1) / a.thin : 0) + (a.num_samples + a.thin - 1) / a.thin;
  P.grad_budget = 2048;
  // diagnostic_file rows (plain runs; a flow run's sampler space is z)
  P.diag = out && out->diagnostics && !rc.flow && !p0 ? 1 : 0;
  P.nrv = P.diag ? 8 : 7;
  // cache the chain vectors in shared memory when four chains fit in a block's
  // budget.  It pays where a launch runs many steps of a chain (fused mode);
  // in round mode a launch runs one step and the copy in / out costs what it
  // saves (measured on the logistic workload: 63.4 us with, 60.0 us without).
  {
    const int nvec = P.metric == 1 ? NCACHE_VEC : NCACHE_VEC_DIAG;
    P.cache_stride = (nvec * P.ld + P.R * 3 + 1) & ~1;
    const size_t bytes = 4 * (size_t)P.cache_stride * sizeof(double);
    const bool rounds = use_rounds(m) && !p0 && !rc.flow;
    P.cache = bytes <= 160 * 1024 && !rounds;
    if (P.cache) {
      GN_CUDA(fused_set_smem(m.dev.kind, (int)bytes));
      GN_CUDA((advance_set_smem_k<0, 32>((int)bytes)));
      GN_CUDA((advance_set_smem_k<1, 32>((int)bytes)));
      GN_CUDA((advance_set_smem_k<2, 32>((int)bytes)));
    } else if (!rounds && (size_t)P.cache_stride * sizeof(double) <= 200 * 1024) {
      // large chains: the cache can still hold one or two chains per CTA
      // (the fused-mode autotuner decides whether that pays)
      const size_t one = (size_t)P.cache_stride * sizeof(double);
      GN_CUDA(fused_set_smem(m.dev.kind, (int)std::min<size_t>(2 * one <= 200 * 1024 ? 2 * one : one, 200 * 1024)));
    }
    // a wide dense-metric chain on the mixed path: its team does the metric
    // product, momentum draw and covariance updates in FP32
    P.dense32 = rc.metric == 1 && rounds && !P.cache && a.precision == GNUTS_PRECISION_MIXED && D >= TEAM_MIN_D &&
                D <= DENSE32_MAXD;
  }

  Arena ar;
  Bufs B{};
  const size_t vec = (size_t)C * P.ld;
  const size_t mat = P.metric == 1 ? (size_t)C * D * P.ld : vec;
  double** vecs[] = {&B.Wq, &B.Wp, &B.Wg, &B.Fq, &B.Fp, &B.Fg, &B.Bq, &B.Bp, &B.Bg, &B.Sq, &B.Sg,
                     &B.Tpb, &B.Tsb, &B.Tpe, &B.Tse, &B.Trho, &B.wm, &B.tmp};
  for (double** v : vecs) GN_CUDA(ar.alloc(v, vec));
  GN_CUDA(ar.alloc(&B.rec, vec * P.R * P.nrv));
  if (P.diag) {
    GN_CUDA(ar.alloc(&B.Sp, vec));
    GN_CUDA(ar.alloc(&B.diag_draws, (size_t)C * P.n_saved * (7 + 3 * (size_t)D)));
  }
  GN_CUDA(ar.alloc(&B.recs, (size_t)C * P.R * 3));
  GN_CUDA(ar.alloc(&B.minv, mat));
  GN_CUDA(ar.alloc(&B.wm2, mat));
  if (P.metric == 1) GN_CUDA(ar.alloc(&B.chol, mat));
  if (P.dense32) {
    GN_CUDA(ar.alloc(&B.minv32, mat));
    GN_CUDA(ar.alloc(&B.chol32, mat));
    GN_CUDA(ar.alloc(&B.wm2_32, mat));
    GN_CUDA(ar.alloc(&B.wm2_32lo, mat));
    GN_CUDA(ar.alloc(&B.wpend, vec * 4));
    GN_CUDA(ar.alloc(&B.wlist, (size_t)C + 2));
  }
  GN_CUDA(ar.alloc(&B.draws, (size_t)C * P.n_saved * P.ncol));
  GN_CUDA(ar.alloc(&B.out_eps, C));
  const size_t msz = P.metric == 1 ? (size_t)D * D : (size_t)D;
  GN_CUDA(ar.alloc(&B.out_minv, (size_t)C * msz));
  GN_CUDA(ar.alloc(&B.sc, C));
  GN_CUDA(ar.alloc(&B.done_count, 1));
  double* d_inv = nullptr;
  if (inv_metric) {
    GN_CUDA(ar.alloc(&d_inv, (size_t)C * msz));
    GN_CUDA(cudaMemcpy(d_inv, inv_metric, sizeof(double) * C * msz, cudaMemcpyHostToDevice));
  }
  if (inits) {
    double* d;
    GN_CUDA(ar.alloc(&d, (size_t)C * D));
    GN_CUDA(cudaMemcpy(d, inits, sizeof(double) * C * D, cudaMemcpyHostToDevice));
    B.init_q = d;
  }
  if (p0) {
    double* d;
    GN_CUDA(ar.alloc(&d, (size_t)C * D));
    GN_CUDA(cudaMemcpy(d, p0, sizeof(double) * C * D, cudaMemcpyHostToDevice));
    B.p0 = d;
  }
  if (rc.stepsizes) {
    double* d;
    GN_CUDA(ar.alloc(&d, (size_t)C));
    GN_CUDA(cudaMemcpy(d, rc.stepsizes, sizeof(double) * C, cudaMemcpyHostToDevice));
    B.init_eps = d;
  }
  if (rc.flow) {
    if (rc.flow->d != D || p0) {
      err = "flow dimension does not match the model's";
      return GNUTS_ERR_ARGUMENT;
    }
    GN_CUDA(ar.alloc(&B.zdraws, (size_t)C * P.n_saved * D));
  }
  ReplayBufs RB{nullptr, nullptr};
  if (chain_ids) {
    unsigned* d;
    GN_CUDA(ar.alloc(&d, C));
    GN_CUDA(cudaMemcpy(d, chain_ids, sizeof(unsigned) * C, cudaMemcpyHostToDevice));
    RB.chain_ids = d;
  }
  if (counters) {
    unsigned long long* d;
    GN_CUDA(ar.alloc(&d, C));
    GN_CUDA(cudaMemcpy(d, counters, sizeof(uint64_t) * C, cudaMemcpyHostToDevice));
    RB.rng_start = d;
  }

  const int threads = 128;
  const int blocks = (C * 32 + threads - 1) / threads;
  k_init<<<blocks, threads>>>(P, B, m.dev, d_inv, RB);
  GN_CUDA(cudaGetLastError());

  // Upper bound on launches: every transition needs at most 2^max_depth
  // gradients; step-size searches are bounded by the 1e7 / 0 step-size
  // limits (about 1100 halvings or 24 doublings per search).
  const double per_chain_max = (double)(a.num_warmup + a.num_samples) * (double)(1 << std::min(a.max_depth, 20)) +
                               8.0 * 1200.0 + 200.0;
  int done = 0;
  RunStats stats;
  // draw sink and interrupt callback of this thread (not for replayed transitions)
  DrawStreamer streamer(P, B, !p0);
  if (rc.flow) {
    double fs[6] = {0, 0, 0, 0, 0, 4};
    st = run_flow_fused(m, *rc.flow, P, B, per_chain_max, fs, err);
    if (st) return st;
    stats.rounds = fs[0];
    stats.device_ms = fs[1];
    stats.launches = fs[2];
    stats.grad_us = fs[3];
    stats.advance_us = fs[4];
    stats.chains_per_cta = fs[5];
    GN_CUDA(cudaMemcpy(&done, B.done_count, sizeof(int), cudaMemcpyDeviceToHost));
    if (done >= C) {
      st = flow_finalize_draws(m, *rc.flow, C * P.n_saved, B.zdraws, B.draws, P.ncol, err);
      if (st) return st;
      stats.launches += 1;
    }
  } else if (use_rounds(m) && !p0) {
    st = run_rounds(m, P, B, a.precision, per_chain_max, a.refresh, progress, ctx, streamer, stats, err);
    if (st) return st;
    GN_CUDA(cudaMemcpy(&done, B.done_count, sizeof(int), cudaMemcpyDeviceToHost));
  } else {
    const long long max_launches = (long long)(per_chain_max / P.grad_budget) + 16;
    int last_reported = -1;
    cudaEvent_t f0, f1;
    GN_CUDA(cudaEventCreate(&f0));
    GN_CUDA(cudaEventCreate(&f1));
    struct FEv { cudaEvent_t a, b; ~FEv() { cudaEventDestroy(a); cudaEventDestroy(b); } } fev{f0, f1};
    GN_CUDA(cudaEventRecord(f0));
    // Launch shape autotuner: chains per CTA (1, 2 or 4 warps) and whether the
    // chain vectors are cached in shared memory.  Each candidate runs one
    // short launch of the real run (the chains advance; what a chain computes
    // does not depend on the launch shape), and the fastest one is kept.
    int warps = 4;
    if (C >= 64 && !p0) {
      cudaEvent_t t0, t1;
      GN_CUDA(cudaEventCreate(&t0));
      GN_CUDA(cudaEventCreate(&t1));
      struct TEv { cudaEvent_t a, b; ~TEv() { cudaEventDestroy(a); cudaEventDestroy(b); } } tev{t0, t1};
      Params Pt = P;
      Pt.grad_budget = 32;
      float best = 1e30f;
      int best_w = 4, best_c = P.cache;
      for (int w : {4, 2, 1})
        for (int cch = 1; cch >= 0; --cch) {
          // shared-memory budget of a CTA's cached chains (as set above)
          if (cch && (size_t)w * P.cache_stride * sizeof(double) > (w == 4 ? 160 : 200) * 1024) continue;
          Pt.cache = cch;
          const int bl = (C + w - 1) / w;
          const size_t sm = cch ? (size_t)w * P.cache_stride * sizeof(double) : 0;
          GN_CUDA(cudaEventRecord(t0));
          GN_CUDA(fused_launch(m.dev.kind, bl, 32 * w, sm, Pt, B, m.dev, RB));
          GN_CUDA(cudaEventRecord(t1));
          GN_CUDA(cudaEventSynchronize(t1));
          float ms = 0;
          cudaEventElapsedTime(&ms, t0, t1);
          stats.rounds += 1;
          stats.launches += 1;
          if (ms < best) {
            best = ms;
            best_w = w;
            best_c = cch;
          }
        }
      warps = best_w;
      P.cache = best_c;
      stats.chains_per_cta = warps;
      GN_CUDA(cudaMemcpy(&done, B.done_count, sizeof(int), cudaMemcpyDeviceToHost));
    }
    const int fthreads = 32 * warps, fblocks = (C + warps - 1) / warps;
    const size_t fsmem = P.cache ? (size_t)warps * P.cache_stride * sizeof(double) : 0;
    for (long long l = 0; l < max_launches && done < C; ++l) {
      GN_CUDA(fused_launch(m.dev.kind, fblocks, fthreads, fsmem, P, B, m.dev, RB));
      stats.rounds += 1;
      stats.launches += 1;
      GN_CUDA(cudaMemcpy(&done, B.done_count, sizeof(int), cudaMemcpyDeviceToHost));
      if (streamer.active()) {
        if ((st = streamer.request_rows(0, 0, err))) return st;
        GN_CUDA(cudaStreamSynchronize(0));
        if ((st = streamer.deliver(0, err))) return st;
      }
      if (!p0 && interrupt_requested()) {
        err = kInterrupted;
        return GNUTS_ERR_INTERRUPTED;
      }
      if (progress && a.refresh > 0) {
        Scal s0;
        GN_CUDA(cudaMemcpy(&s0, B.sc, sizeof(Scal), cudaMemcpyDeviceToHost));
        int it = s0.iter;
        if (it / a.refresh != last_reported) {
          last_reported = it / a.refresh;
          progress(ctx, 0, it, a.num_warmup + a.num_samples, it < a.num_warmup);
        }
      }
      if (done >= C) break;
    }
    GN_CUDA(cudaEventRecord(f1));
    GN_CUDA(cudaEventSynchronize(f1));
    float ms = 0;
    cudaEventElapsedTime(&ms, f0, f1);
    stats.device_ms = ms;
    stats.advance_us = stats.rounds > 0 ? 1e3 * ms / stats.rounds : 0;
  }
  stats.launches += 1;  // k_init
  GN_CUDA(cudaDeviceSynchronize());
  if (done < C) {
    err = "sampler did not finish within its launch bound";
    return GNUTS_ERR_TIMEOUT;
  }

  if ((st = streamer.finish(err))) return st;
  NvtxRange out_range("gnuts.nuts.copy_out");
  std::vector<Scal> sc(C);
  GN_CUDA(cudaMemcpy(sc.data(), B.sc, sizeof(Scal) * C, cudaMemcpyDeviceToHost));
  if (out) {
    if (out->draws)
      GN_CUDA(cudaMemcpy(out->draws, B.draws, sizeof(double) * C * P.n_saved * P.ncol, cudaMemcpyDeviceToHost));
    if (P.diag)
      GN_CUDA(cudaMemcpy(out->diagnostics, B.diag_draws, sizeof(double) * C * P.n_saved * (7 + 3 * (size_t)D),
                         cudaMemcpyDeviceToHost));
    if (out->stepsize) GN_CUDA(cudaMemcpy(out->stepsize, B.out_eps, sizeof(double) * C, cudaMemcpyDeviceToHost));
    if (out->inv_metric)
      GN_CUDA(cudaMemcpy(out->inv_metric, B.out_minv, sizeof(double) * C * msz, cudaMemcpyDeviceToHost));
    for (int c = 0; c < C; ++c) {
      if (out->warmup_seconds) out->warmup_seconds[c] = (double)(sc[c].t_warm - sc[c].t_start) * 1e-9;
      if (out->sampling_seconds) out->sampling_seconds[c] = (double)(sc[c].t_end - sc[c].t_warm) * 1e-9;
      if (out->n_grad) out->n_grad[c] = sc[c].n_grad;
      if (out->n_leapfrog) out->n_leapfrog[c] = sc[c].n_lf_total;
      if (out->chain_status) out->chain_status[c] = sc[c].err ? (sc[c].err == CE_INIT ? GNUTS_ERR_INIT : GNUTS_ERR_SAMPLER) : GNUTS_OK;
    }
    if (out->timing) {
      for (int i = 0; i < GNUTS_TIMING_FIELDS; ++i) out->timing[i] = 0;
      out->timing[GNUTS_TIMING_ROUNDS] = stats.rounds;
      out->timing[GNUTS_TIMING_GRAD_US] = stats.grad_us;
      out->timing[GNUTS_TIMING_ADVANCE_US] = stats.advance_us;
      out->timing[GNUTS_TIMING_DEVICE_MS] = stats.device_ms;
      out->timing[GNUTS_TIMING_LAUNCHES] = stats.launches;
      out->timing[GNUTS_TIMING_REDUCE_US] = stats.reduce_us;
      out->timing[GNUTS_TIMING_CHAINS_PER_CTA] = stats.chains_per_cta;
    }
  }
  if (counters)
    for (int c = 0; c < C; ++c) counters[c] = sc[c].rng_n;
  for (int c = 0; c < C; ++c) {
    if (sc[c].err) {
      char buf[64];
      snprintf(buf, sizeof buf, "chain %u: ", (chain_ids ? chain_ids[c] : a.chain_id + c));
      err = std::string(buf) + chain_error_message(sc[c].err);
      return sc[c].err == CE_INIT ? GNUTS_ERR_INIT : GNUTS_ERR_SAMPLER;
    }
  }
  if (replay_q_out)
    GN_CUDA(cudaMemcpy2D(replay_q_out, sizeof(double) * D, B.Sq, sizeof(double) * P.ld, sizeof(double) * D, C,
                         cudaMemcpyDeviceToHost));
  if (rc.q_last)
    GN_CUDA(cudaMemcpy2D(rc.q_last, sizeof(double) * D, B.Sq, sizeof(double) * P.ld, sizeof(double) * D, C,
                         cudaMemcpyDeviceToHost));
  return GNUTS_OK;
}

int run_transition(Model& m, int metric, const double* inv_metric, int n, const double* q0, const double* p0,
                   double eps, int max_depth, unsigned seed, const unsigned* chain_ids, uint64_t* counters,
                   double* q_out, double* stats, std::string& err) {
  gnuts_sample_args a;
  gnuts_sample_args_default(&a);
  a.num_chains = n;
  a.seed = seed;
  a.num_warmup = 0;
  a.num_samples = 1;
  a.thin = 1;
  a.save_warmup = 0;
  a.stepsize = eps;
  a.stepsize_jitter = 0;
  a.max_depth = max_depth;
  const int D = m.dev.D;
  const size_t msz = metric == 1 ? (size_t)D * D : (size_t)D;
  std::vector<double> im;
  if (metric != 2 && inv_metric) {
    im.resize((size_t)n * msz);
    for (int i = 0; i < n; ++i) std::memcpy(&im[(size_t)i * msz], inv_metric, sizeof(double) * msz);
  }
  const int ncol = 7 + m.dev.ncon;
  std::vector<double> draws((size_t)n * ncol);
  gnuts_output out{};
  out.draws = draws.data();
  RunConfig rc{metric, 0};
  int st = run_nuts_impl(m, a, rc, q0, im.empty() ? nullptr : im.data(), p0, chain_ids, counters, q_out, &out,
                         nullptr, nullptr, err);
  if (st) return st;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 7; ++k) stats[(size_t)i * 7 + k] = draws[(size_t)i * ncol + k];
  return GNUTS_OK;
}

static int check_points(const Model& m, int n, std::string& err) {
  if (m.dev.n_members && n % m.dev.n_members != 0) {
    err = "a posterior set evaluates a multiple of its " + std::to_string(m.dev.n_members) +
          " posteriors' points (point i belongs to posterior i / (n / P))";
    return GNUTS_ERR_ARGUMENT;
  }
  return GNUTS_OK;
}

int run_log_prob_grad(Model& m, int n, const double* q, int jacobian, int precision, double* lp, double* grad,
                      std::string& err) {
  int st = upload(m, err);
  if (st) return st;
  if (n <= 0) return GNUTS_OK;
  if ((st = check_points(m, n, err))) return st;
  const int D = m.dev.D;
  Arena ar;
  double *dq, *dg, *dl;
  GN_CUDA(ar.alloc(&dq, (size_t)n * D));
  GN_CUDA(ar.alloc(&dg, (size_t)n * D));
  GN_CUDA(ar.alloc(&dl, n));
  GN_CUDA(cudaMemcpy(dq, q, sizeof(double) * n * D, cudaMemcpyHostToDevice));
  if (!use_rounds(m) && (st = check_warp_limits(m, err))) return st;
  if (use_rounds(m)) {
    st = batched_log_prob_grad(m.dev, n, dq, jacobian, dl, dg, precision, err);
    if (st) return st;
  } else {
    const int threads = 128, blocks = (n * 32 + threads - 1) / threads;
    k_log_prob_grad<<<blocks, threads>>>(m.dev, n, dq, jacobian, dl, dg);
    GN_CUDA(cudaGetLastError());
  }
  GN_CUDA(cudaMemcpy(lp, dl, sizeof(double) * n, cudaMemcpyDeviceToHost));
  GN_CUDA(cudaMemcpy(grad, dg, sizeof(double) * n * D, cudaMemcpyDeviceToHost));
  return GNUTS_OK;
}

int run_write_array(Model& m, int n, const double* q, double* out, std::string& err) {
  int st = upload(m, err);
  if (st) return st;
  if (n <= 0) return GNUTS_OK;
  if ((st = check_points(m, n, err))) return st;
  const int D = m.dev.D, K = m.dev.ncon;
  Arena ar;
  double *dq, *dout;
  GN_CUDA(ar.alloc(&dq, (size_t)n * D));
  GN_CUDA(ar.alloc(&dout, (size_t)n * K));
  GN_CUDA(cudaMemcpy(dq, q, sizeof(double) * n * D, cudaMemcpyHostToDevice));
  const int threads = 128, blocks = (n * 32 + threads - 1) / threads;
  k_write_array<<<blocks, threads>>>(m.dev, n, dq, dout);
  GN_CUDA(cudaGetLastError());
  GN_CUDA(cudaMemcpy(out, dout, sizeof(double) * n * K, cudaMemcpyDeviceToHost));
  return GNUTS_OK;
}

}  // namespace gnuts
