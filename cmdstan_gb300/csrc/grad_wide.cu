// Batched logistic-likelihood gradient for wide designs (more predictors than
// the tcgen05 kernel's 128-column tile: the regularised-horseshoe workload,
// X 200,000 x 1000) on the tensor cores through cuBLASLt.  The two
// contractions of the likelihood gradient are plain GEMMs with an elementwise
// step between them, so they go to the library; the elementwise step is a
// kernel of this project:
//
//   GEMM1  H = X [beta_hi | beta_lo]          BF16 x BF16 -> FP32, N x 2C
//   epi    eta = H_hi + H_lo + b0;  lp += y eta - softplus(eta);
//          r = y - inv_logit(eta) -> BF16;  per-block sums of lp and r
//   GEMM2  G = X^T R                          BF16 x BF16 -> FP32, K x C
//   final  partials [1][C][K+1] (intercept from the r sums) and lp [1][C],
//          the layout the state machine's reduce_gradient consumes
//
// The likelihood is the one of stan::model::log_prob_grad for the logistic
// GLM (the gradient contract of src/cmdstan/command_helper.hpp:589-593);
// coefficient transforms and priors stay in stage_request / reduce_gradient.
// Precision matches the tcgen05 path: X BF16-exact, coefficients split into
// two BF16 parts (16 significant bits), FP32 accumulation, residuals BF16,
// per-warp sums in FP32 and per-block / per-chain sums in FP64, all in a
// fixed order (bitwise reproducible run to run).
#include <cublasLt.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <string>
#include "internal.h"
#include "batched.cuh"
#include "grad_wide.h"

namespace gnuts {

namespace {
constexpr int WE_THREADS = 256;
constexpr int WE_ROWS = 4 * WE_THREADS;  // rows per epilogue block
constexpr size_t WIDE_WS_BYTES = 64ull << 20;
}  // namespace

struct WidePlan {
  cublasLtHandle_t lt = nullptr;
  cublasLtMatmulDesc_t d1 = nullptr, d2 = nullptr;
  cublasLtMatrixLayout_t a1 = nullptr, b1 = nullptr, c1 = nullptr, a2 = nullptr, b2 = nullptr, c2 = nullptr;
  cublasLtMatmulAlgo_t algo1{}, algo2{};
  void* ws = nullptr;
  __nv_bfloat16* bcat = nullptr;  // K x 2C column-major: chain c's hi in column c, lo in column C + c
  float* h = nullptr;             // N x 2C column-major
  __nv_bfloat16* r = nullptr;     // N x C column-major (residuals)
  float* gk = nullptr;            // K x C column-major
  double *plp = nullptr, *pr = nullptr;  // [NB][C] block sums of lp and of r
  double* coef64 = nullptr;               // [C][K+1] coefficient rows (stage_request)
  double *part_lp = nullptr, *part_g = nullptr;  // [1][C], [1][C][K+1] for reduce_gradient
  int C = 0, K = 0, N = 0, NB = 0;
};

bool wide_supported(const DevModel& M) {
  return (M.kind == MK_LOGISTIC || M.kind == MK_HORSESHOE) && M.Xb && M.yi && M.K % 8 == 0 && M.N % 8 == 0 &&
         M.N > 0 && M.K >= 8;
}

// coefficient rows -> the two BF16 parts of GEMM1's B operand
__global__ void k_wide_stage(const double* coef64, int C, int K, __nv_bfloat16* bcat) {
  const size_t n = (size_t)C * K;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / K), k = (int)(i % K);
    const double v = coef64[(size_t)c * (K + 1) + 1 + k];
    const __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
    bcat[i] = hi;
    bcat[(size_t)C * K + i] = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
  }
}

// eta, the likelihood's lp terms and residuals of chain blockIdx.y over rows
// [blockIdx.x * WE_ROWS, +WE_ROWS).  FP32 per element and per warp (shuffle
// sums in a fixed order); the block's eight warp sums are added in FP64 by
// one thread: the block does two FP64 additions per warp, not a tree of them
// (this part's FP64 pipe is narrow).
__global__ void __launch_bounds__(WE_THREADS) k_wide_epi(const float* __restrict__ h, const double* coef64,
                                                         const int* __restrict__ y, int N, int C, int K,
                                                         __nv_bfloat16* __restrict__ r, double* plp,
                                                         double* pr) {
  const int c = blockIdx.y;
  const float b0 = (float)coef64[(size_t)c * (K + 1)];
  const float* hh = h + (size_t)c * N;
  const float* hl = h + ((size_t)C + c) * N;
  __nv_bfloat16* rr = r + (size_t)c * N;
  float lp = 0.f, rs = 0.f;
  const int n0 = blockIdx.x * WE_ROWS + threadIdx.x;
  float eh[4], el[4], yv[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int n = n0 + j * WE_THREADS;
    const bool ok = n < N;
    eh[j] = ok ? hh[n] : 0.f;
    el[j] = ok ? hl[n] : 0.f;
    yv[j] = ok ? (float)y[n] : 0.f;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int n = n0 + j * WE_THREADS;
    if (n < N) {
      const float eta = eh[j] + el[j] + b0;
      // softplus(eta) = max(eta, 0) + log1p(exp(-|eta|)); inv_logit from the same exponential
      const float e = __expf(-fabsf(eta));
      const float d = 1.f + e;
      const float sp = fmaxf(eta, 0.f) + __logf(d);
      const float sig = __fdividef(eta >= 0.f ? 1.f : e, d);
      lp += fmaf(yv[j], eta, -sp);
      const float res = yv[j] - sig;
      rs += res;
      rr[n] = __float2bfloat16_rn(res);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lp += __shfl_xor_sync(0xffffffffu, lp, o);
    rs += __shfl_xor_sync(0xffffffffu, rs, o);
  }
  __shared__ float s_lp[WE_THREADS / 32], s_r[WE_THREADS / 32];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_lp[w] = lp;
    s_r[w] = rs;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int k = 0; k < WE_THREADS / 32; ++k) {
      a += (double)s_lp[k];
      b += (double)s_r[k];
    }
    plp[(size_t)blockIdx.x * C + c] = a;
    pr[(size_t)blockIdx.x * C + c] = b;
  }
}

// block sums and GEMM2's columns -> the consumer's partials.  One warp per
// chain: lane l sums blocks l, l + 32, ... in order, then a fixed butterfly.
__global__ void k_wide_final(const double* plp, const double* pr, const float* gk, int NB, int C, int K,
                             double* part_lp, double* part_g) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (c >= C) return;
  double a = 0, b = 0;
  for (int s = lane; s < NB; s += 32) {
    a += plp[(size_t)s * C + c];
    b += pr[(size_t)s * C + c];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  double* g = part_g + (size_t)c * (K + 1);
  if (lane == 0) {
    part_lp[c] = a;
    g[0] = b;
  }
  const float* src = gk + (size_t)c * K;
  for (int k = lane; k < K; k += 32) g[1 + k] = (double)src[k];
}

namespace {
const char* lt_name(cublasStatus_t s) {
  switch (s) {
    case CUBLAS_STATUS_SUCCESS: return "success";
    case CUBLAS_STATUS_NOT_INITIALIZED: return "not initialized";
    case CUBLAS_STATUS_ALLOC_FAILED: return "allocation failed";
    case CUBLAS_STATUS_INVALID_VALUE: return "invalid value";
    case CUBLAS_STATUS_ARCH_MISMATCH: return "architecture mismatch";
    case CUBLAS_STATUS_EXECUTION_FAILED: return "execution failed";
    case CUBLAS_STATUS_NOT_SUPPORTED: return "not supported";
    default: return "error";
  }
}
}  // namespace

#define WL_CHECK(call)                                                                 \
  do {                                                                                 \
    cublasStatus_t s_ = (call);                                                        \
    if (s_ != CUBLAS_STATUS_SUCCESS) {                                                 \
      err = std::string("cuBLASLt ") + lt_name(s_) + " at " #call;                    \
      wide_destroy(p);                                                                 \
      return GNUTS_ERR_CUDA;                                                           \
    }                                                                                  \
  } while (0)
#define WC_CHECK(call)                                                                 \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      err = std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call;      \
      wide_destroy(p);                                                                 \
      return GNUTS_ERR_CUDA;                                                           \
    }                                                                                  \
  } while (0)

void wide_destroy(WidePlan* p) {
  if (!p) return;
  for (auto* l : {p->a1, p->b1, p->c1, p->a2, p->b2, p->c2})
    if (l) cublasLtMatrixLayoutDestroy(l);
  if (p->d1) cublasLtMatmulDescDestroy(p->d1);
  if (p->d2) cublasLtMatmulDescDestroy(p->d2);
  if (p->lt) cublasLtDestroy(p->lt);
  for (void* q : {(void*)p->ws, (void*)p->bcat, (void*)p->h, (void*)p->r, (void*)p->gk, (void*)p->plp, (void*)p->pr,
                  (void*)p->coef64, (void*)p->part_lp, (void*)p->part_g})
    if (q) cudaFree(q);
  delete p;
}

int wide_create(const DevModel& M, int C, WidePlan** out, double** coef64, double** part_lp, double** part_g,
                std::string& err) {
  *out = nullptr;
  if (C < 1 || C > 65535) {  // the epilogue's grid has one y-block per chain
    err = "the wide-design gradient takes 1 to 65535 chains";
    return GNUTS_ERR_ARGUMENT;
  }
  WidePlan* p = new WidePlan();
  p->C = C;
  p->K = M.K;
  p->N = M.N;
  p->NB = (M.N + WE_ROWS - 1) / WE_ROWS;
  const size_t N = (size_t)M.N, K = (size_t)M.K, C2 = 2 * (size_t)C;
  WC_CHECK(cudaMalloc(&p->ws, WIDE_WS_BYTES));
  WC_CHECK(cudaMalloc(&p->bcat, sizeof(__nv_bfloat16) * K * C2));
  WC_CHECK(cudaMalloc(&p->h, sizeof(float) * N * C2));
  WC_CHECK(cudaMalloc(&p->r, sizeof(__nv_bfloat16) * N * C));
  WC_CHECK(cudaMalloc(&p->gk, sizeof(float) * K * C));
  WC_CHECK(cudaMalloc(&p->plp, sizeof(double) * p->NB * C));
  WC_CHECK(cudaMalloc(&p->pr, sizeof(double) * p->NB * C));
  WC_CHECK(cudaMalloc(&p->coef64, sizeof(double) * C * (K + 1)));
  WC_CHECK(cudaMalloc(&p->part_lp, sizeof(double) * C));
  WC_CHECK(cudaMalloc(&p->part_g, sizeof(double) * C * (K + 1)));
  WC_CHECK(cudaMemset(p->coef64, 0, sizeof(double) * C * (K + 1)));
  WL_CHECK(cublasLtCreate(&p->lt));
  const cublasOperation_t T = CUBLAS_OP_T, Nn = CUBLAS_OP_N;
  // GEMM1: H (N x 2C) = X^T-view (N x K) * Bcat (K x 2C); X is K x N column-major (row-major N x K)
  WL_CHECK(cublasLtMatmulDescCreate(&p->d1, CUBLAS_COMPUTE_32F, CUDA_R_32F));
  WL_CHECK(cublasLtMatmulDescSetAttribute(p->d1, CUBLASLT_MATMUL_DESC_TRANSA, &T, sizeof(T)));
  WL_CHECK(cublasLtMatmulDescSetAttribute(p->d1, CUBLASLT_MATMUL_DESC_TRANSB, &Nn, sizeof(Nn)));
  WL_CHECK(cublasLtMatrixLayoutCreate(&p->a1, CUDA_R_16BF, K, N, K));
  WL_CHECK(cublasLtMatrixLayoutCreate(&p->b1, CUDA_R_16BF, K, C2, K));
  WL_CHECK(cublasLtMatrixLayoutCreate(&p->c1, CUDA_R_32F, N, C2, N));
  // GEMM2: G (K x C) = X (K x N) * R (N x C)
  WL_CHECK(cublasLtMatmulDescCreate(&p->d2, CUBLAS_COMPUTE_32F, CUDA_R_32F));
  WL_CHECK(cublasLtMatmulDescSetAttribute(p->d2, CUBLASLT_MATMUL_DESC_TRANSA, &Nn, sizeof(Nn)));
  WL_CHECK(cublasLtMatmulDescSetAttribute(p->d2, CUBLASLT_MATMUL_DESC_TRANSB, &Nn, sizeof(Nn)));
  WL_CHECK(cublasLtMatrixLayoutCreate(&p->a2, CUDA_R_16BF, K, N, K));
  WL_CHECK(cublasLtMatrixLayoutCreate(&p->b2, CUDA_R_16BF, N, C, N));
  WL_CHECK(cublasLtMatrixLayoutCreate(&p->c2, CUDA_R_32F, K, C, K));
  cublasLtMatmulPreference_t pref = nullptr;
  WL_CHECK(cublasLtMatmulPreferenceCreate(&pref));
  size_t wsb = WIDE_WS_BYTES;
  cublasStatus_t s = cublasLtMatmulPreferenceSetAttribute(pref, CUBLASLT_MATMUL_PREF_MAX_WORKSPACE_BYTES, &wsb,
                                                          sizeof(wsb));
  cublasLtMatmulHeuristicResult_t h1{}, h2{};
  int n1 = 0, n2 = 0;
  if (s == CUBLAS_STATUS_SUCCESS)
    s = cublasLtMatmulAlgoGetHeuristic(p->lt, p->d1, p->a1, p->b1, p->c1, p->c1, pref, 1, &h1, &n1);
  if (s == CUBLAS_STATUS_SUCCESS)
    s = cublasLtMatmulAlgoGetHeuristic(p->lt, p->d2, p->a2, p->b2, p->c2, p->c2, pref, 1, &h2, &n2);
  cublasLtMatmulPreferenceDestroy(pref);
  WL_CHECK(s);
  if (n1 < 1 || n2 < 1) {
    err = "cuBLASLt found no algorithm for the wide gradient's GEMMs";
    wide_destroy(p);
    return GNUTS_ERR_CUDA;
  }
  p->algo1 = h1.algo;
  p->algo2 = h2.algo;
  *coef64 = p->coef64;
  *part_lp = p->part_lp;
  *part_g = p->part_g;
  *out = p;
  return GNUTS_OK;
}

int wide_launch(const WidePlan* p, const GradOut& G, const DevModel& M, cudaStream_t st) {
  const float one = 1.f, zero = 0.f;
  const int C = p->C, K = p->K, N = p->N;
  k_wide_stage<<<std::min(4096, (C * K + 255) / 256), 256, 0, st>>>(G.coef64, C, K, p->bcat);
  if (cublasLtMatmul(p->lt, p->d1, &one, M.Xb, p->a1, p->bcat, p->b1, &zero, p->h, p->c1, p->h, p->c1, &p->algo1,
                     p->ws, WIDE_WS_BYTES, st) != CUBLAS_STATUS_SUCCESS)
    return GNUTS_ERR_CUDA;
  k_wide_epi<<<dim3(p->NB, C), WE_THREADS, 0, st>>>(p->h, G.coef64, M.yi, N, C, K, p->r, p->plp, p->pr);
  if (cublasLtMatmul(p->lt, p->d2, &one, M.Xb, p->a2, p->r, p->b2, &zero, p->gk, p->c2, p->gk, p->c2, &p->algo2,
                     p->ws, WIDE_WS_BYTES, st) != CUBLAS_STATUS_SUCCESS)
    return GNUTS_ERR_CUDA;
  k_wide_final<<<(C * 32 + 255) / 256, 256, 0, st>>>(p->plp, p->pr, p->gk, p->NB, C, K, G.part_lp, G.part_g);
  return cudaGetLastError() == cudaSuccess ? GNUTS_OK : GNUTS_ERR_CUDA;
}

}  // namespace gnuts
