// Internal declarations shared by the C-ABI layer (abi.cpp) and the CUDA
// translation units.  Not part of the public interface.
#pragma once
#include <stdint.h>
#include <string>
#include <vector>
#include <nvtx3/nvToolsExt.h>
#include "../../include/gnuts.h"

namespace gnuts {

// NVTX range for the duration of a scope (visible in Nsight timelines; a no-op
// when no tool is attached)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

enum ModelKind : int {
  MK_BERNOULLI = 0,
  MK_NORMAL = 1,
  MK_LOGISTIC = 2,
  MK_HIER = 3,
  MK_FUNNEL = 4,
  MK_VARINT = 5,
  MK_HORSESHOE = 6,
};

// Device-resident model data.  Plain struct copied by value into kernels.
struct DevModel {
  int kind;
  int D;       // unconstrained dimension
  int ncon;    // write_array columns
  int N, J, K; // sizes (meaning depends on kind)
  int ysum;    // bernoulli: sum(y)
  const int* yi;
  const double* yr;
  const double* X;       // FP64 row-major N x (D or K)
  const float* Xf;       // FP32 copy (same values)
  const uint16_t* Xb;    // BF16 copy (same values when X is bf16-representable)
  const int* group;      // varint: 1-based group ids, rows sorted by group
  const int* gstart;     // varint: J+1 row offsets
  const double* sigma;
  const double* scales;
  double scale_global, slab_scale, slab_df;
  // tensor-core layout (logistic, K + 1 <= 128): X as BF16 rows of XTC_LD
  // elements [x_1..x_K, 1, 0...] (the ones column carries the intercept) and
  // y packed 32 rows per word
  const uint16_t* Xtc;
  const uint32_t* ybits;
  // Xtc^T (y - 1/2) in FP64, XTC_LD entries: the linear part of the
  // likelihood is B . xtc_ym for a coefficient row B in Xtc's column order
  const double* xtc_ym;
  // varint: parameter order [beta, log sigma_y, log tau, alpha] (posterior
  // sets, so that the shared parameters sit in the same columns for every
  // posterior) and FP32 likelihood rows (FP64 sums across groups)
  int alpha_last, fp32;
  // posterior set: chain (or point) c of C uses members[c / (C / n_members)]
  const DevModel* members;
  int n_members;
};
constexpr int XTC_LD = 104;  // row stride in elements (208 B, a multiple of 16 B)
constexpr int TC_GSTRIDE = 128;  // FP32 gradient partials per chain of the tensor-core path

struct Model {
  std::string id, name;
  DevModel dev{};
  bool x_bf16_exact = false;
  std::vector<std::string> con_names, unc_names;
  // host copies used for unconstraining / write_array on the host
  std::vector<double> host_X;
  std::vector<int> host_yi;
  std::vector<void*> device_allocs;
  int device = -1;
  // posterior set: members with row / group offsets into the shared arrays
  struct Member { int N, J, D; long row_off, g_off; };
  std::vector<Member> members;
  ~Model();
};

// Affine-coupling flow (flow.cu): host-side layout plus device buffers.
struct Flow {
  int d = 0, L = 0, H = 0;
  float clamp = 4.0f;
  std::vector<int> nb, na, idx, idx_off;  // idx: per layer b list then a list
  std::vector<long> th_off, w_off;        // th_off has L + 1 entries (th_off[L] = mu)
  std::vector<long> wt_off;               // tensor-core weight blocks (zero-padded, see flow.cuh)
  long th_rho = 0, n_params = 0, n_w16 = 0, n_w16t = 0;
  int stage_max = 0, stage_max_tc = 0;
  int device = -1;
  float *theta = nullptr, *adam_m = nullptr, *adam_v = nullptr, *grad = nullptr;
  uint16_t* w16 = nullptr;
  uint16_t* w16t = nullptr;
  int* didx = nullptr;
  int* nvalid = nullptr;  // [2] valid-point counters of the training steps
  ~Flow();
};

struct RunConfig {
  int metric;   // 0 diag, 1 dense, 2 unit
  int adapt;
  const Flow* flow = nullptr;      // sample z with x = T(z) (learned preconditioner)
  const double* stepsizes = nullptr;  // per-chain initial step size (NULL: the argument's)
  double* q_last = nullptr;        // [C][D] final sampler-space position of every chain
};

// thread-local callbacks of the sampling services (gnuts_set_interrupt,
// gnuts_set_draw_sink); sampler.cu and flow.cu poll them between launches
struct RunHooks {
  gnuts_interrupt_fn interrupt = nullptr;
  void* interrupt_ctx = nullptr;
  gnuts_draws_fn sink = nullptr;
  void* sink_ctx = nullptr;
};
RunHooks& run_hooks();
inline bool interrupt_requested() {
  const RunHooks& h = run_hooks();
  return h.interrupt && h.interrupt(h.interrupt_ctx) != 0;
}

// sampler.cu
int run_nuts(Model& m, const gnuts_sample_args& a, const RunConfig& rc, const double* inits,
             const double* inv_metric, gnuts_output* out, gnuts_progress_fn progress, void* ctx,
             std::string& err);
int run_transition(Model& m, int metric, const double* inv_metric, int n, const double* q0,
                   const double* p0, double eps, int max_depth, unsigned seed,
                   const unsigned* chain_ids, uint64_t* counters, double* q_out, double* stats,
                   std::string& err);
int run_log_prob_grad(Model& m, int n, const double* q, int jacobian, int precision, double* lp, double* grad,
                      std::string& err);
int run_write_array(Model& m, int n, const double* q, double* out, std::string& err);
int upload(Model& m, std::string& err);
// abi.cpp: record the calling thread's last error (returns code); argument checks of the services
int api_fail(int code, const std::string& msg);
int validate_args(const Model& m, const gnuts_sample_args* a, int adapt, int metric);

// flow.cu
int flow_create(int d, int L, int H, double clamp, Flow** out, std::string& err);
int flow_set_params(Flow& f, const double* theta, std::string& err);
int flow_get_params(const Flow& f, double* theta, std::string& err);
int flow_forward(Flow& f, int n, const double* z, double* x, double* logdet, std::string& err);
int flow_inverse(Flow& f, int n, const double* x, double* z, double* logdet, std::string& err);
int flow_log_prob_grad(Model& m, Flow& f, int n, const double* z, int jacobian, double* lp, double* grad_z,
                       double* grad_theta, std::string& err);
int flow_adam_step(Flow& f, const double* grad, int t, double lr, double b1, double b2, double eps,
                   std::string& err);
int flow_log_prob_grad_tc(Model& m, Flow& f, int n, const double* z, double* lp, double* grad_z, std::string& err);
int flow_train(Model& m, Flow& f, const gnuts_train_args& ta, double* loss_trace, std::string& err);
// noalloc.cu: the allocation-free batched gradient (device pointers)
int noalloc_log_prob_grad(const Model& m, int n, const double* q, int jac, double* lp, double* g, std::string& err);

}  // namespace gnuts
