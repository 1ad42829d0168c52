/*
 * gnuts -- GB300-native NUTS sampler behind a plain C ABI.
 *
 * This is the drop-in boundary for CmdStan's sampling path.  Each entry
 * point replaces one reference interface; the reference location is cited
 * beside it (paths relative to the CmdStan source tree).  No C++ types,
 * exceptions or device pointers cross this boundary: inputs and outputs are
 * host arrays owned by the caller, errors are integer codes plus a message
 * retrievable with gnuts_last_error().
 *
 * Threading: a model handle may be used by one thread at a time.
 */
#ifndef GNUTS_H
#define GNUTS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes (0 = OK like stan::services::error_codes::OK;
 *      src/cmdstan/return_codes.hpp:7 maps every non-zero to NOT_OK) ---- */
#define GNUTS_OK 0
#define GNUTS_ERR_ARGUMENT 1    /* invalid argument (bad value, bad combination) */
#define GNUTS_ERR_DATA 2        /* missing / malformed data variable */
#define GNUTS_ERR_INIT 3        /* initialisation failed (non-finite lp or gradient) */
#define GNUTS_ERR_SAMPLER 4     /* sampler error (improper posterior, metric overflow) */
#define GNUTS_ERR_CUDA 5        /* CUDA runtime error / no device */
#define GNUTS_ERR_TIMEOUT 6     /* a bounded device wait ran out */
#define GNUTS_ERR_INTERRUPTED 7 /* the caller's interrupt callback asked the run to stop */

/* gradient precision for data-heavy models */
#define GNUTS_PRECISION_FP64 0   /* FP64 everywhere (CUDA cores) */
#define GNUTS_PRECISION_MIXED 1  /* BF16 split-compensated tensor-core contractions, FP64 energy */

/* ---- data: the C form of stan::io::var_context
 *      (built by get_var_context, src/cmdstan/command_helper.hpp:116-133) ---- */
#define GNUTS_VAR_INT 0
#define GNUTS_VAR_REAL 1
typedef struct {
  const char* name;
  int type;              /* GNUTS_VAR_INT (int32 data) or GNUTS_VAR_REAL (double data) */
  int ndim;              /* 0 for scalars */
  const int64_t* dims;   /* ndim extents, row-major data */
  const void* data;
} gnuts_var;

typedef struct gnuts_model gnuts_model;

/* Replaces new_model(var_context&, seed, &cout) (src/cmdstan/command.hpp:170-171)
 * for the stanc-generated model.  model_id names one of the built-in models:
 *   "bernoulli", "normal", "logistic", "hier", "funnel", "varint", "horseshoe". */
int gnuts_model_create(const char* model_id, const gnuts_var* vars, int n_vars, unsigned int seed,
                       gnuts_model** out);
/* Same, with the data given as Stan JSON text (command_helper.hpp:116-133, JSON branch). */
int gnuts_model_create_json(const char* model_id, const char* json_text, unsigned int seed,
                            gnuts_model** out);
void gnuts_model_destroy(gnuts_model* m);

/* model_base::num_params_r and the number of write_array columns
 * (command_helper.hpp:253-264). */
int gnuts_model_dims(const gnuts_model* m, int* num_params_r, int* num_constrained);
/* model_base::model_name (write_model.hpp) */
int gnuts_model_name(const gnuts_model* m, char* buf, size_t len);
/* model_base::constrained_param_names (unconstrained == 0) and
 * unconstrained_param_names (unconstrained != 0), CSV spelling "beta.3" */
int gnuts_model_param_name(const gnuts_model* m, int index, int unconstrained, char* buf, size_t len);

/* stan::model::log_prob_grad<true, jacobian> at n points (command_helper.hpp:589-593),
 * evaluated on the GPU.  q is n x num_params_r, grad is n x num_params_r. */
int gnuts_log_prob_grad(const gnuts_model* m, int n, const double* q, int jacobian, double* lp,
                        double* grad);
/* The same contract (command_helper.hpp:589-593) evaluated with the gradient
 * precision the sampler uses for data-heavy models: GNUTS_PRECISION_MIXED
 * selects the BF16-split tensor-core contraction, FP64 the CUDA-core one. */
int gnuts_log_prob_grad_precision(const gnuts_model* m, int n, const double* q, int jacobian,
                                  int precision, double* lp, double* grad);
/* model_base::transform_inits / unconstrain_array (command_helper.hpp:334-351) */
int gnuts_unconstrain(const gnuts_model* m, const double* constrained, double* unconstrained);
/* model_base::write_array for n unconstrained points -> n x num_constrained */
int gnuts_write_array(const gnuts_model* m, int n, const double* q, double* out);

/* ---- sampler arguments: the values command() reads for the sample branch
 *      (src/cmdstan/command.hpp:554-655) ---- */
typedef struct {
  int num_chains;            /* num_chains (command_helper.hpp:613-642) */
  unsigned int chain_id;     /* id: chain k has id chain_id + k */
  unsigned int seed;         /* random seed */
  double init_radius;        /* init = R (default 2); 0 = all zeros */
  int num_warmup, num_samples, thin, save_warmup;
  int refresh;               /* progress lines every `refresh` iterations (0 = none) */
  double stepsize, stepsize_jitter;
  int max_depth;
  double delta, gamma, kappa, t0;
  unsigned int init_buffer, term_buffer, window;
  int precision;             /* GNUTS_PRECISION_* */
} gnuts_sample_args;

/* Fills the CmdStan defaults (arg_sample.hpp, arg_adapt.hpp, arg_hmc.hpp,
 * arg_nuts.hpp, arg_init.hpp, arg_id.hpp, arg_seed.hpp). */
void gnuts_sample_args_default(gnuts_sample_args* a);

/* Outputs, all caller-allocated host arrays (NULL = not wanted).
 * n_saved = (save_warmup ? ceil(num_warmup/thin) : 0) + ceil(num_samples/thin). */
typedef struct {
  double* draws;             /* [num_chains][n_saved][7 + num_constrained]: lp__, accept_stat__,
                                stepsize__, treedepth__, n_leapfrog__, divergent__, energy__,
                                then write_array values */
  double* stepsize;          /* [num_chains] step size after adaptation */
  double* inv_metric;        /* [num_chains][D] (diag/unit) or [num_chains][D][D] (dense) */
  double* warmup_seconds;    /* [num_chains] */
  double* sampling_seconds;  /* [num_chains] */
  int64_t* n_grad;           /* [num_chains] gradient evaluations incl. init and step-size search */
  int* chain_status;         /* [num_chains] GNUTS_OK or the chain's error code */
  int64_t* n_leapfrog;       /* [num_chains] sum of n_leapfrog__ over all warmup + sampling iterations */
  double* timing;            /* [GNUTS_TIMING_FIELDS] run telemetry, see GNUTS_TIMING_* */
  double* diagnostics;       /* [num_chains][n_saved][7 + 3 * num_params_r]: the rows of CmdStan's
                                diagnostic_file (command.hpp:225-247): the seven sampler columns,
                                then the selected point's unconstrained position q, its momentum p
                                and the gradient g.  Plain (not learned-map) runs; NULL = not wanted */
} gnuts_output;

/* timing[] fields: device-side measurements of one run */
#define GNUTS_TIMING_ROUNDS 0        /* gradient rounds (round mode) or fused launches */
#define GNUTS_TIMING_GRAD_US 1       /* mean duration of the batched gradient kernel, us (CUDA events) */
#define GNUTS_TIMING_ADVANCE_US 2    /* mean duration of the state-machine kernel, us (CUDA events) */
#define GNUTS_TIMING_DEVICE_MS 3     /* device time from first to last launch, ms */
#define GNUTS_TIMING_LAUNCHES 4      /* kernels launched by the run */
#define GNUTS_TIMING_REDUCE_US 5     /* 0: the row-split sums run inside the state-machine kernel */
#define GNUTS_TIMING_CHAINS_PER_CTA 6  /* launch shape the fused-mode autotuner picked (chains per CTA) */
#define GNUTS_TIMING_FIELDS 8

/* Progress callback, called from the calling thread between device launches
 * (mirrors the `Iteration: k / n [pct%]` logger lines). May be NULL. */
typedef void (*gnuts_progress_fn)(void* ctx, int chain, int iteration, int total, int warmup);

/* stan::callbacks::interrupt (created at command.hpp:186 and passed to every
 * service at :609-688): a callback the service polls between device
 * launches (every few milliseconds of sampling); a nonzero return stops the
 * run, which then returns GNUTS_ERR_INTERRUPTED (rows already handed to a
 * draw sink stay delivered; the gnuts_output arrays are not filled).
 * Thread-local: it applies to the service calls of the calling thread made
 * after it is set; NULL removes it. */
typedef int (*gnuts_interrupt_fn)(void* ctx);
void gnuts_set_interrupt(gnuts_interrupt_fn fn, void* ctx);

/* Streaming draw output, the role of the sample_writers CmdStan hands the
 * services (command.hpp:191-192, written per iteration): while a run of
 * this thread proceeds, rows first_row .. first_row + n_rows - 1 of every
 * chain are passed as soon as all chains have written them, as one
 * [num_chains][n_rows][7 + num_constrained] block (same columns as
 * gnuts_output.draws; the pointer is valid during the call).  With a sink
 * set, gnuts_output.draws may be NULL, so the caller never holds all draws at
 * once.  Blocks hold at most 64 MB; the last rows come when the run ends.
 * Thread-local like gnuts_set_interrupt; NULL removes it.  Learned-map runs
 * deliver their rows at the end of the run. */
typedef void (*gnuts_draws_fn)(void* ctx, int first_row, int n_rows, const double* rows);
void gnuts_set_draw_sink(gnuts_draws_fn fn, void* ctx);

/* stan::services::sample::hmc_nuts_diag_e_adapt (command.hpp:673-688):
 * inits NULL -> random inits; inv_metric NULL -> unit diagonal start
 * (metric_file given -> command.hpp:673-680). */
int gnuts_hmc_nuts_diag_e_adapt(gnuts_model* m, const gnuts_sample_args* a, const double* inits,
                                const double* inv_metric, gnuts_output* out,
                                gnuts_progress_fn progress, void* ctx);
/* stan::services::sample::hmc_nuts_dense_e_adapt (command.hpp:657-672) */
int gnuts_hmc_nuts_dense_e_adapt(gnuts_model* m, const gnuts_sample_args* a, const double* inits,
                                 const double* inv_metric, gnuts_output* out,
                                 gnuts_progress_fn progress, void* ctx);
/* stan::services::sample::hmc_nuts_unit_e_adapt (command.hpp:689-697 branch) */
int gnuts_hmc_nuts_unit_e_adapt(gnuts_model* m, const gnuts_sample_args* a, const double* inits,
                                gnuts_output* out, gnuts_progress_fn progress, void* ctx);
/* Non-adapting services hmc_nuts_{diag,dense,unit}_e (command.hpp:609-632) */
int gnuts_hmc_nuts_diag_e(gnuts_model* m, const gnuts_sample_args* a, const double* inits,
                          const double* inv_metric, gnuts_output* out, gnuts_progress_fn progress,
                          void* ctx);
int gnuts_hmc_nuts_dense_e(gnuts_model* m, const gnuts_sample_args* a, const double* inits,
                           const double* inv_metric, gnuts_output* out, gnuts_progress_fn progress,
                           void* ctx);
int gnuts_hmc_nuts_unit_e(gnuts_model* m, const gnuts_sample_args* a, const double* inits,
                          gnuts_output* out, gnuts_progress_fn progress, void* ctx);

/* One NUTS transition per point with the momentum supplied (replay of
 * base_nuts::transition with injected draws; no reference counterpart as an
 * API, it exposes the transition that hmc_nuts_* run internally).
 * metric: 0 diag, 1 dense, 2 unit.  inv_metric: D or D*D (shared by all points).
 * counters[n]: stream-0 Philox draw counters, advanced on return.
 * stats[n][7]: lp__, accept_stat__, stepsize__, treedepth__, n_leapfrog__, divergent__, energy__. */
int gnuts_transition(gnuts_model* m, int metric, const double* inv_metric, int n, const double* q0,
                     const double* p0, double stepsize, int max_depth, unsigned int seed,
                     const unsigned int* chain_ids, uint64_t* counters, double* q_out, double* stats);

/* stansummary statistics of one quantity (stansummary_helper.hpp:397-428,
 * chainset mean / mcse_mean / sd / med_abs_deviation / quantiles /
 * split_rank_normalized_ess / split_rank_normalized_rhat).
 * x[c * stride_chain + i * stride_iter] is draw i of chain c.
 * out: mean, mcse, sd, mad, quantiles[n_probs], ess_bulk, ess_tail, rhat. */
int gnuts_summary(const double* x, int n_chains, int n_iter, int64_t stride_chain, int64_t stride_iter,
                  const double* probs, int n_probs, double* out);
/* The same for n_cols quantities at once (threads over columns); out is
 * n_cols x (7 + n_probs). */
int gnuts_summary_columns(const double* draws, int n_chains, int n_iter, int n_cols, int64_t stride_chain,
                          int64_t stride_iter, const int* cols, const double* probs, int n_probs,
                          int n_threads, double* out);

/* The same statistics as gnuts_summary_columns (stansummary_helper.hpp:397-428),
 * computed on the GPU, one CTA per quantity: the pooled draws are radix
 * sorted on the device (draws, then their distances to the median) and every
 * autocovariance is a CTA-wide reduction.  Results equal the host version's
 * up to floating-point summation order.  n_iter >= 4 and n_chains * n_iter
 * < 2^31.  Returns GNUTS_ERR_CUDA without a device. */
int gnuts_summary_columns_gpu(const double* draws, int n_chains, int n_iter, int n_cols, int64_t stride_chain,
                              int64_t stride_iter, const int* cols, const double* probs, int n_probs,
                              double* out);

/* Diagnostic checks of a run (CmdStan's bin/diagnose, src/cmdstan/diagnose.cpp:84-221):
 * transitions at the maximum tree depth, divergences, E-BFMI < 0.3 (energy__
 * over all chains' draws taken chain after chain), parameters with
 * min(bulk, tail) ESS per draw < 0.001 and with max(bulk, tail) R-hat >
 * 1.01499 (diagnose.cpp:12).  draws[c * stride_chain + i * stride_iter + col];
 * a column index < 0 skips that check; param_names is '\n'-separated, in
 * Stan CSV form ("mu.1" is reported as "mu[1]", as the CSV reader does).  The
 * ESS / R-hat statistics run on host threads (use_gpu = 0) or on the GPU.
 * report receives the reference's report text (NUL-terminated; an argument
 * error if report_cap is too small). */
typedef struct {
  long n_treedepth_max;  /* transitions with treedepth__ >= max_depth */
  long n_divergent;
  double e_bfmi;         /* NaN without an energy column */
  int n_low_ess;         /* parameters below 0.001 effective draws per transition */
  int n_high_rhat;       /* parameters with R-hat above 1.01499 */
  int has_problems;
} gnuts_diagnosis;
int gnuts_diagnose(const double* draws, int n_chains, int n_iter, int64_t stride_chain, int64_t stride_iter,
                   int treedepth_col, int divergent_col, int energy_col, const int* param_cols, int n_params,
                   const char* param_names, int max_depth, int use_gpu, int n_threads, char* report,
                   size_t report_cap, gnuts_diagnosis* result);

/* Allocation-free gradient for callers that cannot allocate device memory.
 * No counterpart in the reference: CmdStan computes gradients on the host.
 * It exists for callers that run where cudaMalloc is not allowed -- code
 * inside a memory pool or arena that owns all device memory, a host callback
 * of another library, an allocator-free real-time loop -- but that can pass
 * device buffers they already own.  Same contract as gnuts_log_prob_grad
 * (lp and gradient, FP64), for the batched models "logistic" and "horseshoe",
 * with q, lp and grad given as DEVICE pointers (n x num_params_r, n, n x
 * num_params_r).  Its scratch (coefficients, row-split partial sums) lives in
 * a fixed static device array of GNUTS_NOALLOC_SCRATCH_BYTES that every GPU
 * loading the library holds until the process exits; it calls no cudaMalloc,
 * cudaFree or allocating library routine.  Limits: n <= GNUTS_NOALLOC_MAX_POINTS
 * and num_params_r of the coefficient row (predictors + 1) <= GNUTS_NOALLOC_MAX_COEF;
 * larger requests fail with GNUTS_ERR_ARGUMENT.  The model's data must
 * already be on the current device (any earlier device call on the handle,
 * e.g. gnuts_log_prob_grad, uploads it).  The first call on each device looks
 * up the scratch array's device address; make that first call before any
 * stream capture.  All calls share the one scratch array and work on the
 * legacy default stream, returning after the result is written: calls that
 * overlap on the GPU (from several host threads) race. */
#define GNUTS_NOALLOC_MAX_POINTS 64
#define GNUTS_NOALLOC_MAX_COEF 128
#define GNUTS_NOALLOC_MAX_SPLITS 32
#define GNUTS_NOALLOC_SCRATCH_BYTES \
  (8 * (GNUTS_NOALLOC_MAX_SPLITS * GNUTS_NOALLOC_MAX_POINTS * (GNUTS_NOALLOC_MAX_COEF + 1) + \
        GNUTS_NOALLOC_MAX_POINTS * GNUTS_NOALLOC_MAX_COEF))
int gnuts_log_prob_grad_noalloc(const gnuts_model* m, int n, const double* q_device, int jacobian,
                                double* lp_device, double* grad_device);


/* ---- learned preconditioner: affine-coupling flow ----
 * No counterpart in the reference: CmdStan's NUTS samples the model's own
 * unconstrained space.  A flow T maps z to x (RealNVP coupling layers with a
 * tanh hidden layer and a soft-clamped log-scale, then x = mu + exp(rho) .* u);
 * NUTS then samples z with target lp_x(T(z)) + log|det dT/dz|.  Parameters are
 * one vector theta: per layer W1 [n_b][H], b1 [H], W2 [H][2 n_a], b2 [2 n_a];
 * then mu [d], rho [d].  Layer l keeps the indices i whose bit (l mod B) equals
 * (l div B) mod 2 (B = ceil(log2 d)) and transforms the others. */
typedef struct gnuts_flow gnuts_flow;
/* dim 2..128, layers 1..16, hidden 32 / 64 / 128, clamp > 0 (log-scale bound) */
int gnuts_flow_create(int dim, int layers, int hidden, double clamp, gnuts_flow** out);
void gnuts_flow_destroy(gnuts_flow* f);
long gnuts_flow_num_params(const gnuts_flow* f);
int gnuts_flow_set_params(gnuts_flow* f, const double* theta);
int gnuts_flow_get_params(const gnuts_flow* f, double* theta);
/* identity coupling layers (W2 = b2 = 0, b1 = 0, W1 ~ N(0, w1_scale^2 / n_b)
 * from seed) around the affine map x = mean + scale .* z */
int gnuts_flow_init_affine(gnuts_flow* f, const double* mean, const double* scale, unsigned int seed,
                           double w1_scale);
/* x = T(z) and log|det| for n points (n x dim) */
int gnuts_flow_forward(gnuts_flow* f, int n, const double* z, double* x, double* logdet);
/* z = T^-1(x); logdet receives log|det dT/dz| at that z (may be NULL) */
int gnuts_flow_inverse(gnuts_flow* f, int n, const double* x, double* z, double* logdet);
/* pulled-back log density lp = lp_x(T(z)) + log|det| (model log_prob_grad
 * contract, command_helper.hpp:589-593, evaluated at x), its gradient in z
 * (n x dim) and, when grad_theta is not NULL, the sum over the n points of its
 * gradient in theta (num_params) */
int gnuts_flow_log_prob_grad(gnuts_model* m, gnuts_flow* f, int n, const double* z, int jacobian, double* lp,
                             double* grad_z, double* grad_theta);
/* the sampler's gradient pass at n points: lp = lp_x(T(z)) + log|det|
 * (jacobian on) and its gradient in z, from the tensor-core evaluation the
 * learned sampler uses (BF16 weights, activations carried as three BF16
 * parts, FP32 accumulation; the model at x in FP64) */
int gnuts_flow_log_prob_grad_tc(gnuts_model* m, gnuts_flow* f, int n, const double* z, double* lp,
                                double* grad_z);
/* one Adam step (bias-corrected, step t >= 1) with the given gradient */
int gnuts_flow_adam_step(gnuts_flow* f, const double* grad, int t, double lr, double beta1, double beta2,
                         double eps);
/* Reverse-KL training.  Each step draws `batch` base points
 * z ~ N(0, base_scale^2 I) (Philox stream 2 of (seed, point)) and takes one
 * Adam step (0.9, 0.999, 1e-8; learning rate decaying linearly from
 * learning_rate to a tenth of it) on the mean of
 * -(beta * lp_x(T(z)) + log|det|).  beta rises linearly from beta0 to 1 over
 * the first anneal_fraction of the steps (a tempered, wider target first, so
 * the map does not collapse onto one region), then stays 1.  At beta = 1 the
 * minimiser pulls the posterior back to N(0, base_scale^2 I): base_scale 1 is
 * the reverse KL; larger values weight the tails more. */
typedef struct {
  int steps, batch;         /* default 2000, 256 */
  double learning_rate;     /* default 2e-3 */
  double base_scale;        /* default 1.25 */
  double beta0;             /* default 1 */
  double anneal_fraction;   /* default 0 (no annealing) */
  unsigned int seed;
} gnuts_train_args;
void gnuts_train_args_default(gnuts_train_args* ta);
/* loss_trace (steps, may be NULL) receives each step's mean loss */
int gnuts_flow_train(gnuts_model* m, gnuts_flow* f, const gnuts_train_args* ta, double* loss_trace);

/* hmc_nuts_diag_e_adapt (command.hpp:673-688) run on z with x = T(z): inits
 * and the returned step size / inverse metric are in z; draws hold lp__ =
 * the model's lp at x and write_array(x), like a plain run's */
int gnuts_hmc_nuts_flow_diag_e_adapt(gnuts_model* m, gnuts_flow* f, const gnuts_sample_args* a,
                                     const double* inits_z, const double* inv_metric, gnuts_output* out,
                                     gnuts_progress_fn progress, void* ctx);

typedef struct {
  int layers, hidden;       /* default 8, 128 */
  double clamp;             /* default 6 */
  gnuts_train_args train;   /* gnuts_train_args_default; the seed is derived from the sampler's */
  int flow_warmup;          /* z-space warmup iterations, default 300 */
  double flow_delta;        /* adaptation target of the z-space sampler, default 0.95 */
  int pilot_samples;        /* draws per chain each sampler produces for the judge, default 200 */
  double moment_tolerance;  /* combined MCSE, default 4 */
  double rhat_max;          /* convergence bound on the pilots' max split R-hat, default 1.01 */
} gnuts_learned_args;
void gnuts_learned_args_default(gnuts_learned_args* la);

typedef struct {
  int used_flow;                    /* 1: the learned map produced the draws; 0: plain fallback */
  double plain_ess_per_grad, flow_ess_per_grad;  /* min bulk ESS / sampling gradients, pilots */
  double plain_divergence_rate, flow_divergence_rate;
  double max_moment_z;              /* max over parameters |mean_f - mean_p| / sqrt(mcse_f^2 + mcse_p^2) */
  double loss_first, loss_last;     /* mean training loss of the first / last 10 steps */
  double plain_seconds, train_seconds, flow_seconds, final_seconds;
  int64_t plain_grads, flow_grads, final_grads;
  double plain_max_rhat, flow_max_rhat;  /* max over parameters of the pilots' split R-hat */
} gnuts_learned_report;

/* Learned-preconditioner variant of hmc_nuts_diag_e_adapt (command.hpp:
 * 673-688): (1) plain diag_e NUTS, num_warmup adaptive iterations and
 * pilot_samples draws; (2) flow initialised from those chains (median and
 * MAD-based scale of their final positions, pooled across chains) and trained by
 * reverse KL through the model's own gradient kernels; (3) NUTS on z with
 * flow_warmup adaptive iterations and pilot_samples draws; (4) the judge
 * keeps the flow only if its ESS per gradient is not lower, its divergence
 * rate not higher, its max R-hat not above max(rhat_max, the plain pilot's)
 * and (when the plain pilot is free of divergences) every posterior mean
 * agrees within moment_tolerance combined MCSE; (5) the kept
 * sampler continues, non-adapting, for num_samples draws into out. */
int gnuts_hmc_nuts_learned_diag_e_adapt(gnuts_model* m, const gnuts_sample_args* a, const gnuts_learned_args* la,
                                        const double* inits, gnuts_output* out, gnuts_learned_report* report,
                                        gnuts_progress_fn progress, void* ctx);

/* Message of the last failing call on this thread. */
int gnuts_last_error(char* buf, size_t len);
/* Library version string, e.g. "gnuts 0.1 (sm_103a)". */
const char* gnuts_version(void);

#ifdef __cplusplus
}
#endif
#endif
