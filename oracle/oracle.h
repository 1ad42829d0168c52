/*
 * CPU FP64 oracle for the NUTS sampling path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library is the checker, never the product: only tests/, the smoke
 * check and bench.py's CPU-baseline leg load it.  It restates, in plain
 * C++ written for this project, the algorithms that CmdStan reaches through
 * its service calls (src/cmdstan/command.hpp:657-688):
 *
 *   - stan::mcmc base_nuts transition / build_tree (multinomial sampling,
 *     generalized no-U-turn criterion with the two extra checks across
 *     merged subtrees, divergence at Delta-H > 1000), written RECURSIVELY
 *     like the published algorithm so that the device's iterative state
 *     machine is checked against an independent formulation;
 *   - expl_leapfrog and the diag_e / dense_e / unit_e Euclidean metrics;
 *   - dual-averaging step-size adaptation and windowed Welford variance /
 *     covariance adaptation with the defaults of
 *     src/cmdstan/arguments/arg_adapt.hpp:19-37;
 *   - stan::services::util::initialize (random inits on (-R, R), up to 100
 *     attempts) and run_adaptive_sampler / run_sampler;
 *   - chainset split rank-normalized ESS and R-hat plus mean / MCSE / SD /
 *     MAD / quantiles as used by src/cmdstan/stansummary_helper.hpp:397-428.
 *
 * Parity pins: the summary statistics are pinned to the exact goldens of
 * src/test/interface/stansummary_test.cpp:481-495 and :622-637 (fixture
 * draws extracted by tests/golden/make_golden.py).  The NUTS transition and
 * the adaptation cannot be pinned to the reference (its stan submodule is
 * empty): they follow the public algorithm descriptions and are checked by
 * analytic posteriors, finite differences and moment tests ("parity
 * unpinned" for trajectories).
 *
 * The random numbers come from Philox-4x32-10 keyed by (seed, chain id);
 * the draw schedule is defined in philox.h and is shared by contract (not by
 * code) with the device sampler.
 */
#ifndef GNUTS_ORACLE_H
#define GNUTS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Philox ---- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* uniform [0,1) / normal pair draws at an explicit stream position */
double orc_uniform(uint32_t seed, uint32_t chain, uint32_t stream, uint64_t counter);
void orc_normal_pair(uint32_t seed, uint32_t chain, uint32_t stream, uint64_t counter, double out[2]);

/* ---- models ---- */
typedef struct orc_model orc_model;
orc_model* orc_bernoulli(int N, const int* y);
orc_model* orc_normal(int K, const double* scales);
orc_model* orc_logistic(int N, int D, const double* X, const int* y);
orc_model* orc_hier(int J, const double* y, const double* sigma);
orc_model* orc_funnel(int K);
orc_model* orc_varint(int N, int J, int K, const int* group, const double* X, const double* y);
orc_model* orc_horseshoe(int N, int D, const double* X, const int* y, double scale_global,
                         double slab_scale, double slab_df);
void orc_model_free(orc_model* m);
int orc_model_dim(const orc_model* m);
int orc_model_num_constrained(const orc_model* m);
/* lp (propto, with or without the Jacobian) and its gradient on the unconstrained scale */
double orc_log_prob_grad(const orc_model* m, const double* q, int jacobian, double* grad);
void orc_write_array(const orc_model* m, const double* q, double* out);
int orc_unconstrain(const orc_model* m, const double* constrained, double* q);

/* ---- sampler ---- */
typedef struct {
  int num_warmup, num_samples, thin, save_warmup;
  double stepsize, stepsize_jitter;
  int max_depth;
  int adapt_engaged;
  double delta, gamma, kappa, t0;
  unsigned init_buffer, term_buffer, window;
  int metric;           /* 0 diag_e, 1 dense_e, 2 unit_e */
  uint32_t seed;
  double init_radius;
} orc_args;

/* Columns of a draw row: lp__, accept_stat__, stepsize__, treedepth__,
 * n_leapfrog__, divergent__, energy__, then the D unconstrained values. */
#define ORC_NSAMPLER_COLS 7

/* One chain.  init_q (D) may be NULL for random inits.  inv_metric may be
 * NULL (unit) or D / D*D values.  draws must hold n_saved*(7+D) doubles.
 * adapted_metric holds D (diag/unit) or D*D (dense).  Returns 0 on success,
 * non-zero (and a message) on failure. */
int orc_run_chain(const orc_model* m, const orc_args* a, uint32_t chain_id, const double* init_q,
                  const double* inv_metric, double* draws, double* adapted_stepsize,
                  double* adapted_metric, long long* n_grad, char* errbuf, int errlen);

/* Independent chains on n_threads host threads (the timed CPU baseline). */
int orc_run_chains(const orc_model* m, const orc_args* a, int n_chains, uint32_t first_chain_id,
                   int n_threads, const double* init_q, const double* inv_metric, double* draws,
                   double* adapted_stepsize, double* adapted_metric, long long* n_grad);

/* One NUTS transition with explicit momentum (replay test).  q0/p0 are D
 * vectors; the uniforms come from stream 0 of (seed, chain) starting at
 * *counter, which is advanced.  out_q receives the selected point. */
int orc_transition(const orc_model* m, int metric, const double* inv_metric, const double* q0,
                   const double* p0, double eps, int max_depth, uint32_t seed, uint32_t chain,
                   uint64_t* counter, double* out_q, double* out_stats /* 7 sampler cols */);

/* ---- summary statistics (chainset restatement) ----
 * x is [n_chains][n_draws] row-major. */
double orc_ess_bulk(const double* x, int n_chains, int n_draws);
double orc_ess_tail(const double* x, int n_chains, int n_draws);
double orc_ess_basic(const double* x, int n_chains, int n_draws);
double orc_rhat(const double* x, int n_chains, int n_draws);
/* out: mean, mcse, sd, mad, q[0..n_probs-1], ess_bulk, ess_tail, rhat */
void orc_summary(const double* x, int n_chains, int n_draws, const double* probs, int n_probs,
                 double* out);


/* ---- affine-coupling flow (flow.cpp; no counterpart in the reference) ----
 * theta layout and the map are defined at the top of flow.cpp. */
long orc_flow_num_params(int d, int L, int H);
void orc_flow_mask(int d, int L, int H, int l, int* out);
double orc_flow_forward(int d, int L, int H, double clamp, const double* theta, const double* z, double* x);
double orc_flow_inverse(int d, int L, int H, double clamp, const double* theta, const double* x, double* z);
double orc_flow_log_prob_grad(const orc_model* m, int L, int H, double clamp, const double* theta,
                              const double* z, int jacobian, double* grad_z, double* thbar, double* x_out,
                              double* lp_x_out);
void orc_adam(long n, double* theta, double* m, double* v, const double* g, int t, double lr, double b1,
              double b2, double eps);

#ifdef __cplusplus
}
#endif
#endif
