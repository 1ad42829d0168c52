// C-ABI of the learned preconditioner (include/gnuts.h, "learned
// preconditioner" section): flow handles, reverse-KL training, NUTS on z,
// and the learned variant of hmc_nuts_diag_e_adapt with plain NUTS as
// fallback and judge.
//
// No counterpart in the reference: CmdStan's sample method
// (src/cmdstan/command.hpp:673-688) runs plain NUTS on the model's
// unconstrained space.  The learned service keeps that service's arguments
// and output contract (draws of lp__, sampler columns and write_array values)
// so a caller can switch between the two.
#include <algorithm>
#include <chrono>
#include <memory>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "internal.h"

namespace gnuts {
namespace {

Flow* F(gnuts_flow* f) { return reinterpret_cast<Flow*>(f); }
const Flow* F(const gnuts_flow* f) { return reinterpret_cast<const Flow*>(f); }
Model* Mo(gnuts_model* m) { return reinterpret_cast<Model*>(m); }

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// per-sampler judge statistics over the constrained columns of pilot draws
struct PilotStats {
  double min_ess = 0, grads = 0, div_rate = 0, max_rhat = 0;
  std::vector<double> mean, mcse;
};

PilotStats pilot_stats(const std::vector<double>& draws, int C, int n, int ncol) {
  PilotStats ps;
  const int ncon = ncol - 7;
  std::vector<int> cols(ncon);
  for (int k = 0; k < ncon; ++k) cols[k] = 7 + k;
  std::vector<double> out((size_t)ncon * 7);
  gnuts_summary_columns(draws.data(), C, n, ncon, (int64_t)n * ncol, ncol, cols.data(), nullptr, 0, 0, out.data());
  ps.min_ess = INFINITY;
  for (int k = 0; k < ncon; ++k) {
    const double* o = &out[(size_t)k * 7];
    ps.mean.push_back(o[0]);
    ps.mcse.push_back(o[1]);
    const double ess = std::isfinite(o[4]) ? o[4] : 0.0;
    ps.min_ess = std::min(ps.min_ess, ess);
    ps.max_rhat = std::max(ps.max_rhat, std::isfinite(o[6]) ? o[6] : INFINITY);
  }
  double div = 0;
  for (int c = 0; c < C; ++c)
    for (int i = 0; i < n; ++i) {
      const double* row = &draws[((size_t)c * n + i) * ncol];
      ps.grads += row[4];
      div += row[5];
    }
  ps.div_rate = div / std::max(1, C * n);
  return ps;
}

struct RunBufs {
  std::vector<double> draws, eps, minv, tw, ts, timing;
  std::vector<int64_t> ng, nlf;
  std::vector<int> status;
  gnuts_output out{};
  RunBufs(int C, int n_saved, int ncol, int D) {
    draws.assign((size_t)C * n_saved * ncol, 0.0);
    eps.assign(C, 0.0);
    minv.assign((size_t)C * D, 0.0);
    tw.assign(C, 0.0);
    ts.assign(C, 0.0);
    timing.assign(GNUTS_TIMING_FIELDS, 0.0);
    ng.assign(C, 0);
    nlf.assign(C, 0);
    status.assign(C, 0);
    out.draws = draws.data();
    out.stepsize = eps.data();
    out.inv_metric = minv.data();
    out.warmup_seconds = tw.data();
    out.sampling_seconds = ts.data();
    out.n_grad = ng.data();
    out.chain_status = status.data();
    out.n_leapfrog = nlf.data();
    out.timing = timing.data();
  }
};

}  // namespace
}  // namespace gnuts

using namespace gnuts;

extern "C" {

int gnuts_flow_create(int dim, int layers, int hidden, double clamp, gnuts_flow** out) {
  if (!out) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  std::string err;
  Flow* f = nullptr;
  int rc = flow_create(dim, layers, hidden, clamp, &f, err);
  if (rc) return api_fail(rc, err);
  *out = reinterpret_cast<gnuts_flow*>(f);
  return GNUTS_OK;
}

void gnuts_flow_destroy(gnuts_flow* f) { delete F(f); }

long gnuts_flow_num_params(const gnuts_flow* f) { return f ? F(f)->n_params : 0; }

int gnuts_flow_set_params(gnuts_flow* f, const double* theta) {
  if (!f || !theta) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  for (long i = 0; i < F(f)->n_params; ++i)
    if (!std::isfinite(theta[i])) return api_fail(GNUTS_ERR_ARGUMENT, "flow parameters must be finite");
  std::string err;
  int rc = flow_set_params(*F(f), theta, err);
  return rc ? api_fail(rc, err) : GNUTS_OK;
}

int gnuts_flow_get_params(const gnuts_flow* f, double* theta) {
  if (!f || !theta) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  std::string err;
  int rc = flow_get_params(*F(f), theta, err);
  return rc ? api_fail(rc, err) : GNUTS_OK;
}

int gnuts_flow_init_affine(gnuts_flow* fh, const double* mean, const double* scale, unsigned int seed,
                           double w1_scale) {
  if (!fh || !mean || !scale) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  const Flow& f = *F(fh);
  std::vector<double> th(f.n_params, 0.0);
  std::mt19937_64 rng(seed);
  std::normal_distribution<double> nd(0.0, 1.0);
  for (int l = 0; l < f.L; ++l) {
    const long nb = f.nb[l];
    const double sd = w1_scale / std::sqrt((double)std::max<long>(1, nb));
    for (long i = 0; i < nb * f.H; ++i) th[f.th_off[l] + i] = sd * nd(rng);
  }
  for (int i = 0; i < f.d; ++i) {
    if (!(scale[i] > 0) || !std::isfinite(scale[i]) || !std::isfinite(mean[i]))
      return api_fail(GNUTS_ERR_ARGUMENT, "flow affine start needs finite means and positive scales");
    th[f.th_off[f.L] + i] = mean[i];
    th[f.th_rho + i] = std::log(scale[i]);
  }
  std::string err;
  int rc = flow_set_params(*F(fh), th.data(), err);
  return rc ? api_fail(rc, err) : GNUTS_OK;
}

int gnuts_flow_forward(gnuts_flow* f, int n, const double* z, double* x, double* logdet) {
  if (!f || (n > 0 && (!z || !x || !logdet))) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  std::string err;
  int rc = flow_forward(*F(f), n, z, x, logdet, err);
  return rc ? api_fail(rc, err) : GNUTS_OK;
}

int gnuts_flow_inverse(gnuts_flow* f, int n, const double* x, double* z, double* logdet) {
  if (!f || (n > 0 && (!x || !z))) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  std::string err;
  int rc = flow_inverse(*F(f), n, x, z, logdet, err);
  return rc ? api_fail(rc, err) : GNUTS_OK;
}

int gnuts_flow_log_prob_grad(gnuts_model* m, gnuts_flow* f, int n, const double* z, int jacobian, double* lp,
                             double* grad_z, double* grad_theta) {
  if (!m || !f || (n > 0 && (!z || !lp || !grad_z))) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  std::string err;
  int rc = flow_log_prob_grad(*Mo(m), *F(f), n, z, jacobian, lp, grad_z, grad_theta, err);
  return rc ? api_fail(rc, err) : GNUTS_OK;
}

int gnuts_flow_log_prob_grad_tc(gnuts_model* m, gnuts_flow* f, int n, const double* z, double* lp,
                                double* grad_z) {
  if (!m || !f || (n > 0 && (!z || !lp || !grad_z))) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  std::string err;
  int rc = flow_log_prob_grad_tc(*Mo(m), *F(f), n, z, lp, grad_z, err);
  return rc ? api_fail(rc, err) : GNUTS_OK;
}

int gnuts_flow_adam_step(gnuts_flow* f, const double* grad, int t, double lr, double beta1, double beta2,
                         double eps) {
  if (!f || !grad) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  if (t < 1 || !(lr > 0) || !(beta1 >= 0 && beta1 < 1) || !(beta2 >= 0 && beta2 < 1) || !(eps > 0))
    return api_fail(GNUTS_ERR_ARGUMENT, "invalid Adam hyper-parameters");
  std::string err;
  int rc = flow_adam_step(*F(f), grad, t, lr, beta1, beta2, eps, err);
  return rc ? api_fail(rc, err) : GNUTS_OK;
}

void gnuts_train_args_default(gnuts_train_args* ta) {
  if (!ta) return;
  ta->steps = 2000;
  ta->batch = 256;
  ta->learning_rate = 2e-3;
  ta->base_scale = 1.25;
  ta->beta0 = 1.0;
  ta->anneal_fraction = 0.0;
  ta->seed = 0;
}

static int check_train_args(const gnuts_train_args& t) {
  if (t.steps < 0 || t.batch < 1 || t.batch > 65536 || !(t.learning_rate > 0) || !(t.base_scale > 0) ||
      !(t.beta0 > 0 && t.beta0 <= 1) || !(t.anneal_fraction >= 0 && t.anneal_fraction <= 1))
    return api_fail(GNUTS_ERR_ARGUMENT, "training needs steps >= 0, 1 <= batch <= 65536, learning_rate > 0, "
                                        "base_scale > 0, 0 < beta0 <= 1, 0 <= anneal_fraction <= 1");
  return GNUTS_OK;
}

int gnuts_flow_train(gnuts_model* m, gnuts_flow* f, const gnuts_train_args* ta, double* loss_trace) {
  if (!m || !f || !ta) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  int rc = check_train_args(*ta);
  if (rc) return rc;
  std::string err;
  rc = flow_train(*Mo(m), *F(f), *ta, loss_trace, err);
  return rc ? api_fail(rc, err) : GNUTS_OK;
}

int gnuts_hmc_nuts_flow_diag_e_adapt(gnuts_model* m, gnuts_flow* f, const gnuts_sample_args* a,
                                     const double* inits_z, const double* inv_metric, gnuts_output* out,
                                     gnuts_progress_fn progress, void* ctx) {
  if (!m || !f) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  Model& mm = *Mo(m);
  int rc = validate_args(mm, a, 1, 0);
  if (rc) return rc;
  if (F(f)->d != mm.dev.D) return api_fail(GNUTS_ERR_ARGUMENT, "flow dimension does not match the model's");
  if (F(f)->device < 0) return api_fail(GNUTS_ERR_ARGUMENT, "flow parameters not set");
  RunConfig cfg{0, 1};
  cfg.flow = F(f);
  std::string err;
  rc = run_nuts(mm, *a, cfg, inits_z, inv_metric, out, progress, ctx, err);
  return rc ? api_fail(rc, err) : GNUTS_OK;
}

void gnuts_learned_args_default(gnuts_learned_args* la) {
  if (!la) return;
  la->layers = 8;
  la->hidden = 128;
  la->clamp = 6.0;
  gnuts_train_args_default(&la->train);
  la->flow_warmup = 300;
  la->flow_delta = 0.95;
  la->pilot_samples = 200;
  la->moment_tolerance = 4.0;
  la->rhat_max = 1.01;
}

int gnuts_hmc_nuts_learned_diag_e_adapt(gnuts_model* mh, const gnuts_sample_args* a, const gnuts_learned_args* la,
                                        const double* inits, gnuts_output* out, gnuts_learned_report* report,
                                        gnuts_progress_fn progress, void* ctx) {
  if (!mh || !a || !la) return api_fail(GNUTS_ERR_ARGUMENT, "null argument");
  Model& m = *Mo(mh);
  int rc = validate_args(m, a, 1, 0);
  if (rc) return rc;
  if (la->pilot_samples < 20 || la->flow_warmup < 20 || !(la->flow_delta > 0 && la->flow_delta < 1))
    return api_fail(GNUTS_ERR_ARGUMENT,
                    "learned sampler needs pilot_samples >= 20, flow_warmup >= 20 and 0 < flow_delta < 1");
  if ((rc = check_train_args(la->train))) return rc;
  const int C = a->num_chains, D = m.dev.D, ncol = 7 + m.dev.ncon, P = la->pilot_samples;
  if (D < 2) return api_fail(GNUTS_ERR_ARGUMENT, "the learned map needs at least 2 parameters");
  std::string err;
  gnuts_learned_report rep{};
  Flow* fl = nullptr;
  rc = flow_create(D, la->layers, la->hidden, la->clamp, &fl, err);
  if (rc) return api_fail(rc, err);
  std::unique_ptr<Flow> flow_owner(fl);

  NvtxRange range("gnuts.learned");
  // (1) plain diag_e NUTS: adaptive warmup and a pilot
  double t0 = now_s();
  gnuts_sample_args ap = *a;
  ap.num_samples = P;
  ap.save_warmup = 0;
  ap.thin = 1;
  RunBufs rp(C, P, ncol, D);
  std::vector<double> q_plain((size_t)C * D);
  {
    RunConfig cfg{0, 1};
    cfg.q_last = q_plain.data();
    rc = run_nuts(m, ap, cfg, inits, nullptr, &rp.out, progress, ctx, err);
    if (rc) return api_fail(rc, err);
  }
  rep.plain_seconds = now_s() - t0;
  for (int c = 0; c < C; ++c) rep.plain_grads += rp.nlf[c];

  // (2) flow start from the plain chains, then reverse-KL training.  The
  // affine part starts at the median and the MAD-based scale of the chains'
  // final positions, pooled across chains: chains that each cover only part
  // of the posterior (a funnel's chains stuck at different v) still spread
  // across it together, and the median / MAD ignore the few far-out ones.
  t0 = now_s();
  std::vector<double> mean(D, 0.0), scale(D, 0.0);
  {
    std::vector<double> col(C);
    for (int i = 0; i < D; ++i) {
      for (int c = 0; c < C; ++c) col[c] = q_plain[(size_t)c * D + i];
      std::sort(col.begin(), col.end());
      const double med = C % 2 ? col[C / 2] : 0.5 * (col[C / 2 - 1] + col[C / 2]);
      for (int c = 0; c < C; ++c) col[c] = std::fabs(col[c] - med);
      std::sort(col.begin(), col.end());
      const double mad = C % 2 ? col[C / 2] : 0.5 * (col[C / 2 - 1] + col[C / 2]);
      double ms = 0;  // fallback: the adapted metric (within-chain scale)
      for (int c = 0; c < C; ++c) ms += rp.minv[(size_t)c * D + i] / C;
      mean[i] = med;
      scale[i] = mad > 0 ? 1.4826 * mad : std::sqrt(std::max(ms, 1e-12));
    }
  }
  rc = gnuts_flow_init_affine(reinterpret_cast<gnuts_flow*>(fl), mean.data(), scale.data(), a->seed + 1u, 0.5);
  if (rc) return rc;
  const int steps = la->train.steps;
  std::vector<double> trace(std::max(1, steps));
  gnuts_train_args ta = la->train;
  ta.seed = a->seed + 1u;
  rc = flow_train(m, *fl, ta,
                  trace.data(), err);
  if (rc) return api_fail(rc, err);
  rep.train_seconds = now_s() - t0;
  if (steps > 0) {
    const int k = std::min(10, steps);
    for (int i = 0; i < k; ++i) {
      rep.loss_first += trace[i] / k;
      rep.loss_last += trace[steps - 1 - i] / k;
    }
  }

  // (3) NUTS on z: warmup and a pilot, started from the plain chains' positions
  t0 = now_s();
  std::vector<double> z0((size_t)C * D);
  rc = flow_inverse(*fl, C, q_plain.data(), z0.data(), nullptr, err);
  if (rc) return api_fail(rc, err);
  for (double v : z0)
    if (!std::isfinite(v)) return api_fail(GNUTS_ERR_SAMPLER, "flow inverse of a chain position is not finite");
  gnuts_sample_args af = *a;
  af.num_warmup = la->flow_warmup;
  af.num_samples = P;
  af.save_warmup = 0;
  af.thin = 1;
  af.seed = a->seed + 2u;
  af.delta = la->flow_delta;
  RunBufs rf(C, P, ncol, D);
  std::vector<double> z_flow((size_t)C * D);
  {
    RunConfig cfg{0, 1};
    cfg.flow = fl;
    cfg.q_last = z_flow.data();
    rc = run_nuts(m, af, cfg, z0.data(), nullptr, &rf.out, nullptr, nullptr, err);
  }
  rep.flow_seconds = now_s() - t0;
  bool flow_ok = rc == GNUTS_OK;
  if (flow_ok)
    for (int c = 0; c < C; ++c) rep.flow_grads += rf.nlf[c];

  // (4) judge
  NvtxRange judge_range("gnuts.learned.judge");
  const PilotStats sp = pilot_stats(rp.draws, C, P, ncol);
  rep.plain_ess_per_grad = sp.min_ess / std::max(1.0, sp.grads);
  rep.plain_divergence_rate = sp.div_rate;
  rep.plain_max_rhat = sp.max_rhat;
  if (flow_ok) {
    const PilotStats sf = pilot_stats(rf.draws, C, P, ncol);
    rep.flow_ess_per_grad = sf.min_ess / std::max(1.0, sf.grads);
    rep.flow_divergence_rate = sf.div_rate;
    rep.flow_max_rhat = sf.max_rhat;
    double zmax = 0;
    for (size_t k = 0; k < sp.mean.size(); ++k) {
      const double den = std::sqrt(sp.mcse[k] * sp.mcse[k] + sf.mcse[k] * sf.mcse[k]);
      const double zz = den > 0 ? std::fabs(sf.mean[k] - sp.mean[k]) / den : 0.0;
      zmax = std::max(zmax, std::isfinite(zz) ? zz : INFINITY);
    }
    rep.max_moment_z = zmax;
    const bool plain_clean = sp.div_rate <= 1e-3;
    // the flow may not mix worse than the plain sampler, nor miss the
    // convergence bound that the plain pilot meets
    const bool rhat_ok = sf.max_rhat <= std::max(la->rhat_max, sp.max_rhat);
    flow_ok = rep.flow_ess_per_grad >= rep.plain_ess_per_grad && sf.div_rate <= sp.div_rate && rhat_ok &&
              (!plain_clean || zmax <= la->moment_tolerance);
  } else {
    rep.flow_ess_per_grad = 0;
    rep.flow_divergence_rate = 1;
    rep.max_moment_z = INFINITY;
    rep.flow_max_rhat = INFINITY;
  }
  rep.used_flow = flow_ok ? 1 : 0;

  // (5) the kept sampler continues without adaptation
  t0 = now_s();
  gnuts_sample_args afin = *a;
  afin.num_warmup = 0;
  afin.save_warmup = 0;
  afin.seed = a->seed + 3u;
  RunConfig cfg{0, 0};
  cfg.flow = flow_ok ? fl : nullptr;
  cfg.stepsizes = flow_ok ? rf.eps.data() : rp.eps.data();
  const double* final_minv = flow_ok ? rf.minv.data() : rp.minv.data();
  std::vector<double> pooled_eps, pooled_minv;
  if (flow_ok) {
    // The pulled-back space is one shared coordinate system, so the kept
    // flow sampler runs every chain with the chains' median adapted step size
    // and elementwise median inverse metric.  A chain whose own adaptation
    // collapsed in a poorly mapped region (tiny step, trees at max_depth)
    // would otherwise set the wall time of the whole launch.
    auto median = [](std::vector<double> v) {
      std::sort(v.begin(), v.end());
      const size_t n = v.size();
      return n % 2 ? v[n / 2] : 0.5 * (v[n / 2 - 1] + v[n / 2]);
    };
    pooled_eps.assign(C, median(rf.eps));
    pooled_minv.assign((size_t)C * D, 0.0);
    std::vector<double> col(C);
    for (int i = 0; i < D; ++i) {
      for (int c = 0; c < C; ++c) col[c] = rf.minv[(size_t)c * D + i];
      const double v = median(col);
      for (int c = 0; c < C; ++c) pooled_minv[(size_t)c * D + i] = v;
    }
    cfg.stepsizes = pooled_eps.data();
    final_minv = pooled_minv.data();
  }
  std::vector<int64_t> nlf_fin(C, 0);
  int64_t* user_nlf = out ? out->n_leapfrog : nullptr;
  gnuts_output fin = out ? *out : gnuts_output{};
  if (!fin.n_leapfrog) fin.n_leapfrog = nlf_fin.data();
  rc = run_nuts(m, afin, cfg, flow_ok ? z_flow.data() : q_plain.data(), final_minv, &fin, progress, ctx, err);
  if (rc) return api_fail(rc, err);
  rep.final_seconds = now_s() - t0;
  for (int c = 0; c < C; ++c) rep.final_grads += fin.n_leapfrog[c];
  (void)user_nlf;
  if (report) *report = rep;
  return GNUTS_OK;
}

}  // extern "C"
