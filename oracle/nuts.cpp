// Oracle NUTS sampler (CPU, FP64, recursive) -- TEST INFRASTRUCTURE ONLY.
//
// Restates the algorithm behind CmdStan's
// stan::services::sample::hmc_nuts_{diag,dense}_e[_adapt] service calls
// (src/cmdstan/command.hpp:609-632 and 657-688).  The stan submodule is empty
// in the reference tree, so this follows the published descriptions:
//   * Hoffman & Gelman (2014) tree doubling, with Betancourt (2017)
//     multinomial sampling: biased progressive sampling between the old
//     trajectory and a new subtree, uniform progressive sampling inside a
//     subtree;
//   * generalized no-U-turn criterion p#-.rho > 0 && p#+.rho > 0 checked on
//     every merged tree and, in addition, on each half extended by the
//     adjacent point of the other half;
//   * divergence when H - H0 > 1000 (NaN energies count as +inf);
//   * accept_stat = mean over all leapfrog leaves of min(1, exp(H0 - h));
//   * dual averaging of log step size (Nesterov 2009 as used by Hoffman &
//     Gelman), mu = log(10 * stepsize);
//   * windowed adaptation: init_buffer / doubling slow windows / term_buffer
//     with the regularised update var <- n/(n+5) var + 1e-3 * 5/(n+5);
//   * step-size search (init_stepsize) after every metric update.
// The recursion below mirrors the shape of that algorithm on purpose: the
// device sampler uses an explicit-stack state machine, and equality of the
// two is what the replay tests check.
#include "oracle.h"
#include "philox.h"
#include <cmath>
#include <cstring>
#include <cstdio>
#include <limits>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>
#include <atomic>

namespace {

using Vec = std::vector<double>;
const double INF = std::numeric_limits<double>::infinity();

inline double lse(double a, double b) {
  if (a == -INF) return b;
  if (b == -INF) return a;
  double m = a > b ? a : b;
  return m + std::log1p(std::exp(-std::fabs(a - b)));
}
inline double dot(const Vec& a, const Vec& b) {
  double s = 0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

struct Point {
  Vec q, p, g;  // g = gradient of lp
  double lp = 0;
};

struct Metric {
  int kind = 0;  // 0 diag, 1 dense, 2 unit
  int D = 0;
  Vec minv;  // D or D*D
  Vec L;     // Cholesky factor of dense minv (lower, row-major)
  void set(int k, int d, const double* init) {
    kind = k; D = d;
    if (kind == 1) {
      minv.assign((size_t)D * D, 0.0);
      if (init) std::memcpy(minv.data(), init, sizeof(double) * D * D);
      else for (int i = 0; i < D; ++i) minv[(size_t)i * D + i] = 1.0;
      factor();
    } else {
      minv.assign(D, 1.0);
      if (init && kind == 0) std::memcpy(minv.data(), init, sizeof(double) * D);
    }
  }
  void factor() {
    L.assign((size_t)D * D, 0.0);
    for (int j = 0; j < D; ++j) {
      double s = minv[(size_t)j * D + j];
      for (int k = 0; k < j; ++k) s -= L[(size_t)j * D + k] * L[(size_t)j * D + k];
      if (!(s > 0)) throw std::runtime_error("inverse metric is not positive definite");
      double d = std::sqrt(s);
      L[(size_t)j * D + j] = d;
      for (int i = j + 1; i < D; ++i) {
        double t = minv[(size_t)i * D + j];
        for (int k = 0; k < j; ++k) t -= L[(size_t)i * D + k] * L[(size_t)j * D + k];
        L[(size_t)i * D + j] = t / d;
      }
    }
  }
  void dtau_dp(const Vec& p, Vec& out) const {
    out.resize(D);
    if (kind == 1) {
      for (int i = 0; i < D; ++i) {
        double s = 0;
        for (int j = 0; j < D; ++j) s += minv[(size_t)i * D + j] * p[j];
        out[i] = s;
      }
    } else {
      for (int i = 0; i < D; ++i) out[i] = minv[i] * p[i];
    }
  }
  double tau(const Vec& p) const {
    Vec t;
    dtau_dp(p, t);
    return 0.5 * dot(p, t);
  }
  // p ~ N(0, M): diag p_i = z_i / sqrt(minv_i); dense p = L^{-T} z
  void sample_p(orc_rng* rng, Vec& p) const {
    p.resize(D);
    Vec z(D);
    orc_next_normals(rng, D, z.data());
    if (kind == 1) {
      for (int i = D - 1; i >= 0; --i) {
        double s = z[i];
        for (int k = i + 1; k < D; ++k) s -= L[(size_t)k * D + i] * p[k];
        p[i] = s / L[(size_t)i * D + i];
      }
    } else {
      for (int i = 0; i < D; ++i) p[i] = z[i] / std::sqrt(minv[i]);
    }
  }
};

struct Sampler {
  const orc_model* model;
  int D;
  Metric metric;
  orc_rng rng;
  double nom_eps = 1, eps = 1, jitter = 0;
  int max_depth = 10;
  double max_dH = 1000;
  long long n_grad = 0;
  // per-transition
  Point z;
  int depth = 0;
  bool divergent = false;

  double H(const Point& a) const { return metric.tau(a.p) - a.lp; }
  void gradient(Point& a) {
    a.g.resize(D);
    a.lp = orc_log_prob_grad(model, a.q.data(), 1, a.g.data());
    ++n_grad;
  }
  void leapfrog(Point& a, double e) {
    for (int i = 0; i < D; ++i) a.p[i] += 0.5 * e * a.g[i];
    Vec v;
    metric.dtau_dp(a.p, v);
    for (int i = 0; i < D; ++i) a.q[i] += e * v[i];
    gradient(a);
    for (int i = 0; i < D; ++i) a.p[i] += 0.5 * e * a.g[i];
  }
  static bool crit(const Vec& ps_minus, const Vec& ps_plus, const Vec& rho) {
    return dot(ps_plus, rho) > 0 && dot(ps_minus, rho) > 0;
  }

  // Recursive subtree of 2^d leapfrogs in direction `sign` starting from z.
  // Outputs follow the published algorithm's argument list.
  bool build_tree(int d, Point& z_propose, Vec& ps_beg, Vec& ps_end, Vec& rho, Vec& p_beg,
                  Vec& p_end, double H0, double sign, int& n_leapfrog, double& lsw,
                  double& sum_metro) {
    if (d == 0) {
      leapfrog(z, sign * eps);
      ++n_leapfrog;
      double h = H(z);
      if (std::isnan(h)) h = INF;
      if (h - H0 > max_dH) divergent = true;
      lsw = lse(lsw, H0 - h);
      sum_metro += (H0 - h > 0) ? 1.0 : std::exp(H0 - h);
      z_propose = z;
      metric.dtau_dp(z.p, ps_beg);
      ps_end = ps_beg;
      for (int i = 0; i < D; ++i) rho[i] += z.p[i];
      p_beg = z.p;
      p_end = p_beg;
      return !divergent;
    }
    double lsw_init = -INF;
    Vec p_init_end(D), ps_init_end(D), rho_init(D, 0.0);
    bool ok = build_tree(d - 1, z_propose, ps_beg, ps_init_end, rho_init, p_beg, p_init_end, H0,
                         sign, n_leapfrog, lsw_init, sum_metro);
    if (!ok) return false;
    Point z_prop_final = z;
    double lsw_final = -INF;
    Vec p_final_beg(D), ps_final_beg(D), rho_final(D, 0.0);
    ok = build_tree(d - 1, z_prop_final, ps_final_beg, ps_end, rho_final, p_final_beg, p_end, H0,
                    sign, n_leapfrog, lsw_final, sum_metro);
    if (!ok) return false;
    double lsw_sub = lse(lsw_init, lsw_final);
    lsw = lse(lsw, lsw_sub);
    if (lsw_final > lsw_sub) {
      z_propose = z_prop_final;
    } else {
      double a = std::exp(lsw_final - lsw_sub);
      if (orc_next_uniform(&rng) < a) z_propose = z_prop_final;
    }
    Vec rho_sub(D);
    for (int i = 0; i < D; ++i) {
      rho_sub[i] = rho_init[i] + rho_final[i];
      rho[i] += rho_sub[i];
    }
    bool persist = crit(ps_beg, ps_end, rho_sub);
    Vec ext(D);
    for (int i = 0; i < D; ++i) ext[i] = rho_init[i] + p_final_beg[i];
    persist = persist && crit(ps_beg, ps_final_beg, ext);
    for (int i = 0; i < D; ++i) ext[i] = rho_final[i] + p_init_end[i];
    persist = persist && crit(ps_init_end, ps_end, ext);
    return persist;
  }

  struct Stats { double lp, accept, eps; int depth, n_leapfrog, divergent; double energy; };

  // One transition from z (with z.g, z.lp valid).  If p0 is given it is used
  // as the momentum instead of a draw (jitter is then not drawn either).
  Stats transition(const double* p0) {
    eps = nom_eps;
    if (!p0 && jitter > 0) eps *= 1.0 + jitter * (2.0 * orc_next_uniform(&rng) - 1.0);
    if (p0) z.p.assign(p0, p0 + D);
    else metric.sample_p(&rng, z.p);

    Point z_fwd = z, z_bck = z, z_sample = z, z_propose = z;
    Vec p_ff = z.p, ps_ff, p_fb = z.p, p_bf = z.p, p_bb = z.p;
    metric.dtau_dp(z.p, ps_ff);
    Vec ps_fb = ps_ff, ps_bf = ps_ff, ps_bb = ps_ff;
    Vec rho = z.p;
    double lsw = 0;
    double H0 = H(z);
    int n_leapfrog = 0;
    double sum_metro = 0;
    depth = 0;
    divergent = false;

    while (depth < max_depth) {
      Vec rho_fwd(D, 0.0), rho_bck(D, 0.0);
      bool valid = false;
      double lsw_sub = -INF;
      if (orc_next_uniform(&rng) > 0.5) {
        z = z_fwd;
        rho_bck = rho;
        p_bf = p_ff;
        ps_bf = ps_ff;
        valid = build_tree(depth, z_propose, ps_fb, ps_ff, rho_fwd, p_fb, p_ff, H0, 1.0, n_leapfrog,
                           lsw_sub, sum_metro);
        z_fwd = z;
      } else {
        z = z_bck;
        rho_fwd = rho;
        p_fb = p_bb;
        ps_fb = ps_bb;
        valid = build_tree(depth, z_propose, ps_bf, ps_bb, rho_bck, p_bf, p_bb, H0, -1.0, n_leapfrog,
                           lsw_sub, sum_metro);
        z_bck = z;
      }
      if (!valid) break;
      ++depth;
      if (lsw_sub > lsw) {
        z_sample = z_propose;
      } else {
        double a = std::exp(lsw_sub - lsw);
        if (orc_next_uniform(&rng) < a) z_sample = z_propose;
      }
      lsw = lse(lsw, lsw_sub);
      for (int i = 0; i < D; ++i) rho[i] = rho_bck[i] + rho_fwd[i];
      bool persist = crit(ps_bb, ps_ff, rho);
      Vec ext(D);
      for (int i = 0; i < D; ++i) ext[i] = rho_bck[i] + p_fb[i];
      persist = persist && crit(ps_bb, ps_fb, ext);
      for (int i = 0; i < D; ++i) ext[i] = rho_fwd[i] + p_bf[i];
      persist = persist && crit(ps_bf, ps_ff, ext);
      if (!persist) break;
    }
    z = z_sample;
    Stats s;
    s.lp = z.lp;
    s.accept = sum_metro / (double)n_leapfrog;
    s.eps = eps;
    s.depth = depth;
    s.n_leapfrog = n_leapfrog;
    s.divergent = divergent ? 1 : 0;
    s.energy = H(z);
    return s;
  }

  // Step-size search run before warmup and after every metric update.
  void init_stepsize() {
    Point z_init = z;
    if (nom_eps == 0 || nom_eps > 1e7 || std::isnan(nom_eps)) return;
    metric.sample_p(&rng, z.p);
    double H0 = H(z);
    leapfrog(z, nom_eps);
    double h = H(z);
    if (std::isnan(h)) h = INF;
    double dH = H0 - h;
    int direction = dH > std::log(0.8) ? 1 : -1;
    while (true) {
      z = z_init;
      metric.sample_p(&rng, z.p);
      double H0b = H(z);
      leapfrog(z, nom_eps);
      double hb = H(z);
      if (std::isnan(hb)) hb = INF;
      double dHb = H0b - hb;
      if (direction == 1 && !(dHb > std::log(0.8))) break;
      if (direction == -1 && !(dHb < std::log(0.8))) break;
      nom_eps = direction == 1 ? 2 * nom_eps : 0.5 * nom_eps;
      if (nom_eps > 1e7) throw std::runtime_error("Posterior is improper. Please check your model.");
      if (nom_eps == 0)
        throw std::runtime_error(
            "No acceptably small step size could be found. Perhaps the posterior is not continuous?");
    }
    z = z_init;
  }
};

struct DualAveraging {
  double mu = 0, delta = 0.8, gamma = 0.05, kappa = 0.75, t0 = 10;
  double counter = 0, s_bar = 0, x_bar = 0;
  void restart() { counter = 0; s_bar = 0; x_bar = 0; }
  void learn(double& eps, double stat) {
    counter += 1;
    stat = stat > 1 ? 1 : stat;
    double eta = 1.0 / (counter + t0);
    s_bar = (1.0 - eta) * s_bar + eta * (delta - stat);
    double x = mu - s_bar * std::sqrt(counter) / gamma;
    double xe = std::pow(counter, -kappa);
    x_bar = (1.0 - xe) * x_bar + xe * x;
    eps = std::exp(x);
  }
  void complete(double& eps) { eps = std::exp(x_bar); }
};

struct Windows {
  unsigned num_warmup = 0, init_buffer = 0, term_buffer = 0, base_window = 0;
  unsigned counter = 0, size = 0, next = 0;
  void restart() {
    counter = 0;
    size = base_window;
    next = init_buffer + size - 1;
  }
  void set(unsigned nw, unsigned ib, unsigned tb, unsigned bw) {
    if (nw < 20) { restart(); return; }
    if (ib + bw + tb > nw) {
      num_warmup = nw;
      init_buffer = (unsigned)(0.15 * nw);
      term_buffer = (unsigned)(0.1 * nw);
      base_window = nw - (init_buffer + term_buffer);
      restart();
      return;
    }
    num_warmup = nw; init_buffer = ib; term_buffer = tb; base_window = bw;
    restart();
  }
  bool in_window() const {
    return counter >= init_buffer && counter < num_warmup - term_buffer && counter != num_warmup;
  }
  bool end_window() const { return counter == next && counter != num_warmup; }
  void compute_next() {
    if (next == num_warmup - term_buffer - 1) return;
    size *= 2;
    next = counter + size;
    if (next != num_warmup - term_buffer - 1) {
      unsigned boundary = next + 2 * size;
      if (boundary >= num_warmup - term_buffer) next = num_warmup - term_buffer - 1;
    }
  }
};

struct Welford {
  int D = 0; bool dense = false; long n = 0;
  Vec m, m2;
  void init(int d, bool de) { D = d; dense = de; restart(); }
  void restart() {
    n = 0;
    m.assign(D, 0.0);
    m2.assign(dense ? (size_t)D * D : (size_t)D, 0.0);
  }
  void add(const Vec& q) {
    ++n;
    Vec delta(D);
    for (int i = 0; i < D; ++i) { delta[i] = q[i] - m[i]; m[i] += delta[i] / n; }
    if (dense) {
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) m2[(size_t)i * D + j] += (q[i] - m[i]) * delta[j];
    } else {
      for (int i = 0; i < D; ++i) m2[i] += (q[i] - m[i]) * delta[i];
    }
  }
};

void record(double* row, const Sampler::Stats& s, const Vec& q, int D) {
  row[0] = s.lp; row[1] = s.accept; row[2] = s.eps; row[3] = s.depth;
  row[4] = s.n_leapfrog; row[5] = s.divergent; row[6] = s.energy;
  for (int i = 0; i < D; ++i) row[7 + i] = q[i];
}

bool finite_point(const Point& z) {
  if (!std::isfinite(z.lp)) return false;
  for (double v : z.g) if (!std::isfinite(v)) return false;
  return true;
}

}  // namespace

extern "C" {

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  orc_philox_impl(ctr, key, out);
}
double orc_uniform(uint32_t seed, uint32_t chain, uint32_t stream, uint64_t counter) {
  orc_rng g{seed, chain, stream, counter};
  return orc_next_uniform(&g);
}
void orc_normal_pair(uint32_t seed, uint32_t chain, uint32_t stream, uint64_t counter, double out[2]) {
  orc_rng g{seed, chain, stream, counter};
  orc_next_normals(&g, 2, out);
}

int orc_run_chain(const orc_model* m, const orc_args* a, uint32_t chain_id, const double* init_q,
                  const double* inv_metric, double* draws, double* adapted_stepsize,
                  double* adapted_metric, long long* n_grad, char* errbuf, int errlen) {
  const int D = orc_model_dim(m);
  Sampler S;
  S.model = m;
  S.D = D;
  S.rng = orc_rng{a->seed, chain_id, 0u, 0ull};
  try {
    S.metric.set(a->metric, D, a->metric == 2 ? nullptr : inv_metric);
  } catch (const std::exception& e) {
    if (errbuf) snprintf(errbuf, errlen, "%s", e.what());
    return 1;
  }
  // ---- initialisation (stan::services::util::initialize) ----
  orc_rng irng{a->seed, chain_id, 1u, 0ull};
  S.z.q.assign(D, 0.0);
  bool ok = false;
  int attempts = (init_q || a->init_radius == 0) ? 1 : 100;
  for (int t = 0; t < attempts && !ok; ++t) {
    if (init_q) {
      S.z.q.assign(init_q, init_q + D);
    } else {
      for (int i = 0; i < D; ++i) S.z.q[i] = a->init_radius * (2.0 * orc_next_uniform(&irng) - 1.0);
    }
    S.gradient(S.z);
    ok = finite_point(S.z);
  }
  if (!ok) {
    if (errbuf) snprintf(errbuf, errlen, "Initialization failed.");
    return 2;
  }
  S.nom_eps = a->stepsize;
  S.jitter = a->stepsize_jitter;
  S.max_depth = a->max_depth;

  DualAveraging da;
  Windows win;
  Welford wf;
  const bool adapt = a->adapt_engaged != 0;
  if (adapt) {
    da.mu = std::log(10.0 * a->stepsize);
    da.delta = a->delta; da.gamma = a->gamma; da.kappa = a->kappa; da.t0 = a->t0;
    da.restart();
    win.set((unsigned)a->num_warmup, a->init_buffer, a->term_buffer, a->window);
    wf.init(D, a->metric == 1);
    try {
      S.init_stepsize();
    } catch (const std::exception& e) {
      if (errbuf) snprintf(errbuf, errlen, "%s", e.what());
      return 3;
    }
  }
  const int ncol = ORC_NSAMPLER_COLS + D;
  long row = 0;
  try {
    for (int it = 0; it < a->num_warmup; ++it) {
      Sampler::Stats s = S.transition(nullptr);
      if (adapt) {
        da.learn(S.nom_eps, s.accept);
        if (a->metric != 2) {
          if (win.in_window()) wf.add(S.z.q);
          if (win.end_window()) {
            win.compute_next();
            double n = (double)wf.n;
            if (a->metric == 1) {
              for (int i = 0; i < D; ++i)
                for (int j = 0; j < D; ++j) {
                  double v = wf.m2[(size_t)i * D + j] / (n - 1.0);
                  v = (n / (n + 5.0)) * v + (i == j ? 1e-3 * (5.0 / (n + 5.0)) : 0.0);
                  S.metric.minv[(size_t)i * D + j] = v;
                }
              S.metric.factor();
            } else {
              for (int i = 0; i < D; ++i) {
                double v = wf.m2[i] / (n - 1.0);
                S.metric.minv[i] = (n / (n + 5.0)) * v + 1e-3 * (5.0 / (n + 5.0));
              }
            }
            for (double v : S.metric.minv)
              if (!std::isfinite(v)) throw std::runtime_error("Numerical overflow in metric adaptation.");
            wf.restart();
            ++win.counter;
            S.init_stepsize();
            da.mu = std::log(10.0 * S.nom_eps);
            da.restart();
          } else {
            ++win.counter;
          }
        }
      }
      if (a->save_warmup && it % a->thin == 0) record(draws + (row++) * ncol, s, S.z.q, D);
    }
    if (adapt) da.complete(S.nom_eps);
    for (int it = 0; it < a->num_samples; ++it) {
      Sampler::Stats s = S.transition(nullptr);
      if (it % a->thin == 0) record(draws + (row++) * ncol, s, S.z.q, D);
    }
  } catch (const std::exception& e) {
    if (errbuf) snprintf(errbuf, errlen, "%s", e.what());
    return 4;
  }
  if (adapted_stepsize) *adapted_stepsize = S.nom_eps;
  if (adapted_metric) std::memcpy(adapted_metric, S.metric.minv.data(), sizeof(double) * S.metric.minv.size());
  if (n_grad) *n_grad = S.n_grad;
  return 0;
}

int orc_run_chains(const orc_model* m, const orc_args* a, int n_chains, uint32_t first_chain_id,
                   int n_threads, const double* init_q, const double* inv_metric, double* draws,
                   double* adapted_stepsize, double* adapted_metric, long long* n_grad) {
  const int D = orc_model_dim(m);
  const long n_saved = (a->save_warmup ? (a->num_warmup + a->thin - 1) / a->thin : 0) +
                       (a->num_samples + a->thin - 1) / a->thin;
  const long per_chain = n_saved * (ORC_NSAMPLER_COLS + D);
  const long msize = a->metric == 1 ? (long)D * D : D;
  std::atomic<int> next{0};
  std::atomic<int> rc{0};
  auto work = [&]() {
    for (;;) {
      int c = next.fetch_add(1);
      if (c >= n_chains) return;
      long long ng = 0;
      int r = orc_run_chain(m, a, first_chain_id + c, init_q ? init_q + (long)c * D : nullptr,
                            inv_metric ? inv_metric + (long)c * msize : nullptr, draws + c * per_chain,
                            adapted_stepsize ? adapted_stepsize + c : nullptr,
                            adapted_metric ? adapted_metric + c * msize : nullptr, &ng, nullptr, 0);
      if (n_grad) n_grad[c] = ng;
      if (r) rc = r;
    }
  };
  if (n_threads < 1) n_threads = 1;
  std::vector<std::thread> th;
  for (int t = 0; t < n_threads; ++t) th.emplace_back(work);
  for (auto& t : th) t.join();
  return rc.load();
}

int orc_transition(const orc_model* m, int metric, const double* inv_metric, const double* q0,
                   const double* p0, double eps, int max_depth, uint32_t seed, uint32_t chain,
                   uint64_t* counter, double* out_q, double* out_stats) {
  const int D = orc_model_dim(m);
  Sampler S;
  S.model = m;
  S.D = D;
  S.rng = orc_rng{seed, chain, 0u, *counter};
  S.metric.set(metric, D, metric == 2 ? nullptr : inv_metric);
  S.z.q.assign(q0, q0 + D);
  S.gradient(S.z);
  S.nom_eps = eps;
  S.max_depth = max_depth;
  Sampler::Stats s = S.transition(p0);
  *counter = S.rng.n;
  std::memcpy(out_q, S.z.q.data(), sizeof(double) * D);
  out_stats[0] = s.lp; out_stats[1] = s.accept; out_stats[2] = s.eps; out_stats[3] = s.depth;
  out_stats[4] = s.n_leapfrog; out_stats[5] = s.divergent; out_stats[6] = s.energy;
  return 0;
}

}  // extern "C"
