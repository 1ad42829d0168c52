// Oracle log densities with analytic gradients -- TEST INFRASTRUCTURE ONLY.
//
// Each model restates, in FP64, the log density that stanc + Stan Math
// would compute for the corresponding Stan program through
// stan::model::log_prob_grad<true, jacobian> (contract visible at
// src/cmdstan/command_helper.hpp:589-593): `propto` drops every term that
// does not depend on parameters, and `jacobian` adds the log-Jacobian of
// the constraining transforms (lower=0 -> exp, (0,1) -> inv_logit).
//
//   bernoulli  src/test/test-models (bernoulli example): theta ~ beta(1,1),
//              y ~ bernoulli(theta)
//   normal     proper.stan / test_model.stan: x_k ~ normal(0, s_k)
//   logistic   alpha ~ normal(0,2.5), beta ~ normal(0,1),
//              y ~ bernoulli_logit(alpha + X beta)
//   hier       eight_schools.stan with mu ~ normal(0,5),
//              tau ~ cauchy(0,5) (half), theta ~ normal(mu,tau),
//              y ~ normal(theta, sigma); unconstrained order mu, theta, tau
//              as declared in eight_schools.stan
//   funnel     v ~ normal(0,3), x_k ~ normal(0, exp(v/2))
//   varint     alpha_j ~ normal(0,tau), beta ~ normal(0,1),
//              sigma_y ~ normal(0,1) (half), tau ~ normal(0,1) (half),
//              y_n ~ normal(alpha[g_n] + x_n beta, sigma_y)
//   horseshoe  regularised horseshoe (Piironen & Vehtari 2017) logistic
//              regression: beta0 ~ normal(0,2.5), z ~ normal(0,1),
//              lambda ~ cauchy(0,1) (half), tau ~ cauchy(0,scale_global)
//              (half), caux ~ inv_gamma(nu/2, nu/2), c = slab_scale*sqrt(caux),
//              lambda_t = sqrt(c^2 lambda^2 / (c^2 + tau^2 lambda^2)),
//              beta = z .* lambda_t * tau, y ~ bernoulli_logit(beta0 + X beta)
#include "oracle.h"
#include <cmath>
#include <cstring>
#include <vector>
#include <string>

namespace {

inline double log1p_exp(double a) { return a > 0 ? a + std::log1p(std::exp(-a)) : std::log1p(std::exp(a)); }
inline double inv_logit(double a) {
  if (a >= 0) return 1.0 / (1.0 + std::exp(-a));
  double e = std::exp(a);
  return e / (1.0 + e);
}

enum Kind { BERN, NORMAL, LOGISTIC, HIER, FUNNEL, VARINT, HORSESHOE };

// x . b in FP64 with four interleaved partial sums, ((s0 + s1) + (s2 + s3))
// plus the tail: the row products of a GLM as a vectorising CPU library
// forms them (a single running sum is one serial add chain per row)
static double dot4(const double* x, const double* b, int D) {
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  int d = 0;
  for (; d + 4 <= D; d += 4) {
    s0 += x[d] * b[d];
    s1 += x[d + 1] * b[d + 1];
    s2 += x[d + 2] * b[d + 2];
    s3 += x[d + 3] * b[d + 3];
  }
  double t = (s0 + s1) + (s2 + s3);
  for (; d < D; ++d) t += x[d] * b[d];
  return t;
}

}  // namespace

struct orc_model {
  Kind kind;
  int N = 0, D = 0, J = 0, K = 0;
  std::vector<int> yi, group;
  std::vector<double> yr, X, sigma, scales;
  double scale_global = 0, slab_scale = 0, slab_df = 0;
  int dim = 0, ncon = 0;
};

extern "C" {

orc_model* orc_bernoulli(int N, const int* y) {
  auto* m = new orc_model{};
  m->kind = BERN; m->N = N; m->yi.assign(y, y + N); m->dim = 1; m->ncon = 1;
  return m;
}
orc_model* orc_normal(int K, const double* scales) {
  auto* m = new orc_model{};
  m->kind = NORMAL; m->K = K; m->scales.assign(scales, scales + K); m->dim = K; m->ncon = K;
  return m;
}
orc_model* orc_logistic(int N, int D, const double* X, const int* y) {
  auto* m = new orc_model{};
  m->kind = LOGISTIC; m->N = N; m->D = D;
  m->X.assign(X, X + (size_t)N * D); m->yi.assign(y, y + N);
  m->dim = D + 1; m->ncon = D + 1;
  return m;
}
orc_model* orc_hier(int J, const double* y, const double* sigma) {
  auto* m = new orc_model{};
  m->kind = HIER; m->J = J; m->yr.assign(y, y + J); m->sigma.assign(sigma, sigma + J);
  m->dim = J + 2; m->ncon = J + 2;
  return m;
}
orc_model* orc_funnel(int K) {
  auto* m = new orc_model{};
  m->kind = FUNNEL; m->K = K; m->dim = K + 1; m->ncon = K + 1;
  return m;
}
orc_model* orc_varint(int N, int J, int K, const int* group, const double* X, const double* y) {
  auto* m = new orc_model{};
  m->kind = VARINT; m->N = N; m->J = J; m->K = K;
  m->group.assign(group, group + N); m->X.assign(X, X + (size_t)N * K); m->yr.assign(y, y + N);
  m->dim = J + K + 2; m->ncon = J + K + 2;
  return m;
}
orc_model* orc_horseshoe(int N, int D, const double* X, const int* y, double scale_global,
                         double slab_scale, double slab_df) {
  auto* m = new orc_model{};
  m->kind = HORSESHOE; m->N = N; m->D = D;
  m->X.assign(X, X + (size_t)N * D); m->yi.assign(y, y + N);
  m->scale_global = scale_global; m->slab_scale = slab_scale; m->slab_df = slab_df;
  m->dim = 2 * D + 3;
  m->ncon = 2 * D + 3 + D;  // beta0, z, tau, lambda, caux, then beta (transformed)
  return m;
}
void orc_model_free(orc_model* m) { delete m; }
int orc_model_dim(const orc_model* m) { return m->dim; }
int orc_model_num_constrained(const orc_model* m) { return m->ncon; }

double orc_log_prob_grad(const orc_model* m, const double* q, int jac, double* g) {
  const double J = jac ? 1.0 : 0.0;
  switch (m->kind) {
    case BERN: {
      double u = q[0];
      int s = 0;
      for (int n = 0; n < m->N; ++n) s += m->yi[n];
      double a = s + J, b = (m->N - s) + J;
      double th = inv_logit(u);
      // log theta = -log1p_exp(-u), log(1-theta) = -log1p_exp(u)
      double lp = -a * log1p_exp(-u) - b * log1p_exp(u);
      g[0] = a * (1.0 - th) - b * th;
      return lp;
    }
    case NORMAL: {
      double lp = 0;
      for (int k = 0; k < m->K; ++k) {
        double s = m->scales[k];
        lp += -0.5 * (q[k] / s) * (q[k] / s);
        g[k] = -q[k] / (s * s);
      }
      return lp;
    }
    case LOGISTIC: {
      const int N = m->N, D = m->D;
      double alpha = q[0];
      const double* beta = q + 1;
      double lp = 0;
      for (int d = 0; d <= D; ++d) g[d] = 0;
      for (int n = 0; n < N; ++n) {
        const double* x = &m->X[(size_t)n * D];
        const double eta = alpha + dot4(x, beta, D);
        int y = m->yi[n];
        lp += y * eta - log1p_exp(eta);
        double r = y - inv_logit(eta);
        g[0] += r;
        for (int d = 0; d < D; ++d) g[1 + d] += r * x[d];
      }
      lp += -0.5 * (alpha / 2.5) * (alpha / 2.5);
      g[0] += -alpha / 6.25;
      for (int d = 0; d < D; ++d) {
        lp += -0.5 * beta[d] * beta[d];
        g[1 + d] += -beta[d];
      }
      return lp;
    }
    case HIER: {
      // unconstrained: [mu, theta_1..J, log tau]  (declaration order of eight_schools.stan)
      const int Jn = m->J;
      double mu = q[0];
      const double* th = q + 1;
      double lt = q[Jn + 1], tau = std::exp(lt);
      double lp = -0.5 * (mu / 5.0) * (mu / 5.0);
      double gmu = -mu / 25.0, glt = 0;
      // half-cauchy(0,5) on tau: -log(1 + (tau/5)^2)
      double t5 = tau / 5.0;
      lp += -std::log1p(t5 * t5);
      glt += -2.0 * t5 * t5 / (1.0 + t5 * t5);
      for (int j = 0; j < Jn; ++j) {
        double z = (th[j] - mu) / tau;
        lp += -lt - 0.5 * z * z;
        g[1 + j] = -z / tau;
        gmu += z / tau;
        glt += -1.0 + z * z;
        double e = (m->yr[j] - th[j]) / m->sigma[j];
        lp += -0.5 * e * e;
        g[1 + j] += e / m->sigma[j];
      }
      lp += J * lt;
      glt += J;
      g[0] = gmu;
      g[Jn + 1] = glt;
      return lp;
    }
    case FUNNEL: {
      double v = q[0];
      double lp = -0.5 * (v / 3.0) * (v / 3.0);
      double gv = -v / 9.0;
      double ev = std::exp(-v);
      for (int k = 0; k < m->K; ++k) {
        double x = q[1 + k];
        lp += -0.5 * v - 0.5 * x * x * ev;
        gv += -0.5 + 0.5 * x * x * ev;
        g[1 + k] = -x * ev;
      }
      g[0] = gv;
      return lp;
    }
    case VARINT: {
      // unconstrained: [alpha_1..J, beta_1..K, log sigma_y, log tau]
      const int Jn = m->J, Kn = m->K, N = m->N;
      const double* al = q;
      const double* be = q + Jn;
      double ls = q[Jn + Kn], lt = q[Jn + Kn + 1];
      double sy = std::exp(ls), tau = std::exp(lt);
      for (int i = 0; i < m->dim; ++i) g[i] = 0;
      double lp = 0, gls = 0, glt = 0;
      for (int j = 0; j < Jn; ++j) {
        double z = al[j] / tau;
        lp += -lt - 0.5 * z * z;
        g[j] += -z / tau;
        glt += -1.0 + z * z;
      }
      for (int k = 0; k < Kn; ++k) {
        lp += -0.5 * be[k] * be[k];
        g[Jn + k] += -be[k];
      }
      lp += -0.5 * sy * sy - 0.5 * tau * tau;
      gls += -sy * sy;
      glt += -tau * tau;
      double isy = 1.0 / sy;
      double ss = 0;
      for (int n = 0; n < N; ++n) {
        const double* x = &m->X[(size_t)n * Kn];
        int gj = m->group[n] - 1;
        double mu = al[gj];
        for (int k = 0; k < Kn; ++k) mu += x[k] * be[k];
        double e = (m->yr[n] - mu) * isy;
        ss += e * e;
        double r = e * isy;  // d/dmu
        g[gj] += r;
        for (int k = 0; k < Kn; ++k) g[Jn + k] += r * x[k];
      }
      lp += -N * ls - 0.5 * ss;
      gls += -N + ss;
      lp += J * (ls + lt);
      gls += J;
      glt += J;
      g[Jn + Kn] = gls;
      g[Jn + Kn + 1] = glt;
      return lp;
    }
    case HORSESHOE: {
      // unconstrained: [beta0, z_1..D, log tau, log lambda_1..D, log caux]
      const int D = m->D, N = m->N;
      double b0 = q[0];
      const double* z = q + 1;
      double lt = q[D + 1], tau = std::exp(lt);
      const double* ll = q + D + 2;
      double lc = q[2 * D + 2], caux = std::exp(lc);
      const double nu = m->slab_df, ss = m->slab_scale, sg = m->scale_global;
      double c2 = ss * ss * caux;
      std::vector<double> beta(D), lamt(D), lam(D);
      for (int d = 0; d < D; ++d) {
        lam[d] = std::exp(ll[d]);
        double l2 = lam[d] * lam[d];
        lamt[d] = std::sqrt(c2 * l2 / (c2 + tau * tau * l2));
        beta[d] = z[d] * lamt[d] * tau;
      }
      // likelihood
      std::vector<double> gb(D, 0.0);
      double lp = 0, gb0 = 0;
      for (int n = 0; n < N; ++n) {
        const double* x = &m->X[(size_t)n * D];
        const double eta = b0 + dot4(x, beta.data(), D);
        int y = m->yi[n];
        lp += y * eta - log1p_exp(eta);
        double r = y - inv_logit(eta);
        gb0 += r;
        for (int d = 0; d < D; ++d) gb[d] += r * x[d];
      }
      // priors
      lp += -0.5 * (b0 / 2.5) * (b0 / 2.5);
      gb0 += -b0 / 6.25;
      double glt = 0, glc = 0;
      for (int d = 0; d < D; ++d) {
        lp += -0.5 * z[d] * z[d];
        lp += -std::log1p(lam[d] * lam[d]);
      }
      double ts = tau / sg;
      lp += -std::log1p(ts * ts);
      glt += -2.0 * ts * ts / (1.0 + ts * ts);
      lp += (-0.5 * nu - 1.0) * lc - 0.5 * nu / caux;
      glc += (-0.5 * nu - 1.0) + 0.5 * nu / caux;
      // chain rule through beta_d = z_d * tau * lamt_d,
      // lamt_d^2 = c2 l2 / (c2 + tau^2 l2)
      // d log lamt / d log lambda = c2 / (c2 + tau^2 l2)
      // d log lamt / d log tau    = -tau^2 l2 / (c2 + tau^2 l2)
      // d log lamt / d log caux   = 0.5 * tau^2 l2 / (c2 + tau^2 l2)
      g[0] = gb0;
      for (int d = 0; d < D; ++d) {
        double l2 = lam[d] * lam[d];
        double den = c2 + tau * tau * l2;
        double a = c2 / den, b = tau * tau * l2 / den;
        double gbd = gb[d] * beta[d];  // d lp / d log|beta| contribution
        g[1 + d] = gb[d] * lamt[d] * tau - z[d];
        glt += gbd * (1.0 - b);
        g[D + 2 + d] = gbd * a - 2.0 * l2 / (1.0 + l2) + J;
        glc += gbd * 0.5 * b;
      }
      lp += J * (lt + lc);
      for (int d = 0; d < D; ++d) lp += J * ll[d];
      glt += J;
      glc += J;
      g[D + 1] = glt;
      g[2 * D + 2] = glc;
      return lp;
    }
  }
  return NAN;
}

void orc_write_array(const orc_model* m, const double* q, double* out) {
  switch (m->kind) {
    case BERN: out[0] = inv_logit(q[0]); return;
    case NORMAL:
    case LOGISTIC:
    case FUNNEL:
      for (int i = 0; i < m->dim; ++i) out[i] = q[i];
      return;
    case HIER:
      for (int i = 0; i < m->J + 1; ++i) out[i] = q[i];
      out[m->J + 1] = std::exp(q[m->J + 1]);
      return;
    case VARINT:
      for (int i = 0; i < m->J + m->K; ++i) out[i] = q[i];
      out[m->J + m->K] = std::exp(q[m->J + m->K]);
      out[m->J + m->K + 1] = std::exp(q[m->J + m->K + 1]);
      return;
    case HORSESHOE: {
      const int D = m->D;
      double tau = std::exp(q[D + 1]), caux = std::exp(q[2 * D + 2]);
      double c2 = m->slab_scale * m->slab_scale * caux;
      out[0] = q[0];
      for (int d = 0; d < D; ++d) out[1 + d] = q[1 + d];
      out[D + 1] = tau;
      for (int d = 0; d < D; ++d) out[D + 2 + d] = std::exp(q[D + 2 + d]);
      out[2 * D + 2] = caux;
      for (int d = 0; d < D; ++d) {
        double l2 = out[D + 2 + d] * out[D + 2 + d];
        double lamt = std::sqrt(c2 * l2 / (c2 + tau * tau * l2));
        out[2 * D + 3 + d] = q[1 + d] * lamt * tau;
      }
      return;
    }
  }
}

int orc_unconstrain(const orc_model* m, const double* c, double* q) {
  switch (m->kind) {
    case BERN:
      if (!(c[0] > 0 && c[0] < 1)) return 1;
      q[0] = std::log(c[0] / (1.0 - c[0]));
      return 0;
    case NORMAL:
    case LOGISTIC:
    case FUNNEL:
      for (int i = 0; i < m->dim; ++i) q[i] = c[i];
      return 0;
    case HIER:
      for (int i = 0; i < m->J + 1; ++i) q[i] = c[i];
      if (!(c[m->J + 1] > 0)) return 1;
      q[m->J + 1] = std::log(c[m->J + 1]);
      return 0;
    case VARINT:
      for (int i = 0; i < m->J + m->K; ++i) q[i] = c[i];
      for (int i = m->J + m->K; i < m->dim; ++i) {
        if (!(c[i] > 0)) return 1;
        q[i] = std::log(c[i]);
      }
      return 0;
    case HORSESHOE: {
      const int D = m->D;
      q[0] = c[0];
      for (int d = 0; d < D; ++d) q[1 + d] = c[1 + d];
      for (int i = D + 1; i < 2 * D + 3; ++i) {
        if (!(c[i] > 0)) return 1;
        q[i] = std::log(c[i]);
      }
      return 0;
    }
  }
  return 1;
}

}  // extern "C"
