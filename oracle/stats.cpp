// Oracle summary statistics -- TEST INFRASTRUCTURE ONLY.
//
// Restates what src/cmdstan/stansummary_helper.hpp:397-428 obtains from
// stan::mcmc::chainset (absent from the reference tree):
//   mean, MCSE of the mean, SD, MAD, quantiles, split rank-normalized
//   bulk / tail ESS and R-hat = max(bulk, tail)  (stansummary_helper.hpp:423-425).
// The published method is Vehtari, Gelman, Simpson, Carpenter & Buerkner
// (2021), "Rank-normalization, folding, and localization: an improved R-hat",
// with Geyer's initial-positive / initial-monotone sequence truncation.
// Pinned to the goldens of src/test/interface/stansummary_test.cpp:481-495
// (bernoulli) and :622-637 (eight schools).
#include "oracle.h"
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace {

using Vec = std::vector<double>;
using Chains = std::vector<Vec>;

// Inverse standard normal CDF: Acklam's rational approximation followed by
// one Halley refinement step using erfc (full double precision).
double qnorm(double p) {
  static const double a[] = {-3.969683028665376e+01, 2.209460984245205e+02, -2.759285104469687e+02,
                             1.383577518672690e+02, -3.066479806614716e+01, 2.506628277459239e+00};
  static const double b[] = {-5.447609879822406e+01, 1.615858368580409e+02, -1.556989798598866e+02,
                             6.680131188771972e+01, -1.328068155288572e+01};
  static const double c[] = {-7.784894002430293e-03, -3.223964580411365e-01, -2.400758277161838e+00,
                             -2.549732539343734e+00, 4.374664141464968e+00, 2.938163982698783e+00};
  static const double d[] = {7.784695709041462e-03, 3.224671290700398e-01, 2.445134137142996e+00,
                             3.754408661907416e+00};
  if (p <= 0) return -INFINITY;
  if (p >= 1) return INFINITY;
  double x;
  const double pl = 0.02425;
  if (p < pl) {
    double q = std::sqrt(-2 * std::log(p));
    x = (((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
        ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1);
  } else if (p <= 1 - pl) {
    double q = p - 0.5, r = q * q;
    x = (((((a[0] * r + a[1]) * r + a[2]) * r + a[3]) * r + a[4]) * r + a[5]) * q /
        (((((b[0] * r + b[1]) * r + b[2]) * r + b[3]) * r + b[4]) * r + 1);
  } else {
    double q = std::sqrt(-2 * std::log(1 - p));
    x = -(((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
        ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1);
  }
  double e = 0.5 * std::erfc(-x / std::sqrt(2.0)) - p;
  double u = e * std::sqrt(2 * M_PI) * std::exp(x * x / 2);
  x = x - u / (1 + x * u / 2);
  return x;
}

Chains to_chains(const double* x, int M, int N) {
  Chains c(M);
  for (int m = 0; m < M; ++m) c[m].assign(x + (long)m * N, x + (long)(m + 1) * N);
  return c;
}

// split each chain in half; an odd middle draw is dropped
Chains split(const Chains& in) {
  Chains out;
  for (const auto& c : in) {
    size_t n = c.size(), h = n / 2;
    out.emplace_back(c.begin(), c.begin() + h);
    out.emplace_back(c.begin() + (n - h), c.end());
  }
  return out;
}

// pooled ranks with average ties -> normal scores (r - 3/8) / (S + 1/4)
Chains rank_normalize(const Chains& in) {
  std::vector<std::pair<double, size_t>> all;
  size_t S = 0;
  for (const auto& c : in) S += c.size();
  all.reserve(S);
  size_t idx = 0;
  for (const auto& c : in)
    for (double v : c) all.emplace_back(v, idx++);
  std::sort(all.begin(), all.end(), [](auto& a, auto& b) { return a.first < b.first; });
  Vec r(S);
  size_t i = 0;
  while (i < S) {
    size_t j = i;
    while (j + 1 < S && all[j + 1].first == all[i].first) ++j;
    double avg = 0.5 * ((double)(i + 1) + (double)(j + 1));
    for (size_t k = i; k <= j; ++k) r[all[k].second] = avg;
    i = j + 1;
  }
  Chains out = in;
  idx = 0;
  for (auto& c : out)
    for (double& v : c) v = qnorm((r[idx++] - 0.375) / ((double)S + 0.25));
  return out;
}

double mean(const Vec& v) { return std::accumulate(v.begin(), v.end(), 0.0) / v.size(); }
double var(const Vec& v) {
  double m = mean(v), s = 0;
  for (double x : v) s += (x - m) * (x - m);
  return s / (v.size() - 1);
}

// biased autocovariance at lag k (divides by n), matching the FFT estimator
double acov(const Vec& v, double m, size_t k) {
  size_t n = v.size();
  double s = 0;
  for (size_t t = 0; t + k < n; ++t) s += (v[t] - m) * (v[t + k] - m);
  return s / n;
}

double ess_chains(const Chains& ch) {
  const size_t M = ch.size(), N = ch[0].size();
  if (N < 4) return NAN;
  Vec cm(M);
  for (size_t m = 0; m < M; ++m) cm[m] = mean(ch[m]);
  // constant chains
  bool constant = true;
  for (size_t m = 0; m < M && constant; ++m)
    for (double x : ch[m])
      if (x != ch[0][0]) { constant = false; break; }
  if (constant) return NAN;
  auto mean_acov = [&](size_t k) {
    double s = 0;
    for (size_t m = 0; m < M; ++m) s += acov(ch[m], cm[m], k);
    return s / M;
  };
  double a0 = mean_acov(0);
  double mean_var = a0 * N / (N - 1.0);
  double var_plus = mean_var * (N - 1.0) / N;
  if (M > 1) var_plus += var(cm);
  Vec rho(N, 0.0);
  size_t t = 0;
  double rho_even = 1.0;
  double rho_odd = 1.0 - (mean_var - mean_acov(1)) / var_plus;
  rho[0] = rho_even;
  rho[1] = rho_odd;
  // signed bound: with split chains of 4 draws, N - 5 is negative
  while ((long)t < (long)N - 5 && !std::isnan(rho_even + rho_odd) && (rho_even + rho_odd > 0)) {
    t += 2;
    rho_even = 1.0 - (mean_var - mean_acov(t)) / var_plus;
    rho_odd = 1.0 - (mean_var - mean_acov(t + 1)) / var_plus;
    if (rho_even + rho_odd >= 0) {
      rho[t] = rho_even;
      rho[t + 1] = rho_odd;
    }
  }
  size_t max_t = t;
  if (rho_even > 0) rho[max_t] = rho_even;
  // initial monotone sequence
  t = 0;
  while (t + 4 <= max_t) {
    t += 2;
    if (rho[t] + rho[t + 1] > rho[t - 2] + rho[t - 1]) {
      rho[t] = (rho[t - 2] + rho[t - 1]) / 2;
      rho[t + 1] = rho[t];
    }
  }
  double ess = (double)M * N;
  double tau = -1.0;
  for (size_t k = 0; k < max_t; ++k) tau += 2.0 * rho[k];
  tau += rho[max_t];
  tau = std::max(tau, 1.0 / std::log10(ess));
  return ess / tau;
}

double rhat_chains(const Chains& ch) {
  const size_t M = ch.size(), N = ch[0].size();
  Vec cm(M), cv(M);
  for (size_t m = 0; m < M; ++m) { cm[m] = mean(ch[m]); cv[m] = var(ch[m]); }
  double vb = N * var(cm);
  double vw = mean(cv);
  return std::sqrt((vb / vw + N - 1.0) / N);
}

// R type-7 quantile of pooled draws
double quantile(Vec v, double p) {
  std::sort(v.begin(), v.end());
  double h = (v.size() - 1) * p;
  size_t lo = (size_t)std::floor(h);
  size_t hi = std::min(lo + 1, v.size() - 1);
  return v[lo] + (h - lo) * (v[hi] - v[lo]);
}

Vec pool(const Chains& c) {
  Vec v;
  for (auto& x : c) v.insert(v.end(), x.begin(), x.end());
  return v;
}

double ess_tail_of(const Chains& ch) {
  Vec all = pool(ch);
  double q05 = quantile(all, 0.05), q95 = quantile(all, 0.95);
  Chains i05 = ch, i95 = ch;
  for (auto& c : i05) for (double& v : c) v = v <= q05 ? 1.0 : 0.0;
  for (auto& c : i95) for (double& v : c) v = v <= q95 ? 1.0 : 0.0;
  double e1 = ess_chains(split(i05)), e2 = ess_chains(split(i95));
  return std::min(e1, e2);
}

double rhat_of(const Chains& ch) {
  double bulk = rhat_chains(rank_normalize(split(ch)));
  Vec all = pool(ch);
  double med = quantile(all, 0.5);
  Chains f = ch;
  for (auto& c : f) for (double& v : c) v = std::fabs(v - med);
  double tail = rhat_chains(rank_normalize(split(f)));
  return std::max(bulk, tail);
}

}  // namespace

extern "C" {

double orc_ess_bulk(const double* x, int M, int N) {
  return ess_chains(rank_normalize(split(to_chains(x, M, N))));
}
double orc_ess_tail(const double* x, int M, int N) { return ess_tail_of(to_chains(x, M, N)); }
double orc_ess_basic(const double* x, int M, int N) { return ess_chains(split(to_chains(x, M, N))); }
double orc_rhat(const double* x, int M, int N) { return rhat_of(to_chains(x, M, N)); }

void orc_summary(const double* x, int M, int N, const double* probs, int n_probs, double* out) {
  Chains ch = to_chains(x, M, N);
  Vec all = pool(ch);
  double mu = mean(all), sd = std::sqrt(var(all));
  // MCSE uses the ESS of the raw, unsplit chains (pinned by the goldens)
  double ess_mean = ess_chains(ch);
  out[0] = mu;
  out[1] = sd / std::sqrt(ess_mean);
  out[2] = sd;
  double med = quantile(all, 0.5);
  Vec dev(all.size());
  for (size_t i = 0; i < all.size(); ++i) dev[i] = std::fabs(all[i] - med);
  out[3] = 1.4826 * quantile(dev, 0.5);
  for (int k = 0; k < n_probs; ++k) out[4 + k] = quantile(all, probs[k]);
  out[4 + n_probs] = orc_ess_bulk(x, M, N);
  out[5 + n_probs] = ess_tail_of(ch);
  out[6 + n_probs] = rhat_of(ch);
}

}  // extern "C"
