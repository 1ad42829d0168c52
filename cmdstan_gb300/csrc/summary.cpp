// stansummary statistics for the sampler's draws (host C++).
//
// Replaces what src/cmdstan/stansummary_helper.hpp:397-428 obtains from
// stan::mcmc::chainset (absent from the reference tree): mean, MCSE of the
// mean, SD, MAD, quantiles, split rank-normalized bulk / tail ESS and
// R-hat = max(bulk, tail) (stansummary_helper.hpp:423-425).  Method:
// Vehtari, Gelman, Simpson, Carpenter & Buerkner (2021) with Geyer's
// initial-positive / initial-monotone sequence truncation; inverse normal CDF
// by Wichura's algorithm AS241 (PPND16).  The MCSE of the mean uses the ESS
// of the raw, unsplit chains, which is what the reference's goldens imply.
// Columns are processed on several host threads.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <utility>
#include <thread>
#include <vector>
#include "../../include/gnuts.h"

namespace {

// Wichura, "Algorithm AS 241: The percentage points of the normal
// distribution", Applied Statistics 37 (1988), PPND16.
double ppnd16(double p) {
  const double q = p - 0.5;
  if (std::fabs(q) <= 0.425) {
    const double r = 0.180625 - q * q;
    return q *
           (((((((2509.0809287301226727 * r + 33430.575583588128105) * r + 67265.770927008700853) * r +
                45921.953931549871457) * r + 13731.693765509461125) * r + 1971.5909503065514427) * r +
             133.14166789178437745) * r + 3.387132872796366608) /
           (((((((5226.495278852545925 * r + 28729.085735721942674) * r + 39307.89580009271061) * r +
                21213.794301586595867) * r + 5394.1960214247511077) * r + 687.1870074920579083) * r +
             42.313330701600911252) * r + 1.0);
  }
  double r = q < 0 ? p : 1.0 - p;
  if (r <= 0) return q < 0 ? -INFINITY : INFINITY;
  r = std::sqrt(-std::log(r));
  double v;
  if (r <= 5.0) {
    r -= 1.6;
    v = (((((((7.7454501427834140764e-4 * r + 0.0227238449892691845833) * r + 0.24178072517745061177) * r +
             1.27045825245236838258) * r + 3.64784832476320460504) * r + 5.7694972214606914055) * r +
          4.6303378461565452959) * r + 1.42343711074968357734) /
        (((((((1.05075007164441684324e-9 * r + 5.475938084995344946e-4) * r + 0.0151986665636164571966) * r +
             0.14810397642748007459) * r + 0.68976733498510000455) * r + 1.6763848301838038494) * r +
          2.05319162663775882187) * r + 1.0);
  } else {
    r -= 5.0;
    v = (((((((2.01033439929228813265e-7 * r + 2.71155556874348757815e-5) * r + 0.0012426609473880784386) * r +
             0.026532189526576123093) * r + 0.29656057182850489123) * r + 1.7848265399172913358) * r +
          5.4637849111641143699) * r + 6.6579046435011037772) /
        (((((((2.04426310338993978564e-15 * r + 1.4215117583164458887e-7) * r + 1.8463183175100546818e-5) * r +
             7.868691311456132591e-4) * r + 0.0148753612908506148525) * r + 0.13692988092273580531) * r +
          0.59983220655588793769) * r + 1.0);
  }
  return q < 0 ? -v : v;
}

// M sequences of equal length n stored contiguously: seq m = data[m*n .. m*n+n)
struct Seqs {
  int M, n;
  std::vector<double> data;
  const double* at(int m) const { return data.data() + (size_t)m * n; }
};

double mean_of(const double* x, int n) {
  double s = 0;
  for (int i = 0; i < n; ++i) s += x[i];
  return s / n;
}
double var_of(const double* x, int n, double m) {
  double s = 0;
  for (int i = 0; i < n; ++i) s += (x[i] - m) * (x[i] - m);
  return s / (n - 1);
}

// effective sample size of M sequences (Geyer truncation, antithetic guard)
double ess_of(const Seqs& S) {
  const int M = S.M, n = S.n;
  if (n < 4) return NAN;
  std::vector<double> cm(M);
  bool constant = true;
  const double first = S.data[0];
  for (int m = 0; m < M; ++m) {
    cm[m] = mean_of(S.at(m), n);
    for (int i = 0; i < n && constant; ++i) constant = S.at(m)[i] == first;
  }
  if (constant) return NAN;
  // mean over sequences of the biased autocovariance at lag k, computed on demand
  std::vector<double> acov_cache;
  auto acov = [&](int k) -> double {
    while ((int)acov_cache.size() <= k) {
      const int kk = (int)acov_cache.size();
      double tot = 0;
      for (int m = 0; m < M; ++m) {
        const double* x = S.at(m);
        const double mu = cm[m];
        double s = 0;
        for (int t = 0; t + kk < n; ++t) s += (x[t] - mu) * (x[t + kk] - mu);
        tot += s / n;
      }
      acov_cache.push_back(tot / M);
    }
    return acov_cache[k];
  };
  const double mean_var = acov(0) * n / (n - 1.0);
  double var_plus = mean_var * (n - 1.0) / n;
  if (M > 1) var_plus += var_of(cm.data(), M, mean_of(cm.data(), M));
  std::vector<double> rho(n + 2, 0.0);
  auto rho_at = [&](int k) { return 1.0 - (mean_var - acov(k)) / var_plus; };
  int t = 0;
  double even = 1.0, odd = rho_at(1);
  rho[0] = even;
  rho[1] = odd;
  while (t < n - 5 && !std::isnan(even + odd) && even + odd > 0) {
    t += 2;
    even = rho_at(t);
    odd = rho_at(t + 1);
    if (even + odd >= 0) {
      rho[t] = even;
      rho[t + 1] = odd;
    }
  }
  const int max_t = t;
  if (even > 0) rho[max_t] = even;
  for (int u = 2; u <= max_t - 2; u += 2) {
    const double prev = rho[u - 2] + rho[u - 1];
    if (rho[u] + rho[u + 1] > prev) {
      rho[u] = prev / 2;
      rho[u + 1] = rho[u];
    }
  }
  double tau = -1.0 + rho[max_t];
  for (int k = 0; k < max_t; ++k) tau += 2.0 * rho[k];
  const double total = (double)M * n;
  tau = std::max(tau, 1.0 / std::log10(total));
  return total / tau;
}

double rhat_of(const Seqs& S) {
  const int M = S.M, n = S.n;
  std::vector<double> cm(M), cv(M);
  for (int m = 0; m < M; ++m) {
    cm[m] = mean_of(S.at(m), n);
    cv[m] = var_of(S.at(m), n, cm[m]);
  }
  const double between = n * var_of(cm.data(), M, mean_of(cm.data(), M));
  const double within = mean_of(cv.data(), M);
  return std::sqrt((between / within + n - 1.0) / n);
}

// type-7 quantile of sorted values
double quantile_sorted(const std::vector<double>& s, double p) {
  const double h = (s.size() - 1) * p;
  const size_t lo = (size_t)std::floor(h);
  const size_t hi = std::min(lo + 1, s.size() - 1);
  return s[lo] + (h - lo) * (s[hi] - s[lo]);
}

Seqs split_of(const Seqs& in) {
  const int h = in.n / 2;
  Seqs out{2 * in.M, h, std::vector<double>((size_t)2 * in.M * h)};
  for (int m = 0; m < in.M; ++m) {
    const double* x = in.at(m);
    std::copy(x, x + h, out.data.begin() + (size_t)(2 * m) * h);
    std::copy(x + (in.n - h), x + in.n, out.data.begin() + (size_t)(2 * m + 1) * h);
  }
  return out;
}

// normal scores of pooled ranks (average ranks for ties).  The draws are
// sorted as contiguous (value, position) pairs: the order among equal values
// does not matter, since tied draws share the mean of their ranks.
// When sorted_out is given it receives the sorted values.
Seqs zscale(const Seqs& in, std::vector<double>* sorted_out = nullptr) {
  const size_t S = in.data.size();
  std::vector<std::pair<double, uint32_t>> vi(S);
  for (size_t k = 0; k < S; ++k) vi[k] = {in.data[k], (uint32_t)k};
  std::sort(vi.begin(), vi.end(),
            [](const std::pair<double, uint32_t>& a, const std::pair<double, uint32_t>& b) { return a.first < b.first; });
  if (sorted_out) {
    sorted_out->resize(S);
    for (size_t k = 0; k < S; ++k) (*sorted_out)[k] = vi[k].first;
  }
  Seqs out = in;
  size_t i = 0;
  while (i < S) {
    size_t j = i + 1;
    while (j < S && vi[j].first == vi[i].first) ++j;
    const double rank = 0.5 * (double)(i + 1 + j);  // mean of ranks i+1 .. j
    const double z = ppnd16((rank - 0.375) / ((double)S + 0.25));
    for (size_t k = i; k < j; ++k) out.data[vi[k].second] = z;
    i = j;
  }
  return out;
}

// type-7 median of v (reordered in place) from its two order statistics
double median_select(std::vector<double>& v) {
  const double h = (v.size() - 1) * 0.5;
  const size_t lo = (size_t)std::floor(h);
  const size_t hi = std::min(lo + 1, v.size() - 1);
  std::nth_element(v.begin(), v.begin() + lo, v.end());
  const double a = v[lo];
  const double b = hi == lo ? a : *std::min_element(v.begin() + lo + 1, v.end());
  return a + (h - lo) * (b - a);
}

void summarize(const double* x, int M, int n, int64_t sc, int64_t si, const double* probs, int np, double* out) {
  Seqs S{M, n, std::vector<double>((size_t)M * n)};
  for (int m = 0; m < M; ++m)
    for (int i = 0; i < n; ++i) S.data[(size_t)m * n + i] = x[m * sc + i * si];
  // split chains: with an even chain length they hold every draw, so the
  // sort behind their normal scores also gives the pooled sorted values
  const Seqs sp = split_of(S);
  std::vector<double> sorted;
  const Seqs zsp = zscale(sp, n % 2 == 0 ? &sorted : nullptr);
  if (n % 2 != 0) {
    sorted = S.data;
    std::sort(sorted.begin(), sorted.end());
  }
  const double mu = mean_of(S.data.data(), (int)S.data.size());
  const double sd = std::sqrt(var_of(S.data.data(), (int)S.data.size(), mu));
  const double med = quantile_sorted(sorted, 0.5);
  std::vector<double> dev(S.data.size());
  for (size_t i = 0; i < dev.size(); ++i) dev[i] = std::fabs(S.data[i] - med);
  out[0] = mu;
  out[1] = sd / std::sqrt(ess_of(S));
  out[2] = sd;
  out[3] = 1.4826 * median_select(dev);
  for (int k = 0; k < np; ++k) out[4 + k] = quantile_sorted(sorted, probs[k]);
  out[4 + np] = ess_of(zsp);
  // tail ESS: indicators of the 5% and 95% quantiles
  const double q05 = quantile_sorted(sorted, 0.05), q95 = quantile_sorted(sorted, 0.95);
  Seqs i05 = sp, i95 = sp;
  for (double& v : i05.data) v = v <= q05 ? 1.0 : 0.0;
  for (double& v : i95.data) v = v <= q95 ? 1.0 : 0.0;
  out[5 + np] = std::min(ess_of(i05), ess_of(i95));
  // R-hat: bulk on ranks, tail on ranks of |x - median|
  Seqs fold = sp;
  for (double& v : fold.data) v = std::fabs(v - med);
  out[6 + np] = std::max(rhat_of(zsp), rhat_of(zscale(fold)));
}

}  // namespace

extern "C" {

int gnuts_summary(const double* x, int n_chains, int n_iter, int64_t stride_chain, int64_t stride_iter,
                  const double* probs, int n_probs, double* out) {
  if (!x || !out || n_chains < 1 || n_iter < 2 || n_probs < 0 || (n_probs > 0 && !probs)) return GNUTS_ERR_ARGUMENT;
  summarize(x, n_chains, n_iter, stride_chain, stride_iter, probs, n_probs, out);
  return GNUTS_OK;
}

int gnuts_summary_columns(const double* draws, int n_chains, int n_iter, int n_cols, int64_t stride_chain,
                          int64_t stride_iter, const int* cols, const double* probs, int n_probs, int n_threads,
                          double* out) {
  if (!draws || !out || !cols || n_chains < 1 || n_iter < 2 || n_cols < 0) return GNUTS_ERR_ARGUMENT;
  if (n_threads < 1) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int j; (j = next.fetch_add(1)) < n_cols;)
      summarize(draws + cols[j], n_chains, n_iter, stride_chain, stride_iter, probs, n_probs,
                out + (size_t)j * (7 + n_probs));
  };
  std::vector<std::thread> th;
  for (int t = 0; t < std::min(n_threads, n_cols); ++t) th.emplace_back(work);
  for (auto& t : th) t.join();
  return GNUTS_OK;
}

}  // extern "C"
