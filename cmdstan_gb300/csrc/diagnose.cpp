// Diagnostic checks of a NUTS run: the checks of CmdStan's bin/diagnose
// (src/cmdstan/diagnose.cpp:84-221) over draws already in memory, so that a
// run of thousands of chains is checked without writing and re-reading CSV
// files.  The report text is the reference's, line for line, since users and
// scripts read it.
//
//   treedepth    transitions with treedepth__ >= max_depth (diagnose.cpp:84-110)
//   divergences  sum of divergent__ (:111-128)
//   E-BFMI       mean squared successive difference of energy__ over the
//                draws of all chains taken chain after chain, divided by
//                their pooled sample variance; below 0.3 is reported (:129-157)
//   ESS          min(bulk, tail) split rank-normalized ESS per draw < 0.001 (:158-163)
//   R-hat        max(bulk, tail) split rank-normalized R-hat > 1.01499 (:12, :165-168)
// ESS and R-hat come from the stansummary statistics (gnuts_summary_columns
// on host threads, or gnuts_summary_columns_gpu: one CTA per quantity).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "internal.h"

namespace {

constexpr double RHAT_MAX = 1.01499;  // reported as 1.01
constexpr double EBFMI_MIN = 0.3;
constexpr double ESS_PER_DRAW_MIN = 0.001;

std::string fixed2(double v) {
  char b[64];
  std::snprintf(b, sizeof b, "%.2f", v);
  return b;
}

// Stan CSV column names carry indices after dots ("mu.1", "Sigma.2.3"); the
// CSV reader reports them in bracket form ("mu[1]", "Sigma[2,3]")
std::string bracket_name(const std::string& n) {
  const size_t d = n.find('.');
  if (d == std::string::npos || d == 0) return n;
  std::string s = n.substr(0, d) + "[";
  for (size_t i = d + 1; i < n.size(); ++i) s += n[i] == '.' ? ',' : n[i];
  return s + "]";
}

std::string join(const std::vector<std::string>& v) {
  std::string s;
  for (size_t i = 0; i < v.size(); ++i) s += (i ? ", " : "") + v[i];
  return s;
}

}  // namespace

extern "C" {

int gnuts_diagnose(const double* draws, int n_chains, int n_iter, int64_t stride_chain, int64_t stride_iter,
                   int treedepth_col, int divergent_col, int energy_col, const int* param_cols, int n_params,
                   const char* param_names, int max_depth, int use_gpu, int n_threads, char* report,
                   size_t report_cap, gnuts_diagnosis* result) {
  if (!draws || n_chains < 1 || n_iter < 4 || n_params < 0 || (n_params > 0 && !param_cols))
    return gnuts::api_fail(GNUTS_ERR_ARGUMENT, "gnuts_diagnose: needs draws of at least one chain of 4 iterations");
  std::vector<std::string> names;
  {
    const char* p = param_names ? param_names : "";
    for (int i = 0; i < n_params; ++i) {
      const char* e = std::strchr(p, '\n');
      names.emplace_back(bracket_name(e ? std::string(p, e) : std::string(p)));
      p = e ? e + 1 : p + std::strlen(p);
      if (names.back().empty()) names.back() = "param" + std::to_string(i + 1);
    }
  }
  auto at = [&](int c, int i, int col) { return draws[c * stride_chain + i * stride_iter + col]; };
  const long total = (long)n_chains * n_iter;
  gnuts_diagnosis r{};
  std::string out;
  bool problems = false;
  if (treedepth_col >= 0) {
    out += "Checking sampler transitions treedepth.\n";
    long n_max = 0;
    for (int c = 0; c < n_chains; ++c)
      for (int i = 0; i < n_iter; ++i) n_max += at(c, i, treedepth_col) >= max_depth;
    r.n_treedepth_max = n_max;
    if (n_max > 0) {
      problems = true;
      out += std::to_string(n_max) + " of " + std::to_string(total) + " (" + fixed2(100.0 * n_max / total) +
             "%) transitions hit the maximum treedepth limit of " + std::to_string(max_depth) + ", or 2^" +
             std::to_string(max_depth) + " leapfrog steps.\n" +
             "Trajectories that are prematurely terminated due to this limit will result in slow exploration.\n"
             "For optimal performance, increase this limit.\n\n";
    } else {
      out += "Treedepth satisfactory for all transitions.\n\n";
    }
  }
  if (divergent_col >= 0) {
    out += "Checking sampler transitions for divergences.\n";
    double sum = 0;
    for (int c = 0; c < n_chains; ++c)
      for (int i = 0; i < n_iter; ++i) sum += at(c, i, divergent_col);
    const long n_div = (long)sum;
    r.n_divergent = n_div;
    if (n_div > 0) {
      problems = true;
      out += std::to_string(n_div) + " of " + std::to_string(total) + " (" + fixed2(100.0 * n_div / total) +
             "%) transitions ended with a divergence.\n"
             "These divergent transitions indicate that HMC is not fully able to explore the posterior "
             "distribution.\n"
             "Try increasing adapt delta closer to 1.\n"
             "If this doesn't remove all divergences, try to reparameterize the model.\n\n";
    } else {
      out += "No divergent transitions found.\n\n";
    }
  }
  r.e_bfmi = NAN;
  if (energy_col >= 0) {
    out += "Checking E-BFMI - sampler transitions HMC potential energy.\n";
    // running mean of the squared successive differences (chain after chain,
    // as the draws are stored), pooled sample variance
    double msq = 0, prev = at(0, 0, energy_col), mean = 0;
    long k = 0;
    for (int c = 0; c < n_chains; ++c)
      for (int i = 0; i < n_iter; ++i) {
        const double e = at(c, i, energy_col);
        mean += e;
        if (c == 0 && i == 0) continue;
        ++k;
        msq += ((e - prev) * (e - prev) - msq) / (double)k;
        prev = e;
      }
    mean /= (double)total;
    double var = 0;
    for (int c = 0; c < n_chains; ++c)
      for (int i = 0; i < n_iter; ++i) {
        const double d = at(c, i, energy_col) - mean;
        var += d * d;
      }
    var /= (double)(total - 1);
    r.e_bfmi = msq / var;
    if (r.e_bfmi < EBFMI_MIN) {
      problems = true;
      out += "The E-BFMI, " + fixed2(r.e_bfmi) + ", is below the nominal threshold of " + fixed2(EBFMI_MIN) +
             " which suggests that HMC may have trouble exploring the target distribution.\n"
             "If possible, try to reparameterize the model.\n\n";
    } else {
      out += "E-BFMI satisfactory.\n\n";
    }
  }
  std::vector<std::string> bad_ess, bad_rhat;
  if (n_params > 0) {
    std::vector<double> st((size_t)n_params * 7);
    int rc = use_gpu ? gnuts_summary_columns_gpu(draws, n_chains, n_iter, n_params, stride_chain, stride_iter,
                                                 param_cols, nullptr, 0, st.data())
                     : gnuts_summary_columns(draws, n_chains, n_iter, n_params, stride_chain, stride_iter,
                                             param_cols, nullptr, 0, n_threads, st.data());
    if (rc) return gnuts::api_fail(rc, "gnuts_diagnose: the ESS / R-hat statistics failed");
    for (int j = 0; j < n_params; ++j) {
      const double* s = st.data() + (size_t)j * 7;  // mean, mcse, sd, mad, ess_bulk, ess_tail, rhat
      const double n_eff = s[4] < s[5] ? s[4] : s[5];
      if (n_eff / (double)total < ESS_PER_DRAW_MIN) bad_ess.push_back(names[j]);
      if (s[6] > RHAT_MAX) bad_rhat.push_back(names[j]);
    }
  }
  r.n_low_ess = (int)bad_ess.size();
  r.n_high_rhat = (int)bad_rhat.size();
  if (!bad_ess.empty()) {
    problems = true;
    out += "The following parameters had fewer than 0.001 effective draws per transition:\n  " + join(bad_ess) +
           "\nSuch low values indicate that the effective sample size estimators may be biased high and actual "
           "performance may be substantially lower than quoted.\n\n";
  } else {
    out += "Rank-normalized split effective sample size satisfactory for all parameters.\n\n";
  }
  if (!bad_rhat.empty()) {
    problems = true;
    out += "The following parameters had rank-normalized split R-hat greater than " + fixed2(RHAT_MAX) + ":\n  " +
           join(bad_rhat) +
           "\nSuch high values indicate incomplete mixing and biased estimation.\n"
           "You should consider regularizating your model with additional prior information or a more effective "
           "parameterization.\n\n";
  } else {
    out += "Rank-normalized split R-hat values satisfactory for all parameters.\n\n";
  }
  out += problems ? "Processing complete.\n" : "Processing complete, no problems detected.\n";
  r.has_problems = problems ? 1 : 0;
  if (result) *result = r;
  if (report && report_cap > 0) {
    const size_t n = out.size() < report_cap - 1 ? out.size() : report_cap - 1;
    std::memcpy(report, out.data(), n);
    report[n] = 0;
    if (out.size() >= report_cap)
      return gnuts::api_fail(GNUTS_ERR_ARGUMENT, "gnuts_diagnose: report buffer too small (" +
                                                      std::to_string(out.size() + 1) + " bytes needed)");
  }
  return GNUTS_OK;
}

}  // extern "C"
