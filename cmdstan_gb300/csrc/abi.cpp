// C-ABI entry points (include/gnuts.h): model registry, Stan-JSON data
// reader, argument validation and the hmc_nuts_* service wrappers.
//
// Error behaviour follows CmdStan: every failure returns a non-zero code and
// a message (command.hpp:110-118 for argument errors, :569-574 for adapt
// with num_warmup = 0, services' init failures -> NOT_OK).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "internal.h"

namespace gnuts {

Model::~Model() {
  for (void* p : device_allocs) cudaFree(p);
}

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
}  // namespace

int api_fail(int code, const std::string& msg) { return fail(code, msg); }

int validate_args(const Model& m, const gnuts_sample_args* a, int adapt, int metric);

namespace {

// ---------------------------------------------------------------- var context
struct Var {
  bool is_int = true;
  std::vector<int64_t> dims;
  std::vector<double> values;
};
using VarMap = std::map<std::string, Var>;

// Minimal Stan JSON reader (stan::json::json_data restated): an object of
// name -> number | (nested) array of numbers; "inf"/"Infinity"/"-inf"/"NaN"
// are accepted as strings or bare words.  Arrays are row-major.
struct JsonReader {
  const char* p;
  const char* end;
  explicit JsonReader(const std::string& s) : p(s.data()), end(s.data() + s.size()) {}
  void ws() {
    while (p < end && std::isspace((unsigned char)*p)) ++p;
  }
  [[noreturn]] void error(const std::string& m) { throw std::runtime_error("JSON data: " + m); }
  std::string str() {
    if (*p != '"') error("expected string");
    ++p;
    std::string s;
    while (p < end && *p != '"') {
      if (*p == '\\' && p + 1 < end) ++p;
      s += *p++;
    }
    if (p >= end) error("unterminated string");
    ++p;
    return s;
  }
  bool special(const std::string& w, double& v) {
    std::string l = w;
    std::transform(l.begin(), l.end(), l.begin(), ::tolower);
    if (l == "inf" || l == "infinity" || l == "+inf" || l == "+infinity") { v = INFINITY; return true; }
    if (l == "-inf" || l == "-infinity") { v = -INFINITY; return true; }
    if (l == "nan") { v = NAN; return true; }
    return false;
  }
  void number(Var& v) {
    ws();
    double x;
    if (*p == '"') {
      std::string s = str();
      if (!special(s, x)) error("bad numeric string '" + s + "'");
      v.is_int = false;
      v.values.push_back(x);
      return;
    }
    const char* b = p;
    while (p < end && (std::isalnum((unsigned char)*p) || *p == '-' || *p == '+' || *p == '.')) ++p;
    std::string tok(b, p);
    if (tok.empty()) error("expected number");
    if (special(tok, x)) {
      v.is_int = false;
    } else {
      char* e = nullptr;
      x = std::strtod(tok.c_str(), &e);
      if (*e) error("bad number '" + tok + "'");
      if (tok.find_first_of(".eE") != std::string::npos) v.is_int = false;
    }
    v.values.push_back(x);
  }
  // returns the extents of this (sub)array
  std::vector<int64_t> array(Var& v) {
    ws();
    if (*p != '[') {
      number(v);
      return {};
    }
    ++p;
    ws();
    std::vector<int64_t> inner;
    int64_t n = 0;
    bool first = true;
    if (*p == ']') {
      ++p;
      return {0};
    }
    while (true) {
      std::vector<int64_t> d = array(v);
      if (first) inner = d;
      else if (d != inner) error("ragged array");
      first = false;
      ++n;
      ws();
      if (*p == ',') { ++p; continue; }
      if (*p == ']') { ++p; break; }
      error("expected , or ]");
    }
    std::vector<int64_t> out{n};
    out.insert(out.end(), inner.begin(), inner.end());
    return out;
  }
  VarMap parse() {
    VarMap m;
    ws();
    if (p >= end) return m;
    if (*p != '{') error("expected object");
    ++p;
    ws();
    if (*p == '}') return m;
    while (true) {
      ws();
      std::string name = str();
      ws();
      if (*p != ':') error("expected :");
      ++p;
      Var v;
      v.dims = array(v);
      m[name] = std::move(v);
      ws();
      if (*p == ',') { ++p; continue; }
      if (*p == '}') { ++p; break; }
      error("expected , or }");
    }
    return m;
  }
};

VarMap vars_from_abi(const gnuts_var* vars, int n) {
  VarMap m;
  for (int i = 0; i < n; ++i) {
    const gnuts_var& g = vars[i];
    if (!g.name) throw std::runtime_error("variable without a name");
    Var v;
    v.is_int = g.type == GNUTS_VAR_INT;
    int64_t count = 1;
    for (int k = 0; k < g.ndim; ++k) {
      if (g.dims[k] < 0) throw std::runtime_error(std::string("negative extent for ") + g.name);
      v.dims.push_back(g.dims[k]);
      count *= g.dims[k];
    }
    v.values.resize(count);
    if (count && !g.data) throw std::runtime_error(std::string("no data for ") + g.name);
    for (int64_t k = 0; k < count; ++k)
      v.values[k] = v.is_int ? (double)((const int32_t*)g.data)[k] : ((const double*)g.data)[k];
    m[g.name] = std::move(v);
  }
  return m;
}

const Var& need(const VarMap& m, const std::string& name) {
  auto it = m.find(name);
  if (it == m.end()) throw std::runtime_error("variable does not exist; processing stage=data initialization; variable name=" + name);
  return it->second;
}
int64_t need_int(const VarMap& m, const std::string& name) {
  const Var& v = need(m, name);
  if (!v.dims.empty() || v.values.size() != 1) throw std::runtime_error("variable " + name + " must be a scalar");
  if (!v.is_int) throw std::runtime_error("variable " + name + " must be an integer");
  return (int64_t)v.values[0];
}
double need_real(const VarMap& m, const std::string& name, double dflt, bool optional) {
  auto it = m.find(name);
  if (it == m.end()) {
    if (optional) return dflt;
    throw std::runtime_error("variable does not exist; variable name=" + name);
  }
  if (it->second.values.size() != 1) throw std::runtime_error("variable " + name + " must be a scalar");
  return it->second.values[0];
}
void check_dims(const Var& v, const std::string& name, std::vector<int64_t> dims) {
  if (v.dims != dims) {
    std::string want, got;
    for (auto d : dims) want += "[" + std::to_string(d) + "]";
    for (auto d : v.dims) got += "[" + std::to_string(d) + "]";
    throw std::runtime_error("mismatch in dimension declared and found in context; variable name=" + name +
                             "; declared dims=" + want + "; found dims=" + got);
  }
}

std::string idx_name(const std::string& base, int i) { return base + "." + std::to_string(i); }

// --------------------------------------------------------------- model build
struct HostData {
  std::vector<int> yi, group, gstart;
  std::vector<double> yr, X, sigma, scales;
};

struct ModelImpl : Model {
  HostData hd;
};

ModelImpl* build_model(const std::string& id, const VarMap& vm) {
  auto m = std::make_unique<ModelImpl>();
  m->id = id;
  DevModel& d = m->dev;
  HostData& h = m->hd;
  auto ints01 = [&](const Var& v, const std::string& name) {
    std::vector<int> out(v.values.size());
    for (size_t i = 0; i < out.size(); ++i) {
      double x = v.values[i];
      if (!(x == 0 || x == 1)) throw std::runtime_error(name + " is " + std::to_string(x) + ", but must be in the interval [0, 1]");
      out[i] = (int)x;
    }
    if (!v.is_int) throw std::runtime_error(name + " must be an integer array");
    return out;
  };
  if (id == "bernoulli") {
    d.kind = MK_BERNOULLI;
    int64_t N = need_int(vm, "N");
    if (N < 0) throw std::runtime_error("N is " + std::to_string(N) + ", but must be greater than or equal to 0");
    const Var& y = need(vm, "y");
    check_dims(y, "y", {N});
    h.yi = ints01(y, "y");
    d.N = (int)N;
    d.ysum = std::accumulate(h.yi.begin(), h.yi.end(), 0);
    d.D = 1;
    d.ncon = 1;
    m->name = "bernoulli_model";
    m->con_names = {"theta"};
  } else if (id == "normal" || id == "proper" || id == "test_model") {
    d.kind = MK_NORMAL;
    if (id == "proper") h.scales = {1.0};
    else if (id == "test_model") h.scales = {10.0, 1.0};
    else {
      auto it = vm.find("scales");
      if (it == vm.end()) h.scales = {1.0};
      else h.scales = it->second.values;
    }
    for (double s : h.scales)
      if (!(s > 0)) throw std::runtime_error("scales must be positive");
    d.K = (int)h.scales.size();
    d.D = d.K;
    d.ncon = d.K;
    if (id == "proper") { m->name = "proper_model"; m->con_names = {"mu"}; }
    else if (id == "test_model") { m->name = "test_model_model"; m->con_names = {"mu1", "mu2"}; }
    else {
      m->name = "normal_model";
      for (int k = 1; k <= d.K; ++k) m->con_names.push_back(idx_name("x", k));
    }
  } else if (id == "logistic") {
    d.kind = MK_LOGISTIC;
    int64_t N = need_int(vm, "N");
    int64_t K = vm.count("D") ? need_int(vm, "D") : need_int(vm, "K");
    if (N < 0 || K < 1) throw std::runtime_error("bad N or D");
    const Var& X = need(vm, "X");
    check_dims(X, "X", {N, K});
    const Var& y = need(vm, "y");
    check_dims(y, "y", {N});
    h.X = X.values;
    h.yi = ints01(y, "y");
    d.N = (int)N;
    d.K = (int)K;
    d.D = (int)K + 1;
    d.ncon = d.D;
    m->name = "logistic_model";
    m->con_names.push_back("alpha");
    for (int k = 1; k <= K; ++k) m->con_names.push_back(idx_name("beta", k));
  } else if (id == "hier") {
    d.kind = MK_HIER;
    int64_t J = need_int(vm, "J");
    if (J < 0) throw std::runtime_error("J must be >= 0");
    const Var& y = need(vm, "y");
    check_dims(y, "y", {J});
    const Var& s = need(vm, "sigma");
    check_dims(s, "sigma", {J});
    for (double v : s.values)
      if (!(v >= 0)) throw std::runtime_error("sigma must be >= 0");
    h.yr = y.values;
    h.sigma = s.values;
    d.J = (int)J;
    d.D = (int)J + 2;
    d.ncon = d.D;
    m->name = "hier_model";
    m->con_names.push_back("mu");
    for (int j = 1; j <= J; ++j) m->con_names.push_back(idx_name("theta", j));
    m->con_names.push_back("tau");
  } else if (id == "funnel") {
    d.kind = MK_FUNNEL;
    int64_t K = vm.count("K") ? need_int(vm, "K") : 100;
    if (K < 0) throw std::runtime_error("K must be >= 0");
    d.K = (int)K;
    d.D = (int)K + 1;
    d.ncon = d.D;
    m->name = "funnel_model";
    m->con_names.push_back("v");
    for (int k = 1; k <= K; ++k) m->con_names.push_back(idx_name("x", k));
  } else if (id == "varint") {
    d.kind = MK_VARINT;
    int64_t N = need_int(vm, "N"), J = need_int(vm, "J"), K = need_int(vm, "K");
    if (N < 0 || J < 1 || K < 0 || K > 16) throw std::runtime_error("varint needs N >= 0, J >= 1, 0 <= K <= 16");
    const Var& g = need(vm, "group");
    check_dims(g, "group", {N});
    const Var& X = need(vm, "X");
    check_dims(X, "X", {N, K});
    const Var& y = need(vm, "y");
    check_dims(y, "y", {N});
    // rows ordered by group (stable) so each group is one contiguous segment
    std::vector<int> order(N);
    std::iota(order.begin(), order.end(), 0);
    for (int64_t n = 0; n < N; ++n) {
      double gv = g.values[n];
      if (gv < 1 || gv > J || gv != std::floor(gv)) throw std::runtime_error("group must be in 1..J");
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return g.values[a] < g.values[b]; });
    h.group.resize(N);
    h.X.resize(N * K);
    h.yr.resize(N);
    h.gstart.assign(J + 1, 0);
    for (int64_t i = 0; i < N; ++i) {
      int n = order[i];
      h.group[i] = (int)g.values[n];
      for (int64_t k = 0; k < K; ++k) h.X[i * K + k] = X.values[n * K + k];
      h.yr[i] = y.values[n];
      h.gstart[h.group[i]]++;
    }
    for (int64_t j = 1; j <= J; ++j) h.gstart[j] += h.gstart[j - 1];
    d.N = (int)N;
    d.J = (int)J;
    d.K = (int)K;
    d.D = (int)(J + K + 2);
    d.ncon = d.D;
    m->name = "varint_model";
    for (int j = 1; j <= J; ++j) m->con_names.push_back(idx_name("alpha", j));
    for (int k = 1; k <= K; ++k) m->con_names.push_back(idx_name("beta", k));
    m->con_names.push_back("sigma_y");
    m->con_names.push_back("tau");
  } else if (id == "varint_set") {
    // P independent varying-intercept regressions sampled in one launch.
    // Data: P, K, J[P], N[P], group (1-based within its posterior), X
    // [sum N][K], y [sum N]; the rows of posterior p follow those of p - 1.
    // fp32 (default 1) evaluates the likelihood rows in FP32.
    d.kind = MK_VARINT;
    int64_t P = need_int(vm, "P"), K = need_int(vm, "K");
    if (P < 1 || K < 0 || K > 16) throw std::runtime_error("varint_set needs P >= 1 and 0 <= K <= 16");
    const Var& Jv = need(vm, "J");
    check_dims(Jv, "J", {P});
    const Var& Nv = need(vm, "N");
    check_dims(Nv, "N", {P});
    int64_t total = 0;
    for (int64_t p = 0; p < P; ++p) {
      if (Jv.values[p] < 1 || Nv.values[p] < 0) throw std::runtime_error("varint_set needs J[p] >= 1 and N[p] >= 0");
      total += (int64_t)Nv.values[p];
    }
    const Var& g = need(vm, "group");
    check_dims(g, "group", {total});
    const Var& X = need(vm, "X");
    check_dims(X, "X", {total, K});
    const Var& y = need(vm, "y");
    check_dims(y, "y", {total});
    d.fp32 = vm.count("fp32") ? (int)need_int(vm, "fp32") : 1;
    d.alpha_last = 1;
    h.X.resize(total * K);
    h.yr.resize(total);
    h.group.resize(total);
    int64_t row = 0, goff = 0, Jmax = 0;
    for (int64_t p = 0; p < P; ++p) {
      const int64_t J = (int64_t)Jv.values[p], Np = (int64_t)Nv.values[p];
      std::vector<int64_t> order(Np);
      std::iota(order.begin(), order.end(), row);
      for (int64_t n = row; n < row + Np; ++n) {
        const double gv = g.values[n];
        if (gv < 1 || gv > J || gv != std::floor(gv)) throw std::runtime_error("group must be in 1..J[p]");
      }
      std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return g.values[a] < g.values[b]; });
      std::vector<int> gs(J + 1, 0);
      for (int64_t i = 0; i < Np; ++i) {
        const int64_t n = order[i];
        h.group[row + i] = (int)g.values[n];
        for (int64_t k = 0; k < K; ++k) h.X[(row + i) * K + k] = X.values[n * K + k];
        h.yr[row + i] = y.values[n];
        gs[(int)g.values[n]]++;
      }
      for (int64_t j = 1; j <= J; ++j) gs[j] += gs[j - 1];
      h.gstart.insert(h.gstart.end(), gs.begin(), gs.end());
      m->members.push_back({(int)Np, (int)J, (int)(J + K + 2), (long)row, (long)goff});
      row += Np;
      goff += J + 1;
      Jmax = std::max(Jmax, J);
    }
    d.N = (int)total;
    d.J = (int)Jmax;
    d.K = (int)K;
    d.D = (int)(Jmax + K + 2);
    d.ncon = d.D;
    d.n_members = (int)P;
    m->name = "varint_set_model";
    for (int k = 1; k <= K; ++k) m->con_names.push_back(idx_name("beta", k));
    m->con_names.push_back("sigma_y");
    m->con_names.push_back("tau");
    for (int j = 1; j <= Jmax; ++j) m->con_names.push_back(idx_name("alpha", j));
  } else if (id == "horseshoe") {
    d.kind = MK_HORSESHOE;
    int64_t N = need_int(vm, "N");
    int64_t K = vm.count("D") ? need_int(vm, "D") : need_int(vm, "K");
    if (N < 0 || K < 1) throw std::runtime_error("bad N or D");
    const Var& X = need(vm, "X");
    check_dims(X, "X", {N, K});
    const Var& y = need(vm, "y");
    check_dims(y, "y", {N});
    h.X = X.values;
    h.yi = ints01(y, "y");
    d.scale_global = need_real(vm, "scale_global", 0.01, true);
    d.slab_scale = need_real(vm, "slab_scale", 2.0, true);
    d.slab_df = need_real(vm, "slab_df", 4.0, true);
    if (!(d.scale_global > 0 && d.slab_scale > 0 && d.slab_df > 0))
      throw std::runtime_error("scale_global, slab_scale and slab_df must be positive");
    d.N = (int)N;
    d.K = (int)K;
    d.D = 2 * (int)K + 3;
    d.ncon = 3 * (int)K + 3;
    m->name = "horseshoe_model";
    m->con_names.push_back("beta0");
    for (int k = 1; k <= K; ++k) m->con_names.push_back(idx_name("z", k));
    m->con_names.push_back("tau");
    for (int k = 1; k <= K; ++k) m->con_names.push_back(idx_name("lambda", k));
    m->con_names.push_back("caux");
    for (int k = 1; k <= K; ++k) m->con_names.push_back(idx_name("beta", k));
  } else {
    throw std::runtime_error("unknown model '" + id + "'");
  }
  // unconstrained names: same order, constrained ones get their transform spelled out
  m->unc_names.assign(m->con_names.begin(), m->con_names.begin() + d.D);
  d.yi = h.yi.empty() ? nullptr : h.yi.data();
  d.yr = h.yr.empty() ? nullptr : h.yr.data();
  d.X = h.X.empty() ? nullptr : h.X.data();
  d.group = h.group.empty() ? nullptr : h.group.data();
  d.gstart = h.gstart.empty() ? nullptr : h.gstart.data();
  d.sigma = h.sigma.empty() ? nullptr : h.sigma.data();
  d.scales = h.scales.empty() ? nullptr : h.scales.data();
  m->host_X = h.X;
  m->host_yi = h.yi;
  // bf16 exactness of X (the mixed-precision path is exact on X only then)
  bool exact = true;
  for (double x : h.X) {
    float f = (float)x;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((double)f != x || (u & 0xffffu) != 0) { exact = false; break; }
  }
  m->x_bf16_exact = exact;
  return m.release();
}

int create(const std::string& id, const VarMap& vm, gnuts_model** out) {
  try {
    // device upload is deferred to the first device call, so a model can be
    // built, inspected and validated on a host without a GPU
    ModelImpl* m = build_model(id, vm);
    *out = reinterpret_cast<gnuts_model*>(m);
    return GNUTS_OK;
  } catch (const std::exception& e) {
    return fail(GNUTS_ERR_DATA, e.what());
  }
}

Model* M(gnuts_model* m) { return reinterpret_cast<Model*>(m); }
const Model* M(const gnuts_model* m) { return reinterpret_cast<const Model*>(m); }

int validate(const Model& m, const gnuts_sample_args* a, int adapt, int metric) { return validate_args(m, a, adapt, metric); }
}  // namespace

int validate_args(const Model& m, const gnuts_sample_args* a, int adapt, int metric) {
  if (!a) return fail(GNUTS_ERR_ARGUMENT, "no arguments");
  if (a->num_chains < 1) return fail(GNUTS_ERR_ARGUMENT, "num_chains must be >= 1");
  if (a->num_warmup < 0) return fail(GNUTS_ERR_ARGUMENT, "num_warmup must be >= 0");
  if (a->num_samples < 0) return fail(GNUTS_ERR_ARGUMENT, "num_samples must be >= 0");
  if (a->thin < 1) return fail(GNUTS_ERR_ARGUMENT, "thin must be > 0");
  if (!(a->stepsize > 0)) return fail(GNUTS_ERR_ARGUMENT, "stepsize must be > 0");
  if (!(a->stepsize_jitter >= 0 && a->stepsize_jitter <= 1)) return fail(GNUTS_ERR_ARGUMENT, "stepsize_jitter must be in [0, 1]");
  if (a->max_depth < 1 || a->max_depth > 16) return fail(GNUTS_ERR_ARGUMENT, "max_depth must be in 1..16");
  if (!(a->init_radius >= 0)) return fail(GNUTS_ERR_ARGUMENT, "init radius must be >= 0");
  if (adapt) {
    if (a->num_warmup == 0)
      return fail(GNUTS_ERR_ARGUMENT, "The number of warmup samples (num_warmup) must be greater than zero if adaptation is enabled.");
    if (!(a->delta > 0 && a->delta < 1)) return fail(GNUTS_ERR_ARGUMENT, "delta must be in (0, 1)");
    if (!(a->gamma > 0)) return fail(GNUTS_ERR_ARGUMENT, "gamma must be > 0");
    if (!(a->kappa > 0)) return fail(GNUTS_ERR_ARGUMENT, "kappa must be > 0");
    if (!(a->t0 > 0)) return fail(GNUTS_ERR_ARGUMENT, "t0 must be > 0");
  }
  if (a->precision != GNUTS_PRECISION_FP64 && a->precision != GNUTS_PRECISION_MIXED)
    return fail(GNUTS_ERR_ARGUMENT, "unknown precision");
  (void)m;
  (void)metric;
  return GNUTS_OK;
}

namespace {

int service(gnuts_model* mh, const gnuts_sample_args* a, const double* inits, const double* inv_metric,
            gnuts_output* out, gnuts_progress_fn progress, void* ctx, int metric, int adapt) {
  if (!mh) return fail(GNUTS_ERR_ARGUMENT, "null model");
  Model& m = *M(mh);
  int rc = validate(m, a, adapt, metric);
  if (rc) return rc;
  if (inv_metric && metric != 2) {
    const int D = m.dev.D;
    const size_t msz = metric == 1 ? (size_t)D * D : (size_t)D;
    for (size_t i = 0; i < (size_t)a->num_chains * msz; ++i)
      if (!std::isfinite(inv_metric[i])) return fail(GNUTS_ERR_ARGUMENT, "inverse metric has non-finite entries");
    if (metric == 0)
      for (size_t i = 0; i < (size_t)a->num_chains * msz; ++i)
        if (!(inv_metric[i] > 0)) return fail(GNUTS_ERR_ARGUMENT, "diagonal inverse metric must be positive");
  }
  std::string err;
  RunConfig cfg{metric, adapt};
  try {
    rc = run_nuts(m, *a, cfg, inits, metric == 2 ? nullptr : inv_metric, out, progress, ctx, err);
  } catch (const std::exception& e) {
    return fail(GNUTS_ERR_SAMPLER, e.what());
  }
  if (rc) return fail(rc, err);
  return GNUTS_OK;
}

}  // namespace
}  // namespace gnuts

using namespace gnuts;

namespace gnuts {
RunHooks& run_hooks() {
  thread_local RunHooks h;
  return h;
}
}  // namespace gnuts

extern "C" {

void gnuts_set_interrupt(gnuts_interrupt_fn fn, void* ctx) {
  gnuts::run_hooks().interrupt = fn;
  gnuts::run_hooks().interrupt_ctx = ctx;
}

void gnuts_set_draw_sink(gnuts_draws_fn fn, void* ctx) {
  gnuts::run_hooks().sink = fn;
  gnuts::run_hooks().sink_ctx = ctx;
}


int gnuts_model_create(const char* model_id, const gnuts_var* vars, int n_vars, unsigned int seed, gnuts_model** out) {
  (void)seed;
  if (!model_id || !out) return fail(GNUTS_ERR_ARGUMENT, "null argument");
  try {
    VarMap vm = vars_from_abi(vars, n_vars);
    return create(model_id, vm, out);
  } catch (const std::exception& e) {
    return fail(GNUTS_ERR_DATA, e.what());
  }
}

int gnuts_model_create_json(const char* model_id, const char* json_text, unsigned int seed, gnuts_model** out) {
  (void)seed;
  if (!model_id || !out) return fail(GNUTS_ERR_ARGUMENT, "null argument");
  try {
    VarMap vm = JsonReader(json_text ? std::string(json_text) : std::string()).parse();
    return create(model_id, vm, out);
  } catch (const std::exception& e) {
    return fail(GNUTS_ERR_DATA, e.what());
  }
}

void gnuts_model_destroy(gnuts_model* m) { delete reinterpret_cast<ModelImpl*>(m); }

int gnuts_model_dims(const gnuts_model* m, int* num_params_r, int* num_constrained) {
  if (!m) return fail(GNUTS_ERR_ARGUMENT, "null model");
  if (num_params_r) *num_params_r = M(m)->dev.D;
  if (num_constrained) *num_constrained = M(m)->dev.ncon;
  return GNUTS_OK;
}

int gnuts_model_name(const gnuts_model* m, char* buf, size_t len) {
  if (!m || !buf) return fail(GNUTS_ERR_ARGUMENT, "null argument");
  snprintf(buf, len, "%s", M(m)->name.c_str());
  return GNUTS_OK;
}

int gnuts_model_param_name(const gnuts_model* m, int index, int unconstrained, char* buf, size_t len) {
  if (!m || !buf) return fail(GNUTS_ERR_ARGUMENT, "null argument");
  const auto& v = unconstrained ? M(m)->unc_names : M(m)->con_names;
  if (index < 0 || index >= (int)v.size()) return fail(GNUTS_ERR_ARGUMENT, "parameter index out of range");
  snprintf(buf, len, "%s", v[index].c_str());
  return GNUTS_OK;
}

int gnuts_log_prob_grad(const gnuts_model* m, int n, const double* q, int jacobian, double* lp, double* grad) {
  if (!m || (n > 0 && (!q || !lp || !grad))) return fail(GNUTS_ERR_ARGUMENT, "null argument");
  std::string err;
  int rc = run_log_prob_grad(*const_cast<Model*>(M(m)), n, q, jacobian, GNUTS_PRECISION_FP64, lp, grad, err);
  return rc ? fail(rc, err) : GNUTS_OK;
}

int gnuts_log_prob_grad_precision(const gnuts_model* m, int n, const double* q, int jacobian, int precision,
                                  double* lp, double* grad) {
  if (!m || (n > 0 && (!q || !lp || !grad))) return fail(GNUTS_ERR_ARGUMENT, "null argument");
  if (precision != GNUTS_PRECISION_FP64 && precision != GNUTS_PRECISION_MIXED)
    return fail(GNUTS_ERR_ARGUMENT, "unknown precision");
  std::string err;
  int rc = run_log_prob_grad(*const_cast<Model*>(M(m)), n, q, jacobian, precision, lp, grad, err);
  return rc ? fail(rc, err) : GNUTS_OK;
}

int gnuts_log_prob_grad_noalloc(const gnuts_model* m, int n, const double* q_device, int jacobian, double* lp_device,
                                double* grad_device) {
  if (!m) return fail(GNUTS_ERR_ARGUMENT, "null model");
  std::string err;
  int rc = noalloc_log_prob_grad(*M(m), n, q_device, jacobian, lp_device, grad_device, err);
  return rc ? fail(rc, err) : GNUTS_OK;
}

int gnuts_unconstrain(const gnuts_model* m, const double* c, double* q) {
  if (!m || !c || !q) return fail(GNUTS_ERR_ARGUMENT, "null argument");
  const DevModel& d = M(m)->dev;
  auto pos = [&](double v, const char* what) {
    if (!(v > 0)) throw std::runtime_error(std::string(what) + " is " + std::to_string(v) + ", but must be positive");
    return std::log(v);
  };
  try {
    switch (d.kind) {
      case MK_BERNOULLI:
        if (!(c[0] > 0 && c[0] < 1)) throw std::runtime_error("theta is " + std::to_string(c[0]) + ", but must be in the interval [0, 1]");
        q[0] = std::log(c[0] / (1.0 - c[0]));
        break;
      case MK_NORMAL:
      case MK_LOGISTIC:
      case MK_FUNNEL:
        for (int i = 0; i < d.D; ++i) q[i] = c[i];
        break;
      case MK_HIER:
        for (int i = 0; i <= d.J; ++i) q[i] = c[i];
        q[d.J + 1] = pos(c[d.J + 1], "tau");
        break;
      case MK_VARINT:
        if (d.n_members) throw std::runtime_error("a posterior set takes unconstrained inits (one row per chain)");
        for (int i = 0; i < d.J + d.K; ++i) q[i] = c[i];
        q[d.J + d.K] = pos(c[d.J + d.K], "sigma_y");
        q[d.J + d.K + 1] = pos(c[d.J + d.K + 1], "tau");
        break;
      case MK_HORSESHOE:
        q[0] = c[0];
        for (int k = 0; k < d.K; ++k) q[1 + k] = c[1 + k];
        q[d.K + 1] = pos(c[d.K + 1], "tau");
        for (int k = 0; k < d.K; ++k) q[d.K + 2 + k] = pos(c[d.K + 2 + k], "lambda");
        q[2 * d.K + 2] = pos(c[2 * d.K + 2], "caux");
        break;
    }
  } catch (const std::exception& e) {
    return fail(GNUTS_ERR_INIT, e.what());
  }
  return GNUTS_OK;
}

int gnuts_write_array(const gnuts_model* m, int n, const double* q, double* out) {
  if (!m || (n > 0 && (!q || !out))) return fail(GNUTS_ERR_ARGUMENT, "null argument");
  std::string err;
  int rc = run_write_array(*const_cast<Model*>(M(m)), n, q, out, err);
  return rc ? fail(rc, err) : GNUTS_OK;
}

void gnuts_sample_args_default(gnuts_sample_args* a) {
  if (!a) return;
  std::memset(a, 0, sizeof(*a));
  a->num_chains = 1;
  a->chain_id = 1;
  a->seed = 0;
  a->init_radius = 2.0;
  a->num_warmup = 1000;
  a->num_samples = 1000;
  a->thin = 1;
  a->save_warmup = 0;
  a->refresh = 100;
  a->stepsize = 1.0;
  a->stepsize_jitter = 0.0;
  a->max_depth = 10;
  a->delta = 0.8;
  a->gamma = 0.05;
  a->kappa = 0.75;
  a->t0 = 10.0;
  a->init_buffer = 75;
  a->term_buffer = 50;
  a->window = 25;
  a->precision = GNUTS_PRECISION_FP64;
}

int gnuts_hmc_nuts_diag_e_adapt(gnuts_model* m, const gnuts_sample_args* a, const double* inits,
                                const double* inv_metric, gnuts_output* out, gnuts_progress_fn progress, void* ctx) {
  return service(m, a, inits, inv_metric, out, progress, ctx, 0, 1);
}
int gnuts_hmc_nuts_dense_e_adapt(gnuts_model* m, const gnuts_sample_args* a, const double* inits,
                                 const double* inv_metric, gnuts_output* out, gnuts_progress_fn progress, void* ctx) {
  return service(m, a, inits, inv_metric, out, progress, ctx, 1, 1);
}
int gnuts_hmc_nuts_unit_e_adapt(gnuts_model* m, const gnuts_sample_args* a, const double* inits, gnuts_output* out,
                                gnuts_progress_fn progress, void* ctx) {
  return service(m, a, inits, nullptr, out, progress, ctx, 2, 1);
}
int gnuts_hmc_nuts_diag_e(gnuts_model* m, const gnuts_sample_args* a, const double* inits, const double* inv_metric,
                          gnuts_output* out, gnuts_progress_fn progress, void* ctx) {
  return service(m, a, inits, inv_metric, out, progress, ctx, 0, 0);
}
int gnuts_hmc_nuts_dense_e(gnuts_model* m, const gnuts_sample_args* a, const double* inits, const double* inv_metric,
                           gnuts_output* out, gnuts_progress_fn progress, void* ctx) {
  return service(m, a, inits, inv_metric, out, progress, ctx, 1, 0);
}
int gnuts_hmc_nuts_unit_e(gnuts_model* m, const gnuts_sample_args* a, const double* inits, gnuts_output* out,
                          gnuts_progress_fn progress, void* ctx) {
  return service(m, a, inits, nullptr, out, progress, ctx, 2, 0);
}

int gnuts_transition(gnuts_model* m, int metric, const double* inv_metric, int n, const double* q0, const double* p0,
                     double stepsize, int max_depth, unsigned int seed, const unsigned int* chain_ids,
                     uint64_t* counters, double* q_out, double* stats) {
  if (!m || !q0 || !p0 || !chain_ids || !counters || !q_out || !stats) return fail(GNUTS_ERR_ARGUMENT, "null argument");
  if (n < 1) return fail(GNUTS_ERR_ARGUMENT, "n must be >= 1");
  if (metric < 0 || metric > 2) return fail(GNUTS_ERR_ARGUMENT, "metric must be 0, 1 or 2");
  if (metric != 2 && !inv_metric) return fail(GNUTS_ERR_ARGUMENT, "inverse metric required");
  if (max_depth < 1 || max_depth > 16) return fail(GNUTS_ERR_ARGUMENT, "max_depth must be in 1..16");
  if (!(stepsize > 0)) return fail(GNUTS_ERR_ARGUMENT, "stepsize must be > 0");
  std::string err;
  int rc = run_transition(*M(m), metric, inv_metric, n, q0, p0, stepsize, max_depth, seed, chain_ids, counters, q_out,
                          stats, err);
  return rc ? fail(rc, err) : GNUTS_OK;
}

int gnuts_last_error(char* buf, size_t len) {
  if (buf && len) snprintf(buf, len, "%s", g_last_error.c_str());
  return (int)g_last_error.size();
}

const char* gnuts_version(void) { return "gnuts 0.1 (sm_103a)"; }

}  // extern "C"
