// The CmdStan argument tree for the sample method.
//
// Mirrors the grammar the reference parses (src/cmdstan/arguments/
// argument_parser.hpp, categorical_argument.hpp, list_argument.hpp,
// singleton_argument.hpp): tokens are `name` or `name=value`; a group
// (`adapt`, `output`, ...) consumes the tokens that follow it while they
// name one of its sub-arguments; a list (`method=sample`, `algorithm=hmc`,
// `engine=nuts`, `metric=diag_e`) selects one option and that option's group
// consumes what follows; each top-level argument may be given once; a bare
// method name is read as `method=<name>`.  The tree is printed in the Stan
// CSV header as `name = value` lines, two spaces of indent per level and
// " (Default)" after values left at their defaults (valued_argument.hpp).
#pragma once
#include <climits>
#include <cmath>
#include <functional>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace gnuts_cli {

struct Arg {
  enum Kind { GROUP, LIST, INT, UINT, REAL, BOOL, STRING };
  Kind kind;
  std::string name, desc;
  // value (INT / UINT / REAL / BOOL / STRING)
  long long ival = 0, idef = 0;
  double rval = 0, rdef = 0;
  bool bval = false, bdef = false;
  std::string sval, sdef;
  std::string valid_text;                  // "Valid values:" text
  std::function<bool(long long)> ivalid;   // INT / UINT
  std::function<bool(double)> rvalid;      // REAL
  // GROUP: sub-arguments in print order; LIST: the options (each a GROUP)
  std::vector<std::unique_ptr<Arg>> children;
  int cursor = 0, def_cursor = 0;
  bool unvalued = false;  // an option without sub-arguments that prints no line (unvalued_argument.hpp)

  Arg(Kind k, std::string n, std::string d) : kind(k), name(std::move(n)), desc(std::move(d)) {}

  Arg* add(std::unique_ptr<Arg> a) {
    children.push_back(std::move(a));
    return children.back().get();
  }
  Arg* child(const std::string& n) const {
    if (kind == LIST) {
      const Arg* sel = children[cursor].get();
      return sel->name == n ? const_cast<Arg*>(sel) : nullptr;
    }
    for (auto& c : children)
      if (c->name == n) return c.get();
    return nullptr;
  }
  bool is_default() const {
    switch (kind) {
      case INT: case UINT: return ival == idef;
      case REAL: return rval == rdef;
      case BOOL: return bval == bdef;
      case STRING: return sval == sdef;
      case LIST: return cursor == def_cursor;
      default: return true;
    }
  }
  std::string value_text() const {
    switch (kind) {
      case INT: case UINT: return std::to_string(ival);
      case REAL: { std::ostringstream s; s << rval; return s.str(); }
      case BOOL: return bval ? "true" : "false";
      case STRING: return sval;
      case LIST: return children[cursor]->name;
      default: return "";
    }
  }
};

inline std::unique_ptr<Arg> group(const std::string& n, const std::string& d) {
  return std::make_unique<Arg>(Arg::GROUP, n, d);
}
inline std::unique_ptr<Arg> unvalued(const std::string& n, const std::string& d) {
  auto a = std::make_unique<Arg>(Arg::GROUP, n, d);
  a->unvalued = true;
  return a;
}
inline std::unique_ptr<Arg> list(const std::string& n, const std::string& d) {
  return std::make_unique<Arg>(Arg::LIST, n, d);
}
inline std::unique_ptr<Arg> int_arg(const std::string& n, const std::string& d, long long def,
                                    std::function<bool(long long)> ok, const std::string& valid) {
  auto a = std::make_unique<Arg>(Arg::INT, n, d);
  a->ival = a->idef = def;
  a->ivalid = std::move(ok);
  a->valid_text = valid;
  return a;
}
inline std::unique_ptr<Arg> uint_arg(const std::string& n, const std::string& d, long long def) {
  auto a = std::make_unique<Arg>(Arg::UINT, n, d);
  a->ival = a->idef = def;
  a->ivalid = [](long long v) { return v >= 0 && v <= (long long)UINT_MAX; };
  a->valid_text = " 0 <= " + n;
  return a;
}
inline std::unique_ptr<Arg> real_arg(const std::string& n, const std::string& d, double def,
                                     std::function<bool(double)> ok, const std::string& valid) {
  auto a = std::make_unique<Arg>(Arg::REAL, n, d);
  a->rval = a->rdef = def;
  a->rvalid = std::move(ok);
  a->valid_text = valid;
  return a;
}
inline std::unique_ptr<Arg> bool_arg(const std::string& n, const std::string& d, bool def) {
  auto a = std::make_unique<Arg>(Arg::BOOL, n, d);
  a->bval = a->bdef = def;
  a->valid_text = " [0, 1, false, true]";
  return a;
}
inline std::unique_ptr<Arg> string_arg(const std::string& n, const std::string& d, const std::string& def) {
  auto a = std::make_unique<Arg>(Arg::STRING, n, d);
  a->sval = a->sdef = def;
  a->valid_text = " Path to existing file";
  return a;
}

inline void split_token(const std::string& t, std::string& name, std::string& value) {
  const size_t eq = t.find('=');
  if (eq == std::string::npos) {
    name = t;
    value.clear();
  } else {
    name = t.substr(0, eq);
    value = t.substr(eq + 1);
  }
}

struct ParseState {
  std::vector<std::string> errors;
  bool help = false;
};

// The parse functions take the remaining tokens in REVERSE order (the next
// token is at the back), like the reference parser.
bool parse_arg(Arg& a, std::vector<std::string>& toks, ParseState& st);

// Value parsing follows the reference's from_string: std::stoi / stoul /
// stod (a numeric prefix is accepted), booleans 0 / 1 / false / true.
inline bool parse_value(Arg& a, const std::string& v) {
  try {
    switch (a.kind) {
      case Arg::INT: {
        long long x = std::stoll(v);
        if (x < INT_MIN || x > INT_MAX || !a.ivalid(x)) return false;
        a.ival = x;
        return true;
      }
      case Arg::UINT: {
        if (!v.empty() && v[0] == '-') return false;
        unsigned long long x = std::stoull(v);
        if (x > UINT_MAX || !a.ivalid((long long)x)) return false;
        a.ival = (long long)x;
        return true;
      }
      case Arg::REAL: {
        double x = std::stod(v);
        if (!a.rvalid(x)) return false;
        a.rval = x;
        return true;
      }
      case Arg::BOOL:
        if (v == "true" || v == "1") { a.bval = true; return true; }
        if (v == "false" || v == "0") { a.bval = false; return true; }
        return false;
      case Arg::STRING:
        a.sval = v;
        return true;
      default:
        return false;
    }
  } catch (...) {
    return false;
  }
}

inline bool parse_group(Arg& g, std::vector<std::string>& toks, ParseState& st) {
  bool valid = true;
  while (!toks.empty()) {
    const std::string t = toks.back();
    if (t == "help" || t == "help-all") {
      st.help = true;
      toks.clear();
      return true;
    }
    std::string n, v;
    split_token(t, n, v);
    if (n == g.name) return false;
    Arg* hit = nullptr;
    bool bare = false;
    for (auto& c : g.children) {
      if (c->name == t) { hit = c.get(); bare = true; break; }
      if (c->name == n) { hit = c.get(); break; }
    }
    if (!hit) break;
    if (bare) toks.pop_back();
    valid &= parse_arg(*hit, toks, st);
    if (!valid) break;
  }
  return valid;
}

inline bool parse_arg(Arg& a, std::vector<std::string>& toks, ParseState& st) {
  if (a.kind == Arg::GROUP) return parse_group(a, toks, st);
  if (toks.empty()) return true;
  std::string n, v;
  split_token(toks.back(), n, v);
  if (n != a.name) return true;
  toks.pop_back();
  if (a.kind == Arg::LIST) {
    for (size_t i = 0; i < a.children.size(); ++i) {
      if (a.children[i]->name != v) continue;
      a.cursor = (int)i;
      return parse_group(*a.children[i], toks, st);
    }
    std::string opts;
    for (auto& c : a.children) opts += " " + c->name;
    st.errors.push_back(v + " is not a valid value for \"" + a.name + "\"");
    st.errors.push_back("  Valid values:" + opts);
    toks.clear();
    return false;
  }
  if (parse_value(a, v)) return true;
  st.errors.push_back(v + " is not a valid value for \"" + a.name + "\"");
  st.errors.push_back("  Valid values:" + a.valid_text);
  toks.clear();
  return false;
}

// `name = value` lines of the tree (valued_argument.hpp / categorical_argument.hpp print)
inline void print_arg(const Arg& a, int depth, std::vector<std::string>& out) {
  const std::string ind(2 * depth, ' ');
  if (a.kind == Arg::GROUP) {
    if (a.unvalued) return;
    out.push_back(ind + a.name);
    for (auto& c : a.children) print_arg(*c, depth + 1, out);
    return;
  }
  std::string line = ind + a.name + " = " + a.value_text();
  if (a.is_default()) line += " (Default)";
  out.push_back(line);
  if (a.kind == Arg::LIST) print_arg(*a.children[a.cursor], depth + 1, out);
}

// ---------------------------------------------------------------- the tree
struct Config {
  std::unique_ptr<Arg> method, id, data, init, random, output, num_threads, gpu;
  std::vector<Arg*> top;        // print / parse order
  unsigned int random_seed = 0; // value used when seed is left at -1

  Config() {
    auto pos_i = [](long long v) { return v > 0; };
    auto nonneg_i = [](long long v) { return v >= 0; };
    auto pos_r = [](double v) { return v > 0; };
    method = list("method", "Analysis method (Note that method= is optional)");
    {
      auto sample = group("sample", "Bayesian inference with Markov Chain Monte Carlo");
      sample->add(int_arg("num_samples", "Number of sampling iterations", 1000, nonneg_i, " 0 <= num_samples"));
      sample->add(int_arg("num_warmup", "Number of warmup iterations", 1000, nonneg_i, " 0 <= num_warmup"));
      sample->add(bool_arg("save_warmup", "Stream warmup samples to output?", false));
      sample->add(int_arg("thin", "Period between saved samples", 1, pos_i, " 0 < thin"));
      auto adapt = group("adapt", "Warmup Adaptation");
      adapt->add(bool_arg("engaged", "Adaptation engaged?", true));
      adapt->add(real_arg("gamma", "Adaptation regularization scale", 0.05, pos_r, " 0 < gamma"));
      adapt->add(real_arg("delta", "Adaptation target acceptance statistic", 0.8,
                          [](double v) { return v >= 0.1 && v <= std::nextafter(1.0, 0.0); },
                          " 0.1 <= delta <= 1"));
      adapt->add(real_arg("kappa", "Adaptation relaxation exponent", 0.75, pos_r, " 0 < kappa"));
      adapt->add(real_arg("t0", "Adaptation iteration offset", 10, pos_r, " 0 < t0"));
      adapt->add(uint_arg("init_buffer", "Width of initial fast adaptation interval", 75));
      adapt->add(uint_arg("term_buffer", "Width of final fast adaptation interval", 50));
      adapt->add(uint_arg("window", "Initial width of slow adaptation interval", 25));
      adapt->add(bool_arg("save_metric", "Save metric as JSON?", false));
      sample->add(std::move(adapt));
      auto algo = list("algorithm", "Sampling algorithm");
      {
        auto hmc = group("hmc", "Hamiltonian Monte Carlo");
        auto engine = list("engine", "Engine for Hamiltonian Monte Carlo");
        auto stat = group("static", "Static integration time");
        stat->add(real_arg("int_time", "Total integration time for Hamiltonian evolution", 2 * M_PI, pos_r,
                           " 0 < int_time"));
        engine->add(std::move(stat));
        auto nuts = group("nuts", "The No-U-Turn Sampler");
        nuts->add(int_arg("max_depth", "Maximum tree depth", 10, pos_i, " 0 < max_depth"));
        engine->add(std::move(nuts));
        engine->cursor = engine->def_cursor = 1;
        hmc->add(std::move(engine));
        auto metric = list("metric", "Geometry of base manifold");
        metric->add(unvalued("unit_e", "Euclidean manifold with unit metric"));
        metric->add(unvalued("diag_e", "Euclidean manifold with diag metric"));
        metric->add(unvalued("dense_e", "Euclidean manifold with dense metric"));
        metric->cursor = metric->def_cursor = 1;
        hmc->add(std::move(metric));
        hmc->add(string_arg("metric_file", "Input file with precomputed Euclidean metric", ""));
        hmc->add(real_arg("stepsize", "Step size for discrete evolution", 1, pos_r, " 0 < stepsize"));
        hmc->add(real_arg("stepsize_jitter", "Uniformly random jitter of the stepsize, in percent", 0,
                          [](double v) { return v >= 0 && v <= 1; }, " 0 <= stepsize_jitter <= 1"));
        algo->add(std::move(hmc));
        algo->add(unvalued("fixed_param", "Fixed Parameter Sampler"));
      }
      sample->add(std::move(algo));
      sample->add(int_arg("num_chains", "Number of chains", 1, pos_i, " 0 < num_chains"));
      method->add(std::move(sample));
      // the other CmdStan methods are recognised (so that they parse like the
      // reference's); log_prob (arg_log_prob.hpp) and diagnose test=gradient
      // (arg_diagnose.hpp, arg_test_gradient.hpp) run, the rest are refused
      // with a message when run
      for (const char* m : {"optimize", "variational"}) method->add(group(m, "not provided by this sampler"));
      {
        auto diag = group("diagnose", "Model diagnostics");
        auto test = list("test", "Diagnostic test");
        auto grad = group("gradient", "Check model gradient against finite differences");
        grad->add(real_arg("epsilon", "Finite difference step size", 1e-6, pos_r, " 0 < epsilon"));
        grad->add(real_arg("error", "Error threshold", 1e-6, pos_r, " 0 < error"));
        test->add(std::move(grad));
        diag->add(std::move(test));
        method->add(std::move(diag));
      }
      for (const char* m : {"generate_quantities", "pathfinder"}) method->add(group(m, "not provided by this sampler"));
      {
        auto lp = group("log_prob", "Return the log density up to a constant and its gradients, given supplied "
                                    "parameters");
        lp->add(string_arg("unconstrained_params", "Input file (JSON or R dump) of parameter values on "
                                                   "unconstrained scale", ""));
        lp->add(string_arg("constrained_params", "Input file (JSON or R dump) of parameter values on "
                                                 "constrained scale", ""));
        lp->add(bool_arg("jacobian", "When true, include change-of-variables adjustment for constraining "
                                     "parameter transforms", true));
        method->add(std::move(lp));
      }
      method->add(group("laplace", "not provided by this sampler"));
    }
    id = int_arg("id", "Unique process identifier", 1, [](long long v) { return v >= 0; }, " id >= 0");
    data = group("data", "Input data options");
    data->add(string_arg("file", "Input data file", ""));
    init = string_arg("init", "Initialization method: \"x\" initialize randomly between [-x, x], \"0\" "
                              "initialize to 0, anything else identifies a file of values",
                      "2");
    init->valid_text = " real number >= 0 or file path";
    random = group("random", "Random number configuration");
    random->add(int_arg("seed", "Random number generator seed", -1,
                        [](long long v) { return (v >= 0 && v <= (long long)UINT_MAX) || v == -1; },
                        " non-negative integer < 4294967296  or -1 to generate seed"));
    output = group("output", "File output options");
    output->add(string_arg("file", "Output file", "output.csv"));
    output->add(string_arg("diagnostic_file", "Auxiliary output file for diagnostic information", ""));
    output->add(int_arg("refresh", "Number of iterations between screen updates", 100,
                        [](long long v) { return v >= 0; }, " 0 <= refresh"));
    output->add(int_arg("sig_figs", "The number of significant figures used for the output CSV files.", -1,
                        [](long long v) { return (v >= 0 && v <= 18) || v == -1; },
                        " 0 <= integer <= 18 or -1 to use the default number of significant figures"));
    output->add(string_arg("profile_file", "File to store profiling information", "profile.csv"));
    output->add(bool_arg("save_cmdstan_config", "Save the CmdStan configuration as JSON?", false));
    num_threads = int_arg("num_threads", "Number of threads available to the program.", 1,
                          [](long long v) { return v > 0 || v == -1; }, " num_threads > 0 || num_threads == -1");
    // options of this sampler that CmdStan does not have, in their own group so
    // that CmdStan's arguments and defaults stay as they are
    gpu = group("gpu", "GB300 sampler options (not part of CmdStan)");
    {
      auto prec = list("precision", "Gradient precision of the data-heavy models");
      prec->add(unvalued("fp64", "FP64 everywhere"));
      prec->add(unvalued("mixed", "BF16-split tensor-core contractions, FP32 accumulation, FP64 energy"));
      gpu->add(std::move(prec));
      gpu->add(bool_arg("learned", "Learned affine-coupling preconditioner with plain NUTS as fallback and judge "
                                   "(metric=diag_e, adaptation engaged)", false));
    }
    top = {method.get(), id.get(), data.get(), init.get(), random.get(), output.get(), num_threads.get(), gpu.get()};
  }

  Arg* sample() const { return method->children[0].get(); }
  Arg* adapt() const { return sample()->child("adapt"); }
  Arg* hmc() const { return sample()->children[5]->children[0].get(); }
  Arg* at(const std::vector<std::string>& path) const {
    Arg* a = nullptr;
    for (Arg* t : top)
      if (t->name == path[0]) a = t;
    for (size_t i = 1; a && i < path.size(); ++i) a = a->child(path[i]);
    return a;
  }

  // parse argv[first..argc) the way argument_parser::parse_args does
  bool parse(int argc, char** argv, int first, ParseState& st) {
    std::vector<std::string> toks;
    for (int i = argc - 1; i >= first; --i) toks.push_back(argv[i]);
    std::vector<Arg*> unset = top;
    bool method_set = false, valid = true, good = true;
    while (good && !toks.empty()) {
      good = false;
      std::string t = toks.back();
      if (!method_set) {
        for (auto& m : method->children)
          if (m->name == t) {
            t = "method=" + t;
            toks.back() = t;
            break;
          }
      }
      std::string n, v;
      split_token(t, n, v);
      if (n == "method") method_set = true;
      for (size_t i = 0; i < unset.size(); ++i) {
        Arg* a = unset[i];
        if (a->name == t) {
          toks.pop_back();
          valid &= parse_arg(*a, toks, st);
          good = true;
        } else if (a->name == n) {
          valid &= parse_arg(*a, toks, st);
          good = true;
        }
        if (good) {
          unset.erase(unset.begin() + i);
          break;
        }
      }
      if (t == "help" || t == "help-all") {
        st.help = true;
        return true;
      }
      if (!good) st.errors.push_back(t + " is either mistyped or misplaced.");
    }
    if (st.help) return true;
    if (!method_set) st.errors.push_back("A method must be specified!");
    return valid && good && method_set;
  }

  std::vector<std::string> lines() const {
    std::vector<std::string> out;
    for (Arg* a : top) {
      if (a == random.get()) {
        // seed -1 prints the seed actually used (arg_seed.hpp print_value)
        out.push_back("random");
        const Arg* s = random->children[0].get();
        std::string l = "  seed = " + std::to_string(s->ival == -1 ? (long long)random_seed : s->ival);
        if (s->is_default()) l += " (Default)";
        out.push_back(l);
        continue;
      }
      print_arg(*a, 0, out);
    }
    return out;
  }
};

}  // namespace gnuts_cli
