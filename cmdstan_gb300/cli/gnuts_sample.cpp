// gnuts-sample: the CmdStan command line for `method=sample algorithm=hmc
// engine=nuts`, running the GPU sampler behind include/gnuts.h.
//
// Replaces the sample branch of cmdstan::command (src/cmdstan/command.hpp:
// 97-118 argument parsing, 166-171 data + model, 180-264 output writers,
// 552-697 the hmc_nuts_* dispatch) and writes Stan CSV the way the
// reference's writers do (write_config.hpp header, column header, the
// adaptation block, draws, the elapsed-time trailer; file.hpp:189-212 file
// names; save_metric JSON, command.hpp:247-261).
//
// A CmdStan model executable is named after its model; the built-in models
// here are selected the same way: run through a link named after the model
// (`ln -s gnuts-sample bernoulli; ./bernoulli sample data file=...`) or
// name it as the first argument (`gnuts-sample model=bernoulli sample ...`).
// Exit status 0 on success, 1 on any error (return_codes.hpp).
#include <gnuts.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <random>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "arg_tree.hpp"
#include "json_lite.hpp"

using namespace gnuts_cli;

namespace {

constexpr int OK = 0, NOT_OK = 1;

std::string read_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("Can't open specified file, \"" + path + "\"");
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}
bool file_exists(const std::string& p) {
  std::ifstream f(p);
  return (bool)f;
}

// file.hpp make_filenames: base + tag + ("_" + (id + i) when several) + suffix
std::vector<std::string> make_filenames(const std::string& file, const std::string& tag, const std::string& type,
                                        int n, unsigned id) {
  std::string base = file, sfx;
  const size_t dot = file.find_last_of('.');
  const size_t sep = file.find_last_of('/');
  if (dot != std::string::npos && (sep == std::string::npos || dot > sep) && dot > 0) {
    base = file.substr(0, dot);
    sfx = file.substr(dot);
  }
  if (type != ".csv" || sfx.empty()) sfx = type;
  std::vector<std::string> out;
  for (int i = 0; i < n; ++i)
    out.push_back(base + tag + (n == 1 ? std::string() : "_" + std::to_string(id + (unsigned)i)) + sfx);
  return out;
}

// command_helper.hpp get_vec_var_context: per-chain files <base>_<id+i><ext>
// when the first exists, else the base file for every chain
std::vector<std::string> per_chain_inputs(const std::string& file, int n, unsigned id) {
  if (n == 1) return {file};
  const size_t dot = file.find_last_of('.');
  if (dot == std::string::npos) throw std::runtime_error("Found: \"" + file + "\" but user specified files must end in .json or .R");
  const std::string ext = file.substr(dot);
  if (ext != ".json") throw std::runtime_error("file ending of " + ext + " is not supported by gnuts-sample (JSON only)");
  auto names = make_filenames(file.substr(0, dot), "", ext, n, id);
  if (!file_exists(names[0])) {
    if (!file_exists(file))
      throw std::runtime_error("Can't open either of specified files,\"" + names[0] + "\" and base file \"" + file + "\"");
    return std::vector<std::string>(n, file);
  }
  for (auto& f : names)
    if (!file_exists(f)) throw std::runtime_error("Found \"" + names[0] + "\" but cannot open \"" + f + "\"");
  return names;
}

std::string fmt(double v, int prec) {
  if (std::isnan(v)) return "nan";
  if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
  char b[64];
  snprintf(b, sizeof b, "%.*g", prec, v);
  return b;
}

std::string utc_now() {
  std::time_t t = std::chrono::system_clock::to_time_t(std::chrono::system_clock::now());
  std::tm tm{};
  gmtime_r(&t, &tm);
  char b[64];
  snprintf(b, sizeof b, "%04d-%02d-%02d %02d:%02d:%02d UTC", 1900 + tm.tm_year, tm.tm_mon + 1, tm.tm_mday,
           tm.tm_hour, tm.tm_min, tm.tm_sec);
  return b;
}

std::string last_error() {
  char b[2048];
  gnuts_last_error(b, sizeof b);
  return b;
}

struct Progress {
  int num_chains;
  unsigned id;
};
void on_progress(void* ctx, int chain, int iteration, int total, int warmup) {
  const Progress* p = static_cast<const Progress*>(ctx);
  const int width = (int)std::to_string(total).size();
  const int it = iteration + 1 > total ? total : iteration + 1;
  char line[160];
  snprintf(line, sizeof line, "Iteration: %*d / %d [%3d%%]  (%s)", width, it, total, (int)(100.0 * it / total),
           warmup ? "Warmup" : "Sampling");
  if (p->num_chains > 1) std::cout << "Chain [" << (p->id + (unsigned)chain) << "] ";
  std::cout << line << std::endl;
}

// Constrained values of the parameters block (the first num_params_r names
// of write_array order) from a JSON object; "beta.3" is element 3 (1-based)
// of the flattened array "beta".
std::vector<double> constrained_from_json(gnuts_model* m, const JValue& obj, int D, const std::string& file) {
  std::vector<double> out(D);
  for (int i = 0; i < D; ++i) {
    char nb[256];
    gnuts_model_param_name(m, i, 0, nb, sizeof nb);
    std::string name = nb, var = name;
    std::vector<int> idx;
    const size_t dot = name.find('.');
    if (dot != std::string::npos) {
      var = name.substr(0, dot);
      std::stringstream ss(name.substr(dot + 1));
      std::string part;
      while (std::getline(ss, part, '.')) idx.push_back(std::stoi(part));
    }
    const JValue* v = obj.get(var);
    if (!v) throw std::runtime_error("variable " + var + " not found in init file " + file);
    for (int k : idx) {
      if (v->type != JValue::ARR || k < 1 || k > (int)v->arr.size())
        throw std::runtime_error("variable " + var + " in init file " + file + " has too few elements");
      v = &v->arr[k - 1];
    }
    if (!v->as_number(out[i])) throw std::runtime_error("variable " + var + " in init file " + file + " is not numeric");
  }
  return out;
}

gnuts_model* create_model(const Config& cfg, const std::string& model_id) {
  const std::string data_file = cfg.data->children[0]->sval;
  const std::string data_text = data_file.empty() ? std::string("{}") : read_file(data_file);
  gnuts_model* model = nullptr;
  if (gnuts_model_create_json(model_id.c_str(), data_text.c_str(), cfg.random_seed, &model) != GNUTS_OK)
    throw std::runtime_error("Error creating model '" + model_id + "': " + last_error());
  return model;
}

void write_csv_header(std::ostream& f, gnuts_model* model, const std::vector<std::string>& cfg_lines) {
  char nb[256];
  gnuts_model_name(model, nb, sizeof nb);
  f << "# stan_version_major = 2\n# stan_version_minor = 36\n# stan_version_patch = 0\n";
  f << "# model = " << nb << "\n# start_datetime = " << utc_now() << "\n";
  for (auto& l : cfg_lines) f << "# " << l << "\n";
  f << "# stanc_version = gnuts built-in model\n# stancflags = \n# gnuts_version = " << gnuts_version() << "\n";
}

std::vector<std::string> split_csv(const std::string& line) {
  std::vector<std::string> out;
  std::stringstream ss(line);
  std::string t;
  while (std::getline(ss, t, ',')) {
    while (!t.empty() && (t.back() == '\r' || t.back() == ' ')) t.pop_back();
    while (!t.empty() && t.front() == ' ') t.erase(t.begin());
    out.push_back(t);
  }
  return out;
}

// Unconstrained parameter sets for method=log_prob (command.hpp:414-446):
// `unconstrained_params` is a JSON file with params_r (one vector, or an array
// of vectors, command_helper.hpp:520-558); `constrained_params` is a JSON file
// of the parameters block or a Stan CSV whose parameter columns are read row
// by row (command_helper.hpp:279-374).
std::vector<double> log_prob_points(gnuts_model* model, const std::string& upars, const std::string& cpars, int D,
                                    int* n_out) {
  std::vector<double> q;
  if (!upars.empty()) {
    JValue obj = JParser(read_file(upars)).parse();
    const JValue* v = obj.get("params_r");
    if (!v) throw std::runtime_error("Unconstrained parameters file has no variable 'params_r' with unconstrained "
                                     "parameter values!");
    std::vector<double> flat;
    v->flatten(flat);
    size_t cols = flat.size();
    if (v->type == JValue::ARR && !v->arr.empty() && v->arr[0].type == JValue::ARR) cols = v->arr[0].arr.size();
    if ((int)cols != D || flat.empty())
      throw std::runtime_error("Incorrect number of unconstrained parameters provided! Model has " + std::to_string(D) +
                               " parameters but " + std::to_string(cols) + " were found.");
    *n_out = (int)(flat.size() / cols);
    return flat;
  }
  std::vector<std::vector<double>> rows;
  const size_t dot = cpars.find_last_of('.');
  if (dot != std::string::npos && cpars.substr(dot) == ".csv") {
    std::ifstream f(cpars);
    if (!f) throw std::runtime_error("Can't open specified file, \"" + cpars + "\"");
    std::string line;
    std::vector<std::string> header;
    std::vector<int> cols(D, -1);
    while (std::getline(f, line)) {
      if (line.empty() || line[0] == '#') continue;
      if (header.empty()) {
        header = split_csv(line);
        for (int i = 0; i < D; ++i) {
          char nb[256];
          gnuts_model_param_name(model, i, 0, nb, sizeof nb);
          for (size_t k = 0; k < header.size(); ++k)
            if (header[k] == nb) cols[i] = (int)k;
          if (cols[i] < 0)
            throw std::runtime_error(std::string("Mismatch between model and fitted_parameters csv file \"") + cpars +
                                     "\": no column " + nb);
        }
        continue;
      }
      const auto vals = split_csv(line);
      std::vector<double> con(D);
      for (int i = 0; i < D; ++i) {
        if (cols[i] >= (int)vals.size()) throw std::runtime_error("short row in " + cpars);
        con[i] = std::stod(vals[cols[i]]);
      }
      rows.push_back(con);
    }
  } else {
    JValue obj = JParser(read_file(cpars)).parse();
    rows.push_back(constrained_from_json(model, obj, D, cpars));
  }
  q.resize(rows.size() * D);
  for (size_t r = 0; r < rows.size(); ++r)
    if (gnuts_unconstrain(model, rows[r].data(), q.data() + r * D) != GNUTS_OK)
      throw std::runtime_error("Error transforming the constrained parameter values of " + cpars + ": " +
                               last_error());
  *n_out = (int)rows.size();
  return q;
}

// method=log_prob: lp and gradient for every parameter set, evaluated on the
// GPU in one batch; written like services_log_prob_grad
// (command_helper.hpp:560-600): header lp__,g_<unconstrained names>, one row
// per set.
int run_log_prob(Config& cfg, const std::string& model_id, Arg* lpg) {
  const std::string upars = lpg->child("unconstrained_params")->sval;
  const std::string cpars = lpg->child("constrained_params")->sval;
  const bool jacobian = lpg->child("jacobian")->bval;
  if (upars.empty() && cpars.empty())
    throw std::runtime_error("No input parameter files provided, cannot calculate log probability density.");
  if (!upars.empty() && !cpars.empty())
    throw std::runtime_error("Cannot specify both input files of both constrained and unconstrained parameter "
                             "values.");
  const long long seed_arg = cfg.random->children[0]->ival;
  cfg.random_seed = seed_arg >= 0 ? (unsigned)seed_arg : 0u;
  const auto cfg_lines = cfg.lines();
  for (auto& l : cfg_lines) std::cout << l << std::endl;
  std::cout << std::endl;
  gnuts_model* model = create_model(cfg, model_id);
  struct ModelGuard { gnuts_model* m; ~ModelGuard() { gnuts_model_destroy(m); } } mg{model};
  int D = 0, ncon = 0;
  gnuts_model_dims(model, &D, &ncon);
  int n = 0;
  std::vector<double> q = log_prob_points(model, upars, cpars, D, &n);
  std::vector<double> lp(n), g((size_t)n * D);
  if (gnuts_log_prob_grad(model, n, q.data(), jacobian ? 1 : 0, lp.data(), g.data()) != GNUTS_OK)
    throw std::runtime_error("Error during log_prob calculation:\n" + last_error());
  Arg* out_grp = cfg.output.get();
  const int sig_figs = (int)out_grp->child("sig_figs")->ival;
  const int prec = sig_figs < 0 ? 6 : sig_figs;
  const std::string file = out_grp->child("file")->sval;
  std::ofstream f(file);
  if (!f) throw std::runtime_error("Can't open output file " + file);
  write_csv_header(f, model, cfg_lines);
  f << "lp__";
  for (int i = 0; i < D; ++i) {
    char nb[256];
    gnuts_model_param_name(model, i, 1, nb, sizeof nb);
    f << ",g_" << nb;
  }
  f << "\n";
  for (int r = 0; r < n; ++r) {
    f << fmt(lp[r], prec);
    for (int i = 0; i < D; ++i) f << "," << fmt(g[(size_t)r * D + i], prec);
    f << "\n";
  }
  if (!f) throw std::runtime_error("error writing " + file);
  return OK;
}

// method=diagnose test=gradient: the model gradient at the initial point
// against central finite differences of the log density (with the Jacobian),
// all 2D + 1 evaluations in one batch on the GPU.  Report as CmdStan's
// gradient test prints it, to the console and as comments in the output file.
int run_diagnose(Config& cfg, const std::string& model_id, Arg* diag) {
  Arg* test = diag->child("test");
  if (test->value_text() != "gradient") throw std::runtime_error("diagnose test=" + test->value_text() + " unknown");
  Arg* grad = test->child("gradient");
  const double eps = grad->child("epsilon")->rval, tol = grad->child("error")->rval;
  const long long seed_arg = cfg.random->children[0]->ival;
  cfg.random_seed = seed_arg >= 0
                        ? (unsigned)seed_arg
                        : (unsigned)(std::chrono::system_clock::now().time_since_epoch().count() & 0xFFFFFFFFu);
  const auto cfg_lines = cfg.lines();
  for (auto& l : cfg_lines) std::cout << l << std::endl;
  std::cout << std::endl;
  gnuts_model* model = create_model(cfg, model_id);
  struct ModelGuard { gnuts_model* m; ~ModelGuard() { gnuts_model_destroy(m); } } mg{model};
  int D = 0, ncon = 0;
  gnuts_model_dims(model, &D, &ncon);
  // initial point: a radius (uniform on (-R, R), seeded) or a JSON file of constrained values
  std::vector<double> q0(D, 0.0);
  const std::string init = cfg.init->sval;
  double radius = 2.0;
  bool is_radius = true;
  try {
    size_t used = 0;
    radius = std::stod(init, &used);
    is_radius = used == init.size();
  } catch (...) {
    is_radius = false;
  }
  if (is_radius) {
    std::mt19937_64 rng(cfg.random_seed);
    std::uniform_real_distribution<double> u(-radius, radius);
    for (double& v : q0) v = radius > 0 ? u(rng) : 0.0;
  } else {
    JValue obj = JParser(read_file(init)).parse();
    auto con = constrained_from_json(model, obj, D, init);
    if (gnuts_unconstrain(model, con.data(), q0.data()) != GNUTS_OK)
      throw std::runtime_error("Error transforming the initial values of " + init + ": " + last_error());
  }
  const int n = 2 * D + 1;
  std::vector<double> q((size_t)n * D), lp(n), g((size_t)n * D);
  for (int r = 0; r < n; ++r) std::copy(q0.begin(), q0.end(), q.begin() + (size_t)r * D);
  for (int i = 0; i < D; ++i) {
    q[(size_t)(1 + 2 * i) * D + i] += eps;
    q[(size_t)(2 + 2 * i) * D + i] -= eps;
  }
  if (gnuts_log_prob_grad(model, n, q.data(), 1, lp.data(), g.data()) != GNUTS_OK)
    throw std::runtime_error("Error during gradient test:\n" + last_error());
  std::ostringstream rep;
  rep << "TEST GRADIENT MODE\n\n Log probability=" << fmt(lp[0], 6) << "\n\n";
  char line[256];
  snprintf(line, sizeof line, " %10s %16s %16s %16s %16s\n", "param idx", "value", "model", "finite diff", "error");
  rep << line;
  int failed = 0;
  for (int i = 0; i < D; ++i) {
    const double fd = (lp[1 + 2 * i] - lp[2 + 2 * i]) / (2 * eps);
    const double e = g[i] - fd;
    if (std::fabs(e) > tol) ++failed;
    snprintf(line, sizeof line, " %10d %16s %16s %16s %16s\n", i, fmt(q0[i], 6).c_str(), fmt(g[i], 6).c_str(),
             fmt(fd, 6).c_str(), fmt(e, 6).c_str());
    rep << line;
  }
  std::cout << rep.str() << std::endl;
  const std::string file = cfg.output->child("file")->sval;
  std::ofstream f(file);
  if (!f) throw std::runtime_error("Can't open output file " + file);
  write_csv_header(f, model, cfg_lines);
  std::istringstream is(rep.str());
  std::string l;
  while (std::getline(is, l)) f << "# " << l << "\n";
  if (failed) std::cout << failed << " of " << D << " gradient components differ by more than error=" << tol << std::endl;
  return OK;
}

}  // namespace

int main(int argc, char** argv) {
  // ---- model selection
  std::string model_id;
  int first = 1;
  if (argc > 1 && std::strncmp(argv[1], "model=", 6) == 0) {
    model_id = argv[1] + 6;
    first = 2;
  } else {
    std::string exe = argv[0];
    const size_t sep = exe.find_last_of('/');
    model_id = sep == std::string::npos ? exe : exe.substr(sep + 1);
  }

  // ---- arguments (command.hpp:97-118)
  Config cfg;
  if (argc <= first) {
    std::cout << "Usage: " << argv[0] << " [model=<id>] sample <subargs> [id=<n>] [data file=<json>] [init=<x|json>]"
              << " [random seed=<n>] [output file=<csv> refresh=<n> sig_figs=<n>]" << std::endl;
    return NOT_OK;
  }
  ParseState st;
  const bool parsed = cfg.parse(argc, argv, first, st);
  for (auto& e : st.errors) std::cerr << e << std::endl;
  if (st.help) {
    std::cout << "Usage: " << argv[0] << " [model=<id>] sample num_samples=<n> num_warmup=<n> save_warmup=<b> thin=<n>"
              << " adapt [engaged=<b> gamma delta kappa t0 init_buffer term_buffer window save_metric=<b>]"
              << " algorithm=hmc engine=nuts max_depth=<n> metric=unit_e|diag_e|dense_e metric_file=<json>"
              << " stepsize=<x> stepsize_jitter=<x> num_chains=<n> id=<n> data file=<json> init=<x|json>"
              << " random seed=<n> output file=<csv> refresh=<n> sig_figs=<n> save_cmdstan_config=<b>" << std::endl;
    return OK;
  }
  if (!parsed) {
    std::cerr << "Failed to parse command arguments, cannot run model." << std::endl;
    return NOT_OK;
  }
  try {
    const std::string method = cfg.method->value_text();
    if (method == "log_prob") return run_log_prob(cfg, model_id, cfg.method->child("log_prob"));
    if (method == "diagnose") return run_diagnose(cfg, model_id, cfg.method->child("diagnose"));
    if (method != "sample")
      throw std::runtime_error("method=" + method + " is not provided by gnuts-sample; it runs method=sample "
                               "(algorithm=hmc engine=nuts)");
    Arg* sample = cfg.sample();
    Arg* adapt = cfg.adapt();
    Arg* algo = sample->child("algorithm");
    if (algo->value_text() != "hmc")
      throw std::runtime_error("algorithm=" + algo->value_text() + " is not provided by gnuts-sample; use algorithm=hmc");
    Arg* hmc = cfg.hmc();
    Arg* engine = hmc->child("engine");
    if (engine->value_text() != "nuts")
      throw std::runtime_error("engine=" + engine->value_text() + " is not provided by gnuts-sample; use engine=nuts");
    const std::string metric = hmc->child("metric")->value_text();
    Arg* out_grp = cfg.output.get();
    const std::string output_file = out_grp->child("file")->sval;
    const std::string diagnostic_file = out_grp->child("diagnostic_file")->sval;
    const int sig_figs = (int)out_grp->child("sig_figs")->ival;
    const int prec = sig_figs < 0 ? 6 : sig_figs;
    const int refresh = (int)out_grp->child("refresh")->ival;
    const unsigned id = (unsigned)cfg.id->ival;
    const int num_chains = (int)sample->child("num_chains")->ival;
    const int num_warmup = (int)sample->child("num_warmup")->ival;
    const int num_samples = (int)sample->child("num_samples")->ival;
    const int thin = (int)sample->child("thin")->ival;
    const bool save_warmup = sample->child("save_warmup")->bval;
    const bool engaged = adapt->child("engaged")->bval;
    const bool save_metric = adapt->child("save_metric")->bval;

    // seed -1: a seed from the clock (arg_seed.hpp)
    const long long seed_arg = cfg.random->children[0]->ival;
    cfg.random_seed = seed_arg >= 0
                          ? (unsigned)seed_arg
                          : (unsigned)(std::chrono::system_clock::now().time_since_epoch().count() & 0xFFFFFFFFu);

    // config echo (command.hpp:153-157)
    const auto cfg_lines = cfg.lines();
    for (auto& l : cfg_lines) std::cout << l << std::endl;
    std::cout << std::endl;

    if (engaged && num_warmup == 0)
      throw std::runtime_error("The number of warmup samples (num_warmup) must be greater than zero if adaptation "
                               "is enabled.");
    if (save_metric && !engaged)
      throw std::runtime_error("Saving the adapted metric (save_metric=1) can only be enabled when adaptation is "
                               "engaged (adapt engaged=1)");

    // ---- data + model (command.hpp:166-171)
    const std::string data_file = cfg.data->children[0]->sval;
    const std::string data_text = data_file.empty() ? std::string("{}") : read_file(data_file);
    gnuts_model* model = nullptr;
    if (gnuts_model_create_json(model_id.c_str(), data_text.c_str(), cfg.random_seed, &model) != GNUTS_OK)
      throw std::runtime_error("Error creating model '" + model_id + "': " + last_error());
    struct ModelGuard { gnuts_model* m; ~ModelGuard() { gnuts_model_destroy(m); } } mg{model};
    int D = 0, ncon = 0;
    gnuts_model_dims(model, &D, &ncon);
    char nb[256];
    gnuts_model_name(model, nb, sizeof nb);
    const std::string model_name = nb;

    // ---- inits (command.hpp:264-276): a radius or JSON file(s) of constrained values
    const std::string init = cfg.init->sval;
    double init_radius = 2.0;
    bool init_is_radius = true;
    try {
      size_t used = 0;
      init_radius = std::stod(init, &used);
      if (used != init.size()) init_is_radius = false;
    } catch (...) {
      init_is_radius = false;
    }
    std::vector<double> inits;
    if (!init_is_radius) {
      auto files = per_chain_inputs(init, num_chains, id);
      inits.resize((size_t)num_chains * D);
      for (int c = 0; c < num_chains; ++c) {
        JValue obj = JParser(read_file(files[c])).parse();
        auto con = constrained_from_json(model, obj, D, files[c]);
        if (gnuts_unconstrain(model, con.data(), inits.data() + (size_t)c * D) != GNUTS_OK)
          throw std::runtime_error("Error transforming the initial values of " + files[c] + ": " + last_error());
      }
      init_radius = 0;
    } else if (init_radius < 0) {
      throw std::runtime_error("init radius must be non-negative");
    }

    // ---- metric file(s) (command.hpp:593-596)
    const std::string metric_file = hmc->child("metric_file")->sval;
    std::vector<double> inv_metric;
    const size_t msz = metric == "dense_e" ? (size_t)D * D : (size_t)D;
    if (!metric_file.empty() && metric != "unit_e") {
      auto files = per_chain_inputs(metric_file, num_chains, id);
      inv_metric.resize((size_t)num_chains * msz);
      for (int c = 0; c < num_chains; ++c) {
        JValue obj = JParser(read_file(files[c])).parse();
        const JValue* v = obj.get("inv_metric");
        if (!v) throw std::runtime_error("variable inv_metric not found in metric file " + files[c]);
        std::vector<double> flat;
        v->flatten(flat);
        if (flat.size() != msz)
          throw std::runtime_error("inv_metric in " + files[c] + " has " + std::to_string(flat.size()) +
                                   " elements; expecting " + std::to_string(msz));
        std::copy(flat.begin(), flat.end(), inv_metric.begin() + (long)(c * msz));
      }
    }

    // ---- run (command.hpp:607-697)
    gnuts_sample_args a;
    gnuts_sample_args_default(&a);
    a.num_chains = num_chains;
    a.chain_id = id;
    a.seed = cfg.random_seed;
    a.init_radius = init_radius;
    a.num_warmup = num_warmup;
    a.num_samples = num_samples;
    a.thin = thin;
    a.save_warmup = save_warmup;
    a.refresh = refresh;
    a.stepsize = hmc->child("stepsize")->rval;
    a.stepsize_jitter = hmc->child("stepsize_jitter")->rval;
    a.max_depth = (int)engine->child("nuts")->child("max_depth")->ival;
    a.delta = adapt->child("delta")->rval;
    a.gamma = adapt->child("gamma")->rval;
    a.kappa = adapt->child("kappa")->rval;
    a.t0 = adapt->child("t0")->rval;
    a.init_buffer = (unsigned)adapt->child("init_buffer")->ival;
    a.term_buffer = (unsigned)adapt->child("term_buffer")->ival;
    a.window = (unsigned)adapt->child("window")->ival;
    a.precision = cfg.gpu->child("precision")->value_text() == "mixed" ? GNUTS_PRECISION_MIXED : GNUTS_PRECISION_FP64;
    if (const char* p = std::getenv("GNUTS_PRECISION")) a.precision = std::string(p) == "mixed" ? 1 : 0;
    const bool learned = cfg.gpu->child("learned")->bval;
    if (learned && (metric != "diag_e" || !engaged))
      throw std::runtime_error("gpu learned=1 needs metric=diag_e with adaptation engaged");

    const int n_saved = (save_warmup ? (num_warmup + thin - 1) / thin : 0) + (num_samples + thin - 1) / thin;
    const int ncol = 7 + ncon;
    std::vector<double> draws((size_t)num_chains * n_saved * ncol), eps(num_chains), minv((size_t)num_chains * msz);
    std::vector<double> wsec(num_chains), ssec(num_chains), timing(GNUTS_TIMING_FIELDS);
    std::vector<int64_t> ngrad(num_chains), nlf(num_chains);
    std::vector<int> status(num_chains);
    // diagnostic_file rows (command.hpp:225-247): sampler columns, q, p, g
    std::vector<double> diag;
    if (!diagnostic_file.empty()) {
      if (learned) throw std::runtime_error("output diagnostic_file is not provided with gpu learned=1");
      diag.resize((size_t)num_chains * n_saved * (7 + 3 * (size_t)D));
    }
    gnuts_output out{};
    out.draws = draws.data();
    out.diagnostics = diag.empty() ? nullptr : diag.data();
    out.stepsize = eps.data();
    out.inv_metric = minv.data();
    out.warmup_seconds = wsec.data();
    out.sampling_seconds = ssec.data();
    out.n_grad = ngrad.data();
    out.chain_status = status.data();
    out.n_leapfrog = nlf.data();
    out.timing = timing.data();
    Progress prog{num_chains, id};
    const double* ip = inits.empty() ? nullptr : inits.data();
    const double* mp = inv_metric.empty() ? nullptr : inv_metric.data();
    int rc;
    gnuts_progress_fn pf = refresh > 0 ? on_progress : nullptr;
    if (learned) {
      // warmup and judge pilots run inside; out receives the kept sampler's draws
      gnuts_learned_args la;
      gnuts_learned_args_default(&la);
      gnuts_learned_report rep;
      rc = gnuts_hmc_nuts_learned_diag_e_adapt(model, &a, &la, ip, &out, &rep, pf, &prog);
      if (rc == GNUTS_OK)
        std::cout << "Learned preconditioner: " << (rep.used_flow ? "kept" : "rejected, plain NUTS kept")
                  << " (pilot ESS per gradient " << fmt(rep.flow_ess_per_grad, 3) << " vs "
                  << fmt(rep.plain_ess_per_grad, 3) << ", divergences " << fmt(rep.flow_divergence_rate, 3)
                  << " vs " << fmt(rep.plain_divergence_rate, 3) << ", max R-hat " << fmt(rep.flow_max_rhat, 4)
                  << " vs " << fmt(rep.plain_max_rhat, 4) << ")" << std::endl;
    } else if (engaged) {
      if (metric == "dense_e") rc = gnuts_hmc_nuts_dense_e_adapt(model, &a, ip, mp, &out, pf, &prog);
      else if (metric == "diag_e") rc = gnuts_hmc_nuts_diag_e_adapt(model, &a, ip, mp, &out, pf, &prog);
      else rc = gnuts_hmc_nuts_unit_e_adapt(model, &a, ip, &out, pf, &prog);
    } else {
      if (metric == "dense_e") rc = gnuts_hmc_nuts_dense_e(model, &a, ip, mp, &out, pf, &prog);
      else if (metric == "diag_e") rc = gnuts_hmc_nuts_diag_e(model, &a, ip, mp, &out, pf, &prog);
      else rc = gnuts_hmc_nuts_unit_e(model, &a, ip, &out, pf, &prog);
    }
    if (rc != GNUTS_OK) throw std::runtime_error(last_error());

    // ---- Stan CSV per chain
    std::vector<std::string> names;
    for (int i = 0; i < ncon; ++i) {
      gnuts_model_param_name(model, i, 0, nb, sizeof nb);
      names.push_back(nb);
    }
    const auto csv_names = make_filenames(output_file, "", ".csv", num_chains, id);
    const int n_warm_saved = save_warmup ? (num_warmup + thin - 1) / thin : 0;
    const std::string datetime = utc_now();
    // one file per chain (file.hpp:189-212), formatted on all host cores:
    // chains are claimed from an atomic counter; the console lines and the
    // first error are reported in chain order afterwards
    std::vector<std::string> chain_msg(num_chains), chain_err(num_chains);
    auto write_chain = [&](int c) {
      std::ofstream f(csv_names[c]);
      if (!f) {
        chain_err[c] = "Can't open output file " + csv_names[c];
        return;
      }
      f << "# stan_version_major = 2\n# stan_version_minor = 36\n# stan_version_patch = 0\n";
      f << "# model = " << model_name << "\n# start_datetime = " << datetime << "\n";
      for (auto& l : cfg_lines) f << "# " << l << "\n";
      f << "# stanc_version = gnuts built-in model\n# stancflags = \n# gnuts_version = " << gnuts_version() << "\n";
      f << "lp__,accept_stat__,stepsize__,treedepth__,n_leapfrog__,divergent__,energy__";
      for (auto& n : names) f << "," << n;
      f << "\n";
      auto write_rows = [&](int r0, int r1) {
        std::string line;
        for (int r = r0; r < r1; ++r) {
          const double* row = draws.data() + ((size_t)c * n_saved + r) * ncol;
          line.clear();
          for (int k = 0; k < ncol; ++k) {
            if (k) line += ',';
            line += fmt(row[k], prec);
          }
          line += '\n';
          f << line;
        }
      };
      write_rows(0, n_warm_saved);
      // the sampler state after warmup (run_adaptive_sampler / run_sampler)
      if (engaged) f << "# Adaptation terminated\n";
      f << "# Step size = " << fmt(eps[c], 6) << "\n";
      const double* mv = minv.data() + (size_t)c * msz;
      if (metric == "diag_e") {
        f << "# Diagonal elements of inverse mass matrix:\n# ";
        for (int i = 0; i < D; ++i) f << (i ? ", " : "") << fmt(mv[i], 6);
        f << "\n";
      } else if (metric == "dense_e") {
        f << "# Elements of inverse mass matrix:\n";
        for (int i = 0; i < D; ++i) {
          f << "# ";
          for (int j = 0; j < D; ++j) f << (j ? ", " : "") << fmt(mv[(size_t)i * D + j], 6);
          f << "\n";
        }
      } else {
        f << "# No free parameters for unit metric\n";
      }
      write_rows(n_warm_saved, n_saved);
      const double w = wsec[c], s = ssec[c];
      f << "# \n#  Elapsed Time: " << fmt(w, 6) << " seconds (Warm-up)\n";
      f << "#                " << fmt(s, 6) << " seconds (Sampling)\n";
      f << "#                " << fmt(w + s, 6) << " seconds (Total)\n# \n";
      if (!f) {
        chain_err[c] = "error writing " + csv_names[c];
        return;
      }
      chain_msg[c] = (num_chains > 1 ? "Chain [" + std::to_string(id + (unsigned)c) + "] " : std::string()) +
                     "Elapsed Time: " + fmt(w, 6) + " seconds (Warm-up), " + fmt(s, 6) + " seconds (Sampling), " +
                     fmt(w + s, 6) + " seconds (Total)";
    };
    {
      const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
      const int nt = std::min(hw, num_chains);
      std::atomic<int> next{0};
      auto worker = [&]() {
        for (int c = next++; c < num_chains; c = next++) write_chain(c);
      };
      std::vector<std::thread> pool;
      for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
      worker();
      for (auto& t : pool) t.join();
    }
    for (int c = 0; c < num_chains; ++c) {
      if (!chain_err[c].empty()) throw std::runtime_error(chain_err[c]);
      std::cout << chain_msg[c] << std::endl;
    }

    // ---- diagnostic_file per chain (file names as the output files', file.hpp:189-212):
    // the config block, then one row per saved iteration
    if (!diag.empty()) {
      std::vector<std::string> unames;
      for (int i = 0; i < D; ++i) {
        gnuts_model_param_name(model, i, 1, nb, sizeof nb);
        unames.push_back(nb);
      }
      const auto dnames = make_filenames(diagnostic_file, "", ".csv", num_chains, id);
      const size_t dcol = 7 + 3 * (size_t)D;
      for (int c = 0; c < num_chains; ++c) {
        std::ofstream f(dnames[c]);
        if (!f) throw std::runtime_error("Can't open diagnostic file " + dnames[c]);
        f << "# stan_version_major = 2\n# stan_version_minor = 36\n# stan_version_patch = 0\n";
        f << "# model = " << model_name << "\n# start_datetime = " << datetime << "\n";
        for (auto& l : cfg_lines) f << "# " << l << "\n";
        f << "lp__,accept_stat__,stepsize__,treedepth__,n_leapfrog__,divergent__,energy__";
        for (auto& n : unames) f << "," << n;
        for (auto& n : unames) f << ",p_" << n;
        for (auto& n : unames) f << ",g_" << n;
        f << "\n";
        std::string line;
        for (int r = 0; r < n_saved; ++r) {
          const double* row = diag.data() + ((size_t)c * n_saved + r) * dcol;
          line.clear();
          for (size_t k = 0; k < dcol; ++k) {
            if (k) line += ',';
            line += fmt(row[k], prec);
          }
          line += '\n';
          f << line;
        }
        if (!f) throw std::runtime_error("error writing " + dnames[c]);
      }
    }

    // ---- adapted metric as JSON (command.hpp:247-261)
    if (save_metric) {
      const auto mnames = make_filenames(output_file, "_metric", ".json", num_chains, id);
      for (int c = 0; c < num_chains; ++c) {
        std::ofstream f(mnames[c]);
        if (!f) throw std::runtime_error("Can't open output file " + mnames[c]);
        const double* mv = minv.data() + (size_t)c * msz;
        f << "{\n  \"stepsize\": " << json_number(eps[c], prec) << ",\n  \"metric_type\": \"" << metric
          << "\",\n  \"inv_metric\": [";
        if (metric == "dense_e") {
          for (int i = 0; i < D; ++i) {
            f << (i ? ", " : "") << "[";
            for (int j = 0; j < D; ++j) f << (j ? ", " : "") << json_number(mv[(size_t)i * D + j], prec);
            f << "]";
          }
        } else {
          for (int i = 0; i < D; ++i) f << (i ? ", " : "") << json_number(mv[i], prec);
        }
        f << "]\n}\n";
      }
    }

    // ---- configuration as JSON (output save_cmdstan_config)
    if (out_grp->child("save_cmdstan_config")->bval) {
      const auto cnames = make_filenames(output_file, "_config", ".json", 1, id);
      std::ofstream f(cnames[0]);
      f << "{\n  \"stan_major_version\": \"2\",\n  \"stan_minor_version\": \"36\",\n  \"stan_patch_version\": \"0\",\n";
      f << "  \"model_name\": \"" << model_name << "\",\n  \"start_datetime\": \"" << datetime << "\",\n";
      f << "  \"method\": \"sample\",\n  \"num_samples\": " << num_samples << ",\n  \"num_warmup\": " << num_warmup
        << ",\n  \"save_warmup\": " << (save_warmup ? "true" : "false") << ",\n  \"thin\": " << thin
        << ",\n  \"adapt_engaged\": " << (engaged ? "true" : "false") << ",\n  \"metric\": \"" << metric
        << "\",\n  \"num_chains\": " << num_chains << ",\n  \"id\": " << id << ",\n  \"seed\": " << cfg.random_seed
        << ",\n  \"data_file\": \"" << data_file << "\",\n  \"output_file\": \"" << output_file << "\"\n}\n";
    }
    bool all_ok = true;
    for (int c = 0; c < num_chains; ++c) all_ok &= status[c] == GNUTS_OK;
    return all_ok ? OK : NOT_OK;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return NOT_OK;
  }
}
