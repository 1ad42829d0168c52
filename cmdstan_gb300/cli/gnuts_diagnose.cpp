// gnuts-diagnose: CmdStan's bin/diagnose (src/cmdstan/diagnose.cpp) over
// Stan CSV files, one chain per file, with the checks computed by
// gnuts_diagnose (include/gnuts.h).  Usage, messages and exit codes follow the
// reference: no arguments print the usage and exit 0; unreadable files are
// reported and skipped; no readable file, or a file that does not parse,
// exits 1 (return_codes::NOT_OK).  --gpu computes the ESS / R-hat statistics
// on the GPU (the first argument only).
#include <gnuts.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

namespace {

struct Csv {
  std::vector<std::string> names;
  std::vector<double> rows;  // row-major, names.size() per draw
  int max_depth = 10;
  size_t n_draws() const { return names.empty() ? 0 : rows.size() / names.size(); }
};

std::vector<std::string> split(const std::string& s, char c) {
  std::vector<std::string> v;
  std::string cur;
  std::istringstream in(s);
  while (std::getline(in, cur, c)) v.push_back(cur);
  return v;
}

// comment lines (config block with "max_depth = N", adaptation block, timing
// trailer), one header line, then one line of numbers per draw
bool parse(std::istream& in, Csv& out, std::string& err) {
  std::string line;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.empty()) continue;
    if (line[0] == '#') {
      const size_t p = line.find("max_depth =");
      if (p != std::string::npos && out.names.empty()) out.max_depth = std::atoi(line.c_str() + p + 11);
      continue;
    }
    if (out.names.empty()) {
      out.names = split(line, ',');
      continue;
    }
    const std::vector<std::string> f = split(line, ',');
    if (f.size() != out.names.size()) {
      err = ": draw line with " + std::to_string(f.size()) + " values, header has " + std::to_string(out.names.size());
      return false;
    }
    for (const std::string& v : f) {
      char* end = nullptr;
      const double x = std::strtod(v.c_str(), &end);
      if (end == v.c_str()) {
        err = ": not a number: " + v;
        return false;
      }
      out.rows.push_back(x);
    }
  }
  if (out.names.empty()) {
    err = ": no header line";
    return false;
  }
  return true;
}

}  // namespace

int main(int argc, const char* argv[]) {
  int first = 1, use_gpu = 0;
  if (argc > 1 && std::string(argv[1]) == "--gpu") {
    use_gpu = 1;
    first = 2;
  }
  if (argc == first) {
    std::cout << "USAGE:  diagnose <filename 1> [<filename 2> ... <filename N>]" << std::endl << std::endl;
    return 0;
  }
  std::vector<std::string> files;
  for (int i = first; i < argc; ++i) {
    std::ifstream f(argv[i]);
    if (f.good()) files.push_back(argv[i]);
    else std::cout << "File " << argv[i] << " not found" << std::endl;
  }
  if (files.empty()) {
    std::cout << "No valid input files, exiting." << std::endl;
    return 1;
  }
  std::vector<Csv> chains(files.size());
  for (size_t i = 0; i < files.size(); ++i) {
    std::ifstream f(files[i]);
    std::string err;
    if (!parse(f, chains[i], err)) {
      std::cout << "Cannot parse input csv file: " << files[i] << err << "." << std::endl;
      return 1;
    }
    if (chains[i].names != chains[0].names || chains[i].n_draws() != chains[0].n_draws()) {
      std::cout << "Cannot parse input csv file: " << files[i] << ": columns or number of draws differ from "
                << files[0] << "." << std::endl;
      return 1;
    }
  }
  const Csv& c0 = chains[0];
  const int C = (int)chains.size(), n = (int)c0.n_draws(), K = (int)c0.names.size();
  std::vector<double> draws;
  for (const Csv& c : chains) draws.insert(draws.end(), c.rows.begin(), c.rows.end());
  auto col = [&](const char* nm) {
    for (int j = 0; j < K; ++j)
      if (c0.names[j] == nm) return j;
    return -1;
  };
  std::vector<int> pcols;
  std::string pnames;
  for (int j = 0; j < K; ++j)
    if (c0.names[j].find("__") == std::string::npos) {
      pcols.push_back(j);
      pnames += (pnames.empty() ? "" : "\n") + c0.names[j];
    }
  std::vector<char> report(65536 + 64 * pnames.size());
  gnuts_diagnosis res;
  const int rc = gnuts_diagnose(draws.data(), C, n, (int64_t)n * K, K, col("treedepth__"), col("divergent__"),
                                col("energy__"), pcols.data(), (int)pcols.size(), pnames.c_str(), c0.max_depth,
                                use_gpu, 0, report.data(), report.size(), &res);
  if (rc != GNUTS_OK) {
    char msg[512];
    gnuts_last_error(msg, sizeof msg);
    std::cout << "diagnose failed: " << msg << std::endl;
    return 1;
  }
  std::cout << report.data();
  return 0;
}
