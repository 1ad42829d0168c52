// Minimal JSON reader / writer for the command line's input files (data,
// inits, metric) and its metric output.  Stan JSON conventions: numbers are
// doubles, "NaN" / "Inf" / "Infinity" / "-Inf" / "-Infinity" strings are the
// IEEE specials, nested arrays are row-major.
#pragma once
#include <cmath>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace gnuts_cli {

struct JValue {
  enum Type { NUL, BOOL, NUM, STR, ARR, OBJ } type = NUL;
  double num = 0;
  bool b = false;
  std::string str;
  std::vector<JValue> arr;
  std::vector<std::pair<std::string, JValue>> obj;

  const JValue* get(const std::string& k) const {
    for (auto& kv : obj)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
  // numeric value (numbers and the special strings)
  bool as_number(double& out) const {
    if (type == NUM) { out = num; return true; }
    if (type == BOOL) { out = b ? 1 : 0; return true; }
    if (type == STR) {
      if (str == "NaN") { out = NAN; return true; }
      if (str == "Inf" || str == "Infinity" || str == "+Inf" || str == "+Infinity") { out = INFINITY; return true; }
      if (str == "-Inf" || str == "-Infinity") { out = -INFINITY; return true; }
    }
    return false;
  }
  // all numbers of a (possibly nested) array in row-major order
  void flatten(std::vector<double>& out) const {
    if (type == ARR) {
      for (auto& e : arr) e.flatten(out);
      return;
    }
    double v;
    if (!as_number(v)) throw std::runtime_error("non-numeric value in array");
    out.push_back(v);
  }
};

class JParser {
 public:
  explicit JParser(const std::string& s) : s_(s) {}
  JValue parse() {
    JValue v = value();
    ws();
    if (i_ != s_.size()) fail("trailing characters");
    return v;
  }

 private:
  const std::string& s_;
  size_t i_ = 0;
  [[noreturn]] void fail(const std::string& m) {
    throw std::runtime_error("JSON parse error at offset " + std::to_string(i_) + ": " + m);
  }
  void ws() {
    while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\t' || s_[i_] == '\n' || s_[i_] == '\r')) ++i_;
  }
  bool lit(const char* w) {
    size_t n = 0;
    while (w[n]) ++n;
    if (s_.compare(i_, n, w) == 0) { i_ += n; return true; }
    return false;
  }
  std::string string_lit() {
    if (s_[i_] != '"') fail("expected string");
    ++i_;
    std::string out;
    while (i_ < s_.size() && s_[i_] != '"') {
      char c = s_[i_++];
      if (c == '\\') {
        if (i_ >= s_.size()) fail("bad escape");
        char e = s_[i_++];
        switch (e) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'u': {
            if (i_ + 4 > s_.size()) fail("bad unicode escape");
            unsigned cp = (unsigned)std::strtoul(s_.substr(i_, 4).c_str(), nullptr, 16);
            i_ += 4;
            if (cp < 0x80) out += (char)cp;
            else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
            else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
            break;
          }
          default: out += e;
        }
      } else {
        out += c;
      }
    }
    if (i_ >= s_.size()) fail("unterminated string");
    ++i_;
    return out;
  }
  JValue value() {
    ws();
    if (i_ >= s_.size()) fail("unexpected end");
    JValue v;
    const char c = s_[i_];
    if (c == '{') {
      ++i_;
      v.type = JValue::OBJ;
      ws();
      if (s_[i_] == '}') { ++i_; return v; }
      for (;;) {
        ws();
        std::string k = string_lit();
        ws();
        if (s_[i_] != ':') fail("expected ':'");
        ++i_;
        v.obj.emplace_back(k, value());
        ws();
        if (s_[i_] == ',') { ++i_; continue; }
        if (s_[i_] == '}') { ++i_; break; }
        fail("expected ',' or '}'");
      }
    } else if (c == '[') {
      ++i_;
      v.type = JValue::ARR;
      ws();
      if (s_[i_] == ']') { ++i_; return v; }
      for (;;) {
        v.arr.push_back(value());
        ws();
        if (s_[i_] == ',') { ++i_; continue; }
        if (s_[i_] == ']') { ++i_; break; }
        fail("expected ',' or ']'");
      }
    } else if (c == '"') {
      v.type = JValue::STR;
      v.str = string_lit();
    } else if (lit("true")) {
      v.type = JValue::BOOL; v.b = true;
    } else if (lit("false")) {
      v.type = JValue::BOOL; v.b = false;
    } else if (lit("null")) {
      v.type = JValue::NUL;
    } else if (lit("NaN")) {
      v.type = JValue::NUM; v.num = NAN;
    } else if (lit("Infinity") || lit("Inf")) {
      v.type = JValue::NUM; v.num = INFINITY;
    } else if (lit("-Infinity") || lit("-Inf")) {
      v.type = JValue::NUM; v.num = -INFINITY;
    } else {
      const char* b = s_.c_str() + i_;
      char* e = nullptr;
      v.num = std::strtod(b, &e);
      if (e == b) fail("unexpected character");
      i_ += (size_t)(e - b);
      v.type = JValue::NUM;
    }
    return v;
  }
};

inline std::string json_number(double v, int prec = 17) {
  if (std::isnan(v)) return "NaN";
  if (std::isinf(v)) return v > 0 ? "Infinity" : "-Infinity";
  char buf[64];
  snprintf(buf, sizeof buf, "%.*g", prec, v);
  return buf;
}

}  // namespace gnuts_cli
