// Minimal JSON value, reader and writer for config.json / result.json.
//
// The reference reads config.json and rewrites result.json through nlohmann::json
// (src/config.h, src/result.h); that library is not part of this build, so the driver uses
// this small one.  Objects keep their keys sorted (as nlohmann's default std::map does), so
// dumps are ordered like the reference's.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace shci_cli {

struct Json {
  enum Type { Null, Bool, Number, String, Array, Object } type = Null;
  bool b = false;
  double num = 0.0;
  bool is_int = false;
  std::string str;
  std::vector<Json> arr;
  std::map<std::string, Json> obj;

  static Json number(double v) {
    Json j;
    j.type = Number;
    j.num = v;
    return j;
  }
  static Json string(const std::string& s) {
    Json j;
    j.type = String;
    j.str = s;
    return j;
  }

  const Json* get(const std::string& path) const {
    const Json* cur = this;
    std::stringstream ss(path);
    std::string key;
    while (std::getline(ss, key, '/')) {
      if (key.empty()) continue;
      if (cur->type != Object) return nullptr;
      auto it = cur->obj.find(key);
      if (it == cur->obj.end()) return nullptr;
      cur = &it->second;
    }
    return cur;
  }
  Json& put(const std::string& path) {
    Json* cur = this;
    std::stringstream ss(path);
    std::string key;
    while (std::getline(ss, key, '/')) {
      if (key.empty()) continue;
      if (cur->type != Object) {
        *cur = Json();
        cur->type = Object;
      }
      cur = &cur->obj[key];
    }
    return *cur;
  }
};

class Parser {
 public:
  explicit Parser(const std::string& s) : s_(s) {}
  Json parse() {
    Json v = value();
    ws();
    if (i_ != s_.size()) fail("trailing characters");
    return v;
  }

 private:
  const std::string& s_;
  size_t i_ = 0;
  [[noreturn]] void fail(const char* m) {
    throw std::runtime_error(std::string("JSON parse error: ") + m + " at offset " +
                             std::to_string(i_));
  }
  void ws() {
    while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\n' || s_[i_] == '\t' || s_[i_] == '\r'))
      i_++;
  }
  Json value() {
    ws();
    if (i_ >= s_.size()) fail("unexpected end");
    const char c = s_[i_];
    if (c == '{') return object();
    if (c == '[') return array();
    if (c == '"') return Json::string(string());
    if (s_.compare(i_, 4, "true") == 0) {
      i_ += 4;
      Json j;
      j.type = Json::Bool;
      j.b = true;
      return j;
    }
    if (s_.compare(i_, 5, "false") == 0) {
      i_ += 5;
      Json j;
      j.type = Json::Bool;
      return j;
    }
    if (s_.compare(i_, 4, "null") == 0) {
      i_ += 4;
      return Json();
    }
    return number();
  }
  Json number() {
    const char* start = s_.c_str() + i_;
    char* end = nullptr;
    const double v = std::strtod(start, &end);
    if (end == start) fail("bad number");
    bool integral = true;
    for (const char* p = start; p < end; p++)
      if (*p == '.' || *p == 'e' || *p == 'E') integral = false;
    i_ += static_cast<size_t>(end - start);
    Json j = Json::number(v);
    j.is_int = integral;
    return j;
  }
  std::string string() {
    std::string out;
    i_++;  // opening quote
    while (i_ < s_.size() && s_[i_] != '"') {
      if (s_[i_] == '\\' && i_ + 1 < s_.size()) {
        i_++;
        const char e = s_[i_];
        out.push_back(e == 'n' ? '\n' : e == 't' ? '\t' : e);
      } else {
        out.push_back(s_[i_]);
      }
      i_++;
    }
    if (i_ >= s_.size()) fail("unterminated string");
    i_++;
    return out;
  }
  Json array() {
    Json j;
    j.type = Json::Array;
    i_++;
    ws();
    if (i_ < s_.size() && s_[i_] == ']') {
      i_++;
      return j;
    }
    while (true) {
      j.arr.push_back(value());
      ws();
      if (i_ < s_.size() && s_[i_] == ',') {
        i_++;
        continue;
      }
      if (i_ < s_.size() && s_[i_] == ']') {
        i_++;
        return j;
      }
      fail("expected , or ]");
    }
  }
  Json object() {
    Json j;
    j.type = Json::Object;
    i_++;
    ws();
    if (i_ < s_.size() && s_[i_] == '}') {
      i_++;
      return j;
    }
    while (true) {
      ws();
      if (i_ >= s_.size() || s_[i_] != '"') fail("expected key");
      const std::string k = string();
      ws();
      if (i_ >= s_.size() || s_[i_] != ':') fail("expected :");
      i_++;
      j.obj[k] = value();
      ws();
      if (i_ < s_.size() && s_[i_] == ',') {
        i_++;
        continue;
      }
      if (i_ < s_.size() && s_[i_] == '}') {
        i_++;
        return j;
      }
      fail("expected , or }");
    }
  }
};

// Shortest representation that reads back to the same double.
inline std::string fmt_double(double v) {
  if (std::isnan(v)) return "NaN";
  if (std::isinf(v)) return v > 0 ? "Infinity" : "-Infinity";
  char buf[40];
  for (int prec = 15; prec <= 17; prec++) {
    std::snprintf(buf, sizeof(buf), "%.*g", prec, v);
    if (std::strtod(buf, nullptr) == v) break;
  }
  std::string s(buf);
  if (s.find_first_of(".eE") == std::string::npos && s.find("inf") == std::string::npos)
    s += ".0";
  return s;
}

inline void dump(const Json& j, std::string& out, int indent, int level) {
  const std::string pad(static_cast<size_t>(indent * (level + 1)), ' ');
  const std::string pad0(static_cast<size_t>(indent * level), ' ');
  switch (j.type) {
    case Json::Null: out += "null"; break;
    case Json::Bool: out += j.b ? "true" : "false"; break;
    case Json::Number:
      if (j.is_int && std::fabs(j.num) < 9e15) {
        out += std::to_string(static_cast<long long>(j.num));
      } else {
        out += fmt_double(j.num);
      }
      break;
    case Json::String: out += "\"" + j.str + "\""; break;
    case Json::Array:
      if (j.arr.empty()) {
        out += "[]";
        break;
      }
      out += "[\n";
      for (size_t k = 0; k < j.arr.size(); k++) {
        out += pad;
        dump(j.arr[k], out, indent, level + 1);
        out += k + 1 < j.arr.size() ? ",\n" : "\n";
      }
      out += pad0 + "]";
      break;
    case Json::Object: {
      if (j.obj.empty()) {
        out += "{}";
        break;
      }
      out += "{\n";
      size_t k = 0;
      for (const auto& kv : j.obj) {
        out += pad + "\"" + kv.first + "\": ";
        dump(kv.second, out, indent, level + 1);
        out += ++k < j.obj.size() ? ",\n" : "\n";
      }
      out += pad0 + "}";
      break;
    }
  }
}

inline std::string dump(const Json& j) {
  std::string s;
  dump(j, s, 2, 0);
  return s;
}

}  // namespace shci_cli
