// Minimal stand-in for the part of nlohmann::json the reference's predictor
// constructors use: `istream >> json`, `items()` with structured bindings,
// `at(key)`, `get<std::vector<double>>()`, `get<std::vector<std::vector<double>>>()`
// and implicit conversion to double.
//
// Test infrastructure only (lets the reference sources compile without the
// library). Written from the JSON grammar (RFC 8259) and nlohmann's documented
// API. Objects iterate in sorted key order, as nlohmann::json (std::map) does.
#ifndef LMC_ORACLE_SHIM_NLOHMANN_JSON_
#define LMC_ORACLE_SHIM_NLOHMANN_JSON_
#include <cctype>
#include <cstdlib>
#include <istream>
#include <iterator>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace nlohmann {
class json {
 public:
  enum class Kind { Null, Bool, Number, String, Array, Object };
  json() = default;

  const json &at(const std::string &key) const {
    if (kind_ != Kind::Object) throw std::out_of_range("json shim: at() on non-object");
    auto it = object_.find(key);
    if (it == object_.end()) throw std::out_of_range("json shim: key '" + key + "' not found");
    return it->second;
  }
  std::vector<std::pair<std::string, const json &>> items() const {
    std::vector<std::pair<std::string, const json &>> out;
    if (kind_ == Kind::Object)
      for (const auto &kv : object_) out.emplace_back(kv.first, kv.second);
    return out;
  }
  operator double() const {  // NOLINT: nlohmann converts implicitly
    if (kind_ != Kind::Number) throw std::invalid_argument("json shim: value is not a number");
    return number_;
  }
  template <typename T>
  T get() const;

  friend std::istream &operator>>(std::istream &is, json &j) {
    std::string text((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
    size_t pos = 0;
    j = Parse(text, pos);
    SkipWs(text, pos);
    if (pos != text.size()) throw std::invalid_argument("json shim: trailing characters");
    return is;
  }

 private:
  static void SkipWs(const std::string &s, size_t &p) {
    while (p < s.size() && std::isspace(static_cast<unsigned char>(s[p]))) ++p;
  }
  static json Parse(const std::string &s, size_t &p) {
    SkipWs(s, p);
    if (p >= s.size()) throw std::invalid_argument("json shim: unexpected end");
    json j;
    const char c = s[p];
    if (c == '{') {
      j.kind_ = Kind::Object;
      ++p;
      SkipWs(s, p);
      if (p < s.size() && s[p] == '}') { ++p; return j; }
      while (true) {
        SkipWs(s, p);
        json key = Parse(s, p);
        if (key.kind_ != Kind::String) throw std::invalid_argument("json shim: object key is not a string");
        SkipWs(s, p);
        if (p >= s.size() || s[p] != ':') throw std::invalid_argument("json shim: expected ':'");
        ++p;
        j.object_[key.string_] = Parse(s, p);
        SkipWs(s, p);
        if (p < s.size() && s[p] == ',') { ++p; continue; }
        if (p < s.size() && s[p] == '}') { ++p; break; }
        throw std::invalid_argument("json shim: expected ',' or '}'");
      }
    } else if (c == '[') {
      j.kind_ = Kind::Array;
      ++p;
      SkipWs(s, p);
      if (p < s.size() && s[p] == ']') { ++p; return j; }
      while (true) {
        j.array_.push_back(Parse(s, p));
        SkipWs(s, p);
        if (p < s.size() && s[p] == ',') { ++p; continue; }
        if (p < s.size() && s[p] == ']') { ++p; break; }
        throw std::invalid_argument("json shim: expected ',' or ']'");
      }
    } else if (c == '"') {
      j.kind_ = Kind::String;
      ++p;
      while (p < s.size() && s[p] != '"') {
        if (s[p] == '\\' && p + 1 < s.size()) { j.string_ += s[p + 1]; p += 2; continue; }
        j.string_ += s[p++];
      }
      if (p >= s.size()) throw std::invalid_argument("json shim: unterminated string");
      ++p;
    } else if (s.compare(p, 4, "true") == 0) {
      j.kind_ = Kind::Bool; j.bool_ = true; p += 4;
    } else if (s.compare(p, 5, "false") == 0) {
      j.kind_ = Kind::Bool; j.bool_ = false; p += 5;
    } else if (s.compare(p, 4, "null") == 0) {
      p += 4;
    } else {
      const char *begin = s.c_str() + p;
      char *end = nullptr;
      j.number_ = std::strtod(begin, &end);
      if (end == begin) throw std::invalid_argument("json shim: bad token");
      j.kind_ = Kind::Number;
      p += static_cast<size_t>(end - begin);
    }
    return j;
  }

  Kind kind_{Kind::Null};
  bool bool_{false};
  double number_{0.0};
  std::string string_{};
  std::vector<json> array_{};
  std::map<std::string, json> object_{};

  friend std::vector<double> ToDoubleVector(const json &j);
};

inline std::vector<double> ToDoubleVector(const json &j) {
  if (j.kind_ != json::Kind::Array) throw std::invalid_argument("json shim: value is not an array");
  std::vector<double> v;
  v.reserve(j.array_.size());
  for (const auto &e : j.array_) v.push_back(static_cast<double>(e));
  return v;
}

template <>
inline std::vector<double> json::get<std::vector<double>>() const {
  return ToDoubleVector(*this);
}
template <>
inline std::vector<std::vector<double>> json::get<std::vector<std::vector<double>>>() const {
  if (kind_ != Kind::Array) throw std::invalid_argument("json shim: value is not an array");
  std::vector<std::vector<double>> v;
  v.reserve(array_.size());
  for (const auto &row : array_) v.push_back(ToDoubleVector(row));
  return v;
}
}  // namespace nlohmann
#endif
