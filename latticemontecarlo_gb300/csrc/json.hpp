// Minimal JSON reader for the coefficient file format of the reference
// ("Base": {"theta": [...]}, "<Element>": {"mu_x_mmm": [...], "U_mmm": [[...]], ...}).
// Supports objects, arrays, numbers, strings, true/false/null (RFC 8259).
#pragma once
#include <cctype>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace lmc {

class JsonValue {
 public:
  enum class Type { Null, Bool, Number, String, Array, Object };

  static JsonValue Parse(const std::string &text) {
    size_t pos = 0;
    JsonValue v = ParseValue(text, pos);
    SkipWs(text, pos);
    if (pos != text.size()) throw std::invalid_argument("JSON: trailing characters at offset " + std::to_string(pos));
    return v;
  }

  Type type() const { return type_; }
  bool IsObject() const { return type_ == Type::Object; }
  bool Has(const std::string &key) const { return type_ == Type::Object && object_.count(key) != 0; }
  const JsonValue &At(const std::string &key) const {
    if (type_ != Type::Object) throw std::invalid_argument("JSON: not an object when looking up '" + key + "'");
    auto it = object_.find(key);
    if (it == object_.end()) throw std::out_of_range("JSON: key '" + key + "' not found");
    return it->second;
  }
  const std::map<std::string, JsonValue> &Object() const { return object_; }
  double Number() const {
    if (type_ != Type::Number) throw std::invalid_argument("JSON: value is not a number");
    return number_;
  }
  std::vector<double> Vector() const {
    if (type_ != Type::Array) throw std::invalid_argument("JSON: value is not an array");
    std::vector<double> v;
    v.reserve(array_.size());
    for (const auto &e : array_) v.push_back(e.Number());
    return v;
  }
  // Row-major matrix from an array of equal-length arrays.
  std::vector<double> Matrix(int *rows, int *cols) const {
    if (type_ != Type::Array) throw std::invalid_argument("JSON: matrix is not an array");
    std::vector<double> m;
    *rows = static_cast<int>(array_.size());
    *cols = 0;
    for (size_t r = 0; r < array_.size(); ++r) {
      auto row = array_[r].Vector();
      if (r == 0) *cols = static_cast<int>(row.size());
      else if (static_cast<int>(row.size()) != *cols) throw std::invalid_argument("JSON: ragged matrix");
      m.insert(m.end(), row.begin(), row.end());
    }
    return m;
  }

 private:
  static void SkipWs(const std::string &s, size_t &p) {
    while (p < s.size() && std::isspace(static_cast<unsigned char>(s[p]))) ++p;
  }
  static JsonValue ParseValue(const std::string &s, size_t &p) {
    SkipWs(s, p);
    if (p >= s.size()) throw std::invalid_argument("JSON: unexpected end of input");
    JsonValue v;
    const char c = s[p];
    if (c == '{') {
      v.type_ = Type::Object;
      ++p;
      SkipWs(s, p);
      if (p < s.size() && s[p] == '}') { ++p; return v; }
      for (;;) {
        SkipWs(s, p);
        JsonValue key = ParseValue(s, p);
        if (key.type_ != Type::String) throw std::invalid_argument("JSON: object key must be a string");
        SkipWs(s, p);
        if (p >= s.size() || s[p] != ':') throw std::invalid_argument("JSON: expected ':'");
        ++p;
        v.object_[key.string_] = ParseValue(s, p);
        SkipWs(s, p);
        if (p < s.size() && s[p] == ',') { ++p; continue; }
        if (p < s.size() && s[p] == '}') { ++p; break; }
        throw std::invalid_argument("JSON: expected ',' or '}' at offset " + std::to_string(p));
      }
    } else if (c == '[') {
      v.type_ = Type::Array;
      ++p;
      SkipWs(s, p);
      if (p < s.size() && s[p] == ']') { ++p; return v; }
      for (;;) {
        v.array_.push_back(ParseValue(s, p));
        SkipWs(s, p);
        if (p < s.size() && s[p] == ',') { ++p; continue; }
        if (p < s.size() && s[p] == ']') { ++p; break; }
        throw std::invalid_argument("JSON: expected ',' or ']' at offset " + std::to_string(p));
      }
    } else if (c == '"') {
      v.type_ = Type::String;
      ++p;
      while (p < s.size() && s[p] != '"') {
        if (s[p] == '\\' && p + 1 < s.size()) {
          v.string_ += s[p + 1];
          p += 2;
          continue;
        }
        v.string_ += s[p++];
      }
      if (p >= s.size()) throw std::invalid_argument("JSON: unterminated string");
      ++p;
    } else if (s.compare(p, 4, "true") == 0) {
      v.type_ = Type::Bool;
      p += 4;
    } else if (s.compare(p, 5, "false") == 0) {
      v.type_ = Type::Bool;
      p += 5;
    } else if (s.compare(p, 4, "null") == 0) {
      p += 4;
    } else {
      const char *b = s.c_str() + p;
      char *e = nullptr;
      v.number_ = std::strtod(b, &e);
      if (e == b) throw std::invalid_argument("JSON: bad token at offset " + std::to_string(p));
      v.type_ = Type::Number;
      p += static_cast<size_t>(e - b);
    }
    return v;
  }

  Type type_{Type::Null};
  double number_{0.0};
  std::string string_;
  std::vector<JsonValue> array_;
  std::map<std::string, JsonValue> object_;
};

}  // namespace lmc
