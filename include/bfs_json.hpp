// bfs_json.hpp -- minimal JSON value for the command line driver's report.
//
// The reference writes its report with a vendored JSON library
// (include/json.hpp, used at src/host.cpp:228-271 and
// src/run_bfs_gpu.hpp:784-790).  This header provides the small subset the
// report needs: objects (keys kept sorted, as the reference's objects are),
// arrays, numbers, strings, booleans and null; `obj["key"] = value`,
// `push_back`, parsing an existing report file and `dump(indent)`.
#pragma once
#include <charconv>
#include <cmath>
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace bfs {

class Json {
 public:
  enum class Type { Null, Bool, Int, UInt, Double, String, Array, Object };

  Json() = default;
  Json(std::nullptr_t) {}
  Json(bool b) : t_(Type::Bool), b_(b) {}
  Json(int v) : t_(Type::Int), i_(v) {}
  Json(long v) : t_(Type::Int), i_(v) {}
  Json(long long v) : t_(Type::Int), i_(v) {}
  Json(unsigned v) : t_(Type::UInt), u_(v) {}
  Json(unsigned long v) : t_(Type::UInt), u_(v) {}
  Json(unsigned long long v) : t_(Type::UInt), u_(v) {}
  Json(double v) : t_(Type::Double), d_(v) {}
  Json(float v) : t_(Type::Double), d_(v) {}
  Json(const char *s) : t_(Type::String), s_(s) {}
  Json(const std::string &s) : t_(Type::String), s_(s) {}
  template <typename T>
  Json(const std::vector<T> &v) : t_(Type::Array) {
    for (const auto &x : v) a_.emplace_back(x);
  }

  static Json object() {
    Json j;
    j.t_ = Type::Object;
    return j;
  }
  static Json array() {
    Json j;
    j.t_ = Type::Array;
    return j;
  }

  Type type() const { return t_; }
  bool is_object() const { return t_ == Type::Object; }
  bool is_array() const { return t_ == Type::Array; }
  bool is_null() const { return t_ == Type::Null; }

  // Object access; a null value becomes an object (like the reference's
  // library does for operator[] on a non-const value).
  Json &operator[](const std::string &k) {
    if (t_ == Type::Null) t_ = Type::Object;
    if (t_ != Type::Object) throw std::runtime_error("json: not an object");
    return o_[k];
  }
  const Json &at(const std::string &k) const {
    auto it = o_.find(k);
    if (t_ != Type::Object || it == o_.end()) throw std::runtime_error("json: no key " + k);
    return it->second;
  }
  bool contains(const std::string &k) const { return t_ == Type::Object && o_.count(k); }
  void push_back(const Json &v) {
    if (t_ == Type::Null) t_ = Type::Array;
    if (t_ != Type::Array) throw std::runtime_error("json: not an array");
    a_.push_back(v);
  }
  size_t size() const { return t_ == Type::Array ? a_.size() : t_ == Type::Object ? o_.size() : 0; }
  const Json &operator[](size_t i) const { return a_.at(i); }

  double as_double() const {
    switch (t_) {
      case Type::Int: return (double)i_;
      case Type::UInt: return (double)u_;
      case Type::Double: return d_;
      case Type::Bool: return b_ ? 1.0 : 0.0;
      default: throw std::runtime_error("json: not a number");
    }
  }
  uint64_t as_uint() const {
    if (t_ == Type::UInt) return u_;
    if (t_ == Type::Int && i_ >= 0) return (uint64_t)i_;
    if (t_ == Type::Double && d_ >= 0) return (uint64_t)d_;
    throw std::runtime_error("json: not an unsigned number");
  }
  const std::string &as_string() const {
    if (t_ != Type::String) throw std::runtime_error("json: not a string");
    return s_;
  }
  bool as_bool() const {
    if (t_ != Type::Bool) throw std::runtime_error("json: not a bool");
    return b_;
  }

  std::string dump(int indent = -1) const {
    std::string out;
    write(out, indent, 0);
    return out;
  }

  static Json parse(const std::string &text) {
    size_t pos = 0;
    Json j = parse_value(text, pos);
    skip_ws(text, pos);
    if (pos != text.size()) throw std::runtime_error("json: trailing characters");
    return j;
  }

 private:
  Type t_ = Type::Null;
  bool b_ = false;
  long long i_ = 0;
  unsigned long long u_ = 0;
  double d_ = 0.0;
  std::string s_;
  std::vector<Json> a_;
  std::map<std::string, Json> o_;

  static void esc(std::string &out, const std::string &s) {
    out += '"';
    for (unsigned char c : s) {
      switch (c) {
        case '"': out += "\\\""; break;
        case '\\': out += "\\\\"; break;
        case '\n': out += "\\n"; break;
        case '\t': out += "\\t"; break;
        case '\r': out += "\\r"; break;
        case '\b': out += "\\b"; break;
        case '\f': out += "\\f"; break;
        default:
          if (c < 0x20) {
            char buf[8];
            std::snprintf(buf, sizeof buf, "\\u%04x", c);
            out += buf;
          } else {
            out += (char)c;
          }
      }
    }
    out += '"';
  }
  static void nl(std::string &out, int indent, int depth) {
    if (indent < 0) return;
    out += '\n';
    out.append((size_t)indent * depth, ' ');
  }
  void write(std::string &out, int indent, int depth) const {
    char buf[64];
    switch (t_) {
      case Type::Null: out += "null"; break;
      case Type::Bool: out += b_ ? "true" : "false"; break;
      case Type::Int: out += std::to_string(i_); break;
      case Type::UInt: out += std::to_string(u_); break;
      case Type::Double: {
        if (!std::isfinite(d_)) {
          out += "null";
          break;
        }
        auto r = std::to_chars(buf, buf + sizeof buf, d_);  // shortest round trip
        std::string s(buf, r.ptr);
        if (s.find_first_of(".eE") == std::string::npos) s += ".0";
        out += s;
        break;
      }
      case Type::String: esc(out, s_); break;
      case Type::Array: {
        out += '[';
        if (a_.empty()) {
          out += ']';
          break;
        }
        for (size_t i = 0; i < a_.size(); i++) {
          if (i) out += ',';
          nl(out, indent, depth + 1);
          a_[i].write(out, indent, depth + 1);
        }
        nl(out, indent, depth);
        out += ']';
        break;
      }
      case Type::Object: {
        out += '{';
        if (o_.empty()) {
          out += '}';
          break;
        }
        bool first = true;
        for (const auto &kv : o_) {
          if (!first) out += ',';
          first = false;
          nl(out, indent, depth + 1);
          esc(out, kv.first);
          out += indent < 0 ? ":" : ": ";
          kv.second.write(out, indent, depth + 1);
        }
        nl(out, indent, depth);
        out += '}';
        break;
      }
    }
  }
  static void skip_ws(const std::string &s, size_t &p) {
    while (p < s.size() && (s[p] == ' ' || s[p] == '\n' || s[p] == '\t' || s[p] == '\r')) p++;
  }
  static std::string parse_string(const std::string &s, size_t &p) {
    if (s[p] != '"') throw std::runtime_error("json: expected string");
    p++;
    std::string out;
    while (p < s.size() && s[p] != '"') {
      char c = s[p++];
      if (c != '\\') {
        out += c;
        continue;
      }
      if (p >= s.size()) break;
      char e = s[p++];
      switch (e) {
        case 'n': out += '\n'; break;
        case 't': out += '\t'; break;
        case 'r': out += '\r'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        case 'u': {
          if (p + 4 > s.size()) throw std::runtime_error("json: bad escape");
          unsigned cp = (unsigned)std::stoul(s.substr(p, 4), nullptr, 16);
          p += 4;
          if (cp < 0x80) {
            out += (char)cp;
          } else if (cp < 0x800) {
            out += (char)(0xC0 | (cp >> 6));
            out += (char)(0x80 | (cp & 0x3F));
          } else {
            out += (char)(0xE0 | (cp >> 12));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
          }
          break;
        }
        default: out += e;
      }
    }
    if (p >= s.size()) throw std::runtime_error("json: unterminated string");
    p++;
    return out;
  }
  static Json parse_value(const std::string &s, size_t &p) {
    skip_ws(s, p);
    if (p >= s.size()) throw std::runtime_error("json: unexpected end");
    const char c = s[p];
    if (c == '{') {
      Json j = object();
      p++;
      skip_ws(s, p);
      if (p < s.size() && s[p] == '}') {
        p++;
        return j;
      }
      for (;;) {
        skip_ws(s, p);
        std::string k = parse_string(s, p);
        skip_ws(s, p);
        if (p >= s.size() || s[p] != ':') throw std::runtime_error("json: expected ':'");
        p++;
        j.o_[k] = parse_value(s, p);
        skip_ws(s, p);
        if (p < s.size() && s[p] == ',') {
          p++;
          continue;
        }
        if (p < s.size() && s[p] == '}') {
          p++;
          return j;
        }
        throw std::runtime_error("json: expected ',' or '}'");
      }
    }
    if (c == '[') {
      Json j = array();
      p++;
      skip_ws(s, p);
      if (p < s.size() && s[p] == ']') {
        p++;
        return j;
      }
      for (;;) {
        j.a_.push_back(parse_value(s, p));
        skip_ws(s, p);
        if (p < s.size() && s[p] == ',') {
          p++;
          continue;
        }
        if (p < s.size() && s[p] == ']') {
          p++;
          return j;
        }
        throw std::runtime_error("json: expected ',' or ']'");
      }
    }
    if (c == '"') return Json(parse_string(s, p));
    if (s.compare(p, 4, "true") == 0) {
      p += 4;
      return Json(true);
    }
    if (s.compare(p, 5, "false") == 0) {
      p += 5;
      return Json(false);
    }
    if (s.compare(p, 4, "null") == 0) {
      p += 4;
      return Json();
    }
    size_t q = p;
    bool is_float = false;
    if (q < s.size() && (s[q] == '-' || s[q] == '+')) q++;
    while (q < s.size() && (std::isdigit((unsigned char)s[q]) || s[q] == '.' || s[q] == 'e' ||
                            s[q] == 'E' || s[q] == '-' || s[q] == '+')) {
      if (s[q] == '.' || s[q] == 'e' || s[q] == 'E') is_float = true;
      q++;
    }
    if (q == p) throw std::runtime_error("json: bad value");
    const std::string num = s.substr(p, q - p);
    p = q;
    if (is_float) return Json(std::stod(num));
    if (num[0] == '-') return Json(std::stoll(num));
    return Json(std::stoull(num));
  }
};

}  // namespace bfs
