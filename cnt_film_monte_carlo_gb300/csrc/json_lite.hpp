// json_lite.hpp -- a small JSON reader/writer for the drop-in driver's input.json.
// Supports objects, arrays, numbers, strings (with \" \\ \/ \b \f \n \r \t \uXXXX escapes, the
// last decoded to UTF-8), true/false/null, and refuses what RFC 8259 does not allow (as the
// reference's nlohmann::json reader does): numbers outside the JSON grammar (nan, inf, hex, a
// leading '+' or zero, a bare '.'), other escapes, raw control characters, unpaired
// surrogates and invalid UTF-8 in strings.  Object key order is kept for writing the file back; a number read from
// text is written back as that text (so integers stay integers and 0.1 stays 0.1); strings are
// written with quote, backslash and control characters escaped.
#pragma once
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace jl {

struct Value {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0;
  std::string lit;  // a number's text as read (empty for numbers made in code)
  std::string str;
  std::vector<Value> arr;
  std::vector<std::pair<std::string, Value>> obj;

  bool has(const std::string& k) const {
    for (auto& kv : obj)
      if (kv.first == k) return true;
    return false;
  }
  const Value& operator[](const std::string& k) const {
    for (auto& kv : obj)
      if (kv.first == k) return kv.second;
    throw std::invalid_argument("json: missing key \"" + k + "\"");
  }
  const Value& operator[](size_t i) const {
    if (kind != Array || i >= arr.size()) throw std::invalid_argument("json: index out of range");
    return arr[i];
  }
  double as_double() const {
    if (kind != Number) throw std::invalid_argument("json: number expected");
    return num;
  }
  // the number truncated toward zero, as nlohmann's get<int>() converts a float; a value outside
  // the range of long long (1e999 reads as infinity) is refused instead of converted
  long long as_int() const {
    const double x = as_double();
    if (!(x > -9223372036854775808.0 && x < 9223372036854775808.0))
      throw std::invalid_argument("json: integer out of range");
    return (long long)x;
  }
  int as_int32() const {
    const long long v = as_int();
    if (v < -2147483648LL || v > 2147483647LL) throw std::invalid_argument("json: integer out of range");
    return (int)v;
  }
  bool as_bool() const {
    if (kind != Bool) throw std::invalid_argument("json: bool expected");
    return b;
  }
  const std::string& as_string() const {
    if (kind != String) throw std::invalid_argument("json: string expected");
    return str;
  }
};

class Parser {
 public:
  explicit Parser(const std::string& s) : s_(s) {}
  Value parse() {
    Value v = value();
    ws();
    if (i_ != s_.size()) fail("trailing characters");
    return v;
  }

 private:
  const std::string& s_;
  size_t i_ = 0;
  // objects and arrays nest at most this deep: the reader and the writer recurse once per level,
  // and a file of a few hundred kilobytes of brackets would otherwise overflow the stack
  static constexpr int kMaxDepth = 512;
  int depth_ = 0;
  [[noreturn]] void fail(const char* what) {
    throw std::invalid_argument(std::string("json: ") + what + " at offset " + std::to_string(i_));
  }
  void ws() {
    while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\n' || s_[i_] == '\t' || s_[i_] == '\r')) ++i_;
  }
  bool eat(char c) {
    ws();
    if (i_ < s_.size() && s_[i_] == c) {
      ++i_;
      return true;
    }
    return false;
  }
  Value value() {
    ws();
    if (i_ >= s_.size()) fail("unexpected end");
    char c = s_[i_];
    Value v;
    if ((c == '{' || c == '[') && ++depth_ > kMaxDepth) fail("objects and arrays nested too deep");
    if (c == '{') {
      ++i_;
      v.kind = Value::Object;
      if (eat('}')) {
        --depth_;
        return v;
      }
      do {
        ws();
        std::string k = string();
        if (!eat(':')) fail("':' expected");
        v.obj.emplace_back(k, value());
      } while (eat(','));
      if (!eat('}')) fail("'}' expected");
      --depth_;
    } else if (c == '[') {
      ++i_;
      v.kind = Value::Array;
      if (eat(']')) {
        --depth_;
        return v;
      }
      do {
        v.arr.push_back(value());
      } while (eat(','));
      if (!eat(']')) fail("']' expected");
      --depth_;
    } else if (c == '"') {
      v.kind = Value::String;
      v.str = string();
    } else if (s_.compare(i_, 4, "true") == 0) {
      i_ += 4;
      v.kind = Value::Bool;
      v.b = true;
    } else if (s_.compare(i_, 5, "false") == 0) {
      i_ += 5;
      v.kind = Value::Bool;
    } else if (s_.compare(i_, 4, "null") == 0) {
      i_ += 4;
    } else {
      number(v);
    }
    return v;
  }
  bool digit_at(size_t j) const { return j < s_.size() && s_[j] >= '0' && s_[j] <= '9'; }
  // -?(0|[1-9][0-9]*)(.[0-9]+)?([eE][+-]?[0-9]+)?, converted by strtod (C locale)
  void number(Value& v) {
    size_t j = i_;
    if (j < s_.size() && s_[j] == '-') ++j;
    if (!digit_at(j)) fail("value expected");
    if (s_[j] == '0') {
      ++j;
    } else {
      while (digit_at(j)) ++j;
    }
    if (j < s_.size() && s_[j] == '.') {
      ++j;
      if (!digit_at(j)) fail("digit expected after '.'");
      while (digit_at(j)) ++j;
    }
    if (j < s_.size() && (s_[j] == 'e' || s_[j] == 'E')) {
      ++j;
      if (j < s_.size() && (s_[j] == '+' || s_[j] == '-')) ++j;
      if (!digit_at(j)) fail("digit expected in exponent");
      while (digit_at(j)) ++j;
    }
    v.lit = s_.substr(i_, j - i_);
    v.num = std::strtod(v.lit.c_str(), nullptr);
    v.kind = Value::Number;
    i_ = j;
  }
  uint32_t hex4() {
    if (i_ + 4 > s_.size()) fail("bad \\u escape");
    uint32_t v = 0;
    for (int k = 0; k < 4; ++k) {
      const char h = s_[i_ + k];
      v <<= 4;
      if (h >= '0' && h <= '9')
        v |= (uint32_t)(h - '0');
      else if (h >= 'a' && h <= 'f')
        v |= (uint32_t)(h - 'a' + 10);
      else if (h >= 'A' && h <= 'F')
        v |= (uint32_t)(h - 'A' + 10);
      else
        fail("bad \\u escape");
    }
    i_ += 4;
    return v;
  }
  static void utf8(std::string& out, uint32_t cp) {
    if (cp < 0x80) {
      out += (char)cp;
    } else if (cp < 0x800) {
      out += (char)(0xC0 | (cp >> 6));
      out += (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
      out += (char)(0xE0 | (cp >> 12));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    } else {
      out += (char)(0xF0 | (cp >> 18));
      out += (char)(0x80 | ((cp >> 12) & 0x3F));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    }
  }
  // One multi-byte UTF-8 character whose lead byte b was just read (RFC 3629: no overlong forms,
  // no surrogates, nothing above U+10FFFF), appended to out as it is.
  void utf8_sequence(unsigned char b, std::string& out) {
    int n;
    unsigned char lo = 0x80, hi = 0xBF;  // range of the first continuation byte
    if (b >= 0xC2 && b <= 0xDF) {
      n = 1;
    } else if (b >= 0xE0 && b <= 0xEF) {
      n = 2;
      if (b == 0xE0) lo = 0xA0;
      if (b == 0xED) hi = 0x9F;
    } else if (b >= 0xF0 && b <= 0xF4) {
      n = 3;
      if (b == 0xF0) lo = 0x90;
      if (b == 0xF4) hi = 0x8F;
    } else {
      fail("invalid UTF-8 in string");
    }
    out += (char)b;
    for (int k = 0; k < n; ++k) {
      if (i_ >= s_.size()) fail("invalid UTF-8 in string");
      const unsigned char t = (unsigned char)s_[i_];
      if (t < (k == 0 ? lo : 0x80) || t > (k == 0 ? hi : 0xBF)) fail("invalid UTF-8 in string");
      out += (char)t;
      ++i_;
    }
  }
  std::string string() {
    if (i_ >= s_.size() || s_[i_] != '"') fail("string expected");
    ++i_;
    std::string out;
    while (i_ < s_.size() && s_[i_] != '"') {
      char c = s_[i_++];
      if ((unsigned char)c < 0x20) fail("control character in string");
      if ((unsigned char)c >= 0x80) {
        utf8_sequence((unsigned char)c, out);
        continue;
      }
      if (c == '\\') {
        if (i_ >= s_.size()) fail("bad escape");
        char e = s_[i_++];
        switch (e) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case '"':
          case '\\':
          case '/': out += e; break;
          case 'u': {
            uint32_t cp = hex4();
            if (cp >= 0xDC00 && cp < 0xE000) fail("unpaired surrogate");
            if (cp >= 0xD800 && cp < 0xDC00) {  // must be the first half of a surrogate pair
              if (s_.compare(i_, 2, "\\u") != 0) fail("unpaired surrogate");
              i_ += 2;
              const uint32_t lo = hex4();
              if (lo < 0xDC00 || lo >= 0xE000) fail("bad surrogate pair");
              cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
            }
            utf8(out, cp);
            break;
          }
          default: fail("bad escape");
        }
      } else {
        out += c;
      }
    }
    if (i_ >= s_.size()) fail("unterminated string");
    ++i_;
    return out;
  }
};

inline Value parse(const std::string& text) { return Parser(text).parse(); }

// a string as a JSON literal: quote, backslash and control characters escaped
inline void write_string(std::ostream& o, const std::string& s) {
  o << '"';
  for (unsigned char c : s) {
    switch (c) {
      case '"': o << "\\\""; break;
      case '\\': o << "\\\\"; break;
      case '\n': o << "\\n"; break;
      case '\t': o << "\\t"; break;
      case '\r': o << "\\r"; break;
      case '\b': o << "\\b"; break;
      case '\f': o << "\\f"; break;
      default:
        if (c < 0x20) {
          static const char hex[] = "0123456789abcdef";
          o << "\\u00" << hex[c >> 4] << hex[c & 15];
        } else {
          o << (char)c;
        }
    }
  }
  o << '"';
}

inline void write(std::ostream& o, const Value& v, int indent = 0) {
  std::string pad(indent, ' '), pad2(indent + 4, ' ');
  switch (v.kind) {
    case Value::Null: o << "null"; break;
    case Value::Bool: o << (v.b ? "true" : "false"); break;
    case Value::Number: {
      if (!v.lit.empty()) {
        o << v.lit;
        break;
      }
      // made in code: the shortest text that reads back as the same double, kept a float
      // literal ("2.0", not "2"); JSON has no infinities or NaNs
      if (!std::isfinite(v.num)) {
        o << "null";
        break;
      }
      char buf[64];
      const auto r = std::to_chars(buf, buf + sizeof buf, v.num);
      std::string t(buf, r.ptr);
      if (t.find_first_of(".e") == std::string::npos) t += ".0";
      o << t;
      break;
    }
    case Value::String: write_string(o, v.str); break;
    case Value::Array:
      o << "[";
      for (size_t i = 0; i < v.arr.size(); ++i) {
        if (i) o << ", ";
        write(o, v.arr[i], indent + 4);
      }
      o << "]";
      break;
    case Value::Object:
      o << "{\n";
      for (size_t i = 0; i < v.obj.size(); ++i) {
        o << pad2;
        write_string(o, v.obj[i].first);
        o << ": ";
        write(o, v.obj[i].second, indent + 4);
        o << (i + 1 < v.obj.size() ? ",\n" : "\n");
      }
      o << pad << "}";
      break;
  }
}

}  // namespace jl
