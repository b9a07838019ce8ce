// Minimal JSON reader for clovers scene files.
//
// Scene files are small (kilobytes), so a DOM with ordered object members is
// enough.  Numbers are kept as double; a field typed f32 in the reference is
// read through double and rounded to float, the same two-step conversion
// serde_json performs for f32 targets (decimal -> f64 -> `as f32`).
#pragma once

#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace clv_json {

struct Value {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Value> arr;
  std::vector<std::pair<std::string, Value>> obj;

  bool is_null() const { return kind == Null; }
  bool is_number() const { return kind == Number; }
  bool is_string() const { return kind == String; }
  bool is_array() const { return kind == Array; }
  bool is_object() const { return kind == Object; }

  const Value* find(const char* key) const {
    if (kind != Object) return nullptr;
    for (auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
  bool has(const char* key) const { return find(key) != nullptr; }
  const Value& at(const char* key) const {
    const Value* v = find(key);
    if (!v) throw std::runtime_error(std::string("missing field `") + key + "`");
    return *v;
  }
  double as_number(const char* what = "value") const {
    if (kind != Number) throw std::runtime_error(std::string("expected a number for ") + what);
    return num;
  }
  float as_f32(const char* what = "value") const { return (float)as_number(what); }
  bool as_bool(const char* what = "value") const {
    if (kind != Bool) throw std::runtime_error(std::string("expected a bool for ") + what);
    return b;
  }
  const std::string& as_string(const char* what = "value") const {
    if (kind != String) throw std::runtime_error(std::string("expected a string for ") + what);
    return str;
  }
};

class Parser {
 public:
  explicit Parser(const std::string& text) : s_(text), p_(0) {}

  Value parse() {
    Value v = value();
    ws();
    if (p_ != s_.size()) fail("trailing characters");
    return v;
  }

 private:
  const std::string& s_;
  size_t p_;

  [[noreturn]] void fail(const char* msg) {
    size_t line = 1, col = 1;
    for (size_t i = 0; i < p_ && i < s_.size(); ++i) {
      if (s_[i] == '\n') { ++line; col = 1; } else { ++col; }
    }
    throw std::runtime_error(std::string("JSON parse error: ") + msg + " at line " +
                             std::to_string(line) + " column " + std::to_string(col));
  }
  void ws() {
    while (p_ < s_.size() && (s_[p_] == ' ' || s_[p_] == '\t' || s_[p_] == '\n' || s_[p_] == '\r')) ++p_;
  }
  bool eat(char c) {
    ws();
    if (p_ < s_.size() && s_[p_] == c) { ++p_; return true; }
    return false;
  }
  void expect(char c) {
    if (!eat(c)) {
      char m[32];
      std::snprintf(m, sizeof m, "expected '%c'", c);
      fail(m);
    }
  }
  Value value() {
    ws();
    if (p_ >= s_.size()) fail("unexpected end of input");
    char c = s_[p_];
    Value v;
    if (c == '{') {
      ++p_;
      v.kind = Value::Object;
      if (eat('}')) return v;
      do {
        ws();
        std::string k = string_lit();
        expect(':');
        v.obj.emplace_back(std::move(k), value());
      } while (eat(','));
      expect('}');
    } else if (c == '[') {
      ++p_;
      v.kind = Value::Array;
      if (eat(']')) return v;
      do { v.arr.push_back(value()); } while (eat(','));
      expect(']');
    } else if (c == '"') {
      v.kind = Value::String;
      v.str = string_lit();
    } else if (s_.compare(p_, 4, "true") == 0) {
      p_ += 4; v.kind = Value::Bool; v.b = true;
    } else if (s_.compare(p_, 5, "false") == 0) {
      p_ += 5; v.kind = Value::Bool; v.b = false;
    } else if (s_.compare(p_, 4, "null") == 0) {
      p_ += 4; v.kind = Value::Null;
    } else if (c == '-' || (c >= '0' && c <= '9')) {
      const char* begin = s_.c_str() + p_;
      char* end = nullptr;
      v.kind = Value::Number;
      v.num = std::strtod(begin, &end);
      if (end == begin) fail("bad number");
      p_ += (size_t)(end - begin);
    } else {
      fail("unexpected character");
    }
    return v;
  }
  static void put_utf8(std::string& out, unsigned cp) {
    if (cp < 0x80) out += (char)cp;
    else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
    else if (cp < 0x10000) {
      out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F));
    } else {
      out += (char)(0xF0 | (cp >> 18)); out += (char)(0x80 | ((cp >> 12) & 0x3F));
      out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F));
    }
  }
  unsigned hex4() {
    if (p_ + 4 > s_.size()) fail("bad \\u escape");
    unsigned v = 0;
    for (int i = 0; i < 4; ++i) {
      char h = s_[p_++];
      v <<= 4;
      if (h >= '0' && h <= '9') v |= (unsigned)(h - '0');
      else if (h >= 'a' && h <= 'f') v |= (unsigned)(h - 'a' + 10);
      else if (h >= 'A' && h <= 'F') v |= (unsigned)(h - 'A' + 10);
      else fail("bad \\u escape");
    }
    return v;
  }
  std::string string_lit() {
    if (p_ >= s_.size() || s_[p_] != '"') fail("expected string");
    ++p_;
    std::string out;
    while (true) {
      if (p_ >= s_.size()) fail("unterminated string");
      char c = s_[p_++];
      if (c == '"') break;
      if (c != '\\') { out += c; continue; }
      if (p_ >= s_.size()) fail("unterminated escape");
      char e = s_[p_++];
      switch (e) {
        case '"': out += '"'; break;
        case '\\': out += '\\'; break;
        case '/': out += '/'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        case 'n': out += '\n'; break;
        case 'r': out += '\r'; break;
        case 't': out += '\t'; break;
        case 'u': {
          unsigned cp = hex4();
          if (cp >= 0xD800 && cp < 0xDC00 && p_ + 1 < s_.size() && s_[p_] == '\\' && s_[p_ + 1] == 'u') {
            p_ += 2;
            unsigned lo = hex4();
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          }
          put_utf8(out, cp);
          break;
        }
        default: fail("bad escape");
      }
    }
    return out;
  }
};

inline Value parse(const std::string& text) { return Parser(text).parse(); }

}  // namespace clv_json
