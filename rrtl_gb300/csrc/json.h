// Minimal JSON reader for the design interchange format.
//
// The interchange format is the serde-JSON encoding of the reference's
// `rrtl_ir::Design` (crates/rrtl-ir/src/lib.rs:651-658, serde derive on every
// IR type). Numbers are kept as their source text so 128-bit literal values
// (serde encodes `i128` as a bare JSON number) survive without loss.
#pragma once

#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace rrtl {
namespace json {

struct Value {
  enum Kind : uint8_t { Null, Bool, Number, String, Array, Object };
  Kind kind = Null;
  bool b = false;
  std::string text;  // String payload or number source text
  std::vector<Value> arr;
  std::vector<std::pair<std::string, Value>> obj;

  bool is_null() const { return kind == Null; }
  bool is_obj() const { return kind == Object; }
  bool is_arr() const { return kind == Array; }
  bool is_str() const { return kind == String; }
  bool is_num() const { return kind == Number; }

  const Value* find(const char* key) const {
    if (kind != Object) return nullptr;
    for (auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
  const Value& at(const char* key) const {
    const Value* v = find(key);
    if (!v) throw std::runtime_error(std::string("json: missing key `") + key + "`");
    return *v;
  }
  const std::string& str() const {
    if (kind != String) throw std::runtime_error("json: expected string");
    return text;
  }
  __int128 i128() const {
    if (kind != Number) throw std::runtime_error("json: expected number");
    const char* p = text.c_str();
    bool neg = false;
    if (*p == '-') { neg = true; ++p; }
    unsigned __int128 v = 0;
    for (; *p; ++p) {
      if (*p < '0' || *p > '9') throw std::runtime_error("json: expected integer, got `" + text + "`");
      v = v * 10 + (unsigned)(*p - '0');
    }
    return neg ? -(__int128)v : (__int128)v;
  }
  uint64_t u64() const { return (uint64_t)i128(); }
  uint32_t u32() const { return (uint32_t)i128(); }
  bool boolean() const {
    if (kind != Bool) throw std::runtime_error("json: expected bool");
    return b;
  }
};

class Parser {
 public:
  Parser(const char* s, size_t n) : p_(s), end_(s + n) {}
  Value parse() {
    Value v = value();
    ws();
    if (p_ != end_) fail("trailing characters");
    return v;
  }

 private:
  const char* p_;
  const char* end_;
  [[noreturn]] void fail(const char* what) { throw std::runtime_error(std::string("json parse: ") + what); }
  void ws() {
    while (p_ < end_ && (*p_ == ' ' || *p_ == '\n' || *p_ == '\r' || *p_ == '\t')) ++p_;
  }
  bool lit(const char* s) {
    size_t n = strlen(s);
    if ((size_t)(end_ - p_) >= n && memcmp(p_, s, n) == 0) {
      p_ += n;
      return true;
    }
    return false;
  }
  std::string string_body() {
    std::string out;
    ++p_;  // opening quote
    while (p_ < end_ && *p_ != '"') {
      char c = *p_++;
      if (c == '\\') {
        if (p_ >= end_) fail("bad escape");
        char e = *p_++;
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
            if (end_ - p_ < 4) fail("bad \\u escape");
            unsigned cp = 0;
            for (int i = 0; i < 4; ++i) {
              char h = *p_++;
              cp <<= 4;
              if (h >= '0' && h <= '9') cp |= h - '0';
              else if (h >= 'a' && h <= 'f') cp |= h - 'a' + 10;
              else if (h >= 'A' && h <= 'F') cp |= h - 'A' + 10;
              else fail("bad hex digit");
            }
            if (cp < 0x80) out += (char)cp;
            else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
            else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
            break;
          }
          default: fail("bad escape");
        }
      } else {
        out += c;
      }
    }
    if (p_ >= end_) fail("unterminated string");
    ++p_;
    return out;
  }
  Value value() {
    ws();
    if (p_ >= end_) fail("unexpected end");
    Value v;
    char c = *p_;
    if (c == '{') {
      v.kind = Value::Object;
      ++p_;
      ws();
      if (p_ < end_ && *p_ == '}') { ++p_; return v; }
      for (;;) {
        ws();
        if (p_ >= end_ || *p_ != '"') fail("expected key");
        std::string k = string_body();
        ws();
        if (p_ >= end_ || *p_ != ':') fail("expected ':'");
        ++p_;
        v.obj.emplace_back(std::move(k), value());
        ws();
        if (p_ < end_ && *p_ == ',') { ++p_; continue; }
        if (p_ < end_ && *p_ == '}') { ++p_; break; }
        fail("expected ',' or '}'");
      }
    } else if (c == '[') {
      v.kind = Value::Array;
      ++p_;
      ws();
      if (p_ < end_ && *p_ == ']') { ++p_; return v; }
      for (;;) {
        v.arr.push_back(value());
        ws();
        if (p_ < end_ && *p_ == ',') { ++p_; continue; }
        if (p_ < end_ && *p_ == ']') { ++p_; break; }
        fail("expected ',' or ']'");
      }
    } else if (c == '"') {
      v.kind = Value::String;
      v.text = string_body();
    } else if (lit("true")) {
      v.kind = Value::Bool; v.b = true;
    } else if (lit("false")) {
      v.kind = Value::Bool; v.b = false;
    } else if (lit("null")) {
      v.kind = Value::Null;
    } else if (c == '-' || (c >= '0' && c <= '9')) {
      v.kind = Value::Number;
      const char* s = p_;
      if (*p_ == '-') ++p_;
      while (p_ < end_ && ((*p_ >= '0' && *p_ <= '9') || *p_ == '.' || *p_ == 'e' || *p_ == 'E' || *p_ == '+' || *p_ == '-')) ++p_;
      v.text.assign(s, p_);
    } else {
      fail("unexpected character");
    }
    return v;
  }
};

inline Value parse(const char* s, size_t n) { return Parser(s, n).parse(); }

}  // namespace json
}  // namespace rrtl
