// json_reader.cpp - recursive-descent JSON reader (see json_reader.h).
#include "json_reader.h"

#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace mintjson {

namespace {

struct Parser {
  const std::string& s;
  size_t i = 0;
  explicit Parser(const std::string& t) : s(t) {}

  [[noreturn]] void error(const char* what) {
    throw std::runtime_error(std::string("JSON: ") + what + " at byte " + std::to_string(i));
  }
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r')) i++;
  }
  bool eat(char c) {
    ws();
    if (i < s.size() && s[i] == c) {
      i++;
      return true;
    }
    return false;
  }
  void expect(char c) {
    if (!eat(c)) error((std::string("expected '") + c + "'").c_str());
  }
  std::string string_lit() {
    ws();
    if (i >= s.size() || s[i] != '"') error("expected string");
    i++;
    std::string out;
    while (i < s.size() && s[i] != '"') {
      char c = s[i++];
      if (c == '\\') {
        if (i >= s.size()) error("bad escape");
        char e = s[i++];
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
            if (i + 4 > s.size()) error("bad \\u escape");
            unsigned cp = (unsigned)std::strtoul(s.substr(i, 4).c_str(), nullptr, 16);
            i += 4;
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
          default: error("bad escape");
        }
      } else {
        out += c;
      }
    }
    if (i >= s.size()) error("unterminated string");
    i++;
    return out;
  }
  Value value() {
    ws();
    if (i >= s.size()) error("unexpected end");
    Value v;
    char c = s[i];
    if (c == '{') {
      i++;
      v.kind = Value::Object;
      if (eat('}')) return v;
      do {
        std::string k = string_lit();
        expect(':');
        v.obj.emplace_back(k, value());
      } while (eat(','));
      expect('}');
    } else if (c == '[') {
      i++;
      v.kind = Value::Array;
      if (eat(']')) return v;
      do v.arr.push_back(value());
      while (eat(','));
      expect(']');
    } else if (c == '"') {
      v.kind = Value::String;
      v.str = string_lit();
    } else if (s.compare(i, 4, "true") == 0) {
      i += 4;
      v.kind = Value::Bool;
      v.b = true;
    } else if (s.compare(i, 5, "false") == 0) {
      i += 5;
      v.kind = Value::Bool;
    } else if (s.compare(i, 4, "null") == 0) {
      i += 4;
    } else {
      const char* start = s.c_str() + i;
      char* end = nullptr;
      errno = 0;
      double d = std::strtod(start, &end);
      if (end == start) error("expected a value");
      i += (size_t)(end - start);
      v.kind = Value::Number;
      v.num = d;
    }
    return v;
  }
};

}  // namespace

const Value* Value::get(const std::string& key) const {
  if (kind != Object) return nullptr;
  for (auto& kv : obj)
    if (kv.first == key) return &kv.second;
  return nullptr;
}

double Value::number(const std::string& key) const {
  const Value* v = get(key);
  if (!v || v->kind != Number) throw std::runtime_error("missing number field '" + key + "'");
  return v->num;
}

double Value::number_or(const std::string& key, double dflt) const {
  const Value* v = get(key);
  return (v && v->kind == Number) ? v->num : dflt;
}

std::string Value::string_or(const std::string& key, const std::string& dflt) const {
  const Value* v = get(key);
  return (v && v->kind == String) ? v->str : dflt;
}

bool Value::bool_or(const std::string& key, bool dflt) const {
  const Value* v = get(key);
  return (v && v->kind == Bool) ? v->b : dflt;
}

Value parse(const std::string& text) {
  Parser p(text);
  Value v = p.value();
  p.ws();
  if (p.i != text.size()) p.error("trailing characters");
  return v;
}

Value parse_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open config file '" + path + "'");
  std::stringstream ss;
  ss << f.rdbuf();
  return parse(ss.str());
}

}  // namespace mintjson
