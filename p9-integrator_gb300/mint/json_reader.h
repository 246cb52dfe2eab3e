// json_reader.h - a small JSON reader for the system-config files of mint.
//
// Parses the subset the configs use (objects, arrays, numbers, strings,
// true/false/null) into a tree of Value nodes.  Numbers are parsed with
// strtod, so every decimal written by a JSON writer round-trips to the same
// binary64 value.  Errors throw std::runtime_error with the byte offset.
#pragma once
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace mintjson {

struct Value {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Value> arr;
  std::vector<std::pair<std::string, Value>> obj;  // insertion order kept

  const Value* get(const std::string& key) const;  // nullptr if absent
  double number(const std::string& key) const;     // throws if absent or not a number
  double number_or(const std::string& key, double dflt) const;
  std::string string_or(const std::string& key, const std::string& dflt) const;
  bool bool_or(const std::string& key, bool dflt) const;
};

Value parse(const std::string& text);
Value parse_file(const std::string& path);

}  // namespace mintjson
