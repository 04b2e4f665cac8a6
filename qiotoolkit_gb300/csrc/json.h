// json.h -- minimal JSON reader/writer for the host shim.
//
// Reads the reference's input documents ({"cost_function": ...}) and params
// ({"params": ...}); writes result documents.  Numbers keep their double
// value and, when they are integral, an exact int64.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace qio
{
namespace json
{
struct Value
{
  enum Type { NUL, BOOL, NUMBER, STRING, ARRAY, OBJECT };
  Type type = NUL;
  bool b = false;
  double num = 0;
  bool is_int = false;
  int64_t i = 0;
  std::string str;
  std::vector<Value> arr;
  std::vector<std::pair<std::string, Value>> obj;

  bool is_null() const { return type == NUL; }
  bool is_number() const { return type == NUMBER; }
  bool is_array() const { return type == ARRAY; }
  bool is_object() const { return type == OBJECT; }
  bool is_string() const { return type == STRING; }
  bool has(const std::string& k) const;
  const Value& operator[](const std::string& k) const;
  const Value* find(const std::string& k) const;
};

// Parse a document; throws std::runtime_error with the offset on bad input.
Value parse(const char* text, size_t len);
Value parse(const std::string& s);

// Writer helpers: numbers printed with %.17g unless `fixed6` (the reference
// renders doubles with std::to_string, i.e. "%f").
std::string quote(const std::string& s);
std::string number(double v);
}  // namespace json
}  // namespace qio
