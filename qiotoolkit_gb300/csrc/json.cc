// json.cc -- recursive-descent JSON reader (RFC 8259 subset sufficient for
// the reference's input and params documents) and small writer helpers.
#include "json.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

namespace qio
{
namespace json
{
static const Value kNull;

bool Value::has(const std::string& k) const { return find(k) != nullptr; }

const Value* Value::find(const std::string& k) const
{
  if (type != OBJECT) return nullptr;
  for (const auto& kv : obj)
    if (kv.first == k) return &kv.second;
  return nullptr;
}

const Value& Value::operator[](const std::string& k) const
{
  const Value* v = find(k);
  return v ? *v : kNull;
}

namespace
{
struct Parser
{
  const char* p;
  const char* end;
  const char* begin;

  [[noreturn]] void fail(const char* what)
  {
    throw std::runtime_error(std::string("JSON parse error: ") + what +
                             " at offset " + std::to_string(p - begin));
  }
  void ws()
  {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) p++;
  }
  bool lit(const char* s)
  {
    size_t n = strlen(s);
    if ((size_t)(end - p) >= n && memcmp(p, s, n) == 0)
    {
      p += n;
      return true;
    }
    return false;
  }
  static void put_utf8(std::string& out, unsigned cp)
  {
    if (cp < 0x80) out += (char)cp;
    else if (cp < 0x800)
    {
      out += (char)(0xC0 | (cp >> 6));
      out += (char)(0x80 | (cp & 0x3F));
    }
    else if (cp < 0x10000)
    {
      out += (char)(0xE0 | (cp >> 12));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    }
    else
    {
      out += (char)(0xF0 | (cp >> 18));
      out += (char)(0x80 | ((cp >> 12) & 0x3F));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    }
  }
  unsigned hex4()
  {
    if (end - p < 4) fail("short \\u escape");
    unsigned v = 0;
    for (int k = 0; k < 4; k++)
    {
      char c = *p++;
      v <<= 4;
      if (c >= '0' && c <= '9') v |= (unsigned)(c - '0');
      else if (c >= 'a' && c <= 'f') v |= (unsigned)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') v |= (unsigned)(c - 'A' + 10);
      else fail("bad \\u escape");
    }
    return v;
  }
  std::string string()
  {
    if (p >= end || *p != '"') fail("expected string");
    p++;
    std::string out;
    while (true)
    {
      if (p >= end) fail("unterminated string");
      char c = *p++;
      if (c == '"') break;
      if (c == '\\')
      {
        if (p >= end) fail("bad escape");
        char e = *p++;
        switch (e)
        {
          case '"': out += '"'; break;
          case '\\': out += '\\'; break;
          case '/': out += '/'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'n': out += '\n'; break;
          case 'r': out += '\r'; break;
          case 't': out += '\t'; break;
          case 'u':
          {
            unsigned cp = hex4();
            if (cp >= 0xD800 && cp < 0xDC00 && end - p >= 6 && p[0] == '\\' &&
                p[1] == 'u')
            {
              p += 2;
              unsigned lo = hex4();
              cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
            }
            put_utf8(out, cp);
            break;
          }
          default: fail("bad escape");
        }
      }
      else
        out += c;
    }
    return out;
  }
  Value number()
  {
    const char* s = p;
    if (p < end && *p == '-') p++;
    bool frac = false;
    while (p < end && ((*p >= '0' && *p <= '9') || *p == '.' || *p == 'e' ||
                       *p == 'E' || *p == '+' || *p == '-'))
    {
      if (*p == '.' || *p == 'e' || *p == 'E') frac = true;
      p++;
    }
    std::string tok(s, p);
    if (tok.empty() || tok == "-") fail("bad number");
    Value v;
    v.type = Value::NUMBER;
    char* ep = nullptr;
    v.num = strtod(tok.c_str(), &ep);
    if (ep == tok.c_str()) fail("bad number");
    if (!frac)
    {
      errno = 0;
      long long ll = strtoll(tok.c_str(), nullptr, 10);
      if (errno == 0)
      {
        v.is_int = true;
        v.i = ll;
      }
    }
    else if (std::isfinite(v.num) && v.num == std::floor(v.num) &&
             std::fabs(v.num) < 9.2e18)
    {
      v.is_int = true;
      v.i = (int64_t)v.num;
    }
    return v;
  }
  Value value(int depth)
  {
    if (depth > 256) fail("nesting too deep");
    ws();
    if (p >= end) fail("unexpected end");
    Value v;
    char c = *p;
    if (c == '{')
    {
      p++;
      v.type = Value::OBJECT;
      ws();
      if (p < end && *p == '}')
      {
        p++;
        return v;
      }
      while (true)
      {
        ws();
        std::string k = string();
        ws();
        if (p >= end || *p != ':') fail("expected ':'");
        p++;
        v.obj.emplace_back(std::move(k), value(depth + 1));
        ws();
        if (p < end && *p == ',')
        {
          p++;
          continue;
        }
        if (p < end && *p == '}')
        {
          p++;
          break;
        }
        fail("expected ',' or '}'");
      }
      return v;
    }
    if (c == '[')
    {
      p++;
      v.type = Value::ARRAY;
      ws();
      if (p < end && *p == ']')
      {
        p++;
        return v;
      }
      while (true)
      {
        v.arr.push_back(value(depth + 1));
        ws();
        if (p < end && *p == ',')
        {
          p++;
          continue;
        }
        if (p < end && *p == ']')
        {
          p++;
          break;
        }
        fail("expected ',' or ']'");
      }
      return v;
    }
    if (c == '"')
    {
      v.type = Value::STRING;
      v.str = string();
      return v;
    }
    if (lit("true"))
    {
      v.type = Value::BOOL;
      v.b = true;
      return v;
    }
    if (lit("false"))
    {
      v.type = Value::BOOL;
      v.b = false;
      return v;
    }
    if (lit("null")) return v;
    return number();
  }
};
}  // namespace

Value parse(const char* text, size_t len)
{
  Parser ps{text, text + len, text};
  Value v = ps.value(0);
  ps.ws();
  if (ps.p != ps.end) ps.fail("trailing characters");
  return v;
}

Value parse(const std::string& s) { return parse(s.data(), s.size()); }

std::string quote(const std::string& s)
{
  std::string o = "\"";
  for (char c : s)
  {
    switch (c)
    {
      case '"': o += "\\\""; break;
      case '\\': o += "\\\\"; break;
      case '\n': o += "\\n"; break;
      case '\t': o += "\\t"; break;
      case '\r': o += "\\r"; break;
      default:
        if ((unsigned char)c < 0x20)
        {
          char b[8];
          snprintf(b, sizeof b, "\\u%04x", (unsigned char)c);
          o += b;
        }
        else
          o += c;
    }
  }
  return o + "\"";
}

std::string number(double v)
{
  if (std::isnan(v)) return "null";
  if (std::isinf(v)) return v > 0 ? "1e308" : "-1e308";
  char b[40];
  snprintf(b, sizeof b, "%.17g", v);
  return b;
}
}  // namespace json
}  // namespace qio
