// dimacs.cc -- DIMACS cnf / wcnf input for MaxSAT models (utils/dimacs.cc,
// read by app/runner.cc:87-89).  Accepted input, as the reference's reader:
// comment lines starting with 'c'; one problem line `p cnf|wcnf <nvar>
// <nclauses> [top]` (top only for wcnf; it is parsed and not used by the
// MaxSat model); clauses of literals terminated by 0, preceded by the
// clause weight for wcnf (weight 1 for cnf).  A clause must not be empty
// and may not repeat a variable or hold it with both signs; the counts of
// clauses and of distinct variables must equal the problem line's.
#include <cctype>
#include <cstdlib>
#include <set>
#include <string>
#include <vector>

#include "host.h"

namespace qio
{
namespace
{
struct DimacsReader
{
  const std::string& s;
  size_t p = 0, line = 1, line_start = 0;
  explicit DimacsReader(const std::string& text) : s(text) {}

  std::string on_line() const { return "on line " + std::to_string(line); }
  std::string at(long offset = 0) const
  {
    return "on line " + std::to_string(line) + ", col " +
           std::to_string((long)p + offset - (long)line_start + 1);
  }
  void eat_ws()
  {
    while (p < s.size() && std::isspace((unsigned char)s[p]))
    {
      if (s[p] == '\n') line++;
      if (s[p] == '\n' || s[p] == '\r') line_start = p;
      p++;
    }
  }
  size_t token_len() const
  {
    size_t e = p;
    while (e < s.size() && !std::isspace((unsigned char)s[e])) e++;
    return e - p;
  }
  void skip_line()
  {
    while (p < s.size() && s[p] != '\n' && s[p] != '\r') p++;
    eat_ws();
  }
  long read_int()
  {
    eat_ws();
    const size_t n = token_len();
    std::string tok = s.substr(p, n);
    char* end = nullptr;
    long v = std::strtol(tok.c_str(), &end, 10);
    if (n == 0 || (size_t)(end - tok.c_str()) != n) fail(1, "Expected number " + at());
    p += n;
    return v;
  }
  double read_double()
  {
    eat_ws();
    const size_t n = token_len();
    std::string tok = s.substr(p, n);
    char* end = nullptr;
    double v = std::strtod(tok.c_str(), &end);
    if (n == 0 || (size_t)(end - tok.c_str()) != n) fail(1, "Expected number " + at());
    p += n;
    return v;
  }
  long read_positive()
  {
    const size_t before = p;
    long v = read_int();
    if (v <= 0) fail(1, "Expected positive number " + at((long)before - (long)p));
    return v;
  }
};
}  // namespace

std::unique_ptr<HostModel> build_model_dimacs(const std::string& text)
{
  DimacsReader r(text);
  std::string type;
  long nvar = 0, ncl = 0;
  std::vector<int64_t> off{0};
  std::vector<int32_t> ids;
  std::vector<double> weights;
  while (r.p < text.size())
  {
    const char c = text[r.p];
    if (c == 'c')
    {
      r.skip_line();
      continue;
    }
    if (c == 'p')
    {
      if (!type.empty()) fail(1, "Multiple problem lines in Dimacs file " + r.on_line());
      if (text.compare(r.p, 2, "p ") != 0) fail(1, "Expected 'p ' " + r.at());
      r.p += 2;
      r.eat_ws();
      const size_t n = r.token_len();
      type = text.substr(r.p, n);
      r.p += n;
      if (type != "cnf" && type != "wcnf")
        fail(1, "Expected `type` to be 'cnf' or 'wcnf' " + r.at(-(long)type.size()));
      nvar = r.read_positive();
      ncl = r.read_positive();
      if (type == "wcnf")
      {
        while (r.p < text.size() && (text[r.p] == ' ' || text[r.p] == '\t')) r.p++;
        if (r.p < text.size() && !std::isspace((unsigned char)text[r.p])) (void)r.read_double();  // top
      }
      r.eat_ws();
      continue;
    }
    // a clause
    const double w = type == "wcnf" ? r.read_double() : 1.0;
    std::set<long> seen;
    size_t count = 0;
    while (true)
    {
      const long v = r.read_int();
      if (v == 0)
      {
        if (count == 0) fail(1, "List of variables in a clause cannot be empty " + r.at());
        break;
      }
      if (seen.count(v)) fail(1, "Variable name " + std::to_string(v) + " appears multiple times in clause.");
      if (seen.count(-v))
        fail(1, "Variable name " + std::to_string(std::labs(v)) + " appears both positive and negative in clause.");
      seen.insert(v);
      ids.push_back((int32_t)v);
      count++;
    }
    off.push_back((int64_t)ids.size());
    weights.push_back(w);
    r.eat_ws();
  }
  if (type.empty()) fail(1, "Missing problem line in dimacs input");
  if ((long)weights.size() != ncl)
    fail(1, "Number of clauses parsed does not match: " + std::to_string(weights.size()) + "!=" +
                std::to_string(ncl));
  std::set<long> vars;
  for (int32_t v : ids) vars.insert(std::labs((long)v));
  if ((long)vars.size() != nvar)
    fail(1, "Number of variables found does not match: " + std::to_string(vars.size()) + "!=" +
                std::to_string(nvar));
  return build_model(K_MAXSAT, (int64_t)weights.size(), off.data(), ids.data(), weights.data());
}
}  // namespace qio
