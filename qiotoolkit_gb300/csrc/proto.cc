// proto.cc -- protobuf model input (utils/proto_reader.h:28-150,
// utils/problem.proto): a folder <name> holding <name>_0.pb, <name>_1.pb,
// ... each a serialised QuantumUtil.Problem.  The first file carries the
// cost function's type and version and the first terms; later files add
// terms.  Decoded here from the proto3 wire format (no protobuf library):
//   Problem      { CostFunction cost_function = 1; Struct metadata = 2; }
//   CostFunction { ProblemType type = 1; string version = 2;
//                  repeated Term terms = 3; map<string,int64> init_config = 4; }
//   Term         { double c = 1; repeated int64 ids = 2; }
//   ProblemType  PUBO = 0, ISING = 1, MAXSAT = 2, SOFTSPIN = 3
// Checks and messages follow the reference reader; the initial
// configuration map and the metadata are skipped.
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "host.h"

namespace qio
{
namespace
{
struct Wire
{
  const uint8_t* p;
  const uint8_t* e;
  bool ok = true;
  bool done() const { return p >= e; }
  uint64_t varint()
  {
    uint64_t v = 0;
    for (int shift = 0; shift < 64; shift += 7)
    {
      if (p >= e)
      {
        ok = false;
        return 0;
      }
      const uint8_t b = *p++;
      v |= (uint64_t)(b & 0x7F) << shift;
      if (!(b & 0x80)) return v;
    }
    ok = false;
    return v;
  }
  uint64_t fixed64()
  {
    if (e - p < 8)
    {
      ok = false;
      p = e;
      return 0;
    }
    uint64_t v = 0;
    for (int i = 0; i < 8; i++) v |= (uint64_t)p[i] << (8 * i);
    p += 8;
    return v;
  }
  Wire sub()
  {
    const uint64_t n = varint();
    if (!ok || (uint64_t)(e - p) < n)
    {
      ok = false;
      p = e;
      return Wire{e, e};
    }
    Wire w{p, p + n};
    p += n;
    return w;
  }
  void skip(int wt)
  {
    if (wt == 0) varint();
    else if (wt == 1) fixed64();
    else if (wt == 2) sub();
    else if (wt == 5)
    {
      if (e - p < 4) ok = false;
      p += 4;
    }
    else ok = false;
  }
};

struct Decoded
{
  bool has_cf = false, has_type = false;
  int type = 0;
  std::string version;
  std::vector<double> c;
  std::vector<std::vector<int64_t>> ids;
};

void decode_term(Wire w, Decoded& d)
{
  double c = 0.0;
  std::vector<int64_t> ids;
  while (!w.done() && w.ok)
  {
    const uint64_t key = w.varint();
    const int field = (int)(key >> 3), wt = (int)(key & 7);
    if (field == 1 && wt == 1)
    {
      const uint64_t bits = w.fixed64();
      std::memcpy(&c, &bits, 8);
    }
    else if (field == 2 && wt == 2)  // packed
    {
      Wire pw = w.sub();
      while (!pw.done() && pw.ok) ids.push_back((int64_t)pw.varint());
      w.ok = w.ok && pw.ok;
    }
    else if (field == 2 && wt == 0)
      ids.push_back((int64_t)w.varint());
    else
      w.skip(wt);
  }
  if (!w.ok) fail(1, "Invalid problem message: malformed term");
  d.c.push_back(c);
  d.ids.push_back(std::move(ids));
}

void decode_cost_function(Wire w, Decoded& d)
{
  d.has_cf = true;
  while (!w.done() && w.ok)
  {
    const uint64_t key = w.varint();
    const int field = (int)(key >> 3), wt = (int)(key & 7);
    if (field == 1 && wt == 0)
    {
      d.type = (int)w.varint();
      d.has_type = true;
    }
    else if (field == 2 && wt == 2)
    {
      Wire sw = w.sub();
      d.version.assign((const char*)sw.p, (size_t)(sw.e - sw.p));
    }
    else if (field == 3 && wt == 2)
      decode_term(w.sub(), d);
    else
      w.skip(wt);
  }
  if (!w.ok) fail(1, "Invalid problem message: malformed cost function");
}

Decoded decode_problem(const std::string& bytes)
{
  Decoded d;
  Wire w{(const uint8_t*)bytes.data(), (const uint8_t*)bytes.data() + bytes.size()};
  while (!w.done() && w.ok)
  {
    const uint64_t key = w.varint();
    const int field = (int)(key >> 3), wt = (int)(key & 7);
    if (field == 1 && wt == 2) decode_cost_function(w.sub(), d);
    else w.skip(wt);
  }
  if (!w.ok) fail(1, "Invalid problem message: malformed protobuf");
  return d;
}

bool read_file(const std::string& path, std::string& out)
{
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) return false;
  out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return true;
}
}  // namespace

std::unique_ptr<HostModel> build_model_proto_folder(const std::string& folder_path)
{
  std::string path = folder_path;
  while (path.size() > 1 && (path.back() == '/' || path.back() == '\\')) path.pop_back();
  const size_t cut = path.find_last_of("/\\");
  const std::string name = cut == std::string::npos ? path : path.substr(cut + 1);
  int kind = -1;
  std::vector<int64_t> off{0};
  std::vector<int32_t> ids;
  std::vector<double> coef;
  for (int k = 0;; k++)
  {
    const std::string file = path + "/" + name + "_" + std::to_string(k) + ".pb";
    std::string bytes;
    if (!read_file(file, bytes))
    {
      if (k == 0) fail(1, "Could not open file: " + file);
      break;
    }
    Decoded d = decode_problem(bytes);
    if (!d.has_cf) fail(1, "Invalid problem message. No cost function found");
    if (k == 0)
    {
      if (d.type < 0 || d.type > 3)
        fail(1, "Expected type to be ising, pubo, maxsat or softspin. Invalid problem type specified. ");
      if (d.type == 3) fail(1, "model type softspin is outside the Metropolis path of this library");
      if (d.version != "1.0" && d.version != "1.1" && !d.version.empty())
        fail(1, "Expected version to be 1.0 or 1.1. Provided: " + d.version);
      if ((d.type == 0 || d.type == 1) && d.c.empty())
        fail(1, "Problem terms cannot be 0. Please add problem terms");
      kind = d.type == 1 ? K_ISING : (d.type == 0 ? K_PUBO : K_MAXSAT);
    }
    for (size_t t = 0; t < d.c.size(); t++)
    {
      for (int64_t v : d.ids[t])
      {
        if (v < INT32_MIN || v > INT32_MAX) fail(1, "variable id " + std::to_string(v) + " out of range");
        ids.push_back((int32_t)v);
      }
      off.push_back((int64_t)ids.size());
      coef.push_back(d.c[t]);
    }
  }
  return build_model(kind, (int64_t)coef.size(), off.data(), ids.data(), coef.data());
}
}  // namespace qio
