// model_host.cc -- model construction and upload, schedules, device setup.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <set>

#include "host.h"

namespace qio
{
void fail(int status, const std::string& msg) { throw Error(status, msg); }

void cuda_check(cudaError_t e, const char* what)
{
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation)
    fail(2, std::string(what) + ": out of device memory");
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    fail(5, std::string(what) + ": " + cudaGetErrorString(e));
  fail(3, std::string(what) + ": " + cudaGetErrorString(e));
}

// Device bytes held in buffers.  QIO_DEVICE_MEMORY_LIMIT (bytes, read at
// each allocation) caps them, for callers that share a GPU: an allocation
// past the cap fails as out of device memory (status 2), as it would on a
// full device.
static std::atomic<long long> g_held{0};

static long long device_memory_limit()
{
  const char* e = std::getenv("QIO_DEVICE_MEMORY_LIMIT");
  return e ? std::atoll(e) : 0;
}

DevBuf::DevBuf(size_t n) : bytes(n)
{
  if (!n) return;
  const long long cap = device_memory_limit();
  if (cap > 0 && g_held.load() + (long long)n > cap)
    fail(2, "cudaMalloc: out of device memory (over QIO_DEVICE_MEMORY_LIMIT)");
  cuda_check(cudaMalloc(&ptr, n), "cudaMalloc");
  g_held += (long long)n;
}
DevBuf::~DevBuf()
{
  if (ptr)
  {
    cudaFree(ptr);
    g_held -= (long long)bytes;
  }
}
DevBuf& DevBuf::operator=(DevBuf&& o) noexcept
{
  if (this != &o)
  {
    if (ptr)
    {
      cudaFree(ptr);
      g_held -= (long long)bytes;
    }
    ptr = o.ptr;
    bytes = o.bytes;
    o.ptr = nullptr;
    o.bytes = 0;
  }
  return *this;
}

static std::mutex g_dev_mu;
static std::map<int, int*> g_err;

int* device_error_flag()
{
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> g(g_dev_mu);
  auto it = g_err.find(dev);
  return it == g_err.end() ? nullptr : it->second;
}

void check_device_error(cudaStream_t s)
{
  int* e = device_error_flag();
  if (!e) return;
  int h = 0;
  cuda_check(cudaMemcpyAsync(&h, e, 4, cudaMemcpyDeviceToHost, s), "D2H error flag");
  cuda_check(cudaStreamSynchronize(s), "sync");
  if (h)
  {
    cuda_check(cudaMemsetAsync(e, 0, 4, s), "memset");
    fail(4, "a device-side wait for a bulk copy gave up (bounded wait); results are invalid");
  }
}

void ensure_device()
{
  static std::mutex& mu = g_dev_mu;
  static std::set<int> ready;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    fail(5, "no CUDA device available: the GB300 library has no CPU fallback");
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> g(mu);
  if (ready.count(dev)) return;
  upload_tables(dev);
  cuda_check(cudaGetLastError(), "upload_tables");
  int* flag = nullptr;
  cuda_check(cudaMalloc(&flag, 4), "cudaMalloc");
  cuda_check(cudaMemset(flag, 0, 4), "cudaMemset");
  g_err[dev] = flag;
  ready.insert(dev);
}

// ---------------------------------------------------------------------------
// Graph models: normalize_edges (graph/graph.h:74-177).  Names are numbered
// in order of first appearance; a repeated name in a term throws for Ising
// ("Duplicated ids detected in term!") and is merged for PUBO
// (model/pubo.h:82); members are sorted; terms without members add to the
// constant cost; each variable lists its terms in ascending term id.
// ---------------------------------------------------------------------------
static void build_graph(HostModel& m, int64_t n_terms, const int64_t* off,
                        const int32_t* ids, const double* coef)
{
  if (n_terms <= 0)
    fail(1, "parameter `terms`: size must be greater than 0, found 0");
  const bool merge = (m.kind == K_PUBO || m.kind == K_PUBO_PLAIN);
  std::map<int32_t, int> name_to_id;
  std::vector<std::vector<int>> members;
  std::vector<std::vector<int>> node_edges;
  m.min_loc = INT32_MAX;
  m.min_coupling = std::numeric_limits<double>::max();
  for (int64_t t = 0; t < n_terms; t++)
  {
    if (off[t + 1] < off[t]) fail(1, "term offsets must be non-decreasing");
    std::vector<int> mem;
    for (int64_t k = off[t]; k < off[t + 1]; k++)
    {
      auto it = name_to_id.find(ids[k]);
      int id;
      if (it == name_to_id.end())
      {
        id = (int)m.names.size();
        name_to_id.emplace(ids[k], id);
        m.names.push_back(ids[k]);
        node_edges.emplace_back();
      }
      else
        id = it->second;
      if (std::find(mem.begin(), mem.end(), id) == mem.end())
      {
        mem.push_back(id);
        node_edges[id].push_back((int)members.size());
      }
      else if (!merge)
        fail(1, "Duplicated ids detected in term!");
    }
    std::sort(mem.begin(), mem.end());
    int loc = (int)mem.size();
    m.max_loc = std::max(m.max_loc, loc);
    m.min_loc = std::min(m.min_loc, loc);
    m.total_loc += loc;
    if (!mem.empty())
    {
      m.accum_dep += (int64_t)loc * (loc - 1);
      m.min_coupling = std::min(m.min_coupling, std::fabs(coef[t]));
      m.max_coupling = std::max(m.max_coupling, std::fabs(coef[t]));
      members.push_back(std::move(mem));
      m.tcost.push_back(coef[t]);
    }
    else
      m.const_cost += coef[t];
  }
  if (m.min_loc == INT32_MAX) m.min_loc = 0;
  m.N = (int64_t)m.names.size();
  m.M = (int64_t)members.size();
  if (m.N > INT32_MAX / 2 || m.M > INT32_MAX / 2) fail(1, "model too large");
  m.row.assign(m.N + 1, 0);
  for (int64_t v = 0; v < m.N; v++) m.row[v + 1] = m.row[v] + (int)node_edges[v].size();
  m.K = m.row[m.N];
  m.inc.resize(m.K);
  m.coef.resize(m.K);
  for (int64_t v = 0; v < m.N; v++)
    for (size_t j = 0; j < node_edges[v].size(); j++)
    {
      int t = node_edges[v][j];
      m.inc[m.row[v] + j] = (uint32_t)t;
      m.coef[m.row[v] + j] = m.tcost[t];
    }
  m.trow.assign(m.M + 1, 0);
  for (int64_t t = 0; t < m.M; t++) m.trow[t + 1] = m.trow[t] + (int)members[t].size();
  m.tvar.resize(m.trow[m.M]);
  for (int64_t t = 0; t < m.M; t++)
    for (size_t j = 0; j < members[t].size(); j++)
      m.tvar[m.trow[t] + j] = (uint32_t)members[t][j];
}

// ---------------------------------------------------------------------------
// MaxSat::configure(clauses) (model/max_sat.h:295-397): clauses containing a
// variable and its negation are always true and dropped; variables used
// only there are free (rendered as 1); the remaining variables are numbered
// by ascending name; clause c (1-based in the reference, c-1 here) lists
// each variable once, negated literals marked.
// ---------------------------------------------------------------------------
static void build_maxsat(HostModel& m, int64_t n_terms, const int64_t* off,
                         const int32_t* ids, const double* coef)
{
  if (n_terms <= 0) fail(1, "parameter `terms` must not be empty");
  std::vector<char> always(n_terms, 0);
  std::set<int32_t> used, maybe_free;
  for (int64_t c = 0; c < n_terms; c++)
  {
    std::set<int32_t> seen;
    for (int64_t k = off[c]; k < off[c + 1]; k++)
    {
      int32_t v = ids[k];
      if (v == 0 || v == INT32_MIN)
        fail(1, "MaxSat variables cannot have the name " + std::to_string(v) +
                    " since it cannot be negated to indicate 'not " +
                    std::to_string(v) + "'.");
      if (seen.count(-v)) always[c] = 1;
      seen.insert(v);
    }
    for (int32_t v : seen) (always[c] ? maybe_free : used).insert(std::abs(v));
  }
  for (int32_t v : maybe_free)
    if (!used.count(v)) m.free_vars.push_back(v);
  m.names.assign(used.begin(), used.end());
  m.N = (int64_t)m.names.size();
  std::map<int32_t, int> name_to_id;
  for (size_t i = 0; i < m.names.size(); i++) name_to_id[m.names[i]] = (int)i;
  std::vector<std::vector<uint32_t>> affected(m.N);
  std::vector<std::vector<uint32_t>> members;
  m.min_loc = INT32_MAX;
  for (int64_t c = 0; c < n_terms; c++)
  {
    if (always[c]) continue;
    int t = (int)members.size();
    m.tcost.push_back(coef[c]);
    m.max_coupling = std::max(m.max_coupling, std::fabs(coef[c]));
    std::vector<uint32_t> mem;
    std::set<int> seen;
    for (int64_t k = off[c]; k < off[c + 1]; k++)
    {
      int32_t name = ids[k];
      int id = name_to_id[std::abs(name)];
      if (seen.count(id)) continue;
      seen.insert(id);
      uint32_t neg = name < 0 ? kNegBit : 0u;
      affected[id].push_back((uint32_t)t | neg);
      mem.push_back((uint32_t)id | neg);
    }
    m.max_loc = std::max(m.max_loc, (int)mem.size());
    m.min_loc = std::min(m.min_loc, (int)mem.size());
    members.push_back(std::move(mem));
  }
  if (m.min_loc == INT32_MAX) m.min_loc = 0;
  m.M = (int64_t)members.size();
  if (m.M == 0)
  {
    // the model is "empty": every clause is always true
    m.N = 0;
    m.names.clear();
  }
  m.row.assign(m.N + 1, 0);
  for (int64_t v = 0; v < m.N; v++) m.row[v + 1] = m.row[v] + (int)affected[v].size();
  m.K = m.row[m.N];
  m.inc.resize(m.K);
  m.coef.resize(m.K);
  for (int64_t v = 0; v < m.N; v++)
    for (size_t j = 0; j < affected[v].size(); j++)
    {
      uint32_t e = affected[v][j];
      m.inc[m.row[v] + j] = e;
      m.coef[m.row[v] + j] = m.tcost[e & ~kNegBit];
    }
  m.trow.assign(m.M + 1, 0);
  for (int64_t t = 0; t < m.M; t++) m.trow[t + 1] = m.trow[t] + (int)members[t].size();
  m.tvar.resize(m.trow[m.M]);
  for (int64_t t = 0; t < m.M; t++)
    for (size_t j = 0; j < members[t].size(); j++) m.tvar[m.trow[t] + j] = members[t][j];
}

// Window-conflict masks: bit d-1 of nbr[v] is set when variable v-d (d in
// 1..32) shares a term with v.
static void build_nbr(HostModel& m)
{
  m.nbr.assign(m.N, 0u);
  std::vector<int> mem;
  for (int64_t t = 0; t < m.M; t++)
  {
    mem.clear();
    for (int k = m.trow[t]; k < m.trow[t + 1]; k++) mem.push_back((int)(m.tvar[k] & ~kNegBit));
    std::sort(mem.begin(), mem.end());
    for (size_t j = 0; j < mem.size(); j++)
      for (size_t i = j; i-- > 0;)
      {
        int d = mem[j] - mem[i];
        if (d > 32) break;
        if (d >= 1) m.nbr[mem[j]] |= 1u << (d - 1);
      }
  }
}

// Later co-members for the per-block field updates: for incidence k of v
// (term t), each member u of t with 0 < u - v <= 31 and a row of at most 32
// incidences, encoded as (u - v, position of t in u's row).  When u flips
// nothing is posted (it has been decided already); when v flips, these are
// the undecided variables of the same 32-variable block whose cost
// difference changes.
static void build_levels(HostModel& m);

static void build_near(HostModel& m)
{
  m.near.assign(m.K, 0ULL);
  for (int64_t v = 0; v < m.N; v++)
    for (int q = m.row[v]; q < m.row[v + 1]; q++)
    {
      uint32_t t = m.inc[q] & ~kNegBit;
      unsigned long long w = 0;
      int cnt = 0;
      bool over = false;
      for (int j = m.trow[t]; j < m.trow[t + 1]; j++)
      {
        int64_t u = (int64_t)(m.tvar[j] & ~kNegBit);
        int64_t d = u - v;
        if (d < 1 || d > 31) continue;
        if (m.row[u + 1] - m.row[u] > 32) continue;
        int kp = -1;
        for (int x = m.row[u]; x < m.row[u + 1]; x++)
          if ((m.inc[x] & ~kNegBit) == t) { kp = x - m.row[u]; break; }
        if (kp < 0) continue;
        if (cnt == 6) { over = true; break; }
        w |= ((unsigned long long)d | ((unsigned long long)kp << 5)) << (10 * cnt);
        cnt++;
      }
      m.near[q] = over ? (7ULL << 61) : (w | ((unsigned long long)cnt << 61));
    }
}

// Records of the field-cached sweep.  The local field of a variable is the
// sum, over its contributing incidences, of the coefficients in fixed point
// q = round(c * 2^S): Ising, every incidence, +q for a term whose parity bit
// is clear and -q otherwise (the cost difference is -2 times the sum);
// counter models, the incidences whose term the flip would switch, +q when
// the variable's literal is true and -q otherwise.  S is the largest scale
// with 2^S * max_v sum_row |c| <= 2^30 (2^22 when the field also carries the
// count of contributing incidences in its low 8 bits), so a field never
// overflows and differs from the reference's FP64 sum by less than deg + 1
// units.  Integer models use S = 0: the field is then the exact difference.
// Eligible: Ising with the term cache or counter models, fewer than 32766
// variables, rows of at most 255 incidences.
static void build_fields(HostModel& m)
{
  m.fc_rec.clear();
  if (!(m.flavor == F_PARITY || m.flavor == F_COUNTER) || m.N == 0 || m.N >= 32766) return;
  double amax = 0;
  for (int64_t v = 0; v < m.N; v++)
  {
    if (m.row[v + 1] - m.row[v] > 255) return;
    double s = 0;
    for (int q = m.row[v]; q < m.row[v + 1]; q++) s += std::fabs(m.coef[q]);
    amax = std::max(amax, s);
  }
  m.fc_pack = !m.int_mode && m.flavor == F_COUNTER;
  if (m.int_mode) m.fc_S = 0;
  else
  {
    const int top = m.fc_pack ? 22 : 30;
    int e = 0;
    if (amax > 0) std::frexp(amax, &e);  // amax < 2^e
    m.fc_S = amax > 0 ? top - e : 0;
    if (m.fc_S < -900 || m.fc_S > 900) return;  // 2^-S must stay a normal double
  }
  m.fc_rec.assign((size_t)m.K * 4, 0u);
  for (int64_t v = 0; v < m.N; v++)
    for (int q = m.row[v]; q < m.row[v + 1]; q++)
    {
      const uint32_t t = m.inc[q] & ~kNegBit;
      long long fq = m.int_mode ? (long long)m.coef_i[q] : std::llrint(std::ldexp(m.coef[q], m.fc_S));
      if (m.fc_pack) fq *= 256;
      uint32_t co[3] = {0xFFFFu, 0xFFFFu, 0xFFFFu};
      int nco = 0;
      for (int j = m.trow[t]; j < m.trow[t + 1]; j++)
      {
        const uint32_t u = m.tvar[j] & ~kNegBit;
        if ((int64_t)u == v) continue;
        if (nco < 3) co[nco] = u | ((m.tvar[j] & kNegBit) ? 0x8000u : 0u);
        nco++;
      }
      if (nco > 3) nco = 15;
      uint32_t* r = &m.fc_rec[(size_t)q * 4];
      r[0] = m.inc[q];
      r[1] = (uint32_t)(int32_t)fq;
      r[2] = co[0] | (co[1] << 16);
      r[3] = co[2] | ((uint32_t)nco << 16);
    }
}

// Integer mode: every coefficient is an integer of magnitude <= 2^20 and the
// per-variable sums stay below 2^30, so int32/int64 arithmetic gives the same
// values as the reference's FP64 sums (all partial sums are exact).
static void detect_int_mode(HostModel& m)
{
  bool ok = m.M > 0;
  for (double c : m.tcost)
    if (!(std::floor(c) == c && std::fabs(c) <= 1048576.0)) { ok = false; break; }
  if (ok)
    for (int64_t v = 0; v < m.N && ok; v++)
    {
      double s = 0;
      for (int q = m.row[v]; q < m.row[v + 1]; q++) s += std::fabs(m.coef[q]);
      if (2 * s >= 1073741824.0) ok = false;
    }
  m.int_mode = ok;
  m.fscreen = true;
  m.scan32 = false;
  if (!ok)
  {
    m.coef_f.resize(m.K);
    for (int64_t q = 0; q < m.K; q++)
    {
      const double a = std::fabs(m.coef[q]);
      if (!(a == 0.0 || (a >= 1e-30 && a <= 1e30))) m.fscreen = false;
      m.coef_f[q] = (float)m.coef[q];
    }
  }
  else
  {
    double mx = 0;
    for (int64_t v = 0; v < m.N; v++)
    {
      double s = 0;
      for (int q = m.row[v]; q < m.row[v + 1]; q++) s += std::fabs(m.coef[q]);
      mx = std::max(mx, 2 * s);
    }
    m.scan32 = 32.0 * mx < 2147483647.0;
  }
  if (ok)
  {
    m.coef_i.resize(m.K);
    for (int64_t q = 0; q < m.K; q++) m.coef_i[q] = (int)m.coef[q];
    m.tcost_i.resize(m.M);
    for (int64_t t = 0; t < m.M; t++) m.tcost_i[t] = (int)m.tcost[t];
  }
}

std::unique_ptr<HostModel> build_model(int kind, int64_t n_terms,
                                       const int64_t* off, const int32_t* ids,
                                       const double* coef)
{
  if (kind < 0 || kind > 4) fail(1, "unknown model kind " + std::to_string(kind));
  if (n_terms < 0 || (n_terms > 0 && (!off || !coef)))
    fail(1, "model arrays must not be null");
  std::unique_ptr<HostModel> m(new HostModel());
  m->kind = kind;
  if (kind == K_MAXSAT) build_maxsat(*m, n_terms, off, ids, coef);
  else build_graph(*m, n_terms, off, ids, coef);
  switch (kind)
  {
    case K_ISING: m->flavor = F_PARITY; break;
    case K_ISING_PLAIN: m->flavor = F_PLAIN_ISING; break;
    case K_PUBO: m->flavor = F_COUNTER; break;
    case K_PUBO_PLAIN: m->flavor = F_PLAIN_PUBO; break;
    default: m->flavor = F_COUNTER; break;
  }
  // byte counters hold up to 255 members; wider PUBO terms use the
  // counter-free evaluation (same results, model::Pubo semantics)
  if (m->flavor == F_COUNTER && m->max_loc > 255)
  {
    if (kind == K_MAXSAT) fail(1, "MaxSat clauses with more than 255 variables are not supported");
    m->flavor = F_PLAIN_PUBO;
  }
  // GraphProperties::rescale (graph/graph_properties.h:24-40)
  // (MaxSat keeps markov::Model's default factor 1, markov/model.h:193)
  m->scale_factor = (kind == K_MAXSAT || m->max_coupling <= 1 || m->max_coupling == 0)
                        ? 1.0
                        : 1.0 / m->max_coupling;
  build_nbr(*m);
  detect_int_mode(*m);
  build_fields(*m);
  if (m->flavor == F_PARITY || m->flavor == F_COUNTER) build_near(*m);
  if (m->flavor == F_PARITY)
  {
    // term parity from the member spins: with one or two members per term
    // the cached term bit is the other member's spin (or a constant)
    bool pair = m->M > 0;
    for (int64_t t = 0; t < m->M && pair; t++) pair = m->trow[t + 1] - m->trow[t] <= 2;
    m->pair_only = pair;
    if (pair)
    {
      m->other.assign(m->K, -1);
      for (int64_t v = 0; v < m->N; v++)
        for (int q = m->row[v]; q < m->row[v + 1]; q++)
        {
          uint32_t t = m->inc[q] & ~kNegBit;
          for (int j = m->trow[t]; j < m->trow[t + 1]; j++)
          {
            int u = (int)(m->tvar[j] & ~kNegBit);
            if (u != v) m->other[q] = u;
          }
        }
      const int pad = (int)(((m->N + 31) / 32) * 32);  // the padding spin
      if (m->int_mode)
      {
        m->rec_i.resize(2 * m->K);
        bool small = pad < (1 << 24);
        for (int64_t q = 0; q < m->K; q++)
        {
          m->rec_i[2 * q] = m->other[q] >= 0 ? m->other[q] : pad;
          m->rec_i[2 * q + 1] = m->coef_i[q];
          small = small && m->coef_i[q] >= -128 && m->coef_i[q] <= 127;
        }
        if (small)
        {
          m->rec_p.resize(m->K);
          for (int64_t q = 0; q < m->K; q++)
            m->rec_p[q] = ((unsigned)m->rec_i[2 * q] << 8) | ((unsigned)m->coef_i[q] & 0xFFu);
        }
        build_levels(*m);
      }
      else
      {
        m->rec_f.resize(2 * m->K);
        for (int64_t q = 0; q < m->K; q++)
        {
          long long u = m->other[q] >= 0 ? m->other[q] : pad;
          double ub;
          memcpy(&ub, &u, 8);
          m->rec_f[2 * q] = ub;
          m->rec_f[2 * q + 1] = m->coef[q];
        }
      }
    }
  }
  return m;
}

// Level schedule of an ordered sweep (levels.cu): level(v) = 1 + the largest
// level among v's neighbours u < v, 0 without one, so neighbours never share
// a level and each variable comes after its lower neighbours and before its
// higher ones.  Entries list the variables level by level (index order
// within a level); with 8-bit coefficients and at most 15 incidences per
// variable an entry carries the variable's records too (4, 8 or 16 words),
// else it is the variable alone.  The kernel sums a lane's differences in
// 32-bit integers: models whose differences could overflow them stay on the
// other kernels.
static void build_levels(HostModel& m)
{
  m.lv_ok = m.lv_d8 = false;
  m.n_levels = m.lv_recs = m.lv_width = 0;
  m.lv_off.clear();
  m.lv_ent.clear();
  m.lv_pos.clear();
  if (m.N <= 0) return;
  std::vector<int> L((size_t)m.N, 0);
  int maxl = 0, maxdeg = 0;
  long long bound = 0, widest = 0;  // sum and largest of the variables' |largest difference|
  for (int64_t v = 0; v < m.N; v++)
  {
    int l = 0;
    for (int q = m.row[v]; q < m.row[v + 1]; q++)
    {
      const int u = m.other[q];
      if (u >= 0 && u < v) l = std::max(l, L[u] + 1);
      bound += 2LL * std::llabs((long long)m.coef_i[q]);
    }
    long long dv = 0;
    for (int q = m.row[v]; q < m.row[v + 1]; q++) dv += 2LL * std::llabs((long long)m.coef_i[q]);
    widest = std::max(widest, dv);
    L[v] = l;
    maxl = std::max(maxl, l);
    maxdeg = std::max(maxdeg, m.row[v + 1] - m.row[v]);
  }
  if (bound >= (1LL << 31)) return;
  const int nl = maxl + 1;
  std::vector<int> off((size_t)nl + 1, 0);
  for (int64_t v = 0; v < m.N; v++) off[L[v] + 1]++;
  int width = 0;
  for (int t = 0; t < nl; t++)
  {
    width = std::max(width, off[t + 1]);
    off[t + 1] += off[t];
  }
  // record slots of an entry: the fewest of 3, 4, 6, 7, 15 that hold the
  // largest row (8-bit coefficients only), else 0 (the variable alone)
  int recs = 0;
  if (!m.rec_p.empty())
    for (int c : {3, 4, 6, 7, 15})
      if (maxdeg <= c)
      {
        recs = c;
        break;
      }
  const int ew = recs ? lv_entry_words(recs) : 1;
  const int pad = (int)(((m.N + 31) / 32) * 32);
  std::vector<int> fill(off.begin(), off.end() - 1);
  std::vector<uint32_t> ent((size_t)m.N * ew, recs ? lv_record(pad, 0) : 0u);
  std::vector<int> pos((size_t)((m.N + 31) / 32) * 32, 0);
  for (int64_t v = 0; v < m.N; v++)
  {
    pos[v] = fill[L[v]];
    uint32_t* e = &ent[(size_t)fill[L[v]]++ * ew];
    e[0] = (uint32_t)v;
    if (recs)
      for (int q = m.row[v], j = 1; q < m.row[v + 1]; q++, j++)
        e[j] = lv_record(m.other[q] >= 0 ? m.other[q] : pad, m.coef_i[q]);
  }
  m.lv_off.swap(off);
  m.lv_ent.swap(ent);
  m.lv_pos.swap(pos);
  m.n_levels = nl;
  m.lv_recs = recs;
  m.lv_width = width;
  m.lv_d8 = widest <= 127;
  m.lv_ok = true;
}

template <class T>
static size_t put(std::vector<char>& blob, const std::vector<T>& v)
{
  size_t o = (blob.size() + 255) & ~(size_t)255;
  blob.resize(o + v.size() * sizeof(T));
  if (!v.empty()) memcpy(blob.data() + o, v.data(), v.size() * sizeof(T));
  return o;
}

void HostModel::upload() const
{
  ensure_device();
  std::vector<char> blob;
  size_t o_row = put(blob, row), o_inc = put(blob, inc), o_coef = put(blob, coef),
         o_ci = put(blob, coef_i), o_nbr = put(blob, nbr), o_trow = put(blob, trow),
         o_tvar = put(blob, tvar), o_tc = put(blob, tcost), o_tci = put(blob, tcost_i),
         o_cf = put(blob, coef_f), o_near = put(blob, near), o_oth = put(blob, other),
         o_ri = put(blob, rec_i), o_rf = put(blob, rec_f), o_rp = put(blob, rec_p),
         o_lo = put(blob, lv_off), o_le = put(blob, lv_ent), o_lp = put(blob, lv_pos),
         o_fc = put(blob, fc_rec);
  // 256 bytes of tail padding: bulk copies of incidence ranges round their
  // end up to 16 bytes
  blob.resize(((blob.size() + 255) & ~(size_t)255) + 256);
  dmem = DevBuf(blob.size());
  cuda_check(cudaMemcpy(dmem.ptr, blob.data(), blob.size(), cudaMemcpyHostToDevice),
             "model upload");
  char* b = (char*)dmem.ptr;
  dev.flavor = flavor;
  dev.n_vars = (int)N;
  dev.n_terms = (int)M;
  dev.sweep_size = (int)N;
  dev.int_mode = int_mode ? 1 : 0;
  dev.row = (const int*)(b + o_row);
  dev.inc = (const uint32_t*)(b + o_inc);
  dev.coef = (const double*)(b + o_coef);
  dev.coef_i = int_mode ? (const int*)(b + o_ci) : nullptr;
  dev.nbr = (const uint32_t*)(b + o_nbr);
  dev.trow = (const int*)(b + o_trow);
  dev.tvar = (const uint32_t*)(b + o_tvar);
  dev.tcost = (const double*)(b + o_tc);
  dev.tcost_i = int_mode ? (const int*)(b + o_tci) : nullptr;
  dev.coef_f = int_mode ? nullptr : (const float*)(b + o_cf);
  dev.near = near.empty() ? nullptr : (const unsigned long long*)(b + o_near);
  dev.fscreen = fscreen ? 1 : 0;
  dev.scan32 = scan32 ? 1 : 0;
  dev.pair_only = pair_only ? 1 : 0;
  int md = 0;
  for (int64_t v = 0; v < N; v++) md = std::max(md, row[v + 1] - row[v]);
  dev.max_deg = md;
  int mb = 0;
  for (int64_t b = 0; b < N; b += 32) mb = std::max(mb, row[std::min<int64_t>(b + 32, N)] - row[b]);
  dev.max_block_inc = mb;
  dev.other = other.empty() ? nullptr : (const int*)(b + o_oth);
  dev.rec_i = rec_i.empty() ? nullptr : (const int2*)(b + o_ri);
  dev.rec_f = rec_f.empty() ? nullptr : (const double2*)(b + o_rf);
  dev.rec_p = rec_p.empty() ? nullptr : (const unsigned int*)(b + o_rp);
  dev.lv_ok = lv_ok ? 1 : 0;
  dev.lv_off = lv_ok ? (const int*)(b + o_lo) : nullptr;
  dev.lv_ent = lv_ok ? (const uint32_t*)(b + o_le) : nullptr;
  dev.lv_pos = lv_ok ? (const int*)(b + o_lp) : nullptr;
  dev.n_levels = lv_ok ? n_levels : 0;
  dev.lv_recs = lv_ok ? lv_recs : 0;
  dev.lv_d8 = lv_d8 ? 1 : 0;
  dev.fc_rec = fc_rec.empty() ? nullptr : (const uint4*)(b + o_fc);
  dev.fc_S = fc_S;
  dev.fc_pack = fc_pack ? 1 : 0;
  dev.fc_inv = std::ldexp(1.0, -fc_S);
  int ordinal = -1;
  cuda_check(cudaGetDevice(&ordinal), "cudaGetDevice");
  upload_device = ordinal;
  uploaded = true;
}

DevModel HostModel::device_view(bool full_maxsat_sweep) const
{
  DevModel d = device();
  // MaxSat does not override get_sweep_size() (markov/model.h:169): one
  // attempt (variable 0) per sweep unless the full sweep is requested.
  if (kind == K_MAXSAT && !full_maxsat_sweep) d.sweep_size = N > 0 ? 1 : 0;
  return d;
}

static std::vector<int32_t> flatten_ids(const json::Value& terms, std::vector<int64_t>& off,
                                        std::vector<double>& coef)
{
  std::vector<int32_t> ids;
  off.assign(1, 0);
  for (const auto& t : terms.arr)
  {
    const json::Value* c = t.find("c");
    const json::Value* i = t.find("ids");
    if (!c || !c->is_number()) fail(1, "parameter `c` is required");
    if (!i || !i->is_array()) fail(1, "parameter `ids` is required");
    coef.push_back(c->num);
    for (const auto& x : i->arr)
    {
      if (!x.is_number() || !x.is_int) fail(1, "ids must be integers");
      ids.push_back((int32_t)x.i);
    }
    off.push_back((int64_t)ids.size());
  }
  return ids;
}

std::unique_ptr<HostModel> build_model_json(const json::Value& doc, int kind)
{
  const json::Value* cf = doc.find("cost_function");
  if (!cf || !cf->is_object()) fail(1, "Input field `cost_function` is required.");
  const json::Value* type = cf->find("type");
  if (kind < 0)
  {
    if (!type || !type->is_string()) fail(1, "parameter `type` is required");
    if (type->str == "ising") kind = K_ISING;
    else if (type->str == "pubo") kind = K_PUBO;
    else if (type->str == "maxsat") kind = K_MAXSAT;
    else fail(1, "Unknown model type: " + type->str);
  }
  const json::Value* ver = cf->find("version");
  if (ver && ver->is_string() && kind != K_MAXSAT && ver->str != "1.0" && ver->str != "1.1")
    fail(1, "Expecting `version` equals 1.0 or 1.1, but found: " + ver->str);
  const json::Value* terms = cf->find("terms");
  if (!terms || !terms->is_array()) fail(1, "parameter `terms` is required");
  std::vector<int64_t> off;
  std::vector<double> coef;
  std::vector<int32_t> ids = flatten_ids(*terms, off, coef);
  return build_model(kind, (int64_t)coef.size(), off.data(), ids.data(), coef.data());
}

// ---------------------------------------------------------------------------
// Schedules.  Linear a + p(b-a) (schedule/linear.cc:15-18), geometric
// a(b/a)^p (schedule/geometric.cc:9-12), lists of constant points
// (Segments of constants, schedule/segments.cc:15-43,45-110), input mapping
// and clamping (schedule/schedule.cc:17-25), discretisation (38-89).
// ---------------------------------------------------------------------------
double Schedule::progress_value(double p) const
{
  switch (type)
  {
    case 0: return initial + p * (final_ - initial);
    case 1: return initial * pow(final_ / initial, p);
    case 2: return initial;
    default:
    {
      double position = get_start() + p * (get_stop() - get_start());
      if (position < 0) return values.front();
      for (size_t i = 0; i < values.size(); i++)
      {
        double stop = (double)i;
        if (position > stop) continue;
        double start = (double)i;
        if (i > 0 && position < start)
        {
          double last_stop = (double)(i - 1);
          double q = (position - last_stop) / (start - last_stop);
          return (1 - q) * values[i - 1] + q * values[i];
        }
        return values[i];
      }
      return values.back();
    }
  }
}
double Schedule::get_start() const { return has_start ? start_ : 0; }
double Schedule::get_stop() const
{
  if (has_stop) return stop_;
  if (type == 3) return (double)values.size() - 1;
  return 1;
}
int Schedule::get_count() const
{
  if (has_count) return count_;
  if (type == 3) return (int)values.size();
  return (int)round(std::abs(get_stop() - get_start()));
}
double Schedule::get_value(double input) const
{
  double start = get_start(), stop = get_stop();
  if (start == stop) return progress_value(0);
  double progress = (input - start) / (stop - start);
  return progress_value(std::min(1., std::max(0., progress)));
}
std::vector<double> Schedule::discretized() const
{
  int count = get_count();
  if (count < 2) fail(1, "Can not get_discretized_values(count) for less than 2 values");
  std::vector<double> d;
  for (int i = 0; i < count; i++) d.push_back(progress_value(double(i) / (count - 1)));
  return d;
}
std::string Schedule::render() const
{
  if (type == 0 || type == 1)
    return std::string("{\"type\":\"") + (type == 0 ? "linear" : "geometric") +
           "\",\"initial\":" + json::number(initial) + ",\"final\":" + json::number(final_) + "}";
  if (type == 2) return json::number(initial);
  std::string s = "{\"type\":\"segments\",\"segments\":[";
  for (size_t i = 0; i < values.size(); i++)
    s += (i ? "," : "") + std::string("{\"value\":") + json::number(values[i]) + "}";
  return s + "]}";
}

Schedule parse_schedule(const json::Value& v, const std::string& name)
{
  Schedule s;
  if (v.is_number())
  {
    s.type = 2;
    s.initial = v.num;
    return s;
  }
  if (v.is_array())
  {
    if (v.arr.empty())
      fail(1, "parameter `" + name + "`: unable to initialize schedule:\n  Linear: parameter `type` is required\n  Geometric: parameter `type` is required\n  Segments: `segments` must be specified as a non-empty array.\n  Constant: expected double, found array");
    s.type = 3;
    for (const auto& x : v.arr)
    {
      if (!x.is_number()) fail(1, "parameter `" + name + "`: list values must be numbers");
      s.values.push_back(x.num);
    }
    return s;
  }
  if (!v.is_object()) fail(1, "parameter `" + name + "`: unable to initialize schedule");
  const json::Value* type = v.find("type");
  std::string t = (type && type->is_string()) ? type->str : "";
  auto num = [&](const char* k, double& out, bool required) {
    const json::Value* x = v.find(k);
    if (!x) { if (required) fail(1, "parameter `" + std::string(k) + "` is required"); return false; }
    if (!x->is_number()) fail(1, "parameter `" + std::string(k) + "`: expected number");
    out = x->num;
    return true;
  };
  if (t == "linear" || t == "geometric")
  {
    s.type = t == "linear" ? 0 : 1;
    num("initial", s.initial, true);
    num("final", s.final_, true);
    if (s.type == 1 && s.initial <= 0) fail(1, "initial must be positive for geometric");
    if (s.type == 1 && s.final_ <= 0) fail(1, "final must be positive for geometric");
  }
  else if (t == "constant")
  {
    s.type = 2;
    num("value", s.initial, true);
  }
  else if (t == "segments")
  {
    s.type = 3;
    const json::Value* segs = v.find("segments");
    if (!segs || !segs->is_array() || segs->arr.empty())
      fail(1, "`segments` must be specified as a non-empty array.");
    for (const auto& x : segs->arr)
    {
      if (x.is_number()) s.values.push_back(x.num);
      else if (x.is_object() && x.find("value") && x["value"].is_number())
        s.values.push_back(x["value"].num);
      else fail(1, "only constant segments are supported");
    }
  }
  else
    fail(1, "parameter `" + name + "`: unable to initialize schedule:\n  Linear: parameter `type` is required");
  double d;
  if (num("start", d, false)) { s.has_start = true; s.start_ = d; }
  if (num("stop", d, false)) { s.has_stop = true; s.stop_ = d; }
  if (num("count", d, false)) { s.has_count = true; s.count_ = (int)d; }
  return s;
}
}  // namespace qio

// ---------------------------------------------------------------------------
// Bounds on a single flip's cost difference, used by the parameter-free
// solvers to place their temperature ranges.
// ---------------------------------------------------------------------------
namespace qio
{
static const double kMinDeltaDefault = 0.1;  // MIN_DELTA_DEFAULT, model/graph_model.h:16

// utils::least_diff_method, utils/utils.cc:43-53: replace the two largest
// values by their difference until one value is left
static double least_diff_one(std::multiset<double> s)
{
  while (s.size() > 1)
  {
    auto a = std::prev(s.end());
    const double x = *a;
    s.erase(a);
    auto b = std::prev(s.end());
    const double y = *b;
    s.erase(b);
    s.insert(x - y);
  }
  return *s.begin();
}

// the two-set form, utils/utils.cc:55-100: the largest of each set cancel;
// the smallest non-zero remainder is kept
static double least_diff_two(std::multiset<double> a, std::multiset<double> b)
{
  double mn = std::numeric_limits<double>::max();
  if (a.empty() && !b.empty()) return *b.begin();
  if (!a.empty() && b.empty()) return *a.begin();
  while (!a.empty() && !b.empty())
  {
    auto ia = std::prev(a.end());
    const double ca = *ia;
    a.erase(ia);
    auto ib = std::prev(b.end());
    const double cb = *ib;
    b.erase(ib);
    double delta = ca - cb;
    if (delta > 0)
      a.insert(delta);
    else if (delta < 0)
    {
      delta = -delta;
      b.insert(delta);
    }
    else if (a.size() < b.size())
      a.insert(ca);
    else
      b.insert(cb);
    if (mn > delta && delta != 0) mn = delta;
  }
  return mn;
}

// Ising: twice the largest sum of |c| over a variable's terms
// (model/ising.h:176-179, graph/graph.h:453-485); PUBO: that sum itself
// (model/graph_model.h:194-197)
double estimate_max_cost_diff(const HostModel& m)
{
  if (m.kind == K_MAXSAT) fail(1, "cost difference estimates are not available for maxsat models");
  double mx = 0;
  for (int64_t v = 0; v < m.N; v++)
  {
    double s = 0;
    for (int q = m.row[v]; q < m.row[v + 1]; q++) s += std::abs(m.coef[q]);
    mx = s > mx ? s : mx;
  }
  return (m.kind == K_ISING || m.kind == K_ISING_PLAIN) ? mx * 2 : mx;
}

// Ising (model/ising.h:181-224): per variable the single-set least
// difference of its |c|, zeros skipped, the smallest doubled; PUBO
// (model/pubo.h:127-184): the two-set least difference of its positive and
// negated negative c.  No non-zero value: MIN_DELTA_DEFAULT (doubled for
// Ising).
double estimate_min_cost_diff(const HostModel& m)
{
  if (m.kind == K_MAXSAT) fail(1, "cost difference estimates are not available for maxsat models");
  const bool ising = m.kind == K_ISING || m.kind == K_ISING_PLAIN;
  double mn = std::numeric_limits<double>::max();
  for (int64_t v = 0; v < m.N; v++)
  {
    double local;
    if (ising)
    {
      std::multiset<double> s;
      for (int q = m.row[v]; q < m.row[v + 1]; q++) s.insert(std::abs(m.coef[q]));
      if (s.empty()) continue;
      local = least_diff_one(s);
    }
    else
    {
      std::multiset<double> pos, neg;
      for (int q = m.row[v]; q < m.row[v + 1]; q++)
      {
        const double c = m.coef[q];
        if (c > 0) pos.insert(c);
        else if (c < 0) neg.insert(-c);
      }
      local = least_diff_two(pos, neg);
    }
    if (local == 0) continue;
    mn = local < mn ? local : mn;
  }
  if (mn == std::numeric_limits<double>::max()) mn = kMinDeltaDefault;
  return ising ? mn * 2 : mn;
}
}  // namespace qio
