// qio_oracle.cc -- CPU oracle for the QIOToolkit Metropolis hot path.
//
// TEST INFRASTRUCTURE ONLY: this file is the checker the CUDA library is
// compared against (and the CPU baseline that bench.py times).  The product
// library never links it.
//
// It restates, in plain C++17 without fast-math, the reference code listed
// below.  Every block cites the reference file:line it follows (paths are
// relative to the reference's cpp/ directory).
//
// Third-party arithmetic at the boundary:
//   * pcg32 (pcg-cpp @ ffd522e7188bef30a00c74dc7eb9de5faff90092, fetched by
//     cmake/pcg.cmake:5-6) is restated from its published algorithm
//     (64-bit LCG, XSH-RR output, default stream increment).
//   * libstdc++ <random>: std::uniform_real_distribution<double> (two 32-bit
//     draws through generate_canonical), std::poisson_distribution<int> and
//     std::mt19937 are used directly, exactly as the reference calls them
//     (utils/random_generator.cc:8-9,49,54-58).
//
// Built with -O2 -ffp-contract=off: the reference's Release flags include
// -Ofast (cpp/CMakeLists.txt:34); the oracle follows the source semantics,
// not a fast-math build.

#include "qio_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <random>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc
{
// ===========================================================================
// Random generators
// ===========================================================================

// pcg32 = pcg_engines::setseq_xsh_rr_64_32 with its default increment.
// Seeding constructs the engine afresh: state = (seed + inc) * mult + inc.
// Follows utils/random_generator.h:79-96, utils/random_generator.cc:37-58.
struct Pcg32
{
  static constexpr uint64_t kMult = 6364136223846793005ULL;
  static constexpr uint64_t kInc = 1442695040888963407ULL;
  using result_type = uint32_t;
  static constexpr result_type min() { return 0; }
  static constexpr result_type max() { return 0xffffffffu; }

  uint64_t state;
  Pcg32() { seed64(0xcafef00dd15ea5e5ULL); }
  explicit Pcg32(uint32_t s) { seed64(s); }
  void seed64(uint64_t s) { state = (s + kInc) * kMult + kInc; }
  static uint32_t output(uint64_t old)
  {
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  uint32_t operator()()
  {
    uint64_t old = state;
    state = old * kMult + kInc;
    return output(old);
  }
};

// Abstract generator with the reference's RandomGenerator surface
// (utils/random_generator.h:19-57).
struct Rng
{
  virtual ~Rng() {}
  virtual uint32_t uint32() = 0;
  virtual double uniform() = 0;
  virtual uint32_t poisson(double mean) = 0;
  virtual std::unique_ptr<Rng> fork() = 0;
};

struct PcgRng : Rng
{
  Pcg32 pcg;
  PcgRng() {}
  explicit PcgRng(uint32_t s) : pcg(s) {}
  uint32_t uint32() override { return pcg(); }
  double uniform() override
  {
    std::uniform_real_distribution<double> u(0.0, 1.0);
    return u(pcg);
  }
  uint32_t poisson(double mean) override
  {
    std::poisson_distribution<> p(mean);
    return p(pcg);
  }
  // fork(): the child is seeded with one draw of the parent
  // (utils/random_generator.cc:35-43).
  std::unique_ptr<Rng> fork() override
  {
    return std::unique_ptr<Rng>(new PcgRng(uint32()));
  }
};

struct TwisterRng : Rng
{
  std::mt19937 tw;
  TwisterRng() {}
  explicit TwisterRng(uint32_t s) { tw.seed(s); }
  uint32_t uint32() override { return tw(); }
  double uniform() override
  {
    std::uniform_real_distribution<double> u(0.0, 1.0);
    return u(tw);
  }
  uint32_t poisson(double mean) override
  {
    std::poisson_distribution<> p(mean);
    return p(tw);
  }
  std::unique_ptr<Rng> fork() override
  {
    return std::unique_ptr<Rng>(new TwisterRng(uint32()));
  }
};

// Counter-based generator (this project's independent-stream mode; no
// reference counterpart).  SplitMix64's finaliser (Steele, Lea & Flood 2014)
// applied to key + counter * golden-gamma gives random access to a stream.
static inline uint64_t mix64(uint64_t z)
{
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static inline uint64_t counter_key(uint32_t seed, uint64_t stream)
{
  return mix64(((uint64_t)seed << 32) ^ mix64(stream + 0x9E3779B97F4A7C15ULL));
}
static inline uint64_t counter_draw(uint64_t key, uint64_t ctr)
{
  return mix64(key + ctr * 0x9E3779B97F4A7C15ULL);
}
static const uint64_t kInitCounterBase = 1ULL << 62;

// ===========================================================================
// ln lookup table and Metropolis acceptance
// ===========================================================================

// uniform_ln[row][i] = log(i / 256^(row+1)), utils/utils.cc:12-32.
static std::vector<double> make_uniform_ln()
{
  std::vector<double> t(4 * 256);
  for (int row = 0; row < 4; row++)
    for (size_t i = 0; i < 256; i++)
      t[row * 256 + i] = log((i) / pow((double)256, (double)(row + 1)));
  return t;
}
static const std::vector<double>& uniform_ln()
{
  static std::vector<double> t = make_uniform_ln();
  return t;
}

// Draw source for the acceptance test: either a stream (replay) or the
// counter-mode draws of one attempt.
struct DrawSource
{
  virtual uint32_t next() = 0;
};
struct RngDraws : DrawSource
{
  Rng* rng;
  explicit RngDraws(Rng* r) : rng(r) {}
  uint32_t next() override { return rng->uint32(); }
};
struct CounterDraws : DrawSource
{
  uint64_t key, ctr;
  int k = 0;
  uint64_t w = 0;
  CounterDraws(uint64_t key_, uint64_t ctr_) : key(key_), ctr(ctr_) {}
  uint32_t next() override
  {
    // draws 0,1 come from word 2*ctr, draws 2,3 from word 2*ctr+1
    if ((k & 1) == 0) w = counter_draw(key, 2 * ctr + (uint64_t)(k >> 1));
    uint32_t v = (k & 1) ? (uint32_t)(w >> 32) : (uint32_t)w;
    k++;
    return v;
  }
};

// Metropolis::accept, markov/metropolis.h:64-104: downhill accepts without a
// draw; uphill draws r, bucket = r & 255, redraws in the next (finer) row
// while bucket == 0 (at most 4 draws, then accept), and interpolates the
// ln table at distance (r >> 8) / 16777214.
static bool metropolis_accept(double cost_diff, double beta, DrawSource& src)
{
  if (cost_diff <= 0) return true;
  size_t bucket = 0;
  int row = -1;
  uint32_t current = 0;
  while (bucket == 0)
  {
    if (row < 3)
    {
      current = src.next();
      bucket = current & 255u;
      row++;
    }
    else
    {
      return true;
    }
  }
  const std::vector<double>& ln = uniform_ln();
  double y0 = ln[row * 256 + bucket - 1];
  double y1 = ln[row * 256 + bucket];
  double distance = ((double)(current >> 8)) /
                    (double)((~((uint32_t)256)) >> 8);
  double value = y0 + distance * (y1 - y0);
  return value < (cost_diff * -beta);
}

// ===========================================================================
// Models
// ===========================================================================

enum Kind
{
  ISING = ORC_ISING,
  ISING_PLAIN = ORC_ISING_PLAIN,
  PUBO = ORC_PUBO,
  PUBO_PLAIN = ORC_PUBO_PLAIN,
  MAXSAT = ORC_MAXSAT
};

struct Model
{
  int kind;
  // Graph models (graph/graph.h): edges in internal ids, node->edge lists.
  int64_t N = 0, M = 0;
  std::vector<std::vector<int32_t>> edge_nodes;
  std::vector<double> cost;
  std::vector<std::vector<int64_t>> node_edges;
  double const_cost = 0;
  double max_coupling = 0;
  double scale_factor = 1.0;
  bool rescaled = false;
  std::vector<int32_t> id_to_name;
  // MaxSAT (model/max_sat.h): 1-based clause weights and signed clause ids
  std::vector<double> weights;
  std::vector<std::vector<int>> affected;
  std::vector<int> free_variables;

  bool empty() const { return N == 0; }
  // sweep size: graph models -> N (ordered sweep over all nodes); MaxSat
  // does not override Model::get_sweep_size() and gets 1
  // (markov/model.h:169).
  int64_t sweep_size(bool full_maxsat) const
  {
    if (kind == MAXSAT) return full_maxsat ? N : 1;
    return N;
  }
};

// normalize_edges, graph/graph.h:74-177: ids renumbered by first appearance,
// duplicate ids in a term throw (Ising) or merge (PUBO), member ids sorted,
// empty terms folded into const_cost, node edge lists in ascending edge id.
static void normalize(Model& m, int64_t n_terms, const int64_t* off,
                      const int32_t* ids, const double* coef, bool allow_dup)
{
  if (n_terms == 0)
    throw std::runtime_error(
        "parameter `terms`: size must be greater than 0, found 0");
  std::map<int, int> name_to_id;
  for (int64_t t = 0; t < n_terms; t++)
  {
    std::set<int> seen;
    std::vector<int32_t> nodes;
    for (int64_t k = off[t]; k < off[t + 1]; k++)
    {
      int input_id = ids[k];
      auto it = name_to_id.find(input_id);
      if (it == name_to_id.end())
      {
        int nid = (int)m.id_to_name.size();
        name_to_id[input_id] = nid;
        m.id_to_name.push_back(input_id);
        m.node_edges.push_back({});
      }
      int internal = name_to_id[input_id];
      if (seen.find(internal) == seen.end())
      {
        seen.insert(internal);
        nodes.push_back(internal);
        m.node_edges[internal].push_back((int64_t)m.edge_nodes.size());
      }
      else if (!allow_dup)
      {
        throw std::runtime_error("Duplicated ids detected in term!");
      }
    }
    std::sort(nodes.begin(), nodes.end());
    if (!nodes.empty())
    {
      double a = fabs(coef[t]);
      if (a > m.max_coupling) m.max_coupling = a;
      m.edge_nodes.push_back(nodes);
      m.cost.push_back(coef[t]);
    }
    else
    {
      m.const_cost += coef[t];
    }
  }
  m.N = (int64_t)m.id_to_name.size();
  m.M = (int64_t)m.edge_nodes.size();
}

// MaxSat::configure(clauses), model/max_sat.h:295-397: always-true clauses
// dropped, variables sorted by name, clauses 1-indexed, negated literals
// stored as negative clause ids, repeated variables in a clause skipped.
static void configure_maxsat(Model& m, int64_t n_terms, const int64_t* off,
                             const int32_t* ids, const double* coef)
{
  size_t active = 0;
  std::vector<bool> always_true(n_terms);
  std::set<int> used, potentially_free;
  for (int64_t i = 0; i < n_terms; i++)
  {
    std::set<int> seen;
    for (int64_t k = off[i]; k < off[i + 1]; k++)
    {
      int v = ids[k];
      if (v == 0 || v == std::numeric_limits<int>::min())
        throw std::runtime_error("MaxSat variables cannot have the name " +
                                 std::to_string(v));
      if (seen.find(-v) != seen.end()) always_true[i] = true;
      seen.insert(v);
    }
    if (always_true[i])
      for (int v : seen) potentially_free.insert(std::abs(v));
    else
    {
      active++;
      for (int v : seen) used.insert(std::abs(v));
    }
  }
  for (int v : potentially_free)
    if (used.find(v) == used.end()) m.free_variables.push_back(v);
  m.id_to_name.assign(used.begin(), used.end());
  m.weights.clear();
  m.affected.clear();
  if (m.id_to_name.empty() || active == 0)
  {
    m.N = 0;
    m.M = 0;
    return;
  }
  std::map<int, int> name_to_id;
  for (size_t id = 0; id < m.id_to_name.size(); id++)
    name_to_id[m.id_to_name[id]] = (int)id;
  m.weights.resize(active + 1);
  m.affected.resize(m.id_to_name.size());
  int clause_id = 1;
  for (int64_t i = 0; i < n_terms; i++)
  {
    if (always_true[i]) continue;
    m.weights[clause_id] = coef[i];
    std::set<int> seen;
    for (int64_t k = off[i]; k < off[i + 1]; k++)
    {
      int name = ids[k];
      int var_id = name_to_id[std::abs(name)];
      if (seen.find(var_id) != seen.end()) continue;
      seen.insert(var_id);
      m.affected[var_id].push_back(name < 0 ? -clause_id : clause_id);
    }
    clause_id++;
  }
  m.N = (int64_t)m.id_to_name.size();
  m.M = (int64_t)active;
}

// State: spins (Ising: true = -1; PUBO: true = "0"; MaxSat: true = variable
// true) plus the per-term cache (Ising parity bits, PUBO zero counters,
// MaxSat clause counters indexed 1..M).
struct State
{
  std::vector<uint8_t> spins;
  std::vector<int64_t> terms;
};

static State create_state(const Model& m)
{
  State s;
  s.spins.assign(m.N, 0);
  if (m.kind == ISING || m.kind == PUBO) s.terms.assign(m.M, 0);
  if (m.kind == MAXSAT)
  {
    // MaxSat::create_state, model/max_sat.h:113-122: all variables false;
    // negated literals are true.
    s.terms.assign(m.M + 1, 0);
    for (int64_t i = 0; i < m.N; i++)
      for (int j : m.affected[i])
        if (j < 0) s.terms[-j]++;
  }
  return s;
}

// IsingTermCached::apply_transition (model/ising.cc:36-44), Ising (26-29),
// PuboWithCounter (model/pubo.h:369-392), Pubo (model/pubo.cc:75-79),
// MaxSat (model/max_sat.h:239-259).
static void apply_transition(const Model& m, int64_t v, State& s)
{
  switch (m.kind)
  {
    case ISING:
      s.spins[v] = !s.spins[v];
      for (int64_t j : m.node_edges[v]) s.terms[j] = !s.terms[j];
      break;
    case ISING_PLAIN:
    case PUBO_PLAIN:
      s.spins[v] = !s.spins[v];
      break;
    case PUBO:
      if (s.spins[v])
      {
        for (int64_t j : m.node_edges[v]) s.terms[j]--;
        s.spins[v] = 0;
      }
      else
      {
        for (int64_t j : m.node_edges[v]) s.terms[j]++;
        s.spins[v] = 1;
      }
      break;
    case MAXSAT:
    {
      bool value = s.spins[v];
      if (value)
      {
        for (int c : m.affected[v])
          if (c > 0) s.terms[c]--; else s.terms[-c]++;
      }
      else
      {
        for (int c : m.affected[v])
          if (c > 0) s.terms[c]++; else s.terms[-c]--;
      }
      s.spins[v] = !value;
      break;
    }
  }
}

// get_ising_term, model/ising.h:233-245 (parity recomputed from members).
static double ising_term_plain(const Model& m, const State& s, int64_t j)
{
  bool term = false;
  for (int32_t i : m.edge_nodes[j]) term ^= (s.spins[i] != 0);
  double c = m.cost[j];
  return term ? -c : c;
}

// calculate_cost: Ising model/ising.h:94-102, PuboWithCounter
// model/pubo.h:301-333, Pubo model/pubo.cc:27-48, MaxSat
// model/max_sat.h:163-170.
static double calculate_cost(const Model& m, const State& s)
{
  double cost = 0.0;
  switch (m.kind)
  {
    case ISING:
      for (int64_t j = 0; j < m.M; j++)
      {
        double c = m.cost[j];
        cost += s.terms[j] ? -c : c;
      }
      break;
    case ISING_PLAIN:
      for (int64_t j = 0; j < m.M; j++) cost += ising_term_plain(m, s, j);
      break;
    case PUBO:
      for (int64_t j = 0; j < m.M; j++)
        if (s.terms[j] == 0) cost += m.cost[j];
      break;
    case PUBO_PLAIN:
      for (int64_t j = 0; j < m.M; j++)
      {
        bool zero = false;
        for (int32_t i : m.edge_nodes[j])
          if (s.spins[i]) { zero = true; break; }
        if (!zero) cost += m.cost[j];
      }
      break;
    case MAXSAT:
      for (int64_t c = 1; c <= m.M; c++)
        if (s.terms[c] == 0) cost += m.weights[c];
      break;
  }
  return cost;
}

// calculate_cost_difference: Ising model/ising.h:108-117, PuboWithCounter
// model/pubo.h:335-367, Pubo model/pubo.cc:50-73, MaxSat
// model/max_sat.h:173-236.
static double cost_difference(const Model& m, const State& s, int64_t v)
{
  double diff = 0.0;
  switch (m.kind)
  {
    case ISING:
      for (int64_t j : m.node_edges[v])
      {
        double c = m.cost[j];
        diff += s.terms[j] ? -c : c;
      }
      return 2.0 * (-diff);
    case ISING_PLAIN:
      for (int64_t j : m.node_edges[v]) diff += ising_term_plain(m, s, j);
      return 2.0 * (-diff);
    case PUBO:
      if (s.spins[v])
      {
        for (int64_t j : m.node_edges[v])
          if (s.terms[j] == 1) diff += m.cost[j];
      }
      else
      {
        for (int64_t j : m.node_edges[v])
          if (s.terms[j] == 0) diff -= m.cost[j];
      }
      return diff;
    case PUBO_PLAIN:
      for (int64_t j : m.node_edges[v])
      {
        bool zero = false;
        for (int32_t i : m.edge_nodes[j])
          if (i != v && s.spins[i]) { zero = true; break; }
        if (!zero) diff += s.spins[v] ? m.cost[j] : -m.cost[j];
      }
      return diff;
    case MAXSAT:
      if (s.spins[v])
      {
        for (int c : m.affected[v])
        {
          if (c > 0) { if (s.terms[c] == 1) diff += m.weights[c]; }
          else { if (s.terms[-c] == 0) diff -= m.weights[-c]; }
        }
      }
      else
      {
        for (int c : m.affected[v])
        {
          if (c > 0) { if (s.terms[c] == 0) diff -= m.weights[c]; }
          else { if (s.terms[-c] == 1) diff += m.weights[-c]; }
        }
      }
      return diff;
  }
  return diff;
}

// Random initial state.  Graph models: one uint32 draw per 32 variables,
// bit (i % 32) set -> apply_transition(i) (model/ising.h:23-41,
// model/pubo.h:16-34).  MaxSat: uniform() < 0.5 per variable
// (model/max_sat.h:144-150).
static State random_state_replay(const Model& m, Rng& rng)
{
  State s = create_state(m);
  if (m.kind == MAXSAT)
  {
    for (int64_t i = 0; i < m.N; i++)
      if (rng.uniform() < 0.5) apply_transition(m, i, s);
    return s;
  }
  uint32_t rv = 0;
  for (int64_t i = 0; i < m.N; i++)
  {
    if (i % 32 == 0) rv = rng.uint32();
    if ((rv >> (i % 32)) & 1u) apply_transition(m, i, s);
  }
  return s;
}

// Counter-mode initial state: bit i comes from draw(key, base + i / 32), bit
// (i % 32) of its low word; MaxSat uses bit 63 of draw(key, base + i) == 0.
static State random_state_counter(const Model& m, uint64_t key)
{
  State s = create_state(m);
  if (m.kind == MAXSAT)
  {
    for (int64_t i = 0; i < m.N; i++)
      if ((counter_draw(key, kInitCounterBase + (uint64_t)i) >> 63) == 0)
        apply_transition(m, i, s);
    return s;
  }
  uint32_t rv = 0;
  for (int64_t i = 0; i < m.N; i++)
  {
    if (i % 32 == 0)
      rv = (uint32_t)counter_draw(key, kInitCounterBase + (uint64_t)(i / 32));
    if ((rv >> (i % 32)) & 1u) apply_transition(m, i, s);
  }
  return s;
}

// ===========================================================================
// Walker / Metropolis (markov/walker.h, markov/metropolis.h)
// ===========================================================================

struct Walker
{
  const Model* model = nullptr;
  Rng* rng = nullptr;          // replay mode
  uint64_t key = 0;            // counter mode
  uint64_t sweep_counter = 0;  // counter mode: sweeps done on this stream
  bool counter_mode = false;
  bool full_maxsat = false;
  State state;
  double cost_ = 0;
  double lowest_cost = 0;
  std::vector<uint8_t> lowest_spins;
  uint64_t diff_evals = 0, accepted = 0;
  uint64_t total_attempts = 0, total_accepts = 0;
  double beta_ = 1.0, temperature_ = 1.0;

  // set_temperature / set_beta, markov/metropolis.h:35-61
  void set_temperature(double t)
  {
    temperature_ = t;
    if (temperature_ <= 0)
    {
      temperature_ = 0.0;
      beta_ = std::numeric_limits<double>::infinity();
    }
    else
      beta_ = 1.0 / temperature_;
  }
  void set_beta(double b)
  {
    beta_ = b;
    if (beta_ <= 0)
    {
      beta_ = 0;
      temperature_ = std::numeric_limits<double>::infinity();
    }
    else
      temperature_ = 1.0 / beta_;
  }
  // save_lowest / check_lowest, markov/walker.h:269-280
  void save_lowest()
  {
    lowest_cost = cost_;
    lowest_spins = state.spins;
  }
  void check_lowest()
  {
    if (cost_ < lowest_cost) save_lowest();
  }
  // init, markov/walker.h:50-58
  void init()
  {
    state = counter_mode ? random_state_counter(*model, key)
                         : random_state_replay(*model, *rng);
    cost_ = calculate_cost(*model, state);
    save_lowest();
  }
  // attempt_transition, markov/walker.h:209-229
  void attempt(int64_t v, uint64_t ctr)
  {
    double d = cost_difference(*model, state, v);
    diff_evals++;
    total_attempts++;
    bool acc;
    if (counter_mode)
    {
      CounterDraws src(key, ctr);
      acc = metropolis_accept(d, beta_, src);
    }
    else
    {
      RngDraws src(rng);
      acc = metropolis_accept(d, beta_, src);
    }
    if (acc)
    {
      apply_transition(*model, v, state);
      accepted++;
      total_accepts++;
      cost_ += d;
      check_lowest();
    }
  }
  // ordered sweep, markov/walker.h:143-153
  void make_sweep()
  {
    int64_t n = model->sweep_size(full_maxsat);
    uint64_t base = sweep_counter * (uint64_t)n;
    for (int64_t i = 0; i < n; i++) attempt(i, base + (uint64_t)i);
    sweep_counter++;
  }
  void make_sweeps(int64_t k)
  {
    for (int64_t i = 0; i < k; i++) make_sweep();
  }
  void swap_state(Walker& o)
  {
    std::swap(state, o.state);
    std::swap(cost_, o.cost_);
  }
};

// ===========================================================================
// Schedules (schedule/*.cc)
// ===========================================================================

struct Schedule
{
  int type = ORC_SCHED_LINEAR;
  double initial = 0, final_ = 0;
  bool has_start = false, has_stop = false, has_count = false;
  double start_ = 0, stop_ = 1;
  int count_ = 1;
  std::vector<double> values;

  // generator value at progress p: Linear schedule/linear.cc:15-18,
  // Geometric schedule/geometric.cc:9-12, constant points of a list
  // (Segments, schedule/segments.cc:15-43 with constant points at
  // positions 0..n-1).
  double progress_value(double p) const
  {
    switch (type)
    {
      case ORC_SCHED_LINEAR: return initial + p * (final_ - initial);
      case ORC_SCHED_GEOMETRIC: return initial * pow(final_ / initial, p);
      case ORC_SCHED_CONSTANT: return initial;
      case ORC_SCHED_LIST:
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
            double progress = (position - last_stop) / (start - last_stop);
            return (1 - progress) * values[i - 1] + progress * values[i];
          }
          return values[i];
        }
        return values.back();
      }
    }
    return 0;
  }
  // ScheduleGenerator defaults, schedule/schedule_generator.cc (start 0,
  // stop 1, count round(|stop-start|)); lists: start 0, stop n-1, count n
  // (Segments::adjust, schedule/segments.cc:45-110).
  double get_start() const
  {
    if (has_start) return start_;
    return 0;
  }
  double get_stop() const
  {
    if (has_stop) return stop_;
    if (type == ORC_SCHED_LIST) return (double)values.size() - 1;
    return 1;
  }
  int get_count() const
  {
    if (has_count) return count_;
    if (type == ORC_SCHED_LIST) return (int)values.size();
    return (int)round(std::abs(get_stop() - get_start()));
  }
  // Schedule::get_value, schedule/schedule.cc:17-25
  double get_value(double input) const
  {
    double start = get_start(), stop = get_stop();
    if (start == stop) return progress_value(0);
    double progress = (input - start) / (stop - start);
    return progress_value(std::min(1., std::max(0., progress)));
  }
  // Schedule::get_discretized_values, schedule/schedule.cc:38-89
  std::vector<double> discretized() const
  {
    int count = get_count();
    if (count < 2)
      throw std::runtime_error(
          "Can not get_discretized_values(count) for less than 2 values");
    std::vector<double> d;
    for (int i = 0; i < count; i++)
      d.push_back(progress_value(double(i) / (count - 1)));
    return d;
  }
};

static Schedule to_schedule(const orc_schedule& s)
{
  Schedule r;
  r.type = s.type;
  r.initial = s.initial;
  r.final_ = s.final_value;
  r.has_start = s.has_start;
  r.has_stop = s.has_stop;
  r.has_count = s.has_count;
  r.start_ = s.start;
  r.stop_ = s.stop;
  r.count_ = s.count;
  if (s.type == ORC_SCHED_LIST)
    r.values.assign(s.values, s.values + s.n_values);
  return r;
}

// ===========================================================================
// Results
// ===========================================================================

struct Result
{
  int64_t n_vars = 0;
  int64_t last_step = 0;
  std::vector<double> cost, lowest;
  std::vector<uint64_t> attempts, accepts;
  std::vector<std::vector<uint8_t>> states, lowest_states;
  bool has_best = false;
  double best_cost = 0;  // lowest + const cost
  std::vector<uint8_t> best_state;
  std::vector<double> sol_costs;
  std::vector<std::vector<uint8_t>> sol_states;
  std::vector<double> pt_obs;  // n * 5
  std::vector<double> pa_beta;
  std::vector<int64_t> pa_pop;
  uint64_t master_out = 0;  // PT: master stream state after the run
};

// ModelSolver::update_lowest_cost, solver/model_solver.h:247-259
struct Lowest
{
  bool has = false;
  double cost = 0;
  std::vector<uint8_t> state;
  void update(double c, const std::vector<uint8_t>& s)
  {
    if (!has || c < cost)
    {
      has = true;
      cost = c;
      state = s;
    }
  }
};

// populate_solutions / copy_solutions, solver/model_solver.h:261-308:
// walkers partially sorted by lowest cost (ties: lower index first here;
// std::partial_sort leaves tie order unspecified).
static void populate(Result& r, const std::vector<Walker*>& ws, Lowest& low,
                     int nsol, const Model& m, bool population,
                     bool pop_lowest_check)
{
  std::vector<size_t> idx(ws.size());
  for (size_t i = 0; i < idx.size(); i++) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) {
    return ws[a]->lowest_cost < ws[b]->lowest_cost;
  });
  unsigned k = std::min((unsigned)nsol, (unsigned)ws.size());
  if (population && pop_lowest_check && low.has &&
      low.cost < ws[idx[0]]->lowest_cost)
  {
    r.sol_costs.push_back(low.cost + m.const_cost);
    r.sol_states.push_back(low.state);
    k--;
  }
  for (unsigned i = 0; i < k; i++)
  {
    r.sol_costs.push_back(ws[idx[i]]->lowest_cost + m.const_cost);
    r.sol_states.push_back(ws[idx[i]]->lowest_spins);
  }
  double c0 = r.sol_costs[0] - m.const_cost;
  low.update(c0, r.sol_states[0]);
  r.has_best = low.has;
  r.best_cost = low.cost + m.const_cost;
  r.best_state = low.state;
}

static void fill_replicas(Result& r, const std::vector<Walker*>& ws)
{
  for (Walker* w : ws)
  {
    r.cost.push_back(w->cost_);
    r.lowest.push_back(w->lowest_cost);
    r.attempts.push_back(w->total_attempts);
    r.accepts.push_back(w->total_accepts);
    r.states.push_back(w->state.spins);
    r.lowest_states.push_back(w->lowest_spins);
  }
}

static void set_threads(int t)
{
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

// ---------------------------------------------------------------------------
// SimulatedAnnealing, solver/simulated_annealing.h:45-110 and the stepping
// loop solver/stepping_solver.h:112-268 (step limit and cost limit).
// ---------------------------------------------------------------------------
static Result run_sa(const Model& m, const orc_params& p)
{
  Result r;
  r.n_vars = m.N;
  Schedule sched = to_schedule(p.sched);
  // stretch (solver/simulated_annealing.h:175-201)
  if (sched.get_start() == 0 && sched.get_stop() == 1 && sched.get_count() == 1)
  {
    if (p.step_limit > 1)
    {
      sched.has_stop = true;
      sched.stop_ = std::max(1, (int)p.step_limit - 1);
    }
    else
      throw std::runtime_error("The number of sweeps must be greater than 1.");
  }
  if (m.empty())
  {
    r.has_best = false;
    r.best_cost = m.const_cost;
    return r;
  }
  size_t R = (size_t)p.restarts;
  PcgRng master(p.seed);
  for (int64_t k = 0; k < p.master_skip; k++) master.uint32();
  std::vector<std::unique_ptr<Rng>> rngs(R);
  for (size_t i = 0; i < R; i++) rngs[i] = master.fork();
  std::vector<Walker> reps(R);
  std::vector<Walker*> wp(R);
  set_threads(p.threads);
#pragma omp parallel for schedule(dynamic, 1)
  for (size_t i = 0; i < R; i++)
  {
    Walker& w = reps[i];
    w.model = &m;
    w.rng = rngs[i].get();
    w.counter_mode = p.rng_mode == ORC_RNG_COUNTER;
    w.key = counter_key(p.seed, i);
    w.full_maxsat = p.full_maxsat_sweep != 0;
    w.init();
  }
  for (size_t i = 0; i < R; i++) wp[i] = &reps[i];
  Lowest low;
  low.update(reps[0].cost_, reps[0].state.spins);
  int64_t step = 0;
  if (!p.has_cost_limit)
  {
    // no per-step interaction between replicas: run each replica's whole
    // anneal in one go (identical results, parallel over replicas)
    std::vector<double> vals(p.step_limit);
    for (int64_t s = 0; s < p.step_limit; s++) vals[s] = sched.get_value((double)s);
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t i = 0; i < R; i++)
      for (int64_t s = 0; s < p.step_limit; s++)
      {
        if (p.use_inverse) reps[i].set_beta(vals[s]);
        else reps[i].set_temperature(vals[s]);
        reps[i].make_sweep();
      }
    step = p.step_limit;
  }
  else
  {
    for (step = 0; step < p.step_limit;)
    {
      double v = sched.get_value((double)step);
#pragma omp parallel for schedule(dynamic, 1)
      for (size_t i = 0; i < R; i++)
      {
        if (p.use_inverse) reps[i].set_beta(v);
        else reps[i].set_temperature(v);
        reps[i].make_sweep();
      }
      for (size_t i = 0; i < R; i++)
        low.update(reps[i].lowest_cost, reps[i].lowest_spins);
      step++;
      if (low.cost <= p.cost_limit) break;
    }
  }
  r.last_step = step;
  fill_replicas(r, wp);
  populate(r, wp, low, p.number_of_solutions, m, false, false);
  return r;
}

// ---------------------------------------------------------------------------
// Tabu search, solver/tabu.h:22-164 with markov/tabu_walker.h:14-218 and the
// hill climber of markov/hill_climbing_walker.h.  Each restart scans the
// variables in order: the first move that would put the cost below the
// lowest is taken (and starts a hill-climbing local search), otherwise the
// lowest-difference move not on the tabu list; a taken move stays tabu for
// `tabu_tenure` sweeps.  Only the initial state draws random numbers.
// ---------------------------------------------------------------------------
struct TabuWalker : Walker
{
  std::vector<uint64_t> tabu;   // expiry iteration per variable
  uint64_t iter = 0, incomplete = 0;
  uint64_t tenure = 0;
  bool local = false;
  // the hill climber (a walker accepting differences <= 0) on a copy
  State hc;
  double hc_cost = 0, hc_low = 0;
  std::vector<uint8_t> hc_low_spins;

  // get_sweep_size(): N, or 1 for MaxSat (markov/model.h:169) unless the
  // full MaxSat sweep is asked for
  int64_t sweep() const { return model->sweep_size(full_maxsat); }
  void tabu_init()
  {
    init();
    tabu.assign((size_t)sweep(), 0);
    iter = incomplete = 0;
    local = false;
  }
  // local_search_init: HillClimbingWalker::init(state), markov/walker.h:63-69
  void local_init()
  {
    local = true;
    hc = state;
    hc_cost = calculate_cost(*model, hc);
    hc_low = hc_cost;
    hc_low_spins = hc.spins;
  }
  // local_search_sweep: one ordered hill-climbing sweep on the copy; its
  // lowest replaces the walker's when it improved, else local search ends
  void local_sweep()
  {
    const double prev = hc_low;
    for (int64_t v = 0; v < sweep(); v++)
    {
      const double d = cost_difference(*model, hc, v);
      diff_evals++;
      total_attempts++;
      if (d <= 0)
      {
        apply_transition(*model, v, hc);
        accepted++;
        total_accepts++;
        hc_cost += d;
        if (hc_cost < hc_low)
        {
          hc_low = hc_cost;
          hc_low_spins = hc.spins;
        }
      }
    }
    if (hc_low < prev)
    {
      lowest_cost = hc_low;
      lowest_spins = hc_low_spins;
    }
    else
      local = false;
  }
  // TabuWalker::make_sweep, markov/tabu_walker.h:60-129
  void tabu_sweep()
  {
    if (local)
    {
      local_sweep();
      return;
    }
    const int64_t n = sweep();
    bool has_best = false, taken = false;
    double best_d = 0;
    int64_t best = 0;
    for (int64_t i = 0; i < n; i++)
    {
      const double cost_before = cost_, low_before = lowest_cost;
      const double d = cost_difference(*model, state, i);
      diff_evals++;
      total_attempts++;
      if (cost_before + d < low_before)
      {
        // attempt_transition accepted it (TabuWalker::accept)
        apply_transition(*model, i, state);
        accepted++;
        total_accepts++;
        cost_ += d;
        check_lowest();
        tabu[i] = iter + tenure;
        local_init();
        incomplete += (uint64_t)i;
        if (incomplete < (uint64_t)n)
          local_sweep();
        else
          incomplete -= (uint64_t)n;
        taken = true;
        break;
      }
      if (tabu[i] >= iter) continue;
      if (!has_best || d < best_d)
      {
        has_best = true;
        best_d = d;
        best = i;
      }
    }
    if (!taken && has_best)
    {
      // Walker::apply_transition(transition, diff)
      apply_transition(*model, best, state);
      cost_ += best_d;
      check_lowest();
      tabu[best] = iter + tenure;
    }
    iter++;
  }
};

static Result run_tabu(const Model& m, const orc_params& p)
{
  Result r;
  r.n_vars = m.N;
  if (m.empty())
  {
    r.has_best = false;
    r.best_cost = m.const_cost;
    return r;
  }
  size_t R = (size_t)p.restarts;
  PcgRng master(p.seed);
  for (int64_t k = 0; k < p.master_skip; k++) master.uint32();
  std::vector<std::unique_ptr<Rng>> rngs(R);
  for (size_t i = 0; i < R; i++) rngs[i] = master.fork();
  std::vector<TabuWalker> reps(R);
  std::vector<Walker*> wp(R);
  set_threads(p.threads);
#pragma omp parallel for schedule(dynamic, 1)
  for (size_t i = 0; i < R; i++)
  {
    TabuWalker& w = reps[i];
    w.model = &m;
    w.rng = rngs[i].get();
    w.counter_mode = p.rng_mode == ORC_RNG_COUNTER;
    w.full_maxsat = p.full_maxsat_sweep != 0;
    w.key = counter_key(p.seed, i);
    // Tabu::make_step sets tabu_tenures_[i] when the list is given
    w.tenure = (uint64_t)(p.tabu_tenures && (int64_t)i < p.n_tabu_tenures ? p.tabu_tenures[i] : p.tabu_tenure);
    w.tabu_init();
  }
  for (size_t i = 0; i < R; i++) wp[i] = &reps[i];
  Lowest low;
  low.update(reps[0].cost_, reps[0].state.spins);
#pragma omp parallel for schedule(dynamic, 1)
  for (size_t i = 0; i < R; i++)
    for (int64_t s = 0; s < p.step_limit; s++) reps[i].tabu_sweep();
  r.last_step = p.step_limit;
  fill_replicas(r, wp);
  populate(r, wp, low, p.number_of_solutions, m, false, false);
  return r;
}

// ---------------------------------------------------------------------------
// ParallelTempering, solver/parallel_tempering.h:68-189.  Generic over the
// walker type so that the reference's toy model can reuse it for the pin.
// ---------------------------------------------------------------------------
template <class W, class CostOf, class Sweep>
static void pt_loop(std::vector<W>& reps, Rng& master, int64_t steps,
                    bool use_inverse, std::vector<double>& obs, Lowest* low,
                    CostOf cost_of, Sweep sweep, bool counter_swaps,
                    uint64_t swap_key, int64_t* last_step, bool has_limit,
                    double limit)
{
  size_t n = reps.size();
  std::vector<int> dir(n, 0);  // UP = 0, DOWN = 1
  std::vector<double> s_acc(n, 0), s_cost(n, 0), s_dir(n, 0), s_swap(n, 0);
  std::vector<double> c_swap(n, 0);
  int64_t step = 0;
  for (step = 0; step < steps;)
  {
    sweep(reps);
    for (size_t i = 0; i < n; i++)
    {
      auto& w = reps[i];
      s_acc[i] += static_cast<double>(w.accepted) /
                  static_cast<double>(w.diff_evals);
      s_cost[i] += cost_of(w);
      if (low) low->update(w.lowest_cost, w.lowest_spins_ref());
      w.accepted = 0;
      w.diff_evals = 0;
      s_dir[i] += dir[i];
    }
    for (size_t i = step & 1; i < n - 1; i += 2)
    {
      auto& a = reps[i];
      auto& b = reps[i + 1];
      double u;
      if (counter_swaps)
      {
        uint64_t w = counter_draw(swap_key, (uint64_t)step * n + i);
        u = (double)(w >> 11) * (1.0 / 9007199254740992.0);
      }
      else
        u = master.uniform();
      bool acc = u < exp((cost_of(a) - cost_of(b)) * (a.beta_ - b.beta_));
      if (acc)
      {
        a.swap_state(b);
        std::swap(dir[i], dir[i + 1]);
        s_swap[i] += 1;
      }
      c_swap[i] += 1;
    }
    dir[0] = 0;
    dir[n - 1] = 1;
    step++;
    if (has_limit && low && low->has && low->cost <= limit) break;
  }
  *last_step = step;
  obs.assign(n * 5, 0);
  for (size_t i = 0; i < n; i++)
  {
    double st = (double)step;
    obs[i * 5 + 0] = use_inverse ? reps[i].beta_ : reps[i].temperature_;
    obs[i * 5 + 1] = s_acc[i] / st;
    obs[i * 5 + 2] = s_cost[i] / st;
    obs[i * 5 + 3] = s_dir[i] / st;
    obs[i * 5 + 4] = c_swap[i] > 0 ? s_swap[i] / c_swap[i] : NAN;
  }
}

struct PtWalker : Walker
{
  const std::vector<uint8_t>& lowest_spins_ref() const { return lowest_spins; }
};

static Result run_pt(const Model& m, const orc_params& p)
{
  Result r;
  r.n_vars = m.N;
  Schedule sched = to_schedule(p.sched);
  std::vector<double> temps = sched.discretized();
  if (p.use_inverse)
    std::sort(temps.begin(), temps.end(), std::greater<double>());
  else
    std::sort(temps.begin(), temps.end(), std::less<double>());
  if (m.empty())
  {
    r.best_cost = m.const_cost;
    return r;
  }
  size_t n = temps.size();
  PcgRng master(p.seed);
  if (p.use_master_state) master.pcg.state = p.master_state;
  std::vector<std::unique_ptr<Rng>> rngs(n);
  for (size_t i = 0; i < n; i++) rngs[i] = master.fork();
  std::vector<PtWalker> reps(n);
  set_threads(p.threads);
#pragma omp parallel for schedule(dynamic, 1)
  for (size_t i = 0; i < n; i++)
  {
    PtWalker& w = reps[i];
    w.model = &m;
    w.rng = rngs[i].get();
    w.counter_mode = p.rng_mode == ORC_RNG_COUNTER;
    w.key = counter_key(p.seed, i);
    w.full_maxsat = p.full_maxsat_sweep != 0;
    if (p.use_inverse) w.set_beta(temps[i]);
    else w.set_temperature(temps[i]);
    w.init();
  }
  Lowest low;
  low.update(reps[0].cost_, reps[0].state.spins);
  int64_t spr = p.sweeps_per_replica;
  auto sweep = [spr](std::vector<PtWalker>& ws) {
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t i = 0; i < ws.size(); i++) ws[i].make_sweeps(spr);
  };
  auto cost_of = [](const PtWalker& w) { return w.cost_; };
  pt_loop(reps, master, p.step_limit, p.use_inverse != 0, r.pt_obs, &low,
          cost_of, sweep, p.rng_mode == ORC_RNG_COUNTER,
          counter_key(p.seed, 0xFFFFFFFFULL), &r.last_step, p.has_cost_limit,
          p.cost_limit);
  std::vector<Walker*> wp(n);
  for (size_t i = 0; i < n; i++) wp[i] = &reps[i];
  fill_replicas(r, wp);
  populate(r, wp, low, p.number_of_solutions, m, false, false);
  r.master_out = master.pcg.state;
  return r;
}

// ---------------------------------------------------------------------------
// PopulationAnnealing, solver/population_annealing.h:102-167,262-616 and
// Population::resample, solver/population.h:171-218.  OpenMP streams are
// emulated: citizen i uses stream (i % pa_threads), streams consumed in
// citizen order (schedule(static, 1)).  Reductions run sequentially in
// citizen order (the reference's OpenMP reduction order is unspecified for
// more than one thread).  Linear/geometric schedules; Poisson (default) or
// constant-population resampling.
// ---------------------------------------------------------------------------
struct Citizen
{
  Walker w;
  size_t count = 1;
  size_t family = 0;
};

// utils::RandomSelector (utils/random_selector.cc:14-125): Fenwick-style
// cumulative weights with select-and-remove.
struct Selector
{
  std::vector<size_t> ids;
  std::vector<double> weight{0, 0};
  double total = 0;
  double cumulative(size_t position) const
  {
    size_t p = 0;
    double w = 0;
    for (size_t k = weight.size() - 1; k > 0; k >>= 1)
      if (position & k)
      {
        p |= k;
        w += weight[p];
      }
    return w;
  }
  double get_weight(size_t position) const
  {
    return cumulative(position + 1) - cumulative(position);
  }
  void add_weight(size_t position, double w)
  {
    for (size_t k = 1; k < weight.size(); k <<= 1)
    {
      if (position & k) position ^= k;
      else weight[position + k] += w;
    }
  }
  void insert(size_t id, double w)
  {
    size_t position = ids.size();
    ids.push_back(id);
    total += w;
    if (position + 1 >= weight.size())
    {
      double t = weight.back();
      weight.resize(2 * weight.size() - 1);
      weight.back() = t;
    }
    add_weight(position, w);
  }
  size_t select_position(double u) const
  {
    if (ids.empty()) throw std::runtime_error("Random selector is empty.");
    if (ids.size() == 1) return 0;
    double w = u * total;
    size_t position = 0;
    for (size_t k = weight.size() - 1; k > 0; k >>= 1)
      if (w >= weight[position + k])
      {
        position += k;
        w -= weight[position];
      }
    if (position >= ids.size()) position = ids.size() - 1;
    return position;
  }
  void remove_position(size_t position)
  {
    ids[position] = ids.back();
    ids.pop_back();
    double before = get_weight(position);
    double after = get_weight(ids.size());
    total -= before;
    add_weight(position, after - before);
    add_weight(ids.size(), -after);
  }
  size_t select_and_remove(double u)
  {
    size_t pos = select_position(u);
    size_t id = ids[pos];
    remove_position(pos);
    return id;
  }
};

// ---------------------------------------------------------------------------
// SubstochasticMonteCarlo, solver/substochastic_monte_carlo.h:36-240: a
// population of random walkers (markov/random_walker.h: every proposed flip
// is accepted).  Each step, every walker attempts steps_per_walker flips,
// each taken with probability alpha(step) / steps_per_walker; then the
// population is resampled with weights exp(beta(step) (max - cost) /
// (max - min)): floor(target * w / W) copies each, the remaining slots drawn
// without replacement by the residual weights (utils::RandomSelector on the
// master stream), copies laid out as Population::resample does.
// Replay streams emulate the reference's OpenMP threads: rngs[t] forked from
// the master, thread t serving a contiguous block of walkers in index order
// (schedule(static)); walker init draws on the same per-thread streams.
// Counter mode: the walker in slot j draws counter_uniform(key_j, 2 c) and
// (key_j, 2 c + 1) for its c-th attempt (c = step * steps_per_walker + k),
// key_j = counter_key(seed, j).
// ---------------------------------------------------------------------------
static double counter_uniform(uint64_t key, uint64_t ctr)
{
  return (double)(counter_draw(key, ctr) >> 11) * 0x1p-53;
}

// libgomp's schedule(static) block of thread t among T for n iterations
static void static_block(size_t n, size_t T, size_t t, size_t& b, size_t& e)
{
  size_t q = n / T, r = n % T;
  if (t < r)
  {
    b = t * (q + 1);
    e = b + q + 1;
  }
  else
  {
    b = t * q + r;
    e = b + q;
  }
}

static void ssmc_schedules(const orc_params& p, Schedule& alpha, Schedule& beta)
{
  alpha = to_schedule(p.sched);
  beta = to_schedule(p.sched2);
  // solver/substochastic_monte_carlo.h:177-227
  if (alpha.get_count() <= 1 && beta.get_count() <= 1)
  {
    alpha.has_stop = beta.has_stop = true;
    alpha.stop_ = beta.stop_ = (double)(int)p.step_limit;
  }
  else if (alpha.get_count() <= 1)
  {
    alpha.has_stop = true;
    alpha.stop_ = (double)(int)beta.get_stop();
  }
  else if (beta.get_count() <= 1)
  {
    beta.has_stop = true;
    beta.stop_ = (double)(int)alpha.get_stop();
  }
  else if (alpha.get_count() != beta.get_count())
    throw std::runtime_error("The schedules for alpha and beta must have the same length");
  if (alpha.progress_value(0) <= alpha.progress_value(1))
    throw std::runtime_error("the schedule for alpha must be decreasing");
  if (beta.progress_value(0) >= beta.progress_value(1))
    throw std::runtime_error("the schedule for beta must be increasing");
}

static Result run_ssmc(const Model& m, const orc_params& p)
{
  Result r;
  r.n_vars = m.N;
  if (m.empty())
  {
    r.has_best = false;
    r.best_cost = m.const_cost;
    return r;
  }
  Schedule alpha, beta;
  ssmc_schedules(p, alpha, beta);
  const size_t R = (size_t)p.population;
  const size_t T = (size_t)std::max(1, p.pa_threads);
  const int64_t spw = std::max<int64_t>(1, p.sweeps_per_replica);
  const bool counter = p.rng_mode == ORC_RNG_COUNTER;
  set_threads(p.threads);
  PcgRng master(p.seed);
  if (p.use_master_state) master.pcg.state = p.master_state;
  std::vector<std::unique_ptr<Rng>> rngs(T);
  for (size_t t = 0; t < T; t++) rngs[t] = master.fork();
  std::vector<Walker> pop(R);
  for (size_t t = 0; t < T; t++)
  {
    size_t b, e;
    static_block(R, T, t, b, e);
    for (size_t i = b; i < e; i++)
    {
      Walker& w = pop[i];
      w.model = &m;
      w.rng = rngs[t].get();
      w.counter_mode = counter;
      w.key = counter_key(p.seed, i);
      w.init();
    }
  }
  Lowest low;
  low.update(pop[0].cost_, pop[0].state.spins);
  const int64_t n = m.N;
  int64_t step = 0;
  for (; step < p.step_limit; step++)
  {
    const double p_step = alpha.get_value((double)step) / (double)spw;
    // make_walker_steps: each emulated thread owns its block and stream
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t t = 0; t < T; t++)
    {
      size_t b, e;
      static_block(R, T, t, b, e);
      for (size_t i = b; i < e; i++)
      {
        Walker& w = pop[i];
        const uint64_t key = counter_key(p.seed, i);
        for (int64_t k = 0; k < spw; k++)
        {
          const uint64_t c = (uint64_t)(step * spw + k);
          const double u = counter ? counter_uniform(key, 2 * c) : rngs[t]->uniform();
          if (u < p_step)
          {
            const double u2 = counter ? counter_uniform(key, 2 * c + 1) : rngs[t]->uniform();
            const int64_t v = (int64_t)(u2 * (double)n);
            const double d = cost_difference(m, w.state, v);
            w.diff_evals++;
            w.total_attempts++;
            apply_transition(m, v, w.state);
            w.accepted++;
            w.total_accepts++;
            w.cost_ += d;
            w.check_lowest();
          }
        }
      }
    }
    // update_population_statistics
    double mn = pop[0].cost_, mx = pop[0].cost_;
    for (size_t i = 0; i < R; i++)
    {
      mn = std::min(mn, pop[i].cost_);
      mx = std::max(mx, pop[i].cost_);
      low.update(pop[i].lowest_cost, pop[i].lowest_spins);
    }
    // resample_population
    const double b = beta.get_value((double)step);
    const double range = mx - mn;
    if (range > 0)
    {
      double total = 0;
      std::vector<double> weight(R);
      for (size_t i = 0; i < R; i++)
      {
        weight[i] = exp(b * (mx - pop[i].cost_) / range);
        total += weight[i];
      }
      size_t resampled = 0;
      std::vector<size_t> count(R);
      Selector sel;
      for (size_t i = 0; i < R; i++)
      {
        const double rel = (double)R * weight[i] / total;
        const size_t iw = (size_t)floor(rel);
        count[i] = iw;
        resampled += iw;
        sel.insert(i, rel - (double)iw);
      }
      while (resampled < R)
      {
        count[sel.select_and_remove(master.uniform())] += 1;
        resampled++;
      }
      std::vector<Walker> next;
      next.reserve(R);
      for (size_t i = 0; i < R; i++)
        for (size_t c = 0; c < count[i]; c++) next.push_back(pop[i]);
      pop.swap(next);
    }
    if (p.has_cost_limit && low.has && low.cost <= p.cost_limit)
    {
      step++;
      break;
    }
  }
  r.last_step = step;
  std::vector<Walker*> wp(R);
  for (size_t i = 0; i < R; i++) wp[i] = &pop[i];
  fill_replicas(r, wp);
  populate(r, wp, low, p.number_of_solutions, m, true, true);
  r.master_out = master.pcg.state;
  return r;
}

// ---------------------------------------------------------------------------
// QuantumMonteCarlo, solver/quantum_monte_carlo.h:44-233 with
// markov/cluster_walker.h and markov/quantum_walker.h: each restart holds
// `trotter_number` slices (imaginary-time copies).  A sweep visits the
// variables in order; for variable v every slice k computes its difference,
// slice k > 0 bonds to slice k-1 with probability bond_prob when both hold the
// same value of v, each run of bonded slices (open boundary: slice 0 starts a
// run) is flipped together when its summed difference (slice order) is below
// 1e-11 or a uniform() of its first slice's stream is below
// exp(-beta_eff * sum); then the flips apply.  beta_eff = beta(step) / P,
// bond_prob = 1 - tanh(field(step) * beta(step) / P).  Slice i = r * P + k
// draws on stream i (forked in that order), or, in counter mode, on
// counter_key(seed, i) at 2 (step * N + v) and 2 (step * N + v) + 1.
// Per slice: attempts count N per sweep, accepts the flips applied.
// ---------------------------------------------------------------------------
static Result run_qmc(const Model& m, const orc_params& p)
{
  Result r;
  r.n_vars = m.N;
  if (m.empty())
  {
    r.has_best = false;
    r.best_cost = m.const_cost;
    return r;
  }
  const size_t R = (size_t)p.restarts, P = (size_t)p.trotter_number, S = R * P;
  const bool counter = p.rng_mode == ORC_RNG_COUNTER;
  Schedule beta = to_schedule(p.sched), field = to_schedule(p.sched2);
  beta.has_stop = field.has_stop = true;
  beta.stop_ = field.stop_ = (double)std::max(1, (int)p.step_limit - 1);
  PcgRng master(p.seed);
  std::vector<std::unique_ptr<Rng>> rngs(S);
  for (size_t i = 0; i < S; i++) rngs[i] = master.fork();
  std::vector<Walker> sl(S);
  for (size_t i = 0; i < S; i++)
  {
    sl[i].model = &m;
    sl[i].rng = rngs[i].get();
    sl[i].counter_mode = counter;
    sl[i].key = counter_key(p.seed, i);
    sl[i].init();
  }
  std::vector<double> low(R, std::numeric_limits<double>::max());
  std::vector<std::vector<uint8_t>> low_state(R);
  auto save_lowest = [&](size_t rr) {
    size_t b = 0;
    for (size_t k = 1; k < P; k++)
      if (sl[rr * P + k].cost_ < sl[rr * P + b].cost_) b = k;
    if (sl[rr * P + b].cost_ < low[rr])
    {
      low[rr] = sl[rr * P + b].cost_;
      low_state[rr] = sl[rr * P + b].state.spins;
    }
  };
  for (size_t rr = 0; rr < R; rr++) save_lowest(rr);
  Lowest best;
  best.update(low[0], low_state[0]);
  const int64_t n = m.N;
  // the sweep visits get_sweep_size() variables (1 for MaxSat unless the
  // full sweep is asked for); draw positions stay indexed by N
  const int64_t sw = m.sweep_size(p.full_maxsat_sweep != 0);
  set_threads(p.threads);
  int64_t step = 0;
  for (; step < p.step_limit; step++)
  {
    const double b = beta.get_value((double)step), g = field.get_value((double)step);
    const double beta_eff = b / (double)P;
    const double bond_prob = 1 - std::tanh(g * b / (double)P);
    // restarts are independent within a step (own slices and streams)
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t rr = 0; rr < R; rr++)
    {
      std::vector<double> diff(P);
      std::vector<char> bond(P), acc(P);
      Walker* w = &sl[rr * P];
      for (int64_t v = 0; v < sw; v++)
      {
        const uint64_t c = 2 * ((uint64_t)step * (uint64_t)n + (uint64_t)v);
        for (size_t k = 0; k < P; k++)
        {
          diff[k] = cost_difference(m, w[k].state, v);
          bond[k] = 0;
          if (k != 0 && w[k - 1].state.spins[v] == w[k].state.spins[v])
          {
            const double u = counter ? counter_uniform(w[k].key, c) : w[k].rng->uniform();
            bond[k] = u < bond_prob;
          }
        }
        for (size_t k = 0; k < P; k++)
        {
          if (bond[k]) continue;
          double sum = diff[k];
          size_t e = k + 1;
          for (; e < P && bond[e]; e++) sum += diff[e];
          bool a = true;
          if (!(sum < 10E-12))
          {
            const double u = counter ? counter_uniform(w[k].key, c + 1) : w[k].rng->uniform();
            a = u < std::exp(-beta_eff * sum);
          }
          for (size_t i = k; i < e; i++) acc[i] = a;
        }
        for (size_t k = 0; k < P; k++)
          if (acc[k])
          {
            apply_transition(m, v, w[k].state);
            w[k].cost_ += diff[k];
            w[k].total_accepts++;
          }
      }
      for (size_t k = 0; k < P; k++) w[k].total_attempts += (uint64_t)sw;
      save_lowest(rr);
    }
    if (p.has_cost_limit)
    {
      for (size_t rr = 0; rr < R; rr++) best.update(low[rr], low_state[rr]);
      if (best.has && best.cost <= p.cost_limit)
      {
        step++;
        break;
      }
    }
  }
  r.last_step = step;
  // per slice: its cost and state; its restart's lowest
  for (size_t i = 0; i < S; i++)
  {
    r.cost.push_back(sl[i].cost_);
    r.lowest.push_back(low[i / P]);
    r.attempts.push_back(sl[i].total_attempts);
    r.accepts.push_back(sl[i].total_accepts);
    r.states.push_back(sl[i].state.spins);
    r.lowest_states.push_back(low_state[i / P]);
  }
  // populate_solutions over the restarts (solver/model_solver.h:261-308)
  std::vector<size_t> idx(R);
  for (size_t i = 0; i < R; i++) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b2) { return low[a] < low[b2]; });
  const size_t k = std::min((size_t)p.number_of_solutions, R);
  for (size_t i = 0; i < k; i++)
  {
    r.sol_costs.push_back(low[idx[i]] + m.const_cost);
    r.sol_states.push_back(low_state[idx[i]]);
  }
  best.update(low[idx[0]], low_state[idx[0]]);
  r.has_best = best.has;
  r.best_cost = best.cost + m.const_cost;
  r.best_state = best.state;
  return r;
}



// ---------------------------------------------------------------------------
// Multinomial resampling mode of the GB300 library (params "resampling":
// "multinomial", counter streams), restated: the library's exp (Cody-Waite
// reduction with the fdlibm split of ln 2, degree-13 Taylor polynomial by
// fused multiply-adds, 2^k by exponent bits), fixed-point weights
// floor(w 2^40), exact integer prefix sums, parent j = first i with
// prefix_i > hi64(draw_j * total).
// ---------------------------------------------------------------------------
static double multinomial_exp(double x)
{
  if (x < -745.2) return 0.0;
  const double k = std::nearbyint(x * 1.4426950408889634);
  double r = std::fma(-k, 6.93147180369123816490e-01, x);
  r = std::fma(-k, 1.90821492927058770002e-10, r);
  static const double inv_fact[14] = {1.0 / 6227020800.0, 1.0 / 479001600.0, 1.0 / 39916800.0,
                                      1.0 / 3628800.0,    1.0 / 362880.0,    1.0 / 40320.0,
                                      1.0 / 5040.0,       1.0 / 720.0,       1.0 / 120.0,
                                      1.0 / 24.0,         1.0 / 6.0,         0.5,
                                      1.0,                1.0};
  double poly = inv_fact[0];
  for (int j = 1; j < 14; j++) poly = std::fma(poly, r, inv_fact[j]);
  int ki = (int)k;
  if (ki < -1020)
  {
    poly *= 5.551115123125783e-17;  // 2^-54
    ki += 54;
  }
  uint64_t bits = (uint64_t)(int64_t)(ki + 1023) << 52;
  double scale;
  std::memcpy(&scale, &bits, 8);
  return poly * scale;
}

static uint64_t mul_hi64(uint64_t a, uint64_t b)
{
  return (uint64_t)(((unsigned __int128)a * (unsigned __int128)b) >> 64);
}

static Result run_pa(Model& m, const orc_params& p)
{
  Result r;
  r.n_vars = m.N;
  Schedule beta = to_schedule(p.sched);
  if (beta.get_count() == 1)
  {
    if (p.step_limit > 1)
    {
      beta.has_stop = true;
      beta.stop_ = std::max(1, (int)p.step_limit - 1);
    }
    else
      throw std::runtime_error(
          "Either a step_limit or schedule.count must be provided.");
  }
  double beta_start = beta.get_value(0);
  if (m.empty())
  {
    r.best_cost = m.const_cost;
    return r;
  }
  size_t T = (size_t)std::max(1, p.pa_threads);
  size_t target = (size_t)p.population;
  PcgRng master(p.seed);
  if (p.use_master_state) master.pcg.state = p.master_state;
  std::vector<std::unique_ptr<Rng>> rngs(T);
  for (size_t t = 0; t < T; t++) rngs[t] = master.fork();
  // GraphProperties::rescale, graph/graph_properties.h:24-40
  if (!m.rescaled)
  {
    m.rescaled = true;
    if (!(m.max_coupling <= 1 || m.max_coupling == 0))
      m.scale_factor = 1.0 / m.max_coupling;
  }
  bool counter = p.rng_mode == ORC_RNG_COUNTER;
  std::vector<std::unique_ptr<Citizen>> pop;
  double cur_beta = beta_start;
  uint64_t restart_base = 0;
  uint64_t epoch = 0;
  set_threads(p.threads);
  auto run_streams = [&](auto&& body) {
    // emulated schedule(static, 1): stream t handles citizens t, t+T, ...
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t t = 0; t < T; t++)
      for (size_t i = t; i < pop.size(); i += T) body(i, t);
  };
  auto init_population = [&]() {
    // init_population, solver/population_annealing.h:141-167: only newly
    // inserted citizens take the current beta (the blueprint's); citizens
    // that already exist keep theirs until the end of the next step, and
    // every citizen (including any beyond the target) is re-initialised.
    for (size_t i = 0; i < target; i++)
    {
      if (pop.size() <= i)
      {
        pop.emplace_back(new Citizen());
        pop.back()->w.model = &m;
        pop.back()->w.set_beta(cur_beta);
      }
      pop[i]->family = i;
    }
    run_streams([&](size_t i, size_t t) {
      Walker& w = pop[i]->w;
      w.rng = rngs[t].get();
      w.counter_mode = counter;
      w.full_maxsat = p.full_maxsat_sweep != 0;
      w.key = counter_key(p.seed, ((0xFFFFFFFFULL - epoch) << 32) | i);
      w.sweep_counter = 0;
      w.init();
      w.diff_evals = w.accepted = 0;
    });
  };
  init_population();
  Lowest low;
  low.update(pop[0]->w.cost_, pop[0]->w.state.spins);
  int64_t step = 0;
  for (step = 0; step < p.step_limit;)
  {
    size_t R = pop.size();
    double Rd = (double)R;
    std::vector<double> before(R), after(R);
    run_streams([&](size_t i, size_t t) {
      Walker& w = pop[i]->w;
      before[i] = w.cost_;
      w.rng = rngs[t].get();
      w.key = counter_key(p.seed, ((uint64_t)(step + 1) << 32) | i);
      w.sweep_counter = 0;
      w.make_sweeps(p.sweeps_per_replica);
      after[i] = w.cost_;
    });
    for (size_t i = 0; i < R; i++)
      low.update(pop[i]->w.lowest_cost, pop[i]->w.lowest_spins);
    double avg_before = 0, avg_after = 0;
    double min_cost = std::numeric_limits<double>::max();
    for (size_t i = 0; i < R; i++)
    {
      avg_before += before[i];
      avg_after += after[i];
      min_cost = (after[i] < min_cost) ? after[i] : min_cost;
    }
    avg_before /= Rd;
    avg_after /= Rd;
    double var_after = 0;
    for (size_t i = 0; i < R; i++)
    {
      double da = after[i] - avg_after;
      var_after += da * da;
    }
    var_after /= Rd;
    for (size_t i = 0; i < R; i++) after[i] -= min_cost;
    double delta_beta = beta.get_value((double)(step + 1 - restart_base)) -
                        beta.get_value((double)(step - restart_base));
    double rho_t = 1.0;
    bool all_equal = false;
    if (p.resampling == 1)
    {
      double cmax = -std::numeric_limits<double>::max();
      for (size_t i = 0; i < R; i++) cmax = std::max(cmax, after[i] + min_cost);
      all_equal = cmax == min_cost;
    }
    if (delta_beta > 0 && p.resampling == 1)
    {
      // multinomial on counter draws: the population size stays R
      std::vector<uint64_t> prefix(R);
      uint64_t run = 0;
      for (size_t i = 0; i < R; i++)
      {
        const double w = multinomial_exp(-(delta_beta * m.scale_factor) * after[i]);
        run += (uint64_t)(w * 1099511627776.0);
        prefix[i] = run;
      }
      const uint64_t key = counter_key(p.seed, (0x7FFFFFFFULL << 32) | (uint64_t)step);
      std::vector<std::unique_ptr<Citizen>> next;
      for (size_t j = 0; j < R; j++)
      {
        const uint64_t u = mul_hi64(counter_draw(key, (uint64_t)j), run);
        const size_t parent = (size_t)(std::upper_bound(prefix.begin(), prefix.end(), u) - prefix.begin());
        std::unique_ptr<Citizen> cp(new Citizen(*pop[parent]));
        cp->count = 1;
        next.push_back(std::move(cp));
      }
      pop.swap(next);
      std::map<size_t, size_t> fam;
      for (auto& c : pop) fam[c->family]++;
      uint64_t sq = 0;
      for (auto& f : fam) sq += (uint64_t)f.second * (uint64_t)f.second;
      rho_t = (double)sq / Rd;
    }
    else if (delta_beta > 0)
    {
      // resample, solver/population_annealing.h:490-616
      double total = 0.0;
      std::vector<double> weight(R);
      for (size_t i = 0; i < R; i++)
      {
        weight[i] = exp(-delta_beta * after[i] * m.scale_factor);
        total += weight[i];
      }
      if (p.constant_population)
      {
        size_t resampled = 0;
        std::vector<double> residual(R);
        for (size_t i = 0; i < R; i++)
        {
          double rel = (double)target * weight[i] / total;
          size_t iw = (size_t)floor(rel);
          residual[i] = rel - (double)iw;
          pop[i]->count = iw;
          resampled += iw;
        }
        Selector sel;
        for (size_t i = 0; i < R; i++) sel.insert(i, residual[i]);
        while (resampled < R)
        {
          size_t id = sel.select_and_remove(master.uniform());
          pop[id]->count += 1;
          resampled++;
        }
      }
      else
      {
        double RRQ = (double)target / total;
        uint64_t cur = R;
        for (size_t i = 0; i < R; i++)
        {
          size_t nc = (RRQ * weight[i]) > 0.0
                          ? (size_t)floor(master.poisson(RRQ * weight[i]))
                          : size_t(0);
          if (nc == 0)
          {
            cur -= pop[i]->count;
            pop[i]->count = 0;
          }
          else if (nc > 1)
          {
            cur += nc - 1;
            pop[i]->count += nc - 1;
          }
        }
        if (cur == 0)
        {
          size_t i = (size_t)floor(master.uniform() * pop.size());
          pop[i]->count += 1;
        }
      }
      // Population::resample, solver/population.h:171-218: dead citizens
      // removed, then for each survivor its (count-1) copies followed by the
      // survivor itself.
      std::vector<std::unique_ptr<Citizen>> next;
      for (size_t i = 0; i < R; i++)
      {
        Citizen& c = *pop[i];
        if (c.count == 0) continue;
        for (size_t k = 1; k < c.count; k++)
        {
          std::unique_ptr<Citizen> cp(new Citizen(c));
          cp->count = 1;
          next.push_back(std::move(cp));
        }
        c.count = 1;
        next.push_back(std::move(pop[i]));
      }
      pop.swap(next);
      std::map<size_t, size_t> fam;
      for (auto& c : pop) fam[c->family]++;
      rho_t = 0;
      for (auto& f : fam) rho_t += (double)f.second * (double)f.second;
      rho_t /= Rd;
    }
    r.pa_beta.push_back(cur_beta);
    r.pa_pop.push_back((int64_t)pop.size());
    if (Rd / rho_t < p.alpha || (p.resampling == 1 ? all_equal : var_after == 0))
    {
      cur_beta = beta_start;
      restart_base = step;
      if (p.exp_repopulation) target *= 2;
      epoch++;
      init_population();
    }
    else
    {
      cur_beta += delta_beta;
      for (auto& c : pop) c->w.set_beta(cur_beta);
    }
    step++;
    if (p.has_cost_limit && low.has && low.cost <= p.cost_limit) break;
  }
  r.last_step = step;
  r.master_out = master.pcg.state;
  std::vector<Walker*> wp;
  for (auto& c : pop) wp.push_back(&c->w);
  fill_replicas(r, wp);
  populate(r, wp, low, p.number_of_solutions, m, true, true);
  return r;
}

// ---------------------------------------------------------------------------
// Toy model of the reference's solver tests (solver/test/test_model.cc:4-38):
// cost |x - 42|, random transition x + 10u - 5, initial x = 100u, sweep size
// 10, random-order sweep (markov/walker.h:155-178).
// ---------------------------------------------------------------------------
struct ToyWalker
{
  Rng* rng = nullptr;
  double x = 0, cost_ = 0, lowest_cost = 0, lowest_x = 0;
  uint64_t diff_evals = 0, accepted = 0;
  double beta_ = 1, temperature_ = 1;
  std::vector<uint8_t> dummy;
  const std::vector<uint8_t>& lowest_spins_ref() const { return dummy; }
  void set_temperature(double t)
  {
    temperature_ = t;
    if (temperature_ <= 0)
    {
      temperature_ = 0.0;
      beta_ = std::numeric_limits<double>::infinity();
    }
    else
      beta_ = 1.0 / temperature_;
  }
  void set_beta(double b)
  {
    beta_ = b;
    if (beta_ <= 0)
    {
      beta_ = 0;
      temperature_ = std::numeric_limits<double>::infinity();
    }
    else
      temperature_ = 1.0 / beta_;
  }
  void init()
  {
    x = rng->uniform() * 100;
    cost_ = std::abs(x - 42);
    lowest_cost = cost_;
    lowest_x = x;
  }
  void make_sweep()
  {
    for (int k = 0; k < 10; k++)
    {
      double t = x + rng->uniform() * 10 - 5;
      double d = std::abs(t - 42) - std::abs(x - 42);
      diff_evals++;
      RngDraws src(rng);
      if (metropolis_accept(d, beta_, src))
      {
        x = t;
        accepted++;
        cost_ += d;
        if (cost_ < lowest_cost)
        {
          lowest_cost = cost_;
          lowest_x = x;
        }
      }
    }
  }
  void swap_state(ToyWalker& o)
  {
    std::swap(x, o.x);
    std::swap(cost_, o.cost_);
  }
};

}  // namespace orc

using namespace orc;

// ===========================================================================
// C interface
// ===========================================================================

static void set_err(char* err, int errlen, const char* msg)
{
  if (err && errlen > 0)
  {
    strncpy(err, msg, errlen - 1);
    err[errlen - 1] = 0;
  }
}

extern "C" {

void orc_pcg_stream(uint32_t seed, int use_default_seed, int n, uint32_t* out)
{
  Pcg32 g;
  if (!use_default_seed) g = Pcg32(seed);
  for (int i = 0; i < n; i++) out[i] = g();
}

// one 32-bit output of the PCG stream in the given state, the state advanced
uint32_t orc_pcg_state_u32(uint64_t* state)
{
  Pcg32 g;
  g.state = *state;
  const uint32_t x = g();
  *state = g.state;
  return x;
}

// one uniform() of the PCG stream in the given state, the state advanced
double orc_pcg_state_uniform(uint64_t* state)
{
  PcgRng g;
  g.pcg.state = *state;
  const double u = g.uniform();
  *state = g.pcg.state;
  return u;
}

void orc_pcg_uniform(uint32_t seed, int use_default_seed, int n, double* out)
{
  PcgRng g;
  if (!use_default_seed) g = PcgRng(seed);
  for (int i = 0; i < n; i++) out[i] = g.uniform();
}

void orc_pcg_fork_uniform(uint32_t seed, int n_forks, int n, double* out)
{
  PcgRng r(seed);
  std::vector<std::unique_ptr<Rng>> f;
  for (int k = 0; k < n_forks; k++) f.push_back(r.fork());
  for (int i = 0; i < n; i++)
  {
    out[i * (n_forks + 1)] = r.uniform();
    for (int k = 0; k < n_forks; k++)
      out[i * (n_forks + 1) + 1 + k] = f[k]->uniform();
  }
}

void orc_twister_uniform(uint32_t seed, int use_default_seed, int n,
                         double* out)
{
  TwisterRng g;
  if (!use_default_seed) g = TwisterRng(seed);
  for (int i = 0; i < n; i++) out[i] = g.uniform();
}

void orc_uniform_ln(double* out)
{
  const std::vector<double>& t = uniform_ln();
  for (size_t i = 0; i < t.size(); i++) out[i] = t[i];
}

int orc_metropolis_accept(double cost_diff, double beta, const uint32_t* draws,
                          int n_draws, int* used)
{
  struct Arr : DrawSource
  {
    const uint32_t* d;
    int n, k = 0;
    uint32_t next() override { return k < n ? d[k++] : (k++, 0u); }
  } src;
  src.d = draws;
  src.n = n_draws;
  bool a = metropolis_accept(cost_diff, beta, src);
  if (used) *used = src.k;
  return a ? 1 : 0;
}

uint64_t orc_counter_draw(uint64_t key, uint64_t ctr)
{
  return counter_draw(key, ctr);
}

double orc_qexp(double x) { return multinomial_exp(x); }
uint64_t orc_counter_key(uint32_t seed, uint64_t stream)
{
  return counter_key(seed, stream);
}

void* orc_model_create(int kind, int64_t n_terms, const int64_t* term_off,
                       const int32_t* ids, const double* coef, char* err,
                       int errlen)
{
  try
  {
    std::unique_ptr<Model> m(new Model());
    m->kind = kind;
    if (kind == MAXSAT)
      configure_maxsat(*m, n_terms, term_off, ids, coef);
    else
      normalize(*m, n_terms, term_off, ids, coef,
                kind == PUBO || kind == PUBO_PLAIN);
    return m.release();
  }
  catch (std::exception& e)
  {
    set_err(err, errlen, e.what());
    return nullptr;
  }
}

void orc_model_destroy(void* m) { delete (Model*)m; }
int64_t orc_model_n_vars(void* m) { return ((Model*)m)->N; }
int64_t orc_model_n_terms(void* m) { return ((Model*)m)->M; }
double orc_model_const_cost(void* m) { return ((Model*)m)->const_cost; }
double orc_model_scale_factor(void* m)
{
  Model* mm = (Model*)m;
  if (mm->max_coupling <= 1 || mm->max_coupling == 0) return 1.0;
  return 1.0 / mm->max_coupling;
}
void orc_model_var_names(void* m, int32_t* out)
{
  Model* mm = (Model*)m;
  for (size_t i = 0; i < mm->id_to_name.size(); i++) out[i] = mm->id_to_name[i];
}

static State state_from_spins(const Model& m, const uint8_t* spins)
{
  State s = create_state(m);
  for (int64_t i = 0; i < m.N; i++)
    if (spins[i]) apply_transition(m, i, s);
  return s;
}

double orc_state_cost(void* m, const uint8_t* spins)
{
  Model& mm = *(Model*)m;
  return calculate_cost(mm, state_from_spins(mm, spins));
}
double orc_state_cost_difference(void* m, const uint8_t* spins, int64_t var)
{
  Model& mm = *(Model*)m;
  return cost_difference(mm, state_from_spins(mm, spins), var);
}
void orc_state_apply(void* m, uint8_t* spins, int64_t var)
{
  (void)m;
  spins[var] = !spins[var];
}

// The reference model tests' Metropolis loop (model/test/ising_test.cc:
// 136-160): random transition from a Mersenne twister, exp acceptance.
double orc_model_twister_min(void* m, uint32_t seed, int iters, double T)
{
  Model& mm = *(Model*)m;
  State s = create_state(mm);
  TwisterRng rng(seed);
  double cost = calculate_cost(mm, s), mn = cost;
  for (int i = 0; i < iters; i++)
  {
    int64_t t;
    if (mm.kind == ISING || mm.kind == ISING_PLAIN)
      t = (int64_t)(rng.uniform() * (double)mm.N);
    else
      t = (int64_t)floor(rng.uniform() * (double)mm.N);
    double d = cost_difference(mm, s, t);
    if (d < 0 || rng.uniform() < exp(-d / T))
    {
      apply_transition(mm, t, s);
      cost += d;
    }
    mn = std::min(mn, cost);
  }
  return mn;
}

void* orc_run(void* m, const orc_params* p, char* err, int errlen)
{
  try
  {
    Model& mm = *(Model*)m;
    std::unique_ptr<Result> r(new Result());
    if (p->solver == ORC_SA) *r = run_sa(mm, *p);
    else if (p->solver == ORC_PT) *r = run_pt(mm, *p);
    else if (p->solver == ORC_PA) *r = run_pa(mm, *p);
    else if (p->solver == ORC_TABU) *r = run_tabu(mm, *p);
    else if (p->solver == ORC_SSMC) *r = run_ssmc(mm, *p);
    else if (p->solver == ORC_QMC) *r = run_qmc(mm, *p);
    else throw std::runtime_error("unknown solver");
    return r.release();
  }
  catch (std::exception& e)
  {
    set_err(err, errlen, e.what());
    return nullptr;
  }
}

int64_t orc_res_n_replicas(void* r) { return (int64_t)((Result*)r)->cost.size(); }
int64_t orc_res_n_vars(void* r) { return ((Result*)r)->n_vars; }
int64_t orc_res_last_step(void* r) { return ((Result*)r)->last_step; }
void orc_res_replicas(void* r, double* cost, double* lowest, uint64_t* attempts,
                      uint64_t* accepts)
{
  Result& rr = *(Result*)r;
  for (size_t i = 0; i < rr.cost.size(); i++)
  {
    if (cost) cost[i] = rr.cost[i];
    if (lowest) lowest[i] = rr.lowest[i];
    if (attempts) attempts[i] = rr.attempts[i];
    if (accepts) accepts[i] = rr.accepts[i];
  }
}
void orc_res_states(void* r, uint8_t* out)
{
  Result& rr = *(Result*)r;
  for (size_t i = 0; i < rr.states.size(); i++)
    memcpy(out + i * rr.n_vars, rr.states[i].data(), rr.n_vars);
}
void orc_res_lowest_states(void* r, uint8_t* out)
{
  Result& rr = *(Result*)r;
  for (size_t i = 0; i < rr.lowest_states.size(); i++)
    memcpy(out + i * rr.n_vars, rr.lowest_states[i].data(), rr.n_vars);
}
double orc_res_best_cost(void* r) { return ((Result*)r)->best_cost; }
uint64_t orc_res_master_state(void* r) { return ((Result*)r)->master_out; }
void orc_res_best_state(void* r, uint8_t* out)
{
  Result& rr = *(Result*)r;
  if (!rr.best_state.empty()) memcpy(out, rr.best_state.data(), rr.n_vars);
}
int64_t orc_res_n_solutions(void* r)
{
  return (int64_t)((Result*)r)->sol_costs.size();
}
void orc_res_solutions(void* r, double* costs, uint8_t* states)
{
  Result& rr = *(Result*)r;
  for (size_t i = 0; i < rr.sol_costs.size(); i++)
  {
    costs[i] = rr.sol_costs[i];
    if (states) memcpy(states + i * rr.n_vars, rr.sol_states[i].data(), rr.n_vars);
  }
}
void orc_res_pt_observables(void* r, double* out5)
{
  Result& rr = *(Result*)r;
  for (size_t i = 0; i < rr.pt_obs.size(); i++) out5[i] = rr.pt_obs[i];
}
void orc_res_pa_trace(void* r, int64_t* n_steps, double* beta_out,
                      int64_t* pop_out, int64_t max_steps)
{
  Result& rr = *(Result*)r;
  *n_steps = (int64_t)rr.pa_beta.size();
  for (int64_t i = 0; i < std::min(max_steps, *n_steps); i++)
  {
    beta_out[i] = rr.pa_beta[i];
    pop_out[i] = rr.pa_pop[i];
  }
}
void orc_res_destroy(void* r) { delete (Result*)r; }

int orc_pt_toy(uint32_t seed, int64_t steps, const double* temps_in, int n,
               int use_inverse, double* obs5, double* best)
{
  std::vector<double> temps(temps_in, temps_in + n);
  if (use_inverse) std::sort(temps.begin(), temps.end(), std::greater<double>());
  else std::sort(temps.begin(), temps.end(), std::less<double>());
  PcgRng master(seed);
  std::vector<std::unique_ptr<Rng>> rngs(n);
  for (int i = 0; i < n; i++) rngs[i] = master.fork();
  std::vector<ToyWalker> reps(n);
  for (int i = 0; i < n; i++)
  {
    reps[i].rng = rngs[i].get();
    if (use_inverse) reps[i].set_beta(temps[i]);
    else reps[i].set_temperature(temps[i]);
    reps[i].init();
  }
  std::vector<double> obs;
  auto sweep = [](std::vector<ToyWalker>& ws) {
    for (auto& w : ws) w.make_sweep();
  };
  auto cost_of = [](const ToyWalker& w) { return w.cost_; };
  int64_t last = 0;
  pt_loop(reps, master, steps, use_inverse != 0, obs, (Lowest*)nullptr,
          cost_of, sweep, false, 0, &last, false, 0.0);
  for (size_t i = 0; i < obs.size(); i++) obs5[i] = obs[i];
  double b = std::numeric_limits<double>::max();
  for (auto& w : reps) b = std::min(b, w.lowest_cost);
  *best = b;
  return 0;
}

}  // extern "C"
