// solvers.cc -- host drivers of the simulated annealing and parallel
// tempering solvers, configured from the reference's params JSON.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <numeric>
#include <thread>

#include "host.h"

namespace qio
{
// ---- host-side PCG32 and counter keys (same algorithms as the kernels) ----
static const uint64_t kMult = 6364136223846793005ULL;
static const uint64_t kInc = 1442695040888963407ULL;
struct Pcg
{
  uint64_t state;
  explicit Pcg(uint32_t s) { state = ((uint64_t)s + kInc) * kMult + kInc; }
  uint32_t next()
  {
    uint64_t old = state;
    state = old * kMult + kInc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
};
static uint64_t mix64(uint64_t z)
{
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
uint64_t host_counter_key(uint32_t seed, uint64_t stream)
{
  return mix64(((uint64_t)seed << 32) ^ mix64(stream + 0x9E3779B97F4A7C15ULL));
}

// ---- params helpers ------------------------------------------------------
struct Params
{
  const json::Value& p;
  explicit Params(const json::Value& v) : p(v) {}
  const json::Value* get(const char* k, const char* alias = nullptr) const
  {
    const json::Value* v = p.find(k);
    if (!v && alias) v = p.find(alias);
    return v;
  }
  double num(const char* k, double def, const char* alias = nullptr) const
  {
    const json::Value* v = get(k, alias);
    if (!v || v->is_null()) return def;
    if (!v->is_number()) fail(1, std::string("parameter `") + k + "`: expected number");
    return v->num;
  }
  int64_t integer(const char* k, int64_t def, const char* alias = nullptr) const
  {
    const json::Value* v = get(k, alias);
    if (!v || v->is_null()) return def;
    if (!v->is_number()) fail(1, std::string("parameter `") + k + "`: expected integer");
    return v->is_int ? v->i : (int64_t)v->num;
  }
  bool boolean(const char* k, bool def) const
  {
    const json::Value* v = get(k);
    if (!v || v->is_null()) return def;
    if (v->type == json::Value::BOOL) return v->b;
    if (v->is_number()) return v->num != 0;
    fail(1, std::string("parameter `") + k + "`: expected boolean");
  }
  std::string str(const char* k, const std::string& def) const
  {
    const json::Value* v = get(k);
    if (!v || v->is_null()) return def;
    if (!v->is_string()) fail(1, std::string("parameter `") + k + "`: expected string");
    return v->str;
  }
};

static int default_threads()
{
  unsigned n = std::thread::hardware_concurrency();
  return n ? (int)n : 1;
}

// Solver::configure + SteppingSolver::configure (solver/solver.h:156-218,
// solver/stepping_solver.h:43-81) + ModelSolver::configure
// (solver/model_solver.h:41-82).
static void configure_common(Solver& s, const json::Value& doc)
{
  if (!doc.is_object() || !doc.find("params"))
    fail(1, "Input field `params` is required.");
  s.params = doc["params"];
  Params p(s.params);
  if (p.get("time_limit", "timeout"))
  {
    s.has_time_limit = true;
    s.time_limit = p.num("time_limit", 0, "timeout");
    if (s.time_limit < 0) fail(1, "timeout value must be non-negative");
  }
  if (p.get("cost_limit"))
  {
    s.has_cost_limit = true;
    s.cost_limit = p.num("cost_limit", 0);
  }
  int t = (int)p.integer("threads", 0);
  s.threads = (t > 0 && t < default_threads()) ? t : default_threads();
  int64_t ns = p.integer("number_of_solutions", 1);
  if (ns <= 0 || ns > 10)
    fail(1, "parameter `number_of_solutions`: must be greater than 0 and less than or equal to 10, found " +
                std::to_string(ns));
  s.number_of_solutions = (int)ns;
  s.step_limit = p.integer("step_limit", 10000, "sweeps");
  if (s.step_limit < 0) fail(1, "parameter `step_limit` must be non-negative");
  int64_t seed = p.integer("seed", (int64_t)std::chrono::system_clock::now().time_since_epoch().count());
  s.seed = (uint32_t)seed;
  std::string mode = p.str("rng_mode", "replay");
  if (mode != "replay" && mode != "counter")
    fail(1, "parameter `rng_mode` must be \"replay\" or \"counter\"");
  s.replay = mode == "replay";
  s.full_maxsat_sweep = p.boolean("maxsat_full_sweep", false);
  s.warps_per_block = (int)p.integer("warps_per_block", 0);
  s.profile = p.boolean("profile_kernels", false);
  s.smem_state = p.boolean("smem_state", true);
  std::string kern = p.str("kernel", "auto");
  if (kern == "auto") s.kernel = 0;
  else if (kern == "warp") s.kernel = 1;
  else if (kern == "lanes") s.kernel = 2;
  else if (kern == "levels") s.kernel = 3;
  else if (kern == "fields") s.kernel = 4;
  else fail(1, "parameter `kernel` must be \"auto\", \"warp\", \"lanes\", \"levels\" or \"fields\"");
  s.output_params.push_back({"seed", std::to_string(s.seed)});
  s.output_params.push_back({"step_limit", std::to_string(s.step_limit)});
}

void configure_common_public(Solver& s, const json::Value& doc) { configure_common(s, doc); }

bool Solver::advance(cudaStream_t, int64_t)
{
  fail(1, "solver " + target() + " cannot run in pieces");
}

void Solver::prof_begin(cudaStream_t s)
{
  if (!profile) return;
  if (prof_used == prof_events.size())
  {
    cudaEvent_t a, b;
    cuda_check(cudaEventCreate(&a), "cudaEventCreate");
    cuda_check(cudaEventCreate(&b), "cudaEventCreate");
    prof_events.push_back({a, b});
  }
  cuda_check(cudaEventRecord(prof_events[prof_used].first, s), "cudaEventRecord");
}

void Solver::prof_end(cudaStream_t s)
{
  if (!profile) return;
  cuda_check(cudaEventRecord(prof_events[prof_used].second, s), "cudaEventRecord");
  prof_used++;
}

double Solver::prof_total_ms()
{
  double t = 0;
  for (size_t i = 0; i < prof_used; i++)
  {
    cuda_check(cudaEventSynchronize(prof_events[i].second), "cudaEventSynchronize");
    float ms = 0;
    cudaEventElapsedTime(&ms, prof_events[i].first, prof_events[i].second);
    t += ms;
  }
  prof_used = 0;
  return t;
}

// ---------------------------------------------------------------------------
// Population of walkers on the device.
// ---------------------------------------------------------------------------
struct Population
{
  DevBuf buf;
  DevPop pop{};
  int n = 0;
  uint64_t* rng = nullptr;
  int* slot_of = nullptr;
  double* beta = nullptr;
  // cached local fields of the field-cached sweep, per slot; fvalid: they
  // match the slots' states (false after anything else changed the states)
  DevBuf fbuf;
  int* field = nullptr;
  bool fvalid = false;

  void ensure_fields(int64_t N)
  {
    if (field) return;
    fbuf = DevBuf((size_t)n * (size_t)fc_words((int)N) * 4);
    field = (int*)fbuf.ptr;
  }

  void alloc(const HostModel& m, int slots, int streams, bool need_slots,
             int64_t n_beta)
  {
    const bool plain = m.flavor == F_PLAIN_ISING || m.flavor == F_PLAIN_PUBO;
    alloc_sizes(m.N, plain ? 0 : m.M, slots, streams, need_slots, n_beta);
  }

  // strides for models of up to N variables and M term-state bytes
  void alloc_sizes(int64_t N, int64_t M, int slots, int streams, bool need_slots, int64_t n_beta)
  {
    n = slots;
    int nw = (int)(((N + 31) / 32 + 3) & ~3LL);
    int mp = std::max(16, (int)((M + 15) & ~15LL));
    size_t S = (size_t)slots;
    size_t off = 0;
    auto take = [&](size_t bytes) {
      size_t o = off;
      off = (off + bytes + 255) & ~(size_t)255;
      return o;
    };
    size_t o_sp = take(S * nw * 4), o_ts = take(S * mp), o_c = take(S * 8),
           o_l = take(S * 8), o_ls = take(S * nw * 4), o_at = take(S * 8),
           o_ac = take(S * 8), o_sa = take(S * 8), o_sc = take(S * 8), o_wi = take(S * 8),
           o_rng = take((size_t)streams * 8), o_slot = take(need_slots ? S * 4 : 0),
           o_beta = take((size_t)n_beta * 8), o_tag = take(need_slots ? S * 8 : 0);
    buf = DevBuf(off);
    char* b = (char*)buf.ptr;
    pop.n = slots;
    pop.nw = nw;
    pop.mp = mp;
    pop.spins = (uint32_t*)(b + o_sp);
    pop.tstate = (uint8_t*)(b + o_ts);
    pop.cost = (double*)(b + o_c);
    pop.lowest = (double*)(b + o_l);
    pop.lspins = (uint32_t*)(b + o_ls);
    pop.attempts = (unsigned long long*)(b + o_at);
    pop.accepts = (unsigned long long*)(b + o_ac);
    pop.step_att = (unsigned long long*)(b + o_sa);
    pop.step_acc = (unsigned long long*)(b + o_sc);
    pop.windows = (unsigned long long*)(b + o_wi);
    rng = (uint64_t*)(b + o_rng);
    slot_of = need_slots ? (int*)(b + o_slot) : nullptr;
    beta = (double*)(b + o_beta);
    // the lowest's launch tags: population kept by slot labels (tempering)
    pop.lowtag = need_slots ? (long long*)(b + o_tag) : nullptr;
  }

  static void unpack(const std::vector<uint32_t>& words, int nw, int64_t N,
                     int64_t count, std::vector<uint8_t>& out)
  {
    out.resize((size_t)count * N);
    unpack_states(words.data(), nw, N, count, out.data());
  }
};

// eight variables per table lookup: byte b of a state word expands to the
// eight output bytes of its bits (hosts are little-endian: x86-64, aarch64)
void unpack_states(const uint32_t* words, int nw, int64_t N, int64_t count, uint8_t* out)
{
  static const std::array<uint64_t, 256> lut = [] {
    std::array<uint64_t, 256> t{};
    for (int b = 0; b < 256; b++)
      for (int k = 0; k < 8; k++) t[b] |= (uint64_t)((b >> k) & 1) << (8 * k);
    return t;
  }();
  const int64_t whole = N / 8;
  for (int64_t r = 0; r < count; r++)
  {
    const uint32_t* w = words + r * nw;
    uint8_t* o = out + r * N;
    for (int64_t q = 0; q < whole; q++)
    {
      const uint32_t byte = (w[q >> 2] >> ((q & 3) * 8)) & 255u;
      memcpy(o + 8 * q, &lut[byte], 8);
    }
    for (int64_t v = whole * 8; v < N; v++) o[v] = (uint8_t)((w[v >> 5] >> (v & 31)) & 1u);
  }
}

uint64_t sum_windows(const DevPop& p, int n)
{
  if (n <= 0 || !p.windows) return 0;
  std::vector<unsigned long long> w(n);
  cuda_check(cudaMemcpy(w.data(), p.windows, (size_t)n * 8, cudaMemcpyDeviceToHost), "D2H");
  uint64_t t = 0;
  for (auto x : w) t += x;
  return t;
}

// warps per block: enough that the grid needs at most one block per SM
// (152 SMs), so every sub-partition runs at most one walker's warp when the
// walkers are fewer than the sub-partitions
int pick_wpb(int requested, int streams)
{
  if (requested > 0) return std::min(8, requested);
  int w = (streams + 151) / 152;
  return std::max(1, std::min(8, w));
}

struct EventTimer
{
  cudaEvent_t a, b;
  cudaStream_t s;
  explicit EventTimer(cudaStream_t st) : s(st)
  {
    cuda_check(cudaEventCreate(&a), "cudaEventCreate");
    cuda_check(cudaEventCreate(&b), "cudaEventCreate");
    cuda_check(cudaEventRecord(a, s), "cudaEventRecord");
  }
  double stop()
  {
    cuda_check(cudaEventRecord(b, s), "cudaEventRecord");
    cuda_check(cudaEventSynchronize(b), "cudaEventSynchronize");
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
  ~EventTimer()
  {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

// Lane-per-walker execution (lanes.cu): the group layout of the walkers,
// the device copy of their model descriptors, and the transposes between the
// population's bit-packed layout and the groups' interleaved bytes.
void LaneRunner::setup(const std::vector<DevModel>& models, const std::vector<int>& model_of, int n_walkers,
                       const std::vector<int>& local_of, bool smem)
{
    max_words = max_terms = 0;
    for (int r = 0; r < n_walkers; r++)
    {
      const DevModel& m = models[model_of.empty() ? 0 : model_of[r]];
      max_words = std::max(max_words, (m.n_vars + 31) / 32);
      max_terms = std::max(max_terms, m.n_terms);
      if (model_of.empty()) break;
    }
    // lanes per group: 32 when a group's words (and the padding word) fit in
    // shared memory, else as many as fit (at least 8), else 32 in global memory
    const int words = max_words + 1;
    int lanes = 32, smem_words = 0;
    if (smem)
    {
      if (32 * words * 4 <= kLwSmemBytes) smem_words = words;
      else if (8 * words * 4 <= kLwSmemBytes)
      {
        lanes = kLwSmemBytes / (words * 4);
        smem_words = words;
      }
    }
    const int G = (n_walkers + lanes - 1) / lanes;
    std::vector<long long> off(G);
    std::vector<int> nv(G);
    long long total = 0;
    for (int g = 0; g < G; g++)
    {
      int n = 0;
      for (int l = 0; l < lanes && g * lanes + l < n_walkers; l++)
      {
        const DevModel& m = models[model_of.empty() ? 0 : model_of[g * lanes + l]];
        n = std::max(n, m.n_vars);
      }
      nv[g] = (n + 31) / 32 + 1;  // spin words per lane, and the padding word
      off[g] = total;
      total += ((long long)nv[g] * 8 * lanes + (long long)kLwLog * 4 * lanes + 255) & ~255LL;
    }

    size_t o_m = 0, o_mo = (models.size() * sizeof(DevModel) + 255) & ~(size_t)255;
    size_t o_off = o_mo + ((model_of.size() * 4 + 255) & ~(size_t)255);
    size_t o_nv = o_off + (((size_t)G * 8 + 255) & ~(size_t)255);
    size_t o_lo = o_nv + (((size_t)G * 4 + 255) & ~(size_t)255);
    size_t bytes = o_lo + local_of.size() * 4 + 16;
    meta = DevBuf(bytes);
    arena = DevBuf((size_t)std::max<long long>(total, 256));
    char* b = (char*)meta.ptr;
    cuda_check(cudaMemcpy(b + o_m, models.data(), models.size() * sizeof(DevModel), cudaMemcpyHostToDevice), "H2D");
    if (!model_of.empty())
      cuda_check(cudaMemcpy(b + o_mo, model_of.data(), model_of.size() * 4, cudaMemcpyHostToDevice), "H2D");
    cuda_check(cudaMemcpy(b + o_off, off.data(), (size_t)G * 8, cudaMemcpyHostToDevice), "H2D");
    cuda_check(cudaMemcpy(b + o_nv, nv.data(), (size_t)G * 4, cudaMemcpyHostToDevice), "H2D");
    if (!local_of.empty())
      cuda_check(cudaMemcpy(b + o_lo, local_of.data(), local_of.size() * 4, cudaMemcpyHostToDevice), "H2D");
    a = LwArgs{};
    a.models = (const DevModel*)(b + o_m);
    a.model_of = model_of.empty() ? nullptr : (const int*)(b + o_mo);
    a.n_walkers = n_walkers;
    a.arena = (uint8_t*)arena.ptr;
    a.g_off = (const long long*)(b + o_off);
    a.g_nw = (const int*)(b + o_nv);
    a.local_of = local_of.empty() ? nullptr : (const int*)(b + o_lo);
    a.G = lanes;
    a.smem_words = smem_words;
    bool packed = true;
    int md = 0;
    for (const DevModel& m : models)
    {
      packed = packed && m.rec_p != nullptr;
      md = std::max(md, m.max_deg);
    }
    a.packed = packed ? 1 : 0;
    a.unroll = md <= 4 ? 4 : (md <= 6 ? 6 : 8);
    ready = true;
}

// The lane kernel runs Ising models whose terms have one or two members.
bool lanes_eligible(const HostModel& m) { return m.flavor == F_PARITY && m.pair_only; }

// kernel choice: one walker per lane when there are enough walkers to fill
// warps of 32 many times over (or when asked for)
bool lanes_for(const Solver& s, const HostModel& m, int64_t walkers)
{
  if (s.kernel == 2)
  {
    if (!lanes_eligible(m))
      fail(1, "parameter `kernel`: \"lanes\" needs an Ising model whose terms have at most two members");
    return true;
  }
  if (s.kernel == 1 || s.kernel == 3) return false;
  return lanes_eligible(m) && walkers >= 1024;
}

// The level kernel runs integer pair-only Ising models whose level schedule
// fits its bounds, with counter streams (its attempts run out of order).
bool levels_eligible(const HostModel& m)
{
  return m.flavor == F_PARITY && m.pair_only && m.int_mode && m.lv_ok && lv_stride_words((int)m.N) > 0;
}

static const size_t kLevelLogBudget = (size_t)4 << 30;

size_t LevelLog::ensure(int R, int64_t K, const HostModel& m, int nw)
{
  const size_t db = m.lv_d8 ? 1 : 4;
  const long long st = lv_diff_stride((int)m.N);
  const size_t per = (size_t)nw * 4 + 16 + (size_t)st * db;  // one walker, one sweep
  const int64_t fit = (int64_t)(kLevelLogBudget / std::max<size_t>(1, per * (size_t)std::max(1, R)));
  const int k = (int)std::max<int64_t>(1, std::min<int64_t>({K, fit, 64}));
  if (buf.ptr && R <= walkers && k <= sweeps) return buf.bytes;
  const size_t n = (size_t)R * k;
  off_cost = (n * nw * 4 + 255) & ~(size_t)255;
  off_diff = (off_cost + n * 16 + 255) & ~(size_t)255;
  buf = DevBuf(off_diff + n * st * db);
  walkers = R;
  sweeps = k;
  stride = st;
  bytes_per_diff = (int)db;
  return buf.bytes;
}

void LevelLog::fill(LvArgs& a) const
{
  a.log_sweeps = sweeps;
  a.start = (uint32_t*)buf.ptr;
  a.cost0 = (long long*)((char*)buf.ptr + off_cost);
  a.diffs = (char*)buf.ptr + off_diff;
  a.diff_stride = stride;
  a.diff_bytes = bytes_per_diff;
}

// auto: large models (a lane group of them would not fit an SM's shared
// memory many times over), counter streams
bool levels_for(const Solver& s, const HostModel& m)
{
  if (s.kernel == 3)
  {
    if (s.replay) fail(1, "parameter `kernel`: \"levels\" needs \"rng_mode\": \"counter\"");
    if (!levels_eligible(m))
      fail(1, "parameter `kernel`: \"levels\" needs an Ising model with integer coefficients whose "
              "terms have at most two members (and differences within 32-bit integers)");
    return true;
  }
  if (s.kernel != 0) return false;
  return !s.replay && levels_eligible(m) && m.N >= 4096;
}

// The field-cached sweep: Ising with the term cache or counter models
// (PUBO, MaxSat with full sweeps) whose walker state, fields and record tiles
// fit a block's shared memory.  auto: Ising models (1.47x the windowed kernel
// on the 1000-spin sparse SA workload); counter models keep the windowed
// kernel, which measured 4 % faster on the 4096-variable PUBO tempering
// workload; "fields" forces it, "warp" keeps the windowed kernel.
bool fields_for(const Solver& s, const HostModel& m, const Population& P, bool full_maxsat_sweep)
{
  const bool ok = !m.empty() && !m.fc_rec.empty() && s.smem_state &&
                  fc_fits(m.device_view(full_maxsat_sweep), P.pop.nw, P.pop.mp);
  if (s.kernel == 4)
  {
    if (!ok)
      fail(1, "parameter `kernel`: \"fields\" needs an Ising (term-cached) or counter model of fewer "
              "than 32766 variables with rows of at most 255 incidences, every variable in a sweep, "
              "and walker state that fits shared memory");
    return true;
  }
  return s.kernel == 0 && s.auto_fields && ok && m.flavor == F_PARITY;
}

// beta as Metropolis::set_beta / set_temperature store it
// (markov/metropolis.h:35-61)
static double beta_of(double value, bool inverse)
{
  if (inverse) return value <= 0 ? 0.0 : value;
  return value <= 0 ? std::numeric_limits<double>::infinity() : 1.0 / value;
}

// ---------------------------------------------------------------------------
// SimulatedAnnealing (solver/simulated_annealing.h:17-224)
// ---------------------------------------------------------------------------
class SimulatedAnnealing : public Solver
{
 public:
  bool use_inverse = false;
  int64_t restarts = 1;
  Schedule schedule;
  Population P;
  std::vector<double> betas;
  LaneRunner L;
  bool lanes = false, levels = false, fields = false;
  LevelLog lvlog;
  Pcg* ext_master = nullptr;  // repeated runs: the restarts fork from this stream

  std::string target() const override { return "simulatedannealing.qiotoolkit"; }

  // A new run of `sweeps` sweeps and `r` restarts on the linear beta schedule
  // b0 -> b1 (SAParameterFree::update_parameters, solver/sa_parameter_free.h:
  // 120-137); the population is sized afresh at the next init.
  void retarget(int64_t sweeps, int64_t r, double b0, double b1)
  {
    step_limit = sweeps;
    restarts = r;
    use_inverse = true;
    schedule = Schedule();
    schedule.type = 0;
    schedule.initial = b0;
    schedule.final_ = b1;
    schedule.has_stop = true;
    schedule.stop_ = (double)std::max<int64_t>(1, sweeps - 1);
    betas.resize(step_limit);
    for (int64_t k = 0; k < step_limit; k++) betas[k] = beta_of(schedule.get_value((double)k), true);
    P = Population();
    L = LaneRunner();
    lvlog = LevelLog();
    initialized = ran = false;
    step_pos = 0;
    launches = 0;
  }

  void configure(const json::Value& doc)
  {
    configure_common(*this, doc);
    Params p(params);
    use_inverse = p.boolean("use_inverse_temperature", false);
    bool qio_format = false;
    if (p.get("schedule"))
      schedule = parse_schedule(params["schedule"], "schedule");
    else
    {
      double b0 = p.num("beta_start", 0);
      double b1 = p.num("beta_stop", 0.01);
      if (b0 < 0)
        fail(1, "parameter `beta_start`: must be greater than or equal to 0, found " + json::number(b0));
      if (!(b1 > b0))
        fail(1, "parameter `beta_stop`: must be greater than " + json::number(b0) + ", found " + json::number(b1));
      use_inverse = true;
      schedule.type = 0;
      schedule.initial = b0;
      schedule.final_ = b1;
      qio_format = true;
      output_params.push_back({"beta_start", json::number(b0)});
      output_params.push_back({"beta_stop", json::number(b1)});
    }
    (void)qio_format;
    // stretch to step_limit (solver/simulated_annealing.h:175-201)
    if (schedule.get_start() == 0 && schedule.get_stop() == 1 && schedule.get_count() == 1)
    {
      if (step_limit > 1)
      {
        schedule.has_stop = true;
        schedule.stop_ = std::max(1, (int)step_limit - 1);
      }
      else
        fail(1, "The number of sweeps must be greater than 1.");
    }
    restarts = p.integer("restarts", threads);
    if (restarts <= 0) fail(1, "parameter `restarts`: must be greater than 0");
    if (restarts > (1 << 24)) fail(1, "parameter `restarts` too large");
    output_params.push_back({"restarts", std::to_string(restarts)});
    betas.resize(step_limit);
    for (int64_t s = 0; s < step_limit; s++)
      betas[s] = beta_of(schedule.get_value((double)s), use_inverse);
    if (kernel == 3 && !model->empty()) levels_for(*this, *model);  // validates the request
  }

  int64_t n_walkers() const override { return model->empty() ? 0 : restarts; }

  void init(cudaStream_t st) override
  {
    initialized = true;
    if (model->empty()) return;
    ensure_device();
    const int R = (int)restarts;
    if (!P.buf.ptr) P.alloc(*model, R, R, false, std::max<int64_t>(1, step_limit));
    device_bytes = (int64_t)P.buf.bytes;
    // rngs_[i] = rng_->fork() in index order (solver/simulated_annealing.h:53-56)
    std::vector<uint64_t> rs(R);
    Pcg own(seed);
    Pcg& master = ext_master ? *ext_master : own;
    for (int i = 0; i < R; i++) rs[i] = Pcg(master.next()).state;
    cuda_check(cudaMemcpyAsync(P.rng, rs.data(), R * 8, cudaMemcpyHostToDevice, st), "H2D rng");
    if (step_limit > 0)
      cuda_check(cudaMemcpyAsync(P.beta, betas.data(), betas.size() * 8, cudaMemcpyHostToDevice, st),
                 "H2D beta");
    InitArgs a{};
    a.m = model->device_view(full_maxsat_sweep);
    a.p = P.pop;
    a.n_walkers = R;
    a.replay = replay ? (model->kind == K_MAXSAT ? 2 : 1) : (model->kind == K_MAXSAT ? 3 : 0);
    a.rng = P.rng;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = (long long)1 << 40;
    levels = levels_for(*this, *model);
    lanes = !levels && lanes_for(*this, *model, restarts);
    fields = !levels && !lanes && fields_for(*this, *model, P, full_maxsat_sweep);
    if (fields)
    {
      P.ensure_fields(model->N);
      P.fvalid = false;
      device_bytes = (int64_t)(P.buf.bytes + P.fbuf.bytes);
    }
    used_kernel = levels ? 3 : (lanes ? 2 : (fields ? 8 : 1));
    // the lane and level sweeps work from the spins and rebuild the term
    // bytes when they finish
    a.skip_terms = (levels || lanes) ? 1 : 0;
    cuda_check(launch_init(a, st), "init kernel");
    launches++;
    if (levels && !lvlog.buf.ptr) device_bytes += (int64_t)lvlog.ensure(R, step_limit, *model, P.pop.nw);
    if (lanes && !L.ready)
    {
      L.setup({model->device_view(full_maxsat_sweep)}, {}, R, {}, smem_state);
      device_bytes += (int64_t)L.bytes();
    }
  }

  LwArgs lane_args() const
  {
    LwArgs a = L.a;
    a.p = P.pop;
    a.slot_of = nullptr;
    a.beta = P.beta;
    a.bs_w = 0;
    a.bs_s = 1;
    a.replay = replay ? 1 : 0;
    a.int_mode = model->int_mode ? 1 : 0;
    a.rng = P.rng;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = (long long)1 << 40;
    return a;
  }

  LvArgs level_args(int64_t base, int64_t n) const
  {
    LvArgs v{};
    v.m = model->device_view(full_maxsat_sweep);
    v.p = P.pop;
    v.n_walkers = (int)restarts;
    v.beta = P.beta;
    v.bs_w = 0;
    v.bs_s = 1;
    v.sweep_base = base;
    v.n_sweeps = (int)n;
    v.seed = seed;
    v.key_base = 0;
    v.key_div = (long long)1 << 40;
    lvlog.fill(v);
    return v;
  }

  // term bytes from the spins once the level kernel is done with them
  void levels_finish(cudaStream_t st)
  {
    cuda_check(launch_lv_terms(model->device_view(full_maxsat_sweep), P.pop, (int)restarts, nullptr, st),
               "term rebuild");
    launches++;
  }

  // one launch of sweeps [base, base + n) with the chosen kernel
  void sweep_launch(SweepArgs& a, LwArgs& la, int wpb, int64_t base, int64_t n, cudaStream_t st)
  {
    prof_begin(st);
    if (levels)
      cuda_check(launch_lv_sweep(level_args(base, n), st), "level sweep kernel");
    else if (lanes)
    {
      la.sweep_base = base;
      la.n_sweeps = (int)n;
      cuda_check(launch_lw_sweep(la, 0, st), "lane sweep kernel");
    }
    else
    {
      a.sweep_base = base;
      a.n_sweeps = (int)n;
      a.field = fields ? P.field : nullptr;
      a.field_valid = P.fvalid ? 1 : 0;
      cuda_check(launch_sweep(a, st, wpb), "sweep kernel");
      P.fvalid = fields;
    }
    prof_end(st);
    launches++;
  }

  SweepArgs sweep_args() const
  {
    SweepArgs a{};
    a.m = model->device_view(full_maxsat_sweep);
    a.p = P.pop;
    a.n_streams = (int)restarts;
    a.n_walkers = (int)restarts;
    a.beta = P.beta;
    a.bs_w = 0;
    a.bs_s = 1;
    a.replay = replay ? 1 : 0;
    a.rng = P.rng;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = (long long)1 << 40;
    a.smem_state = smem_state ? 1 : 0;
    a.err = device_error_flag();
    return a;
  }

  void run(cudaStream_t st) override
  {
    if (!initialized) fail(1, "init() must be called before run()");
    ran = true;
    if (model->empty()) return;
    EventTimer total(st);
    SweepArgs a = sweep_args();
    LwArgs la = lanes ? lane_args() : LwArgs{};
    int wpb = pick_wpb(warps_per_block, a.n_streams);
    if (lanes)
    {
      cuda_check(launch_lw_load(la, L.max_words, st), "lane load");
      launches++;
    }
    if (!has_cost_limit && !has_time_limit)
    {
      if (step_limit > 0) sweep_launch(a, la, wpb, 0, step_limit, st);
      last_step = step_limit;
    }
    else
    {
      // per-step checks of the stepping loop (solver/stepping_solver.h:
      // 124-258): cost limit after every step, time limit between chunks
      auto t0 = std::chrono::steady_clock::now();
      int64_t chunk = has_cost_limit ? 1 : std::max<int64_t>(1, step_limit / 100);
      std::vector<double> low(restarts);
      int64_t s = 0;
      while (s < step_limit)
      {
        const int64_t n = std::min(chunk, step_limit - s);
        sweep_launch(a, la, wpb, s, n, st);
        s += n;
        if (has_cost_limit)
        {
          cuda_check(cudaMemcpyAsync(low.data(), P.pop.lowest, restarts * 8, cudaMemcpyDeviceToHost, st), "D2H");
          cuda_check(cudaStreamSynchronize(st), "sync");
          if (*std::min_element(low.begin(), low.end()) <= cost_limit) break;
        }
        if (has_time_limit)
        {
          cuda_check(cudaStreamSynchronize(st), "sync");
          double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
          if (el >= time_limit) break;
        }
      }
      last_step = s;
    }
    if (lanes)
    {
      cuda_check(launch_lw_store(la, L.max_words, L.max_terms, st), "lane store");
      launches++;
    }
    if (levels) levels_finish(st);
    run_ms = total.stop();
    sweep_ms = profile ? prof_total_ms() : run_ms;
    check_device_error(st);
  }

  bool advance(cudaStream_t st, int64_t n) override
  {
    if (!initialized) fail(1, "init() must be called before advance()");
    ran = true;
    if (model->empty() || step_limit <= 0)
    {
      last_step = step_limit;
      return true;
    }
    SweepArgs a = sweep_args();
    LwArgs la = lanes ? lane_args() : LwArgs{};
    if (lanes && step_pos == 0)
    {
      cuda_check(launch_lw_load(la, L.max_words, st), "lane load");
      launches++;
    }
    const int64_t todo = std::min(n, step_limit - step_pos);
    if (todo > 0) sweep_launch(a, la, pick_wpb(warps_per_block, a.n_streams), step_pos, todo, st);
    step_pos += todo;
    last_step = step_pos;
    if (step_pos < step_limit) return false;
    if (lanes)
    {
      cuda_check(launch_lw_store(la, L.max_words, L.max_terms, st), "lane store");
      launches++;
    }
    if (levels) levels_finish(st);
    return true;
  }

  uint64_t total_windows() override { return sum_windows(P.pop, (int)n_walkers()); }

  void fetch(std::vector<double>& cost, std::vector<double>& lowest,
             std::vector<uint64_t>& att, std::vector<uint64_t>& acc,
             std::vector<uint8_t>* lowest_states, std::vector<uint8_t>* states) override
  {
    int R = (int)n_walkers();
    cost.resize(R);
    lowest.resize(R);
    att.resize(R);
    acc.resize(R);
    if (!R) return;
    cuda_check(cudaMemcpy(cost.data(), P.pop.cost, R * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(lowest.data(), P.pop.lowest, R * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(att.data(), P.pop.attempts, R * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(acc.data(), P.pop.accepts, R * 8, cudaMemcpyDeviceToHost), "D2H");
    std::vector<uint32_t> w((size_t)R * P.pop.nw);
    if (lowest_states)
    {
      cuda_check(cudaMemcpy(w.data(), P.pop.lspins, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      Population::unpack(w, P.pop.nw, model->N, R, *lowest_states);
    }
    if (states)
    {
      cuda_check(cudaMemcpy(w.data(), P.pop.spins, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      Population::unpack(w, P.pop.nw, model->N, R, *states);
    }
  }
};

// ---------------------------------------------------------------------------
// ParallelTempering (solver/parallel_tempering.h:28-253).  The reference has
// no restarts; the GB300 option "restarts" runs that many independent
// tempering ladders, restart k seeded with seed + k (each identical to a
// reference run with that seed).  Swaps exchange slot labels instead of
// states; RNG streams, lowest states and counters stay with the temperature
// position exactly as the reference's walkers do.
// ---------------------------------------------------------------------------
class ParallelTempering : public Solver
{
 public:
  bool use_inverse = false;
  int64_t spr = 1;
  int restarts = 1;
  Schedule ladder;
  std::vector<double> temps;   // sorted
  std::vector<double> betas;   // per position
  Population P;
  bool fields = false;         // field-cached sweep
  DevBuf aux;
  int* dir = nullptr;
  double *obs_acc = nullptr, *obs_cost = nullptr, *obs_dir = nullptr;
  unsigned long long *swap_acc = nullptr, *swap_cnt = nullptr, *ties = nullptr;
  int* hot_first = nullptr;  // walkers by ascending beta (device)
  uint64_t* master = nullptr;
  unsigned long long* swap_key = nullptr;
  Pcg* ext_master = nullptr;  // repeated runs: ladder 0's streams fork from this stream

  std::string target() const override { return "paralleltempering.qiotoolkit"; }

  // A new run of `sweeps` steps on the inverse temperatures `all_betas`, one
  // ladder (PTParameterFree::update_parameters, solver/pt_parameter_free.h:
  // 124-137); buffers are sized afresh at the next init.
  void retarget(int64_t sweeps, const std::vector<double>& all_betas)
  {
    step_limit = sweeps;
    use_inverse = true;
    ladder = Schedule();
    ladder.type = 3;
    ladder.values = all_betas;
    temps = all_betas;
    std::sort(temps.begin(), temps.end(), std::greater<double>());
    betas.resize(temps.size());
    for (size_t i = 0; i < temps.size(); i++) betas[i] = beta_of(temps[i], true);
    restarts = 1;
    P = Population();
    aux = DevBuf();
    initialized = ran = false;
    step_pos = 0;
    launches = 0;
  }

  size_t best_index(const std::vector<double>& low) override { return time_first_lowest(low); }

  // The walker whose lowest the reference's tempering loop would hold: it
  // offers every position's lowest after each step, in position order, and
  // keeps the first strictly lower one (parallel_tempering.h:163-164 with
  // ModelSolver::update_lowest_cost), so among equal lowest costs the one
  // reached at the earliest step, then the lowest position, wins; position
  // 0's initial state is offered first.
  size_t time_first_lowest(const std::vector<double>& low)
  {
    std::vector<long long> tag(low.size(), 0);
    if (P.pop.lowtag && !low.empty())
      cuda_check(cudaMemcpy(tag.data(), P.pop.lowtag, low.size() * 8, cudaMemcpyDeviceToHost), "D2H");
    // only position 0's initial state is offered before the first step
    for (size_t i = 1; i < tag.size(); i++)
      if (tag[i] < 0) tag[i] = 0;
    size_t b = 0;
    for (size_t i = 1; i < low.size(); i++)
      if (low[i] < low[b] || (low[i] == low[b] && tag[i] < tag[b])) b = i;
    return b;
  }

  // the master stream of ladder 0 after the run (the swaps draw from it)
  uint64_t master_after(cudaStream_t st)
  {
    uint64_t v = 0;
    cuda_check(cudaMemcpyAsync(&v, master, 8, cudaMemcpyDeviceToHost, st), "D2H");
    cuda_check(cudaStreamSynchronize(st), "sync");
    return v;
  }

  void configure(const json::Value& doc)
  {
    configure_common(*this, doc);
    if (kernel == 2 || kernel == 3)
      fail(1, std::string("parameter `kernel`: \"") + (kernel == 2 ? "lanes" : "levels") +
                  "\" is not available for parallel tempering (swaps exchange temperature labels between walkers)");
    Params p(params);
    spr = p.integer("sweeps_per_replica", 1);
    if (spr <= 0) fail(1, "parameter `sweeps_per_replica`: must be greater than 0");
    if (p.get("temperatures"))
    {
      ladder = parse_schedule(params["temperatures"], "temperatures");
      use_inverse = false;
    }
    else if (p.get("all_betas"))
    {
      ladder = parse_schedule(params["all_betas"], "all_betas");
      use_inverse = true;
    }
    else
    {
      ladder.type = 3;
      ladder.values = {0.1, 0.5, 1., 2., 4.};
      use_inverse = true;
    }
    output_params.push_back({use_inverse ? "all_betas" : "temperatures", ladder.render()});
    temps = ladder.discretized();
    if (use_inverse) std::sort(temps.begin(), temps.end(), std::greater<double>());
    else std::sort(temps.begin(), temps.end(), std::less<double>());
    betas.resize(temps.size());
    for (size_t i = 0; i < temps.size(); i++) betas[i] = beta_of(temps[i], use_inverse);
    restarts = (int)p.integer("restarts", 1);
    if (restarts <= 0) fail(1, "parameter `restarts`: must be greater than 0");
  }

  int T() const { return (int)temps.size(); }
  int64_t n_walkers() const override { return model->empty() ? 0 : (int64_t)restarts * T(); }

  void init(cudaStream_t st) override
  {
    initialized = true;
    if (model->empty()) return;
    ensure_device();
    const int W = restarts * T();
    if (!P.buf.ptr) P.alloc(*model, W, W, true, W);
    size_t K = (size_t)restarts;
    size_t off = 0;
    auto take = [&](size_t b) { size_t o = off; off = (off + b + 255) & ~(size_t)255; return o; };
    size_t o_dir = take(W * 4), o_oa = take(W * 8), o_oc = take(W * 8), o_od = take(W * 8),
           o_sa = take(W * 8), o_sc = take(W * 8), o_t = take(8), o_m = take(K * 8),
           o_k = take(K * 8), o_ord = take(W * 4);
    if (!aux.ptr) aux = DevBuf(off);
    char* b = (char*)aux.ptr;
    dir = (int*)(b + o_dir);
    obs_acc = (double*)(b + o_oa);
    obs_cost = (double*)(b + o_oc);
    obs_dir = (double*)(b + o_od);
    swap_acc = (unsigned long long*)(b + o_sa);
    swap_cnt = (unsigned long long*)(b + o_sc);
    ties = (unsigned long long*)(b + o_t);
    master = (uint64_t*)(b + o_m);
    swap_key = (unsigned long long*)(b + o_k);
    hot_first = (int*)(b + o_ord);
    cuda_check(cudaMemsetAsync(aux.ptr, 0, off, st), "memset");
    device_bytes = (int64_t)(P.buf.bytes + aux.bytes);
    std::vector<uint64_t> rs(W), ms(K), keys(K);
    std::vector<int> slots(W);
    std::vector<double> bw(W);
    for (int k = 0; k < restarts; k++)
    {
      Pcg own(seed + (uint32_t)k);
      Pcg& m = (ext_master && k == 0) ? *ext_master : own;
      for (int i = 0; i < T(); i++)
      {
        rs[k * T() + i] = Pcg(m.next()).state;
        slots[k * T() + i] = k * T() + i;
        bw[k * T() + i] = betas[i];
      }
      ms[k] = m.state;
      keys[k] = host_counter_key(seed + (uint32_t)k, 0xFFFFFFFFULL);
    }
    cuda_check(cudaMemcpyAsync(P.rng, rs.data(), W * 8, cudaMemcpyHostToDevice, st), "H2D");
    cuda_check(cudaMemcpyAsync(P.slot_of, slots.data(), W * 4, cudaMemcpyHostToDevice, st), "H2D");
    cuda_check(cudaMemcpyAsync(P.beta, bw.data(), W * 8, cudaMemcpyHostToDevice, st), "H2D");
    cuda_check(cudaMemcpyAsync(master, ms.data(), K * 8, cudaMemcpyHostToDevice, st), "H2D");
    cuda_check(cudaMemcpyAsync(swap_key, keys.data(), K * 8, cudaMemcpyHostToDevice, st), "H2D");
    // walkers hottest first (smallest beta; stable): the field-cached
    // sweep's blocks take them in this order
    std::vector<int> ord(W);
    for (int w = 0; w < W; w++) ord[w] = w;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return bw[x] < bw[y]; });
    cuda_check(cudaMemcpyAsync(hot_first, ord.data(), W * 4, cudaMemcpyHostToDevice, st), "H2D");
    InitArgs a{};
    a.m = model->device_view(full_maxsat_sweep);
    a.p = P.pop;
    a.n_walkers = W;
    a.slot_of = nullptr;  // identity at init
    a.replay = replay ? (model->kind == K_MAXSAT ? 2 : 1) : (model->kind == K_MAXSAT ? 3 : 0);
    a.rng = P.rng;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = T();
    cuda_check(launch_init(a, st), "init kernel");
    fields = fields_for(*this, *model, P, full_maxsat_sweep);
    if (fields)
    {
      P.ensure_fields(model->N);
      device_bytes += (int64_t)P.fbuf.bytes;
    }
    P.fvalid = false;
    used_kernel = fields ? 8 : 1;
    cuda_check(cudaStreamSynchronize(st), "sync");
    // the sweep/swap loop keeps its own copies of the stream so that a
    // host-side pageable copy above cannot race with kernels
    launches++;
  }

  void run(cudaStream_t st) override
  {
    if (!initialized) fail(1, "init() must be called before run()");
    ran = true;
    if (model->empty()) return;
    EventTimer total(st);
    const int W = restarts * T();
    SweepArgs a{};
    a.m = model->device_view(full_maxsat_sweep);
    a.p = P.pop;
    a.n_streams = W;
    a.n_walkers = W;
    a.slot_of = P.slot_of;
    a.beta = P.beta;
    a.bs_w = 1;
    a.bs_s = 0;
    a.n_sweeps = (int)spr;
    a.replay = replay ? 1 : 0;
    a.rng = P.rng;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = T();
    a.smem_state = smem_state ? 1 : 0;
    a.err = device_error_flag();
    SwapArgs sw{};
    sw.restarts = restarts;
    sw.n_temps = T();
    sw.slot_of = P.slot_of;
    sw.cost = P.pop.cost;
    sw.beta = P.beta;
    sw.dir = dir;
    sw.step_acc_reset = P.pop.step_acc;
    sw.step_att_reset = P.pop.step_att;
    sw.obs_acc = obs_acc;
    sw.obs_cost = obs_cost;
    sw.obs_dir = obs_dir;
    sw.swap_acc = swap_acc;
    sw.swap_cnt = swap_cnt;
    sw.near_ties = ties;
    sw.replay = replay ? 1 : 0;
    sw.master = master;
    sw.swap_key = swap_key;
    int wpb = pick_wpb(warps_per_block, W);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<double> low(W);
    int64_t s = 0;
    for (s = 0; s < step_limit;)
    {
      a.sweep_base = s * spr;
      a.tag = s;  // the step, for the time order of equal lowest costs
      a.field = fields ? P.field : nullptr;
      a.order = fields ? hot_first : nullptr;
      a.field_valid = P.fvalid ? 1 : 0;
      prof_begin(st);
      cuda_check(launch_sweep(a, st, wpb), "sweep kernel");
      prof_end(st);
      P.fvalid = fields;
      sw.step = s;
      cuda_check(launch_pt_swap(sw, st), "swap kernel");
      launches += 2;
      s++;
      if (has_cost_limit)
      {
        cuda_check(cudaMemcpyAsync(low.data(), P.pop.lowest, W * 8, cudaMemcpyDeviceToHost, st), "D2H");
        cuda_check(cudaStreamSynchronize(st), "sync");
        if (*std::min_element(low.begin(), low.end()) <= cost_limit) break;
      }
      if (has_time_limit && (s % 16 == 0))
      {
        cuda_check(cudaStreamSynchronize(st), "sync");
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() >= time_limit)
          break;
      }
    }
    last_step = s;
    run_ms = total.stop();
    sweep_ms = profile ? prof_total_ms() : run_ms;
    check_device_error(st);
    unsigned long long nt = 0;
    cuda_check(cudaMemcpy(&nt, ties, 8, cudaMemcpyDeviceToHost), "D2H");
    near_ties = nt;
  }

  bool advance(cudaStream_t st, int64_t n) override
  {
    if (!initialized) fail(1, "init() must be called before advance()");
    ran = true;
    if (model->empty())
    {
      last_step = step_limit;
      return true;
    }
    const int W = restarts * T();
    SweepArgs a{};
    a.m = model->device_view(full_maxsat_sweep);
    a.p = P.pop;
    a.n_streams = W;
    a.n_walkers = W;
    a.slot_of = P.slot_of;
    a.beta = P.beta;
    a.bs_w = 1;
    a.bs_s = 0;
    a.n_sweeps = (int)spr;
    a.replay = replay ? 1 : 0;
    a.rng = P.rng;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = T();
    a.smem_state = smem_state ? 1 : 0;
    a.err = device_error_flag();
    SwapArgs sw{};
    sw.restarts = restarts;
    sw.n_temps = T();
    sw.slot_of = P.slot_of;
    sw.cost = P.pop.cost;
    sw.beta = P.beta;
    sw.dir = dir;
    sw.step_acc_reset = P.pop.step_acc;
    sw.step_att_reset = P.pop.step_att;
    sw.obs_acc = obs_acc;
    sw.obs_cost = obs_cost;
    sw.obs_dir = obs_dir;
    sw.swap_acc = swap_acc;
    sw.swap_cnt = swap_cnt;
    sw.near_ties = ties;
    sw.replay = replay ? 1 : 0;
    sw.master = master;
    sw.swap_key = swap_key;
    const int wpb = pick_wpb(warps_per_block, W);
    const int64_t end = std::min(step_limit, step_pos + n);
    for (; step_pos < end; step_pos++)
    {
      a.sweep_base = step_pos * spr;
      a.tag = step_pos;
      a.field = fields ? P.field : nullptr;
      a.order = fields ? hot_first : nullptr;
      a.field_valid = P.fvalid ? 1 : 0;
      cuda_check(launch_sweep(a, st, wpb), "sweep kernel");
      P.fvalid = fields;
      sw.step = step_pos;
      cuda_check(launch_pt_swap(sw, st), "swap kernel");
      launches += 2;
    }
    last_step = step_pos;
    return step_pos >= step_limit;
  }

  uint64_t total_windows() override { return sum_windows(P.pop, (int)n_walkers()); }

  void fetch(std::vector<double>& cost, std::vector<double>& lowest,
             std::vector<uint64_t>& att, std::vector<uint64_t>& acc,
             std::vector<uint8_t>* lowest_states, std::vector<uint8_t>* states) override
  {
    int W = (int)n_walkers();
    cost.resize(W);
    lowest.resize(W);
    att.resize(W);
    acc.resize(W);
    if (!W) return;
    std::vector<double> slot_cost(W);
    std::vector<int> slots(W);
    cuda_check(cudaMemcpy(slot_cost.data(), P.pop.cost, W * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(slots.data(), P.slot_of, W * 4, cudaMemcpyDeviceToHost), "D2H");
    for (int w = 0; w < W; w++) cost[w] = slot_cost[slots[w]];
    cuda_check(cudaMemcpy(lowest.data(), P.pop.lowest, W * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(att.data(), P.pop.attempts, W * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(acc.data(), P.pop.accepts, W * 8, cudaMemcpyDeviceToHost), "D2H");
    std::vector<uint32_t> wds((size_t)W * P.pop.nw);
    if (lowest_states)
    {
      cuda_check(cudaMemcpy(wds.data(), P.pop.lspins, wds.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      Population::unpack(wds, P.pop.nw, model->N, W, *lowest_states);
    }
    if (states)
    {
      cuda_check(cudaMemcpy(wds.data(), P.pop.spins, wds.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      std::vector<uint8_t> by_slot;
      Population::unpack(wds, P.pop.nw, model->N, W, by_slot);
      states->resize(by_slot.size());
      for (int w = 0; w < W; w++)
        memcpy(states->data() + (size_t)w * model->N, by_slot.data() + (size_t)slots[w] * model->N,
               model->N);
    }
  }

  void pt_observables(std::vector<double>& out) override
  {
    int W = (int)n_walkers();
    out.assign((size_t)W * 5, 0);
    if (!W) return;
    std::vector<double> oa(W), oc(W), od(W);
    std::vector<unsigned long long> sa(W), sc(W);
    cuda_check(cudaMemcpy(oa.data(), obs_acc, W * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(oc.data(), obs_cost, W * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(od.data(), obs_dir, W * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(sa.data(), swap_acc, W * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(sc.data(), swap_cnt, W * 8, cudaMemcpyDeviceToHost), "D2H");
    double st = (double)last_step;
    for (int w = 0; w < W; w++)
    {
      int i = w % T();
      out[w * 5 + 0] = use_inverse ? betas[i] : (betas[i] > 0 ? 1.0 / betas[i] : INFINITY);
      if (!use_inverse) out[w * 5 + 0] = temps[i] <= 0 ? 0.0 : temps[i];
      out[w * 5 + 1] = oa[w] / st;
      out[w * 5 + 2] = oc[w] / st;
      out[w * 5 + 3] = od[w] / st;
      out[w * 5 + 4] = sc[w] ? (double)sa[w] / (double)sc[w] : NAN;
    }
  }
};

std::unique_ptr<Solver> make_pa_solver(const HostModel* m, const json::Value& doc);
std::unique_ptr<Solver> make_ssmc_solver(const HostModel* m, const json::Value& doc);
std::unique_ptr<Solver> make_pa_pf_solver(const HostModel* m, const json::Value& doc);
std::unique_ptr<Solver> make_ssmc_pf_solver(const HostModel* m, const json::Value& doc);

// ---------------------------------------------------------------------------
// Tabu search ("tabu.qiotoolkit": solver/tabu.h:22-164 with
// markov/tabu_walker.h).  Restarts fork from the master stream and start
// from random states exactly as the annealing walkers do; the sweeps are
// deterministic (tabu_kernel).
// ---------------------------------------------------------------------------
class TabuSearch : public Solver
{
 public:
  int64_t restarts = 1;
  uint64_t tenure = 0;
  std::vector<uint64_t> tenure_list;  // per restart (parameter-free runs)
  Pcg* ext_master = nullptr;          // repeated runs: the restarts fork from this stream
  Population P;
  DevBuf aux;
  TabuArgs ta{};

  // another run of the parameter-free search: its sweeps, restarts, tenures
  void retarget(int64_t sweeps, int64_t r, const std::vector<uint64_t>& tenures)
  {
    step_limit = sweeps;
    restarts = r;
    tenure_list = tenures;
    P = Population();
    aux = DevBuf();
    initialized = ran = false;
    step_pos = 0;
    launches = 0;
  }

  std::string target() const override { return "tabu.qiotoolkit"; }

  void configure(const json::Value& doc)
  {
    configure_common(*this, doc);
    Params p(params);
    const int64_t t = p.integer("tabu_tenure", 0);
    if (t < 0) fail(1, "parameter `tabu_tenure`: must be greater than or equal to 0, found " + std::to_string(t));
    tenure = (uint64_t)t;
    restarts = p.integer("restarts", threads);
    if (restarts <= 0) fail(1, "parameter `restarts`: must be greater than 0");
    if (restarts > (1 << 24)) fail(1, "parameter `restarts` too large");
    output_params.push_back({"tabu_tenure", std::to_string(tenure)});
    output_params.push_back({"restarts", std::to_string(restarts)});
  }

  int64_t n_walkers() const override { return model->empty() ? 0 : restarts; }

  void init(cudaStream_t st) override
  {
    initialized = true;
    if (model->empty()) return;
    ensure_device();
    const int R = (int)restarts;
    if (!P.buf.ptr) P.alloc(*model, R, R, false, 1);
    const size_t nw = (size_t)P.pop.nw, N = (size_t)model->N;
    size_t off = 0;
    auto take = [&](size_t b) { size_t o = off; off = (off + b + 255) & ~(size_t)255; return o; };
    const size_t o_t = take((size_t)R * N * 8), o_h = take((size_t)R * nw * 4), o_l = take((size_t)R * nw * 4),
                 o_s = take((size_t)R * sizeof(TabuState)), o_d = take((size_t)R * N * 8),
                 o_hd = take((size_t)R * N * 8), o_tn = take((size_t)R * 8);
    if (!aux.ptr) aux = DevBuf(off);
    char* b = (char*)aux.ptr;
    cuda_check(cudaMemsetAsync(aux.ptr, 0, off, st), "memset");
    device_bytes = (int64_t)(P.buf.bytes + aux.bytes);
    // rngs_[i] = rng_->fork() in index order (solver/tabu.h:56-60)
    std::vector<uint64_t> rs(R);
    Pcg own(seed);
    Pcg& master = ext_master ? *ext_master : own;
    for (int i = 0; i < R; i++) rs[i] = Pcg(master.next()).state;
    if (!tenure_list.empty())
    {
      if ((int64_t)tenure_list.size() < R) fail(6, "tabu: fewer tenures than restarts");
      cuda_check(cudaMemcpyAsync(b + o_tn, tenure_list.data(), (size_t)R * 8, cudaMemcpyHostToDevice, st), "H2D");
    }
    cuda_check(cudaMemcpyAsync(P.rng, rs.data(), R * 8, cudaMemcpyHostToDevice, st), "H2D rng");
    InitArgs a{};
    a.m = model->device_view(full_maxsat_sweep);
    a.p = P.pop;
    a.n_walkers = R;
    // MaxSat states draw one uniform() per variable (model/max_sat.h:144-150)
    a.replay = replay ? (model->kind == K_MAXSAT ? 2 : 1) : (model->kind == K_MAXSAT ? 3 : 0);
    a.rng = P.rng;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = (long long)1 << 40;
    a.skip_terms = 1;  // the tabu sweeps gather the member spins
    used_kernel = 4;
    cuda_check(launch_init(a, st), "init kernel");
    launches++;
    ta = TabuArgs{};
    ta.m = model->device_view(full_maxsat_sweep);
    ta.p = P.pop;
    ta.n_walkers = R;
    ta.tenure = tenure;
    ta.tabu = (unsigned long long*)(b + o_t);
    ta.hc = (uint32_t*)(b + o_h);
    ta.hc_low = (uint32_t*)(b + o_l);
    ta.st = (TabuState*)(b + o_s);
    ta.tenures = tenure_list.empty() ? nullptr : (const unsigned long long*)(b + o_tn);
    ta.diff = (double*)(b + o_d);
    ta.hdiff = (double*)(b + o_hd);
    step_pos = 0;
  }

  void run(cudaStream_t st) override
  {
    if (!initialized) fail(1, "init() must be called before run()");
    ran = true;
    if (model->empty()) return;
    EventTimer total(st);
    int64_t s = 0;
    const int64_t chunk = (has_cost_limit || has_time_limit) ? std::max<int64_t>(1, step_limit / 100) : step_limit;
    auto t0 = std::chrono::steady_clock::now();
    std::vector<double> low(restarts);
    while (s < step_limit)
    {
      TabuArgs a = ta;
      a.n_steps = (int)std::min(chunk, step_limit - s);
      prof_begin(st);
      cuda_check(launch_tabu(a, st), "tabu kernel");
      prof_end(st);
      launches++;
      s += a.n_steps;
      if (has_cost_limit)
      {
        cuda_check(cudaMemcpyAsync(low.data(), P.pop.lowest, restarts * 8, cudaMemcpyDeviceToHost, st), "D2H");
        cuda_check(cudaStreamSynchronize(st), "sync");
        if (*std::min_element(low.begin(), low.end()) <= cost_limit) break;
      }
      if (has_time_limit)
      {
        cuda_check(cudaStreamSynchronize(st), "sync");
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() >= time_limit) break;
      }
    }
    last_step = s;
    run_ms = total.stop();
    sweep_ms = profile ? prof_total_ms() : run_ms;
    check_device_error(st);
  }

  // serving pieces: up to n further tabu sweeps per call
  bool advance(cudaStream_t st, int64_t n) override
  {
    if (!initialized) fail(1, "init() must be called before advance()");
    ran = true;
    if (model->empty() || step_limit <= 0)
    {
      last_step = step_limit;
      return true;
    }
    const int64_t todo = std::min(n, step_limit - step_pos);
    if (todo > 0)
    {
      TabuArgs a = ta;
      a.n_steps = (int)todo;
      cuda_check(launch_tabu(a, st), "tabu kernel");
      launches++;
    }
    step_pos += todo;
    last_step = step_pos;
    return step_pos >= step_limit;
  }

  void fetch(std::vector<double>& cost, std::vector<double>& lowest, std::vector<uint64_t>& att,
             std::vector<uint64_t>& acc, std::vector<uint8_t>* lowest_states,
             std::vector<uint8_t>* states) override
  {
    const int R = (int)n_walkers();
    cost.resize(R);
    lowest.resize(R);
    att.resize(R);
    acc.resize(R);
    if (!R) return;
    cuda_check(cudaMemcpy(cost.data(), P.pop.cost, R * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(lowest.data(), P.pop.lowest, R * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(att.data(), P.pop.attempts, R * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(acc.data(), P.pop.accepts, R * 8, cudaMemcpyDeviceToHost), "D2H");
    std::vector<uint32_t> w((size_t)R * P.pop.nw);
    if (lowest_states)
    {
      cuda_check(cudaMemcpy(w.data(), P.pop.lspins, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      Population::unpack(w, P.pop.nw, model->N, R, *lowest_states);
    }
    if (states)
    {
      cuda_check(cudaMemcpy(w.data(), P.pop.spins, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      Population::unpack(w, P.pop.nw, model->N, R, *states);
    }
  }
};

// ---------------------------------------------------------------------------
// Quantum Monte Carlo ("quantummontecarlo.qiotoolkit",
// solver/quantum_monte_carlo.h:22-260): restarts of `trotter_number`
// imaginary-time slices swept by qmc_kernel, beta and the transverse field
// linear over the steps.  Walkers are the slices (slot r * trotter + k); a
// slice's lowest is its restart's.
// ---------------------------------------------------------------------------
class QuantumMonteCarlo : public Solver
{
 public:
  int64_t restarts = 1, trotter = 2;
  double beta_start = 1, beta_stop = 1, field_low = 0, field_high = 5;
  Population P;
  DevBuf aux;
  double* d_low = nullptr;
  uint32_t* d_lspins = nullptr;
  unsigned long long* d_ties = nullptr;
  double* d_beta = nullptr;
  unsigned long long* d_blim = nullptr;
  unsigned char* d_ball = nullptr;
  // level schedule of the counter-stream kernel
  bool use_levels = false;
  int n_levels = 0;
  DevBuf lvbuf;
  int* d_lv_off = nullptr;
  int* d_lv_var = nullptr;
  double* d_dlog = nullptr;

  // level(v) = 1 + the largest level of v's lower-index term co-members (0
  // without one); variables listed by level, in index order within a level
  void build_levels(cudaStream_t st)
  {
    const HostModel& m = *model;
    const int N = (int)m.N;
    std::vector<int> lev(N, 0);
    int top = 0;
    for (int v = 0; v < N; v++)
    {
      int L = 0;
      for (int q = m.row[v]; q < m.row[v + 1]; q++)
      {
        const uint32_t t = m.inc[q] & ~kNegBit;
        for (int u = m.trow[t]; u < m.trow[t + 1]; u++)
        {
          const int x = (int)(m.tvar[u] & ~kNegBit);
          if (x < v) L = std::max(L, lev[x] + 1);
        }
      }
      lev[v] = L;
      top = std::max(top, L);
    }
    n_levels = top + 1;
    std::vector<int> off(n_levels + 1, 0), var(N);
    for (int v = 0; v < N; v++) off[lev[v] + 1]++;
    for (int L = 0; L < n_levels; L++) off[L + 1] += off[L];
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (int v = 0; v < N; v++) var[fill[lev[v]]++] = v;
    const size_t S = (size_t)restarts * trotter;
    size_t o = 0;
    auto take = [&](size_t b) { size_t r = o; o = (o + b + 255) & ~(size_t)255; return r; };
    const size_t o_off = take((size_t)(n_levels + 1) * 4), o_var = take((size_t)N * 4),
                 o_log = take(S * (size_t)N * 8);
    lvbuf = DevBuf(o);
    char* b = (char*)lvbuf.ptr;
    d_lv_off = (int*)(b + o_off);
    d_lv_var = (int*)(b + o_var);
    d_dlog = (double*)(b + o_log);
    cuda_check(cudaMemcpyAsync(d_lv_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice, st), "H2D");
    cuda_check(cudaMemcpyAsync(d_lv_var, var.data(), var.size() * 4, cudaMemcpyHostToDevice, st), "H2D");
  }

  std::string target() const override { return "quantummontecarlo.qiotoolkit"; }
  int64_t n_walkers() const override { return model->empty() ? 0 : restarts * trotter; }
  size_t solution_stride() const override { return (size_t)trotter; }

  void configure(const json::Value& doc)
  {
    configure_common(*this, doc);
    Params p(params);
    // solver/quantum_monte_carlo.h:185-229
    beta_stop = p.num("beta_stop", 1.0);
    if (!(beta_stop > 0)) fail(1, "parameter `beta_stop`: must be greater than 0, found " + json::number(beta_stop));
    beta_start = p.num("beta_start", beta_stop);
    if (!(beta_start <= beta_stop))
      fail(1, "parameter `beta_start`: must be less than or equal to " + json::number(beta_stop) + ", found " +
                  json::number(beta_start));
    if (!params.find("beta_stop") && params.find("beta_start")) beta_stop = beta_start;
    field_low = p.num("transverse_field_low", 0.0);
    if (!(field_low >= 0))
      fail(1, "parameter `transverse_field_low`: must be greater than or equal to 0, found " + json::number(field_low));
    field_high = p.num("transverse_field_high", 5.0);
    if (!(field_high > field_low))
      fail(1, "parameter `transverse_field_high`: must be greater than " + json::number(field_low) + ", found " +
                  json::number(field_high));
    trotter = p.integer("trotter_number", threads);
    if (trotter <= 1) fail(1, "parameter `trotter_number`: must be greater than 1");
    if (trotter > kQmcMaxTrotter) fail(1, "parameter `trotter_number`: at most 1024 slices here");
    restarts = p.integer("restarts", 1);
    if (restarts <= 0) fail(1, "parameter `restarts`: must be greater than 0");
    restarts = std::min<int64_t>(restarts, std::max(threads, 16));
    output_params.push_back({"beta_stop", json::number(beta_stop)});
    output_params.push_back({"beta_start", json::number(beta_start)});
    output_params.push_back({"transverse_field_low", json::number(field_low)});
    output_params.push_back({"transverse_field_high", json::number(field_high)});
    output_params.push_back({"trotter_number", std::to_string(trotter)});
    output_params.push_back({"restarts", std::to_string(restarts)});
  }

  void init(cudaStream_t st) override
  {
    initialized = true;
    if (model->empty()) return;
    ensure_device();
    const int S = (int)(restarts * trotter), R = (int)restarts;
    const int64_t steps = std::max<int64_t>(1, step_limit);
    if (!P.buf.ptr)
    {
      P.alloc(*model, S, S, false, 1);
      size_t off = 0;
      auto take = [&](size_t b) { size_t o = off; off = (off + b + 255) & ~(size_t)255; return o; };
      const size_t o_l = take((size_t)R * 8), o_ls = take((size_t)R * P.pop.nw * 4), o_t = take(8),
                   o_b = take((size_t)steps * 8), o_p = take((size_t)steps * 8), o_a = take((size_t)steps);
      aux = DevBuf(off);
      char* b = (char*)aux.ptr;
      d_low = (double*)(b + o_l);
      d_lspins = (uint32_t*)(b + o_ls);
      d_ties = (unsigned long long*)(b + o_t);
      d_beta = (double*)(b + o_b);
      d_blim = (unsigned long long*)(b + o_p);
      d_ball = (unsigned char*)(b + o_a);
    }
    // counter streams draw by position: the level-parallel kernel runs them
    // ("kernel": "warp" keeps one warp per restart)
    use_levels = !replay && kernel != 1 && kernel != 2 && qmc_level_smem((int)trotter, P.pop.nw) > 0 &&
                 (model->kind != K_MAXSAT || full_maxsat_sweep);
    if (use_levels && !lvbuf.ptr) build_levels(st);
    device_bytes = (int64_t)(P.buf.bytes + aux.bytes + lvbuf.bytes);
    // per step: beta / P and 1 - tanh(field * beta / P), both schedules
    // linear with stop max(1, step_limit - 1)
    Schedule bs, fs;
    bs.type = fs.type = 0;
    bs.initial = beta_start;
    bs.final_ = beta_stop;
    fs.initial = field_low;
    fs.final_ = field_high;
    bs.has_stop = fs.has_stop = true;
    bs.stop_ = fs.stop_ = (double)std::max(1, (int)step_limit - 1);
    std::vector<double> be(steps);
    std::vector<unsigned long long> lim(steps);
    std::vector<unsigned char> all(steps, 0);
    // uniform() of the two 32-bit outputs X = d0 + d1 2^32 (libstdc++'s
    // generate_canonical), monotone in X
    auto canon = [](unsigned long long x) {
      const double sum = (double)(uint32_t)x + (double)(uint32_t)(x >> 32) * 4294967296.0;
      const double u = sum * 5.421010862427522170037e-20;
      return u >= 1.0 ? 0.99999999999999988898 : u;
    };
    for (int64_t s = 0; s < steps; s++)
    {
      const double b = bs.get_value((double)s), g = fs.get_value((double)s);
      be[s] = b / (double)trotter;
      const double bp = 1 - std::tanh(g * b / (double)trotter);
      if (replay)
      {
        // the least X with uniform() >= bp (uniform() < bp below it)
        if (canon(~0ULL) < bp)
          all[s] = 1, lim[s] = ~0ULL;
        else
        {
          unsigned long long lo = 0, hi = ~0ULL;
          while (lo < hi)
          {
            const unsigned long long mid = lo + (hi - lo) / 2;
            if (canon(mid) >= bp) hi = mid;
            else lo = mid + 1;
          }
          lim[s] = lo;
        }
      }
      else
      {
        // (draw >> 11) 2^-53 < bp  <=>  draw >> 11 < ceil(bp 2^53)
        const double t = std::ceil(std::max(0.0, std::min(1.0, bp)) * 9007199254740992.0);
        lim[s] = (unsigned long long)t;
      }
    }
    cuda_check(cudaMemcpyAsync(d_beta, be.data(), steps * 8, cudaMemcpyHostToDevice, st), "H2D");
    cuda_check(cudaMemcpyAsync(d_blim, lim.data(), steps * 8, cudaMemcpyHostToDevice, st), "H2D");
    cuda_check(cudaMemcpyAsync(d_ball, all.data(), steps, cudaMemcpyHostToDevice, st), "H2D");
    cuda_check(cudaStreamSynchronize(st), "sync");
    cuda_check(cudaMemsetAsync(d_ties, 0, 8, st), "memset");
    // rngs_[i] = rng_->fork() for the R * P slices in order (:52-58)
    std::vector<uint64_t> rs(S);
    Pcg master(seed);
    for (int i = 0; i < S; i++) rs[i] = Pcg(master.next()).state;
    cuda_check(cudaMemcpyAsync(P.rng, rs.data(), (size_t)S * 8, cudaMemcpyHostToDevice, st), "H2D rng");
    InitArgs a{};
    a.m = model->device_view(full_maxsat_sweep);
    a.p = P.pop;
    a.n_walkers = S;
    a.replay = replay ? (model->kind == K_MAXSAT ? 2 : 1) : (model->kind == K_MAXSAT ? 3 : 0);
    a.rng = P.rng;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = (long long)1 << 40;
    a.skip_terms = 1;
    cuda_check(launch_init(a, st), "init kernel");
    launches++;
    used_kernel = use_levels ? 7 : 6;
    // save_lowest of every restart on its initial slices
    std::vector<double> c(S), low(R);
    cuda_check(cudaMemcpyAsync(c.data(), P.pop.cost, (size_t)S * 8, cudaMemcpyDeviceToHost, st), "D2H");
    cuda_check(cudaStreamSynchronize(st), "sync");
    for (int r = 0; r < R; r++)
    {
      int b = 0;
      for (int k = 1; k < trotter; k++)
        if (c[(size_t)r * trotter + k] < c[(size_t)r * trotter + b]) b = k;
      low[r] = c[(size_t)r * trotter + b];
      cuda_check(cudaMemcpyAsync(d_lspins + (size_t)r * P.pop.nw, P.pop.spins + ((size_t)r * trotter + b) * P.pop.nw,
                                 P.pop.nw * 4, cudaMemcpyDeviceToDevice, st),
                 "D2D");
    }
    cuda_check(cudaMemcpyAsync(d_low, low.data(), (size_t)R * 8, cudaMemcpyHostToDevice, st), "H2D");
    cuda_check(cudaStreamSynchronize(st), "sync");
    step_pos = 0;
  }

  QmcArgs args() const
  {
    QmcArgs a{};
    a.m = model->device_view(full_maxsat_sweep);
    a.p = P.pop;
    a.restarts = (int)restarts;
    a.trotter = (int)trotter;
    a.beta_eff = d_beta;
    a.bond_lim = d_blim;
    a.bond_all = d_ball;
    a.replay = replay ? 1 : 0;
    a.rng = P.rng;
    a.seed = seed;
    a.low = d_low;
    a.low_spins = d_lspins;
    a.near_ties = d_ties;
    a.n_levels = n_levels;
    a.lv_off = d_lv_off;
    a.lv_var = d_lv_var;
    a.dlog = d_dlog;
    return a;
  }

  void launch(cudaStream_t st, int64_t base, int64_t n)
  {
    QmcArgs a = args();
    a.step_base = base;
    a.n_steps = (int)n;
    prof_begin(st);
    cuda_check(use_levels ? launch_qmc_levels(a, st) : launch_qmc(a, st), "qmc kernel");
    prof_end(st);
    launches++;
  }

  void run(cudaStream_t st) override
  {
    if (!initialized) fail(1, "init() must be called before run()");
    ran = true;
    if (model->empty()) return;
    EventTimer total(st);
    const int64_t chunk = (has_cost_limit || has_time_limit) ? std::max<int64_t>(1, step_limit / 100) : step_limit;
    auto t0 = std::chrono::steady_clock::now();
    std::vector<double> low(restarts);
    int64_t s = step_pos;
    while (s < step_limit)
    {
      const int64_t n = std::min(chunk, step_limit - s);
      launch(st, s, n);
      s += n;
      if (has_cost_limit)
      {
        cuda_check(cudaMemcpyAsync(low.data(), d_low, restarts * 8, cudaMemcpyDeviceToHost, st), "D2H");
        cuda_check(cudaStreamSynchronize(st), "sync");
        if (*std::min_element(low.begin(), low.end()) <= cost_limit) break;
      }
      if (has_time_limit)
      {
        cuda_check(cudaStreamSynchronize(st), "sync");
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() >= time_limit) break;
      }
    }
    step_pos = s;
    last_step = s;
    run_ms = total.stop();
    sweep_ms = profile ? prof_total_ms() : run_ms;
    cuda_check(cudaMemcpy(&near_ties, d_ties, 8, cudaMemcpyDeviceToHost), "D2H");
    check_device_error(st);
  }

  bool advance(cudaStream_t st, int64_t n) override
  {
    if (!initialized) fail(1, "init() must be called before advance()");
    ran = true;
    if (model->empty() || step_limit <= 0)
    {
      last_step = step_limit;
      return true;
    }
    const int64_t todo = std::min(n, step_limit - step_pos);
    if (todo > 0) launch(st, step_pos, todo);
    step_pos += todo;
    last_step = step_pos;
    return step_pos >= step_limit;
  }

  void fetch(std::vector<double>& cost, std::vector<double>& lowest, std::vector<uint64_t>& att,
             std::vector<uint64_t>& acc, std::vector<uint8_t>* lowest_states,
             std::vector<uint8_t>* states) override
  {
    const int S = (int)n_walkers(), R = (int)restarts;
    cost.resize(S);
    lowest.resize(S);
    att.resize(S);
    acc.resize(S);
    if (!S) return;
    std::vector<double> low(R);
    cuda_check(cudaMemcpy(cost.data(), P.pop.cost, (size_t)S * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(low.data(), d_low, (size_t)R * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(att.data(), P.pop.attempts, (size_t)S * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(acc.data(), P.pop.accepts, (size_t)S * 8, cudaMemcpyDeviceToHost), "D2H");
    for (int i = 0; i < S; i++) lowest[i] = low[i / trotter];
    const int nw = P.pop.nw;
    if (lowest_states)
    {
      std::vector<uint32_t> w((size_t)R * nw);
      cuda_check(cudaMemcpy(w.data(), d_lspins, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      std::vector<uint8_t> per;
      Population::unpack(w, nw, model->N, R, per);
      lowest_states->resize((size_t)S * model->N);
      for (int i = 0; i < S; i++)
        std::copy(per.begin() + (size_t)(i / trotter) * model->N, per.begin() + (size_t)(i / trotter + 1) * model->N,
                  lowest_states->begin() + (size_t)i * model->N);
    }
    if (states)
    {
      std::vector<uint32_t> w((size_t)S * nw);
      cuda_check(cudaMemcpy(w.data(), P.pop.spins, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      Population::unpack(w, nw, model->N, S, *states);
    }
  }
};

// ---------------------------------------------------------------------------
// Parameter-free solvers with the linear search ("simulatedannealing-
// parameterfree.qiotoolkit", "paralleltempering-parameterfree.qiotoolkit":
// solver/parameter_free_solver.h:9-257 with solver/parameter_free_linear_
// solver.h and strategy/linear_search.cc; the adapters of
// solver/sa_parameter_free.h and solver/pt_parameter_free.h).  Repeated runs
// of the underlying solver: run j takes sweeps = the next sample point (and,
// for SA, restarts = min_num_restarts x the last sample point / sweeps);
// after each pass over the sample points they are stretched by the change
// factor when the last one gave the lowest cost and shrunk when the first
// did.  The temperature range runs from -ln(max_prob) / (max cost
// difference) to -ln(min_prob) / (min cost difference + factor x (max -
// min)).  The runs draw from one master stream that continues from run to
// run.  The search stops when `nonimprovement_limit` runs in a row find no
// lower cost, or at the time limit (default 5 s), checked between runs (the
// reference also hands the remaining time to the run itself).  The result is
// the lowest cost found and its state; the parameters shown are those of the
// run that found it (with equal costs, the cheaper run's).
// ---------------------------------------------------------------------------
class ParameterFreeSearch : public Solver
{
 public:
  double max_prob = 0.5, min_prob = 0.0001, adjust = 0.001, change = 1.5;
  double beta_start = 0.01, beta_stop = 10.0;
  std::vector<int> samples{10, 20, 30, 50};
  int nonimprovement_limit = 8;
  // linear search state (strategy/linear_search.cc)
  std::vector<int> points;
  std::vector<double> objs;
  int cur = -1, init_min = 0;
  Pcg master{0};
  // best so far (ParameterFreeSolver::update_best)
  bool has_best = false;
  double best = 0, best_exec = 0;
  int stable = 0;
  int64_t best_sweeps = 0, best_restarts = 0;
  std::vector<uint8_t> best_state;
  std::vector<std::array<double, 3>> trace;  // per run: sweeps, restarts, lowest cost
  uint64_t att_total = 0, acc_total = 0;
  std::string stop_reason;

  // one run of the underlying solver with `sweeps` sweeps (the last sample
  // point `back`), its master stream continuing `master`: the restarts used
  // (or replicas), its lowest cost and state, and its cost estimate
  virtual void one_run(int sweeps, int back, cudaStream_t st, int64_t& sl, int64_t& r, double& obj,
                       std::vector<uint8_t>& state, double& exec) = 0;
  virtual void render_params(int64_t sweeps, int64_t r) = 0;

  // the parameters shared by both adapters, the time limit, the estimates
  void configure_search(bool estimates = true)
  {
    if (!replay) fail(1, "parameter-free solvers run with \"rng_mode\": \"replay\"");
    if (number_of_solutions != 1) fail(1, "parameter-free solvers return one solution: `number_of_solutions` must be 1");
    Params p(params);
    auto prob = [&](const char* k, double def) {
      const double v = p.num(k, def);
      if (!(v > 0 && v <= 1)) fail(1, std::string("parameter `") + k + "`: must be in (0, 1], found " + json::number(v));
      return v;
    };
    max_prob = prob("max_prob", 0.5);
    min_prob = prob("min_prob", 0.0001);
    adjust = prob("min_cost_diff_adjustment_factor", 0.001);
    change = p.num("search_interval_change_factor", 1.5);
    if (const json::Value* v = p.get("initial_sweeps_sample_points"))
    {
      if (!v->is_array() || v->arr.size() <= 2)
        fail(1, "parameter `initial_sweeps_sample_points`: expected an array of more than 2 integers");
      samples.clear();
      for (const auto& x : v->arr)
      {
        if (!x.is_number() || x.num < 1) fail(1, "parameter `initial_sweeps_sample_points`: expected positive integers");
        samples.push_back((int)x.num);
      }
    }
    nonimprovement_limit = (int)p.integer("nonimprovement_limit", 8);
    if (nonimprovement_limit <= 0) fail(1, "parameter `nonimprovement_limit`: must be greater than 0");
    if (!has_time_limit)
    {
      has_time_limit = true;  // a time limit must be set (parameter_free_solver.h:56-61)
      time_limit = 5.0;
    }
    if (!model->empty() && estimates)
    {
      const double mx = estimate_max_cost_diff(*model), mn = estimate_min_cost_diff(*model);
      if (mx <= 0) fail(1, "max cost difference should be > 0, found :" + json::number(mx));
      if (mn <= 0) fail(1, "min cost difference should be > 0, found :" + json::number(mn));
      if (mn > mx)
        fail(1, "min cost difference should be <= max cost difference, found :" + json::number(mn) + " > " +
                    json::number(mx));
      beta_start = -std::log(max_prob) / mx;
      beta_stop = -std::log(min_prob) / (mn + adjust * (mx - mn));
    }
  }

  int64_t n_walkers() const override { return (model->empty() || !has_best) ? 0 : 1; }

  void init(cudaStream_t) override
  {
    initialized = true;
    ran = false;
    master = Pcg(seed);
    points = samples;  // LinearSearchOpt::set_ranges
    objs.assign(points.size(), std::numeric_limits<double>::max());
    init_min = points[0];
    cur = -1;
    has_best = false;
    stable = 0;
    trace.clear();
    att_total = acc_total = 0;
    best_state.clear();
    stop_reason.clear();
    last_step = 0;
    launches = 0;
  }

  // LinearSearchOpt::fit_sample_points: shrink when the first point gave the
  // lowest cost (unless already at the initial first point), stretch when
  // the last one did
  void fit_points()
  {
    const int lowest = (int)(std::min_element(objs.begin(), objs.end()) - objs.begin());
    if (lowest == 0)
    {
      if (points[0] > init_min)
        for (int& x : points) x = (int)((double)x / change);
    }
    else if (lowest == (int)points.size() - 1)
      for (int& x : points) x = (int)((double)x * change);
    objs.assign(points.size(), std::numeric_limits<double>::max());
  }

  void run(cudaStream_t st) override
  {
    if (!initialized) fail(1, "init() must be called before run()");
    ran = true;
    if (model->empty()) return;
    auto t0 = std::chrono::steady_clock::now();
    auto elapsed = [&] { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
    for (int64_t step = 0;; step++)
    {
      // LinearSearchOpt::recommend_parameter_values (two dimensions)
      cur++;
      if (cur >= (int)points.size())
      {
        cur = 0;
        fit_points();
      }
      if (elapsed() >= time_limit && has_best)
      {
        stop_reason = "time limit";
        break;
      }
      int64_t sl = 0, r = 0;
      double obj = 0, exec = 0;
      std::vector<uint8_t> state;
      one_run(points[cur], points.back(), st, sl, r, obj, state, exec);
      objs[cur] = obj;  // LinearSearchOpt::add_new_sample
      trace.push_back({(double)sl, (double)r, obj + model->const_cost});
      auto update_best = [&] {
        best = obj;
        best_exec = exec;
        best_sweeps = sl;
        best_restarts = r;
        best_state = state;
      };
      // ParameterFreeSolver::make_step, solver/parameter_free_solver.h:123-151
      bool done = false;
      if (has_best && std::abs(best - obj) < 10E-12)
      {
        stable++;
        if (exec < best_exec) update_best();
      }
      if (stable >= nonimprovement_limit)
      {
        done = true;
        stop_reason = "no improvement";
      }
      if (!has_best || best - obj > 10E-12)
      {
        stable = 0;
        has_best = true;
        update_best();
      }
      last_step = step + 1;
      if (done) break;
      if (has_cost_limit && best <= cost_limit)
      {
        stop_reason = "cost limit";
        break;
      }
    }
    render_params(best_sweeps, best_restarts);
    run_ms = elapsed() * 1e3;
  }

  // the lowest state and cost of a finished run (the first walker holding
  // the smallest lowest), with the run's counters added to the totals
  void take_lowest(Solver& w, double& obj, std::vector<uint8_t>& state,
                   const std::function<size_t(const std::vector<double>&)>& pick = nullptr)
  {
    std::vector<double> c, low;
    std::vector<uint64_t> at, ac;
    std::vector<uint8_t> ls;
    w.fetch(c, low, at, ac, &ls, nullptr);
    size_t b = 0;
    if (pick)
      b = pick(low);
    else
      for (size_t i = 1; i < low.size(); i++)
        if (low[i] < low[b]) b = i;
    obj = low[b];
    state.assign(ls.begin() + b * model->N, ls.begin() + (b + 1) * model->N);
    for (size_t i = 0; i < at.size(); i++)
    {
      att_total += at[i];
      acc_total += ac[i];
    }
    launches += w.launches;
  }

  void fetch(std::vector<double>& cost, std::vector<double>& lowest, std::vector<uint64_t>& att,
             std::vector<uint64_t>& acc, std::vector<uint8_t>* lowest_states,
             std::vector<uint8_t>* states) override
  {
    // one entry: the best state found over all runs
    cost.clear();
    lowest.clear();
    att.clear();
    acc.clear();
    if (model->empty() || !has_best) return;
    cost.push_back(best);
    lowest.push_back(best);
    att.push_back(att_total);
    acc.push_back(acc_total);
    if (lowest_states) *lowest_states = best_state;
    if (states) *states = best_state;
  }

  std::string extra_benchmark() override
  {
    std::string s = ",\"parameter_free\":{\"runs\":[";
    for (size_t i = 0; i < trace.size(); i++)
      s += (i ? "," : "") + std::string("{\"sweeps\":") + std::to_string((int64_t)trace[i][0]) +
           ",\"restarts\":" + std::to_string((int64_t)trace[i][1]) + ",\"lowest\":" + json::number(trace[i][2]) +
           "}";
    s += "],\"stop\":" + json::quote(stop_reason) + "}";
    return s;
  }
};

// SAParameterFree (solver/sa_parameter_free.h): restarts = min_num_restarts
// x last sample point / sweeps, a linear beta schedule over the run
class SAParameterFree : public ParameterFreeSearch
{
 public:
  std::unique_ptr<SimulatedAnnealing> w;
  int64_t min_restarts = 1;

  std::string target() const override { return "simulatedannealing-parameterfree.qiotoolkit"; }

  void configure(const json::Value& doc)
  {
    configure_common(*this, doc);
    Params p(params);
    min_restarts = p.integer("min_num_restarts", threads);
    if (min_restarts <= 0) fail(1, "parameter `min_num_restarts`: must be greater than 0");
    configure_search();
    w.reset(new SimulatedAnnealing());
    w->model = model;
    w->configure(doc);
    render_params(samples[0], min_restarts);
  }

  void render_params(int64_t sweeps, int64_t r) override
  {
    output_params.clear();
    output_params.push_back({"seed", std::to_string(seed)});
    output_params.push_back({"beta_start", json::number(beta_start)});
    output_params.push_back({"beta_stop", json::number(beta_stop)});
    output_params.push_back({"restarts", std::to_string(r)});
    output_params.push_back({"sweeps", std::to_string(sweeps)});
  }

  // SAParameterFree::update_parameters, solver/sa_parameter_free.h:120-137;
  // estimate_execution_cost 139-145 (up to the thread divisor)
  void one_run(int sweeps, int back, cudaStream_t st, int64_t& sl, int64_t& r, double& obj,
               std::vector<uint8_t>& state, double& exec) override
  {
    sl = std::max(sweeps, 2);
    r = (int64_t)((int)min_restarts * back / sweeps);
    if (r <= 0) fail(1, "parameter-free search reached a run with no restarts");
    w->retarget(sl, r, beta_start, beta_stop);
    w->ext_master = &master;
    w->init(st);
    w->run(st);
    take_lowest(*w, obj, state);
    exec = (double)sl * (double)r;
  }
};

// TabuParameterFree (solver/tabu_parameter_free.h): restarts as the SA
// adapter, each restart with its own tenure (determine_all_tenures_, 86-124);
// configure() already forked replica_rng_ from the master, so the runs'
// restarts fork from the master's second draw on.
class TabuParameterFree : public ParameterFreeSearch
{
 public:
  std::unique_ptr<TabuSearch> w;
  int64_t min_restarts = 1;

  std::string target() const override { return "tabu-parameterfree.qiotoolkit"; }

  void configure(const json::Value& doc)
  {
    configure_common(*this, doc);
    Params p(params);
    min_restarts = p.integer("min_num_restarts", threads);
    if (min_restarts <= 0) fail(1, "parameter `min_num_restarts`: must be greater than 0");
    configure_search(false);
    w.reset(new TabuSearch());
    w->model = model;
    w->configure(doc);
    render_params(samples[0], min_restarts);
  }

  void init(cudaStream_t st) override
  {
    ParameterFreeSearch::init(st);
    master.next();  // replica_rng_ = rng_->fork()
  }

  void render_params(int64_t sweeps, int64_t r) override
  {
    output_params.clear();
    output_params.push_back({"seed", std::to_string(seed)});
    output_params.push_back({"restarts", std::to_string(r)});
    output_params.push_back({"sweeps", std::to_string(sweeps)});
  }

  static std::vector<uint64_t> tenures(size_t n, size_t nv)
  {
    const size_t den = 4, cap = 20;
    const size_t opt = std::min(cap, nv / den);
    std::vector<uint64_t> out;
    size_t todo = n;
    while (todo > 0)
    {
      out.push_back(opt);
      todo--;
      if (todo > 0 && opt > cap / 2)
      {
        out.push_back(opt / 2);
        todo--;
      }
      if (todo > 0)
      {
        const size_t inc = std::max((nv - opt) / (todo * den), (size_t)1);
        size_t t = opt + inc;
        while (todo > 0 && t < nv)
        {
          out.push_back(t);
          todo--;
          t += inc;
        }
      }
    }
    return out;
  }

  // TabuParameterFree::update_parameters, solver/tabu_parameter_free.h:48-60
  void one_run(int sweeps, int back, cudaStream_t st, int64_t& sl, int64_t& r, double& obj,
               std::vector<uint8_t>& state, double& exec) override
  {
    sl = std::max(sweeps, 2);
    r = (int64_t)((int)min_restarts * back / sweeps);
    if (r <= 0) fail(1, "parameter-free search reached a run with no restarts");
    // num_variables = get_sweep_size() (solver/tabu_parameter_free.h:78-83)
    const size_t nv = model->kind == K_MAXSAT && !full_maxsat_sweep ? 1 : (size_t)model->N;
    w->retarget(sl, r, tenures((size_t)r, nv));
    w->ext_master = &master;
    w->init(st);
    w->run(st);
    take_lowest(*w, obj, state);
    exec = (double)sl * (double)r;
  }
};

// PTParameterFree (solver/pt_parameter_free.h): min_num_betas inverse
// temperatures from geometric ladders of 4, 9, 14, ... values between the
// two ends (determine_all_betas_, 155-173), the run length from the search
class PTParameterFree : public ParameterFreeSearch
{
 public:
  std::unique_ptr<ParallelTempering> w;
  int64_t min_betas = 1;
  std::vector<double> all_betas;
  static const int kIncrement = 5;  // tempering_size_increment_

  std::string target() const override { return "paralleltempering-parameterfree.qiotoolkit"; }

  void configure(const json::Value& doc)
  {
    configure_common(*this, doc);
    Params p(params);
    min_betas = p.integer("min_num_betas", threads);
    if (min_betas <= 0) fail(1, "parameter `min_num_betas`: must be greater than 0");
    configure_search();
    w.reset(new ParallelTempering());
    w->model = model;
    w->configure(doc);
    // determine_all_betas_
    all_betas.clear();
    Schedule g;
    g.type = 1;
    g.initial = beta_start;
    g.final_ = beta_stop;
    g.has_stop = true;
    for (int size = kIncrement; (int64_t)all_betas.size() < min_betas; size += kIncrement)
    {
      const int n = size - 1;
      g.stop_ = (double)(n - 1);
      for (int i = 0; i < n && (int64_t)all_betas.size() < min_betas; i++) all_betas.push_back(g.get_value((double)i));
    }
    render_params(samples[0], (int64_t)all_betas.size());
  }

  void render_params(int64_t sweeps, int64_t) override
  {
    Schedule list;
    list.type = 3;
    list.values = all_betas;
    output_params.clear();
    output_params.push_back({"seed", std::to_string(seed)});
    output_params.push_back({"all_betas", list.render()});
    output_params.push_back({"sweeps", std::to_string(sweeps)});
  }

  // update_parameters 124-137; estimate_execution_cost 139-144 (up to the
  // thread divisor)
  void one_run(int sweeps, int, cudaStream_t st, int64_t& sl, int64_t& r, double& obj,
               std::vector<uint8_t>& state, double& exec) override
  {
    sl = std::max(sweeps, 2);
    r = (int64_t)all_betas.size();
    w->retarget(sl, all_betas);
    w->ext_master = &master;
    w->init(st);
    w->run(st);
    master.state = w->master_after(st);
    take_lowest(*w, obj, state, [&](const std::vector<double>& low) { return w->time_first_lowest(low); });
    exec = (double)sl * (double)r;
  }
};

std::unique_ptr<Solver> make_solver(const HostModel* m, const std::string& target,
                                    const json::Value& doc)
{
  if (target == "simulatedannealing.qiotoolkit")
  {
    std::unique_ptr<SimulatedAnnealing> s(new SimulatedAnnealing());
    s->model = m;
    s->configure(doc);
    return std::unique_ptr<Solver>(s.release());
  }
  if (target == "paralleltempering.qiotoolkit")
  {
    std::unique_ptr<ParallelTempering> s(new ParallelTempering());
    s->model = m;
    s->configure(doc);
    return std::unique_ptr<Solver>(s.release());
  }
  if (target == "populationannealing.cpu") return make_pa_solver(m, doc);
  if (target == "substochasticmontecarlo.cpu") return make_ssmc_solver(m, doc);
  if (target == "populationannealing-parameterfree.cpu") return make_pa_pf_solver(m, doc);
  if (target == "substochasticmontecarlo-parameterfree.cpu") return make_ssmc_pf_solver(m, doc);
  if (target == "simulatedannealing-parameterfree.qiotoolkit")
  {
    std::unique_ptr<SAParameterFree> s(new SAParameterFree());
    s->model = m;
    s->configure(doc);
    return std::unique_ptr<Solver>(s.release());
  }
  if (target == "tabu-parameterfree.qiotoolkit")
  {
    std::unique_ptr<TabuParameterFree> s(new TabuParameterFree());
    s->model = m;
    s->configure(doc);
    return std::unique_ptr<Solver>(s.release());
  }
  if (target == "quantummontecarlo.qiotoolkit")
  {
    std::unique_ptr<QuantumMonteCarlo> s(new QuantumMonteCarlo());
    s->model = m;
    s->configure(doc);
    return std::unique_ptr<Solver>(s.release());
  }
  if (target == "tabu.qiotoolkit")
  {
    std::unique_ptr<TabuSearch> s(new TabuSearch());
    s->model = m;
    s->configure(doc);
    return std::unique_ptr<Solver>(s.release());
  }
  if (target == "paralleltempering-parameterfree.qiotoolkit")
  {
    std::unique_ptr<PTParameterFree> s(new PTParameterFree());
    s->model = m;
    s->configure(doc);
    return std::unique_ptr<Solver>(s.release());
  }
  fail(1, "Unknown solver: " + target);
}

// ---------------------------------------------------------------------------
// Batches: independent simulated-annealing solves of many models with the
// same params, in one population and one captured CUDA graph (the init
// kernels, and one sweep launch for all instances when every model runs on
// the lane kernel; one sweep launch per instance otherwise).  Instance i's
// walkers, streams and results equal a plain solve of model i with the same
// params: its walkers are numbered 0..restarts-1 for stream forks and
// counter keys, exactly as in its own solve.
// ---------------------------------------------------------------------------
class BatchView : public SimulatedAnnealing
{
 public:
  const Population* BP = nullptr;
  int first = 0;

  void fetch(std::vector<double>& cost, std::vector<double>& lowest,
             std::vector<uint64_t>& att, std::vector<uint64_t>& acc,
             std::vector<uint8_t>* lowest_states, std::vector<uint8_t>* states) override
  {
    const int R = (int)n_walkers();
    cost.resize(R);
    lowest.resize(R);
    att.resize(R);
    acc.resize(R);
    if (!R) return;
    const DevPop& p = BP->pop;
    cuda_check(cudaMemcpy(cost.data(), p.cost + first, R * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(lowest.data(), p.lowest + first, R * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(att.data(), p.attempts + first, R * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(acc.data(), p.accepts + first, R * 8, cudaMemcpyDeviceToHost), "D2H");
    std::vector<uint32_t> w((size_t)R * p.nw);
    if (lowest_states)
    {
      cuda_check(cudaMemcpy(w.data(), p.lspins + (size_t)first * p.nw, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      Population::unpack(w, p.nw, model->N, R, *lowest_states);
    }
    if (states)
    {
      cuda_check(cudaMemcpy(w.data(), p.spins + (size_t)first * p.nw, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      Population::unpack(w, p.nw, model->N, R, *states);
    }
  }
};

static DevPop pop_slice(const DevPop& p, int first, int count)
{
  DevPop v = p;
  v.n = count;
  v.spins = p.spins + (size_t)first * p.nw;
  v.tstate = p.tstate + (size_t)first * p.mp;
  v.cost = p.cost + first;
  v.lowest = p.lowest + first;
  v.lspins = p.lspins + (size_t)first * p.nw;
  v.attempts = p.attempts + first;
  v.accepts = p.accepts + first;
  v.step_att = p.step_att + first;
  v.step_acc = p.step_acc + first;
  v.windows = p.windows ? p.windows + first : nullptr;
  return v;
}

class SABatch : public Batch
{
 public:
  std::vector<const HostModel*> models;
  std::vector<std::unique_ptr<BatchView>> views;
  int R = 0, W = 0;
  int64_t steps = 0;
  bool replay = true, lanes = false, autotune = true, use_graph = true, smem = true;
  bool full_sweep = false;  // maxsat_full_sweep: every MaxSat variable in a sweep
  int wpb_param = 0;         // warps_per_block: the plan without autotune (0: spread)
  uint32_t seed = 0;
  int kernel = 0;
  Population P;
  LaneRunner L;
  DevBuf rng0;
  bool prepared = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t graph_stream = nullptr;
  int plan_wpb = 0, plan_smem = 1;
  int64_t graph_launches = 0;
  // the population's layout: instances grouped by kernel flavour and
  // coefficient kind, longest first within a group (largest N first), so
  // that the warps of the lane kernel hold instances of equal size and the
  // longest solves start first; instance i's walkers are block pos[i]
  std::vector<int> order, pos;
  // windowed-kernel batches: one persistent launch per group of walkers
  // [first, last) that share a flavour and coefficient kind, fed by a device
  // queue in population order (so longest first)
  bool queued = false;
  struct Group
  {
    int first, last;
    const HostModel* model;  // any member (flavour and coefficient kind)
    int max_block_inc;       // the members' largest 32-variable block
  };
  std::vector<Group> groups;
  DevBuf qbuf;  // DevModel per instance, model_of, local_of, one queue counter per group
  const DevModel* d_models = nullptr;
  int* d_model_of = nullptr;
  int* d_local_of = nullptr;
  int* d_queue = nullptr;
  bool profile = false;  // events around the sweep launches (runs without a graph)
  double sweep_ms = 0;

  ~SABatch() override
  {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }

  void configure(const std::vector<const HostModel*>& ms, const json::Value& doc)
  {
    if (ms.empty()) fail(1, "a batch needs at least one model");
    models = ms;
    for (size_t i = 0; i < ms.size(); i++)
    {
      if (!ms[i]) fail(1, "batch model " + std::to_string(i) + " is null");
      if (ms[i]->empty()) fail(1, "batch model " + std::to_string(i) + " has no variables");
      std::unique_ptr<BatchView> v(new BatchView());
      v->model = ms[i];
      v->configure(doc);
      if (v->has_cost_limit || v->has_time_limit)
        fail(1, "batches run every instance for its full sweep count: `cost_limit` and `timeout` are not supported");
      views.push_back(std::move(v));
    }
    const BatchView& v0 = *views[0];
    R = (int)v0.restarts;
    if ((int64_t)R * (int64_t)ms.size() > (1 << 26)) fail(1, "batch too large");
    W = R * (int)ms.size();
    steps = v0.step_limit;
    replay = v0.replay;
    seed = v0.seed;
    kernel = v0.kernel;
    smem = v0.smem_state;
    full_sweep = v0.full_maxsat_sweep;
    wpb_param = v0.warps_per_block;
    Params p(doc["params"]);
    autotune = p.boolean("autotune", true);
    use_graph = p.boolean("graph", true);
    profile = v0.profile && !use_graph;
    bool eligible = true;
    for (auto* m : ms)
      eligible = eligible && lanes_eligible(*m) && m->int_mode == ms[0]->int_mode;
    if (kernel == 3) fail(1, "parameter `kernel`: \"levels\" is not available for batches");
    if (kernel == 2 && !eligible)
      fail(1, "parameter `kernel`: \"lanes\" needs Ising models whose terms have at most two members "
              "and the same coefficient kind");
    lanes = eligible && kernel != 1;
  }

  int n_instances() const override { return (int)models.size(); }

  void prepare(cudaStream_t st)
  {
    ensure_device();
    int64_t N = 0, M = 0;
    for (auto* m : models)
    {
      N = std::max(N, m->N);
      const bool plain = m->flavor == F_PLAIN_ISING || m->flavor == F_PLAIN_PUBO;
      M = std::max(M, plain ? (int64_t)0 : m->M);
    }
    P.alloc_sizes(N, M, W, W, false, std::max<int64_t>(1, steps));
    // every model on the device before any capture (uploads allocate)
    for (auto* m : models) m->device_view(full_sweep);
    order.resize(models.size());
    for (size_t i = 0; i < models.size(); i++) order[i] = (int)i;
    auto kind_of = [&](int x) { return models[x]->flavor * 2 + (models[x]->int_mode ? 1 : 0); };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      if (kind_of(x) != kind_of(y)) return kind_of(x) < kind_of(y);
      return models[x]->N > models[y]->N;
    });
    pos.resize(models.size());
    for (size_t k = 0; k < order.size(); k++) pos[order[k]] = (int)k;
    for (size_t i = 0; i < views.size(); i++)
    {
      views[i]->BP = &P;
      views[i]->first = pos[i] * R;
    }
    // stream forks of each instance: rngs_[i] = rng_->fork() in index order
    // (solver/simulated_annealing.h:53-56), the same for every instance
    std::vector<uint64_t> rs(W);
    Pcg master(seed);
    for (int i = 0; i < R; i++) rs[i] = Pcg(master.next()).state;
    for (int k = 1; k < (int)models.size(); k++) std::copy(rs.begin(), rs.begin() + R, rs.begin() + (size_t)k * R);
    rng0 = DevBuf((size_t)W * 8);
    cuda_check(cudaMemcpy(rng0.ptr, rs.data(), (size_t)W * 8, cudaMemcpyHostToDevice), "H2D rng");
    const auto& betas = views[0]->betas;
    if (steps > 0)
      cuda_check(cudaMemcpy(P.beta, betas.data(), betas.size() * 8, cudaMemcpyHostToDevice), "H2D beta");
    if (lanes)
    {
      std::vector<DevModel> dm;
      for (auto* m : models) dm.push_back(m->device_view(full_sweep));
      std::vector<int> model_of(W), local_of(W);
      for (int r = 0; r < W; r++)
      {
        model_of[r] = order[r / R];
        local_of[r] = r % R;
      }
      L.setup(dm, model_of, W, local_of, smem);
    }
    else
      plan_queue();
    (void)st;
    prepared = true;
  }

  // The windowed kernel's queue plan: groups of one flavour and coefficient
  // kind whose walker state fits a warp's shared memory; otherwise (or with
  // `smem_state` off) one launch per instance.
  void plan_queue()
  {
    groups.clear();
    queued = smem;
    for (size_t k = 0; k < order.size() && queued; k++)
    {
      const HostModel* m = models[order[k]];
      const int first = (int)k * R;
      const int mb = m->device_view(full_sweep).max_block_inc;
      if (groups.empty() || groups.back().model->flavor != m->flavor ||
          groups.back().model->int_mode != m->int_mode)
        groups.push_back({first, first + R, m, mb});
      else
      {
        groups.back().last = first + R;
        groups.back().max_block_inc = std::max(groups.back().max_block_inc, mb);
      }
      SweepArgs a{};
      a.m = m->device_view(full_sweep);
      a.m.max_block_inc = groups.back().max_block_inc;
      a.p = P.pop;
      queued = sweep_state_fits(a);
    }
    if (!queued)
    {
      groups.clear();
      return;
    }
    const size_t n = models.size();
    const size_t o_mo = (n * sizeof(DevModel) + 255) & ~(size_t)255;
    const size_t o_lo = o_mo + (((size_t)W * 4 + 255) & ~(size_t)255);
    const size_t o_q = o_lo + (((size_t)W * 4 + 255) & ~(size_t)255);
    qbuf = DevBuf(o_q + groups.size() * 4);
    std::vector<DevModel> dm(n);
    for (size_t i = 0; i < n; i++) dm[i] = models[i]->device_view(full_sweep);
    std::vector<int> model_of(W), local_of(W);
    for (int r = 0; r < W; r++)
    {
      model_of[r] = order[r / R];
      local_of[r] = r % R;
    }
    char* b = (char*)qbuf.ptr;
    cuda_check(cudaMemcpy(b, dm.data(), n * sizeof(DevModel), cudaMemcpyHostToDevice), "H2D models");
    cuda_check(cudaMemcpy(b + o_mo, model_of.data(), (size_t)W * 4, cudaMemcpyHostToDevice), "H2D");
    cuda_check(cudaMemcpy(b + o_lo, local_of.data(), (size_t)W * 4, cudaMemcpyHostToDevice), "H2D");
    d_models = (const DevModel*)b;
    d_model_of = (int*)(b + o_mo);
    d_local_of = (int*)(b + o_lo);
    d_queue = (int*)(b + o_q);
  }

  // one group's persistent sweep launch (its queue reset first)
  void launch_group(size_t g, int64_t sweeps, int wpb, cudaStream_t st)
  {
    const Group& G = groups[g];
    cuda_check(cudaMemsetAsync(d_queue + g, 0, 4, st), "memset");
    SweepArgs a{};
    a.m = G.model->device_view(full_sweep);
    a.p = pop_slice(P.pop, G.first, G.last - G.first);
    a.n_streams = G.last - G.first;
    a.n_walkers = G.last - G.first;
    a.beta = P.beta;
    a.bs_w = 0;
    a.bs_s = 1;
    a.replay = replay ? 1 : 0;
    a.rng = P.rng + G.first;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = (long long)1 << 40;
    a.smem_state = 1;
    a.err = device_error_flag();
    a.sweep_base = 0;
    a.n_sweeps = (int)sweeps;
    a.models = d_models;
    a.model_of = d_model_of + G.first;
    a.local_of = d_local_of + G.first;
    a.queue = d_queue + g;
    a.m.max_block_inc = G.max_block_inc;  // tiles sized for the group's largest block
    cuda_check(launch_sweep(a, st, wpb), "sweep kernel");
  }

  LwArgs lane_args() const
  {
    LwArgs a = L.a;
    a.p = P.pop;
    a.slot_of = nullptr;
    a.beta = P.beta;
    a.bs_w = 0;
    a.bs_s = 1;
    a.replay = replay ? 1 : 0;
    a.int_mode = models[0]->int_mode ? 1 : 0;
    a.rng = P.rng;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = (long long)1 << 40;
    return a;
  }

  // the whole solve, enqueued on st: streams reset, init, sweeps
  void enqueue(cudaStream_t st, int64_t n_sweeps, int& n_launch)
  {
    n_launch = 0;
    cuda_check(cudaMemcpyAsync(P.rng, rng0.ptr, (size_t)W * 8, cudaMemcpyDeviceToDevice, st), "D2D rng");
    for (size_t i = 0; i < models.size(); i++)
    {
      InitArgs a{};
      a.m = models[i]->device_view(full_sweep);
      a.p = pop_slice(P.pop, pos[i] * R, R);
      a.n_walkers = R;
      // a MaxSat walker draws its state one uniform() per variable
      // (model/max_sat.h:144-150)
      const bool ms = models[i]->kind == K_MAXSAT;
      a.replay = replay ? (ms ? 2 : 1) : (ms ? 3 : 0);
      a.rng = P.rng + (size_t)pos[i] * R;
      a.seed = seed;
      a.key_base = 0;
      a.key_div = (long long)1 << 40;
      a.skip_terms = (lanes && n_sweeps > 0) ? 1 : 0;  // the lane store rebuilds them
      cuda_check(launch_init(a, st), "init kernel");
      n_launch++;
    }
    if (n_sweeps <= 0) return;
    if (lanes)
    {
      LwArgs la = lane_args();
      la.sweep_base = 0;
      la.n_sweeps = (int)n_sweeps;
      cuda_check(launch_lw_load(la, L.max_words, st), "lane load");
      std::unique_ptr<EventTimer> t(profile ? new EventTimer(st) : nullptr);
      if (!plan_smem) la.smem_words = 0;
      cuda_check(launch_lw_sweep(la, plan_wpb, st), "lane sweep kernel");
      if (t) sweep_ms = t->stop();
      cuda_check(launch_lw_store(la, L.max_words, L.max_terms, st), "lane store");
      n_launch += 3;
    }
    else if (queued)
    {
      std::unique_ptr<EventTimer> t(profile ? new EventTimer(st) : nullptr);
      for (size_t g = 0; g < groups.size(); g++)
      {
        launch_group(g, n_sweeps, plan_wpb > 0 ? plan_wpb : 4, st);
        n_launch++;
      }
      if (t) sweep_ms = t->stop();
    }
    else
    {
      std::unique_ptr<EventTimer> t(profile ? new EventTimer(st) : nullptr);
      for (size_t i = 0; i < models.size(); i++)
      {
        SweepArgs a{};
        a.m = models[i]->device_view(full_sweep);
        a.p = pop_slice(P.pop, pos[i] * R, R);
        a.n_streams = R;
        a.n_walkers = R;
        a.beta = P.beta;
        a.bs_w = 0;
        a.bs_s = 1;
        a.replay = replay ? 1 : 0;
        a.rng = P.rng + (size_t)pos[i] * R;
        a.seed = seed;
        a.key_base = 0;
        a.key_div = (long long)1 << 40;
        a.smem_state = plan_smem;
        a.err = device_error_flag();
        a.sweep_base = 0;
        a.n_sweeps = (int)n_sweeps;
        cuda_check(launch_sweep(a, st, pick_wpb(plan_wpb, R)), "sweep kernel");
        n_launch++;
      }
      if (t) sweep_ms = t->stop();
    }
  }

  // Launch plan, timed on a short trial of the batch itself: for the lane
  // kernel warps per block and shared-memory groups; for the windowed
  // kernel's queues warps per block (walkers per block: 1, 2, 4 or 8).
  void tune(cudaStream_t st)
  {
    plan_smem = smem ? 1 : 0;
    plan_wpb = wpb_param;
    if (!autotune || steps <= 0) return;
    const int64_t trial = std::max<int64_t>(1, std::min<int64_t>(steps, (steps + 99) / 100));
    if (queued)
    {
      double best = 1e300;
      int best_wpb = 4;
      for (int wpb : {1, 2, 4, 8})
      {
        int n;
        enqueue(st, 0, n);
        EventTimer t(st);
        for (size_t g = 0; g < groups.size(); g++) launch_group(g, trial, wpb, st);
        const double ms = t.stop();
        if (ms < best)
        {
          best = ms;
          best_wpb = wpb;
        }
      }
      plan_wpb = best_wpb;
      return;
    }
    if (!lanes) return;
    double best = 1e300;
    int best_wpb = 0, best_sm = plan_smem;
    for (int sm = L.a.smem_words > 0 ? 1 : 0; sm >= 0; sm--)
      for (int wpb : {1, 2, 4})
      {
        int n;
        plan_wpb = wpb;
        plan_smem = sm;
        enqueue(st, 0, n);
        LwArgs la = lane_args();
        la.sweep_base = 0;
        la.n_sweeps = (int)trial;
        if (!sm) la.smem_words = 0;
        cuda_check(launch_lw_load(la, L.max_words, st), "lane load");
        EventTimer t(st);
        cuda_check(launch_lw_sweep(la, wpb, st), "lane sweep kernel");
        double ms = t.stop();
        if (ms < best)
        {
          best = ms;
          best_wpb = wpb;
          best_sm = sm;
        }
      }
    plan_wpb = best_wpb;
    plan_smem = best_sm;
  }

  void run(cudaStream_t st) override
  {
    if (!prepared)
    {
      prepare(st);
      tune(st);
    }
    EventTimer total(st);
    int n = 0;
    if (use_graph)
    {
      if (!exec || graph_stream != st)
      {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        // a private stream for the capture (the caller's may be the legacy
        // default stream, which cannot be captured)
        cudaStream_t cs;
        cuda_check(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate");
        cuda_check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        try
        {
          enqueue(cs, steps, n);
        }
        catch (...)
        {
          cudaGraph_t g;
          cudaStreamEndCapture(cs, &g);
          if (g) cudaGraphDestroy(g);
          cudaStreamDestroy(cs);
          throw;
        }
        cuda_check(cudaStreamEndCapture(cs, &graph), "cudaStreamEndCapture");
        cudaStreamDestroy(cs);
        cuda_check(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
        graph_stream = st;
        graph_launches = n;
      }
      cuda_check(cudaGraphLaunch(exec, st), "cudaGraphLaunch");
      n = (int)graph_launches;
    }
    else
      enqueue(st, steps, n);
    const double ms = total.stop();
    check_device_error(st);
    for (auto& v : views)
    {
      v->initialized = v->ran = true;
      v->last_step = steps;
      v->run_ms = ms;
      v->launches = (uint64_t)n;
    }
    stats_.run_ms = ms;
    stats_.launches = n;
    stats_.kernel = lanes ? 2 : 1;
    stats_.warps_per_block = plan_wpb;
    stats_.smem = plan_smem;
    stats_.graph = use_graph ? 1 : 0;
    stats_.walkers = W;
    stats_.device_bytes = (int64_t)(P.buf.bytes + L.bytes() + rng0.bytes + qbuf.bytes);
    stats_.sweep_kernel_ms = profile ? sweep_ms : 0.0;
  }

  std::string result_json(int i) override
  {
    if (i < 0 || i >= (int)views.size()) fail(1, "instance " + std::to_string(i) + " out of range");
    if (!views[i]->ran) fail(1, "run() must be called before reading results");
    return views[i]->result_json();
  }

  void lowest(double* out) override
  {
    std::vector<double> low(W);
    if (!views[0]->ran) fail(1, "run() must be called before reading results");
    cuda_check(cudaMemcpy(low.data(), P.pop.lowest, (size_t)W * 8, cudaMemcpyDeviceToHost), "D2H");
    for (size_t i = 0; i < models.size(); i++)
    {
      const size_t f = (size_t)pos[i] * R;
      double b = low[f];
      for (int k = 1; k < R; k++) b = std::min(b, low[f + k]);
      out[i] = b + models[i]->const_cost;
    }
  }
};

std::unique_ptr<Batch> make_batch(const std::vector<const HostModel*>& models, const std::string& target,
                                  const json::Value& doc)
{
  if (target != "simulatedannealing.qiotoolkit")
    fail(1, "batches run \"simulatedannealing.qiotoolkit\"; found " + target);
  std::unique_ptr<SABatch> b(new SABatch());
  b->configure(models, doc);
  return std::unique_ptr<Batch>(b.release());
}

// ---------------------------------------------------------------------------
// Results: populate_solutions / get_solutions (solver/model_solver.h:111-150,
// 261-308): walkers ordered by lowest cost (ties by walker index), the first
// number_of_solutions of them returned, costs include the constant terms.
// ---------------------------------------------------------------------------
static std::string render_config(const HostModel& m, const uint8_t* s)
{
  std::string o = "{";
  for (int64_t v = 0; v < m.N; v++)
  {
    int val;
    if (m.kind == K_ISING || m.kind == K_ISING_PLAIN) val = s[v] ? -1 : 1;
    else if (m.kind == K_MAXSAT) val = s[v] ? 1 : 0;
    else val = s[v] ? 0 : 1;
    o += (v ? "," : "") + json::quote(std::to_string(m.names[v])) + ":" + std::to_string(val);
  }
  for (size_t i = 0; i < m.free_vars.size(); i++)
    o += ((m.N || i) ? "," : "") + json::quote(std::to_string(m.free_vars[i])) + ":1";
  return o + "}";
}

void Solver::best(double& cost, std::vector<uint8_t>& state)
{
  std::vector<double> c, low;
  std::vector<uint64_t> at, ac;
  std::vector<uint8_t> ls;
  fetch(c, low, at, ac, &ls, nullptr);
  if (low.empty())
  {
    cost = model->const_cost;
    state.clear();
    return;
  }
  const size_t b = best_index(low);
  cost = low[b] + model->const_cost;
  state.assign(ls.begin() + b * model->N, ls.begin() + (b + 1) * model->N);
  double hc;
  std::vector<uint8_t> hs;
  if (historical_lowest(hc, hs) && hc < low[b])
  {
    cost = hc + model->const_cost;
    state = hs;
  }
}

std::string Solver::result_json()
{
  std::vector<double> c, low;
  std::vector<uint64_t> at, ac;
  std::vector<uint8_t> ls;
  fetch(c, low, at, ac, &ls, nullptr);
  uint64_t attempts = 0, accepts = 0;
  for (size_t i = 0; i < at.size(); i++)
  {
    attempts += at[i];
    accepts += ac[i];
  }
  std::string sol = "{\"version\":\"1.0\"";
  if (!low.empty())
  {
    const size_t stride = solution_stride();
    std::vector<size_t> idx;
    for (size_t i = 0; i < low.size(); i += stride) idx.push_back(i);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return low[a] < low[b]; });
    // the solver's lowest first (ModelSolver::populate_solutions keeps it
    // as the result's cost and configuration)
    const size_t b0 = best_index(low);
    idx.erase(std::find(idx.begin(), idx.end(), b0));
    idx.insert(idx.begin(), b0);
    size_t k = std::min((size_t)number_of_solutions, idx.size());
    // population solvers may have lost their historical lowest
    // (solver/model_solver.h:280-290): it then comes first
    std::vector<std::pair<double, const uint8_t*>> list;
    double hc;
    std::vector<uint8_t> hs;
    if (historical_lowest(hc, hs) && hc < low[idx[0]])
    {
      list.push_back({hc, hs.data()});
      k--;
    }
    for (size_t j = 0; j < k; j++) list.push_back({low[idx[j]], ls.data() + idx[j] * model->N});
    sol += ",\"cost\":" + json::number(list[0].first + model->const_cost);
    sol += ",\"configuration\":" + render_config(*model, list[0].second);
    sol += ",\"solutions\":[";
    for (size_t j = 0; j < list.size(); j++)
      sol += (j ? "," : "") + std::string("{\"cost\":") + json::number(list[j].first + model->const_cost) +
             ",\"configuration\":" + render_config(*model, list[j].second) + "}";
    sol += "]";
  }
  else
    sol += ",\"cost\":" + json::number(model->const_cost);
  sol += ",\"parameters\":{";
  for (size_t i = 0; i < output_params.size(); i++)
    sol += (i ? "," : "") + json::quote(output_params[i].first) + ":" + output_params[i].second;
  sol += "}}";
  // Solver::get_benchmark (solver/solver.h:78-145): evaluation counts, the
  // graph size properties of graph models under the keys of utils/config.h
  // (-1 localities otherwise, as MaxSat has no graph properties), and the
  // counters / solver / model extensions
  const bool graph = model->kind != K_MAXSAT;
  std::string counters = "{\"accepted_transitions\":" + std::to_string(accepts) +
                         ",\"difference_evaluations\":" + std::to_string(attempts) +
                         ",\"function_evaluations\":" + std::to_string(n_walkers()) + "}";
  std::string size;
  if (graph)
    size = "{\"nodes\":" + std::to_string(model->N) + ",\"edges\":" + std::to_string(model->M) +
           ",\"locality\":" + std::to_string(model->max_loc) +
           ",\"min_locality\":" + std::to_string(model->min_loc) +
           ",\"avg_locality\":" + json::number(model->M ? (double)model->total_loc / (double)model->M : 0.0) +
           ",\"sum_coefficient_degrees_total\":" + std::to_string(model->total_loc) +
           ",\"accumulated_dependent_vars\":" + std::to_string(model->accum_dep) +
           ",\"max_coupling_magnitude\":" + json::number(model->max_coupling) +
           ",\"min_coupling_magnitude\":" + json::number(model->min_coupling) + "}";
  std::string bench = "{\"cost_function_evaluation_count\":" + std::to_string(n_walkers()) +
                      ",\"cost_difference_evaluation_count\":" + std::to_string(attempts);
  if (graph)
  {
    // the size entries, copied to the top level as solver.h does
    bench += ",\"num_variables\":" + std::to_string(model->N) + ",\"num_terms\":" + std::to_string(model->M) +
             "," + size.substr(size.find("\"locality\""), size.size() - size.find("\"locality\"") - 1);
  }
  else
    bench += ",\"locality\":-1,\"min_locality\":-1,\"avg_locality\":-1";
  bench += ",\"extensions\":[{\"name\":\"counters\",\"value\":" + counters +
           "},{\"name\":\"solver\",\"value\":{\"last_step\":" + std::to_string(last_step) +
           (ran ? "" : ",\"not_run\":true") + "}},{\"name\":\"model\",\"value\":" +
           (graph ? "{\"graph\":{\"size\":" + size + "}}" : std::string("{}")) + "}]" +
           ",\"gb300\":{\"run_ms\":" + json::number(run_ms) +
           ",\"kernel_launches\":" + std::to_string(launches) +
           ",\"rng_mode\":" + json::quote(replay ? "replay" : "counter") + "}" + extra_benchmark() +
           runner_benchmark + "}";
  return "{\"benchmark\":" + bench + ",\"solutions\":" + sol + "}";
}
}  // namespace qio
