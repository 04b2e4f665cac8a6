// pa.cc -- population annealing driver (solver/population_annealing.h).
//
// Sweeps and replica copies run on the device.  The O(R) bookkeeping between
// sweeps -- cost statistics, Boltzmann weights, resampling counts, family
// census, restart test -- runs on the host in the reference's arithmetic
// (sequential sums, the C library's exp, libstdc++'s Poisson and uniform
// distributions on the master PCG stream), so that trajectories replay the
// reference exactly.  Only R doubles and R ints cross PCIe per step; the
// O(R * N) state traffic stays in HBM.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <numeric>
#include <random>

#include "bayes.h"
#include "host.h"

namespace qio
{
uint64_t host_counter_key(uint32_t seed, uint64_t stream);
void configure_common_public(Solver& s, const json::Value& doc);
uint64_t sum_windows(const DevPop& p, int n);
int pick_wpb(int requested, int streams);

namespace
{
const uint64_t kMult = 6364136223846793005ULL;
const uint64_t kInc = 1442695040888963407ULL;

// pcg32 as a UniformRandomBitGenerator for the libstdc++ distributions the
// reference uses (utils/random_generator.cc:47-58).
struct PcgEngine
{
  using result_type = uint32_t;
  static constexpr result_type min() { return 0; }
  static constexpr result_type max() { return 0xffffffffu; }
  uint64_t state = 0;
  explicit PcgEngine(uint32_t s) { state = ((uint64_t)s + kInc) * kMult + kInc; }
  result_type operator()()
  {
    uint64_t old = state;
    state = old * kMult + kInc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  double uniform()
  {
    std::uniform_real_distribution<double> u(0.0, 1.0);
    return u(*this);
  }
  uint32_t poisson(double mean)
  {
    std::poisson_distribution<> p(mean);
    return (uint32_t)p(*this);
  }
};

// LCG jump: state after k further steps.
uint64_t jump(uint64_t s, uint64_t k)
{
  uint64_t A = kMult, C = kInc;
  while (k)
  {
    if (k & 1) s = A * s + C;
    C = A * C + C;
    A = A * A;
    k >>= 1;
  }
  return s;
}

// utils::RandomSelector (utils/random_selector.cc:14-125) for the
// constant-population residual draw.
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
  double get_weight(size_t position) const { return cumulative(position + 1) - cumulative(position); }
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
  size_t select_and_remove(double u)
  {
    if (ids.empty()) fail(6, "Random selector is empty.");
    size_t position = 0;
    if (ids.size() > 1)
    {
      double w = u * total;
      for (size_t k = weight.size() - 1; k > 0; k >>= 1)
        if (w >= weight[position + k])
        {
          position += k;
          w -= weight[position];
        }
      if (position >= ids.size()) position = ids.size() - 1;
    }
    size_t id = ids[position];
    ids[position] = ids.back();
    ids.pop_back();
    double before = get_weight(position);
    double after = get_weight(ids.size());
    total -= before;
    add_weight(position, after - before);
    add_weight(ids.size(), -after);
    return id;
  }
};

struct Pool
{
  DevBuf buf;
  DevPop pop{};
  int cap = 0;
  void alloc(const HostModel& m, int capacity)
  {
    cap = capacity;
    int nw = (int)(((m.N + 31) / 32 + 3) & ~3LL);
    int mp = (int)((m.M + 15) & ~15LL);
    if (m.flavor == F_PLAIN_ISING || m.flavor == F_PLAIN_PUBO) mp = 16;
    size_t S = (size_t)capacity, off = 0;
    auto take = [&](size_t b) { size_t o = off; off = (off + b + 255) & ~(size_t)255; return o; };
    size_t o_sp = take(S * nw * 4), o_ts = take(S * mp), o_c = take(S * 8), o_l = take(S * 8),
           o_ls = take(S * nw * 4), o_at = take(S * 8), o_ac = take(S * 8), o_sa = take(S * 8),
           o_sc = take(S * 8), o_wi = take(S * 8);
    buf = DevBuf(off);
    char* b = (char*)buf.ptr;
    pop.n = capacity;
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
  }
};
}  // namespace

class PopulationAnnealing : public Solver
{
 public:
  double alpha = 2.0;
  size_t target_pop = 0;
  size_t target_initial = 0;
  bool constant_population = false;
  std::string strategy = "linear_schedule";
  Schedule beta;
  double beta_start = 0;
  int64_t spr = 1;
  bool exp_repop = false;
  int T = 1;  // emulated OpenMP threads = replay streams

  Pool pools[2];
  int cur = 0;
  DevBuf aux;  // streams (T), per-walker init streams, src_of, beta
  uint64_t* d_streams = nullptr;
  uint64_t* d_init_rng = nullptr;
  int* d_src = nullptr;
  double* d_beta = nullptr;
  int aux_cap = 0;

  PcgEngine master{0};
  PcgEngine* ext_master = nullptr;  // repeated runs: the master stream continues from run to run
  uint64_t swept = 0;  // attempts made since init (walkers swept x sweeps x sweep size)
  std::vector<uint64_t> streams;  // host mirror of the replay streams
  std::vector<size_t> family;
  std::vector<double> wbeta;
  size_t R = 0;
  double cur_beta = 0;
  uint64_t restart_base = 0, epoch = 0;
  bool has_low = false;
  double low_cost = 0;
  std::vector<uint32_t> low_words;
  std::vector<double> trace_beta;
  std::vector<int64_t> trace_pop;

  bool streams_on_device = false;

  // multinomial device resampling (counter streams) and lane-kernel sweeps
  bool multinomial = false;
  bool lanes = false, levels = false;
  LevelLog lvlog;  // level kernel sweep log
  DevBuf dres;  // prefix sums, two family arrays, census counts, scalars
  unsigned long long* d_prefix = nullptr;
  int* d_family[2] = {nullptr, nullptr};
  unsigned int* d_counts = nullptr;
  PaScalars* d_scal = nullptr;
  int res_cap = 0, fcur = 0;
  LaneRunner L;
  int lane_walkers = 0;

  std::string target_name() const { return "populationannealing.cpu"; }

  bool historical_lowest(double& c, std::vector<uint8_t>& st) override
  {
    if (!has_low) return false;
    c = low_cost;
    st.assign(model->N, 0);
    for (int64_t v = 0; v < model->N; v++) st[v] = (low_words[v / 32] >> (v % 32)) & 1u;
    return true;
  }
  std::string target() const override { return target_name(); }
  uint64_t total_windows() override { return sum_windows(pools[cur].pop, (int)n_walkers()); }

  void configure(const json::Value& doc)
  {
    configure_common_pa(doc);
    if (kernel == 3 && !model->empty()) levels_for(*this, *model);  // validates the request
  }

  void configure_common_pa(const json::Value& doc);

  int64_t n_walkers() const override { return model->empty() ? 0 : (int64_t)R; }

  int draws_per_init() const
  {
    return model->kind == K_MAXSAT ? (int)(2 * model->N) : (int)((model->N + 31) / 32);
  }

  void ensure_aux(int capacity)
  {
    if (capacity <= aux_cap) return;
    size_t off = 0;
    auto take = [&](size_t b) { size_t o = off; off = (off + b + 255) & ~(size_t)255; return o; };
    size_t o_s = take((size_t)T * 8), o_i = take((size_t)capacity * 8), o_src = take((size_t)capacity * 4),
           o_b = take((size_t)capacity * 8);
    DevBuf nb(off);
    // carry the replay streams over
    if (aux.ptr) cuda_check(cudaMemcpy((char*)nb.ptr + o_s, d_streams, (size_t)T * 8, cudaMemcpyDeviceToDevice), "D2D");
    aux = std::move(nb);
    char* b = (char*)aux.ptr;
    d_streams = (uint64_t*)(b + o_s);
    d_init_rng = (uint64_t*)(b + o_i);
    d_src = (int*)(b + o_src);
    d_beta = (double*)(b + o_b);
    aux_cap = capacity;
    if (multinomial) ensure_res(capacity);
  }

  void ensure_res(int capacity)
  {
    if (capacity <= res_cap) return;
    size_t off = 0;
    auto take = [&](size_t b) { size_t o = off; off = (off + b + 255) & ~(size_t)255; return o; };
    size_t o_p = take((size_t)capacity * 8), o_f0 = take((size_t)capacity * 4), o_f1 = take((size_t)capacity * 4),
           o_c = take((size_t)capacity * 4), o_s = take(sizeof(PaScalars));
    DevBuf nb(off);
    char* b = (char*)nb.ptr;
    int* nf0 = (int*)(b + o_f0);
    if (res_cap > 0 && R > 0)  // carry the families over
      cuda_check(cudaMemcpy(nf0, d_family[fcur], R * 4, cudaMemcpyDeviceToDevice), "D2D");
    dres = std::move(nb);
    d_prefix = (unsigned long long*)(b + o_p);
    d_family[0] = nf0;
    d_family[1] = (int*)(b + o_f1);
    d_counts = (unsigned int*)(b + o_c);
    d_scal = (PaScalars*)(b + o_s);
    fcur = 0;
    res_cap = capacity;
  }

  void ensure_capacity(int n, cudaStream_t st)
  {
    if (n <= pools[cur].cap)
    {
      ensure_aux(pools[cur].cap);
      return;
    }
    int cap = std::max(n + n / 2, 64);
    Pool np[2];
    np[0].alloc(*model, cap);
    np[1].alloc(*model, cap);
    ensure_aux(cap);
    if (R > 0 && pools[cur].cap > 0)
    {
      std::vector<int> ident(R);
      std::iota(ident.begin(), ident.end(), 0);
      cuda_check(cudaMemcpyAsync(d_src, ident.data(), R * 4, cudaMemcpyHostToDevice, st), "H2D");
      cuda_check(launch_pa_copy(pools[cur].pop, np[0].pop, d_src, (int)R, st), "copy");
      cuda_check(cudaStreamSynchronize(st), "sync");
    }
    pools[0] = std::move(np[0]);
    pools[1] = std::move(np[1]);
    cur = 0;
    device_bytes = (int64_t)(pools[0].buf.bytes + pools[1].buf.bytes + aux.bytes);
  }

  void upload_beta(cudaStream_t st)
  {
    cuda_check(cudaMemcpyAsync(d_beta, wbeta.data(), R * 8, cudaMemcpyHostToDevice, st), "H2D beta");
  }

  // init_population (solver/population_annealing.h:141-167)
  void init_population(cudaStream_t st)
  {
    size_t old = R;
    if (R < target_pop)
    {
      ensure_capacity((int)target_pop, st);
      wbeta.resize(target_pop, 0.0);
      family.resize(target_pop, 0);
      for (size_t i = old; i < target_pop; i++)
        wbeta[i] = cur_beta <= 0 ? 0.0 : cur_beta;  // Metropolis::set_beta
      R = target_pop;
    }
    for (size_t i = 0; i < target_pop; i++) family[i] = i;
    InitArgs a{};
    // citizens that already exist keep their counters across a restart;
    // new ones start from zero (their slots are cleared first)
    a.keep_counters = 1;
    if (old < R)
    {
      cuda_check(cudaMemsetAsync(pools[cur].pop.attempts + old, 0, (R - old) * 8, st), "memset");
      cuda_check(cudaMemsetAsync(pools[cur].pop.accepts + old, 0, (R - old) * 8, st), "memset");
    }
    a.m = model->device_view(full_maxsat_sweep);
    a.p = pools[cur].pop;
    a.n_walkers = (int)R;
    // the lane and level sweeps work from the spins alone
    a.skip_terms = (lanes || levels) ? 1 : 0;
    if (replay)
    {
      if (streams_on_device)
      {
        cuda_check(cudaMemcpyAsync(streams.data(), d_streams, (size_t)T * 8, cudaMemcpyDeviceToHost, st), "D2H");
        cuda_check(cudaStreamSynchronize(st), "sync");
      }
      streams_on_device = true;
      // walker i draws from stream i % T after the walkers before it
      const uint64_t D = (uint64_t)draws_per_init();
      std::vector<uint64_t> per(R);
      for (size_t i = 0; i < R; i++) per[i] = jump(streams[i % T], (uint64_t)(i / T) * D);
      for (int t = 0; t < T; t++)
      {
        uint64_t n_t = (R > (size_t)t) ? (uint64_t)((R - t + T - 1) / T) : 0;
        streams[t] = jump(streams[t], n_t * D);
      }
      cuda_check(cudaMemcpyAsync(d_init_rng, per.data(), R * 8, cudaMemcpyHostToDevice, st), "H2D");
      cuda_check(cudaMemcpyAsync(d_streams, streams.data(), (size_t)T * 8, cudaMemcpyHostToDevice, st), "H2D");
      a.replay = model->kind == K_MAXSAT ? 2 : 1;
      a.rng = d_init_rng;
      cuda_check(launch_init(a, st), "init kernel");
      cuda_check(cudaStreamSynchronize(st), "sync");
    }
    else
    {
      a.replay = model->kind == K_MAXSAT ? 3 : 0;
      a.seed = seed;
      a.key_base = (0xFFFFFFFFULL - epoch) << 32;
      a.key_div = (long long)1 << 40;
      cuda_check(launch_init(a, st), "init kernel");
    }
    launches++;
    upload_beta(st);
    if (multinomial)
    {
      ensure_res(pools[cur].cap);
      cuda_check(launch_pa_iota(d_family[fcur], (int)R, st), "family ids");
      launches++;
    }
  }

  void init(cudaStream_t st) override
  {
    initialized = true;
    if (model->empty()) return;
    ensure_device();
    streams_on_device = false;
    has_low = false;
    trace_beta.clear();
    trace_pop.clear();
    swept = 0;
    epoch = 0;
    target_pop = target_initial;
    master = ext_master ? *ext_master : PcgEngine(seed);
    streams.assign(T, 0);
    for (int t = 0; t < T; t++) streams[t] = PcgEngine(master()).state;  // rngs_[t] = fork()
    cur_beta = beta_start;
    restart_base = 0;
    R = 0;
    // lanes need independent streams per walker: counter mode only
    levels = levels_for(*this, *model);
    lanes = !levels && !replay && lanes_for(*this, *model, (int64_t)target_pop);
    if (replay && kernel == 2) fail(1, "parameter `kernel`: \"lanes\" needs \"rng_mode\": \"counter\" here");
    used_kernel = levels ? 3 : (lanes ? 2 : 1);
    init_population(st);
    // update_lowest_cost(population_[0]->cost(), population_[0]->state())
    double c0;
    cuda_check(cudaMemcpy(&c0, pools[cur].pop.cost, 8, cudaMemcpyDeviceToHost), "D2H");
    has_low = true;
    low_cost = c0;
    low_words.resize(pools[cur].pop.nw);
    cuda_check(cudaMemcpy(low_words.data(), pools[cur].pop.spins, low_words.size() * 4,
                          cudaMemcpyDeviceToHost), "D2H");
  }

  void run(cudaStream_t st) override;
  void step_multinomial(cudaStream_t st, int64_t step);

  void fetch(std::vector<double>& cost, std::vector<double>& lowest, std::vector<uint64_t>& att,
             std::vector<uint64_t>& acc, std::vector<uint8_t>* lowest_states,
             std::vector<uint8_t>* states) override
  {
    int n = (int)n_walkers();
    cost.resize(n);
    lowest.resize(n);
    att.resize(n);
    acc.resize(n);
    if (!n) return;
    const DevPop& p = pools[cur].pop;
    cuda_check(cudaMemcpy(cost.data(), p.cost, n * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(lowest.data(), p.lowest, n * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(att.data(), p.attempts, n * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(acc.data(), p.accepts, n * 8, cudaMemcpyDeviceToHost), "D2H");
    std::vector<uint32_t> w((size_t)n * p.nw);
    auto unpack = [&](std::vector<uint8_t>& out) {
      out.resize((size_t)n * model->N);
      unpack_states(w.data(), p.nw, model->N, n, out.data());
    };
    if (lowest_states)
    {
      cuda_check(cudaMemcpy(w.data(), p.lspins, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      unpack(*lowest_states);
    }
    if (states)
    {
      cuda_check(cudaMemcpy(w.data(), p.spins, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      unpack(*states);
    }
  }
};

void PopulationAnnealing::configure_common_pa(const json::Value& doc)
{
  configure_common_public(*this, doc);
  const json::Value& p = params;
  auto num = [&](const char* k, double def) {
    const json::Value* v = p.find(k);
    if (!v || v->is_null()) return def;
    if (!v->is_number()) fail(1, std::string("parameter `") + k + "`: expected number");
    return v->num;
  };
  alpha = num("alpha", 2.0);
  if (!(alpha > 1.0)) fail(1, "parameter `alpha`: must be greater than 1, found " + json::number(alpha));
  double pop = num("population", (double)threads);
  if (!(pop > 0)) fail(1, "parameter `population`: must be greater than 0");
  target_pop = (size_t)pop;
  target_initial = target_pop;
  const json::Value* cp = p.find("constant_population");
  constant_population = cp && ((cp->type == json::Value::BOOL && cp->b) || (cp->is_number() && cp->num != 0));
  const json::Value* rs = p.find("resampling_strategy");
  if (rs && rs->is_string()) strategy = rs->str;
  if (strategy != "linear_schedule" && strategy != "geometric_schedule")
    fail(1, "`resampling strategy` must be one of ['linear_schedule', 'geometric_schedule'] on this solver");
  bool geometric = strategy == "geometric_schedule";
  if (p.find("beta"))
    beta = parse_schedule(p["beta"], "beta");
  else
  {
    double b0 = num("beta_start", geometric ? 0.01 : 0.0);
    double b1 = num("beta_stop", 5.0);
    if (!(b1 >= b0)) fail(1, "parameter `beta_stop`: must be greater than or equal to beta_start");
    if (!geometric && b0 < 0) fail(1, "parameter `beta_start`: must be greater than or equal to 0");
    if (geometric && (b0 <= 0 || b1 <= 0)) fail(1, "beta_start and beta_stop must be positive for geometric");
    beta.type = geometric ? 1 : 0;
    beta.initial = b0;
    beta.final_ = b1;
  }
  if (beta.get_count() == 1)
  {
    if (step_limit > 1)
    {
      beta.has_stop = true;
      beta.stop_ = std::max(1, (int)step_limit - 1);
    }
    else
      fail(1, "Either a step_limit or schedule.count must be provided. "
              "You can also set beta.{start,stop} to define the range.");
  }
  if (beta.progress_value(0) >= beta.progress_value(1))
    fail(1, "the schedule for beta must be increasing (i.e., beta.initial < beta.final).");
  beta_start = beta.get_value(0);
  int64_t s = 1;
  const json::Value* v = p.find("sweeps_per_replica");
  if (v && v->is_number()) s = (int64_t)v->num;
  if (s <= 0) fail(1, "parameter `sweeps_per_replica`: must be greater than 0");
  spr = s;
  // feature 2 = PA exponential repopulation (utils/config.h:49-61)
  const json::Value* en = p.find("enabled_features");
  if (en && en->is_array())
    for (const auto& x : en->arr)
      if (x.is_number() && x.num == 2) exp_repop = true;
  const json::Value* rsm = p.find("resampling");
  if (rsm && !rsm->is_null())
  {
    if (!rsm->is_string() || (rsm->str != "reference" && rsm->str != "multinomial"))
      fail(1, "parameter `resampling` must be \"reference\" or \"multinomial\"");
    multinomial = rsm->str == "multinomial";
    if (multinomial && replay)
      fail(1, "parameter `resampling`: \"multinomial\" needs \"rng_mode\": \"counter\"");
  }
  // OpenMP stream emulation for replay: one stream per reference thread
  T = threads;
  output_params.push_back({"population", std::to_string(target_pop)});
  output_params.push_back({"beta", beta.render()});
  output_params.push_back({"alpha", json::number(alpha)});
}

// One resampling step on the device (pa_device.cu): weights, prefix sums,
// parents, replica copies and the family census run as kernels; the host
// reads back one small record (cost range, best lowest, census).
void PopulationAnnealing::step_multinomial(cudaStream_t st, int64_t step)
{
  const double scale = model->scale_factor;
  const size_t Rn = R;
  const double Rd = (double)Rn;
  Pool& P = pools[cur];
  double delta_beta = beta.get_value((double)(step + 1 - (int64_t)restart_base)) -
                      beta.get_value((double)(step - (int64_t)restart_base));
  trace_beta.push_back(cur_beta);
  cuda_check(launch_pa_weights(P.pop.cost, P.pop.lowest, (int)Rn, delta_beta > 0 ? delta_beta * scale : 0.0,
                               d_prefix, d_scal, st),
             "weights kernel");
  launches++;
  if (delta_beta > 0)
  {
    const uint64_t key = host_counter_key(seed, (0x7FFFFFFFULL << 32) | (uint64_t)step);
    Pool& Pn = pools[1 - cur];
    cuda_check(launch_pa_parents(d_prefix, (int)Rn, (int)Rn, key, d_scal, d_family[fcur], d_src,
                                 d_family[1 - fcur], st),
               "parents kernel");
    cuda_check(launch_pa_copy(P.pop, Pn.pop, d_src, (int)Rn, st), "copy kernel");
    fcur = 1 - fcur;
    cuda_check(launch_pa_census(d_family[fcur], (int)Rn, d_counts, (int)Rn, d_scal, st), "census");
    launches += 4;
  }
  PaScalars sc{};
  cuda_check(cudaMemcpyAsync(&sc, d_scal, sizeof sc, cudaMemcpyDeviceToHost, st), "D2H");
  cuda_check(cudaStreamSynchronize(st), "sync");
  // update_lowest_cost (solver/population_annealing.h:301-308): the first
  // citizen with the smallest lowest cost, on the population swept this step
  if (!has_low || sc.best_lowest < low_cost)
  {
    has_low = true;
    low_cost = sc.best_lowest;
    low_words.resize(P.pop.nw);
    cuda_check(cudaMemcpy(low_words.data(), P.pop.lspins + (size_t)sc.best_index * P.pop.nw,
                          P.pop.nw * 4, cudaMemcpyDeviceToHost), "D2H");
  }
  double rho_t = 1.0;
  if (delta_beta > 0)
  {
    cur = 1 - cur;
    rho_t = (double)sc.census / Rd;
  }
  trace_pop.push_back((int64_t)R);
  if (Rd / rho_t < alpha || sc.cmax == sc.cmin)
  {
    cur_beta = beta_start;
    restart_base = (uint64_t)step;
    if (exp_repop) target_pop *= 2;
    epoch++;
    init_population(st);
  }
  else
  {
    cur_beta += delta_beta;
    const double b = cur_beta <= 0 ? 0.0 : cur_beta;
    std::fill(wbeta.begin(), wbeta.begin() + R, b);  // host mirror for a later restart
    cuda_check(launch_pa_fill(d_beta, (int)R, b, st), "beta fill");
    launches++;
  }
}

void PopulationAnnealing::run(cudaStream_t st)
{
  if (!initialized) fail(1, "init() must be called before run()");
  ran = true;
  if (model->empty()) return;
  const double scale = model->scale_factor;  // rescale() at init
  std::vector<double> after, lowest;
  int64_t step = 0;
  const auto t0 = std::chrono::steady_clock::now();
  // the time limit, checked between steps (SteppingSolver::run)
  auto out_of_time = [&] {
    return has_time_limit &&
           std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() >= time_limit;
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, st);
  for (step = 0; step < step_limit;)
  {
    Pool& P = pools[cur];
    const size_t Rn = R;
    after.resize(Rn);
    lowest.resize(Rn);
    SweepArgs a{};
    a.m = model->device_view(full_maxsat_sweep);
    a.p = P.pop;
    a.n_walkers = (int)Rn;
    a.n_streams = replay ? std::min<int>(T, (int)Rn) : (int)Rn;
    a.beta = d_beta;
    a.bs_w = 1;
    a.bs_s = 0;
    a.sweep_base = 0;
    a.n_sweeps = (int)spr;
    swept += (uint64_t)Rn * (uint64_t)spr *
             (uint64_t)((model->kind == K_MAXSAT && !full_maxsat_sweep) ? 1 : model->N);
    a.replay = replay ? 1 : 0;
    a.rng = d_streams;
    a.seed = seed;
    a.key_base = (unsigned long long)(step + 1) << 32;
    a.key_div = (long long)1 << 40;
    a.smem_state = smem_state ? 1 : 0;
    a.err = device_error_flag();
    int wpb = pick_wpb(warps_per_block, a.n_streams);
    if (levels)
    {
      lvlog.ensure((int)Rn, spr, *model, P.pop.nw);
      LvArgs v{};
      v.m = a.m;
      v.p = P.pop;
      v.n_walkers = (int)Rn;
      v.beta = d_beta;
      v.bs_w = 1;
      v.bs_s = 0;
      v.sweep_base = 0;
      v.n_sweeps = (int)spr;
      v.seed = seed;
      v.key_base = a.key_base;
      v.key_div = a.key_div;
      lvlog.fill(v);
      prof_begin(st);
      cuda_check(launch_lv_sweep(v, st), "level sweep kernel");
      prof_end(st);
      // the term bytes are not kept up to date: every reader of this
      // population in this mode uses the spins
      launches++;
    }
    else if (lanes)
    {
      if (!L.ready || lane_walkers < (int)Rn)
      {
        L.setup({model->device_view(full_maxsat_sweep)}, {}, (int)Rn, {}, smem_state);
        lane_walkers = (int)Rn;
      }
      LwArgs la = L.a;
      la.p = P.pop;
      la.n_walkers = (int)Rn;
      la.beta = d_beta;
      la.bs_w = 1;
      la.bs_s = 0;
      la.sweep_base = 0;
      la.n_sweeps = (int)spr;
      la.replay = 0;
      la.int_mode = model->int_mode ? 1 : 0;
      la.seed = seed;
      la.key_base = a.key_base;
      la.key_div = a.key_div;
      cuda_check(launch_lw_load(la, L.max_words, st), "lane load");
      prof_begin(st);
      cuda_check(launch_lw_sweep(la, 0, st), "lane sweep kernel");
      prof_end(st);
      // the term bytes are not kept up to date: every reader of this
      // population in this mode uses the spins
      cuda_check(launch_lw_store(la, L.max_words, 0, st), "lane store");
      launches += 3;
    }
    else
    {
      prof_begin(st);
      cuda_check(launch_sweep(a, st, wpb), "sweep kernel");
      prof_end(st);
      launches++;
    }
    if (multinomial)
    {
      step_multinomial(st, step);
      step++;
      if (has_cost_limit && has_low && low_cost <= cost_limit) break;
      if (out_of_time()) break;
      continue;
    }
    cuda_check(cudaMemcpyAsync(after.data(), P.pop.cost, Rn * 8, cudaMemcpyDeviceToHost, st), "D2H");
    cuda_check(cudaMemcpyAsync(lowest.data(), P.pop.lowest, Rn * 8, cudaMemcpyDeviceToHost, st), "D2H");
    cuda_check(cudaStreamSynchronize(st), "sync");
    // update_lowest_cost over the citizens (solver/population_annealing.h:301-308)
    int best = -1;
    for (size_t i = 0; i < Rn; i++)
      if (!has_low || lowest[i] < low_cost)
      {
        has_low = true;
        low_cost = lowest[i];
        best = (int)i;
      }
    if (best >= 0)
    {
      low_words.resize(P.pop.nw);
      cuda_check(cudaMemcpy(low_words.data(), P.pop.lspins + (size_t)best * P.pop.nw,
                            P.pop.nw * 4, cudaMemcpyDeviceToHost), "D2H");
    }
    // statistics (solver/population_annealing.h:310-382)
    const double Rd = (double)Rn;
    double avg_after = 0, min_cost = std::numeric_limits<double>::max();
    for (size_t i = 0; i < Rn; i++)
    {
      avg_after += after[i];
      min_cost = (after[i] < min_cost) ? after[i] : min_cost;
    }
    avg_after /= Rd;
    double var_after = 0;
    for (size_t i = 0; i < Rn; i++)
    {
      double d = after[i] - avg_after;
      var_after += d * d;
    }
    var_after /= Rd;
    for (size_t i = 0; i < Rn; i++) after[i] -= min_cost;
    double delta_beta = beta.get_value((double)(step + 1 - (int64_t)restart_base)) -
                        beta.get_value((double)(step - (int64_t)restart_base));
    double rho_t = 1.0;
    trace_beta.push_back(cur_beta);
    if (delta_beta > 0)
    {
      // resample (solver/population_annealing.h:490-616)
      std::vector<double> weight(Rn);
      double total = 0.0;
      for (size_t i = 0; i < Rn; i++)
      {
        weight[i] = exp(-delta_beta * after[i] * scale);
        total += weight[i];
      }
      std::vector<size_t> count(Rn, 1);
      if (constant_population)
      {
        size_t resampled = 0;
        std::vector<double> residual(Rn);
        for (size_t i = 0; i < Rn; i++)
        {
          double rel = (double)target_pop * weight[i] / total;
          size_t iw = (size_t)floor(rel);
          residual[i] = rel - (double)iw;
          count[i] = iw;
          resampled += iw;
        }
        Selector sel;
        for (size_t i = 0; i < Rn; i++) sel.insert(i, residual[i]);
        while (resampled < Rn)
        {
          count[sel.select_and_remove(master.uniform())] += 1;
          resampled++;
        }
      }
      else
      {
        double RRQ = (double)target_pop / total;
        uint64_t curp = Rn;
        for (size_t i = 0; i < Rn; i++)
        {
          size_t nc = (RRQ * weight[i]) > 0.0 ? (size_t)floor(master.poisson(RRQ * weight[i])) : 0;
          if (nc == 0)
          {
            curp -= count[i];
            count[i] = 0;
          }
          else if (nc > 1)
          {
            curp += nc - 1;
            count[i] += nc - 1;
          }
        }
        if (curp == 0)
        {
          size_t i = (size_t)floor(master.uniform() * Rn);
          count[i] += 1;
        }
      }
      // Population::resample: survivors in order, each followed... copies of
      // citizen i (count - 1) precede the moved original; all are identical.
      std::vector<int> src;
      std::vector<size_t> fam;
      std::vector<double> nb;
      for (size_t i = 0; i < Rn; i++)
        for (size_t c = 0; c < count[i]; c++)
        {
          src.push_back((int)i);
          fam.push_back(family[i]);
          nb.push_back(wbeta[i]);
        }
      size_t Rnew = src.size();
      ensure_capacity((int)Rnew, st);
      Pool& Pc = pools[cur];
      Pool& Pn = pools[1 - cur];
      cuda_check(cudaMemcpyAsync(d_src, src.data(), Rnew * 4, cudaMemcpyHostToDevice, st), "H2D");
      cuda_check(launch_pa_copy(Pc.pop, Pn.pop, d_src, (int)Rnew, st), "copy kernel");
      launches++;
      cur = 1 - cur;
      family.swap(fam);
      wbeta.swap(nb);
      R = Rnew;
      std::map<size_t, size_t> census;
      for (size_t f : family) census[f]++;
      rho_t = 0;
      for (auto& kv : census) rho_t += (double)kv.second * (double)kv.second;
      rho_t /= Rd;
    }
    trace_pop.push_back((int64_t)R);
    if (Rd / rho_t < alpha || var_after == 0)
    {
      cur_beta = beta_start;
      restart_base = (uint64_t)step;
      if (exp_repop) target_pop *= 2;
      epoch++;
      init_population(st);
    }
    else
    {
      cur_beta += delta_beta;
      for (size_t i = 0; i < R; i++) wbeta[i] = cur_beta <= 0 ? 0.0 : cur_beta;
      upload_beta(st);
    }
    step++;
    if (has_cost_limit && has_low && low_cost <= cost_limit) break;
    if (out_of_time()) break;
  }
  last_step = step;
  if (ext_master) *ext_master = master;
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  run_ms = ms;
  sweep_ms = profile ? prof_total_ms() : ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  check_device_error(st);
}

// ---------------------------------------------------------------------------
// Substochastic Monte Carlo ("substochasticmontecarlo.cpu",
// solver/substochastic_monte_carlo.h:22-311): a population of random walkers
// resampled every step.  The walker steps run on the device
// (ssmc_walk_kernel); the O(R) statistics and resampling run on the host in
// the reference's arithmetic (sequential sums, the C library's exp, the
// RandomSelector on the master PCG stream), the copies on the device.
// Replay streams emulate the reference's OpenMP threads (`threads` streams,
// each serving a contiguous block of walkers); counter streams key each
// walker slot.
// ---------------------------------------------------------------------------
class SubstochasticMonteCarlo : public Solver
{
 public:
  int64_t target_pop = 1, spw = 1;
  Schedule alpha, beta;
  Pool pools[2];
  int cur = 0;
  DevBuf aux;  // src map (R ints), chain streams (T), init streams (R), best spins
  int* d_src = nullptr;
  uint64_t* d_chain = nullptr;
  uint64_t* d_init = nullptr;
  uint32_t* d_best = nullptr;
  PcgEngine master{0};
  PcgEngine* ext_master = nullptr;  // repeated runs: the master stream continues from run to run
  uint64_t swept = 0;  // walker steps since init (each attempts a move with probability p_step)
  bool has_low = false;
  double low_cost = 0;
  int T = 1;
  int cap_R = 0;  // walkers the buffers hold
  // page-locked host copies of the costs, lowest costs and the copy map
  double* h_cost = nullptr;
  double* h_low = nullptr;
  int* h_src = nullptr;
  int host_R = 0;

  ~SubstochasticMonteCarlo() override
  {
    if (h_cost) cudaFreeHost(h_cost);
    if (h_low) cudaFreeHost(h_low);
    if (h_src) cudaFreeHost(h_src);
  }

  std::string target() const override { return "substochasticmontecarlo.cpu"; }
  int64_t n_walkers() const override { return model->empty() ? 0 : target_pop; }

  static std::string num6(double x)
  {
    char b[64];
    snprintf(b, sizeof b, "%g", x);
    return b;
  }

  void configure(const json::Value& doc)
  {
    configure_common_public(*this, doc);
    auto num = [&](const char* k, double def) {
      const json::Value* v = params.find(k);
      if (!v || v->is_null()) return def;
      if (!v->is_number()) fail(1, std::string("parameter `") + k + "`: expected number");
      return v->num;
    };
    target_pop = (int64_t)num("target_population", (double)threads);
    if (target_pop <= 0) fail(1, "parameter `target_population`: must be greater than 0");
    if (target_pop > (1 << 24)) fail(1, "parameter `target_population` too large");
    spw = (int64_t)num("steps_per_walker", 1.0);
    if (spw <= 0) fail(1, "parameter `steps_per_walker`: must be greater than 0");
    alpha = Schedule{};
    alpha.type = 0;
    alpha.initial = 1.0;
    alpha.final_ = 0.0;
    beta = Schedule{};
    beta.type = 0;
    beta.initial = 0.0;
    beta.final_ = 5.0;
    if (params.find("alpha")) alpha = parse_schedule(params["alpha"], "alpha");
    if (params.find("beta")) beta = parse_schedule(params["beta"], "beta");
    // equal lengths (solver/substochastic_monte_carlo.h:177-209)
    if (alpha.get_count() <= 1 && beta.get_count() <= 1)
    {
      alpha.has_stop = beta.has_stop = true;
      alpha.stop_ = beta.stop_ = (double)(int)step_limit;
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
      fail(1, "The schedules for alpha and beta must have the same length");
    const double a0 = alpha.progress_value(0), a1 = alpha.progress_value(1);
    if (a0 <= a1)
      fail(1, "the schedule for alpha must be decreasing (i.e., alpha.initial > alpha.final). Found alpha.initial = " +
                  num6(a0) + " <= " + num6(a1) + " = alpha.final.");
    const double b0 = beta.progress_value(0), b1 = beta.progress_value(1);
    if (b0 >= b1)
      fail(1, "the schedule for beta must be increasing (i.e., beta.initial < beta.final). Found beta.initial = " +
                  num6(b0) + " >= " + num6(b1) + " = beta.final.");
    T = threads;
    output_params.push_back({"target_population", std::to_string(target_pop)});
    output_params.push_back({"steps_per_walker", std::to_string(spw)});
    output_params.push_back({"alpha", alpha.render()});
    output_params.push_back({"beta", beta.render()});
  }

  bool historical_lowest(double& c, std::vector<uint8_t>& st) override
  {
    if (!has_low) return false;
    c = low_cost;
    std::vector<uint32_t> w(pools[0].pop.nw);
    cuda_check(cudaMemcpy(w.data(), d_best, w.size() * 4, cudaMemcpyDeviceToHost), "D2H best");
    st.assign(model->N, 0);
    for (int64_t v = 0; v < model->N; v++) st[v] = (w[v / 32] >> (v % 32)) & 1u;
    return true;
  }

  void init(cudaStream_t st) override
  {
    initialized = true;
    if (model->empty()) return;
    ensure_device();
    const int R = (int)target_pop;
    if (!pools[0].buf.ptr || cap_R < R)
    {
      cap_R = R;
      pools[0].alloc(*model, R);
      pools[1].alloc(*model, R);
      size_t off = 0;
      auto take = [&](size_t b) { size_t o = off; off = (off + b + 255) & ~(size_t)255; return o; };
      const size_t o_src = take((size_t)R * 4), o_ch = take((size_t)T * 8), o_in = take((size_t)R * 8),
                   o_b = take((size_t)pools[0].pop.nw * 4);
      aux = DevBuf(off);
      char* b = (char*)aux.ptr;
      d_src = (int*)(b + o_src);
      d_chain = (uint64_t*)(b + o_ch);
      d_init = (uint64_t*)(b + o_in);
      d_best = (uint32_t*)(b + o_b);
    }
    if (h_cost && host_R < R)
    {
      cudaFreeHost(h_cost);
      cudaFreeHost(h_low);
      cudaFreeHost(h_src);
      h_cost = h_low = nullptr;
      h_src = nullptr;
    }
    if (!h_cost)
    {
      host_R = R;
      cuda_check(cudaMallocHost((void**)&h_cost, (size_t)R * 8), "cudaMallocHost");
      cuda_check(cudaMallocHost((void**)&h_low, (size_t)R * 8), "cudaMallocHost");
      cuda_check(cudaMallocHost((void**)&h_src, (size_t)R * 4), "cudaMallocHost");
    }
    device_bytes = (int64_t)(pools[0].buf.bytes + pools[1].buf.bytes + aux.bytes);
    cur = 0;
    has_low = false;
    step_pos = 0;
    swept = 0;
    // rngs_[t] = rng_->fork() (solver/substochastic_monte_carlo.h:47-51);
    // thread t initialises its block of walkers in index order, each walker
    // taking one draw per 32 variables (model/ising.h:23-41), or one
    // uniform() -- two draws -- per variable for MaxSat (model/max_sat.h:
    // 144-150)
    master = ext_master ? *ext_master : PcgEngine(seed);
    const bool ms = model->kind == K_MAXSAT;
    const uint64_t per = ms ? (uint64_t)(2 * model->N) : (uint64_t)((model->N + 31) / 32);
    std::vector<uint64_t> chain(T), wi(R);
    for (int t = 0; t < T; t++)
    {
      uint64_t f = PcgEngine((uint32_t)master()).state;
      const int q = R / T, r = R % T;
      const int b0 = t < r ? t * (q + 1) : t * q + r, e0 = b0 + (t < r ? q + 1 : q);
      for (int i = b0; i < e0; i++) wi[i] = jump(f, (uint64_t)(i - b0) * per);
      chain[t] = jump(f, (uint64_t)(e0 - b0) * per);
    }
    cuda_check(cudaMemcpyAsync(d_chain, chain.data(), T * 8, cudaMemcpyHostToDevice, st), "H2D");
    cuda_check(cudaMemcpyAsync(d_init, wi.data(), (size_t)R * 8, cudaMemcpyHostToDevice, st), "H2D");
    InitArgs a{};
    a.m = model->device_view(false);
    a.p = pools[0].pop;
    a.n_walkers = R;
    a.replay = replay ? (ms ? 2 : 1) : (ms ? 3 : 0);
    a.rng = d_init;
    a.seed = seed;
    a.key_base = 0;
    a.key_div = (long long)1 << 40;
    a.skip_terms = 1;  // the walker steps work from the spins
    cuda_check(launch_init(a, st), "init kernel");
    launches++;
    used_kernel = 5;
    // update_lowest_cost(population_[0]->cost(), state())
    cuda_check(cudaMemcpyAsync(&low_cost, pools[0].pop.cost, 8, cudaMemcpyDeviceToHost, st), "D2H");
    cuda_check(cudaMemcpyAsync(d_best, pools[0].pop.spins, pools[0].pop.nw * 4, cudaMemcpyDeviceToDevice, st),
               "D2D");
    cuda_check(cudaStreamSynchronize(st), "sync");
    has_low = true;
  }

  // one step: walker steps, statistics, resampling (make_step, :67-84)
  void step(cudaStream_t st, int64_t s)
  {
    const double* cost = h_cost;
    const double* low = h_low;
    const int R = (int)target_pop;
    SsmcArgs a{};
    a.m = model->device_view(false);
    a.p = pools[cur].pop;
    a.n_walkers = R;
    a.steps_per_walker = (int)spw;
    a.p_step = alpha.get_value((double)s) / (double)spw;
    a.step = s;
    a.n_chains = T;
    a.rng = d_chain;
    a.seed = seed;
    a.replay = replay ? 1 : 0;
    prof_begin(st);
    cuda_check(launch_ssmc_walk(a, st), "ssmc walk kernel");
    swept += (uint64_t)R * (uint64_t)spw;
    prof_end(st);
    launches++;
    const DevPop& p = pools[cur].pop;
    cuda_check(cudaMemcpyAsync(h_cost, p.cost, (size_t)R * 8, cudaMemcpyDeviceToHost, st), "D2H");
    cuda_check(cudaMemcpyAsync(h_low, p.lowest, (size_t)R * 8, cudaMemcpyDeviceToHost, st), "D2H");
    cuda_check(cudaStreamSynchronize(st), "sync");
    // update_population_statistics (:114-126)
    double mn = cost[0], mx = cost[0];
    int best = -1;
    for (int i = 0; i < R; i++)
    {
      mn = std::min(mn, cost[i]);
      mx = std::max(mx, cost[i]);
      if (low[i] < low_cost)
      {
        low_cost = low[i];
        best = i;
      }
    }
    if (best >= 0)
      cuda_check(cudaMemcpyAsync(d_best, p.lspins + (size_t)best * p.nw, p.nw * 4, cudaMemcpyDeviceToDevice, st),
                 "D2D");
    // resample_population (:128-169)
    const double b = beta.get_value((double)s);
    const double range = mx - mn;
    if (range > 0)
    {
      double total = 0;
      std::vector<double> weight(R);
      for (int i = 0; i < R; i++)
      {
        weight[i] = exp(b * (mx - cost[i]) / range);
        total += weight[i];
      }
      size_t resampled = 0;
      std::vector<size_t> count(R);
      Selector sel;
      for (int i = 0; i < R; i++)
      {
        const double rel = (double)target_pop * weight[i] / total;
        const size_t iw = (size_t)floor(rel);
        count[i] = iw;
        resampled += iw;
        sel.insert((size_t)i, rel - (double)iw);
      }
      while (resampled < (size_t)R)
      {
        count[sel.select_and_remove(master.uniform())] += 1;
        resampled++;
      }
      // the previous step's sync (the D2H above) has retired the last
      // upload of the map, so the page-locked buffer is free to refill
      int n_src = 0;
      for (int i = 0; i < R; i++)
        for (size_t c = 0; c < count[i]; c++) h_src[n_src++] = i;
      cuda_check(cudaMemcpyAsync(d_src, h_src, (size_t)R * 4, cudaMemcpyHostToDevice, st), "H2D");
      cuda_check(launch_pa_copy(pools[cur].pop, pools[1 - cur].pop, d_src, R, st), "copy kernel");
      launches++;
      cur = 1 - cur;
    }
  }

  void run(cudaStream_t st) override
  {
    if (!initialized) fail(1, "init() must be called before run()");
    ran = true;
    if (model->empty()) return;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    auto t0 = std::chrono::steady_clock::now();
    int64_t s = step_pos;
    for (; s < step_limit; s++)
    {
      step(st, s);
      if (has_cost_limit && low_cost <= cost_limit)
      {
        s++;
        break;
      }
      if (has_time_limit &&
          std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() >= time_limit)
      {
        s++;
        break;
      }
    }
    step_pos = s;
    last_step = s;
    if (ext_master) *ext_master = master;
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    run_ms = ms;
    sweep_ms = profile ? prof_total_ms() : ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
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
    const int64_t end = std::min(step_limit, step_pos + n);
    for (; step_pos < end; step_pos++) step(st, step_pos);
    last_step = step_pos;
    return step_pos >= step_limit;
  }

  void fetch(std::vector<double>& cost, std::vector<double>& lowest, std::vector<uint64_t>& att,
             std::vector<uint64_t>& acc, std::vector<uint8_t>* lowest_states,
             std::vector<uint8_t>* states) override
  {
    const int n = (int)n_walkers();
    cost.resize(n);
    lowest.resize(n);
    att.resize(n);
    acc.resize(n);
    if (!n) return;
    const DevPop& p = pools[cur].pop;
    cuda_check(cudaMemcpy(cost.data(), p.cost, n * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(lowest.data(), p.lowest, n * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(att.data(), p.attempts, n * 8, cudaMemcpyDeviceToHost), "D2H");
    cuda_check(cudaMemcpy(acc.data(), p.accepts, n * 8, cudaMemcpyDeviceToHost), "D2H");
    std::vector<uint32_t> w((size_t)n * p.nw);
    auto unpack = [&](std::vector<uint8_t>& out) {
      out.resize((size_t)n * model->N);
      unpack_states(w.data(), p.nw, model->N, n, out.data());
    };
    if (lowest_states)
    {
      cuda_check(cudaMemcpy(w.data(), p.lspins, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      unpack(*lowest_states);
    }
    if (states)
    {
      cuda_check(cudaMemcpy(w.data(), p.spins, w.size() * 4, cudaMemcpyDeviceToHost), "D2H");
      unpack(*states);
    }
  }
};

// ---------------------------------------------------------------------------
// Parameter-free population annealing and substochastic Monte Carlo
// ("populationannealing-parameterfree.cpu", "substochasticmontecarlo-
// parameterfree.cpu"): solver/parameter_free_solver.h:9-257 with the
// Bayesian strategy (bayes.h) and the adapters of solver/pa_parameter_free.h
// and solver/ssmc_parameter_free.h.  Repeated runs of the underlying solver
// on one master stream that continues from run to run (the adapter's rng_,
// which also draws the initial samples' jitter).  The first
// `initial_samples` runs take the adapter's initial parameter vectors; later
// runs take the strategy's recommendations over the adapter's ranges (whose
// step range follows the measured seconds per step), or, when the strategy
// cannot fit its model, the best vector so far with its first entry x 1.5.
// Each run is handed the time left as its time limit.  The search stops at
// the time limit (default 5 s), when the time left is shorter than the last
// search step took (the reference's tick then holds no step), after
// `nonimprovement_limit` runs in a row without a lower cost, or after
// `step_limit` runs.  The result is the lowest cost found and its state; the
// parameters shown are those of the best run (with equal costs, the cheaper
// run's), as ParameterFreeSolver::finalize renders them.
// ---------------------------------------------------------------------------
class BayesParameterFree : public Solver
{
 public:
  BayesOpt strategy;
  int initial_samples = 4, nonimprovement_limit = 8;
  PcgEngine master{0};
  double min_diff = 0, max_diff = 0;
  int initial_counter = 0;
  double worker_time_limit = 0;  // the adapter's time limit: the time left at its last run
  double steps_accum = 0, secs_accum = 0;
  bool has_best = false;
  double best = 0, best_exec = 0;
  int stable = 0;
  std::vector<double> best_params;
  std::vector<uint8_t> best_state;
  struct Run
  {
    std::vector<double> params;
    int64_t steps = 0, step_limit = 0;
    uint64_t attempts = 0;
    double lowest = 0;
    bool recommended = false;
  };
  std::vector<Run> trace;
  std::string stop_reason;
  uint64_t att_total = 0, acc_total = 0;

  virtual Solver& worker() = 0;
  // the work of the worker's last run, under the trace key work_key():
  // flip attempts (PA) or walker steps (SSMC)
  virtual uint64_t worker_attempts() const = 0;
  virtual const char* work_key() const = 0;
  virtual int dims() const = 0;
  virtual std::vector<std::pair<double, double>> ranges() = 0;
  virtual void initial_values(std::vector<double>& v) = 0;
  virtual void update(const std::vector<double>& v) = 0;
  virtual double exec_cost() = 0;
  virtual void render() = 0;
  virtual void prepare() {}

  int64_t sweep_size() const { return model->kind == K_MAXSAT ? 1 : model->N; }

  // ModelSolver::max_replicas_adjusted_state: the walkers that 58 % of the
  // free device memory holds (a walker's two population slots), at most
  // threads x mult, at least one
  size_t max_states(uint32_t mult) const
  {
    const size_t cap = (size_t)threads * mult;
    size_t free_b = 0, total_b = 0;
    cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    const double nw = (double)((model->N + 31) / 32 + 4);
    const double per = 2.0 * (2.0 * nw * 4.0 + (double)model->M + 80.0);
    const double adjust = (double)free_b / per * 0.58;
    if (adjust < 1.0) return 1;
    return std::min((size_t)adjust, cap);
  }
  // ModelSolver::adjust_states
  size_t adjust_states(double x, uint32_t mult) const
  {
    const size_t mx = max_states(mult);
    size_t r = std::min((size_t)x, mx);
    if (mx > (size_t)threads)
      r = std::max(r, (size_t)threads);
    else
      r = mx;
    return r;
  }

  // parameters of the search itself (ParameterFreeSolver::training_parameters,
  // BayesianOpt::configure)
  void configure_search(const json::Value& p)
  {
    if (number_of_solutions != 1)
      fail(1, "parameter-free solvers return one solution: `number_of_solutions` must be 1");
    auto integer = [&](const char* k, int64_t def) -> int64_t {
      const json::Value* v = p.find(k);
      if (!v || v->is_null()) return def;
      if (!v->is_number()) fail(1, std::string("parameter `") + k + "`: expected integer");
      return (int64_t)v->num;
    };
    initial_samples = (int)integer("initial_samples", 4);
    if (initial_samples <= 0) fail(1, "parameter `initial_samples`: must be greater than 0");
    nonimprovement_limit = (int)integer("nonimprovement_limit", 8);
    if (nonimprovement_limit <= 0) fail(1, "parameter `nonimprovement_limit`: must be greater than 0");
    const int64_t rs = integer("reserved_samples", 64);
    if (rs <= 10) fail(1, "parameter `reserved_samples`: must be greater than 10");
    // BayesianOpt::init resets the reserve to 128 samples whatever the
    // parameter says (strategy/bayesian.cc:25-51, 53-57)
    strategy.reserved = 128;
    if (const json::Value* st = p.find("search_training"))
      if (st->is_object())
        if (const json::Value* v = st->find("num_to_sample"))
        {
          if (!v->is_number() || v->num < 1) fail(1, "parameter `num_to_sample`: expected a positive integer");
          strategy.num_to_sample = (int)v->num;
        }
    if (!has_time_limit)
    {
      has_time_limit = true;  // a time limit must be set (parameter_free_solver.h:56-61)
      time_limit = 5.0;
    }
  }

  int64_t n_walkers() const override { return (model->empty() || !has_best) ? 0 : 1; }

  void init(cudaStream_t) override
  {
    initialized = true;
    ran = false;
    master = PcgEngine(seed);
    strategy.init(dims(), seed);
    initial_counter = 0;
    worker_time_limit = time_limit;
    steps_accum = secs_accum = 0;
    has_best = false;
    best = best_exec = 0;
    stable = 0;
    best_params.clear();
    best_state.clear();
    trace.clear();
    stop_reason.clear();
    att_total = acc_total = 0;
    last_step = 0;
    launches = 0;
    if (!model->empty()) prepare();
  }

  void run(cudaStream_t st) override
  {
    if (!initialized) fail(1, "init() must be called before run()");
    ran = true;
    if (model->empty()) return;
    using clock = std::chrono::steady_clock;
    const auto t0 = clock::now();
    auto since = [](clock::time_point a) { return std::chrono::duration<double>(clock::now() - a).count(); };
    double last = 0;
    for (int64_t step = 0; step < step_limit; step++)
    {
      const double left0 = time_limit - since(t0);
      if (left0 <= 0 || (step > 0 && left0 < last))
      {
        stop_reason = "time limit";
        break;
      }
      const auto ts = clock::now();
      // ParameterFreeSolver::make_step, solver/parameter_free_solver.h:65-151
      std::vector<double> v;
      bool rec = false;
      if (step < initial_samples)
        initial_values(v);
      else
      {
        strategy.set_ranges(ranges());
        rec = strategy.recommend(v);
        if (!rec)
        {
          if (stable < nonimprovement_limit)
          {
            v = best_params;
            v[0] *= 1.5;  // update_parameters_linearly
          }
          else
          {
            stop_reason = "no improvement";
            break;
          }
        }
      }
      const double left = time_limit - since(t0);
      if (left <= 0 && has_best)
      {
        stop_reason = "time limit";
        break;
      }
      update(v);
      Solver& w = worker();
      // counter streams: each run keys them with one master draw, so that the
      // runs' walkers draw independently
      if (!replay) w.seed = master();
      w.has_time_limit = true;
      w.time_limit = left;
      worker_time_limit = left;
      const uint64_t l0 = w.launches;  // the workers count on across runs
      w.init(st);
      const auto tr = clock::now();
      w.run(st);
      secs_accum += since(tr);  // update_accumulated_info
      steps_accum += (double)w.last_step;
      launches += w.launches - l0;
      double obj = 0;
      std::vector<uint8_t> state;
      lowest_of(w, obj, state);
      strategy.add_sample(v, obj);
      Run r;
      r.params = v;
      r.steps = w.last_step;
      r.step_limit = w.step_limit;
      r.lowest = obj + model->const_cost;
      r.attempts = worker_attempts();
      r.recommended = rec;
      trace.push_back(r);
      const double exec = exec_cost();
      auto update_best = [&] {
        best = obj;
        best_exec = exec;
        best_params = v;
        best_state = state;
      };
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
      last = since(ts);
      if (done) break;
      if (has_cost_limit && best <= cost_limit)
      {
        stop_reason = "cost limit";
        break;
      }
    }
    if (stop_reason.empty()) stop_reason = "step limit";
    if (has_best)
    {
      update(best_params);  // finalize: the best run's parameters
      render();
    }
    run_ms = since(t0) * 1e3;
  }

  // a finished run's lowest cost and state (the lowest it ever saw), with its
  // counters added to the totals
  void lowest_of(Solver& w, double& obj, std::vector<uint8_t>& state)
  {
    std::vector<double> c, low;
    std::vector<uint64_t> at, ac;
    std::vector<uint8_t> ls;
    w.fetch(c, low, at, ac, &ls, nullptr);
    for (size_t i = 0; i < at.size(); i++)
    {
      att_total += at[i];
      acc_total += ac[i];
    }
    if (w.historical_lowest(obj, state)) return;
    size_t b = 0;
    for (size_t i = 1; i < low.size(); i++)
      if (low[i] < low[b]) b = i;
    obj = low[b];
    state.assign(ls.begin() + b * model->N, ls.begin() + (b + 1) * model->N);
  }

  void fetch(std::vector<double>& cost, std::vector<double>& lowest, std::vector<uint64_t>& att,
             std::vector<uint64_t>& acc, std::vector<uint8_t>* lowest_states,
             std::vector<uint8_t>* states) override
  {
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
    {
      const Run& r = trace[i];
      s += (i ? "," : "") + std::string("{\"params\":[");
      for (size_t k = 0; k < r.params.size(); k++) s += (k ? "," : "") + json::number(r.params[k]);
      s += "],\"steps\":" + std::to_string(r.steps) + ",\"step_limit\":" + std::to_string(r.step_limit) +
           ",\"" + work_key() + "\":" + std::to_string(r.attempts) +
           ",\"lowest\":" + json::number(r.lowest) + ",\"recommended\":" + (r.recommended ? "true" : "false") + "}";
    }
    s += "],\"stop\":" + json::quote(stop_reason) + ",\"training\":{\"learning_time_ms\":" +
         json::number(strategy.learning_ms) + ",\"model_time_ms\":" + json::number(strategy.model_ms) + "}}";
    return s;
  }

 protected:
  // a range parameter {"initial": a, "final": b} (utils/range.cc:16-30)
  static void range_param(const json::Value& p, const char* k, std::pair<double, double>& r)
  {
    const json::Value* v = p.find(k);
    if (!v || v->is_null()) return;
    const json::Value* a = v->is_object() ? v->find("initial") : nullptr;
    const json::Value* b = v->is_object() ? v->find("final") : nullptr;
    if (!a || !b || !a->is_number() || !b->is_number())
      fail(1, std::string("parameter `") + k + "`: expected {\"initial\": number, \"final\": number}");
    if (a->num > b->num)
      fail(1, "initial value: " + json::number(a->num) + ", is larger than final value:" + json::number(b->num));
    r = {a->num, b->num};
  }
  static double num_param(const json::Value& p, const char* k, double def)
  {
    const json::Value* v = p.find(k);
    if (!v || v->is_null()) return def;
    if (!v->is_number()) fail(1, std::string("parameter `") + k + "`: expected number");
    return v->num;
  }
};

// PAParameterFree (solver/pa_parameter_free.h:18-410): five parameters --
// sweeps, population, alpha, sweeps per replica and the negative log of the
// smallest acceptance probability, which sets beta_stop; a geometric beta
// schedule from -ln(max_prob) / (max cost difference).  The linear-schedule
// resampling strategy (the reference's default; its other strategies are
// experimental and not built).
class PAParameterFree : public BayesParameterFree
{
 public:
  std::unique_ptr<PopulationAnnealing> w;
  double max_step_divider = 160, min_population_mult = 4, initial_alpha = 2, initial_min_prob_log = 2;
  double max_prob = 0.5, final_min_prob_log = 15, start_min_prob_log = 0, beta_start = 0;
  uint32_t initial_sweeps = 20, max_population_mult = 128;
  std::pair<double, double> alpha_range{1.00000001, 3}, spr_range{1, 4};
  uint64_t max_steps = std::numeric_limits<uint32_t>::max() / 8;
  double population_start = 0, population_end = 0;

  std::string target() const override { return "populationannealing-parameterfree.cpu"; }
  Solver& worker() override { return *w; }
  uint64_t worker_attempts() const override { return w->swept; }
  const char* work_key() const override { return "attempts"; }
  int dims() const override { return 5; }

  void configure(const json::Value& doc)
  {
    configure_common_public(*this, doc);
    w.reset(new PopulationAnnealing());
    w->model = model;
    w->configure(doc);
    if (w->strategy != "linear_schedule")
      fail(1, "parameter-free population annealing supports `resampling_strategy` \"linear_schedule\" only");
    const json::Value& p = params;
    configure_search(p);
    max_step_divider = num_param(p, "max_step_divider", 160.);
    if (!(max_step_divider > 1.0)) fail(1, "parameter `max_step_divider`: must be greater than 1");
    min_population_mult = num_param(p, "min_population_mult", 4);
    if (!(min_population_mult > 0)) fail(1, "parameter `min_population_mult`: must be greater than 0");
    const double is = num_param(p, "initial_sweeps", 20);
    if (!(is >= 1)) fail(1, "parameter `initial_sweeps`: must be greater than 0");
    initial_sweeps = (uint32_t)is;
    initial_alpha = num_param(p, "initial_alpha", 2);
    if (!(initial_alpha > 1)) fail(1, "parameter `initial_alpha`: must be greater than 1");
    initial_min_prob_log = num_param(p, "initial_min_prob_log", 2);
    if (!(initial_min_prob_log >= 0)) fail(1, "parameter `initial_min_prob_log`: must be at least 0");
    max_prob = num_param(p, "max_prob", 0.5);
    if (!(max_prob > 0 && max_prob <= 1)) fail(1, "parameter `max_prob`: must be in (0, 1]");
    const double mpm = num_param(p, "max_population_mult", 128);
    if (!(mpm > (double)((uint32_t)min_population_mult + 1)))
      fail(1, "parameter `max_population_mult`: must be greater than min_population_mult + 1");
    max_population_mult = (uint32_t)mpm;
    range_param(p, "alpha_range", alpha_range);
    range_param(p, "sweeps_per_replica_range", spr_range);
    if (num_param(p, "reserved_population", 0) != 0)
      fail(1, "parameter `reserved_population`: only 0 (no replicas carried between runs) is supported");
    const double limit = std::sqrt((double)sweep_size()) * (double)model->M;
    if (limit < (double)std::numeric_limits<uint32_t>::max())
      max_steps = std::max<uint64_t>(max_steps, (uint64_t)limit);
    else
      max_steps = std::numeric_limits<uint32_t>::max();
    if (p.find("max_steps"))
    {
      const double ms = num_param(p, "max_steps", (double)max_steps);
      if (!(ms > 65535)) fail(1, "parameter `max_steps`: must be greater than 65535");
      max_steps = (uint64_t)ms;
    }
    if (!model->empty())
    {
      if (model->kind == K_MAXSAT)
        fail(1, "parameter-free population annealing runs Ising and PUBO models (it needs cost-difference "
                "estimates)");
      max_diff = estimate_max_cost_diff(*model);
      min_diff = estimate_min_cost_diff(*model);
      if (!(max_diff > 0)) fail(1, "max cost difference should be > 0, found :" + json::number(max_diff));
      if (!(min_diff > 0)) fail(1, "min cost difference should be > 0, found :" + json::number(min_diff));
      beta_start = -std::log(max_prob) / max_diff;
      start_min_prob_log = min_diff * beta_start * 2;
      const json::Value* f = p.find("final_min_prob_log");
      if (f && !f->is_null())
      {
        if (!f->is_number() || !(f->num > start_min_prob_log))
          fail(1, "parameter `final_min_prob_log`: must be greater than " + json::number(start_min_prob_log));
        final_min_prob_log = f->num;
      }
      start_min_prob_log = std::max(initial_min_prob_log, start_min_prob_log);
      final_min_prob_log = std::max(final_min_prob_log, start_min_prob_log * 5);
    }
    output_params.clear();
    output_params.push_back({"seed", std::to_string(seed)});
    output_params.push_back({"beta_start", json::number(beta_start)});
  }

  void prepare() override
  {
    ensure_device();
    population_end = (double)max_states(max_population_mult);
    population_start = (double)threads * min_population_mult;
    if (population_start >= population_end) population_start = population_end - 1.;
    w->ext_master = &master;
  }

  std::vector<std::pair<double, double>> ranges() override
  {
    const double sps = secs_accum / steps_accum;
    double ms = worker_time_limit / (sps * max_step_divider);
    ms = std::max(ms, (double)initial_sweeps + 1);
    ms = std::min((double)max_steps, ms);
    return {{(double)initial_sweeps, ms},
            {population_start, population_end},
            alpha_range,
            spr_range,
            {start_min_prob_log, final_min_prob_log}};
  }

  void initial_values(std::vector<double>& v) override
  {
    const int k = initial_counter;
    v.clear();
    v.push_back((double)(initial_sweeps + k * 10));
    v.push_back((double)adjust_states((double)threads * (k + 1), max_population_mult));
    v.push_back(initial_alpha + 0.5 * (master.uniform() - 0.5));
    v.push_back(k + 1.0);
    v.push_back(initial_min_prob_log + k * 2);
    initial_counter++;
  }

  void update(const std::vector<double>& v) override
  {
    w->spr = std::max<int64_t>(1, std::lround(v[3]));
    w->step_limit = std::max<int64_t>((int64_t)std::ceil(v[0] / (double)w->spr), 2);
    w->target_initial = adjust_states(v[1], max_population_mult);
    w->alpha = std::max(v[2], alpha_range.first);
    const double beta_stop = v[4] / min_diff;
    Schedule b;
    b.type = 1;
    b.initial = beta_start;
    b.final_ = beta_stop;
    b.has_stop = true;
    b.stop_ = std::max(1, (int)w->step_limit - 1);
    w->beta = b;
    w->beta_start = b.get_value(0);
  }

  double exec_cost() override
  {
    const size_t t = (size_t)threads;
    return (double)w->step_limit * (double)w->spr * (double)((w->target_initial + t - 1) / t);
  }

  void render() override
  {
    output_params.clear();
    output_params.push_back({"seed", std::to_string(seed)});
    output_params.push_back({"beta_start", json::number(beta_start)});
    output_params.push_back({"beta_stop", json::number(w->beta.final_)});
    output_params.push_back({"beta", w->beta.render()});
    output_params.push_back({"sweeps", std::to_string(w->step_limit)});
    output_params.push_back({"sweeps_per_replica", std::to_string(w->spr)});
    output_params.push_back({"population", std::to_string(w->target_initial)});
    output_params.push_back({"alpha", json::number(w->alpha)});
  }
};

// SSMCParameterFree (solver/ssmc_parameter_free.h:10-280): seven parameters
// -- steps, target population, steps per walker, alpha's final value and
// scope (a linear schedule from final + scope down to final) and beta's
// initial value and scope (linear, initial up to initial + scope).
class SSMCParameterFree : public BayesParameterFree
{
 public:
  std::unique_ptr<SubstochasticMonteCarlo> w;
  uint32_t max_replica_mult = 3, initial_sweeps = 20, initial_spw = 1;
  double max_step_divider = 40, initial_alpha_final = 0.00001, initial_alpha_scope = 0.8;
  double initial_beta_initial = 0.00001, initial_beta_scope = 5;
  uint64_t max_steps = std::numeric_limits<uint16_t>::max();
  std::pair<double, double> steps_range{1., 5.}, alpha_final_range{0.00001, 0.2}, alpha_scope_range{0.8, 1.0},
      beta_initial_range{0.00001, 8.0}, beta_scope_range{1, 8.0};
  double population_start = 0, population_end = 0;

  std::string target() const override { return "substochasticmontecarlo-parameterfree.cpu"; }
  Solver& worker() override { return *w; }
  uint64_t worker_attempts() const override { return w->swept; }
  const char* work_key() const override { return "walker_steps"; }
  int dims() const override { return 7; }

  void configure(const json::Value& doc)
  {
    configure_common_public(*this, doc);
    w.reset(new SubstochasticMonteCarlo());
    w->model = model;
    w->configure(doc);
    const json::Value& p = params;
    configure_search(p);
    range_param(p, "steps_range", steps_range);
    range_param(p, "alpha_final_range", alpha_final_range);
    range_param(p, "alpha_scope_range", alpha_scope_range);
    range_param(p, "beta_initial_range", beta_initial_range);
    range_param(p, "beta_scope_range", beta_scope_range);
    auto positive = [&](const char* k, double def) {
      const double x = num_param(p, k, def);
      if (!(x > 0)) fail(1, std::string("parameter `") + k + "`: must be greater than 0");
      return x;
    };
    max_replica_mult = (uint32_t)positive("max_replica_mult", 3);
    max_step_divider = num_param(p, "max_step_divider", 40.);
    if (!(max_step_divider > 1.0)) fail(1, "parameter `max_step_divider`: must be greater than 1");
    initial_sweeps = (uint32_t)positive("initial_sweeps", 20);
    initial_spw = (uint32_t)positive("initial_steps_per_walker", 1);
    initial_alpha_final = positive("initial_alpha_final", 0.00001);
    initial_alpha_scope = positive("initial_alpha_scope", 0.8);
    initial_beta_initial = positive("initial_beta_initial", 0.00001);
    initial_beta_scope = positive("initial_beta_scope", 5);
    if (num_param(p, "reserved_population", 0) != 0)
      fail(1, "parameter `reserved_population`: only 0 (no walkers carried between runs) is supported");
    const double ss = (double)sweep_size();
    const double limit = std::sqrt(ss) * (double)model->M * ss;
    if (limit < (double)std::numeric_limits<uint32_t>::max())
      max_steps = std::max<uint64_t>(max_steps, (uint64_t)limit);
    else
      max_steps = std::numeric_limits<uint32_t>::max();
    if (p.find("max_steps"))
    {
      const double ms = num_param(p, "max_steps", (double)max_steps);
      if (!(ms > 65535)) fail(1, "parameter `max_steps`: must be greater than 65535");
      max_steps = (uint64_t)ms;
    }
    output_params.clear();
    output_params.push_back({"seed", std::to_string(seed)});
  }

  void prepare() override
  {
    ensure_device();
    population_end = (double)max_states(max_replica_mult);
    population_start = (double)threads;
    if (population_start >= population_end) population_start = population_end - 1.;
    w->ext_master = &master;
  }

  std::vector<std::pair<double, double>> ranges() override
  {
    const double sps = secs_accum / steps_accum;
    const double ss = (double)sweep_size();
    double ms = worker_time_limit / (sps * max_step_divider);
    ms = std::max(ms, 100.0);
    ms = std::max(ms, initial_sweeps * ss + 1.0);
    ms = std::min((double)max_steps, ms);
    return {{initial_sweeps * ss, ms},    {population_start, population_end}, steps_range, alpha_final_range,
            alpha_scope_range,            beta_initial_range,                 beta_scope_range};
  }

  void initial_values(std::vector<double>& v) override
  {
    const int k = initial_counter;
    v.clear();
    v.push_back((double)((uint64_t)initial_sweeps * (uint64_t)sweep_size() * (uint64_t)(1 + k)));
    v.push_back(std::min((double)threads + k, (double)max_states(max_replica_mult)));
    v.push_back((double)initial_spw);
    v.push_back(initial_alpha_final);
    v.push_back(initial_alpha_scope);
    v.push_back(initial_beta_initial);
    v.push_back(initial_beta_scope + 1.0 * master.uniform());
    initial_counter++;
  }

  void update(const std::vector<double>& v) override
  {
    w->step_limit = std::max<int64_t>((int64_t)std::floor(v[0]), 2);
    w->target_pop = (int64_t)adjust_states(v[1], max_replica_mult);
    w->spw = std::max<int64_t>((int64_t)(size_t)v[2], 1);
    Schedule a, b;
    a.type = 0;
    a.initial = v[3] + v[4];
    a.final_ = v[3];
    a.has_stop = true;
    a.stop_ = (double)w->step_limit;
    b.type = 0;
    b.initial = v[5];
    b.final_ = v[5] + v[6];
    b.has_stop = true;
    b.stop_ = (double)w->step_limit;
    w->alpha = a;
    w->beta = b;
  }

  double exec_cost() override
  {
    const int64_t t = threads;
    return (double)w->step_limit * (double)w->spw * (double)((w->target_pop + t - 1) / t);
  }

  void render() override
  {
    output_params.clear();
    output_params.push_back({"seed", std::to_string(seed)});
    output_params.push_back({"step_limit", std::to_string(w->step_limit)});
    output_params.push_back({"target_population", std::to_string(w->target_pop)});
    output_params.push_back({"steps_per_walker", std::to_string(w->spw)});
    output_params.push_back({"alpha", w->alpha.render()});
    output_params.push_back({"beta", w->beta.render()});
  }
};

std::unique_ptr<Solver> make_pa_pf_solver(const HostModel* m, const json::Value& doc)
{
  std::unique_ptr<PAParameterFree> s(new PAParameterFree());
  s->model = m;
  s->configure(doc);
  return std::unique_ptr<Solver>(s.release());
}

std::unique_ptr<Solver> make_ssmc_pf_solver(const HostModel* m, const json::Value& doc)
{
  std::unique_ptr<SSMCParameterFree> s(new SSMCParameterFree());
  s->model = m;
  s->configure(doc);
  return std::unique_ptr<Solver>(s.release());
}

std::unique_ptr<Solver> make_ssmc_solver(const HostModel* m, const json::Value& doc)
{
  std::unique_ptr<SubstochasticMonteCarlo> s(new SubstochasticMonteCarlo());
  s->model = m;
  s->configure(doc);
  return std::unique_ptr<Solver>(s.release());
}

std::unique_ptr<Solver> make_pa_solver(const HostModel* m, const json::Value& doc)
{
  std::unique_ptr<PopulationAnnealing> s(new PopulationAnnealing());
  s->model = m;
  s->configure(doc);
  return std::unique_ptr<Solver>(s.release());
}
}  // namespace qio
