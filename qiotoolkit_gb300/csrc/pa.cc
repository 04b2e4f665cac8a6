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
    epoch = 0;
    target_pop = target_initial;
    master = PcgEngine(seed);
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
  }
  last_step = step;
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
  bool has_low = false;
  double low_cost = 0;
  int T = 1;
  // page-locked host copies of the costs, lowest costs and the copy map
  double* h_cost = nullptr;
  double* h_low = nullptr;
  int* h_src = nullptr;

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
    if (!pools[0].buf.ptr)
    {
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
    if (!h_cost)
    {
      cuda_check(cudaMallocHost((void**)&h_cost, (size_t)R * 8), "cudaMallocHost");
      cuda_check(cudaMallocHost((void**)&h_low, (size_t)R * 8), "cudaMallocHost");
      cuda_check(cudaMallocHost((void**)&h_src, (size_t)R * 4), "cudaMallocHost");
    }
    device_bytes = (int64_t)(pools[0].buf.bytes + pools[1].buf.bytes + aux.bytes);
    cur = 0;
    has_low = false;
    step_pos = 0;
    // rngs_[t] = rng_->fork() (solver/substochastic_monte_carlo.h:47-51);
    // thread t initialises its block of walkers in index order, each walker
    // taking one draw per 32 variables (model/ising.h:23-41), or one
    // uniform() -- two draws -- per variable for MaxSat (model/max_sat.h:
    // 144-150)
    master = PcgEngine(seed);
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
