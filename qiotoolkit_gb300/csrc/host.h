// host.h -- host-side model and solver objects behind the C ABI.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "json.h"
#include "qio_internal.h"

namespace qio
{
// Errors carry the C-ABI status they map to.
struct Error : std::runtime_error
{
  int status;
  Error(int st, const std::string& m) : std::runtime_error(m), status(st) {}
};
[[noreturn]] void fail(int status, const std::string& msg);
void cuda_check(cudaError_t e, const char* what);

// Device buffer owned by RAII.
struct DevBuf
{
  void* ptr = nullptr;
  size_t bytes = 0;
  DevBuf() {}
  explicit DevBuf(size_t n);
  ~DevBuf();
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : ptr(o.ptr), bytes(o.bytes)
  {
    o.ptr = nullptr;
    o.bytes = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept;
  template <class T> T* as() const { return (T*)ptr; }
};

void ensure_device();  // selects the device, uploads tables once per device
// bit-packed walker states (32 variables per word, rows of nw words) to one
// byte per variable, `count` rows of N bytes
void unpack_states(const uint32_t* words, int nw, int64_t N, int64_t count, uint8_t* out);
int* device_error_flag();       // per-device int set by kernels whose bounded waits gave up
void check_device_error(cudaStream_t s);  // throws QIO_TIMEOUT (status 4) when set

struct HostModel
{
  int kind = K_ISING;
  int flavor = F_PARITY;
  int64_t N = 0, M = 0, K = 0;
  // variable -> incident terms (ascending term id), incidence payloads
  std::vector<int> row;
  std::vector<uint32_t> inc;
  std::vector<double> coef;
  std::vector<int> coef_i;
  std::vector<float> coef_f;
  std::vector<unsigned long long> near;
  bool fscreen = true, scan32 = false;
  // Ising models whose terms all have one or two members: the other member
  // of each incidence (-1 for a one-member term)
  bool pair_only = false;
  std::vector<int> other;
  // per incidence (other member, coefficient) records of the lane kernel; a
  // one-member term points at the padding spin n_words * 32 (always 0)
  std::vector<int> rec_i;     // 2 ints per incidence (integer mode)
  std::vector<double> rec_f;  // 2 doubles per incidence: (other as bits, coef)
  std::vector<unsigned int> rec_p;  // other << 8 | coefficient, when |coef| <= 127
  // field-cached sweep records (16 bytes per incidence; see DevModel::fc_rec)
  std::vector<uint32_t> fc_rec;
  int fc_S = 0;
  bool fc_pack = false;
  // level schedule (levels.cu): entries grouped by level, their offsets
  std::vector<int> lv_off, lv_pos;
  std::vector<uint32_t> lv_ent;
  int n_levels = 0, lv_recs = 0, lv_width = 0;
  bool lv_ok = false, lv_d8 = false;
  std::vector<uint32_t> nbr;
  // term -> members
  std::vector<int> trow;
  std::vector<uint32_t> tvar;
  std::vector<double> tcost;
  std::vector<int> tcost_i;
  double const_cost = 0, max_coupling = 0, scale_factor = 1.0;
  int max_loc = 0, min_loc = 0;
  // graph::Size properties (graph/properties.h:52-68, accumulated in
  // normalize_edges, graph/graph.h:134-176): sum of term orders, sum of
  // order * (order - 1) over non-constant terms, smallest |c| of those
  int64_t total_loc = 0, accum_dep = 0;
  double min_coupling = 0;
  std::vector<int32_t> names;  // internal id -> input name
  std::vector<int32_t> free_vars;  // MaxSat free variables
  bool int_mode = false;
  // device copy, made on first use (model construction needs no GPU)
  mutable DevBuf dmem;
  mutable DevModel dev{};
  mutable bool uploaded = false;
  mutable int upload_device = -1;  // CUDA ordinal that holds dmem

  bool empty() const { return N == 0; }
  void upload() const;
  const DevModel& device() const
  {
    if (!uploaded) upload();
    return dev;
  }
  DevModel device_view(bool full_maxsat_sweep) const;
};

// Build from the raw term list (reference input order).
std::unique_ptr<HostModel> build_model(int kind, int64_t n_terms,
                                       const int64_t* off, const int32_t* ids,
                                       const double* coef);
std::unique_ptr<HostModel> build_model_json(const json::Value& doc, int kind);
// DIMACS cnf / wcnf text -> MaxSat model (dimacs.cc)
std::unique_ptr<HostModel> build_model_dimacs(const std::string& text);
// protobuf problem folder <name>/<name>_<k>.pb -> model (proto.cc)
std::unique_ptr<HostModel> build_model_proto_folder(const std::string& folder_path);
// bounds on one flip's cost difference (parameter-free solvers)
double estimate_max_cost_diff(const HostModel& m);
double estimate_min_cost_diff(const HostModel& m);

// Schedule (schedule/schedule.cc, linear.cc, geometric.cc, segments.cc).
struct Schedule
{
  int type = 0;  // 0 linear, 1 geometric, 2 constant, 3 list
  double initial = 0, final_ = 0;
  bool has_start = false, has_stop = false, has_count = false;
  double start_ = 0, stop_ = 1;
  int count_ = 1;
  std::vector<double> values;
  double progress_value(double p) const;
  double get_start() const;
  double get_stop() const;
  int get_count() const;
  double get_value(double input) const;
  std::vector<double> discretized() const;
  std::string render() const;
};
Schedule parse_schedule(const json::Value& v, const std::string& name);

class Solver;
std::unique_ptr<Solver> make_solver(const HostModel* m, const std::string& target,
                                    const json::Value& params_doc);

class Solver
{
 public:
  virtual ~Solver() {}
  virtual void init(cudaStream_t s) = 0;
  virtual void run(cudaStream_t s) = 0;
  // results
  virtual int64_t n_walkers() const = 0;
  virtual void fetch(std::vector<double>& cost, std::vector<double>& lowest,
                     std::vector<uint64_t>& att, std::vector<uint64_t>& acc,
                     std::vector<uint8_t>* lowest_states,
                     std::vector<uint8_t>* states) = 0;
  virtual void pt_observables(std::vector<double>& out) { out.clear(); }
  // lowest state ever seen by a population solver (it may have died)
  virtual bool historical_lowest(double&, std::vector<uint8_t>&) { return false; }
  virtual std::string target() const = 0;
  virtual uint64_t total_windows() { return 0; }
  // the walker whose lowest is the solver's lowest (default: the first with
  // the smallest lowest cost)
  virtual size_t best_index(const std::vector<double>& low)
  {
    size_t b = 0;
    for (size_t i = 1; i < low.size(); i++)
      if (low[i] < low[b]) b = i;
    return b;
  }
  // extra members of the result's benchmark block (JSON, starting with ',')
  virtual std::string extra_benchmark() { return ""; }
  // walkers per solution candidate: the solutions list takes walkers
  // 0, stride, 2 stride, ... (QMC: one candidate per restart, not per slice)
  virtual size_t solution_stride() const { return 1; }
  // Serving: the solve in pieces.  After init(), advance() enqueues up to n
  // further steps on the stream and returns true once the step budget is
  // spent (results are read after the stream has finished).  The pieces
  // give the same trajectory as run().
  virtual bool advance(cudaStream_t s, int64_t n);
  int64_t step_pos = 0;
  std::string result_json();
  // keys a runner adds to the benchmark object (app/runner.cc:546-631)
  std::string runner_benchmark;
  void best(double& cost, std::vector<uint8_t>& state);

  const HostModel* model = nullptr;
  json::Value params;            // the "params" object as given
  std::vector<std::pair<std::string, std::string>> output_params;  // rendered
  uint32_t seed = 0;
  int64_t step_limit = 10000;
  int64_t last_step = 0;
  bool has_cost_limit = false;
  double cost_limit = 0;
  bool has_time_limit = false;
  double time_limit = 0;
  int threads = 1;
  int number_of_solutions = 1;
  bool replay = true;
  bool full_maxsat_sweep = false;
  int warps_per_block = 0;  // 0: pick from the walker count
  uint64_t launches = 0;
  double sweep_ms = 0, run_ms = 0;
  uint64_t near_ties = 0;
  int64_t device_bytes = 0;
  int used_kernel = 1;     // kernel of the last sweeps (numbered as `kernel`)
  bool initialized = false, ran = false;
  bool profile = false;  // bracket every sweep launch with CUDA events
  bool smem_state = true;  // walker state in shared memory when it fits
  int kernel = 0;          // sweep kernel: 0 auto, 1 one walker per warp, 2 one walker per lane,
                           // 3 level schedule (one walker per warp, counter streams),
                           // 4 cached local fields (two warps per walker)
  bool auto_fields = true;  // "auto" may pick the cached-field sweep (the server's solves do not)
  // CUDA-event pairs around sweep launches (profile mode)
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_events;
  size_t prof_used = 0;
  void prof_begin(cudaStream_t s);
  void prof_end(cudaStream_t s);
  double prof_total_ms();  // synchronises; resets the pairs
};
// Lane-per-walker execution (lanes.cu): the group layout of the walkers,
// the device copy of their model descriptors, and the transposes between a
// population's bit-packed layout and the groups' interleaved words.
// Sweep log of the level kernel (levels.cu): per walker and logged sweep its
// start spins, start cost and attempt differences.  Launches longer than the
// log's sweeps are cut into pieces of that many sweeps.
struct LevelLog
{
  DevBuf buf;
  int walkers = 0, sweeps = 0;
  size_t off_cost = 0, off_diff = 0;
  long long stride = 0;
  int bytes_per_diff = 1;
  // room for R walkers and up to K sweeps (fewer when the log would exceed
  // its byte budget); returns the bytes held
  size_t ensure(int R, int64_t K, const HostModel& m, int nw);
  void fill(LvArgs& a) const;
};

struct LaneRunner
{
  DevBuf meta, arena;
  LwArgs a{};
  int max_words = 0, max_terms = 0;
  bool ready = false;
  // walker r runs models[model_of[r]] (model_of empty: models[0] for all);
  // local_of[r]: its index within its own solve, for counter keys
  // smem: hold the group words in shared memory when they fit (with fewer
  // than 32 lanes per group if that is what makes them fit)
  void setup(const std::vector<DevModel>& models, const std::vector<int>& model_of, int n_walkers,
             const std::vector<int>& local_of = {}, bool smem = true);
  size_t bytes() const { return meta.bytes + arena.bytes; }
};
bool lanes_eligible(const HostModel& m);
// the lane kernel for this solver and walker count (params "kernel"; auto:
// eligible models with at least 1024 walkers)
bool lanes_for(const Solver& s, const HostModel& m, int64_t walkers);
bool levels_eligible(const HostModel& m);
bool levels_for(const Solver& s, const HostModel& m);

// Many independent solves of the same target and params (one per model).
struct BatchStats
{
  double run_ms = 0;
  int64_t launches = 0, walkers = 0, device_bytes = 0;
  int kernel = 0, warps_per_block = 0, smem = 0, graph = 0;
  double sweep_kernel_ms = 0;
};
class Batch
{
 public:
  virtual ~Batch() {}
  virtual void run(cudaStream_t s) = 0;
  virtual int n_instances() const = 0;
  virtual std::string result_json(int instance) = 0;
  virtual void lowest(double* out) = 0;  // per instance: best lowest cost + const cost
  const BatchStats& stats() const { return stats_; }

 protected:
  BatchStats stats_;
};
std::unique_ptr<Batch> make_batch(const std::vector<const HostModel*>& models, const std::string& target,
                                  const json::Value& params_doc);
// Continuous batching of solve requests (serve.cc).
struct ServerStats
{
  int64_t submitted = 0, completed = 0, failed = 0, active = 0, pending = 0;
  int64_t used_bytes = 0, budget_bytes = 0, peak_active = 0;
  double elapsed_s = 0, p50_ms = 0, p99_ms = 0, max_ms = 0;
};
class Server
{
 public:
  virtual ~Server() {}
  // validates params; the model must stay alive until the request finishes
  virtual int64_t submit(const HostModel* m, const std::string& target, const json::Value& params_doc) = 0;
  // 0 pending, 1 running, 2 done (out: result JSON), 3 failed (out: message)
  virtual int poll(int64_t id, std::string* out) = 0;
  virtual int wait(int64_t id, double timeout_s, std::string* out) = 0;
  virtual void forget(int64_t id) = 0;
  virtual int64_t request_bytes(int64_t id) = 0;  // device footprint used for admission
  virtual ServerStats stats() = 0;
};
// budget_bytes <= 0: half of the device's free memory
std::unique_ptr<Server> make_server(int64_t budget_bytes, int max_active, int64_t sa_piece, int64_t pt_piece);
}  // namespace qio
