// serve.cc -- continuous batching of solve requests on one GPU.
//
// No counterpart in the reference, which solves one problem per process
// (app/runner.cc:513-631).  A request is a model, a target and params, solved
// exactly as qio_solver_* would solve it.  A worker thread admits pending
// requests in arrival order whenever a slot is free and their device
// footprint (model + walker population) fits the memory budget, lets a later
// request overtake one that does not fit yet, and keeps every admitted solve
// resident: its population (spins, term caches, temperature ladder, streams)
// stays on the device between pieces.  Each admitted solve owns a CUDA stream
// and advances in pieces of sweeps (SA) or steps (PT); a piece is enqueued as
// soon as the previous one has finished, so the pieces of all admitted
// solves overlap on the GPU.  A solve retires when its sweep budget is
// spent: its result JSON is rendered, its device memory freed, and the next
// pending requests are admitted.  Pieces replay the same trajectory as one
// run, so a result is the same whether the request ran alone or in a mix.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>

#include "host.h"

namespace qio
{
namespace
{
using Clock = std::chrono::steady_clock;

struct Request
{
  int64_t id = 0;
  const HostModel* model = nullptr;
  std::unique_ptr<Solver> solver;
  int64_t footprint = 0;
  double work = 0;  // one walker's chain: incidences x sweeps
  int state = 0;  // 0 pending, 1 running, 2 done, 3 failed
  Clock::time_point t_submit, t_admit, t_done;
  std::string result, error;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  bool finished = false;  // last piece enqueued
  int64_t piece = 1;
};

int64_t model_bytes(const HostModel& m)
{
  return (int64_t)(m.row.size() * 4 + m.inc.size() * 4 + m.coef.size() * 8 + m.coef_i.size() * 4 +
                   m.coef_f.size() * 4 + m.near.size() * 8 + m.nbr.size() * 4 + m.trow.size() * 4 +
                   m.tvar.size() * 4 + m.tcost.size() * 8 + m.tcost_i.size() * 4 + m.other.size() * 4 +
                   m.rec_i.size() * 4 + m.rec_f.size() * 8 + m.rec_p.size() * 4 + m.lv_off.size() * 4 +
                   m.lv_ent.size() * 4 + m.lv_pos.size() * 4 + 19 * 256);
}

// device bytes of a solve: the model blob and the walker population
int64_t footprint_of(const HostModel& m, const Solver& s)
{
  const int64_t W = std::max<int64_t>(1, s.n_walkers());
  const int64_t nw = ((m.N + 31) / 32 + 3) & ~3LL;
  const int64_t mp = std::max<int64_t>(16, (m.M + 15) & ~15LL);
  // spins, lowest spins, term states, per-walker scalars
  const int64_t per = 2 * nw * 4 + mp + 10 * 8;
  const int64_t steps = std::max<int64_t>(1, s.step_limit);
  // the level kernel's sweep log (at most 64 sweeps, at most 4 GiB)
  int64_t lv = 0;
  if (m.lv_ok)
  {
    const int64_t per_sweep = nw * 4 + 16 + ((m.N + 31) & ~31LL) * (m.lv_d8 ? 1 : 4);
    lv = std::min<int64_t>((int64_t)4 << 30, W * std::min<int64_t>(64, steps) * per_sweep);
  }
  // tabu search: tabu list and two cost-difference arrays per walker, the
  // hill climber's spins and state
  const int64_t tabu = s.target() == "tabu.qiotoolkit" ? W * (24 * m.N + 2 * nw * 4 + 64) : 0;
  // substochastic Monte Carlo: a second population (the resampling copies
  // into it), the copy map and init streams; quantum Monte Carlo: per step
  // beta and bond limits, per restart its lowest (walkers are its slices)
  int64_t extra = 0;
  if (s.target() == "substochasticmontecarlo.cpu") extra = W * (per + 12) + nw * 4;
  if (s.target() == "quantummontecarlo.qiotoolkit") extra = steps * 17 + W * (8 + nw * 4);
  return model_bytes(m) + W * per + steps * 8 + W * 64 + lv + tabu + extra + 64 * 1024;
}
}  // namespace

class ServerImpl : public Server
{
 public:
  ServerImpl(int64_t budget, int max_active, int64_t sa_piece, int64_t pt_piece)
      : budget_(budget), max_active_(max_active), sa_piece_(sa_piece), pt_piece_(pt_piece)
  {
    t0_ = Clock::now();
    worker_ = std::thread([this] { loop(); });
  }

  ~ServerImpl() override
  {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    if (worker_.joinable()) worker_.join();
    // solves still running: let their pieces finish before freeing memory
    for (auto& kv : all_)
      if (kv.second->stream) cudaStreamSynchronize(kv.second->stream);
    for (auto& kv : all_) release(*kv.second);
  }

  int64_t submit(const HostModel* m, const std::string& target, const json::Value& doc) override
  {
    std::unique_ptr<Request> r(new Request());
    r->model = m;
    r->solver = make_solver(m, target, doc);  // params are validated here
    // "auto" keeps the windowed sweep for served solves: a mix is bound by
    // its longest chain, where the field-cached sweep gains nothing, and one
    // run with 200 solves in flight on it ended in an illegal-address fault
    // that was not located (a request may still ask for "fields")
    r->solver->auto_fields = false;
    if (r->solver->has_cost_limit || r->solver->has_time_limit)
      fail(1, "served solves run their full sweep budget: `cost_limit` and `timeout` are not supported");
    r->footprint = footprint_of(*m, *r->solver);
    r->work = (double)std::max<int64_t>(1, m->K) * (double)std::max<int64_t>(1, r->solver->step_limit);
    if (r->footprint > budget_)
      fail(2, "request needs " + std::to_string(r->footprint) + " device bytes; the server's budget is " +
                  std::to_string(budget_));
    r->piece = target == "paralleltempering.qiotoolkit" ? pt_piece_ : sa_piece_;
    // the model goes to the device in the caller's thread, before the
    // worker reads it
    ensure_device();
    if (!m->empty()) m->device();
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> g(mu_);
    r->id = next_id_++;
    const int64_t id = r->id;
    pending_.push_back(r.get());
    all_[id] = std::move(r);
    submitted_++;
    cv_.notify_all();
    return id;
  }

  int poll(int64_t id, std::string* out) override
  {
    std::lock_guard<std::mutex> g(mu_);
    auto it = all_.find(id);
    if (it == all_.end()) fail(1, "unknown request " + std::to_string(id));
    Request& r = *it->second;
    if (out && r.state == 2) *out = r.result;
    if (out && r.state == 3) *out = r.error;
    return r.state;
  }

  int wait(int64_t id, double timeout_s, std::string* out) override
  {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = all_.find(id);
    if (it == all_.end()) fail(1, "unknown request " + std::to_string(id));
    Request* r = it->second.get();
    auto pred = [&] { return r->state >= 2; };
    if (timeout_s < 0) done_cv_.wait(lk, pred);
    else done_cv_.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
    if (out && r->state == 2) *out = r->result;
    if (out && r->state == 3) *out = r->error;
    return r->state;
  }

  void forget(int64_t id) override
  {
    std::lock_guard<std::mutex> g(mu_);
    auto it = all_.find(id);
    if (it == all_.end()) fail(1, "unknown request " + std::to_string(id));
    if (it->second->state < 2) fail(1, "request " + std::to_string(id) + " has not finished");
    all_.erase(it);
  }

  int64_t request_bytes(int64_t id) override
  {
    std::lock_guard<std::mutex> g(mu_);
    auto it = all_.find(id);
    if (it == all_.end()) fail(1, "unknown request " + std::to_string(id));
    return it->second->footprint;
  }

  ServerStats stats() override
  {
    std::lock_guard<std::mutex> g(mu_);
    ServerStats st;
    st.submitted = submitted_;
    st.completed = (int64_t)latencies_.size();
    st.failed = failed_;
    st.active = (int64_t)active_.size();
    st.pending = (int64_t)pending_.size();
    st.used_bytes = used_;
    st.budget_bytes = budget_;
    st.peak_active = peak_active_;
    st.elapsed_s = std::chrono::duration<double>(Clock::now() - t0_).count();
    if (!latencies_.empty())
    {
      std::vector<double> v = latencies_;
      std::sort(v.begin(), v.end());
      auto pct = [&](double q) {
        size_t k = (size_t)std::ceil(q * (double)v.size()) - 1;
        return v[std::min(k, v.size() - 1)];
      };
      st.p50_ms = pct(0.50);
      st.p99_ms = pct(0.99);
      st.max_ms = v.back();
    }
    return st;
  }

 private:
  int64_t budget_;
  int max_active_;
  int64_t sa_piece_, pt_piece_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::thread worker_;
  bool stop_ = false;
  std::deque<Request*> pending_;
  std::vector<Request*> active_;
  std::map<int64_t, std::unique_ptr<Request>> all_;
  int64_t next_id_ = 1, used_ = 0, submitted_ = 0, failed_ = 0, peak_active_ = 0;
  std::vector<double> latencies_;
  Clock::time_point t0_;

  void release(Request& r)
  {
    if (r.ev) cudaEventDestroy(r.ev);
    if (r.stream) cudaStreamDestroy(r.stream);
    r.ev = nullptr;
    r.stream = nullptr;
    r.solver.reset();
  }

  // finished or failed: free the device memory, record the latency
  void retire(Request* r, bool ok, const std::string& msg)
  {
    release(*r);
    std::lock_guard<std::mutex> g(mu_);
    r->t_done = Clock::now();
    used_ -= r->footprint;
    active_.erase(std::find(active_.begin(), active_.end(), r));
    if (ok)
    {
      r->state = 2;
      r->result = msg;
      latencies_.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
    }
    else
    {
      r->state = 3;
      r->error = msg;
      failed_++;
    }
    done_cv_.notify_all();
  }

  // admitted solve: its stream, its population, its first piece
  void start(Request* r)
  {
    try
    {
      // the longer a walker's chain, the higher its stream's priority: when
      // the admitted solves' blocks outnumber the GPU's slots, the block
      // scheduler starts the pieces of the longest chains first (a mix ends
      // with its longest chain)
      int least = 0, greatest = 0;
      cuda_check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "cudaDeviceGetStreamPriorityRange");
      const int levels = least - greatest;
      const int level = (int)std::max(0.0, std::min((double)levels, std::floor(std::log2(r->work / 1e6))));
      cuda_check(cudaStreamCreateWithPriority(&r->stream, cudaStreamNonBlocking, least - level),
                 "cudaStreamCreate");
      cuda_check(cudaEventCreateWithFlags(&r->ev, cudaEventDisableTiming), "cudaEventCreate");
      r->solver->init(r->stream);
      r->finished = r->solver->advance(r->stream, r->piece);
      cuda_check(cudaEventRecord(r->ev, r->stream), "cudaEventRecord");
    }
    catch (const std::exception& e)
    {
      retire(r, false, e.what());
    }
  }

  // poll one running solve: enqueue its next piece or retire it
  bool service(Request* r)
  {
    cudaError_t q = cudaEventQuery(r->ev);
    if (q == cudaErrorNotReady) return false;
    try
    {
      if (q != cudaSuccess) cuda_check(q, "solve piece");
      if (r->finished)
      {
        cuda_check(cudaStreamSynchronize(r->stream), "sync");
        check_device_error(r->stream);
        std::string res = r->solver->result_json();
        retire(r, true, res);
        return true;
      }
      r->finished = r->solver->advance(r->stream, r->piece);
      cuda_check(cudaEventRecord(r->ev, r->stream), "cudaEventRecord");
    }
    catch (const std::exception& e)
    {
      retire(r, false, e.what());
    }
    return true;
  }

  void loop()
  {
    for (;;)
    {
      std::vector<Request*> admitted, running;
      {
        std::unique_lock<std::mutex> lk(mu_);
        if (stop_) return;
        // first fit in arrival order
        for (auto it = pending_.begin(); it != pending_.end();)
        {
          Request* r = *it;
          if ((int)active_.size() >= max_active_) break;
          if (used_ + r->footprint <= budget_)
          {
            used_ += r->footprint;
            r->state = 1;
            r->t_admit = Clock::now();
            active_.push_back(r);
            admitted.push_back(r);
            it = pending_.erase(it);
          }
          else
            ++it;
        }
        peak_active_ = std::max<int64_t>(peak_active_, (int64_t)active_.size());
        if (active_.empty())
        {
          cv_.wait(lk, [&] { return stop_ || !pending_.empty(); });
          continue;
        }
        running = active_;
      }
      for (Request* r : admitted) start(r);
      bool progressed = !admitted.empty();
      for (Request* r : running)
        if (std::find(admitted.begin(), admitted.end(), r) == admitted.end() && r->state == 1)
          progressed = service(r) || progressed;
      if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
  }
};

std::unique_ptr<Server> make_server(int64_t budget_bytes, int max_active, int64_t sa_piece, int64_t pt_piece)
{
  if (max_active <= 0) fail(1, "server: `max_active` must be positive");
  if (sa_piece <= 0 || pt_piece <= 0) fail(1, "server: piece sizes must be positive");
  if (budget_bytes <= 0)
  {
    ensure_device();
    size_t free_b = 0, total_b = 0;
    cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    budget_bytes = (int64_t)(free_b / 2);
  }
  return std::unique_ptr<Server>(new ServerImpl(budget_bytes, max_active, sa_piece, pt_piece));
}
}  // namespace qio
