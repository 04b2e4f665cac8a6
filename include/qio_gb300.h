/*
 * qio_gb300.h -- C ABI of the GB300 Metropolis library (libqio_gb300.so).
 *
 * The reference (QIOToolkit) binds models and solvers at compile time as C++
 * templates; this header is the plain-C boundary that a reference-side
 * plugin binds instead.  Each entry point names the reference interface it
 * replaces (paths relative to the reference's cpp/ directory).
 *
 * Conventions
 *   - Every call returns qio_status; on failure qio_last_error_message()
 *     (thread-local) holds the reason, worded like the reference's
 *     exceptions where the reference pins a message.
 *   - Host buffers only cross this boundary; device memory is owned by the
 *     library.  `stream` arguments are cudaStream_t values passed as void*
 *     (NULL = the legacy default stream).
 *   - Spin/variable states are arrays of uint8 in the model's internal
 *     variable order (0 = false, 1 = true).  For Ising, true = spin -1; for
 *     PUBO, true = variable value 0 (the reference's convention,
 *     model/pubo.h:191-276); for MaxSAT, true = variable true.
 *   - Handles are independent; one handle is used by one host thread at a
 *     time.
 */
#ifndef QIO_GB300_H
#define QIO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum qio_status {
  QIO_OK = 0,
  QIO_INVALID_ARGUMENT = 1, /* utils::ValueException and friends           */
  QIO_OUT_OF_MEMORY = 2,    /* utils::MemoryLimitedException               */
  QIO_CUDA_ERROR = 3,       /* a CUDA call failed                          */
  QIO_TIMEOUT = 4,          /* a bounded device wait gave up               */
  QIO_NO_DEVICE = 5,        /* no CUDA device: there is no CPU fallback    */
  QIO_INTERNAL = 6
} qio_status;

typedef enum qio_model_kind {
  QIO_ISING = 0,       /* model::IsingTermCached, model/ising.h:331-342      */
  QIO_ISING_PLAIN = 1, /* model::Ising, model/ising.h:292-301                */
  QIO_PUBO = 2,        /* model::PuboWithCounter<T>, model/pubo.h:285-399    */
  QIO_PUBO_PLAIN = 3,  /* model::Pubo, model/pubo.h:221-231                  */
  QIO_MAXSAT = 4       /* model::MaxSat<T>, model/max_sat.h:96-599           */
} qio_model_kind;

typedef struct qio_model qio_model;
typedef struct qio_solver qio_solver;

typedef struct qio_model_info {
  int32_t kind;
  int32_t integer_weights; /* 1: all coefficients are small integers (exact
                              integer arithmetic on the device)            */
  int64_t n_vars;
  int64_t n_terms;
  int64_t n_incidences;    /* sum of term orders                          */
  int32_t max_locality;
  int32_t min_locality;
  double const_cost;       /* Graph::get_const_cost, graph/graph.h:214   */
  double scale_factor;     /* GraphProperties::rescale factor (1/max|c| if
                              max|c| > 1), graph/graph_properties.h:24-40 */
  double max_coupling;
  int64_t device_bytes;    /* HBM held by the model                       */
  int32_t n_levels;        /* level schedule of the ordered sweep (integer
                              Ising models with one- or two-member terms):
                              its levels and the most variables in one
                              level, or 0                                 */
  int32_t max_level_width;
  int32_t level_kernel;    /* 1: the level kernel can run this model      */
  /* graph::Size properties (graph/properties.h:52-68; graph models only):
   * the mean term order over non-constant terms, the sum of term orders,
   * the sum of order * (order - 1), the smallest |coefficient| */
  double avg_locality;
  int64_t sum_coefficient_degrees_total;
  int64_t accumulated_dependent_vars;
  double min_coupling;
} qio_model_info;

typedef struct qio_solver_stats {
  int64_t replicas;        /* walkers (SA restarts, PT slots, PA citizens) */
  int64_t last_step;       /* SteppingSolver step_, solver/stepping_solver.h:369 */
  uint64_t attempts;       /* difference evaluations (flip attempts)       */
  uint64_t accepts;        /* accepted transitions                         */
  uint64_t kernel_launches;/* kernels launched by qio_solver_run           */
  double sweep_kernel_ms;  /* CUDA-event time of the sweep kernels         */
  double run_ms;           /* CUDA-event time of the whole run             */
  uint64_t near_ties;      /* PT swaps whose uniform draw was within 1e-15 of
                              the device exp(), decided with the correctly
                              rounded exp instead                          */
  int64_t device_bytes;    /* HBM held by the solver                       */
  uint64_t windows;        /* 32-variable evaluation windows committed; the
                              mean committed window is attempts / windows */
  int32_t sweep_kernel;    /* kernel of the last sweeps: 1 one walker per
                              warp, 2 one walker per lane, 3 level schedule,
                              4 tabu search (one walker per warp),
                              5 substochastic Monte Carlo walker steps,
                              6 quantum Monte Carlo (one warp per restart),
                              7 quantum Monte Carlo level schedule (counter
                              streams, one block per restart), 8 cached
                              local fields (two warps per walker) */
} qio_solver_stats;

/* ---- library ---------------------------------------------------------- */
const char* qio_last_error_message(void);
const char* qio_version(void);
/* Releases a buffer returned by the library (result JSON). */
void qio_free(void* p);

/* ---- model ------------------------------------------------------------ */

/* Build a model from the raw term list of the reference's input format
 * ("cost_function": {"terms": [{"c": c, "ids": [...]}, ...]}).
 * Replaces GraphModel::configure -> Graph::init -> normalize_edges
 * (graph/graph.h:368-397,517-534,74-177) for graph models and
 * MaxSat::configure(clauses) (model/max_sat.h:262-397) for QIO_MAXSAT:
 * ids are renumbered by first appearance (MaxSAT: sorted by name), member ids
 * are sorted, duplicate ids throw (Ising) or merge (PUBO), empty terms fold
 * into the constant cost.
 *   term_offsets: n_terms + 1 offsets into term_ids
 *   term_ids:     variable names (MaxSAT: signed literals, -v = negated) */
qio_status qio_model_create(int32_t kind, int64_t n_terms,
                            const int64_t* term_offsets,
                            const int32_t* term_ids,
                            const double* coefficients, qio_model** out);

/* Same, from the reference's JSON input document ({"cost_function": {...}}).
 * kind < 0 selects by "type" as app/runner.cc:255-429 does (ising ->
 * QIO_ISING, pubo -> QIO_PUBO, maxsat -> QIO_MAXSAT). */
qio_status qio_model_create_json(const char* input_json, int32_t kind,
                                 qio_model** out);

/* MaxSAT model from DIMACS cnf / wcnf text (utils/dimacs.cc, read by
 * app/runner.cc:87-89 into model::MaxSat): the same accepted input and
 * error messages. */
qio_status qio_model_create_dimacs(const char* text, qio_model** out);
/* Model from a protobuf problem folder <name>/<name>_0.pb, _1.pb, ...
 * (utils/proto_reader.h:28-150, schema utils/problem.proto, read by
 * utils::configure_from_proto_folder): the first file holds the type,
 * version and first terms, later files more terms. */
qio_status qio_model_create_proto_folder(const char* folder_path, qio_model** out);
/* Bounds on one flip's cost difference that the parameter-free solvers
 * derive their temperature ranges from: GraphModel / Ising / Pubo
 * estimate_min_cost_diff and estimate_max_cost_diff (model/ising.h:176-224,
 * model/pubo.h:127-184, graph/graph.h:453-485).  Ising and PUBO models. */
qio_status qio_model_cost_diff_bounds(const qio_model* model, double* min_diff, double* max_diff);
/* The Bayesian search strategy of the population-annealing and
 * substochastic parameter-free solvers (strategy/bayesian.h:14-78,
 * BayesianOpt::add_new_sample + recommend_parameter_values), for callers
 * that run their own parameter searches: from n >= 2 samples xs (n x dims,
 * row-major) with objectives ys, `count` points (count x dims) inside the
 * box [lo, hi] that a Gaussian-process model expects to improve on the
 * lowest objective.  Deterministic for a seed; host only. */
qio_status qio_bayes_recommend(int32_t dims, const double* lo, const double* hi, int32_t n,
                               const double* xs, const double* ys, uint32_t seed, int32_t count,
                               double* out);

qio_status qio_model_get_info(const qio_model* model, qio_model_info* out);
/* Original variable name of each internal variable (Graph::output_map,
 * graph/graph.h:407-413; MaxSat variable_names_, model/max_sat.h:596). */
qio_status qio_model_get_var_names(const qio_model* model, int32_t* names);
qio_status qio_model_destroy(qio_model* model);

/* ---- per-state contract (markov/model.h:79-149), evaluated on the GPU --- */

/* calculate_cost for n_states states (n_states x n_vars bytes); the sum runs
 * in the reference's term order, so results are bit-identical to it. */
qio_status qio_states_cost(const qio_model* model, int64_t n_states,
                           const uint8_t* states, double* costs, void* stream);
/* calculate_cost for n_states states that are already in device memory
 * (states: n_states x n_vars bytes, costs: n_states doubles, both device
 * pointers), with no allocation: no counterpart in the reference.  For
 * callers that must not allocate device memory during a call (a serving
 * loop whose HBM is held by resident solves; a thread that cannot take the
 * device-wide synchronisation of cudaMalloc/cudaFree).  Scratch is a fixed
 * 1 MiB array inside the library: n_states * ceil(n_vars / 32) must not
 * exceed 262144 words (QIO_INVALID_ARGUMENT otherwise).  All calls share it:
 * overlapping calls (other streams or threads) race and must be serialised
 * by the caller.  The first call on a device looks up the array's address
 * and loads the kernels of every model flavour; make it before any stream
 * capture.  The model must already be on the current device (an earlier
 * qio_states_cost or solver call there; another current device is
 * QIO_INVALID_ARGUMENT), and states / costs must be device (or managed)
 * memory of that device (host pointers are QIO_INVALID_ARGUMENT).  Results
 * equal qio_states_cost's; the call is asynchronous on `stream`. */
qio_status qio_states_cost_noalloc(const qio_model* model, int64_t n_states,
                                   const uint8_t* states, double* costs, void* stream);
/* calculate_cost_difference(state q, vars[q]) for n queries. */
qio_status qio_states_cost_difference(const qio_model* model, int64_t n,
                                      const uint8_t* states,
                                      const int64_t* vars, double* diffs,
                                      void* stream);
/* apply_transition(vars[q]) on each state (host buffers, in place). */
qio_status qio_states_apply(const qio_model* model, int64_t n,
                            uint8_t* states, const int64_t* vars);

/* ---- solvers ---------------------------------------------------------- */

/* Create a solver for `target` ("simulatedannealing.qiotoolkit",
 * "paralleltempering.qiotoolkit", "populationannealing.cpu", and beside the
 * path "tabu.qiotoolkit", "substochasticmontecarlo.cpu",
 * "quantummontecarlo.qiotoolkit" and the parameter-free searches
 * "simulatedannealing-parameterfree.qiotoolkit",
 * "paralleltempering-parameterfree.qiotoolkit",
 * "tabu-parameterfree.qiotoolkit", "populationannealing-parameterfree.cpu",
 * "substochasticmontecarlo-parameterfree.cpu") configured from
 * the reference's params JSON ({"params": {...}}): replaces
 * create_model_solver (app/runner.cc:134-193) + Solver::configure
 * (solver/solver.h:156-218 and the solver-specific configure()).  Options
 * beyond the reference's ride in the same object:
 *   "rng_mode": "replay" (default; the reference's PCG streams, trajectories
 *               identical to it) or "counter" (independent counter-based
 *               streams keyed by walker, sweep and variable);
 *   "restarts" (PT): independent tempering ladders, ladder k seeded seed+k;
 *   "maxsat_full_sweep": attempt every MaxSAT variable per sweep (the
 *               reference's MaxSat sweep is one attempt, markov/model.h:169);
 *   "warps_per_block", "profile_kernels": launch shape and per-launch
 *               CUDA-event timing of the sweep kernels. */
qio_status qio_solver_create(const qio_model* model, const char* target,
                             const char* params_json, qio_solver** out);
/* Solver::init (random initial states, solver/simulated_annealing.h:45-74). */
qio_status qio_solver_init(qio_solver* s, void* stream);
/* SteppingSolver::run (solver/stepping_solver.h:112-268): all steps on the
 * device; returns after the stream has drained. */
qio_status qio_solver_run(qio_solver* s, void* stream);
/* finalize + get_result (solver/model_solver.h:111-150,301-308,
 * solver/solver.h:147-153): result JSON {"benchmark": ..., "solutions": ...}.
 * The string is released with qio_free. */
qio_status qio_solver_result_json(qio_solver* s, char** out_json);
/* Per-walker results (NULL outputs are skipped); *n receives the count.
 * lowest_states / states: n x n_vars bytes. */
qio_status qio_solver_replicas(qio_solver* s, int64_t* n, double* cost,
                               double* lowest, uint64_t* attempts,
                               uint64_t* accepts, uint8_t* lowest_states,
                               uint8_t* states);
/* Best solution over all walkers: cost includes the constant terms. */
qio_status qio_solver_best(qio_solver* s, double* cost, uint8_t* state);
qio_status qio_solver_get_stats(qio_solver* s, qio_solver_stats* out);
/* PT observables averaged over steps per temperature slot and restart:
 * (T or beta, acc_rate, avg_cost, avg_dir, swap_rate) x slots x restarts,
 * as the reference's observer renders them
 * (solver/parallel_tempering.h:142-186). */
qio_status qio_solver_pt_observables(qio_solver* s, double* out5);
qio_status qio_solver_destroy(qio_solver* s);

/* ---- batches: many independent solves in one device graph ------------
 * No counterpart in the reference, which solves one model per run
 * (app/runner.cc:513-631).  Every instance gets the same target and params;
 * instance i's result equals a plain solve of models[i] with them (the same
 * walkers, streams, counters and result JSON).  Target
 * "simulatedannealing.qiotoolkit".  Extra params keys: "autotune" (time the
 * lane-kernel launch shapes on a short trial, default true), "graph"
 * (capture the whole run in one CUDA graph, default true), "kernel".
 * The models must outlive the batch. */
typedef struct qio_batch qio_batch;
typedef struct qio_batch_stats {
  double run_ms;            /* last run: CUDA events around it              */
  int64_t launches;         /* kernel launches per run (one init per
                               instance; one sweep launch per kind of model
                               with the windowed kernel's queue, else one
                               per instance)                               */
  int64_t walkers;          /* instances x restarts                         */
  int64_t device_bytes;     /* population + lane groups                     */
  int32_t kernel;           /* 1: one walker per warp, 2: one walker per lane */
  int32_t warps_per_block;  /* lane plan (0: spread the groups over the SMs);
                               windowed kernel: walkers per block of its
                               persistent queue launches                   */
  int32_t smem;             /* 1: walker words in shared memory             */
  int32_t graph;            /* 1: each run is one captured CUDA graph       */
  double sweep_kernel_ms;   /* "graph": false with "profile_kernels": true:
                               CUDA events around the sweep launches       */
} qio_batch_stats;
qio_status qio_batch_create(const qio_model* const* models, int32_t n_models, const char* target,
                            const char* params_json, qio_batch** out);
/* init + all sweeps of every instance; returns when they are done */
qio_status qio_batch_run(qio_batch* batch, void* stream);
/* instance's result JSON, the shape qio_solver_result_json gives */
qio_status qio_batch_result_json(qio_batch* batch, int32_t instance, char** out_json);
/* best cost per instance (lowest over its walkers + constant terms) */
qio_status qio_batch_lowest(qio_batch* batch, double* costs);
qio_status qio_batch_get_stats(const qio_batch* batch, qio_batch_stats* out);
qio_status qio_batch_destroy(qio_batch* batch);

/* ---- serving: continuous batching of solve requests -------------------
 * No counterpart in the reference (one solve per process).  A worker thread
 * admits requests in arrival order when a slot is free and their device
 * footprint (model + walker population) fits the memory budget (a later
 * request may overtake one that does not fit yet), keeps each admitted
 * solve resident on the device, advances all of them in overlapping pieces
 * on their own streams, and retires a solve when its sweep budget is spent.
 * A request's result JSON equals qio_solver_*'s for the same model, target
 * and params, alone or in any mix.  Targets: simulated annealing and
 * parallel tempering; `cost_limit` / `timeout` are rejected.
 * config_json: {"memory_budget_bytes": B (default: half the free device
 * memory), "max_active": A (default 64), "sa_sweeps_per_piece": 64,
 * "pt_steps_per_piece": 16}. */
typedef struct qio_server qio_server;
typedef struct qio_server_stats {
  int64_t submitted, completed, failed, active, pending;
  int64_t used_bytes, budget_bytes, peak_active;
  double elapsed_s;          /* since creation                               */
  double p50_ms, p99_ms, max_ms;  /* submit-to-done latency of completed ones */
} qio_server_stats;
qio_status qio_server_create(const char* config_json, qio_server** out);
/* the model must stay alive until the request has finished */
qio_status qio_server_submit(qio_server* server, const qio_model* model, const char* target,
                             const char* params_json, int64_t* request_id);
/* state: 0 pending, 1 running, 2 done (*out_json = result), 3 failed
 * (*out_json = message); *out_json is set only then (free with qio_free) */
qio_status qio_server_poll(qio_server* server, int64_t request_id, int32_t* state, char** out_json);
/* as poll, blocking until the request is done or failed (timeout_s < 0:
 * no limit) */
qio_status qio_server_wait(qio_server* server, int64_t request_id, double timeout_s, int32_t* state,
                           char** out_json);
/* drop a finished request's stored result */
qio_status qio_server_forget(qio_server* server, int64_t request_id);
/* the device footprint the server admits the request by */
qio_status qio_server_request_bytes(qio_server* server, int64_t request_id, int64_t* bytes);
qio_status qio_server_get_stats(qio_server* server, qio_server_stats* out);
/* stops the worker; requests not yet finished are dropped */
qio_status qio_server_destroy(qio_server* server);

/* ---- runner ----------------------------------------------------------- */

/* app::Runner::run (app/runner.cc:215-631): problem JSON + params JSON +
 * target -> the reference's result JSON ({"benchmark", "solutions"}). */
qio_status qio_run_json(const char* input_json, const char* params_json,
                        const char* target, char** out_json);

#ifdef __cplusplus
}
#endif
#endif /* QIO_GB300_H */
