/*
 * qio_oracle.h -- C interface of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a plain C++ restatement of the
 * QIOToolkit Metropolis hot path (random generator, ln lookup table, walker,
 * Ising / PUBO / MaxSAT models, schedules, SA / PT / PA drivers).  It is the
 * checker that the CUDA library is compared against; nothing in the product
 * library links or calls it.  The only other user is bench.py's CPU-baseline
 * leg, which times it as "CPU restatement of the reference".
 *
 * Every function in qio_oracle.cc cites the reference file:line it follows.
 */
#ifndef QIO_ORACLE_H
#define QIO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* model kinds (same numbering as the product C-ABI) */
enum {
  ORC_ISING = 0,        /* model::IsingTermCached (default "ising")   */
  ORC_ISING_PLAIN = 1,  /* model::Ising (no term cache)                */
  ORC_PUBO = 2,         /* model::PuboWithCounter (default "pubo")     */
  ORC_PUBO_PLAIN = 3,   /* model::Pubo (no counters)                   */
  ORC_MAXSAT = 4        /* model::MaxSat                               */
};

enum { ORC_SA = 0, ORC_PT = 1, ORC_PA = 2, ORC_TABU = 3, ORC_SSMC = 4, ORC_QMC = 5 };
enum { ORC_RNG_REPLAY = 0, ORC_RNG_COUNTER = 1 };
enum { ORC_SCHED_LINEAR = 0, ORC_SCHED_GEOMETRIC = 1, ORC_SCHED_CONSTANT = 2,
       ORC_SCHED_LIST = 3 };

typedef struct orc_schedule {
  int type;
  double initial, final_value;
  int has_start, has_stop, has_count;
  double start, stop;
  int count;
  int n_values;          /* ORC_SCHED_LIST: explicit values */
  const double* values;
} orc_schedule;

typedef struct orc_params {
  int solver;
  uint32_t seed;
  int64_t step_limit;
  int64_t restarts;           /* SA */
  int use_inverse;            /* SA/PT: schedule holds beta (1) or T (0) */
  orc_schedule sched;         /* SA: beta/T(step); PT: ladder; PA: beta(step) */
  int64_t sweeps_per_replica; /* PT, PA */
  int64_t population;         /* PA */
  double alpha;               /* PA restart ratio */
  int constant_population;    /* PA */
  int exp_repopulation;       /* PA feature 2 */
  int pa_threads;             /* PA: emulated OpenMP thread count (streams) */
  int rng_mode;
  int threads;                /* OpenMP threads used by the oracle itself */
  int number_of_solutions;
  int has_cost_limit;
  double cost_limit;
  int full_maxsat_sweep;      /* MaxSAT: N attempts per sweep instead of 1 */
  int resampling;             /* PA: 0 the reference's (Poisson / constant),
                                 1 multinomial on counter draws (the GB300
                                 library's device mode, restated here) */
  int64_t master_skip;        /* SA: draws taken from the master stream before
                                 the restarts fork (a run that continues the
                                 stream of earlier runs, as the parameter-free
                                 solvers' repeated SA runs do) */
  int use_master_state;       /* PT: start the master stream at master_state
                                 instead of seeding it (repeated runs) */
  uint64_t master_state;
  int64_t tabu_tenure;        /* tabu: sweeps a taken move stays tabu */
  orc_schedule sched2;        /* SSMC: beta (resampling) schedule; `sched`
                                 holds alpha, `sweeps_per_replica` the steps
                                 per walker, `population` the target
                                 population, `pa_threads` the emulated
                                 OpenMP thread count (streams) */
  const int64_t* tabu_tenures;/* tabu: per-restart tenures (parameter-free
                                 runs), or NULL for tabu_tenure everywhere */
  int64_t n_tabu_tenures;
  int64_t trotter_number;     /* QMC: slices per restart; `sched` holds beta
                                 (linear), `sched2` the transverse field
                                 (linear), both stretched over the steps */
} orc_params;

/* ---- random generator pins ---- */
void orc_pcg_stream(uint32_t seed, int use_default_seed, int n, uint32_t* out);
void orc_pcg_uniform(uint32_t seed, int use_default_seed, int n, double* out);
void orc_pcg_fork_uniform(uint32_t seed, int n_forks, int n, double* out);
void orc_twister_uniform(uint32_t seed, int use_default_seed, int n,
                         double* out);
void orc_uniform_ln(double* out /* 4*256 */);
int orc_metropolis_accept(double cost_diff, double beta, const uint32_t* draws,
                          int n_draws, int* used);
uint64_t orc_counter_draw(uint64_t key, uint64_t ctr);
/* exp(x) for x <= 0 as the multinomial resampling mode defines it */
double orc_qexp(double x);
uint64_t orc_counter_key(uint32_t seed, uint64_t stream);

/* ---- model ---- */
void* orc_model_create(int kind, int64_t n_terms, const int64_t* term_off,
                       const int32_t* ids, const double* coef, char* err,
                       int errlen);
void orc_model_destroy(void* m);
int64_t orc_model_n_vars(void* m);
int64_t orc_model_n_terms(void* m);
double orc_model_const_cost(void* m);
double orc_model_scale_factor(void* m);
void orc_model_var_names(void* m, int32_t* out);
double orc_state_cost(void* m, const uint8_t* spins);
double orc_state_cost_difference(void* m, const uint8_t* spins, int64_t var);
void orc_state_apply(void* m, uint8_t* spins, int64_t var);
/* Metropolis on a ring with a Mersenne twister, as in the reference model
   tests: returns the minimum cost reached. */
double orc_model_twister_min(void* m, uint32_t seed, int iters, double T);

/* ---- solvers ---- */
void* orc_run(void* m, const orc_params* p, char* err, int errlen);
int64_t orc_res_n_replicas(void* r);
int64_t orc_res_n_vars(void* r);
int64_t orc_res_last_step(void* r);
void orc_res_replicas(void* r, double* cost, double* lowest, uint64_t* attempts,
                      uint64_t* accepts);
void orc_res_states(void* r, uint8_t* out);
void orc_res_lowest_states(void* r, uint8_t* out);
double orc_res_best_cost(void* r);
/* PT: the master stream's state after the run */
uint64_t orc_res_master_state(void* r);
void orc_res_best_state(void* r, uint8_t* out);
int64_t orc_res_n_solutions(void* r);
void orc_res_solutions(void* r, double* costs, uint8_t* states);
/* PT observables averaged per temperature slot (T or beta, acc_rate,
   avg_cost, avg_dir, swap_rate); swap_rate of the last slot is NaN. */
void orc_res_pt_observables(void* r, double* out5);
void orc_res_pa_trace(void* r, int64_t* n_steps, double* beta_out,
                      int64_t* pop_out, int64_t max_steps);
void orc_res_destroy(void* r);

/* toy model of the reference's solver tests (cost |x - 42|) under PT */
int orc_pt_toy(uint32_t seed, int64_t steps, const double* temps, int n,
               int use_inverse, double* obs5 /* n*5 */, double* best);

#ifdef __cplusplus
}
#endif
#endif
