// qio_internal.h -- structures shared by the host shim (.cc) and the sm_103a
// kernels (.cu).  No torch types, no C++ standard-library types cross into
// device code.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace qio
{
// Model kinds, numbered as qio_model_kind in include/qio_gb300.h.
enum Kind
{
  K_ISING = 0,
  K_ISING_PLAIN = 1,
  K_PUBO = 2,
  K_PUBO_PLAIN = 3,
  K_MAXSAT = 4
};

// Kernel flavour of a model.
//   F_PARITY : Ising with a per-term parity byte (IsingTermCached)
//   F_COUNTER: per-term counter byte with signed literals (PuboWithCounter is
//              MaxSat with every literal positive: a PUBO variable whose
//              spin is true has value 0, i.e. its "literal" is true)
//   F_PLAIN_ISING / F_PLAIN_PUBO: no term state, members gathered per term
enum Flavor
{
  F_PARITY = 0,
  F_COUNTER = 1,
  F_PLAIN_ISING = 2,
  F_PLAIN_PUBO = 3
};

static const uint32_t kNegBit = 0x80000000u;

// Read-only model in HBM.  Incidence k of variable v lies in
// [row[v], row[v+1]) in ascending term id, the reference's order
// (graph/graph.h:123).  inc[k] = term | kNegBit for a negated literal.
struct DevModel
{
  int flavor;
  int n_vars;
  int n_terms;
  int sweep_size;   // attempts per sweep (n_vars; 1 for MaxSat strict)
  int int_mode;     // coefficients are small integers
  const int* row;          // n_vars + 1
  const uint32_t* inc;     // K
  const double* coef;      // K  coefficient of the incidence's term
  const int* coef_i;       // K  same, integer mode
  const float* coef_f;     // K  same rounded to float (FP32 screen), FP64 mode
  // near[k]: the later members u of incidence k's term (0 < u - v <= 31)
  // whose rows hold at most 32 incidences, as 10-bit entries (u - v: bits
  // 0-4, the term's position in u's row: bits 5-9), up to six of them; the
  // count is in bits 61-63, 7 meaning "too many to list"
  const unsigned long long* near;
  int fscreen;             // FP64 coefficients all within the FP32 screen's range
  int pair_only;           // Ising, every term has one or two members
  const int* other;        // K  the other member of the incidence's term, or -1
  const int2* rec_i;       // K  (other or padding spin, integer coefficient), pair-only
  const double2* rec_f;    // K  (other as an integer in the low word, coefficient)
  const unsigned int* rec_p;  // K  other << 8 | 8-bit coefficient (small integer ones)
  int max_deg;             // largest row (incidences of one variable)
  int max_block_inc;       // most incidences of one 32-variable block of the sweep
  // level schedule (levels.cu), integer pair-only Ising models: level(v) =
  // 1 + the largest level of v's lower neighbours (0 without one); the
  // variables of level t are entries lv_off[t] .. lv_off[t+1] of lv_ent, in
  // index order.  With lv_recs > 0 an entry is the variable and lv_recs
  // records lv_record(u, c) of its terms (padded with zero-coefficient
  // padding-spin records), lv_entry_words(lv_recs) words in all; with
  // lv_recs == 0 it is the variable alone (records from row / rec)
  const int* lv_off;
  const uint32_t* lv_ent;
  const int* lv_pos;       // entry of each variable (n_vars rounded up to 32)
  int n_levels;
  int lv_recs;             // 0, 3, 4, 6, 7 or 15
  int lv_ok;               // the level kernel can run this model
  int lv_d8;               // every cost difference within -128 .. 127
  int scan32;              // 32 cost differences always sum within int32
  const uint32_t* nbr;     // n_vars: bit d-1 set if v-d shares a term with v
  const int* trow;         // n_terms + 1
  const uint32_t* tvar;    // K  members (| kNegBit for negated literals)
  const double* tcost;     // n_terms
  const int* tcost_i;      // n_terms
  // field-cached sweep (fields.cu): one 16-byte record per incidence, in
  // row order: x = inc (term | kNegBit), y = the coefficient in fixed point
  // (round(c * 2^fc_S), shifted left 8 when fc_pack), z = co-members 0 and 1,
  // w = co-member 2 | count << 16 (count 15: more than three, read trow /
  // tvar); a co-member is id | 0x8000 for a negated literal, 0xFFFF none
  const uint4* fc_rec;     // K, or null when the model does not qualify
  int fc_S;                // fixed-point scale exponent
  int fc_pack;             // FP64 counter models: field = fixed << 8 | count
  double fc_inv;           // 2^-fc_S
};

// Walker population in HBM (structure of arrays).  Spins are bit-packed,
// 32 variables per word; term state is one byte per term.
struct DevPop
{
  int n;                 // slots
  int nw;                // words per spin vector
  int mp;                // bytes per term-state vector
  uint32_t* spins;       // n * nw
  uint8_t* tstate;       // n * mp
  double* cost;          // n (per slot)
  double* lowest;        // n (per walker)
  uint32_t* lspins;      // n * nw (per walker)
  unsigned long long* attempts;   // n (per walker)
  unsigned long long* accepts;    // n (per walker)
  unsigned long long* step_att;   // n (per walker, since last observation)
  unsigned long long* step_acc;   // n
  unsigned long long* windows;    // n (per walker: window iterations), or null
  long long* lowtag;     // n (per walker): the tag of the launch in which its
                         // lowest last dropped (-1: its initial state), or null
};

struct SweepArgs
{
  DevModel m;
  DevPop p;
  int n_streams;        // one warp per stream
  int n_walkers;        // stream w serves walkers w, w + n_streams, ...
  const int* slot_of;   // walker -> slot (PT label swaps) or null
  const double* beta;   // beta[walker * bs_w + sweep * bs_s]
  long long bs_w, bs_s;
  long long sweep_base; // absolute sweep index of this launch's first sweep
  int n_sweeps;
  int replay;           // 1: PCG streams (replay); 0: counter mode
  uint64_t* rng;        // replay: PCG state per stream
  uint32_t seed;        // counter mode: key = counter_key(seed + w / key_div,
  unsigned long long key_base;  //                      key_base + w % key_div)
  long long key_div;
  int smem_state;       // stage spins + term state in shared memory
  int* err;             // device error flag (a bounded wait gave up)
  long long tag;        // written to p.lowtag[walker] when its lowest drops
  // field-cached sweep: per slot the fixed-point local field of every
  // variable (fc_words(N) ints), kept between launches; null selects the
  // windowed kernel.  field_valid = 0: rebuild the fields from the state.
  int* field;
  int field_valid;
  // batches (windowed kernel): walker r runs models[model_of[r]] with the
  // counter key of walker local_of[r] of its own solve; with `queue` set,
  // each warp takes walkers from the counter *queue (reset to 0 before the
  // launch) until n_walkers are taken, in index order, and keeps walker r's
  // PCG state in rng[r].  Null: a.m for every walker, stream w serving
  // walkers w, w + n_streams, ...
  const DevModel* models;
  const int* model_of;
  const int* local_of;
  int* queue;
  // windowed kernel: incidences a shared-memory record tile holds (a
  // multiple of 8; 0: launch_sweep sizes it to the model's largest block,
  // at most 640, 768 for integer models); larger blocks are read from HBM
  int tile_cap;
  // field-cached sweep: stream w runs walker order[w] (null: walker w); set
  // only with one walker per stream.  Tempering puts its hottest replicas
  // first, so that their long chains start in the first wave of blocks.
  const int* order;
};

struct InitArgs
{
  DevModel m;
  DevPop p;
  int n_walkers;
  const int* slot_of;
  int replay;
  uint64_t* rng;        // replay: per walker stream state (advanced in place)
  uint32_t seed;
  unsigned long long key_base;
  long long key_div;
  const uint8_t* given;     // optional: explicit states (n_walkers * n_vars)
  int keep_counters;        // 1: keep attempt/accept totals (population re-init)
  int skip_terms;           // 1: leave the term state bytes alone (the sweeps
                            //    that follow work from the spins)
};

// ---- launchers (kernels.cu) -------------------------------------------
void upload_tables(int device);  // ln table + PCG jump tables
cudaError_t launch_init(const InitArgs& a, cudaStream_t s);
cudaError_t launch_sweep(const SweepArgs& a, cudaStream_t s, int warps_per_block);
// one warp's walker state (term bytes, spins, lowest) fits shared memory
// beside the windowed kernel's tables and tiles (required by batch queues)
bool sweep_state_fits(const SweepArgs& a);
// field-cached sweep (fields.cu): ints of one slot's fields, and whether the
// kernel can run this model with this population layout
int64_t fc_words(int n_vars);
bool fc_fits(const DevModel& m, int nw, int mp);
cudaError_t launch_fc_sweep(const SweepArgs& a, cudaStream_t s);
cudaError_t launch_eval_cost(const DevModel& m, int n_states,
                             const uint32_t* spins, int nw, double* out,
                             cudaStream_t s);
// Lane-per-walker sweeps (lanes.cu) for Ising models with one- or
// two-member terms.  Walker r is lane r % G of group r / G (G <= 32 lanes of
// one warp); a group's block in the arena holds 32-bit words [spins gw*G]
// [lowest spins gw*G][flip log kLwLog*G], word w of lane l at index w*G + l.
static const int kLwLog = 64;
static const int kLwSmemBytes = 227 * 1024;  // dynamic shared memory per block
struct LwArgs
{
  const DevModel* models;   // device array
  const int* model_of;      // per walker (null: every walker runs models[0])
  int n_walkers;
  DevPop p;                 // per-walker cost, lowest, counters; spins for the transposes
  const int* slot_of;       // null: slot = walker
  uint8_t* arena;
  const long long* g_off;   // per group: byte offset of its block
  const int* g_nw;          // per group: spin words per lane (block layout)
  const double* beta;       // beta[r * bs_w + sweep * bs_s]
  long long bs_w, bs_s;
  long long sweep_base;
  int n_sweeps;
  int replay, int_mode;
  uint64_t* rng;
  uint32_t seed;
  long long key_div;
  unsigned long long key_base;
  const int* local_of;      // per walker: index within its solve for counter keys (null: r)
  int G;                    // walkers (lanes) per group
  int smem_words;           // group words per lane held in shared memory (0: global)
  int packed;               // every model has 32-bit records (rec_p)
  int unroll;               // records per attempt held in registers: 4, 6 or 8
};
// wpb: warps per block (0: spread the groups over the SMs)
cudaError_t launch_lw_sweep(const LwArgs& a, int wpb, cudaStream_t s);
cudaError_t launch_lw_load(const LwArgs& a, int max_words, cudaStream_t s);
cudaError_t launch_lw_store(const LwArgs& a, int max_words, int max_terms, cudaStream_t s);
void lw_upload(const double* ln, const float* scr);

// Level-scheduled sweeps (levels.cu): one warp per walker, counter streams,
// integer pair-only Ising models with lv_ok.  The walker's spins stay in
// shared memory for the launch (word w at w + w / 32); each sweep is logged
// and a second kernel finds the lowest from the log.
static const int kLvMaxWarps = 28;
static const int kLvSmemBytes = 227 * 1024;
struct LvArgs
{
  DevModel m;
  DevPop p;
  int n_walkers;
  const int* slot_of;       // null: slot = walker
  const double* beta;       // beta[r * bs_w + sweep * bs_s]
  long long bs_w, bs_s;
  long long sweep_base;
  int n_sweeps;
  uint32_t seed;            // key of walker r: counter_key(seed + r / key_div,
  unsigned long long key_base;  //                   key_base + r % key_div)
  long long key_div;
  // the sweep log, log_sweeps sweeps per walker (sweep k of walker r at
  // r * log_sweeps + k): start spins (p.nw words), start cost and a bound
  // below the sweep's running cost (two per sweep), and the difference of
  // every attempt (0 when rejected) at its level entry
  int log_sweeps;
  uint32_t* start;
  long long* cost0;
  void* diffs;
  long long diff_stride;    // elements per logged sweep (>= n_vars, a multiple of 32)
  int diff_bytes;           // 1 (models with lv_d8) or 4
};
// lowest pass: threads per block (one block per walker), log bytes staged
// in shared memory per block
static const int kLvLowThreads = 512;
static const int kLvRowBytes = 96 * 1024;
// shared-memory word of spin word w in the level kernel's layout (one
// padding word after every 32 so that lanes spread over the banks)
__host__ __device__ inline int lv_phys(int w) { return w + (w >> 5); }
// a term record of a level entry: the other member's shared-memory word and
// bit, and the 8-bit coefficient
inline uint32_t lv_record(int u, int c)
{
  return ((uint32_t)lv_phys(u >> 5) << 13) | ((uint32_t)(u & 31) << 8) | ((uint32_t)c & 0xFFu);
}
__host__ __device__ constexpr int lv_entry_words(int recs) { return recs <= 3 ? 4 : (recs <= 7 ? 8 : 16); }
// bytes per logged difference for a model (1 or 4)
inline int lv_diff_bytes(const DevModel& m) { return m.lv_d8 ? 1 : 4; }
inline long long lv_diff_stride(int n_vars) { return ((long long)n_vars + 31) & ~31LL; }
// shared-memory words per walker, 0 when the model does not fit
int lv_stride_words(int n_vars);
cudaError_t launch_lv_sweep(const LvArgs& a, cudaStream_t s);
// term parity bytes from the spins (after level sweeps)
cudaError_t launch_lv_terms(const DevModel& m, const DevPop& p, int n_walkers, const int* slot_of,
                            cudaStream_t s);
void lv_upload(const double* ln, const float* scr);

// Device resampling of population annealing (pa_device.cu, multinomial).
struct PaScalars
{
  double cmin, cmax, best_lowest;
  int best_index;
  unsigned long long total;   // sum of the fixed-point weights
  unsigned long long census;  // sum over families of count^2
};
cudaError_t launch_pa_weights(const double* cost, const double* lowest, int R, double dbeta_scale,
                              unsigned long long* prefix, PaScalars* out, cudaStream_t s);
cudaError_t launch_pa_parents(const unsigned long long* prefix, int R, int R_new, uint64_t key,
                              const PaScalars* sc, const int* family, int* src, int* family_new,
                              cudaStream_t s);
cudaError_t launch_pa_census(const int* family, int R, unsigned int* counts, int n_families, PaScalars* out,
                             cudaStream_t s);
cudaError_t launch_pa_iota(int* a, int n, cudaStream_t s);
cudaError_t launch_pa_fill(double* a, int n, double v, cudaStream_t s);
cudaError_t launch_qexp(const double* x, double* y, int n, cudaStream_t s);

// Allocation-free variant: states are n x n_vars bytes on the device, packed
// into a fixed file-scope scratch array of kNoAllocScratchWords words.
static const int kNoAllocScratchWords = 1 << 18;
static const int kMaxDevices = 64;
cudaError_t launch_eval_cost_noalloc(const DevModel& m, int n, const uint8_t* states, int n_vars,
                                     int nw, double* out, cudaStream_t s);
cudaError_t launch_eval_diff(const DevModel& m, int n, const uint32_t* spins,
                             int nw, const long long* vars, double* out,
                             cudaStream_t s);

// Tabu search (kernels.cu): one warp per walker; per walker the tabu list
// (expiry sweep per variable), the hill climber's copy and its lowest state,
// and the scalars below.
struct TabuState
{
  double hc_cost, hc_low;        // the hill climber's cost and lowest
  unsigned long long iter;       // tabu sweeps so far
  unsigned long long incomplete; // compensation count (markov/tabu_walker.h:88-101)
  int local;                     // 1: local-search mode
  int ready;                     // 1: the cached differences are filled
};
struct TabuArgs
{
  DevModel m;
  DevPop p;
  int n_walkers;
  int n_steps;
  unsigned long long tenure;
  const unsigned long long* tenures;  // per walker (parameter-free runs), or null
  unsigned long long* tabu;  // n_walkers * n_vars
  uint32_t* hc;              // n_walkers * p.nw
  uint32_t* hc_low;          // n_walkers * p.nw
  double* diff;              // n_walkers * n_vars: each variable's cost difference
  double* hdiff;             // n_walkers * n_vars: the same for the hill climber's copy
  TabuState* st;             // n_walkers
};
cudaError_t launch_tabu(const TabuArgs& a, cudaStream_t s);

// Substochastic Monte Carlo walker steps (solver/substochastic_monte_carlo.h:
// 86-112): every walker attempts steps_per_walker random flips, each made
// with probability p_step and always accepted (markov/random_walker.h).
struct SsmcArgs
{
  DevModel m;
  DevPop p;
  int n_walkers;
  int steps_per_walker;
  double p_step;
  long long step;           // absolute step (counter mode draw positions)
  int n_chains;             // replay: emulated OpenMP threads, each serving a
                            // contiguous block of walkers in index order
  uint64_t* rng;            // replay: PCG state per chain
  uint32_t seed;            // counter mode: slot j draws on counter_key(seed, j)
  int replay;
};
cudaError_t launch_ssmc_walk(const SsmcArgs& a, cudaStream_t s);

// Quantum Monte Carlo sweeps (solver/quantum_monte_carlo.h:128-175 with
// markov/cluster_walker.h): one warp per restart, slice k of restart r in
// population slot r * trotter + k.
static const int kQmcMaxTrotter = 1024;
struct QmcArgs
{
  DevModel m;
  DevPop p;                  // trotter * restarts slots
  int restarts, trotter;
  long long step_base;       // absolute step of the launch's first sweep
  int n_steps;
  const double* beta_eff;    // per absolute step: beta / trotter
  // per absolute step, the bond probability bp = 1 - tanh(field * beta /
  // trotter) as an integer limit on the draw: replay, uniform() < bp exactly
  // when the two 32-bit outputs X = d0 + d1 2^32 lie below bond_lim (all X
  // when bond_all); counter, when draw >> 11 lies below bond_lim
  const unsigned long long* bond_lim;
  const unsigned char* bond_all;
  int replay;
  uint64_t* rng;             // replay: PCG state per slot
  uint32_t seed;             // counter mode: slot i draws on counter_key(seed, i)
  double* low;               // per restart: lowest cost of its slices
  uint32_t* low_spins;       // per restart: that slice's spins (p.nw words)
  unsigned long long* near_ties;  // exp() within 1e-15 of its uniform draw
  // level schedule (counter streams only): variables lv_var[lv_off[t] ..
  // lv_off[t+1]) share no term and follow all their lower-index neighbours'
  // levels; dlog holds each slice's flip differences of a sweep (restarts *
  // trotter * n_vars) for the cost sums in variable order
  int n_levels;
  const int* lv_off;
  const int* lv_var;
  double* dlog;
};
cudaError_t launch_qmc(const QmcArgs& a, cudaStream_t s);
static const int kQmcLevelWarps = 32;
// dynamic shared memory of the level kernel (0 when it cannot run)
size_t qmc_level_smem(int trotter, int nw);
cudaError_t launch_qmc_levels(const QmcArgs& a, cudaStream_t s);

// PT: label swaps + observables, one warp per restart (lanes over the ladder,
// then over the step's pairs).
struct SwapArgs
{
  int restarts;
  int n_temps;
  int* slot_of;             // restarts * n_temps
  const double* cost;       // per slot
  const double* beta;       // per walker (position)
  int* dir;                 // per walker
  const unsigned long long* step_att;
  unsigned long long* step_acc_reset;  // step counters (reset after reading)
  unsigned long long* step_att_reset;
  double* obs_acc;          // per walker: sum of per-step acc_rate
  double* obs_cost;         // per walker: sum of costs
  double* obs_dir;          // per walker: sum of directions
  unsigned long long* swap_acc;  // per walker
  unsigned long long* swap_cnt;  // per walker
  unsigned long long* near_ties;
  long long step;
  int replay;
  uint64_t* master;         // replay: per restart master PCG state
  const unsigned long long* swap_key;  // counter: per restart key
};
cudaError_t launch_pt_swap(const SwapArgs& a, cudaStream_t s);

// PA: bit-exact replica copies src -> dst (walker j of dst copies walker
// src_of[j]); step counters of the copies start at zero.
cudaError_t launch_pa_copy(const DevPop& src, const DevPop& dst, const int* src_of,
                           int n_dst, cudaStream_t s);
}  // namespace qio
