// kernels.cu -- sm_103a kernels of the Metropolis hot path.
//
// The ordered sweep of the reference (markov/walker.h:143-153) is a strictly
// sequential chain: attempt i reads the state left by attempt i-1.  One warp
// owns one walker and evaluates a WINDOW of 32 consecutive variables at once
// (lane l takes variable i+l), each lane summing its own cost difference in
// the reference's term order (bit-identical FP64).  Decisions are then
// committed in lane order up to the first lane whose terms intersect an
// earlier accepted flip in the window (its difference was computed on a
// stale state) or that needs the Metropolis redraw path; the next window
// starts there.  Replay streams are PCG32 positions: lane l's draw is the
// stream advanced by the number of uphill lanes before it (an LCG jump), so
// the committed prefix consumes exactly the draws the sequential chain would.
// The result is the reference's trajectory, evaluated up to 32-wide.
#include <cstdio>
#include <mutex>

#include "exp_cr.cuh"
#include "qio_internal.h"

namespace qio
{
static const unsigned kFull = 0xffffffffu;
static const unsigned long long kMult = 6364136223846793005ULL;
static const unsigned long long kInc = 1442695040888963407ULL;
static const unsigned long long kGamma = 0x9E3779B97F4A7C15ULL;
static const unsigned long long kInitCounterBase = 1ULL << 62;

// ln table (utils/utils.cc:12-32, computed on the host with the C library's
// log) and LCG jump tables: k steps (k = 0..64) and 2^k steps.
__constant__ double c_ln[1024];
__constant__ unsigned long long c_jA[65], c_jC[65];
__constant__ unsigned long long c_pA[64], c_pC[64];

__device__ __forceinline__ uint32_t pcg_out(uint64_t old)
{
  uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  uint32_t rot = (uint32_t)(old >> 59u);
  return __funnelshift_r(xs, xs, rot);
}

__device__ __forceinline__ uint64_t jump_any(uint64_t s, unsigned long long k)
{
  for (int b = 0; k; b++, k >>= 1)
    if (k & 1ULL) s = c_pA[b] * s + c_pC[b];
  return s;
}

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t counter_key(uint32_t seed, uint64_t stream)
{
  return mix64(((uint64_t)seed << 32) ^ mix64(stream + kGamma));
}
__device__ __forceinline__ uint64_t counter_draw(uint64_t key, uint64_t ctr)
{
  return mix64(key + ctr * kGamma);
}

// libstdc++ generate_canonical<double,53> over a 32-bit engine: two draws,
// sum = a + b * 2^32 rounded once, divided by 2^64, clamped below 1.
__device__ __forceinline__ double canonical(uint32_t a, uint32_t b)
{
  double s = __dadd_rn((double)a, __dmul_rn((double)b, 4294967296.0));
  double u = __dmul_rn(s, 5.421010862427522170037e-20);  // 2^-64
  if (u >= 1.0) u = 0.99999999999999988898;              // nextafter(1, 0)
  return u;
}

// value < -dE * beta with value interpolated in ln[row] at bucket r & 255,
// distance (r >> 8) / 16777214 (markov/metropolis.h:96-103).  Explicit _rn
// intrinsics keep the reference's rounding (no fused multiply-add).
__device__ __forceinline__ bool lut_less(const double* ln, uint32_t r, int row,
                                         double thr)
{
  int b = (int)(r & 255u);
  double y0 = ln[row * 256 + b - 1];
  double y1 = ln[row * 256 + b];
  // (r >> 8) / 16777214 correctly rounded: reciprocal product corrected by
  // one fused residual step (Markstein); equal to the IEEE quotient for all
  // 2^24 inputs (checked exhaustively by the oracle's test).
  const double x = (double)(r >> 8);
  const double inv = 5.9604648328104515e-08;  // RN(1 / 16777214)
  const double d0 = __dmul_rn(x, inv);
  const double dist = __fma_rn(__fma_rn(-d0, 16777214.0, x), inv, d0);
  double value = __dadd_rn(y0, __dmul_rn(dist, __dsub_rn(y1, y0)));
  return value < thr;
}

// Metropolis::accept (markov/metropolis.h:64-104) for an uphill move with
// the draws supplied by `draw(k)`; `used` receives the draw count.
template <class F>
__device__ __forceinline__ bool metropolis_uphill(double thr, const double* ln,
                                                  F draw, int& used)
{
  int row = -1, b = 0;
  uint32_t cur = 0;
  used = 0;
  while (b == 0)
  {
    if (row < 3)
    {
      cur = draw(used);
      used++;
      b = (int)(cur & 255u);
      row++;
    }
    else
      return true;
  }
  return lut_less(ln, cur, row, thr);
}

__device__ __forceinline__ uint32_t spin_of(const uint32_t* spins, int v)
{
  return (spins[v >> 5] >> (v & 31)) & 1u;
}

// Value of term t under `spins` for the full cost (calculate_cost) and a
// skip flag for counter models (terms that do not contribute are skipped,
// as the reference does, rather than added as 0).
template <int FL, bool INT>
__device__ __forceinline__ void term_value(const DevModel& m,
                                           const uint32_t* spins, int t,
                                           double& val, long long& ival,
                                           bool& skip)
{
  int b = m.trow[t], e = m.trow[t + 1];
  if (FL == F_PARITY || FL == F_PLAIN_ISING)
  {
    uint32_t par = 0;
    for (int k = b; k < e; k++) par ^= spin_of(spins, (int)(m.tvar[k] & ~kNegBit));
    skip = false;
    if (INT) ival = par ? -(long long)m.tcost_i[t] : (long long)m.tcost_i[t];
    else val = par ? -m.tcost[t] : m.tcost[t];
  }
  else
  {
    // counter: number of true literals; the term contributes when it is 0
    int cnt = 0;
    for (int k = b; k < e; k++)
    {
      uint32_t x = m.tvar[k];
      cnt += (int)(spin_of(spins, (int)(x & ~kNegBit)) ^ (x >> 31));
    }
    skip = cnt != 0;
    if (INT) ival = skip ? 0 : (long long)m.tcost_i[t];
    else val = skip ? 0.0 : m.tcost[t];
  }
}

// Sum of term values by one warp: lanes evaluate 32 terms in parallel; the
// FP64 sum runs sequentially in term order (bit-identical to a loop), the
// integer sum (exact in any order) as per-lane partial sums and a reduction.
template <int FL, bool INT>
__device__ void warp_cost(const DevModel& m, const uint32_t* spins, int lane,
                          double& cost, long long& icost)
{
  double c = 0.0;
  long long ic = 0;
  for (int t0 = 0; t0 < m.n_terms; t0 += 32)
  {
    int t = t0 + lane;
    double v = 0.0;
    long long iv = 0;
    bool skip = true;
    if (t < m.n_terms) term_value<FL, INT>(m, spins, t, v, iv, skip);
    if (INT)
    {
      // integer sums are exact in any order: per-lane partial sums
      if (!skip) ic += iv;
      continue;
    }
    unsigned keep = __ballot_sync(kFull, !skip);
    while (keep)
    {
      int j = __ffs(keep) - 1;
      keep &= keep - 1;
      c = __dadd_rn(c, __shfl_sync(kFull, v, j));
    }
  }
  if (INT)
  {
#pragma unroll
    for (int d = 16; d; d >>= 1) ic += __shfl_xor_sync(kFull, ic, d);
  }
  cost = c;
  icost = ic;
}

// Term state bytes (written to ts unless it is null) and the cost of a state
// by one warp in a single pass over the terms; each lane takes four terms at
// a time so that their loads overlap.  FP64 values are added in term order
// (bit-identical to a loop), integers per lane and reduced.
template <int FL, bool INT>
__device__ void warp_terms_cost(const DevModel& m, const uint32_t* spins, uint8_t* ts, int lane,
                                double& cost, long long& icost)
{
  constexpr int U = 4;
  constexpr bool PAR = FL == F_PARITY || FL == F_PLAIN_ISING;
  double c = 0.0;
  long long ic = 0;
  const int M = m.n_terms;
  for (int t0 = 0; t0 < M; t0 += 32 * U)
  {
    int b[U], e[U];
    uint32_t acc[U];
#pragma unroll
    for (int u = 0; u < U; u++)
    {
      const int t = t0 + u * 32 + lane;
      b[u] = t < M ? __ldg(m.trow + t) : 0;
      e[u] = t < M ? __ldg(m.trow + t + 1) : 0;
      acc[u] = 0;
    }
    // the members of the four terms, position by position
    for (int k = 0;; k++)
    {
      bool more = false;
#pragma unroll
      for (int u = 0; u < U; u++)
        if (b[u] + k < e[u])
        {
          const uint32_t x = __ldg(m.tvar + b[u] + k);
          const uint32_t sx = spin_of(spins, (int)(x & ~kNegBit));
          if (PAR) acc[u] ^= sx;
          else acc[u] += sx ^ (x >> 31);
          more = more || b[u] + k + 1 < e[u];
        }
      if (!more) break;
    }
#pragma unroll
    for (int u = 0; u < U; u++)
    {
      const int t = t0 + u * 32 + lane;
      double v = 0.0;
      long long iv = 0;
      bool skip = true;
      if (t < M)
      {
        if (ts && (FL == F_PARITY || FL == F_COUNTER)) ts[t] = (uint8_t)acc[u];
        // parity: the term's sign; counter: the term counts when no literal is true
        skip = PAR ? false : acc[u] != 0;
        if (INT) iv = skip ? 0 : (PAR && acc[u] ? -(long long)m.tcost_i[t] : (long long)m.tcost_i[t]);
        else v = skip ? 0.0 : (PAR && acc[u] ? -m.tcost[t] : m.tcost[t]);
      }
      if (INT)
      {
        if (!skip) ic += iv;
        continue;
      }
      unsigned keep = __ballot_sync(kFull, !skip);
      while (keep)
      {
        const int j = __ffs(keep) - 1;
        keep &= keep - 1;
        c = __dadd_rn(c, __shfl_sync(kFull, v, j));
      }
    }
  }
  if (INT)
  {
#pragma unroll
    for (int d = 16; d; d >>= 1) ic += __shfl_xor_sync(kFull, ic, d);
  }
  cost = c;
  icost = ic;
}

// Term state byte from spins: parity (Ising) or true-literal count.
template <int FL>
__device__ __forceinline__ uint8_t term_state(const DevModel& m,
                                              const uint32_t* spins, int t)
{
  int b = m.trow[t], e = m.trow[t + 1];
  uint32_t acc = 0;
  for (int k = b; k < e; k++)
  {
    uint32_t x = m.tvar[k];
    uint32_t s = spin_of(spins, (int)(x & ~kNegBit));
    if (FL == F_PARITY) acc ^= s;
    else acc += s ^ (x >> 31);
  }
  return (uint8_t)acc;
}

// ---------------------------------------------------------------------------
// init: random (or given) state, term cache, cost, lowest = current.
// Walker::init (markov/walker.h:50-58) with get_random_spin_state /
// get_random_binary_state (model/ising.h:23-41, model/pubo.h:16-34) or the
// MaxSat per-variable uniform() < 0.5 (model/max_sat.h:144-150).
// ---------------------------------------------------------------------------
template <int FL, bool INT>
__global__ void __launch_bounds__(128) init_kernel(InitArgs a)
{
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= a.n_walkers) return;
  const DevModel& m = a.m;
  const int N = m.n_vars;
  const int nwd = (N + 31) >> 5;
  const int slot = a.slot_of ? a.slot_of[w] : w;
  uint32_t* spins = a.p.spins + (size_t)slot * a.p.nw;
  uint8_t* ts = a.p.tstate + (size_t)slot * a.p.mp;
  uint32_t* lsp = a.p.lspins + (size_t)w * a.p.nw;
  // a.replay: 0 counter, 1 PCG replay (one draw per 32 variables);
  // 2 PCG replay / 3 counter with one uniform() per variable (MaxSat)
  const bool var_uniform = (a.replay == 2 || a.replay == 3);
  const bool replay = (a.replay == 1 || a.replay == 2);
  uint64_t key = 0;
  if (!replay)
    key = counter_key(a.seed + (uint32_t)(w / a.key_div),
                      a.key_base + (unsigned long long)(w % a.key_div));
  uint64_t rs = replay ? a.rng[w] : 0;
  for (int q0 = 0; q0 < nwd; q0 += 32)
  {
    int q = q0 + lane;
    uint32_t word = 0;
    if (a.given)
    {
      if (q < nwd)
        for (int b = 0; b < 32; b++)
        {
          int v = q * 32 + b;
          if (v < N && a.given[(size_t)w * N + v]) word |= 1u << b;
        }
    }
    else if (!var_uniform)
    {
      if (q < nwd)
      {
        if (replay) word = pcg_out(jump_any(rs, (unsigned long long)q));
        else word = (uint32_t)counter_draw(key, kInitCounterBase + (unsigned long long)q);
      }
    }
    else
    {
      // MaxSat: bit b of word q0+j is variable 32*(q0+j)+b; lanes take one
      // variable each, 32 words per pass
      for (int j = 0; j < 32 && q0 + j < nwd; j++)
      {
        int v = (q0 + j) * 32 + lane;
        bool bit = false;
        if (v < N)
        {
          if (replay)
          {
            uint64_t s0 = jump_any(rs, 2ULL * (unsigned long long)v);
            uint32_t d0 = pcg_out(s0);
            uint32_t d1 = pcg_out(s0 * kMult + kInc);
            bit = canonical(d0, d1) < 0.5;
          }
          else
            bit = (counter_draw(key, kInitCounterBase + (unsigned long long)v) >> 63) == 0;
        }
        unsigned bw = __ballot_sync(kFull, bit);
        if (lane == j) word = bw;
      }
    }
    if (q < nwd)
    {
      if (q == nwd - 1 && (N & 31)) word &= (1u << (N & 31)) - 1u;
      spins[q] = word;
    }
  }
  for (int q = nwd + lane; q < a.p.nw; q += 32) spins[q] = 0;
  if (replay && lane == 0)
    a.rng[w] = jump_any(rs, var_uniform ? 2ULL * (unsigned long long)N
                                        : (unsigned long long)nwd);
  __syncwarp();
  double cost;
  long long icost;
  warp_terms_cost<FL, INT>(m, spins, a.skip_terms ? nullptr : ts, lane, cost, icost);
  if (INT) cost = (double)icost;
  for (int q = lane; q < a.p.nw; q += 32) lsp[q] = spins[q];
  if (lane == 0)
  {
    a.p.cost[slot] = cost;
    a.p.lowest[w] = cost;
    if (a.p.lowtag) a.p.lowtag[w] = -1;
    if (!a.keep_counters)
    {
      a.p.attempts[w] = 0;
      a.p.accepts[w] = 0;
    }
    a.p.step_att[w] = 0;
    a.p.step_acc[w] = 0;
    if (a.p.windows) a.p.windows[w] = 0;
  }
}

// ---------------------------------------------------------------------------
// Evaluation kernels for the per-state contract.
// ---------------------------------------------------------------------------
template <int FL, bool INT>
__global__ void eval_cost_kernel(DevModel m, int n, const uint32_t* spins,
                                 int nw, double* out)
{
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= n) return;
  double c;
  long long ic;
  warp_cost<FL, INT>(m, spins + (size_t)w * nw, lane, c, ic);
  if (lane == 0) out[w] = INT ? (double)ic : c;
}

// calculate_cost_difference for query q: incident terms evaluated in
// parallel, summed in order (model/ising.h:108-117, model/pubo.h:335-367,
// model/pubo.cc:50-73, model/max_sat.h:173-236).
template <int FL, bool INT>
__global__ void eval_diff_kernel(DevModel m, int n, const uint32_t* spins,
                                 int nw, const long long* vars, double* out)
{
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= n) return;
  const uint32_t* sp = spins + (size_t)w * nw;
  const int v = (int)vars[w];
  const uint32_t sv = spin_of(sp, v);
  const int rb = m.row[v], re = m.row[v + 1];
  double diff = 0.0;
  long long idiff = 0;
  for (int q0 = rb; q0 < re; q0 += 32)
  {
    int q = q0 + lane;
    double val = 0.0;
    long long ival = 0;
    bool skip = true;
    if (q < re)
    {
      uint32_t e = m.inc[q];
      int t = (int)(e & ~kNegBit);
      int tb = m.trow[t], te = m.trow[t + 1];
      if (FL == F_PARITY || FL == F_PLAIN_ISING)
      {
        uint32_t par = 0;
        for (int u = tb; u < te; u++) par ^= spin_of(sp, (int)(m.tvar[u] & ~kNegBit));
        skip = false;
        if (INT) ival = par ? -(long long)m.coef_i[q] : (long long)m.coef_i[q];
        else val = par ? -m.coef[q] : m.coef[q];
      }
      else
      {
        int cnt = 0;
        for (int u = tb; u < te; u++)
        {
          uint32_t x = m.tvar[u];
          cnt += (int)(spin_of(sp, (int)(x & ~kNegBit)) ^ (x >> 31));
        }
        const bool lit = (sv ^ (e >> 31)) != 0;
        if (lit && cnt == 1)
        {
          skip = false;
          if (INT) ival = m.coef_i[q]; else val = m.coef[q];
        }
        else if (!lit && cnt == 0)
        {
          skip = false;
          if (INT) ival = -(long long)m.coef_i[q]; else val = -m.coef[q];
        }
      }
    }
    unsigned keep = __ballot_sync(kFull, !skip);
    while (keep)
    {
      int j = __ffs(keep) - 1;
      keep &= keep - 1;
      if (INT) idiff += __shfl_sync(kFull, ival, j);
      else diff = __dadd_rn(diff, __shfl_sync(kFull, val, j));
    }
  }
  if (lane == 0)
  {
    if (FL == F_PARITY || FL == F_PLAIN_ISING)
      out[w] = INT ? (double)(-2 * idiff) : __dmul_rn(2.0, -diff);
    else
      out[w] = INT ? (double)idiff : diff;
  }
}

// ---------------------------------------------------------------------------
// Tabu search (solver/tabu.h:22-164, markov/tabu_walker.h:14-218), one warp
// per walker.  A tabu sweep prices every variable against the current state
// (lanes take 32 variables at a time, each difference summed in the
// reference's term order), takes the first move that puts the cost below the
// lowest -- then hill-climbs on a copy (accepting differences <= 0, one
// variable after the other) while that improves the lowest -- or else the
// lowest-difference move not on the tabu list.  No random numbers after the
// initial state.
// ---------------------------------------------------------------------------
// FP64 instructions occupy a GB300 sub-partition's FP64 unit for ~64 cycles
// each, so the tabu kernel orders, signs and scales differences with integer
// bit operations where that is exact.
// fkey: unsigned key ordered as the doubles (finite values; -0 keyed as +0,
// as -0 == +0 compares)
__device__ __forceinline__ unsigned long long fkey(double x)
{
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if (b == 0x8000000000000000ull) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
// -2 * x for a normal x by the exponent and sign bits (__dmul_rn otherwise)
__device__ __forceinline__ double times_minus2(double x)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
  if (e == 0 || e >= 0x7FEu) return __dmul_rn(2.0, -x);
  return __longlong_as_double((long long)((b + (1ull << 52)) ^ 0x8000000000000000ull));
}

// calculate_cost_difference of variable v by one thread, terms in row order
template <int FL, bool INT>
__device__ double lane_diff(const DevModel& m, const uint32_t* sp, int v)
{
  const uint32_t sv = spin_of(sp, v);
  double diff = 0.0;
  long long idiff = 0;
  if (FL == F_PARITY && m.pair_only)
  {
    // one- or two-member terms: the parity is the spin of v xor that of the
    // other member; four incidences' loads in flight, added in row order
    const int qe = m.row[v + 1];
    for (int q = m.row[v]; q < qe; q += 4)
    {
      int o[4];
      double c[4];
      int ci[4];
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (q + u < qe)
        {
          o[u] = __ldg(m.other + q + u);
          if (INT) ci[u] = __ldg(m.coef_i + q + u);
          else c[u] = __ldg(m.coef + q + u);
        }
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (q + u < qe)
        {
          const uint32_t par = sv ^ (o[u] >= 0 ? spin_of(sp, o[u]) : 0u);
          if (INT) idiff += par ? -(long long)ci[u] : (long long)ci[u];
          else diff = __dadd_rn(diff, par ? -c[u] : c[u]);
        }
    }
    return INT ? (double)(-2 * idiff) : times_minus2(diff);
  }
  for (int q = m.row[v], qe = m.row[v + 1]; q < qe; q++)
  {
    const uint32_t e = m.inc[q];
    const int t = (int)(e & ~kNegBit);
    const int tb = m.trow[t], te = m.trow[t + 1];
    if (FL == F_PARITY || FL == F_PLAIN_ISING)
    {
      uint32_t par = 0;
      for (int u = tb; u < te; u++) par ^= spin_of(sp, (int)(m.tvar[u] & ~kNegBit));
      if (INT) idiff += par ? -(long long)m.coef_i[q] : (long long)m.coef_i[q];
      else diff = __dadd_rn(diff, par ? -m.coef[q] : m.coef[q]);
    }
    else
    {
      int cnt = 0;
      for (int u = tb; u < te; u++)
      {
        const uint32_t x = m.tvar[u];
        cnt += (int)(spin_of(sp, (int)(x & ~kNegBit)) ^ (x >> 31));
      }
      const bool lit = (sv ^ (e >> 31)) != 0;
      if (lit && cnt == 1)
      {
        if (INT) idiff += m.coef_i[q];
        else diff = __dadd_rn(diff, m.coef[q]);
      }
      else if (!lit && cnt == 0)
      {
        if (INT) idiff -= m.coef_i[q];
        else diff = __dadd_rn(diff, -m.coef[q]);
      }
    }
  }
  if (FL == F_PARITY || FL == F_PLAIN_ISING) return INT ? (double)(-2 * idiff) : times_minus2(diff);
  return INT ? (double)idiff : diff;
}

__device__ __forceinline__ void warp_copy(uint32_t* dst, const uint32_t* src, int n, int lane)
{
  for (int q = lane; q < n; q += 32) dst[q] = src[q];
  __syncwarp();
}

// Every walker keeps the cost difference of each of its variables (and its
// hill climber those of the copy) in HBM.  A flip of variable i changes only
// the differences of i and of the members of i's terms; those are summed
// afresh from the spins (term order, as calculate_cost_difference), so a
// cached value always equals a fresh evaluation bit for bit.
template <int FL, bool INT>
__device__ void tabu_refresh(const DevModel& m, const uint32_t* sp, double* df, int i, int lane)
{
  const int rb = m.row[i], re = m.row[i + 1];
  // i itself on the first lane without an incidence of i's row, so its sum
  // runs beside the co-members' instead of after one of them
  if (lane == min(re - rb, 31)) df[i] = lane_diff<FL, INT>(m, sp, i);
  if (FL == F_PARITY && m.pair_only)
  {
    for (int q = rb + lane; q < re; q += 32)
    {
      const int x = __ldg(m.other + q);
      if (x >= 0) df[x] = lane_diff<FL, INT>(m, sp, x);
    }
    __syncwarp();
    return;
  }
  for (int q = rb + lane; q < re; q += 32)
  {
    const int t = (int)(m.inc[q] & ~kNegBit);
    for (int u = m.trow[t], ue = m.trow[t + 1]; u < ue; u++)
    {
      const int x = (int)(m.tvar[u] & ~kNegBit);
      if (x != i) df[x] = lane_diff<FL, INT>(m, sp, x);
    }
  }
  __syncwarp();
}

template <int FL, bool INT>
__global__ void __launch_bounds__(128) tabu_kernel(TabuArgs a)
{
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= a.n_walkers) return;  // whole warps leave together
  const DevModel& m = a.m;
  // N strides the per-walker arrays; SW variables are swept (get_sweep_size:
  // N, or 1 for MaxSat unless the full sweep is asked for)
  const int N = m.n_vars, SW = m.sweep_size, nw = a.p.nw;
  uint32_t* sp = a.p.spins + (size_t)w * nw;
  uint32_t* ls = a.p.lspins + (size_t)w * nw;
  uint32_t* hs = a.hc + (size_t)w * nw;
  uint32_t* hl = a.hc_low + (size_t)w * nw;
  unsigned long long* tb = a.tabu + (size_t)w * N;
  double* df = a.diff + (size_t)w * N;
  double* hd = a.hdiff + (size_t)w * N;
  TabuState S = a.st[w];
  double cost = a.p.cost[w], low = a.p.lowest[w];
  unsigned long long att = 0, acc = 0;
  const unsigned long long tenure = a.tenures ? a.tenures[w] : a.tenure;
  if (!S.ready)
  {
    for (int v = lane; v < N; v += 32) df[v] = lane_diff<FL, INT>(m, sp, v);
    S.ready = 1;
    __syncwarp();
  }

  // HillClimbingWalker::make_sweep on the copy, then local_search_sweep's
  // bookkeeping (markov/tabu_walker.h:183-207).  The ordered sweep runs in
  // windows of 32 variables read at once: the lanes before the first
  // accepted one (d <= 0) hold what the sequential sweep would have seen and
  // were rejected; the window restarts after each accepted flip.
  auto local_sweep = [&]() {
    const double prev = S.hc_low;
    int v0 = 0;
    while (v0 < SW)
    {
      const int v = v0 + lane;
      const bool ok = v < SW;
      const double d = ok ? hd[v] : 0.0;
      // d <= 0 for a non-NaN double: its bits as a signed integer are <= 0
      const unsigned take = __ballot_sync(kFull, ok && __double_as_longlong(d) <= 0);
      if (!take)
      {
        att += (unsigned long long)min(32, SW - v0);
        v0 += 32;
        continue;
      }
      const int j = __ffs(take) - 1;
      const double dj = __shfl_sync(kFull, d, j);
      const int i = v0 + j;
      att += (unsigned long long)(j + 1);
      if (lane == 0) hs[i >> 5] ^= 1u << (i & 31);
      __syncwarp();
      acc++;
      S.hc_cost = __dadd_rn(S.hc_cost, dj);
      if (S.hc_cost < S.hc_low)
      {
        S.hc_low = S.hc_cost;
        warp_copy(hl, hs, nw, lane);
      }
      tabu_refresh<FL, INT>(m, hs, hd, i, lane);
      v0 = i + 1;
    }
    if (S.hc_low < prev)
    {
      low = S.hc_low;
      warp_copy(ls, hl, nw, lane);
    }
    else
      S.local = 0;
  };

  for (int step = 0; step < a.n_steps; step++)
  {
    if (S.local)
    {
      local_sweep();
      continue;
    }
    // the scan, markov/tabu_walker.h:68-127: 128 variables per round (four
    // loads in flight per lane), each lane keeping its own first-lowest
    // candidate off the tabu list.  fl(cost + d) < low is monotone in d, so
    // with t = fl(low - cost) and e = 2^-48 max(|cost|, |low|, |t|) every
    // d < fl(t - e) is taken and every d > fl(t + e) is not (the rounding
    // errors are below e / 16); only differences in between are added in FP64.
    bool taken = false;
    double bd = 0.0;
    unsigned long long bk = ~0ull;
    int bv = INT_MAX;
    const unsigned long long it = S.iter;
    const double t = __dadd_rn(low, -cost);
    const double e = fmax(__dmul_rn(fmax(fmax(fabs(cost), fabs(low)), fabs(t)), 0x1p-48), 0x1p-1000);
    const unsigned long long klo = fkey(__dadd_rn(t, -e)), khi = fkey(__dadd_rn(t, e));
    for (int c0 = 0; c0 < SW && !taken; c0 += 128)
    {
      double d[4];
      unsigned long long x[4];
#pragma unroll
      for (int u = 0; u < 4; u++)
      {
        const int v = c0 + 32 * u + lane;
        d[u] = v < SW ? df[v] : 0.0;
        x[u] = v < SW ? tb[v] : 0ull;
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
      {
        const int v = c0 + 32 * u + lane;
        const bool ok = v < SW;
        const unsigned long long k = fkey(d[u]);
        unsigned take = __ballot_sync(kFull, ok && k < klo);
        const unsigned near = __ballot_sync(kFull, ok && k >= klo && k <= khi);
        if (near) take |= __ballot_sync(kFull, ((near >> lane) & 1) && __dadd_rn(cost, d[u]) < low);
        if (take)
        {
          const int j = __ffs(take) - 1;
          const int i = c0 + 32 * u + j;
          const double di = __shfl_sync(kFull, d[u], j);
          taken = true;
          // attempt_transition accepted it: flip, cost, lowest
          if (lane == 0) sp[i >> 5] ^= 1u << (i & 31);
          __syncwarp();
          acc++;
          cost = __dadd_rn(cost, di);
          low = cost;
          warp_copy(ls, sp, nw, lane);
          if (lane == 0) tb[i] = it + tenure;
          tabu_refresh<FL, INT>(m, sp, df, i, lane);
          // local_search_init: a hill climber on a copy, its cost computed afresh
          warp_copy(hs, sp, nw, lane);
          warp_copy(hl, sp, nw, lane);
          for (int q = lane; q < N; q += 32) hd[q] = df[q];
          __syncwarp();
          double c;
          long long ic;
          warp_terms_cost<FL, INT>(m, hs, nullptr, lane, c, ic);
          S.hc_cost = INT ? (double)ic : c;
          S.hc_low = S.hc_cost;
          S.local = 1;
          S.incomplete += (unsigned long long)i;
          att += (unsigned long long)(i + 1);
          if (S.incomplete < (unsigned long long)SW)
            local_sweep();
          else
            S.incomplete -= (unsigned long long)SW;
          break;
        }
        if (ok && !(x[u] >= it) && k < bk)
        {
          bk = k;
          bd = d[u];
          bv = v;
        }
      }
    }
    if (!taken)
    {
      att += (unsigned long long)SW;
      // the lowest difference off the tabu list, the first on ties
#pragma unroll
      for (int sh = 16; sh; sh >>= 1)
      {
        const unsigned long long ok_ = __shfl_xor_sync(kFull, bk, sh);
        const double od = __shfl_xor_sync(kFull, bd, sh);
        const int ov = __shfl_xor_sync(kFull, bv, sh);
        if (ov != INT_MAX && (bv == INT_MAX || ok_ < bk || (ok_ == bk && ov < bv)))
        {
          bk = ok_;
          bd = od;
          bv = ov;
        }
      }
      if (bv != INT_MAX)
      {
        // Walker::apply_transition(transition, diff)
        if (lane == 0) sp[bv >> 5] ^= 1u << (bv & 31);
        __syncwarp();
        cost = __dadd_rn(cost, bd);
        if (cost < low)
        {
          low = cost;
          warp_copy(ls, sp, nw, lane);
        }
        if (lane == 0) tb[bv] = it + tenure;
        tabu_refresh<FL, INT>(m, sp, df, bv, lane);
      }
    }
    S.iter++;
    __syncwarp();
  }
  if (lane == 0)
  {
    a.st[w] = S;
    a.p.cost[w] = cost;
    a.p.lowest[w] = low;
    a.p.attempts[w] += att;
    a.p.accepts[w] += acc;
  }
}

// ---------------------------------------------------------------------------
// Substochastic Monte Carlo walker steps.  Replay: one thread per emulated
// OpenMP thread t of the reference, serving walkers [b_t, e_t) (libgomp's
// schedule(static) blocks) in index order on its PCG stream: per attempt one
// uniform() against p_step, then, when taken, one uniform() for the variable
// (floor(u * N), model/ising.h:138-143, model/pubo.h:102-107).  Counter
// mode: one thread per walker slot j, its c-th attempt drawing
// counter_draw(counter_key(seed, j), 2c) and (.., 2c + 1) as 53-bit uniforms.
// Every flip is accepted: cost += the difference (term order), lowest kept.
// ---------------------------------------------------------------------------
template <int FL, bool INT>
__device__ __forceinline__ void ssmc_flip(const DevModel& m, const DevPop& p, int w, int v)
{
  uint32_t* sp = p.spins + (size_t)w * p.nw;
  const double d = lane_diff<FL, INT>(m, sp, v);
  sp[v >> 5] ^= 1u << (v & 31);
  const double c = __dadd_rn(p.cost[w], d);
  p.cost[w] = c;
  p.attempts[w] += 1;
  p.accepts[w] += 1;
  if (c < p.lowest[w])
  {
    p.lowest[w] = c;
    uint32_t* ls = p.lspins + (size_t)w * p.nw;
    for (int q = 0; q < p.nw; q++) ls[q] = sp[q];
  }
}

template <int FL, bool INT>
__global__ void __launch_bounds__(128) ssmc_walk_kernel(SsmcArgs a)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int N = a.m.n_vars;
  const int spw = a.steps_per_walker;
  if (a.replay)
  {
    if (t >= a.n_chains) return;
    const int R = a.n_walkers, T = a.n_chains;
    const int q = R / T, r = R % T;
    const int b = t < r ? t * (q + 1) : t * q + r;
    const int e = b + (t < r ? q + 1 : q);
    uint64_t s = a.rng[t];
    auto uni = [&]() {
      const uint32_t d0 = pcg_out(s);
      s = s * kMult + kInc;
      const uint32_t d1 = pcg_out(s);
      s = s * kMult + kInc;
      return canonical(d0, d1);
    };
    for (int w = b; w < e; w++)
      for (int k = 0; k < spw; k++)
        if (uni() < a.p_step)
        {
          const int v = (int)__dmul_rn(uni(), (double)N);
          ssmc_flip<FL, INT>(a.m, a.p, w, v);
        }
    a.rng[t] = s;
  }
  else
  {
    if (t >= a.n_walkers) return;
    const uint64_t key = counter_key(a.seed, (uint64_t)t);
    for (int k = 0; k < spw; k++)
    {
      const unsigned long long c = (unsigned long long)a.step * (unsigned long long)spw + (unsigned long long)k;
      const double u = (double)(counter_draw(key, 2 * c) >> 11) * 0x1p-53;
      if (u < a.p_step)
      {
        const double u2 = (double)(counter_draw(key, 2 * c + 1) >> 11) * 0x1p-53;
        ssmc_flip<FL, INT>(a.m, a.p, t, (int)__dmul_rn(u2, (double)N));
      }
    }
  }
}

template <int FL, bool I>
static void ssmc_dispatch(const SsmcArgs& a, cudaStream_t s)
{
  const int n = a.replay ? a.n_chains : a.n_walkers;
  const int blocks = (n + 127) / 128;
  if (blocks > 0) ssmc_walk_kernel<FL, I><<<blocks, 128, 0, s>>>(a);
}

cudaError_t launch_ssmc_walk(const SsmcArgs& a, cudaStream_t s)
{
  if (a.n_walkers <= 0 || a.steps_per_walker <= 0) return cudaSuccess;
  const bool I = a.m.int_mode != 0;
  switch (a.m.flavor)
  {
    case F_PARITY: I ? ssmc_dispatch<F_PARITY, true>(a, s) : ssmc_dispatch<F_PARITY, false>(a, s); break;
    case F_COUNTER: I ? ssmc_dispatch<F_COUNTER, true>(a, s) : ssmc_dispatch<F_COUNTER, false>(a, s); break;
    case F_PLAIN_ISING: I ? ssmc_dispatch<F_PLAIN_ISING, true>(a, s) : ssmc_dispatch<F_PLAIN_ISING, false>(a, s); break;
    default: I ? ssmc_dispatch<F_PLAIN_PUBO, true>(a, s) : ssmc_dispatch<F_PLAIN_PUBO, false>(a, s); break;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Quantum Monte Carlo: one warp per restart, lanes over its slices (slice k
// on lane k % 32).  For each variable v of the ordered sweep: every slice
// computes its difference and, for k > 0 with the same value of v as slice
// k-1, its bond (a uniform() below bond_prob); each run of bonded slices
// (slice 0 and every unbonded slice start one) sums its differences in slice
// order, is accepted below 1e-11 or on a uniform() of its first slice below
// exp(-beta_eff * sum), and all its slices flip together.  The per-warp
// differences, bonds and acceptances sit in shared memory.  After each sweep
// the restart keeps the first lowest-cost slice if it beats its lowest.
// ---------------------------------------------------------------------------
// the 64 random bits of one uniform(): replay, the stream's next two
// outputs X = d0 + d1 2^32 (canonical(d0, d1) = fl(X) 2^-64, clamped below
// 1); counter, one counter draw (uniform = (draw >> 11) 2^-53)
__device__ __forceinline__ unsigned long long qmc_bits(const QmcArgs& a, int slot, unsigned long long ctr)
{
  if (a.replay)
  {
    uint64_t s = a.rng[slot];
    const uint32_t d0 = pcg_out(s);
    s = s * kMult + kInc;
    const uint32_t d1 = pcg_out(s);
    a.rng[slot] = s * kMult + kInc;
    return ((unsigned long long)d1 << 32) | d0;
  }
  return counter_draw(counter_key(a.seed, (uint64_t)slot), ctr);
}
__device__ __forceinline__ double qmc_uniform(const QmcArgs& a, unsigned long long x)
{
  if (a.replay) return canonical((uint32_t)x, (uint32_t)(x >> 32));
  return (double)(x >> 11) * 0x1p-53;
}

template <int FL, bool INT>
__global__ void __launch_bounds__(128) qmc_kernel(QmcArgs a)
{
  extern __shared__ unsigned char qsm[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int r = blockIdx.x * (blockDim.x >> 5) + wib;
  if (r >= a.restarts) return;  // whole warps leave together
  // SW variables are swept (1 for MaxSat unless the full sweep is asked
  // for); draw positions stay indexed by N
  const int P = a.trotter, N = a.m.n_vars, SW = a.m.sweep_size, nw = a.p.nw;
  const size_t per_warp = (size_t)P * 8 + (((size_t)P * 2 + 7) & ~(size_t)7);
  double* dif = (double*)(qsm + (size_t)wib * per_warp);
  uint8_t* bond = (uint8_t*)(dif + P);
  uint8_t* acc = bond + P;
  const int base = r * P;
  for (int st = 0; st < a.n_steps; st++)
  {
    const long long S = a.step_base + st;
    const double be = a.beta_eff[S];
    const float bef = (float)be;
    const unsigned long long blim = a.bond_lim[S];
    const bool ball = a.bond_all[S] != 0;
    for (int v = 0; v < SW; v++)
    {
      const unsigned long long c = 2ull * ((unsigned long long)S * (unsigned long long)N + (unsigned long long)v);
      for (int k = lane; k < P; k += 32)
      {
        const uint32_t* sp = a.p.spins + (size_t)(base + k) * nw;
        dif[k] = lane_diff<FL, INT>(a.m, sp, v);
        uint8_t b = 0;
        if (k > 0 && spin_of(sp - nw, v) == spin_of(sp, v))
        {
          const unsigned long long x = qmc_bits(a, base + k, c);
          b = a.replay ? (ball || x < blim) : ((x >> 11) < blim);
        }
        bond[k] = b;
      }
      __syncwarp();
      for (int k = lane; k < P; k += 32)
      {
        if (bond[k]) continue;
        double sum = dif[k];
        int e = k + 1;
        for (; e < P && bond[e]; e++) sum = __dadd_rn(sum, dif[e]);
        uint8_t ok = 1;
        if (!(sum < 10E-12))
        {
          const unsigned long long ub = qmc_bits(a, base + k, c + 1);
          // FP32 screen: the draw's top 24 bits are within 2^-23 of it;
          // x = -be sum rounded through float and expf's error stay below
          // ef (|xf| + 2) 2^-20; the FP64 exp decides only near the draw
          const float uf = (float)(uint32_t)(ub >> 40) * 0x1p-24f;
          const float xf = -bef * (float)sum, ef = expf(xf);
          const float te = ef * (fabsf(xf) + 2.0f) * 0x1p-20f;
          if (uf + 0x1p-23f < ef - te)
            ok = 1;
          else if (uf - 0x1p-23f > ef + te)
            ok = 0;
          else
          {
            const double u = qmc_uniform(a, ub);
            const double e = exp(__dmul_rn(-be, sum));
            if (fabs(u - e) <= 1e-15 * e) atomicAdd(a.near_ties, 1ULL);
            ok = u < e;
          }
        }
        for (int i = k; i < e; i++) acc[i] = ok;
      }
      __syncwarp();
      for (int k = lane; k < P; k += 32)
        if (acc[k])
        {
          uint32_t* sp = a.p.spins + (size_t)(base + k) * nw;
          sp[v >> 5] ^= 1u << (v & 31);
          a.p.cost[base + k] = __dadd_rn(a.p.cost[base + k], dif[k]);
          a.p.accepts[base + k] += 1;
        }
      __syncwarp();
    }
    // add_difference_evaluations + save_lowest (first lowest slice)
    double bc = 0.0;
    int bk = INT_MAX;
    for (int k = lane; k < P; k += 32)
    {
      a.p.attempts[base + k] += (unsigned long long)SW;
      const double ck = a.p.cost[base + k];
      if (bk == INT_MAX || ck < bc)
      {
        bc = ck;
        bk = k;
      }
    }
#pragma unroll
    for (int sh = 16; sh; sh >>= 1)
    {
      const double oc = __shfl_xor_sync(kFull, bc, sh);
      const int ok = __shfl_xor_sync(kFull, bk, sh);
      if (ok != INT_MAX && (bk == INT_MAX || oc < bc || (oc == bc && ok < bk)))
      {
        bc = oc;
        bk = ok;
      }
    }
    if (bc < a.low[r])
    {
      const uint32_t* src = a.p.spins + (size_t)(base + bk) * nw;
      for (int q = lane; q < nw; q += 32) a.low_spins[(size_t)r * nw + q] = src[q];
      __syncwarp();
      if (lane == 0) a.low[r] = bc;
    }
    __syncwarp();
  }
}

// Level-parallel QMC sweeps for counter streams (positional draws): one
// block per restart, its slices' spins in shared memory, the warps taking the
// variables of one level at a time (no two share a term, and every
// lower-index neighbour sits in an earlier level, so each variable sees the
// spins the ordered sweep would).  Flips are logged per slice; after the
// sweep each slice adds its flips' differences to its cost in variable order,
// as the ordered sweep's cost += diff does.
size_t qmc_level_smem(int trotter, int nw)
{
  if (trotter < 2 || trotter > 256) return 0;
  const size_t per_warp = (size_t)trotter * 8 + (((size_t)trotter * 2 + 7) & ~(size_t)7);
  const size_t b = 2 * (size_t)trotter * nw * 4 + kQmcLevelWarps * per_warp;
  return b <= 200 * 1024 ? b : 0;
}

template <int FL, bool INT>
__global__ void __launch_bounds__(kQmcLevelWarps * 32) qmc_level_kernel(QmcArgs a)
{
  extern __shared__ __align__(16) unsigned char qls[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int r = blockIdx.x;
  const int P = a.trotter, N = a.m.n_vars, nw = a.p.nw;
  uint32_t* sps = (uint32_t*)qls;
  uint32_t* flp = sps + (size_t)P * nw;
  const size_t per_warp = (size_t)P * 8 + (((size_t)P * 2 + 7) & ~(size_t)7);
  double* dif = (double*)((unsigned char*)(flp + (size_t)P * nw) + (size_t)wib * per_warp);
  uint8_t* bond = (uint8_t*)(dif + P);
  uint8_t* acc = bond + P;
  const int base = r * P;
  double* dl = a.dlog + (size_t)base * N;
  for (int i = threadIdx.x; i < P * nw; i += blockDim.x) sps[i] = a.p.spins[(size_t)base * nw + i];
  __syncthreads();
  for (int st = 0; st < a.n_steps; st++)
  {
    const long long S = a.step_base + st;
    const double be = a.beta_eff[S];
    const float bef = (float)be;
    const unsigned long long blim = a.bond_lim[S];
    for (int i = threadIdx.x; i < P * nw; i += blockDim.x) flp[i] = 0;
    __syncthreads();
    for (int L = 0; L < a.n_levels; L++)
    {
      const int e1 = a.lv_off[L + 1];
      for (int e = a.lv_off[L] + wib; e < e1; e += nwarps)
      {
        const int v = a.lv_var[e];
        const unsigned long long c =
            2ull * ((unsigned long long)S * (unsigned long long)N + (unsigned long long)v);
        for (int k = lane; k < P; k += 32)
        {
          const uint32_t* sp = sps + (size_t)k * nw;
          dif[k] = lane_diff<FL, INT>(a.m, sp, v);
          uint8_t b = 0;
          if (k > 0 && spin_of(sp - nw, v) == spin_of(sp, v))
            b = (counter_draw(counter_key(a.seed, (uint64_t)(base + k)), c) >> 11) < blim;
          bond[k] = b;
        }
        __syncwarp();
        for (int k = lane; k < P; k += 32)
        {
          if (bond[k]) continue;
          double sum = dif[k];
          int q = k + 1;
          for (; q < P && bond[q]; q++) sum = __dadd_rn(sum, dif[q]);
          uint8_t ok = 1;
          if (!(sum < 10E-12))
          {
            const unsigned long long ub = counter_draw(counter_key(a.seed, (uint64_t)(base + k)), c + 1);
            const float uf = (float)(uint32_t)(ub >> 40) * 0x1p-24f;
            const float xf = -bef * (float)sum, ef = expf(xf);
            const float te = ef * (fabsf(xf) + 2.0f) * 0x1p-20f;
            if (uf + 0x1p-23f < ef - te)
              ok = 1;
            else if (uf - 0x1p-23f > ef + te)
              ok = 0;
            else
            {
              const double u = (double)(ub >> 11) * 0x1p-53;
              const double x = exp(__dmul_rn(-be, sum));
              if (fabs(u - x) <= 1e-15 * x) atomicAdd(a.near_ties, 1ULL);
              ok = u < x;
            }
          }
          for (int i = k; i < q; i++) acc[i] = ok;
        }
        __syncwarp();
        for (int k = lane; k < P; k += 32)
          if (acc[k])
          {
            atomicXor(&sps[(size_t)k * nw + (v >> 5)], 1u << (v & 31));
            atomicOr(&flp[(size_t)k * nw + (v >> 5)], 1u << (v & 31));
            dl[(size_t)k * N + v] = dif[k];
          }
        __syncwarp();
      }
      __syncthreads();
    }
    // cost += diff over the sweep's flips in variable order, per slice
    for (int k = threadIdx.x; k < P; k += blockDim.x)
    {
      double cst = a.p.cost[base + k];
      unsigned long long nf = 0;
      for (int q = 0; q < nw; q++)
      {
        uint32_t f = flp[(size_t)k * nw + q];
        while (f)
        {
          const int b = __ffs(f) - 1;
          f &= f - 1;
          cst = __dadd_rn(cst, dl[(size_t)k * N + q * 32 + b]);
          nf++;
        }
      }
      a.p.cost[base + k] = cst;
      a.p.accepts[base + k] += nf;
      a.p.attempts[base + k] += (unsigned long long)N;
    }
    __syncthreads();
    if (wib == 0)
    {
      double bc = 0.0;
      int bk = INT_MAX;
      for (int k = lane; k < P; k += 32)
      {
        const double ck = a.p.cost[base + k];
        if (bk == INT_MAX || ck < bc)
        {
          bc = ck;
          bk = k;
        }
      }
#pragma unroll
      for (int sh = 16; sh; sh >>= 1)
      {
        const double oc = __shfl_xor_sync(kFull, bc, sh);
        const int ok = __shfl_xor_sync(kFull, bk, sh);
        if (ok != INT_MAX && (bk == INT_MAX || oc < bc || (oc == bc && ok < bk)))
        {
          bc = oc;
          bk = ok;
        }
      }
      if (bc < a.low[r])
      {
        for (int q = lane; q < nw; q += 32) a.low_spins[(size_t)r * nw + q] = sps[(size_t)bk * nw + q];
        __syncwarp();
        if (lane == 0) a.low[r] = bc;
      }
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < P * nw; i += blockDim.x) a.p.spins[(size_t)base * nw + i] = sps[i];
}

template <int FL, bool I>
static cudaError_t qmc_level_dispatch(const QmcArgs& a, cudaStream_t s)
{
  const size_t smem = qmc_level_smem(a.trotter, a.p.nw);
  if (smem > 48 * 1024)
  {
    cudaError_t e =
        cudaFuncSetAttribute(qmc_level_kernel<FL, I>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  qmc_level_kernel<FL, I><<<a.restarts, kQmcLevelWarps * 32, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_qmc_levels(const QmcArgs& a, cudaStream_t s)
{
  if (a.restarts <= 0 || a.n_steps <= 0) return cudaSuccess;
  if (a.replay || !qmc_level_smem(a.trotter, a.p.nw) || !a.lv_off || !a.lv_var || !a.dlog)
    return cudaErrorInvalidValue;
  const bool I = a.m.int_mode != 0;
  switch (a.m.flavor)
  {
    case F_PARITY: return I ? qmc_level_dispatch<F_PARITY, true>(a, s) : qmc_level_dispatch<F_PARITY, false>(a, s);
    case F_COUNTER: return I ? qmc_level_dispatch<F_COUNTER, true>(a, s) : qmc_level_dispatch<F_COUNTER, false>(a, s);
    case F_PLAIN_ISING:
      return I ? qmc_level_dispatch<F_PLAIN_ISING, true>(a, s) : qmc_level_dispatch<F_PLAIN_ISING, false>(a, s);
    default: return I ? qmc_level_dispatch<F_PLAIN_PUBO, true>(a, s) : qmc_level_dispatch<F_PLAIN_PUBO, false>(a, s);
  }
}

template <int FL, bool I>
static cudaError_t qmc_dispatch(const QmcArgs& a, cudaStream_t s)
{
  const size_t per_warp = (size_t)a.trotter * 8 + (((size_t)a.trotter * 2 + 7) & ~(size_t)7);
  const int blocks = (a.restarts + 3) / 4;
  const size_t smem = 4 * per_warp;
  if (smem > 48 * 1024)
  {
    cudaError_t e = cudaFuncSetAttribute(qmc_kernel<FL, I>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  if (blocks > 0) qmc_kernel<FL, I><<<blocks, 128, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_qmc(const QmcArgs& a, cudaStream_t s)
{
  if (a.restarts <= 0 || a.n_steps <= 0) return cudaSuccess;
  if (a.trotter < 2 || a.trotter > kQmcMaxTrotter) return cudaErrorInvalidValue;
  const bool I = a.m.int_mode != 0;
  switch (a.m.flavor)
  {
    case F_PARITY: return I ? qmc_dispatch<F_PARITY, true>(a, s) : qmc_dispatch<F_PARITY, false>(a, s);
    case F_COUNTER: return I ? qmc_dispatch<F_COUNTER, true>(a, s) : qmc_dispatch<F_COUNTER, false>(a, s);
    case F_PLAIN_ISING: return I ? qmc_dispatch<F_PLAIN_ISING, true>(a, s) : qmc_dispatch<F_PLAIN_ISING, false>(a, s);
    default: return I ? qmc_dispatch<F_PLAIN_PUBO, true>(a, s) : qmc_dispatch<F_PLAIN_PUBO, false>(a, s);
  }
}

// ---------------------------------------------------------------------------
// PT: observations then alternating-parity neighbour swaps of the slot
// labels (solver/parallel_tempering.h:134-189); one thread per restart.
// ---------------------------------------------------------------------------
__global__ void pt_swap_kernel(SwapArgs a)
{
  // one warp per restart: lanes over the ladder's walkers, then over the
  // step's pairs (pairs of one parity share no walker)
  const int lane = threadIdx.x & 31;
  const int k = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (k >= a.restarts) return;
  const int T = a.n_temps;
  const int base = k * T;
  for (int p = lane; p < T; p += 32)
  {
    const int w = base + p;
    const double att = (double)a.step_att_reset[w];
    const double acc = (double)a.step_acc_reset[w];
    a.obs_acc[w] = __dadd_rn(a.obs_acc[w], __ddiv_rn(acc, att));
    a.obs_cost[w] = __dadd_rn(a.obs_cost[w], a.cost[a.slot_of[w]]);
    a.obs_dir[w] = __dadd_rn(a.obs_dir[w], (double)a.dir[w]);
    a.step_att_reset[w] = 0;
    a.step_acc_reset[w] = 0;
  }
  __syncwarp();
  // pair j of the step is (i, i + 1), i = (step & 1) + 2j; replayed, it
  // takes draws 2j and 2j + 1 of the master stream (the reference's loop
  // draws them in pair order)
  const int first = (int)(a.step & 1);
  const int npairs = T - 1 > first ? (T - first) / 2 : 0;
  uint64_t ms = a.replay ? a.master[k] : 0;
  for (int j0 = 0; j0 < npairs; j0 += 32)
  {
    const int j = j0 + lane;
    if (j < npairs)
    {
      const int i = first + 2 * j;
      double u;
      if (a.replay)
      {
        uint64_t sj = c_jA[2 * lane] * ms + c_jC[2 * lane];
        const uint32_t d0 = pcg_out(sj);
        sj = sj * kMult + kInc;
        const uint32_t d1 = pcg_out(sj);
        u = canonical(d0, d1);
      }
      else
      {
        const uint64_t wd = counter_draw(a.swap_key[k], (unsigned long long)a.step * (unsigned long long)T +
                                                            (unsigned long long)i);
        u = __dmul_rn((double)(wd >> 11), 1.0 / 9007199254740992.0);
      }
      const int wa = base + i, wb = base + i + 1;
      const double x = __dmul_rn(__dsub_rn(a.cost[a.slot_of[wa]], a.cost[a.slot_of[wb]]),
                                 __dsub_rn(a.beta[wa], a.beta[wb]));
      double e = exp(x);
      if (fabs(u - e) <= 1e-15 * e)
      {
        // near tie: the correctly rounded exp, which the C library's exp
        // (the reference's) returns except for its rare misroundings
        e = dd::exp_cr(x);
        atomicAdd(a.near_ties, 1ULL);
      }
      if (u < e)
      {
        const int t = a.slot_of[wa];
        a.slot_of[wa] = a.slot_of[wb];
        a.slot_of[wb] = t;
        const int d = a.dir[wa];
        a.dir[wa] = a.dir[wb];
        a.dir[wb] = d;
        a.swap_acc[wa] += 1;
      }
      a.swap_cnt[wa] += 1;
    }
    // the master stream moves past this chunk's draws (at most 64)
    const int nin = min(32, npairs - j0);
    if (a.replay) ms = c_jA[2 * nin] * ms + c_jC[2 * nin];
  }
  __syncwarp();
  if (lane == 0)
  {
    a.dir[base] = 0;
    a.dir[base + T - 1] = 1;
    if (a.replay) a.master[k] = ms;
  }
}

// ---------------------------------------------------------------------------
// PA resampling copies (Population::resample, solver/population.h:171-218):
// every destination walker is an integer copy of its source walker.
// ---------------------------------------------------------------------------
__global__ void pa_copy_kernel(DevPop src, DevPop dst, const int* src_of, int n_dst)
{
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= n_dst) return;
  const int i = src_of[j];
  const uint4* a = (const uint4*)(src.spins + (size_t)i * src.nw);
  uint4* b = (uint4*)(dst.spins + (size_t)j * dst.nw);
  for (int q = lane; q < src.nw / 4; q += 32) b[q] = a[q];
  a = (const uint4*)(src.lspins + (size_t)i * src.nw);
  b = (uint4*)(dst.lspins + (size_t)j * dst.nw);
  for (int q = lane; q < src.nw / 4; q += 32) b[q] = a[q];
  a = (const uint4*)(src.tstate + (size_t)i * src.mp);
  b = (uint4*)(dst.tstate + (size_t)j * dst.mp);
  for (int q = lane; q < src.mp / 16; q += 32) b[q] = a[q];
  if (lane == 0)
  {
    dst.cost[j] = src.cost[i];
    dst.lowest[j] = src.lowest[i];
    dst.attempts[j] = src.attempts[i];
    dst.accepts[j] = src.accepts[i];
    dst.step_att[j] = 0;
    dst.step_acc[j] = 0;
    if (dst.windows) dst.windows[j] = src.windows ? src.windows[i] : 0;
  }
}

cudaError_t launch_pa_copy(const DevPop& src, const DevPop& dst, const int* src_of,
                           int n_dst, cudaStream_t s)
{
  int blocks = (n_dst + 7) / 8;
  if (blocks > 0) pa_copy_kernel<<<blocks, 256, 0, s>>>(src, dst, src_of, n_dst);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void sw_upload(const double* ln, const float* scr, const unsigned long long* jA,
               const unsigned long long* jC);
void fc_upload(const double* ln, const float* scr, const unsigned long long* jA,
               const unsigned long long* jC);

void upload_tables(int)
{
  double ln[1024];
  for (int row = 0; row < 4; row++)
    for (int i = 0; i < 256; i++)
      ln[row * 256 + i] = log((i) / pow((double)256, (double)(row + 1)));
  unsigned long long jA[65], jC[65], pA[64], pC[64];
  jA[0] = 1;
  jC[0] = 0;
  for (int k = 1; k < 65; k++)
  {
    jA[k] = jA[k - 1] * kMult;
    jC[k] = jC[k - 1] * kMult + kInc;
  }
  pA[0] = kMult;
  pC[0] = kInc;
  for (int k = 1; k < 64; k++)
  {
    pA[k] = pA[k - 1] * pA[k - 1];
    pC[k] = pA[k - 1] * pC[k - 1] + pC[k - 1];
  }
  cudaMemcpyToSymbol(c_ln, ln, sizeof ln);
  cudaMemcpyToSymbol(c_jA, jA, sizeof jA);
  cudaMemcpyToSymbol(c_jC, jC, sizeof jC);
  cudaMemcpyToSymbol(c_pA, pA, sizeof pA);
  cudaMemcpyToSymbol(c_pC, pC, sizeof pC);
  // FP32 screen of the ln-table comparison: per (row, bucket) the double
  // y0 and RN(y1 - y0) rounded to float, and an error margin 2^-19 (|y0| +
  // |dy|) that covers the float rounding of y0, dy, the distance and the
  // multiply-add against the double expression
  float scr[3072];
  for (int row = 0; row < 4; row++)
    for (int b = 0; b < 256; b++)
    {
      float* e = scr + (row * 256 + b) * 3;
      if (b < 2)
      {
        e[0] = e[1] = e[2] = 0.f;
        continue;
      }
      double y0 = ln[row * 256 + b - 1], dy = ln[row * 256 + b] - y0;
      e[0] = (float)y0;
      e[1] = (float)dy;
      e[2] = (float)(ldexp(fabs(y0) + fabs(dy), -19));
    }
  sw_upload(ln, scr, jA, jC);
  fc_upload(ln, scr, jA, jC);
  lw_upload(ln, scr);
  lv_upload(ln, scr);
}

template <int FL, bool INT>
static void init_dispatch(const InitArgs& a, cudaStream_t s)
{
  const int wpb = 4;
  int blocks = (a.n_walkers + wpb - 1) / wpb;
  if (blocks > 0) init_kernel<FL, INT><<<blocks, 32 * wpb, 0, s>>>(a);
}

cudaError_t launch_init(const InitArgs& a, cudaStream_t s)
{
  const bool I = a.m.int_mode != 0;
  switch (a.m.flavor)
  {
    case F_PARITY: I ? init_dispatch<F_PARITY, true>(a, s) : init_dispatch<F_PARITY, false>(a, s); break;
    case F_COUNTER: I ? init_dispatch<F_COUNTER, true>(a, s) : init_dispatch<F_COUNTER, false>(a, s); break;
    case F_PLAIN_ISING: I ? init_dispatch<F_PLAIN_ISING, true>(a, s) : init_dispatch<F_PLAIN_ISING, false>(a, s); break;
    default: I ? init_dispatch<F_PLAIN_PUBO, true>(a, s) : init_dispatch<F_PLAIN_PUBO, false>(a, s); break;
  }
  return cudaGetLastError();
}

template <int FL, bool I>
static void cost_dispatch(const DevModel& m, int n, const uint32_t* sp, int nw,
                          double* out, cudaStream_t s)
{
  int blocks = (n + 3) / 4;
  if (blocks > 0) eval_cost_kernel<FL, I><<<blocks, 128, 0, s>>>(m, n, sp, nw, out);
}

cudaError_t launch_eval_cost(const DevModel& m, int n, const uint32_t* sp,
                             int nw, double* out, cudaStream_t s)
{
  const bool I = m.int_mode != 0;
  switch (m.flavor)
  {
    case F_PARITY: I ? cost_dispatch<F_PARITY, true>(m, n, sp, nw, out, s) : cost_dispatch<F_PARITY, false>(m, n, sp, nw, out, s); break;
    case F_COUNTER: I ? cost_dispatch<F_COUNTER, true>(m, n, sp, nw, out, s) : cost_dispatch<F_COUNTER, false>(m, n, sp, nw, out, s); break;
    case F_PLAIN_ISING: I ? cost_dispatch<F_PLAIN_ISING, true>(m, n, sp, nw, out, s) : cost_dispatch<F_PLAIN_ISING, false>(m, n, sp, nw, out, s); break;
    default: I ? cost_dispatch<F_PLAIN_PUBO, true>(m, n, sp, nw, out, s) : cost_dispatch<F_PLAIN_PUBO, false>(m, n, sp, nw, out, s); break;
  }
  return cudaGetLastError();
}

template <int FL, bool I>
static void diff_dispatch(const DevModel& m, int n, const uint32_t* sp, int nw,
                          const long long* vars, double* out, cudaStream_t s)
{
  int blocks = (n + 3) / 4;
  if (blocks > 0) eval_diff_kernel<FL, I><<<blocks, 128, 0, s>>>(m, n, sp, nw, vars, out);
}

cudaError_t launch_eval_diff(const DevModel& m, int n, const uint32_t* sp,
                             int nw, const long long* vars, double* out,
                             cudaStream_t s)
{
  const bool I = m.int_mode != 0;
  switch (m.flavor)
  {
    case F_PARITY: I ? diff_dispatch<F_PARITY, true>(m, n, sp, nw, vars, out, s) : diff_dispatch<F_PARITY, false>(m, n, sp, nw, vars, out, s); break;
    case F_COUNTER: I ? diff_dispatch<F_COUNTER, true>(m, n, sp, nw, vars, out, s) : diff_dispatch<F_COUNTER, false>(m, n, sp, nw, vars, out, s); break;
    case F_PLAIN_ISING: I ? diff_dispatch<F_PLAIN_ISING, true>(m, n, sp, nw, vars, out, s) : diff_dispatch<F_PLAIN_ISING, false>(m, n, sp, nw, vars, out, s); break;
    default: I ? diff_dispatch<F_PLAIN_PUBO, true>(m, n, sp, nw, vars, out, s) : diff_dispatch<F_PLAIN_PUBO, false>(m, n, sp, nw, vars, out, s); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_pt_swap(const SwapArgs& a, cudaStream_t s)
{
  const int threads = 128;  // four restarts per block, a warp each
  const int blocks = (a.restarts * 32 + threads - 1) / threads;
  if (blocks > 0) pt_swap_kernel<<<blocks, threads, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free cost evaluation.  Callers that must not allocate device
// memory while they run -- a serving loop that has handed the free HBM to
// resident solves, or a host thread that cannot afford the device-wide
// synchronisation cudaMalloc / cudaFree bring -- evaluate the cost of states
// that already sit on the device here.  The packed spin words, the only
// scratch the cost kernel needs, go to the fixed file-scope array below
// instead of a buffer allocated per call.
//
// Limits and sharing: the array holds kNoAllocScratchWords 32-bit words
// (1 MiB); a call needs n_states * ceil(n_vars / 32) words, and the entry
// point rejects larger requests before launching.  Every word a call uses
// is written before it is read, so nothing in the array has to start at
// zero.  All calls on one device share the array: calls that overlap in
// time (different streams or host threads) race on it and must be
// serialised by the caller.  The first call on each device looks up the
// array's device address (cudaGetSymbolAddress) with that device current and
// loads the kernel of every model flavour (cudaFuncGetAttributes), so later
// calls load nothing; make that first call before any stream capture.
// ---------------------------------------------------------------------------
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchWords];

template <int FL, bool INT>
__global__ void eval_cost_noalloc_kernel(DevModel m, int n, const uint8_t* states, int n_vars,
                                         int nw, uint32_t* scratch, double* out)
{
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= n) return;
  // pack this state's bytes into its own scratch words (coalesced reads)
  const uint8_t* st = states + (size_t)w * n_vars;
  uint32_t* sp = scratch + (size_t)w * nw;
  for (int q = 0; q < nw; q++)
  {
    const int v = q * 32 + lane;
    const unsigned word = __ballot_sync(kFull, v < n_vars && st[v] != 0);
    if (lane == 0) sp[q] = word;
  }
  __syncwarp();
  double c;
  long long ic;
  warp_cost<FL, INT>(m, sp, lane, c, ic);
  if (lane == 0) out[w] = INT ? (double)ic : c;
}

template <int FL, bool I>
static void cost_noalloc_dispatch(const DevModel& m, int n, const uint8_t* st, int n_vars, int nw,
                                  uint32_t* scratch, double* out, cudaStream_t s)
{
  int blocks = (n + 3) / 4;
  if (blocks > 0) eval_cost_noalloc_kernel<FL, I><<<blocks, 128, 0, s>>>(m, n, st, n_vars, nw, scratch, out);
}

cudaError_t launch_eval_cost_noalloc(const DevModel& m, int n, const uint8_t* states, int n_vars,
                                     int nw, double* out, cudaStream_t s)
{
  if ((long long)n * (long long)nw > (long long)kNoAllocScratchWords) return cudaErrorInvalidValue;
  // set-up once per device, with that device current: the array's address
  static std::mutex mu;
  static uint32_t* addr[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  uint32_t* scratch = nullptr;
  {
    std::lock_guard<std::mutex> g(mu);
    if (!addr[dev])
    {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return e;
      // load every flavour's kernel now, so that no later call (another model
      // flavour) loads a module lazily inside a capture
      cudaFuncAttributes fa;
      const void* fns[] = {
          (const void*)eval_cost_noalloc_kernel<F_PARITY, true>,
          (const void*)eval_cost_noalloc_kernel<F_PARITY, false>,
          (const void*)eval_cost_noalloc_kernel<F_COUNTER, true>,
          (const void*)eval_cost_noalloc_kernel<F_COUNTER, false>,
          (const void*)eval_cost_noalloc_kernel<F_PLAIN_ISING, true>,
          (const void*)eval_cost_noalloc_kernel<F_PLAIN_ISING, false>,
          (const void*)eval_cost_noalloc_kernel<F_PLAIN_PUBO, true>,
          (const void*)eval_cost_noalloc_kernel<F_PLAIN_PUBO, false>};
      for (const void* f : fns)
      {
        e = cudaFuncGetAttributes(&fa, f);
        if (e != cudaSuccess) return e;
      }
      addr[dev] = (uint32_t*)p;
    }
    scratch = addr[dev];
  }
  const bool I = m.int_mode != 0;
  switch (m.flavor)
  {
    case F_PARITY: I ? cost_noalloc_dispatch<F_PARITY, true>(m, n, states, n_vars, nw, scratch, out, s) : cost_noalloc_dispatch<F_PARITY, false>(m, n, states, n_vars, nw, scratch, out, s); break;
    case F_COUNTER: I ? cost_noalloc_dispatch<F_COUNTER, true>(m, n, states, n_vars, nw, scratch, out, s) : cost_noalloc_dispatch<F_COUNTER, false>(m, n, states, n_vars, nw, scratch, out, s); break;
    case F_PLAIN_ISING: I ? cost_noalloc_dispatch<F_PLAIN_ISING, true>(m, n, states, n_vars, nw, scratch, out, s) : cost_noalloc_dispatch<F_PLAIN_ISING, false>(m, n, states, n_vars, nw, scratch, out, s); break;
    default: I ? cost_noalloc_dispatch<F_PLAIN_PUBO, true>(m, n, states, n_vars, nw, scratch, out, s) : cost_noalloc_dispatch<F_PLAIN_PUBO, false>(m, n, states, n_vars, nw, scratch, out, s); break;
  }
  return cudaGetLastError();
}
template <int FL, bool I>
static void tabu_dispatch(const TabuArgs& a, cudaStream_t s)
{
  const int blocks = (a.n_walkers + 3) / 4;
  if (blocks > 0) tabu_kernel<FL, I><<<blocks, 128, 0, s>>>(a);
}

cudaError_t launch_tabu(const TabuArgs& a, cudaStream_t s)
{
  if (a.n_walkers <= 0 || a.n_steps <= 0) return cudaSuccess;
  const bool I = a.m.int_mode != 0;
  switch (a.m.flavor)
  {
    case F_PARITY: I ? tabu_dispatch<F_PARITY, true>(a, s) : tabu_dispatch<F_PARITY, false>(a, s); break;
    case F_COUNTER: I ? tabu_dispatch<F_COUNTER, true>(a, s) : tabu_dispatch<F_COUNTER, false>(a, s); break;
    case F_PLAIN_ISING: I ? tabu_dispatch<F_PLAIN_ISING, true>(a, s) : tabu_dispatch<F_PLAIN_ISING, false>(a, s); break;
    default: I ? tabu_dispatch<F_PLAIN_PUBO, true>(a, s) : tabu_dispatch<F_PLAIN_PUBO, false>(a, s); break;
  }
  return cudaGetLastError();
}
}  // namespace qio
