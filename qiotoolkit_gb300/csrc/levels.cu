// levels.cu -- level-scheduled ordered sweeps for Ising models with one- or
// two-member terms and integer coefficients, counter streams.
//
// One warp runs one walker.  The reference's ordered sweep visits the
// variables 0..N-1 in turn (markov/walker.h:143-153); the attempt at v sums
// its incident terms from the spins as they are at that moment (the new
// value of a neighbour u < v, the old one of a neighbour u > v;
// model/ising.h:108-117) and decides with the draws of attempt v.  In
// counter mode those draws are a function of (walker, sweep, v) alone, so any
// schedule that runs v after all its lower neighbours and before all its
// higher ones makes the same decisions and reaches the same spins.  The host
// gives each variable level(v) = 1 + the largest level of its lower
// neighbours (0 without one): the variables of one level share no term, run
// at once across the warp, and the levels run in order.  An L x L periodic
// lattice has 2L - 1 levels of up to L variables.
//
// Cost and lowest: the reference adds each accepted difference to the cost
// and keeps the first state whose cost drops below the lowest seen
// (markov/walker.h:209-229,269-280).  The host cuts 0..N-1 into chunks,
// maximal runs of consecutive variables whose level does not decrease: a
// chunk's variables are visited in index order, those of one level by its
// lane one after the other.  Lane l owns
// chunks l, l + 32, ... and keeps for each the sum of its accepted
// differences, the smallest of its prefix sums and the variable where that
// first occurred.  After the sweep a scan over the chunks in index order puts
// the running cost of the reference at every accepted flip within reach: its
// minimum, and the first variable reaching it, are the sweep's candidate for
// a new lowest (all in integers, so the sums are the reference's exactly).
// The lowest spins are then the end-of-sweep spins up to that variable and
// the start-of-sweep spins (copied out when the sweep starts) after it.
//
// Spins live in shared memory for the whole launch, bit-packed, word w at
// w + w / 32 so that lanes walking rows of a lattice hit different banks.
// Flips are shared-memory XORs: two variables of one level may share a word.
#include <algorithm>
#include <climits>

#include "metropolis.cuh"
#include "qio_internal.h"

namespace qio
{
namespace lv
{
using namespace qio::mc;

__device__ double g_ln[1024];
__device__ float g_scr[1024 * 3];

__host__ __device__ __forceinline__ int phys(int w) { return w + (w >> 5); }

template <bool PACK>
struct Rec;
template <>
struct Rec<true>
{
  using T = unsigned int;
  static __device__ __forceinline__ int other(T r) { return (int)(r >> 8); }
  static __device__ __forceinline__ int coef(T r) { return (int)(signed char)(r & 0xFFu); }
};
template <>
struct Rec<false>
{
  using T = int2;
  static __device__ __forceinline__ int other(T r) { return r.x; }
  static __device__ __forceinline__ int coef(T r) { return r.y; }
};

// Running sum of a chunk's accepted differences and its smallest prefix sum:
// two ints, or one word of two 16-bit halves (low: sum, high: minimum) when
// every chunk's differences add up to less than 2^15 in magnitude.
template <bool P16>
struct ChunkSum;
template <>
struct ChunkSum<false>
{
  int s, m;
  __device__ __forceinline__ void init()
  {
    s = 0;
    m = INT_MAX;
  }
  __device__ __forceinline__ bool add(int d)  // true: a new smallest prefix
  {
    s += d;
    if (s < m)
    {
      m = s;
      return true;
    }
    return false;
  }
  __device__ __forceinline__ int sum() const { return s; }
  __device__ __forceinline__ int min() const { return m; }
};
template <>
struct ChunkSum<true>
{
  unsigned w;
  __device__ __forceinline__ void init() { w = 0x7FFF0000u; }
  __device__ __forceinline__ bool add(int d)
  {
    const int s = (int)(short)(w & 0xFFFFu) + d;
    if (s < ((int)w >> 16))
    {
      w = ((unsigned)s << 16) | ((unsigned)s & 0xFFFFu);
      return true;
    }
    w = (w & 0xFFFF0000u) | ((unsigned)s & 0xFFFFu);
    return false;
  }
  __device__ __forceinline__ int sum() const { return (int)(short)(w & 0xFFFFu); }
  __device__ __forceinline__ int min() const { return (int)w >> 16; }
};

// warps per block the kernel is compiled for: 28 (72 registers) up to 8
// chunks per lane, 16 (128 registers) for 16
template <int CPL>
struct LvWarps
{
  static const int value = CPL >= 16 ? 16 : kLvMaxWarps;
};

// CPL: chunks per lane (the model's chunks <= 32 * CPL)
template <int CPL, bool PACK, bool P16>
__global__ void __launch_bounds__(LvWarps<CPL>::value * 32, 1) lv_sweep_kernel(LvArgs a, int stride)
{
  using R = typename Rec<PACK>::T;
  extern __shared__ __align__(16) uint32_t lv_smem[];
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int r = blockIdx.x * (blockDim.x >> 5) + wib;
  if (r >= a.n_walkers) return;  // whole warps leave together
  const int N = a.m.n_vars, nwd = (N + 31) >> 5;
  const int* __restrict__ row = a.m.row;
  const unsigned short* __restrict__ lvl = a.m.lvl;
  const int* __restrict__ chunk = a.m.chunk;
  const R* __restrict__ rec = PACK ? (const R*)a.m.rec_p : (const R*)a.m.rec_i;
  const int nch = a.m.n_chunks, nlev = a.m.n_levels;
  const double* ln = g_ln;
  const float* scr = g_scr;

  uint32_t* sp = lv_smem + (size_t)wib * stride;
  const int slot = a.slot_of ? a.slot_of[r] : r;
  uint32_t* gs = a.p.spins + (size_t)slot * a.p.nw;
  uint32_t* ls = a.p.lspins + (size_t)r * a.p.nw;
  uint32_t* st = a.start + (size_t)r * a.p.nw;
  for (int w = lane; w < nwd; w += 32) sp[phys(w)] = gs[w];
  if (lane == 0) sp[phys(nwd)] = 0u;  // the padding spin of one-member terms
  __syncwarp();

  long long icost = (long long)a.p.cost[slot], ilow = (long long)a.p.lowest[r];
  const uint64_t key = counter_key(a.seed + (uint32_t)((long long)r / a.key_div),
                                   a.key_base + (unsigned long long)((long long)r % a.key_div));
  unsigned long long nacc = 0;
  auto spin = [&](int u) -> uint32_t { return (sp[phys(u >> 5)] >> (u & 31)) & 1u; };

  for (int k = 0; k < a.n_sweeps; k++)
  {
    const long long swp = a.sweep_base + k;
    const double beta = a.beta[(long long)r * a.bs_w + swp * a.bs_s];
    const bool beta_inf =
        ((unsigned long long)__double_as_longlong(beta) & 0x7FFFFFFFFFFFFFFFULL) == 0x7FF0000000000000ULL;
    const float nbeta_f = -approx_float(beta);
    const unsigned long long ctr0 = (unsigned long long)swp * (unsigned long long)N;
    for (int w = lane; w < nwd; w += 32) st[w] = sp[phys(w)];

    // per chunk: next variable, (variables left after it << 16 | its level),
    // sum of accepted differences, smallest prefix sum and where it fell
    int pos[CPL], ppos[CPL];
    ChunkSum<P16> cs[CPL];
    unsigned rl[CPL];
    unsigned int sacc = 0;
#pragma unroll
    for (int c = 0; c < CPL; c++)
    {
      const int kc = c * 32 + lane;
      cs[c].init();
      ppos[c] = -1;
      pos[c] = 0;
      rl[c] = 0xFFFFu;
      if (kc < nch)
      {
        const int b = __ldg(chunk + kc), e = __ldg(chunk + kc + 1);
        pos[c] = b;
        rl[c] = ((unsigned)(e - b - 1) << 16) | (unsigned)__ldg(lvl + b);
      }
    }
    for (int t = 0; t < nlev; t++)
    {
#pragma unroll
      for (int c = 0; c < CPL; c++)
      {
        // the chunk's variables at this level, in index order
        while ((int)(rl[c] & 0xFFFFu) == t)
        {
        const int v = pos[c];
        const uint32_t sv = spin(v);
        const int qb = __ldg(row + v), qe = __ldg(row + v + 1);
        int iacc = 0;
#pragma unroll 4
        for (int q = qb; q < qe; q++)
        {
          const R rq = __ldg(rec + q);
          const int cf = Rec<PACK>::coef(rq);
          iacc += (sv ^ spin(Rec<PACK>::other(rq))) ? -cf : cf;
        }
        const int idE = -2 * iacc;
        bool acc = idE <= 0;
        if (!acc)
        {
          // Metropolis::accept (markov/metropolis.h:64-104) on the draws of
          // attempt ctr0 + v: words 2 ctr and 2 ctr + 1, two draws each
          const unsigned long long ctr = ctr0 + (unsigned long long)v;
          const uint64_t w0 = counter_draw(key, 2ULL * ctr);
          uint32_t cur = (uint32_t)w0;
          int rw = 0;
          if ((cur & 255u) == 0u)
          {
            cur = (uint32_t)(w0 >> 32);
            rw = 1;
            if ((cur & 255u) == 0u)
            {
              const uint64_t w1 = counter_draw(key, 2ULL * ctr + 1ULL);
              cur = (uint32_t)w1;
              rw = 2;
              if ((cur & 255u) == 0u)
              {
                cur = (uint32_t)(w1 >> 32);
                rw = 3;
              }
            }
          }
          if ((cur & 255u) == 0u) acc = true;  // four zero buckets: accept
          else if (beta_inf) acc = false;
          else
          {
            // the difference is an integer: its float is exact below 2^24,
            // within the screen's margin above
            const int d = lut_screen(scr, cur, rw, __fmul_rn((float)idE, nbeta_f));
            acc = d >= 0 ? d == 1 : lut_less_exact(ln, cur, rw, __dmul_rn((double)idE, -beta));
          }
        }
        if (acc)
        {
          atomicXor(&sp[phys(v >> 5)], 1u << (v & 31));
          sacc++;
          if (cs[c].add(idE)) ppos[c] = v;
        }
        if (rl[c] >> 16)
        {
          pos[c] = v + 1;
          rl[c] = (((rl[c] >> 16) - 1u) << 16) | (unsigned)__ldg(lvl + v + 1);
        }
        else
          rl[c] = 0xFFFFu;
        }
      }
      __syncwarp();
    }
    nacc += sacc;

    // chunks in index order (c major, lane minor): running cost at each
    // chunk's start, the sweep's lowest point and its first variable
    long long carry = 0, best = LLONG_MAX;
    int bestk = INT_MAX, bestv = -1;
#pragma unroll
    for (int c = 0; c < CPL; c++)
    {
      const int csum = cs[c].sum();
      long long x = csum;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1)
      {
        const long long y = __shfl_up_sync(kFull, x, d);
        if (lane >= d) x += y;
      }
      const long long before = carry + x - csum;
      carry += __shfl_sync(kFull, x, 31);
      if (ppos[c] >= 0)
      {
        const long long cand = before + cs[c].min();
        if (cand < best)
        {
          best = cand;
          bestk = c * 32 + lane;
          bestv = ppos[c];
        }
      }
    }
#pragma unroll
    for (int d = 16; d; d >>= 1)
    {
      const long long ob = __shfl_xor_sync(kFull, best, d);
      const int ok = __shfl_xor_sync(kFull, bestk, d);
      const int ov = __shfl_xor_sync(kFull, bestv, d);
      if (ob < best || (ob == best && ok < bestk))
      {
        best = ob;
        bestk = ok;
        bestv = ov;
      }
    }
    if (bestv >= 0 && icost + best < ilow)
    {
      ilow = icost + best;
      const int ws = bestv >> 5;
      const uint32_t keep = (2u << (bestv & 31)) - 1u;  // bits 0 .. bestv % 32
      for (int w = lane; w < nwd; w += 32)
      {
        const uint32_t now = sp[phys(w)], old = st[w];
        ls[w] = w < ws ? now : (w > ws ? old : ((now & keep) | (old & ~keep)));
      }
    }
    icost += carry;
    __syncwarp();
  }

  for (int w = lane; w < nwd; w += 32) gs[w] = sp[phys(w)];
#pragma unroll
  for (int d = 16; d; d >>= 1) nacc += __shfl_xor_sync(kFull, nacc, d);
  if (lane == 0)
  {
    const unsigned long long natt = (unsigned long long)a.n_sweeps * (unsigned long long)N;
    a.p.cost[slot] = (double)icost;
    a.p.lowest[r] = (double)ilow;
    a.p.attempts[r] += natt;
    a.p.accepts[r] += nacc;
    a.p.step_att[r] += natt;
    a.p.step_acc[r] += nacc;
    if (a.p.windows) a.p.windows[r] += natt;
  }
}

// term parity bytes of the population from its spins, one thread per
// (walker, term), grid-stride
__global__ void lv_terms_kernel(DevModel m, DevPop p, int n_walkers, const int* slot_of)
{
  const long long total = (long long)n_walkers * m.n_terms;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x)
  {
    const int r = (int)(i / m.n_terms);
    const int t = (int)(i - (long long)r * m.n_terms);
    const int slot = slot_of ? slot_of[r] : r;
    const uint32_t* s = p.spins + (size_t)slot * p.nw;
    uint32_t par = 0;
    for (int k = m.trow[t]; k < m.trow[t + 1]; k++)
    {
      const uint32_t x = m.tvar[k] & ~kNegBit;
      par ^= (s[x >> 5] >> (x & 31)) & 1u;
    }
    p.tstate[(size_t)slot * p.mp + t] = (uint8_t)par;
  }
}
}  // namespace lv

void lv_upload(const double* ln, const float* scr)
{
  cudaMemcpyToSymbol(lv::g_ln, ln, 1024 * sizeof(double));
  cudaMemcpyToSymbol(lv::g_scr, scr, 3072 * sizeof(float));
}

int lv_stride_words(int n_vars)
{
  const int nwd = (n_vars + 31) / 32;
  const int words = lv::phys(nwd) + 1;
  return words * 4 <= kLvSmemBytes ? words : 0;
}

// Warps (walkers) per block: as many as the shared memory and the kernel's
// register budget allow, then evened out so that the last wave's blocks are
// as full as the others.
template <int CPL, bool PACK, bool P16>
static cudaError_t lv_go(const LvArgs& a, int stride, cudaStream_t s)
{
  auto k = lv::lv_sweep_kernel<CPL, PACK, P16>;
  const long long sms = 152;
  const int cap = std::min(lv::LvWarps<CPL>::value, kLvSmemBytes / (stride * 4));  // warps per SM
  const long long waves = ((long long)a.n_walkers + sms * cap - 1) / (sms * cap);
  const long long even = ((long long)a.n_walkers + sms * waves - 1) / (sms * waves);
  const int wpb = (int)std::max(1LL, std::min<long long>(cap, even));
  const int bytes = wpb * stride * 4;
  static int configured = 48 * 1024;
  if (bytes > configured)
  {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kLvSmemBytes);
    if (e != cudaSuccess) return e;
    configured = kLvSmemBytes;
  }
  const int blocks = (a.n_walkers + wpb - 1) / wpb;
  k<<<blocks, 32 * wpb, bytes, s>>>(a, stride);
  return cudaGetLastError();
}

template <bool PACK>
static cudaError_t lv_go_cpl(const LvArgs& a, int stride, cudaStream_t s)
{
  const int need = (a.m.n_chunks + 31) / 32;
  const bool p16 = a.m.lv_p16 != 0;
  if (need <= 1) return lv_go<1, PACK, false>(a, stride, s);
  if (need <= 2) return lv_go<2, PACK, false>(a, stride, s);
  if (need <= 4) return lv_go<4, PACK, false>(a, stride, s);
  if (need <= 8) return p16 ? lv_go<8, PACK, true>(a, stride, s) : lv_go<8, PACK, false>(a, stride, s);
  return p16 ? lv_go<16, PACK, true>(a, stride, s) : lv_go<16, PACK, false>(a, stride, s);
}

cudaError_t launch_lv_sweep(const LvArgs& a, cudaStream_t s)
{
  if (a.n_walkers <= 0 || a.n_sweeps <= 0) return cudaSuccess;
  if (!a.m.lv_ok || a.m.n_chunks > kLvMaxChunks || !a.m.rec_i || !a.start) return cudaErrorInvalidValue;
  const int stride = lv_stride_words(a.m.n_vars);
  if (stride == 0) return cudaErrorInvalidValue;
  return a.m.rec_p ? lv_go_cpl<true>(a, stride, s) : lv_go_cpl<false>(a, stride, s);
}

cudaError_t launch_lv_terms(const DevModel& m, const DevPop& p, int n_walkers, const int* slot_of,
                            cudaStream_t s)
{
  const long long total = (long long)n_walkers * m.n_terms;
  if (total <= 0) return cudaSuccess;
  const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 64);
  lv::lv_terms_kernel<<<blocks, 256, 0, s>>>(m, p, n_walkers, slot_of);
  return cudaGetLastError();
}
}  // namespace qio
