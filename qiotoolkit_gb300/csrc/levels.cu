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
// neighbours (0 without one): the variables of one level share no term, are
// spread over the warp's lanes, and the levels run in order.  An L x L
// periodic lattice has about 2L levels of up to L variables.
//
// Cost and lowest: the reference adds each accepted difference to the cost
// and keeps the first state whose cost drops below the lowest seen
// (markov/walker.h:209-229,269-280).  The sweep kernel adds up each sweep's
// accepted differences for the cost and logs, per sweep, its start spins,
// its start cost, the start cost plus its negative differences (a bound
// below its running cost) and the difference of every attempt (0 when
// rejected) at the attempt's level entry, where consecutive lanes write
// consecutive bytes.  The lowest kernel then replays the log sweep by sweep
// (skipping sweeps whose bound is not below the lowest): it puts the
// differences back in variable order (through each variable's entry),
// follows the running cost in index order -- integers, the reference's
// exact sums --, and keeps the first variable where it drops below the
// lowest.  Each variable is tried once per sweep, so the state at that point
// is the sweep's end spins up to the variable and its start spins after it.
//
// Spins live in shared memory for the whole sweep launch, bit-packed, word w
// at w + w / 32 so that the lanes' words fall in different banks.  Flips are
// shared-memory XORs: two variables of one level may share a word.
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

__host__ __device__ __forceinline__ int phys(int w) { return lv_phys(w); }

__device__ __forceinline__ int rec_other(unsigned int r) { return (int)(r >> 8); }
__device__ __forceinline__ int rec_coef(unsigned int r) { return (int)(signed char)(r & 0xFFu); }

// Metropolis::accept (markov/metropolis.h:64-104) for an uphill integer
// difference on the draws of attempt ctr: words 2 ctr and 2 ctr + 1, two
// draws each
__device__ __forceinline__ bool accept_up(uint64_t key, unsigned long long ctr, int idE, double beta,
                                          bool beta_inf, float nbeta_f)
{
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
  if ((cur & 255u) == 0u) return true;  // four zero buckets: accept
  if (beta_inf) return false;
  // the difference is an integer: its float is exact below 2^24, within the
  // screen's margin above
  const int d = lut_screen(g_scr, cur, rw, __fmul_rn((float)idE, nbeta_f));
  return d >= 0 ? d == 1 : lut_less_exact(g_ln, cur, rw, __dmul_rn((double)idE, -beta));
}

// RECS: record slots of a level entry (0: the entry is the variable alone,
// its terms come from row / rec).  PACK: 32-bit records in rec_p.
// D8: every cost difference fits in 8 bits (logged as bytes, else as 32-bit
// integers).
template <int RECS, bool PACK, bool D8>
__global__ void __launch_bounds__(kLvMaxWarps * 32, 1) lv_sweep_kernel(LvArgs a, int stride)
{
  extern __shared__ __align__(16) uint32_t lv_smem[];
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int r = blockIdx.x * (blockDim.x >> 5) + wib;
  if (r >= a.n_walkers) return;  // whole warps leave together
  const int N = a.m.n_vars, nwd = (N + 31) >> 5;
  const int* __restrict__ row = a.m.row;
  const unsigned int* __restrict__ recp = a.m.rec_p;
  const int2* __restrict__ reci = a.m.rec_i;
  const int* __restrict__ loff = a.m.lv_off;
  const uint32_t* __restrict__ ent = a.m.lv_ent;
  const int nlev = a.m.n_levels;

  uint32_t* sp = lv_smem + (size_t)wib * stride;
  const int slot = a.slot_of ? a.slot_of[r] : r;
  uint32_t* gs = a.p.spins + (size_t)slot * a.p.nw;
  for (int w = lane; w < nwd; w += 32) sp[phys(w)] = gs[w];
  if (lane == 0) sp[phys(nwd)] = 0u;  // the padding spin of one-member terms
  __syncwarp();

  long long icost = (long long)a.p.cost[slot];
  const uint64_t key = counter_key(a.seed + (uint32_t)((long long)r / a.key_div),
                                   a.key_base + (unsigned long long)((long long)r % a.key_div));
  unsigned long long nacc = 0;
  auto spin = [&](int u) -> uint32_t { return (sp[phys(u >> 5)] >> (u & 31)) & 1u; };
  // a variable's terms from the row arrays
  auto row_sum = [&](int v, uint32_t sv) -> int {
    int iacc = 0;
    for (int q = __ldg(row + v), qe = __ldg(row + v + 1); q < qe; q++)
    {
      int u, cf;
      if (PACK)
      {
        const unsigned int rq = __ldg(recp + q);
        u = rec_other(rq);
        cf = rec_coef(rq);
      }
      else
      {
        const int2 rq = __ldg(reci + q);
        u = rq.x;
        cf = rq.y;
      }
      iacc += (sv ^ spin(u)) ? -cf : cf;
    }
    return iacc;
  };

  for (int k = 0; k < a.n_sweeps; k++)
  {
    const long long swp = a.sweep_base + k;
    const double beta = a.beta[(long long)r * a.bs_w + swp * a.bs_s];
    const bool beta_inf =
        ((unsigned long long)__double_as_longlong(beta) & 0x7FFFFFFFFFFFFFFFULL) == 0x7FF0000000000000ULL;
    const float nbeta_f = -approx_float(beta);
    const unsigned long long ctr0 = (unsigned long long)swp * (unsigned long long)N;
    // the log of this sweep: start spins, start cost, differences by entry
    const size_t lk = (size_t)r * a.log_sweeps + k;
    uint32_t* st = a.start + lk * a.p.nw;
    for (int w = lane; w < nwd; w += 32) st[w] = sp[phys(w)];
    const long long c_start = icost;
    signed char* de8 = (signed char*)a.diffs + lk * a.diff_stride;
    int* de32 = (int*)a.diffs + lk * a.diff_stride;

    int tot = 0, neg = 0;  // this lane's accepted differences, their negative part
    unsigned int sacc = 0;
    auto attempt = [&](int e, int v, int iacc) {
      const int idE = -2 * iacc;
      const bool acc = idE <= 0 || accept_up(key, ctr0 + (unsigned long long)v, idE, beta, beta_inf, nbeta_f);
      if (D8) de8[e] = (signed char)(acc ? idE : 0);
      else de32[e] = acc ? idE : 0;
      if (acc)
      {
        atomicXor(&sp[phys(v >> 5)], 1u << (v & 31));
        sacc++;
        tot += idE;
        neg += min(idE, 0);
      }
    };
    int e1 = __ldg(loff);
    for (int t = 0; t < nlev; t++)
    {
      const int e0 = e1;
      e1 = __ldg(loff + t + 1);
      if constexpr (RECS == 0)
      {
        for (int e = e0 + lane; e < e1; e += 32)
        {
          const int v = (int)__ldg(ent + e);
          attempt(e, v, row_sum(v, spin(v)));
        }
      }
      else
      {
        // entries of this level, one per lane at a time; the next entry's
        // words are loaded while this one is tried
        constexpr int EW = RECS ? lv_entry_words(RECS) : 4;
        constexpr int NQ = EW / 4;
        int e = e0 + lane;
        uint4 nx[NQ];
        if (e < e1)
        {
#pragma unroll
          for (int j = 0; j < NQ; j++) nx[j] = __ldg((const uint4*)(ent + (size_t)e * EW) + j);
        }
        while (e < e1)
        {
          uint32_t w[4 * NQ];
#pragma unroll
          for (int j = 0; j < NQ; j++)
          {
            w[4 * j] = nx[j].x;
            w[4 * j + 1] = nx[j].y;
            w[4 * j + 2] = nx[j].z;
            w[4 * j + 3] = nx[j].w;
          }
          const int en = e + 32;
          if (en < e1)
          {
#pragma unroll
            for (int j = 0; j < NQ; j++) nx[j] = __ldg((const uint4*)(ent + (size_t)en * EW) + j);
          }
          const int v = (int)w[0];
          const uint32_t sv = spin(v);
          int iacc = 0;
#pragma unroll
          for (int j = 1; j <= RECS; j++)
          {
            // record: shared-memory word << 13 | bit << 8 | 8-bit coefficient
            const uint32_t rq = w[j];
            const int cf = (int)(signed char)(rq & 0xFFu);
            const uint32_t z = (sv ^ (sp[rq >> 13] >> ((rq >> 8) & 31u))) & 1u;
            iacc += z ? -cf : cf;
          }
          attempt(e, v, iacc);
          e = en;
        }
      }
      __syncwarp();
    }
    nacc += sacc;
    long long total = tot, dip = neg;
#pragma unroll
    for (int d = 16; d; d >>= 1)
    {
      total += __shfl_xor_sync(kFull, total, d);
      dip += __shfl_xor_sync(kFull, dip, d);
    }
    // the start cost, and a bound below every running cost of the sweep
    if (lane == 0)
    {
      a.cost0[2 * lk] = c_start;
      a.cost0[2 * lk + 1] = c_start + dip;
    }
    icost += total;
  }

  for (int w = lane; w < nwd; w += 32) gs[w] = sp[phys(w)];
#pragma unroll
  for (int d = 16; d; d >>= 1) nacc += __shfl_xor_sync(kFull, nacc, d);
  if (lane == 0)
  {
    const unsigned long long natt = (unsigned long long)a.n_sweeps * (unsigned long long)N;
    a.p.cost[slot] = (double)icost;
    a.p.attempts[r] += natt;
    a.p.accepts[r] += nacc;
    a.p.step_att[r] += natt;
    a.p.step_acc[r] += nacc;
    if (a.p.windows) a.p.windows[r] += natt;
  }
}

// The lowest of the logged sweeps, one block per walker (a persistent grid
// over the walkers).  STAGE: each logged sweep's differences are copied into
// shared memory and read there in variable order; otherwise they are read
// through L1.  Thread i follows a contiguous run of variables; a block scan
// places its running sum in the sweep's running cost, and the smallest
// (value, thread) pair gives the first variable where the cost is lowest.
template <bool D8, bool STAGE>
__global__ void __launch_bounds__(kLvLowThreads, 2) lv_lowest_kernel(LvArgs a)
{
  extern __shared__ __align__(16) unsigned char lv_row[];
  __shared__ long long s_tot[kLvLowThreads / 32], s_val[kLvLowThreads / 32];
  __shared__ int s_thr[kLvLowThreads / 32], s_var[kLvLowThreads / 32];
  __shared__ long long s_low;
  __shared__ int s_k, s_v;
  const unsigned kFull = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  constexpr int kW = kLvLowThreads / 32;
  const int N = a.m.n_vars, nwd = (N + 31) >> 5;
  const int* __restrict__ epos = a.m.lv_pos;
  const int vpt = ((N + kLvLowThreads - 1) / kLvLowThreads + 3) & ~3;  // a multiple of 4
  const int v0 = min(N, tid * vpt), v1 = min(N, v0 + vpt);
  for (int r = blockIdx.x; r < a.n_walkers; r += gridDim.x)
  {
    const int slot = a.slot_of ? a.slot_of[r] : r;
    if (tid == 0)
    {
      s_low = (long long)a.p.lowest[r];
      s_k = -1;
      s_v = -1;
    }
    for (int k = 0; k < a.n_sweeps; k++)
    {
      const size_t lk = (size_t)r * a.log_sweeps + k;
      const long long c0 = a.cost0[2 * lk];
      const signed char* de8 = (const signed char*)a.diffs + lk * a.diff_stride;
      const int* de32 = (const int*)a.diffs + lk * a.diff_stride;
      // the previous sweep's readers are done with the row and s_low holds
      // the lowest so far; a sweep whose running cost cannot get below it is
      // skipped
      __syncthreads();
      if (a.cost0[2 * lk + 1] >= s_low) continue;
      if (STAGE)
      {
        const int n16 = (int)((a.diff_stride * (D8 ? 1 : 4)) >> 4);
        const uint4* src = D8 ? (const uint4*)de8 : (const uint4*)de32;
#pragma unroll 4
        for (int i = tid; i < n16; i += kLvLowThreads) ((uint4*)lv_row)[i] = src[i];
        __syncthreads();
      }
      const signed char* r8 = STAGE ? (const signed char*)lv_row : de8;
      const int* r32 = STAGE ? (const int*)lv_row : de32;
      long long run = 0, mn = LLONG_MAX;
      int pos = -1;
      for (int v = v0; v < v1; v += 4)
      {
        const int4 p4 = __ldg((const int4*)(epos + v));
        const int pp[4] = {p4.x, p4.y, p4.z, p4.w};
        int dv[4];
#pragma unroll
        for (int j = 0; j < 4; j++) dv[j] = v + j < v1 ? (D8 ? (int)r8[pp[j]] : r32[pp[j]]) : 0;
#pragma unroll
        for (int j = 0; j < 4; j++)
          if (dv[j] != 0)
          {
            run += dv[j];
            if (run < mn)
            {
              mn = run;
              pos = v + j;
            }
          }
      }
      // exclusive scan of the threads' sums, in thread (= variable) order
      long long x = run;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1)
      {
        const long long y = __shfl_up_sync(kFull, x, d);
        if (lane >= d) x += y;
      }
      if (lane == 31) s_tot[wid] = x;
      __syncthreads();
      long long before = x - run;
      for (int w = 0; w < wid; w++) before += s_tot[w];
      long long best = pos >= 0 ? before + mn : LLONG_MAX;
      int bt = pos >= 0 ? tid : INT_MAX, bv = pos;
#pragma unroll
      for (int d = 16; d; d >>= 1)
      {
        const long long ob = __shfl_xor_sync(kFull, best, d);
        const int ot = __shfl_xor_sync(kFull, bt, d);
        const int ov = __shfl_xor_sync(kFull, bv, d);
        if (ob < best || (ob == best && ot < bt))
        {
          best = ob;
          bt = ot;
          bv = ov;
        }
      }
      if (lane == 0)
      {
        s_val[wid] = best;
        s_thr[wid] = bt;
        s_var[wid] = bv;
      }
      __syncthreads();
      if (tid == 0)
      {
        for (int w = 1; w < kW; w++)
          if (s_val[w] < best || (s_val[w] == best && s_thr[w] < bt))
          {
            best = s_val[w];
            bt = s_thr[w];
            bv = s_var[w];
          }
        if (bv >= 0 && c0 + best < s_low)
        {
          s_low = c0 + best;
          s_k = k;
          s_v = bv;
        }
      }
      // s_tot is rewritten by the next sweep only after the barrier above it
    }
    __syncthreads();
    const int best_k = s_k, best_v = s_v;
    if (best_k >= 0)
    {
      // the end spins of that sweep up to best_v, its start spins after
      const size_t lk = (size_t)r * a.log_sweeps + best_k;
      const uint32_t* s0 = a.start + lk * a.p.nw;
      const uint32_t* s1 = best_k + 1 < a.n_sweeps ? a.start + (lk + 1) * a.p.nw
                                                    : a.p.spins + (size_t)slot * a.p.nw;
      uint32_t* ls = a.p.lspins + (size_t)r * a.p.nw;
      const int ws = best_v >> 5;
      const uint32_t keep = (2u << (best_v & 31)) - 1u;  // bits 0 .. best_v % 32
      for (int w = tid; w < nwd; w += kLvLowThreads)
      {
        const uint32_t now = s1[w], old = s0[w];
        ls[w] = w < ws ? now : (w > ws ? old : ((now & keep) | (old & ~keep)));
      }
      if (tid == 0) a.p.lowest[r] = (double)s_low;
    }
    __syncthreads();  // s_low / s_k / s_v are reset for the next walker
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

// Warps (walkers) per block: as many as the shared memory and the register
// budget allow, then evened out so that the last wave's blocks are as full
// as the others.
template <int RECS, bool PACK, bool D8>
static cudaError_t lv_go(const LvArgs& a, int stride, cudaStream_t s)
{
  auto k = lv::lv_sweep_kernel<RECS, PACK, D8>;
  const long long sms = 152;
  const int cap = std::min(kLvMaxWarps, kLvSmemBytes / (stride * 4));  // warps per SM
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

template <bool D8, bool STAGE>
static cudaError_t lv_low(const LvArgs& a, cudaStream_t s)
{
  auto k = lv::lv_lowest_kernel<D8, STAGE>;
  const int bytes = STAGE ? (int)(a.diff_stride * (D8 ? 1 : 4)) : 0;
  static int configured = 48 * 1024;
  if (bytes > configured)
  {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kLvRowBytes);
    if (e != cudaSuccess) return e;
    configured = kLvRowBytes;
  }
  const int blocks = (int)std::min<long long>(152LL * 4, a.n_walkers);  // persistent over the walkers
  k<<<blocks, kLvLowThreads, bytes, s>>>(a);
  return cudaGetLastError();
}

static cudaError_t lv_sweep_only(const LvArgs& a, int stride, bool d8, cudaStream_t s)
{
  if (a.m.lv_recs > 0 && !a.m.rec_p) return cudaErrorInvalidValue;
  switch (a.m.lv_recs)
  {
    case 3: return d8 ? lv_go<3, true, true>(a, stride, s) : lv_go<3, true, false>(a, stride, s);
    case 4: return d8 ? lv_go<4, true, true>(a, stride, s) : lv_go<4, true, false>(a, stride, s);
    case 6: return d8 ? lv_go<6, true, true>(a, stride, s) : lv_go<6, true, false>(a, stride, s);
    case 7: return d8 ? lv_go<7, true, true>(a, stride, s) : lv_go<7, true, false>(a, stride, s);
    case 15: return d8 ? lv_go<15, true, true>(a, stride, s) : lv_go<15, true, false>(a, stride, s);
    case 0:
      if (a.m.rec_p) return d8 ? lv_go<0, true, true>(a, stride, s) : lv_go<0, true, false>(a, stride, s);
      return d8 ? lv_go<0, false, true>(a, stride, s) : lv_go<0, false, false>(a, stride, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_lv_sweep(const LvArgs& a0, cudaStream_t s)
{
  if (a0.n_walkers <= 0 || a0.n_sweeps <= 0) return cudaSuccess;
  if (!a0.m.lv_ok || !a0.m.lv_ent || !a0.m.lv_pos || !a0.m.rec_i || !a0.start || !a0.cost0 || !a0.diffs ||
      a0.log_sweeps < 1)
    return cudaErrorInvalidValue;
  const int stride = lv_stride_words(a0.m.n_vars);
  if (stride == 0) return cudaErrorInvalidValue;
  const bool d8 = a0.m.lv_d8 != 0;
  if (a0.diff_bytes != (d8 ? 1 : 4) || a0.diff_stride < a0.m.n_vars || (a0.diff_stride & 31) ||
      ((uintptr_t)a0.diffs & 255))
    return cudaErrorInvalidValue;
  const bool stage = a0.diff_stride * a0.diff_bytes <= kLvRowBytes;
  // the log holds log_sweeps sweeps: sweep launches of at most that many,
  // each followed by its lowest pass
  for (int done = 0; done < a0.n_sweeps; done += a0.log_sweeps)
  {
    LvArgs a = a0;
    a.sweep_base = a0.sweep_base + done;
    a.n_sweeps = std::min(a0.log_sweeps, a0.n_sweeps - done);
    cudaError_t e = lv_sweep_only(a, stride, d8, s);
    if (e != cudaSuccess) return e;
    if (d8) e = stage ? lv_low<true, true>(a, s) : lv_low<true, false>(a, s);
    else e = stage ? lv_low<false, true>(a, s) : lv_low<false, false>(a, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
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
