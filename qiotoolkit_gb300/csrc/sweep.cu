// sweep.cu -- the windowed Metropolis sweep (sm_103a).
//
// One warp owns one walker.  A window of 32 consecutive variables is
// evaluated at once (lane l takes variable i + l), each lane summing its own
// cost difference in the reference's term order; decisions are committed in
// lane order up to the first lane whose terms intersect an earlier accepted
// flip in the window, or whose draw needs the redraw path (markov/
// metropolis.h:93-103); the next window starts there.  Replay streams are
// PCG32 positions: lane l's draw is the stream advanced by the number of
// uphill lanes before it, so the committed prefix consumes exactly the
// draws of the sequential chain (markov/walker.h:143-153,209-229).
//
// GB300 specifics.  A warp-wide FP64 instruction costs one sub-partition
// ~64 cycles whatever its active mask, so FP64 is spent only where the
// reference's rounding must be reproduced: the ordered cost-difference sums
// (compacted to the terms that contribute, for PUBO/MaxSAT) and the running
// cost.  Sign tests and cost comparisons use integer keys of the IEEE bit
// patterns, the x(-2) of the Ising difference is an exponent increment, and
// the ln-table comparison runs in FP32 with a rigorous error margin, falling
// back to the exact FP64 expression only inside the margin.  Walker state
// (term bytes, spins, lowest spins) lives in shared memory when it fits.
#include <algorithm>
#include <climits>
#include <type_traits>

#include "metropolis.cuh"
#include "qio_internal.h"

namespace qio
{
namespace sw
{
using namespace qio::mc;
static const unsigned kFull = 0xffffffffu;
static const int kHdr = 160;  // per-warp header: 2 mbarriers, 33 dirty words

__constant__ double c_ln[1024];
__constant__ float c_scr[1024 * 3];  // y0, dy, err per (row, bucket)
__constant__ unsigned long long c_jA[65], c_jC[65];
static const int kTableBytes = 6208;  // per block: ln and screen row 0, jump tables

// Per-block tables: row 0 of the ln table and of its FP32 screen (every
// uphill attempt reads them) in shared memory; rows 1-3 (redraws after a
// zero bucket, 1 in 256 uphill attempts) stay in constant memory.
struct Smem
{
  double* ln;
  const float* scr;
  unsigned long long* jA;
  unsigned long long* jC;
};
__device__ __forceinline__ const double* ln_rows(const Smem& S, int row) { return row ? c_ln : S.ln; }
__device__ __forceinline__ const float* scr_rows(const Smem& S, int row) { return row ? c_scr : S.scr; }

template <bool INT>
__device__ __forceinline__ bool uphill_accept(const Smem& S, uint32_t r0, int row, double dE,
                                              long long idE, double beta, float nbeta_f)
{
  float thr_f = INT ? __fmul_rn((float)idE, nbeta_f) : __fmul_rn(approx_float(dE), nbeta_f);
  int d = lut_screen(scr_rows(S, row), r0, row, thr_f);
  if (d >= 0) return d == 1;
  return lut_less_exact(ln_rows(S, row), r0, row, __dmul_rn(INT ? (double)idE : dE, -beta));
}

__device__ __forceinline__ uint32_t spin_of(const uint32_t* spins, int v)
{
  return (spins[v >> 5] >> (v & 31)) & 1u;
}

// any contributing incidence (rows of more than 32 incidences are "wide")
__device__ __forceinline__ bool nq_nonzero(uint32_t qm, bool wide) { return wide || qm != 0u; }

// Exact reference-order FP64 difference for a row of more than 32
// incidences, recomputed from the term states (rare: high-degree variables).
template <int FL, class C>
__device__ __forceinline__ double exact_dE_wide(bool part, uint32_t sv, const uint8_t* ts,
                                                const uint32_t* pinc, const C* pcoef, int deg)
{
  double diff = 0.0;
  const int n = part ? deg : 0;
  for (int k = 0; k < n; k++)
  {
    uint32_t e = pinc[k];
    uint8_t z = ts[e & ~kNegBit];
    double c = (double)pcoef[k];
    if (FL == F_PARITY) diff = __dadd_rn(diff, z ? -c : c);
    else
    {
      const bool lit = (sv ^ (e >> 31)) != 0;
      if (lit ? (z == 1) : (z == 0)) diff = lit ? __dadd_rn(diff, c) : __dsub_rn(diff, c);
    }
  }
  return (FL == F_PARITY) ? neg2x(diff) : diff;
}

// warp-cooperative copy of `words` 32-bit words (16-byte aligned, multiple of 4)
__device__ __forceinline__ void copy_words(uint32_t* dst, const uint32_t* src, int words, int lane)
{
  const uint4* s = (const uint4*)src;
  uint4* d = (uint4*)dst;
  for (int q = lane; q < words / 4; q += 32) d[q] = s[q];
}

// ---- TMA bulk copies into shared memory, completion on an mbarrier -------
__device__ __forceinline__ unsigned smem_u32(const void* p)
{
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned long long* bar, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_1d(void* dst, const void* src, unsigned bytes,
                                       unsigned long long* bar)
{
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned long long* bar, unsigned parity)
{
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; false when the copy never completed (error reported)
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int* err)
{
  for (int it = 0; it < (1 << 22); it++)
    if (mbar_try(bar, parity)) return true;
  if (err) atomicExch(err, 1);
  return false;
}

// Per-warp tile of the CSR incidences of one 32-variable block: term ids,
// coefficients and later-co-member words of [q0, q0 + n) brought in by bulk
// copies.  Bulk copies move 16-byte aligned, 16-byte multiple ranges, so each
// starts at the aligned address below its first element and records the
// element offset.  FP64 models carry the coefficients twice: rounded to float
// for the screen and exact for the reference-order sums.
// The capacity is set per launch (a multiple of 8, the model's largest block
// or less); each array starts on a 16-byte boundary and holds cap + 8
// entries, the slack that the rounding of the copies' ends needs.
template <bool INT>
struct Tile
{
  static const int kMaxCap = INT ? 768 : 640;  // incidences held in shared memory, at most
  uint32_t* inc;
  float* coef_f;
  typename std::conditional<INT, int, double>::type* coef;
  unsigned long long* near;
};
template <bool INT>
__host__ __device__ inline int tile_bytes(int cap)
{
  const int e = cap + 8;
  return e * 4 + (INT ? 16 : e * 4) + e * (INT ? 4 : 8) + e * 8;
}
template <bool INT>
__device__ __forceinline__ Tile<INT> tile_at(unsigned char* base, int cap)
{
  using C = typename std::conditional<INT, int, double>::type;
  const int e = cap + 8;
  Tile<INT> t;
  t.inc = (uint32_t*)base;
  t.coef_f = (float*)(base + e * 4);
  t.coef = (C*)(base + e * 4 + (INT ? 16 : e * 4));
  t.near = (unsigned long long*)(base + e * 4 + (INT ? 16 : e * 4) + e * (INT ? 4 : 8));
  return t;
}

template <bool INT>
__device__ __forceinline__ void tile_issue(const Tile<INT>& t, int cap, unsigned long long* bar,
                                           const DevModel& m, int q0, int q1, int* off)
{
  using C = typename std::conditional<INT, int, double>::type;
  const int n = min(q1 - q0, cap);
  const C* cbase = INT ? (const C*)m.coef_i : (const C*)m.coef;
  const void* src[4] = {m.inc + q0, cbase + q0, m.near + q0,
                        INT ? (const void*)m.inc : (const void*)(m.coef_f + q0)};
  const int esz[4] = {4, (int)sizeof(C), 8, 4};
  void* dst[4] = {t.inc, t.coef, t.near, t.coef_f};
  const int ncopy = INT ? 3 : 4;
  unsigned bytes[4];
  const char* start[4];
  unsigned total = 0;
#pragma unroll
  for (int c = 0; c < ncopy; c++)
  {
    const char* a = (const char*)src[c];
    start[c] = (const char*)((size_t)a & ~(size_t)15);
    off[c] = (int)((a - start[c]) / esz[c]);
    bytes[c] = (unsigned)(((a + (size_t)esz[c] * (size_t)(n > 0 ? n : 1)) - start[c] + 15) & ~(size_t)15);
    total += bytes[c];
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_expect(bar, total);
#pragma unroll
  for (int c = 0; c < ncopy; c++) tma_1d(dst[c], start[c], bytes[c], bar);
}

// Mutable per-walker state of the sweep.
struct Walk
{
  double cost, low;
  long long icost, ilow, klow;
  unsigned long long natt, nacc, nwin;
  uint64_t rs, key;
};

// warp-inclusive prefix sums
__device__ __forceinline__ long long warp_scan64(long long x, int lane)
{
#pragma unroll
  for (int d = 1; d < 32; d <<= 1)
  {
    long long y = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x += y;
  }
  return x;
}
__device__ __forceinline__ int warp_scan32(int x, int lane)
{
#pragma unroll
  for (int d = 1; d < 32; d <<= 1)
  {
    int y = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x += y;
  }
  return x;
}

// Exact reference-order FP64 cost difference from the masks: bit k of qm =
// incidence k contributes, bit k of sm = its sign (counter: literal true ->
// +c; parity: term bit set -> -c).  The warp issues one FP64 add per set bit
// of the longest mask among participating lanes.
template <int FL>
__device__ __forceinline__ double exact_dE(bool part, uint32_t qm, uint32_t sm, const double* pc)
{
  double diff = 0.0;
  uint32_t q = part ? qm : 0u;
  const int n = (int)__reduce_max_sync(kFull, (unsigned)__popc(q));
#pragma unroll 2
  for (int i = 0; i < n; i++)
  {
    if (q)
    {
      const int k = __ffs(q) - 1;
      q &= q - 1;
      long long cb = __double_as_longlong(pc[k]);
      const bool neg = (FL == F_PARITY) ? ((sm >> k) & 1u) != 0u : ((sm >> k) & 1u) == 0u;
      cb ^= (long long)neg << 63;
      diff = __dadd_rn(diff, __longlong_as_double(cb));
    }
  }
  return (FL == F_PARITY) ? neg2x(diff) : diff;
}

// All rounds of one 32-variable block.  Lane l holds variable i0 + l.  On
// entry every lane reads its row once into per-incidence masks (qm: the
// incidence contributes to the cost difference, sm: its sign) and a field
// (the integer difference, or an FP32 estimate with a rigorous error bound).
// A round decides the undecided lanes from their fields, commits the prefix
// up to the first lane that shares a term with an earlier accepted lane of
// the round (or that needs the redraw path), and applies the committed
// flips: term bytes change by shared-memory atomics and each flip marks the
// incidences of later undecided lanes that share its terms (the per-lane
// dirty words, dirty[32] = "recompute all"), which those lanes re-read at
// the start of the next round.  Rows of more than 32 incidences ("wide")
// are recomputed every round.  FP64 cost differences are summed exactly, in
// the reference's term order, only for lanes whose sign or comparison the
// screen leaves open and for the flips that may be committed.
// TILE: the block's incidences are in the shared tile; otherwise they are
// read from global memory.
template <int FL, bool REPLAY, bool INT, bool TILE>
__device__ __forceinline__ void block_rounds(const Smem& S, const DevModel& m, Walk& W,
                                             uint8_t* ts, uint32_t* spins, uint32_t* lsp,
                                             uint32_t* dirty, const uint32_t* tinc,
                                             const typename std::conditional<INT, int, double>::type* tcoef,
                                             const float* tcf, const unsigned long long* tnear,
                                             int i0, int Sz, int nwd, double beta, float nbeta_f,
                                             bool beta_inf, unsigned long long ctr0)
{
  using C = typename std::conditional<INT, int, double>::type;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int v = i0 + lane;
  const bool valid = v < Sz;
  const int nvalid = min(32, Sz - i0);
  // rows of lanes past the end start at the block's first row (the row
  // pointers below and the owner offsets of the apply step rely on it)
  int rb = __ldg(m.row + (valid ? v : i0)), deg = 0;
  uint32_t sv = 0, nb = 0;
  if (valid)
  {
    deg = __ldg(m.row + v + 1) - rb;
    sv = spin_of(spins, v);
    nb = __ldg(m.nbr + v);
  }
  const uint32_t* pinc = TILE ? tinc : (const uint32_t*)(m.inc + rb);
  const C* pcoef = TILE ? tcoef : (INT ? (const C*)(m.coef_i + rb) : (const C*)(m.coef + rb));
  const float* pcf = TILE ? tcf : (INT ? nullptr : m.coef_f + rb);
  const unsigned long long* pnear = TILE ? tnear : m.near + rb;
  auto INC = [&](int k) -> uint32_t { return TILE ? pinc[k] : __ldg(pinc + k); };
  auto COEF = [&](int k) -> C { return TILE ? pcoef[k] : __ldg(pcoef + k); };
  auto CF = [&](int k) -> float { return TILE ? pcf[k] : __ldg(pcf + k); };
  auto NEAR = [&](int k) -> unsigned long long { return TILE ? pnear[k] : __ldg(pnear + k); };
  const bool wide = deg > 32;
  const bool narrow = valid && !wide;
  uint32_t* ts32 = (uint32_t*)ts;

  uint32_t qm = 0, sm = 0;
  int ifield = 0;
  float ffield = 0.f, fsabs = 0.f;
  int nops = 0;
  // the whole row: masks (first 32 incidences) and field
  auto gather = [&]() {
    uint32_t q = 0, sg = 0;
    int ia = 0;
    float fa = 0.f, fs = 0.f;
    for (int k = 0; k < deg; k++)
    {
      const uint32_t e = INC(k);
      const uint32_t z = ts[e & ~kNegBit];
      if (FL == F_PARITY)
      {
        if (INT)
        {
          const int c = (int)COEF(k);
          ia += z ? -c : c;
        }
        else
        {
          const float c = CF(k);
          fa = __fadd_rn(fa, z ? -c : c);
          fs = __fadd_rn(fs, fabsf(c));
        }
        if (k < 32) sg |= z << k;
      }
      else
      {
        const uint32_t lit = (sv ^ (e >> 31)) & 1u;
        const uint32_t qual = lit ? (z == 1u) : (z == 0u);
        if (INT)
        {
          const int c = (int)COEF(k);
          ia += qual ? (lit ? c : -c) : 0;
        }
        else
        {
          const float c = CF(k);
          fa = __fadd_rn(fa, qual ? (lit ? c : -c) : 0.f);
          fs = __fadd_rn(fs, fabsf(c));
        }
        if (k < 32)
        {
          q |= qual << k;
          sg |= lit << k;
        }
      }
    }
    qm = (FL == F_PARITY) ? ((deg >= 32) ? kFull : ((1u << deg) - 1u)) : q;
    sm = sg;
    ifield = ia;
    ffield = fa;
    fsabs = fs;
    nops = deg;
  };
  // re-read the marked incidences and correct the field
  auto fix = [&](int k, uint32_t e, uint32_t z) {
    if (FL == F_PARITY)
    {
      if (z != ((sm >> k) & 1u))
      {
        sm ^= 1u << k;
        if (INT)
        {
          const int c = (int)COEF(k);
          ifield += z ? -2 * c : 2 * c;
        }
        else
        {
          const float c = CF(k);
          ffield = __fadd_rn(ffield, z ? -2.f * c : 2.f * c);
          nops += 2;
        }
      }
    }
    else
    {
      const uint32_t lit = (sm >> k) & 1u;
      const uint32_t qual = lit ? (z == 1u) : (z == 0u);
      if (qual != ((qm >> k) & 1u))
      {
        qm ^= 1u << k;
        if (INT)
        {
          const int c = (int)COEF(k);
          const int d = lit ? c : -c;
          ifield += qual ? d : -d;
        }
        else
        {
          const float c = CF(k);
          const float d = lit ? c : -c;
          ffield = __fadd_rn(ffield, qual ? d : -d);
          nops += 2;
        }
      }
    }
  };
  auto refresh = [&](uint32_t dm) {
    while (dm)
    {
      // two marked incidences at a time: their loads overlap
      const int k1 = __ffs(dm) - 1;
      dm &= dm - 1;
      const int k2 = dm ? __ffs(dm) - 1 : k1;
      dm &= dm - 1;
      const uint32_t e1 = INC(k1), e2 = INC(k2);
      const uint32_t z1 = ts[e1 & ~kNegBit], z2 = ts[e2 & ~kNegBit];
      fix(k1, e1, z1);
      if (k2 != k1) fix(k2, e2, z2);
    }
  };

  if (narrow) gather();
  dirty[lane] = 0u;
  if (lane == 0) dirty[32] = 0u;
  __syncwarp();

  int cursor = 0;
  bool pending = false;  // the last round flipped something: marks may be set
  unsigned blk_flips = 0;  // committed flips of the block
  long long fidE = 0;      // a flipped lane's difference (integer mode)
  double fdE = 0.0;        // ... FP64, exact when fexact
  bool fexact = false;
  while (cursor < nvalid)
  {
    const bool active = valid && lane >= cursor;
    if (pending)
    {
      const uint32_t all = dirty[32];
      const uint32_t dm = dirty[lane];
      __syncwarp();
      if (active && narrow)
      {
        if (all) gather();
        else refresh(dm);
      }
      if (dm) dirty[lane] = 0u;
      if (lane == 0 && all) dirty[32] = 0u;
      __syncwarp();
    }

    // ---- cost difference: exact where known, screened otherwise --------
    long long idE = 0;
    double dE = 0.0;
    bool have_exact = false;
    float dEf = 0.f, bound = 0.f;
    if constexpr (INT)
    {
      if (active && wide) gather();
      idE = (FL == F_PARITY) ? -2LL * (long long)ifield : (long long)ifield;
    }
    else
    {
      if (__any_sync(kFull, active && wide))
      {
        const double ex = exact_dE_wide<FL>(active && wide, sv, ts, pinc, pcoef, deg);
        if (active && wide)
        {
          dE = ex;
          have_exact = true;
        }
      }
      if (active && narrow)
      {
        dEf = (FL == F_PARITY) ? -2.f * ffield : ffield;
        bound = m.fscreen ? __fmaf_rn((FL == F_PARITY ? 2.f : 1.f) * fsabs,
                                      (float)(nops + 2) * 9.5367431640625e-07f, 1e-35f)  // 2^-20
                          : INFINITY;
        // no contributing term: the reference's sum is exactly +0.0
        if (FL != F_PARITY && qm == 0u) have_exact = true;
      }
      const bool undecided = active && narrow && !have_exact && !(fabsf(dEf) > bound);
      if (__any_sync(kFull, undecided))
      {
        const double ex = exact_dE<FL>(undecided, qm, sm, pcoef);
        if (undecided)
        {
          dE = ex;
          have_exact = true;
        }
      }
    }

    // ---- acceptance (markov/metropolis.h:64-104) ----------------------
    const unsigned before = lt & ~((1u << cursor) - 1u);  // lanes in [cursor, lane)
    bool uphill;
    if (INT) uphill = active && idE > 0;
    else uphill = active && (have_exact ? !le_zero(dE) : (dEf > 0.f));
    bool acc = active && !uphill;
    bool redraw = false;
    unsigned U = 0;
    int pos = 0;
    // FP32-screened comparison value < dE * (-beta); -1 inside the margin
    auto decide = [&](uint32_t r, int row) -> int {
      if (beta_inf) return 0;
      if (INT || have_exact)
      {
        const float thr_f = INT ? __fmul_rn((float)idE, nbeta_f) : __fmul_rn(approx_float(dE), nbeta_f);
        return lut_screen(scr_rows(S, row), r, row, thr_f);
      }
      const float thr_f = __fmul_rn(dEf, nbeta_f);
      // widen the margin by the screen's own error times beta
      const float et_extra = __fmul_rn(bound, -nbeta_f) * 1.0000002f;
      const int b = (int)(r & 255u);
      if (b == 1) return 0;
      const int kk = (row * 256 + b) * 3;
      const float* scr = scr_rows(S, row);
      const float y0 = scr[kk], dy = scr[kk + 1], ev = scr[kk + 2];
      const float dist = __fmul_rn((float)(r >> 8), 5.96046483e-08f);
      const float value = __fmaf_rn(dist, dy, y0);
      const float et = __fmaf_rn(fabsf(thr_f), 1.9073486328125e-06f, 1e-30f) + et_extra;
      if (__fadd_rn(value, ev) < __fsub_rn(thr_f, et)) return 1;
      if (__fsub_rn(value, ev) > __fadd_rn(thr_f, et)) return 0;
      return -1;
    };
    if (REPLAY)
    {
      U = __ballot_sync(kFull, uphill);
      pos = __popc(U & before);
    }
    uint32_t dr = 0;
    int drow = 0;
    int dec = 1;  // 1 accept, 0 reject, -1 needs the exact expression
    if (uphill)
    {
      if (REPLAY)
      {
        dr = pcg_out(S.jA[pos] * W.rs + S.jC[pos]);
        redraw = (dr & 255u) == 0;
        if (!redraw) dec = decide(dr, 0);
      }
      else
      {
        const unsigned long long ctr = ctr0 + (unsigned long long)v;
        const uint64_t w0 = counter_draw(W.key, 2ULL * ctr);
        int row = -1, b = 0, used = 0;
        uint32_t cur = 0;
        bool all_zero = false;
        while (b == 0)
        {
          if (row < 3)
          {
            if (used == 0) cur = (uint32_t)w0;
            else if (used == 1) cur = (uint32_t)(w0 >> 32);
            else
            {
              uint64_t w1 = counter_draw(W.key, 2ULL * ctr + 1ULL);
              cur = used == 2 ? (uint32_t)w1 : (uint32_t)(w1 >> 32);
            }
            used++;
            b = (int)(cur & 255u);
            row++;
          }
          else
          {
            all_zero = true;
            break;
          }
        }
        dr = cur;
        drow = row;
        dec = all_zero ? 1 : decide(cur, row);
      }
    }
    const unsigned Rm = REPLAY ? __ballot_sync(kFull, redraw) : 0u;
    if constexpr (!INT)
    {
      if (__any_sync(kFull, uphill && !redraw && dec < 0))
      {
        // Exact differences for the lanes inside the LUT margin that may be
        // committed: up to the first stop under the surely accepted lanes
        // (more acceptances can only move the stop earlier).  Committed flips
        // get theirs at the end of the block.
        const bool sure = active && (!uphill || (!redraw && dec == 1));
        const unsigned As = __ballot_sync(kFull, sure);
        bool cs = false;
        if (active && lane > cursor)
          cs = (nb & (__brev(As) >> (32 - lane)) & ((1u << (lane - cursor)) - 1u)) != 0u;
        const unsigned stop_s = __ballot_sync(kFull, cs) | Rm;
        const int fs = stop_s ? (__ffs(stop_s) - 1) : 32;
        const bool cand = active && lane <= fs && !have_exact && uphill && !redraw && dec < 0;
        if (__any_sync(kFull, cand))
        {
          const double ex = exact_dE<FL>(cand, qm, sm, pcoef);
          if (cand)
          {
            dE = ex;
            have_exact = true;
          }
        }
        if (lane > fs && dec < 0) dec = 0;  // cannot be committed this round
      }
    }
    // lanes inside the screen's margin: exact comparison
    if (uphill && !redraw && dec < 0)
      dec = lut_less_exact(ln_rows(S, drow), dr, drow, __dmul_rn(INT ? (double)idE : dE, -beta)) ? 1 : 0;
    if (uphill && !redraw) acc = dec == 1;
    const unsigned A = __ballot_sync(kFull, acc);
    bool conf = false;
    if (active && lane > cursor)
      conf = (nb & (__brev(A) >> (32 - lane)) & ((1u << (lane - cursor)) - 1u)) != 0u;
    const unsigned Cm = __ballot_sync(kFull, conf);
    const unsigned stop = Cm | Rm;
    int f = stop ? (__ffs(stop) - 1) : 32;
    if (f > nvalid) f = nvalid;
    const bool slow = REPLAY && f < nvalid && ((Rm >> f) & 1u) && !((Cm >> f) & 1u);
    const unsigned commit = ((f >= 32) ? kFull : ((1u << f) - 1u)) & ~((1u << cursor) - 1u);
    unsigned flips = A & commit;
    int draws = REPLAY ? __popc(U & commit) : 0;
    if (REPLAY && slow)
    {
      // lane f drew a zero bucket: its redraw chain (markov/metropolis.h:93-103)
      if constexpr (!INT)
      {
        const bool nx = lane == f && !have_exact;
        if (__any_sync(kFull, nx))
        {
          const double ex = exact_dE<FL>(nx, qm, sm, pcoef);
          if (nx)
          {
            dE = ex;
            have_exact = true;
          }
        }
      }
      int sacc = 0, used = 0;
      if (lane == f)
      {
        int row = -1, b = 0;
        uint32_t cur = 0;
        bool decided = false;
        while (b == 0)
        {
          if (row < 3)
          {
            cur = pcg_out(S.jA[pos + used] * W.rs + S.jC[pos + used]);
            used++;
            b = (int)(cur & 255u);
            row++;
          }
          else
          {
            decided = true;
            break;
          }
        }
        bool ok;
        if (decided) ok = true;
        else if (beta_inf) ok = false;
        else ok = lut_less_exact(ln_rows(S, row), cur, row, __dmul_rn(INT ? (double)idE : dE, -beta));
        sacc = ok ? 1 : 0;
      }
      sacc = __shfl_sync(kFull, sacc, f);
      used = __shfl_sync(kFull, used, f);
      if (sacc) flips |= 1u << f;
      draws += used;
    }
    const int adv = f + (slow ? 1 : 0) - cursor;
    const bool mine = ((flips >> lane) & 1u) != 0u;
    if (mine)
    {
      // a committed lane keeps its masks: its exact difference can wait
      // for the end of the block
      fidE = idE;
      fdE = dE;
      fexact = INT || have_exact;
    }

    // ---- apply: the flips' incidences spread over the warp; term bytes
    // change by atomics (different terms may share a word), and each
    // incidence marks the later co-members of its term ----------------------
    pending = flips != 0u;
    // apply: term bytes change by atomics (different terms may share a
    // word) and each incidence marks the later co-members of its term
    auto apply_one = [&](int j, int kk, uint32_t svj) {
      const uint32_t e = INC(kk);
      const unsigned long long nw = NEAR(kk);
      const uint32_t t = e & ~kNegBit;
      const unsigned sh = (t & 3u) << 3;
      if (FL == F_PARITY) atomicXor(ts32 + (t >> 2), 1u << sh);
      else atomicAdd(ts32 + (t >> 2), ((svj ^ (e >> 31)) & 1u) ? (0u - (1u << sh)) : (1u << sh));
      const int cnt = (int)(nw >> 61);
      if (cnt == 7) atomicOr(dirty + 32, 1u);
      else
        for (int i = 0; i < cnt; i++)
        {
          const int u = j + (int)((nw >> (10 * i)) & 31u);
          if (u < 32) atomicOr(dirty + u, 1u << (unsigned)((nw >> (10 * i + 5)) & 31u));
        }
    };
    if (__popc(flips) <= 2)
    {
      // few flips: one flipping lane at a time, the warp over its incidences
      unsigned fl = flips;
      while (fl)
      {
        const int j = __ffs(fl) - 1;
        fl &= fl - 1;
        const int dj = __shfl_sync(kFull, deg, j);
        const int rj = __shfl_sync(kFull, rb, j);
        const uint32_t svj = __shfl_sync(kFull, sv, j);
        for (int k0 = 0; k0 < dj; k0 += 32)
          if (k0 + lane < dj) apply_one(j, k0 + lane + (rj - rb), svj);
      }
    }
    else
    {
      // many flips: their incidences laid out back to back over the warp
      const int mydeg = mine ? deg : 0;
      const int incl = warp_scan32(mydeg, lane);
      const int excl = incl - mydeg;
      const int total = __shfl_sync(kFull, incl, 31);
      const unsigned F = __ballot_sync(kFull, mine && mydeg > 0);
      for (int base = 0; base < total; base += 32)
      {
        // start positions of the flips' runs inside this chunk
        const int rel = excl - base;
        const unsigned starts = __reduce_or_sync(kFull, (mine && mydeg > 0 && rel >= 0 && rel < 32) ? (1u << rel) : 0u);
        const int nbefore = __popc(__ballot_sync(kFull, mine && mydeg > 0 && rel < 0));
        const int g = base + lane;
        const int idx = nbefore + __popc(starts & ((2u << lane) - 1u)) - 1;
        // the idx-th flipping lane with a non-empty row: smallest j with
        // popc(F & bits 0..j) > idx
        int j = 0;
#pragma unroll
        for (int step = 16; step; step >>= 1)
          if (__popc(F & ((2u << (j + step - 1)) - 1u)) <= idx) j += step;
        const int ej = __shfl_sync(kFull, excl, j & 31);
        const int rj = __shfl_sync(kFull, rb, j & 31);
        const uint32_t svj = __shfl_sync(kFull, sv, j & 31);
        if (g < total) apply_one(j, g - ej + (rj - rb), svj);
      }
    }
    const int wi = i0 >> 5;
    if (lane == 0 && flips) spins[wi] ^= flips;
    W.natt += (unsigned long long)adv;
    W.nacc += (unsigned long long)__popc(flips);
    W.nwin++;
    if (REPLAY) W.rs = S.jA[draws] * W.rs + S.jC[draws];
    cursor += adv;
    blk_flips |= flips;
  }
  __syncwarp();

  // ---- running cost and lowest state over the block's flips, in attempt
  // order (they are in lane order) -----------------------------------------
  if (blk_flips == 0u) return;
  const bool fl_mine = ((blk_flips >> lane) & 1u) != 0u;
  int lowpos = -1;
  if constexpr (INT)
  {
    if (m.scan32)
    {
      const int d = fl_mine ? (int)fidE : 0;
      const int dsum = __reduce_add_sync(kFull, d);
      const int negsum = __reduce_add_sync(kFull, d < 0 ? d : 0);
      // the lowest prefix cost is at least icost + negsum
      if ((long long)negsum < W.ilow - W.icost)
      {
        const int pre = warp_scan32(d, lane);
        const int mn = __reduce_min_sync(kFull, fl_mine ? pre : INT_MAX);
        if ((long long)mn < W.ilow - W.icost)
        {
          lowpos = __ffs(__ballot_sync(kFull, fl_mine && pre == mn)) - 1;
          W.ilow = W.icost + mn;
        }
      }
      W.icost += dsum;
    }
    else
    {
      const long long pre = warp_scan64(fl_mine ? fidE : 0LL, lane);
      const long long ci = W.icost + pre;
      long long mn = fl_mine ? ci : LLONG_MAX;
#pragma unroll
      for (int d = 16; d; d >>= 1) mn = min(mn, __shfl_xor_sync(kFull, mn, d));
      if (mn < W.ilow)
      {
        lowpos = __ffs(__ballot_sync(kFull, fl_mine && ci == mn)) - 1;
        W.ilow = mn;
      }
      W.icost += __shfl_sync(kFull, pre, 31);
    }
  }
  else
  {
    const bool nx = fl_mine && !fexact;
    if (__any_sync(kFull, nx))
    {
      const double ex = exact_dE<FL>(nx, qm, sm, pcoef);
      if (nx) fdE = ex;
    }
    unsigned fl = blk_flips;
    int j = __ffs(fl) - 1;
    fl &= fl - 1;
    double d = __shfl_sync(kFull, fdE, j);
    while (true)
    {
      const int jn = fl ? (__ffs(fl) - 1) : j;
      const double dn = __shfl_sync(kFull, fdE, jn);  // ahead of the dependent add
      W.cost = __dadd_rn(W.cost, d);
      const long long kc = order_key(W.cost);
      if (kc < W.klow)
      {
        W.klow = kc;
        W.low = W.cost;
        lowpos = j;
      }
      if (!fl) break;
      fl &= fl - 1;
      j = jn;
      d = dn;
    }
  }
  if (lowpos >= 0)
  {
    // the state at the last improvement: the block's later flips undone
    for (int q = lane; q < nwd; q += 32) lsp[q] = spins[q];
    __syncwarp();
    const unsigned undo = blk_flips & ~((2u << lowpos) - 1u);
    if (lane == 0 && undo) lsp[i0 >> 5] ^= undo;
    __syncwarp();
  }
}

// Counter-free models (model::Ising, model::Pubo): the cost difference
// gathers the member spins of each incident term; windows slide.
template <int FL, bool REPLAY, bool INT>
__device__ __forceinline__ void block_rounds_plain(const Smem& S, const DevModel& m, Walk& W,
                                                   uint32_t* spins, uint32_t* lsp, int i0, int Sz,
                                                   int nwd, double beta, float nbeta_f,
                                                   bool beta_inf, unsigned long long ctr0)
{
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int v = i0 + lane;
  const bool valid = v < Sz;
  const int nvalid = min(32, Sz - i0);
  int rb = 0, re = 0;
  uint32_t sv = 0, nb = 0;
  if (valid)
  {
    rb = __ldg(m.row + v);
    re = __ldg(m.row + v + 1);
    sv = spin_of(spins, v);
    nb = __ldg(m.nbr + v);
  }
  int cursor = 0;
  while (cursor < nvalid)
  {
    const bool active = valid && lane >= cursor;
    double dE = 0.0;
    long long idE = 0;
    if (active)
    {
      double diff = 0.0;
      long long iacc = 0;
      for (int q = rb; q < re; q++)
      {
        int t = (int)__ldg(m.inc + q);
        int tb = __ldg(m.trow + t), te = __ldg(m.trow + t + 1);
        if (FL == F_PLAIN_ISING)
        {
          uint32_t par = 0;
          for (int u = tb; u < te; u++) par ^= spin_of(spins, (int)__ldg(m.tvar + u));
          if (INT) iacc += par ? -(long long)__ldg(m.coef_i + q) : (long long)__ldg(m.coef_i + q);
          else diff = __dadd_rn(diff, par ? -__ldg(m.coef + q) : __ldg(m.coef + q));
        }
        else
        {
          bool zero = false;
          for (int u = tb; u < te; u++)
          {
            int x = (int)__ldg(m.tvar + u);
            if (x != v && spin_of(spins, x)) { zero = true; break; }
          }
          if (!zero)
          {
            if (INT) iacc += sv ? (long long)__ldg(m.coef_i + q) : -(long long)__ldg(m.coef_i + q);
            else diff = sv ? __dadd_rn(diff, __ldg(m.coef + q)) : __dsub_rn(diff, __ldg(m.coef + q));
          }
        }
      }
      if (FL == F_PLAIN_ISING)
      {
        if (INT) idE = -2 * iacc;
        else dE = neg2x(diff);
      }
      else
      {
        if (INT) idE = iacc;
        else dE = diff;
      }
    }
    const unsigned before = lt & ~((1u << cursor) - 1u);
    const bool uphill = active && (INT ? (idE > 0) : !le_zero(dE));
    bool acc = active && !uphill;
    bool redraw = false;
    unsigned U = 0;
    int pos = 0;
    if (REPLAY)
    {
      U = __ballot_sync(kFull, uphill);
      pos = __popc(U & before);
      if (uphill)
      {
        uint32_t r0 = pcg_out(S.jA[pos] * W.rs + S.jC[pos]);
        redraw = (r0 & 255u) == 0;
        if (!redraw) acc = !beta_inf && uphill_accept<INT>(S, r0, 0, dE, idE, beta, nbeta_f);
      }
    }
    else if (uphill)
    {
      const unsigned long long ctr = ctr0 + (unsigned long long)v;
      const uint64_t w0 = counter_draw(W.key, 2ULL * ctr);
      int row = -1, b = 0, used = 0;
      uint32_t cur = 0;
      bool decided = false;
      while (b == 0)
      {
        if (row < 3)
        {
          if (used == 0) cur = (uint32_t)w0;
          else if (used == 1) cur = (uint32_t)(w0 >> 32);
          else
          {
            uint64_t w1 = counter_draw(W.key, 2ULL * ctr + 1ULL);
            cur = used == 2 ? (uint32_t)w1 : (uint32_t)(w1 >> 32);
          }
          used++;
          b = (int)(cur & 255u);
          row++;
        }
        else
        {
          decided = true;
          break;
        }
      }
      acc = decided ? true : (!beta_inf && uphill_accept<INT>(S, cur, row, dE, idE, beta, nbeta_f));
    }
    const unsigned A = __ballot_sync(kFull, acc);
    bool conf = false;
    if (active && lane > cursor)
      conf = (nb & (__brev(A) >> (32 - lane)) & ((1u << (lane - cursor)) - 1u)) != 0u;
    const unsigned Cm = __ballot_sync(kFull, conf);
    const unsigned Rm = REPLAY ? __ballot_sync(kFull, redraw) : 0u;
    const unsigned stop = Cm | Rm;
    int f = stop ? (__ffs(stop) - 1) : 32;
    if (f > nvalid) f = nvalid;
    const bool slow = REPLAY && f < nvalid && ((Rm >> f) & 1u) && !((Cm >> f) & 1u);
    const unsigned commit = ((f >= 32) ? kFull : ((1u << f) - 1u)) & ~((1u << cursor) - 1u);
    unsigned flips = A & commit;
    int draws = REPLAY ? __popc(U & commit) : 0;
    if (REPLAY && slow)
    {
      int sacc = 0, used = 0;
      if (lane == f)
      {
        int row = -1, b = 0;
        uint32_t cur = 0;
        bool decided = false;
        while (b == 0)
        {
          if (row < 3)
          {
            cur = pcg_out(S.jA[pos + used] * W.rs + S.jC[pos + used]);
            used++;
            b = (int)(cur & 255u);
            row++;
          }
          else
          {
            decided = true;
            break;
          }
        }
        bool ok = decided ? true
                          : (!beta_inf && uphill_accept<INT>(S, cur, row, dE, idE, beta, nbeta_f));
        sacc = ok ? 1 : 0;
      }
      sacc = __shfl_sync(kFull, sacc, f);
      used = __shfl_sync(kFull, used, f);
      if (sacc) flips |= 1u << f;
      draws += used;
    }
    const int adv = f + (slow ? 1 : 0) - cursor;
    const int wi = i0 >> 5;
    if (lane == 0 && flips) spins[wi] ^= flips;
    int lowpos = -1;
    unsigned fl = flips;
    while (fl)
    {
      const int j = __ffs(fl) - 1;
      fl &= fl - 1;
      if (INT)
      {
        W.icost += __shfl_sync(kFull, idE, j);
        if (W.icost < W.ilow)
        {
          W.ilow = W.icost;
          lowpos = j;
        }
      }
      else
      {
        W.cost = __dadd_rn(W.cost, __shfl_sync(kFull, dE, j));
        long long kc = order_key(W.cost);
        if (kc < W.klow)
        {
          W.klow = kc;
          W.low = W.cost;
          lowpos = j;
        }
      }
    }
    __syncwarp();
    if (lowpos >= 0)
    {
      for (int q = lane; q < nwd; q += 32) lsp[q] = spins[q];
      __syncwarp();
      const unsigned undo = flips & ~((2u << lowpos) - 1u);
      if (lane == 0 && undo) lsp[wi] ^= undo;
      __syncwarp();
    }
    W.natt += (unsigned long long)adv;
    W.nacc += (unsigned long long)__popc(flips);
    W.nwin++;
    if (REPLAY) W.rs = S.jA[draws] * W.rs + S.jC[draws];
    cursor += adv;
  }
  __syncwarp();
}

template <int FL, bool REPLAY, bool INT, bool SMEM, bool BATCH>
__global__ void __launch_bounds__(256, 1) sweep2_kernel(SweepArgs a)
{
  using C = typename std::conditional<INT, int, double>::type;
  extern __shared__ __align__(16) unsigned char smem[];
  double* s_ln = (double*)smem;                                   // row 0: 2048 B
  float* s_scr = (float*)(smem + 2048);                           // row 0: 3072 B
  unsigned long long* s_A = (unsigned long long*)(smem + 5120);  // 520 B
  unsigned long long* s_C = s_A + 65;                             // 520 B
  unsigned char* s_warp = smem + kTableBytes;
  for (int t = threadIdx.x; t < 256; t += blockDim.x) s_ln[t] = c_ln[t];
  for (int t = threadIdx.x; t < 768; t += blockDim.x) s_scr[t] = c_scr[t];
  for (int t = threadIdx.x; t < 65; t += blockDim.x)
  {
    s_A[t] = c_jA[t];
    s_C[t] = c_jC[t];
  }
  __syncthreads();
  const Smem S{s_ln, s_scr, s_A, s_C};

  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int w = blockIdx.x * (blockDim.x >> 5) + wib;
  if (w >= a.n_streams) return;
  const bool staged = (FL == F_PARITY || FL == F_COUNTER);
  // per-warp region: [bars 16][dirty words 144][tiles 2][term bytes][spins][lowest]
  const int cap = a.tile_cap > 0 ? a.tile_cap : Tile<INT>::kMaxCap;
  const int tile_b = staged ? tile_bytes<INT>(cap) : 0;
  const int state_bytes = SMEM ? (a.p.mp + 8 * a.p.nw) : 0;
  unsigned char* my = s_warp + (size_t)wib * (kHdr + 2 * tile_b + state_bytes);
  unsigned long long* bars = (unsigned long long*)my;
  uint32_t* dirty = (uint32_t*)(my + 16);
  unsigned char* tile_base = my + kHdr;  // tile b at tile_base + b * tile_b
  unsigned char* my_state = my + kHdr + 2 * tile_b;
  if (staged && lane == 0)
  {
    mbar_init(&bars[0]);
    mbar_init(&bars[1]);
  }
  __syncwarp();
  unsigned phase0 = 0, phase1 = 0;
  Walk W;
  W.rs = (REPLAY && !BATCH) ? a.rng[w] : 0;
  // batches: the warp takes walkers from the queue in index order (the
  // population lies longest instance first) until every walker is taken
  auto take = [&]() -> int {
    int q = 0;
    if (lane == 0) q = atomicAdd(a.queue, 1);
    return __shfl_sync(kFull, q, 0);
  };

  for (int r = BATCH ? take() : w; r < a.n_walkers; r = BATCH ? take() : r + a.n_streams)
  {
    const DevModel m = BATCH ? a.models[a.model_of[r]] : a.m;
    const int Sz = m.sweep_size;
    const int nwd = (m.n_vars + 31) >> 5;
    if (BATCH && REPLAY) W.rs = a.rng[r];
    const int slot = a.slot_of ? a.slot_of[r] : r;
    uint32_t* g_spins = a.p.spins + (size_t)slot * a.p.nw;
    uint8_t* g_ts = a.p.tstate + (size_t)slot * a.p.mp;
    uint32_t* g_lsp = a.p.lspins + (size_t)r * a.p.nw;
    uint8_t* ts;
    uint32_t* spins;
    uint32_t* lsp;
    if (SMEM)
    {
      ts = my_state;
      spins = (uint32_t*)(my_state + a.p.mp);
      lsp = spins + a.p.nw;
      copy_words((uint32_t*)ts, (const uint32_t*)g_ts, a.p.mp / 4, lane);
      copy_words(spins, g_spins, a.p.nw, lane);
      copy_words(lsp, g_lsp, a.p.nw, lane);
      __syncwarp();
    }
    else
    {
      ts = g_ts;
      spins = g_spins;
      lsp = g_lsp;
    }
    W.cost = a.p.cost[slot];
    W.low = a.p.lowest[r];
    W.icost = INT ? (long long)W.cost : 0;
    W.ilow = INT ? (long long)W.low : 0;
    W.klow = order_key(W.low);
    W.natt = W.nacc = W.nwin = 0;
    W.key = 0;
    if (!REPLAY)
    {
      const long long lr = BATCH ? a.local_of[r] : r;
      W.key = counter_key(a.seed + (uint32_t)(lr / a.key_div),
                          a.key_base + (unsigned long long)(lr % a.key_div));
    }
    const int nblocks = (Sz + 31) >> 5;
    const int total_blocks = nblocks * a.n_sweeps;
    int toff[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}}, tq0[2] = {0, 0}, tq1[2] = {0, 0};
    if (staged && total_blocks > 0 && lane == 0)
    {
      int q0 = __ldg(m.row + 0), q1 = __ldg(m.row + min(32, Sz));
      tile_issue<INT>(tile_at<INT>(tile_base, cap), cap, &bars[0], m, q0, q1, toff[0]);
      tq0[0] = q0;
      tq1[0] = q1;
    }
    bool aborted = false;
    for (int gb = 0; gb < total_blocks; gb++)
    {
      const int k = gb / nblocks;
      const int bi = gb - k * nblocks;
      const int buf = gb & 1;
      const long long swp = a.sweep_base + k;
      const double beta = a.beta[(long long)r * a.bs_w + swp * a.bs_s];
      const bool beta_inf =
          ((unsigned long long)__double_as_longlong(beta) & 0x7FFFFFFFFFFFFFFFULL) ==
          0x7FF0000000000000ULL;
      const float nbeta_f = -approx_float(beta);
      const unsigned long long ctr0 = (unsigned long long)swp * (unsigned long long)Sz;
      const int i0 = bi << 5;
      if (staged)
      {
        // issue the next block's tile into the other buffer, then wait for ours
        if (gb + 1 < total_blocks && lane == 0)
        {
          int nb = (bi + 1 < nblocks) ? bi + 1 : 0;
          int q0 = __ldg(m.row + (nb << 5)), q1 = __ldg(m.row + min((nb << 5) + 32, Sz));
          tile_issue<INT>(tile_at<INT>(tile_base + (buf ^ 1) * tile_b, cap), cap, &bars[buf ^ 1], m, q0, q1,
                          toff[buf ^ 1]);
          tq0[buf ^ 1] = q0;
          tq1[buf ^ 1] = q1;
        }
        bool ok = mbar_wait(&bars[buf], buf ? phase1 : phase0, a.err);
        if (buf) phase1 ^= 1u; else phase0 ^= 1u;
        if (!__all_sync(kFull, ok))
        {
          aborted = true;
          break;
        }
        const int t_q0 = __shfl_sync(kFull, tq0[buf], 0);
        const int t_q1 = __shfl_sync(kFull, tq1[buf], 0);
        const int t_oi = __shfl_sync(kFull, toff[buf][0], 0);
        const int t_oc = __shfl_sync(kFull, toff[buf][1], 0);
        const int t_on = __shfl_sync(kFull, toff[buf][2], 0);
        const int t_of = __shfl_sync(kFull, toff[buf][3], 0);
        if (t_q1 - t_q0 <= cap)
        {
          const int v = i0 + lane;
          const int rb = (v < Sz) ? __ldg(m.row + v) : t_q0;
          const Tile<INT> tile = tile_at<INT>(tile_base + buf * tile_b, cap);
          block_rounds<FL, REPLAY, INT, true>(S, m, W, ts, spins, lsp, dirty,
                                              tile.inc + t_oi + (rb - t_q0),
                                              tile.coef + t_oc + (rb - t_q0),
                                              tile.coef_f + t_of + (rb - t_q0),
                                              tile.near + t_on + (rb - t_q0), i0, Sz, nwd,
                                              beta, nbeta_f, beta_inf, ctr0);
        }
        else
          block_rounds<FL, REPLAY, INT, false>(S, m, W, ts, spins, lsp, dirty, nullptr, nullptr,
                                               nullptr, nullptr, i0, Sz, nwd, beta, nbeta_f,
                                               beta_inf, ctr0);
      }
      else
        block_rounds_plain<FL, REPLAY, INT>(S, m, W, spins, lsp, i0, Sz, nwd, beta, nbeta_f,
                                            beta_inf, ctr0);
    }
    if (aborted) return;
    if (SMEM)
    {
      __syncwarp();
      copy_words((uint32_t*)g_ts, (const uint32_t*)ts, a.p.mp / 4, lane);
      copy_words(g_spins, spins, a.p.nw, lane);
      copy_words(g_lsp, lsp, a.p.nw, lane);
    }
    if (lane == 0)
    {
      a.p.cost[slot] = INT ? (double)W.icost : W.cost;
      const double nlow = INT ? (double)W.ilow : W.low;
      if (a.p.lowtag && nlow < a.p.lowest[r]) a.p.lowtag[r] = a.tag;
      a.p.lowest[r] = nlow;
      a.p.attempts[r] += W.natt;
      a.p.accepts[r] += W.nacc;
      a.p.step_att[r] += W.natt;
      a.p.step_acc[r] += W.nacc;
      if (a.p.windows) a.p.windows[r] += W.nwin;
      if (BATCH && REPLAY) a.rng[r] = W.rs;
    }
    __syncwarp();
  }
  if (REPLAY && !BATCH && lane == 0) a.rng[w] = W.rs;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

int warp_region_bytes(const SweepArgs& a, bool smem_state)
{
  const bool INT = a.m.int_mode != 0;
  const bool staged = (a.m.flavor == F_PARITY || a.m.flavor == F_COUNTER);
  const int cap = a.tile_cap > 0 ? a.tile_cap : (INT ? Tile<true>::kMaxCap : Tile<false>::kMaxCap);
  const int tile = staged ? (INT ? tile_bytes<true>(cap) : tile_bytes<false>(cap)) : 0;
  return kHdr + 2 * tile + (smem_state ? a.p.mp + 8 * a.p.nw : 0);
}

// the tile capacity for a model: its largest block, rounded up to a
// multiple of 8, at most the kernel's maximum
int tile_cap_for(const DevModel& m)
{
  const int mx = m.int_mode ? Tile<true>::kMaxCap : Tile<false>::kMaxCap;
  return std::max(8, std::min(mx, (m.max_block_inc + 7) & ~7));
}

template <int FL, bool R, bool I, bool SM, bool B>
static cudaError_t go(const SweepArgs& a, cudaStream_t s, int wpb, int smem)
{
  auto k = sweep2_kernel<FL, R, I, SM, B>;
  static int configured = -1;
  if (smem > 48 * 1024 && configured < smem)
  {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    configured = smem;
  }
  int blocks = (a.n_streams + wpb - 1) / wpb;
  if (B)
  {
    // persistent: as many blocks as stay resident, the queue feeds them
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 32 * wpb, smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    blocks = std::max(1, std::min((a.n_walkers + wpb - 1) / wpb, std::max(1, per_sm) * sms));
    SweepArgs b = a;
    b.n_streams = blocks * wpb;
    k<<<blocks, 32 * wpb, smem, s>>>(b);
    return cudaGetLastError();
  }
  if (blocks > 0) k<<<blocks, 32 * wpb, smem, s>>>(a);
  return cudaGetLastError();
}

template <int FL, bool R, bool I>
static cudaError_t go_sm(const SweepArgs& a, cudaStream_t s, int wpb, int smem, bool sm)
{
  if (a.queue) return go<FL, R, I, true, true>(a, s, wpb, smem);  // batches stage their state
  return sm ? go<FL, R, I, true, false>(a, s, wpb, smem) : go<FL, R, I, false, false>(a, s, wpb, smem);
}

template <int FL>
static cudaError_t go_fl(const SweepArgs& a, cudaStream_t s, int wpb, int smem, bool sm)
{
  const bool I = a.m.int_mode != 0;
  if (a.replay)
    return I ? go_sm<FL, true, true>(a, s, wpb, smem, sm) : go_sm<FL, true, false>(a, s, wpb, smem, sm);
  return I ? go_sm<FL, false, true>(a, s, wpb, smem, sm) : go_sm<FL, false, false>(a, s, wpb, smem, sm);
}

void upload_sweep_tables(const double* ln, const float* scr, const unsigned long long* jA,
                         const unsigned long long* jC)
{
  cudaMemcpyToSymbol(c_ln, ln, 1024 * sizeof(double));
  cudaMemcpyToSymbol(c_scr, scr, 3072 * sizeof(float));
  cudaMemcpyToSymbol(c_jA, jA, 65 * sizeof(unsigned long long));
  cudaMemcpyToSymbol(c_jC, jC, 65 * sizeof(unsigned long long));
}
}  // namespace sw

bool sweep_state_fits(const SweepArgs& a)
{
  SweepArgs b = a;
  if (b.tile_cap <= 0) b.tile_cap = sw::tile_cap_for(b.m);
  return sw::kTableBytes + sw::warp_region_bytes(b, true) <= 227 * 1024;
}

// Launch: warps per block chosen so that the grid spreads over the SMs;
// walker state goes to shared memory when the per-warp region fits.
cudaError_t launch_sweep(const SweepArgs& a_in, cudaStream_t s, int wpb)
{
  using namespace sw;
  // the field-cached sweep when the caller keeps fields for this population
  if (a_in.field && a_in.smem_state && fc_fits(a_in.m, a_in.p.nw, a_in.p.mp)) return launch_fc_sweep(a_in, s);
  // record tiles sized to the largest block (a batch passes its largest)
  SweepArgs a = a_in;
  if (a.tile_cap <= 0) a.tile_cap = tile_cap_for(a.m);
  if (wpb < 1) wpb = 1;
  if (wpb > 8) wpb = 8;
  const int max_smem = 227 * 1024;
  bool sm = a.smem_state != 0;
  int per = warp_region_bytes(a, sm);
  if (sm)
  {
    while (wpb > 1 && kTableBytes + wpb * per > max_smem) wpb--;
    if (kTableBytes + wpb * per > max_smem)
    {
      sm = false;
      per = warp_region_bytes(a, false);
    }
  }
  if (a.queue && !sm) return cudaErrorInvalidValue;  // batches stage their state
  int smem = kTableBytes + wpb * per;
  switch (a.m.flavor)
  {
    case F_PARITY: return go_fl<F_PARITY>(a, s, wpb, smem, sm);
    case F_COUNTER: return go_fl<F_COUNTER>(a, s, wpb, smem, sm);
    case F_PLAIN_ISING: return go_fl<F_PLAIN_ISING>(a, s, wpb, smem, sm);
    default: return go_fl<F_PLAIN_PUBO>(a, s, wpb, smem, sm);
  }
}
}  // namespace qio

namespace qio
{
void sw_upload(const double* ln, const float* scr, const unsigned long long* jA,
               const unsigned long long* jC)
{
  sw::upload_sweep_tables(ln, scr, jA, jC);
}
}  // namespace qio
