// fields.cu -- the field-cached Metropolis sweep (sm_103a).
//
// Two warps own one walker.  The DECIDER runs the reference's ordered sweep
// (markov/walker.h:143-153,209-229) in 32-variable windows, like the
// windowed kernel, but it reads each variable's cost difference from a
// cached local field instead of summing its row: the field is the
// difference in fixed point (DevModel::fc_rec), kept exact under every flip
// by integer shared-memory atomics on the co-members of the flipped
// variable's terms.  A field differs from the reference's FP64 sum by less
// than deg + 1 units, so its sign and the FP32-screened ln-table comparison
// (markov/metropolis.h:64-104) are decided from it with a rigorous margin;
// only inside the margin is the exact FP64 sum taken, in the reference's
// term order.  Committed flips go to a flip log in shared memory, with the
// contributing-incidence masks read before the flip.
//
// The ACCOUNTANT consumes the log in batches of up to 32 flips: every lane
// recomputes one flip's exact FP64 cost difference from its masks (the
// reference's order and rounding, model/ising.h:108-117, model/pubo.h:
// 335-367), then the running cost is accumulated in flip order exactly as
// cost_ += diff (markov/walker.h:225) and the lowest state is taken at the
// first strict improvement (markov/walker.h:269-280) from the accountant's
// own copy of the spins.  Neither the decisions nor the draws depend on the
// running cost, so moving it off the decider changes nothing in the chain.
//
// Waits between the two warps poll shared-memory counters (acquire/release)
// with a time limit on lack of progress; on expiry the kernel raises the
// device error flag and both warps return.
#include <algorithm>
#include <climits>

#include "metropolis.cuh"
#include "qio_internal.h"

namespace qio
{
namespace fc
{
using namespace qio::mc;
static const unsigned kFull = 0xffffffffu;
static const int kCap = 512;      // tile records (16 B each) per buffer
static const int kLog = 128;      // flip-log entries per walker (power of 2)
static const int kCtrl = 64;      // per-walker control block
static const int kTable = 6208;   // per-block tables (ln row 0, screen row 0, jumps)
static const unsigned kExactF = 0x80000000u;  // log entry: exact FP64 difference
static const unsigned kExactI = 0x40000000u;  // log entry: exact integer difference
static const unsigned long long kTimeoutNs = 4000000000ULL;  // 4 s without progress

__constant__ double c_ln[1024];
__constant__ float c_scr[3072];
__constant__ unsigned long long c_jA[65], c_jC[65];

// ---- shared-memory synchronisation between the two warps -----------------
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
  unsigned v;
  asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];"
               : "=r"(v)
               : "r"((unsigned)__cvta_generic_to_shared(p))
               : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v)
{
  asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)),
               "r"(v)
               : "memory");
}
__device__ __forceinline__ unsigned long long now_ns()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void pair_sync(int id)
{
  asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory");
}

// ---- TMA bulk copy of a tile of records, completion on an mbarrier --------
__device__ __forceinline__ unsigned smem_u32(const void* p)
{
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void tile_issue(uint4* dst, const uint4* src, int n, unsigned long long* bar)
{
  const unsigned bytes = (unsigned)(n > 0 ? n : 1) * 16u;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
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
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity)
{
  for (int it = 0; it < (1 << 22); it++)
    if (mbar_try(bar, parity)) return true;
  return false;
}

// ---- ln-table comparison ---------------------------------------------------
// rows 1..3 (redraws, 1 in 256 uphill attempts) stay in constant memory
__device__ __forceinline__ const double* ln_base(const double* s_ln0, int row)
{
  return row ? c_ln : s_ln0;
}
__device__ __forceinline__ const float* scr_base(const float* s_scr0, int row)
{
  return row ? c_scr : s_scr0;
}
// value(r) < thr in FP32 with the screen's margins plus `extra` (the field's
// own deviation from the exact threshold); 1 accept, 0 reject, -1 undecided
__device__ __forceinline__ int screen(const float* scr, uint32_t r, int row, float thr_f, float extra)
{
  const int b = (int)(r & 255u);
  if (b == 1) return 0;  // y0 = log(0): NaN, never less
  const int k = (row * 256 + b) * 3;
  const float y0 = scr[k], dy = scr[k + 1], ev = scr[k + 2];
  const float dist = __fmul_rn((float)(r >> 8), 5.96046483e-08f);
  const float value = __fmaf_rn(dist, dy, y0);
  const float et = __fmaf_rn(fabsf(thr_f), 1.9073486328125e-06f, 1e-30f) + extra;  // 2^-19
  if (__fadd_rn(value, ev) < __fsub_rn(thr_f, et)) return 1;
  if (__fsub_rn(value, ev) > __fadd_rn(thr_f, et)) return 0;
  return -1;
}

__device__ __forceinline__ uint32_t spin_of(const uint32_t* spins, int v)
{
  return (spins[v >> 5] >> (v & 31)) & 1u;
}

// Exact cost difference of flipping v (FP64 models): the reference's sum
// over the row in ascending term id, from the current term states.
template <int FL>
__device__ double exact_dE(const DevModel& m, int v, uint32_t sv, const uint8_t* z)
{
  const int rb = __ldg(m.row + v), re = __ldg(m.row + v + 1);
  double d = 0.0;
  for (int k = rb; k < re; k++)
  {
    const uint32_t e = __ldg(m.inc + k);
    const uint32_t zz = z[e & ~kNegBit];
    const double c = __ldg(m.coef + k);
    if (FL == F_PARITY) d = __dadd_rn(d, zz ? -c : c);
    else
    {
      const bool lit = ((sv ^ (e >> 31)) & 1u) != 0u;
      if (lit ? (zz == 1u) : (zz == 0u)) d = lit ? __dadd_rn(d, c) : __dsub_rn(d, c);
    }
  }
  return (FL == F_PARITY) ? neg2x(d) : d;
}

// Exact cost difference from a log entry's masks (accountant): qm = the
// contributing incidences, sm = their signs.
template <int FL>
__device__ __forceinline__ double dE_from_masks(const DevModel& m, int v, int deg, uint32_t qm,
                                                uint32_t sm)
{
  const double* pc = m.coef + __ldg(m.row + v);
  uint32_t q = (FL == F_PARITY) ? ((deg >= 32) ? kFull : ((1u << deg) - 1u)) : qm;
  double d = 0.0;
  while (q)
  {
    // four loads in flight ahead of the dependent adds
    double c[4];
    int k[4];
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
      k[i] = q ? __ffs(q) - 1 : -1;
      q &= q - 1;
      c[i] = k[i] >= 0 ? __ldg(pc + k[i]) : 0.0;
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
      if (k[i] >= 0)
      {
        const bool s = ((sm >> k[i]) & 1u) != 0u;
        if (FL == F_PARITY) d = __dadd_rn(d, s ? -c[i] : c[i]);
        else d = s ? __dadd_rn(d, c[i]) : __dsub_rn(d, c[i]);
      }
  }
  return (FL == F_PARITY) ? neg2x(d) : d;
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

// Per-walker shared-memory region.
struct Region
{
  unsigned long long* bars;  // 2 mbarriers
  unsigned* head;            // log entries published by the decider
  unsigned* tail;            // log entries consumed by the accountant
  unsigned* done;            // the decider finished the walker
  unsigned* beat;            // decider progress (blocks processed)
  unsigned* abort;           // a wait gave up: both warps leave
  uint4* log;                // kLog entries
  uint4* tiles;              // 2 x kCap records
  int* G;                    // fields, fc_words(N)
  uint8_t* z;                // term states, mp bytes
  uint32_t* spins;           // nw words
  uint32_t* aspins;          // the accountant's spins, nw words
};

__host__ __device__ inline int region_bytes(int n_vars, int nw, int mp)
{
  const int np = ((n_vars + 31) / 32) * 32;
  return kCtrl + kLog * 16 + 2 * kCap * 16 + np * 4 + mp + 8 * nw;
}

__device__ __forceinline__ Region carve(unsigned char* base, int n_vars, int nw, int mp)
{
  Region R;
  R.bars = (unsigned long long*)base;
  unsigned* c = (unsigned*)(base + 16);
  R.head = c;
  R.tail = c + 1;
  R.done = c + 2;
  R.beat = c + 3;
  R.abort = c + 4;
  R.log = (uint4*)(base + kCtrl);
  R.tiles = R.log + kLog;
  R.G = (int*)(R.tiles + 2 * kCap);
  const int np = ((n_vars + 31) / 32) * 32;
  R.z = (uint8_t*)(R.G + np);
  R.spins = (uint32_t*)(R.z + mp);
  R.aspins = R.spins + nw;
  return R;
}

__device__ __forceinline__ void raise_abort(const Region& R, int* err)
{
  if (err) atomicExch(err, 1);
  st_release(R.abort, 1u);
}

// Field of variable v from the term states and spins (fresh populations).
template <int FL>
__device__ __forceinline__ int field_of(const DevModel& m, int v, const uint8_t* z, const uint32_t* spins)
{
  const int rb = __ldg(m.row + v), re = __ldg(m.row + v + 1);
  const uint32_t sv = spin_of(spins, v);
  const int pack = m.fc_pack;
  int acc = 0;
  for (int k = rb; k < re; k++)
  {
    const uint4 rec = __ldg(m.fc_rec + k);
    const uint32_t zz = z[rec.x & ~kNegBit];
    const int q = (int)rec.y;
    if (FL == F_PARITY) acc += zz ? -q : q;
    else
    {
      const uint32_t lit = (sv ^ (rec.x >> 31)) & 1u;
      if (lit ? (zz == 1u) : (zz == 0u)) acc += (lit ? q : -q) + pack;
    }
  }
  return acc;
}

// change of co-member w's field when a term's state goes zo -> zn
template <int FL>
__device__ __forceinline__ int co_delta(uint32_t cw, uint32_t zo, uint32_t zn, int q, int pack,
                                        const uint32_t* spins)
{
  if (FL == F_PARITY) return zo ? 2 * q : -2 * q;  // the term's contribution changes sign
  const uint32_t litw = (spin_of(spins, (int)(cw & 0x7FFFu)) ^ (cw >> 15)) & 1u;
  const int qo = litw ? (zo == 1u) : (zo == 0u);
  const int qn = litw ? (zn == 1u) : (zn == 0u);
  return (qn - qo) * ((litw ? q : -q) + pack);
}

// Apply one incidence of a committed flip: the term's state moves, and the
// fields of the term's other members change by the exact integer amounts.
// Returns this incidence's bits for the flip's log masks: bit 0 = the
// incidence contributes to the flip's cost difference, bit 1 = its sign.
template <int FL>
__device__ __forceinline__ unsigned apply_incidence(const DevModel& m, const Region& R, const uint4 rec,
                                                    uint32_t sv, int vj, int pack)
{
  const uint32_t e = rec.x & ~kNegBit;
  const uint32_t zo = R.z[e];
  const int q = (int)rec.y;
  uint32_t zn;
  unsigned bits;
  if (FL == F_PARITY)
  {
    bits = 1u | (zo ? 2u : 0u);
    zn = zo ^ 1u;
  }
  else
  {
    const uint32_t lit = (sv ^ (rec.x >> 31)) & 1u;
    bits = ((lit ? (zo == 1u) : (zo == 0u)) ? 1u : 0u) | (lit << 1);
    zn = lit ? zo - 1u : zo + 1u;
  }
  R.z[e] = (uint8_t)zn;
  const int nco = (int)(rec.w >> 16);
  if (nco <= 3)
  {
    const uint32_t cws[3] = {rec.z & 0xFFFFu, rec.z >> 16, rec.w & 0xFFFFu};
#pragma unroll
    for (int i = 0; i < 3; i++)
      if (i < nco)
      {
        const int d = co_delta<FL>(cws[i], zo, zn, q, pack, R.spins);
        if (d) atomicAdd(R.G + (cws[i] & 0x7FFFu), d);
      }
  }
  else
  {
    for (int x = __ldg(m.trow + e); x < __ldg(m.trow + e + 1); x++)
    {
      const uint32_t tv = __ldg(m.tvar + x);
      const uint32_t u = tv & ~kNegBit;
      if ((int)u == vj) continue;
      const uint32_t cw = u | ((tv & kNegBit) ? 0x8000u : 0u);
      const int d = co_delta<FL>(cw, zo, zn, q, pack, R.spins);
      if (d) atomicAdd(R.G + u, d);
    }
  }
  return bits;
}

// ---------------------------------------------------------------------------
// The decider: one walker's sweeps.  Returns false when a wait gave up.
// Committed flips are logged at head + i and published to the accountant at
// the end of each 32-variable block (a block logs at most 32 flips; the log
// is checked for room for them when the block starts).
// ---------------------------------------------------------------------------
template <int FL, bool REPLAY, bool INT>
__device__ bool decide_sweeps(const SweepArgs& a, const Region& R, const double* s_ln0, const float* s_scr0,
                              const unsigned long long* s_jA, const unsigned long long* s_jC, int r,
                              unsigned* phase, uint64_t& rs, unsigned long long& natt,
                              unsigned long long& nacc, unsigned long long& nwin)
{
  const DevModel& m = a.m;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int N = m.n_vars;
  const int pack = m.fc_pack;
  uint64_t key = 0;
  if (!REPLAY)
    key = counter_key(a.seed + (uint32_t)(r / a.key_div), a.key_base + (unsigned long long)(r % a.key_div));
  const int nblocks = (N + 31) >> 5;
  const int total = nblocks * a.n_sweeps;
  unsigned head = 0;       // entries written (published at block ends)
  unsigned tail_seen = 0;  // lane 0: the accountant's count last seen
  // per-lane row data of the current and the next block (prefetched)
  auto row_data = [&](int blk, int& rb, int& deg, uint32_t& nb) {
    const int v = (blk << 5) + lane;
    rb = 0;
    deg = 0;
    nb = 0;
    if (v < N)
    {
      rb = __ldg(m.row + v);
      deg = __ldg(m.row + v + 1) - rb;
      nb = __ldg(m.nbr + v);
    }
  };
  int n_rb, n_deg;
  uint32_t n_nb;
  row_data(0, n_rb, n_deg, n_nb);
  int tq0 = 0, tq1 = 0;  // lane 0: record range of the tile in flight
  if (total > 0 && lane == 0)
  {
    tq0 = __ldg(m.row + 0);
    tq1 = __ldg(m.row + min(32, N));
    tile_issue(R.tiles, m.fc_rec + tq0, min(tq1 - tq0, kCap), &R.bars[0]);
  }
  double beta = 0.0;
  bool beta_inf = false;
  float nbeta_f = 0.f, fscale = 0.f, fsa = 0.f;
  unsigned long long ctr0 = 0;
  for (int gb = 0; gb < total; gb++)
  {
    const int k = gb / nblocks;
    const int bi = gb - k * nblocks;
    const int buf = gb & 1;
    if (bi == 0)
    {
      const long long swp = a.sweep_base + k;
      beta = a.beta[(long long)r * a.bs_w + swp * a.bs_s];
      beta_inf = ((unsigned long long)__double_as_longlong(beta) & 0x7FFFFFFFFFFFFFFFULL) ==
                 0x7FF0000000000000ULL;
      nbeta_f = -approx_float(beta);
      // thr = field * fscale approximates dE * (-beta)
      fscale = INT ? 0.f : (float)(beta * m.fc_inv * (FL == F_PARITY ? 2.0 : -1.0));
      fsa = fabsf(fscale) * 1.0001f;
      ctr0 = (unsigned long long)swp * (unsigned long long)N;
    }
    const int i0 = bi << 5;
    // this block's record range, then the next block's tile into the other buffer
    const int b_q0 = __shfl_sync(kFull, tq0, 0);
    const int b_q1 = __shfl_sync(kFull, tq1, 0);
    if (gb + 1 < total && lane == 0)
    {
      const int nbk = (bi + 1 < nblocks) ? bi + 1 : 0;
      tq0 = __ldg(m.row + (nbk << 5));
      tq1 = __ldg(m.row + min((nbk << 5) + 32, N));
      tile_issue(R.tiles + (buf ^ 1) * kCap, m.fc_rec + tq0, min(tq1 - tq0, kCap), &R.bars[buf ^ 1]);
    }
    const int rb = n_rb, deg = n_deg;
    const uint32_t nb = n_nb;
    if (gb + 1 < total) row_data((bi + 1 < nblocks) ? bi + 1 : 0, n_rb, n_deg, n_nb);
    // room in the log for this block's flips
    bool ok = true;
    if (lane == 0 && head + 32u - tail_seen > (unsigned)kLog)
    {
      unsigned long long t0 = 0;
      unsigned last = tail_seen;
      while (true)
      {
        tail_seen = ld_acquire(R.tail);
        if (head + 32u - tail_seen <= (unsigned)kLog) break;
        if (tail_seen != last)
        {
          last = tail_seen;
          t0 = 0;
        }
        if (ld_acquire(R.abort))
        {
          ok = false;
          break;
        }
        const unsigned long long t = now_ns();
        if (t0 == 0) t0 = t;
        else if (t - t0 > kTimeoutNs)
        {
          raise_abort(R, a.err);
          ok = false;
          break;
        }
        __nanosleep(64);
      }
    }
    const bool tile_ok = mbar_wait(&R.bars[buf], phase[buf]);
    phase[buf] ^= 1u;
    if (!__all_sync(kFull, ok && tile_ok))
    {
      if (lane == 0)
      {
        if (!tile_ok) raise_abort(R, a.err);
        // the copy in flight lands before the walker's region is given up
        if (gb + 1 < total)
        {
          mbar_wait(&R.bars[buf ^ 1], phase[buf ^ 1]);
          phase[buf ^ 1] ^= 1u;
        }
      }
      __syncwarp();
      return false;
    }
    const bool staged = b_q1 - b_q0 <= kCap;
    const uint4* tile = R.tiles + buf * kCap;

    const int v = i0 + lane;
    const bool valid = v < N;
    const int nvalid = min(32, N - i0);
    uint32_t sv = valid ? spin_of(R.spins, v) : 0u;
    const int bnd = deg + 1;  // |field - exact| < bnd units
    const unsigned head0 = head;

    int cursor = 0;
    while (cursor < nvalid)
    {
      const bool active = valid && lane >= cursor;
      // replay: the draw at stream position `lane` and its screen value,
      // ahead of the field (an uphill lane takes the draw of its position)
      uint32_t pd = 0;
      float pval = 0.f, pev = 0.f;
      if (REPLAY)
      {
        pd = pcg_out(s_jA[lane] * rs + s_jC[lane]);
        const int b = (int)(pd & 255u);
        if (b >= 2)
        {
          const float* e = s_scr0 + b * 3;
          pval = __fmaf_rn(__fmul_rn((float)(pd >> 8), 5.96046483e-08f), e[1], e[0]);
          pev = e[2];
        }
      }
      const int g = active ? R.G[v] : 0;
      // ---- cost difference: sign from the field, exact inside its margin
      bool have_exact = false, uphill = false;
      double dE = 0.0;
      long long idE = 0;
      int F = 0;
      if (INT)
      {
        idE = (FL == F_PARITY) ? -2LL * (long long)g : (long long)g;
        uphill = active && idE > 0;
      }
      else
      {
        bool need = false;
        if (FL == F_PARITY)
        {
          F = g;
          need = active && F <= bnd && F >= -bnd;
          uphill = active && F < -bnd;
        }
        else
        {
          F = g >> 8;
          if (active && (g & 255) == 0) have_exact = true;  // nothing contributes: +0.0
          need = active && !have_exact && F <= bnd && F >= -bnd;
          uphill = active && !have_exact && F > bnd;
        }
        if (__any_sync(kFull, need))
        {
          if (need)
          {
            dE = exact_dE<FL>(m, v, sv, R.z);
            have_exact = true;
            uphill = !le_zero(dE);
          }
        }
      }
      bool acc = active && !uphill;
      const unsigned before = lt & ~((1u << cursor) - 1u);
      unsigned U = 0;
      int pos = 0;
      if (REPLAY)
      {
        U = __ballot_sync(kFull, uphill);
        pos = __popc(U & before);
      }
      uint32_t dr = 0;
      int drow = 0;
      bool redraw = false;
      int dec = 1;
      auto decide = [&](uint32_t rr, int row) -> int {
        if (beta_inf) return 0;
        const float* sc = scr_base(s_scr0, row);
        if (INT) return screen(sc, rr, row, __fmul_rn((float)idE, nbeta_f), 0.f);
        if (have_exact) return screen(sc, rr, row, __fmul_rn(approx_float(dE), nbeta_f), 0.f);
        return screen(sc, rr, row, __fmul_rn((float)F, fscale), fsa * (float)(bnd + 1));
      };
      if (REPLAY)
      {
        const uint32_t d0 = __shfl_sync(kFull, pd, pos & 31);
        const float v0 = __shfl_sync(kFull, pval, pos & 31);
        const float e0 = __shfl_sync(kFull, pev, pos & 31);
        if (uphill)
        {
          dr = d0;
          redraw = (dr & 255u) == 0;
          if (!redraw)
          {
            if (beta_inf || (dr & 255u) == 1u) dec = 0;
            else
            {
              float thr, extra = 0.f;
              if (INT) thr = __fmul_rn((float)idE, nbeta_f);
              else if (have_exact) thr = __fmul_rn(approx_float(dE), nbeta_f);
              else
              {
                thr = __fmul_rn((float)F, fscale);
                extra = fsa * (float)(bnd + 1);
              }
              const float et = __fmaf_rn(fabsf(thr), 1.9073486328125e-06f, 1e-30f) + extra;  // 2^-19
              if (__fadd_rn(v0, e0) < __fsub_rn(thr, et)) dec = 1;
              else if (__fsub_rn(v0, e0) > __fadd_rn(thr, et)) dec = 0;
              else dec = -1;
            }
          }
        }
      }
      else if (uphill)
      {
        const unsigned long long ctr = ctr0 + (unsigned long long)v;
        const uint64_t w0 = counter_draw(key, 2ULL * ctr);
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
              const uint64_t w1 = counter_draw(key, 2ULL * ctr + 1ULL);
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
      const unsigned Rm = REPLAY ? __ballot_sync(kFull, redraw) : 0u;
      if (!INT && __any_sync(kFull, uphill && !redraw && dec < 0))
      {
        // exact differences for the lanes inside the margin that can still
        // be committed: up to the first stop under the surely accepted lanes
        const bool sure = active && (!uphill || (!redraw && dec == 1));
        const unsigned As = __ballot_sync(kFull, sure);
        bool cs = false;
        if (active && lane > cursor)
          cs = (nb & (__brev(As) >> (32 - lane)) & ((1u << (lane - cursor)) - 1u)) != 0u;
        const unsigned stop_s = __ballot_sync(kFull, cs) | Rm;
        const int fs = stop_s ? (__ffs(stop_s) - 1) : 32;
        const bool cand = active && lane <= fs && !have_exact && uphill && !redraw && dec < 0;
        if (cand)
        {
          dE = exact_dE<FL>(m, v, sv, R.z);
          have_exact = true;
        }
        if (lane > fs && dec < 0) dec = 0;  // not committed this round
      }
      if (uphill && !redraw && dec < 0)
        dec = lut_less_exact(ln_base(s_ln0, drow), dr, drow, __dmul_rn(INT ? (double)idE : dE, -beta)) ? 1 : 0;
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
        if (!INT && lane == f && !have_exact)
        {
          dE = exact_dE<FL>(m, v, sv, R.z);
          have_exact = true;
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
              cur = pcg_out(s_jA[pos + used] * rs + s_jC[pos + used]);
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
          bool okk;
          if (decided) okk = true;
          else if (beta_inf) okk = false;
          else
            okk = lut_less_exact(ln_base(s_ln0, row), cur, row, __dmul_rn(INT ? (double)idE : dE, -beta));
          sacc = okk ? 1 : 0;
        }
        sacc = __shfl_sync(kFull, sacc, f);
        used = __shfl_sync(kFull, used, f);
        if (sacc) flips |= 1u << f;
        draws += used;
      }
      const int adv = f + (slow ? 1 : 0) - cursor;
      const bool mine = ((flips >> lane) & 1u) != 0u;
      const int nfl = __popc(flips);

      if (nfl)
      {
        // a wide row keeps no masks: its exact difference is taken now,
        // before the flips change the term states
        if (!INT && mine && !have_exact && deg > 32)
        {
          dE = exact_dE<FL>(m, v, sv, R.z);
          have_exact = true;
        }
        const bool keep_masks = !INT && mine && !have_exact;
        const int eslot = (int)((head + (unsigned)__popc(flips & lt)) & (unsigned)(kLog - 1));
        // the log entry: x = v | deg << 16 | kind, y/z = masks or the difference
        uint4 ent;
        ent.x = (unsigned)v | ((unsigned)deg << 16);
        ent.y = 0u;
        ent.z = 0u;
        ent.w = 0u;
        if (INT)
        {
          ent.x |= kExactI;
          ent.y = (unsigned)(unsigned long long)idE;
          ent.z = (unsigned)((unsigned long long)idE >> 32);
        }
        else if (have_exact)
        {
          ent.x |= kExactF;
          const unsigned long long bits = (unsigned long long)__double_as_longlong(dE);
          ent.y = (unsigned)bits;
          ent.z = (unsigned)(bits >> 32);
        }
        if (nfl <= 2)
        {
          // one flip at a time, the warp over its incidences (masks by ballot)
          unsigned fl = flips;
          while (fl)
          {
            const int j = __ffs(fl) - 1;
            fl &= fl - 1;
            const int dj = __shfl_sync(kFull, deg, j);
            const int rbj = __shfl_sync(kFull, rb, j);
            const uint32_t svj = __shfl_sync(kFull, sv, j);
            unsigned qm = 0, sm = 0;
            for (int k0 = 0; k0 < dj; k0 += 32)
            {
              const int kk = k0 + lane;
              unsigned bits = 0;
              if (kk < dj)
              {
                const uint4 rec = staged ? tile[rbj - b_q0 + kk] : __ldg(m.fc_rec + rbj + kk);
                bits = apply_incidence<FL>(m, R, rec, svj, i0 + j, pack);
              }
              if (k0 == 0)
              {
                qm = __ballot_sync(kFull, bits & 1u);
                sm = __ballot_sync(kFull, (bits >> 1) & 1u);
              }
            }
            if (lane == j)
            {
              if (keep_masks)
              {
                ent.y = (FL == F_PARITY) ? 0u : qm;
                ent.z = sm;
              }
              R.log[eslot] = ent;
            }
          }
        }
        else
        {
          // many flips: their incidences laid out back to back over the warp
          if (mine) R.log[eslot] = ent;
          __syncwarp();
          const int mydeg = mine ? deg : 0;
          const int incl = warp_scan32(mydeg, lane);
          const int excl = incl - mydeg;
          const int tot = __shfl_sync(kFull, incl, 31);
          const unsigned Fm = __ballot_sync(kFull, mine && mydeg > 0);
          const unsigned KM = __ballot_sync(kFull, keep_masks);
          for (int base = 0; base < tot; base += 32)
          {
            const int rel = excl - base;
            const unsigned starts =
                __reduce_or_sync(kFull, (mine && mydeg > 0 && rel >= 0 && rel < 32) ? (1u << rel) : 0u);
            const int nbefore = __popc(__ballot_sync(kFull, mine && mydeg > 0 && rel < 0));
            const int gi = base + lane;
            const int idx = nbefore + __popc(starts & ((2u << lane) - 1u)) - 1;
            int j = 0;
#pragma unroll
            for (int step = 16; step; step >>= 1)
              if (__popc(Fm & ((2u << (j + step - 1)) - 1u)) <= idx) j += step;
            j &= 31;
            const int ej = __shfl_sync(kFull, excl, j);
            const int rbj = __shfl_sync(kFull, rb, j);
            const uint32_t svj = __shfl_sync(kFull, sv, j);
            const int slj = __shfl_sync(kFull, eslot, j);
            if (gi < tot)
            {
              const int kk = gi - ej;
              const uint4 rec = staged ? tile[rbj - b_q0 + kk] : __ldg(m.fc_rec + rbj + kk);
              const unsigned bits = apply_incidence<FL>(m, R, rec, svj, i0 + j, pack);
              if ((KM >> j) & 1u)
              {
                if (FL != F_PARITY && (bits & 1u)) atomicOr(&R.log[slj].y, 1u << kk);
                if (bits & 2u) atomicOr(&R.log[slj].z, 1u << kk);
              }
            }
          }
        }
        __syncwarp();
        if (mine)
        {
          // the flipped variable's own field changes sign (the same terms
          // contribute, with the other sign); the count stays
          const int gv = R.G[v];
          R.G[v] = pack ? (-gv + 2 * (gv & 255)) : -gv;
          sv ^= 1u;
        }
        if (lane == 0) R.spins[i0 >> 5] ^= flips;
        __syncwarp();
        head += (unsigned)nfl;
      }
      natt += (unsigned long long)adv;
      nacc += (unsigned long long)nfl;
      nwin++;
      if (REPLAY) rs = s_jA[draws] * rs + s_jC[draws];
      cursor += adv;
    }
    // publish the block's flips
    if (head != head0)
    {
      __threadfence_block();
      __syncwarp();
    }
    if (lane == 0)
    {
      if (head != head0) st_release(R.head, head);
      st_release(R.beat, (unsigned)gb + 1u);
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// The accountant: running cost, lowest cost and lowest state from the log.
// ---------------------------------------------------------------------------
template <int FL, bool INT>
__device__ bool account(const SweepArgs& a, const Region& R, double& cost, double& low, long long& icost,
                        long long& ilow, uint32_t* g_lsp)
{
  const DevModel& m = a.m;
  const int lane = threadIdx.x & 31;
  const int nw = a.p.nw;
  unsigned tail = 0;
  long long klow = order_key(low);
  while (true)
  {
    // wait for a batch (16 entries, or whatever is left once the decider is done)
    unsigned h = 0;
    int fin = 0;
    if (lane == 0)
    {
      unsigned long long t0 = 0;
      unsigned last_h = tail, last_b = ld_acquire(R.beat);
      while (true)
      {
        h = ld_acquire(R.head);
        if (h - tail >= 16u) break;
        if (ld_acquire(R.done))
        {
          h = ld_acquire(R.head);
          fin = 1;
          break;
        }
        if (ld_acquire(R.abort))
        {
          fin = 2;
          break;
        }
        const unsigned b = ld_acquire(R.beat);
        if (h != last_h || b != last_b)
        {
          last_h = h;
          last_b = b;
          t0 = 0;
        }
        const unsigned long long t = now_ns();
        if (t0 == 0) t0 = t;
        else if (t - t0 > kTimeoutNs)
        {
          raise_abort(R, a.err);
          fin = 2;
          break;
        }
        __nanosleep(128);
      }
    }
    h = __shfl_sync(kFull, h, 0);
    fin = __shfl_sync(kFull, fin, 0);
    if (fin == 2) return false;
    while (h != tail)
    {
      const int n = (int)min(32u, h - tail);
      int v = 0;
      double d = 0.0;
      long long id = 0;
      if (lane < n)
      {
        const uint4 ent = R.log[(tail + (unsigned)lane) & (unsigned)(kLog - 1)];
        v = (int)(ent.x & 0x7FFFu);
        const int deg = (int)((ent.x >> 16) & 255u);
        const unsigned long long bits = (unsigned long long)ent.y | ((unsigned long long)ent.z << 32);
        if (INT) id = (long long)bits;
        else if (ent.x & kExactF) d = __longlong_as_double((long long)bits);
        else d = dE_from_masks<FL>(m, v, deg, ent.y, ent.z);
      }
      __syncwarp();
      tail += (unsigned)n;
      if (lane == 0) st_release(R.tail, tail);
      // running cost in flip order (markov/walker.h:225) and the first
      // strict improvement of the lowest (markov/walker.h:269-280)
      int lowpos = -1;
      if (INT)
      {
        const long long pre = warp_scan64(lane < n ? id : 0LL, lane);
        const long long ci = icost + pre;
        long long mn = lane < n ? ci : LLONG_MAX;
#pragma unroll
        for (int s = 16; s; s >>= 1) mn = min(mn, __shfl_xor_sync(kFull, mn, s));
        if (mn < ilow)
        {
          lowpos = __ffs(__ballot_sync(kFull, lane < n && ci == mn)) - 1;
          ilow = mn;
        }
        icost += __shfl_sync(kFull, pre, 31);
      }
      else
      {
        double dn = __shfl_sync(kFull, d, 0);
        for (int i = 0; i < n; i++)
        {
          const double di = dn;
          dn = __shfl_sync(kFull, d, (i + 1) & 31);  // ahead of the dependent add
          cost = __dadd_rn(cost, di);
          const long long kc = order_key(cost);
          if (kc < klow)
          {
            klow = kc;
            low = cost;
            lowpos = i;
          }
        }
      }
      // the accountant's spins, and the lowest state at lowpos
      if (lane < n && lane <= lowpos) atomicXor(R.aspins + (v >> 5), 1u << (v & 31));
      __syncwarp();
      if (lowpos >= 0)
      {
        for (int q = lane; q < nw; q += 32) g_lsp[q] = R.aspins[q];
        __syncwarp();
      }
      if (lane < n && lane > lowpos) atomicXor(R.aspins + (v >> 5), 1u << (v & 31));
      __syncwarp();
    }
    if (fin == 1) return true;
  }
}

template <int FL, bool REPLAY, bool INT>
__global__ void __launch_bounds__(256, 1) fc_sweep_kernel(SweepArgs a, int wpc)
{
  extern __shared__ __align__(128) unsigned char smem[];
  double* s_ln0 = (double*)smem;                                  // 2048 B
  float* s_scr0 = (float*)(smem + 2048);                          // 3072 B
  unsigned long long* s_jA = (unsigned long long*)(smem + 5120);  // 520 B
  unsigned long long* s_jC = s_jA + 65;                            // 520 B
  for (int t = threadIdx.x; t < 256; t += blockDim.x) s_ln0[t] = c_ln[t];
  for (int t = threadIdx.x; t < 768; t += blockDim.x) s_scr0[t] = c_scr[t];
  for (int t = threadIdx.x; t < 65; t += blockDim.x)
  {
    s_jA[t] = c_jA[t];
    s_jC[t] = c_jC[t];
  }
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const bool decider = wib < wpc;
  const int ws = decider ? wib : wib - wpc;  // walker slot in the block
  const int w = blockIdx.x * wpc + ws;
  if (w >= a.n_streams) return;
  const DevModel& m = a.m;
  const int N = m.n_vars;
  const int nw = a.p.nw, mp = a.p.mp;
  const int np = ((N + 31) / 32) * 32;
  unsigned char* base = smem + kTable + (size_t)ws * region_bytes(N, nw, mp);
  const Region R = carve(base, N, nw, mp);
  const int bar_id = 1 + ws;
  if (decider && lane == 0)
  {
    mbar_init(&R.bars[0]);
    mbar_init(&R.bars[1]);
  }
  uint64_t rs = (REPLAY && decider) ? a.rng[w] : 0;
  unsigned phase[2] = {0u, 0u};  // mbarrier phases, kept across walkers

  for (int r = w; r < a.n_walkers; r += a.n_streams)
  {
    const int slot = a.slot_of ? a.slot_of[r] : r;
    uint32_t* g_spins = a.p.spins + (size_t)slot * nw;
    uint8_t* g_ts = a.p.tstate + (size_t)slot * mp;
    int* g_field = a.field + (size_t)slot * np;
    if (decider)
    {
      if (lane == 0)
      {
        *R.head = 0u;
        *R.tail = 0u;
        *R.done = 0u;
        *R.beat = 0u;
        *R.abort = 0u;
      }
      for (int q = lane; q < mp / 4; q += 32) ((uint32_t*)R.z)[q] = ((const uint32_t*)g_ts)[q];
      for (int q = lane; q < nw; q += 32) R.spins[q] = g_spins[q];
      if (a.field_valid)
        for (int q = lane; q < np / 4; q += 32) ((int4*)R.G)[q] = ((const int4*)g_field)[q];
    }
    pair_sync(bar_id);
    if (!a.field_valid)
    {
      // fields from the state: both warps
      for (int v = (decider ? 0 : 32) + lane; v < N; v += 64) R.G[v] = field_of<FL>(m, v, R.z, R.spins);
    }
    if (!decider)
      for (int q = lane; q < nw; q += 32) R.aspins[q] = R.spins[q];
    pair_sync(bar_id);

    bool ok;
    if (decider)
    {
      unsigned long long natt = 0, nacc = 0, nwin = 0;
      ok = decide_sweeps<FL, REPLAY, INT>(a, R, s_ln0, s_scr0, s_jA, s_jC, r, phase, rs, natt, nacc,
                                          nwin);
      if (lane == 0) st_release(R.done, 1u);
      pair_sync(bar_id);
      if (ok && !*(volatile unsigned*)R.abort)
      {
        for (int q = lane; q < mp / 4; q += 32) ((uint32_t*)g_ts)[q] = ((const uint32_t*)R.z)[q];
        for (int q = lane; q < nw; q += 32) g_spins[q] = R.spins[q];
        for (int q = lane; q < np / 4; q += 32) ((int4*)g_field)[q] = ((const int4*)R.G)[q];
        if (lane == 0)
        {
          a.p.attempts[r] += natt;
          a.p.accepts[r] += nacc;
          a.p.step_att[r] += natt;
          a.p.step_acc[r] += nacc;
          if (a.p.windows) a.p.windows[r] += nwin;
        }
      }
    }
    else
    {
      double cost = a.p.cost[slot], low = a.p.lowest[r];
      long long icost = INT ? (long long)cost : 0, ilow = INT ? (long long)low : 0;
      ok = account<FL, INT>(a, R, cost, low, icost, ilow, a.p.lspins + (size_t)r * nw);
      pair_sync(bar_id);
      if (ok && !*(volatile unsigned*)R.abort && lane == 0)
      {
        a.p.cost[slot] = INT ? (double)icost : cost;
        const double nlow = INT ? (double)ilow : low;
        if (a.p.lowtag && nlow < a.p.lowest[r]) a.p.lowtag[r] = a.tag;
        a.p.lowest[r] = nlow;
      }
    }
    if (*(volatile unsigned*)R.abort) return;
    pair_sync(bar_id);  // the region is reused by the next walker
  }
  if (REPLAY && decider && lane == 0) a.rng[w] = rs;
}

template <int FL, bool R, bool I>
static cudaError_t go(const SweepArgs& a, cudaStream_t s, int wpc, int smem)
{
  auto k = fc_sweep_kernel<FL, R, I>;
  static int configured = -1;
  if (smem > 48 * 1024 && configured < smem)
  {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    configured = smem;
  }
  const int blocks = (a.n_streams + wpc - 1) / wpc;
  if (blocks > 0) k<<<blocks, 64 * wpc, smem, s>>>(a, wpc);
  return cudaGetLastError();
}

template <int FL>
static cudaError_t go_fl(const SweepArgs& a, cudaStream_t s, int wpc, int smem)
{
  const bool I = a.m.int_mode != 0;
  if (a.replay) return I ? go<FL, true, true>(a, s, wpc, smem) : go<FL, true, false>(a, s, wpc, smem);
  return I ? go<FL, false, true>(a, s, wpc, smem) : go<FL, false, false>(a, s, wpc, smem);
}
}  // namespace fc

static const int kFcMaxSmem = 227 * 1024;
static const int kSms = 152;

int64_t fc_words(int n_vars) { return ((int64_t)(n_vars + 31) / 32) * 32; }

bool fc_fits(const DevModel& m, int nw, int mp)
{
  if (!m.fc_rec || m.sweep_size != m.n_vars || m.n_vars <= 0) return false;
  if (!(m.flavor == F_PARITY || m.flavor == F_COUNTER)) return false;
  return fc::kTable + fc::region_bytes(m.n_vars, nw, mp) <= kFcMaxSmem;
}

cudaError_t launch_fc_sweep(const SweepArgs& a, cudaStream_t s)
{
  if (!fc_fits(a.m, a.p.nw, a.p.mp) || !a.field) return cudaErrorInvalidValue;
  const int per = fc::region_bytes(a.m.n_vars, a.p.nw, a.p.mp);
  const int wmax = std::min(4, (kFcMaxSmem - fc::kTable) / per);
  // spread the walkers over the SMs: as few per block as fills them
  int wpc = (a.n_streams + kSms - 1) / kSms;
  wpc = std::max(1, std::min(wpc, wmax));
  const int smem = fc::kTable + wpc * per;
  switch (a.m.flavor)
  {
    case F_PARITY: return fc::go_fl<F_PARITY>(a, s, wpc, smem);
    default: return fc::go_fl<F_COUNTER>(a, s, wpc, smem);
  }
}

void fc_upload(const double* ln, const float* scr, const unsigned long long* jA,
               const unsigned long long* jC)
{
  cudaMemcpyToSymbol(fc::c_ln, ln, 1024 * sizeof(double));
  cudaMemcpyToSymbol(fc::c_scr, scr, 3072 * sizeof(float));
  cudaMemcpyToSymbol(fc::c_jA, jA, 65 * sizeof(unsigned long long));
  cudaMemcpyToSymbol(fc::c_jC, jC, 65 * sizeof(unsigned long long));
}
}  // namespace qio
