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

// the exact ln-table comparison (markov/metropolis.h:96-103), kept out of
// line: the FP64 instructions stay off the common path
__device__ __noinline__ bool exact_less(const double* ln, uint32_t r, int row, double dE, double beta)
{
  return lut_less_exact(ln, r, row, __dmul_rn(dE, -beta));
}

// The redraw chain of an uphill attempt whose first replayed draw had
// bucket 0 (markov/metropolis.h:93-103): draws at positions pos, pos + 1, ...
// Returns 1 accept / 0 reject, the draws used in *used.
__device__ __noinline__ int redraw_chain(const unsigned long long* jA, const unsigned long long* jC,
                                         uint64_t rs, int pos, const double* s_ln0, bool beta_inf,
                                         double dE, double beta, int* used)
{
  int row = -1, b = 0, u = 0;
  uint32_t cur = 0;
  bool decided = false;
  while (b == 0)
  {
    if (row < 3)
    {
      cur = pcg_out(jA[pos + u] * rs + jC[pos + u]);
      u++;
      b = (int)(cur & 255u);
      row++;
    }
    else
    {
      decided = true;
      break;
    }
  }
  *used = u;
  if (decided) return 1;
  if (beta_inf) return 0;
  return lut_less_exact(row ? c_ln : s_ln0, cur, row, __dmul_rn(dE, -beta)) ? 1 : 0;
}

__device__ __forceinline__ uint32_t spin_of(const uint32_t* spins, int v)
{
  return (spins[v >> 5] >> (v & 31)) & 1u;
}

// Exact cost difference of flipping v (FP64 models): the reference's sum
// over the row in ascending term id, from the current term states.
template <int FL>
__device__ __noinline__ double exact_dE(const DevModel& m, int v, uint32_t sv, const uint8_t* z)
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
__device__ __noinline__ void apply_overflow(const DevModel& m, const Region& R, uint32_t e, uint32_t zo,
                                            uint32_t zn, int q, int vj, int pack)
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

template <int FL>
__device__ __forceinline__ unsigned apply_incidence(const DevModel& m, const Region& R, const uint4 rec,
                                                    uint32_t sv, int vj, int pack)
{
  // every shared-memory load before the stores: the term state and the
  // co-members' spin words
  const uint32_t e = rec.x & ~kNegBit;
  const int nco = (int)(rec.w >> 16);
  const uint32_t cws[3] = {rec.z & 0xFFFFu, rec.z >> 16, rec.w & 0xFFFFu};
  const uint32_t zo = R.z[e];
  uint32_t sw[3] = {0u, 0u, 0u};
  if (FL != F_PARITY)
  {
#pragma unroll
    for (int i = 0; i < 3; i++)
      if (i < nco) sw[i] = R.spins[(cws[i] & 0x7FFFu) >> 5];
  }
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
  int d[3] = {0, 0, 0};
#pragma unroll
  for (int i = 0; i < 3; i++)
    if (i < nco && nco <= 3)
    {
      if (FL == F_PARITY) d[i] = zo ? 2 * q : -2 * q;  // the term's contribution changes sign
      else
      {
        const uint32_t litw = ((sw[i] >> (cws[i] & 31u)) ^ (cws[i] >> 15)) & 1u;
        const int qo = litw ? (zo == 1u) : (zo == 0u);
        const int qn = litw ? (zn == 1u) : (zn == 0u);
        d[i] = (qn - qo) * ((litw ? q : -q) + pack);
      }
    }
  R.z[e] = (uint8_t)zn;
#pragma unroll
  for (int i = 0; i < 3; i++)
    if (d[i]) atomicAdd(R.G + (cws[i] & 0x7FFFu), d[i]);
  // terms of more than three co-members (count 15): after the pass
  return bits | ((nco > 3) ? 4u : 0u) | (zo << 8) | (zn << 16);
}

// The co-members of a term with more than three (read from the term lists),
// for the incidences the pass marked; called by the whole warp after it.
template <int FL>
__device__ __noinline__ void apply_overflow_lane(const DevModel& m, const Region& R, bool mine, uint4 rec,
                                                 unsigned bits, int vj, int pack)
{
  if (!mine) return;
  const uint32_t e = rec.x & ~kNegBit;
  const uint32_t zo = (bits >> 8) & 255u, zn = (bits >> 16) & 255u;
  apply_overflow<FL>(m, R, e, zo, zn, (int)rec.y, vj, pack);
}

// Counter-stream draw of an attempt whose first byte was 0 (rare): the
// reference's redraw loop over the two 64-bit counter words.  Returns the
// draw and its ln-table row; *all_zero when every try came up 0.
__device__ __noinline__ uint32_t counter_redraw(uint64_t key, unsigned long long ctr, uint64_t w0, int* row_out,
                                               bool* all_zero)
{
  int row = -1, b = 0, used = 0;
  uint32_t cur = 0;
  *all_zero = false;
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
      *all_zero = true;
      break;
    }
  }
  *row_out = row;
  return cur;
}

// One wide flip (a row of more than 32 incidences): the warp over its
// incidences, 32 at a time.  Its log entry carries the exact difference.
template <int FL>
__device__ __noinline__ void apply_wide(const DevModel& m, const Region& R, const uint4* tile, bool staged,
                                        int b_q0, int rbj, int dj, uint32_t svj, int vj, int pack)
{
  const int lane = threadIdx.x & 31;
  for (int k0 = 0; k0 < dj; k0 += 32)
  {
    const int kk = k0 + lane;
    uint4 rec = make_uint4(0u, 0u, 0u, 0u);
    unsigned bits = 0;
    if (kk < dj)
    {
      rec = staged ? tile[rbj - b_q0 + kk] : __ldg(m.fc_rec + rbj + kk);
      bits = apply_incidence<FL>(m, R, rec, svj, vj, pack);
    }
    if (bits & 4u)
      apply_overflow<FL>(m, R, rec.x & ~kNegBit, (bits >> 8) & 255u, (bits >> 16) & 255u, (int)rec.y, vj, pack);
  }
}

// One window round in full generality (out of line): exact differences for
// fields inside their margin, ln-table comparisons inside the screen's
// margin, counter draws that needed the redraw loop, the replayed redraw
// chain of a zero bucket.  The fast path hands a round here whenever any
// of these occurs in it; this function decides the round from scratch.
struct RoundIo
{
  // in (per lane)
  bool active;
  int v, cursor, nvalid, bnd, g;
  uint32_t nb, sv, pd;
  uint64_t w0;
  float xmargin;
  // in (uniform)
  uint64_t rs, key;
  unsigned long long ctr0;
  double beta;
  bool beta_inf;
  float nbeta_f, fscale;
  // out
  unsigned flips;
  int draws, adv;
  bool have_exact;
  double dE;
  long long idE;
};

template <int FL, bool REPLAY, bool INT>
__device__ __noinline__ void general_round(const DevModel& m, const uint8_t* z, const double* s_ln0,
                                           const float* s_scr0, const unsigned long long* s_jA,
                                           const unsigned long long* s_jC, RoundIo& io)
{
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const bool active = io.active;
  const int v = io.v, cursor = io.cursor, bnd = io.bnd, g = io.g;
  const uint32_t nb = io.nb, sv = io.sv;
  const double beta = io.beta;
  const bool beta_inf = io.beta_inf;
  const float nbeta_f = io.nbeta_f, fscale = io.fscale;
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
    if (need)
    {
      dE = exact_dE<FL>(m, v, sv, z);
      have_exact = true;
      uphill = !le_zero(dE);
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
  auto decide = [&](uint32_t rr, int row) -> int {
    if (beta_inf) return 0;
    const float* sc = scr_base(s_scr0, row);
    if (INT) return screen(sc, rr, row, __fmul_rn((float)idE, nbeta_f), 0.f);
    if (have_exact) return screen(sc, rr, row, __fmul_rn(approx_float(dE), nbeta_f), 0.f);
    return screen(sc, rr, row, __fmul_rn((float)F, fscale), io.xmargin);
  };
  uint32_t dr = 0;
  int drow = 0;
  bool redraw = false;
  int dec = 1;
  if (REPLAY)
  {
    const uint32_t d0 = __shfl_sync(kFull, io.pd, pos & 31);
    if (uphill)
    {
      dr = d0;
      redraw = (dr & 255u) == 0;
      if (!redraw) dec = decide(dr, 0);
    }
  }
  else if (uphill)
  {
    const uint32_t cur0 = io.pd;
    if ((cur0 & 255u) != 0u)
    {
      dr = cur0;
      dec = decide(cur0, 0);
    }
    else
    {
      bool all_zero;
      dr = counter_redraw(io.key, io.ctr0 + (unsigned long long)v, io.w0, &drow, &all_zero);
      dec = all_zero ? 1 : decide(dr, drow);
    }
  }
  const unsigned Rm = REPLAY ? __ballot_sync(kFull, redraw) : 0u;
  if (!INT && __any_sync(kFull, uphill && !redraw && dec < 0))
  {
    // exact differences for the lanes inside the margin that can still be
    // committed: up to the first stop under the surely accepted lanes (more
    // acceptances can only move the stop earlier)
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
      dE = exact_dE<FL>(m, v, sv, z);
      have_exact = true;
    }
    if (lane > fs && dec < 0) dec = 0;  // not committed this round
  }
  if (uphill && !redraw && dec < 0)
    dec = exact_less(ln_base(s_ln0, drow), dr, drow, INT ? (double)idE : dE, beta) ? 1 : 0;
  if (uphill && !redraw) acc = dec == 1;
  const unsigned A = __ballot_sync(kFull, acc);
  bool conf = false;
  if (active && lane > cursor)
    conf = (nb & (__brev(A) >> (32 - lane)) & ((1u << (lane - cursor)) - 1u)) != 0u;
  const unsigned Cm = __ballot_sync(kFull, conf);
  const unsigned stop = Cm | Rm;
  int f = stop ? (__ffs(stop) - 1) : 32;
  if (f > io.nvalid) f = io.nvalid;
  const bool slow = REPLAY && f < io.nvalid && ((Rm >> f) & 1u) && !((Cm >> f) & 1u);
  const unsigned commit = ((f >= 32) ? kFull : ((1u << f) - 1u)) & ~((1u << cursor) - 1u);
  unsigned flips = A & commit;
  int draws = REPLAY ? __popc(U & commit) : 0;
  if (REPLAY && slow)
  {
    // lane f drew a zero bucket: its redraw chain (markov/metropolis.h:93-103)
    if (!INT && lane == f && !have_exact)
    {
      dE = exact_dE<FL>(m, v, sv, z);
      have_exact = true;
    }
    int sacc = 0, used = 0;
    if (lane == f)
      sacc = redraw_chain(s_jA, s_jC, io.rs, pos, s_ln0, beta_inf, INT ? (double)idE : dE, beta, &used);
    sacc = __shfl_sync(kFull, sacc, f);
    used = __shfl_sync(kFull, used, f);
    if (sacc) flips |= 1u << f;
    draws += used;
  }
  io.flips = flips;
  io.draws = draws;
  io.adv = f + (slow ? 1 : 0) - cursor;
  io.have_exact = have_exact;
  io.dE = dE;
  io.idE = idE;
}

// ---------------------------------------------------------------------------
// The decider: one walker's sweeps.  Returns false when a wait gave up.
// Committed flips are logged at head + i and published to the accountant at
// the end of each 32-variable block (a block logs at most 32 flips; the log
// is checked for room for them when the block starts).
//
// A window round, common path: every lane turns the draw at stream position
// `lane` into the screen interval [lo, hi] of the ln-table value; each
// uphill lane takes the interval of its position (the uphill lanes before it)
// and compares it with its threshold field * fscale +- margin.  Inside the
// margin, the exact FP64 difference and comparison are taken (rare).  Flips
// are applied in lane segments of 8, 16 or 32 per flip.
// ---------------------------------------------------------------------------
template <int FL, bool REPLAY, bool INT>
__device__ __forceinline__ bool decide_sweeps(const SweepArgs& a, const Region R, const double* s_ln0, const float* s_scr0,
                              const unsigned long long* s_jA, const unsigned long long* s_jC, int r,
                              unsigned& phases, uint64_t& rs, unsigned long long& natt,
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
  // per-lane row data of the next block (prefetched a block ahead)
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
  // lane 0: record range of the tile in flight (tq) and of the next one (nq),
  // loaded a block ahead of its copy
  int tq0 = 0, tq1 = 0, nq0 = 0, nq1 = 0;
  auto range_of = [&](int blk, int& q0, int& q1) {
    q0 = __ldg(m.row + (blk << 5));
    q1 = __ldg(m.row + min((blk << 5) + 32, N));
  };
  if (total > 0 && lane == 0)
  {
    range_of(0, tq0, tq1);
    tile_issue(R.tiles, m.fc_rec + tq0, min(tq1 - tq0, kCap), &R.bars[0]);
    if (total > 1) range_of(nblocks > 1 ? 1 : 0, nq0, nq1);
  }
  double beta = 0.0;
  bool beta_inf = false;
  float nbeta_f = 0.f, fscale = 0.f, fsa = 0.f;
  unsigned long long ctr0 = 0;
  // the sweep's beta, loaded a block ahead of its first use
  const double* betas = a.beta + (long long)r * a.bs_w;
  double beta_next = total > 0 ? betas[a.sweep_base * a.bs_s] : 0.0;
  int k = 0, bi = 0;                              // sweep and block of gb
  int bi2 = nblocks > 2 ? 2 : (nblocks == 2 ? 0 : 0);  // block of gb + 2
  for (int gb = 0; gb < total; gb++, bi++)
  {
    if (bi == nblocks)
    {
      bi = 0;
      k++;
    }
    const int buf = gb & 1;
    if (bi == 0)
    {
      const long long swp = a.sweep_base + k;
      beta = beta_next;
      beta_inf = ((unsigned long long)__double_as_longlong(beta) & 0x7FFFFFFFFFFFFFFFULL) ==
                 0x7FF0000000000000ULL;
      nbeta_f = -approx_float(beta);
      // thr = field * fscale approximates dE * (-beta)
      fscale = INT ? 0.f : (float)(beta * m.fc_inv * (FL == F_PARITY ? 2.0 : -1.0));
      fsa = fabsf(fscale) * 1.0001f;
      ctr0 = (unsigned long long)swp * (unsigned long long)N;
    }
    if (bi == nblocks - 1 && gb + 1 < total) beta_next = betas[(a.sweep_base + k + 1) * a.bs_s];
    const int i0 = bi << 5;
    // this block's record range, then the next block's tile into the other buffer
    const int b_q0 = __shfl_sync(kFull, tq0, 0);
    const int b_q1 = __shfl_sync(kFull, tq1, 0);
    if (gb + 1 < total && lane == 0)
    {
      tq0 = nq0;
      tq1 = nq1;
      tile_issue(R.tiles + (buf ^ 1) * kCap, m.fc_rec + tq0, min(tq1 - tq0, kCap), &R.bars[buf ^ 1]);
      if (gb + 2 < total) range_of(bi2, nq0, nq1);
    }
    bi2 = (bi2 + 1 == nblocks) ? 0 : bi2 + 1;
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
    const bool tile_ok = mbar_wait(&R.bars[buf], (phases >> buf) & 1u);
    phases ^= 1u << buf;
    if (!__all_sync(kFull, ok && tile_ok))
    {
      if (lane == 0)
      {
        if (!tile_ok) raise_abort(R, a.err);
        // the copy in flight lands before the walker's region is given up
        if (gb + 1 < total)
        {
          mbar_wait(&R.bars[buf ^ 1], (phases >> (buf ^ 1)) & 1u);
          phases ^= 1u << (buf ^ 1);
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
    const float xmargin = INT ? 0.f : fsa * (float)(bnd + 1);
    const unsigned head0 = head;
    unsigned b_att = 0, b_acc = 0, b_win = 0;

    // the draws of the first round (replay: stream positions 0..31)
    uint32_t pd = 0;
    uint64_t w0 = 0;
    float plo = 0.f, phi = 0.f;
    unsigned Zm = 0;
    auto draws_for = [&](int cur) {
      if (REPLAY) pd = pcg_out(s_jA[lane] * rs + s_jC[lane]);
      else
      {
        w0 = counter_draw(key, 2ULL * (ctr0 + (unsigned long long)(i0 + lane)));
        pd = (uint32_t)w0;
      }
      const int pb = (int)(pd & 255u);
      const float* e = s_scr0 + pb * 3;
      const float val = __fmaf_rn(__fmul_rn((float)(pd >> 8), 5.96046483e-08f), e[1], e[0]);
      plo = pb == 1 ? INFINITY : __fsub_rn(val, e[2]);
      phi = pb == 1 ? INFINITY : __fadd_rn(val, e[2]);
      Zm = __ballot_sync(kFull, pb == 0);
      (void)cur;
    };
    if (!REPLAY) draws_for(0);  // counter draws: fixed for the block

    int cursor = 0;
    while (cursor < nvalid)
    {
      if (REPLAY) draws_for(0);
      const bool active = valid && lane >= cursor;
      const unsigned before = lt & ~((1u << cursor) - 1u);
      const int g = active ? R.G[v] : 0;
      // ---- fast path: the field's sign and the screened comparison
      bool up, rare;
      float thr, xm;
      if (INT)
      {
        const long long idE = (FL == F_PARITY) ? -2LL * (long long)g : (long long)g;
        up = active && idE > 0;
        thr = __fmul_rn((float)idE, nbeta_f);
        xm = 0.f;
        rare = false;
      }
      else if (FL == F_PARITY)
      {
        up = active && g < -bnd;
        rare = active && g <= bnd && g >= -bnd;
        thr = __fmul_rn((float)g, fscale);
        xm = xmargin;
      }
      else
      {
        const int F = g >> 8;
        const bool zero = (g & 255) == 0;  // nothing contributes: +0.0
        up = active && !zero && F > bnd;
        rare = active && !zero && F <= bnd && F >= -bnd;
        thr = __fmul_rn((float)F, fscale);
        xm = xmargin;
      }
      unsigned U = 0;
      float lo = plo, hi = phi;
      bool rd = false;
      if (REPLAY)
      {
        U = __ballot_sync(kFull, up);
        const int pos = __popc(U & before);
        lo = __shfl_sync(kFull, plo, pos);
        hi = __shfl_sync(kFull, phi, pos);
        rd = up && ((Zm >> pos) & 1u);
      }
      else
        rare = rare || (up && (pd & 255u) == 0u);
      const float et = __fmaf_rn(fabsf(thr), 1.9073486328125e-06f, 1e-30f) + xm;  // 2^-19
      const bool acc_u = up && !rd && !beta_inf && hi < __fsub_rn(thr, et);
      const bool rej_u = up && !rd && (beta_inf || lo > __fadd_rn(thr, et));
      rare = rare || (up && !rd && !acc_u && !rej_u);
      const unsigned A = __ballot_sync(kFull, active && (!up || acc_u));
      const unsigned Rm = __ballot_sync(kFull, rd);
      bool conf = false;
      if (active && lane > cursor)
        conf = (nb & (__brev(A) >> (32 - lane)) & ((1u << (lane - cursor)) - 1u)) != 0u;
      const unsigned Cm = __ballot_sync(kFull, conf);
      const unsigned stop = Cm | Rm;
      int f = stop ? (__ffs(stop) - 1) : 32;
      if (f > nvalid) f = nvalid;
      const unsigned commit = ((f >= 32) ? kFull : ((1u << f) - 1u)) & ~((1u << cursor) - 1u);
      unsigned flips = A & commit;
      int draws = REPLAY ? __popc(U & commit) : 0;
      int adv = f - cursor;
      bool have_exact = false;
      double dE = 0.0;
      long long idE = (FL == F_PARITY) ? -2LL * (long long)g : (long long)g;
      if (!INT && FL == F_COUNTER && active && (g & 255) == 0) have_exact = true;  // dE = +0.0
      // the general round: a field inside its margin, a comparison inside
      // the screen's margin, a counter redraw, or a replayed zero bucket at
      // the stop
      const bool slow = REPLAY && f < nvalid && ((Rm >> f) & 1u) && !((Cm >> f) & 1u);
      const bool any_rare = __any_sync(kFull, rare);
      if (!any_rare && slow)
      {
        // lane f drew a zero bucket: its redraw chain (markov/metropolis.h:93-103)
        int sacc = 0, used = 0;
        if (lane == f)
        {
          double d = 0.0;
          if (!INT) d = exact_dE<FL>(m, v, sv, R.z);
          const int pos = __popc(U & before);
          sacc = redraw_chain(s_jA, s_jC, rs, pos, s_ln0, beta_inf, INT ? (double)idE : d, beta, &used);
          have_exact = !INT;
          dE = d;
        }
        sacc = __shfl_sync(kFull, sacc, f);
        used = __shfl_sync(kFull, used, f);
        if (sacc) flips |= 1u << f;
        draws += used;
        adv += 1;
      }
      if (any_rare)
      {
        RoundIo io;
        io.active = active;
        io.v = v;
        io.cursor = cursor;
        io.nvalid = nvalid;
        io.bnd = bnd;
        io.g = g;
        io.nb = nb;
        io.sv = sv;
        io.pd = pd;
        io.w0 = w0;
        io.xmargin = xmargin;
        io.rs = rs;
        io.key = key;
        io.ctr0 = ctr0;
        io.beta = beta;
        io.beta_inf = beta_inf;
        io.nbeta_f = nbeta_f;
        io.fscale = fscale;
        general_round<FL, REPLAY, INT>(m, R.z, s_ln0, s_scr0, s_jA, s_jC, io);
        flips = io.flips;
        draws = io.draws;
        adv = io.adv;
        have_exact = io.have_exact;
        dE = io.dE;
        idE = io.idE;
      }
      const bool mine = ((flips >> lane) & 1u) != 0u;
      const int nfl = __popc(flips);
      // the next round's draws, ahead of the apply (independent of it)
      if (REPLAY) rs = s_jA[draws] * rs + s_jC[draws];

      if (nfl)
      {
        // a wide row keeps no masks: its exact difference is taken now,
        // before the flips change the term states
        const bool wide = mine && deg > 32;
        if (!INT && __any_sync(kFull, wide && !have_exact))
          if (wide && !have_exact)
          {
            dE = exact_dE<FL>(m, v, sv, R.z);
            have_exact = true;
          }
        const int fi = __popc(flips & lt);  // this flip's index among the round's
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
        const int maxdeg = (int)__reduce_max_sync(kFull, (unsigned)(mine ? deg : 0));
        if (maxdeg <= 32)
        {
          // segments of sg lanes, one flip each, pp flips per pass
          const int lsg = maxdeg <= 8 ? 3 : (maxdeg <= 16 ? 4 : 5);
          const int sg = 1 << lsg;
          const int pp = 32 >> lsg;
          const int grp = lane >> lsg;
          const int kk = lane & (sg - 1);
          unsigned qm = 0, sm = 0;
          unsigned fw = flips;  // flips not yet applied
          for (int p0 = 0; p0 < nfl; p0 += pp)
          {
            // the lanes of the pass's first pp flips: successive lowest bits
            const int q0 = __ffs(fw) - 1;
            const unsigned f1 = fw & (fw - 1);
            const int q1 = f1 ? __ffs(f1) - 1 : q0;
            const unsigned f2 = f1 & (f1 - 1);
            const int q2 = f2 ? __ffs(f2) - 1 : q0;
            const unsigned f3 = f2 & (f2 - 1);
            const int q3 = f3 ? __ffs(f3) - 1 : q0;
            const int j = grp == 0 ? q0 : (grp == 1 ? q1 : (grp == 2 ? q2 : q3));
            const bool live = p0 + grp < nfl;
            fw = (pp == 1) ? f1 : ((pp == 2) ? f2 : (f3 & (f3 - 1)));
            const int dj = __shfl_sync(kFull, deg, j);
            const int rbj = __shfl_sync(kFull, rb, j);
            const uint32_t svj = __shfl_sync(kFull, sv, j);
            unsigned bits = 0;
            const bool act = live && kk < dj;
            uint4 rec = make_uint4(0u, 0u, 0u, 0u);
            if (act)
            {
              rec = staged ? tile[rbj - b_q0 + kk] : __ldg(m.fc_rec + rbj + kk);
              bits = apply_incidence<FL>(m, R, rec, svj, i0 + j, pack);
            }
            if (__any_sync(kFull, bits & 4u))
              apply_overflow_lane<FL>(m, R, (bits & 4u) != 0u, rec, bits, i0 + j, pack);
            if (!INT)
            {
              const unsigned Bq = __ballot_sync(kFull, bits & 1u);
              const unsigned Bs = __ballot_sync(kFull, (bits >> 1) & 1u);
              if (mine && fi >= p0 && fi < p0 + pp)
              {
                const int sh = (fi - p0) << lsg;
                const unsigned w = (sg == 32) ? kFull : ((1u << sg) - 1u);
                qm = (Bq >> sh) & w;
                sm = (Bs >> sh) & w;
              }
            }
          }
          if (mine && !INT && !have_exact)
          {
            ent.y = (FL == F_PARITY) ? 0u : qm;
            ent.z = sm;
          }
        }
        else
        {
          // a wide flip among them (rare): one flip at a time
          unsigned fl = flips;
          while (fl)
          {
            const int j = __ffs(fl) - 1;
            fl &= fl - 1;
            const int dj = __shfl_sync(kFull, deg, j);
            const int rbj = __shfl_sync(kFull, rb, j);
            const uint32_t svj = __shfl_sync(kFull, sv, j);
            unsigned bits = 0;
            if (dj <= 32)
            {
              uint4 rec = make_uint4(0u, 0u, 0u, 0u);
              if (lane < dj)
              {
                rec = staged ? tile[rbj - b_q0 + lane] : __ldg(m.fc_rec + rbj + lane);
                bits = apply_incidence<FL>(m, R, rec, svj, i0 + j, pack);
              }
              if (__any_sync(kFull, bits & 4u))
                apply_overflow_lane<FL>(m, R, (bits & 4u) != 0u, rec, bits, i0 + j, pack);
            }
            else
              apply_wide<FL>(m, R, tile, staged, b_q0, rbj, dj, svj, i0 + j, pack);
            if (!INT)
            {
              const unsigned Bq = __ballot_sync(kFull, bits & 1u);
              const unsigned Bs = __ballot_sync(kFull, (bits >> 1) & 1u);
              if (lane == j && !have_exact)
              {
                ent.y = (FL == F_PARITY) ? 0u : Bq;
                ent.z = Bs;
              }
            }
          }
        }
        __syncwarp();
        if (mine)
        {
          R.log[(head + (unsigned)fi) & (unsigned)(kLog - 1)] = ent;
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
      b_att += (unsigned)adv;
      b_acc += (unsigned)nfl;
      b_win++;
      cursor += adv;
    }
    natt += b_att;
    nacc += b_acc;
    nwin += b_win;
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
__device__ __forceinline__ bool account(const SweepArgs& a, const Region R, double& cost, double& low, long long& icost,
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
  const int ws0 = blockIdx.x * wpc + ws;
  if (ws0 >= a.n_streams) return;
  const int w = a.order ? a.order[ws0] : ws0;
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
  unsigned phases = 0u;  // mbarrier phase bits of the two tile buffers, kept across walkers

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
      ok = decide_sweeps<FL, REPLAY, INT>(a, R, s_ln0, s_scr0, s_jA, s_jC, r, phases, rs, natt, nacc,
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
