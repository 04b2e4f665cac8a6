// lanes.cu -- lane-per-walker Metropolis sweeps for Ising models whose terms
// have one or two members (lattices, sparse graphs with fields).
//
// Each thread runs one walker's sweeps exactly as the reference's ordered
// sweep does (markov/walker.h:143-153,209-229): variable by variable, the
// cost difference summed over the incident terms in ascending term order
// (model/ising.h:108-117), the Metropolis decision (markov/metropolis.h:
// 64-104) on the walker's own stream, the flip, cost += diff and the lowest
// check.  The G walkers of a warp (G <= 32 lanes; fewer when a group's
// spins would not fit in shared memory otherwise) form a group whose spins
// are stored bit-packed and interleaved: word w (spins 32w .. 32w+31) of
// lane l at group word w*G + l, so the warp's accesses to one word index are
// one line, and the row loads of a model are shared by the lanes that run
// it.
//
// Term parity from spins: with at most two members, the cached term bit of
// IsingTermCached is the XOR of the variable's own spin and the other
// member's spin (or the own spin alone), so the state is the spins alone
// and a flip is one word update.
//
// Lowest state: the reference copies the spins whenever the cost drops below
// the lowest (markov/walker.h:269-280).  Here a new lowest only records that
// the current state is the lowest; later flips are logged, and the lowest
// spins are written out (current words with the logged flips undone) when
// the log fills or the launch ends -- the same state, fewer copies.  The
// Metropolis tables are read through L1 from global memory: lanes look up
// different buckets, which constant memory would serialise.
#include <algorithm>

#include "metropolis.cuh"
#include "qio_internal.h"

namespace qio
{
namespace lw
{
using namespace qio::mc;
static const unsigned long long kMult = 6364136223846793005ULL;
static const unsigned long long kInc = 1442695040888963407ULL;

__device__ double g_ln[1024];
__device__ float g_scr[1024 * 3];

// Metropolis decision for an uphill move with threshold dE * (-beta):
// FP32 screen first, the exact FP64 expression inside its margin.
__device__ __forceinline__ bool lut_accept(const double* ln, const float* scr, uint32_t r, int row,
                                           double dE, double beta, float nbeta_f)
{
  const float thr_f = __fmul_rn(approx_float(dE), nbeta_f);
  const int d = lut_screen(scr, r, row, thr_f);
  if (d >= 0) return d == 1;
  return lut_less_exact(ln, r, row, __dmul_rn(dE, -beta));
}

// SMEM: the group's current spin words live in shared memory for the launch
// (copied in at the start, out at the end); the lowest words stay in global
// memory.  Tables in the block's first 20 KB, group words after them.
// per incidence record: (other member or the padding spin, coefficient), as
// int2, packed into 32 bits (other << 8 | 8-bit coefficient) when every
// coefficient fits, or as double2 (other's bits in x) for FP64 models
enum RecKind
{
  RK_INT2 = 0,
  RK_PACK = 1,
  RK_F64 = 2
};
template <int RK>
struct Rec;
template <>
struct Rec<RK_INT2>
{
  using T = int2;
  static __device__ __forceinline__ int other(const T& r) { return r.x; }
  static __device__ __forceinline__ int icoef(const T& r) { return r.y; }
  static __device__ __forceinline__ double dcoef(const T& r) { return (double)r.y; }
};
template <>
struct Rec<RK_PACK>
{
  using T = unsigned int;
  static __device__ __forceinline__ int other(const T& r) { return (int)(r >> 8); }
  static __device__ __forceinline__ int icoef(const T& r) { return (int)(signed char)(r & 0xFFu); }
  static __device__ __forceinline__ double dcoef(const T& r) { return (double)icoef(r); }
};
template <>
struct Rec<RK_F64>
{
  using T = double2;
  static __device__ __forceinline__ int other(const T& r) { return (int)__double_as_longlong(r.x); }
  static __device__ __forceinline__ int icoef(const T&) { return 0; }
  static __device__ __forceinline__ double dcoef(const T& r) { return r.y; }
};
// KPRE: records of the next variable loaded one attempt ahead (4, 6 or 8,
// at least the largest row when it is that small)
template <bool REPLAY, int RK, bool SMEM, int KPRE>
__global__ void __launch_bounds__(128) lw_sweep_kernel(LwArgs a)
{
  constexpr int kPre = KPRE;
  constexpr bool INT = RK != RK_F64;
  using R = typename Rec<RK>::T;
  extern __shared__ __align__(16) unsigned char lw_smem[];
  const double* s_ln = g_ln;
  const float* s_scr = g_scr;
  const int G = a.G;
  const int lane = threadIdx.x & 31;
  const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int r = g * G + lane;
  if (lane >= G || r >= a.n_walkers) return;  // no warp-wide operations below
  const int smem_words = a.smem_words;
  const DevModel* md = a.models + (a.model_of ? a.model_of[r] : 0);
  const int* __restrict__ row = md->row;
  const R* __restrict__ rec = RK == RK_PACK ? (const R*)md->rec_p
                              : (RK == RK_INT2 ? (const R*)md->rec_i : (const R*)md->rec_f);
  const int Sz = md->sweep_size;
  const int nwd = (md->n_vars + 31) >> 5;  // word nwd is the padding spin word (0)
  const int gw = a.g_nw[g];
  uint32_t* base = (uint32_t*)(a.arena + a.g_off[g]);
  uint32_t* gsp = base + lane;              // word w at gsp[w * G]
  uint32_t* lsp = base + (size_t)gw * G + lane;
  uint32_t* lg = base + (size_t)gw * 2 * G + lane;
  uint32_t* sp = gsp;
  if (SMEM)
  {
    sp = (uint32_t*)lw_smem + (size_t)(threadIdx.x >> 5) * smem_words * G + lane;
    for (int w = 0; w < nwd; w++) sp[(size_t)w * G] = gsp[(size_t)w * G];
  }
  sp[(size_t)nwd * G] = 0u;

  const int slot = a.slot_of ? a.slot_of[r] : r;
  double cost = a.p.cost[slot], low = a.p.lowest[r];
  long long icost = INT ? (long long)cost : 0, ilow = INT ? (long long)low : 0;
  long long klow = order_key(low);
  uint64_t rs = REPLAY ? a.rng[r] : 0;
  uint64_t key = 0;
  if (!REPLAY)
  {
    const long long lr = a.local_of ? a.local_of[r] : r;
    key = counter_key(a.seed + (uint32_t)(lr / a.key_div), a.key_base + (unsigned long long)(lr % a.key_div));
  }
  unsigned long long natt = 0, nacc = 0;
  bool pend = false;  // the lowest is the current state with the logged flips undone
  int nlog = 0;
  auto write_lowest = [&]() {
    for (int w = 0; w < nwd; w++) lsp[(size_t)w * G] = sp[(size_t)w * G];
    for (int i = 0; i < nlog; i++)
    {
      const uint32_t v = lg[(size_t)i * G];
      lsp[(size_t)(v >> 5) * G] ^= 1u << (v & 31);
    }
    pend = false;
    nlog = 0;
  };
  auto spin = [&](int u) -> uint32_t { return (sp[(size_t)(u >> 5) * G] >> (u & 31)) & 1u; };

  for (int k = 0; k < a.n_sweeps; k++)
  {
    const long long swp = a.sweep_base + k;
    const double beta = a.beta[(long long)r * a.bs_w + swp * a.bs_s];
    const bool beta_inf =
        ((unsigned long long)__double_as_longlong(beta) & 0x7FFFFFFFFFFFFFFFULL) == 0x7FF0000000000000ULL;
    const float nbeta_f = -approx_float(beta);
    const unsigned long long ctr0 = (unsigned long long)swp * (unsigned long long)Sz;
    natt += (unsigned long long)Sz;
    // records two attempts ahead and row offsets three ahead: no attempt
    // waits on a dependent pair of L2 loads (row offset, then records)
    const int nrow = md->n_vars;  // row has nrow + 1 entries
    int qb = __ldg(row), qe = __ldg(row + 1);
    int qe1 = (Sz > 1) ? __ldg(row + min(2, nrow)) : qe;
    int qe2 = (Sz > 2) ? __ldg(row + min(3, nrow)) : qe1;
    R cur[kPre], nx1[kPre];
#pragma unroll
    for (int j = 0; j < kPre; j++)
    {
      if (qb + j < qe) cur[j] = __ldg(rec + qb + j);
      if (qe + j < qe1) nx1[j] = __ldg(rec + qe + j);
    }
    uint32_t cw = 0;  // current word of v
    for (int v = 0; v < Sz; v++)
    {
      // variable v + 2's records and v + 4's row end
      const int qe3 = (v + 3 < Sz) ? __ldg(row + min(v + 4, nrow)) : qe2;
      R nx2[kPre];
#pragma unroll
      for (int j = 0; j < kPre; j++)
        if (qe1 + j < qe2) nx2[j] = __ldg(rec + qe1 + j);
      if ((v & 31) == 0) cw = sp[(size_t)(v >> 5) * G];
      const uint32_t sv = (cw >> (v & 31)) & 1u;
      long long idE = 0;
      double dE = 0.0;
      {
        int iacc = 0;
        double diff = 0.0;
#pragma unroll
        for (int j = 0; j < kPre; j++)
          if (qb + j < qe)
          {
            const uint32_t z = sv ^ spin(Rec<RK>::other(cur[j]));
            if (INT)
            {
              const int c = Rec<RK>::icoef(cur[j]);
              iacc += z ? -c : c;
            }
            else
            {
              const double c = Rec<RK>::dcoef(cur[j]);
              diff = __dadd_rn(diff, z ? -c : c);
            }
          }
        for (int q = qb + kPre; q < qe; q++)
        {
          const R rq = __ldg(rec + q);
          const uint32_t z = sv ^ spin(Rec<RK>::other(rq));
          if (INT)
          {
            const int c = Rec<RK>::icoef(rq);
            iacc += z ? -c : c;
          }
          else
          {
            const double c = Rec<RK>::dcoef(rq);
            diff = __dadd_rn(diff, z ? -c : c);
          }
        }
        if (INT) idE = -2LL * (long long)iacc;
        else dE = neg2x(diff);
      }
#pragma unroll
      for (int j = 0; j < kPre; j++)
      {
        cur[j] = nx1[j];
        nx1[j] = nx2[j];
      }
      qb = qe;
      qe = qe1;
      qe1 = qe2;
      qe2 = qe3;
      bool acc;
      if (INT ? idE <= 0 : le_zero(dE)) acc = true;
      else
      {
        int rw = -1, b = 0;
        uint32_t cur = 0;
        bool all_zero = false;
        if (REPLAY)
        {
          while (b == 0)
          {
            if (rw < 3)
            {
              cur = pcg_out(rs);
              rs = rs * kMult + kInc;
              b = (int)(cur & 255u);
              rw++;
            }
            else
            {
              all_zero = true;
              break;
            }
          }
        }
        else
        {
          const unsigned long long ctr = ctr0 + (unsigned long long)v;
          const uint64_t w0 = counter_draw(key, 2ULL * ctr);
          int used = 0;
          while (b == 0)
          {
            if (rw < 3)
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
              rw++;
            }
            else
            {
              all_zero = true;
              break;
            }
          }
        }
        if (all_zero) acc = true;
        else if (beta_inf) acc = false;
        else if (INT)
        {
          // integer difference: its float is exact below 2^24, within the
          // screen's 2^-19 margin above
          const int d = lut_screen(s_scr, cur, rw, __fmul_rn((float)idE, nbeta_f));
          acc = d >= 0 ? d == 1 : lut_less_exact(s_ln, cur, rw, __dmul_rn((double)idE, -beta));
        }
        else acc = lut_accept(s_ln, s_scr, cur, rw, dE, beta, nbeta_f);
      }
      if (acc)
      {
        nacc++;
        cw ^= 1u << (v & 31);
        sp[(size_t)(v >> 5) * G] = cw;
        bool newlow;
        if (INT)
        {
          icost += idE;
          newlow = icost < ilow;
          if (newlow) ilow = icost;
        }
        else
        {
          cost = __dadd_rn(cost, dE);
          const long long kc = order_key(cost);
          newlow = kc < klow;
          if (newlow)
          {
            klow = kc;
            low = cost;
          }
        }
        if (newlow)
        {
          pend = true;
          nlog = 0;
        }
        else if (pend)
        {
          if (nlog == kLwLog)
          {
            // the log is full: write the lowest out, this flip excluded
            write_lowest();
            lsp[(size_t)(v >> 5) * G] ^= 1u << (v & 31);
          }
          else
          {
            lg[(size_t)nlog * G] = (uint32_t)v;
            nlog++;
          }
        }
      }
    }
  }
  if (pend) write_lowest();
  if (SMEM)
    for (int w = 0; w < nwd; w++) gsp[(size_t)w * G] = sp[(size_t)w * G];
  a.p.cost[slot] = INT ? (double)icost : cost;
  a.p.lowest[r] = INT ? (double)ilow : low;
  a.p.attempts[r] += natt;
  a.p.accepts[r] += nacc;
  a.p.step_att[r] += natt;
  a.p.step_acc[r] += nacc;
  if (a.p.windows) a.p.windows[r] += natt;
  if (REPLAY) a.rng[r] = rs;
}

// Population (bit-packed spins per slot, lowest spins per walker) <-> group
// words.  Thread (g, lane) of block (g, word block) moves words of walker
// g*G + lane; a warp's accesses to one word index are one line.
template <bool LOAD>
__global__ void lw_move_kernel(LwArgs a, int words_per_block)
{
  const int G = a.G;
  const int g = blockIdx.x, lane = threadIdx.x;
  const int r = g * G + lane;
  if (lane >= G || r >= a.n_walkers) return;
  const DevModel* md = a.models + (a.model_of ? a.model_of[r] : 0);
  const int nwd = (md->n_vars + 31) >> 5;
  const int slot = a.slot_of ? a.slot_of[r] : r;
  const int gw = a.g_nw[g];
  uint32_t* base = (uint32_t*)(a.arena + a.g_off[g]);
  const int q0 = blockIdx.y * words_per_block, q1 = min(nwd, q0 + words_per_block);
  for (int q = q0; q < q1; q++)
  {
    uint32_t* sp = base + (size_t)q * G + lane;
    uint32_t* lsp = base + (size_t)(gw + q) * G + lane;
    uint32_t* ps = a.p.spins + (size_t)slot * a.p.nw + q;
    uint32_t* pl = a.p.lspins + (size_t)r * a.p.nw + q;
    if (LOAD)
    {
      *sp = *ps;
      *lsp = *pl;
    }
    else
    {
      *ps = *sp;
      *pl = *lsp;
    }
  }
}

// term parity bytes of the population from its spins (IsingTermCachedState),
// one thread per (walker, term) pair, grid-stride
__global__ void lw_terms_kernel(LwArgs a, int max_terms)
{
  const long long total = (long long)a.n_walkers * max_terms;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x)
  {
    const int r = (int)(i / max_terms);
    const int t = (int)(i - (long long)r * max_terms);
    const DevModel* md = a.models + (a.model_of ? a.model_of[r] : 0);
    if (t >= md->n_terms) continue;
    const int slot = a.slot_of ? a.slot_of[r] : r;
    const uint32_t* s = a.p.spins + (size_t)slot * a.p.nw;
    uint32_t par = 0;
    for (int k = md->trow[t]; k < md->trow[t + 1]; k++)
    {
      const uint32_t x = md->tvar[k] & ~kNegBit;
      par ^= (s[x >> 5] >> (x & 31)) & 1u;
    }
    a.p.tstate[(size_t)slot * a.p.mp + t] = (uint8_t)par;
  }
}
}  // namespace lw

void lw_upload(const double* ln, const float* scr)
{
  cudaMemcpyToSymbol(lw::g_ln, ln, 1024 * sizeof(double));
  cudaMemcpyToSymbol(lw::g_scr, scr, 3072 * sizeof(float));
}

template <bool R, int RK, bool SM, int KP>
static cudaError_t lw_go_k(const LwArgs& a, cudaStream_t s, int wpb)
{
  auto k = lw::lw_sweep_kernel<R, RK, SM, KP>;
  const int bytes = SM ? wpb * a.smem_words * a.G * 4 : 0;
  static int configured = 48 * 1024;
  if (bytes > configured)
  {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    configured = bytes;
  }
  const int groups = (a.n_walkers + a.G - 1) / a.G;
  const int blocks = (groups + wpb - 1) / wpb;
  if (blocks > 0) k<<<blocks, 32 * wpb, bytes, s>>>(a);
  return cudaGetLastError();
}

template <bool R, int RK, bool SM>
static cudaError_t lw_go(const LwArgs& a, cudaStream_t s, int wpb)
{
  if (a.unroll == 4) return lw_go_k<R, RK, SM, 4>(a, s, wpb);
  if (a.unroll == 6) return lw_go_k<R, RK, SM, 6>(a, s, wpb);
  return lw_go_k<R, RK, SM, 8>(a, s, wpb);
}

template <bool R, int RK>
static cudaError_t lw_go_sm(const LwArgs& a, cudaStream_t s, int wpb)
{
  return a.smem_words > 0 ? lw_go<R, RK, true>(a, s, wpb) : lw_go<R, RK, false>(a, s, wpb);
}

template <bool R>
static cudaError_t lw_go_rk(const LwArgs& a, cudaStream_t s, int wpb)
{
  if (!a.int_mode) return lw_go_sm<R, lw::RK_F64>(a, s, wpb);
  return a.packed ? lw_go_sm<R, lw::RK_PACK>(a, s, wpb) : lw_go_sm<R, lw::RK_INT2>(a, s, wpb);
}

// Warps per block: enough that the groups spread over the 152 SMs, as many
// as the groups' shared-memory words allow.
cudaError_t launch_lw_sweep(const LwArgs& a, int wpb, cudaStream_t s)
{
  if (a.G < 1 || a.G > 32) return cudaErrorInvalidValue;
  const int groups = (a.n_walkers + a.G - 1) / a.G;
  if (groups == 0) return cudaSuccess;
  if (wpb <= 0) wpb = std::max(1, std::min(4, (groups + 151) / 152));
  wpb = std::min(wpb, 4);
  if (a.smem_words > 0)
  {
    while (wpb > 1 && wpb * a.smem_words * a.G * 4 > kLwSmemBytes) wpb--;
    if (a.smem_words * a.G * 4 > kLwSmemBytes) return cudaErrorInvalidValue;
  }
  return a.replay ? lw_go_rk<true>(a, s, wpb) : lw_go_rk<false>(a, s, wpb);
}

static const int kMoveWords = 64;  // words per thread in the transposes

cudaError_t launch_lw_load(const LwArgs& a, int max_words, cudaStream_t s)
{
  const int groups = (a.n_walkers + a.G - 1) / a.G;
  if (groups == 0 || max_words == 0) return cudaSuccess;
  const int wb = (max_words + kMoveWords - 1) / kMoveWords;
  lw::lw_move_kernel<true><<<dim3(groups, wb), 32, 0, s>>>(a, kMoveWords);
  return cudaGetLastError();
}

cudaError_t launch_lw_store(const LwArgs& a, int max_words, int max_terms, cudaStream_t s)
{
  const int groups = (a.n_walkers + a.G - 1) / a.G;
  if (groups == 0 || max_words == 0) return cudaSuccess;
  const int wb = (max_words + kMoveWords - 1) / kMoveWords;
  lw::lw_move_kernel<false><<<dim3(groups, wb), 32, 0, s>>>(a, kMoveWords);
  if (max_terms > 0)
  {
    const long long total = (long long)a.n_walkers * max_terms;
    const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 64);
    lw::lw_terms_kernel<<<blocks, 256, 0, s>>>(a, max_terms);
  }
  return cudaGetLastError();
}
}  // namespace qio
