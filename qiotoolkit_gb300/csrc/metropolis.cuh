// metropolis.cuh -- device helpers shared by the sweep kernels: PCG32
// output, counter-based draws, IEEE bit tricks and the Metropolis ln-table
// comparison of markov/metropolis.h:64-104 (exact, and screened in FP32).
#pragma once
#include <cstdint>

namespace qio
{
namespace mc
{
static const unsigned long long kGamma = 0x9E3779B97F4A7C15ULL;

__device__ __forceinline__ uint32_t pcg_out(uint64_t old)
{
  uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  uint32_t rot = (uint32_t)(old >> 59u);
  return __funnelshift_r(xs, xs, rot);
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

// ---- IEEE bit helpers (integer pipe) ------------------------------------
// x <= 0 for a non-NaN double
__device__ __forceinline__ bool le_zero(double x)
{
  long long b = __double_as_longlong(x);
  if (b == 0) return true;
  unsigned long long mag = (unsigned long long)b & 0x7FFFFFFFFFFFFFFFULL;
  return b < 0 && mag <= 0x7FF0000000000000ULL;
}
// monotone integer key: key(a) < key(b) <=> a < b (non-NaN; -0 taken as +0)
__device__ __forceinline__ long long order_key(double x)
{
  long long b = __double_as_longlong(x);
  if (b == (long long)0x8000000000000000LL) b = 0;
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
// exact -2x (Ising: 2.0 * (-diff), model/ising.h:116) by exponent arithmetic
__device__ __forceinline__ double neg2x(double x)
{
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  unsigned long long mag = b & 0x7FFFFFFFFFFFFFFFULL;
  unsigned long long sgn = (b ^ 0x8000000000000000ULL) & 0x8000000000000000ULL;
  if (mag < 0x0010000000000000ULL) return __longlong_as_double((long long)(sgn | (mag << 1)));
  if (mag < 0x7FE0000000000000ULL)
    return __longlong_as_double((long long)(sgn | (mag + 0x0010000000000000ULL)));
  return __dmul_rn(2.0, -x);
}
// float approximation of a double from its bits, |rel err| < 2^-23
__device__ __forceinline__ float approx_float(double x)
{
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  unsigned s = (unsigned)(b >> 63) << 31;
  int e = (int)((b >> 52) & 0x7FF);
  if (e < 1023 - 126) return __int_as_float((int)s);
  if (e > 1023 + 127) return __int_as_float((int)(s | 0x7F800000u));
  unsigned m = (unsigned)((b >> 29) & 0x7FFFFFu);
  return __int_as_float((int)(s | ((unsigned)(e - 1023 + 127) << 23) | m));
}

// exact comparison of markov/metropolis.h:96-103 with the distance
// (r >> 8) / 16777214 correctly rounded via a corrected reciprocal
__device__ __forceinline__ bool lut_less_exact(const double* ln, uint32_t r, int row,
                                               double thr)
{
  int b = (int)(r & 255u);
  double y0 = ln[row * 256 + b - 1];
  double y1 = ln[row * 256 + b];
  const double x = (double)(r >> 8);
  const double inv = 5.9604648328104515e-08;  // RN(1 / 16777214)
  const double d0 = __dmul_rn(x, inv);
  const double dist = __fma_rn(__fma_rn(-d0, 16777214.0, x), inv, d0);
  double value = __dadd_rn(y0, __dmul_rn(dist, __dsub_rn(y1, y0)));
  return value < thr;
}

// value < thr decided in FP32 when the margin allows it.  thr = dE * (-beta)
// rounded to double; thr_f approximates it within 2^-21.7 |thr_f|; the margin
// used is 2^-19 |thr_f| (+1e-30).  The value side uses the per-bucket margin
// 2^-19 (|y0| + |dy|) against a bound of 2^-21.5 (|y0| + |dy|).
// Returns 1 accept, 0 reject, -1 undecided.
__device__ __forceinline__ int lut_screen(const float* scr, uint32_t r, int row, float thr_f)
{
  int b = (int)(r & 255u);
  if (b == 1) return 0;  // y0 = log(0): the value is NaN and never less
  int k = (row * 256 + b) * 3;
  float y0 = scr[k], dy = scr[k + 1], ev = scr[k + 2];
  float dist = __fmul_rn((float)(r >> 8), 5.96046483e-08f);
  float value = __fmaf_rn(dist, dy, y0);
  float et = __fmaf_rn(fabsf(thr_f), 1.9073486328125e-06f, 1e-30f);  // 2^-19
  if (__fadd_rn(value, ev) < __fsub_rn(thr_f, et)) return 1;
  if (__fsub_rn(value, ev) > __fadd_rn(thr_f, et)) return 0;
  return -1;
}
}  // namespace mc
}  // namespace qio
