// pa_device.cu -- device-side resampling step of population annealing
// (params "resampling": "multinomial", counter-based streams).
//
// The reference resamples on the host from its master stream (Poisson
// counts, or floor + residual selection; solver/population_annealing.h:
// 490-616).  This mode keeps the whole step on the device and is defined so
// that any implementation computes the same integers:
//   * shifted costs E_i - min(E), Boltzmann weights w_i = qexp(-dbeta *
//     (E_i - min E) * scale) in FP64 with the library's own exp (below:
//     only +, *, fma and exponent arithmetic, so it rounds the same on
//     every IEEE machine), converted to fixed point W_i = floor(w_i 2^40);
//   * an inclusive prefix sum of W in 64-bit integers (exact, any order);
//   * replica j of the next population takes parent p_j, the first i with
//     prefix_i > u_j, u_j = high 64 bits of draw_j * total, draw_j the
//     counter-based draw j of the step's resampling key;
//   * family census sum_f n_f^2 in integers; restart when R / rho < alpha
//     or every cost is equal.
// Replica copies are exact integer copies (pa_copy_kernel).
#include "metropolis.cuh"
#include "qio_internal.h"

namespace qio
{
namespace pad
{
using namespace qio::mc;

// exp(x), x <= 0: Cody-Waite reduction x = k ln2 + r (ln2 split into a
// 32-bit head and its tail, the classic fdlibm constants), |r| <= ln2/2,
// exp(r) by the degree-13 Taylor polynomial in Horner form with fused
// multiply-adds (truncation error below 5e-18), then 2^k by exponent bits.
__device__ __forceinline__ double qexp(double x)
{
  if (x < -745.2) return 0.0;
  const double k = rint(x * 1.4426950408889634);
  double r = fma(-k, 6.93147180369123816490e-01, x);
  r = fma(-k, 1.90821492927058770002e-10, r);
  double p = 1.0 / 6227020800.0;
  p = fma(p, r, 1.0 / 479001600.0);
  p = fma(p, r, 1.0 / 39916800.0);
  p = fma(p, r, 1.0 / 3628800.0);
  p = fma(p, r, 1.0 / 362880.0);
  p = fma(p, r, 1.0 / 40320.0);
  p = fma(p, r, 1.0 / 5040.0);
  p = fma(p, r, 1.0 / 720.0);
  p = fma(p, r, 1.0 / 120.0);
  p = fma(p, r, 1.0 / 24.0);
  p = fma(p, r, 1.0 / 6.0);
  p = fma(p, r, 0.5);
  p = fma(p, r, 1.0);
  p = fma(p, r, 1.0);
  int ki = (int)k;
  if (ki < -1020)
  {
    p *= 5.551115123125783e-17;  // 2^-54
    ki += 54;
  }
  return p * __longlong_as_double((long long)(ki + 1023) << 52);
}

// One block: cost min/max, the best lowest (smallest value, then smallest
// index), fixed-point weights and their inclusive prefix sum.
__global__ void __launch_bounds__(1024) pa_weights_kernel(const double* cost, const double* lowest, int R,
                                                        double dbeta_scale, unsigned long long* prefix,
                                                        PaScalars* out)
{
  __shared__ double s_min[32], s_max[32], s_low[32];
  __shared__ int s_idx[32];
  __shared__ unsigned long long s_sum[1024];
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nt = blockDim.x;
  const int chunk = (R + nt - 1) / nt;
  const int b = t * chunk, e = min(R, b + chunk);
  double mn = INFINITY, mx = -INFINITY, lo = INFINITY;
  int li = 0x7fffffff;
  for (int i = b; i < e; i++)
  {
    const double c = cost[i];
    mn = fmin(mn, c);
    mx = fmax(mx, c);
    const double l = lowest[i];
    if (l < lo)
    {
      lo = l;
      li = i;
    }
  }
  for (int d = 16; d; d >>= 1)
  {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, d));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, d));
    const double ol = __shfl_xor_sync(0xffffffffu, lo, d);
    const int oi = __shfl_xor_sync(0xffffffffu, li, d);
    if (ol < lo || (ol == lo && oi < li))
    {
      lo = ol;
      li = oi;
    }
  }
  if (lane == 0)
  {
    s_min[wid] = mn;
    s_max[wid] = mx;
    s_low[wid] = lo;
    s_idx[wid] = li;
  }
  __syncthreads();
  if (wid == 0)
  {
    const int nw = nt >> 5;
    mn = lane < nw ? s_min[lane] : INFINITY;
    mx = lane < nw ? s_max[lane] : -INFINITY;
    lo = lane < nw ? s_low[lane] : INFINITY;
    li = lane < nw ? s_idx[lane] : 0x7fffffff;
    for (int d = 16; d; d >>= 1)
    {
      mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, d));
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, d));
      const double ol = __shfl_xor_sync(0xffffffffu, lo, d);
      const int oi = __shfl_xor_sync(0xffffffffu, li, d);
      if (ol < lo || (ol == lo && oi < li))
      {
        lo = ol;
        li = oi;
      }
    }
    if (lane == 0)
    {
      s_min[0] = mn;
      s_max[0] = mx;
      s_low[0] = lo;
      s_idx[0] = li;
    }
  }
  __syncthreads();
  const double cmin = s_min[0];
  // weights of this thread's chunk, kept in the prefix array for now
  unsigned long long part = 0;
  for (int i = b; i < e; i++)
  {
    const double w = qexp(-dbeta_scale * (cost[i] - cmin));
    const unsigned long long W = (unsigned long long)(w * 1099511627776.0);  // 2^40
    part += W;
    prefix[i] = W;
  }
  s_sum[t] = part;
  __syncthreads();
  // inclusive scan of the per-thread sums (Hillis-Steele; integers: exact)
  for (int d = 1; d < nt; d <<= 1)
  {
    const unsigned long long v = t >= d ? s_sum[t - d] : 0ULL;
    __syncthreads();
    s_sum[t] += v;
    __syncthreads();
  }
  unsigned long long run = t ? s_sum[t - 1] : 0ULL;
  for (int i = b; i < e; i++)
  {
    run += prefix[i];
    prefix[i] = run;
  }
  if (t == nt - 1)
  {
    out->cmin = cmin;
    out->cmax = s_max[0];
    out->best_lowest = s_low[0];
    out->best_index = s_idx[0];
    out->total = s_sum[nt - 1];
  }
}

// parents of the next population and their families
__global__ void pa_parents_kernel(const unsigned long long* prefix, int R, int R_new, uint64_t key,
                                  const PaScalars* sc, const int* family, int* src, int* family_new)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= R_new) return;
  const unsigned long long total = sc->total;
  const unsigned long long u = __umul64hi(counter_draw(key, (unsigned long long)j), total);
  // first i with prefix[i] > u
  int lo = 0, hi = R - 1;
  while (lo < hi)
  {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] > u) hi = mid;
    else lo = mid + 1;
  }
  src[j] = lo;
  family_new[j] = family[lo];
}

__global__ void pa_census_count_kernel(const int* family, int R, unsigned int* counts)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < R) atomicAdd(&counts[family[j]], 1u);
}

__global__ void __launch_bounds__(1024) pa_census_sum_kernel(const unsigned int* counts, int n, PaScalars* out)
{
  __shared__ unsigned long long s[32];
  unsigned long long acc = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
  {
    const unsigned long long c = counts[i];
    acc += c * c;
  }
  for (int d = 16; d; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32)
  {
    acc = threadIdx.x < (blockDim.x >> 5) ? s[threadIdx.x] : 0ULL;
    for (int d = 16; d; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
    if (threadIdx.x == 0) out->census = acc;
  }
}

__global__ void pa_iota_kernel(int* a, int n)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) a[j] = j;
}

__global__ void pa_fill_kernel(double* a, int n, double v)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) a[j] = v;
}

__global__ void qexp_kernel(const double* x, double* y, int n)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) y[j] = qexp(x[j]);
}
}  // namespace pad

cudaError_t launch_pa_weights(const double* cost, const double* lowest, int R, double dbeta_scale,
                              unsigned long long* prefix, PaScalars* out, cudaStream_t s)
{
  pad::pa_weights_kernel<<<1, 1024, 0, s>>>(cost, lowest, R, dbeta_scale, prefix, out);
  return cudaGetLastError();
}

cudaError_t launch_pa_parents(const unsigned long long* prefix, int R, int R_new, uint64_t key,
                              const PaScalars* sc, const int* family, int* src, int* family_new,
                              cudaStream_t s)
{
  if (R_new > 0) pad::pa_parents_kernel<<<(R_new + 255) / 256, 256, 0, s>>>(prefix, R, R_new, key, sc, family, src, family_new);
  return cudaGetLastError();
}

cudaError_t launch_pa_census(const int* family, int R, unsigned int* counts, int n_families, PaScalars* out,
                             cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(counts, 0, (size_t)n_families * 4, s);
  if (e != cudaSuccess) return e;
  if (R > 0) pad::pa_census_count_kernel<<<(R + 255) / 256, 256, 0, s>>>(family, R, counts);
  pad::pa_census_sum_kernel<<<1, 1024, 0, s>>>(counts, n_families, out);
  return cudaGetLastError();
}

cudaError_t launch_pa_iota(int* a, int n, cudaStream_t s)
{
  if (n > 0) pad::pa_iota_kernel<<<(n + 255) / 256, 256, 0, s>>>(a, n);
  return cudaGetLastError();
}

cudaError_t launch_pa_fill(double* a, int n, double v, cudaStream_t s)
{
  if (n > 0) pad::pa_fill_kernel<<<(n + 255) / 256, 256, 0, s>>>(a, n, v);
  return cudaGetLastError();
}

cudaError_t launch_qexp(const double* x, double* y, int n, cudaStream_t s)
{
  if (n > 0) pad::qexp_kernel<<<(n + 255) / 256, 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}
}  // namespace qio
