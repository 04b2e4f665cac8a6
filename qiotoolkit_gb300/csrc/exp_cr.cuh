// exp_cr.cuh -- exp(x) rounded correctly to double, by double-double
// arithmetic (error-free sums and products: Knuth's two-sum, Dekker's
// fast two-sum, products by fused multiply-add), for deciding the rare
// parallel-tempering swaps whose uniform draw lies within 1e-15 of exp(x):
// there the device's exp and the host C library's exp (which the reference
// calls) may round to neighbouring doubles.
//
// Method: Cody-Waite reduction x = k ln2 + r with ln 2 split in three
// doubles (k ln2_hi and k ln2_mid exact for |k| < 2^11), |r| <= ~0.35, the
// Taylor sum of exp(r) to 27 terms in double-double (truncation below 1e-40),
// scaled by 2^k.  The double-double value is within ~1e-30 relative of
// exp(x), so its rounding to double is the correctly rounded exp except
// within that distance of a rounding midpoint.  Compiles as host code (tested
// there against exact values) and as device code.
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define QIO_HD __host__ __device__ __forceinline__
#else
#define QIO_HD inline
#endif

namespace qio
{
namespace dd
{
struct DD
{
  double hi, lo;
};
QIO_HD DD two_sum(double a, double b)
{
  const double s = a + b;
  const double bb = s - a;
  const double e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
QIO_HD DD fast_two_sum(double a, double b)
{
  const double s = a + b;
  return {s, b - (s - a)};
}
QIO_HD DD two_prod(double a, double b)
{
  const double p = a * b;
  return {p, fma(a, b, -p)};
}
QIO_HD DD add(DD a, DD b)
{
  DD s = two_sum(a.hi, b.hi);
  const DD t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
QIO_HD DD mul(DD a, DD b)
{
  DD p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return fast_two_sum(p.hi, p.lo);
}
// a / n for a small positive integer n
QIO_HD DD div_small(DD a, double n)
{
  const double q1 = a.hi / n;
  const double r = fma(-q1, n, a.hi) + a.lo;
  return fast_two_sum(q1, r / n);
}

QIO_HD double exp_cr(double x)
{
  if (x != x) return x;
  if (x > 709.79) return INFINITY;
  if (x < -745.2) return 0.0;
  const double k = rint(x * 1.4426950408889634);  // round(x / ln 2)
  // ln 2 = c1 + c2 + c3 to ~160 bits
  const double c1 = 0x1.62e42fefa39efp-1, c2 = 0x1.abc9e3b39803fp-56, c3 = 0x1.7b57a079a1934p-111;
  const DD p1 = two_prod(k, c1), p2 = two_prod(k, c2);
  DD r = two_sum(x, -p1.hi);
  r = add(r, DD{-p1.lo, 0.0});
  r = add(r, DD{-p2.hi, -p2.lo});
  r = add(r, DD{-(k * c3), 0.0});
  DD term{1.0, 0.0}, sum{1.0, 0.0};
  for (int n = 1; n <= 27; n++)
  {
    term = div_small(mul(term, r), (double)n);
    sum = add(sum, term);
  }
  const DD s = fast_two_sum(sum.hi, sum.lo);
  return ldexp(s.hi, (int)k);
}
}  // namespace dd
}  // namespace qio
