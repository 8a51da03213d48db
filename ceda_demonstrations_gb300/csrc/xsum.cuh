// Exact, order-independent accumulation of doubles (host + device).
//
// Every term x is truncated toward zero to a multiple of 2^-160 and added exactly into
// ten signed 64-bit limbs, limb k carrying 32-bit digits of weight 2^(32k-160). A term
// touches at most three limbs and never propagates a carry, so per-thread accumulators,
// warp shuffles, block trees and global atomics can combine partial sums in any order and
// the total is the same integer. The result is that integer rounded once to the nearest
// double. Terms with |x| >= 2^128 (or inf) set the overflow flag, NaN sets the NaN flag.
// Up to 2^31 terms fit without limb overflow.
//
// This replaces the order-dependent allreduce of the reference's NVECTOR reductions
// (gkeyll_diffusion/src/nvector_gkylzero.c:234-404): the value a reduction returns here is
// independent of the grid shape, the SM count and the kernel that produced the terms.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define XS_HD __host__ __device__ __forceinline__
#else
#define XS_HD inline
#endif

namespace xsum {

constexpr int NL = 10;
constexpr unsigned FLAG_NAN = 1u, FLAG_OVF = 2u;

struct Limbs {
  long long l[NL];
};

XS_HD void zero(Limbs& a)
{
#pragma unroll
  for (int k = 0; k < NL; ++k) a.l[k] = 0;
}

XS_HD unsigned long long bits_of(double x)
{
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}

XS_HD void add(Limbs& a, double x, unsigned& flags)
{
  unsigned long long b = bits_of(x);
  const bool neg       = (b >> 63) != 0;
  const int e          = (int)((b >> 52) & 0x7ff);
  unsigned long long m = b & ((1ULL << 52) - 1);
  if (e == 0x7ff)
  {
    flags |= m ? FLAG_NAN : FLAG_OVF;
    return;
  }
  int exp2;
  if (e == 0) exp2 = -1074;
  else
  {
    m |= (1ULL << 52);
    exp2 = e - 1075;
  }
  if (exp2 > 75)
  { // |x| >= 2^128
    flags |= FLAG_OVF;
    return;
  }
  int sh = exp2 + 160;
  if (sh < 0)
  {
    m  = (sh <= -64) ? 0ULL : (m >> (-sh));
    sh = 0;
  }
  const int k  = sh >> 5; // 0 .. 7 (sh <= 235)
  const int bs = sh & 31;
  // v = m << bs spans up to 85 bits: digits d0 | d1 | d2
  const unsigned long long lo = m << bs;
  const unsigned long long hi = bs ? (m >> (64 - bs)) : 0ULL;
  long long d0                = (long long)(lo & 0xffffffffULL);
  long long d1                = (long long)(lo >> 32);
  long long d2                = (long long)hi;
  if (neg)
  {
    d0 = -d0;
    d1 = -d1;
    d2 = -d2;
  }
  // three adds into limbs k, k+1, k+2; one branch per term (the terms of one warp usually
  // share k) instead of a select on every limb
  switch (k)
  {
#define XS_CASE(K)                                                                                                   \
  case K:                                                                                                            \
    a.l[K] += d0;                                                                                                    \
    a.l[K + 1] += d1;                                                                                                \
    a.l[K + 2] += d2;                                                                                                \
    break;
    XS_CASE(0)
    XS_CASE(1)
    XS_CASE(2)
    XS_CASE(3)
    XS_CASE(4)
    XS_CASE(5)
    XS_CASE(6)
    XS_CASE(7)
#undef XS_CASE
  default: break;
  }
}

XS_HD void merge(Limbs& a, const Limbs& b)
{
#pragma unroll
  for (int k = 0; k < NL; ++k) a.l[k] += b.l[k];
}

XS_HD double from_bits(unsigned long long b)
{
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

// Normalise the limbs into a two's-complement integer of 32-bit digits and round it to the
// nearest double (ties to even). Integer arithmetic only, so host and device produce the
// same bits.
XS_HD double finalize(const long long* limbs, unsigned flags)
{
  if (flags & FLAG_NAN) return from_bits(0x7ff8000000000000ULL);
  if (flags & FLAG_OVF) return from_bits(0x7ff0000000000000ULL);
  constexpr int ND = NL + 1; // digit NL holds the sign extension
  unsigned int dg[ND];
  long long carry = 0;
  for (int k = 0; k < NL; ++k)
  {
    long long v = limbs[k] + carry;
    dg[k]       = (unsigned int)(v & 0xffffffffLL);
    carry       = v >> 32; // arithmetic shift: floor division by 2^32
  }
  const bool negative = carry < 0;
  dg[NL]              = (unsigned int)(carry & 0xffffffffLL);
  if (negative)
  { // magnitude = two's-complement negation
    unsigned long long c = 1;
    for (int k = 0; k < ND; ++k)
    {
      unsigned long long s = (unsigned long long)(unsigned int)(~dg[k]) + c;
      dg[k]                = (unsigned int)s;
      c                    = s >> 32;
    }
  }
  int top = -1;
  for (int k = ND - 1; k >= 0 && top < 0; --k)
    if (dg[k])
    {
      int msb = 31;
      while (!((dg[k] >> msb) & 1u)) --msb;
      top = k * 32 + msb;
    }
  if (top < 0) return 0.0;
  int shift = top - 52;
  unsigned long long mant;
  if (shift <= 0)
  { // the magnitude fits in 53 bits: exact
    mant  = (unsigned long long)dg[0] | ((unsigned long long)dg[1] << 32);
    shift = 0;
  }
  else
  {
    const int k = shift >> 5, b = shift & 31;
    unsigned long long w0 = dg[k];
    unsigned long long w1 = (k + 1 < ND) ? dg[k + 1] : 0ULL;
    unsigned long long w2 = (k + 2 < ND) ? dg[k + 2] : 0ULL;
    unsigned long long c  = w0 | (w1 << 32);
    mant                  = (c >> b) | (b ? (w2 << (64 - b)) : 0ULL);
    mant &= ((1ULL << 53) - 1);
    const int r  = shift - 1;
    const bool rb = ((dg[r >> 5] >> (r & 31)) & 1u) != 0;
    bool sticky   = (dg[r >> 5] & ((1u << (r & 31)) - 1u)) != 0;
    for (int q = 0; q < (r >> 5); ++q) sticky = sticky || (dg[q] != 0);
    if (rb && (sticky || (mant & 1ULL)))
    {
      mant++;
      if (mant == (1ULL << 53))
      {
        mant >>= 1;
        shift++;
      }
    }
  }
  // value = mant * 2^(shift - 160): exact power-of-two scaling in steps of 2^60
  double v = (double)mant;
  int ex   = shift - 160;
  while (ex <= -60)
  {
    v *= 0x1p-60;
    ex += 60;
  }
  while (ex >= 60)
  {
    v *= 0x1p60;
    ex -= 60;
  }
  v *= (ex < 0) ? 1.0 / (double)(1ULL << (-ex)) : (double)(1ULL << ex);
  return negative ? -v : v;
}

} // namespace xsum
