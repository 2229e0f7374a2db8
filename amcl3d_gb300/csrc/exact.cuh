// Exact, order-independent sums of floats on the integer pipe.
//
// A float is m * 2^(k-149) with an integer m < 2^24 and 0 <= k <= 253, so every
// float is an integer multiple of 2^-149.  X320 holds such a multiple as a 320-bit
// two's-complement integer (5 x 64-bit words, least significant first, value =
// integer * 2^-149).  Sums of up to 2^32 floats of any magnitude fit without
// overflow, integer addition is associative, and so a block/grid reduction over
// X320 gives the exact real sum whatever the launch shape or summation order.
// Rounding to double happens once, at the end (round to nearest, ties to even),
// which is what math.fsum returns for the same floats.
//
// GB300 runs FP64 at a small fraction of its FP32/INT rate; these sums replace the
// FP64 accumulations of the weight normalisation, the resampling prefix and the
// pose mean with exact integer arithmetic.
#pragma once
#include <stdint.h>

namespace amcl
{
struct X320
{
  uint64_t w[5];
};

__host__ __device__ inline X320 x320_zero()
{
  X320 r;
#pragma unroll
  for (int i = 0; i < 5; ++i)
    r.w[i] = 0;
  return r;
}

__device__ __forceinline__ X320 x320_add(const X320& a, const X320& b)
{
  X320 r;
  asm("add.cc.u64 %0, %5, %10;\n\t"
      "addc.cc.u64 %1, %6, %11;\n\t"
      "addc.cc.u64 %2, %7, %12;\n\t"
      "addc.cc.u64 %3, %8, %13;\n\t"
      "addc.u64 %4, %9, %14;"
      : "=l"(r.w[0]), "=l"(r.w[1]), "=l"(r.w[2]), "=l"(r.w[3]), "=l"(r.w[4])
      : "l"(a.w[0]), "l"(a.w[1]), "l"(a.w[2]), "l"(a.w[3]), "l"(a.w[4]), "l"(b.w[0]), "l"(b.w[1]),
        "l"(b.w[2]), "l"(b.w[3]), "l"(b.w[4]));
  return r;
}

__device__ __forceinline__ X320 x320_neg(const X320& a)
{
  X320 n;
#pragma unroll
  for (int i = 0; i < 5; ++i)
    n.w[i] = ~a.w[i];
  X320 one = x320_zero();
  one.w[0] = 1;
  return x320_add(n, one);
}

// Exact conversion of a finite float (NaN/Inf give 0 and set *bad).
__device__ __forceinline__ X320 x320_from_float(float f, bool* bad = nullptr)
{
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xFFu;
  uint32_t m = b & 0x7FFFFFu;
  X320 r = x320_zero();
  if (e == 0xFFu)
  {
    if (bad)
      *bad = true;
    return r;
  }
  if (e)
    m |= 0x800000u;
  const int k = e ? static_cast<int>(e) - 1 : 0;
  const int word = k >> 6, sh = k & 63;
  const uint64_t lo = static_cast<uint64_t>(m) << sh;
  const uint64_t hi = sh ? (static_cast<uint64_t>(m) >> (64 - sh)) : 0ull;
#pragma unroll
  for (int i = 0; i < 5; ++i)
    r.w[i] = (i == word) ? lo : ((i == word + 1) ? hi : 0ull);
  return (b >> 31) ? x320_neg(r) : r;
}

__device__ __forceinline__ X320 x320_shfl_xor(const X320& a, int lane_mask)
{
  X320 r;
#pragma unroll
  for (int i = 0; i < 5; ++i)
    r.w[i] = __shfl_xor_sync(0xFFFFFFFFu, a.w[i], lane_mask);
  return r;
}

// Every lane of the warp ends with the warp total.
__device__ __forceinline__ X320 x320_warp_sum(X320 a)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    a = x320_add(a, x320_shfl_xor(a, o));
  return a;
}

// Signed compare: -1, 0, 1.
__device__ __forceinline__ int x320_cmp(const X320& a, const X320& b)
{
  const int64_t ta = static_cast<int64_t>(a.w[4]), tb = static_cast<int64_t>(b.w[4]);
  if (ta != tb)
    return ta < tb ? -1 : 1;
#pragma unroll
  for (int i = 3; i >= 0; --i)
    if (a.w[i] != b.w[i])
      return a.w[i] < b.w[i] ? -1 : 1;
  return 0;
}

__host__ __device__ inline int clz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
  return __clzll(static_cast<long long>(x));
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// Bits [p, p+64) of a 320-bit magnitude, 0 <= p < 320 (bits past the top are 0).
__host__ __device__ inline uint64_t x320_bits64(const X320& a, int p)
{
  const int w = p >> 6, s = p & 63;
  const uint64_t lo = w < 5 ? a.w[w] : 0ull;
  const uint64_t hi = w + 1 < 5 ? a.w[w + 1] : 0ull;
  return s ? ((lo >> s) | (hi << (64 - s))) : lo;
}

// True when any bit below position p (exclusive) is set.
__host__ __device__ inline bool x320_any_below(const X320& a, int p)
{
  if (p <= 0)
    return false;
  const int w = p >> 6, s = p & 63;
  for (int i = 0; i < w && i < 5; ++i)
    if (a.w[i])
      return true;
  if (w < 5 && s && (a.w[w] & ((1ull << s) - 1ull)))
    return true;
  return false;
}

// Correctly rounded (nearest, ties to even) conversion to double.
__host__ __device__ inline double x320_to_double(const X320& v)
{
  X320 a = v;
  const bool neg = (a.w[4] >> 63) != 0;
  if (neg)
  {
    // two's complement negate on the host/device without PTX
    uint64_t carry = 1;
    for (int i = 0; i < 5; ++i)
    {
      const uint64_t x = ~a.w[i];
      a.w[i] = x + carry;
      carry = (carry && a.w[i] == 0) ? 1 : 0;
    }
  }
  int top = -1;
  for (int i = 4; i >= 0; --i)
    if (a.w[i])
    {
      top = i * 64 + 63 - clz64(a.w[i]);
      break;
    }
  if (top < 0)
    return neg ? -0.0 : 0.0;
  const int lsb = top - 52;  // position of the last kept bit
  uint64_t mant = lsb >= 0 ? (x320_bits64(a, lsb) & ((1ull << 53) - 1ull)) : x320_bits64(a, 0);
  int exp2 = (lsb >= 0 ? lsb : 0) - 149;  // value = mant * 2^exp2
  if (lsb > 0)
  {
    const uint64_t guard = (x320_bits64(a, lsb - 1) & 1ull);
    const bool sticky = x320_any_below(a, lsb - 1);
    if (guard && (sticky || (mant & 1ull)))
    {
      mant += 1;
      if (mant >> 53)
      {
        mant >>= 1;
        exp2 += 1;
      }
    }
  }
  // mant < 2^53 is exact in double; the scaling by a power of two is exact too
  // (results stay far above the double subnormal range: |value| >= 2^-149).
  double r = static_cast<double>(mant);
  int e = exp2;
  while (e > 0)
  {
    const int s = e > 60 ? 60 : e;
    r *= static_cast<double>(1ull << s);
    e -= s;
  }
  while (e < 0)
  {
    const int s = -e > 60 ? 60 : -e;
    r /= static_cast<double>(1ull << s);
    e += s;
  }
  return neg ? -r : r;
}

// 32-bit digit split for grid-wide atomic accumulation: digits 0..8 are unsigned,
// digit 9 carries the sign.  Sums of up to 2^31 such digit vectors fit in int64.
struct Digits10
{
  unsigned long long d[10];
};

__device__ __forceinline__ void x320_atomic_add(unsigned long long* dst10, const X320& v)
{
#pragma unroll
  for (int j = 0; j < 10; ++j)
  {
    const uint64_t word = v.w[j >> 1];
    uint64_t digit = (j & 1) ? (word >> 32) : (word & 0xFFFFFFFFull);
    if (j == 9)
      digit = static_cast<uint64_t>(static_cast<int64_t>(static_cast<int32_t>(static_cast<uint32_t>(digit))));
    if (digit)
      atomicAdd(dst10 + j, static_cast<unsigned long long>(digit));
  }
}

// Rebuilds the X320 total from accumulated digits (carry propagation).
__host__ __device__ inline X320 x320_from_digits(const unsigned long long* d10)
{
  X320 r = x320_zero();
  // value = sum_j d_j * 2^(32 j), d_9 signed
  int64_t carry = 0;  // running carry in units of 2^(32 j)
  uint32_t digit[10];
  for (int j = 0; j < 10; ++j)
  {
    // d_j plus incoming carry; for j < 9 the sum is non-negative and < 2^64 + 2^32
    if (j < 9)
    {
      const unsigned long long dj = d10[j];
      const unsigned long long s = dj + static_cast<unsigned long long>(carry);
      const bool ovf = s < dj;  // carry >= 0 for j < 9
      digit[j] = static_cast<uint32_t>(s & 0xFFFFFFFFull);
      carry = static_cast<int64_t>((s >> 32) | (ovf ? (1ull << 32) : 0ull));
    }
    else
    {
      const int64_t s = static_cast<int64_t>(d10[j]) + carry;
      digit[j] = static_cast<uint32_t>(static_cast<uint64_t>(s) & 0xFFFFFFFFull);
    }
  }
  for (int i = 0; i < 5; ++i)
    r.w[i] = static_cast<uint64_t>(digit[2 * i]) | (static_cast<uint64_t>(digit[2 * i + 1]) << 32);
  return r;
}

}  // namespace amcl
