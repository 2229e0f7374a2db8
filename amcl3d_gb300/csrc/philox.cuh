// Counter-based random numbers for the particle filter.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC'11): a 4x32-bit counter and a 2x32-bit key go through ten rounds of
// two 32x32->64 multiplies with the published multipliers and Weyl key increments.
// Every (filter seed, draw step, particle) triple addresses its own 128 random bits,
// so draws are independent of launch shape and batching and need no stored state
// beyond a per-filter step counter.
//
// The reference draws from std::mt19937 seeded by std::random_device
// (ParticleFilter.cpp:22, ParticleFilter.h:211-212), which is not reproducible;
// the stream here is a different generator by design, checked statistically.
#pragma once
#include <stdint.h>

namespace amcl
{
struct Philox4
{
  uint32_t v[4];
};

__host__ __device__ inline void philox_mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo)
{
  const uint64_t p = static_cast<uint64_t>(a) * static_cast<uint64_t>(b);
  hi = static_cast<uint32_t>(p >> 32);
  lo = static_cast<uint32_t>(p);
}

__host__ __device__ inline Philox4 philox4x32_10(Philox4 c, uint32_t k0, uint32_t k1)
{
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r)
  {
    uint32_t hi0, lo0, hi1, lo1;
    philox_mulhilo(M0, c.v[0], hi0, lo0);
    philox_mulhilo(M1, c.v[2], hi1, lo1);
    Philox4 n;
    n.v[0] = hi1 ^ c.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ k1;
    n.v[3] = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// Counter layout: (particle index, step low, step high, stream tag).
enum : uint32_t
{
  RNG_TAG_PREDICT = 1,
  RNG_TAG_INIT = 2,
  RNG_TAG_RESAMPLE = 3
};

// Uniform in (0, 1]: (x + 1) * 2^-32 rounded to float.
__device__ __forceinline__ float u01_open0(uint32_t x) { return (static_cast<float>(x) + 1.0f) * 2.3283064365386963e-10f; }
// Uniform in [0, 1): top 24 bits.
__host__ __device__ inline float u01_closed0(uint32_t x) { return static_cast<float>(x >> 8) * 5.9604644775390625e-08f; }

// Four standard normals from one Philox block (Box-Muller on two pairs).
__device__ __forceinline__ void normals4(const Philox4& r, float z[4])
{
#pragma unroll
  for (int j = 0; j < 2; ++j)
  {
    const float u1 = u01_open0(r.v[2 * j]);
    const float u2 = u01_closed0(r.v[2 * j + 1]);
    const float rad = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    z[2 * j] = rad * c;
    z[2 * j + 1] = rad * s;
  }
}

}  // namespace amcl
