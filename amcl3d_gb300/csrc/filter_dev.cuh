// Device bodies of the per-particle filter stages (ParticleFilter.cpp:46-222), shared
// by the single-filter kernels (filter.cu) and the batched kernels (batch.cu).
// Each body handles one block of NT particles of one filter; `blk` is the block's
// index within that filter.
#pragma once
#include <stdint.h>

#include "exact.cuh"
#include "locate.cuh"
#include "philox.cuh"

namespace amcl
{
enum Acc
{
  ACC_WP = 0,
  ACC_WR,
  ACC_W,
  ACC_W2,               // sum of the normalised weights
  ACC_M1,               // 4 accumulators: sum w*x, w*y, w*z, w*a
  ACC_M2 = ACC_M1 + 4,  // 4 accumulators: sum w*x^2, ...
  ACC_COUNT = ACC_M2 + 4
};
constexpr int NDIG = 10;
constexpr int NT = 256;  // threads per block of the per-particle kernels
constexpr int ACC_WORDS = ACC_COUNT * NDIG;

struct PFStats
{
  double sum_wp, sum_wr, sum_w, sum_w2;
  double mean[4];
  double var[4];
  float mean_f[4];
  int err;
  int pad;
};

__device__ __forceinline__ double acc_value(const unsigned long long* acc, int k)
{
  return x320_to_double(x320_from_digits(acc + k * NDIG));
}

// Exact two-product of floats via FMA: a*b = p + e exactly (e rounded only if it
// underflows; the oracle rounds the same residual the same way).
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e)
{
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// Block-wide exact sum of one value per thread added to digits `dst`.
__device__ __forceinline__ void block_exact_add(X320 v, unsigned long long* dst, X320* s_part)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = x320_warp_sum(v);
  __syncthreads();
  if (lane == 0)
    s_part[wid] = v;
  __syncthreads();
  if (wid == 0)
  {
    X320 t = lane < nw ? s_part[lane] : x320_zero();
    t = x320_warp_sum(t);
    if (lane == 0)
      x320_atomic_add(dst, t);
  }
}

// Block-wide exact sum returned to thread 0 (others: unspecified).
__device__ __forceinline__ X320 block_exact_sum(X320 v, X320* s_part)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = x320_warp_sum(v);
  __syncthreads();
  if (lane == 0)
    s_part[wid] = v;
  __syncthreads();
  X320 t = x320_zero();
  if (wid == 0)
  {
    t = lane < nw ? s_part[lane] : x320_zero();
    t = x320_warp_sum(t);
  }
  return t;
}

// ---- update: blend (ParticleFilter.cpp:157-180) ----------------------------------------------
// wp /= wtp, wr /= wtr for every particle (stale values of out-of-map particles
// included); w = alpha*wp + (1-alpha)*wr in double for in-map particles, else 0.
__device__ __forceinline__ void blend_block(uint32_t blk, uint32_t n, const uint8_t* inmap, float* wp, float* wr,
                                            float* w, double alpha, unsigned long long* acc, double* s_sum,
                                            X320* s_part)
{
  __syncthreads();
  if (threadIdx.x == 0)
    s_sum[0] = acc_value(acc, ACC_WP);
  if (threadIdx.x == 32)
    s_sum[1] = acc_value(acc, ACC_WR);
  __syncthreads();
  const double sp = s_sum[0], sr = s_sum[1];
  const uint32_t i = blk * NT + threadIdx.x;
  float wv = 0.0f;
  if (i < n)
  {
    const float a = sp > 0 ? __double2float_rn(__ddiv_rn(static_cast<double>(wp[i]), sp)) : 0.0f;
    const float b = sr > 0 ? __double2float_rn(__ddiv_rn(static_cast<double>(wr[i]), sr)) : 0.0f;
    wp[i] = a;
    wr[i] = b;
    if (inmap[i])
      wv = __double2float_rn(
          __dadd_rn(__dmul_rn(static_cast<double>(a), alpha), __dmul_rn(static_cast<double>(b), __dsub_rn(1.0, alpha))));
    w[i] = wv;
  }
  block_exact_add(x320_from_float(wv), acc + ACC_W * NDIG, s_part);
}

// ---- normalise w, mean terms, per-block resample sums (ParticleFilter.cpp:182-195, :79-92) ----
// Nine exact block sums (w, then w*c and w*c^2 per pose component c): each warp sums
// them one after the other into s_part[quantity][warp] without a barrier, then one
// barrier and the cross-warp sums run on separate warps.
constexpr int NORM_Q = 9;

__device__ __forceinline__ void normalize_block(uint32_t blk, uint32_t n, const float4* pose, float* w,
                                                unsigned long long* acc, X320* blocksum, double* s_sum,
                                                X320* s_part /* NORM_Q x (NT / 32) */)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (threadIdx.x == 0)
    s_sum[0] = acc_value(acc, ACC_W);
  __syncthreads();
  const double tot = s_sum[0];
  const uint32_t i = blk * NT + threadIdx.x;
  float wv = 0.0f;
  float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
  if (i < n)
  {
    wv = tot > 0 ? __double2float_rn(__ddiv_rn(static_cast<double>(w[i]), tot)) : 0.0f;
    w[i] = wv;
    p = pose[i];
  }
  X320 q = x320_warp_sum(x320_from_float(wv));
  if (lane == 0)
    s_part[wid] = q;
  const float c[4] = { p.x, p.y, p.z, p.w };
#pragma unroll
  for (int k = 0; k < 4; ++k)
  {
    float hi, lo;
    two_prod(wv, c[k], hi, lo);
    q = x320_warp_sum(x320_add(x320_from_float(hi), x320_from_float(lo)));
    if (lane == 0)
      s_part[(1 + k) * nw + wid] = q;
    // w*c^2 = w*(s + t) with c*c = s + t exactly; each product split again.
    float s, t, h1, l1, h2, l2;
    two_prod(c[k], c[k], s, t);
    two_prod(wv, s, h1, l1);
    two_prod(wv, t, h2, l2);
    q = x320_warp_sum(x320_add(x320_add(x320_from_float(h1), x320_from_float(l1)),
                               x320_add(x320_from_float(h2), x320_from_float(l2))));
    if (lane == 0)
      s_part[(5 + k) * nw + wid] = q;
  }
  __syncthreads();
  for (int j = wid; j < NORM_Q; j += nw)
  {
    X320 t = lane < nw ? s_part[j * nw + lane] : x320_zero();
    t = x320_warp_sum(t);
    if (lane == 0)
    {
      if (j == 0)
      {
        blocksum[blk] = t;  // the resample prefix of this block
        x320_atomic_add(acc + ACC_W2 * NDIG, t);
      }
      else
        x320_atomic_add(acc + (j <= 4 ? ACC_M1 + (j - 1) : ACC_M2 + (j - 5)) * NDIG, t);
    }
  }
}

// Sums, mean and variance from the exact accumulators, by one warp: lane k converts
// accumulator k, lanes 0-3 finish pose component k.
__device__ __forceinline__ void finalize_stats_warp(const unsigned long long* acc, PFStats* st)
{
  const int lane = threadIdx.x & 31;
  const double v = lane < ACC_COUNT ? acc_value(acc, lane) : 0.0;
  const double s2 = __shfl_sync(0xFFFFFFFFu, v, ACC_W2);
  const double m1 = __shfl_sync(0xFFFFFFFFu, v, ACC_M1 + (lane & 3));
  const double m2 = __shfl_sync(0xFFFFFFFFu, v, ACC_M2 + (lane & 3));
  if (lane == ACC_WP)
    st->sum_wp = v;
  if (lane == ACC_WR)
    st->sum_wr = v;
  if (lane == ACC_W)
    st->sum_w = v;
  if (lane == ACC_W2)
    st->sum_w2 = v;
  if (lane < 4)
  {
    st->mean[lane] = m1;  // the reference's mean is sum w*x of the normalised weights
    st->mean_f[lane] = __double2float_rn(m1);
    if (s2 > 0)
    {
      const double mu = __ddiv_rn(m1, s2);
      st->var[lane] = __dsub_rn(__ddiv_rn(m2, s2), __dmul_rn(mu, mu));
    }
    else
      st->var[lane] = 0.0;
  }
}

// ---- predict (ParticleFilter.cpp:97-119) --------------------------------------------------------
struct PredictArgs
{
  uint32_t n;
  uint32_t seed_lo, seed_hi;
  uint64_t step;
  float sx, sy, sz, sa;  // (float) |delta * mod|, the normal_distribution<float> stddev
  double dx, dy, dz, da;
  float* draws;  // optional 4 per particle
};

__device__ __forceinline__ void predict_particle(uint32_t i, float4* pose, const PredictArgs& a)
{
  Philox4 c;
  c.v[0] = i;
  c.v[1] = static_cast<uint32_t>(a.step);
  c.v[2] = static_cast<uint32_t>(a.step >> 32);
  c.v[3] = RNG_TAG_PREDICT;
  float z[4];
  normals4(philox4x32_10(c, a.seed_lo, a.seed_hi), z);
  if (a.draws)
    reinterpret_cast<float4*>(a.draws)[i] = make_float4(z[0], z[1], z[2], z[3]);
  float4 p = pose[i];
  // ranGaussian(0, dev) = z * (float)dev + 0.0f  (normal_distribution<float>)
  const float gx = fadd(fmul(z[0], a.sx), 0.0f);
  const float gy = fadd(fmul(z[1], a.sy), 0.0f);
  const float gz = fadd(fmul(z[2], a.sz), 0.0f);
  const float ga = fadd(fmul(z[3], a.sa), 0.0f);
  double sd, cd;
  sincos(static_cast<double>(p.w), &sd, &cd);
  const float sa = __double2float_rn(sd), ca = __double2float_rn(cd);
  const float rx = __double2float_rn(__dadd_rn(a.dx, static_cast<double>(gx)));
  const float ry = __double2float_rn(__dadd_rn(a.dy, static_cast<double>(gy)));
  p.x = fadd(p.x, fsub(fmul(ca, rx), fmul(sa, ry)));
  p.y = fadd(p.y, fadd(fmul(sa, rx), fmul(ca, ry)));
  p.z = __double2float_rn(__dadd_rn(static_cast<double>(p.z), __dadd_rn(a.dz, static_cast<double>(gz))));
  p.w = __double2float_rn(__dadd_rn(static_cast<double>(p.w), __dadd_rn(a.da, static_cast<double>(ga))));
  pose[i] = p;
}

// ---- resample (ParticleFilter.cpp:198-222) ---------------------------------------------------
// u_m = r + factor*m in float; index[m] = first i with C_i >= u_m where C is the
// inclusive prefix of w; for each particle hi_i = #{m : u_m <= C_i} (u is
// non-decreasing in m), so index[m] = first i with hi_i > m.

__device__ __forceinline__ float u_of(float r, float factor, uint32_t m)
{
  return fadd(r, fmul(factor, static_cast<float>(m)));
}

__device__ __forceinline__ void block_sum_block(uint32_t blk, uint32_t n, const float* w, X320* blocksum,
                                                X320* s_part)
{
  const uint32_t i = blk * NT + threadIdx.x;
  const X320 t = block_exact_sum(x320_from_float(i < n ? w[i] : 0.0f), s_part);
  if (threadIdx.x == 0)
    blocksum[blk] = t;
}

// Exact inclusive prefix C_i, then hi_i by binary search over m.
__device__ __forceinline__ void prefix_hi_block(uint32_t blk, uint32_t n, const float* w, const X320* blocksum,
                                                float r, float factor, int32_t* hi, X320* s_scan, X320* s_base)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (wid == 0)
  {
    X320 t = x320_zero();
    for (uint32_t b = lane; b < blk; b += 32)
      t = x320_add(t, blocksum[b]);
    t = x320_warp_sum(t);
    if (lane == 0)
      *s_base = t;
  }
  const uint32_t i = blk * NT + threadIdx.x;
  const X320 own = x320_from_float(i < n ? w[i] : 0.0f);
  X320 x = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    X320 y;
#pragma unroll
    for (int k = 0; k < 5; ++k)
      y.w[k] = __shfl_up_sync(0xFFFFFFFFu, x.w[k], o);
    if (lane >= o)
      x = x320_add(x, y);
  }
  if (lane == 31)
    s_scan[wid] = x;
  __syncthreads();
  X320 c = *s_base;
  for (int k = 0; k < wid; ++k)
    c = x320_add(c, s_scan[k]);
  c = x320_add(c, x);  // inclusive prefix C_i
  if (i >= n)
    return;
  uint32_t lo = 0, up = n;
  while (lo < up)
  {
    const uint32_t mid = (lo + up) >> 1;
    if (x320_cmp(x320_from_float(u_of(r, factor, mid)), c) <= 0)
      lo = mid + 1;
    else
      up = mid;
  }
  hi[i] = static_cast<int32_t>(lo);
}

__device__ __forceinline__ void gather_particle(uint32_t m, uint32_t n, const int32_t* hi, const float4* pose,
                                                const float* wp, const float* wr, float4* pose_o, float* w_o,
                                                float* wp_o, float* wr_o, float factor, int32_t* idx_o)
{
  uint32_t lo = 0, up = n;
  while (lo < up)
  {
    const uint32_t mid = (lo + up) >> 1;
    if (static_cast<uint32_t>(hi[mid]) > m)
      up = mid;
    else
      lo = mid + 1;
  }
  // lo == n: the reference runs past its array (reads p_[N]); clamp to the last particle.
  const uint32_t src = lo < n ? lo : n - 1;
  pose_o[m] = pose[src];
  wp_o[m] = wp[src];
  wr_o[m] = wr[src];
  w_o[m] = factor;  // new_p[m].w = factor (ParticleFilter.cpp:217)
  if (idx_o)
    idx_o[m] = static_cast<int32_t>(src);
}

}  // namespace amcl
