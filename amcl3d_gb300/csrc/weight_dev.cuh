// Device helpers of the cloud weighting shared by the single-filter kernels
// (weight.cu) and the batched kernels (batch.cu).
#pragma once
#include "exact.cuh"
#include "grid.cuh"
#include "locate.cuh"

namespace amcl
{
constexpr int UNROLL = 8;
constexpr int YAW_UNROLL = 8;  // points per group of the paired yaw-only loop
constexpr int FAST_UNROLL = 8;  // points per group of the loop with floor constants
constexpr int GEN_UNROLL = 4;   // points per group of the general yaw loop
constexpr int MAX_RANGES = 64;

__device__ __forceinline__ float exp_f32_via_f64(float x) { return __double2float_rn(exp(static_cast<double>(x))); }

// ParticleFilter::computeRangeWeight (ParticleFilter.cpp:224-244), float overloads.
__device__ __forceinline__ float range_weight(float x, float y, float z, const float4* rg, int nr, float k1, float k2)
{
  if (nr == 0)
    return 0.0f;
  float w = 1.0f;
  for (int b = 0; b < nr; ++b)
  {
    const float4 R = rg[b];  // (r, ax, ay, az)
    const float dx = fsub(x, R.y), dy = fsub(y, R.z), dz = fsub(z, R.w);
    const float r = __fsqrt_rn(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)));
    const float d = fsub(r, R.x);
    const float e = exp_f32_via_f64(fmul(fmul(-k2, d), d));
    w = fmul(w, fmul(k1, e));
  }
  return w;
}

// Running sum of the probabilities: the reference's float `weight += prob`
// (Grid3d.cpp:191) or a Neumaier-compensated float sum.
template <int SUM>
struct CloudSum
{
  float sum = 0.0f, comp = 0.0f;
  int n = 0;
  __device__ __forceinline__ void add(float v)
  {
    if (SUM == 0)
    {
      sum = fadd(sum, v);
    }
    else
    {
      const float t = fadd(sum, v);
      comp = fadd(comp, fabsf(sum) >= fabsf(v) ? fadd(fsub(sum, t), v) : fadd(fsub(v, t), sum));
      sum = t;
    }
    n += 1;
  }
  // The compensated add without the count (the loops with floor constants count apart).
  __device__ __forceinline__ void add_uncounted(float v)
  {
    const float t = fadd(sum, v);
    comp = fadd(comp, fabsf(sum) >= fabsf(v) ? fadd(fsub(sum, t), v) : fadd(fsub(v, t), sum));
    sum = t;
  }
  // Grid3d.cpp:198: 0 with 10 or fewer points, else the mean.
  __device__ __forceinline__ float weight() const
  {
    const float tot = SUM == 0 ? sum : fadd(sum, comp);
    return (n <= 10) ? 0.0f : __fdiv_rn(tot, static_cast<float>(n));
  }
};

// Adds the points [0, cnt) of a staged chunk (cnt a multiple of UNROLL, padding
// points NaN) in order.  Points are float4 (x, y, z + 0, -), or with YL the
// yaw-only staging: (x, x, y, y) in s_pts and z + 0 in s_z.
template <int STORAGE, int SUM, int MODE, bool YL, int TAB>
__device__ __forceinline__ void weigh_chunk(const float4* s_pts, const float* s_z, uint32_t cnt, const float2* s_tab,
                                            const GridView& g, const PartXf& xf, CloudSum<SUM>& acc)
{
  for (uint32_t k = 0; k < cnt; k += UNROLL)
  {
    uint32_t cell[UNROLL];
#pragma unroll
    for (int j = 0; j < UNROLL; ++j)
    {
      const float4 s = s_pts[k + j];
      cell[j] = YL ? cell_of_point<MODE, TAB>(g, s_tab, xf, s.x, s.z, s_z[k + j])
                   : cell_of_point<MODE, TAB>(g, s_tab, xf, s.x, s.y, s.z);
    }
    float v[UNROLL];
#pragma unroll
    for (int j = 0; j < UNROLL; ++j)
      v[j] = cell[j] != 0xFFFFFFFFu ? gather_prob<STORAGE>(g, cell[j]) : 0.0f;
#pragma unroll
    for (int j = 0; j < UNROLL; ++j)
      if (cell[j] != 0xFFFFFFFFu)
        acc.add(v[j]);
  }
}

// weigh_chunk of the yaw-only mode on the yaw-only staging, x and y paired, YAW_UNROLL
// points per group (cnt a multiple of it).
template <int STORAGE, int SUM, int TAB>
__device__ __forceinline__ void weigh_chunk_yaw2(const float4* s_pts, const float* s_z, uint32_t cnt,
                                                 const float2* s_tab, const GridView& g, const PartYaw2& q,
                                                 CloudSum<SUM>& acc)
{
  static_assert(YAW_UNROLL % 4 == 0, "z is read a float4 at a time");
  for (uint32_t k = 0; k < cnt; k += YAW_UNROLL)
  {
    float zs[YAW_UNROLL];
#pragma unroll
    for (int j = 0; j < YAW_UNROLL; j += 4)
    {
      const float4 z4 = *reinterpret_cast<const float4*>(s_z + k + j);
      zs[j] = z4.x;
      zs[j + 1] = z4.y;
      zs[j + 2] = z4.z;
      zs[j + 3] = z4.w;
    }
    uint32_t cell[YAW_UNROLL];
#pragma unroll
    for (int j = 0; j < YAW_UNROLL; ++j)
      cell[j] = cell_of_point_yaw2<TAB>(g, s_tab, q, s_pts[k + j], zs[j]);
    float v[YAW_UNROLL];
#pragma unroll
    for (int j = 0; j < YAW_UNROLL; ++j)
      v[j] = cell[j] != 0xFFFFFFFFu ? gather_prob<STORAGE>(g, cell[j]) : 0.0f;
#pragma unroll
    for (int j = 0; j < YAW_UNROLL; ++j)
      if (cell[j] != 0xFFFFFFFFu)
        acc.add(v[j]);
  }
}

// ---- yaw-only loop with the grid's floor constants (GridView::fast_idx) -------------------
// The cheaper form of weigh_chunk_yaw2: the floors use the constants mag[a], so the
// bits of the round-down FMAs weighted by the strides are the cell index with nothing
// to subtract; a rejected point gathers the zero cell stored after the grid (pad_cell)
// and is not counted, and adding +0.0 to the running sum (never below +0) leaves it
// unchanged, so the sum and the count are the reference's (Grid3d.cpp:185-195).

// Cell of one point from its coordinates X and round-down floors lo, pad_cell when the
// reference skips it; `near` marks floors that may be one cell off (the pair table
// settles them).
template <int TAB>
__device__ __forceinline__ uint32_t settle_fast(const GridView& g, const float2* tab, float2 Xxy, float Xz, float2 loxy,
                                                float loz, bool near, int& n)
{
  bool valid = (__float_as_uint(Xxy.x) < __float_as_uint(g.V[0])) &
               (__float_as_uint(Xxy.y) < __float_as_uint(g.V[1])) & (__float_as_uint(Xz) < __float_as_uint(g.V[2]));
  uint32_t idx = __float_as_uint(loxy.x) + __float_as_uint(loxy.y) * g.step_y + __float_as_uint(loz) * g.step_z;
  if (near && valid)
  {
    const int kx = locate_pair<TAB>(Xxy.x, tab, g, 0);
    const int ky = locate_pair<TAB>(Xxy.y, tab, g, 1);
    const int kz = locate_pair<TAB>(Xz, tab, g, 2);
    valid = (kx | ky | kz) >= 0;
    idx = static_cast<uint32_t>(kx) + static_cast<uint32_t>(ky) * g.step_y + static_cast<uint32_t>(kz) * g.step_z;
  }
  n += valid ? 1 : 0;
  return valid ? idx : g.pad_cell;
}

// One branch per point (the table settles a point near a cell boundary in place).
template <int STORAGE, int SUM, int TAB, int U = FAST_UNROLL>
__device__ __forceinline__ void weigh_chunk_yaw2_fast(const float4* s_pts, const float* s_z, uint32_t cnt,
                                                      const float2* s_tab, const GridView& g, const PartYaw2& q,
                                                      CloudSum<SUM>& acc)
{
  const float2 mxy = make_float2(g.mag[0], g.mag[1]);
  for (uint32_t k = 0; k < cnt; k += U)
  {
    float zs[U];
#pragma unroll
    for (int j = 0; j < U; j += 4)
    {
      const float4 z4 = *reinterpret_cast<const float4*>(s_z + k + j);
      zs[j] = z4.x;
      zs[j + 1] = z4.y;
      zs[j + 2] = z4.z;
      zs[j + 3] = z4.w;
    }
    uint32_t cell[U];
#pragma unroll
    for (int j = 0; j < U; ++j)
    {
      const float4 xxyy = s_pts[k + j];
      const float2 s01 = __fadd2_rn(__ffma2_rn(make_float2(xxyy.x, xxyy.y), q.rx, q.nz),
                                    __ffma2_rn(make_float2(xxyy.z, xxyy.w), q.ry, q.nz));
      const float2 X01 = __fadd2_rn(s01, q.h);
      const float2 lo = __ffma2_rd(X01, q.lo, mxy), hi = __ffma2_rd(X01, q.hi, mxy);
      const float Xz = fadd(zs[j], q.hz);
      const float loz = __fmaf_rd(Xz, q.loz, g.mag[2]), hiz = __fmaf_rd(Xz, q.hiz, g.mag[2]);
      const bool near = !(lo.x == hi.x) | !(lo.y == hi.y) | !(loz == hiz);
      cell[j] = settle_fast<TAB>(g, s_tab, X01, Xz, lo, loz, near, acc.n);
    }
    float v[U];
#pragma unroll
    for (int j = 0; j < U; ++j)
      v[j] = gather_prob<STORAGE>(g, cell[j]);
#pragma unroll
    for (int j = 0; j < U; ++j)
    {
      if (SUM == 0)
        acc.sum = fadd(acc.sum, v[j]);
      else
        acc.add_uncounted(v[j]);
    }
  }
}

// ---- yaw-only loop for offsets that are not floats (GridView::gen_fast) --------------------
// A map whose minimum is not a float multiple of the coordinates (any real octomap
// map) gives offsets off = double(t) - min that are not floats, and the reference's
// X = fl32(double(f) + off) is then no single float add.  With off = H + L (H its float
// rounding, L the float rounding of the rest) the float estimate v = (f + H) + L lies
// within 3.125 * 2^-24 * |v| + 2^-47 * |H| of X; so wherever |v| >= 2^-20 * |H| the
// reference's cell lies between the floors of v against 1/res bracketed 2^-22 relative
// below and above (GridView::inv_lo2 / inv_hi2), X has v's sign, and when the two floors
// agree they are the cell and the bounds of v are those of X (every axis's bound being
// the threshold of its last cell).  Points near 0 or whose floors disagree take the
// reference's X from a float two-sum (gen_exact_x), after the group's other points.
struct PartYawG
{
  float2 rx, ry;  // (r00, r10), (r01, r11)
  float2 h, l;    // (H_x, H_y), (L_x, L_y)
  float zb;       // 2^-20 max_a |H_a|: |v| below it on any axis takes the exact path
  float2 nz;      // (-0.0, -0.0), opaque to the compiler
  float hz, lz;
};

__device__ __forceinline__ PartYawG gen_yaw(const GridView& g, const PartXf& p)
{
  PartYawG q;
  q.rx = make_float2(p.r[0], p.r[3]);
  q.ry = make_float2(p.r[1], p.r[4]);
  q.h = make_float2(p.H[0], p.H[1]);
  q.l = make_float2(p.L[0], p.L[1]);
  q.zb = ldexpf(fmaxf(fmaxf(fabsf(p.H[0]), fabsf(p.H[1])), fabsf(p.H[2])), -20);
  q.nz = make_float2(g.neg_zero, g.neg_zero);
  q.hz = p.H[2];
  q.lz = p.L[2];
  return q;
}

// The reference's X = fl32(double(s) + off) on one axis from float arithmetic, with
// off = H + L + r (|r| <= 2^-48 |H|): Knuth's two-sum gives a + e = s + H exactly, then
// t = fl(e + L), X = fl(a + t) and the residual w = fl((a - X) + t) (a - X is exact while
// |a| >= 2^-20 |H|), so (s + off) - X = w within 2^-24 (|w| + |t|) + |r|.  X is the
// reference's rounding unless |w| lies within twice that of half an ulp of X, X is a
// power of two, or |a| < 2^-20 |H|: then `amb` is set and the caller takes the double
// add.  L = 0 means off is the float H (make_partxf keeps L nonzero otherwise): then X is
// a = fl(s + H), which is fl32(fl64(s + H)) (ties included), and nothing is undecided.
__device__ __forceinline__ float gen_exact_x(float s, float H, float L, bool& amb)
{
  const float a = fadd(s, H);
  const float bv = fsub(a, s);
  const float av = fsub(a, bv);
  const float e = fadd(fsub(s, av), fsub(H, bv));
  const float t = fadd(e, L);
  const float X = fadd(a, t);
  const float w = fadd(fsub(a, X), t);
  const uint32_t xb = __float_as_uint(X) & 0x7FFFFFFFu;
  const float half_ulp = __uint_as_float((xb & 0x7F800000u) - (24u << 23));
  const float margin = fadd(fmul(fadd(fabsf(w), fabsf(t)), 1.1920928955078125e-07f),   // 2^-23
                            fmul(fabsf(H), 7.105427357601002e-15f));                   // 2^-47
  amb |= (L != 0.0f) & (!(fabsf(fsub(fabsf(w), half_ulp)) > margin) | ((xb & 0x007FFFFFu) == 0u) |
                        (xb < 0x0D000000u) | !(fabsf(a) >= fmul(fabsf(H), 9.5367431640625e-07f)));  // 2^-20
  return X;
}

// The reference's X on one axis: fl32(double(s) + (double(t) - min)) (Grid3d.cpp:155-157).
// Out of line, so that the double arithmetic is branched around rather than issued,
// predicated off, for every open point.
static __device__ __noinline__ float reference_x(float s, float t, double mn)
{
  return __double2float_rn(__dadd_rn(static_cast<double>(s), __dsub_rn(static_cast<double>(t), mn)));
}

// The reference's cell of a point that the widened floors left open (`near`), or
// 0xFFFFFFFF where the reference rejects it: X per axis from gen_exact_x, or from the
// reference's double add where that cannot decide.  Out of line with scalar arguments
// and the grid by address (a __grid_constant__ kernel parameter), so that the loop
// around it keeps its registers for the common case.
template <int TAB>
static __device__ __noinline__ uint32_t open_cell(const GridView* gp, const float2* tab, float sx, float sy, float sz,
                                                  float hx, float hy, float hz, float lx, float ly, float lz,
                                                  const float4* pose, uint32_t p)
{
  const GridView& g = *gp;
  bool amb = false;
  float X[3] = { gen_exact_x(sx, hx, lx, amb), gen_exact_x(sy, hy, ly, amb), gen_exact_x(sz, hz, lz, amb) };
  if (amb)
  {
    const float4 t = pose[p];
    X[0] = reference_x(sx, t.x, g.min[0]);
    X[1] = reference_x(sy, t.y, g.min[1]);
    X[2] = reference_x(sz, t.z, g.min[2]);
  }
  const int kx = locate_pair<TAB>(X[0], tab, g, 0);
  const int ky = locate_pair<TAB>(X[1], tab, g, 1);
  const int kz = locate_pair<TAB>(X[2], tab, g, 2);
  if ((kx | ky | kz) < 0)
    return 0xFFFFFFFFu;
  return static_cast<uint32_t>(kx) + static_cast<uint32_t>(ky) * g.step_y + static_cast<uint32_t>(kz) * g.step_z;
}

template <int STORAGE, int SUM, int TAB>
__device__ __forceinline__ void weigh_chunk_yaw2_gen(const float4* s_pts, const float* s_z, uint32_t cnt,
                                                     const float2* s_tab, const GridView& g, const PartYawG& q,
                                                     const float4* pose, uint32_t p, CloudSum<SUM>& acc)
{
  const float2 mxy = make_float2(g.mag[0], g.mag[1]);
  const float2 ilo = make_float2(g.inv_lo2[0], g.inv_lo2[1]), ihi = make_float2(g.inv_hi2[0], g.inv_hi2[1]);
  for (uint32_t k = 0; k < cnt; k += GEN_UNROLL)
  {
    float zs[GEN_UNROLL];
#pragma unroll
    for (int j = 0; j < GEN_UNROLL; j += 4)
    {
      const float4 z4 = *reinterpret_cast<const float4*>(s_z + k + j);
      zs[j] = z4.x;
      zs[j + 1] = z4.y;
      zs[j + 2] = z4.z;
      zs[j + 3] = z4.w;
    }
    uint32_t cell[GEN_UNROLL];
    uint32_t open = 0;  // points whose floors leave the cell open, fixed after the group
#pragma unroll
    for (int j = 0; j < GEN_UNROLL; ++j)
    {
      const float4 xxyy = s_pts[k + j];
      const float2 s01 = __fadd2_rn(__ffma2_rn(make_float2(xxyy.x, xxyy.y), q.rx, q.nz),
                                    __ffma2_rn(make_float2(xxyy.z, xxyy.w), q.ry, q.nz));
      const float2 v01 = __fadd2_rn(__fadd2_rn(s01, q.h), q.l);
      const float vz = fadd(fadd(zs[j], q.hz), q.lz);
      const float2 lo = __ffma2_rd(v01, ilo, mxy), hi = __ffma2_rd(v01, ihi, mxy);
      const float loz = __fmaf_rd(vz, g.inv_lo2[2], g.mag[2]), hiz = __fmaf_rd(vz, g.inv_hi2[2], g.mag[2]);
      const bool near = !(lo.x == hi.x) | !(lo.y == hi.y) | !(loz == hiz) | (fabsf(v01.x) < q.zb) |
                        (fabsf(v01.y) < q.zb) | (fabsf(vz) < q.zb);
      const bool valid = (__float_as_uint(v01.x) < __float_as_uint(g.V[0])) &
                         (__float_as_uint(v01.y) < __float_as_uint(g.V[1])) &
                         (__float_as_uint(vz) < __float_as_uint(g.V[2])) & !near;
      const uint32_t idx =
          __float_as_uint(lo.x) + __float_as_uint(lo.y) * g.step_y + __float_as_uint(loz) * g.step_z;
      acc.n += valid ? 1 : 0;
      cell[j] = valid ? idx : g.pad_cell;
      open |= near ? (1u << j) : 0u;
    }
    if (open)
    {
#pragma unroll
      for (int j = 0; j < GEN_UNROLL; ++j)
      {
        if (open & (1u << j))
        {
          const float4 xxyy = s_pts[k + j];
          const float2 s01 = __fadd2_rn(__ffma2_rn(make_float2(xxyy.x, xxyy.y), q.rx, q.nz),
                                        __ffma2_rn(make_float2(xxyy.z, xxyy.w), q.ry, q.nz));
          const uint32_t idx = open_cell<TAB>(&g, s_tab, s01.x, s01.y, zs[j], q.h.x, q.h.y, q.hz, q.l.x, q.l.y,
                                              q.lz, pose, p);
          const bool ok = idx != 0xFFFFFFFFu;
          acc.n += ok ? 1 : 0;
          cell[j] = ok ? idx : g.pad_cell;
        }
      }
    }
    float v[GEN_UNROLL];
#pragma unroll
    for (int j = 0; j < GEN_UNROLL; ++j)
      v[j] = gather_prob<STORAGE>(g, cell[j]);
#pragma unroll
    for (int j = 0; j < GEN_UNROLL; ++j)
    {
      if (SUM == 0)
        acc.sum = fadd(acc.sum, v[j]);
      else
        acc.add_uncounted(v[j]);
    }
  }
}

// Point-parallel weighting (a warp = 32 particles, one per lane, over `npts` staged
// points from k0): each lane writes its particle's cell probability, or -1 for a
// point the reference skips, to out[(base + k) * 32] for k < cnt, the
// [tile][point][lane] slab that an in-order pass sums afterwards.
template <int STORAGE, int MODE, int TAB>
__device__ __forceinline__ void tile_values(const float4* s_pts, uint32_t k0, uint32_t npts, uint32_t cnt,
                                            const float2* s_tab, const GridView& g, const PartXf& xf, float* out,
                                            uint32_t base)
{
  for (uint32_t kk = 0; kk < npts; kk += UNROLL)
  {
    uint32_t cell[UNROLL];
#pragma unroll
    for (int j = 0; j < UNROLL; ++j)
    {
      const float4 s = s_pts[k0 + kk + j];
      cell[j] = cell_of_point<MODE, TAB>(g, s_tab, xf, s.x, s.y, s.z);
    }
#pragma unroll
    for (int j = 0; j < UNROLL; ++j)
    {
      const uint32_t k = k0 + kk + j;
      if (k >= cnt)
        continue;
      const float v = cell[j] != 0xFFFFFFFFu ? gather_prob<STORAGE>(g, cell[j]) : -1.0f;
      out[static_cast<uint64_t>(base + k) * 32] = v;
    }
  }
}

// The in-order pass over one lane's column of a [point][lane] slab of n points:
// the reference's running sum of the probabilities (skipped points are -1).  Loads
// bypass L1 (the slab was written by other blocks).
template <int SUM>
__device__ __forceinline__ void slab_sum(const float* slab, uint32_t n, CloudSum<SUM>& acc)
{
  constexpr uint32_t U = 16;
  uint32_t k = 0;
  for (; k + U <= n; k += U)
  {
    float v[U];
#pragma unroll
    for (uint32_t j = 0; j < U; ++j)
      v[j] = __ldcg(slab + static_cast<uint64_t>(k + j) * 32);
#pragma unroll
    for (uint32_t j = 0; j < U; ++j)
      if (v[j] >= 0.0f)
        acc.add(v[j]);
  }
  for (; k < n; ++k)
  {
    const float v = __ldcg(slab + static_cast<uint64_t>(k) * 32);
    if (v >= 0.0f)
      acc.add(v);
  }
}

// Block-wide exact sums of (a, b) added to the grid-wide digit accumulators.
__device__ __forceinline__ void block_exact_pair(float va, float vb, bool take, unsigned long long* acc_a,
                                                 unsigned long long* acc_b, X320* s_part)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  X320 xa = take ? x320_from_float(va) : x320_zero();
  X320 xb = take ? x320_from_float(vb) : x320_zero();
  xa = x320_warp_sum(xa);
  xb = x320_warp_sum(xb);
  if (lane == 0)
  {
    s_part[2 * wid] = xa;
    s_part[2 * wid + 1] = xb;
  }
  __syncthreads();
  if (wid == 0)
  {
    X320 ta = lane < nw ? s_part[2 * lane] : x320_zero();
    X320 tb = lane < nw ? s_part[2 * lane + 1] : x320_zero();
    ta = x320_warp_sum(ta);
    tb = x320_warp_sum(tb);
    if (lane == 0)
    {
      if (acc_a)
        x320_atomic_add(acc_a, ta);
      if (acc_b)
        x320_atomic_add(acc_b, tb);
    }
  }
}


// Copies the grid's locate thresholds into shared memory (all threads of the block),
// as single floats: axis a's T[0..size+1] at float offset toff[a] + a (T[size+1] = +inf
// from the last pair's upper half), table_staged_floats(g) floats in all.  Half the
// bytes of the pairs leaves the SM's L1 more room for the cell gathers.
__device__ __forceinline__ void load_tables(const GridView& g, float2* s_tab)
{
  float* sT = reinterpret_cast<float*>(s_tab);
  const uint32_t ntab = table_entries(g);
  for (uint32_t i = threadIdx.x; i < ntab; i += blockDim.x)
  {
    const int a = i >= g.toff[2] ? 2 : (i >= g.toff[1] ? 1 : 0);
    const float2 t = g.T2[i];
    sT[i + a] = t.x;
    if (i == g.toff[a] + g.size[a])
      sT[i + a + 1] = t.y;
  }
}

// FS (chosen by the launcher, fast_variant): 1 = the grid has floor constants and a zero
// minimum (every offset a float), so yaw-only warps take weigh_chunk_yaw2_fast; 2 = the
// grid has the general loop's constants (GridView::gen_fast) and a non-zero minimum, so
// every yaw-only point takes weigh_chunk_yaw2_gen; 0 = neither.
// One block of particles [p0, p0 + blockDim) of one filter, one thread per particle
// over the whole cloud in cloud order (the fused weighting).  The caller has loaded
// s_tab (when a.N > 0) and s_rg.  s_pts holds `chunk` float4 (a multiple of UNROLL):
// as many points per stage, or 4/5 as many (a multiple of YAW_UNROLL) in the yaw-only
// staging.  Every thread of the block must call this.
template <int STORAGE, int SUM, int TAB, int FS = 0, int U = FAST_UNROLL>
__device__ __forceinline__ void weigh_block(const WeightArgs& a, const GridView& g, uint32_t p0, uint32_t chunk,
                                            float4* s_pts, const float4* s_rg, X320* s_part, const float2* s_tab)
{
  const uint32_t p = p0 + threadIdx.x;
  const bool active = p < a.P;
  float4 pose = make_float4(0.f, 0.f, 0.f, 0.f);
  if (active)
    pose = a.pose[p];
  const bool inm = active && (a.ignore_map || into_map(g, pose.x, pose.y, pose.z));
  PartXf xf;
  xf.exact = 1;
  if (inm)
    make_partxf(g, a.sr, a.cr, a.sp, a.cp, pose.x, pose.y, pose.z, pose.w, xf);
  // Transform mode, uniform per warp.
  const bool warp_exact = __all_sync(0xFFFFFFFFu, xf.exact != 0);
  const int mode = warp_exact ? (a.yaw_only ? XF_YAW : XF_EXACT) : XF_GENERAL;

  // Yaw-only filters stage (x, x, y, y) and z separately: 20 B per point, so a
  // chunk holds 4/5 as many points in the same shared memory.
  const bool yl = a.yaw_only != 0;
  const uint32_t al = yl ? YAW_UNROLL : UNROLL;  // padding of a staged chunk (NaN points)
  const uint32_t ch = yl ? (chunk * 4 / 5) / al * al : chunk;
  float* s_z = reinterpret_cast<float*>(s_pts + ch);
  PartYaw2 q{};
  if (inm && mode == XF_YAW)
    q = pair_yaw(g, xf);
  PartYawG qg{};
  if (FS == 2 && inm && yl)
    qg = gen_yaw(g, xf);

  CloudSum<SUM> acc;
  for (uint32_t base = 0; base < a.N; base += ch)
  {
    const uint32_t cnt = min(ch, a.N - base);
    const uint32_t cnt8 = (cnt + al - 1) / al * al;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < cnt8; i += blockDim.x)
    {
      const float nan = __int_as_float(0x7FC00000);
      const float4 c = i < cnt ? stage_point(a.cloud[base + i], yl) : make_float4(nan, nan, nan, 0.0f);
      if (yl)
      {
        s_pts[i] = make_float4(c.x, c.x, c.y, c.y);
        s_z[i] = c.z;
      }
      else
      {
        s_pts[i] = c;
      }
    }
    __syncthreads();
    if (!inm)
      continue;
    if (FS == 1 && mode == XF_YAW)
      weigh_chunk_yaw2_fast<STORAGE, SUM, TAB, U>(s_pts, s_z, cnt8, s_tab, g, q, acc);
    else if (FS == 2 && yl)
      weigh_chunk_yaw2_gen<STORAGE, SUM, TAB>(s_pts, s_z, cnt8, s_tab, g, qg, a.pose, p, acc);
    else if (mode == XF_YAW)
      weigh_chunk_yaw2<STORAGE, SUM, TAB>(s_pts, s_z, cnt8, s_tab, g, q, acc);
    else if (mode == XF_EXACT)
      weigh_chunk<STORAGE, SUM, XF_EXACT, false, TAB>(s_pts, s_z, cnt8, s_tab, g, xf, acc);
    else if (yl)
      weigh_chunk<STORAGE, SUM, XF_GENERAL, true, TAB>(s_pts, s_z, cnt8, s_tab, g, xf, acc);
    else
      weigh_chunk<STORAGE, SUM, XF_GENERAL, false, TAB>(s_pts, s_z, cnt8, s_tab, g, xf, acc);
  }
  float wpv = 0.0f, wrv = 0.0f;
  if (inm)
  {
    wpv = acc.weight();
    wrv = range_weight(pose.x, pose.y, pose.z, s_rg, static_cast<int>(a.nr), a.k1, a.k2);
    a.wp[p] = wpv;
    a.wr[p] = wrv;
  }
  if (active && a.inmap)
    a.inmap[p] = inm ? 1 : 0;
  if (a.acc_wp || a.acc_wr)
  {
    __syncthreads();
    block_exact_pair(wpv, wrv, inm, a.acc_wp, a.acc_wr, s_part);
  }
}

}  // namespace amcl
