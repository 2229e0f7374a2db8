// Per-point arithmetic of Grid3d::computeCloudWeight (amcl3d/src/Grid3d.cpp:133-199),
// reproduced bit for bit in float arithmetic on the GPU.
//
// The reference computes, per scan point s and particle (t, yaw):
//   f   = (s.x*r00 + s.y*r01) + (s.z + 0)*r02          float, no FMA  (Grid3d.cpp:174)
//   X   = (float)((double)f + (double(t.x) - min.x))   one double add  (Grid3d.cpp:155,174)
//   ok  = X >= 0 && X < (max.x - min.x)                double compare  (Grid3d.cpp:178)
//   ix  = (uint32)floor((double)X / res)               double divide   (Grid3d.cpp:181)
//   ok &= ix < size_x                                                  (Grid3d.cpp:185)
// FP64 runs at a small fraction of the FP32 rate on GB300, so the hot loop avoids
// it:
//  * the divide/floor/compare chain is replaced by exact float comparisons against a
//    per-axis table T[k] = the smallest float X with floor(fl64(X / res)) >= k and a
//    bound V = the smallest float X that fails a bound check (both computed on the
//    host with the reference's own double arithmetic); the kernels keep the table
//    as pairs (T[k], T[k+1]) so one 64-bit shared load settles a cell;
//  * when the particle's offset double(t) - min is exactly a float (always when the
//    map minimum is 0, and whenever the subtraction happens to be exact), the double
//    add of two floats followed by the rounding to float is exactly the float add, so
//    X = s + H in one instruction;
//  * otherwise the double add is evaluated as a float-float sum (the offset split
//    into H + L, Knuth's two-sum), which lands within one float ulp of the exact X;
//    when any threshold lies within a safe margin of that estimate the point takes
//    the exact FP64 path (one double add and a rounding);
//  * with roll = pitch = 0 the products with the zero rotation coefficients only ever
//    change the sign of a zero sum, which moves no point to another cell, so they are
//    skipped (non-finite points, which those products turn into NaN, are rejected
//    explicitly instead).
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/amcl3d_gpu.h"

namespace amcl
{
// Device view of one grid, passed by value to the weighting kernels.
struct GridView
{
  const float* prob_f32;
  const __half* prob_f16;
  const uint8_t* prob_u8;
  float u8_scale;
  int storage;  // AMCL_GRID_*
  uint32_t size[3];
  uint32_t step_y, step_z;
  // isIntoMap as float compares: x >= lo[a] && x < hi[a]  (Grid3d.cpp:207)
  float in_lo[3], in_hi[3];
  // locate tables: (T[k], T[k+1]) for k = 0..size (T[size+1] = +inf), per axis at toff[a]
  const float2* T2;
  uint32_t toff[3];
  float V[3];
  float inv_res[3];
  // 1/res bracketed by floats a little more than 2^-53 relative below and above it
  // (inv_hi = +inf on an axis of 2^21 cells or more)
  float inv_lo[3], inv_hi[3];
  float neg_zero;  // -0.0f, read at run time (see PartYaw2)
  double min[3];
  uint64_t cells;
  int built;
  // Floor constants of the yaw-only loop: mag[a] = 2^23 + m[a] with
  // sum_a bits(mag[a]) * stride[a] = 0 (mod 2^32), strides (1, step_y, step_z), so the
  // bits of fma_rd(X[a], inv_lo[a], mag[a]) = bits(mag[a]) + floor(X[a] * inv_lo[a]),
  // weighted by the strides, sum to the cell index itself with no bias to remove.
  float mag[3];
  uint32_t pad_cell;  // index of the zero cell stored after the last cell of every prob array
  int fast_idx;       // mag[] exists and pad_cell < 2^32
  // The yaw-only loop for offsets that are not floats (weigh_chunk_yaw2_gen): 1/res
  // bracketed 2^-22 relative below and above, wide enough for the float estimate of a
  // transformed coordinate; usable when every axis's bound V is the threshold of its
  // last cell (V = T[size], so the cell range decides the bounds) and is below 2^21 cells.
  float inv_lo2[3], inv_hi2[3];
  int gen_fast;
};

// Per-particle constants of the transform.
struct PartXf
{
  float r[9];
  float H[3], L[3];
  double off[3];
  // All three offsets are exact floats (off == H): then fl64(s + H) is the exact sum
  // of two floats, or rounds only bits far below the float rounding point, so
  // X = fl32(fl64(s + H)) equals the single float add s + H.
  int exact;
};

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// Rotation of Grid3d.cpp:139-149 with the float overloads of sin/cos (what a ROS
// build gets through <math.h>); sin/cos of the yaw are the double functions
// rounded to float.
__device__ __forceinline__ void make_rotation(float sr, float cr, float sp, float cp, float yaw, float r[9])
{
  double sd, cd;
  sincos(static_cast<double>(yaw), &sd, &cd);
  const float sy = __double2float_rn(sd), cy = __double2float_rn(cd);
  r[0] = fmul(cy, cp);
  r[1] = fsub(fmul(fmul(cy, sp), sr), fmul(sy, cr));
  r[2] = fadd(fmul(fmul(cy, sp), cr), fmul(sy, sr));
  r[3] = fmul(sy, cp);
  r[4] = fadd(fmul(fmul(sy, sp), sr), fmul(cy, cr));
  r[5] = fsub(fmul(fmul(sy, sp), cr), fmul(cy, sr));
  r[6] = -sp;
  r[7] = fmul(cp, sr);
  r[8] = fmul(cp, cr);
}

__device__ __forceinline__ void make_partxf(const GridView& g, float sr, float cr, float sp, float cp, float tx,
                                            float ty, float tz, float yaw, PartXf& p)
{
  make_rotation(sr, cr, sp, cp, yaw, p.r);
  const float t[3] = { tx, ty, tz };
#pragma unroll
  for (int a = 0; a < 3; ++a)
  {
    const double off = __dsub_rn(static_cast<double>(t[a]), g.min[a]);  // Grid3d.cpp:155-157
    p.off[a] = off;
    p.H[a] = fadd(__double2float_rn(off), 0.0f);  // -0.0 becomes +0.0: the same cell, never a -0.0 sum
    // L = 0 exactly when off is the float H (a rest below the smallest subnormal keeps it)
    const double rest = __dsub_rn(off, static_cast<double>(p.H[a]));
    const float L = __double2float_rn(rest);
    p.L[a] = (L == 0.0f && rest != 0.0) ? copysignf(1.401298464324817e-45f, static_cast<float>(rest)) : L;
  }
  p.exact = (p.off[0] == static_cast<double>(p.H[0]) && p.off[1] == static_cast<double>(p.H[1]) &&
             p.off[2] == static_cast<double>(p.H[2]) && isfinite(p.H[0]) && isfinite(p.H[1]) && isfinite(p.H[2]))
                ? 1
                : 0;
}

// Locate-table entries staged in shared memory by the weighting kernels (32 KB as
// single floats, load_tables).  A grid with more (its three sizes summing above about 8,190 cells)
// keeps its table in global memory: the table is read only for points near a cell
// boundary, and staging it would cost occupancy or not fit at all.
constexpr uint32_t SMEM_TABLE_MAX = 8192;

__host__ __device__ __forceinline__ uint32_t table_entries(const GridView& g)
{
  return g.size[0] + g.size[1] + g.size[2] + 3;
}
__host__ __device__ __forceinline__ bool tables_staged(const GridView& g) { return table_entries(g) <= SMEM_TABLE_MAX; }
// Floats of the shared-memory copy (load_tables): size + 2 thresholds per axis.
__host__ __device__ __forceinline__ uint32_t table_staged_floats(const GridView& g) { return table_entries(g) + 3; }

// Where a kernel reads the locate tables: its shared-memory copy, global memory, or
// whichever tables_staged(g) says (a branch, taken only near cell boundaries).  The
// hot kernels fix it at compile time: a run-time choice between the two in the hot
// loop costs a few percent even though the loads are rare.
enum : int
{
  TAB_SHARED = 0,
  TAB_GLOBAL = 1,
  TAB_EITHER = 2
};

// Pair (T[k], T[k+1]) of axis a (typed loads, so the shared copy keeps its address
// space): two adjacent floats of the staged copy, or one pair from global memory.
template <int TAB>
__device__ __forceinline__ float2 table_pair(const float2* s_tab, const GridView& g, int a, int k)
{
  if (TAB == TAB_SHARED || (TAB == TAB_EITHER && tables_staged(g)))
  {
    const float* sT = reinterpret_cast<const float*>(s_tab);
    const int j = static_cast<int>(g.toff[a]) + a + k;
    return make_float2(sT[j], sT[j + 1]);
  }
  return __ldg(g.T2 + g.toff[a] + k);
}

// Cell index along axis a for an exact X, -1 when the reference rejects the point
// (X < 0, X >= V, NaN).  floor(X / res) in float is within one cell of the
// reference's floor(fl64(X / res)); the pair (T[k], T[k+1]) settles it exactly.
template <int TAB>
__device__ __forceinline__ int locate_pair(float X, const float2* s_tab, const GridView& g, int a)
{
  int k = __float2int_rd(fmul(X, g.inv_res[a]));
  k = min(max(k, 0), static_cast<int>(g.size[a]));
  const float2 t = table_pair<TAB>(s_tab, g, a, k);
  k = (X < t.x) ? k - 1 : ((X >= t.y) ? k + 1 : k);  // X < 0 ends at -1 (T[0] = 0)
  return (X < g.V[a]) ? k : -1;
}

// Same result as locate_pair for a valid X (0 <= X < V), reading the table only
// near a cell boundary.  inv_lo <= 1/res <= inv_hi with more than 2^-53 relative
// room on each side, and fl64 moves X / res by at most 2^-53 relative, so for X >= 0
//   floor(X * inv_lo) <= floor(fl64(X / res)) <= floor(X * inv_hi);
// when the two floors agree they are the reference's cell, otherwise (for about
// X / res * 2^-22 of the points) `near` is set and the pair table settles it.  Each
// floor is one fused multiply-add rounded toward -inf: X * inv + 1.5 * 2^23 lies in
// [2^23, 2^24), where the floats are the integers, for 0 <= X * inv < 2^22, so the
// rounded sum is 1.5 * 2^23 + floor(X * inv) exactly, read off its bit pattern.  A
// valid X keeps X * inv_hi below size + 1 < 2^22; an axis of 2^21 cells or more has
// inv_hi = +inf, which makes the floors disagree (or NaN) for every point.
__device__ __forceinline__ int floor_bracket(float X, float inv_lo, float inv_hi, bool& near)
{
  const float lo = __fmaf_rd(X, inv_lo, 12582912.0f);
  const float hi = __fmaf_rd(X, inv_hi, 12582912.0f);
  near |= !(lo == hi);
  return __float_as_int(lo) - 0x4B400000;
}

// True when a threshold lies within m of X (the estimate may then be on the wrong side).
template <int TAB>
__device__ __forceinline__ bool near_threshold(float X, int k, const float2* s_tab, const GridView& g, int a, float m)
{
  if (fabsf(X) <= m || fabsf(g.V[a] - X) <= m)
    return true;
  if (k < 0)
    return false;
  const float2 t = table_pair<TAB>(s_tab, g, a, k);
  return (X - t.x <= m) || (t.y - X <= m);
}

// Transformed coordinate, estimated in float-float; m receives the safe margin.
__device__ __forceinline__ float xform_axis(float s, float H, float L, float& m)
{
  const float a = fadd(s, H);
  const float bv = fsub(a, s);
  const float av = fsub(a, bv);
  const float br = fsub(H, bv);
  const float ar = fsub(s, av);
  const float e = fadd(ar, br);
  const float X = fadd(a, fadd(e, L));
  // |X - exact| <= 1.25 ulp(X) + 2^-47 (|s| + |H|); the margin covers it with room.
  m = fmul(fadd(fadd(fabsf(X), fabsf(H)), fabsf(s)), 2.384185791015625e-07f /* 2^-22 */);
  return X;
}

// uint32 index arithmetic of Grid3d.cpp:187; 0xFFFFFFFF marks a skipped point (a
// valid index is below the cell count, itself below 2^32).
__device__ __forceinline__ uint32_t cell_index(const GridView& g, int kx, int ky, int kz)
{
  if ((kx | ky | kz) < 0)
    return 0xFFFFFFFFu;
  return static_cast<uint32_t>(kx) + static_cast<uint32_t>(ky) * g.step_y + static_cast<uint32_t>(kz) * g.step_z;
}

// Loop variant of the fused weighting for a grid (the FS template argument): 1 when
// every offset is a float (zero minimum) and the floor constants exist, 2 when the
// minimum is not zero and the general yaw loop's constants exist, else 0.
__host__ __forceinline__ int fast_variant(const GridView& g)
{
  if (!g.fast_idx)
    return 0;
  if (g.min[0] == 0.0 && g.min[1] == 0.0 && g.min[2] == 0.0)
    return 1;
  return g.gen_fast ? 2 : 0;
}

// Point-transform modes of the weighting loops.
enum : int
{
  XF_GENERAL = 0,  // any offsets: float-float estimate + exact FP64 fallback
  XF_EXACT = 1,    // offsets are floats: X = s + H
  XF_YAW = 2       // offsets are floats and roll = pitch = 0
};

// Cell index from exact coordinates X and their bracket floors k (floor_bracket),
// 0xFFFFFFFF when the reference skips the point: the bound checks of
// Grid3d.cpp:178-179 and 185 as 0 <= X < V, one unsigned compare of the bit
// patterns per axis (X is never -0.0, H being canonicalised; negative X and NaN have
// patterns above V's), and one branch for the rare point near a cell boundary.
template <int TAB>
__device__ __forceinline__ uint32_t settle_cell(const GridView& g, const float2* tab, const float X[3], int k[3],
                                                bool near)
{
  bool valid = true;
#pragma unroll
  for (int a = 0; a < 3; ++a)
    valid &= __float_as_uint(X[a]) < __float_as_uint(g.V[a]);
  if (near && valid)
  {
#pragma unroll
    for (int a = 0; a < 3; ++a)
      k[a] = locate_pair<TAB>(X[a], tab, g, a);
    valid = (k[0] | k[1] | k[2]) >= 0;
  }
  if (!valid)
    return 0xFFFFFFFFu;
  return static_cast<uint32_t>(k[0]) + static_cast<uint32_t>(k[1]) * g.step_y + static_cast<uint32_t>(k[2]) * g.step_z;
}

// Grid cell of scan point (px, py, pz0) for the particle, 0xFFFFFFFF when the
// reference skips it.  pz0 is s.z + 0.0f (Grid3d.cpp:174-176).  `tab` is the pair
// table (in shared memory in the kernels).
template <int MODE, int TAB>
__device__ __forceinline__ uint32_t cell_of_point(const GridView& g, const float2* tab, const PartXf& p, float px,
                                                  float py, float pz0)
{
  float s[3];
  if (MODE == XF_YAW)
  {
    s[0] = fadd(fmul(px, p.r[0]), fmul(py, p.r[1]));
    s[1] = fadd(fmul(px, p.r[3]), fmul(py, p.r[4]));
    s[2] = pz0;
  }
  else
  {
    s[0] = fadd(fadd(fmul(px, p.r[0]), fmul(py, p.r[1])), fmul(pz0, p.r[2]));
    s[1] = fadd(fadd(fmul(px, p.r[3]), fmul(py, p.r[4])), fmul(pz0, p.r[5]));
    s[2] = fadd(fadd(fmul(px, p.r[6]), fmul(py, p.r[7])), fmul(pz0, p.r[8]));
  }
  int k[3];
  if (MODE != XF_GENERAL)
  {
    // X = s + H exactly (float offsets)
    float X[3];
    bool near = false;
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
      X[a] = fadd(s[a], p.H[a]);
      k[a] = floor_bracket(X[a], g.inv_lo[a], g.inv_hi[a], near);
    }
    return settle_cell<TAB>(g, tab, X, k, near);
  }
  bool amb = false;
#pragma unroll
  for (int a = 0; a < 3; ++a)
  {
    float m;
    const float X = xform_axis(s[a], p.H[a], p.L[a], m);
    k[a] = locate_pair<TAB>(X, tab, g, a);
    amb |= near_threshold<TAB>(X, k[a], tab, g, a, m);
  }
  if (amb)
  {
    // Exact path: the reference's double add, rounded to float once more.
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
      const float X = __double2float_rn(__dadd_rn(static_cast<double>(s[a]), p.off[a]));
      k[a] = locate_pair<TAB>(X, tab, g, a);
    }
  }
  return cell_index(g, k[0], k[1], k[2]);
}

// A scan point as staged in shared memory: z + 0.0f applied; in the yaw-only mode a
// point with a non-finite coordinate becomes NaN (the skipped products would have
// turned it into NaN).
__device__ __forceinline__ float4 stage_point(float4 c, bool yaw_only)
{
  c.z = fadd(c.z, 0.0f);  // (point->z + error_z), error_z = 0 (Grid3d.cpp:166,174-176)
  if (yaw_only && !(isfinite(c.x) && isfinite(c.y) && isfinite(c.z)))
    c.x = __int_as_float(0x7FC00000);
  return c;
}

// The yaw-only transform with the x and y axes paired in the two-wide float
// instructions of sm_100 and later (each half rounds as the scalar instruction): the
// same operations as cell_of_point<XF_YAW> in fewer issues.  The scan point is
// staged as (x, x, y, y) so that both products of a coordinate come from one register
// pair.  The reference rounds the two products and their sum separately, but the
// code generator contracts a two-wide multiply feeding a two-wide add into a fused
// multiply-add even when both carry an explicit round-to-nearest; so each product is
// a fused multiply-add with an addend of -0.0 that the compiler cannot see as a
// constant (GridView::neg_zero, a kernel argument).  fma(a, b, -0) is the rounded
// product a * b for every input, signed zeros included, and nothing contracts a
// fused multiply-add into a following add.
struct PartYaw2
{
  float2 rx, ry;  // (r00, r10), (r01, r11)
  float2 h;       // (H_x, H_y)
  float2 lo, hi;  // (inv_lo, inv_hi) of the x and y axes
  float2 nz;      // (-0.0, -0.0), opaque to the compiler
  float hz, loz, hiz;
};

__device__ __forceinline__ PartYaw2 pair_yaw(const GridView& g, const PartXf& p)
{
  PartYaw2 q;
  q.rx = make_float2(p.r[0], p.r[3]);
  q.ry = make_float2(p.r[1], p.r[4]);
  q.h = make_float2(p.H[0], p.H[1]);
  q.lo = make_float2(g.inv_lo[0], g.inv_lo[1]);
  q.hi = make_float2(g.inv_hi[0], g.inv_hi[1]);
  q.nz = make_float2(g.neg_zero, g.neg_zero);
  q.hz = p.H[2];
  q.loz = g.inv_lo[2];
  q.hiz = g.inv_hi[2];
  return q;
}

template <int TAB>
__device__ __forceinline__ uint32_t cell_of_point_yaw2(const GridView& g, const float2* tab, const PartYaw2& q,
                                                       float4 xxyy, float pz0)
{
  const float2 s01 = __fadd2_rn(__ffma2_rn(make_float2(xxyy.x, xxyy.y), q.rx, q.nz),
                                __ffma2_rn(make_float2(xxyy.z, xxyy.w), q.ry, q.nz));
  const float2 X01 = __fadd2_rn(s01, q.h);
  const float2 c2 = make_float2(12582912.0f, 12582912.0f);
  const float2 lo = __ffma2_rd(X01, q.lo, c2), hi = __ffma2_rd(X01, q.hi, c2);
  const float Xz = fadd(pz0, q.hz);
  const float loz = __fmaf_rd(Xz, q.loz, 12582912.0f), hiz = __fmaf_rd(Xz, q.hiz, 12582912.0f);
  const bool near = !(lo.x == hi.x) | !(lo.y == hi.y) | !(loz == hiz);
  const float X[3] = { X01.x, X01.y, Xz };
  int k[3] = { __float_as_int(lo.x) - 0x4B400000, __float_as_int(lo.y) - 0x4B400000,
               __float_as_int(loz) - 0x4B400000 };
  return settle_cell<TAB>(g, tab, X, k, near);
}

template <int STORAGE>
__device__ __forceinline__ float gather_prob(const GridView& g, uint32_t idx)
{
  if (STORAGE == AMCL_GRID_F32)
    return __ldg(g.prob_f32 + idx);
  else if (STORAGE == AMCL_GRID_F16)
    return __half2float(__ldg(g.prob_f16 + idx));
  else
    return fmul(static_cast<float>(__ldg(g.prob_u8 + idx)), g.u8_scale);
}

// isIntoMap (Grid3d.cpp:201-208) as exact float compares.
__device__ __forceinline__ bool into_map(const GridView& g, float x, float y, float z)
{
  return g.built && x >= g.in_lo[0] && x < g.in_hi[0] && y >= g.in_lo[1] && y < g.in_hi[1] && z >= g.in_lo[2] &&
         z < g.in_hi[2];
}

}  // namespace amcl
