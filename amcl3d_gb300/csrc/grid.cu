// Grid3d on the device: the distance field (computeGrid), its reduced-precision
// copies, the z-slice message, the .grid file and isIntoMap.
//
// Device layout in HBM: two separate cell arrays in the reference's linear order
// (ix + iy*size_x + iz*size_x*size_y, Grid3d.cpp:187): `prob` (4 B/cell, the
// only array the filter gathers) and `dist` (4 B/cell, kept for parity and for
// the .grid file).  Optional FP16 (2 B/cell) and uint8 (1 B/cell) copies of
// `prob` shrink the gather footprint.
#include <cfloat>
#include <cmath>
#include <cstring>

#include "grid.cuh"

using namespace amcl;

namespace amcl
{
// ---- host helpers: float thresholds equal to the reference's double compares -------

// Smallest float F with F >= v (v finite).
static float float_ceil(double v)
{
  float f = static_cast<float>(v);
  if (static_cast<double>(f) < v)
    f = std::nextafter(f, INFINITY);
  while (true)
  {
    const float d = std::nextafter(f, -INFINITY);
    if (static_cast<double>(d) >= v)
      f = d;
    else
      break;
  }
  return f;
}

// Smallest float X >= 0 with floor((double)X / res) >= k (Grid3d.cpp:181-183).
static float table_threshold(double res, uint32_t k)
{
  if (k == 0)
    return 0.0f;
  auto ok = [&](float x) { return std::floor(static_cast<double>(x) / res) >= static_cast<double>(k); };
  float x = static_cast<float>(static_cast<double>(k) * res);
  while (!ok(x))
    x = std::nextafter(x, INFINITY);
  while (true)
  {
    const float d = std::nextafter(x, -INFINITY);
    if (d >= 0.0f && ok(d))
      x = d;
    else
      break;
  }
  return x;
}

// Floor constants mag[a] = 2^23 + m[a] of the hot loop: with B = bits(2^23) =
// 0x4B000000 the index sum_a (B + m[a] + k[a]) * stride[a] equals
// sum_a k[a] * stride[a] (mod 2^32) when sum_a m[a] * stride[a] = R = -B * (1 + sy + sz);
// R is written in the mixed radix of the strides (m2 = R / sz, m1 = (R % sz) / sy,
// m0 = R % sy).  Each m[a] must leave room for the floors of a valid coordinate (up to
// size + 1 cells below 2^23 past the constant), which holds whenever
// size_x * size_y >= 1024 and every axis is below 2^22 cells.
static void grid_floor_constants(GridView& v)
{
  const uint64_t two32 = 1ull << 32;
  const uint64_t sy = v.step_y, sz = v.step_z;
  v.fast_idx = 0;
  v.pad_cell = 0;
  for (int a = 0; a < 3; ++a)
    v.mag[a] = 12582912.0f;
  if (v.cells == 0 || v.cells >= two32 - 1 || sy == 0 || sz == 0 || sz >= two32)
    return;
  const uint64_t B = 0x4B000000ull;
  const uint64_t R = (two32 - (B * ((1 + sy + sz) % two32)) % two32) % two32;
  const uint64_t m2 = R / sz, r2 = R % sz;
  const uint64_t m1 = r2 / sy, m0 = r2 % sy;
  const uint64_t m[3] = { m0, m1, m2 };
  for (int a = 0; a < 3; ++a)
    if (m[a] + v.size[a] + 2 > (1ull << 23))
      return;
  uint64_t chk = 0;
  const uint64_t stride[3] = { 1, sy, sz };
  for (int a = 0; a < 3; ++a)
    chk = (chk + ((B + m[a]) % two32) * stride[a]) % two32;
  if (chk != 0)
    return;
  for (int a = 0; a < 3; ++a)
    v.mag[a] = static_cast<float>(8388608.0 + static_cast<double>(m[a]));
  v.pad_cell = static_cast<uint32_t>(v.cells);
  v.fast_idx = 1;
}

size_t grid_table_floats(const amcl_grid_s* g)
{
  return static_cast<size_t>(g->info.size[0]) + g->info.size[1] + g->info.size[2] + 3;
}

int grid_prepare_view(amcl_grid_s* g)
{
  GridView& v = g->view;
  const amcl_grid_info& in = g->info;
  g->tabs_host.assign(grid_table_floats(g), 0.0f);
  uint32_t off = 0;
  for (int a = 0; a < 3; ++a)
  {
    v.size[a] = in.size[a];
    v.toff[a] = off;
    for (uint32_t k = 0; k <= in.size[a]; ++k)
      g->tabs_host[off + k] = table_threshold(in.resolution, k);
    const double octo_size = in.max[a] - in.min[a];  // Grid3d.cpp:151-153
    const float U = float_ceil(octo_size);
    const float Tsz = g->tabs_host[off + in.size[a]];
    v.V[a] = std::min(U, Tsz);
    const double ir = 1.0 / in.resolution;
    v.inv_res[a] = static_cast<float>(ir);
    // 1/res is rounded by at most 2^-53 relative in ir; 2^-50 of room covers it
    float lo = v.inv_res[a], hi = v.inv_res[a];
    while (static_cast<double>(lo) > ir * (1.0 - std::ldexp(1.0, -50)))
      lo = std::nextafter(lo, 0.0f);
    while (static_cast<double>(hi) < ir * (1.0 + std::ldexp(1.0, -50)))
      hi = std::nextafter(hi, INFINITY);
    v.inv_lo[a] = lo;
    v.inv_hi[a] = in.size[a] < (1u << 21) ? hi : INFINITY;
    float lo2 = v.inv_res[a], hi2 = v.inv_res[a];
    while (static_cast<double>(lo2) > ir * (1.0 - std::ldexp(1.0, -22)))
      lo2 = std::nextafter(lo2, 0.0f);
    while (static_cast<double>(hi2) < ir * (1.0 + std::ldexp(1.0, -22)))
      hi2 = std::nextafter(hi2, INFINITY);
    v.inv_lo2[a] = lo2;
    v.inv_hi2[a] = hi2;
    v.min[a] = in.min[a];
    v.in_lo[a] = float_ceil(in.min[a]);
    v.in_hi[a] = float_ceil(in.max[a]);
    off += in.size[a] + 1;
  }
  v.neg_zero = -0.0f;
  v.step_y = in.size[0];
  v.step_z = in.size[0] * in.size[1];
  v.cells = g->cells();
  grid_floor_constants(v);
  v.gen_fast = v.fast_idx;
  for (int a = 0; a < 3; ++a)
    if (in.size[a] >= (1u << 20) || v.V[a] != g->tabs_host[v.toff[a] + in.size[a]])
      v.gen_fast = 0;
  // Pairs (T[k], T[k+1]) per axis, T[size+1] = +inf: one 64-bit load settles a cell.
  std::vector<float2> pairs(g->tabs_host.size());
  for (int a = 0; a < 3; ++a)
    for (uint32_t k = 0; k <= in.size[a]; ++k)
      pairs[v.toff[a] + k] = make_float2(g->tabs_host[v.toff[a] + k],
                                         k < in.size[a] ? g->tabs_host[v.toff[a] + k + 1] : INFINITY);
  int rc = g->tabs.ensure(pairs.size() * sizeof(float2));
  if (rc)
    return rc;
  AMCL_CUDA_TRY(cudaMemcpyAsync(g->tabs.p, pairs.data(), pairs.size() * sizeof(float2), cudaMemcpyHostToDevice,
                                g->st.s));
  v.T2 = g->tabs.as<float2>();
  v.prob_f32 = g->prob.as<float>();
  v.prob_f16 = g->prob16.as<__half>();
  v.prob_u8 = g->prob8.as<uint8_t>();
  v.u8_scale = in.u8_scale;
  v.storage = static_cast<int>(in.storage);
  v.built = g->built ? 1 : 0;
  AMCL_CUDA_TRY(cudaStreamSynchronize(g->st.s));
  return AMCL_OK;
}

void grid_apply_l2_window(amcl_grid_s* g, cudaStream_t s)
{
  cudaStreamAttrValue attr;
  std::memset(&attr, 0, sizeof(attr));
  if (g->l2_window && g->built)
  {
    int dev = 0, maxw = 0, maxp = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxAccessPolicyWindowSize, dev);
    cudaDeviceGetAttribute(&maxp, cudaDevAttrMaxPersistingL2CacheSize, dev);
    const void* base = g->info.storage == AMCL_GRID_F16 ? g->prob16.p
                       : g->info.storage == AMCL_GRID_U8 ? g->prob8.p
                                                         : g->prob.p;
    const size_t elem = g->info.storage == AMCL_GRID_F16 ? 2 : g->info.storage == AMCL_GRID_U8 ? 1 : 4;
    const size_t bytes = static_cast<size_t>(g->cells()) * elem;
    const size_t win = std::min<size_t>(bytes, static_cast<size_t>(maxw));
    if (maxp > 0)
      cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, static_cast<size_t>(maxp));
    attr.accessPolicyWindow.base_ptr = const_cast<void*>(base);
    attr.accessPolicyWindow.num_bytes = win;
    attr.accessPolicyWindow.hitRatio =
        win ? std::min(1.0f, static_cast<float>(maxp) / static_cast<float>(win)) : 0.0f;
    attr.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attr.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
  }
  cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &attr);
  cudaGetLastError();
}
}  // namespace amcl

// ---- distance field: exact nearest occupied point per cell corner ----------------------
//
// computeGrid (PointCloudTools.cpp:84-149) asks a FLANN kd-tree for the nearest
// occupied leaf centre of every cell corner min + i*res (as float) and stores the
// squared distance, accumulated in float as ((0 + dx*dx) + dy*dy) + dz*dz
// (flann::L2_Simple over pcl::PointXYZ), plus prob = c1 * expf(-d2*d2*c2).
//
// Here: points are bucketed in cubes of DF_B^3 cells; one warp owns DF_LPW z-layers of
// a DF_B^3 brick (2 * DF_LPW cells per lane, sharing their x) and scans the buckets on
// the surface of each Chebyshev ring around the brick with warp-uniform (broadcast)
// point loads, skipping buckets whose box is farther from every cell than each cell's
// best, and stopping once every cell's best squared distance is below the squared
// distance to the first unscanned ring.  The minimum of the same float expression
// over all points is exact: the bounds keep margins far above float rounding.

namespace
{
constexpr int DF_B = 8;

struct DFGeom
{
  int nb[3];       // buckets per axis
  double min[3];   // map min
  double bsize;    // bucket edge in metres
  uint64_t nbtot;
};

__global__ void k_df_count(const float* __restrict__ xyz, uint64_t n, uint32_t stride, DFGeom gm,
                           uint32_t* __restrict__ counts, uint32_t* __restrict__ bucket_of)
{
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
  {
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
      const double v = (static_cast<double>(xyz[i * stride + a]) - gm.min[a]) / gm.bsize;
      long long b = static_cast<long long>(floor(v));
      b = b < 0 ? 0 : (b >= gm.nb[a] ? gm.nb[a] - 1 : b);
      if (!(v == v))
        b = 0;
      c[a] = static_cast<int>(b);
    }
    const uint32_t bid = static_cast<uint32_t>((static_cast<uint64_t>(c[2]) * gm.nb[1] + c[1]) * gm.nb[0] + c[0]);
    bucket_of[i] = bid;
    atomicAdd(counts + bid, 1u);
  }
}

// Exclusive scan of counts into start (nb + 1 entries), single block, chunked.
__global__ void k_scan_single(const uint32_t* __restrict__ counts, uint64_t nb, uint32_t* __restrict__ start)
{
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0)
    carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint64_t base = 0; base < nb; base += blockDim.x)
  {
    const uint64_t i = base + threadIdx.x;
    const uint32_t v = i < nb ? counts[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= o)
        x += y;
    }
    if (lane == 31)
      warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0)
    {
      uint32_t t = lane < static_cast<int>(blockDim.x >> 5) ? warp_tot[lane] : 0u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1)
      {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, t, o);
        if (lane >= o)
          t += y;
      }
      warp_tot[lane] = t;  // inclusive
    }
    __syncthreads();
    const uint32_t before = (wid ? warp_tot[wid - 1] : 0u) + carry;
    if (i < nb)
      start[i] = before + x - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1)
      carry = before + x;
    __syncthreads();
  }
  if (threadIdx.x == 0)
    start[nb] = carry;
}

__global__ void k_df_scatter(const float* __restrict__ xyz, uint64_t n, uint32_t stride,
                             const uint32_t* __restrict__ bucket_of, const uint32_t* __restrict__ start,
                             uint32_t* __restrict__ fill, float4* __restrict__ out)
{
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
  {
    const uint32_t b = bucket_of[i];
    const uint32_t pos = start[b] + atomicAdd(fill + b, 1u);
    out[pos] = make_float4(xyz[i * stride], xyz[i * stride + 1], xyz[i * stride + 2], 0.0f);
  }
}

struct DFQuery
{
  const float* qx;  // query coordinate per axis index: (float)(min + i*res)
  const float* qy;
  const float* qz;
  uint32_t size[3];
  float c1, c2;
  int empty;  // no occupied points at all
};

constexpr int DF_LPW = 4;                         // z-layers of the brick per warp
constexpr int DF_THREADS = 32 * DF_B / DF_LPW;    // warps per brick block
constexpr int DF_NC = 2 * DF_LPW;                 // cells per lane

__global__ __launch_bounds__(DF_THREADS) void k_df_search(DFGeom gm, DFQuery q, const float4* __restrict__ pts,
                                                          const uint32_t* __restrict__ start, float* __restrict__ dist,
                                                          float* __restrict__ prob)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t brick = blockIdx.x;
  const int bx = static_cast<int>(brick % gm.nb[0]);
  const int by = static_cast<int>((brick / gm.nb[0]) % gm.nb[1]);
  const int bz = static_cast<int>(brick / (static_cast<uint64_t>(gm.nb[0]) * gm.nb[1]));
  // cells of this lane: x = lane & 7, y in {lane >> 3, (lane >> 3) + 4}, the warp's DF_LPW z-layers
  const int cx = bx * DF_B + (lane & 7);
  const int cy0 = by * DF_B + (lane >> 3);
  int cy[DF_NC], cz[DF_NC];
  float qxv, qyv[DF_NC], qzv[DF_NC];
  bool valid[DF_NC];
  bool any = false;
  qxv = cx < static_cast<int>(q.size[0]) ? q.qx[cx] : 0.0f;
#pragma unroll
  for (int j = 0; j < DF_NC; ++j)
  {
    cy[j] = cy0 + 4 * (j & 1);
    cz[j] = bz * DF_B + wid * DF_LPW + (j >> 1);
    valid[j] = cx < static_cast<int>(q.size[0]) && cy[j] < static_cast<int>(q.size[1]) &&
               cz[j] < static_cast<int>(q.size[2]);
    qyv[j] = valid[j] ? q.qy[cy[j]] : 0.0f;
    qzv[j] = valid[j] ? q.qz[cz[j]] : 0.0f;
    any |= valid[j];
  }
  float best[DF_NC];
#pragma unroll
  for (int j = 0; j < DF_NC; ++j)
    best[j] = INFINITY;
  if (!__any_sync(0xFFFFFFFFu, any))
    return;
  // This warp's cells span [qlo, qhi] per axis (corner coordinates ascend with the index).
  const int x1 = min(bx * DF_B + DF_B, static_cast<int>(q.size[0])) - 1;
  const int y1 = min(by * DF_B + DF_B, static_cast<int>(q.size[1])) - 1;
  const int z0 = min(bz * DF_B + wid * DF_LPW, static_cast<int>(q.size[2]) - 1);
  const int z1 = min(bz * DF_B + wid * DF_LPW + DF_LPW - 1, static_cast<int>(q.size[2]) - 1);
  const float qlo[3] = { q.qx[bx * DF_B], q.qy[by * DF_B], q.qz[z0] };
  const float qhi[3] = { q.qx[x1], q.qy[y1], q.qz[z1] };
  const float bminf[3] = { static_cast<float>(gm.min[0]), static_cast<float>(gm.min[1]),
                           static_cast<float>(gm.min[2]) };
  const float bsizef = static_cast<float>(gm.bsize);
  float worst = INFINITY;  // the largest best distance among the warp's cells, as of the last ring
  if (!q.empty)
  {
    const int rmax = max(gm.nb[0], max(gm.nb[1], gm.nb[2]));
    for (int r = 0; r <= rmax; ++r)
    {
      // The buckets at Chebyshev distance r form the surface of a (2r + 1)^3 cube:
      // two z faces (2r + 1)^2, two y faces (2r + 1) x (2r - 1), two x faces (2r - 1)^2.
      const int side = 2 * r + 1, inner = 2 * r - 1;
      const int fz = side * side, fy = side * inner, fx = inner * inner;
      const int nsurf = r == 0 ? 1 : 2 * (fz + fy + fx);
      for (int base = 0; base < nsurf; base += 32)
      {
        const int li = base + lane;
        uint32_t s0 = 0, s1 = 0;
        bool have = false;
        if (li < nsurf)
        {
          int dx = 0, dy = 0, dz = 0;
          if (r > 0)
          {
            int t = li;
            if (t < 2 * fz)
            {
              dz = t < fz ? -r : r;
              t %= fz;
              dx = t % side - r;
              dy = t / side - r;
            }
            else if ((t -= 2 * fz) < 2 * fy)
            {
              dy = t < fy ? -r : r;
              t %= fy;
              dx = t % side - r;
              dz = t / side - (r - 1);
            }
            else
            {
              t -= 2 * fy;
              dx = t < fx ? -r : r;
              t %= fx;
              dy = t % inner - (r - 1);
              dz = t / inner - (r - 1);
            }
          }
          const int ux = bx + dx, uy = by + dy, uz = bz + dz;
          bool reach = ux >= 0 && uy >= 0 && uz >= 0 && ux < gm.nb[0] && uy < gm.nb[1] && uz < gm.nb[2];
          if (reach && worst < INFINITY)
          {
            // Skip a bucket whose box is farther from every cell than each cell's best:
            // per axis the gap between the cells' span and the bucket's box (edge buckets
            // are open outward: clamped points lie there), less a slack far above the
            // float rounding of the coordinates.
            const int u[3] = { ux, uy, uz };
            float d2 = 0.0f;
#pragma unroll
            for (int a = 0; a < 3; ++a)
            {
              const float blo = u[a] == 0 ? -INFINITY : bminf[a] + static_cast<float>(u[a]) * bsizef;
              const float bhi = u[a] == gm.nb[a] - 1 ? INFINITY : bminf[a] + static_cast<float>(u[a] + 1) * bsizef;
              const float slack = 1e-4f + 1e-6f * fmaxf(fabsf(qlo[a]), fabsf(qhi[a]));
              const float gap = fmaxf(fmaxf(blo - qhi[a], qlo[a] - bhi) - slack, 0.0f);
              d2 += gap * gap;
            }
            reach = !(d2 > worst * 1.00001f);
          }
          if (reach)
          {
            const uint64_t b = (static_cast<uint64_t>(uz) * gm.nb[1] + uy) * gm.nb[0] + ux;
            s0 = __ldg(start + b);
            s1 = __ldg(start + b + 1);
            have = s1 > s0;
          }
        }
        uint32_t mask = __ballot_sync(0xFFFFFFFFu, have);
        while (mask)
        {
          const int src = __ffs(mask) - 1;
          mask &= mask - 1;
          const uint32_t a0 = __shfl_sync(0xFFFFFFFFu, s0, src);
          const uint32_t a1 = __shfl_sync(0xFFFFFFFFu, s1, src);
          for (uint32_t i = a0; i < a1; ++i)
          {
            const float4 p = __ldg(pts + i);  // same address across the warp: broadcast
            const float ddx = __fsub_rn(qxv, p.x);
            const float dxx = __fmul_rn(ddx, ddx);
#pragma unroll
            for (int j = 0; j < DF_NC; ++j)
            {
              const float ddy = __fsub_rn(qyv[j], p.y);
              const float ddz = __fsub_rn(qzv[j], p.z);
              const float d = __fadd_rn(__fadd_rn(dxx, __fmul_rn(ddy, ddy)), __fmul_rn(ddz, ddz));
              best[j] = d < best[j] ? d : best[j];
            }
          }
        }
      }
      // Unscanned buckets are >= r full buckets away from every cell of the brick.
      worst = 0.0f;
#pragma unroll
      for (int j = 0; j < DF_NC; ++j)
        worst = fmaxf(worst, valid[j] ? best[j] : 0.0f);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        worst = fmaxf(worst, __shfl_xor_sync(0xFFFFFFFFu, worst, o));
      const double bound = static_cast<double>(r) * gm.bsize;
      if (static_cast<double>(worst) < bound * bound * (1.0 - 1e-5))
        break;
    }
  }
#pragma unroll
  for (int j = 0; j < DF_NC; ++j)
  {
    if (!valid[j])
      continue;
    const uint64_t idx = (static_cast<uint64_t>(cz[j]) * q.size[1] + cy[j]) * q.size[0] + cx;
    if (q.empty)
    {
      dist[idx] = -1.0f;  // PointCloudTools.cpp:142-143
      prob[idx] = 0.0f;
    }
    else
    {
      const float d = best[j];
      const float arg = __fmul_rn(__fmul_rn(-d, d), q.c2);  // -dist * dist * gauss_const2
      const float e = __double2float_rn(exp(static_cast<double>(arg)));
      dist[idx] = d;
      prob[idx] = __fmul_rn(q.c1, e);
    }
  }
}

__global__ void k_max_prob(const float* __restrict__ p, uint64_t n, unsigned int* __restrict__ out_bits)
{
  float m = 0.0f;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    m = fmaxf(m, p[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    m = fmaxf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
  if ((threadIdx.x & 31) == 0)
    atomicMax(out_bits, __float_as_uint(m));  // non-negative floats order like their bits
}

__global__ void k_quantize(const float* __restrict__ p, uint64_t n, __half* __restrict__ h, uint8_t* __restrict__ q,
                           float inv_scale)
{
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
  {
    const float v = p[i];
    if (h)
      h[i] = __float2half_rn(v);
    if (q)
    {
      float c = rintf(v * inv_scale);
      c = fminf(fmaxf(c, 0.0f), 255.0f);
      q[i] = static_cast<uint8_t>(c);
    }
  }
}

// Grid3d::buildGridSliceMsg max over [init, end) then int8(prob * 100/max).
__global__ void k_slice_max(const float* __restrict__ p, uint64_t first, uint64_t count, unsigned int* out_bits)
{
  float m = -1.0f;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    m = fmaxf(m, p[first + i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    m = fmaxf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
  if ((threadIdx.x & 31) == 0 && m >= 0.0f)
    atomicMax(out_bits, __float_as_uint(m));
}

__global__ void k_slice_scale(const float* __restrict__ p, uint64_t first, uint64_t count, const unsigned int* mbits,
                              int8_t* __restrict__ out)
{
  float maxp = __uint_as_float(*mbits);
  if (maxp < 0.000001f)
    maxp = 0.000001f;
  const float s = __fdiv_rn(100.f, maxp);
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    out[i] = static_cast<int8_t>(__float2int_rz(__fmul_rn(p[first + i], s)));
}
}  // namespace

// ---- C ABI --------------------------------------------------------------------------------

extern "C" int amcl_grid_create(amcl_grid_t* out, void* stream)
{
  if (!out)
    return fail(AMCL_EINVAL, "amcl_grid_create: null out");
  amcl_grid_s* g = new amcl_grid_s();
  const int rc = g->st.init(stream);
  if (rc)
  {
    delete g;
    return rc;
  }
  *out = g;
  return AMCL_OK;
}

extern "C" int amcl_grid_destroy(amcl_grid_t g)
{
  if (!g)
    return AMCL_OK;
  cudaStreamSynchronize(g->st.s);
  delete g;
  return AMCL_OK;
}

static int grid_set_info(amcl_grid_s* g, const double mn[3], const double mx[3], double res, double sensor_dev)
{
  if (!(res > 0.0) || !std::isfinite(res))
    return fail(AMCL_EINVAL, "grid: resolution must be positive");
  uint64_t total = 1;
  for (int a = 0; a < 3; ++a)
  {
    if (!std::isfinite(mn[a]) || !std::isfinite(mx[a]) || !(mx[a] > mn[a]))
      return fail(AMCL_EINVAL, "grid: bounds must be finite with max > min");
    const double sz = std::ceil((mx[a] - mn[a]) / res);  // PointCloudTools.cpp:96-101
    if (sz < 1.0 || sz > 4294967295.0)
      return fail(AMCL_ERANGE, "grid: axis size out of range");
    g->info.size[a] = static_cast<uint32_t>(sz);
    g->info.min[a] = mn[a];
    g->info.max[a] = mx[a];
    total *= g->info.size[a];
    if (total > 0xFFFFFFFFull)
      return fail(AMCL_ERANGE, "grid: more than 2^32-1 cells (uint32 cell index of Grid3d.cpp:187)");
  }
  g->info.resolution = res;
  g->info.sensor_dev = sensor_dev;
  return AMCL_OK;
}

extern "C" int amcl_grid_build(amcl_grid_t g, const float* xyz, uint64_t n, uint32_t stride_floats, const double min[3],
                               const double max[3], double resolution, double sensor_dev)
{
  if (!g || !min || !max || (n && !xyz) || stride_floats < 3)
    return fail(AMCL_EINVAL, "amcl_grid_build: bad arguments");
  g->built = false;
  int rc = grid_set_info(g, min, max, resolution, sensor_dev);
  if (rc)
    return rc;
  const uint64_t cells = g->cells();
  cudaStream_t s = g->st.s;
  if ((rc = g->dist.ensure(cells * 4)) || (rc = g->prob.ensure((cells + 1) * 4)))
    return rc;
  g->prob16.release();
  g->prob8.release();
  g->info.storage = AMCL_GRID_F32;
  g->info.u8_scale = 0.0f;
  AMCL_CUDA_TRY(cudaMemsetAsync(g->prob.as<float>() + cells, 0, 4, s));  // the zero pad cell

  // Query coordinates (float)(min + i*res) per axis (PointCloudTools.cpp:127-129).
  std::vector<float> q[3];
  for (int a = 0; a < 3; ++a)
  {
    q[a].resize(g->info.size[a]);
    for (uint32_t i = 0; i < g->info.size[a]; ++i)
      q[a][i] = static_cast<float>(min[a] + (static_cast<double>(i) * resolution));
  }
  DFGeom gm;
  gm.bsize = DF_B * resolution;
  gm.nbtot = 1;
  for (int a = 0; a < 3; ++a)
  {
    gm.nb[a] = static_cast<int>((g->info.size[a] + DF_B - 1) / DF_B);
    gm.min[a] = min[a];
    gm.nbtot *= gm.nb[a];
  }
  DevBuf d_xyz, d_counts, d_bof, d_start, d_fill, d_pts, d_q;
  const size_t qn = q[0].size() + q[1].size() + q[2].size();
  if ((rc = d_q.ensure(qn * 4)) || (rc = d_counts.ensure(gm.nbtot * 4)) || (rc = d_start.ensure((gm.nbtot + 1) * 4)) ||
      (rc = d_fill.ensure(gm.nbtot * 4)))
    return rc;
  std::vector<float> qall;
  qall.reserve(qn);
  for (int a = 0; a < 3; ++a)
    qall.insert(qall.end(), q[a].begin(), q[a].end());
  AMCL_CUDA_TRY(cudaMemcpyAsync(d_q.p, qall.data(), qn * 4, cudaMemcpyHostToDevice, s));
  AMCL_CUDA_TRY(cudaMemsetAsync(d_counts.p, 0, gm.nbtot * 4, s));
  AMCL_CUDA_TRY(cudaMemsetAsync(d_fill.p, 0, gm.nbtot * 4, s));
  if (n)
  {
    if ((rc = d_xyz.ensure(n * stride_floats * 4)) || (rc = d_bof.ensure(n * 4)) || (rc = d_pts.ensure(n * 16)))
      return rc;
    AMCL_CUDA_TRY(cudaMemcpyAsync(d_xyz.p, xyz, n * stride_floats * 4, cudaMemcpyHostToDevice, s));
    const unsigned nbk = std::min<uint64_t>(ceil_div(n, 256), 65535u * 16);
    k_df_count<<<nbk, 256, 0, s>>>(d_xyz.as<float>(), n, stride_floats, gm, d_counts.as<uint32_t>(),
                                   d_bof.as<uint32_t>());
    AMCL_LAUNCH_CHECK("k_df_count");
  }
  k_scan_single<<<1, 1024, 0, s>>>(d_counts.as<uint32_t>(), gm.nbtot, d_start.as<uint32_t>());
  AMCL_LAUNCH_CHECK("k_scan_single");
  if (n)
  {
    const unsigned nbk = std::min<uint64_t>(ceil_div(n, 256), 65535u * 16);
    k_df_scatter<<<nbk, 256, 0, s>>>(d_xyz.as<float>(), n, stride_floats, d_bof.as<uint32_t>(),
                                     d_start.as<uint32_t>(), d_fill.as<uint32_t>(), d_pts.as<float4>());
    AMCL_LAUNCH_CHECK("k_df_scatter");
  }
  DFQuery dq;
  dq.qx = d_q.as<float>();
  dq.qy = dq.qx + q[0].size();
  dq.qz = dq.qy + q[1].size();
  for (int a = 0; a < 3; ++a)
    dq.size[a] = g->info.size[a];
  dq.c1 = static_cast<float>(1. / (sensor_dev * std::sqrt(2 * M_PI)));  // PointCloudTools.cpp:114
  dq.c2 = static_cast<float>(1. / (2. * sensor_dev * sensor_dev));      // PointCloudTools.cpp:115
  dq.empty = n == 0;
  k_df_search<<<static_cast<unsigned>(gm.nbtot), DF_THREADS, 0, s>>>(gm, dq, d_pts.as<float4>(), d_start.as<uint32_t>(),
                                                                g->dist.as<float>(), g->prob.as<float>());
  AMCL_LAUNCH_CHECK("k_df_search");
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  g->built = true;
  return grid_prepare_view(g);
}

extern "C" int amcl_grid_load_cells(amcl_grid_t g, const amcl_grid_info* info, const float* dist, const float* prob)
{
  if (!g || !info || !prob)
    return fail(AMCL_EINVAL, "amcl_grid_load_cells: bad arguments");
  g->built = false;
  int rc = grid_set_info(g, info->min, info->max, info->resolution, info->sensor_dev);
  if (rc)
    return rc;
  for (int a = 0; a < 3; ++a)
    if (info->size[a] != g->info.size[a])
      return fail(AMCL_EINVAL, "amcl_grid_load_cells: sizes do not match ceil((max-min)/res)");
  const uint64_t cells = g->cells();
  if ((rc = g->dist.ensure(cells * 4)) || (rc = g->prob.ensure((cells + 1) * 4)))
    return rc;
  g->prob16.release();
  g->prob8.release();
  g->info.storage = AMCL_GRID_F32;
  g->info.u8_scale = 0.0f;
  AMCL_CUDA_TRY(cudaMemsetAsync(g->prob.as<float>() + cells, 0, 4, g->st.s));  // the zero pad cell
  if (dist)
    AMCL_CUDA_TRY(cudaMemcpyAsync(g->dist.p, dist, cells * 4, cudaMemcpyHostToDevice, g->st.s));
  else
    AMCL_CUDA_TRY(cudaMemsetAsync(g->dist.p, 0, cells * 4, g->st.s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(g->prob.p, prob, cells * 4, cudaMemcpyHostToDevice, g->st.s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(g->st.s));
  g->built = true;
  return grid_prepare_view(g);
}

extern "C" int amcl_grid_info_get(amcl_grid_t g, amcl_grid_info* out)
{
  if (!g || !out)
    return fail(AMCL_EINVAL, "amcl_grid_info_get: bad arguments");
  if (!g->built)
    return fail(AMCL_ESTATE, "amcl_grid_info_get: grid not built");
  *out = g->info;
  return AMCL_OK;
}

extern "C" int amcl_grid_weight_loop(amcl_grid_t g, int* loop)
{
  if (!g || !loop)
    return fail(AMCL_EINVAL, "amcl_grid_weight_loop: bad arguments");
  if (!g->built)
    return fail(AMCL_ESTATE, "amcl_grid_weight_loop: grid not built");
  *loop = fast_variant(g->view);
  return AMCL_OK;
}

extern "C" int amcl_grid_read_cells(amcl_grid_t g, uint64_t first, uint64_t count, float* dist, float* prob)
{
  if (!g)
    return fail(AMCL_EINVAL, "amcl_grid_read_cells: null grid");
  if (!g->built)
    return fail(AMCL_ESTATE, "amcl_grid_read_cells: grid not built");
  if (first > g->cells() || count > g->cells() - first)
    return fail(AMCL_ERANGE, "amcl_grid_read_cells: range outside the grid");
  if (dist)
    AMCL_CUDA_TRY(cudaMemcpyAsync(dist, g->dist.as<float>() + first, count * 4, cudaMemcpyDeviceToHost, g->st.s));
  if (prob)
    AMCL_CUDA_TRY(cudaMemcpyAsync(prob, g->prob.as<float>() + first, count * 4, cudaMemcpyDeviceToHost, g->st.s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(g->st.s));
  return AMCL_OK;
}

extern "C" int amcl_grid_set_storage(amcl_grid_t g, int storage)
{
  if (!g || storage < AMCL_GRID_F32 || storage > AMCL_GRID_U8)
    return fail(AMCL_EINVAL, "amcl_grid_set_storage: bad arguments");
  if (!g->built)
    return fail(AMCL_ESTATE, "amcl_grid_set_storage: grid not built");
  const uint64_t cells = g->cells();
  cudaStream_t s = g->st.s;
  const unsigned nb = std::min<uint64_t>(ceil_div(cells, 256), 152u * 64);
  int rc;
  if (storage == AMCL_GRID_F16 && !g->prob16.p)
  {
    if ((rc = g->prob16.ensure((cells + 1) * 2)))
      return rc;
    AMCL_CUDA_TRY(cudaMemsetAsync(g->prob16.as<__half>() + cells, 0, 2, s));
    k_quantize<<<nb, 256, 0, s>>>(g->prob.as<float>(), cells, g->prob16.as<__half>(), nullptr, 0.0f);
    AMCL_LAUNCH_CHECK("k_quantize(f16)");
  }
  if (storage == AMCL_GRID_U8 && !g->prob8.p)
  {
    if ((rc = g->prob8.ensure(cells + 1)))
      return rc;
    AMCL_CUDA_TRY(cudaMemsetAsync(g->prob8.as<uint8_t>() + cells, 0, 1, s));
    DevBuf mbits;
    if ((rc = mbits.ensure(4)))
      return rc;
    AMCL_CUDA_TRY(cudaMemsetAsync(mbits.p, 0, 4, s));
    k_max_prob<<<nb, 256, 0, s>>>(g->prob.as<float>(), cells, mbits.as<unsigned int>());
    AMCL_LAUNCH_CHECK("k_max_prob");
    unsigned int bits = 0;
    AMCL_CUDA_TRY(cudaMemcpyAsync(&bits, mbits.p, 4, cudaMemcpyDeviceToHost, s));
    AMCL_CUDA_TRY(cudaStreamSynchronize(s));
    float mx;
    std::memcpy(&mx, &bits, 4);
    const float scale = mx > 0.0f ? mx / 255.0f : 1.0f;
    g->info.u8_scale = scale;
    k_quantize<<<nb, 256, 0, s>>>(g->prob.as<float>(), cells, nullptr, g->prob8.as<uint8_t>(), 1.0f / scale);
    AMCL_LAUNCH_CHECK("k_quantize(u8)");
  }
  g->info.storage = static_cast<uint32_t>(storage);
  g->view.prob_f16 = g->prob16.as<__half>();
  g->view.prob_u8 = g->prob8.as<uint8_t>();
  g->view.u8_scale = g->info.u8_scale;
  g->view.storage = storage;
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  return AMCL_OK;
}

extern "C" int amcl_grid_set_l2_window(amcl_grid_t g, int enable)
{
  if (!g)
    return fail(AMCL_EINVAL, "amcl_grid_set_l2_window: null grid");
  g->l2_window = enable != 0;
  grid_apply_l2_window(g, g->st.s);
  return AMCL_OK;
}

extern "C" int amcl_grid_is_into_map(amcl_grid_t g, float x, float y, float z, int* inside)
{
  if (!g || !inside)
    return fail(AMCL_EINVAL, "amcl_grid_is_into_map: bad arguments");
  if (!g->built)
  {
    *inside = 0;  // Grid3d.cpp:203-204
    return AMCL_OK;
  }
  const GridView& v = g->view;
  *inside = (x >= v.in_lo[0] && x < v.in_hi[0] && y >= v.in_lo[1] && y < v.in_hi[1] && z >= v.in_lo[2] &&
             z < v.in_hi[2])
                ? 1
                : 0;
  return AMCL_OK;
}

extern "C" int amcl_grid_slice(amcl_grid_t g, double z, int8_t* out, uint64_t cap, uint64_t* len, uint32_t* width,
                               uint32_t* height)
{
  if (!g || !len || !width || !height)
    return fail(AMCL_EINVAL, "amcl_grid_slice: bad arguments");
  if (!g->built)
    return fail(AMCL_ESTATE, "amcl_grid_slice: grid not built");  // Grid3d.cpp:82-83
  const amcl_grid_info& in = g->info;
  if (z < in.min[2] || z > in.max[2])
    return fail(AMCL_EINVAL, "amcl_grid_slice: z outside the map");  // Grid3d.cpp:85-86
  // point2grid (Grid3d.cpp:277-282) of the slice corners; x, y passed as float.
  auto p2g = [&](float x, float y, float zz) -> uint32_t {
    return static_cast<uint32_t>((x - in.min[0]) / in.resolution) +
           static_cast<uint32_t>((y - in.min[1]) / in.resolution) * in.size[0] +
           static_cast<uint32_t>((zz - in.min[2]) / in.resolution) * (in.size[0] * in.size[1]);
  };
  const uint32_t init = p2g(static_cast<float>(in.min[0]), static_cast<float>(in.min[1]), static_cast<float>(z));
  const uint32_t end = p2g(static_cast<float>(in.max[0]), static_cast<float>(in.max[1]), static_cast<float>(z));
  const uint64_t count = end > init ? end - init : 0;
  if (static_cast<uint64_t>(init) + count > g->cells())
    return fail(AMCL_ERANGE, "amcl_grid_slice: slice runs past the grid (reference reads out of bounds here)");
  *len = count;
  *width = in.size[0];
  *height = in.size[1];
  if (!out || !count)
    return AMCL_OK;
  cudaStream_t s = g->st.s;
  DevBuf mbits, dout;
  int rc;
  if ((rc = mbits.ensure(4)) || (rc = dout.ensure(count)))
    return rc;
  // max starts at -1 (Grid3d.cpp:103); all probs are >= 0 so the float-bits max
  // starting from the bits of 0.0 gives the same result whenever count > 0.
  AMCL_CUDA_TRY(cudaMemsetAsync(mbits.p, 0, 4, s));
  const unsigned nb = std::min<uint64_t>(ceil_div(count, 256), 152u * 8);
  k_slice_max<<<nb, 256, 0, s>>>(g->prob.as<float>(), init, count, mbits.as<unsigned int>());
  AMCL_LAUNCH_CHECK("k_slice_max");
  k_slice_scale<<<nb, 256, 0, s>>>(g->prob.as<float>(), init, count, mbits.as<unsigned int>(), dout.as<int8_t>());
  AMCL_LAUNCH_CHECK("k_slice_scale");
  AMCL_CUDA_TRY(cudaMemcpyAsync(out, dout.p, std::min(cap, count), cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  return AMCL_OK;
}

// ---- .grid file (Grid3d::saveGrid / loadGrid) -------------------------------------------

extern "C" int amcl_grid_save(amcl_grid_t g, const char* path)
{
  if (!g || !path)
    return fail(AMCL_EINVAL, "amcl_grid_save: bad arguments");
  if (!g->built)
    return fail(AMCL_ESTATE, "amcl_grid_save: grid not built");  // Grid3d.cpp:212-213
  FILE* f = std::fopen(path, "wb");
  if (!f)
    return fail(AMCL_EIO, std::string("amcl_grid_save: cannot open ") + path);
  const uint64_t cells = g->cells();
  bool ok = std::fwrite(&g->info.size[0], 4, 1, f) == 1 && std::fwrite(&g->info.size[1], 4, 1, f) == 1 &&
            std::fwrite(&g->info.size[2], 4, 1, f) == 1 && std::fwrite(&g->info.sensor_dev, 8, 1, f) == 1;
  const uint64_t chunk = 1ull << 24;
  std::vector<float> d(std::min(cells, chunk)), p(std::min(cells, chunk)), cell(2 * std::min(cells, chunk));
  for (uint64_t first = 0; ok && first < cells; first += chunk)
  {
    const uint64_t c = std::min(chunk, cells - first);
    int rc = amcl_grid_read_cells(g, first, c, d.data(), p.data());
    if (rc)
    {
      std::fclose(f);
      return rc;
    }
    for (uint64_t i = 0; i < c; ++i)
    {
      cell[2 * i] = d[i];
      cell[2 * i + 1] = p[i];
    }
    ok = std::fwrite(cell.data(), 8, c, f) == c;
  }
  std::fclose(f);
  return ok ? AMCL_OK : fail(AMCL_EIO, std::string("amcl_grid_save: short write to ") + path);
}

extern "C" int amcl_grid_load(amcl_grid_t g, const char* path, const double min[3], const double max[3],
                              double resolution, double sensor_dev)
{
  if (!g || !path || !min || !max)
    return fail(AMCL_EINVAL, "amcl_grid_load: bad arguments");
  FILE* f = std::fopen(path, "rb");
  if (!f)
    return fail(AMCL_EIO, std::string("amcl_grid_load: cannot open ") + path);
  uint32_t sz[3];
  double dev = 0;
  bool ok = std::fread(sz, 4, 3, f) == 3 && std::fread(&dev, 8, 1, f) == 1;
  if (!ok)
  {
    std::fclose(f);
    return fail(AMCL_EIO, "amcl_grid_load: truncated header");
  }
  if (std::fabs(dev - sensor_dev) >= std::numeric_limits<double>::epsilon())
  {
    std::fclose(f);
    return fail(AMCL_ESTATE, "amcl_grid_load: sensor_dev differs from the file's");  // Grid3d.cpp:256-260
  }
  amcl_grid_info info{};
  for (int a = 0; a < 3; ++a)
  {
    info.min[a] = min[a];
    info.max[a] = max[a];
    info.size[a] = sz[a];
  }
  info.resolution = resolution;
  info.sensor_dev = sensor_dev;
  const uint64_t cells = static_cast<uint64_t>(sz[0]) * sz[1] * sz[2];
  std::vector<float> d(cells), p(cells);
  const uint64_t chunk = 1ull << 24;
  std::vector<float> cell(2 * std::min<uint64_t>(std::max<uint64_t>(cells, 1), chunk));
  for (uint64_t first = 0; ok && first < cells; first += chunk)
  {
    const uint64_t c = std::min(chunk, cells - first);
    ok = std::fread(cell.data(), 8, c, f) == c;
    for (uint64_t i = 0; ok && i < c; ++i)
    {
      d[first + i] = cell[2 * i];
      p[first + i] = cell[2 * i + 1];
    }
  }
  std::fclose(f);
  if (!ok)
    return fail(AMCL_EIO, "amcl_grid_load: truncated cell data");
  return amcl_grid_load_cells(g, &info, d.data(), p.data());
}

extern "C" int amcl_grid_stream(amcl_grid_t g, void** stream)
{
  if (!g || !stream)
    return fail(AMCL_EINVAL, "amcl_grid_stream: bad arguments");
  *stream = g->st.s;
  return AMCL_OK;
}
