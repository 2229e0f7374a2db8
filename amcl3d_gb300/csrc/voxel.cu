// Scan voxel downsample (pcl::VoxelGrid<pcl::PointXYZ>, called by Node.cpp:130-137 on
// every accepted scan, just before ParticleFilter::update).
//
// PCL is a third-party dependency whose source is not part of the reference tree; its
// published algorithm (VoxelGrid::applyFilter) is:
//   inverse leaf 1.0f / leaf; min / max over the finite points (float);
//   voxel counts (int64)((max - min) * inverse) + 1 per axis, and if their product
//     exceeds INT32_MAX the filter returns its input unchanged;
//   min_b = (int)floor(min * inverse), div_b = (int)floor(max * inverse) - min_b + 1;
//   key = i + j * div_b.x + k * div_b.x * div_b.y with ijk = (int)(floor(p * inverse) - min_b);
//   sort the (key, point) pairs by key; per run of one key the centroid is the first
//     point plus each further one (float), divided by the count; output in key order.
//
// On the device: one pass for the bounds (order-preserving integer atomics), one for
// the keys, a stable least-significant-digit radix sort of the 32-bit keys (4 passes
// of 8 bits; per tile a digit histogram, one scan, then a scatter in which each warp
// ranks its keys in input order with __match_any_sync), a head count / scan / write
// that gives each voxel's first sorted position, and one thread per voxel summing its
// points in sorted order.  The sort is stable, so the points of a voxel are summed in
// input order; std::sort's order among equal keys is unspecified, which matters only
// for voxels of three or more points (two-term float sums commute).
// Keys are sorted as unsigned 32-bit values with 0xFFFFFFFF for non-finite points; a
// key space div_b.x * div_b.y * div_b.z beyond 2^32 - 1 (which PCL's int arithmetic
// would wrap) is treated like the int32 overflow: the input is returned unchanged.
#include <cmath>
#include <cstring>

#include "grid.cuh"
#include "voxel.cuh"

namespace amcl
{
namespace
{
constexpr int VX_THREADS = 256;
constexpr int VX_ITEMS = 8;
constexpr int VX_TILE = VX_THREADS * VX_ITEMS;  // keys per tile
constexpr int VX_WARPS = VX_THREADS / 32;
constexpr uint32_t VX_INVALID = 0xFFFFFFFFu;
constexpr uint32_t VX_MAX_POINTS = 1u << 30;

__device__ __forceinline__ uint32_t f2ord(float f)
{
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u)
{
  return (u & 0x80000000u) ? __uint_as_float(u & 0x7FFFFFFFu) : __uint_as_float(~u);
}
__device__ __forceinline__ bool finite3(const float4& p)
{
  return isfinite(p.x) && isfinite(p.y) && isfinite(p.z);
}

// Per-call constants derived from the bounds (every thread recomputes them).
struct VoxelKeyParams
{
  int32_t min_b[3];
  uint32_t mul1, mul2;
  bool overflow;
};

__device__ __forceinline__ VoxelKeyParams key_params(const VoxelMeta* m, float3 inv)
{
  VoxelKeyParams k{};
  const float iv[3] = { inv.x, inv.y, inv.z };
  double dprod = 1.0, bprod = 1.0;
  int32_t div_b[3];
  for (int a = 0; a < 3; ++a)
  {
    const float lo = ord2f(m->mm[a]), hi = ord2f(m->mm[3 + a]);
    const float span = __fmul_rn(__fsub_rn(hi, lo), iv[a]);
    // (int64)span + 1; spans of 2^31 or more overflow the product on their own
    dprod *= (span < 2147483648.0f) ? static_cast<double>(static_cast<long long>(span) + 1) : 4294967296.0;
    k.min_b[a] = static_cast<int32_t>(floorf(__fmul_rn(lo, iv[a])));
    div_b[a] = static_cast<int32_t>(floorf(__fmul_rn(hi, iv[a]))) - k.min_b[a] + 1;
    bprod *= static_cast<double>(div_b[a]);
  }
  k.overflow = m->n_finite != 0 && (dprod > 2147483647.0 || bprod > 4294967295.0);
  k.mul1 = static_cast<uint32_t>(div_b[0]);
  k.mul2 = static_cast<uint32_t>(div_b[0]) * static_cast<uint32_t>(div_b[1]);
  return k;
}

__global__ void k_vx_bounds(const float4* __restrict__ in, uint32_t n, VoxelMeta* __restrict__ meta)
{
  uint32_t lo[3] = { VX_INVALID, VX_INVALID, VX_INVALID }, hi[3] = { 0, 0, 0 }, cnt = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    const float4 p = in[i];
    if (!finite3(p))
      continue;
    ++cnt;
    const uint32_t o[3] = { f2ord(p.x), f2ord(p.y), f2ord(p.z) };
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
      lo[a] = min(lo[a], o[a]);
      hi[a] = max(hi[a], o[a]);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
  {
    lo[a] = __reduce_min_sync(0xFFFFFFFFu, lo[a]);
    hi[a] = __reduce_max_sync(0xFFFFFFFFu, hi[a]);
  }
  cnt = __reduce_add_sync(0xFFFFFFFFu, cnt);
  if ((threadIdx.x & 31) == 0 && cnt)
  {
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
      atomicMin(&meta->mm[a], lo[a]);
      atomicMax(&meta->mm[3 + a], hi[a]);
    }
    atomicAdd(&meta->n_finite, cnt);
  }
}

__global__ void k_vx_keys(const float4* __restrict__ in, uint32_t n, float3 inv, VoxelMeta* __restrict__ meta,
                          uint32_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
  const VoxelKeyParams k = key_params(meta, inv);
  if (blockIdx.x == 0 && threadIdx.x == 0)
    meta->overflow = k.overflow ? 1u : 0u;
  const float iv[3] = { inv.x, inv.y, inv.z };
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    const float4 p = in[i];
    uint32_t key = VX_INVALID;
    if (!k.overflow && finite3(p))
    {
      const float c[3] = { p.x, p.y, p.z };
      uint32_t ijk[3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
        ijk[a] = static_cast<uint32_t>(
            static_cast<int32_t>(__fsub_rn(floorf(__fmul_rn(c[a], iv[a])), static_cast<float>(k.min_b[a]))));
      key = ijk[0] + ijk[1] * k.mul1 + ijk[2] * k.mul2;
    }
    keys[i] = key;
    vals[i] = i;
  }
}

// Digit histogram of one tile: hist[digit * ntiles + tile].
__global__ void __launch_bounds__(VX_THREADS) k_vx_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                        uint32_t* __restrict__ hist, uint32_t ntiles)
{
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * VX_TILE;
  for (uint32_t i = threadIdx.x; i < VX_TILE; i += VX_THREADS)
    if (base + i < n)
      atomicAdd(&h[(keys[base + i] >> shift) & 255u], 1u);
  __syncthreads();
  hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of L counters in place by one block; *total receives the sum.  With
// STAGE the counters pass through shared memory (coalesced in and out; L <= VX_SCAN_SMEM).
constexpr uint32_t VX_SCAN_SMEM = 24576;  // counters staged in 96 KB of shared memory

template <bool STAGE>
__global__ void __launch_bounds__(1024) k_vx_scan(uint32_t* __restrict__ ga, uint32_t L, uint32_t* __restrict__ total)
{
  extern __shared__ uint32_t s_a[];
  __shared__ uint32_t ws[32];
  uint32_t* a = ga;
  if (STAGE)
  {
    for (uint32_t i = threadIdx.x; i < L; i += 1024)
      s_a[i] = ga[i];
    __syncthreads();
    a = s_a;
  }
  const uint32_t per = (L + 1023) / 1024;
  const uint32_t lo = min(L, threadIdx.x * per), hi = min(L, lo + per);
  uint32_t s = 0;
  for (uint32_t i = lo; i < hi; ++i)
    s += a[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o)
      incl += t;
  }
  if (lane == 31)
    ws[warp] = incl;
  __syncthreads();
  if (warp == 0)
  {
    const uint32_t v = ws[lane];
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= o)
        x += t;
    }
    ws[lane] = x - v;
  }
  __syncthreads();
  uint32_t run = ws[warp] + incl - s;
  for (uint32_t i = lo; i < hi; ++i)
  {
    const uint32_t v = a[i];
    a[i] = run;
    run += v;
  }
  if (threadIdx.x == 1023 && total)
    *total = run;
  if (STAGE)
  {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < L; i += 1024)
      ga[i] = s_a[i];
  }
}

int launch_vx_scan(uint32_t* a, uint32_t L, uint32_t* total, cudaStream_t s)
{
  if (L <= VX_SCAN_SMEM)
  {
    static bool attr = false;
    if (!attr)
    {
      AMCL_CUDA_TRY(cudaFuncSetAttribute(k_vx_scan<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(VX_SCAN_SMEM * 4)));
      attr = true;
    }
    k_vx_scan<true><<<1, 1024, L * 4, s>>>(a, L, total);
  }
  else
    k_vx_scan<false><<<1, 1024, 0, s>>>(a, L, total);
  AMCL_LAUNCH_CHECK("k_vx_scan");
  return AMCL_OK;
}

// Stable scatter of one tile by one digit.  Warp w owns the tile's keys
// [w * 256, (w + 1) * 256) in rounds of 32 consecutive keys, so ranks follow input
// order: lanes of one digit in a round are ranked by lane, rounds in order, warps by
// the per-warp digit prefix, tiles by the scanned histogram (digit-major, tile-minor).
__global__ void __launch_bounds__(VX_THREADS) k_vx_scatter(const uint32_t* __restrict__ kin,
                                                           const uint32_t* __restrict__ vin,
                                                           uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           uint32_t n, int shift, const uint32_t* __restrict__ hist,
                                                           uint32_t ntiles)
{
  __shared__ uint32_t cnt[VX_WARPS][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < VX_WARPS * 256; i += VX_THREADS)
    (&cnt[0][0])[i] = 0;
  __syncthreads();
  const uint32_t seg = blockIdx.x * VX_TILE + warp * (VX_TILE / VX_WARPS);
  uint32_t kr[VX_ITEMS], vr[VX_ITEMS], dr[VX_ITEMS];
#pragma unroll
  for (int r = 0; r < VX_ITEMS; ++r)
  {
    const uint32_t j = seg + r * 32 + lane;
    kr[r] = j < n ? kin[j] : 0u;
    vr[r] = j < n ? vin[j] : 0u;
    dr[r] = j < n ? ((kr[r] >> shift) & 255u) : 256u;  // 256: no key (tail of the last tile)
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, dr[r]);
    if (dr[r] < 256u && lane == __ffs(peers) - 1)
      cnt[warp][dr[r]] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    const int d = threadIdx.x;  // VX_THREADS == 256 digits
    uint32_t run = hist[d * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < VX_WARPS; ++w)
    {
      const uint32_t c = cnt[w][d];
      cnt[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < VX_ITEMS; ++r)
  {
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, dr[r]);
    uint32_t pos = 0;
    if (dr[r] < 256u)
    {
      pos = cnt[warp][dr[r]] + __popc(peers & lt);
      kout[pos] = kr[r];
      vout[pos] = vr[r];
    }
    __syncwarp();
    if (dr[r] < 256u && lane == __ffs(peers) - 1)
      cnt[warp][dr[r]] += __popc(peers);
    __syncwarp();
  }
}

// Voxel heads (first sorted position of each key) per tile: count (starts == nullptr)
// or write their positions at the scanned tile offsets.
__global__ void __launch_bounds__(VX_THREADS) k_vx_heads(const uint32_t* __restrict__ keys, uint32_t n,
                                                         uint32_t* __restrict__ tiles, uint32_t* __restrict__ starts)
{
  __shared__ uint32_t ws[VX_WARPS];
  const uint32_t base = blockIdx.x * VX_TILE + threadIdx.x * VX_ITEMS;
  uint32_t flags = 0, c = 0;
  uint32_t prev = base > 0 && base - 1 < n ? keys[base - 1] : VX_INVALID;
#pragma unroll
  for (int k = 0; k < VX_ITEMS; ++k)
  {
    const uint32_t j = base + k;
    if (j < n)
    {
      const uint32_t key = keys[j];
      if (key != VX_INVALID && (j == 0 || key != prev))
      {
        flags |= 1u << k;
        ++c;
      }
      prev = key;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o)
      incl += t;
  }
  if (lane == 31)
    ws[warp] = incl;
  __syncthreads();
  if (!starts)
  {
    if (threadIdx.x == 0)
    {
      uint32_t t = 0;
      for (int w = 0; w < VX_WARPS; ++w)
        t += ws[w];
      tiles[blockIdx.x] = t;
    }
    return;
  }
  uint32_t pos = tiles[blockIdx.x] + incl - c;
  for (int w = 0; w < warp; ++w)
    pos += ws[w];
#pragma unroll
  for (int k = 0; k < VX_ITEMS; ++k)
    if (flags & (1u << k))
      starts[pos++] = base + k;
}

// One thread per voxel: first point + each further point in sorted order, / count.
// On overflow the input is copied through instead.
__global__ void k_vx_centroids(const float4* __restrict__ in, uint32_t n, const uint32_t* __restrict__ vals,
                               const uint32_t* __restrict__ starts, VoxelMeta* __restrict__ meta,
                               float4* __restrict__ out)
{
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (meta->overflow)
  {
    if (v < n)
    {
      const float4 p = in[v];
      out[v] = make_float4(p.x, p.y, p.z, 1.0f);
    }
    if (v == 0)
      meta->n_out = n;
    return;
  }
  const uint32_t total = meta->n_out;
  if (v >= total)
    return;
  const uint32_t s = starts[v];
  const uint32_t e = v + 1 < total ? starts[v + 1] : meta->n_finite;
  const float4 p0 = in[vals[s]];
  float cx = p0.x, cy = p0.y, cz = p0.z;
  for (uint32_t j = s + 1; j < e; ++j)
  {
    const float4 q = in[vals[j]];
    cx = __fadd_rn(cx, q.x);
    cy = __fadd_rn(cy, q.y);
    cz = __fadd_rn(cz, q.z);
  }
  const float cnt = __uint2float_rn(e - s);
  out[v] = make_float4(__fdiv_rn(cx, cnt), __fdiv_rn(cy, cnt), __fdiv_rn(cz, cnt), 1.0f);
}

inline unsigned blocks_for(uint64_t n, int threads, unsigned cap)
{
  const uint64_t b = (n + threads - 1) / threads;
  return static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(b, cap)));
}
}  // namespace

int voxel_enqueue(amcl_voxel_s* v, const float4* in, uint32_t n, const float leaf[3], float4* out, cudaStream_t s)
{
  int rc;
  const uint32_t ntiles = std::max<uint32_t>(1, (n + VX_TILE - 1) / VX_TILE);
  const size_t nk = std::max<uint32_t>(n, 1);
  if ((rc = v->keys[0].ensure(nk * 4)) || (rc = v->keys[1].ensure(nk * 4)) || (rc = v->vals[0].ensure(nk * 4)) ||
      (rc = v->vals[1].ensure(nk * 4)) || (rc = v->hist.ensure(256ull * ntiles * 4)) ||
      (rc = v->tiles.ensure(ntiles * 4ull)) || (rc = v->starts.ensure(nk * 4)) ||
      (rc = v->meta.ensure(sizeof(VoxelMeta))))
    return rc;
  VoxelMeta* meta = v->meta.as<VoxelMeta>();
  // bounds start empty: min encodings all-ones, max encodings and counters zero
  AMCL_CUDA_TRY(cudaMemsetAsync(meta, 0xFF, 3 * sizeof(uint32_t), s));
  AMCL_CUDA_TRY(cudaMemsetAsync(&meta->mm[3], 0, sizeof(VoxelMeta) - 3 * sizeof(uint32_t), s));
  // host float division, as PCL computes its inverse leaf size
  const float3 inv = make_float3(1.0f / leaf[0], 1.0f / leaf[1], 1.0f / leaf[2]);
  const unsigned grid_n = blocks_for(n, VX_THREADS, 4 * 152);
  if (n)
  {
    k_vx_bounds<<<grid_n, VX_THREADS, 0, s>>>(in, n, meta);
    AMCL_LAUNCH_CHECK("k_vx_bounds");
  }
  uint32_t* kA = v->keys[0].as<uint32_t>();
  uint32_t* kB = v->keys[1].as<uint32_t>();
  uint32_t* vA = v->vals[0].as<uint32_t>();
  uint32_t* vB = v->vals[1].as<uint32_t>();
  uint32_t* hist = v->hist.as<uint32_t>();
  uint32_t* tiles = v->tiles.as<uint32_t>();
  uint32_t* starts = v->starts.as<uint32_t>();
  if (n)
  {
    k_vx_keys<<<grid_n, VX_THREADS, 0, s>>>(in, n, inv, meta, kA, vA);
    AMCL_LAUNCH_CHECK("k_vx_keys");
    for (int pass = 0; pass < 4; ++pass)
    {
      const int shift = 8 * pass;
      k_vx_hist<<<ntiles, VX_THREADS, 0, s>>>(kA, n, shift, hist, ntiles);
      AMCL_LAUNCH_CHECK("k_vx_hist");
      if ((rc = launch_vx_scan(hist, 256u * ntiles, nullptr, s)))
        return rc;
      k_vx_scatter<<<ntiles, VX_THREADS, 0, s>>>(kA, vA, kB, vB, n, shift, hist, ntiles);
      AMCL_LAUNCH_CHECK("k_vx_scatter");
      std::swap(kA, kB);
      std::swap(vA, vB);
    }
    // after an even number of passes the sorted keys are back in keys[0] / vals[0]
    k_vx_heads<<<ntiles, VX_THREADS, 0, s>>>(kA, n, tiles, nullptr);
    AMCL_LAUNCH_CHECK("k_vx_heads");
    if ((rc = launch_vx_scan(tiles, ntiles, &meta->n_out, s)))
      return rc;
    k_vx_heads<<<ntiles, VX_THREADS, 0, s>>>(kA, n, tiles, starts);
    AMCL_LAUNCH_CHECK("k_vx_heads");
    k_vx_centroids<<<blocks_for(n, VX_THREADS, 1u << 30), VX_THREADS, 0, s>>>(in, n, vA, starts, meta, out);
    AMCL_LAUNCH_CHECK("k_vx_centroids");
  }
  return AMCL_OK;
}

int voxel_read_count(amcl_voxel_s* v, cudaStream_t s, uint32_t* n_out)
{
  int rc;
  if ((rc = v->h_meta.ensure(sizeof(VoxelMeta))))
    return rc;
  AMCL_CUDA_TRY(cudaMemcpyAsync(v->h_meta.p, v->meta.p, sizeof(VoxelMeta), cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  *n_out = v->h_meta.as<VoxelMeta>()->n_out;
  return AMCL_OK;
}

int voxel_check_leaf(const float leaf[3], const char* fn)
{
  for (int a = 0; a < 3; ++a)
    if (!(leaf[a] > 0.0f) || !std::isfinite(leaf[a]) || !std::isfinite(1.0f / leaf[a]))
      return fail(AMCL_EINVAL, std::string(fn) + ": leaf sizes must be positive and finite");
  return AMCL_OK;
}
}  // namespace amcl

using namespace amcl;

extern "C" int amcl_voxel_create(amcl_voxel_t* out, void* stream)
{
  if (!out)
    return fail(AMCL_EINVAL, "amcl_voxel_create: null out");
  auto* v = new (std::nothrow) amcl_voxel_s();
  if (!v)
    return fail(AMCL_ENOMEM, "amcl_voxel_create: host allocation");
  int rc = v->st.init(stream);
  if (rc)
  {
    delete v;
    return rc;
  }
  *out = v;
  return AMCL_OK;
}

extern "C" int amcl_voxel_destroy(amcl_voxel_t v)
{
  if (!v)
    return AMCL_OK;
  cudaStreamSynchronize(v->st.s);
  delete v;
  return AMCL_OK;
}

extern "C" int amcl_voxel_stream(amcl_voxel_t v, void** stream)
{
  if (!v || !stream)
    return fail(AMCL_EINVAL, "amcl_voxel_stream: bad arguments");
  *stream = v->st.s;
  return AMCL_OK;
}

extern "C" int amcl_voxel_filter(amcl_voxel_t v, const float* xyz, uint64_t n, uint32_t stride_floats, float leaf_x,
                                 float leaf_y, float leaf_z, float* out4, uint64_t cap, uint64_t* n_out)
{
  if (!v || (n && !xyz) || stride_floats < 3 || !n_out || (cap && !out4))
    return fail(AMCL_EINVAL, "amcl_voxel_filter: bad arguments");
  if (n > VX_MAX_POINTS)
    return fail(AMCL_ERANGE, "amcl_voxel_filter: more than 2^30 points");
  const float leaf[3] = { leaf_x, leaf_y, leaf_z };
  int rc;
  if ((rc = voxel_check_leaf(leaf, "amcl_voxel_filter")))
    return rc;
  std::lock_guard<std::mutex> lock(v->mu);
  cudaStream_t s = v->st.s;
  const size_t nb = std::max<uint64_t>(n, 1) * 16;
  if ((rc = v->h_in.ensure(nb)) || (rc = v->in.ensure(nb)) || (rc = v->out.ensure(nb)))
    return rc;
  pack_cloud(xyz, static_cast<uint32_t>(n), stride_floats, v->h_in.as<float4>());
  if (n)
    AMCL_CUDA_TRY(cudaMemcpyAsync(v->in.p, v->h_in.p, n * 16, cudaMemcpyHostToDevice, s));
  if ((rc = voxel_enqueue(v, v->in.as<float4>(), static_cast<uint32_t>(n), leaf, v->out.as<float4>(), s)))
    return rc;
  uint32_t m = 0;
  if (n && (rc = voxel_read_count(v, s, &m)))
    return rc;
  *n_out = m;
  if (m > cap)
    return fail(AMCL_ERANGE, "amcl_voxel_filter: output holds fewer points than the filter produced");
  if (m)
  {
    if ((rc = v->h_out.ensure(m * 16ull)))
      return rc;
    AMCL_CUDA_TRY(cudaMemcpyAsync(v->h_out.p, v->out.p, m * 16ull, cudaMemcpyDeviceToHost, s));
    AMCL_CUDA_TRY(cudaStreamSynchronize(s));
    std::memcpy(out4, v->h_out.p, m * 16ull);
  }
  return AMCL_OK;
}

extern "C" int amcl_voxel_filter_dev(amcl_voxel_t v, const void* in_f4_dev, uint64_t n, float leaf_x, float leaf_y,
                                     float leaf_z, void* out_f4_dev, uint64_t* n_out)
{
  if (!v || (n && (!in_f4_dev || !out_f4_dev)) || !n_out || (reinterpret_cast<uintptr_t>(in_f4_dev) & 15) ||
      (reinterpret_cast<uintptr_t>(out_f4_dev) & 15))
    return fail(AMCL_EINVAL, "amcl_voxel_filter_dev: bad arguments (16-byte aligned float4 buffers)");
  if (n > VX_MAX_POINTS)
    return fail(AMCL_ERANGE, "amcl_voxel_filter_dev: more than 2^30 points");
  const float leaf[3] = { leaf_x, leaf_y, leaf_z };
  int rc;
  if ((rc = voxel_check_leaf(leaf, "amcl_voxel_filter_dev")))
    return rc;
  std::lock_guard<std::mutex> lock(v->mu);
  cudaStream_t s = v->st.s;
  if ((rc = voxel_enqueue(v, static_cast<const float4*>(in_f4_dev), static_cast<uint32_t>(n), leaf,
                          static_cast<float4*>(out_f4_dev), s)))
    return rc;
  uint32_t m = 0;
  if (n && (rc = voxel_read_count(v, s, &m)))
    return rc;
  *n_out = m;
  return AMCL_OK;
}
