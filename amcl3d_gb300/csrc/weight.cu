// Per-particle scan-to-map likelihood: Grid3d::computeCloudWeight
// (amcl3d/src/Grid3d.cpp:133-199) for every in-map particle, fused with the
// range-beacon weight ParticleFilter::computeRangeWeight (ParticleFilter.cpp:224-244)
// and with the exact sums of both weights over the in-map particles that the
// normalisation of ParticleFilter::update needs (ParticleFilter.cpp:129-153).
//
// Two kernels compute the same bits:
//  * fused: one thread per particle walks the whole cloud in cloud order (the
//    scan is staged through shared memory as float4 chunks read by every thread of
//    the block: a broadcast), gathering the cell probability and summing it in
//    float in the reference's order.  Used when there are enough particles to fill
//    the GPU.
//  * two-phase: for few particles, phase 1 spreads (particle tile x point slice)
//    blocks over every SM, each warp holding 32 particles (one per lane) and
//    writing the gathered probability (or -1 for a skipped point) to a scratch
//    slab laid out [tile][point][lane]; phase 2 gives each tile one warp that
//    bulk-copies its slab through shared memory (cp.async.bulk on an mbarrier
//    ring) and adds the values in cloud order, so the float sum is the same as the
//    reference's running sum.
// Both are issue-bound on the per-point arithmetic (the gathers hit L2), so the
// point loop is specialised per transform mode (locate.cuh) and chunks are padded
// with NaN points to a multiple of the unroll so the loop carries no bounds checks.
#include "bulk.cuh"
#include "exact.cuh"
#include "grid.cuh"
#include "weight_dev.cuh"

using namespace amcl;

namespace
{
constexpr int WT_THREADS = 192;  // 6 warps; 4 blocks per SM by registers (80 per thread)
constexpr int WT_CHUNK = 1024;  // points staged per block iteration (16 KB)

template <int STORAGE, int SUM, int TAB, int FS = 0>
__global__ __launch_bounds__(WT_THREADS, 4) void k_weight_fused(WeightArgs a, const __grid_constant__ GridView g)
{
  extern __shared__ __align__(16) unsigned char smem[];
  float4* s_pts = reinterpret_cast<float4*>(smem);
  float4* s_rg = s_pts + WT_CHUNK;
  X320* s_part = reinterpret_cast<X320*>(s_rg + MAX_RANGES);
  float2* s_tab = reinterpret_cast<float2*>(s_part + 2 * (WT_THREADS / 32));
  // The locate tables are only read per point (a range-only update has no grid).
  if (a.N && TAB == TAB_SHARED)
    load_tables(g, s_tab);
  for (uint32_t i = threadIdx.x; i < a.nr; i += blockDim.x)
    s_rg[i] = a.ranges[i];
  weigh_block<STORAGE, SUM, TAB, FS>(a, g, blockIdx.x * blockDim.x, WT_CHUNK, s_pts, s_rg, s_part, s_tab);
}

// ---- two-phase ----------------------------------------------------------------------------
constexpr int TP_WARPS = 8;
constexpr int TP_PTS_PER_WARP = 32;
constexpr int TP_PTS_PER_BLOCK = TP_WARPS * TP_PTS_PER_WARP;

struct __align__(16) PartRec
{
  PartXf xf;
  int inm;
};

template <int STORAGE>
__global__ __launch_bounds__(TP_WARPS * 32) void k_weight_tile_vals(WeightArgs a, GridView g)
{
  extern __shared__ __align__(16) unsigned char smem[];
  float4* s_pts = reinterpret_cast<float4*>(smem);
  PartRec* s_rec = reinterpret_cast<PartRec*>(s_pts + TP_PTS_PER_BLOCK);
  float2* tab = reinterpret_cast<float2*>(s_rec + 32);  // used only when the grid's tables are staged
  if (tables_staged(g))
    load_tables(g, tab);
  const uint32_t tile = blockIdx.x;
  const uint32_t base = blockIdx.y * TP_PTS_PER_BLOCK;
  const uint32_t cnt = base < a.N ? min(static_cast<uint32_t>(TP_PTS_PER_BLOCK), a.N - base) : 0u;
  for (uint32_t i = threadIdx.x; i < TP_PTS_PER_BLOCK; i += blockDim.x)
  {
    const float nan = __int_as_float(0x7FC00000);
    s_pts[i] = i < cnt ? stage_point(a.cloud[base + i], a.yaw_only != 0) : make_float4(nan, nan, nan, 0.0f);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (wid == 0)
  {
    const uint32_t p = tile * 32 + lane;
    PartRec r;
    r.inm = 0;
    r.xf.exact = 1;
    if (p < a.P)
    {
      const float4 pose = a.pose[p];
      r.inm = (a.ignore_map || into_map(g, pose.x, pose.y, pose.z)) ? 1 : 0;
      if (r.inm)
        make_partxf(g, a.sr, a.cr, a.sp, a.cp, pose.x, pose.y, pose.z, pose.w, r.xf);
    }
    s_rec[lane] = r;
  }
  __syncthreads();
  const PartRec rec = s_rec[lane];
  const bool warp_exact = __all_sync(0xFFFFFFFFu, rec.xf.exact != 0);
  if (!rec.inm)
    return;
  float* out = a.scratch + (static_cast<uint64_t>(tile) * a.N) * 32 + lane;
  const uint32_t k0 = wid * TP_PTS_PER_WARP;
  if (warp_exact && a.yaw_only)
    tile_values<STORAGE, XF_YAW, TAB_EITHER>(s_pts, k0, TP_PTS_PER_WARP, cnt, tab, g, rec.xf, out, base);
  else if (warp_exact)
    tile_values<STORAGE, XF_EXACT, TAB_EITHER>(s_pts, k0, TP_PTS_PER_WARP, cnt, tab, g, rec.xf, out, base);
  else
    tile_values<STORAGE, XF_GENERAL, TAB_EITHER>(s_pts, k0, TP_PTS_PER_WARP, cnt, tab, g, rec.xf, out, base);
}

constexpr int TR_STAGE_PTS = 128;  // points per stage: 128 x 32 lanes x 4 B = 16 KB
constexpr int TR_STAGES = 4;

template <int SUM>
__global__ __launch_bounds__(32) void k_weight_tile_reduce(WeightArgs a, GridView g)
{
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_buf = reinterpret_cast<float*>(smem);  // TR_STAGES x TR_STAGE_PTS x 32
  __shared__ __align__(8) uint64_t s_bar[TR_STAGES];
  __shared__ __align__(8) uint64_t s_probe;  // AMCL_OPT_WAIT_PROBE: a barrier nothing completes
  __shared__ float4 s_rg[MAX_RANGES];
  const int lane = threadIdx.x;
  const uint32_t tile = blockIdx.x;
  const uint32_t p = tile * 32 + lane;
  for (uint32_t i = lane; i < a.nr; i += 32)
    s_rg[i] = a.ranges[i];
  float4 pose = make_float4(0.f, 0.f, 0.f, 0.f);
  const bool active = p < a.P;
  if (active)
    pose = a.pose[p];
  const bool inm = active && (a.ignore_map || into_map(g, pose.x, pose.y, pose.z));
  const bool any = __any_sync(0xFFFFFFFFu, inm);
  if (lane == 0)
  {
    for (int s = 0; s < TR_STAGES; ++s)
      mbar_init(&s_bar[s], 1);
    mbar_init(&s_probe, 1);
  }
  mbar_fence_init();
  __syncwarp();
  const float* slab = a.scratch + static_cast<uint64_t>(tile) * a.N * 32;
  const uint32_t nst = (a.N + TR_STAGE_PTS - 1) / TR_STAGE_PTS;
  CloudSum<SUM> acc;
  // The wait probe gives up (short budget) before any copy is issued, so the kernel
  // leaves with nothing in flight; it exercises the error path of the bounded waits.
  bool ok = a.wait_probe ? __all_sync(0xFFFFFFFFu, mbar_wait_bounded(&s_probe, 0, a.err, 1024u)) : true;
  if (ok && any && a.N)
  {
    if (lane == 0)
      for (uint32_t st = 0; st < min(nst, static_cast<uint32_t>(TR_STAGES)); ++st)
      {
        const uint32_t pts = min(static_cast<uint32_t>(TR_STAGE_PTS), a.N - st * TR_STAGE_PTS);
        mbar_arrive_expect_tx(&s_bar[st], pts * 128u);
        bulk_g2s(s_buf + st * TR_STAGE_PTS * 32, slab + static_cast<uint64_t>(st) * TR_STAGE_PTS * 32, pts * 128u,
                 &s_bar[st]);
      }
    uint32_t failed = 0;
    for (uint32_t st = 0; st < nst; ++st)
    {
      const int slot = st % TR_STAGES;
      const uint32_t parity = (st / TR_STAGES) & 1u;
      // every lane leaves together if any lane's wait gave up (the loop holds warp syncs)
      if (!__all_sync(0xFFFFFFFFu, mbar_wait_bounded(&s_bar[slot], parity, a.err)))
      {
        ok = false;
        failed = st;
        break;
      }
      const uint32_t pts = min(static_cast<uint32_t>(TR_STAGE_PTS), a.N - st * TR_STAGE_PTS);
      const float* buf = s_buf + slot * TR_STAGE_PTS * 32;
      if (inm)
      {
        for (uint32_t k = 0; k < pts; ++k)
        {
          const float v = buf[k * 32 + lane];
          if (v >= 0.0f)
            acc.add(v);
        }
      }
      __syncwarp();
      const uint32_t nxt = st + TR_STAGES;
      if (lane == 0 && nxt < nst)
      {
        const uint32_t np = min(static_cast<uint32_t>(TR_STAGE_PTS), a.N - nxt * TR_STAGE_PTS);
        mbar_arrive_expect_tx(&s_bar[slot], np * 128u);
        bulk_g2s(s_buf + slot * TR_STAGE_PTS * 32, slab + static_cast<uint64_t>(nxt) * TR_STAGE_PTS * 32, np * 128u,
                 &s_bar[slot]);
      }
    }
    if (!ok)
    {
      // Drain what is still in flight (bounded) before leaving: the wait gave up at
      // stage `failed`, when stages [failed, issued) had been issued; stage j lands on
      // slot j % TR_STAGES in the phase of parity (j / TR_STAGES) & 1.
      const uint32_t issued = min(nst, failed + static_cast<uint32_t>(TR_STAGES));
      for (uint32_t j = failed; j < issued; ++j)
        mbar_wait_bounded(&s_bar[j % TR_STAGES], (j / TR_STAGES) & 1u, nullptr);
    }
  }
  float wpv = 0.0f, wrv = 0.0f;
  if (inm && ok)
  {
    wpv = acc.weight();
    wrv = range_weight(pose.x, pose.y, pose.z, s_rg, static_cast<int>(a.nr), a.k1, a.k2);
    a.wp[p] = wpv;
    a.wr[p] = wrv;
  }
  if (active && a.inmap)
    a.inmap[p] = inm ? 1 : 0;
  X320 xa = (inm && ok) ? x320_from_float(wpv) : x320_zero();
  X320 xb = (inm && ok) ? x320_from_float(wrv) : x320_zero();
  xa = x320_warp_sum(xa);
  xb = x320_warp_sum(xb);
  if (lane == 0)
  {
    if (a.acc_wp)
      x320_atomic_add(a.acc_wp, xa);
    if (a.acc_wr)
      x320_atomic_add(a.acc_wr, xb);
  }
}

size_t table_bytes(const GridView& g)
{
  return static_cast<size_t>(table_staged_floats(g)) * sizeof(float);
}

template <int STORAGE, int SUM>
int launch_fused(const WeightArgs& a, const GridView& g, cudaStream_t s)
{
  const size_t smem = WT_CHUNK * sizeof(float4) + MAX_RANGES * sizeof(float4) + 2 * (WT_THREADS / 32) * sizeof(X320) +
                      (a.N && tables_staged(g) ? table_bytes(g) : 0);
  static std::atomic<uint64_t> attr_done{ 0 };
  const int rc = once_per_device(attr_done, [] {
    AMCL_CUDA_TRY(cudaFuncSetAttribute(k_weight_fused<STORAGE, SUM, TAB_SHARED>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    AMCL_CUDA_TRY(cudaFuncSetAttribute(k_weight_fused<STORAGE, SUM, TAB_GLOBAL>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    AMCL_CUDA_TRY(cudaFuncSetAttribute(k_weight_fused<STORAGE, SUM, TAB_SHARED, 1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    AMCL_CUDA_TRY(cudaFuncSetAttribute(k_weight_fused<STORAGE, SUM, TAB_GLOBAL, 1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    AMCL_CUDA_TRY(cudaFuncSetAttribute(k_weight_fused<STORAGE, SUM, TAB_SHARED, 2>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    AMCL_CUDA_TRY(cudaFuncSetAttribute(k_weight_fused<STORAGE, SUM, TAB_GLOBAL, 2>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    return static_cast<int>(AMCL_OK);
  });
  if (rc)
    return rc;
  const int fv = fast_variant(g);
  const unsigned nb = ceil_div(a.P, WT_THREADS);
  if (fv == 1 && tables_staged(g))
    k_weight_fused<STORAGE, SUM, TAB_SHARED, 1><<<nb, WT_THREADS, smem, s>>>(a, g);
  else if (fv == 1)
    k_weight_fused<STORAGE, SUM, TAB_GLOBAL, 1><<<nb, WT_THREADS, smem, s>>>(a, g);
  else if (fv == 2 && tables_staged(g))
    k_weight_fused<STORAGE, SUM, TAB_SHARED, 2><<<nb, WT_THREADS, smem, s>>>(a, g);
  else if (fv == 2)
    k_weight_fused<STORAGE, SUM, TAB_GLOBAL, 2><<<nb, WT_THREADS, smem, s>>>(a, g);
  else if (tables_staged(g))
    k_weight_fused<STORAGE, SUM, TAB_SHARED><<<ceil_div(a.P, WT_THREADS), WT_THREADS, smem, s>>>(a, g);
  else
    k_weight_fused<STORAGE, SUM, TAB_GLOBAL><<<ceil_div(a.P, WT_THREADS), WT_THREADS, smem, s>>>(a, g);
  AMCL_LAUNCH_CHECK("k_weight_fused");
  return AMCL_OK;
}

template <int STORAGE, int SUM>
int launch_two_phase(const WeightArgs& a, const GridView& g, cudaStream_t s)
{
  const size_t smem1 = TP_PTS_PER_BLOCK * sizeof(float4) + 32 * sizeof(PartRec) + (tables_staged(g) ? table_bytes(g) : 0);
  const size_t smem2 = static_cast<size_t>(TR_STAGES) * TR_STAGE_PTS * 32 * sizeof(float);
  static std::atomic<uint64_t> attr_done{ 0 };
  const int rc = once_per_device(attr_done, [] {
    AMCL_CUDA_TRY(
        cudaFuncSetAttribute(k_weight_tile_vals<STORAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    AMCL_CUDA_TRY(
        cudaFuncSetAttribute(k_weight_tile_reduce<SUM>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    return static_cast<int>(AMCL_OK);
  });
  if (rc)
    return rc;
  const unsigned tiles = ceil_div(a.P, 32);
  if (a.N)
  {
    dim3 grid1(tiles, ceil_div(a.N, TP_PTS_PER_BLOCK));
    k_weight_tile_vals<STORAGE><<<grid1, TP_WARPS * 32, smem1, s>>>(a, g);
    AMCL_LAUNCH_CHECK("k_weight_tile_vals");
  }
  k_weight_tile_reduce<SUM><<<tiles, 32, smem2, s>>>(a, g);
  AMCL_LAUNCH_CHECK("k_weight_tile_reduce");
  return AMCL_OK;
}

template <int STORAGE>
int launch_storage(const WeightArgs& a, const GridView& g, cudaStream_t s)
{
  const bool tp = a.kernel == 2;
  if (a.cloud_sum == 0)
    return tp ? launch_two_phase<STORAGE, 0>(a, g, s) : launch_fused<STORAGE, 0>(a, g, s);
  return tp ? launch_two_phase<STORAGE, 1>(a, g, s) : launch_fused<STORAGE, 1>(a, g, s);
}
}  // namespace

namespace amcl
{
uint64_t two_phase_scratch_floats(uint32_t P, uint32_t N)
{
  return static_cast<uint64_t>(ceil_div(P, 32)) * 32ull * N;
}

int choose_weight_kernel(uint32_t P, uint32_t N)
{
  // Fused when one thread per particle already gives every SM several warps.
  const uint64_t warps = ceil_div(P, 32);
  if (warps >= 8ull * static_cast<uint64_t>(device_sm_count()))
    return 1;
  if (two_phase_scratch_floats(P, N) * 4ull > (1ull << 30))
    return 1;
  return 2;
}

void pack_cloud(const float* xyz, uint32_t n, uint32_t stride, float4* out)
{
  for (uint32_t i = 0; i < n; ++i)
    out[i] = make_float4(xyz[static_cast<uint64_t>(i) * stride], xyz[static_cast<uint64_t>(i) * stride + 1],
                         xyz[static_cast<uint64_t>(i) * stride + 2], 0.0f);
}

int launch_cloud_weight(amcl_grid_s* g, const WeightArgs& a, cudaStream_t s)
{
  if (a.nr > MAX_RANGES)
    return fail(AMCL_ERANGE, "update: more than 64 range measurements");
  if (a.P == 0)
    return AMCL_OK;
  WeightArgs b = a;
  if (b.N == 0)
    b.kernel = 1;  // no points: nothing to spread, the fused kernel writes wp = 0
  if (b.kernel == 2 && (!b.scratch || b.scratch_floats < two_phase_scratch_floats(b.P, b.N)))
    return fail(AMCL_EINVAL, "two-phase weighting without a large enough scratch buffer");
  if (b.N && !g->view.T2)
    return fail(AMCL_ESTATE, "cloud weighting without a built grid");
  // roll = pitch = 0 (as the float parameters of computeCloudWeight): yaw-only points.
  b.yaw_only = (b.sr == 0.0f && b.sp == 0.0f && b.cr == 1.0f && b.cp == 1.0f) ? 1 : 0;
  switch (g->view.storage)
  {
    case AMCL_GRID_F16:
      return launch_storage<AMCL_GRID_F16>(b, g->view, s);
    case AMCL_GRID_U8:
      return launch_storage<AMCL_GRID_U8>(b, g->view, s);
    default:
      return launch_storage<AMCL_GRID_F32>(b, g->view, s);
  }
}
}  // namespace amcl

// ---- batch of Grid3d::computeCloudWeight calls ---------------------------------------------

extern "C" int amcl_grid_cloud_weights(amcl_grid_t g, const float* poses4, uint32_t P, const float* xyz, uint32_t n,
                                       uint32_t stride_floats, float roll, float pitch, float* out)
{
  if (!g || (P && (!poses4 || !out)) || (n && !xyz) || stride_floats < 3)
    return fail(AMCL_EINVAL, "amcl_grid_cloud_weights: bad arguments");
  if (!P)
    return AMCL_OK;
  if (!g->built)
  {
    for (uint32_t i = 0; i < P; ++i)
      out[i] = 0.0f;  // Grid3d.cpp:136-137
    return AMCL_OK;
  }
  cudaStream_t s = g->st.s;
  DevBuf d_pose, d_cloud, d_wp, d_wr, d_scratch, d_err;
  int rc;
  if ((rc = d_pose.ensure(P * 16ull)) || (rc = d_cloud.ensure(std::max<uint64_t>(n, 1) * 16)) ||
      (rc = d_wp.ensure(P * 4ull)) || (rc = d_wr.ensure(P * 4ull)) || (rc = d_err.ensure(4)))
    return rc;
  std::vector<float4> hc(n);
  pack_cloud(xyz, n, stride_floats, hc.data());
  AMCL_CUDA_TRY(cudaMemcpyAsync(d_pose.p, poses4, P * 16ull, cudaMemcpyHostToDevice, s));
  if (n)
    AMCL_CUDA_TRY(cudaMemcpyAsync(d_cloud.p, hc.data(), n * 16ull, cudaMemcpyHostToDevice, s));
  AMCL_CUDA_TRY(cudaMemsetAsync(d_err.p, 0, 4, s));
  WeightArgs a{};
  a.pose = d_pose.as<float4>();
  a.P = P;
  a.cloud = d_cloud.as<float4>();
  a.N = n;
  a.sr = sinf(roll);
  a.cr = cosf(roll);
  a.sp = sinf(pitch);
  a.cp = cosf(pitch);
  a.wp = d_wp.as<float>();
  a.wr = d_wr.as<float>();
  a.err = d_err.as<int>();
  a.ignore_map = 1;
  a.kernel = choose_weight_kernel(P, n);
  if (a.kernel == 2)
  {
    if ((rc = d_scratch.ensure(two_phase_scratch_floats(P, n) * 4)))
      return rc;
    a.scratch = d_scratch.as<float>();
    a.scratch_floats = d_scratch.bytes / 4;
  }
  grid_apply_l2_window(g, s);
  if ((rc = launch_cloud_weight(g, a, s)))
    return rc;
  int e = 0;
  AMCL_CUDA_TRY(cudaMemcpyAsync(out, d_wp.p, P * 4ull, cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(&e, d_err.p, 4, cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  if (e)
    return fail(AMCL_ETIMEDOUT, "amcl_grid_cloud_weights: a bounded device-side wait gave up");
  return AMCL_OK;
}
