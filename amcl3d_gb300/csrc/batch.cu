// Many particle filters stepped together: one launch sequence (predict, cloud
// weights, blend, normalise + mean, resample) for every filter with a staged step,
// captured once in a CUDA graph and replayed.
//
// Memory: fixed arenas sized at creation (the HBM budget new filters are admitted
// against): particle SoA arrays double-buffered like a single filter's, one range of
// 256-aligned particles per filter slot; clouds, ranges and the per-step descriptors
// are packed each step into pinned staging and copied with one transfer each.
//
// Work distribution: every kernel runs a fixed grid (a multiple of the SM count) and
// walks a list of work items, so grid shapes never change with the batch composition
// and the captured graph stays valid; only the copy sizes are updated per step.  The
// cloud weighting takes (filter, particle tile) items, longest first, from a global
// atomic counter (no spin-waits).  Each item is the fused one-thread-per-particle
// weighting of a single filter, so every filter's weights, sums, mean and resample
// indices are bit-identical to stepping it alone (the normalisation sums are exact
// integer sums, independent of how items interleave).  Items are queued per (storage,
// sum) class and grid slot: up to four distinct grids are launch arguments, so their
// fields come from the constant bank (three 256-thread blocks per SM fit in registers).
//
// Small steps (too few particle tiles to fill the GPU, the served case) split the
// scan instead: items are (32-particle tile, 512-point slice) pairs spread over every
// SM, each writing its probabilities to a [tile][point][lane] scratch slab; the block
// that completes a tile's last slice (a per-tile atomic counter) sums the tile's slab
// in cloud order while it is still in L2.  The float sums, and so every result, are
// the same as the fused path's.  The per-particle transforms of a split step are
// computed once, after predict.  Each step's graph holds only the weighting launches
// of the fused queues and split classes it uses.
//
// Tuning: the particle tile (threads per block of the weighting kernel) and the point
// tile (scan points staged in shared memory per iteration) are chosen by
// amcl_batch_autotune, which times the weighting phase of the staged step under each
// candidate shape.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "bulk.cuh"
#include "filter_dev.cuh"
#include "grid.cuh"
#include "weight_dev.cuh"

using namespace amcl;

namespace
{
enum : uint32_t
{
  ST_PREDICT = 1,
  ST_UPDATE = 2,
  ST_RESAMPLE = 4
};

struct SlotStep
{
  uint32_t slot, flags, P, N, nr, cur;
  uint32_t split, tile_base;  // split: point-parallel weighting; first 32-particle tile counter
  uint64_t p_off, c_off;
  uint64_t sc_off, xf_off;    // split: slab offset (floats), transform record offset
  uint32_t r_off, cloud_sum;
  float sr, cr, sp, cp, k1, k2;
  int yaw_only;
  double alpha;
  PredictArgs pred;
  float factor, r;
  int32_t gslot;  // index of g in the launch's GridSet, -1: read g from here
  GridView g;
};

// The grids of a batch passed by value to the fused weighting launches: a step whose
// grid is in the set reads the grid's fields (bounds, strides, cell array) from the
// kernel's constant bank, as the single-filter kernel does, rather than holding them
// in registers after a load from the step descriptor.
constexpr int BATCH_GRIDS = 4;
struct GridSet
{
  GridView g[BATCH_GRIDS];
};

// Per-particle transform of a split step (computed once per step).
struct SplitRec
{
  PartXf xf;
  int inm;
};

struct BatchDev
{
  float4* pose[2];
  float* w[2];
  float* wp[2];
  float* wr[2];
  uint8_t* inmap;
  int32_t* hi;
  X320* blocksum;
  unsigned long long* acc;  // per slot ACC_WORDS
  PFStats* stats;           // per slot
  const float4* cloud;
  const float4* ranges;
  const SlotStep* steps;
  const uint32_t* counts;  // [0] steps, [1] block items, [2] weight items, then the queues' item ranges
  const uint2* blk_items;  // (step, local block)
  const uint2* wt_items;   // (step, particle tile)
  unsigned int* counter;   // weighting work queues: fused classes, then split classes
  SplitRec* xf;            // split steps' particle transforms
  float* scratch;          // split steps' probability slabs
  unsigned int* tile_done; // split: slices finished per 32-particle tile (reset by the last)
};

constexpr int GRID_BLOCKS_PER_SM = 4;

__global__ __launch_bounds__(NT) void k_b_predict(BatchDev d)
{
  const uint32_t nitems = d.counts[1];
  for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x)
  {
    const uint2 bi = d.blk_items[it];
    const SlotStep& st = d.steps[bi.x];
    if (!(st.flags & ST_PREDICT))
      continue;
    const uint32_t i = bi.y * NT + threadIdx.x;
    if (i < st.P)
      predict_particle(i, d.pose[st.cur] + st.p_off, st.pred);
  }
}

template <int STORAGE, int SUM, int TAB, int FS>
__device__ __forceinline__ void b_weigh(const BatchDev& d, const SlotStep& st, const GridView& g, uint32_t tile,
                                        uint32_t chunk, float4* s_pts, const float4* s_rg, X320* s_part,
                                        const float2* s_tab)
{
  WeightArgs a{};
  a.pose = d.pose[st.cur] + st.p_off;
  a.P = st.P;
  a.cloud = d.cloud + st.c_off;
  a.N = st.N;
  a.sr = st.sr;
  a.cr = st.cr;
  a.sp = st.sp;
  a.cp = st.cp;
  a.nr = st.nr;
  a.k1 = st.k1;
  a.k2 = st.k2;
  a.wp = d.wp[st.cur] + st.p_off;
  a.wr = d.wr[st.cur] + st.p_off;
  a.inmap = d.inmap + st.p_off;
  a.acc_wp = d.acc + static_cast<uint64_t>(st.slot) * ACC_WORDS + ACC_WP * NDIG;
  a.acc_wr = d.acc + static_cast<uint64_t>(st.slot) * ACC_WORDS + ACC_WR * NDIG;
  a.yaw_only = st.yaw_only;
  weigh_block<STORAGE, SUM, TAB, FS>(a, g, tile * blockDim.x, chunk, s_pts, s_rg, s_part, s_tab);
}

// Persistent: blocks take (filter, particle tile) items of one fused queue until it is
// empty.  A fused queue holds the items of one (storage, sum) class on one grid slot:
// slots 0..BATCH_GRIDS-1 are launched with their grid as a kernel argument (its fields
// read from the constant bank: fewer registers, three 256-thread blocks per SM), the
// last slot reads each step's grid from its descriptor.
constexpr int N_CLASSES = 6;                         // 3 storages x 2 sum modes
constexpr int N_GSLOTS = BATCH_GRIDS + 1;            // grid slots + the descriptor path
constexpr int N_FUSED_Q = N_CLASSES * N_GSLOTS;      // fused queues
constexpr int N_COUNTERS = N_FUSED_Q + N_CLASSES;    // fused queues, then split classes
constexpr int SPLIT_MASK_SHIFT = 32;                 // class mask: bit q fused queue q, bit 32 + c split class c
static_assert(N_FUSED_Q <= SPLIT_MASK_SHIFT, "fused queues fit below the split bits");
// counts: [0] steps, [1] block items, [2] weight items, [FQ_BASE + 2q, FQ_BASE + 2q + 1)
// fused queue q's items, [SQ_BASE + 2c, SQ_BASE + 2c + 1) split class c's items
constexpr int FQ_BASE = 4;
constexpr int SQ_BASE = FQ_BASE + 2 * N_FUSED_Q;
constexpr int COUNT_WORDS = SQ_BASE + 2 * N_CLASSES;
__host__ __device__ inline int weight_class(int storage, int cloud_sum) { return storage * 2 + (cloud_sum ? 1 : 0); }
__host__ __device__ inline int fused_queue(int cls, int gslot) { return cls * N_GSLOTS + (gslot < 0 ? BATCH_GRIDS : gslot); }

// FS: the slot grid has floor constants (only with PG; set by the launcher).  The general
// yaw loop (FS 2) runs 2 blocks of 256 per SM, whose 128 registers a thread hold it
// without spilling.
template <int STORAGE, int SUM, bool PG, int MAXT, int FS = 0>
__global__ __launch_bounds__(MAXT, MAXT >= 512 ? 1 : (FS == 2 ? 2 : 3)) void k_b_weight(BatchDev d,
                                                                                        const __grid_constant__ GridView gp,
                                                                                        uint32_t q, uint32_t chunk)
{
  extern __shared__ __align__(16) unsigned char smem[];
  float4* s_pts = reinterpret_cast<float4*>(smem);
  float4* s_rg = s_pts + chunk;
  X320* s_part = reinterpret_cast<X320*>(s_rg + MAX_RANGES);
  float2* s_tab = reinterpret_cast<float2*>(s_part + 2 * 32);
  __shared__ uint32_t s_item;
  __shared__ int s_loaded;
  const uint32_t begin = d.counts[FQ_BASE + 2 * q], end = d.counts[FQ_BASE + 2 * q + 1];
  if (threadIdx.x == 0)
    s_loaded = -1;
  while (true)
  {
    __syncthreads();
    if (threadIdx.x == 0)
      s_item = begin + atomicAdd(d.counter + q, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    if (it >= end)
      break;
    const uint2 wi = d.wt_items[it];
    const SlotStep& st = d.steps[wi.x];
    if (s_loaded != static_cast<int>(wi.x))
    {
      if (st.N && tables_staged(st.g))
        load_tables(st.g, s_tab);  // larger tables stay in global memory
      for (uint32_t i = threadIdx.x; i < st.nr; i += blockDim.x)
        s_rg[i] = d.ranges[st.r_off + i];
      __syncthreads();
      if (threadIdx.x == 0)
        s_loaded = static_cast<int>(wi.x);
    }
    // slot grids always have staged tables (assign_grid_slots); descriptor grids may not
    b_weigh<STORAGE, SUM, PG ? TAB_SHARED : TAB_EITHER, FS>(d, st, PG ? gp : st.g, wi.y, chunk, s_pts, s_rg, s_part,
                                                        s_tab);
  }
}

// Transforms of the particles of split steps (after predict, before the weighting).
__global__ __launch_bounds__(NT) void k_b_xf(BatchDev d)
{
  const uint32_t nitems = d.counts[1];
  for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x)
  {
    const uint2 bi = d.blk_items[it];
    const SlotStep& st = d.steps[bi.x];
    if (!st.split)
      continue;
    const uint32_t i = bi.y * NT + threadIdx.x;
    if (i >= st.P)
      continue;
    const float4 pose = d.pose[st.cur][st.p_off + i];
    SplitRec r;
    r.xf.exact = 1;
    r.inm = into_map(st.g, pose.x, pose.y, pose.z) ? 1 : 0;
    if (r.inm)
      make_partxf(st.g, st.sr, st.cr, st.sp, st.cp, pose.x, pose.y, pose.z, pose.w, r.xf);
    d.xf[st.xf_off + i] = r;
  }
}

constexpr int SP_WARPS = 8;
constexpr uint32_t SP_WARP_PTS = 64;                 // points per warp per split item
constexpr uint32_t SP_PTS = SP_WARPS * SP_WARP_PTS;  // points per split item
constexpr uint32_t SP_RED_PTS = 64;                  // slab points per reduction stage (8 KB)
constexpr uint32_t SP_RED_STAGES = 4;                // reduction stages in shared memory

__device__ __forceinline__ unsigned int atomic_add_acq_rel_gpu(unsigned int* p, unsigned int v)
{
  unsigned int r;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(r) : "l"(p), "r"(v) : "memory");
  return r;
}

// Offset (floats) of the reduction buffers in a split block's shared memory.
__host__ __device__ inline uint32_t split_red_offset(uint32_t tab_cap)
{
  const uint32_t bytes = SP_PTS * 16 + MAX_RANGES * 16 + (tab_cap + 3) * 4;  // staged tables: floats
  return ((bytes + 15) & ~15u) / 4;
}

// Persistent: blocks take (split step, tile * slices + slice) items of one class.
// Each warp covers SP_WARP_PTS points of the slice for the tile's 32 particles.  The
// block whose count completes the tile streams the tile's slab through shared memory
// (all warps copy, 8 KB stages, 3 in flight; warp 0 adds in cloud order).
template <int STORAGE, int SUM>
__global__ __launch_bounds__(SP_WARPS * 32, 3) void k_b_split(BatchDev d, uint32_t tab_cap)
{
  extern __shared__ __align__(16) unsigned char smem[];
  float4* s_pts = reinterpret_cast<float4*>(smem);
  float4* s_rg = s_pts + SP_PTS;
  float2* s_tab = reinterpret_cast<float2*>(s_rg + MAX_RANGES);
  float* s_red = reinterpret_cast<float*>(smem) + split_red_offset(tab_cap);  // SP_RED_STAGES x SP_RED_PTS x 32
  __shared__ uint32_t s_item;
  __shared__ int s_loaded;
  __shared__ int s_last;
  constexpr int cls = STORAGE * 2 + SUM;
  const uint32_t begin = d.counts[SQ_BASE + 2 * cls], end = d.counts[SQ_BASE + 2 * cls + 1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0)
    s_loaded = -1;
  while (true)
  {
    __syncthreads();
    if (threadIdx.x == 0)
      s_item = begin + atomicAdd(d.counter + N_FUSED_Q + cls, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    if (it >= end)
      break;
    const uint2 wi = d.wt_items[it];
    const SlotStep& st = d.steps[wi.x];
    const uint32_t nsl = (st.N + SP_PTS - 1) / SP_PTS;
    const uint32_t tile = wi.y / nsl, slice = wi.y - tile * nsl;
    const bool load = s_loaded != static_cast<int>(wi.x);  // read by all before thread 0 updates it below
    if (load)
    {
      if (tables_staged(st.g))
        load_tables(st.g, s_tab);  // larger tables stay in global memory
      for (uint32_t i = threadIdx.x; i < st.nr; i += blockDim.x)
        s_rg[i] = d.ranges[st.r_off + i];
    }
    const uint32_t base = slice * SP_PTS;
    const uint32_t cnt = min(SP_PTS, st.N - base);
    for (uint32_t i = threadIdx.x; i < SP_PTS; i += blockDim.x)
    {
      const float nan = __int_as_float(0x7FC00000);
      s_pts[i] = i < cnt ? stage_point(d.cloud[st.c_off + base + i], st.yaw_only != 0)
                         : make_float4(nan, nan, nan, 0.0f);
    }
    __syncthreads();
    if (load && threadIdx.x == 0)
      s_loaded = static_cast<int>(wi.x);
    const uint32_t p = tile * 32 + lane;
    SplitRec rec;
    rec.inm = 0;
    rec.xf.exact = 1;
    if (p < st.P)
      rec = d.xf[st.xf_off + p];
    const bool warp_exact = __all_sync(0xFFFFFFFFu, rec.xf.exact != 0);
    const float* slab = d.scratch + st.sc_off + static_cast<uint64_t>(tile) * st.N * 32;
    if (rec.inm)
    {
      float* out = const_cast<float*>(slab) + lane;
      const uint32_t k0 = wid * SP_WARP_PTS;
      if (warp_exact && st.yaw_only)
        tile_values<STORAGE, XF_YAW, TAB_EITHER>(s_pts, k0, SP_WARP_PTS, cnt, s_tab, st.g, rec.xf, out, base);
      else if (warp_exact)
        tile_values<STORAGE, XF_EXACT, TAB_EITHER>(s_pts, k0, SP_WARP_PTS, cnt, s_tab, st.g, rec.xf, out, base);
      else
        tile_values<STORAGE, XF_GENERAL, TAB_EITHER>(s_pts, k0, SP_WARP_PTS, cnt, s_tab, st.g, rec.xf, out, base);
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
      // Release: the block's slab writes (ordered before by the barrier) are visible
      // device-wide before the count; acquire: the last block sees every slice's.
      const unsigned int done = atomic_add_acq_rel_gpu(d.tile_done + st.tile_base + tile, 1u);
      s_last = done == nsl - 1 ? 1 : 0;
    }
    __syncthreads();
    if (!s_last)
      continue;
    // The tile's last slice: sum the slab in cloud order.  Every thread copies its
    // 16-byte pieces of the next stages with cp.async (SP_RED_STAGES - 1 in flight);
    // warp 0 adds each landed stage.
    const float4* slab4 = reinterpret_cast<const float4*>(slab);
    const uint32_t nst = (st.N + SP_RED_PTS - 1) / SP_RED_PTS;
    constexpr uint32_t F4_PER_STAGE = SP_RED_PTS * 8;  // 32 floats per point
    constexpr uint32_t F4_PER_THREAD = F4_PER_STAGE / (SP_WARPS * 32);
    const uint32_t f4_total = st.N * 8;
    float4* red4 = reinterpret_cast<float4*>(s_red);
    auto issue = [&](uint32_t sg) {
#pragma unroll
      for (uint32_t q = 0; q < F4_PER_THREAD; ++q)
      {
        const uint32_t f = q * SP_WARPS * 32 + threadIdx.x;
        const uint32_t gidx = sg * F4_PER_STAGE + f;
        if (gidx < f4_total)
          cp_async16(red4 + (sg % SP_RED_STAGES) * F4_PER_STAGE + f, slab4 + gidx);
      }
    };
#pragma unroll
    for (uint32_t sg = 0; sg + 1 < SP_RED_STAGES; ++sg)
    {
      if (sg < nst)
        issue(sg);
      cp_async_commit();
    }
    CloudSum<SUM> acc;
    for (uint32_t sg = 0; sg < nst; ++sg)
    {
      if (sg + SP_RED_STAGES - 1 < nst)
        issue(sg + SP_RED_STAGES - 1);
      cp_async_commit();
      cp_async_wait<SP_RED_STAGES - 1>();  // this thread's copies of stage sg have landed
      __syncthreads();                     // everyone's have
      if (wid == 0 && rec.inm)
      {
        const float* buf = s_red + (sg % SP_RED_STAGES) * SP_RED_PTS * 32;
        const uint32_t pts = min(SP_RED_PTS, st.N - sg * SP_RED_PTS);
        for (uint32_t k = 0; k < pts; ++k)
        {
          const float v = buf[k * 32 + lane];
          if (v >= 0.0f)
            acc.add(v);
        }
      }
      __syncthreads();  // the stage's buffer is free for the copy issued next
    }
    if (wid == 0)
    {
      float wpv = 0.0f, wrv = 0.0f;
      if (rec.inm)
      {
        const float4 pose = d.pose[st.cur][st.p_off + p];
        wpv = acc.weight();
        wrv = range_weight(pose.x, pose.y, pose.z, s_rg, static_cast<int>(st.nr), st.k1, st.k2);
        d.wp[st.cur][st.p_off + p] = wpv;
        d.wr[st.cur][st.p_off + p] = wrv;
      }
      if (p < st.P)
        d.inmap[st.p_off + p] = rec.inm ? 1 : 0;
      X320 xa = rec.inm ? x320_from_float(wpv) : x320_zero();
      X320 xb = rec.inm ? x320_from_float(wrv) : x320_zero();
      xa = x320_warp_sum(xa);
      xb = x320_warp_sum(xb);
      if (lane == 0)
      {
        unsigned long long* acc_s = d.acc + static_cast<uint64_t>(st.slot) * ACC_WORDS;
        x320_atomic_add(acc_s + ACC_WP * NDIG, xa);
        x320_atomic_add(acc_s + ACC_WR * NDIG, xb);
        d.tile_done[st.tile_base + tile] = 0u;  // ready for the next step
      }
    }
  }
}

__global__ __launch_bounds__(NT) void k_b_blend(BatchDev d)
{
  __shared__ double s_sum[2];
  __shared__ X320 s_part[NT / 32];
  const uint32_t nitems = d.counts[1];
  for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x)
  {
    const uint2 bi = d.blk_items[it];
    const SlotStep& st = d.steps[bi.x];
    if (!(st.flags & ST_UPDATE))
      continue;
    blend_block(bi.y, st.P, d.inmap + st.p_off, d.wp[st.cur] + st.p_off, d.wr[st.cur] + st.p_off,
                d.w[st.cur] + st.p_off, st.alpha, d.acc + static_cast<uint64_t>(st.slot) * ACC_WORDS, s_sum, s_part);
  }
}

__global__ __launch_bounds__(NT) void k_b_normalize(BatchDev d)
{
  __shared__ double s_sum[2];
  __shared__ X320 s_part[NORM_Q * (NT / 32)];
  const uint32_t nitems = d.counts[1];
  for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x)
  {
    const uint2 bi = d.blk_items[it];
    const SlotStep& st = d.steps[bi.x];
    if (!(st.flags & ST_UPDATE))
      continue;
    normalize_block(bi.y, st.P, d.pose[st.cur] + st.p_off, d.w[st.cur] + st.p_off,
                    d.acc + static_cast<uint64_t>(st.slot) * ACC_WORDS, d.blocksum + st.p_off / NT, s_sum, s_part);
  }
}

// One warp per step.
__global__ void k_b_finalize(BatchDev d)
{
  const uint32_t n = d.counts[0];
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t s = warp; s < n; s += nwarps)
  {
    const SlotStep& st = d.steps[s];
    if (st.flags & ST_UPDATE)
      finalize_stats_warp(d.acc + static_cast<uint64_t>(st.slot) * ACC_WORDS, d.stats + st.slot);
  }
}

__global__ __launch_bounds__(NT) void k_b_prefix(BatchDev d)
{
  __shared__ X320 s_scan[NT / 32];
  __shared__ X320 s_base;
  const uint32_t nitems = d.counts[1];
  for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x)
  {
    const uint2 bi = d.blk_items[it];
    const SlotStep& st = d.steps[bi.x];
    if (!(st.flags & ST_RESAMPLE))
      continue;
    prefix_hi_block(bi.y, st.P, d.w[st.cur] + st.p_off, d.blocksum + st.p_off / NT, st.r, st.factor,
                    d.hi + st.p_off, s_scan, &s_base);
  }
}

__global__ __launch_bounds__(NT) void k_b_gather(BatchDev d)
{
  const uint32_t nitems = d.counts[1];
  for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x)
  {
    const uint2 bi = d.blk_items[it];
    const SlotStep& st = d.steps[bi.x];
    if (!(st.flags & ST_RESAMPLE))
      continue;
    const uint32_t m = bi.y * NT + threadIdx.x;
    if (m < st.P)
    {
      const uint32_t o = 1 - st.cur;
      gather_particle(m, st.P, d.hi + st.p_off, d.pose[st.cur] + st.p_off, d.wp[st.cur] + st.p_off,
                      d.wr[st.cur] + st.p_off, d.pose[o] + st.p_off, d.w[o] + st.p_off, d.wp[o] + st.p_off,
                      d.wr[o] + st.p_off, st.factor, nullptr);
    }
  }
}
}  // namespace

// ---- host side ------------------------------------------------------------------------------------

struct BatchSlot
{
  bool used = false;
  amcl_grid_s* grid = nullptr;
  uint32_t cap = 0;
  uint64_t p_off = 0;
  uint32_t P = 0;
  uint64_t seed = 0, step = 0;
  int cur = 0;
  bool initialized = false;
  int cloud_sum = 0;
  // staged step
  bool staged = false;
  std::vector<float4> cloud;
  std::vector<float4> ranges;
  bool predict = false;
  double odom[8] = {};
  double alpha = 0.5, sigma = 0.1, roll = 0, pitch = 0;
  bool resample = false;
  bool stats_valid = false;
};

// Side streams and events that let a step's weighting launches (one per fused queue)
// run as parallel branches: forked from the batch stream, joined back before blend.
constexpr int N_SIDE = 5;
struct Branches
{
  cudaStream_t side[N_SIDE] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[64] = {};
  int init()
  {
    for (auto& s : side)
      AMCL_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    AMCL_CUDA_TRY(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    for (auto& e : join)
      AMCL_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return AMCL_OK;
  }
  ~Branches()
  {
    for (auto s : side)
      if (s)
        cudaStreamDestroy(s);
    if (fork)
      cudaEventDestroy(fork);
    for (auto e : join)
      if (e)
        cudaEventDestroy(e);
  }
};

// The batch's own stream-ordered memory pool (allocations that grow while the
// batch runs come from it, so growing waits only on the batch's stream; a cudaFree
// would synchronise the whole device, every other batch and server lane included).
struct PoolHolder
{
  cudaMemPool_t pool = nullptr;
  int init()
  {
    int dev = 0;
    AMCL_CUDA_TRY(cudaGetDevice(&dev));
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    AMCL_CUDA_TRY(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = UINT64_MAX;  // keep freed memory in the pool for the next growth
    AMCL_CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    return AMCL_OK;
  }
  ~PoolHolder()
  {
    if (pool)
      cudaMemPoolDestroy(pool);  // released once the buffers' stream-ordered frees have run
  }
};

// A device buffer allocated and freed in stream order from a PoolHolder's pool.
struct StreamBuf
{
  void* p = nullptr;
  size_t bytes = 0;
  cudaMemPool_t pool = nullptr;
  cudaStream_t s = nullptr;
  int ensure(size_t want)
  {
    if (want <= bytes && p)
      return AMCL_OK;
    if (p)
      AMCL_CUDA_TRY(cudaFreeAsync(p, s));
    p = nullptr;
    bytes = 0;
    if (want == 0)
      return AMCL_OK;
    const cudaError_t e = cudaMallocFromPoolAsync(&p, want, pool, s);
    if (e != cudaSuccess)
    {
      p = nullptr;
      return fail(AMCL_ENOMEM, std::string("cudaMallocFromPoolAsync ") + std::to_string(want) + " B: " +
                                   cudaGetErrorString(e));
    }
    bytes = want;
    return AMCL_OK;
  }
  template <typename T>
  T* as() const
  {
    return static_cast<T*>(p);
  }
  ~StreamBuf()
  {
    if (p)
      cudaFreeAsync(p, s);
  }
};

struct amcl_batch_s
{
  StreamHolder st;
  Branches br;
  PoolHolder mem;  // declared before the StreamBufs: destroyed after them
  uint32_t max_filters = 0;
  uint64_t max_particles = 0, max_points = 0;
  std::vector<BatchSlot> slots;
  std::vector<std::pair<uint64_t, uint64_t>> free_ranges;  // particle arena [off, len)
  DevBuf pose[2], w[2], wp[2], wr[2], inmap, hi, blocksum, acc, stats, cloud, ranges, steps, counts, blk_items,
      wt_items, counter;
  StreamBuf xf, scratch, tile_done;  // the split path's, sized by the steps as they come
  PinnedBuf h_cloud, h_ranges, h_steps, h_counts, h_blk, h_wt, h_stats;
  uint32_t n_steps = 0, n_blk = 0, n_wt = 0;
  uint64_t class_mask = 0;  // weighting queues of the packed step: bit q fused queue q, bit 32 + c split class c
  int split_mode = 0;       // 0 auto, 1 never, 2 always (when the scratch fits)
  uint64_t scratch_cap = 4ull << 30;  // bytes of probability slab a split step may use
  uint64_t n_cloud = 0, n_ranges = 0;
  std::vector<uint32_t> step_slots;  // slot of each step in the last launch
  int threads = 256, chunk = 1024;
  uint32_t tab_cap = 0;
  // Grids given to the fused weighting launches by value (GridSet): the grid handle of
  // each entry (null: free) and the views as last packed.
  const amcl_grid_s* gset_grid[BATCH_GRIDS] = {};
  GridSet gset{};
  // One instantiated graph per (particle tile, point tile, class mask, grid set) in use;
  // all are dropped when a buffer the kernels point at is reallocated, the tables grow
  // or the grid set changes.
  struct Graph
  {
    int threads = 0, chunk = 0;
    uint64_t mask = 0;
    GridSet gset{};  // baked into the captured weighting launches
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t n_cloud_cp = nullptr, n_ranges_cp = nullptr, n_steps_cp = nullptr, n_counts_cp = nullptr,
                    n_blk_cp = nullptr, n_wt_cp = nullptr;
  };
  std::vector<Graph> graphs;
  void drop_graphs()
  {
    for (Graph& g : graphs)
    {
      if (g.exec)
        cudaGraphExecDestroy(g.exec);
      if (g.graph)
        cudaGraphDestroy(g.graph);
    }
    graphs.clear();
  }
  bool in_flight = false;
  uint64_t steps_done = 0;
  uint64_t graphs_built = 0, reallocs = 0;  // amcl_batch_counters
  std::mutex mu;
  ~amcl_batch_s() { drop_graphs(); }
};

namespace
{
uint64_t align256(uint64_t v) { return (v + 255) & ~255ull; }

BatchDev batch_dev(amcl_batch_s* b)
{
  BatchDev d;
  for (int k = 0; k < 2; ++k)
  {
    d.pose[k] = b->pose[k].as<float4>();
    d.w[k] = b->w[k].as<float>();
    d.wp[k] = b->wp[k].as<float>();
    d.wr[k] = b->wr[k].as<float>();
  }
  d.inmap = b->inmap.as<uint8_t>();
  d.hi = b->hi.as<int32_t>();
  d.blocksum = b->blocksum.as<X320>();
  d.acc = b->acc.as<unsigned long long>();
  d.stats = b->stats.as<PFStats>();
  d.cloud = b->cloud.as<float4>();
  d.ranges = b->ranges.as<float4>();
  d.steps = b->steps.as<SlotStep>();
  d.counts = b->counts.as<uint32_t>();
  d.blk_items = b->blk_items.as<uint2>();
  d.wt_items = b->wt_items.as<uint2>();
  d.counter = b->counter.as<unsigned int>();
  d.xf = b->xf.as<SplitRec>();
  d.scratch = b->scratch.as<float>();
  d.tile_done = b->tile_done.as<unsigned int>();
  return d;
}

size_t weight_smem(const amcl_batch_s* b, int chunk)
{
  return static_cast<size_t>(chunk) * sizeof(float4) + MAX_RANGES * sizeof(float4) + 64 * sizeof(X320) +
         (static_cast<size_t>(b->tab_cap) + 3) * sizeof(float);  // staged tables: floats (load_tables)
}

size_t split_smem(const amcl_batch_s* b)
{
  return static_cast<size_t>(split_red_offset(b->tab_cap)) * 4 +
         static_cast<size_t>(SP_RED_STAGES) * SP_RED_PTS * 32 * sizeof(float);
}

// Persistent launches of one (storage, sum) class: one per fused queue in `mask`, sized
// to the blocks that fit on every SM at once.
// Hands out the stream of each fused-queue launch of a step: the batch stream when
// there is one launch, else a side stream forked from it (joined by join()), so the
// queues' persistent kernels (one per grid slot) run side by side and their tails overlap.
struct Fork
{
  amcl_batch_s* b;
  cudaStream_t main;
  int launches;
  int used = 0;
  int next(cudaStream_t* out)
  {
    if (launches <= 1)
    {
      *out = main;
      return AMCL_OK;
    }
    if (used == 0)
      AMCL_CUDA_TRY(cudaEventRecord(b->br.fork, main));
    if (used >= 64)
      return fail(AMCL_ERANGE, "batch: more than 64 weighting launches in one step");
    *out = b->br.side[used % N_SIDE];
    AMCL_CUDA_TRY(cudaStreamWaitEvent(*out, b->br.fork, 0));
    return AMCL_OK;
  }
  int done(cudaStream_t s)  // after the launch on s
  {
    if (launches <= 1)
      return AMCL_OK;
    AMCL_CUDA_TRY(cudaEventRecord(b->br.join[used], s));
    ++used;
    return AMCL_OK;
  }
  int join()
  {
    for (int i = 0; i < used; ++i)
      AMCL_CUDA_TRY(cudaStreamWaitEvent(main, b->br.join[i], 0));
    return AMCL_OK;
  }
};

template <int STORAGE, int SUM, int MAXT>
int launch_fused_class(amcl_batch_s* b, const BatchDev& d, int threads, uint32_t chunk, size_t smem, Fork& fk,
                       uint64_t mask)
{
  const int cls = weight_class(STORAGE, SUM);
  for (int slot = 0; slot < N_GSLOTS; ++slot)
  {
    const int q = fused_queue(cls, slot < BATCH_GRIDS ? slot : -1);
    if (!(mask >> q & 1u))
      continue;
    cudaStream_t s = nullptr;
    int rc = fk.next(&s);
    if (rc)
      return rc;
    int per_sm = 0;
    if (slot < BATCH_GRIDS)
    {
      const GridView& gv = b->gset.g[slot];
      const int fv = fast_variant(gv);
      AMCL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm,
          fv == 1   ? k_b_weight<STORAGE, SUM, true, MAXT, 1>
          : fv == 2 ? k_b_weight<STORAGE, SUM, true, MAXT, 2>
                    : k_b_weight<STORAGE, SUM, true, MAXT, 0>,
          threads, smem));
      const unsigned grid = static_cast<unsigned>(device_sm_count() * std::max(per_sm, 1));
      if (fv == 1)
        k_b_weight<STORAGE, SUM, true, MAXT, 1><<<grid, threads, smem, s>>>(d, gv, static_cast<uint32_t>(q), chunk);
      else if (fv == 2)
        k_b_weight<STORAGE, SUM, true, MAXT, 2><<<grid, threads, smem, s>>>(d, gv, static_cast<uint32_t>(q), chunk);
      else
        k_b_weight<STORAGE, SUM, true, MAXT, 0><<<grid, threads, smem, s>>>(d, gv, static_cast<uint32_t>(q), chunk);
    }
    else
    {
      AMCL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_b_weight<STORAGE, SUM, false, MAXT>,
                                                                  threads, smem));
      const unsigned grid = static_cast<unsigned>(device_sm_count() * std::max(per_sm, 1));
      k_b_weight<STORAGE, SUM, false, MAXT><<<grid, threads, smem, s>>>(d, GridView{}, static_cast<uint32_t>(q),
                                                                         chunk);
    }
    AMCL_LAUNCH_CHECK("k_b_weight");
    if ((rc = fk.done(s)))
      return rc;
  }
  return AMCL_OK;
}

template <int MAXT>
int launch_fused_classes(amcl_batch_s* b, const BatchDev& d, int threads, uint32_t chunk, size_t smem, cudaStream_t s,
                         uint64_t mask)
{
  Fork fk{ b, s, __builtin_popcountll(mask & ((1ull << N_FUSED_Q) - 1)) };
  int rc;
  if ((rc = launch_fused_class<AMCL_GRID_F32, 0, MAXT>(b, d, threads, chunk, smem, fk, mask)) ||
      (rc = launch_fused_class<AMCL_GRID_F32, 1, MAXT>(b, d, threads, chunk, smem, fk, mask)) ||
      (rc = launch_fused_class<AMCL_GRID_F16, 0, MAXT>(b, d, threads, chunk, smem, fk, mask)) ||
      (rc = launch_fused_class<AMCL_GRID_F16, 1, MAXT>(b, d, threads, chunk, smem, fk, mask)) ||
      (rc = launch_fused_class<AMCL_GRID_U8, 0, MAXT>(b, d, threads, chunk, smem, fk, mask)) ||
      (rc = launch_fused_class<AMCL_GRID_U8, 1, MAXT>(b, d, threads, chunk, smem, fk, mask)))
    return rc;
  return fk.join();
}

// The weighting of a packed step: the fused queues in `mask` (bits 0 .. N_FUSED_Q-1),
// then the split classes (bits SPLIT_MASK_SHIFT + c).
int launch_weight_classes(amcl_batch_s* b, const BatchDev& d, int threads, int chunk, cudaStream_t s, uint64_t mask)
{
  const unsigned sgrid = static_cast<unsigned>(device_sm_count() * 3);
  const size_t smem = weight_smem(b, chunk), ssmem = split_smem(b);
  const uint32_t c = static_cast<uint32_t>(chunk);
  int rc = threads > 256 ? launch_fused_classes<512>(b, d, threads, c, smem, s, mask)
                         : launch_fused_classes<256>(b, d, threads, c, smem, s, mask);
  if (rc)
    return rc;
  const uint64_t sm = mask >> SPLIT_MASK_SHIFT;
  if (sm & (1u << 0))
    k_b_split<AMCL_GRID_F32, 0><<<sgrid, SP_WARPS * 32, ssmem, s>>>(d, b->tab_cap);
  if (sm & (1u << 1))
    k_b_split<AMCL_GRID_F32, 1><<<sgrid, SP_WARPS * 32, ssmem, s>>>(d, b->tab_cap);
  if (sm & (1u << 2))
    k_b_split<AMCL_GRID_F16, 0><<<sgrid, SP_WARPS * 32, ssmem, s>>>(d, b->tab_cap);
  if (sm & (1u << 3))
    k_b_split<AMCL_GRID_F16, 1><<<sgrid, SP_WARPS * 32, ssmem, s>>>(d, b->tab_cap);
  if (sm & (1u << 4))
    k_b_split<AMCL_GRID_U8, 0><<<sgrid, SP_WARPS * 32, ssmem, s>>>(d, b->tab_cap);
  if (sm & (1u << 5))
    k_b_split<AMCL_GRID_U8, 1><<<sgrid, SP_WARPS * 32, ssmem, s>>>(d, b->tab_cap);
  AMCL_LAUNCH_CHECK("k_b_split");
  return AMCL_OK;
}

template <typename K>
int smem_attr(K kernel, size_t smem)
{
  AMCL_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  return AMCL_OK;
}

template <int STORAGE, int SUM>
int fused_smem_attr(size_t smem)
{
  int rc;
  if ((rc = smem_attr(k_b_weight<STORAGE, SUM, true, 256>, smem)) ||
      (rc = smem_attr(k_b_weight<STORAGE, SUM, false, 256>, smem)) ||
      (rc = smem_attr(k_b_weight<STORAGE, SUM, true, 512>, smem)) ||
      (rc = smem_attr(k_b_weight<STORAGE, SUM, false, 512>, smem)) ||
      (rc = smem_attr(k_b_weight<STORAGE, SUM, true, 256, 1>, smem)) ||
      (rc = smem_attr(k_b_weight<STORAGE, SUM, true, 512, 1>, smem)) ||
      (rc = smem_attr(k_b_weight<STORAGE, SUM, true, 256, 2>, smem)) ||
      (rc = smem_attr(k_b_weight<STORAGE, SUM, true, 512, 2>, smem)))
    return rc;
  return AMCL_OK;
}

int set_weight_smem(size_t smem, size_t ssmem)
{
  int rc;
  if ((rc = fused_smem_attr<AMCL_GRID_F32, 0>(smem)) || (rc = fused_smem_attr<AMCL_GRID_F32, 1>(smem)) ||
      (rc = fused_smem_attr<AMCL_GRID_F16, 0>(smem)) || (rc = fused_smem_attr<AMCL_GRID_F16, 1>(smem)) ||
      (rc = fused_smem_attr<AMCL_GRID_U8, 0>(smem)) || (rc = fused_smem_attr<AMCL_GRID_U8, 1>(smem)) ||
      (rc = smem_attr(k_b_split<AMCL_GRID_F32, 0>, ssmem)) || (rc = smem_attr(k_b_split<AMCL_GRID_F32, 1>, ssmem)) ||
      (rc = smem_attr(k_b_split<AMCL_GRID_F16, 0>, ssmem)) || (rc = smem_attr(k_b_split<AMCL_GRID_F16, 1>, ssmem)) ||
      (rc = smem_attr(k_b_split<AMCL_GRID_U8, 0>, ssmem)) || (rc = smem_attr(k_b_split<AMCL_GRID_U8, 1>, ssmem)))
    return rc;
  return AMCL_OK;
}

// Enqueues the whole step on the batch stream (also what the graph captures).
int enqueue_step(amcl_batch_s* b, int threads, int chunk, bool copies, uint64_t mask)
{
  cudaStream_t s = b->st.s;
  BatchDev d = batch_dev(b);
  const int sms = device_sm_count();
  const unsigned grid = static_cast<unsigned>(sms * GRID_BLOCKS_PER_SM);
  if (copies)
  {
    AMCL_CUDA_TRY(cudaMemcpyAsync(b->counts.p, b->h_counts.p, COUNT_WORDS * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    AMCL_CUDA_TRY(cudaMemcpyAsync(b->steps.p, b->h_steps.p, std::max<uint64_t>(b->n_steps, 1) * sizeof(SlotStep),
                                  cudaMemcpyHostToDevice, s));
    AMCL_CUDA_TRY(cudaMemcpyAsync(b->blk_items.p, b->h_blk.p, std::max<uint64_t>(b->n_blk, 1) * sizeof(uint2),
                                  cudaMemcpyHostToDevice, s));
    AMCL_CUDA_TRY(cudaMemcpyAsync(b->wt_items.p, b->h_wt.p, std::max<uint64_t>(b->n_wt, 1) * sizeof(uint2),
                                  cudaMemcpyHostToDevice, s));
    AMCL_CUDA_TRY(cudaMemcpyAsync(b->cloud.p, b->h_cloud.p, std::max<uint64_t>(b->n_cloud, 1) * sizeof(float4),
                                  cudaMemcpyHostToDevice, s));
    AMCL_CUDA_TRY(cudaMemcpyAsync(b->ranges.p, b->h_ranges.p, std::max<uint64_t>(b->n_ranges, 1) * sizeof(float4),
                                  cudaMemcpyHostToDevice, s));
  }
  k_b_predict<<<grid, NT, 0, s>>>(d);
  AMCL_LAUNCH_CHECK("k_b_predict");
  if (mask >> SPLIT_MASK_SHIFT)
  {
    k_b_xf<<<grid, NT, 0, s>>>(d);
    AMCL_LAUNCH_CHECK("k_b_xf");
  }
  AMCL_CUDA_TRY(cudaMemsetAsync(b->acc.p, 0, static_cast<size_t>(b->max_filters) * ACC_WORDS * 8, s));
  AMCL_CUDA_TRY(cudaMemsetAsync(b->counter.p, 0, N_COUNTERS * sizeof(unsigned int), s));
  int rc = launch_weight_classes(b, d, threads, chunk, s, mask);
  if (rc)
    return rc;
  k_b_blend<<<grid, NT, 0, s>>>(d);
  AMCL_LAUNCH_CHECK("k_b_blend");
  k_b_normalize<<<grid, NT, 0, s>>>(d);
  AMCL_LAUNCH_CHECK("k_b_normalize");
  k_b_finalize<<<static_cast<unsigned>(sms), 256, 0, s>>>(d);
  AMCL_LAUNCH_CHECK("k_b_finalize");
  k_b_prefix<<<grid, NT, 0, s>>>(d);
  AMCL_LAUNCH_CHECK("k_b_prefix");
  k_b_gather<<<grid, NT, 0, s>>>(d);
  AMCL_LAUNCH_CHECK("k_b_gather");
  if (copies)
    AMCL_CUDA_TRY(cudaMemcpyAsync(b->h_stats.p, b->stats.p, static_cast<size_t>(b->max_filters) * sizeof(PFStats),
                                  cudaMemcpyDeviceToHost, s));
  return AMCL_OK;
}

// Grid slots of the packed steps: grids already in the batch's GridSet keep their
// slot; a new grid takes a free slot or one whose grid no step of this pack uses;
// beyond BATCH_GRIDS distinct grids, and for grids whose locate tables are too large to
// stage in shared memory, a step reads its grid from its descriptor.  The
// set's views are refreshed from the grids, and a changed set drops the captured graphs
// (the set is a launch argument baked into them).
void assign_grid_slots(amcl_batch_s* b, SlotStep* hs, const std::vector<const amcl_grid_s*>& step_grid)
{
  bool used[BATCH_GRIDS] = {};
  auto slot_of = [&](const amcl_grid_s* g) {
    for (int j = 0; j < BATCH_GRIDS; ++j)
      if (b->gset_grid[j] == g)
        return j;
    return -1;
  };
  for (const amcl_grid_s* g : step_grid)
    if (g && slot_of(g) >= 0)
      used[slot_of(g)] = true;
  for (const amcl_grid_s* g : step_grid)
  {
    if (!g || slot_of(g) >= 0 || !tables_staged(g->view))  // large tables: descriptor queue
      continue;
    for (int j = 0; j < BATCH_GRIDS; ++j)
      if (!used[j])
      {
        b->gset_grid[j] = g;
        used[j] = true;
        break;
      }
  }
  // Only grids of this pack are read (an entry may name a grid destroyed since).
  GridSet fresh;
  std::memcpy(&fresh, &b->gset, sizeof(GridSet));
  for (const amcl_grid_s* g : step_grid)
    if (g && slot_of(g) >= 0)
      std::memcpy(&fresh.g[slot_of(g)], &g->view, sizeof(GridView));
  if (std::memcmp(&fresh, &b->gset, sizeof(GridSet)) != 0)
  {
    b->drop_graphs();
    std::memcpy(&b->gset, &fresh, sizeof(GridSet));
  }
  // a slot's launch reads the tables from shared memory: grids whose tables are not
  // staged (a grid reloaded at a larger size keeps its entry) use the descriptor queue
  for (size_t i = 0; i < step_grid.size(); ++i)
    hs[i].gslot = step_grid[i] && tables_staged(step_grid[i]->view) ? slot_of(step_grid[i]) : -1;
}

// Grows a device or pinned buffer to at least `need` bytes, at least doubling (up to
// `cap`): a workload that creeps upwards reallocates, and so frees (a device-wide
// synchronisation) and drops the captured graphs, only a few times.
template <typename Buf>
int grow(amcl_batch_s* b, Buf& buf, size_t need, size_t cap = SIZE_MAX, size_t first = 1u << 20)
{
  if (buf.p && need <= buf.bytes)
    return AMCL_OK;
  const size_t dbl = std::max<size_t>(2 * buf.bytes, first);
  b->reallocs += 1;
  return buf.ensure(std::max(need, std::min(dbl, cap)));
}

// Weighting work items of the packed steps.  Fused steps: (step, particle tile of
// `threads`), grouped by fused queue ((storage, sum) class and grid slot), longest
// scans first within a queue (stable, so a filter's tiles stay adjacent and reuse the
// staged tables).  Split steps: (step, 32-particle tile * slices + 512-point slice),
// tile-major so a tile's slices run together and its slab is summed while still in
// L2.  Sets the class mask.
void build_weight_items(amcl_batch_s* b, int threads)
{
  const SlotStep* hs = b->h_steps.as<SlotStep>();
  // Queue of a step: fused queue q (0 .. N_FUSED_Q-1), or N_FUSED_Q + c for split class c.
  auto step_queue = [&](uint32_t s) {
    const int cls = weight_class(hs[s].g.storage, static_cast<int>(hs[s].cloud_sum));
    return hs[s].split ? N_FUSED_Q + cls : fused_queue(cls, hs[s].gslot);
  };
  // Steps ordered by queue, longest scan first (stable): the items follow step by step.
  std::vector<uint32_t> order(b->n_steps);
  for (uint32_t s = 0; s < b->n_steps; ++s)
    order[s] = s;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
    const int cx = step_queue(x), cy = step_queue(y);
    return cx != cy ? cx < cy : std::max<uint32_t>(hs[x].N, 1) > std::max<uint32_t>(hs[y].N, 1);
  });
  uint2* hw = b->h_wt.as<uint2>();
  uint32_t* hcnt = b->h_counts.as<uint32_t>();
  for (int w = FQ_BASE; w < COUNT_WORDS; ++w)
    hcnt[w] = 0;
  uint64_t mask = 0;
  uint32_t k = 0;
  int prev = -1;
  for (uint32_t s : order)
  {
    const int qi = step_queue(s);
    const bool split = qi >= N_FUSED_Q;
    const int w = split ? SQ_BASE + 2 * (qi - N_FUSED_Q) : FQ_BASE + 2 * qi;
    const uint32_t n = split ? ceil_div(hs[s].P, 32) * ceil_div(hs[s].N, SP_PTS) : ceil_div(hs[s].P, threads);
    if (qi != prev)
      hcnt[w] = k;
    prev = qi;
    for (uint32_t j = 0; j < n; ++j)
      hw[k++] = make_uint2(s, j);
    hcnt[w + 1] = k;
    if (n)
      mask |= 1ull << (split ? SPLIT_MASK_SHIFT + (qi - N_FUSED_Q) : qi);
  }
  // Every grid slot of a fused class with work is launched (a slot without items returns
  // at once), so the captured graph depends on the classes present rather than on which
  // maps this step's filters happen to use: fewer graphs to build while serving.
  for (int cls = 0; cls < N_CLASSES; ++cls)
  {
    bool any = false;
    for (int j = 0; j < N_GSLOTS; ++j)
      any |= (mask >> fused_queue(cls, j < BATCH_GRIDS ? j : -1)) & 1u;
    if (any)
      for (int j = 0; j < BATCH_GRIDS; ++j)
        mask |= 1ull << fused_queue(cls, j);
  }
  b->n_wt = k;
  b->class_mask = mask;
  hcnt[2] = b->n_wt;
}

// Weighting item capacity the packed steps need (fused and split).
uint64_t weight_items_needed(const amcl_batch_s* b, int threads)
{
  const SlotStep* hs = b->h_steps.as<SlotStep>();
  uint64_t n = 0;
  for (uint32_t s = 0; s < b->n_steps; ++s)
    n += hs[s].split ? static_cast<uint64_t>(ceil_div(hs[s].P, 32)) * ceil_div(hs[s].N, SP_PTS)
                     : ceil_div(hs[s].P, threads);
  return n;
}

// Split decision for the packed steps: point-parallel weighting (all steps with
// points) when the fused tiles cannot fill the GPU and the slabs fit the scratch
// budget; assigns the tile counters, slab and transform offsets and sizes the buffers
// (their reallocation drops the captured graphs).
constexpr uint32_t SPLIT_BELOW_TILES_PER_SM = 1;

int plan_split(amcl_batch_s* b, int threads)
{
  SlotStep* hs = b->h_steps.as<SlotStep>();
  uint64_t fused_tiles = 0, slab = 0;
  for (uint32_t s = 0; s < b->n_steps; ++s)
  {
    hs[s].split = 0;
    if (!hs[s].N)
      continue;
    fused_tiles += ceil_div(hs[s].P, threads);
    slab += static_cast<uint64_t>(ceil_div(hs[s].P, 32)) * 32ull * hs[s].N;
  }
  bool split = b->split_mode == 2 ||
               (b->split_mode == 0 && fused_tiles < SPLIT_BELOW_TILES_PER_SM * static_cast<uint64_t>(device_sm_count()));
  if (!fused_tiles || slab * 4 > b->scratch_cap)
    split = false;
  if (!split)
    return AMCL_OK;
  uint64_t tiles = 0, sc = 0, xo = 0;
  for (uint32_t s = 0; s < b->n_steps; ++s)
  {
    SlotStep& st = hs[s];
    if (!st.N)
      continue;
    st.split = 1;
    st.tile_base = static_cast<uint32_t>(tiles);
    st.sc_off = sc;
    st.xf_off = xo;
    tiles += ceil_div(st.P, 32);
    sc += static_cast<uint64_t>(ceil_div(st.P, 32)) * 32ull * st.N;
    xo += st.P;
  }
  const void* old[3] = { b->xf.p, b->scratch.p, b->tile_done.p };
  const size_t old_tiles = b->tile_done.bytes;
  int rc;
  // first reservations: the transforms and tile counters of as many particles as a split
  // step can hold (fewer fused tiles than SMs, 512-particle tiles at most), 256 MB of slab
  const size_t split_p = static_cast<size_t>(device_sm_count()) * SPLIT_BELOW_TILES_PER_SM * 512;
  if ((rc = grow(b, b->xf, xo * sizeof(SplitRec), SIZE_MAX, split_p * sizeof(SplitRec))) ||
      (rc = grow(b, b->scratch, sc * 4, b->scratch_cap, std::min<size_t>(b->scratch_cap, 256u << 20))) ||
      (rc = grow(b, b->tile_done, tiles * 4, SIZE_MAX, split_p / 32 * 4)))
    return rc;
  if (b->tile_done.bytes != old_tiles || b->tile_done.p != old[2])
    AMCL_CUDA_TRY(cudaMemsetAsync(b->tile_done.p, 0, b->tile_done.bytes, b->st.s));
  if (b->xf.p != old[0] || b->scratch.p != old[1] || b->tile_done.p != old[2])
    b->drop_graphs();
  return AMCL_OK;
}

// Packs the staged steps of every slot into the pinned staging buffers.
int pack_steps(amcl_batch_s* b)
{
  SlotStep* hs = b->h_steps.as<SlotStep>();
  uint2* hb = b->h_blk.as<uint2>();
  float4* hc = b->h_cloud.as<float4>();
  float4* hr = b->h_ranges.as<float4>();
  uint32_t ns = 0, nb = 0;
  uint64_t nc = 0, nr = 0;
  b->step_slots.clear();
  struct Copy
  {
    void* dst;
    const void* src;
    size_t bytes;
  };
  std::vector<Copy> copies;  // into the pinned staging buffers, run together below
  uint64_t copy_bytes = 0;
  const int threads = b->threads;
  std::vector<const amcl_grid_s*> step_grid;  // grid of each step that gathers
  for (uint32_t si = 0; si < b->slots.size(); ++si)
  {
    BatchSlot& sl = b->slots[si];
    if (!sl.used || !sl.staged)
      continue;
    if (!sl.P)
    {
      sl.staged = false;
      continue;
    }
    SlotStep st{};
    st.slot = si;
    st.P = sl.P;
    st.cur = static_cast<uint32_t>(sl.cur);
    st.p_off = sl.p_off;
    const bool upd = sl.grid && sl.grid->built;
    st.N = upd ? static_cast<uint32_t>(sl.cloud.size()) : 0;
    st.nr = static_cast<uint32_t>(sl.ranges.size());
    if (nc + st.N > b->max_points)
      return fail(AMCL_ERANGE, "batch: staged clouds exceed max_points_per_step");
    st.c_off = nc;
    if (st.N)
      copies.push_back({ hc + nc, sl.cloud.data(), st.N * sizeof(float4) });
    nc += st.N;
    st.r_off = static_cast<uint32_t>(nr);
    if (st.nr)
      copies.push_back({ hr + nr, sl.ranges.data(), st.nr * sizeof(float4) });
    nr += st.nr;
    copy_bytes += (st.N + st.nr) * sizeof(float4);
    st.flags = ST_UPDATE | (sl.predict ? ST_PREDICT : 0u) | (sl.resample ? ST_RESAMPLE : 0u);
    st.cloud_sum = static_cast<uint32_t>(sl.cloud_sum);
    const float rollf = static_cast<float>(sl.roll), pitchf = static_cast<float>(sl.pitch);
    st.sr = sinf(rollf);
    st.cr = cosf(rollf);
    st.sp = sinf(pitchf);
    st.cp = cosf(pitchf);
    st.yaw_only = (st.sr == 0.0f && st.sp == 0.0f && st.cr == 1.0f && st.cp == 1.0f) ? 1 : 0;
    st.k1 = static_cast<float>(1.f / (sl.sigma * std::sqrt(2 * M_PI)));
    st.k2 = static_cast<float>(0.5f / (sl.sigma * sl.sigma));
    st.alpha = sl.alpha;
    st.gslot = -1;
    if (upd)
      st.g = sl.grid->view;
    else
    {
      st.g = GridView{};  // no grid: every particle is outside the map
    }
    step_grid.push_back(upd && st.N ? sl.grid : nullptr);
    if (sl.predict)
    {
      st.pred.n = sl.P;
      st.pred.seed_lo = static_cast<uint32_t>(sl.seed);
      st.pred.seed_hi = static_cast<uint32_t>(sl.seed >> 32);
      st.pred.step = sl.step++;
      st.pred.sx = static_cast<float>(std::fabs(sl.odom[4] * sl.odom[0]));
      st.pred.sy = static_cast<float>(std::fabs(sl.odom[5] * sl.odom[1]));
      st.pred.sz = static_cast<float>(std::fabs(sl.odom[6] * sl.odom[2]));
      st.pred.sa = static_cast<float>(std::fabs(sl.odom[7] * sl.odom[3]));
      st.pred.dx = sl.odom[4];
      st.pred.dy = sl.odom[5];
      st.pred.dz = sl.odom[6];
      st.pred.da = sl.odom[7];
      st.pred.draws = nullptr;
    }
    if (sl.resample)
    {
      Philox4 c;
      c.v[0] = 0;
      c.v[1] = static_cast<uint32_t>(sl.step);
      c.v[2] = static_cast<uint32_t>(sl.step >> 32);
      c.v[3] = RNG_TAG_RESAMPLE;
      const Philox4 r = philox4x32_10(c, static_cast<uint32_t>(sl.seed), static_cast<uint32_t>(sl.seed >> 32));
      sl.step += 1;
      const float u = u01_closed0(r.v[0]);
      st.factor = 1.f / static_cast<float>(sl.P);
      st.r = st.factor * u;
    }
    const uint32_t nblk = ceil_div(sl.P, NT);
    for (uint32_t k = 0; k < nblk; ++k)
      hb[nb++] = make_uint2(ns, k);
    hs[ns++] = st;
    b->step_slots.push_back(si);
    sl.staged = false;
  }
  host_parallel_for(static_cast<uint32_t>(copies.size()), copy_threads(copy_bytes),
                    [&](uint32_t i) { std::memcpy(copies[i].dst, copies[i].src, copies[i].bytes); });
  assign_grid_slots(b, hs, step_grid);
  b->n_steps = ns;
  b->n_blk = nb;
  b->n_cloud = nc;
  b->n_ranges = nr;
  uint32_t* hcnt = b->h_counts.as<uint32_t>();
  hcnt[0] = ns;
  hcnt[1] = nb;
  hcnt[3] = 0;
  int rc;
  if ((rc = plan_split(b, threads)))
    return rc;
  const uint64_t items = weight_items_needed(b, threads);
  if (items * sizeof(uint2) > b->wt_items.bytes)
  {
    b->drop_graphs();
    if ((rc = grow(b, b->wt_items, items * sizeof(uint2))) || (rc = grow(b, b->h_wt, items * sizeof(uint2))))
      return rc;
  }
  build_weight_items(b, threads);
  return AMCL_OK;
}

int graph_update_copies(amcl_batch_s* b, amcl_batch_s::Graph& G)
{
  // The copies in the graph move only what the packed step uses.
  struct Cp
  {
    cudaGraphNode_t node;
    void* dst;
    const void* src;
    size_t bytes;
  };
  const Cp cps[] = {
    { G.n_steps_cp, b->steps.p, b->h_steps.p, std::max<uint64_t>(b->n_steps, 1) * sizeof(SlotStep) },
    { G.n_blk_cp, b->blk_items.p, b->h_blk.p, std::max<uint64_t>(b->n_blk, 1) * sizeof(uint2) },
    { G.n_wt_cp, b->wt_items.p, b->h_wt.p, std::max<uint64_t>(b->n_wt, 1) * sizeof(uint2) },
    { G.n_cloud_cp, b->cloud.p, b->h_cloud.p, std::max<uint64_t>(b->n_cloud, 1) * sizeof(float4) },
    { G.n_ranges_cp, b->ranges.p, b->h_ranges.p, std::max<uint64_t>(b->n_ranges, 1) * sizeof(float4) },
  };
  for (const Cp& c : cps)
    AMCL_CUDA_TRY(cudaGraphExecMemcpyNodeSetParams1D(G.exec, c.node, c.dst, c.src, c.bytes, cudaMemcpyHostToDevice));
  return AMCL_OK;
}

// Captures and instantiates the step for the current shape and class mask.
int build_graph(amcl_batch_s* b, uint64_t mask, amcl_batch_s::Graph& G)
{
  cudaStream_t s = b->st.s;
  AMCL_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step(b, b->threads, b->chunk, true, mask);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &g);
  if (rc)
  {
    if (g)
      cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess)
    return fail(AMCL_ECUDA, std::string("batch graph capture: ") + cudaGetErrorString(e));
  G.graph = g;
  G.threads = b->threads;
  G.chunk = b->chunk;
  G.mask = mask;
  std::memcpy(&G.gset, &b->gset, sizeof(GridSet));
  // Find the memcpy nodes by their destinations.
  size_t nn = 0;
  AMCL_CUDA_TRY(cudaGraphGetNodes(g, nullptr, &nn));
  std::vector<cudaGraphNode_t> nodes(nn);
  AMCL_CUDA_TRY(cudaGraphGetNodes(g, nodes.data(), &nn));
  for (cudaGraphNode_t n : nodes)
  {
    cudaGraphNodeType t;
    AMCL_CUDA_TRY(cudaGraphNodeGetType(n, &t));
    if (t != cudaGraphNodeTypeMemcpy)
      continue;
    cudaMemcpy3DParms p;
    AMCL_CUDA_TRY(cudaGraphMemcpyNodeGetParams(n, &p));
    const void* dst = p.dstPtr.ptr;
    if (dst == b->steps.p)
      G.n_steps_cp = n;
    else if (dst == b->blk_items.p)
      G.n_blk_cp = n;
    else if (dst == b->wt_items.p)
      G.n_wt_cp = n;
    else if (dst == b->cloud.p)
      G.n_cloud_cp = n;
    else if (dst == b->ranges.p)
      G.n_ranges_cp = n;
  }
  if (!G.n_steps_cp || !G.n_blk_cp || !G.n_wt_cp || !G.n_cloud_cp || !G.n_ranges_cp)
    return fail(AMCL_ECUDA, "batch graph: copy nodes not found");
  AMCL_CUDA_TRY(cudaGraphInstantiate(&G.exec, g, 0));
  return AMCL_OK;
}

int batch_wait(amcl_batch_s* b)
{
  if (!b->in_flight)
    return AMCL_OK;
  AMCL_CUDA_TRY(cudaStreamSynchronize(b->st.s));
  b->in_flight = false;
  for (uint32_t si : b->step_slots)
  {
    b->slots[si].stats_valid = true;
  }
  return AMCL_OK;
}

int slot_check(amcl_batch_s* b, int slot)
{
  if (slot < 0 || static_cast<uint32_t>(slot) >= b->slots.size() || !b->slots[slot].used)
    return fail(AMCL_EINVAL, "batch: no such filter slot");
  return AMCL_OK;
}

// Single-slot helper kernels (init, set/get) reuse the filter bodies directly.
__global__ __launch_bounds__(NT) void k_slot_init(float4* pose, float* w, float* wp, float* wr, uint32_t n, float x,
                                                 float y, float z, float a, float xd, float yd, float zd, float ad,
                                                 float gc1, float gc2, uint32_t seed_lo, uint32_t seed_hi,
                                                 uint64_t step, unsigned long long* acc)
{
  __shared__ X320 s_part[NT / 32];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float wv = 0.0f;
  if (i < n)
  {
    float4 p = make_float4(x, y, z, a);
    wv = gc1;
    if (i > 0)
    {
      Philox4 c;
      c.v[0] = i;
      c.v[1] = static_cast<uint32_t>(step);
      c.v[2] = static_cast<uint32_t>(step >> 32);
      c.v[3] = RNG_TAG_INIT;
      float zz[4];
      normals4(philox4x32_10(c, seed_lo, seed_hi), zz);
      p.x = fadd(x, fadd(fmul(zz[0], xd), 0.0f));
      p.y = fadd(y, fadd(fmul(zz[1], yd), 0.0f));
      p.z = fadd(z, fadd(fmul(zz[2], zd), 0.0f));
      p.w = fadd(a, fadd(fmul(zz[3], ad), 0.0f));
      const float dx = fsub(p.x, x), dy = fsub(p.y, y), dz = fsub(p.z, z);
      const float dist = __fsqrt_rn(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)));
      wv = fmul(gc1, __double2float_rn(exp(static_cast<double>(fmul(fmul(-dist, dist), gc2)))));
    }
    pose[i] = p;
    w[i] = wv;
    wp[i] = 0.0f;
    wr[i] = 0.0f;
  }
  block_exact_add(x320_from_float(wv), acc + ACC_W * NDIG, s_part);
}

__global__ __launch_bounds__(NT) void k_slot_normalize(uint32_t n, const float4* pose, float* w,
                                                      unsigned long long* acc, X320* blocksum)
{
  __shared__ double s_sum[2];
  __shared__ X320 s_part[NORM_Q * (NT / 32)];
  normalize_block(blockIdx.x, n, pose, w, acc, blocksum, s_sum, s_part);
}

__global__ void k_slot_finalize(const unsigned long long* acc, PFStats* st)
{
  finalize_stats_warp(acc, st);  // one warp
}
}  // namespace

extern "C" int amcl_batch_create(amcl_batch_t* out, uint32_t max_filters, uint64_t max_particles,
                                 uint64_t max_points_per_step, void* stream)
{
  if (!out || !max_filters || !max_particles || max_filters > (1u << 20) || max_particles > (1ull << 31))
    return fail(AMCL_EINVAL, "amcl_batch_create: bad arguments");
  amcl_batch_s* b = new amcl_batch_s();
  int rc = b->st.init(stream);
  if (!rc)
    rc = b->br.init();
  if (!rc)
    rc = b->mem.init();
  for (StreamBuf* sb : { &b->xf, &b->scratch, &b->tile_done })
  {
    sb->pool = b->mem.pool;
    sb->s = b->st.s;
  }
  const uint64_t cap = align256(max_particles) + 256ull * max_filters;  // per-slot alignment slack
  const uint64_t pts = std::max<uint64_t>(max_points_per_step, 1);
  const uint64_t rng = 64ull * max_filters;
  const uint64_t items = cap / 64 + max_filters;  // weight tiles of >= 64 particles
  for (int k = 0; k < 2 && !rc; ++k)
    if ((rc = b->pose[k].ensure(cap * 16)) || (rc = b->w[k].ensure(cap * 4)) || (rc = b->wp[k].ensure(cap * 4)) ||
        (rc = b->wr[k].ensure(cap * 4)))
      break;
  if (!rc)
    (rc = b->inmap.ensure(cap)) || (rc = b->hi.ensure(cap * 4)) || (rc = b->blocksum.ensure(cap / NT * sizeof(X320))) ||
        (rc = b->acc.ensure(static_cast<size_t>(max_filters) * ACC_WORDS * 8)) ||
        (rc = b->stats.ensure(static_cast<size_t>(max_filters) * sizeof(PFStats))) ||
        (rc = b->cloud.ensure(pts * 16)) || (rc = b->ranges.ensure(rng * 16)) ||
        (rc = b->steps.ensure(static_cast<size_t>(max_filters) * sizeof(SlotStep))) ||
        (rc = b->counts.ensure(COUNT_WORDS * 4)) || (rc = b->blk_items.ensure((cap / NT + max_filters) * sizeof(uint2))) ||
        (rc = b->wt_items.ensure(items * sizeof(uint2))) || (rc = b->counter.ensure(N_COUNTERS * sizeof(unsigned int))) ||
        (rc = b->h_cloud.ensure(pts * 16)) || (rc = b->h_ranges.ensure(rng * 16)) ||
        (rc = b->h_steps.ensure(static_cast<size_t>(max_filters) * sizeof(SlotStep))) ||
        (rc = b->h_counts.ensure(COUNT_WORDS * 4)) || (rc = b->h_blk.ensure((cap / NT + max_filters) * sizeof(uint2))) ||
        (rc = b->h_wt.ensure(items * sizeof(uint2))) ||
        (rc = b->h_stats.ensure(static_cast<size_t>(max_filters) * sizeof(PFStats)));
  if (!rc && cudaMemsetAsync(b->stats.p, 0, static_cast<size_t>(max_filters) * sizeof(PFStats), b->st.s) != cudaSuccess)
    rc = fail(AMCL_ECUDA, "amcl_batch_create: memset");
  if (rc)
  {
    delete b;
    return rc;
  }
  std::memset(b->h_stats.p, 0, static_cast<size_t>(max_filters) * sizeof(PFStats));
  b->max_filters = max_filters;
  b->max_particles = cap;
  b->max_points = pts;
  b->slots.resize(max_filters);
  b->free_ranges.push_back({ 0, cap });
  *out = b;
  return AMCL_OK;
}

extern "C" int amcl_batch_destroy(amcl_batch_t b)
{
  if (!b)
    return AMCL_OK;
  cudaStreamSynchronize(b->st.s);
  delete b;
  return AMCL_OK;
}

extern "C" int amcl_batch_add(amcl_batch_t b, amcl_grid_t grid, uint32_t capacity, uint64_t seed, int* slot)
{
  if (!b || !slot || !capacity)
    return fail(AMCL_EINVAL, "amcl_batch_add: bad arguments");
  std::lock_guard<std::mutex> lock(b->mu);
  int free_slot = -1;
  for (uint32_t i = 0; i < b->slots.size(); ++i)
    if (!b->slots[i].used)
    {
      free_slot = static_cast<int>(i);
      break;
    }
  if (free_slot < 0)
    return fail(AMCL_ENOMEM, "amcl_batch_add: all filter slots are in use");
  const uint64_t need = align256(capacity);
  for (size_t k = 0; k < b->free_ranges.size(); ++k)
  {
    auto& fr = b->free_ranges[k];
    if (fr.second >= need)
    {
      BatchSlot& sl = b->slots[free_slot];
      sl = BatchSlot();
      sl.used = true;
      sl.grid = grid;
      sl.cap = static_cast<uint32_t>(need);
      sl.p_off = fr.first;
      sl.seed = seed;
      fr.first += need;
      fr.second -= need;
      if (!fr.second)
        b->free_ranges.erase(b->free_ranges.begin() + static_cast<long>(k));
      *slot = free_slot;
      return AMCL_OK;
    }
  }
  return fail(AMCL_ENOMEM, "amcl_batch_add: no particle arena range left (HBM budget)");
}

extern "C" int amcl_batch_remove(amcl_batch_t b, int slot)
{
  if (!b)
    return fail(AMCL_EINVAL, "amcl_batch_remove: null batch");
  std::lock_guard<std::mutex> lock(b->mu);
  int rc = slot_check(b, slot);
  if (rc)
    return rc;
  if ((rc = batch_wait(b)))
    return rc;
  BatchSlot& sl = b->slots[slot];
  b->free_ranges.push_back({ sl.p_off, sl.cap });
  std::sort(b->free_ranges.begin(), b->free_ranges.end());
  // coalesce neighbours
  std::vector<std::pair<uint64_t, uint64_t>> merged;
  for (auto& fr : b->free_ranges)
  {
    if (!merged.empty() && merged.back().first + merged.back().second == fr.first)
      merged.back().second += fr.second;
    else
      merged.push_back(fr);
  }
  b->free_ranges.swap(merged);
  sl = BatchSlot();
  return AMCL_OK;
}

extern "C" int amcl_batch_set_grid(amcl_batch_t b, int slot, amcl_grid_t grid)
{
  if (!b)
    return fail(AMCL_EINVAL, "amcl_batch_set_grid: null batch");
  std::lock_guard<std::mutex> lock(b->mu);
  int rc = slot_check(b, slot);
  if (rc)
    return rc;
  b->slots[slot].grid = grid;
  return AMCL_OK;
}

extern "C" int amcl_batch_init(amcl_batch_t b, int slot, int num_particles, float x, float y, float z, float a,
                               float x_dev, float y_dev, float z_dev, float a_dev)
{
  if (!b)
    return fail(AMCL_EINVAL, "amcl_batch_init: null batch");
  std::lock_guard<std::mutex> lock(b->mu);
  int rc = slot_check(b, slot);
  if (rc || (rc = batch_wait(b)))
    return rc;
  BatchSlot& sl = b->slots[slot];
  const long long np = num_particles < 0 ? -static_cast<long long>(num_particles) : num_particles;
  if (np == 0 || static_cast<uint64_t>(np) > sl.cap)
    return fail(AMCL_ERANGE, "amcl_batch_init: particle count is 0 or above the slot's capacity");
  sl.P = static_cast<uint32_t>(np);
  sl.cur = 0;
  const float dev = std::max(std::max(x_dev, y_dev), z_dev);
  const float gc1 = static_cast<float>(1. / (dev * std::sqrt(2 * M_PI)));
  const float two_dev_dev = (2 * dev) * dev;
  const float gc2 = static_cast<float>(1. / two_dev_dev);
  cudaStream_t s = b->st.s;
  unsigned long long* acc = b->acc.as<unsigned long long>() + static_cast<uint64_t>(slot) * ACC_WORDS;
  AMCL_CUDA_TRY(cudaMemsetAsync(acc, 0, ACC_WORDS * 8, s));
  const uint64_t off = sl.p_off;
  k_slot_init<<<ceil_div(sl.P, NT), NT, 0, s>>>(b->pose[0].as<float4>() + off, b->w[0].as<float>() + off,
                                                b->wp[0].as<float>() + off, b->wr[0].as<float>() + off, sl.P, x, y, z,
                                                a, x_dev, y_dev, z_dev, a_dev, gc1, gc2, static_cast<uint32_t>(sl.seed),
                                                static_cast<uint32_t>(sl.seed >> 32), sl.step++, acc);
  AMCL_LAUNCH_CHECK("k_slot_init");
  k_slot_normalize<<<ceil_div(sl.P, NT), NT, 0, s>>>(sl.P, b->pose[0].as<float4>() + off, b->w[0].as<float>() + off,
                                                     acc, b->blocksum.as<X320>() + off / NT);
  AMCL_LAUNCH_CHECK("k_slot_normalize");
  k_slot_finalize<<<1, 32, 0, s>>>(acc, b->stats.as<PFStats>() + slot);
  AMCL_LAUNCH_CHECK("k_slot_finalize");
  AMCL_CUDA_TRY(cudaMemcpyAsync(b->h_stats.as<PFStats>() + slot, b->stats.as<PFStats>() + slot, sizeof(PFStats),
                                cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  sl.initialized = true;
  sl.stats_valid = true;
  return AMCL_OK;
}

extern "C" int amcl_batch_set_particles(amcl_batch_t b, int slot, const float* p7, uint32_t n)
{
  if (!b || !p7 || !n)
    return fail(AMCL_EINVAL, "amcl_batch_set_particles: bad arguments");
  std::lock_guard<std::mutex> lock(b->mu);
  int rc = slot_check(b, slot);
  if (rc || (rc = batch_wait(b)))
    return rc;
  BatchSlot& sl = b->slots[slot];
  if (n > sl.cap)
    return fail(AMCL_ERANGE, "amcl_batch_set_particles: above the slot's capacity");
  std::vector<float4> pose(n);
  std::vector<float> w(n), wp(n), wr(n);
  for (uint32_t i = 0; i < n; ++i)
  {
    const float* q = p7 + 7ull * i;
    pose[i] = make_float4(q[0], q[1], q[2], q[3]);
    w[i] = q[4];
    wp[i] = q[5];
    wr[i] = q[6];
  }
  cudaStream_t s = b->st.s;
  const uint64_t off = sl.p_off;
  AMCL_CUDA_TRY(cudaMemcpyAsync(b->pose[0].as<float4>() + off, pose.data(), n * 16ull, cudaMemcpyHostToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(b->w[0].as<float>() + off, w.data(), n * 4ull, cudaMemcpyHostToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(b->wp[0].as<float>() + off, wp.data(), n * 4ull, cudaMemcpyHostToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(b->wr[0].as<float>() + off, wr.data(), n * 4ull, cudaMemcpyHostToDevice, s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  sl.P = n;
  sl.cur = 0;
  sl.initialized = true;
  return AMCL_OK;
}

extern "C" int amcl_batch_get_particles(amcl_batch_t b, int slot, float* p7, uint32_t cap)
{
  if (!b || (!p7 && cap))
    return fail(AMCL_EINVAL, "amcl_batch_get_particles: bad arguments");
  std::lock_guard<std::mutex> lock(b->mu);
  int rc = slot_check(b, slot);
  if (rc || (rc = batch_wait(b)))
    return rc;
  BatchSlot& sl = b->slots[slot];
  const uint32_t m = std::min(cap, sl.P);
  if (!m)
    return AMCL_OK;
  std::vector<float4> pose(m);
  std::vector<float> w(m), wp(m), wr(m);
  cudaStream_t s = b->st.s;
  const uint64_t off = sl.p_off;
  const int c = sl.cur;
  AMCL_CUDA_TRY(cudaMemcpyAsync(pose.data(), b->pose[c].as<float4>() + off, m * 16ull, cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(w.data(), b->w[c].as<float>() + off, m * 4ull, cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(wp.data(), b->wp[c].as<float>() + off, m * 4ull, cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(wr.data(), b->wr[c].as<float>() + off, m * 4ull, cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  for (uint32_t i = 0; i < m; ++i)
  {
    float* q = p7 + 7ull * i;
    q[0] = pose[i].x;
    q[1] = pose[i].y;
    q[2] = pose[i].z;
    q[3] = pose[i].w;
    q[4] = w[i];
    q[5] = wp[i];
    q[6] = wr[i];
  }
  return AMCL_OK;
}

namespace
{
// One filter's staged step (the batch lock held by the caller).
int stage_locked(amcl_batch_s* b, int slot, const float* xyz, uint32_t n, uint32_t stride_floats,
                 const float* ranges4, uint32_t nr, const double* odom8, double alpha, double sigma, double roll,
                 double pitch, int resample)
{
  if ((n && !xyz) || (nr && !ranges4) || stride_floats < 3)
    return fail(AMCL_EINVAL, "amcl_batch_stage: bad arguments");
  if (nr > MAX_RANGES)
    return fail(AMCL_ERANGE, "amcl_batch_stage: more than 64 range measurements");
  int rc = slot_check(b, slot);
  if (rc)
    return rc;
  BatchSlot& sl = b->slots[slot];
  if (!sl.initialized)
    return fail(AMCL_ESTATE, "amcl_batch_stage: filter not initialised");
  sl.cloud.resize(n);
  pack_cloud(xyz, n, stride_floats, sl.cloud.data());
  sl.ranges.resize(nr);
  if (nr)
    std::memcpy(sl.ranges.data(), ranges4, nr * 16ull);
  sl.predict = odom8 != nullptr;
  if (odom8)
    std::memcpy(sl.odom, odom8, sizeof(sl.odom));
  sl.alpha = alpha;
  sl.sigma = sigma;
  sl.roll = roll;
  sl.pitch = pitch;
  sl.resample = resample != 0;
  sl.staged = true;
  return AMCL_OK;
}
}  // namespace

extern "C" int amcl_batch_stage(amcl_batch_t b, int slot, const float* xyz, uint32_t n, uint32_t stride_floats,
                                const float* ranges4, uint32_t nr, const double* odom8, double alpha, double sigma,
                                double roll, double pitch, int resample)
{
  if (!b)
    return fail(AMCL_EINVAL, "amcl_batch_stage: null batch");
  std::lock_guard<std::mutex> lock(b->mu);
  return stage_locked(b, slot, xyz, n, stride_floats, ranges4, nr, odom8, alpha, sigma, roll, pitch, resample);
}

extern "C" int amcl_batch_stage_many(amcl_batch_t b, uint32_t count, const int* slots, const float* const* clouds,
                                     const uint32_t* n, uint32_t stride_floats, const float* const* ranges4,
                                     const uint32_t* nr, const double* odom8, double alpha, double sigma, double roll,
                                     double pitch, int resample)
{
  if (!b || (count && (!slots || !clouds || !n)))
    return fail(AMCL_EINVAL, "amcl_batch_stage_many: bad arguments");
  std::lock_guard<std::mutex> lock(b->mu);
  for (uint32_t k = 0; k < count; ++k)
  {
    const uint32_t nrk = nr ? nr[k] : 0;
    const int rc = stage_locked(b, slots[k], clouds[k], n[k], stride_floats, nrk && ranges4 ? ranges4[k] : nullptr,
                                nrk, odom8 ? odom8 + 8ull * k : nullptr, alpha, sigma, roll, pitch, resample);
    if (rc)
      return rc;
  }
  return AMCL_OK;
}

extern "C" int amcl_batch_stage_packed(amcl_batch_t b, uint32_t count, const int* slots, const float* xyz,
                                       const uint32_t* n, uint32_t stride_floats, const float* ranges4,
                                       const uint32_t* nr, const double* odom8, double alpha, double sigma,
                                       double roll, double pitch, int resample)
{
  if (!b || (count && (!slots || !n)) || stride_floats < 3)
    return fail(AMCL_EINVAL, "amcl_batch_stage_packed: bad arguments");
  std::lock_guard<std::mutex> lock(b->mu);
  // offsets into the packed arrays, and every check before anything is copied
  std::vector<uint64_t> c_off(count), r_off(count);
  uint64_t pts = 0, rgs = 0;
  std::vector<uint8_t> seen(b->slots.size(), 0);
  for (uint32_t k = 0; k < count; ++k)
  {
    c_off[k] = pts;
    r_off[k] = rgs;
    pts += n[k];
    rgs += nr ? nr[k] : 0;
    int rc = slot_check(b, slots[k]);
    if (rc)
      return rc;
    if (!b->slots[slots[k]].initialized)
      return fail(AMCL_ESTATE, "amcl_batch_stage_packed: filter not initialised");
    if (seen[slots[k]]++)
      return fail(AMCL_EINVAL, "amcl_batch_stage_packed: a slot appears twice");
    if (nr && nr[k] > MAX_RANGES)
      return fail(AMCL_ERANGE, "amcl_batch_stage_packed: more than 64 range measurements");
  }
  if ((pts && !xyz) || (rgs && !ranges4))
    return fail(AMCL_EINVAL, "amcl_batch_stage_packed: null cloud or ranges");
  for (uint32_t k = 0; k < count; ++k)  // sizes first (allocation stays on this thread)
  {
    BatchSlot& sl = b->slots[slots[k]];
    sl.cloud.resize(n[k]);
    sl.ranges.resize(nr ? nr[k] : 0);
  }
  host_parallel_for(count, copy_threads((pts + rgs) * 16), [&](uint32_t k) {
    BatchSlot& sl = b->slots[slots[k]];
    pack_cloud(xyz + c_off[k] * stride_floats, n[k], stride_floats, sl.cloud.data());
    if (!sl.ranges.empty())
      std::memcpy(sl.ranges.data(), ranges4 + 4 * r_off[k], sl.ranges.size() * 16);
  });
  for (uint32_t k = 0; k < count; ++k)
  {
    BatchSlot& sl = b->slots[slots[k]];
    sl.predict = odom8 != nullptr;
    if (odom8)
      std::memcpy(sl.odom, odom8 + 8ull * k, sizeof(sl.odom));
    sl.alpha = alpha;
    sl.sigma = sigma;
    sl.roll = roll;
    sl.pitch = pitch;
    sl.resample = resample != 0;
    sl.staged = true;
  }
  return AMCL_OK;
}

extern "C" int amcl_batch_counters(amcl_batch_t b, uint64_t* steps, uint64_t* graphs_built, uint64_t* reallocs)
{
  if (!b)
    return fail(AMCL_EINVAL, "amcl_batch_counters: null batch");
  std::lock_guard<std::mutex> lock(b->mu);
  if (steps)
    *steps = b->steps_done;
  if (graphs_built)
    *graphs_built = b->graphs_built;
  if (reallocs)
    *reallocs = b->reallocs;
  return AMCL_OK;
}

extern "C" int amcl_batch_step(amcl_batch_t b)
{
  if (!b)
    return fail(AMCL_EINVAL, "amcl_batch_step: null batch");
  std::lock_guard<std::mutex> lock(b->mu);
  int rc;
  if ((rc = batch_wait(b)))
    return rc;
  // table capacity in shared memory: the largest grid among the staged filters whose
  // table is staged at all (tables_staged)
  uint32_t tab = 0;
  for (auto& sl : b->slots)
    if (sl.used && sl.staged && sl.grid && sl.grid->built && tables_staged(sl.grid->view))
      tab = std::max<uint32_t>(tab, table_entries(sl.grid->view));
  if ((rc = pack_steps(b)))
    return rc;
  if (!b->n_steps)
    return AMCL_OK;
  if (tab > b->tab_cap)
  {
    b->tab_cap = tab;
    b->drop_graphs();
  }
  const uint64_t mask = b->class_mask;
  amcl_batch_s::Graph* G = nullptr;
  for (auto& g : b->graphs)
    if (g.threads == b->threads && g.chunk == b->chunk && g.mask == mask &&
        std::memcmp(&g.gset, &b->gset, sizeof(GridSet)) == 0)
      G = &g;
  if (!G)
  {
    const size_t smem = weight_smem(b, b->chunk), ssmem = split_smem(b);
    if (smem > 227 * 1024 || ssmem > 227 * 1024)
      return fail(AMCL_ERANGE, "amcl_batch_step: grid tables and point tile exceed shared memory");
    if ((rc = set_weight_smem(smem, ssmem)))
      return rc;
    amcl_batch_s::Graph fresh;
    if ((rc = build_graph(b, mask, fresh)))
    {
      if (fresh.exec)
        cudaGraphExecDestroy(fresh.exec);
      if (fresh.graph)
        cudaGraphDestroy(fresh.graph);
      return rc;
    }
    b->graphs.push_back(fresh);
    b->graphs_built += 1;
    G = &b->graphs.back();
  }
  if ((rc = graph_update_copies(b, *G)))
    return rc;
  AMCL_CUDA_TRY(cudaGraphLaunch(G->exec, b->st.s));
  for (uint32_t si : b->step_slots)
  {
    BatchSlot& sl = b->slots[si];
    if (sl.resample)
      sl.cur = 1 - sl.cur;
    sl.stats_valid = false;
  }
  b->in_flight = true;
  b->steps_done += 1;
  const int kernels = 6 + (mask >> SPLIT_MASK_SHIFT ? 1 : 0) + __builtin_popcountll(mask);  // the graph's kernels
  for (int k = 0; k < kernels; ++k)
    count_launch();
  return AMCL_OK;
}

extern "C" int amcl_batch_wait(amcl_batch_t b)
{
  if (!b)
    return fail(AMCL_EINVAL, "amcl_batch_wait: null batch");
  std::lock_guard<std::mutex> lock(b->mu);
  return batch_wait(b);
}

extern "C" int amcl_batch_get_mean(amcl_batch_t b, int slot, float mean7[7], double mean_var[8])
{
  if (!b || !mean7)
    return fail(AMCL_EINVAL, "amcl_batch_get_mean: bad arguments");
  std::lock_guard<std::mutex> lock(b->mu);
  int rc = slot_check(b, slot);
  if (rc || (rc = batch_wait(b)))
    return rc;
  const PFStats* st = b->h_stats.as<PFStats>() + slot;
  for (int k = 0; k < 7; ++k)
    mean7[k] = k < 4 ? st->mean_f[k] : 0.0f;
  if (mean_var)
    for (int k = 0; k < 4; ++k)
    {
      mean_var[k] = st->mean[k];
      mean_var[4 + k] = st->var[k];
    }
  return AMCL_OK;
}

extern "C" int amcl_batch_set_tuning(amcl_batch_t b, int threads, int chunk)
{
  if (!b || (threads != 64 && threads != 128 && threads != 256 && threads != 512) || chunk < 64 || chunk > 4096 ||
      chunk % UNROLL)
    return fail(AMCL_EINVAL, "amcl_batch_set_tuning: threads in {64,128,256,512}, chunk a multiple of 8 in [64,4096]");
  std::lock_guard<std::mutex> lock(b->mu);
  b->threads = threads;
  b->chunk = chunk;
  return AMCL_OK;
}

extern "C" int amcl_batch_set_split(amcl_batch_t b, int mode, uint64_t scratch_bytes)
{
  if (!b || mode < 0 || mode > 2)
    return fail(AMCL_EINVAL, "amcl_batch_set_split: mode 0 (auto), 1 (never) or 2 (always)");
  std::lock_guard<std::mutex> lock(b->mu);
  b->split_mode = mode;
  if (scratch_bytes)
    b->scratch_cap = scratch_bytes;
  return AMCL_OK;
}

extern "C" int amcl_batch_get_tuning(amcl_batch_t b, int* threads, int* chunk)
{
  if (!b || !threads || !chunk)
    return fail(AMCL_EINVAL, "amcl_batch_get_tuning: bad arguments");
  *threads = b->threads;
  *chunk = b->chunk;
  return AMCL_OK;
}

extern "C" int amcl_batch_stream(amcl_batch_t b, void** stream)
{
  if (!b || !stream)
    return fail(AMCL_EINVAL, "amcl_batch_stream: bad arguments");
  *stream = b->st.s;
  return AMCL_OK;
}

extern "C" int amcl_batch_capacity(amcl_batch_t b, uint64_t* free_particles, uint32_t* free_slots)
{
  if (!b)
    return fail(AMCL_EINVAL, "amcl_batch_capacity: null batch");
  std::lock_guard<std::mutex> lock(b->mu);
  uint64_t fp = 0;
  for (auto& fr : b->free_ranges)
    fp = std::max(fp, fr.second);
  uint32_t fs = 0;
  for (auto& sl : b->slots)
    fs += sl.used ? 0 : 1;
  if (free_particles)
    *free_particles = fp;
  if (free_slots)
    *free_slots = fs;
  return AMCL_OK;
}

// ---- autotuner --------------------------------------------------------------------------------

namespace
{
}  // namespace

extern "C" int amcl_batch_autotune(amcl_batch_t b, int reps, int* best_threads, int* best_chunk, double* best_ms)
{
  if (!b || reps < 1)
    return fail(AMCL_EINVAL, "amcl_batch_autotune: bad arguments");
  std::lock_guard<std::mutex> lock(b->mu);
  int rc = batch_wait(b);
  if (rc)
    return rc;
  if (!b->n_steps)
    return fail(AMCL_ESTATE, "amcl_batch_autotune: run at least one step first");
  cudaStream_t s = b->st.s;
  const uint64_t cap = b->max_particles;
  // Save what the weighting kernel overwrites.
  DevBuf save;
  const size_t fbytes = cap * 4;
  if ((rc = save.ensure(4 * fbytes + cap)))
    return rc;
  char* sp = save.as<char>();
  AMCL_CUDA_TRY(cudaMemcpyAsync(sp, b->wp[0].p, fbytes, cudaMemcpyDeviceToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(sp + fbytes, b->wp[1].p, fbytes, cudaMemcpyDeviceToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(sp + 2 * fbytes, b->wr[0].p, fbytes, cudaMemcpyDeviceToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(sp + 3 * fbytes, b->wr[1].p, fbytes, cudaMemcpyDeviceToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(sp + 4 * fbytes, b->inmap.p, cap, cudaMemcpyDeviceToDevice, s));
  const int cand_t[] = { 128, 256, 512 };
  const int cand_c[] = { 256, 512, 1024, 2048 };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  BatchDev d = batch_dev(b);
  const int sms = device_sm_count();
  double best = 1e300;
  int bt = b->threads, bc = b->chunk;
  for (int t : cand_t)
  {
    build_weight_items(b, t);
    AMCL_CUDA_TRY(cudaMemcpyAsync(b->wt_items.p, b->h_wt.p, std::max<uint64_t>(b->n_wt, 1) * sizeof(uint2),
                                  cudaMemcpyHostToDevice, s));
    AMCL_CUDA_TRY(cudaMemcpyAsync(b->counts.p, b->h_counts.p, COUNT_WORDS * 4, cudaMemcpyHostToDevice, s));
    for (int c : cand_c)
    {
      const size_t smem = weight_smem(b, c);
      if (smem > 227 * 1024)
        continue;
      if ((rc = set_weight_smem(smem, split_smem(b))))
        return rc;
      float total = 0;
      for (int r = -1; r < reps; ++r)
      {
        AMCL_CUDA_TRY(cudaMemsetAsync(b->acc.p, 0, static_cast<size_t>(b->max_filters) * ACC_WORDS * 8, s));
        AMCL_CUDA_TRY(cudaMemsetAsync(b->counter.p, 0, N_COUNTERS * sizeof(unsigned int), s));
        cudaEventRecord(e0, s);
        if ((rc = launch_weight_classes(b, d, t, c, s, b->class_mask)))
          return rc;
        cudaEventRecord(e1, s);
        AMCL_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r >= 0)
          total += ms;
      }
      const double avg = total / reps;
      if (avg < best)
      {
        best = avg;
        bt = t;
        bc = c;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // Restore the filters' state and the item list of the chosen shape.
  AMCL_CUDA_TRY(cudaMemcpyAsync(b->wp[0].p, sp, fbytes, cudaMemcpyDeviceToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(b->wp[1].p, sp + fbytes, fbytes, cudaMemcpyDeviceToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(b->wr[0].p, sp + 2 * fbytes, fbytes, cudaMemcpyDeviceToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(b->wr[1].p, sp + 3 * fbytes, fbytes, cudaMemcpyDeviceToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(b->inmap.p, sp + 4 * fbytes, cap, cudaMemcpyDeviceToDevice, s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  b->threads = bt;
  b->chunk = bc;
  b->drop_graphs();
  if (best_threads)
    *best_threads = bt;
  if (best_chunk)
    *best_chunk = bc;
  if (best_ms)
    *best_ms = best;
  return AMCL_OK;
}
