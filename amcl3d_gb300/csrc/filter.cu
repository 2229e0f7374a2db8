// ParticleFilter on the device: init, predict, update (blend, normalise, mean),
// resample (ParticleFilter.cpp:46-222).
//
// Device layout: particles as structure-of-arrays, pose float4 (x, y, z, yaw) plus
// w, wp, wr float arrays, double-buffered so resample gathers into the spare copy.
// All normalisation sums, the mean and the resampling prefix are exact (integer
// X320 sums, see exact.cuh): they do not depend on summation order, launch shape
// or batching, and each is rounded once (to double) where a value is needed.
#include <cmath>
#include <cstring>
#include <mutex>

#include "bulk.cuh"
#include "exact.cuh"
#include "grid.cuh"
#include "filter_dev.cuh"
#include "philox.cuh"
#include "voxel.cuh"

using namespace amcl;

namespace
{
// ---- single-filter kernels: one block of NT particles each --------------------------------------

__global__ __launch_bounds__(NT) void k_blend(uint32_t n, const uint8_t* __restrict__ inmap, float* __restrict__ wp,
                                             float* __restrict__ wr, float* __restrict__ w, double alpha,
                                             unsigned long long* acc)
{
  __shared__ double s_sum[2];
  __shared__ X320 s_part[NT / 32];
  blend_block(blockIdx.x, n, inmap, wp, wr, w, alpha, acc, s_sum, s_part);
}

__global__ __launch_bounds__(NT) void k_normalize(uint32_t n, const float4* __restrict__ pose, float* __restrict__ w,
                                                 unsigned long long* acc, X320* __restrict__ blocksum)
{
  __shared__ double s_sum[2];
  __shared__ X320 s_part[NORM_Q * (NT / 32)];
  normalize_block(blockIdx.x, n, pose, w, acc, blocksum, s_sum, s_part);
}

__global__ void k_finalize_stats(const unsigned long long* acc, PFStats* st)
{
  finalize_stats_warp(acc, st);  // one warp
}

__global__ __launch_bounds__(NT) void k_predict(float4* __restrict__ pose, PredictArgs a)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n)
    predict_particle(i, pose, a);
}

// ---- init (ParticleFilter.cpp:46-77) ----------------------------------------------------------
struct InitArgs
{
  uint32_t n;
  uint32_t seed_lo, seed_hi;
  uint64_t step;
  float x, y, z, a;
  float xd, yd, zd, ad;
  float gc1, gc2;
  float* draws;
};

__global__ __launch_bounds__(NT) void k_init(float4* __restrict__ pose, float* __restrict__ w, float* __restrict__ wp,
                                            float* __restrict__ wr, InitArgs a, unsigned long long* acc)
{
  __shared__ X320 s_part[NT / 32];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float wv = 0.0f;
  if (i < a.n)
  {
    float4 p = make_float4(a.x, a.y, a.z, a.a);
    wv = a.gc1;
    if (i > 0)
    {
      Philox4 c;
      c.v[0] = i;
      c.v[1] = static_cast<uint32_t>(a.step);
      c.v[2] = static_cast<uint32_t>(a.step >> 32);
      c.v[3] = RNG_TAG_INIT;
      float zz[4];
      normals4(philox4x32_10(c, a.seed_lo, a.seed_hi), zz);
      if (a.draws)
        reinterpret_cast<float4*>(a.draws)[i] = make_float4(zz[0], zz[1], zz[2], zz[3]);
      p.x = fadd(a.x, fadd(fmul(zz[0], a.xd), 0.0f));
      p.y = fadd(a.y, fadd(fmul(zz[1], a.yd), 0.0f));
      p.z = fadd(a.z, fadd(fmul(zz[2], a.zd), 0.0f));
      p.w = fadd(a.a, fadd(fmul(zz[3], a.ad), 0.0f));
      const float dx = fsub(p.x, a.x), dy = fsub(p.y, a.y), dz = fsub(p.z, a.z);
      const float dist = __fsqrt_rn(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)));
      const float e = __double2float_rn(exp(static_cast<double>(fmul(fmul(-dist, dist), a.gc2))));
      wv = fmul(a.gc1, e);
    }
    else if (a.draws)
      reinterpret_cast<float4*>(a.draws)[0] = make_float4(0.f, 0.f, 0.f, 0.f);
    pose[i] = p;
    w[i] = wv;
    wp[i] = 0.0f;  // Particle() zero-initialises wp, wr (ParticleFilter.h:46)
    wr[i] = 0.0f;
  }
  block_exact_add(x320_from_float(wv), acc + ACC_W * NDIG, s_part);
}

__global__ __launch_bounds__(NT) void k_block_sums(uint32_t n, const float* __restrict__ w, X320* __restrict__ blocksum)
{
  __shared__ X320 s_part[NT / 32];
  block_sum_block(blockIdx.x, n, w, blocksum, s_part);
}

__global__ __launch_bounds__(NT) void k_prefix_hi(uint32_t n, const float* __restrict__ w,
                                                 const X320* __restrict__ blocksum, float r, float factor,
                                                 int32_t* __restrict__ hi)
{
  __shared__ X320 s_scan[NT / 32];
  __shared__ X320 s_base;
  prefix_hi_block(blockIdx.x, n, w, blocksum, r, factor, hi, s_scan, &s_base);
}

// The reference's float running sum c += w (ParticleFilter.cpp:203,214), one thread.
__global__ void k_prefix_f32(uint32_t n, const float* __restrict__ w, float* __restrict__ cum)
{
  if (threadIdx.x != 0 || blockIdx.x != 0)
    return;
  float c = 0.0f;
  for (uint32_t i = 0; i < n; ++i)
  {
    c = i == 0 ? w[0] : fadd(c, w[i]);
    cum[i] = c;
  }
}

__global__ __launch_bounds__(NT) void k_hi_from_f32(uint32_t n, const float* __restrict__ cum, float r, float factor,
                                                   int32_t* __restrict__ hi)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const float c = cum[i];
  uint32_t lo = 0, up = n;
  while (lo < up)
  {
    const uint32_t mid = (lo + up) >> 1;
    if (!(u_of(r, factor, mid) > c))  // the reference advances while u > c
      lo = mid + 1;
    else
      up = mid;
  }
  hi[i] = static_cast<int32_t>(lo);
}

__global__ __launch_bounds__(NT) void k_gather(uint32_t n, const int32_t* __restrict__ hi, const float4* __restrict__ pose,
                                              const float* __restrict__ wp, const float* __restrict__ wr,
                                              float4* __restrict__ pose_o, float* __restrict__ w_o,
                                              float* __restrict__ wp_o, float* __restrict__ wr_o, float factor,
                                              int32_t* __restrict__ idx_o)
{
  const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < n)
    gather_particle(m, n, hi, pose, wp, wr, pose_o, w_o, wp_o, wr_o, factor, idx_o);
}
}  // namespace

// ---- host handle ----------------------------------------------------------------------------------

struct amcl_pf_s
{
  StreamHolder st;
  uint32_t n = 0;
  uint32_t cap = 0;
  bool initialized = false;
  uint64_t seed = 0;
  uint64_t step = 0;
  int cur = 0;
  DevBuf pose[2], w[2], wp[2], wr[2];
  DevBuf inmap, acc, stats, blocksum, hi, ridx, cum, scratch, cloud, ranges, draws, err;
  PinnedBuf h_cloud, h_ranges, h_stats;
  DevBuf down;          // voxel-downsampled cloud (amcl_pf_update_voxel)
  PinnedBuf h_down;
  cudaEvent_t staged = nullptr;
  cudaEvent_t down_ev = nullptr;
  bool staged_pending = false;
  bool blocksum_valid = false;
  bool record = false;
  bool have_ridx = false;
  int opt_cloud_sum = 0, opt_prefix = 0, opt_kernel = 0, opt_wait_probe = 0;
  Profiler prof;
  std::mutex mu;
};

namespace
{
int pf_reserve(amcl_pf_s* pf, uint32_t n)
{
  if (n <= pf->cap && pf->pose[0].p)
    return AMCL_OK;
  int rc;
  const size_t nb = ceil_div(n, NT);
  for (int b = 0; b < 2; ++b)
    if ((rc = pf->pose[b].ensure(n * 16ull)) || (rc = pf->w[b].ensure(n * 4ull)) || (rc = pf->wp[b].ensure(n * 4ull)) ||
        (rc = pf->wr[b].ensure(n * 4ull)))
      return rc;
  if ((rc = pf->inmap.ensure(n)) || (rc = pf->blocksum.ensure(nb * sizeof(X320))) || (rc = pf->hi.ensure(n * 4ull)) ||
      (rc = pf->ridx.ensure(n * 4ull)) || (rc = pf->draws.ensure(n * 16ull)))
    return rc;
  pf->cap = n;
  return AMCL_OK;
}

int pf_common_alloc(amcl_pf_s* pf)
{
  int rc;
  if ((rc = pf->acc.ensure(ACC_COUNT * NDIG * 8)) || (rc = pf->stats.ensure(sizeof(PFStats))) ||
      (rc = pf->err.ensure(sizeof(int))) || (rc = pf->h_stats.ensure(sizeof(PFStats))))
    return rc;
  return AMCL_OK;
}

int pf_check_err(amcl_pf_s* pf)
{
  int e = 0;
  AMCL_CUDA_TRY(cudaMemcpyAsync(&e, pf->err.p, sizeof(int), cudaMemcpyDeviceToHost, pf->st.s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(pf->st.s));
  if (e)
  {
    cudaMemsetAsync(pf->err.p, 0, sizeof(int), pf->st.s);
    return fail(AMCL_ETIMEDOUT, "a bounded device-side wait gave up (error code " + std::to_string(e) + ")");
  }
  return AMCL_OK;
}

// Normalise w (exact total), accumulate mean terms, write block sums, finalize stats.
int pf_normalize_and_stats(amcl_pf_s* pf)
{
  const unsigned nb = ceil_div(pf->n, NT);
  unsigned long long* acc = pf->acc.as<unsigned long long>();
  k_normalize<<<nb, NT, 0, pf->st.s>>>(pf->n, pf->pose[pf->cur].as<float4>(), pf->w[pf->cur].as<float>(), acc,
                                        pf->blocksum.as<X320>());
  AMCL_LAUNCH_CHECK("k_normalize");
  k_finalize_stats<<<1, 32, 0, pf->st.s>>>(acc, pf->stats.as<PFStats>());
  AMCL_LAUNCH_CHECK("k_finalize_stats");
  pf->blocksum_valid = true;
  return AMCL_OK;
}

int pf_update_impl(amcl_pf_s* pf, amcl_grid_s* g, const float4* cloud_dev, uint32_t n_pts, const float* ranges4,
                   uint32_t nr, double alpha, double sigma, double roll, double pitch, bool ranges_only)
{
  cudaStream_t s = pf->st.s;
  int rc;
  if (nr > 64)
    return fail(AMCL_ERANGE, "update: more than 64 range measurements");
  // Ranges to the device through pinned staging.
  if (nr)
  {
    if ((rc = pf->h_ranges.ensure(nr * 16)) || (rc = pf->ranges.ensure(nr * 16)))
      return rc;
    std::memcpy(pf->h_ranges.p, ranges4, nr * 16);
    AMCL_CUDA_TRY(cudaMemcpyAsync(pf->ranges.p, pf->h_ranges.p, nr * 16, cudaMemcpyHostToDevice, s));
  }
  AMCL_CUDA_TRY(cudaMemsetAsync(pf->acc.p, 0, ACC_COUNT * NDIG * 8, s));
  WeightArgs a{};
  a.pose = pf->pose[pf->cur].as<float4>();
  a.P = pf->n;
  a.cloud = cloud_dev;
  a.N = n_pts;
  // roll/pitch: float parameters of computeCloudWeight (Node passes doubles, narrowed
  // at the call, ParticleFilter.cpp:145); sin/cos as float overloads.
  const float rollf = static_cast<float>(roll), pitchf = static_cast<float>(pitch);
  a.sr = sinf(rollf);  // computed once per update on the host, with the same libm
  a.cr = cosf(rollf);
  a.sp = sinf(pitchf);
  a.cp = cosf(pitchf);
  a.ranges = pf->ranges.as<float4>();
  a.nr = nr;
  a.k1 = static_cast<float>(1.f / (sigma * std::sqrt(2 * M_PI)));  // ParticleFilter.cpp:231
  a.k2 = static_cast<float>(0.5f / (sigma * sigma));              // ParticleFilter.cpp:232
  a.wp = pf->wp[pf->cur].as<float>();
  a.wr = pf->wr[pf->cur].as<float>();
  a.inmap = pf->inmap.as<uint8_t>();
  unsigned long long* acc = pf->acc.as<unsigned long long>();
  a.acc_wp = acc + ACC_WP * NDIG;
  a.acc_wr = acc + ACC_WR * NDIG;
  a.err = pf->err.as<int>();
  a.cloud_sum = pf->opt_cloud_sum;
  a.kernel = pf->opt_kernel ? pf->opt_kernel : choose_weight_kernel(pf->n, n_pts);
  amcl_grid_s local;  // ranges-only: every particle counts as inside, no cloud
  amcl_grid_s* gg = g;
  if (ranges_only)
  {
    local.view = GridView{};
    local.view.built = 1;
    for (int k = 0; k < 3; ++k)
    {
      local.view.in_lo[k] = -INFINITY;
      local.view.in_hi[k] = INFINITY;
    }
    local.view.storage = AMCL_GRID_F32;
    a.N = 0;
    a.kernel = 1;
    gg = &local;
  }
  else if (!g->built)
  {
    // No grid: isIntoMap is false for every particle (Grid3d.cpp:203-204), so no
    // point is ever weighed; every w becomes 0.
    a.N = 0;
    a.kernel = 1;
  }
  else
    grid_apply_l2_window(g, s);
  if (a.kernel == 2)
  {
    const uint64_t need = two_phase_scratch_floats(pf->n, a.N);
    if ((rc = pf->scratch.ensure(need * 4)))
      return rc;
    a.scratch = pf->scratch.as<float>();
    a.scratch_floats = pf->scratch.bytes / 4;
    a.wait_probe = pf->opt_wait_probe;
    pf->opt_wait_probe = 0;
  }
  {
    ProfScope ps(&pf->prof, s, AMCL_PROF_CLOUD_WEIGHT);
    if ((rc = launch_cloud_weight(gg, a, s)))
      return rc;
  }
  {
    ProfScope ps(&pf->prof, s, AMCL_PROF_NORMALIZE);
    const unsigned nb = ceil_div(pf->n, NT);
    k_blend<<<nb, NT, 0, s>>>(pf->n, pf->inmap.as<uint8_t>(), pf->wp[pf->cur].as<float>(), pf->wr[pf->cur].as<float>(),
                              pf->w[pf->cur].as<float>(), alpha, acc);
    AMCL_LAUNCH_CHECK("k_blend");
    if ((rc = pf_normalize_and_stats(pf)))
      return rc;
  }
  return AMCL_OK;
}

int stage_host_cloud(amcl_pf_s* pf, const float* xyz, uint32_t n, uint32_t stride)
{
  int rc;
  if ((rc = pf->h_cloud.ensure(std::max<size_t>(n, 1) * 16)) || (rc = pf->cloud.ensure(std::max<size_t>(n, 1) * 16)))
    return rc;
  if (pf->staged_pending)
  {
    cudaEventSynchronize(pf->staged);  // previous copy out of the pinned buffer done
    pf->staged_pending = false;
  }
  pack_cloud(xyz, n, stride, pf->h_cloud.as<float4>());
  if (n)
    AMCL_CUDA_TRY(cudaMemcpyAsync(pf->cloud.p, pf->h_cloud.p, n * 16ull, cudaMemcpyHostToDevice, pf->st.s));
  AMCL_CUDA_TRY(cudaEventRecord(pf->staged, pf->st.s));
  pf->staged_pending = true;
  return AMCL_OK;
}

int do_resample(amcl_pf_s* pf, float u01)
{
  cudaStream_t s = pf->st.s;
  const uint32_t n = pf->n;
  ProfScope ps(&pf->prof, s, AMCL_PROF_RESAMPLE);
  // Host float arithmetic (IEEE single; the library is built with -ffp-contract=off).
  const float factor = 1.f / static_cast<float>(n);  // ParticleFilter.cpp:201
  const float r = factor * u01;                       // ParticleFilter.cpp:202
  const unsigned nb = ceil_div(n, NT);
  const int c = pf->cur, o = 1 - pf->cur;
  if (pf->opt_prefix == 1)
  {
    int rc;
    if ((rc = pf->cum.ensure(n * 4ull)))
      return rc;
    k_prefix_f32<<<1, 32, 0, s>>>(n, pf->w[c].as<float>(), pf->cum.as<float>());
    AMCL_LAUNCH_CHECK("k_prefix_f32");
    k_hi_from_f32<<<nb, NT, 0, s>>>(n, pf->cum.as<float>(), r, factor, pf->hi.as<int32_t>());
    AMCL_LAUNCH_CHECK("k_hi_from_f32");
  }
  else
  {
    if (!pf->blocksum_valid)
    {
      k_block_sums<<<nb, NT, 0, s>>>(n, pf->w[c].as<float>(), pf->blocksum.as<X320>());
      AMCL_LAUNCH_CHECK("k_block_sums");
    }
    k_prefix_hi<<<nb, NT, 0, s>>>(n, pf->w[c].as<float>(), pf->blocksum.as<X320>(), r, factor, pf->hi.as<int32_t>());
    AMCL_LAUNCH_CHECK("k_prefix_hi");
  }
  k_gather<<<nb, NT, 0, s>>>(n, pf->hi.as<int32_t>(), pf->pose[c].as<float4>(), pf->wp[c].as<float>(),
                             pf->wr[c].as<float>(), pf->pose[o].as<float4>(), pf->w[o].as<float>(),
                             pf->wp[o].as<float>(), pf->wr[o].as<float>(), factor, pf->ridx.as<int32_t>());
  AMCL_LAUNCH_CHECK("k_gather");
  pf->cur = o;
  pf->blocksum_valid = false;
  pf->have_ridx = true;
  return AMCL_OK;
}

float pf_next_uniform(amcl_pf_s* pf)
{
  Philox4 c;
  c.v[0] = 0;
  c.v[1] = static_cast<uint32_t>(pf->step);
  c.v[2] = static_cast<uint32_t>(pf->step >> 32);
  c.v[3] = RNG_TAG_RESAMPLE;
  const Philox4 r = philox4x32_10(c, static_cast<uint32_t>(pf->seed), static_cast<uint32_t>(pf->seed >> 32));
  pf->step += 1;
  return u01_closed0(r.v[0]);
}
}  // namespace

// ---- C ABI ----------------------------------------------------------------------------------------

#define PF_GUARD(pf)                                  \
  if (!(pf))                                          \
    return fail(AMCL_EINVAL, "null filter handle");   \
  std::lock_guard<std::mutex> lock_((pf)->mu)

extern "C" int amcl_pf_create(amcl_pf_t* out, uint64_t seed, void* stream)
{
  if (!out)
    return fail(AMCL_EINVAL, "amcl_pf_create: null out");
  amcl_pf_s* pf = new amcl_pf_s();
  int rc = pf->st.init(stream);
  if (!rc)
    rc = pf_common_alloc(pf);
  if (!rc && cudaEventCreateWithFlags(&pf->staged, cudaEventDisableTiming) != cudaSuccess)
    rc = fail(AMCL_ECUDA, "amcl_pf_create: cudaEventCreate failed");
  if (!rc && (cudaMemsetAsync(pf->err.p, 0, sizeof(int), pf->st.s) != cudaSuccess ||
              cudaMemsetAsync(pf->stats.p, 0, sizeof(PFStats), pf->st.s) != cudaSuccess))
    rc = fail(AMCL_ECUDA, "amcl_pf_create: cudaMemset failed");
  if (rc)
  {
    delete pf;
    return rc;
  }
  pf->seed = seed;
  *out = pf;
  return AMCL_OK;
}

extern "C" int amcl_pf_destroy(amcl_pf_t pf)
{
  if (!pf)
    return AMCL_OK;
  cudaStreamSynchronize(pf->st.s);
  if (pf->staged)
    cudaEventDestroy(pf->staged);
  if (pf->down_ev)
    cudaEventDestroy(pf->down_ev);
  delete pf;
  return AMCL_OK;
}

extern "C" int amcl_pf_init(amcl_pf_t pf, int num_particles, float x, float y, float z, float a, float x_dev,
                            float y_dev, float z_dev, float a_dev)
{
  PF_GUARD(pf);
  const long long np = num_particles < 0 ? -static_cast<long long>(num_particles) : num_particles;  // abs()
  if (np == 0)
    return fail(AMCL_EINVAL, "amcl_pf_init: zero particles (the reference indexes p_[0])");
  if (np > (1ll << 30))
    return fail(AMCL_ERANGE, "amcl_pf_init: more than 2^30 particles");
  int rc;
  if ((rc = pf_reserve(pf, static_cast<uint32_t>(np))))
    return rc;
  pf->n = static_cast<uint32_t>(np);
  pf->cur = 0;
  cudaStream_t s = pf->st.s;
  const float dev = std::max(std::max(x_dev, y_dev), z_dev);  // ParticleFilter.cpp:54
  InitArgs ia{};
  ia.n = pf->n;
  ia.seed_lo = static_cast<uint32_t>(pf->seed);
  ia.seed_hi = static_cast<uint32_t>(pf->seed >> 32);
  ia.step = pf->step++;
  ia.x = x;
  ia.y = y;
  ia.z = z;
  ia.a = a;
  ia.xd = static_cast<float>(static_cast<double>(x_dev));
  ia.yd = static_cast<float>(static_cast<double>(y_dev));
  ia.zd = static_cast<float>(static_cast<double>(z_dev));
  ia.ad = static_cast<float>(static_cast<double>(a_dev));
  ia.gc1 = static_cast<float>(1. / (dev * std::sqrt(2 * M_PI)));  // ParticleFilter.cpp:55
  const float two_dev_dev = (2 * dev) * dev;
  ia.gc2 = static_cast<float>(1. / two_dev_dev);                   // ParticleFilter.cpp:56
  ia.draws = pf->record ? pf->draws.as<float>() : nullptr;
  AMCL_CUDA_TRY(cudaMemsetAsync(pf->acc.p, 0, ACC_COUNT * NDIG * 8, s));
  k_init<<<ceil_div(pf->n, NT), NT, 0, s>>>(pf->pose[0].as<float4>(), pf->w[0].as<float>(), pf->wp[0].as<float>(),
                                           pf->wr[0].as<float>(), ia, pf->acc.as<unsigned long long>());
  AMCL_LAUNCH_CHECK("k_init");
  if ((rc = pf_normalize_and_stats(pf)))
    return rc;
  pf->initialized = true;
  pf->have_ridx = false;
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  return AMCL_OK;
}

extern "C" int amcl_pf_predict(amcl_pf_t pf, double odom_x_mod, double odom_y_mod, double odom_z_mod,
                               double odom_a_mod, double delta_x, double delta_y, double delta_z, double delta_a)
{
  PF_GUARD(pf);
  if (!pf->n)
    return AMCL_OK;
  PredictArgs pa{};
  pa.n = pf->n;
  pa.seed_lo = static_cast<uint32_t>(pf->seed);
  pa.seed_hi = static_cast<uint32_t>(pf->seed >> 32);
  pa.step = pf->step++;
  pa.sx = static_cast<float>(std::fabs(delta_x * odom_x_mod));  // ParticleFilter.cpp:101-104
  pa.sy = static_cast<float>(std::fabs(delta_y * odom_y_mod));
  pa.sz = static_cast<float>(std::fabs(delta_z * odom_z_mod));
  pa.sa = static_cast<float>(std::fabs(delta_a * odom_a_mod));
  pa.dx = delta_x;
  pa.dy = delta_y;
  pa.dz = delta_z;
  pa.da = delta_a;
  pa.draws = pf->record ? pf->draws.as<float>() : nullptr;
  ProfScope ps(&pf->prof, pf->st.s, AMCL_PROF_PREDICT);
  k_predict<<<ceil_div(pf->n, NT), NT, 0, pf->st.s>>>(pf->pose[pf->cur].as<float4>(), pa);
  AMCL_LAUNCH_CHECK("k_predict");
  return AMCL_OK;
}

extern "C" int amcl_pf_update(amcl_pf_t pf, amcl_grid_t g, const float* xyz, uint32_t n, uint32_t stride_floats,
                              const float* ranges4, uint32_t nr, double alpha, double sigma, double roll, double pitch)
{
  PF_GUARD(pf);
  if (!g || (n && !xyz) || (nr && !ranges4) || stride_floats < 3)
    return fail(AMCL_EINVAL, "amcl_pf_update: bad arguments");
  if (!pf->n)
    return AMCL_OK;
  int rc;
  if ((rc = stage_host_cloud(pf, xyz, n, stride_floats)))
    return rc;
  return pf_update_impl(pf, g, pf->cloud.as<float4>(), n, ranges4, nr, alpha, sigma, roll, pitch, false);
}

extern "C" int amcl_pf_update_dev(amcl_pf_t pf, amcl_grid_t g, const void* cloud_f4_dev, uint32_t n,
                                  const float* ranges4, uint32_t nr, double alpha, double sigma, double roll,
                                  double pitch)
{
  PF_GUARD(pf);
  if (!g || (n && !cloud_f4_dev) || (nr && !ranges4) || (reinterpret_cast<uintptr_t>(cloud_f4_dev) & 15))
    return fail(AMCL_EINVAL, "amcl_pf_update_dev: bad arguments (cloud must be 16-byte aligned float4)");
  if (!pf->n)
    return AMCL_OK;
  return pf_update_impl(pf, g, static_cast<const float4*>(cloud_f4_dev), n, ranges4, nr, alpha, sigma, roll, pitch,
                        false);
}

extern "C" int amcl_pf_update_voxel(amcl_pf_t pf, amcl_grid_t g, amcl_voxel_t v, const float* xyz, uint32_t n,
                                    uint32_t stride_floats, float leaf_x, float leaf_y, float leaf_z,
                                    const float* ranges4, uint32_t nr, double alpha, double sigma, double roll,
                                    double pitch, float* down4, uint64_t down_cap, uint64_t* n_down)
{
  PF_GUARD(pf);
  if (!g || !v || (n && !xyz) || (nr && !ranges4) || stride_floats < 3 || !n_down || (down_cap && !down4))
    return fail(AMCL_EINVAL, "amcl_pf_update_voxel: bad arguments");
  const float leaf[3] = { leaf_x, leaf_y, leaf_z };
  int rc;
  if ((rc = voxel_check_leaf(leaf, "amcl_pf_update_voxel")))
    return rc;
  std::lock_guard<std::mutex> lock_v(v->mu);
  cudaStream_t s = pf->st.s;
  if ((rc = stage_host_cloud(pf, xyz, n, stride_floats)) || (rc = pf->down.ensure(std::max<size_t>(n, 1) * 16)))
    return rc;
  // Node.cpp:130-137: the voxel filter, on this filter's stream, device to device
  if ((rc = voxel_enqueue(v, pf->cloud.as<float4>(), n, leaf, pf->down.as<float4>(), s)))
    return rc;
  uint32_t m = 0;
  if (n && (rc = voxel_read_count(v, s, &m)))
    return rc;
  *n_down = m;
  const bool copy_out = down4 && m;
  if (down4 && m > down_cap)
    return fail(AMCL_ERANGE, "amcl_pf_update_voxel: down4 holds fewer points than the filter produced");
  if (copy_out)
  {
    if (!pf->down_ev && cudaEventCreateWithFlags(&pf->down_ev, cudaEventDisableTiming) != cudaSuccess)
      return fail(AMCL_ECUDA, "amcl_pf_update_voxel: cudaEventCreate failed");
    if ((rc = pf->h_down.ensure(m * 16ull)))
      return rc;
    AMCL_CUDA_TRY(cudaMemcpyAsync(pf->h_down.p, pf->down.p, m * 16ull, cudaMemcpyDeviceToHost, s));
    AMCL_CUDA_TRY(cudaEventRecord(pf->down_ev, s));
  }
  // Node.cpp:162: the update weighs the downsampled cloud straight from device memory
  if (pf->n && (rc = pf_update_impl(pf, g, pf->down.as<float4>(), m, ranges4, nr, alpha, sigma, roll, pitch, false)))
    return rc;
  if (copy_out)
  {
    AMCL_CUDA_TRY(cudaEventSynchronize(pf->down_ev));
    std::memcpy(down4, pf->h_down.p, m * 16ull);
  }
  return AMCL_OK;
}

extern "C" int amcl_pf_update_ranges(amcl_pf_t pf, const float* ranges4, uint32_t nr, double alpha, double sigma)
{
  PF_GUARD(pf);
  if (nr && !ranges4)
    return fail(AMCL_EINVAL, "amcl_pf_update_ranges: bad arguments");
  if (!pf->n)
    return AMCL_OK;
  return pf_update_impl(pf, nullptr, nullptr, 0, ranges4, nr, alpha, sigma, 0.0, 0.0, true);
}

extern "C" int amcl_pf_resample(amcl_pf_t pf)
{
  PF_GUARD(pf);
  if (!pf->n)
    return AMCL_OK;
  const float u = pf_next_uniform(pf);
  return do_resample(pf, u);
}

extern "C" int amcl_pf_resample_with(amcl_pf_t pf, float u01)
{
  PF_GUARD(pf);
  if (!(u01 >= 0.0f && u01 < 1.0f))
    return fail(AMCL_EINVAL, "amcl_pf_resample_with: u01 must be in [0, 1)");
  if (!pf->n)
    return AMCL_OK;
  return do_resample(pf, u01);
}

extern "C" int amcl_pf_get_mean(amcl_pf_t pf, float mean7[7], double mean_var[8])
{
  PF_GUARD(pf);
  if (!mean7)
    return fail(AMCL_EINVAL, "amcl_pf_get_mean: null output");
  for (int k = 0; k < 7; ++k)
    mean7[k] = 0.0f;
  if (mean_var)
    for (int k = 0; k < 8; ++k)
      mean_var[k] = 0.0;
  if (!pf->initialized)
    return AMCL_OK;  // mean_ of a fresh filter is Particle() = zeros
  AMCL_CUDA_TRY(cudaMemcpyAsync(pf->h_stats.p, pf->stats.p, sizeof(PFStats), cudaMemcpyDeviceToHost, pf->st.s));
  int rc = pf_check_err(pf);  // synchronises
  if (rc)
    return rc;
  const PFStats* st = pf->h_stats.as<PFStats>();
  for (int k = 0; k < 4; ++k)
    mean7[k] = st->mean_f[k];
  if (mean_var)
    for (int k = 0; k < 4; ++k)
    {
      mean_var[k] = st->mean[k];
      mean_var[4 + k] = st->var[k];
    }
  return AMCL_OK;
}

extern "C" int amcl_pf_is_initialized(amcl_pf_t pf, int* initialized)
{
  PF_GUARD(pf);
  if (!initialized)
    return fail(AMCL_EINVAL, "amcl_pf_is_initialized: null output");
  *initialized = pf->initialized ? 1 : 0;
  return AMCL_OK;
}

extern "C" int amcl_pf_size(amcl_pf_t pf, uint32_t* n)
{
  PF_GUARD(pf);
  if (!n)
    return fail(AMCL_EINVAL, "amcl_pf_size: null output");
  *n = pf->n;
  return AMCL_OK;
}

extern "C" int amcl_pf_get_particles(amcl_pf_t pf, float* p7, uint32_t cap)
{
  PF_GUARD(pf);
  if (!p7 && cap)
    return fail(AMCL_EINVAL, "amcl_pf_get_particles: null output");
  const uint32_t m = std::min(cap, pf->n);
  if (!m)
    return AMCL_OK;
  std::vector<float4> pose(m);
  std::vector<float> w(m), wp(m), wr(m);
  cudaStream_t s = pf->st.s;
  AMCL_CUDA_TRY(cudaMemcpyAsync(pose.data(), pf->pose[pf->cur].p, m * 16ull, cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(w.data(), pf->w[pf->cur].p, m * 4ull, cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(wp.data(), pf->wp[pf->cur].p, m * 4ull, cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(wr.data(), pf->wr[pf->cur].p, m * 4ull, cudaMemcpyDeviceToHost, s));
  int rc = pf_check_err(pf);
  if (rc)
    return rc;
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

extern "C" int amcl_pf_set_particles(amcl_pf_t pf, const float* p7, uint32_t n)
{
  PF_GUARD(pf);
  if (!p7 || !n)
    return fail(AMCL_EINVAL, "amcl_pf_set_particles: need at least one particle");
  if (n > (1u << 30))
    return fail(AMCL_ERANGE, "amcl_pf_set_particles: more than 2^30 particles");
  int rc;
  if ((rc = pf_reserve(pf, n)))
    return rc;
  AMCL_CUDA_TRY(cudaStreamSynchronize(pf->st.s));
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
  pf->n = n;
  pf->cur = 0;
  cudaStream_t s = pf->st.s;
  AMCL_CUDA_TRY(cudaMemcpyAsync(pf->pose[0].p, pose.data(), n * 16ull, cudaMemcpyHostToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(pf->w[0].p, w.data(), n * 4ull, cudaMemcpyHostToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(pf->wp[0].p, wp.data(), n * 4ull, cudaMemcpyHostToDevice, s));
  AMCL_CUDA_TRY(cudaMemcpyAsync(pf->wr[0].p, wr.data(), n * 4ull, cudaMemcpyHostToDevice, s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  pf->initialized = true;
  pf->blocksum_valid = false;
  pf->have_ridx = false;
  return AMCL_OK;
}

extern "C" int amcl_pf_set_option(amcl_pf_t pf, int option, int64_t value)
{
  PF_GUARD(pf);
  switch (option)
  {
    case AMCL_OPT_CLOUD_SUM:
      if (value < 0 || value > 1)
        return fail(AMCL_EINVAL, "AMCL_OPT_CLOUD_SUM: 0 or 1");
      pf->opt_cloud_sum = static_cast<int>(value);
      return AMCL_OK;
    case AMCL_OPT_RESAMPLE_PREFIX:
      if (value < 0 || value > 1)
        return fail(AMCL_EINVAL, "AMCL_OPT_RESAMPLE_PREFIX: 0 or 1");
      pf->opt_prefix = static_cast<int>(value);
      return AMCL_OK;
    case AMCL_OPT_WEIGHT_KERNEL:
      if (value < 0 || value > 2)
        return fail(AMCL_EINVAL, "AMCL_OPT_WEIGHT_KERNEL: 0, 1 or 2");
      pf->opt_kernel = static_cast<int>(value);
      return AMCL_OK;
    case AMCL_OPT_SEED:
      pf->seed = static_cast<uint64_t>(value);
      pf->step = 0;
      return AMCL_OK;
    case AMCL_OPT_WAIT_PROBE:
      if (value < 0 || value > 1)
        return fail(AMCL_EINVAL, "AMCL_OPT_WAIT_PROBE: 0 or 1");
      pf->opt_wait_probe = static_cast<int>(value);
      return AMCL_OK;
    default:
      return fail(AMCL_ENOTSUP, "amcl_pf_set_option: unknown option");
  }
}

extern "C" int amcl_pf_record_draws(amcl_pf_t pf, int enable)
{
  PF_GUARD(pf);
  pf->record = enable != 0;
  return AMCL_OK;
}

extern "C" int amcl_pf_get_draws(amcl_pf_t pf, float* out, uint32_t cap_floats)
{
  PF_GUARD(pf);
  if (!out && cap_floats)
    return fail(AMCL_EINVAL, "amcl_pf_get_draws: null output");
  const uint64_t m = std::min<uint64_t>(cap_floats, 4ull * pf->n);
  if (m)
    AMCL_CUDA_TRY(cudaMemcpyAsync(out, pf->draws.p, m * 4, cudaMemcpyDeviceToHost, pf->st.s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(pf->st.s));
  return AMCL_OK;
}

extern "C" int amcl_pf_get_resample_index(amcl_pf_t pf, int32_t* out, uint32_t cap)
{
  PF_GUARD(pf);
  if (!pf->have_ridx)
    return fail(AMCL_ESTATE, "amcl_pf_get_resample_index: no resample since the last init/set");
  const uint32_t m = std::min(cap, pf->n);
  if (m)
    AMCL_CUDA_TRY(cudaMemcpyAsync(out, pf->ridx.p, m * 4ull, cudaMemcpyDeviceToHost, pf->st.s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(pf->st.s));
  return AMCL_OK;
}

extern "C" int amcl_pf_stream(amcl_pf_t pf, void** stream)
{
  if (!pf || !stream)
    return fail(AMCL_EINVAL, "amcl_pf_stream: bad arguments");
  *stream = pf->st.s;
  return AMCL_OK;
}

extern "C" int amcl_pf_profile(amcl_pf_t pf, int enable)
{
  PF_GUARD(pf);
  pf->prof.on = enable != 0;
  return AMCL_OK;
}

extern "C" int amcl_pf_profile_read(amcl_pf_t pf, double ms[AMCL_PROF_COUNT], uint64_t launches[AMCL_PROF_COUNT],
                                    int reset)
{
  PF_GUARD(pf);
  pf->prof.collect();
  for (int k = 0; k < AMCL_PROF_COUNT; ++k)
  {
    if (ms)
      ms[k] = pf->prof.ms[k];
    if (launches)
      launches[k] = pf->prof.n[k];
    if (reset)
    {
      pf->prof.ms[k] = 0;
      pf->prof.n[k] = 0;
    }
  }
  return AMCL_OK;
}
