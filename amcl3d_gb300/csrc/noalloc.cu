// amcl_grid_cloud_weights_noalloc: the cloud weighting for callers that may not
// allocate device memory.
//
// Some callers cannot call cudaMalloc at all: code running where the allocator is
// owned by someone else (a real-time loop that must not page or block inside the
// CUDA allocator, a process whose device memory is handed out by a host
// framework's pool, code inside a memory budget that forbids new allocations).
// This entry point computes the same per-particle cloud weights as
// amcl_grid_cloud_weights with the two-phase kernel, but its scratch slab lives in
// a file-scope __device__ array of fixed size instead of a buffer allocated per
// call.  Inputs and outputs are the caller's device buffers.
//
// Limits: at most NOALLOC_MAX_PARTICLES particles and
// ceil(P / 32) * 32 * N <= NOALLOC_MAX_SCRATCH_FLOATS (16 MiB of floats).  The
// array occupies that memory on every GPU that loads the library until the process
// exits.  All calls share it: calls that overlap on the GPU (on different streams,
// or from different threads without ordering) race on it and give wrong results.
// The first call on each device looks the array's device address up
// (cudaGetSymbolAddress) with that device current; make that first call before
// any stream capture.
#include <mutex>

#include "grid.cuh"

namespace
{
constexpr uint32_t NOALLOC_MAX_PARTICLES = 65536;
constexpr uint64_t NOALLOC_MAX_SCRATCH_FLOATS = 4ull * 1024 * 1024;
constexpr uint64_t NOALLOC_ERR_FLOATS = 64;  // one int, padded to 256 bytes
constexpr uint64_t NOALLOC_FLOATS = NOALLOC_ERR_FLOATS + NOALLOC_MAX_PARTICLES + NOALLOC_MAX_SCRATCH_FLOATS;

// [0, 64): error word; [64, 64 + MAX_P): range-weight sink (the kernel writes wr);
// then the two-phase scratch slab.
static __device__ __align__(256) float g_noalloc_scratch[NOALLOC_FLOATS];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
float* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};

// Device address of the array on the current device (looked up once per device).
int noalloc_base(float** out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return amcl::fail(AMCL_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return amcl::fail(AMCL_ERANGE, "amcl_grid_cloud_weights_noalloc: device ordinal beyond 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev])
  {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return amcl::fail(AMCL_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_noalloc_addr[dev] = static_cast<float*>(p);
  }
  *out = g_noalloc_addr[dev];
  return AMCL_OK;
}
}  // namespace

extern "C" int amcl_grid_cloud_weights_noalloc(amcl_grid_t g, const void* poses_f4_dev, uint32_t P,
                                                const void* cloud_f4_dev, uint32_t n, float roll, float pitch,
                                                float* out_dev, void* stream)
{
  using namespace amcl;
  if (!g || (P && (!poses_f4_dev || !out_dev)) || (n && !cloud_f4_dev) ||
      (reinterpret_cast<uintptr_t>(poses_f4_dev) & 15) || (reinterpret_cast<uintptr_t>(cloud_f4_dev) & 15) ||
      (reinterpret_cast<uintptr_t>(out_dev) & 3))
    return fail(AMCL_EINVAL, "amcl_grid_cloud_weights_noalloc: bad arguments (float4 inputs 16-byte aligned)");
  if (P > NOALLOC_MAX_PARTICLES)
    return fail(AMCL_ERANGE, "amcl_grid_cloud_weights_noalloc: more than 65536 particles");
  if (two_phase_scratch_floats(P, n) > NOALLOC_MAX_SCRATCH_FLOATS)
    return fail(AMCL_ERANGE,
                "amcl_grid_cloud_weights_noalloc: ceil(P/32)*32*N exceeds the 4194304-float (16 MiB) scratch array");
  if (!P)
    return AMCL_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!g->built)
  {
    // computeCloudWeight of a grid never opened is 0 (Grid3d.cpp:136-137)
    AMCL_CUDA_TRY(cudaMemsetAsync(out_dev, 0, P * sizeof(float), s));
    AMCL_CUDA_TRY(cudaStreamSynchronize(s));
    return AMCL_OK;
  }
  float* base = nullptr;
  int rc = noalloc_base(&base);
  if (rc)
    return rc;
  int* err = reinterpret_cast<int*>(base);
  AMCL_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));  // the error word starts at zero every call
  WeightArgs a{};
  a.pose = static_cast<const float4*>(poses_f4_dev);
  a.P = P;
  a.cloud = static_cast<const float4*>(cloud_f4_dev);
  a.N = n;
  a.sr = sinf(roll);
  a.cr = cosf(roll);
  a.sp = sinf(pitch);
  a.cp = cosf(pitch);
  a.wp = out_dev;
  a.wr = base + NOALLOC_ERR_FLOATS;
  a.err = err;
  a.ignore_map = 1;
  a.kernel = 2;
  a.scratch = base + NOALLOC_ERR_FLOATS + NOALLOC_MAX_PARTICLES;
  a.scratch_floats = NOALLOC_MAX_SCRATCH_FLOATS;
  if ((rc = launch_cloud_weight(g, a, s)))
    return rc;
  int e = 0;
  AMCL_CUDA_TRY(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  AMCL_CUDA_TRY(cudaStreamSynchronize(s));
  if (e)
    return fail(AMCL_ETIMEDOUT, "amcl_grid_cloud_weights_noalloc: a bounded device-side wait gave up");
  return AMCL_OK;
}
