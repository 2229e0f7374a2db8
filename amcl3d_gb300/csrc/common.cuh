// Shared host/device plumbing of the amcl3d GB300 library: status reporting,
// CUDA error checks, launch accounting and the per-family event profiler.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/amcl3d_gpu.h"

namespace amcl
{
// ---- status -------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);

#define AMCL_CUDA_TRY(expr)                                                                   \
  do                                                                                          \
  {                                                                                           \
    cudaError_t e_ = (expr);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return ::amcl::fail(e_ == cudaErrorMemoryAllocation ? AMCL_ENOMEM : AMCL_ECUDA,         \
                          std::string(#expr) + ": " + cudaGetErrorString(e_));                \
  } while (0)

#define AMCL_LAUNCH_CHECK(name)                                                               \
  do                                                                                          \
  {                                                                                           \
    ::amcl::count_launch();                                                                   \
    cudaError_t e_ = cudaGetLastError();                                                      \
    if (e_ != cudaSuccess)                                                                    \
      return ::amcl::fail(AMCL_ECUDA, std::string("launch ") + name + ": " + cudaGetErrorString(e_)); \
  } while (0)

void count_launch();

// ---- streams ---------------------------------------------------------------------
struct StreamHolder
{
  cudaStream_t s = nullptr;
  bool owned = false;
  int init(void* user)
  {
    if (user)
    {
      s = static_cast<cudaStream_t>(user);
      owned = false;
      return AMCL_OK;
    }
    AMCL_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    owned = true;
    return AMCL_OK;
  }
  ~StreamHolder()
  {
    if (owned && s)
      cudaStreamDestroy(s);
  }
};

// ---- device buffers ----------------------------------------------------------------
struct DevBuf
{
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t want)
  {
    if (want <= bytes && p)
      return AMCL_OK;
    if (p)
      cudaFree(p);
    p = nullptr;
    bytes = 0;
    if (want == 0)
      return AMCL_OK;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess)
    {
      p = nullptr;
      return fail(AMCL_ENOMEM, std::string("cudaMalloc ") + std::to_string(want) + " B: " + cudaGetErrorString(e));
    }
    bytes = want;
    return AMCL_OK;
  }
  void release()
  {
    if (p)
      cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T* as() const
  {
    return static_cast<T*>(p);
  }
  ~DevBuf() { release(); }
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

struct PinnedBuf
{
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t want)
  {
    if (want <= bytes && p)
      return AMCL_OK;
    if (p)
      cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    if (want == 0)
      return AMCL_OK;
    cudaError_t e = cudaMallocHost(&p, want);
    if (e != cudaSuccess)
    {
      p = nullptr;
      return fail(AMCL_ENOMEM, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    bytes = want;
    return AMCL_OK;
  }
  template <typename T>
  T* as() const
  {
    return static_cast<T*>(p);
  }
  ~PinnedBuf()
  {
    if (p)
      cudaFreeHost(p);
  }
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
};

// ---- event profiler ------------------------------------------------------------------
struct Profiler
{
  bool on = false;
  struct Pair
  {
    cudaEvent_t a, b;
    int kind;
  };
  std::vector<Pair> pending;
  std::vector<cudaEvent_t> pool;
  double ms[AMCL_PROF_COUNT] = {};
  uint64_t n[AMCL_PROF_COUNT] = {};

  cudaEvent_t get()
  {
    if (!pool.empty())
    {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  // Returns the index of an open pair, or -1 when profiling is off.
  int begin(cudaStream_t s, int kind)
  {
    if (!on)
      return -1;
    Pair p{ get(), get(), kind };
    cudaEventRecord(p.a, s);
    pending.push_back(p);
    return static_cast<int>(pending.size()) - 1;
  }
  void end(cudaStream_t s, int idx)
  {
    if (idx >= 0)
      cudaEventRecord(pending[idx].b, s);
  }
  void collect()
  {
    for (auto& p : pending)
    {
      cudaEventSynchronize(p.b);
      float t = 0;
      cudaEventElapsedTime(&t, p.a, p.b);
      ms[p.kind] += t;
      n[p.kind] += 1;
      pool.push_back(p.a);
      pool.push_back(p.b);
    }
    pending.clear();
  }
  ~Profiler()
  {
    for (auto& p : pending)
    {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    for (auto e : pool)
      cudaEventDestroy(e);
  }
};

struct ProfScope
{
  Profiler* p;
  cudaStream_t s;
  int idx;
  ProfScope(Profiler* p_, cudaStream_t s_, int kind) : p(p_), s(s_), idx(p_ ? p_->begin(s_, kind) : -1) {}
  ~ProfScope()
  {
    if (p)
      p->end(s, idx);
  }
};

inline unsigned ceil_div(uint64_t a, uint64_t b) { return static_cast<unsigned>((a + b - 1) / b); }

// Runs f(i) for i in [0, n) on up to `threads` host threads (the caller's included),
// items taken in order from a shared counter; serial for threads <= 1.
template <typename F>
void host_parallel_for(uint32_t n, unsigned threads, F f)
{
  threads = std::min<unsigned>(threads, n);
  if (threads <= 1)
  {
    for (uint32_t i = 0; i < n; ++i)
      f(i);
    return;
  }
  std::atomic<uint32_t> next{ 0 };
  auto work = [&] {
    for (uint32_t i = next.fetch_add(1); i < n; i = next.fetch_add(1))
      f(i);
  };
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < threads; ++t)
    pool.emplace_back(work);
  work();
  for (auto& th : pool)
    th.join();
}

// Host threads for copies of `bytes` in total: one below 1 MB, else up to 8 (or half
// the hardware threads).
inline unsigned copy_threads(uint64_t bytes)
{
  if (bytes < (1u << 20))
    return 1;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency() / 2);
  return std::min(8u, hw);
}

// Runs `set` (returning an AMCL status) once for the current device and remembers
// success per device ordinal (0-63) in `done`: kernel attributes are per device.
template <typename F>
int once_per_device(std::atomic<uint64_t>& done, F set)
{
  int dev = 0;
  AMCL_CUDA_TRY(cudaGetDevice(&dev));
  const uint64_t bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit))
    return AMCL_OK;
  const int rc = set();
  if (rc == AMCL_OK && bit)
    done.fetch_or(bit, std::memory_order_acq_rel);
  return rc;
}

int device_sm_count();

}  // namespace amcl
