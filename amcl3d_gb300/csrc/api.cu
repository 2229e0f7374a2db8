// Status reporting and process-wide counters of the C ABI.
#include "common.cuh"

namespace
{
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{ 0 };
}  // namespace

namespace amcl
{
void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int status, const std::string& msg)
{
  g_last_error = msg;
  return status;
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int device_sm_count()
{
  static int cached = 0;
  if (!cached)
  {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
      cached = n;
    else
      cached = 152;
  }
  return cached;
}
}  // namespace amcl

extern "C" const char* amcl_status_string(int status)
{
  switch (status)
  {
    case AMCL_OK:
      return "ok";
    case AMCL_EINVAL:
      return "invalid argument";
    case AMCL_ENOMEM:
      return "out of memory";
    case AMCL_ECUDA:
      return "CUDA error";
    case AMCL_ETIMEDOUT:
      return "device wait timed out";
    case AMCL_ESTATE:
      return "invalid state";
    case AMCL_EIO:
      return "I/O error";
    case AMCL_ERANGE:
      return "size out of range";
    case AMCL_ENOTSUP:
      return "not supported";
    default:
      return "unknown status";
  }
}

extern "C" const char* amcl_last_error(void) { return g_last_error.c_str(); }

extern "C" int amcl_version(int* major, int* minor)
{
  if (major)
    *major = 0;
  if (minor)
    *minor = 1;
  return AMCL_OK;
}

extern "C" uint64_t amcl_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }
