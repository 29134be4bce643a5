// Library-level C ABI: version, status strings, error reporting, device check.
#include "jfg_internal.cuh"

#include <atomic>

namespace jfg {
namespace {
thread_local int g_last_cuda_error = 0;
thread_local bool g_capturing = false;
std::atomic<long long> g_launches{0};
}  // namespace
void set_last_cuda_error(cudaError_t e) { g_last_cuda_error = (int)e; }
void count_launches(long long n) {
  if (!g_capturing) g_launches.fetch_add(n, std::memory_order_relaxed);
}
void set_capturing(bool on) { g_capturing = on; }
}  // namespace jfg

extern "C" long long jfg_launch_count(void) { return jfg::g_launches.load(); }
extern "C" void jfg_reset_launch_count(void) { jfg::g_launches.store(0); }

extern "C" const char* jfg_version(void) { return "jaxfun_gb300 0.1.0 (sm_103a)"; }

extern "C" const char* jfg_status_string(int s) {
  switch (s) {
    case JFG_OK:
      return "ok";
    case JFG_ERR_ARG:
      return "invalid argument";
    case JFG_ERR_CUDA:
      return "CUDA error";
    case JFG_ERR_NOT_CONVERGED:
      return "not converged";
    case JFG_ERR_DEVICE_TIMEOUT:
      return "device wait timed out";
    case JFG_ERR_UNSUPPORTED:
      return "unsupported device or configuration";
    case JFG_ERR_WORKSPACE:
      return "workspace too small";
    default:
      return "unknown status";
  }
}

extern "C" int jfg_last_cuda_error(void) { return jfg::g_last_cuda_error; }

extern "C" int jfg_device_supported(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  return (major == 10 && minor == 3) ? 1 : 0;
}
