// Fast-diagonalisation solve that allocates nothing: the scratch buffers the
// solve needs between its per-axis passes live in a fixed device array that
// the library carries, instead of a workspace the caller provides.
//
// Who needs this: callers that cannot call cudaMalloc (or any allocating
// routine) at the point where they solve -- for example a custom-call handler
// inside another runtime that owns all device memory and hands out no
// workspace, or a real-time loop that must not block on the allocator.  They
// pass only the inputs and the output.
//
// Limits and sharing: the scratch array is JFG_NOALLOC_SCRATCH_BYTES (32 MiB)
// and every GPU that loads this library holds one copy until the process
// exits.  Requests whose scratch need exceeds it are rejected with
// JFG_ERR_WORKSPACE before anything is launched.  All calls on a device share
// the one array, so two calls whose kernels overlap on the GPU (different
// streams without ordering between them) race and corrupt each other's
// results; calls on one stream are ordered and safe.  The array keeps the
// previous call's contents; this solve writes every scratch element it later
// reads, so nothing needs clearing.
//
// Set-up: the first call on each device looks up the device address of the
// array (cudaGetSymbolAddress) with that device current, and caches it for
// the life of the process.  Make that first call before any stream capture.
// The cache is not refreshed after cudaDeviceReset: a process that resets a
// device must not call this entry point on it again.
#include <mutex>

#include "jfg_internal.cuh"

#define JFG_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)

namespace {

static __device__ __align__(256) unsigned char g_fd_scratch[JFG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_ptr[kMaxDevices] = {};

// Device address of g_fd_scratch on the current device (looked up once per
// device).  In host code the symbol name itself is only a host-side stand-in
// and must never be handed to a kernel.
int scratch_ptr(void** out) {
  int dev = 0;
  JFG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return JFG_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_ptr[dev]) {
    void* p = nullptr;
    JFG_CUDA_TRY(cudaGetSymbolAddress(&p, g_fd_scratch));
    if (!p) return JFG_ERR_CUDA;
    g_ptr[dev] = p;
  }
  *out = g_ptr[dev];
  return JFG_OK;
}

}  // namespace

extern "C" size_t jfg_fd_solve_noalloc_max_bytes(void) { return JFG_NOALLOC_SCRATCH_BYTES; }

extern "C" int jfg_fd_solve_f64_noalloc(int ndim, int n, int batch, const double* E,
                                        const double* W, const double* lam, const double* c0,
                                        const double* c1, const double* rhs, double* out,
                                        void* stream) {
  if ((ndim != 2 && ndim != 3) || n < 1 || batch < 0) return JFG_ERR_ARG;
  // Size check by division, so that no product below can wrap around: one
  // field of the batch (batch * n^ndim doubles) must fit in the array.
  const size_t cap_elems = JFG_NOALLOC_SCRATCH_BYTES / sizeof(double);
  size_t per = 1;
  for (int i = 0; i < ndim; ++i) {
    if (per > cap_elems / (size_t)n) return JFG_ERR_WORKSPACE;
    per *= (size_t)n;
  }
  if ((size_t)batch > cap_elems / per) return JFG_ERR_WORKSPACE;
  const size_t need = jfg::fd_ws(ndim, n, batch, (int)sizeof(double));
  if (need > JFG_NOALLOC_SCRATCH_BYTES) return JFG_ERR_WORKSPACE;
  void* scratch = nullptr;
  JFG_TRY(scratch_ptr(&scratch));
  return jfg::fd_solve<double>(jfg::Engine::F64, ndim, n, batch,
                               jfg::OpRef<double>{E, nullptr}, jfg::OpRef<double>{W, nullptr},
                               lam, c0, c1, rhs, out, scratch, JFG_NOALLOC_SCRATCH_BYTES,
                               (cudaStream_t)stream);
}
