// XLA FFI handlers over the C ABI: the custom calls that jaxfun's jit-compiled
// methods make to reach the GB300 kernels.
//
//   TensorProductSpace.forward / backward / scalar_product
//     (src/jaxfun/galerkin/tensorproductspace.py:330-417)   -> jfg_tp_apply_{1,2,3}d
//   TPMatricesLUFactors.solve (src/jaxfun/la/tpmatrix.py:545-587)
//                                                           -> jfg_fd_solve_{2,3}d
//   TensorMatrix.__matmul__ for kappa*Dot(Grad(u), Grad(v))
//     (src/jaxfun/la/tensormatrix.py:54-56)                 -> jfg_varcoef_apply
//   PCG on that operator, FD-preconditioned                 -> jfg_pcg_varcoef
//
// Every handler takes XLA's CUDA stream (PlatformStream), draws its workspace
// from XLA's scratch allocator (so the library itself allocates nothing) and
// turns a non-zero status into an ffi::Error.  Shapes come from the buffers:
// a leading batch axis, then the per-axis extents, row-major like jax.Array.
// Built by jaxfun_gb300/build.py only when xla/ffi/api/ffi.h is available
// (jaxlib's include directory, or JFG_XLA_INCLUDE); linked against
// libjaxfun_gb300.so.
#include <cuda_runtime.h>

#include <cstdint>
#include <optional>
#include <string>
#include <vector>

#include "jaxfun_gb300.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

ffi::Error status_error(int s, const char* what) {
  if (s == JFG_OK) return ffi::Error::Success();
  return ffi::Error(ffi::ErrorCode::kInternal,
                    std::string(what) + ": " + jfg_status_string(s));
}

std::optional<void*> scratch_bytes(ffi::ScratchAllocator& scratch, size_t bytes) {
  if (bytes == 0) return std::optional<void*>(nullptr);
  return scratch.Allocate(bytes, 256);
}

// y[b] = (x_ax mats[ax]) x[b]: mats[ax] is (rows_ax, cols_ax), x is
// (batch, cols_0, ..., cols_{ND-1}), y is (batch, rows_0, ...).
template <int ND>
ffi::Error tp_apply(cudaStream_t st, ffi::ScratchAllocator& scratch,
                    ffi::Buffer<ffi::F64> x, const ffi::Buffer<ffi::F64>* mats,
                    ffi::ResultBuffer<ffi::F64> y) {
  auto xd = x.dimensions();
  if ((int)xd.size() != ND + 1)
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "x must be (batch, axes...)");
  int rows[3], cols[3];
  const double* mp[3];
  for (int a = 0; a < ND; ++a) {
    auto md = mats[a].dimensions();
    if (md.size() != 2 || md[1] != xd[a + 1])
      return ffi::Error(ffi::ErrorCode::kInvalidArgument, "operator shape mismatch");
    rows[a] = (int)md[0];
    cols[a] = (int)md[1];
    mp[a] = mats[a].typed_data();
  }
  const int batch = (int)xd[0];
  const size_t ws = jfg_tp_apply_workspace_size(ND, rows, cols, batch, 8);
  auto w = scratch_bytes(scratch, ws);
  if (!w) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "tp_apply workspace");
  return status_error(jfg_tp_apply_f64(ND, rows, cols, batch, mp, x.typed_data(),
                                       y->typed_data(), *w, ws, st),
                      "jfg_tp_apply_f64");
}

ffi::Error TpApply1Impl(cudaStream_t st, ffi::ScratchAllocator scratch,
                        ffi::Buffer<ffi::F64> x, ffi::Buffer<ffi::F64> m0,
                        ffi::ResultBuffer<ffi::F64> y) {
  const ffi::Buffer<ffi::F64> mats[1] = {m0};
  return tp_apply<1>(st, scratch, x, mats, y);
}

ffi::Error TpApply2Impl(cudaStream_t st, ffi::ScratchAllocator scratch,
                        ffi::Buffer<ffi::F64> x, ffi::Buffer<ffi::F64> m0,
                        ffi::Buffer<ffi::F64> m1, ffi::ResultBuffer<ffi::F64> y) {
  const ffi::Buffer<ffi::F64> mats[2] = {m0, m1};
  return tp_apply<2>(st, scratch, x, mats, y);
}

ffi::Error TpApply3Impl(cudaStream_t st, ffi::ScratchAllocator scratch,
                        ffi::Buffer<ffi::F64> x, ffi::Buffer<ffi::F64> m0,
                        ffi::Buffer<ffi::F64> m1, ffi::Buffer<ffi::F64> m2,
                        ffi::ResultBuffer<ffi::F64> y) {
  const ffi::Buffer<ffi::F64> mats[3] = {m0, m1, m2};
  return tp_apply<3>(st, scratch, x, mats, y);
}

// U = (x W) [(x E) F / (c0[b] + c1[b] * sum lam)], F (batch, n, ..., n)
ffi::Error FdSolveImpl(cudaStream_t st, ffi::ScratchAllocator scratch,
                       ffi::Buffer<ffi::F64> E, ffi::Buffer<ffi::F64> W,
                       ffi::Buffer<ffi::F64> lam, ffi::Buffer<ffi::F64> c0,
                       ffi::Buffer<ffi::F64> c1, ffi::Buffer<ffi::F64> rhs,
                       ffi::ResultBuffer<ffi::F64> out) {
  auto rd = rhs.dimensions();
  const int ndim = (int)rd.size() - 1;
  if (ndim != 2 && ndim != 3)
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "rhs must be (batch, n, n[, n])");
  const int n = (int)rd[1], batch = (int)rd[0];
  if ((int)lam.element_count() != n || (int)c0.element_count() != batch ||
      (int)c1.element_count() != batch)
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "lam / c0 / c1 size mismatch");
  const size_t ws = jfg_fd_solve_workspace_size(ndim, n, batch, 8);
  auto w = scratch_bytes(scratch, ws);
  if (!w) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "fd_solve workspace");
  return status_error(jfg_fd_solve_f64(ndim, n, batch, E.typed_data(), W.typed_data(),
                                       lam.typed_data(), c0.typed_data(), c1.typed_data(),
                                       rhs.typed_data(), out->typed_data(), *w, ws, st),
                      "jfg_fd_solve_f64");
}

// v = A(kappa) u: ops from jfg_varcoef_pack_ops_host, kw (batch, nq^ndim),
// u (batch, n^ndim)
ffi::Error VarcoefApplyImpl(cudaStream_t st, ffi::ScratchAllocator scratch,
                            ffi::Buffer<ffi::F64> ops, ffi::Buffer<ffi::F64> kw,
                            ffi::Buffer<ffi::F64> u, ffi::ResultBuffer<ffi::F64> v) {
  auto ud = u.dimensions();
  auto kd = kw.dimensions();
  const int ndim = (int)ud.size() - 1;
  if ((ndim != 2 && ndim != 3) || kd.size() != ud.size() || kd[0] != ud[0])
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "u / kw shape mismatch");
  const int batch = (int)ud[0], n = (int)ud[1], nq = (int)kd[1];
  if ((size_t)ops.element_count() != jfg_varcoef_ops_count(ndim, n, nq))
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "packed operator size mismatch");
  const size_t ws = jfg_varcoef_workspace_size(ndim, n, nq, batch, 8);
  auto w = scratch_bytes(scratch, ws);
  if (!w) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "varcoef workspace");
  return status_error(jfg_varcoef_apply_f64(ndim, n, nq, batch, ops.typed_data(),
                                            kw.typed_data(), u.typed_data(), v->typed_data(),
                                            *w, ws, st),
                      "jfg_varcoef_apply_f64");
}

// Batched FP64 PCG with the constant-coefficient FD preconditioner; x from a
// zero start, iteration counts per problem in iters (int32).
ffi::Error PcgVarcoefImpl(cudaStream_t st, ffi::ScratchAllocator scratch,
                          ffi::Buffer<ffi::F64> ops, ffi::Buffer<ffi::F64> kw,
                          ffi::Buffer<ffi::F64> E, ffi::Buffer<ffi::F64> W,
                          ffi::Buffer<ffi::F64> lam, ffi::Buffer<ffi::F64> fd_scale,
                          ffi::Buffer<ffi::F64> rhs, ffi::ResultBuffer<ffi::F64> x,
                          ffi::ResultBuffer<ffi::S32> iters, double tol, int64_t maxiter) {
  auto rd = rhs.dimensions();
  auto kd = kw.dimensions();
  const int ndim = (int)rd.size() - 1;
  if ((ndim != 2 && ndim != 3) || kd.size() != rd.size())
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "rhs / kw shape mismatch");
  const int batch = (int)rd[0], n = (int)rd[1], nq = (int)kd[1];
  const size_t ws = jfg_pcg_workspace_size(ndim, n, nq, batch, 8);
  auto w = scratch_bytes(scratch, ws);
  if (!w) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "pcg workspace");
  // the iteration counts come back through a host array, then to the device
  // result (ordered on the stream)
  std::vector<int> it(batch, 0);
  const int s = jfg_pcg_varcoef_f64(ndim, n, nq, batch, ops.typed_data(), kw.typed_data(),
                                    E.typed_data(), W.typed_data(), lam.typed_data(),
                                    fd_scale.typed_data(), rhs.typed_data(), x->typed_data(), 0,
                                    tol, (int)maxiter, it.data(), *w, ws, st);
  if (s != JFG_OK && s != JFG_ERR_NOT_CONVERGED) return status_error(s, "jfg_pcg_varcoef_f64");
  if (cudaMemcpyAsync(iters->typed_data(), it.data(), sizeof(int) * batch,
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return ffi::Error(ffi::ErrorCode::kInternal, "iteration count copy");
  return ffi::Error::Success();
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(JfgTpApply1d, TpApply1Impl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>());

XLA_FFI_DEFINE_HANDLER_SYMBOL(JfgTpApply2d, TpApply2Impl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>());

XLA_FFI_DEFINE_HANDLER_SYMBOL(JfgTpApply3d, TpApply3Impl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>());

XLA_FFI_DEFINE_HANDLER_SYMBOL(JfgFdSolve, FdSolveImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>());

XLA_FFI_DEFINE_HANDLER_SYMBOL(JfgVarcoefApply, VarcoefApplyImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>());

XLA_FFI_DEFINE_HANDLER_SYMBOL(JfgPcgVarcoef, PcgVarcoefImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Ctx<ffi::ScratchAllocator>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::S32>>()
                                  .Attr<double>("tol")
                                  .Attr<int64_t>("maxiter"));
