// Internal PCG problem description shared by the plain and mixed solvers.
#pragma once

#include <vector>

#include "jfg_internal.cuh"

namespace jfg {

template <typename T>
struct PcgProblem {
  Engine engine = Engine::F64;
  Engine m_engine = Engine::F64;   // engine of the preconditioner (E, W point at BF16
                                   // pairs when it is Engine::TB)
  int ndim = 2, n = 0, nq = 0, batch = 0;
  OpRef<T> ops{nullptr, nullptr};  // packed variable-coefficient operators (FP16 pairs
                                   // when engine is Engine::TH)
  const float* ops_inv = nullptr;  // Engine::TH: inverse row scales of the operators
  const T* kw = nullptr;           // (batch, nq^ndim) kappa * quadrature weights
  OpRef<T> E{nullptr, nullptr};    // fast-diagonalisation forward (n x n)
  OpRef<T> W{nullptr, nullptr};    // fast-diagonalisation backward (n x n)
  const T* lam = nullptr;          // (n)
  const T* fd_scale = nullptr;     // (batch) constant kappa of the preconditioner
  const T* rhs = nullptr;          // (batch, n^ndim)
  // with an initial guess: keep it per problem only if its preconditioned
  // residual beats the zero start, and stop relative to the right-hand side
  bool judge_x0 = false;
  // fused dots (FP32 tensor-core engines): bit 0 p.Ap from the operator's
  // field pass, bit 1 r.M^-1 r from the preconditioner's divide pass (only
  // when its forward factor is the transpose of its backward factor)
  int fuse_dots = 0;
};

template <typename T>
size_t pcg_ws(int ndim, int n, int nq, int batch);

// out32 (padded nq per axis) = in64 (n per axis) * scale[b]; zero padding
int launch_pad_scale(int ndim, int n, int nq, int batch, const double* in, const double* scale,
                     float* out, cudaStream_t st);
// x64 (n per axis) += sign * s[b] * d32 (padded); problems with s[b] == 0 untouched
int launch_unpad_axpy(int ndim, int n, int nq, int batch, const float* d, const double* s,
                      double* x, double sign, cudaStream_t st);
// 2-norms of the batch's vectors (length N each); synchronises the stream.
// part_dev holds batch * 16 doubles.
int batch_norms(long long N, int batch, const double* x, double* part_dev,
                std::vector<double>& norms, cudaStream_t st);

template <typename T>
int pcg_run(const PcgProblem<T>& pb, T* x, int use_x0, double tol, int maxiter,
            int* iters_host, void* work, size_t work_bytes, cudaStream_t st);

}  // namespace jfg
