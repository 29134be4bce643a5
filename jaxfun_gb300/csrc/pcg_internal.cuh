// Internal PCG problem description shared by the plain and mixed solvers.
#pragma once

#include <vector>

#include <cuda_runtime.h>

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

// Key of a cached instantiated graph: the sizes, switches and scalars it was
// captured with, and every pointer its kernels use.
struct GraphKey {
  std::vector<long long> ints;
  std::vector<const void*> ptrs;
  bool operator==(const GraphKey& o) const { return ints == o.ints && ptrs == o.ptrs; }
};

// The batched PCG as reusable steps on a workspace (pcg_ws bytes): problems
// can (re)start one list at a time and leave through the ready list, so
// different problems may be at different points of their solves.
template <typename T>
struct PcgCtx {
  static constexpr int CH = 10;  // iterations per captured chunk
  PcgProblem<T> pb;
  cudaStream_t st = 0;
  int ndim = 2, n = 0, nq = 0, batch = 0, vb = 1;
  long long N = 0;
  T *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
  T *pq_part = nullptr, *rz_part[2] = {nullptr, nullptr}, *rz0 = nullptr;
  int *iters = nullptr, *alist = nullptr, *nactive = nullptr, *nready = nullptr;
  int *inner_it = nullptr, *ready = nullptr;
  int* keep = nullptr;  // per problem: stays active after this iteration (k_update_xp)
  double* tolv = nullptr;   // per-problem tolerance (device)
  unsigned* slots = nullptr;
  void* inner = nullptr;
  size_t inner_bytes = 0;
  void* work_ptr = nullptr;
  size_t work_size = 0;
  bool th = false, fuse_pq = false, fuse_rz = false;
  int nb_pq = 16, nb_rz = 16;
  H16Ops h16;
  int maxit = 0;             // per-problem iteration cap since its start (0: none)
  bool track_ready = false;  // problems leaving the active list go to the ready list

  // x: the (batch, n^ndim) iterate; pb.rhs the right-hand sides; clears the
  // active and ready counts and the iteration counts
  int init(const PcgProblem<T>& problem, T* x, void* work, size_t work_bytes, cudaStream_t st);
  // (re)start the listed problems (list NULL: all) from x = 0, or from x with
  // use_x0 (judged against the zero start with judge); tolv must be set
  int start(const int* list, const int* count, int use_x0, bool judge);
  int iteration(int it);
  int chunk();  // CH iterations through the cached graph (launched directly on the
                // legacy default stream, which cannot be captured)

  int applyA(const T* in, T* out, Active a, DotOut* dot = nullptr);
  int applyM(const T* in, T* out, Active a, DotOut* dot = nullptr);
  int applyM_dot(const T* in, T* out, Active a, T* part, int& nb);
  int record_max(const T* v, Active a);
};

}  // namespace jfg
