// Batched preconditioned conjugate gradients for the variable-coefficient
// operator with the constant-coefficient fast-diagonalisation preconditioner.
//
// Per-problem scalars live on the device as block partial sums (warp-shuffle
// reductions), so no kernel waits on the host.  The problems still iterating
// form a device-side active list, rebuilt after every iteration by a one-block
// compaction kernel; every kernel of the iteration (the tensor-core or CUDA-core
// contraction passes included) reads the list when it starts and works on the
// listed problems only, so a converged problem costs nothing from then on and
// the batch pays for the mean iteration count, not the maximum.  Chunks of
// iterations are captured once into a CUDA graph and replayed; the host reads
// the active count once per chunk.
#include <math.h>
#include <string.h>

#include <mutex>
#include <type_traits>
#include <vector>

#include "jfg_internal.cuh"
#include "pcg_internal.cuh"

namespace jfg {

namespace {

constexpr int NB = 16;    // partial sums per problem of the explicit dot kernel
constexpr int PS = DOT_NBMAX;  // partial-sum slots per problem (fused dots use up to PS)
constexpr int DOT_T = 256;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T block_sum(T v) {
  __shared__ T red[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? red[threadIdx.x] : T(0);
  if (w == 0) v = warp_sum(v);
  __syncthreads();
  return v;  // valid in thread 0
}

// part[b*PS + j] = sum over chunk j < NB of x[b]*y[b]  (listed problems, or all)
template <typename T>
__global__ void __launch_bounds__(DOT_T)
    k_dot_part(const T* __restrict__ x, const T* __restrict__ y, long long N,
               T* __restrict__ part, const int* __restrict__ list, const int* count, int batch) {
  const int b = active_problem(list, active_count(list, count, batch), batch, blockIdx.y);
  if (b < 0) return;
  const int j = blockIdx.x;
  const long long chunk = (N + NB - 1) / NB;
  const long long lo = j * chunk, hi = min(N, lo + chunk);
  const T* xb = x + (long long)b * N;
  const T* yb = y + (long long)b * N;
  T s = T(0);
  for (long long i = lo + threadIdx.x; i < hi; i += DOT_T) s += xb[i] * yb[i];
  s = block_sum(s);
  if (threadIdx.x == 0) part[b * PS + j] = s;
}

__device__ __forceinline__ float block_max(float v) {
  __shared__ float red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? red[threadIdx.x] : 0.f;
  if (w == 0)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  return v;  // valid in thread 0
}

// slot[b] = max(slot[b], max |x[b]|) (float bits; non-negative floats order
// like unsigned integers), listed problems or all
template <typename T>
__global__ void k_absmax(const T* __restrict__ x, long long N, unsigned* __restrict__ slot,
                         const int* __restrict__ list, const int* count, int batch) {
  const int b = active_problem(list, active_count(list, count, batch), batch, blockIdx.y);
  if (b < 0) return;
  float m = 0.f;
  const T* xb = x + (long long)b * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf((float)xb[i]));
  m = block_max(m);
  if (threadIdx.x == 0) atomicMax(slot + b, __float_as_uint(m));
}

template <typename T>
__device__ __forceinline__ T sum_part(const T* part, int b, int nb) {
  T s = T(0);
#pragma unroll
  for (int j = 0; j < nb; ++j) s += part[b * PS + j];
  return s;
}

template <typename T>
__device__ __forceinline__ bool is_active(T rz, T rz0, double tol) {
  return rz0 > T(0) && rz > T(0) && (double)rz > tol * tol * (double)rz0;
}

// x += alpha p ; r -= alpha q ; alpha = rz / (p.q) while active
// slots (optional, [4][batch]): the scaled split-FP16 apply's max slots of
// this problem are cleared here, after the apply read them and before the
// p update and the next apply's passes record new maxima
template <typename T>
__global__ void k_update_xr(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                            const T* __restrict__ q, long long N, const T* __restrict__ pq_part,
                            const T* __restrict__ rz_prev, const T* __restrict__ rz0,
                            const double* __restrict__ tolp, const int* __restrict__ list,
                            const int* count, int batch, unsigned* __restrict__ slots, int nb_pq,
                            int nb_rz) {
  const int b = active_problem(list, active_count(list, count, batch), batch, blockIdx.y);
  if (b < 0) return;
  const double tol = *tolp;
  const T rz = sum_part(rz_prev, b, nb_rz);
  if (!is_active(rz, rz0[b], tol)) return;
  if (slots && blockIdx.x == 0 && threadIdx.x < 4) slots[(long long)threadIdx.x * batch + b] = 0u;
  const T pq = sum_part(pq_part, b, nb_pq);
  const T alpha = rz / pq;
  const long long off = (long long)b * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    x[off + i] += alpha * p[off + i];
    r[off + i] -= alpha * q[off + i];
  }
}

// p = z + beta p ; beta = rz_new / rz_prev while active; counts iterations
// pmax (optional): max |p| of each problem recorded for the next apply
template <typename T>
__global__ void k_update_p(T* __restrict__ p, const T* __restrict__ z, long long N,
                           const T* __restrict__ rz_new_part, const T* __restrict__ rz_prev_part,
                           const T* __restrict__ rz0, const double* __restrict__ tolp,
                           int* __restrict__ iters, const int* __restrict__ list,
                           const int* count, int batch, unsigned* __restrict__ pmax, int nb_rz) {
  const int b = active_problem(list, active_count(list, count, batch), batch, blockIdx.y);
  if (b < 0) return;
  const double tol = *tolp;
  const T rzp = sum_part(rz_prev_part, b, nb_rz);
  if (!is_active(rzp, rz0[b], tol)) return;
  const T rzn = sum_part(rz_new_part, b, nb_rz);
  const T beta = rzn / rzp;
  const long long off = (long long)b * N;
  float m = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    const T v = z[off + i] + beta * p[off + i];
    p[off + i] = v;
    m = fmaxf(m, fabsf((float)v));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) iters[b] += 1;
  if (pmax) {
    m = block_max(m);
    if (threadIdx.x == 0) atomicMax(pmax + b, __float_as_uint(m));
  }
}

// Active list: keep the problems whose r.z is still above tol^2 r0.z0.  With
// init the candidates are 0..batch-1, else the current list (filtered in
// place: an entry moves only to a lower slot, after its chunk has been read).
// One block; the order of the problems is kept.
constexpr int CMP_T = 256;
template <typename T>
__global__ void __launch_bounds__(CMP_T)
    k_compact(const T* __restrict__ rz_part, const T* __restrict__ rz0,
              const double* __restrict__ tolp, int* __restrict__ list, int* __restrict__ count,
              int batch, int init, int nb_rz) {
  const double tol = *tolp;
  __shared__ int wcnt[CMP_T / 32];
  __shared__ int base;
  const int n = init ? batch : active_count(list, count, batch);
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j0 = 0; j0 < n; j0 += CMP_T) {
    const int j = j0 + threadIdx.x;
    int b = -1;
    if (j < n) b = init ? j : list[j];
    const bool keep =
        b >= 0 && b < batch && is_active(sum_part(rz_part, b, nb_rz), rz0[b], tol);
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wcnt[w] = __popc(m);
    __syncthreads();  // every list[j] of this chunk has been read
    int off = base + __popc(m & ((1u << lane) - 1u));
    for (int i = 0; i < w; ++i) off += wcnt[i];
    if (keep) list[off] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int i = 0; i < CMP_T / 32; ++i) t += wcnt[i];
      base += t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = base;
}

// the convergence tolerance of this solve, read by the (graph-replayed)
// iteration kernels from device memory
__global__ void k_set_tol(double* __restrict__ tolp, double tol) { *tolp = tol; }

template <typename T>
__global__ void k_set_rz0(const T* __restrict__ part, T* __restrict__ rz0, int batch, int nb) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) rz0[b] = sum_part(part, b, nb);
}

// Per problem: if the guess residual is not better than the zero start
// (r.z >= b.M^-1 b), restart from zero: x = 0, r = b, z = M^-1 b.
template <typename T>
__global__ void k_judge_guess(T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                              const T* __restrict__ b, const T* __restrict__ zb, long long N,
                              const T* __restrict__ rz_part, const T* __restrict__ bz_part,
                              int nb) {
  const int bi = blockIdx.y;
  if (sum_part(rz_part, bi, nb) < sum_part(bz_part, bi, nb)) return;
  const long long off = (long long)bi * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    x[off + i] = T(0);
    r[off + i] = b[off + i];
    z[off + i] = zb[off + i];
  }
}

// rz partials of problems that fell back to the zero start become b.M^-1 b
template <typename T>
__global__ void k_fix_rz(T* __restrict__ rz_part, const T* __restrict__ bz_part, int batch,
                         int nb) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  if (bi >= batch) return;
  if (sum_part(rz_part, bi, nb) >= sum_part(bz_part, bi, nb))
    for (int j = 0; j < nb; ++j) rz_part[bi * PS + j] = bz_part[bi * PS + j];
}

// y = a - y  (r = rhs - A x)
template <typename T>
__global__ void k_sub_from(const T* __restrict__ a, T* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = a[i] - y[i];
}

inline int vec_blocks(long long N) {
  long long b = (N + 255) / 256;
  if (b > 64) b = 64;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace

// ---------------------------------------------------------------------------

// ---- cache of instantiated iteration graphs -------------------------------

struct GraphKey {
  std::vector<long long> ints;
  std::vector<const void*> ptrs;
  bool operator==(const GraphKey& o) const { return ints == o.ints && ptrs == o.ptrs; }
};
struct GraphEntry {
  GraphKey key;
  cudaGraphExec_t exec;
  long long kernels;
  unsigned long long used;
};
std::mutex g_graph_mu;
std::vector<GraphEntry> g_graphs;
unsigned long long g_graph_clock = 0;
constexpr size_t GRAPH_CACHE_MAX = 16;

void graph_cache_find(const GraphKey& k, cudaGraphExec_t* exec, long long* kernels) {
  std::lock_guard<std::mutex> lk(g_graph_mu);
  for (GraphEntry& e : g_graphs)
    if (e.key == k) {
      e.used = ++g_graph_clock;
      *exec = e.exec;
      *kernels = e.kernels;
      return;
    }
}

// Keep a new graph; the least recently used one goes when the cache is full
// (its earlier launches are already ordered on their streams).
void graph_cache_put(const GraphKey& k, cudaGraphExec_t exec, long long kernels) {
  std::lock_guard<std::mutex> lk(g_graph_mu);
  if (g_graphs.size() >= GRAPH_CACHE_MAX) {
    size_t lru = 0;
    for (size_t i = 1; i < g_graphs.size(); ++i)
      if (g_graphs[i].used < g_graphs[lru].used) lru = i;
    cudaGraphExecDestroy(g_graphs[lru].exec);
    g_graphs.erase(g_graphs.begin() + lru);
  }
  g_graphs.push_back(GraphEntry{k, exec, kernels, ++g_graph_clock});
}

template <typename T>
size_t pcg_ws(int ndim, int n, int nq, int batch) {
  long long N = 1;
  for (int i = 0; i < ndim; ++i) N *= n;
  const size_t vec = align_up((size_t)N * batch * sizeof(T), 256);
  const size_t scal = align_up((size_t)batch * PS * sizeof(T), 256);
  const size_t small = align_up((size_t)batch * sizeof(T), 256) +
                       2 * align_up((size_t)batch * sizeof(int), 256) + 256 +
                       align_up((size_t)4 * batch * sizeof(unsigned), 256);
  size_t inner = varcoef_ws(ndim, n, nq, batch, sizeof(T));
  const size_t f = fd_ws(ndim, n, batch, sizeof(T));
  if (f > inner) inner = f;
  return 4 * vec + 3 * scal + small + inner;
}

template size_t pcg_ws<double>(int, int, int, int);
template size_t pcg_ws<float>(int, int, int, int);

template <typename T>
int pcg_run(const PcgProblem<T>& pb, T* x, int use_x0, double tol, int maxiter, int* iters_host,
            void* work, size_t work_bytes, cudaStream_t st) {
  const int ndim = pb.ndim, n = pb.n, nq = pb.nq, batch = pb.batch;
  if ((ndim != 2 && ndim != 3) || n < 1 || nq < n || batch < 1 || !pb.rhs || !x ||
      !(tol > 0.0) || maxiter < 0)
    return JFG_ERR_ARG;
  const size_t need = pcg_ws<T>(ndim, n, nq, batch);
  if (!work || work_bytes < need) return JFG_ERR_WORKSPACE;
  long long N = 1;
  for (int i = 0; i < ndim; ++i) N *= n;
  const size_t vec = align_up((size_t)N * batch * sizeof(T), 256);
  const size_t scal = align_up((size_t)batch * PS * sizeof(T), 256);
  char* w = (char*)work;
  T* r = (T*)w;
  T* z = (T*)(w + vec);
  T* p = (T*)(w + 2 * vec);
  T* q = (T*)(w + 3 * vec);
  T* pq_part = (T*)(w + 4 * vec);
  T* rz_part[2] = {(T*)(w + 4 * vec + scal), (T*)(w + 4 * vec + 2 * scal)};
  char* sm = w + 4 * vec + 3 * scal;
  T* rz0 = (T*)sm;
  int* iters = (int*)(sm + align_up((size_t)batch * sizeof(T), 256));
  int* alist = (int*)(sm + align_up((size_t)batch * sizeof(T), 256) +
                      align_up((size_t)batch * sizeof(int), 256));
  int* nactive = (int*)((char*)alist + align_up((size_t)batch * sizeof(int), 256));
  double* tol_dev = (double*)((char*)nactive + 8);  // inside nactive's 256-byte block
  unsigned* slots = (unsigned*)((char*)nactive + 256);
  void* inner = (char*)slots + align_up((size_t)4 * batch * sizeof(unsigned), 256);
  const size_t inner_bytes = work_bytes - (size_t)((char*)inner - w);

  const Active all, act{alist, nactive};
  const bool th = pb.engine == Engine::TH;
  if (th && (ndim != 2 || !pb.ops_inv)) return JFG_ERR_ARG;
  H16Ops h16;
  h16.op_inv = pb.ops_inv;
  h16.slots = th ? slots : nullptr;
  unsigned* slot_p = th ? slots : nullptr;
  // Fused dots (FP32 tensor-core engines): p.Ap from the operator's field
  // pass and r.M^-1 r from the preconditioner's divide pass; each launch
  // reports its partial count (0: not fused, then explicit dot kernels).
  const bool fuse_pq = std::is_same<T, float>::value && pb.engine != Engine::F32 &&
                       ndim == 2 && (pb.fuse_dots & 1);
  const bool fuse = std::is_same<T, float>::value && pb.m_engine != Engine::F32 &&
                    (pb.fuse_dots & 2);
  int nb_pq = NB, nb_rz = NB;
  auto applyA = [&](const T* in, T* out, Active a, DotOut* dot = nullptr) -> int {
    return varcoef_apply<T>(pb.engine, ndim, n, nq, batch, pb.ops, pb.kw, in, out, inner,
                            inner_bytes, st, a, th ? &h16 : nullptr, dot);
  };
  // TH: clear the max slots and record max |v| of every problem in slot 0
  // (the input of the next apply)
  auto record_max = [&](const T* v) -> int {
    if (!th) return JFG_OK;
    JFG_CUDA_TRY(cudaMemsetAsync(slots, 0, sizeof(unsigned) * 4 * batch, st));
    k_absmax<T><<<dim3(vec_blocks(N), batch), 256, 0, st>>>(v, N, slots, nullptr, nullptr,
                                                            batch);
    JFG_LAUNCHED();
    return JFG_OK;
  };
  auto applyM = [&](const T* in, T* out, Active a, DotOut* dot = nullptr) -> int {
    return fd_solve<T>(pb.m_engine, ndim, n, batch, pb.E, pb.W, pb.lam, nullptr, pb.fd_scale, in,
                       out, inner, inner_bytes, st, a, dot);
  };
  // out . M^-1 in into part: fused into the preconditioner when possible
  auto applyM_dot = [&](const T* in, T* out, Active a, T* part, int& nb) -> int {
    int got = 0;
    DotOut d;
    d.part = fuse ? (float*)part : nullptr;
    d.nb = &got;
    JFG_TRY(applyM(in, out, a, fuse ? &d : nullptr));
    if (got > 0) {
      nb = got;
      return JFG_OK;
    }
    nb = NB;
    k_dot_part<T><<<dim3(NB, batch), DOT_T, 0, st>>>(in, out, N, part, a.list, a.count, batch);
    JFG_LAUNCHED();
    return JFG_OK;
  };

  const int vb = vec_blocks(N);
  const dim3 vgrid(vb, batch);
  const dim3 dgrid(NB, batch);
  const long long total = N * batch;

  // ---- setup: r = rhs - A x (or x = 0, r = rhs); z = M^-1 r; p = z
  JFG_CUDA_TRY(cudaMemsetAsync(iters, 0, sizeof(int) * batch, st));
  if (use_x0) {
    JFG_TRY(record_max(x));
    JFG_TRY(applyA(x, r, all));
    k_sub_from<T><<<vec_blocks(total), 256, 0, st>>>(pb.rhs, r, total);
    JFG_LAUNCHED();
  } else {
    JFG_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(T) * total, st));
    JFG_CUDA_TRY(cudaMemcpyAsync(r, pb.rhs, sizeof(T) * total, cudaMemcpyDeviceToDevice, st));
  }
  JFG_TRY(applyM_dot(r, z, all, rz_part[1], nb_rz));
  if (use_x0 && pb.judge_x0) {
    // Judge the initial guess against the zero start: keep it only where its
    // preconditioned residual is smaller than that of the right-hand side,
    // and measure convergence relative to the right-hand side either way.
    int nb_bz = NB;
    JFG_TRY(applyM_dot(pb.rhs, q, all, pq_part, nb_bz));
    if (nb_bz != nb_rz) return JFG_ERR_UNSUPPORTED;  // same launch signature: cannot differ
    k_judge_guess<T><<<vgrid, 256, 0, st>>>(x, r, z, pb.rhs, q, N, rz_part[1], pq_part, nb_rz);
    JFG_LAUNCHED();
    k_set_rz0<T><<<(batch + 127) / 128, 128, 0, st>>>(pq_part, rz0, batch, nb_rz);
    JFG_LAUNCHED();
    k_fix_rz<T><<<(batch + 127) / 128, 128, 0, st>>>(rz_part[1], pq_part, batch, nb_rz);
    JFG_LAUNCHED();
  } else {
    k_set_rz0<T><<<(batch + 127) / 128, 128, 0, st>>>(rz_part[1], rz0, batch, nb_rz);
    JFG_LAUNCHED();
  }
  JFG_CUDA_TRY(cudaMemcpyAsync(p, z, sizeof(T) * total, cudaMemcpyDeviceToDevice, st));
  JFG_TRY(record_max(p));
  // the problems that start active (r0.z0 > 0)
  k_set_tol<<<1, 1, 0, st>>>(tol_dev, tol);
  JFG_LAUNCHED();
  k_compact<T><<<1, CMP_T, 0, st>>>(rz_part[1], rz0, tol_dev, alist, nactive, batch, 1, nb_rz);
  JFG_LAUNCHED();

  auto iteration = [&](int it) -> int {
    const int prev = (it + 1) & 1, cur = it & 1;
    {
      int got = 0;
      DotOut d;
      d.part = fuse_pq ? (float*)pq_part : nullptr;
      d.nb = &got;
      JFG_TRY(applyA(p, q, act, fuse_pq ? &d : nullptr));
      if (got > 0) {
        nb_pq = got;
      } else {
        nb_pq = NB;
        k_dot_part<T><<<dgrid, DOT_T, 0, st>>>(p, q, N, pq_part, alist, nactive, batch);
        JFG_LAUNCHED();
      }
    }
    k_update_xr<T><<<vgrid, 256, 0, st>>>(x, r, p, q, N, pq_part, rz_part[prev], rz0, tol_dev,
                                          alist, nactive, batch, slot_p, nb_pq, nb_rz);
    JFG_LAUNCHED();
    int nb_new = NB;
    JFG_TRY(applyM_dot(r, z, act, rz_part[cur], nb_new));
    if (nb_new != nb_rz) return JFG_ERR_UNSUPPORTED;  // same launch signature: cannot differ
    k_update_p<T><<<vgrid, 256, 0, st>>>(p, z, N, rz_part[cur], rz_part[prev], rz0, tol_dev,
                                         iters, alist, nactive, batch, slot_p, nb_rz);
    JFG_LAUNCHED();
    k_compact<T><<<1, CMP_T, 0, st>>>(rz_part[cur], rz0, tol_dev, alist, nactive, batch, 0,
                                      nb_rz);
    JFG_LAUNCHED();
    return JFG_OK;
  };

  // ---- iterate in chunks of CH iterations (CH even: the partial-sum
  // ping-pong then lines up with the captured graph)
  const int CH = 10;
  const bool use_graph = (st != 0) && (maxiter >= CH);
  cudaGraphExec_t exec = nullptr;
  long long graph_kernels = 0;
  // The chunk of CH iterations depends only on the buffers, operators, sizes
  // and engines (the tolerance is read from device memory), so its
  // instantiated graph is kept and replayed by later calls with the same key.
  GraphKey key;
  if (use_graph) {
    int dev = 0;
    JFG_CUDA_TRY(cudaGetDevice(&dev));
    const long long v[] = {dev, (long long)sizeof(T), (long long)pb.engine,
                           (long long)pb.m_engine, ndim, n, nq, batch, pb.fuse_dots, nb_rz,
                           (long long)work_bytes};
    const void* ptrs[] = {x, work, pb.ops.hi, pb.ops.lo, pb.ops_inv, pb.kw, pb.E.hi, pb.E.lo,
                          pb.W.hi, pb.W.lo, pb.lam, pb.fd_scale};
    key.ints.assign(v, v + sizeof(v) / sizeof(v[0]));
    key.ptrs.assign(ptrs, ptrs + sizeof(ptrs) / sizeof(ptrs[0]));
    graph_cache_find(key, &exec, &graph_kernels);
  }
  if (use_graph && !exec) {
    cudaGraph_t graph = nullptr;
    JFG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    set_capturing(true);
    int s = JFG_OK;
    for (int i = 0; i < CH && s == JFG_OK; ++i) s = iteration(i);
    set_capturing(false);
    cudaError_t ec = cudaStreamEndCapture(st, &graph);
    if (s != JFG_OK) {
      if (graph) cudaGraphDestroy(graph);
      return s;
    }
    JFG_CUDA_TRY(ec);
    size_t nn = 0;
    cudaGraphGetNodes(graph, nullptr, &nn);
    if (nn > 0) {
      cudaGraphNode_t nodes[4096];
      if (nn > 4096) nn = 4096;
      cudaGraphGetNodes(graph, nodes, &nn);
      for (size_t i = 0; i < nn; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
          ++graph_kernels;
      }
    }
    cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    JFG_CUDA_TRY(ei);
    graph_cache_put(key, exec, graph_kernels);
  }
  int done_iters = 0;
  int status = JFG_OK;
  int h_active = 1;
  while (done_iters < maxiter) {
    if (use_graph && maxiter - done_iters >= CH) {
      cudaError_t e = cudaGraphLaunch(exec, st);
      if (e != cudaSuccess) {
        set_last_cuda_error(e);
        status = JFG_ERR_CUDA;
        break;
      }
      count_launches(graph_kernels);
      done_iters += CH;
    } else {
      const int todo = (maxiter - done_iters < CH) ? maxiter - done_iters : CH;
      for (int i = 0; i < todo && status == JFG_OK; ++i)
        status = iteration(done_iters + i);
      if (status != JFG_OK) break;
      done_iters += todo;
    }
    cudaError_t e = cudaMemcpyAsync(&h_active, nactive, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_last_cuda_error(e);
      status = JFG_ERR_CUDA;
      break;
    }
    if (h_active == 0) break;
  }
  if (status != JFG_OK) return status;
  if (iters_host) {
    JFG_CUDA_TRY(cudaMemcpyAsync(iters_host, iters, sizeof(int) * batch,
                                 cudaMemcpyDeviceToHost, st));
    JFG_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return h_active == 0 ? JFG_OK : JFG_ERR_NOT_CONVERGED;
}

template int pcg_run<double>(const PcgProblem<double>&, double*, int, double, int, int*, void*,
                             size_t, cudaStream_t);
template int pcg_run<float>(const PcgProblem<float>&, float*, int, double, int, int*, void*,
                            size_t, cudaStream_t);

}  // namespace jfg

extern "C" size_t jfg_pcg_workspace_size(int ndim, int n, int nq, int batch, int elem_bytes) {
  if (elem_bytes == 8) return jfg::pcg_ws<double>(ndim, n, nq, batch);
  return jfg::pcg_ws<float>(ndim, n, nq, batch);
}

extern "C" int jfg_pcg_varcoef_f64(int ndim, int n, int nq, int batch, const double* ops,
                                   const double* kw, const double* E, const double* W,
                                   const double* lam, const double* fd_scale, const double* rhs,
                                   double* x, int use_x0, double tol, int maxiter, int* iters,
                                   void* work, size_t work_bytes, void* stream) {
  if (!ops || !kw || !E || !W || !lam) return JFG_ERR_ARG;
  jfg::PcgProblem<double> pb;
  pb.engine = jfg::Engine::F64;
  pb.m_engine = jfg::Engine::F64;
  pb.ndim = ndim;
  pb.n = n;
  pb.nq = nq;
  pb.batch = batch;
  pb.ops = jfg::OpRef<double>{ops, nullptr};
  pb.kw = kw;
  pb.E = jfg::OpRef<double>{E, nullptr};
  pb.W = jfg::OpRef<double>{W, nullptr};
  pb.lam = lam;
  pb.fd_scale = fd_scale;
  pb.rhs = rhs;
  return jfg::pcg_run<double>(pb, x, use_x0, tol, maxiter, iters, work, work_bytes,
                              (cudaStream_t)stream);
}
