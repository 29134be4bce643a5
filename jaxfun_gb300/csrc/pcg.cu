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

// 16-byte vectors of T for the per-iteration updates
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int n = 4;
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int n = 2;
};
template <typename V>
__device__ __forceinline__ float vabsmax(const V& v);
template <>
__device__ __forceinline__ float vabsmax(const float4& v) {
  return fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w)));
}
template <>
__device__ __forceinline__ float vabsmax(const double2& v) {
  return fmaxf(fabsf((float)v.x), fabsf((float)v.y));
}
__device__ __forceinline__ float4 vaxpy(float a, const float4& x, const float4& y) {
  return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}
__device__ __forceinline__ double2 vaxpy(double a, const double2& x, const double2& y) {
  return make_double2(fma(a, x.x, y.x), fma(a, x.y, y.y));
}

__device__ __forceinline__ bool al16(const void* ptr) {
  return ((uintptr_t)ptr & 15u) == 0;
}

// The per-problem scalars of an update are computed once per block (thread
// 0, the same partial-sum order everywhere) and shared: every thread doing
// them cost more than the vector traffic (the FP64 tolerance test alone).
// Vector part: 16-byte accesses when N is a multiple of the vector width,
// else element by element.

// r -= alpha q ; alpha = rz / (p.q) while active (x takes its alpha p in
// k_update_xp, which reads p anyway)
// slots (optional, [H16_SLOTS][batch]): the scaled split-FP16 apply's max slots of
// this problem are cleared here, after the apply read them and before the
// p update and the next apply's passes record new maxima
template <typename T>
__global__ void k_update_r(T* __restrict__ r, const T* __restrict__ q, long long N,
                           const T* __restrict__ pq_part, const T* __restrict__ rz_prev,
                           const T* __restrict__ rz0, const double* __restrict__ tolp,
                           const int* __restrict__ list, const int* count, int batch,
                           unsigned* __restrict__ slots, int nb_pq, int nb_rz) {
  __shared__ T s_alpha;
  __shared__ int s_act;
  const int b = active_problem(list, active_count(list, count, batch), batch, blockIdx.y);
  if (b < 0) return;
  if (threadIdx.x == 0) {
    const T rz = sum_part(rz_prev, b, nb_rz);
    s_act = is_active(rz, rz0[b], tolp[b]) ? 1 : 0;
    s_alpha = s_act ? rz / sum_part(pq_part, b, nb_pq) : T(0);
    if (s_act && slots && blockIdx.x == 0)
      for (int k = 0; k < H16_SLOTS; ++k) slots[(long long)k * batch + b] = 0u;
  }
  __syncthreads();
  if (!s_act) return;
  const T alpha = -s_alpha;
  const long long off = (long long)b * N;
  using V = typename Vec16<T>::type;
  constexpr int VN = Vec16<T>::n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (N % VN == 0 && al16(r + off) && al16(q + off)) {
    V* rv = reinterpret_cast<V*>(r + off);
    const V* qv = reinterpret_cast<const V*>(q + off);
    for (long long i = t0; i < N / VN; i += stride) rv[i] = vaxpy(alpha, qv[i], rv[i]);
  } else {
    for (long long i = t0; i < N; i += stride) r[off + i] = fma(alpha, q[off + i], r[off + i]);
  }
}

// x += alpha p ; p = z + beta p ; alpha = rz_prev / (p.q), beta = rz_new /
// rz_prev while active; counts iterations.  pmax (optional): max |p| of each
// problem recorded for the next apply
template <typename T>
__global__ void k_update_xp(T* __restrict__ x, T* __restrict__ p, const T* __restrict__ z,
                            long long N, const T* __restrict__ pq_part,
                            const T* __restrict__ rz_new_part, const T* __restrict__ rz_prev_part,
                            const T* __restrict__ rz0, const double* __restrict__ tolp,
                            int* __restrict__ iters, const int* __restrict__ list,
                            const int* count, int batch, unsigned* __restrict__ pmax, int nb_pq,
                            int nb_rz, int* __restrict__ inner_it, int maxit,
                            int* __restrict__ keep) {
  __shared__ T s_alpha, s_beta;
  __shared__ int s_act;
  const int b = active_problem(list, active_count(list, count, batch), batch, blockIdx.y);
  if (b < 0) return;
  if (threadIdx.x == 0) {
    const T rzp = sum_part(rz_prev_part, b, nb_rz);
    s_act = is_active(rzp, rz0[b], tolp[b]) ? 1 : 0;
    int kp = 0;
    if (s_act) {
      const T rzn = sum_part(rz_new_part, b, nb_rz);
      s_alpha = rzp / sum_part(pq_part, b, nb_pq);
      s_beta = rzn / rzp;
      // whether the problem stays in the active list (read by k_compact)
      kp = is_active(rzn, rz0[b], tolp[b]) ? 1 : 0;
      if (blockIdx.x == 0) {
        iters[b] += 1;
        if (inner_it) {
          const int it = inner_it[b] + 1;
          inner_it[b] = it;
          if (maxit > 0 && it >= maxit) kp = 0;
        }
      }
    }
    if (blockIdx.x == 0) keep[b] = kp;
  }
  __syncthreads();
  if (!s_act) return;
  const T alpha = s_alpha, beta = s_beta;
  const long long off = (long long)b * N;
  using V = typename Vec16<T>::type;
  constexpr int VN = Vec16<T>::n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float m = 0.f;
  if (N % VN == 0 && al16(x + off) && al16(p + off) && al16(z + off)) {
    V* xv = reinterpret_cast<V*>(x + off);
    V* pv = reinterpret_cast<V*>(p + off);
    const V* zv = reinterpret_cast<const V*>(z + off);
    for (long long i = t0; i < N / VN; i += stride) {
      const V po = pv[i];
      xv[i] = vaxpy(alpha, po, xv[i]);
      const V pn = vaxpy(beta, po, zv[i]);
      pv[i] = pn;
      m = fmaxf(m, vabsmax(pn));
    }
  } else {
    for (long long i = t0; i < N; i += stride) {
      const T po = p[off + i];
      x[off + i] = fma(alpha, po, x[off + i]);
      const T v = fma(beta, po, z[off + i]);
      p[off + i] = v;
      m = fmaxf(m, fabsf((float)v));
    }
  }
  if (pmax) {
    m = block_max(m);
    if (threadIdx.x == 0) atomicMax(pmax + b, __float_as_uint(m));
  }
}

// Active list: keep the problems k_update_xp flagged (r.z still above
// tol_b^2 r0.z0 and, with an iteration cap, fewer than maxit iterations since
// their start).  The list is filtered in place: an entry moves only to a lower
// slot, after its chunk has been read.  ready (optional): the problems dropped
// here are appended to ready[*nready] (their inner solve is over).  One block;
// the order of the problems is kept.
constexpr int CMP_T = 256;
__global__ void __launch_bounds__(CMP_T)
    k_compact(const int* __restrict__ keep, int* __restrict__ list, int* __restrict__ count,
              int batch, int* __restrict__ ready, int* __restrict__ nready) {
  __shared__ int wcnt[CMP_T / 32], wdrop[CMP_T / 32];
  __shared__ int base, dbase;
  const int n = active_count(list, count, batch);
  if (threadIdx.x == 0) {
    base = 0;
    dbase = ready ? *nready : 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j0 = 0; j0 < n; j0 += CMP_T) {
    const int j = j0 + threadIdx.x;
    int b = -1;
    if (j < n) b = list[j];
    const bool valid = b >= 0 && b < batch;
    const bool kp = valid && keep[b] != 0;
    const bool drop = valid && !kp && ready != nullptr;
    const unsigned m = __ballot_sync(0xffffffffu, kp);
    const unsigned md = __ballot_sync(0xffffffffu, drop);
    if (lane == 0) {
      wcnt[w] = __popc(m);
      wdrop[w] = __popc(md);
    }
    __syncthreads();  // every list[j] of this chunk has been read
    int off = base + __popc(m & ((1u << lane) - 1u));
    int doff = dbase + __popc(md & ((1u << lane) - 1u));
    for (int i = 0; i < w; ++i) {
      off += wcnt[i];
      doff += wdrop[i];
    }
    if (kp) list[off] = b;
    if (drop) ready[doff] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0, td = 0;
      for (int i = 0; i < CMP_T / 32; ++i) {
        t += wcnt[i];
        td += wdrop[i];
      }
      base += t;
      dbase += td;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *count = base;
    if (ready) *nready = dbase;
  }
}

// the convergence tolerance of every problem, read by the (graph-replayed)
// iteration kernels from device memory
__global__ void k_set_tol(double* __restrict__ tolp, double tol, int batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) tolp[b] = tol;
}

// ---- restarts of listed problems (the flat mixed-precision schedule) ----

// x = 0 (unless keep_x), r = rhs for the listed problems
template <typename T>
__global__ void k_restart_vec(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ rhs,
                              long long N, int keep_x, const int* __restrict__ list,
                              const int* count, int batch) {
  const int b = active_problem(list, active_count(list, count, batch), batch, blockIdx.y);
  if (b < 0) return;
  const long long off = (long long)b * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    if (!keep_x) x[off + i] = T(0);
    r[off + i] = rhs[off + i];
  }
}

// y = a - y for the listed problems
template <typename T>
__global__ void k_sub_from_list(const T* __restrict__ a, T* __restrict__ y, long long N,
                                const int* __restrict__ list, const int* count, int batch) {
  const int b = active_problem(list, active_count(list, count, batch), batch, blockIdx.y);
  if (b < 0) return;
  const long long off = (long long)b * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x)
    y[off + i] = a[off + i] - y[off + i];
}

// dst = src for the listed problems
template <typename T>
__global__ void k_copy_list(T* __restrict__ dst, const T* __restrict__ src, long long N,
                            const int* __restrict__ list, const int* count, int batch) {
  const int b = active_problem(list, active_count(list, count, batch), batch, blockIdx.y);
  if (b < 0) return;
  const long long off = (long long)b * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x)
    dst[off + i] = src[off + i];
}

// per listed problem: clear its four max slots and its iteration count since
// the start (one thread each)
__global__ void k_restart_scalars(unsigned* __restrict__ slots, int* __restrict__ inner_it,
                                  const int* __restrict__ list, const int* count, int batch) {
  const int n = active_count(list, count, batch);
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int b = list ? list[j] : j;
    if (b < 0 || b >= batch) continue;
    if (slots)
      for (int k = 0; k < H16_SLOTS; ++k) slots[(long long)k * batch + b] = 0u;
    if (inner_it) inner_it[b] = 0;
  }
}

// Append the listed problems whose r.z is above tol_b^2 r0.z0 to the active
// list, the others to the ready list (one block; order kept).
template <typename T>
__global__ void __launch_bounds__(CMP_T)
    k_append_active(const T* __restrict__ rz_part, const T* __restrict__ rz0,
                    const double* __restrict__ tolp, int nb_rz, const int* __restrict__ list,
                    const int* count, int batch, int* __restrict__ alist,
                    int* __restrict__ nactive, int* __restrict__ ready,
                    int* __restrict__ nready) {
  __shared__ int wcnt[CMP_T / 32], wdrop[CMP_T / 32];
  __shared__ int base, dbase;
  const int n = active_count(list, count, batch);
  if (threadIdx.x == 0) {
    base = *nactive;
    dbase = ready ? *nready : 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j0 = 0; j0 < n; j0 += CMP_T) {
    const int j = j0 + threadIdx.x;
    const int b = j < n ? (list ? list[j] : j) : -1;
    const bool valid = b >= 0 && b < batch;
    const bool keep = valid && is_active(sum_part(rz_part, b, nb_rz), rz0[b], tolp[b]);
    const bool drop = valid && !keep && ready != nullptr;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const unsigned md = __ballot_sync(0xffffffffu, drop);
    if (lane == 0) {
      wcnt[w] = __popc(m);
      wdrop[w] = __popc(md);
    }
    __syncthreads();
    int off = base + __popc(m & ((1u << lane) - 1u));
    int doff = dbase + __popc(md & ((1u << lane) - 1u));
    for (int i = 0; i < w; ++i) {
      off += wcnt[i];
      doff += wdrop[i];
    }
    if (keep) alist[off] = b;
    if (drop) ready[doff] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int i = 0; i < CMP_T / 32; ++i) {
        base += wcnt[i];
        dbase += wdrop[i];
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *nactive = base;
    if (ready) *nready = dbase;
  }
}

template <typename T>
__global__ void k_set_rz0(const T* __restrict__ part, T* __restrict__ rz0, int batch, int nb,
                          const int* __restrict__ list = nullptr, const int* count = nullptr) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = active_problem(list, active_count(list, count, batch), batch, j);
  if (b >= 0) rz0[b] = sum_part(part, b, nb);
}

// Per problem: if the guess residual is not better than the zero start
// (r.z >= b.M^-1 b), restart from zero: x = 0, r = b, z = M^-1 b.
template <typename T>
__global__ void k_judge_guess(T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                              const T* __restrict__ b, const T* __restrict__ zb, long long N,
                              const T* __restrict__ rz_part, const T* __restrict__ bz_part,
                              int nb, const int* __restrict__ list = nullptr,
                              const int* count = nullptr, int batch = 0) {
  const int bi = list ? active_problem(list, active_count(list, count, batch), batch, blockIdx.y)
                      : (int)blockIdx.y;
  if (bi < 0) return;
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
                         int nb, const int* __restrict__ list = nullptr,
                         const int* count = nullptr) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int bi = active_problem(list, active_count(list, count, batch), batch, j);
  if (bi < 0) return;
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

// blocks per problem of the per-iteration updates: ~16 vector elements per
// thread
inline int upd_blocks(long long N) {
  long long b = (N + 256 * 16 - 1) / (256 * 16);
  if (b > 64) b = 64;
  return (int)(b < 1 ? 1 : b);
}

inline int vec_blocks(long long N) {
  long long b = (N + 255) / 256;
  if (b > 64) b = 64;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace

// ---------------------------------------------------------------------------

// ---- cache of instantiated iteration graphs -------------------------------

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
                       5 * align_up((size_t)batch * sizeof(int), 256) + 256 +
                       align_up((size_t)batch * sizeof(double), 256) +
                       align_up((size_t)H16_SLOTS * batch * sizeof(unsigned), 256);
  size_t inner = varcoef_ws(ndim, n, nq, batch, sizeof(T));
  const size_t f = fd_ws(ndim, n, batch, sizeof(T));
  if (f > inner) inner = f;
  return 4 * vec + 3 * scal + small + inner;
}

template size_t pcg_ws<double>(int, int, int, int);
template size_t pcg_ws<float>(int, int, int, int);

// ---- the batched PCG context -----------------------------------------------

template <typename T>
int PcgCtx<T>::init(const PcgProblem<T>& problem, T* x_, void* work, size_t work_bytes,
                    cudaStream_t stream) {
  pb = problem;
  st = stream;
  x = x_;
  ndim = pb.ndim;
  n = pb.n;
  nq = pb.nq;
  batch = pb.batch;
  if ((ndim != 2 && ndim != 3) || n < 1 || nq < n || batch < 1 || !pb.rhs || !x)
    return JFG_ERR_ARG;
  const size_t need = pcg_ws<T>(ndim, n, nq, batch);
  if (!work || work_bytes < need) return JFG_ERR_WORKSPACE;
  N = 1;
  for (int i = 0; i < ndim; ++i) N *= n;
  const size_t vec = align_up((size_t)N * batch * sizeof(T), 256);
  const size_t scal = align_up((size_t)batch * PS * sizeof(T), 256);
  const size_t ib = align_up((size_t)batch * sizeof(int), 256);
  char* w = (char*)work;
  r = (T*)w;
  z = (T*)(w + vec);
  p = (T*)(w + 2 * vec);
  q = (T*)(w + 3 * vec);
  pq_part = (T*)(w + 4 * vec);
  rz_part[0] = (T*)(w + 4 * vec + scal);
  rz_part[1] = (T*)(w + 4 * vec + 2 * scal);
  char* sm = w + 4 * vec + 3 * scal;
  rz0 = (T*)sm;
  sm += align_up((size_t)batch * sizeof(T), 256);
  iters = (int*)sm;
  sm += ib;
  alist = (int*)sm;
  sm += ib;
  nactive = (int*)sm;  // the control block: active count, then ready count
  nready = nactive + 1;
  sm += 256;
  tolv = (double*)sm;
  sm += align_up((size_t)batch * sizeof(double), 256);
  inner_it = (int*)sm;
  sm += ib;
  ready = (int*)sm;
  sm += ib;
  keep = (int*)sm;
  sm += ib;
  slots = (unsigned*)sm;
  sm += align_up((size_t)H16_SLOTS * batch * sizeof(unsigned), 256);
  inner = sm;
  inner_bytes = work_bytes - (size_t)(sm - w);
  work_ptr = work;
  work_size = work_bytes;
  th = pb.engine == Engine::TH;
  if (th && !pb.ops_inv) return JFG_ERR_ARG;
  h16.op_inv = pb.ops_inv;
  h16.slots = th ? slots : nullptr;
  // Fused dots (FP32 tensor-core engines): p.Ap from the operator's field
  // pass and r.M^-1 r from the preconditioner's divide pass; each launch
  // reports its partial count (0: not fused, then explicit dot kernels).
  fuse_pq = std::is_same<T, float>::value && pb.engine != Engine::F32 && ndim == 2 &&
            (pb.fuse_dots & 1);
  fuse_rz = std::is_same<T, float>::value && pb.m_engine != Engine::F32 && (pb.fuse_dots & 2);
  nb_pq = NB;
  nb_rz = NB;
  vb = vec_blocks(N);
  JFG_CUDA_TRY(cudaMemsetAsync(nactive, 0, 2 * sizeof(int), st));
  JFG_CUDA_TRY(cudaMemsetAsync(iters, 0, sizeof(int) * batch, st));
  return JFG_OK;
}

template <typename T>
int PcgCtx<T>::applyA(const T* in, T* out, Active a, DotOut* dot) {
  return varcoef_apply<T>(pb.engine, ndim, n, nq, batch, pb.ops, pb.kw, in, out, inner,
                          inner_bytes, st, a, th ? &h16 : nullptr, dot);
}

template <typename T>
int PcgCtx<T>::applyM(const T* in, T* out, Active a, DotOut* dot) {
  return fd_solve<T>(pb.m_engine, ndim, n, batch, pb.E, pb.W, pb.lam, nullptr, pb.fd_scale, in,
                     out, inner, inner_bytes, st, a, dot);
}

// out . M^-1 in into part: fused into the preconditioner when possible
template <typename T>
int PcgCtx<T>::applyM_dot(const T* in, T* out, Active a, T* part, int& nb) {
  int got = 0;
  DotOut d;
  d.part = fuse_rz ? (float*)part : nullptr;
  d.nb = &got;
  JFG_TRY(applyM(in, out, a, fuse_rz ? &d : nullptr));
  if (got > 0) {
    nb = got;
    return JFG_OK;
  }
  nb = NB;
  k_dot_part<T><<<dim3(NB, batch), DOT_T, 0, st>>>(in, out, N, part, a.list, a.count, batch);
  JFG_LAUNCHED();
  return JFG_OK;
}

// TH: clear the listed problems' max slots and record max |v| in slot 0 (the
// input of the next apply)
template <typename T>
int PcgCtx<T>::record_max(const T* v, Active a) {
  if (!th) return JFG_OK;
  k_restart_scalars<<<(batch + 255) / 256, 256, 0, st>>>(slots, nullptr, a.list, a.count, batch);
  JFG_LAUNCHED();
  k_absmax<T><<<dim3(vb, batch), 256, 0, st>>>(v, N, slots, a.list, a.count, batch);
  JFG_LAUNCHED();
  return JFG_OK;
}

template <typename T>
int PcgCtx<T>::start(const int* list, const int* count, int use_x0, bool judge) {
  const Active a{list, count};
  const dim3 vgrid(vb, batch);
  // r = rhs - A x (or x = 0, r = rhs); z = M^-1 r; p = z
  k_restart_vec<T><<<vgrid, 256, 0, st>>>(x, r, pb.rhs, N, use_x0, list, count, batch);
  JFG_LAUNCHED();
  k_restart_scalars<<<(batch + 255) / 256, 256, 0, st>>>(nullptr, inner_it, list, count, batch);
  JFG_LAUNCHED();
  if (use_x0) {
    JFG_TRY(record_max(x, a));
    JFG_TRY(applyA(x, r, a));
    k_sub_from_list<T><<<vgrid, 256, 0, st>>>(pb.rhs, r, N, list, count, batch);
    JFG_LAUNCHED();
  }
  JFG_TRY(applyM_dot(r, z, a, rz_part[1], nb_rz));
  const int sb = (batch + 127) / 128;
  if (use_x0 && judge) {
    // Judge the initial guess against the zero start: keep it only where its
    // preconditioned residual is smaller than that of the right-hand side,
    // and measure convergence relative to the right-hand side either way.
    int nb_bz = NB;
    JFG_TRY(applyM_dot(pb.rhs, q, a, pq_part, nb_bz));
    if (nb_bz != nb_rz) return JFG_ERR_UNSUPPORTED;  // same launch signature: cannot differ
    k_judge_guess<T><<<vgrid, 256, 0, st>>>(x, r, z, pb.rhs, q, N, rz_part[1], pq_part, nb_rz,
                                            list, count, batch);
    JFG_LAUNCHED();
    k_set_rz0<T><<<sb, 128, 0, st>>>(pq_part, rz0, batch, nb_rz, list, count);
    JFG_LAUNCHED();
    k_fix_rz<T><<<sb, 128, 0, st>>>(rz_part[1], pq_part, batch, nb_rz, list, count);
    JFG_LAUNCHED();
  } else {
    k_set_rz0<T><<<sb, 128, 0, st>>>(rz_part[1], rz0, batch, nb_rz, list, count);
    JFG_LAUNCHED();
  }
  k_copy_list<T><<<vgrid, 256, 0, st>>>(p, z, N, list, count, batch);
  JFG_LAUNCHED();
  JFG_TRY(record_max(p, a));
  // the listed problems that start active (r0.z0 > 0) join the active list;
  // with ready tracking the others are ready at once
  k_append_active<T><<<1, CMP_T, 0, st>>>(rz_part[1], rz0, tolv, nb_rz, list, count, batch,
                                          alist, nactive, track_ready ? ready : nullptr, nready);
  JFG_LAUNCHED();
  return JFG_OK;
}

template <typename T>
int PcgCtx<T>::iteration(int it) {
  const int prev = (it + 1) & 1, cur = it & 1;
  const Active act{alist, nactive};
  const dim3 vgrid(vb, batch);
  unsigned* slot_p = th ? slots : nullptr;
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
      k_dot_part<T><<<dim3(NB, batch), DOT_T, 0, st>>>(p, q, N, pq_part, alist, nactive, batch);
      JFG_LAUNCHED();
    }
  }
  const dim3 ugrid(upd_blocks(N), batch);
  k_update_r<T><<<ugrid, 256, 0, st>>>(r, q, N, pq_part, rz_part[prev], rz0, tolv, alist,
                                       nactive, batch, slot_p, nb_pq, nb_rz);
  JFG_LAUNCHED();
  int nb_new = NB;
  JFG_TRY(applyM_dot(r, z, act, rz_part[cur], nb_new));
  if (nb_new != nb_rz) return JFG_ERR_UNSUPPORTED;  // same launch signature: cannot differ
  k_update_xp<T><<<ugrid, 256, 0, st>>>(x, p, z, N, pq_part, rz_part[cur], rz_part[prev], rz0,
                                        tolv, iters, alist, nactive, batch, slot_p, nb_pq, nb_rz,
                                        inner_it, maxit, keep);
  JFG_LAUNCHED();
  k_compact<<<1, CMP_T, 0, st>>>(keep, alist, nactive, batch, track_ready ? ready : nullptr,
                                 nready);
  JFG_LAUNCHED();
  return JFG_OK;
}

// CH iterations: the cached graph of this context (captured on first use).
// The chunk depends only on the buffers, operators, sizes, engines and the
// per-problem iteration cap (the tolerances are read from device memory).
template <typename T>
int PcgCtx<T>::chunk() {
  if (st == 0) {
    // the legacy default stream cannot be captured: launch the iterations
    for (int i = 0; i < CH; ++i) JFG_TRY(iteration(i));
    return JFG_OK;
  }
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;
  int dev = 0;
  JFG_CUDA_TRY(cudaGetDevice(&dev));
  GraphKey key;
  const long long v[] = {dev, (long long)sizeof(T), (long long)pb.engine, (long long)pb.m_engine,
                         ndim, n, nq, batch, pb.fuse_dots, nb_rz, (long long)work_size, maxit,
                         track_ready ? 1 : 0, CH};
  const void* ptrs[] = {x, work_ptr, pb.ops.hi, pb.ops.lo, pb.ops_inv, pb.kw, pb.E.hi, pb.E.lo,
                        pb.W.hi, pb.W.lo, pb.lam, pb.fd_scale};
  key.ints.assign(v, v + sizeof(v) / sizeof(v[0]));
  key.ptrs.assign(ptrs, ptrs + sizeof(ptrs) / sizeof(ptrs[0]));
  graph_cache_find(key, &exec, &kernels);
  if (!exec) {
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
      std::vector<cudaGraphNode_t> nodes(nn);
      cudaGraphGetNodes(graph, nodes.data(), &nn);
      for (size_t i = 0; i < nn; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
          ++kernels;
      }
    }
    cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    JFG_CUDA_TRY(ei);
    graph_cache_put(key, exec, kernels);
  }
  cudaError_t e = cudaGraphLaunch(exec, st);
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return JFG_ERR_CUDA;
  }
  count_launches(kernels);
  return JFG_OK;
}

template <typename T>
int pcg_run(const PcgProblem<T>& pb, T* x, int use_x0, double tol, int maxiter, int* iters_host,
            void* work, size_t work_bytes, cudaStream_t st) {
  if (!(tol > 0.0) || maxiter < 0) return JFG_ERR_ARG;
  PcgCtx<T> c;
  JFG_TRY(c.init(pb, x, work, work_bytes, st));
  k_set_tol<<<(pb.batch + 127) / 128, 128, 0, st>>>(c.tolv, tol, pb.batch);
  JFG_LAUNCHED();
  JFG_TRY(c.start(nullptr, nullptr, use_x0, pb.judge_x0));
  // iterate in chunks of CH iterations (CH even: the partial-sum ping-pong
  // then lines up with the captured graph); a default stream or fewer than
  // CH iterations left run without the graph
  const bool use_graph = (st != 0) && (maxiter >= PcgCtx<T>::CH);
  int done_iters = 0;
  int status = JFG_OK;
  int h_active = 1;
  while (done_iters < maxiter) {
    if (use_graph && maxiter - done_iters >= PcgCtx<T>::CH) {
      status = c.chunk();
      if (status != JFG_OK) break;
      done_iters += PcgCtx<T>::CH;
    } else {
      const int todo = (maxiter - done_iters < PcgCtx<T>::CH) ? maxiter - done_iters
                                                               : PcgCtx<T>::CH;
      for (int i = 0; i < todo && status == JFG_OK; ++i) status = c.iteration(done_iters + i);
      if (status != JFG_OK) break;
      done_iters += todo;
    }
    cudaError_t e = cudaMemcpyAsync(&h_active, c.nactive, sizeof(int), cudaMemcpyDeviceToHost, st);
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
    JFG_CUDA_TRY(cudaMemcpyAsync(iters_host, c.iters, sizeof(int) * pb.batch,
                                 cudaMemcpyDeviceToHost, st));
    JFG_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return h_active == 0 ? JFG_OK : JFG_ERR_NOT_CONVERGED;
}

template struct PcgCtx<float>;
template struct PcgCtx<double>;
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
