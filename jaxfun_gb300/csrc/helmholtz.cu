// Structured FP64 apply of the 2-D Dirichlet Helmholtz operator
//
//   v_b = alpha2[b] (M (x) M) u_b + (K (x) M) u_b + (M (x) K) u_b
//
// for Legendre or Chebyshev Dirichlet composites phi_k = P_k - P_{k+2}
// (src/jaxfun/galerkin/composite.py:786-789) with M = S diag(h) S^T
// (composite.py:330-333) and K = -S D2 S^T, where D2[i][j] are the closed-form
// second-derivative couplings of src/jaxfun/galerkin/Legendre.py:19-33
// (j(j+1) - i(i+1)) and src/jaxfun/galerkin/Chebyshev.py:21-35
// (pi/2 j (j^2 - i^2)), nonzero for j >= i+2 with j - i even.
//
// Along one line of length n (orthogonal length n+2) one backward sweep
// i = n+1 .. 0 computes t_i = (S^T x)_i = x_i - x_{i-2}, w_i = (diag(h) t)_i
// and w_i = -(D2 t)_i (a two-term recurrence per parity class), and the output
// y_i = (S w)_i = w_i - w_{i+2}; everything stays in registers, so the apply
// costs O(n^2) per problem instead of the O(n^3) of dense matrices.  Rows apply
// M and K in one sweep, columns the whole (a2 M + K) U1 + M U2 in one sweep.
// This is the FP64 residual of iterative refinement for the Helmholtz batches.
#include <vector>

#include "jfg_internal.cuh"
#include "pcg_internal.cuh"

namespace jfg {
namespace {

constexpr double PI = 3.14159265358979323846;
constexpr double PI2 = 1.5707963267948966192;

// Per-row coefficients of the sweeps, filled once per block into shared memory
// (the sweep then spends its FP64 issue slots on the arithmetic only):
//   h[i] = (P_i, P_i)_w                       diagonal of the orthogonal mass
//   c[i] = -(4i+6)       (Legendre)           stiffness recurrence coefficient,
//        = -(pi/2)(4i+4) (Chebyshev)          sign and scale of w folded in
//   s[i] = 1 (Legendre), i (Chebyshev)        weight of t_i in the suffix sum
// With t = S^T x and w_i = -(D2 t)_i = -sum_{j >= i+2, j = i mod 2} c(i, j) t_j,
// the closed forms c(i, j) = j(j+1) - i(i+1) (Legendre) and (pi/2) j (j^2 - i^2)
// (Chebyshev) give, per parity class, the two-term recurrence
//   w_i = V(i) = V(i+2) + c[i] * sum_{j >= i+2} s[j] t_j
// so no large suffix sums cancel and each row costs two FMAs.
constexpr int HTAB = 1026;  // rows per line supported: n + 2 <= HTAB

struct HelmTab {
  double h[HTAB], c[HTAB], s[HTAB];
};

__device__ __forceinline__ void fill_tab(int family, int m, HelmTab& T) {
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    const double di = (double)i;
    T.h[i] = family == 0 ? 2.0 / (2.0 * di + 1.0) : (i == 0 ? PI : PI2);
    T.c[i] = family == 0 ? -(4.0 * di + 6.0) : -PI2 * (4.0 * di + 4.0);
    T.s[i] = family == 0 ? 1.0 : di;
  }
  __syncthreads();
}

// One row (stride sx): U1 = M x and U2 = K x in a single backward sweep
// i = n+1 .. 0 over t_i = x_i - x_{i-2}, w = diag(h) t or -(D2 t), y_i = w_i - w_{i+2}.
// The two parity classes are independent recurrences, each with its state in
// registers; the sweep runs in chunks of SW steps whose loads are all issued
// before the chunk's arithmetic (memory-level parallelism for the serial walk).
constexpr int SW = 8;  // steps per chunk (even: a chunk starts on the class of n+1)

struct RowClass {
  double S = 0.0, V = 0.0, x = 0.0;  // suffix sums and the class's pending x_i
};

__device__ __forceinline__ void helm_row(const HelmTab& T, int n, const double* __restrict__ x,
                                         long long sx, double* __restrict__ U1,
                                         double* __restrict__ U2) {
  RowClass A, B;  // A: the parity of n+1, B: the other
  double wm1 = 0.0, wm2 = 0.0, wk1 = 0.0, wk2 = 0.0;  // w at i+1, i+2
  for (int i0 = n + 1; i0 >= 0; i0 -= SW) {
    double xl[SW];
#pragma unroll
    for (int k = 0; k < SW; ++k) {
      const int i = i0 - k;
      xl[k] = i >= 2 ? x[(long long)(i - 2) * sx] : 0.0;
    }
#pragma unroll
    for (int k = 0; k < SW; ++k) {
      const int i = i0 - k;
      if (i < 0) break;
      RowClass& c = (k & 1) ? B : A;
      const double t = c.x - xl[k];  // c.x = x_i (loaded as x_{(i+2)-2}); 0 beyond n-1
      c.x = xl[k];
      const double wm = T.h[i] * t;
      c.V = fma(T.c[i], c.S, c.V);
      c.S = fma(T.s[i], t, c.S);
      const double wk = c.V;
      if (i < n) {
        U1[(long long)i * sx] = wm - wm2;
        U2[(long long)i * sx] = wk - wk2;
      }
      wm2 = wm1;
      wm1 = wm;
      wk2 = wk1;
      wk1 = wk;
    }
  }
}

// One column (stride sx): v = M (a2 U1 + U2) + K U1 = (a2 M + K) U1 + M U2 in a
// single sweep; r = b - v when b is given, else r = v.
struct ColClass {
  double S = 0.0, V = 0.0, u1 = 0.0, u2 = 0.0;
};

__device__ __forceinline__ void helm_col(const HelmTab& T, int n, const double* __restrict__ U1,
                                         const double* __restrict__ U2, long long sx, double a2,
                                         const double* __restrict__ b, double* __restrict__ r) {
  ColClass A, B;
  double w1 = 0.0, w2 = 0.0;
  for (int i0 = n + 1; i0 >= 0; i0 -= SW) {
    double l1[SW], l2[SW], lb[SW];
#pragma unroll
    for (int k = 0; k < SW; ++k) {
      const int i = i0 - k;
      l1[k] = i >= 2 ? U1[(long long)(i - 2) * sx] : 0.0;
      l2[k] = i >= 2 ? U2[(long long)(i - 2) * sx] : 0.0;
      lb[k] = (b && i >= 0 && i < n) ? b[(long long)i * sx] : 0.0;
    }
#pragma unroll
    for (int k = 0; k < SW; ++k) {
      const int i = i0 - k;
      if (i < 0) break;
      ColClass& c = (k & 1) ? B : A;
      const double t1 = c.u1 - l1[k];
      const double tz = fma(a2, t1, c.u2 - l2[k]);
      c.u1 = l1[k];
      c.u2 = l2[k];
      c.V = fma(T.c[i], c.S, c.V);
      c.S = fma(T.s[i], t1, c.S);
      const double w = fma(T.h[i], tz, c.V);
      if (i < n) {
        const double v = w - w2;
        r[(long long)i * sx] = b ? lb[k] - v : v;
      }
      w2 = w1;
      w1 = w;
    }
  }
}

// axis 1 (contiguous): U1 = rows through M, U2 = rows through K
__global__ void k_helm_rows(int family, int n, long long nlines, const double* __restrict__ u,
                            double* __restrict__ U1, double* __restrict__ U2) {
  __shared__ HelmTab T;
  fill_tab(family, n + 2, T);
  const long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (line >= nlines) return;
  helm_row(T, n, u + line * n, 1, U1 + line * n, U2 + line * n);
}

// axis 0 (stride n): v = (alpha2 M + K) U1 + M U2 (columns), optionally r = b - v
__global__ void k_helm_cols(int family, int n, int batch, const double* __restrict__ U1,
                            const double* __restrict__ U2, const double* __restrict__ alpha2,
                            const double* __restrict__ b, double* __restrict__ v) {
  __shared__ HelmTab T;
  fill_tab(family, n + 2, T);
  const long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (line >= (long long)batch * n) return;
  const long long bi = line / n, j = line % n;
  const long long off = bi * (long long)n * n + j;
  const double a2 = alpha2 ? alpha2[bi] : 0.0;
  helm_col(T, n, U1 + off, U2 + off, n, a2, b ? b + off : nullptr, v + off);
}

}  // namespace
}  // namespace jfg

extern "C" size_t jfg_helmholtz_workspace_size(int n, int batch) {
  return 2 * jfg::align_up((size_t)batch * n * n * sizeof(double), 256);
}

extern "C" int jfg_helmholtz_apply_f64(int family, int n, int batch, const double* alpha2,
                                       const double* u, const double* b, double* v, void* work,
                                       size_t work_bytes, void* stream) {
  if ((family != 0 && family != 1) || n < 1 || batch < 0 || !u || !v) return JFG_ERR_ARG;
  if (n + 2 > jfg::HTAB) return JFG_ERR_UNSUPPORTED;
  const size_t need = jfg_helmholtz_workspace_size(n, batch);
  if (!work || work_bytes < need) return JFG_ERR_WORKSPACE;
  if (batch == 0) return JFG_OK;
  double* U1 = (double*)work;
  double* U2 = (double*)((char*)work + need / 2);
  const long long nl = (long long)batch * n;
  const int blocks = (int)((nl + 127) / 128);
  cudaStream_t st = (cudaStream_t)stream;
  jfg::k_helm_rows<<<blocks, 128, 0, st>>>(family, n, nl, u, U1, U2);
  JFG_LAUNCHED();
  jfg::k_helm_cols<<<blocks, 128, 0, st>>>(family, n, batch, U1, U2, alpha2, b, v);
  JFG_LAUNCHED();
  return JFG_OK;
}

// ---------------------------------------------------------------------------
// mixed-precision batch solve: tensor-core FD corrections, FP64 residuals
// ---------------------------------------------------------------------------

namespace {
struct HelmLayout {
  size_t vec64, part, sc, vec32, fdws, hws, total;
};
HelmLayout helm_layout(int n, int nq, int batch) {
  HelmLayout L;
  L.vec64 = jfg::align_up((size_t)batch * n * n * 8, 256);
  L.part = jfg::align_up((size_t)batch * 16 * 8, 256);
  L.sc = jfg::align_up((size_t)batch * 8, 256);
  L.vec32 = jfg::align_up((size_t)batch * nq * nq * 4, 256);
  L.fdws = jfg::align_up(jfg::fd_ws(2, nq, batch, 4), 256);
  L.hws = jfg::align_up(jfg_helmholtz_workspace_size(n, batch), 256);
  L.total = L.vec64 + L.part + 2 * L.sc + 2 * L.vec32 + L.fdws + L.hws;
  return L;
}
}  // namespace

extern "C" size_t jfg_helmholtz_solve_workspace_size(int n, int nq, int batch) {
  if (n < 1 || nq < n || batch < 1) return 0;
  return helm_layout(n, nq, batch).total;
}

extern "C" int jfg_helmholtz_solve_mixed(int family, int n, int nq, int batch, const float* E_hi,
                                         const float* E_lo, const float* W_hi,
                                         const float* W_lo, const float* lam32,
                                         const double* alpha2, const float* alpha2_32,
                                         const double* rhs, double* x, double tol,
                                         int max_refine, int* refinements, void* work,
                                         size_t work_bytes, void* stream) {
  using namespace jfg;
  if ((family != 0 && family != 1) || n < 1 || nq < n || (nq & 3) || batch < 1 || !E_hi ||
      !E_lo || !W_hi || !W_lo || !lam32 || !rhs || !x || !(tol > 0.0) || max_refine < 1)
    return JFG_ERR_ARG;
  const HelmLayout Lo = helm_layout(n, nq, batch);
  if (!work || work_bytes < Lo.total) return JFG_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = (char*)work;
  double* r64 = (double*)w;
  w += Lo.vec64;
  double* part = (double*)w;
  w += Lo.part;
  double* sc_in = (double*)w;
  w += Lo.sc;
  double* sc_out = (double*)w;
  w += Lo.sc;
  float* r32 = (float*)w;
  w += Lo.vec32;
  float* d32 = (float*)w;
  w += Lo.vec32;
  void* fdws = w;
  w += Lo.fdws;
  void* hws = w;
  const long long N = (long long)n * n;
  std::vector<double> bn, rn, hin(batch), hout(batch);
  std::vector<int> nref(batch, 0);
  JFG_TRY(batch_norms(N, batch, rhs, part, bn, st));
  JFG_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * N * batch, st));
  JFG_CUDA_TRY(cudaMemcpyAsync(r64, rhs, sizeof(double) * N * batch, cudaMemcpyDeviceToDevice, st));
  bool done = false;
  for (int it = 0; it <= max_refine; ++it) {
    JFG_TRY(batch_norms(N, batch, r64, part, rn, st));
    int active = 0;
    for (int b = 0; b < batch; ++b) {
      const bool act = rn[b] > tol * bn[b];
      hin[b] = act ? 1.0 / rn[b] : 0.0;
      hout[b] = act ? rn[b] : 0.0;
      nref[b] += (act && it < max_refine) ? 1 : 0;
      active += act;
    }
    if (!active) {
      done = true;
      break;
    }
    if (it == max_refine) break;
    JFG_CUDA_TRY(cudaMemcpyAsync(sc_in, hin.data(), sizeof(double) * batch,
                                 cudaMemcpyHostToDevice, st));
    JFG_CUDA_TRY(cudaMemcpyAsync(sc_out, hout.data(), sizeof(double) * batch,
                                 cudaMemcpyHostToDevice, st));
    JFG_TRY(launch_pad_scale(2, n, nq, batch, r64, sc_in, r32, st));
    JFG_TRY(fd_solve<float>(Engine::TC, 2, nq, batch, OpRef<float>{E_hi, E_lo},
                            OpRef<float>{W_hi, W_lo}, lam32, alpha2_32, nullptr, r32, d32, fdws,
                            Lo.fdws, st));
    JFG_TRY(launch_unpad_axpy(2, n, nq, batch, d32, sc_out, x, 1.0, st));
    JFG_TRY(jfg_helmholtz_apply_f64(family, n, batch, alpha2, x, rhs, r64, hws, Lo.hws, st));
  }
  if (refinements)
    for (int b = 0; b < batch; ++b) refinements[b] = nref[b];
  return done ? JFG_OK : JFG_ERR_NOT_CONVERGED;
}

// ---------------------------------------------------------------------------
// grouped uneven-N batch: one solve over all size groups
// ---------------------------------------------------------------------------
//
// Problems are stored group-major in flat buffers (problem p of size n_p at
// off64[p] in FP64, padded nq_p at off32[p] in FP32).  One refinement step is
//   scale -> pad (FP32) -> 4 grouped tensor-core FD passes over all groups ->
//   x += ||r|| d -> structured FP64 residual over all lines -> norms -> flags
// with every per-problem scalar on the device, so the step is captured once
// into a CUDA graph and replayed; the host reads one active count per step.

namespace jfg {
namespace {

struct HelmProb {
  int n, nq;
  long long off64, off32, line0;  // flat offsets; first line index of the problem
};

constexpr int HNB = 16;  // partial sums per problem

// part[p*HNB + j] = sum of squares of chunk j of problem p's FP64 vector
__global__ void k_rag_sq_part(const HelmProb* __restrict__ tb, const double* __restrict__ v,
                              const double* __restrict__ gate, double* __restrict__ part) {
  const int p = blockIdx.y, j = blockIdx.x;
  if (gate && gate[p] == 0.0) return;  // unchanged vector: keep its partial sums
  const HelmProb q = tb[p];
  const long long N = (long long)q.n * q.n;
  const long long chunk = (N + HNB - 1) / HNB;
  const long long lo = j * chunk, hi = min(N, lo + chunk);
  const double* x = v + q.off64;
  double s = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) s += x[i] * x[i];
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) part[p * HNB + j] = s;
  }
}

// One block: norms from the partial sums.  init: bn = ||rhs||.  Otherwise
// active_p = ||r_p|| > tol ||rhs_p||, hin = 1/||r|| and hout = ||r|| for active
// problems (0 else), count = number of active problems, and per group g (its
// problems gp0[g] .. gp0[g+1]-1) the list of its active problems' local
// indices at glist + gp0[g] with their number in gcnt[g] -- the active subsets
// the grouped tensor-core passes read.
__global__ void k_rag_flags(int nprob, int ngroups, const int* __restrict__ gp0,
                            const double* __restrict__ part, double* __restrict__ bn, double tol,
                            int init, double* __restrict__ hin, double* __restrict__ hout,
                            int* __restrict__ count, int* __restrict__ glist,
                            int* __restrict__ gcnt) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  int mine = 0;
  for (int p = threadIdx.x; p < nprob; p += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < HNB; ++j) s += part[p * HNB + j];
    const double r = sqrt(s);
    if (init) {
      bn[p] = r;
      continue;
    }
    const bool act = r > tol * bn[p];
    hin[p] = act ? 1.0 / r : 0.0;
    hout[p] = act ? r : 0.0;
    mine += act ? 1 : 0;
  }
  if (init) return;
  if (mine) atomicAdd(&cnt, mine);
  __syncthreads();  // hout of every problem written (global, this block)
  if (threadIdx.x == 0) *count = cnt;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int g = w; g < ngroups; g += nw) {
    const int p0 = gp0[g], p1 = gp0[g + 1];
    int base = 0;
    for (int k0 = p0; k0 < p1; k0 += 32) {
      const int p = k0 + lane;
      const bool act = p < p1 && hout[p] != 0.0;
      const unsigned m = __ballot_sync(0xffffffffu, act);
      if (act) glist[p0 + base + __popc(m & ((1u << lane) - 1u))] = p - p0;
      base += __popc(m);
    }
    if (lane == 0) gcnt[g] = base;
  }
}

// r32 (padded nq) = r64 (n) * hin[p]
__global__ void k_rag_pad(const HelmProb* __restrict__ tb, const double* __restrict__ r64,
                          const double* __restrict__ hin, float* __restrict__ r32) {
  const int p = blockIdx.y;
  const double s = hin[p];
  if (s == 0.0) return;  // inactive: not in the tensor-core passes' lists
  const HelmProb q = tb[p];
  const long long NQ = (long long)q.nq * q.nq;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < NQ;
       i += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(i / q.nq), c = (int)(i % q.nq);
    float v = 0.f;
    if (a < q.n && c < q.n) v = (float)(r64[q.off64 + (long long)a * q.n + c] * s);
    r32[q.off32 + i] = v;
  }
}

// x64 += hout[p] * d32 (unpadded); counts one refinement for active problems
__global__ void k_rag_axpy(const HelmProb* __restrict__ tb, const float* __restrict__ d32,
                           const double* __restrict__ hout, double* __restrict__ x,
                           int* __restrict__ nref) {
  const int p = blockIdx.y;
  const double s = hout[p];
  if (s == 0.0) return;
  const HelmProb q = tb[p];
  const long long N = (long long)q.n * q.n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(i / q.n), c = (int)(i % q.n);
    x[q.off64 + i] += s * (double)d32[q.off32 + (long long)a * q.nq + c];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) nref[p] += 1;
}

__device__ __forceinline__ int find_prob(const HelmProb* tb, int nprob, long long line) {
  int lo = 0, hi = nprob - 1;
  while (lo < hi) {  // last p with line0 <= line
    const int mid = (lo + hi + 1) >> 1;
    if (tb[mid].line0 <= line) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// rows (contiguous axis) of every problem: U1 = rows through M, U2 through K
__global__ void k_rag_rows(int family, int nprob, int mmax, long long nlines,
                           const HelmProb* __restrict__ tb, const double* __restrict__ gate,
                           const double* __restrict__ u, double* __restrict__ U1,
                           double* __restrict__ U2) {
  __shared__ HelmTab T;
  fill_tab(family, mmax, T);
  const long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (line >= nlines) return;
  const int p = find_prob(tb, nprob, line);
  if (gate[p] == 0.0) return;  // x unchanged: its residual stands
  const HelmProb q = tb[p];
  const long long off = q.off64 + (line - q.line0) * q.n;
  helm_row(T, q.n, u + off, 1, U1 + off, U2 + off);
}

// columns: r = b - [(alpha2 M + K) U1 + M U2]
__global__ void k_rag_cols(int family, int nprob, int mmax, long long nlines,
                           const HelmProb* __restrict__ tb, const double* __restrict__ gate,
                           const double* __restrict__ U1, const double* __restrict__ U2,
                           const double* __restrict__ alpha2, const double* __restrict__ b,
                           double* __restrict__ r) {
  __shared__ HelmTab T;
  fill_tab(family, mmax, T);
  const long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (line >= nlines) return;
  const int p = find_prob(tb, nprob, line);
  if (gate[p] == 0.0) return;
  const HelmProb q = tb[p];
  const long long off = q.off64 + (line - q.line0);
  helm_col(T, q.n, U1 + off, U2 + off, q.n, alpha2[p], b + off, r + off);
}

struct GroupedLayout {
  int nprob = 0;
  long long tot64 = 0, tot32 = 0, lines = 0, maxnq2 = 0;
  size_t tb, vec64, part, sc, cnt, lists, vec32, total;
};

GroupedLayout grouped_layout(int ng, const int* n, const int* nq, const int* batch) {
  GroupedLayout L;
  for (int g = 0; g < ng; ++g) {
    L.nprob += batch[g];
    L.tot64 += (long long)batch[g] * n[g] * n[g];
    L.tot32 += (long long)batch[g] * nq[g] * nq[g];
    L.lines += (long long)batch[g] * n[g];
    if ((long long)nq[g] * nq[g] > L.maxnq2) L.maxnq2 = (long long)nq[g] * nq[g];
  }
  L.tb = align_up((size_t)L.nprob * sizeof(HelmProb), 256);
  L.vec64 = align_up((size_t)L.tot64 * 8, 256);
  L.part = align_up((size_t)L.nprob * HNB * 8, 256);
  L.sc = align_up((size_t)L.nprob * 8, 256);
  L.cnt = align_up((size_t)L.nprob * 4, 256) + 256;
  L.lists = 2 * align_up((size_t)L.nprob * 4, 256) + 2 * align_up((size_t)(ng + 1) * 4, 256);
  L.vec32 = align_up((size_t)L.tot32 * 4, 256);
  // table | r64 U1 U2 | part | bn hin hout | nref + count | r32 d32 buf0 buf1
  L.total = L.tb + 3 * L.vec64 + L.part + 3 * L.sc + L.cnt + L.lists + 4 * L.vec32;
  return L;
}

}  // namespace
}  // namespace jfg

extern "C" size_t jfg_helmholtz_grouped_workspace_size(int ngroups, const int* n, const int* nq,
                                                       const int* batch) {
  if (ngroups < 1 || !n || !nq || !batch) return 0;
  for (int g = 0; g < ngroups; ++g)
    if (n[g] < 1 || nq[g] < n[g] || batch[g] < 1) return 0;
  return jfg::grouped_layout(ngroups, n, nq, batch).total;
}

extern "C" int jfg_helmholtz_solve_grouped(
    int family, int ngroups, const int* n, const int* nq, const int* batch,
    const float* const* E_hi, const float* const* E_lo, const float* const* W_hi,
    const float* const* W_lo, const float* const* lam32, const double* alpha2,
    const float* alpha2_32, const double* rhs, double* x, double tol, int max_refine,
    int* refinements, const jfg_tc_config* cfg, void* work, size_t work_bytes, void* stream) {
  using namespace jfg;
  if ((family != 0 && family != 1) || ngroups < 1 || !n || !nq || !batch || !E_hi || !E_lo ||
      !W_hi || !W_lo || !lam32 || !alpha2 || !alpha2_32 || !rhs || !x || !(tol > 0.0) ||
      max_refine < 1)
    return JFG_ERR_ARG;
  int mmax = 0;
  for (int g = 0; g < ngroups; ++g) {
    if (n[g] < 1 || nq[g] < n[g] || (nq[g] & 3) || batch[g] < 1 || !E_hi[g] || !E_lo[g] ||
        !W_hi[g] || !W_lo[g] || !lam32[g])
      return JFG_ERR_ARG;
    if (n[g] + 2 > mmax) mmax = n[g] + 2;
  }
  if (mmax > HTAB) return JFG_ERR_UNSUPPORTED;
  const GroupedLayout Lo = grouped_layout(ngroups, n, nq, batch);
  if (!work || work_bytes < Lo.total) return JFG_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = (char*)work;
  HelmProb* tb = (HelmProb*)w;
  w += Lo.tb;
  double* r64 = (double*)w;
  w += Lo.vec64;
  double* U1 = (double*)w;
  w += Lo.vec64;
  double* U2 = (double*)w;
  w += Lo.vec64;
  double* part = (double*)w;
  w += Lo.part;
  double* bn = (double*)w;
  w += Lo.sc;
  double* hin = (double*)w;
  w += Lo.sc;
  double* hout = (double*)w;
  w += Lo.sc;
  int* nref = (int*)w;
  int* count = (int*)(w + align_up((size_t)Lo.nprob * 4, 256));
  w += Lo.cnt;
  int* glist = (int*)w;  // per-group active lists (group g at gp0[g])
  int* gp0 = (int*)(w + align_up((size_t)Lo.nprob * 4, 256));
  int* gcnt = (int*)((char*)gp0 + align_up((size_t)(ngroups + 1) * 4, 256));
  w += Lo.lists;
  float* r32 = (float*)w;
  w += Lo.vec32;
  float* d32 = (float*)w;
  w += Lo.vec32;
  float* buf0 = (float*)w;
  w += Lo.vec32;
  float* buf1 = (float*)w;

  // problem table
  std::vector<HelmProb> ht(Lo.nprob);
  std::vector<long long> g32(ngroups);
  {
    long long o64 = 0, o32 = 0, l0 = 0;
    int p = 0;
    for (int g = 0; g < ngroups; ++g) {
      g32[g] = o32;
      for (int k = 0; k < batch[g]; ++k, ++p) {
        ht[p] = HelmProb{n[g], nq[g], o64, o32, l0};
        o64 += (long long)n[g] * n[g];
        o32 += (long long)nq[g] * nq[g];
        l0 += n[g];
      }
    }
  }
  JFG_CUDA_TRY(cudaMemcpyAsync(tb, ht.data(), sizeof(HelmProb) * Lo.nprob,
                               cudaMemcpyHostToDevice, st));
  std::vector<int> hp0(ngroups + 1, 0);
  for (int g = 0; g < ngroups; ++g) hp0[g + 1] = hp0[g] + batch[g];
  JFG_CUDA_TRY(cudaMemcpyAsync(gp0, hp0.data(), sizeof(int) * (ngroups + 1),
                               cudaMemcpyHostToDevice, st));

  // per-pass group descriptors of the fast-diagonalisation solve
  std::vector<jfg_contract_desc> ds(ngroups);
  std::vector<const float*> ohE(ngroups), olE(ngroups), ohW(ngroups), olW(ngroups);
  std::vector<const float*> in0(ngroups), in1(ngroups), in2(ngroups), in3(ngroups);
  std::vector<float*> out0(ngroups), out1(ngroups), out2(ngroups), out3(ngroups);
  std::vector<jfg_contract_desc> dsE(ngroups);
  {
    int p0 = 0;
    for (int g = 0; g < ngroups; ++g) {
      // only the group's active problems (lists rebuilt on the device every step)
      jfg_contract_desc d = make_desc(batch[g], nq[g], nq[g], nq[g],
                                      Active{glist + hp0[g], gcnt + g});
      ds[g] = d;
      d.epilogue = JFG_EPI_DIV_EIG;
      d.lam_m = lam32[g];
      d.lam_p = lam32[g];
      d.c0 = alpha2_32 + p0;
      d.c1 = nullptr;
      dsE[g] = d;
      ohE[g] = E_hi[g];
      olE[g] = E_lo[g];
      ohW[g] = W_hi[g];
      olW[g] = W_lo[g];
      in0[g] = r32 + g32[g];
      out0[g] = buf0 + g32[g];
      in1[g] = buf0 + g32[g];
      out1[g] = buf1 + g32[g];
      in2[g] = buf1 + g32[g];
      out2[g] = buf0 + g32[g];
      in3[g] = buf0 + g32[g];
      out3[g] = d32 + g32[g];
      p0 += batch[g];
    }
  }
  const jfg_tc_config tc = cfg ? *cfg : tc_default_config();
  const int np = Lo.nprob;
  const dim3 sgrid(HNB, np);
  const long long avg32 = Lo.tot32 / np + 1;
  const dim3 vgrid((unsigned)((avg32 + 255) / 256 < 64 ? (avg32 + 255) / 256 : 64), np);
  const unsigned lblocks = (unsigned)((Lo.lines + 127) / 128);

  auto step = [&]() -> int {
    k_rag_pad<<<vgrid, 256, 0, st>>>(tb, r64, hin, r32);
    JFG_LAUNCHED();
    JFG_TRY(contract_tc_grouped(ngroups, ds.data(), ohE.data(), olE.data(), in0.data(),
                                out0.data(), tc, st));
    JFG_TRY(contract_tc_grouped(ngroups, dsE.data(), ohE.data(), olE.data(), in1.data(),
                                out1.data(), tc, st));
    JFG_TRY(contract_tc_grouped(ngroups, ds.data(), ohW.data(), olW.data(), in2.data(),
                                out2.data(), tc, st));
    JFG_TRY(contract_tc_grouped(ngroups, ds.data(), ohW.data(), olW.data(), in3.data(),
                                out3.data(), tc, st));
    k_rag_axpy<<<vgrid, 256, 0, st>>>(tb, d32, hout, x, nref);
    JFG_LAUNCHED();
    k_rag_rows<<<lblocks, 128, 0, st>>>(family, np, mmax, Lo.lines, tb, hout, x, U1, U2);
    JFG_LAUNCHED();
    k_rag_cols<<<lblocks, 128, 0, st>>>(family, np, mmax, Lo.lines, tb, hout, U1, U2, alpha2, rhs,
                                        r64);
    JFG_LAUNCHED();
    k_rag_sq_part<<<sgrid, 256, 0, st>>>(tb, r64, hout, part);
    JFG_LAUNCHED();
    k_rag_flags<<<1, 1024, 0, st>>>(np, ngroups, gp0, part, bn, tol, 0, hin, hout, count,
                                    glist, gcnt);
    JFG_LAUNCHED();
    return JFG_OK;
  };

  // x = 0, r = rhs, ||rhs||, first flags
  JFG_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * Lo.tot64, st));
  JFG_CUDA_TRY(cudaMemsetAsync(nref, 0, sizeof(int) * np, st));
  JFG_CUDA_TRY(cudaMemcpyAsync(r64, rhs, sizeof(double) * Lo.tot64, cudaMemcpyDeviceToDevice,
                               st));
  k_rag_sq_part<<<sgrid, 256, 0, st>>>(tb, rhs, nullptr, part);
  JFG_LAUNCHED();
  k_rag_flags<<<1, 1024, 0, st>>>(np, ngroups, gp0, part, bn, tol, 1, hin, hout, count, glist,
                                  gcnt);
  JFG_LAUNCHED();
  k_rag_flags<<<1, 1024, 0, st>>>(np, ngroups, gp0, part, bn, tol, 0, hin, hout, count, glist,
                                  gcnt);
  JFG_LAUNCHED();

  // capture one refinement step (the legacy default stream cannot be captured:
  // there the step is launched directly)
  JFG_TRY(tc_setup());
  const bool use_graph = st != 0;
  cudaGraphExec_t exec = nullptr;
  long long graph_kernels = 0;
  if (use_graph) {
    cudaGraph_t graph = nullptr;
    JFG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    set_capturing(true);
    const int cs = step();
    set_capturing(false);
    cudaError_t ec = cudaStreamEndCapture(st, &graph);
    if (cs != JFG_OK) {
      if (graph) cudaGraphDestroy(graph);
      return cs;
    }
    JFG_CUDA_TRY(ec);
    size_t nn = 0;
    cudaGraphGetNodes(graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(graph, nodes.data(), &nn);
    for (size_t i = 0; i < nn; ++i) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
        ++graph_kernels;
    }
    cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    JFG_CUDA_TRY(ei);
  }

  int status = JFG_ERR_NOT_CONVERGED;
  int h_count = 0;
  for (int it = 0; it <= max_refine; ++it) {
    cudaError_t e = cudaMemcpyAsync(&h_count, count, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_last_cuda_error(e);
      status = JFG_ERR_CUDA;
      break;
    }
    if (h_count == 0) {
      status = JFG_OK;
      break;
    }
    if (it == max_refine) break;
    if (use_graph) {
      e = cudaGraphLaunch(exec, st);
      if (e != cudaSuccess) {
        set_last_cuda_error(e);
        status = JFG_ERR_CUDA;
        break;
      }
      count_launches(graph_kernels);
    } else {
      const int s2 = step();
      if (s2 != JFG_OK) {
        status = s2;
        break;
      }
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (refinements && status != JFG_ERR_CUDA) {
    cudaError_t e = cudaMemcpyAsync(refinements, nref, sizeof(int) * np, cudaMemcpyDeviceToHost,
                                    st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_last_cuda_error(e);
      return JFG_ERR_CUDA;
    }
  }
  return status;
}
