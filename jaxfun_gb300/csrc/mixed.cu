// Mixed-precision variable-coefficient solve: FP64 iterative refinement around
// a tensor-core (split-TF32) PCG.
//
//   r = rhs - A x              FP64 operator on the CUDA cores (unpadded layout)
//   d = PCG_tc(A, r / ||r||)   FP32 storage, tcgen05 contractions (padded layout)
//   x += ||r|| d
//
// repeated per problem until ||r|| <= tol ||rhs||.  A problem that has
// converged gets a zero inner right-hand side, so its inner PCG is inactive
// from the first iteration and its x is left untouched.
#include <math.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "jfg_internal.cuh"
#include "pcg_internal.cuh"

namespace jfg {

namespace {

constexpr int NBS = 16;

__global__ void k_sq_part(const double* __restrict__ x, long long N, double* __restrict__ part,
                          const int* __restrict__ list = nullptr, const int* count = nullptr,
                          int batch = 0) {
  __shared__ double red[32];
  const int b = list ? active_problem(list, active_count(list, count, batch), batch, blockIdx.y)
                     : (int)blockIdx.y;
  if (b < 0) return;
  const int j = blockIdx.x;
  const long long chunk = (N + NBS - 1) / NBS;
  const long long lo = j * chunk, hi = min(N, lo + chunk);
  const double* xb = x + (long long)b * N;
  double s = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) s += xb[i] * xb[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) part[b * NBS + j] = s;
  }
}

// out32[b][padded] = in64[b][unpadded] * scale[b] (zero in the padding)
__global__ void k_pad_scale(int ndim, int n, int nq, long long Npad, long long Nun,
                            const double* __restrict__ in, const double* __restrict__ scale,
                            float* __restrict__ out, const int* __restrict__ list = nullptr,
                            const int* count = nullptr, int batch = 0) {
  const int b = list ? active_problem(list, active_count(list, count, batch), batch, blockIdx.y)
                     : (int)blockIdx.y;
  if (b < 0) return;
  const double sc = scale[b];
  // per-problem indices fit 32 bits (the launchers check Npad < 2^31): the
  // digit loop divides in 32-bit arithmetic
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (int)Npad; i += gridDim.x * blockDim.x) {
    int r = i, src = 0, mul = 1;
    bool inside = true;
    for (int a = 0; a < ndim; ++a) {
      const int q = r / nq, c = r - q * nq;
      r = q;
      if (c >= n) inside = false;
      src += c * mul;
      mul *= n;
    }
    out[(long long)b * Npad + i] = inside ? (float)(in[(long long)b * Nun + src] * sc) : 0.f;
  }
}

// x64[b][unpadded] += sign * s[b] * d32[b][padded]
__global__ void k_unpad_axpy(int ndim, int n, int nq, long long Npad, long long Nun,
                             const float* __restrict__ d, const double* __restrict__ s,
                             double* __restrict__ x, double sign,
                             const int* __restrict__ list = nullptr, const int* count = nullptr,
                             int batch = 0) {
  const int b = list ? active_problem(list, active_count(list, count, batch), batch, blockIdx.y)
                     : (int)blockIdx.y;
  if (b < 0) return;
  const double sc = sign * s[b];
  if (sc == 0.0) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (int)Nun; i += gridDim.x * blockDim.x) {
    int r = i, src = 0, mul = 1;
    for (int a = 0; a < ndim; ++a) {
      const int q = r / n, c = r - q * n;
      r = q;
      src += c * mul;
      mul *= nq;
    }
    x[(long long)b * Nun + i] += sc * (double)d[(long long)b * Npad + src];
  }
}

__global__ void k_sub_from64(const double* __restrict__ a, double* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = a[i] - y[i];
}

// y[b] = a[b] - y[b] for the listed problems (length N each)
__global__ void k_sub_from64_list(const double* __restrict__ a, double* __restrict__ y,
                                  long long N, const int* __restrict__ list, const int* count,
                                  int batch) {
  const int b = active_problem(list, active_count(list, count, batch), batch, blockIdx.y);
  if (b < 0) return;
  const long long off = (long long)b * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x)
    y[off + i] = a[off + i] - y[off + i];
}

// ---- per-problem outer steps (the flat schedule) -------------------------

// bn[b] = ||rhs_b|| from its partial sums
__global__ void k_norms_from(const double* __restrict__ part, double* __restrict__ out,
                             int batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  double s = 0.0;
  for (int j = 0; j < NBS; ++j) s += part[b * NBS + j];
  out[b] = sqrt(s);
}

constexpr int OT = 256;

// Outer decision for the listed problems (all with list NULL) from the norms
// of their new residuals: a problem above tol ||rhs_b|| with outer steps left
// restarts its inner solve (scales 1/||r|| and ||r||, inner tolerance
// max(inner_tol, min(0.1, 0.3 tol / relres)), residual kind of its next outer
// step: FP32 update once relres <= 1e-4 when allowed); the others stop
// (state 2 converged, 3 out of outer steps).  The restart list keeps the
// order.  One block.
__global__ void __launch_bounds__(OT)
    k_outer_decide(const double* __restrict__ part, const double* __restrict__ bn, double tol,
                   double inner_tol, int max_outer, int fp32_ok, const int* __restrict__ list,
                   const int* count, int batch, double* __restrict__ sc_in,
                   double* __restrict__ sc_out, double* __restrict__ tolv,
                   int* __restrict__ outer_cnt, int* __restrict__ res_mode,
                   int* __restrict__ state, int* __restrict__ rlist, int* __restrict__ nr) {
  __shared__ int wcnt[OT / 32];
  __shared__ int base;
  const int n = active_count(list, count, batch);
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j0 = 0; j0 < n; j0 += OT) {
    const int j = j0 + threadIdx.x;
    const int b = j < n ? (list ? list[j] : j) : -1;
    bool act = false;
    if (b >= 0 && b < batch) {
      double s = 0.0;
      for (int k = 0; k < NBS; ++k) s += part[b * NBS + k];
      const double rn = sqrt(s), bb = bn[b];
      const double relres = bb > 0.0 ? rn / bb : 0.0;
      act = rn > tol * bb && outer_cnt[b] < max_outer;
      if (act) {
        sc_in[b] = 1.0 / rn;
        sc_out[b] = rn;
        double tk = inner_tol;
        const double need = relres > 0.0 ? 0.3 * tol / relres : 0.1;
        if (need > tk) tk = need < 0.1 ? need : 0.1;
        tolv[b] = tk;
        res_mode[b] = (fp32_ok && relres <= 1e-4) ? 1 : 0;
        outer_cnt[b] += 1;
        state[b] = 1;
      } else {
        sc_in[b] = 0.0;
        sc_out[b] = 0.0;
        state[b] = rn <= tol * bb ? 2 : 3;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, act);
    if (lane == 0) wcnt[w] = __popc(m);
    __syncthreads();
    int off = base + __popc(m & ((1u << lane) - 1u));
    for (int i = 0; i < w; ++i) off += wcnt[i];
    if (act) rlist[off] = b;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int i = 0; i < OT / 32; ++i) base += wcnt[i];
    __syncthreads();
  }
  if (threadIdx.x == 0) *nr = base;
}

// The ready problems (inner solve over) into all / recompute-residual /
// FP32-update lists; the ready count is cleared.  One block.
__global__ void __launch_bounds__(OT)
    k_split_ready(const int* __restrict__ ready, int* __restrict__ nready,
                  const int* __restrict__ res_mode, int batch, int* __restrict__ rall,
                  int* __restrict__ ctrl /* [0] all, [1] recompute, [2] update */,
                  int* __restrict__ rdf, int* __restrict__ rup) {
  __shared__ int wa[OT / 32], wb[OT / 32];
  __shared__ int ba, bb2;
  const int n = min(max(*nready, 0), batch);
  if (threadIdx.x == 0) ba = bb2 = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j0 = 0; j0 < n; j0 += OT) {
    const int j = j0 + threadIdx.x;
    const int b = j < n ? ready[j] : -1;
    const bool valid = b >= 0 && b < batch;
    if (valid) rall[j] = b;
    const bool up = valid && res_mode[b] == 1;
    const bool df = valid && !up;
    const unsigned mu = __ballot_sync(0xffffffffu, up), md = __ballot_sync(0xffffffffu, df);
    if (lane == 0) {
      wa[w] = __popc(md);
      wb[w] = __popc(mu);
    }
    __syncthreads();
    int od = ba + __popc(md & ((1u << lane) - 1u)), ou = bb2 + __popc(mu & ((1u << lane) - 1u));
    for (int i = 0; i < w; ++i) {
      od += wa[i];
      ou += wb[i];
    }
    if (df) rdf[od] = b;
    if (up) rup[ou] = b;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int i = 0; i < OT / 32; ++i) {
        ba += wa[i];
        bb2 += wb[i];
      }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ctrl[0] = n;
    ctrl[1] = ba;
    ctrl[2] = bb2;
    *nready = 0;
  }
}

// ---- control of the solve loop inside one CUDA graph ----------------------
// ctrl[8] body iterations, ctrl[9] outer steps taken, ctrl[10] chunks run,
// ctrl[11] set when the iteration guard ended the loop.
constexpr int CT_LOOPS = 8, CT_READY = 9, CT_CHUNKS = 10, CT_GUARD = 11;

// Before the loop: it runs while some problem is active or ready.
__global__ void k_loop_init(cudaGraphConditionalHandle h_loop, const int* __restrict__ pcg_ctl) {
  if (threadIdx.x == 0 && blockIdx.x == 0)
    cudaGraphSetConditional(h_loop, (pcg_ctl[0] > 0 || pcg_ctl[1] > 0) ? 1u : 0u);
}

// Head of each loop body: the ready problems take their outer step now
// (schedule 1: whenever some are ready; schedule 0: once no problem is still
// iterating), else the active ones run a chunk of iterations.
__global__ void k_loop_branch(cudaGraphConditionalHandle h_ready, const int* __restrict__ pcg_ctl,
                              int flat, int* __restrict__ ctrl) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int na = pcg_ctl[0], nr = pcg_ctl[1];
  const bool ready = nr > 0 && (flat || na <= 0);
  cudaGraphSetConditional(h_ready, ready ? 1u : 0u);
  ctrl[ready ? CT_READY : CT_CHUNKS] += 1;
}

// Tail of each loop body: go on while problems are active or ready, at most
// guard times.
__global__ void k_loop_next(cudaGraphConditionalHandle h_loop, const int* __restrict__ pcg_ctl,
                            int* __restrict__ ctrl, int guard) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int loops = ++ctrl[CT_LOOPS];
  bool more = pcg_ctl[0] > 0 || pcg_ctl[1] > 0;
  if (more && loops >= guard) {
    ctrl[CT_GUARD] = 1;
    more = false;
  }
  cudaGraphSetConditional(h_loop, more ? 1u : 0u);
}

inline int blocks_for(long long n, int cap) {
  long long b = (n + 255) / 256;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

struct MixedLayout {
  long long Nun, Npad;
  size_t vec64, part, sc, vec32, ws64, wsin, opdf, outer, total;
};

MixedLayout layout(int ndim, int n, int nq, int batch) {
  MixedLayout L;
  L.Nun = 1;
  L.Npad = 1;
  for (int i = 0; i < ndim; ++i) L.Nun *= n, L.Npad *= nq;
  L.vec64 = align_up((size_t)L.Nun * batch * 8, 256);
  L.part = align_up((size_t)batch * NBS * 8, 256);
  L.sc = align_up((size_t)batch * 8, 256);
  L.vec32 = align_up((size_t)L.Npad * batch * 4, 256);
  L.ws64 = align_up(varcoef_ws(ndim, n, nq, batch, 8), 256);
  L.wsin = pcg_ws<float>(ndim, nq, nq, batch);
  // the FP64 operator split once per solve into (hi, lo) pairs for the
  // double-FP32 residual passes
  L.opdf = align_up((size_t)8 * n * nq * sizeof(float2), 256);
  // per-problem outer state: ||rhs||, outer count, state, residual kind, four
  // lists and a control block
  L.outer = align_up((size_t)batch * 8, 256) + 7 * align_up((size_t)batch * 4, 256) + 256;
  L.total = L.vec64 + L.part + 2 * L.sc + 2 * L.vec32 + L.ws64 + L.wsin + L.opdf + L.outer;
  return L;
}

// ---- cache of instantiated solve graphs ------------------------------------
// A solve graph: the prologue, then a loop (conditional WHILE node) whose body
// picks (conditional IF/ELSE node) the outer step of the ready problems or a
// chunk of inner iterations.  Kernel nodes per part, for the launch count.
struct SolveGraph {
  GraphKey key;
  cudaGraphExec_t exec = nullptr;
  long long k_top = 0, k_ready = 0, k_chunk = 0, k_body = 0;
  unsigned long long used = 0;
};
std::mutex g_solve_mu;
std::vector<SolveGraph> g_solves;
unsigned long long g_solve_clock = 0;
constexpr size_t SOLVE_CACHE_MAX = 8;

bool solve_cache_find(const GraphKey& k, SolveGraph* out) {
  std::lock_guard<std::mutex> lk(g_solve_mu);
  for (SolveGraph& e : g_solves)
    if (e.key == k) {
      e.used = ++g_solve_clock;
      *out = e;
      return true;
    }
  return false;
}

void solve_cache_put(const SolveGraph& g) {
  std::lock_guard<std::mutex> lk(g_solve_mu);
  if (g_solves.size() >= SOLVE_CACHE_MAX) {
    size_t lru = 0;
    for (size_t i = 1; i < g_solves.size(); ++i)
      if (g_solves[i].used < g_solves[lru].used) lru = i;
    cudaGraphExecDestroy(g_solves[lru].exec);
    g_solves.erase(g_solves.begin() + lru);
  }
  g_solves.push_back(g);
  g_solves.back().used = ++g_solve_clock;
}

long long kernel_nodes(cudaGraph_t g) {
  size_t nn = 0;
  if (cudaGraphGetNodes(g, nullptr, &nn) != cudaSuccess || nn == 0) return 0;
  std::vector<cudaGraphNode_t> nodes(nn);
  if (cudaGraphGetNodes(g, nodes.data(), &nn) != cudaSuccess) return 0;
  long long k = 0;
  for (size_t i = 0; i < nn; ++i) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

// Add a conditional node after everything captured so far on st (which keeps
// capturing after it); its body graphs are returned in bodies.
int add_conditional(cudaStream_t st, cudaGraph_t g, cudaGraphConditionalHandle h,
                    cudaGraphConditionalNodeType type, unsigned size, cudaGraph_t* bodies) {
  cudaStreamCaptureStatus cs;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  JFG_CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd));
  if (cs != cudaStreamCaptureStatusActive) return JFG_ERR_CUDA;
  cudaGraphNodeParams np = {};  // every reserved and unused byte zero
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = type;
  np.conditional.size = size;
  cudaGraphNode_t node;
  JFG_CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, nd, &np));
  for (unsigned i = 0; i < size; ++i) bodies[i] = np.conditional.phGraph_out[i];
  JFG_CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                                   cudaStreamSetCaptureDependencies));
  return JFG_OK;
}

// Capture fill() into graph g on st; on failure the capture is ended and the
// error returned.
template <typename F>
int capture_into(cudaStream_t st, cudaGraph_t g, F&& fill) {
  JFG_CUDA_TRY(cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0,
                                             cudaStreamCaptureModeThreadLocal));
  const int s = fill();
  cudaGraph_t out = nullptr;
  const cudaError_t e = cudaStreamEndCapture(st, &out);
  if (s != JFG_OK) return s;
  JFG_CUDA_TRY(e);
  return JFG_OK;
}

}  // namespace

// ---- refinement glue shared with the Helmholtz batch solver -------------

int launch_pad_scale(int ndim, int n, int nq, int batch, const double* in, const double* scale,
                     float* out, cudaStream_t st) {
  long long Nun = 1, Npad = 1;
  for (int i = 0; i < ndim; ++i) Nun *= n, Npad *= nq;
  if (Npad > 2147483647LL) return JFG_ERR_ARG;
  k_pad_scale<<<dim3(blocks_for(Npad, 256), batch), 256, 0, st>>>(ndim, n, nq, Npad, Nun, in,
                                                                    scale, out);
  JFG_LAUNCHED();
  return JFG_OK;
}

int launch_unpad_axpy(int ndim, int n, int nq, int batch, const float* d, const double* s,
                      double* x, double sign, cudaStream_t st) {
  long long Nun = 1, Npad = 1;
  for (int i = 0; i < ndim; ++i) Nun *= n, Npad *= nq;
  if (Npad > 2147483647LL) return JFG_ERR_ARG;
  k_unpad_axpy<<<dim3(blocks_for(Nun, 256), batch), 256, 0, st>>>(ndim, n, nq, Npad, Nun, d, s,
                                                                    x, sign);
  JFG_LAUNCHED();
  return JFG_OK;
}

int batch_norms(long long N, int batch, const double* x, double* part_dev,
                std::vector<double>& norms, cudaStream_t st) {
  k_sq_part<<<dim3(NBS, batch), 256, 0, st>>>(x, N, part_dev);
  JFG_LAUNCHED();
  std::vector<double> hp((size_t)batch * NBS);
  JFG_CUDA_TRY(cudaMemcpyAsync(hp.data(), part_dev, sizeof(double) * batch * NBS,
                               cudaMemcpyDeviceToHost, st));
  JFG_CUDA_TRY(cudaStreamSynchronize(st));
  norms.assign(batch, 0.0);
  for (int b = 0; b < batch; ++b) {
    double s = 0.0;
    for (int j = 0; j < NBS; ++j) s += hp[(size_t)b * NBS + j];
    norms[b] = sqrt(s);
  }
  return JFG_OK;
}

}  // namespace jfg

extern "C" size_t jfg_pcg_mixed_workspace_size(int ndim, int n, int nq, int batch) {
  if ((ndim != 2 && ndim != 3) || n < 1 || nq < n || batch < 1) return 0;
  return jfg::layout(ndim, n, nq, batch).total;
}

extern "C" int jfg_pcg_varcoef_mixed_guess(const jfg_mixed_plan* plan, const double* rhs,
                                           double* x, const double* guess, int use_x0,
                                           double tol, double inner_tol, int max_outer,
                                           int maxiter_inner, int* inner_iters,
                                           int* outer_iters, void* work, size_t work_bytes,
                                           void* stream);

// Tune the tensor-core passes of the inner solve: one operator apply and one
// preconditioner solve on zeroed workspace vectors with autotuning on, so
// every distinct pass signature gets its fastest configuration (kept for the
// process) before the solve captures its iteration graph.
extern "C" int jfg_pcg_mixed_autotune(const jfg_mixed_plan* plan, void* work, size_t work_bytes,
                                      void* stream) {
  using namespace jfg;
  if (!plan) return JFG_ERR_ARG;
  const jfg_mixed_plan& P = *plan;
  if ((P.ndim != 2 && P.ndim != 3) || P.n < 1 || P.nq < P.n || P.batch < 1 || !P.ops_hi ||
      !P.ops_lo || !P.kw32 || !P.E_hi || !P.E_lo || !P.W_hi || !P.W_lo || !P.lam ||
      (P.precond_bf16 != 0 && P.precond_bf16 != 1 && P.precond_bf16 != 2) ||
      (P.precond_bf16 && (!P.E_hi16 || !P.W_hi16)) ||
      (P.precond_bf16 == 1 && (!P.E_lo16 || !P.W_lo16)) ||
      (P.apply_f16 && ((P.nq & 7) || !P.ops_hi16 || !P.ops_lo16 || !P.ops_inv16)))
    return JFG_ERR_ARG;
  const int ndim = P.ndim, nq = P.nq, batch = P.batch;
  const MixedLayout Lo = layout(ndim, P.n, nq, batch);
  if (!work || work_bytes < Lo.total) return JFG_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  char* w = (char*)work + Lo.vec64 + Lo.part + 2 * Lo.sc;
  float* r32 = (float*)w;
  float* d32 = (float*)(w + Lo.vec32);
  char* wsin = w + 2 * Lo.vec32 + Lo.ws64;
  unsigned* slots = (unsigned*)wsin;
  const size_t sb = align_up((size_t)H16_SLOTS * batch * sizeof(unsigned), 256);
  void* inner = wsin + sb;
  const size_t inner_bytes = Lo.wsin - sb;
  JFG_CUDA_TRY(cudaMemsetAsync(r32, 0, Lo.vec32, st));
  JFG_CUDA_TRY(cudaMemsetAsync(slots, 0, sb, st));
  H16Ops h16;
  h16.op_inv = P.ops_inv16;
  h16.slots = slots;
  const bool th = P.apply_f16 != 0;
  const bool pbf = P.precond_bf16 != 0;
  const OpRef<float> ops = th ? OpRef<float>{(const float*)P.ops_hi16, (const float*)P.ops_lo16}
                              : OpRef<float>{P.ops_hi, P.ops_lo};
  // plain BF16 (precond_bf16 2): no lo halves, one product per term
  const bool p1 = P.precond_bf16 == 2;
  const OpRef<float> E =
      pbf ? OpRef<float>{(const float*)P.E_hi16, p1 ? nullptr : (const float*)P.E_lo16}
          : OpRef<float>{P.E_hi, P.E_lo};
  const OpRef<float> W =
      pbf ? OpRef<float>{(const float*)P.W_hi16, p1 ? nullptr : (const float*)P.W_lo16}
          : OpRef<float>{P.W_hi, P.W_lo};
  const int prev = single_autotune();
  set_single_autotune(1);
  int s = varcoef_apply<float>(th ? Engine::TH : Engine::TC, ndim, nq, nq, batch, ops, P.kw32,
                               r32, d32, inner, inner_bytes, st, Active(), th ? &h16 : nullptr);
  if (s == JFG_OK)
    s = fd_solve<float>(pbf ? Engine::TB : Engine::TC, ndim, nq, batch, E, W, P.lam, nullptr,
                        P.fd_scale, r32, d32, inner, inner_bytes, st);
  set_single_autotune(prev);
  if (s != JFG_OK) return s;
  JFG_CUDA_TRY(cudaStreamSynchronize(st));
  return JFG_OK;
}

extern "C" int jfg_pcg_varcoef_mixed(const jfg_mixed_plan* plan, const double* rhs, double* x,
                                     int use_x0, double tol, double inner_tol, int max_outer,
                                     int maxiter_inner, int* inner_iters, int* outer_iters,
                                     void* work, size_t work_bytes, void* stream) {
  return jfg_pcg_varcoef_mixed_guess(plan, rhs, x, nullptr, use_x0, tol, inner_tol, max_outer,
                                     maxiter_inner, inner_iters, outer_iters, work, work_bytes,
                                     stream);
}

extern "C" int jfg_pcg_varcoef_mixed_guess(const jfg_mixed_plan* plan, const double* rhs,
                                           double* x, const double* guess, int use_x0,
                                           double tol, double inner_tol, int max_outer,
                                           int maxiter_inner, int* inner_iters,
                                           int* outer_iters, void* work, size_t work_bytes,
                                           void* stream) {
  using namespace jfg;
  if (!plan || !rhs || !x || !(tol > 0.0) || !(inner_tol > 0.0) || max_outer < 1 ||
      maxiter_inner < 1)
    return JFG_ERR_ARG;
  const jfg_mixed_plan& P = *plan;
  if ((P.ndim != 2 && P.ndim != 3) || P.n < 1 || P.nq < P.n || P.batch < 1 || !P.ops64 ||
      !P.kw64 || !P.ops_hi || !P.ops_lo || !P.kw32 || !P.E_hi || !P.E_lo || !P.W_hi ||
      !P.W_lo || !P.lam || (P.residual != 0 && P.residual != 1) ||
      (P.precond_bf16 != 0 && P.precond_bf16 != 1 && P.precond_bf16 != 2) ||
      (P.precond_bf16 && (!P.E_hi16 || !P.W_hi16)) ||
      (P.precond_bf16 == 1 && (!P.E_lo16 || !P.W_lo16)) ||
      (P.apply_f16 != 0 && P.apply_f16 != 1) ||
      (P.apply_f16 && ((P.nq & 7) || !P.ops_hi16 || !P.ops_lo16 || !P.ops_inv16)) ||
      (P.schedule != 0 && P.schedule != 1))
    return JFG_ERR_ARG;
  const int ndim = P.ndim, n = P.n, nq = P.nq, batch = P.batch;
  const MixedLayout Lo = layout(ndim, n, nq, batch);
  if (Lo.Npad > 2147483647LL) return JFG_ERR_ARG;  // per-problem indices are 32-bit
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
  void* ws64 = w;
  w += Lo.ws64;
  void* wsin = w;
  w += Lo.wsin;
  float2* opdf = (float2*)w;
  if (P.residual == 1) JFG_TRY(split_pairs_f64(P.ops64, opdf, 8LL * n * nq, st));

  PcgProblem<float> pb;
  pb.engine = P.apply_f16 ? Engine::TH : Engine::TC;
  const bool pbf = P.precond_bf16 != 0;
  pb.m_engine = pbf ? Engine::TB : Engine::TC;
  pb.ndim = ndim;
  pb.n = nq;
  pb.nq = nq;
  pb.batch = batch;
  pb.ops = P.apply_f16 ? OpRef<float>{(const float*)P.ops_hi16, (const float*)P.ops_lo16}
                       : OpRef<float>{P.ops_hi, P.ops_lo};
  pb.ops_inv = P.apply_f16 ? P.ops_inv16 : nullptr;
  pb.fuse_dots = P.fused_dots & 3;
  pb.kw = P.kw32;
  // plain BF16 (precond_bf16 2): no lo halves, one product per term
  const bool p1 = P.precond_bf16 == 2;
  pb.E = pbf ? OpRef<float>{(const float*)P.E_hi16, p1 ? nullptr : (const float*)P.E_lo16}
             : OpRef<float>{P.E_hi, P.E_lo};
  pb.W = pbf ? OpRef<float>{(const float*)P.W_hi16, p1 ? nullptr : (const float*)P.W_lo16}
             : OpRef<float>{P.W_hi, P.W_lo};
  pb.lam = P.lam;
  pb.fd_scale = P.fd_scale;
  pb.rhs = r32;

  const long long tot64 = Lo.Nun * batch;
  const dim3 pgrid(blocks_for(Lo.Npad, 256), batch);
  const dim3 ugrid(blocks_for(Lo.Nun, 256), batch);
  const dim3 sgrid(NBS, batch);
  auto residual = [&]() -> int {
    JFG_TRY(varcoef_apply<double>(
        P.residual == 1 ? Engine::DF : Engine::F64, ndim, n, nq, batch,
        OpRef<double>{P.ops64, P.residual == 1 ? (const double*)opdf : nullptr}, P.kw64, x, r64,
        ws64, Lo.ws64, st));
    k_sub_from64<<<blocks_for(tot64, 4096), 256, 0, st>>>(rhs, r64, tot64);
    JFG_LAUNCHED();
    return JFG_OK;
  };

  // ---- per-problem outer steps, decided on the device ----
  // A problem whose inner solve has converged (or hit maxiter_inner) leaves
  // the active list for the ready list.  The ready problems then take their
  // outer step together -- x += ||r|| d, the new residual (recomputed in
  // FP64-class arithmetic, or updated in FP32 once it is small), its norm and
  // the decision -- and restart.  Schedule 0 takes that step once no problem
  // is still iterating (the batch's outer steps stay in step); schedule 1 at
  // the next chunk boundary while the others keep iterating.  On a stream
  // that can be captured the whole solve is ONE cached CUDA graph: the
  // prologue, then a conditional WHILE node whose body chooses (conditional
  // IF/ELSE node, set by a one-thread kernel) between the outer step and a
  // chunk of inner iterations; the host waits once, at the end.
  char* ob = (char*)opdf + Lo.opdf;
  const size_t ib = align_up((size_t)batch * 4, 256);
  double* bnd = (double*)ob;
  ob += align_up((size_t)batch * 8, 256);
  int* outer_cnt = (int*)ob;
  int* state = (int*)(ob + ib);
  int* res_mode = (int*)(ob + 2 * ib);
  int* rall = (int*)(ob + 3 * ib);
  int* rdf = (int*)(ob + 4 * ib);
  int* rup = (int*)(ob + 5 * ib);
  int* rlist = (int*)(ob + 6 * ib);
  // [0] ready, [1] recompute, [2] update, [3] restart, [CT_*] loop control
  int* ctrl = (int*)(ob + 7 * ib);
  PcgCtx<float> c;
  c.maxit = maxiter_inner;
  c.track_ready = true;
  JFG_TRY(c.init(pb, d32, wsin, Lo.wsin, st));
  const int fp32_ok = P.ops32 ? 1 : 0;
  const int flat = P.schedule == 1 ? 1 : 0;
  const dim3 lgrid(NBS, batch);
  const bool from_guess = guess != nullptr && !use_x0;
  const long long guard_ll =
      (long long)(max_outer + 1) * (maxiter_inner / PcgCtx<float>::CH + 2) + 8;
  const int guard = guard_ll > (1LL << 30) ? (1 << 30) : (int)guard_ll;

  // ||rhs_b||, the first residual, the first decision (all problems) and the
  // start of the first inner solves
  auto prologue = [&]() -> int {
    JFG_CUDA_TRY(cudaMemsetAsync(c.nactive, 0, 2 * sizeof(int), st));
    JFG_CUDA_TRY(cudaMemsetAsync(c.iters, 0, sizeof(int) * batch, st));
    JFG_CUDA_TRY(cudaMemsetAsync(outer_cnt, 0, 3 * ib, st));
    JFG_CUDA_TRY(cudaMemsetAsync(ctrl, 0, 256, st));
    k_sq_part<<<lgrid, 256, 0, st>>>(rhs, Lo.Nun, part);
    JFG_LAUNCHED();
    k_norms_from<<<(batch + 127) / 128, 128, 0, st>>>(part, bnd, batch);
    JFG_LAUNCHED();
    if (use_x0) {
      JFG_TRY(residual());
    } else {
      JFG_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * tot64, st));
      JFG_CUDA_TRY(
          cudaMemcpyAsync(r64, rhs, sizeof(double) * tot64, cudaMemcpyDeviceToDevice, st));
    }
    k_sq_part<<<lgrid, 256, 0, st>>>(r64, Lo.Nun, part);
    JFG_LAUNCHED();
    k_outer_decide<<<1, OT, 0, st>>>(part, bnd, tol, inner_tol, max_outer, fp32_ok, nullptr,
                                     nullptr, batch, sc_in, sc_out, c.tolv, outer_cnt, res_mode,
                                     state, rlist, ctrl + 3);
    JFG_LAUNCHED();
    k_pad_scale<<<pgrid, 256, 0, st>>>(ndim, n, nq, Lo.Npad, Lo.Nun, r64, sc_in, r32, rlist,
                                       ctrl + 3, batch);
    JFG_LAUNCHED();
    if (from_guess) {
      // the learned guess starts each first inner solve, judged per problem
      k_pad_scale<<<pgrid, 256, 0, st>>>(ndim, n, nq, Lo.Npad, Lo.Nun, guess, sc_in, d32, rlist,
                                         ctrl + 3, batch);
      JFG_LAUNCHED();
    }
    return c.start(rlist, ctrl + 3, from_guess ? 1 : 0, from_guess);
  };

  // the outer step of the ready problems, then their restart
  auto ready_step = [&]() -> int {
    k_split_ready<<<1, OT, 0, st>>>(c.ready, c.nready, res_mode, batch, rall, ctrl, rdf, rup);
    JFG_LAUNCHED();
    k_unpad_axpy<<<ugrid, 256, 0, st>>>(ndim, n, nq, Lo.Npad, Lo.Nun, d32, sc_out, x, 1.0, rall,
                                        ctrl, batch);
    JFG_LAUNCHED();
    // recomputed residuals r = rhs - A x
    JFG_TRY(varcoef_apply<double>(
        P.residual == 1 ? Engine::DF : Engine::F64, ndim, n, nq, batch,
        OpRef<double>{P.ops64, P.residual == 1 ? (const double*)opdf : nullptr}, P.kw64, x, r64,
        ws64, Lo.ws64, st, Active{rdf, ctrl + 1}));
    k_sub_from64_list<<<ugrid, 256, 0, st>>>(rhs, r64, Lo.Nun, rdf, ctrl + 1, batch);
    JFG_LAUNCHED();
    // updated residuals r -= ||r|| A32 d (the apply's scratch is the inner
    // solve's pass scratch, free between chunks).  FP32 on the CUDA cores:
    // the scaled split-FP16 tensor-core apply here measured a larger answer
    // error (1.6e-10 against 1e-10 at inner tolerance 1e-5).
    if (fp32_ok) {
      JFG_TRY(varcoef_apply<float>(Engine::F32, ndim, nq, nq, batch,
                                   OpRef<float>{P.ops32, nullptr}, P.kw32, d32, r32, c.inner,
                                   c.inner_bytes, st, Active{rup, ctrl + 2}));
      k_unpad_axpy<<<ugrid, 256, 0, st>>>(ndim, n, nq, Lo.Npad, Lo.Nun, r32, sc_out, r64, -1.0,
                                          rup, ctrl + 2, batch);
      JFG_LAUNCHED();
    }
    k_sq_part<<<lgrid, 256, 0, st>>>(r64, Lo.Nun, part, rall, ctrl, batch);
    JFG_LAUNCHED();
    k_outer_decide<<<1, OT, 0, st>>>(part, bnd, tol, inner_tol, max_outer, fp32_ok, rall, ctrl,
                                     batch, sc_in, sc_out, c.tolv, outer_cnt, res_mode, state,
                                     rlist, ctrl + 3);
    JFG_LAUNCHED();
    k_pad_scale<<<pgrid, 256, 0, st>>>(ndim, n, nq, Lo.Npad, Lo.Nun, r64, sc_in, r32, rlist,
                                       ctrl + 3, batch);
    JFG_LAUNCHED();
    return c.start(rlist, ctrl + 3, 0, false);
  };

  int status = JFG_OK;
  int hctl[4] = {0, 0, 0, 0};  // body iterations, outer steps, chunks, guard hit
  SolveGraph sg;
  const bool graphed = st != 0;
  if (!graphed) {
    // the legacy default stream cannot be captured: the host drives the loop
    JFG_TRY(prologue());
    int hc[2] = {0, 0};
    for (long long loops = 0;; ++loops) {
      JFG_CUDA_TRY(cudaMemcpyAsync(hc, c.nactive, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
      JFG_CUDA_TRY(cudaStreamSynchronize(st));
      if (hc[0] <= 0 && hc[1] <= 0) break;
      if (loops >= guard) {
        status = JFG_ERR_NOT_CONVERGED;
        break;
      }
      if (hc[1] > 0 && (flat || hc[0] <= 0)) {
        JFG_TRY(ready_step());
      } else {
        JFG_TRY(c.chunk());
      }
    }
  } else {
    int dev = 0;
    JFG_CUDA_TRY(cudaGetDevice(&dev));
    GraphKey key;
    long long tb[2];
    const double tv[2] = {tol, inner_tol};
    memcpy(tb, tv, sizeof(tb));
    const long long v[] = {dev,
                           ndim,
                           n,
                           nq,
                           batch,
                           use_x0,
                           from_guess ? 1 : 0,
                           max_outer,
                           maxiter_inner,
                           flat,
                           P.residual,
                           P.precond_bf16,
                           P.apply_f16,
                           P.fused_dots,
                           fp32_ok,
                           (long long)work_bytes,
                           tb[0],
                           tb[1]};
    key.ints.assign(v, v + sizeof(v) / sizeof(v[0]));
    const void* ptrs[] = {rhs,        x,         guess,      work,      P.ops64,   P.kw64,
                          P.ops32,    P.kw32,    P.ops_hi,   P.ops_lo,  P.ops_hi16, P.ops_lo16,
                          P.ops_inv16, P.E_hi,   P.E_lo,     P.W_hi,    P.W_lo,    P.E_hi16,
                          P.E_lo16,   P.W_hi16,  P.W_lo16,   P.lam,     P.fd_scale};
    key.ptrs.assign(ptrs, ptrs + sizeof(ptrs) / sizeof(ptrs[0]));
    if (!solve_cache_find(key, &sg)) {
      sg.key = key;
      cudaGraph_t g = nullptr, body = nullptr, br[2] = {nullptr, nullptr};
      JFG_CUDA_TRY(cudaGraphCreate(&g, 0));
      cudaGraphConditionalHandle h_loop = 0, h_ready = 0;
      set_capturing(true);
      int s = JFG_OK;
      // the loop condition starts at 0 on every launch; only k_loop_init and
      // k_loop_next (bounded by the guard) set it
      if (cudaGraphConditionalHandleCreate(&h_loop, g, 0, cudaGraphCondAssignDefault) !=
          cudaSuccess)
        s = JFG_ERR_CUDA;
      if (s == JFG_OK)
        s = capture_into(st, g, [&]() -> int {
          JFG_TRY(prologue());
          k_loop_init<<<1, 32, 0, st>>>(h_loop, c.nactive);
          JFG_CHECK_LAUNCH();
          return add_conditional(st, g, h_loop, cudaGraphCondTypeWhile, 1, &body);
        });
      if (s == JFG_OK && cudaGraphConditionalHandleCreate(&h_ready, body, 0, 0) != cudaSuccess)
        s = JFG_ERR_CUDA;
      if (s == JFG_OK)
        s = capture_into(st, body, [&]() -> int {
          k_loop_branch<<<1, 32, 0, st>>>(h_ready, c.nactive, flat, ctrl);
          JFG_CHECK_LAUNCH();
          JFG_TRY(add_conditional(st, body, h_ready, cudaGraphCondTypeIf, 2, br));
          k_loop_next<<<1, 32, 0, st>>>(h_loop, c.nactive, ctrl, guard);
          JFG_CHECK_LAUNCH();
          return JFG_OK;
        });
      if (s == JFG_OK) s = capture_into(st, br[0], ready_step);
      if (s == JFG_OK)
        s = capture_into(st, br[1], [&]() -> int {
          for (int i = 0; i < PcgCtx<float>::CH; ++i) JFG_TRY(c.iteration(i));
          return JFG_OK;
        });
      set_capturing(false);
      if (s == JFG_OK) {
        sg.k_top = kernel_nodes(g);
        sg.k_body = kernel_nodes(body);
        sg.k_ready = kernel_nodes(br[0]);
        sg.k_chunk = kernel_nodes(br[1]);
        const cudaError_t ei = cudaGraphInstantiate(&sg.exec, g, 0);
        if (ei != cudaSuccess) {
          set_last_cuda_error(ei);
          s = JFG_ERR_CUDA;
        }
      }
      cudaGraphDestroy(g);
      if (s != JFG_OK) return s;
      solve_cache_put(sg);
    }
    const cudaError_t e = cudaGraphLaunch(sg.exec, st);
    if (e != cudaSuccess) {
      set_last_cuda_error(e);
      return JFG_ERR_CUDA;
    }
    JFG_CUDA_TRY(
        cudaMemcpyAsync(hctl, ctrl + CT_LOOPS, sizeof(hctl), cudaMemcpyDeviceToHost, st));
  }
  std::vector<int> hst(batch);
  JFG_CUDA_TRY(cudaMemcpyAsync(hst.data(), state, sizeof(int) * batch, cudaMemcpyDeviceToHost,
                               st));
  if (inner_iters)
    JFG_CUDA_TRY(cudaMemcpyAsync(inner_iters, c.iters, sizeof(int) * batch,
                                 cudaMemcpyDeviceToHost, st));
  if (outer_iters)
    JFG_CUDA_TRY(cudaMemcpyAsync(outer_iters, outer_cnt, sizeof(int) * batch,
                                 cudaMemcpyDeviceToHost, st));
  JFG_CUDA_TRY(cudaStreamSynchronize(st));
  if (graphed) {
    // kernels the graph ran: its top level, and per body iteration the two
    // control kernels plus the chosen branch
    count_launches(sg.k_top + (long long)hctl[0] * sg.k_body +
                   (long long)hctl[1] * sg.k_ready + (long long)hctl[2] * sg.k_chunk);
    if (hctl[3]) status = JFG_ERR_NOT_CONVERGED;
  }
  if (status != JFG_OK) return status;
  for (int b = 0; b < batch; ++b)
    if (hst[b] != 2) return JFG_ERR_NOT_CONVERGED;
  return JFG_OK;
}
