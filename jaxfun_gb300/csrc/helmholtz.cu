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
// or w_i = -(D2 t)_i from parity-split suffix sums of t, and the output
// y_i = (S w)_i = w_i - w_{i+2}; everything stays in registers, so the apply
// costs O(n^2) per problem instead of the O(n^3) of dense matrices.  This is
// the FP64 residual of iterative refinement for the uneven Helmholtz batch.
#include <vector>

#include "jfg_internal.cuh"
#include "pcg_internal.cuh"

namespace jfg {
namespace {

// y (+)= sc * Op x along a line; op 0 = M, 1 = K; family 0 Legendre, 1 Chebyshev.
__device__ __forceinline__ void sweep(int family, int op, int n, const double* __restrict__ x,
                                      long long sx, double* __restrict__ y, long long sy,
                                      double sc, bool acc) {
  const int m = n + 2;
  double s0[2] = {0.0, 0.0}, s1[2] = {0.0, 0.0}, s3[2] = {0.0, 0.0};
  double w1 = 0.0, w2 = 0.0;  // w_{i+1}, w_{i+2}
  for (int i = m - 1; i >= 0; --i) {
    const double xi = i < n ? x[(long long)i * sx] : 0.0;
    const double xim2 = (i >= 2 && i - 2 < n) ? x[(long long)(i - 2) * sx] : 0.0;
    const double t = xi - xim2;
    const double di = (double)i;
    double w;
    if (op == 0) {
      const double h = family == 0 ? 2.0 / (2.0 * di + 1.0)
                                   : (i == 0 ? 3.14159265358979323846 : 1.5707963267948966192);
      w = h * t;
    } else {
      const int p = i & 1;
      // row i uses j >= i+2 of its parity: the sums hold exactly those
      if (family == 0)
        w = -(s1[p] - di * (di + 1.0) * s0[p]);
      else
        w = -1.5707963267948966192 * (s3[p] - di * di * s1[p]);
      if (family == 0) {
        s0[p] += t;
        s1[p] += di * (di + 1.0) * t;
      } else {
        s1[p] += di * t;
        s3[p] += di * di * di * t;
      }
    }
    if (i < n) {
      const double yi = sc * (w - w2);
      double* o = y + (long long)i * sy;
      *o = acc ? *o + yi : yi;
    }
    w2 = w1;
    w1 = w;
  }
}

// axis 1 (contiguous): U1 = rows through M, U2 = rows through K
__global__ void k_helm_rows(int family, int n, long long nlines, const double* __restrict__ u,
                            double* __restrict__ U1, double* __restrict__ U2) {
  const long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (line >= nlines) return;
  const double* x = u + line * n;
  sweep(family, 0, n, x, 1, U1 + line * n, 1, 1.0, false);
  sweep(family, 1, n, x, 1, U2 + line * n, 1, 1.0, false);
}

// axis 0 (stride n): v = (alpha2 M + K) U1 + M U2 (columns), optionally r = b - v
__global__ void k_helm_cols(int family, int n, int batch, const double* __restrict__ U1,
                            const double* __restrict__ U2, const double* __restrict__ alpha2,
                            const double* __restrict__ b, double* __restrict__ v) {
  const long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (line >= (long long)batch * n) return;
  const long long bi = line / n, j = line % n;
  const long long off = bi * (long long)n * n + j;
  const double a2 = alpha2 ? alpha2[bi] : 0.0;
  sweep(family, 0, n, U1 + off, n, v + off, n, a2, false);
  sweep(family, 1, n, U1 + off, n, v + off, n, 1.0, true);
  sweep(family, 0, n, U2 + off, n, v + off, n, 1.0, true);
  if (b)
    for (int i = 0; i < n; ++i) v[off + (long long)i * n] = b[off + (long long)i * n] - v[off + (long long)i * n];
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
