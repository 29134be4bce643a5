// Batched banded LU without pivoting and its solve, one thread per system:
// the per-wavenumber 1-D polynomial systems of Fourier x polynomial problems
// (TPMatricesWavenumberSolver, src/jaxfun/la/tpmatrix.py:590-1013, whose
// elimination is _lu_banded_no_pivot_kernel, src/jaxfun/la/diamatrix.py:1937-1973).
//
// Input band data use jaxfun's column-aligned DIA convention: for diagonal d
// with offset off_d, data[s][d][j] = A_s[j - off_d][j].  The factors are kept
// interleaved across systems, lu[(p + off) * n + j][s], so the threads of a warp
// (consecutive systems) touch consecutive addresses at every step.  The work is
// O(n (p + q)) per system and memory bound.
#include "jfg_internal.cuh"

namespace jfg {
namespace {

constexpr int MAX_DIAG = 64;

struct Offsets {
  int v[MAX_DIAG];
};

__global__ void k_band_pack(int nsys, int n, int ndiag, const Offsets off, int p, int q,
                            const double* __restrict__ data, double* __restrict__ lu) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const int bw = p + q + 1;
  for (int r = 0; r < bw; ++r)
    for (int j = 0; j < n; ++j) lu[((long long)r * n + j) * nsys + s] = 0.0;
  for (int d = 0; d < ndiag; ++d) {
    const int r = p + off.v[d];
    const double* src = data + ((long long)s * ndiag + d) * n;
    for (int j = 0; j < n; ++j) lu[((long long)r * n + j) * nsys + s] = src[j];
  }
}

// Doolittle elimination in the band: L below the diagonal (unit diagonal
// implied), U on and above it.  A zero pivot leaves inf/nan in the factors.
__global__ void k_band_lu(int nsys, int n, int p, int q, double* __restrict__ lu) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  auto at = [&](int r, int j) -> double& { return lu[((long long)r * n + j) * nsys + s]; };
  for (int k = 0; k < n; ++k) {
    const double piv = at(p, k);
    for (int t = 1; t <= p && k + t < n; ++t) {
      const double f = at(p - t, k) / piv;  // A[k+t][k] / A[k][k]
      at(p - t, k) = f;
      for (int u = 1; u <= q && k + u < n; ++u) at(p + u - t, k + u) -= f * at(p + u, k + u);
    }
  }
}

// x = U^-1 L^-1 b; element i of system s at b[s * ss + i * si] (same for x;
// x may alias b)
__global__ void k_band_solve(int nsys, int n, int p, int q, const double* __restrict__ lu,
                             const double* b, double* x, long long ss, long long si) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  auto at = [&](int r, int j) -> double { return lu[((long long)r * n + j) * nsys + s]; };
  const double* bs = b + (long long)s * ss;
  double* xs = x + (long long)s * ss;
  for (int i = 0; i < n; ++i) {  // forward: y_i = b_i - sum_t L[i][i-t] y_{i-t}
    double y = bs[(long long)i * si];
    for (int t = 1; t <= p && i - t >= 0; ++t) y -= at(p - t, i - t) * xs[(long long)(i - t) * si];
    xs[(long long)i * si] = y;
  }
  for (int i = n - 1; i >= 0; --i) {  // backward: x_i = (y_i - sum_u U[i][i+u] x_{i+u}) / U[i][i]
    double v = xs[(long long)i * si];
    for (int u = 1; u <= q && i + u < n; ++u) v -= at(p + u, i + u) * xs[(long long)(i + u) * si];
    xs[(long long)i * si] = v / at(p, i);
  }
}

}  // namespace
}  // namespace jfg

extern "C" size_t jfg_banded_lu_size(int nsys, int n, int p, int q) {
  if (nsys < 0 || n < 1 || p < 0 || q < 0) return 0;
  return (size_t)(p + q + 1) * n * nsys * sizeof(double);
}

extern "C" int jfg_banded_lu_factor_f64(int nsys, int n, int ndiag, const int* offsets_host,
                                        const double* data, double* lu, void* stream) {
  if (nsys < 0 || n < 1 || ndiag < 1 || ndiag > jfg::MAX_DIAG || !offsets_host || !data || !lu)
    return JFG_ERR_ARG;
  jfg::Offsets off;
  int p = 0, q = 0;
  bool has_main = false;
  for (int d = 0; d < ndiag; ++d) {
    const int o = offsets_host[d];
    if (o <= -n || o >= n) return JFG_ERR_ARG;
    for (int e = 0; e < d; ++e)
      if (off.v[e] == o) return JFG_ERR_ARG;  // each offset once
    off.v[d] = o;
    if (-o > p) p = -o;
    if (o > q) q = o;
    has_main |= o == 0;
  }
  if (!has_main) return JFG_ERR_ARG;
  if (nsys == 0) return JFG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  // one warp per block: few thousand systems still spread over every SM
  const int blocks = (nsys + 31) / 32;
  jfg::k_band_pack<<<blocks, 32, 0, st>>>(nsys, n, ndiag, off, p, q, data, lu);
  JFG_LAUNCHED();
  jfg::k_band_lu<<<blocks, 32, 0, st>>>(nsys, n, p, q, lu);
  JFG_LAUNCHED();
  return JFG_OK;
}

extern "C" int jfg_banded_lu_solve_f64(int nsys, int n, int p, int q, const double* lu,
                                       const double* rhs, double* x, long long sys_stride,
                                       long long elem_stride, void* stream) {
  if (nsys < 0 || n < 1 || p < 0 || q < 0 || p >= n || q >= n || !lu || !rhs || !x)
    return JFG_ERR_ARG;
  if (nsys == 0) return JFG_OK;
  jfg::k_band_solve<<<(nsys + 31) / 32, 32, 0, (cudaStream_t)stream>>>(
      nsys, n, p, q, lu, rhs, x, sys_stride, elem_stride);
  JFG_LAUNCHED();
  return JFG_OK;
}
