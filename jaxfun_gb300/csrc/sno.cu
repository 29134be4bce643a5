// CUDA-core kernels of the spectral neural operator that are too small or too
// irregular for the tensor cores: per-mode channel mixing (forward/backward),
// bias gradients, the loss and its gradient, and the Adam update.
#include <algorithm>
#include <cuda_bf16.h>
#include <math.h>

#include "jfg_internal.cuh"

namespace jfg {
namespace {

constexpr int MAXC = 64;  // channel width limit of the mode-mixing kernels

// out[b][co][q] = sum_ci R[q][co][ci] x[b][q][ci]
//
// A block owns MM_Q consecutive modes and a slice of the samples; thread
// (co, ql) keeps the row R[q0+ql][co][:] in registers for the whole slice.
// Per sample the block stages x[b][q0 .. q0+MM_Q)[:] (contiguous, one float
// per thread) in shared memory, double-buffered so one barrier per sample
// suffices, and the MM_Q threads of one output channel write MM_Q
// consecutive modes (16 bytes).  The number of modes must be a multiple of
// MM_Q (checked by the launcher).
constexpr int MM_Q = 8;

constexpr int MM_LD = MAXC + 4;  // 16-byte rows; the MM_Q rows of a warp's float4 reads hit distinct banks

__global__ void __launch_bounds__(MM_Q * MAXC) k_modemix_fwd(
    int batch, int nq, int C, int per_block, const float* __restrict__ R,
    const float* __restrict__ x, __nv_bfloat16* __restrict__ out) {
  __shared__ __align__(16) float xs[2][MM_Q][MM_LD];
  const int t = threadIdx.x;
  // channels ci >= C stay zero (their R entries are zero too)
  for (int i = t; i < 2 * MM_Q * MM_LD; i += blockDim.x) (&xs[0][0][0])[i] = 0.f;
  __syncthreads();
  const int ql = t % MM_Q;
  const int co = t / MM_Q;
  const int q0 = blockIdx.x * MM_Q;
  const int b0 = blockIdx.y * per_block;
  const int b1 = min(batch, b0 + per_block);
  const bool active = co < C;
  float r[MAXC];
  const float* Rrow = R + ((long long)(q0 + ql) * C + (active ? co : 0)) * C;
#pragma unroll
  for (int ci = 0; ci < MAXC; ++ci) r[ci] = (active && ci < C) ? __ldg(Rrow + ci) : 0.f;
  const int nload = MM_Q * C;
  // each thread's element of the next PF samples is loaded ahead, so the
  // loop over samples does not wait on a load every iteration
  constexpr int PF = 4;
  float nxt[PF];
#pragma unroll
  for (int u = 0; u < PF; ++u)
    nxt[u] = (t < nload && b0 + u < b1) ? x[((long long)(b0 + u) * nq + q0) * C + t] : 0.f;
  for (int b = b0; b < b1; ++b) {
    float (*xb)[MM_LD] = xs[b & 1];
    if (t < nload) xb[t / C][t % C] = nxt[0];
#pragma unroll
    for (int u = 0; u + 1 < PF; ++u) nxt[u] = nxt[u + 1];
    nxt[PF - 1] =
        (t < nload && b + PF < b1) ? x[((long long)(b + PF) * nq + q0) * C + t] : 0.f;
    __syncthreads();
    if (active) {
      const float4* xv = reinterpret_cast<const float4*>(xb[ql]);
      float s = 0.f;
#pragma unroll
      for (int c4 = 0; c4 < MAXC / 4; ++c4) {
        const float4 v = xv[c4];
        s = fmaf(r[4 * c4], v.x, s);
        s = fmaf(r[4 * c4 + 1], v.y, s);
        s = fmaf(r[4 * c4 + 2], v.z, s);
        s = fmaf(r[4 * c4 + 3], v.w, s);
      }
      out[((long long)b * C + co) * nq + q0 + ql] = __float2bfloat16(s);
    }
  }
}

// dx[b][ci][q] = sum_co R[q][co][ci] dy[b][q][co];  dR[q][co][ci] = sum_b dy[b][q][co] x[b][q][ci]
__global__ void k_modemix_bwd(int batch, int nq, int C, const float* __restrict__ R,
                              const float* __restrict__ x, const float* __restrict__ dy,
                              __nv_bfloat16* __restrict__ dx, float* __restrict__ dR) {
  __shared__ float Rs[MAXC * (MAXC + 1)];
  __shared__ float xs[MAXC], ds[MAXC];
  const int q = blockIdx.x;
  const int t = threadIdx.x;
  for (int i = t; i < C * C; i += blockDim.x) Rs[(i / C) * (C + 1) + i % C] = R[(long long)q * C * C + i];
  float acc[MAXC / 2];  // dR row co = t, columns [0, C): two halves processed in turn
  for (int half = 0; half < 2; ++half) {
    const int c0 = half * (C / 2 > 0 ? (C + 1) / 2 : C);
    const int cn = half == 0 ? (C + 1) / 2 : C - (C + 1) / 2;
#pragma unroll 4
    for (int j = 0; j < MAXC / 2; ++j) acc[j] = 0.f;
    __syncthreads();
    for (int b = 0; b < batch; ++b) {
      if (t < C) {
        xs[t] = x[((long long)b * nq + q) * C + t];
        ds[t] = dy[((long long)b * nq + q) * C + t];
      }
      __syncthreads();
      if (t < C) {
        const float dyt = ds[t];
#pragma unroll
        for (int j = 0; j < MAXC / 2; ++j)
          if (j < cn) acc[j] += dyt * xs[c0 + j];
        if (half == 0) {
          float s = 0.f;
          for (int co = 0; co < C; ++co) s += Rs[co * (C + 1) + t] * ds[co];
          dx[((long long)b * C + t) * nq + q] = __float2bfloat16(s);
        }
      }
      __syncthreads();
    }
    if (t < C) {
#pragma unroll
      for (int j = 0; j < MAXC / 2; ++j)
        if (j < cn) dR[((long long)q * C + t) * C + c0 + j] = acc[j];
    }
  }
}

__global__ void k_colsum_bf16(long long rows, int n, const __nv_bfloat16* __restrict__ src,
                              float* __restrict__ out, long long rows_per_block) {
  const int c = threadIdx.x;
  if (c >= n) return;
  const long long r0 = blockIdx.x * rows_per_block;
  const long long r1 = min(rows, r0 + rows_per_block);
  float s = 0.f;
  for (long long r = r0; r < r1; ++r) s += __bfloat162float(src[r * n + c]);
  atomicAdd(out + c, s);
}

__global__ void k_adam(long long n, float* __restrict__ p, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                       float eps, float c1, float c2, __nv_bfloat16* __restrict__ pb,
                       __nv_bfloat16* __restrict__ ptb, int rows, int cols) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    const __nv_bfloat16 h = __float2bfloat16(pi);
    if (pb) pb[i] = h;
    if (ptb && rows > 0 && cols > 0) {
      const long long r = i / cols, c = i % cols;
      ptb[c * rows + r] = h;
    }
  }
}

__global__ void k_mse(long long rows, const float* __restrict__ pred, long long ld,
                      const float* __restrict__ target, __nv_bfloat16* __restrict__ dq,
                      __nv_bfloat16* __restrict__ dqt, float* __restrict__ loss) {
  __shared__ float red[32];
  float s = 0.f;
  const float inv = 1.0f / (float)rows;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows;
       r += (long long)gridDim.x * blockDim.x) {
    const float e = pred[r * ld] - target[r];
    s += e * e;
    const __nv_bfloat16 h = __float2bfloat16(e * inv);
    const __nv_bfloat16 z = __float2bfloat16(0.f);
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      if (dq) dq[r * 16 + c] = c == 0 ? h : z;
      if (dqt) dqt[c * rows + r] = c == 0 ? h : z;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    atomicAdd(loss, t);
  }
}

inline int nblocks(long long n, int cap) {
  long long b = (n + 255) / 256;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace
}  // namespace jfg

using namespace jfg;

extern "C" int jfg_sno_modemix_fwd(int batch, int nmodes, int C, const float* R, const float* x,
                                   void* out, void* stream) {
  if (batch < 0 || nmodes < 0 || C < 1 || C > MAXC || !R || !x || !out) return JFG_ERR_ARG;
  if (batch == 0 || nmodes == 0) return JFG_OK;
  if (nmodes % MM_Q != 0) return JFG_ERR_ARG;
  // enough blocks for every SM, at least 8 samples per block
  const int mblocks = nmodes / MM_Q;
  int groups = (2 * 152 + mblocks - 1) / mblocks;
  groups = std::max(1, std::min(groups, (batch + 7) / 8));
  const int per_block = (batch + groups - 1) / groups;
  groups = (batch + per_block - 1) / per_block;
  k_modemix_fwd<<<dim3(mblocks, groups), MM_Q * MAXC, 0, (cudaStream_t)stream>>>(
      batch, nmodes, C, per_block, R, x, (__nv_bfloat16*)out);
  JFG_LAUNCHED();
  return JFG_OK;
}

extern "C" int jfg_sno_modemix_bwd(int batch, int nmodes, int C, const float* R, const float* x,
                                   const float* dy, void* dx, float* dR, void* stream) {
  if (batch < 0 || nmodes < 0 || C < 1 || C > MAXC || !R || !x || !dy || !dx || !dR)
    return JFG_ERR_ARG;
  if (nmodes == 0) return JFG_OK;
  k_modemix_bwd<<<nmodes, ((C + 31) / 32) * 32, 0, (cudaStream_t)stream>>>(
      batch, nmodes, C, R, x, dy, (__nv_bfloat16*)dx, dR);
  JFG_LAUNCHED();
  return JFG_OK;
}

extern "C" int jfg_colsum_bf16(long long rows, int n, const void* src, float* out,
                               int accumulate, void* stream) {
  if (rows < 0 || n < 1 || n > 1024 || !src || !out) return JFG_ERR_ARG;
  if (!accumulate) JFG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * n, (cudaStream_t)stream));
  if (rows == 0) return JFG_OK;
  const long long rpb = 256;
  const long long nb = (rows + rpb - 1) / rpb;
  if (nb > 2147483647LL) return JFG_ERR_ARG;
  k_colsum_bf16<<<(int)nb, ((n + 31) / 32) * 32, 0, (cudaStream_t)stream>>>(
      rows, n, (const __nv_bfloat16*)src, out, rpb);
  JFG_LAUNCHED();
  return JFG_OK;
}

extern "C" int jfg_adam_step(long long n, float* p, const float* g, float* m, float* v, float lr,
                             float beta1, float beta2, float eps, int step, void* p_bf16,
                             void* pt_bf16, int rows, int cols, void* stream) {
  if (n < 0 || !p || !g || !m || !v || step < 1) return JFG_ERR_ARG;
  if (pt_bf16 && ((long long)rows * cols != n)) return JFG_ERR_ARG;
  if (n == 0) return JFG_OK;
  const float c1 = 1.f - powf(beta1, (float)step);
  const float c2 = 1.f - powf(beta2, (float)step);
  k_adam<<<nblocks(n, 8192), 256, 0, (cudaStream_t)stream>>>(
      n, p, g, m, v, lr, beta1, beta2, eps, c1, c2, (__nv_bfloat16*)p_bf16,
      (__nv_bfloat16*)pt_bf16, rows, cols);
  JFG_LAUNCHED();
  return JFG_OK;
}

extern "C" int jfg_sno_mse(long long rows, const float* pred, long long ld_pred,
                           const float* target, void* dq, void* dqt, float* loss_out,
                           void* stream) {
  if (rows < 1 || !pred || !target || !loss_out || ld_pred < 1) return JFG_ERR_ARG;
  k_mse<<<nblocks(rows, 2048), 256, 0, (cudaStream_t)stream>>>(
      rows, pred, ld_pred, target, (__nv_bfloat16*)dq, (__nv_bfloat16*)dqt, loss_out);
  JFG_LAUNCHED();
  return JFG_OK;
}
