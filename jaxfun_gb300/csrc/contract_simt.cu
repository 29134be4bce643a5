// Per-axis contraction on the CUDA cores (FP64 DFMA and FP32 FFMA).
//
// out[b][s][m][p] = alpha * epi(sum_k op[s][m][k] * in[b][s][p][k]) + beta * out[b][s][m][p]
//
// This is the plain-precision path: FP64 is the parity path (<= 1e-12 against
// the FP64 oracle) and the FP64 residual of iterative refinement.  GB300's
// FP64 rate is ~1.2 TFLOP/s (about 2 DFMA/clk/SM), so a 64x64 register-tiled
// kernel is DFMA-bound long before it is memory-bound.
#include <stdio.h>

#include <type_traits>

#include "jfg_internal.cuh"

namespace jfg {

namespace {

constexpr int TK = 16;   // contraction step
constexpr int NT = 256;  // threads: 16 x 16, each R x R outputs

// Tile (16 R) x (16 R): R = 4 (64 x 64) for large launches; small launches
// take R = 2 or 1 so that they still spread over the SMs (on GB300 one SM
// issues only about 2 DFMA per clock, so a lone 64 x 64 FP64 tile is slow).
// block sum over the NT threads (every thread gets the total)
__device__ __forceinline__ double block_sum_nt(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
#pragma unroll
  for (int i = 0; i < NT / 32; ++i) t += red[i];
  return t;
}

template <typename T, int EPI, int R>
__global__ void __launch_bounds__(NT)
    k_contract_simt(const jfg_contract_desc d, const T* __restrict__ op,
                    const T* __restrict__ in, T* __restrict__ out, T* __restrict__ aux = nullptr,
                    float* __restrict__ aux32 = nullptr, double* __restrict__ part = nullptr) {
  constexpr int TM = 16 * R;  // rows of the operator per CTA
  constexpr int TP = 16 * R;  // columns (p) per CTA
  __shared__ T As[TK][TM + 4];
  __shared__ T Bs[TK][TP + 4];

  const int bz = blockIdx.z;
  const int slot = bz / d.nseg;
  const int s = bz - slot * d.nseg;
  const int b = active_problem(d.batch_list, active_count(d.batch_list, d.batch_count, d.batch),
                               d.batch, slot);
  if (b < 0) return;
  const int m0 = blockIdx.y * TM;
  const int p0 = blockIdx.x * TP;
  const T* opS = op + (long long)s * d.op_seg;
  const T* inS = in + (long long)b * d.in_batch + (long long)s * d.in_seg;

  const int tid = threadIdx.x;
  const int tx = tid & 15;
  const int ty = tid >> 4;

  T acc[R][R];
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int j = 0; j < R; ++j) acc[i][j] = T(0);

  for (int k0 = 0; k0 < d.K; k0 += TK) {
#pragma unroll
    for (int i = 0; i < (TM * TK) / NT; ++i) {
      const int idx = tid + i * NT;
      const int r = idx / TK;
      const int kk = idx % TK;
      const int m = m0 + r, k = k0 + kk;
      As[kk][r] = (m < d.M && k < d.K) ? opS[(long long)m * d.op_ld + k] : T(0);
      const int p = p0 + r;
      Bs[kk][r] = (p < d.P && k < d.K) ? inS[(long long)p * d.in_ld + k] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      T a[R], bb[R];
#pragma unroll
      for (int i = 0; i < R; ++i) a[i] = As[kk][ty * R + i];
#pragma unroll
      for (int j = 0; j < R; ++j) bb[j] = Bs[kk][tx * R + j];
#pragma unroll
      for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < R; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
    }
    __syncthreads();
  }

  T* outS = out + (long long)b * d.out_batch + (long long)s * d.out_seg;
  const T alpha = T(d.alpha);
  const T beta = T(d.beta);
  if constexpr (EPI == EPI_EXP_WEIGHT) {
    // kappa = exp(scale (v - shift)), kw = kappa wm[m] wp[p] (FP64, optional
    // FP32 copy at the field strides); kappa itself into aux when given
    const T sh = d.c0 ? ((const T*)d.c0)[b] : T(0);
    const T sc = d.c1 ? ((const T*)d.c1)[b] : T(1);
    T* auxS = aux ? aux + (long long)b * d.out_batch + (long long)s * d.out_seg : nullptr;
    float* a32 = aux32 ? aux32 + (long long)b * d.field_batch + (long long)s * d.field_seg
                       : nullptr;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int m = m0 + ty * R + i;
      if (m >= d.M) continue;
      const T wm = ((const T*)d.lam_m)[m];
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const int p = p0 + tx * R + j;
        if (p >= d.P) continue;
        const T k = exp(sc * (alpha * acc[i][j] - sh));
        const T v = k * wm * ((const T*)d.lam_p)[p];
        outS[(long long)m * d.out_ld + p] = v;
        if (auxS) auxS[(long long)m * d.out_ld + p] = k;
        if (a32) a32[(long long)m * d.field_ld + p] = (float)v;
      }
    }
  } else if constexpr (EPI == EPI_MOMENTS) {
    // out = alpha v, and this tile's count, mean and sum of squared
    // deviations (two passes over the registers) at part[b][tile][3]
    __shared__ double red[NT / 32];
    double cnt = 0.0, sum = 0.0;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int m = m0 + ty * R + i;
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const int p = p0 + tx * R + j;
        if (m < d.M && p < d.P) {
          const T v = alpha * acc[i][j];
          outS[(long long)m * d.out_ld + p] = v;
          cnt += 1.0;
          sum += (double)v;
        }
      }
    }
    const double n_t = block_sum_nt(cnt, red);
    const double mu = n_t > 0.0 ? block_sum_nt(sum, red) / n_t : 0.0;
    double q = 0.0;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int m = m0 + ty * R + i;
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const int p = p0 + tx * R + j;
        if (m < d.M && p < d.P) {
          const double dv = (double)(alpha * acc[i][j]) - mu;
          q = fma(dv, dv, q);
        }
      }
    }
    const double m2 = block_sum_nt(q, red);
    if (threadIdx.x == 0) {
      const long long tiles = (long long)gridDim.x * gridDim.y * d.nseg;
      const long long t = ((long long)s * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
      double* pt = part + ((long long)b * tiles + t) * 3;
      pt[0] = n_t;
      pt[1] = mu;
      pt[2] = m2;
    }
  } else {
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int m = m0 + ty * R + i;
      if (m >= d.M) continue;
      T denom_m = T(0), c0 = T(0), c1 = T(1);
      if (EPI == JFG_EPI_DIV_EIG) {
        denom_m = ((const T*)d.lam_m)[m];
        c0 = d.c0 ? ((const T*)d.c0)[b] : T(0);
        c1 = d.c1 ? ((const T*)d.c1)[b] : T(1);
      }
#pragma unroll
      for (int j = 0; j < R; ++j) {
        const int p = p0 + tx * R + j;
        if (p >= d.P) continue;
        T v = acc[i][j];
        if (EPI == JFG_EPI_MUL_FIELD) {
          const T* f = (const T*)d.field;
          v *= f[(long long)b * d.field_batch + (long long)s * d.field_seg +
                 (long long)m * d.field_ld + p];
        } else if (EPI == JFG_EPI_DIV_EIG) {
          v = v / (c0 + c1 * (denom_m + ((const T*)d.lam_p)[p]));
        }
        T* o = outS + (long long)m * d.out_ld + p;
        v = alpha * v;
        if (beta != T(0)) v += beta * *o;
        *o = v;
      }
    }
  }
}

// 128 x 128 tiles for FP32 only (64 FP64 accumulators would not fit)
template <typename T, int E>
void launch_r8(dim3 grid, const jfg_contract_desc& d, const T* op, const T* in, T* out,
               cudaStream_t st) {
  if constexpr (std::is_same<T, float>::value)
    k_contract_simt<T, E, 8><<<grid, NT, 0, st>>>(d, op, in, out);
}

template <typename T>
int launch_simt(const jfg_contract_desc& d, const T* op, const T* in, T* out,
                cudaStream_t st) {
  JFG_TRY(validate_desc(d));
  if (!op || !in || !out) return JFG_ERR_ARG;
  if (d.batch == 0 || d.M == 0 || d.P == 0) return JFG_OK;
  const long long gz = (long long)d.batch * d.nseg;
  if (gz > 65535) return JFG_ERR_ARG;
  if (d.epilogue != JFG_EPI_NONE && d.epilogue != JFG_EPI_MUL_FIELD &&
      d.epilogue != JFG_EPI_DIV_EIG)
    return JFG_ERR_ARG;
  // largest tile that still gives two CTAs per SM (the list-restricted
  // launches count their full batch: the active count is not known here)
  static int nsm[64] = {};
  int dev = 0;
  JFG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return JFG_ERR_UNSUPPORTED;
  if (!nsm[dev]) JFG_CUDA_TRY(cudaDeviceGetAttribute(&nsm[dev], cudaDevAttrMultiProcessorCount, dev));
  auto ctas = [&](int t) {
    return (long long)((d.P + t - 1) / t) * ((d.M + t - 1) / t) * gz;
  };
  // FP32 launches big enough for 128 x 128 tiles take them (8 x 8 outputs per
  // thread: half the shared-memory loads per FMA of the 64 x 64 tile)
  const bool r8 = std::is_same<T, float>::value && ctas(128) >= 2 * nsm[dev];
  const int R = r8 ? 8 : ctas(64) >= 2 * nsm[dev] ? 4 : ctas(32) >= 2 * nsm[dev] ? 2 : 1;
  const int tile = 16 * R;
  dim3 grid((d.P + tile - 1) / tile, (d.M + tile - 1) / tile, (unsigned)gz);
  if (grid.y > 65535) return JFG_ERR_ARG;
#define JFG_SIMT_LAUNCH(E)                                                         \
  if (R == 8)                                                                     \
    launch_r8<T, E>(grid, d, op, in, out, st);                                    \
  else if (R == 4)                                                                \
    k_contract_simt<T, E, 4><<<grid, NT, 0, st>>>(d, op, in, out);                \
  else if (R == 2)                                                                \
    k_contract_simt<T, E, 2><<<grid, NT, 0, st>>>(d, op, in, out);                \
  else                                                                            \
    k_contract_simt<T, E, 1><<<grid, NT, 0, st>>>(d, op, in, out)
  switch (d.epilogue) {
    case JFG_EPI_NONE:
      JFG_SIMT_LAUNCH(JFG_EPI_NONE);
      break;
    case JFG_EPI_MUL_FIELD:
      JFG_SIMT_LAUNCH(JFG_EPI_MUL_FIELD);
      break;
    default:
      JFG_SIMT_LAUNCH(JFG_EPI_DIV_EIG);
      break;
  }
#undef JFG_SIMT_LAUNCH
  JFG_CHECK_LAUNCH();
  count_launches(1);
  return JFG_OK;
}

}  // namespace

// Last pass of a backward transform with a coefficient epilogue (FP64,
// internal: not reachable through jfg_contract_*).  EPI_EXP_WEIGHT: out = kw
// (lam_m, lam_p the per-row and per-column quadrature weights, c0 / c1 the
// per-problem shift / scale), aux = kappa, aux32 = FP32 kw.  EPI_MOMENTS: out
// = the values, part = (count, mean, M2) per tile; *tiles = tiles per problem.
int contract_f64_coef(const jfg_contract_desc& d, int kind, const double* op, const double* in,
                      double* out, double* aux, float* aux32, double* part, long long* tiles,
                      cudaStream_t st) {
  if ((kind != EPI_EXP_WEIGHT && kind != EPI_MOMENTS) || !op || !in || !out) return JFG_ERR_ARG;
  if (d.batch < 0 || d.nseg < 1 || d.M < 0 || d.P < 0 || d.K < 1 || d.op_ld < d.K ||
      d.in_ld < d.K || d.out_ld < d.P || d.batch_list || d.beta != 0.0)
    return JFG_ERR_ARG;
  if (kind == EPI_EXP_WEIGHT && (!d.lam_m || !d.lam_p || (aux32 && d.field_ld < d.P)))
    return JFG_ERR_ARG;
  if (kind == EPI_MOMENTS && !part) return JFG_ERR_ARG;
  const long long gz = (long long)d.batch * d.nseg;
  if (gz > 65535) return JFG_ERR_ARG;
  constexpr int tile = 64;  // R = 4
  const dim3 grid((d.P + tile - 1) / tile, (d.M + tile - 1) / tile, (unsigned)gz);
  if (grid.y > 65535) return JFG_ERR_ARG;
  if (tiles) *tiles = (long long)grid.x * grid.y * d.nseg;
  if (gz == 0 || d.M == 0 || d.P == 0) return JFG_OK;
  if (kind == EPI_EXP_WEIGHT)
    k_contract_simt<double, EPI_EXP_WEIGHT, 4><<<grid, NT, 0, st>>>(d, op, in, out, aux, aux32,
                                                                     nullptr);
  else
    k_contract_simt<double, EPI_MOMENTS, 4><<<grid, NT, 0, st>>>(d, op, in, out, nullptr,
                                                                  nullptr, part);
  JFG_CHECK_LAUNCH();
  count_launches(1);
  return JFG_OK;
}

int validate_desc(const jfg_contract_desc& d) {
  if (d.batch < 0 || d.nseg < 1 || d.M < 0 || d.P < 0 || d.K < 1) return JFG_ERR_ARG;
  if (d.op_ld < d.K || d.in_ld < d.K || d.out_ld < d.P) return JFG_ERR_ARG;
  if (d.epilogue == JFG_EPI_MUL_FIELD && (!d.field || d.field_ld < d.P)) return JFG_ERR_ARG;
  if (d.epilogue == JFG_EPI_DIV_EIG && (!d.lam_m || !d.lam_p)) return JFG_ERR_ARG;
  if (d.epilogue < 0 || d.epilogue > 2) return JFG_ERR_ARG;
  if ((d.batch_list == nullptr) != (d.batch_count == nullptr)) return JFG_ERR_ARG;
  return JFG_OK;
}

int contract_f64(const jfg_contract_desc& d, const double* op, const double* in, double* out,
                 cudaStream_t st) {
  return launch_simt<double>(d, op, in, out, st);
}

int contract_f32(const jfg_contract_desc& d, const float* op, const float* in, float* out,
                 cudaStream_t st) {
  return launch_simt<float>(d, op, in, out, st);
}

}  // namespace jfg

extern "C" int jfg_contract_f64(const jfg_contract_desc* d, const double* op, const double* in,
                                double* out, void* stream) {
  if (!d) return JFG_ERR_ARG;
  return jfg::contract_f64(*d, op, in, out, (cudaStream_t)stream);
}

extern "C" int jfg_contract_f32(const jfg_contract_desc* d, const float* op, const float* in,
                                float* out, void* stream) {
  if (!d) return JFG_ERR_ARG;
  return jfg::contract_f32(*d, op, in, out, (cudaStream_t)stream);
}
