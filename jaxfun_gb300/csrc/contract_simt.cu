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
template <typename T, int EPI, int R>
__global__ void __launch_bounds__(NT)
    k_contract_simt(const jfg_contract_desc d, const T* __restrict__ op,
                    const T* __restrict__ in, T* __restrict__ out) {
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
