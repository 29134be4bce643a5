// Per-axis contraction in double-FP32 ("double-float") arithmetic on the FP32
// CUDA cores, FP64 in and out:
//
//   out[b][s][m][p] = alpha * epi(sum_k op[s][m][k] * in[b][s][p][k]) + beta * out
//
// GB300 issues about 2 FP64 FMAs per clock per SM but 128 FP32 FMAs.  Each
// FP64 operand is split into an unevaluated sum hi + lo of two FP32 values
// (48 significant bits), every product is formed error-free from FP32 FMAs
// (TwoProduct: p = a_hi b_hi, e = fma(a_hi, b_hi, -p) + a_hi b_lo + a_lo b_hi)
// and accumulated with Knuth's TwoSum into an (s_hi, s_lo) pair -- 11 FP32
// operations per multiply-add instead of one FP64 FMA at 1/64 of the rate.
// Relative error per product is about 2^-46, so a K-term sum carries about
// sqrt(K) 2^-46 relative to its terms: ample for the FP64 residual of
// iterative refinement, whose target is 1e-11 of the right-hand side.  (The
// algorithms are Dekker's and Knuth's error-free transformations, as used in
// the double-double literature.)
#include "jfg_internal.cuh"

namespace jfg {

namespace {

constexpr int TM = 64;   // operator rows per CTA
constexpr int TP = 64;   // p columns per CTA
constexpr int TK = 16;   // contraction step
constexpr int NT = 256;  // 16 x 16 threads, 4 x 4 outputs each

__device__ __forceinline__ void split2(double v, float& h, float& l) {
  h = __double2float_rn(v);
  l = __double2float_rn(v - (double)h);
}

// (sh, sl) += (ah + al) (bh + bl).  The _rn intrinsics keep the compiler from
// contracting a multiply and an add into one FMA, which would break TwoSum.
__device__ __forceinline__ void df_mac(float ah, float al, float bh, float bl, float& sh,
                                       float& sl) {
  const float p = __fmul_rn(ah, bh);
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  const float t = __fadd_rn(sh, p);
  const float v = __fsub_rn(t, sh);
  const float w = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, v)), __fsub_rn(p, v));
  sl = __fadd_rn(sl, __fadd_rn(w, e));
  sh = t;
}

__global__ void k_split_pairs(const double* __restrict__ src, float2* __restrict__ dst,
                              long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    float h, l;
    split2(src[i], h, l);
    dst[i] = make_float2(h, l);
  }
}

// op_pairs (optional): the operator pre-split into (hi, lo) pairs, so the
// operator tile, which every p tile reloads, costs no FP64 work per load
// in_pairs / out_pairs: the input / output arrays hold (hi, lo) FP32 pairs
// (8 bytes, the same element indexing as FP64): a chain of passes keeps its
// intermediates split, so no tile load needs FP64 work
template <int EPI>
__global__ void __launch_bounds__(NT)
    k_contract_df(const jfg_contract_desc d, const double* __restrict__ op,
                  const float2* __restrict__ op_pairs, const double* __restrict__ in,
                  double* __restrict__ out, bool in_pairs, bool out_pairs) {
  __shared__ __align__(16) float Ah[TK][TM + 4], Al[TK][TM + 4];
  __shared__ __align__(16) float Bh[TK][TP + 4], Bl[TK][TP + 4];

  const int bz = blockIdx.z;
  const int slot = bz / d.nseg;
  const int s = bz - slot * d.nseg;
  const int b = active_problem(d.batch_list, active_count(d.batch_list, d.batch_count, d.batch),
                               d.batch, slot);
  if (b < 0) return;
  const int m0 = blockIdx.y * TM;
  const int p0 = blockIdx.x * TP;
  const double* opS = op + (long long)s * d.op_seg;
  const double* inS = in + (long long)b * d.in_batch + (long long)s * d.in_seg;

  const int tid = threadIdx.x;
  const int tx = tid & 15;
  const int ty = tid >> 4;

  float sh[4][4], sl[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) sh[i][j] = sl[i][j] = 0.f;

  for (int k0 = 0; k0 < d.K; k0 += TK) {
#pragma unroll
    for (int i = 0; i < (TM * TK) / NT; ++i) {
      const int idx = tid + i * NT;
      const int r = idx / TK;
      const int kk = idx % TK;
      const int m = m0 + r, k = k0 + kk;
      float h, l;
      if (op_pairs) {
        const float2 t = (m < d.M && k < d.K)
                             ? op_pairs[(long long)s * d.op_seg + (long long)m * d.op_ld + k]
                             : make_float2(0.f, 0.f);
        h = t.x;
        l = t.y;
      } else {
        split2((m < d.M && k < d.K) ? opS[(long long)m * d.op_ld + k] : 0.0, h, l);
      }
      Ah[kk][r] = h;
      Al[kk][r] = l;
      const int p = p0 + r;
      if (in_pairs) {
        const float2 t = (p < d.P && k < d.K)
                             ? ((const float2*)inS)[(long long)p * d.in_ld + k]
                             : make_float2(0.f, 0.f);
        h = t.x;
        l = t.y;
      } else {
        split2((p < d.P && k < d.K) ? inS[(long long)p * d.in_ld + k] : 0.0, h, l);
      }
      Bh[kk][r] = h;
      Bl[kk][r] = l;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      const float4 ah = *(const float4*)&Ah[kk][ty * 4];
      const float4 al = *(const float4*)&Al[kk][ty * 4];
      const float4 bh = *(const float4*)&Bh[kk][tx * 4];
      const float4 bl = *(const float4*)&Bl[kk][tx * 4];
      const float a_h[4] = {ah.x, ah.y, ah.z, ah.w}, a_l[4] = {al.x, al.y, al.z, al.w};
      const float b_h[4] = {bh.x, bh.y, bh.z, bh.w}, b_l[4] = {bl.x, bl.y, bl.z, bl.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) df_mac(a_h[i], a_l[i], b_h[j], b_l[j], sh[i][j], sl[i][j]);
    }
    // renormalise each accumulator pair (FastTwoSum, |sh| >= |sl|)
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float t = __fadd_rn(sh[i][j], sl[i][j]);
        sl[i][j] = __fsub_rn(sl[i][j], __fsub_rn(t, sh[i][j]));
        sh[i][j] = t;
      }
    __syncthreads();
  }

  double* outS = out + (long long)b * d.out_batch + (long long)s * d.out_seg;
  const double alpha = d.alpha, beta = d.beta;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= d.M) continue;
    double lm = 0.0, c0 = 0.0, c1 = 1.0;
    if (EPI == JFG_EPI_DIV_EIG) {
      lm = ((const double*)d.lam_m)[m];
      c0 = d.c0 ? ((const double*)d.c0)[b] : 0.0;
      c1 = d.c1 ? ((const double*)d.c1)[b] : 1.0;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int p = p0 + tx * 4 + j;
      if (p >= d.P) continue;
      double v = (double)sh[i][j] + (double)sl[i][j];
      if (EPI == JFG_EPI_MUL_FIELD) {
        v *= ((const double*)d.field)[(long long)b * d.field_batch +
                                      (long long)s * d.field_seg +
                                      (long long)m * d.field_ld + p];
      } else if (EPI == JFG_EPI_DIV_EIG) {
        v = v / (c0 + c1 * (lm + ((const double*)d.lam_p)[p]));
      }
      double* o = outS + (long long)m * d.out_ld + p;
      v = alpha * v;
      if (out_pairs) {
        float2* o2 = (float2*)o;
        if (beta != 0.0) {
          const float2 t = *o2;
          v += beta * ((double)t.x + (double)t.y);
        }
        float h, l;
        split2(v, h, l);
        *o2 = make_float2(h, l);
      } else {
        if (beta != 0.0) v += beta * *o;
        *o = v;
      }
    }
  }
}

}  // namespace

int split_pairs_f64(const double* src, float2* dst, long long n, cudaStream_t st) {
  if (n < 0 || (n > 0 && (!src || !dst))) return JFG_ERR_ARG;
  if (n == 0) return JFG_OK;
  long long blocks = (n + 255) / 256;
  if (blocks > 4 * 152) blocks = 4 * 152;
  k_split_pairs<<<(int)blocks, 256, 0, st>>>(src, dst, n);
  JFG_LAUNCHED();
  return JFG_OK;
}

int contract_df64(const jfg_contract_desc& d, const double* op, const float2* op_pairs,
                  const double* in, double* out, cudaStream_t st, bool in_pairs,
                  bool out_pairs) {
  JFG_TRY(validate_desc(d));
  if (!op || !in || !out) return JFG_ERR_ARG;
  if (d.batch == 0 || d.M == 0 || d.P == 0) return JFG_OK;
  const long long gz = (long long)d.batch * d.nseg;
  if (gz > 65535) return JFG_ERR_ARG;
  dim3 grid((d.P + TP - 1) / TP, (d.M + TM - 1) / TM, (unsigned)gz);
  if (grid.y > 65535) return JFG_ERR_ARG;
  switch (d.epilogue) {
    case JFG_EPI_NONE:
      k_contract_df<JFG_EPI_NONE><<<grid, NT, 0, st>>>(d, op, op_pairs, in, out, in_pairs,
                                                        out_pairs);
      break;
    case JFG_EPI_MUL_FIELD:
      k_contract_df<JFG_EPI_MUL_FIELD><<<grid, NT, 0, st>>>(d, op, op_pairs, in, out,
                                                             in_pairs, out_pairs);
      break;
    case JFG_EPI_DIV_EIG:
      k_contract_df<JFG_EPI_DIV_EIG><<<grid, NT, 0, st>>>(d, op, op_pairs, in, out, in_pairs,
                                                           out_pairs);
      break;
    default:
      return JFG_ERR_ARG;
  }
  JFG_LAUNCHED();
  return JFG_OK;
}

}  // namespace jfg

extern "C" int jfg_contract_df64(const jfg_contract_desc* d, const double* op, const double* in,
                                 double* out, void* stream) {
  if (!d) return JFG_ERR_ARG;
  return jfg::contract_df64(*d, op, nullptr, in, out, (cudaStream_t)stream);
}
