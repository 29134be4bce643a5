// BF16 tensor-core GEMM with fused epilogues for the spectral neural operator
// (training and inference).
//
//   D[b][m][n] = alpha * sum_k A[b][m][k] B[b][n][k]      (kind::f16, BF16 in, FP32 TMEM)
//
// One CTA computes a 128 x N tile (N <= 256): TMA loads 64-wide K blocks of A
// and B (128-byte swizzle) into a multi-stage ring, one thread issues
// tcgen05.mma (4 x K=16 per block) into a TMEM accumulator, four epilogue warps
// read it back with tcgen05.ld (one TMEM lane quarter each; thread = row m) and
// apply add / bias / GELU-derivative / GELU, writing any of FP32 row-major
// (optionally atomically, for split-K), BF16 row-major and BF16 transposed.
#include <cuda_bf16.h>
#include <math.h>

#include "tc_common.cuh"

namespace jfg {

__device__ int g_gemm_status = 0;

EncodeTiledFn tensor_map_encoder() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

namespace {

constexpr int TM = 128;
constexpr int KBE = 64;  // BF16 elements per K block (128 B)
constexpr int NTH = 192;
constexpr uint32_t ABYTES = TM * KBE * 2;  // 16 KB

struct GemmParams {
  jfg_gemm_desc d;
  int Nt, stages, tmem_cols, kb_per_split, a_bat, b_bat;
  int nb;              // samples per CTA: B tiles of nb consecutive samples side by side (N = nb * Nt)
  int a_perm, b_perm;  // 1: tensor map dims ordered (K, batch, rows)
  int vec_ok;          // 1: every row-major operand allows 16-byte vector access
};

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
         x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__global__ void __launch_bounds__(NTH, 1)
    k_gemm_bf16(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                const __grid_constant__ GemmParams prm) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const jfg_gemm_desc& d = prm.d;
  const int Nt = prm.Nt, S = prm.stages, NB = prm.nb;
  const uint32_t bbytes = (uint32_t)(NB * Nt) * KBE * 2;
  const uint32_t bbytes1 = (uint32_t)Nt * KBE * 2;  // one sample's B tile
  const uint32_t stage_bytes = ABYTES + bbytes;
  uint64_t* full = (uint64_t*)(smem + (size_t)S * stage_bytes);
  uint64_t* empty = full + S;
  uint64_t* accum = full + 2 * S;
  uint32_t* tmem_slot = (uint32_t*)(full + 2 * S + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * TM;
  const int b0 = blockIdx.y * NB;  // first sample of this CTA
  const int nkb_all = (d.K + KBE - 1) / KBE;
  const int kb0 = blockIdx.z * prm.kb_per_split;
  const int kb1 = min(nkb_all, kb0 + prm.kb_per_split);
  const int nkb = kb1 > kb0 ? kb1 - kb0 : 0;

  if (threadIdx.x == 0) {
    for (int i = 0; i < S; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    tc::mbar_init(accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc::smem_u32(tmem_slot)),
                 "r"(prm.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0 && nkb > 0) {
      int issued = 0;
      int st = 0;       // i % S, kept running (no division per K block)
      uint32_t ph = 0;  // (i / S) & 1
      for (int i = 0; i < nkb; ++i) {
        if (i >= S && !tc::mbar_wait(&empty[st], ph ^ 1u, &g_gemm_status)) break;
        uint8_t* sa = smem + (size_t)st * stage_bytes;
        tc::mbar_expect_tx(&full[st], stage_bytes);
        const int ab = prm.a_bat ? b0 : 0, bb = prm.b_bat ? b0 : 0;
        if (prm.a_perm)
          tc::tma_load_3d(sa, &tmA, &full[st], (kb0 + i) * KBE, ab, m0);
        else
          tc::tma_load_3d(sa, &tmA, &full[st], (kb0 + i) * KBE, m0, ab);
        for (int j = 0; j < NB; ++j) {  // sample j's rows follow sample j-1's
          uint8_t* sbj = sa + ABYTES + (size_t)j * bbytes1;
          if (prm.b_perm)
            tc::tma_load_3d(sbj, &tmB, &full[st], (kb0 + i) * KBE, bb + j, 0);
          else
            tc::tma_load_3d(sbj, &tmB, &full[st], (kb0 + i) * KBE, 0, bb + j);
        }
        issued = i + 1;
        if (++st == S) {
          st = 0;
          ph ^= 1u;
        }
      }
      for (int i = (issued > S ? issued - S : 0); i < issued; ++i)
        tc::mbar_wait(&full[i % S], (uint32_t)(i / S) & 1u, &g_gemm_status);
    }
  } else if (warp == 1) {
    if (lane == 0 && nkb > 0) {
      const uint32_t idesc = tc::idesc_bf16(TM, NB * Nt);
      bool ok = true;
      int st = 0;       // i % S
      uint32_t ph = 0;  // (i / S) & 1
      for (int i = 0; i < nkb; ++i) {
        if (!tc::mbar_wait(&full[st], ph, &g_gemm_status)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t sa = tc::smem_u32(smem + (size_t)st * stage_bytes);
        const uint32_t sb = sa + ABYTES;
#pragma unroll
        for (int kk = 0; kk < KBE / 16; ++kk) {
          const uint32_t off = kk * 32;  // 16 BF16 = 32 B per MMA
          tc::mma_bf16(tmem, tc::sdesc_sw128(sa + off), tc::sdesc_sw128(sb + off), idesc,
                       (i | kk) ? 1u : 0u);
        }
        tc::mma_commit(&empty[st]);
        if (++st == S) {
          st = 0;
          ph ^= 1u;
        }
      }
      if (ok) tc::mma_commit(accum);
    }
  } else if (nkb > 0) {
    // ---------------- epilogue ----------------
    const int q = warp & 3;
    const int m = m0 + 32 * q + lane;
    if (tc::mbar_wait(accum, 0, &g_gemm_status)) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const bool mok = m < d.M;
      const bool split = prm.kb_per_split < nkb_all || d.d32_accumulate;
      for (int cc = 0; cc < NB * Nt / 16; ++cc) {
        float v[16];
        tc::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(cc * 16), v);
        if (!mok) continue;
        // TMEM columns [j Nt, (j+1) Nt) belong to sample b0 + j (Nt % 16 == 0)
        const int b = b0 + (cc * 16) / Nt;
        const int c = ((cc * 16) % Nt) / 16;
        if (!split && c * 16 + 16 <= d.N && prm.vec_ok) {
          // whole 16-column group of this thread's row: 16-byte vector accesses
          const int n0 = c * 16;
          float r[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) r[j] = d.alpha * v[j];
          if (d.add) {
            const float4* a4 = (const float4*)(d.add + (long long)b * d.add_batch +
                                                (long long)m * d.ld_add + n0);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const float4 t = a4[j];
              r[4 * j] += t.x, r[4 * j + 1] += t.y, r[4 * j + 2] += t.z, r[4 * j + 3] += t.w;
            }
          }
          if (d.bias) {
#pragma unroll
            for (int j = 0; j < 16; ++j) r[j] += d.bias[n0 + j];
          }
          if (d.gg) {
            const float4* g4 = (const float4*)(d.gg + (long long)b * d.gg_batch +
                                                (long long)m * d.ld_gg + n0);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const float4 t = g4[j];
              r[4 * j] *= gelu_grad(t.x), r[4 * j + 1] *= gelu_grad(t.y);
              r[4 * j + 2] *= gelu_grad(t.z), r[4 * j + 3] *= gelu_grad(t.w);
            }
          }
          if (d.pre) {
            float4* p4 = (float4*)(d.pre + (long long)b * d.pre_batch + (long long)m * d.ld_pre + n0);
#pragma unroll
            for (int j = 0; j < 4; ++j)
              p4[j] = make_float4(r[4 * j], r[4 * j + 1], r[4 * j + 2], r[4 * j + 3]);
          }
          if (d.act == 1) {
#pragma unroll
            for (int j = 0; j < 16; ++j) r[j] = gelu(r[j]);
          }
          if (d.d32) {
            float4* o4 = (float4*)(d.d32 + (long long)b * d.d32_batch + (long long)m * d.ld_d32 + n0);
#pragma unroll
            for (int j = 0; j < 4; ++j)
              o4[j] = make_float4(r[4 * j], r[4 * j + 1], r[4 * j + 2], r[4 * j + 3]);
          }
          if (d.dbf || d.dtbf) {
            __nv_bfloat16 h[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) h[j] = __float2bfloat16(r[j]);
            if (d.dbf) {
              uint32_t w[8];
#pragma unroll
              for (int j = 0; j < 8; ++j)
                w[j] = (uint32_t)__bfloat16_as_ushort(h[2 * j]) |
                       ((uint32_t)__bfloat16_as_ushort(h[2 * j + 1]) << 16);
              uint4* o = (uint4*)((__nv_bfloat16*)d.dbf + (long long)b * d.dbf_batch +
                                  (long long)m * d.ld_dbf + n0);
              o[0] = make_uint4(w[0], w[1], w[2], w[3]);
              o[1] = make_uint4(w[4], w[5], w[6], w[7]);
            }
            if (d.dtbf) {
              __nv_bfloat16* t = (__nv_bfloat16*)d.dtbf + (long long)b * d.dtbf_batch + m;
#pragma unroll
              for (int j = 0; j < 16; ++j) t[(long long)(n0 + j) * d.ld_dtbf] = h[j];
            }
          }
          continue;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = c * 16 + j;
          if (n >= d.N) break;
          float r = d.alpha * v[j];
          if (!split) {
            if (d.add) r += d.add[(long long)b * d.add_batch + (long long)m * d.ld_add + n];
            if (d.bias) r += d.bias[n];
            if (d.gg)
              r *= gelu_grad(d.gg[(long long)b * d.gg_batch + (long long)m * d.ld_gg + n]);
            if (d.pre) d.pre[(long long)b * d.pre_batch + (long long)m * d.ld_pre + n] = r;
            if (d.act == 1) r = gelu(r);
            if (d.d32) d.d32[(long long)b * d.d32_batch + (long long)m * d.ld_d32 + n] = r;
          } else if (d.d32) {
            atomicAdd(d.d32 + (long long)b * d.d32_batch + (long long)m * d.ld_d32 + n, r);
          }
          if (!split) {
            const __nv_bfloat16 h = __float2bfloat16(r);
            if (d.dbf)
              ((__nv_bfloat16*)d.dbf)[(long long)b * d.dbf_batch + (long long)m * d.ld_dbf + n] = h;
            if (d.dtbf)
              ((__nv_bfloat16*)d.dtbf)[(long long)b * d.dtbf_batch + (long long)n * d.ld_dtbf + m] = h;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(prm.tmem_cols)
                 : "memory");
  }
}

// 3-D BF16 tensor map over (K, rows, batch); when the batch stride is smaller
// than the row stride (samples interleaved inside each row) the dimensions are
// ordered (K, batch, rows) so that strides increase, with a box of one sample.
int make_map_bf16(CUtensorMap* map, const void* base, cuuint64_t K, cuuint64_t rows,
                  cuuint64_t nb, cuuint64_t ld, cuuint64_t bstride, cuuint32_t box_rows,
                  bool perm) {
  EncodeTiledFn fn = tensor_map_encoder();
  if (!fn) return JFG_ERR_UNSUPPORTED;
  cuuint64_t dims[3] = {K, rows, nb};
  cuuint64_t str[2] = {ld * 2, bstride * 2};
  cuuint32_t box[3] = {KBE, box_rows, 1};
  if (perm) {
    dims[1] = nb;
    dims[2] = rows;
    str[0] = bstride * 2;
    str[1] = ld * 2;
    box[1] = 1;
    box[2] = box_rows;
  }
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void*)base, dims, str, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? JFG_OK : JFG_ERR_ARG;
}

}  // namespace

}  // namespace jfg

extern "C" int jfg_gemm_bf16(const jfg_gemm_desc* dp, const void* A, const void* B,
                             void* stream) {
  using namespace jfg;
  if (!dp || !A || !B) return JFG_ERR_ARG;
  const jfg_gemm_desc& d = *dp;
  if (d.batch < 0 || d.M < 0 || d.N < 1 || d.N > 256 || d.K < 1 || d.ksplit < 1 ||
      d.ksplit > 1024)
    return JFG_ERR_ARG;
  if (d.batch == 0 || d.M == 0) return JFG_OK;
  if ((d.lda & 7) || (d.ldb & 7) || (d.a_batch & 7) || (d.b_batch & 7) || d.lda < d.K ||
      d.ldb < d.K)
    return JFG_ERR_ARG;
  if (((uintptr_t)A & 15) || ((uintptr_t)B & 15)) return JFG_ERR_ARG;
  if (d.ksplit > 1 && (d.add || d.bias || d.gg || d.act || d.pre || d.dbf || d.dtbf || !d.d32))
    return JFG_ERR_ARG;
  if (d.batch > 65535) return JFG_ERR_ARG;
  GemmParams prm;
  prm.d = d;
  prm.Nt = (d.N + 15) / 16 * 16;
  const int nkb = (d.K + KBE - 1) / KBE;
  prm.kb_per_split = (nkb + d.ksplit - 1) / d.ksplit;
  prm.a_bat = (d.batch > 1 && d.a_batch != 0) ? 1 : 0;
  prm.b_bat = (d.batch > 1 && d.b_batch != 0) ? 1 : 0;
  // A shared by every sample and narrow per-sample B (the spectral transforms:
  // N = 64 channels): up to 256 / N samples per CTA in one N <= 256 MMA, so
  // the shared A tile is staged once for all of them
  prm.nb = 1;
  if (prm.b_bat && !prm.a_bat && d.ksplit == 1 && d.N % 16 == 0)
    for (int nb = 256 / d.N; nb > 1; --nb)
      if (d.batch % nb == 0) {
        prm.nb = nb;
        break;
      }
  const int ntot = prm.nb * prm.Nt;
  int cols = 32;
  while (cols < ntot) cols <<= 1;
  prm.tmem_cols = cols;
  const size_t stage = ABYTES + (size_t)ntot * KBE * 2;
  // pipeline depth: no deeper than the K blocks a CTA has (the channel-mixing
  // GEMMs have one, so several CTAs share an SM and their epilogues overlap);
  // long-K GEMMs keep >= 3 stages but leave room for a second CTA per SM
  int stages = (int)((200 * 1024) / stage);
  if (stages > 6) stages = 6;
  const int two_per_sm = (int)((113 * 1024 - 1100) / stage);
  if (stages > 3 && two_per_sm >= 3 && two_per_sm < stages) stages = two_per_sm;
  if (stages > prm.kb_per_split) stages = prm.kb_per_split;
  if (stages < 1) stages = 1;
  prm.stages = stages;
  const int ksplit = (nkb + prm.kb_per_split - 1) / prm.kb_per_split;
  {
    auto f4 = [](const void* p, long long ld, long long bs) {
      return p == nullptr || ((((uintptr_t)p) & 15) == 0 && (ld & 3) == 0 && (bs & 3) == 0);
    };
    auto h8 = [](const void* p, long long ld, long long bs) {
      return p == nullptr || ((((uintptr_t)p) & 15) == 0 && (ld & 7) == 0 && (bs & 7) == 0);
    };
    prm.vec_ok = f4(d.add, d.ld_add, d.add_batch) && f4(d.gg, d.ld_gg, d.gg_batch) &&
                 f4(d.pre, d.ld_pre, d.pre_batch) && f4(d.d32, d.ld_d32, d.d32_batch) &&
                 h8(d.dbf, d.ld_dbf, d.dbf_batch);
  }
  prm.a_perm = (prm.a_bat && d.a_batch < d.lda) ? 1 : 0;
  prm.b_perm = (prm.b_bat && d.b_batch < d.ldb) ? 1 : 0;
  if ((prm.a_perm && d.a_batch < d.K) || (prm.b_perm && d.b_batch < d.K)) return JFG_ERR_ARG;
  CUtensorMap ma, mb;
  JFG_TRY(make_map_bf16(&ma, A, d.K, d.M, prm.a_bat ? d.batch : 1, d.lda,
                        prm.a_bat ? d.a_batch : d.lda * d.M, TM, prm.a_perm != 0));
  JFG_TRY(make_map_bf16(&mb, B, d.K, d.N, prm.b_bat ? d.batch : 1, d.ldb,
                        prm.b_bat ? d.b_batch : d.ldb * d.N, (cuuint32_t)prm.Nt,
                        prm.b_perm != 0));
  const size_t smem = 1024 + stages * stage + (2 * stages + 1) * 8 + 16;
  static bool attr_done[64] = {};
  int dev = 0;
  JFG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return JFG_ERR_UNSUPPORTED;
  if (!attr_done[dev]) {
    JFG_CUDA_TRY(cudaFuncSetAttribute(k_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      227 * 1024));
    attr_done[dev] = true;
  }
  dim3 grid((d.M + TM - 1) / TM, d.batch / prm.nb, ksplit);
  k_gemm_bf16<<<grid, NTH, smem, (cudaStream_t)stream>>>(ma, mb, prm);
  JFG_LAUNCHED();
  return JFG_OK;
}

namespace jfg {
int gemm_status_take(int* status) {
  int zero = 0;
  JFG_CUDA_TRY(cudaMemcpyFromSymbol(status, g_gemm_status, sizeof(int)));
  JFG_CUDA_TRY(cudaMemcpyToSymbol(g_gemm_status, &zero, sizeof(int)));
  return JFG_OK;
}
}  // namespace jfg
