// Per-axis contraction on the 5th-generation tensor cores (sm_103a):
// TMA -> shared memory -> tcgen05.mma (kind::tf32) -> TMEM -> epilogue.
//
//   out[b][s][m][p] = alpha * epi( sum_k op[s][m][k] * in[b][s][p][k] ) + beta * out
//
// Precision: three-term split TF32.  Each FP32 input x is split exactly into
// hi = x with its low 13 mantissa bits cleared (a TF32 value) and lo = x - hi;
// the operator is pre-split the same way on the host.  The tensor cores then
// accumulate hi*hi + hi*lo + lo*hi in FP32, which gives FP32-level accuracy
// (about 2^-22 relative per product) at three TF32 MMAs per block.
//
// Tile: 128 rows of p (the MMA M dimension, one TMEM lane per row) by up to 128
// operator rows m (the MMA N dimension, one TMEM column each), K in blocks of
// 32 FP32 (128 B rows, 128-byte swizzle), 3 pipeline stages.  The kernel is
// persistent (one CTA per SM walking the tile list) with two TMEM accumulator
// buffers.  Warp roles:
//   warp 0     TMA producer (one thread)
//   warp 1     TMEM allocator and MMA issuer (one thread)
//   warps 2-5  split each staged input tile into TF32 hi (in place) and lo
//   warps 6-13 epilogue: two warps per TMEM lane quarter, tcgen05.ld 32 lanes
//              x 16 columns, fused field multiply / eigenvalue divide / beta
//              accumulate
// Every mbarrier wait is bounded by a global-timer budget; on expiry the
// kernel records JFG_ERR_DEVICE_TIMEOUT in a device status word, drains its own
// TMA copies (bounded), frees its TMEM and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "jfg_internal.cuh"

namespace jfg {

__device__ int g_tc_status = 0;
// Budget of the pipeline waits (ns) and the test hook that makes the epilogue
// first wait on a barrier nothing arrives on (jfg_tc_set_wait_budget_ns,
// jfg_tc_test_hold): the timeout path can then be exercised without any
// broken kernel.  Drain waits always use the full WAIT_NS budget.
constexpr unsigned long long WAIT_NS_DEFAULT = 2000000000ull;
__device__ unsigned long long g_tc_wait_ns = WAIT_NS_DEFAULT;
__device__ int g_tc_test_hold = 0;

// Kernel variant: 1 keeps the split input tile in TMEM (default), 0 in shared
// memory (jfg_tc_set_variant).
static int g_operand_a_in_tmem = 1;
// Epilogue output path: 1 TMA stores through shared memory where the layout
// allows (default), 0 plain coalesced stores (jfg_tc_set_store_path).
static int g_tma_store = 1;
// Operator-stationary schedule for single-group 16-bit launches whose
// operator chunk fits in shared memory: 0 (default) off, 1 when every CTA gets
// >= 2 tiles, 2 whenever the chunk fits (jfg_tc_set_op_resident); a launch
// configuration's schedule field overrides it.
static int g_op_resident = 0;

namespace {

constexpr int TILE_P = 128;
constexpr int KB = 32;                     // FP32 elements per K block (128 B)
constexpr int MT_MAX = 128;                // operator rows per tile (MMA N)
constexpr int NTHREADS = 448;  // 14 warps
constexpr uint32_t XBYTES = TILE_P * KB * 4;  // 16 KB
// K elements per block of the 16-bit operator paths (split BF16, scaled split
// FP16): 64 (two 128-byte FP32 input rows, one 128-byte operator row; 64 KB
// stages, three of them), except for the field-multiply epilogue: its two
// field boxes per epilogue warp leave room for only two such stages, and with
// 32-element blocks (one input row, a 64-byte operator row under the 64-byte
// swizzle; 32 KB stages) five fit.  Measured on the variable-coefficient
// passes: the field pass 74.5 -> 66.3 us with 32, every other pass slower
// with 32 (more handshakes per unit of work).
__host__ __device__ constexpr int b16_ke(int epi) { return epi == JFG_EPI_MUL_FIELD ? 32 : 64; }
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s budget per wait

constexpr int GMAX = 40;  // groups per launch of the grouped kernel

// One group of problems of a (grouped) launch.
struct TcGroup {
  jfg_contract_desc d;
  float* out;
  int Mtile;       // padded operator rows per tile (multiple of 16, <= MT_MAX)
  int seg_in_map;  // 1 if the input map has a segment dimension
  int bat_in_map;  // 1 if the input map has a batch dimension
  int seg_op_map;  // 1 if the operator maps have a segment dimension
  int mc_inner;    // tile order: operator chunks innermost (inputs beyond L2)
  int tma_store;   // epilogue stores 32 x 32 boxes through shared memory with TMA
  // scaled split-FP16 variant: per-problem max |input| (float bits) that sets
  // the power-of-two input scale, per-problem max |output| recorded for the
  // next pass, and the inverse power-of-two row scales of the operator
  const unsigned* in_max;
  unsigned* out_max;
  const float* op_inv;  // op_inv[s * op_inv_seg + m]
  long long op_inv_seg;
  // field-multiply epilogue of a single-group launch: the field's 32 x 32
  // boxes are fetched by TMA (L.fmap) into the warp's output staging box
  int tma_field;
  int fld_seg;  // the field map has a segment dimension (field_seg != 0)
  int fld_bat;  // the field map has a batch dimension (field_batch != 0)
  // fused dot (field / divide epilogues): partials of sum(acc * out) per
  // problem at dot_part[b * DOT_NBMAX + tile-of-problem * 8 + epilogue warp]
  float* dot_part;
};

// Kernel parameter block (__grid_constant__): groups and their tensor maps
// (input X, operator hi, operator lo, output for TMA stores).
constexpr uint32_t STAGE_OUT = 32 * 32 * 4;  // one epilogue warp's output box (4 KB)
constexpr int SMEM_MAX = 227 * 1024 - 1024;   // dynamic shared memory (static use < 1 KB)
template <int G>
struct TcLaunch {
  CUtensorMap maps[G][4];
  CUtensorMap fmap;  // field of group 0 (TcGroup::tma_field)
  TcGroup g[G];
  int ngroups;
  int stages;
  int tmem_cols;
  int tmem_a;   // 1: split input tile (MMA operand A) kept in TMEM, not shared memory
  int mt_max;   // largest Mtile: sets the stage layout
  int out_stage; // 32 x 32 staging boxes per epilogue warp after the stages: 0, 1 (TMA
                 // stores) or 2 (field-multiply launches: both of a warp's field boxes
                 // of a tile are fetched ahead and stored from separate boxes)
  // 1 (16-bit operators, one group): operator-stationary schedule.  CTA c
  // serves the operator slot c % nslots, slot = s * mchunks + mc, loads that
  // operator chunk (all K blocks, hi and lo) into shared memory once and
  // streams only the input tiles of its (problem, p-tile) pairs.
  int op_res;
  int nslots;
};

// TMEM column map when operand A lives in TMEM: accumulator buffers at
// columns [0, 128) and [128, 256); stage s keeps A hi at 256 + 64 s and A lo
// at 256 + 64 s + 32 (32 TF32 columns each).
constexpr int ACC_STRIDE_TA = 128;
constexpr int A_COL0 = 256;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred P1;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, P1;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false (and the status word set) if the budget runs out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          unsigned long long budget) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (true) {
    for (int i = 0; i < 256; ++i)
      if (mbar_try(bar, parity)) return true;
    if (gtimer() - t0 > budget) {
      atomicExch(&g_tc_status, JFG_ERR_DEVICE_TIMEOUT);
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2),
      "r"(c3)
      : "memory");
}

// Bulk tensor store of a shared-memory box (no swizzle) to global, tracked in
// this thread's bulk async-group.
__device__ __forceinline__ void tma_store_4d(const CUtensorMap* map, const void* src, int c0,
                                             int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%2, %3, %4, %5}], [%1];" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(smem_u32(src)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// core-matrix groups 1024 B apart.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                     // leading byte offset (unused, SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;           // stride byte offset
  d |= (uint64_t)1 << 46;                     // descriptor version
  d |= (uint64_t)2 << 61;                     // SWIZZLE_128B
  return d;
}

// The same for 64-byte rows (64-byte swizzle): 8-row groups 512 B apart.
__device__ __forceinline__ uint64_t sdesc64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                     // leading byte offset (unused, swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;            // stride byte offset
  d |= (uint64_t)1 << 46;                     // descriptor version
  d |= (uint64_t)4 << 61;                     // SWIZZLE_64B
  return d;
}

// Instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accum));
}

// Same MMA with operand A read from TMEM (128 lanes x 8 TF32 columns).
__device__ __forceinline__ void mma_tf32_ta(uint32_t tmem, uint32_t a_tmem, uint64_t b,
                                            uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem),
      "r"(a_tmem), "l"(b), "r"(idesc), "r"(accum));
}

// Instruction descriptor: kind::f16 with BF16 A/B, D = F32, both K-major.
__host__ __device__ constexpr uint32_t idesc_b16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// BF16 MMA (K = 16) with operand A read from TMEM (128 lanes x 8 columns of
// packed BF16 pairs).
__device__ __forceinline__ void mma_b16_ta(uint32_t tmem, uint32_t a_tmem, uint64_t b,
                                           uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem),
      "r"(a_tmem), "l"(b), "r"(idesc), "r"(accum));
}

// Two FP32 -> packed BF16 pair (round to nearest even): lo16 <- a, hi16 <- b.
__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  uint32_t d;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
  return d;
}

// Two FP32 -> packed FP16 pair (round to nearest even): lo16 <- a, hi16 <- b.
__device__ __forceinline__ uint32_t pack_f16x2(float a, float b) {
  uint32_t d;
  asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
  return d;
}

__device__ __forceinline__ float2 unpack_f16x2(uint32_t h) {
  return __half22float2(*reinterpret_cast<const __half2*>(&h));
}

// Instruction descriptor: kind::f16 with FP16 A/B, D = F32, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Power-of-two input scale of the split-FP16 variant from the float bits of
// an upper bound on max |x|: the scaled values are below 2^15 (FP16 max is
// 65504) and the largest is at least 2^14, so FP16 hi and lo keep ~22 bits
// relative to the maximum and nothing overflows.  Zero, non-finite or
// missing bounds give scale 1; the exponent is clamped to [2^-126, 2^126]
// so the inverse is exact as well.
__device__ __forceinline__ void h16_scale_bits(unsigned bits, float& sc, float& inv) {
  sc = inv = 1.f;
  bits &= 0x7FFFFFFFu;
  const int e = (int)(bits >> 23);
  if (bits == 0 || e == 0xFF) return;
  int eb = 268 - e;  // biased exponent of 2^(15 - E), max |x| < 2^E, E = e - 126
  eb = eb < 1 ? 1 : (eb > 253 ? 253 : eb);
  sc = __uint_as_float((unsigned)eb << 23);
  inv = __uint_as_float((unsigned)(254 - eb) << 23);
}
// the recorded bound of problem b (0: none, scale 1)
__device__ __forceinline__ unsigned h16_bits(const unsigned* in_max, int b) {
  return (in_max && b >= 0) ? __ldg(in_max + b) : 0u;
}
__device__ __forceinline__ void h16_scale(const unsigned* in_max, int b, float& sc, float& inv) {
  h16_scale_bits(h16_bits(in_max, b), sc, inv);
}

// Store 32 consecutive 32-bit columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, "
      "%17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};" ::"r"(
          taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
      "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]),
      "r"(v[15]), "r"(v[16]), "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]),
      "r"(v[22]), "r"(v[23]), "r"(v[24]), "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]),
      "r"(v[29]), "r"(v[30]), "r"(v[31])
      : "memory");
}

// Store 16 consecutive 32-bit columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
      "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]),
      "r"(v[15])
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tf32_hi(float x) {
  return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
}

// Persistent kernel over one or more groups of problems.  Group gi has its own
// descriptor, operator tile height Mtile and tensor maps; its tiles are
// t = tb[gi] + ((slot * nseg + s) * mchunks + mc) * nptiles + pt (or, for inputs
// larger than L2, ((slot * nseg + s) * nptiles + pt) * mchunks + mc), covering p rows
// [pt*128, +128) and operator rows [mc*Mtile, +Mtile) of problem slot / segment
// s.  Each CTA walks t = blockIdx.x, blockIdx.x + gridDim.x, ...; two TMEM
// accumulator buffers let the epilogue of tile i overlap the main loop of
// tile i+1.  The tile prefix tb[] is formed on the device from the active
// counts, so listed (active-subset) groups need no host round trip.
template <int EPI, bool BETA, int G, int PREC>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_contract_tc(const __grid_constant__ TcLaunch<G> L) {
  // PREC: 0 split TF32 (kind::tf32), 1 split BF16, 2 scaled split FP16 (both
  // kind::f16: 16-bit operator pairs, 64-element K blocks), 3 plain BF16 (one
  // product hi*hi, the operator's hi only: ~2^-8 relative per product)
  constexpr bool B16 = PREC != 0;
  constexpr bool H16 = PREC == 2;
  constexpr bool B1 = PREC == 3;
  constexpr uint32_t NOP = B1 ? 1u : 2u;  // operator pieces per stage (hi, lo)
  // K elements per block: 32 TF32 (one 128-byte row) or 64 BF16 (one 128-byte
  // operator row; the FP32 input block then takes two TMA boxes)
  constexpr int KE = B16 ? b16_ke(EPI) : KB;
  constexpr uint32_t XB = B16 ? (uint32_t)(KE / KB) * XBYTES : XBYTES;
  constexpr uint32_t OROW = B16 ? 2u * KE : 128u;  // bytes per operator row of a stage
  // TMEM columns per stage of operand A (hi then lo)
  constexpr uint32_t A_SLOT = B16 ? (uint32_t)KE : 2u * KB;
  extern __shared__ uint8_t smem_raw[];
  __shared__ long long tb[G + 1];
  __shared__ int nbs[G];
  __shared__ unsigned long long s_budget;
  __shared__ int s_hold;
  // scaled split FP16: the input bound of each stage's problem, written by the
  // producer with the stage's loads (it reads the list and the bound well
  // ahead), read by the split warps after the stage's full barrier
  __shared__ unsigned s_xbits[16];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int S = L.stages;
  const bool ta = B16 || L.tmem_a != 0;
  const bool res = B16 && !B1 && L.op_res != 0;
  const uint32_t omax = (uint32_t)L.mt_max * OROW;  // Mtile operator rows (hi or lo)
  const uint32_t xbuf = ta ? XB : 2 * XBYTES;  // X block (+ its lo part when in SMEM)
  const uint32_t stage_bytes = res ? xbuf : xbuf + NOP * omax;
  const uint32_t acc_stride = ta ? ACC_STRIDE_TA : 256;
  // operator-stationary schedule: this CTA's operator slot and tile stride
  const int r_slot = res ? (int)(blockIdx.x % (unsigned)L.nslots) : 0;
  const int r_mchunks = res ? (L.g[0].d.M + L.g[0].Mtile - 1) / L.g[0].Mtile : 1;
  const int r_s = r_slot / r_mchunks, r_mc = r_slot - r_s * r_mchunks;
  const long long r_j0 = res ? (long long)(blockIdx.x / (unsigned)L.nslots) : 0;
  const long long r_step =
      res ? (long long)((gridDim.x - (unsigned)r_slot + (unsigned)L.nslots - 1) / L.nslots) : 1;
  const int r_nkb = res ? (L.g[0].d.K + KE - 1) / KE : 0;
  const uint32_t res_bytes = res ? (uint32_t)r_nkb * 2 * omax : 0;

  if (threadIdx.x == 0) {
    long long acc = 0;
    for (int gi = 0; gi < L.ngroups; ++gi) {
      const TcGroup& q = L.g[gi];
      const int nb = active_count(q.d.batch_list, q.d.batch_count, q.d.batch);
      nbs[gi] = nb;
      tb[gi] = acc;
      acc += (long long)((q.d.P + TILE_P - 1) / TILE_P) * ((q.d.M + q.Mtile - 1) / q.Mtile) *
             nb * q.d.nseg;
    }
    tb[L.ngroups] = acc;
    s_budget = g_tc_wait_ns;
    s_hold = g_tc_test_hold;
  }
  __syncthreads();
  const unsigned long long budget = s_budget;
  const long long ntiles = tb[L.ngroups];
  const int r_nptiles = (L.g[0].d.P + TILE_P - 1) / TILE_P;
  const long long r_cnt = res ? (long long)nbs[0] * r_nptiles : 0;  // tiles of one slot
  if (!res && (long long)blockIdx.x >= ntiles) return;  // no tile for this CTA (uniform)
  if (res && r_j0 >= r_cnt) return;

  uint8_t* sbase = smem + res_bytes;                   // input (and operator) stages
  uint8_t* ostage = sbase + (size_t)S * stage_bytes;  // epilogue output boxes (if used)
  uint64_t* bars = (uint64_t*)(ostage + (size_t)8 * STAGE_OUT * L.out_stage);
  uint64_t* full = bars;
  uint64_t* conv = bars + S;
  uint64_t* empty = bars + 2 * S;
  uint64_t* tfull = bars + 3 * S;       // [2] accumulator ready
  uint64_t* tempty = bars + 3 * S + 2;  // [2] accumulator drained
  uint64_t* hold = bars + 3 * S + 4;    // test hook: nothing arrives on it
  uint64_t* mma_done = bars + 3 * S + 5;  // MMA drain after a timeout
  uint64_t* opfull = bars + 3 * S + 6;    // resident operator chunk landed
  uint64_t* fbar = bars + 3 * S + 7;      // [16] field box landed (two per epilogue warp)
  uint32_t* tmem_slot = (uint32_t*)(bars + 3 * S + 23);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int i = 0; i < S; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&conv[i], 4);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], 8);
    }
    mbar_init(hold, 1);
    mbar_init(mma_done, 1);
    mbar_init(opfull, 1);
    for (int i = 0; i < 16; ++i) mbar_init(&fbar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(L.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  auto Xh = [&](int st) { return sbase + (size_t)st * stage_bytes; };
  auto Xl = [&](int st) { return sbase + (size_t)st * stage_bytes + XBYTES; };
  auto Oh = [&](int st) { return sbase + (size_t)st * stage_bytes + xbuf; };
  auto Ol = [&](int st) { return sbase + (size_t)st * stage_bytes + xbuf + omax; };
  // resident operator chunk: K block kb of hi at 2 kb omax, lo right after it
  auto OhR = [&](int kb) { return smem + (size_t)kb * 2 * omax; };
  auto OlR = [&](int kb) { return smem + (size_t)kb * 2 * omax + omax; };
  // b = problem index (-1: an out-of-range list entry, computed but not stored);
  // roles that do not use b (need_b false) skip its list load.  Tile indices
  // below 2^32 take 32-bit division: the 64-bit one is a long software
  // sequence, paid by every role at every tile.
  auto decode = [&](long long t, int& gi, int& pt, int& mc, int& b, int& s, bool need_b) {
    gi = 0;
    while (gi + 1 < L.ngroups && t >= tb[gi + 1]) ++gi;
    const TcGroup& q = L.g[gi];
    const unsigned nptiles = (unsigned)((q.d.P + TILE_P - 1) / TILE_P);
    const unsigned mchunks = (unsigned)((q.d.M + q.Mtile - 1) / q.Mtile);
    const long long r = t - tb[gi];
    int bs;
    if (r <= 0xFFFFFFFFLL) {
      unsigned ru = (unsigned)r;
      if (q.mc_inner) {  // the CTAs that share an input tile run it at the same time
        mc = (int)(ru % mchunks);
        ru /= mchunks;
        pt = (int)(ru % nptiles);
        bs = (int)(ru / nptiles);
      } else {           // the CTAs that share an operator chunk run it at the same time
        pt = (int)(ru % nptiles);
        ru /= nptiles;
        mc = (int)(ru % mchunks);
        bs = (int)(ru / mchunks);
      }
    } else if (q.mc_inner) {
      mc = (int)(r % mchunks);
      pt = (int)((r / mchunks) % nptiles);
      bs = (int)(r / mchunks / nptiles);
    } else {
      pt = (int)(r % nptiles);
      mc = (int)((r / nptiles) % mchunks);
      bs = (int)(r / nptiles / mchunks);
    }
    const int slot = bs / q.d.nseg;
    s = bs - slot * q.d.nseg;
    b = need_b ? active_problem(q.d.batch_list, nbs[gi], q.d.batch, slot) : 0;
  };
  auto nkb_of = [&](int gi) { return (L.g[gi].d.K + KE - 1) / KE; };
  // tile li of this CTA (false past the last one)
  auto tile_of = [&](long long li, int& gi, int& pt, int& mc, int& b, int& s,
                     bool need_b = true) -> bool {
    if (!res) {
      const long long t = (long long)blockIdx.x + li * (long long)gridDim.x;
      if (t >= ntiles) return false;
      decode(t, gi, pt, mc, b, s, need_b);
      return true;
    }
    const long long j = r_j0 + li * r_step;
    if (j >= r_cnt) return false;
    const TcGroup& q = L.g[0];
    gi = 0;
    pt = (int)(j % r_nptiles);
    b = need_b ? active_problem(q.d.batch_list, nbs[0], q.d.batch, (int)(j / r_nptiles)) : 0;
    s = r_s;
    mc = r_mc;
    return true;
  };

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      long long g = 0, issued = 0;
      bool ok = true;
      if (res) {
        // the operator chunk of this CTA's slot, once: every K block, hi and lo
        const TcGroup& q = L.g[0];
        const uint32_t obytes = (uint32_t)q.Mtile * OROW;
        const int os = q.seg_op_map ? r_s : 0;
        mbar_expect_tx(opfull, (uint32_t)r_nkb * 2 * obytes);
        for (int kb = 0; kb < r_nkb; ++kb) {
          tma_load_3d(OhR(kb), &L.maps[0][1], opfull, kb * KE, r_mc * q.Mtile, os);
          tma_load_3d(OlR(kb), &L.maps[0][2], opfull, kb * KE, r_mc * q.Mtile, os);
        }
      }
      int gi, pt, mc, b, s;
      int st = 0;       // stage of K block g (g % S, kept running: no division)
      uint32_t ph = 0;  // (g / S) & 1
      for (long long li = 0; ok && tile_of(li, gi, pt, mc, b, s); ++li) {
        const TcGroup& q = L.g[gi];
        const int cs = q.seg_in_map ? s : 0;
        const int cb = (q.bat_in_map && b > 0) ? b : 0;
        const int os = q.seg_op_map ? s : 0;
        const uint32_t obytes = (uint32_t)q.Mtile * OROW;
        const int nkb = nkb_of(gi);
        const unsigned xbits = H16 ? h16_bits(q.in_max, b) : 0u;
        for (int kb = 0; kb < nkb; ++kb, ++g) {
          if (g >= S && !mbar_wait(&empty[st], ph ^ 1u, budget)) {
            ok = false;
            break;
          }
          if (H16) s_xbits[st] = xbits;
          mbar_expect_tx(&full[st], res ? XB : XB + NOP * obytes);
          tma_load_4d(Xh(st), &L.maps[gi][0], &full[st], kb * KE, pt * TILE_P, cs, cb);
          if (B16 && KE > KB)
            tma_load_4d(Xh(st) + XBYTES, &L.maps[gi][0], &full[st], kb * KE + KB,
                        pt * TILE_P, cs, cb);
          if (!res) {
            tma_load_3d(Oh(st), &L.maps[gi][1], &full[st], kb * KE, mc * q.Mtile, os);
            if (!B1)
              tma_load_3d(Ol(st), &L.maps[gi][2], &full[st], kb * KE, mc * q.Mtile, os);
          }
          issued = g + 1;
          if (++st == S) {
            st = 0;
            ph ^= 1u;
          }
        }
      }
      // drain: the latest use of every stage (and the resident operator) must
      // have landed before exit
      for (long long q = (issued > S ? issued - S : 0); q < issued; ++q)
        mbar_wait(&full[q % S], (uint32_t)(q / S) & 1u, WAIT_NS);
      if (res) mbar_wait(opfull, 0, WAIT_NS);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      long long g = 0;
      int li = 0;
      bool ok = true, issued_any = false;
      if (res && !mbar_wait(opfull, 0, budget)) ok = false;
      int gi, pt, mc, b, s;
      int st = 0;       // stage of K block g
      uint32_t ph = 0;  // (g / S) & 1
      for (; ok && tile_of(li, gi, pt, mc, b, s, false); ++li) {
        const uint32_t idesc = H16   ? idesc_f16(TILE_P, L.g[gi].Mtile)
                               : B16 ? idesc_b16(TILE_P, L.g[gi].Mtile)
                                     : idesc_tf32(TILE_P, L.g[gi].Mtile);
        const int nkb = nkb_of(gi);
        const int buf = li & 1;
        const uint32_t use = (uint32_t)(li >> 1);
        if (li >= 2 && !mbar_wait(&tempty[buf], (use & 1u) ^ 1u, budget)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t acc = tmem + (uint32_t)buf * acc_stride;
        for (int kb = 0; kb < nkb; ++kb, ++g) {
          if (!mbar_wait(&conv[st], ph, budget)) {
            ok = false;
            break;
          }
          issued_any = true;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t oh = smem_u32(res ? OhR(kb) : Oh(st));
          const uint32_t ol = smem_u32(res ? OlR(kb) : Ol(st));
          if (B16) {
            const uint32_t ah = tmem + (uint32_t)A_COL0 + A_SLOT * (uint32_t)st,
                           al = ah + A_SLOT / 2;
#pragma unroll
            for (int kk = 0; kk < KE / 16; ++kk) {
              const uint32_t off = kk * 32;  // 16 BF16 = 32 B of B per MMA, 8 A columns
              const uint64_t bh = KE == 64 ? sdesc(oh + off) : sdesc64(oh + off);
              const uint64_t bl = KE == 64 ? sdesc(ol + off) : sdesc64(ol + off);
              mma_b16_ta(acc, ah + 8 * kk, bh, idesc, (kb | kk) ? 1u : 0u);
              if (!B1) {
                mma_b16_ta(acc, ah + 8 * kk, bl, idesc, 1u);
                mma_b16_ta(acc, al + 8 * kk, bh, idesc, 1u);
              }
            }
          } else if (ta) {
            const uint32_t ah = tmem + (uint32_t)A_COL0 + A_SLOT * (uint32_t)st, al = ah + 32;
#pragma unroll
            for (int kk = 0; kk < KB / 8; ++kk) {
              const uint32_t off = kk * 32;  // 8 TF32 = 32 B of B per MMA, 8 A columns
              mma_tf32_ta(acc, ah + 8 * kk, sdesc(oh + off), idesc, (kb | kk) ? 1u : 0u);
              mma_tf32_ta(acc, ah + 8 * kk, sdesc(ol + off), idesc, 1u);
              mma_tf32_ta(acc, al + 8 * kk, sdesc(oh + off), idesc, 1u);
            }
          } else {
            const uint32_t xh = smem_u32(Xh(st)), xl = smem_u32(Xl(st));
#pragma unroll
            for (int kk = 0; kk < KB / 8; ++kk) {
              const uint32_t off = kk * 32;  // 8 TF32 = 32 B per MMA
              mma_tf32(acc, sdesc(xh + off), sdesc(oh + off), idesc, (kb | kk) ? 1u : 0u);
              mma_tf32(acc, sdesc(xh + off), sdesc(ol + off), idesc, 1u);
              mma_tf32(acc, sdesc(xl + off), sdesc(oh + off), idesc, 1u);
            }
          }
          mma_commit(&empty[st]);
          if (++st == S) {
            st = 0;
            ph ^= 1u;
          }
        }
        if (ok) mma_commit(&tfull[buf]);
      }
      // after a timeout the MMAs already issued must finish before the TMEM
      // they write is freed: one more commit tracks all of them
      if (!ok && issued_any) {
        mma_commit(mma_done);
        mbar_wait(mma_done, 0, WAIT_NS);
      }
    }
  } else if (warp < 6) {
    // ---------------- split staged input tiles into TF32 hi (in place) / lo ----------------
    const int ct = threadIdx.x - 64;  // 0..127
    // TMEM mode: thread = row r of the tile (its warp's lane quarter), reads
    // its 32 values from the 128-byte-swizzled tile and stores hi / lo into
    // its TMEM lane with tcgen05.st.
    const int row = 32 * (warp & 3) + lane;
    bool ok = true;
    int gi, pt, mc, b, s;
    int st = 0;       // stage of the current K block
    uint32_t ph = 0;  // its use count parity
    for (long long li = 0; ok && tile_of(li, gi, pt, mc, b, s, false); ++li) {
      const int nkb = nkb_of(gi);
      float xsc = 1.f, xinv = 1.f;
      for (int kb = 0; kb < nkb; ++kb) {
        if (!mbar_wait(&full[st], ph, budget)) {
          ok = false;
          break;
        }
        if (H16 && kb == 0) h16_scale_bits(s_xbits[st], xsc, xinv);
        if (H16) {
          // 64 FP32 of this row, scaled by 2^k, -> FP16 hi / lo pairs; one
          // 32-element half at a time (16 hi and 16 lo columns) keeps the
          // live registers low
          const uint32_t tbase = tmem + ((uint32_t)(32 * (warp & 3)) << 16) +
                                 (uint32_t)A_COL0 + A_SLOT * (uint32_t)st;
#pragma unroll
          for (int half = 0; half < KE / KB; ++half) {
            uint32_t h[16], l[16];
            const float4* xr = (const float4*)(Xh(st) + half * XBYTES + row * 128);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
              const float4 v = xr[c ^ (row & 7)];
              const float a0 = v.x * xsc, a1 = v.y * xsc, a2 = v.z * xsc, a3 = v.w * xsc;
              const uint32_t h0 = pack_f16x2(a0, a1), h1 = pack_f16x2(a2, a3);
              const float2 f0 = unpack_f16x2(h0), f1 = unpack_f16x2(h1);
              h[2 * c] = h0;
              h[2 * c + 1] = h1;
              l[2 * c] = pack_f16x2(a0 - f0.x, a1 - f0.y);
              l[2 * c + 1] = pack_f16x2(a2 - f1.x, a3 - f1.y);
            }
            tmem_st16(tbase + 16 * half, h);
            tmem_st16(tbase + A_SLOT / 2 + 16 * half, l);
          }
          asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        } else if (B16) {
          // 64 FP32 of this row (two swizzled 128-byte rows) -> BF16 hi / lo,
          // packed in pairs (lower k in the lower half) into 32 TMEM columns
          // each, one 32-element half (16 + 16 columns) at a time
          const uint32_t tbase = tmem + ((uint32_t)(32 * (warp & 3)) << 16) +
                                 (uint32_t)A_COL0 + A_SLOT * (uint32_t)st;
#pragma unroll
          for (int half = 0; half < KE / KB; ++half) {
            uint32_t h[16], l[16];
            const float4* xr = (const float4*)(Xh(st) + half * XBYTES + row * 128);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
              const float4 v = xr[c ^ (row & 7)];
              const uint32_t h0 = pack_bf16x2(v.x, v.y), h1 = pack_bf16x2(v.z, v.w);
              h[2 * c] = h0;
              h[2 * c + 1] = h1;
              if (!B1) {
                l[2 * c] = pack_bf16x2(v.x - __uint_as_float(h0 << 16),
                                       v.y - __uint_as_float(h0 & 0xFFFF0000u));
                l[2 * c + 1] = pack_bf16x2(v.z - __uint_as_float(h1 << 16),
                                           v.w - __uint_as_float(h1 & 0xFFFF0000u));
              }
            }
            tmem_st16(tbase + 16 * half, h);
            if (!B1) tmem_st16(tbase + A_SLOT / 2 + 16 * half, l);
          }
          asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        } else if (ta) {
          const float4* xr = (const float4*)(Xh(st) + row * 128);
          uint32_t h[32], l[32];
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            const float4 v = xr[c ^ (row & 7)];
            const float hv[4] = {tf32_hi(v.x), tf32_hi(v.y), tf32_hi(v.z), tf32_hi(v.w)};
            const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              h[4 * c + e] = __float_as_uint(hv[e]);
              l[4 * c + e] = __float_as_uint(vv[e] - hv[e]);
            }
          }
          const uint32_t tbase = tmem + ((uint32_t)(32 * (warp & 3)) << 16) +
                                 (uint32_t)A_COL0 + A_SLOT * (uint32_t)st;
          tmem_st32(tbase, h);
          tmem_st32(tbase + 32, l);
          asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        } else {
          float4* xh = (float4*)Xh(st);
          float4* xl = (float4*)Xl(st);
#pragma unroll
          for (int i = 0; i < (int)(XBYTES / 16 / 128); ++i) {
            const int idx = ct + i * 128;
            float4 v = xh[idx];
            float4 h = make_float4(tf32_hi(v.x), tf32_hi(v.y), tf32_hi(v.z), tf32_hi(v.w));
            xh[idx] = h;
            xl[idx] = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
          }
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&conv[st]);
        if (++st == S) {
          st = 0;
          ph ^= 1u;
        }
      }
    }
  } else {
    // ---------------- epilogue: TMEM -> registers -> global ----------------
    // Eight warps: two per TMEM lane quarter, each taking every other group
    // of 32 accumulator columns; field / eigenvalue loads of a group are all
    // issued before its TMEM load so they are in flight together.
    const int q4 = warp & 3;  // TMEM lane quarter this warp may access
    const int half = (warp - 6) >> 2;
    const int row = 32 * q4 + lane;
    int li = 0;
    // test hook: a barrier nothing arrives on; its wait runs out (status set)
    // and this warp skips its tiles, so every other role's waits run out too
    const bool held = s_hold != 0 && !mbar_wait(hold, 0, budget);
    const int ew = warp - 6;   // this warp's staging boxes and field barriers
    uint32_t fph = 0;          // phase bit j of fbar[2 ew + j]
    uint32_t fpend = 0;        // bit j: a field box load into box j is in flight
    bool fok = true;
    const int nbox = L.out_stage > 0 ? L.out_stage : 1;
    auto box_of = [&](int j) {
      return (float*)(ostage + ((size_t)ew * nbox + (j < nbox ? j : 0)) * STAGE_OUT);
    };
    int gi, pt, mc, b, s;
    for (; !held && fok && tile_of(li, gi, pt, mc, b, s); ++li) {
      const TcGroup& q = L.g[gi];
      const jfg_contract_desc& d = q.d;
      const int Mt = q.Mtile;
      const float alpha = (float)d.alpha, beta = (float)d.beta;
      const int buf = li & 1;
      const int p = pt * TILE_P + row;
      const bool pin = p < d.P && b >= 0;
      const int bb = b < 0 ? 0 : b;
      float* outS = q.out + (long long)bb * d.out_batch + (long long)s * d.out_seg;
      float c0 = 0.f, c1 = 1.f, lp = 0.f;
      const float* __restrict__ lam_m = (const float*)d.lam_m;
      if (EPI == JFG_EPI_DIV_EIG) {
        c0 = d.c0 ? __ldg((const float*)d.c0 + bb) : 0.f;
        c1 = d.c1 ? __ldg((const float*)d.c1 + bb) : 1.f;
        lp = pin ? __ldg((const float*)d.lam_p + p) : 0.f;
      }
      const float* __restrict__ fld = nullptr;
      if (EPI == JFG_EPI_MUL_FIELD)
        fld = (const float*)d.field + (long long)bb * d.field_batch + (long long)s * d.field_seg;
      float xsc = 1.f, xinv = 1.f, omax = 0.f, dsum = 0.f;
      const float* __restrict__ oinv = nullptr;
      if (H16) {
        h16_scale(q.in_max, b, xsc, xinv);
        oinv = q.op_inv + (long long)s * q.op_inv_seg;
      }
      const bool fdot = EPI != JFG_EPI_NONE && q.dot_part != nullptr;
      // This warp's 16-column blocks of the tile: cb(k) = 2 half + 4 (k / 2) +
      // k % 2 (pairs form the 32 x 32 boxes of the TMA stores).  The per-column
      // factors of block k+1 (field values, eigenvalues, operator scales) are
      // loaded while block k is processed, and those of block 0 before the
      // accumulator wait, so their latency overlaps the main loop.
      const int ncb = Mt / 16;
      auto cb_of = [&](int k) { return half * 2 + 4 * (k >> 1) + (k & 1); };
      // field-multiply epilogue with TMA: the field's 32 x 32 box of each
      // output box is fetched into the staging box by one bulk tensor copy
      const bool tfld = EPI == JFG_EPI_MUL_FIELD && !BETA && q.tma_store && q.tma_field;
      const bool dbl = tfld && nbox == 2;
      // field box of output box j (blocks k = 2j, 2j+1) into staging box j
      auto issue_field = [&](int j, int cbk) {
        if (lane == 0) {
          mbar_expect_tx(&fbar[2 * ew + j], STAGE_OUT);
          tma_load_4d(box_of(j), &L.fmap, &fbar[2 * ew + j], pt * TILE_P + 32 * q4,
                      mc * Mt + (cbk & ~1) * 16, q.fld_seg ? s : 0, q.fld_bat ? bb : 0);
        }
        fpend |= 1u << j;
      };
      auto load_aux = [&](int cbk, float* a) {
        const int m0 = mc * Mt + cbk * 16;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int m = m0 + j;
          const bool ok = pin && m < d.M;
          float v = 1.f;
          if (EPI == JFG_EPI_MUL_FIELD && !tfld)
            v = ok ? __ldg(fld + (long long)m * d.field_ld + p) : 0.f;
          if (EPI == JFG_EPI_DIV_EIG) v = ok ? __ldg(lam_m + m) : 1.f;
          if (H16 && EPI != JFG_EPI_DIV_EIG) {
            // the row's inverse scale alone: the problem's (a power of two,
            // xs) is applied where aux is used, so these loads stay in flight
            // while the block before is processed
            const float oi = ok ? __ldg(oinv + m) : 0.f;
            v = (EPI == JFG_EPI_MUL_FIELD && !tfld) ? v * oi : oi;
          }
          a[j] = v;
        }
      };
      const float xs = (H16 && EPI != JFG_EPI_DIV_EIG) ? xinv : 1.f;
      float aux[16], nxt[16];
      if (cb_of(0) < ncb) {
        load_aux(cb_of(0), aux);
        if (tfld) {
          // the staging boxes are free once the previous stores have read them
          if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
          __syncwarp();
          issue_field(0, cb_of(0));
          if (dbl && cb_of(2) < ncb) issue_field(1, cb_of(2));
        }
      }
      if (!mbar_wait(&tfull[buf], (uint32_t)(li >> 1) & 1u, budget)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tacc = tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)buf * acc_stride;
      const bool tstore = !BETA && q.tma_store;
      for (int k = 0; cb_of(k) < ncb; ++k) {
        const int cb = cb_of(k);
        const bool more = cb_of(k + 1) < ncb;
        if (more) load_aux(cb_of(k + 1), nxt);
        const int mh = mc * Mt + cb * 16;
        float osc[16], prev[16];
        if (pin) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int m = mh + j;
            const bool ok = m < d.M;
            if (H16 && EPI == JFG_EPI_DIV_EIG) osc[j] = ok ? __ldg(oinv + m) * xinv : 0.f;
            if (BETA) prev[j] = ok ? outS[(long long)m * d.out_ld + p] : 0.f;
          }
        }
        float v[16];
        tmem_ld16(tacc + (uint32_t)(cb * 16), v);
        float* cbox = box_of(dbl ? (k >> 1) : 0);  // this output box's staging box
        if (tstore) {
          // stage this warp's 32 (p) x 32 (m) box in shared memory, [m][p] with
          // p contiguous, and store it with one bulk tensor copy (out-of-range
          // rows and columns are clipped by the copy)
          if ((k & 1) == 0) {
            if (tfld) {
              const int j = dbl ? (k >> 1) : 0;
              if (!dbl && k > 0) {
                if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                __syncwarp();
                issue_field(0, cb);
              }
              if (!mbar_wait(&fbar[2 * ew + j], (fph >> j) & 1u, budget)) {
                fok = false;
                break;
              }
              fph ^= 1u << j;
              fpend &= ~(1u << j);
            } else {
              if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
              __syncwarp();
            }
          }
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            float r = v[j];  // rows outside the problem are clipped by the store
            // a = the contraction before the epilogue factor (operator and
            // input scales applied), for the fused dot sum(a * out)
            float a = r;
            if (EPI != JFG_EPI_NONE || H16)
              r *= (EPI == JFG_EPI_DIV_EIG) ? 1.f : (pin ? aux[j] * xs : 0.f);
            if (tfld) a = r;  // aux held only the scales; the field comes next
            if (tfld) r *= cbox[(16 * (k & 1) + j) * 32 + lane];
            if (H16 && EPI == JFG_EPI_DIV_EIG) r *= pin ? osc[j] : 0.f;
            if (EPI == JFG_EPI_DIV_EIG) {
              a = r;
              r = __fdividef(r, c0 + c1 * ((pin ? aux[j] : 1.f) + lp));
            }
            r *= alpha;
            if (fdot) dsum = fmaf(a, r, dsum);
            if (H16) omax = fmaxf(omax, fabsf(r));
            cbox[(16 * (k & 1) + j) * 32 + lane] = r;
          }
          if ((k & 1) == 1 || !more || cb_of(k + 1) != cb + 1) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0 && b >= 0)
              tma_store_4d(&L.maps[gi][3], cbox, pt * TILE_P + 32 * q4, mc * Mt + (cb & ~1) * 16,
                           s, b);
            if (lane == 0) asm volatile("cp.async.bulk.commit_group;" ::: "memory");
          }
        } else if (pin) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int m = mh + j;
            if (m < d.M) {
              float r = v[j];
              float a = r;  // (split FP16 with the field in aux fuses no dot)
              if (EPI != JFG_EPI_NONE || H16) r *= (EPI == JFG_EPI_DIV_EIG) ? 1.f : aux[j] * xs;
              if (H16 && EPI == JFG_EPI_DIV_EIG) r *= osc[j];
              if (EPI == JFG_EPI_DIV_EIG) {
                a = r;
                r = __fdividef(r, c0 + c1 * (aux[j] + lp));
              }
              r *= alpha;
              if (fdot) dsum = fmaf(a, r, dsum);
              if (BETA) r += beta * prev[j];
              if (H16) omax = fmaxf(omax, fabsf(r));
              outS[(long long)m * d.out_ld + p] = r;
            }
          }
        }
        if (more) {
#pragma unroll
          for (int j = 0; j < 16; ++j) aux[j] = nxt[j];
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[buf]);
      if (fdot) {
        // this warp's partial of the tile, one deterministic slot each
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
        const int mch = (d.M + Mt - 1) / Mt, npt = (d.P + TILE_P - 1) / TILE_P;
        if (lane == 0 && b >= 0)
          q.dot_part[(long long)b * DOT_NBMAX + ((s * mch + mc) * npt + pt) * 8 + ew] = dsum;
      }
      if (H16 && q.out_max != nullptr) {
        // max |output| of this tile for the next pass's input scale (float
        // bits of non-negative values order like unsigned integers)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) omax = fmaxf(omax, __shfl_xor_sync(0xffffffffu, omax, o));
        if (lane == 0 && b >= 0) atomicMax(q.out_max + b, __float_as_uint(omax));
      }
    }
    // field box loads still in flight (after a timeout) land before exit
    for (int j = 0; j < 2; ++j)
      if (fpend & (1u << j)) mbar_wait(&fbar[2 * ew + j], (fph >> j) & 1u, WAIT_NS);
    // bulk tensor stores of this warp complete before the kernel ends
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(L.tmem_cols)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
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

int make_map(CUtensorMap* map, const void* base, int rank, const cuuint64_t* dims,
             const cuuint64_t* strides_bytes, const cuuint32_t* box,
             CUtensorMapDataType dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
             CUtensorMapSwizzle sw = CU_TENSOR_MAP_SWIZZLE_128B) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return JFG_ERR_UNSUPPORTED;
  cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  CUresult r = fn(map, dt, (cuuint32_t)rank, (void*)base, dims,
                  strides_bytes, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? JFG_OK : JFG_ERR_ARG;
}

// the plain BF16 kernel exists for the epilogues of the fast diagonalisation
template <int E>
int set_attr_b1(int mx) {
  if constexpr (E != JFG_EPI_MUL_FIELD)
    JFG_CUDA_TRY(cudaFuncSetAttribute(k_contract_tc<E, false, 1, 3>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
  return JFG_OK;
}

// Opt every kernel variant into the largest dynamic shared-memory size once
// per device (before any stream capture can be active in the caller).
int setup_kernel_attr() {
  static bool done[64] = {};
  int dev = 0;
  JFG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return JFG_ERR_UNSUPPORTED;
  if (!done[dev]) {
    const int mx = SMEM_MAX;
#define JFG_SET_ATTR(E, B, G)                                                              \
  JFG_CUDA_TRY(cudaFuncSetAttribute(k_contract_tc<E, B, G, 0>,                             \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, mx));     \
  JFG_CUDA_TRY(cudaFuncSetAttribute(k_contract_tc<E, B, G, 1>,                             \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, mx));     \
  if (G == 1)                                                                              \
  JFG_CUDA_TRY(cudaFuncSetAttribute(k_contract_tc<E, B, 1, 2>,                             \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, mx));     \
  if (G == 1 && !B) JFG_TRY(set_attr_b1<E>(mx))
#define JFG_SET_ATTR_G(G)                   \
  JFG_SET_ATTR(JFG_EPI_NONE, false, G);     \
  JFG_SET_ATTR(JFG_EPI_NONE, true, G);      \
  JFG_SET_ATTR(JFG_EPI_MUL_FIELD, false, G); \
  JFG_SET_ATTR(JFG_EPI_MUL_FIELD, true, G); \
  JFG_SET_ATTR(JFG_EPI_DIV_EIG, false, G);  \
  JFG_SET_ATTR(JFG_EPI_DIV_EIG, true, G)
    JFG_SET_ATTR_G(1);
    JFG_SET_ATTR_G(GMAX);
#undef JFG_SET_ATTR_G
#undef JFG_SET_ATTR
    done[dev] = true;
  }
  return JFG_OK;
}

// Validate one group and fill its descriptor, tile height and tensor maps.
// prec: 0 the operator is TF32 in FP32 words; 1 BF16 (hi, lo) and 2 FP16
// (hi, lo), both with 64-element K blocks; 3 BF16 hi only (op_lo unused).
int fill_group(const jfg_contract_desc& d, const void* op_hi, const void* op_lo,
               const float* in, float* out, TcGroup& q, CUtensorMap* maps, int prec,
               int mt_cap) {
  const bool b16 = prec != 0;
  JFG_TRY(validate_desc(d));
  const bool lo = prec != 3;
  if (!op_hi || (lo && !op_lo) || !in || !out) return JFG_ERR_ARG;
  // TMA: 16-byte aligned bases and strides
  auto al16 = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
  if (!al16(op_hi) || (lo && !al16(op_lo)) || !al16(in)) return JFG_ERR_ARG;
  const int om = b16 ? 7 : 3;  // operator strides in elements: multiples of 16 bytes
  if ((d.op_ld & om) || (d.in_ld & 3) || (d.op_seg & om) || (d.in_seg & 3) || (d.in_batch & 3))
    return JFG_ERR_ARG;
  if ((long long)d.batch * d.nseg > 65535) return JFG_ERR_ARG;
  q.d = d;
  q.out = out;
  const int cap = (mt_cap > 0 && mt_cap < MT_MAX) ? mt_cap : MT_MAX;
  q.Mtile = ((d.M > cap ? cap : d.M) + 15) / 16 * 16;
  q.seg_in_map = (d.nseg > 1 && d.in_seg != 0) ? 1 : 0;
  q.bat_in_map = (d.batch > 1 && d.in_batch != 0) ? 1 : 0;
  q.seg_op_map = (d.nseg > 1 && d.op_seg != 0) ? 1 : 0;
  // inputs that do not stay in L2 are read once if their operator chunks run together
  q.mc_inner = (double)d.P * d.K * 4.0 * d.batch * d.nseg > 64.0 * 1024 * 1024 ? 1 : 0;
  {
    cuuint64_t dims[4] = {(cuuint64_t)d.K, (cuuint64_t)d.P,
                          (cuuint64_t)(q.seg_in_map ? d.nseg : 1),
                          (cuuint64_t)(q.bat_in_map ? d.batch : 1)};
    cuuint64_t str[3] = {(cuuint64_t)d.in_ld * 4,
                         (cuuint64_t)(q.seg_in_map ? d.in_seg : d.in_ld * d.P) * 4,
                         (cuuint64_t)(q.bat_in_map ? d.in_batch : d.in_ld * d.P) * 4};
    cuuint32_t box[4] = {KB, TILE_P, 1, 1};
    JFG_TRY(make_map(&maps[0], in, 4, dims, str, box));
  }
  {
    const int eb = b16 ? 2 : 4;
    cuuint64_t dims[3] = {(cuuint64_t)d.K, (cuuint64_t)d.M,
                          (cuuint64_t)(q.seg_op_map ? d.nseg : 1)};
    cuuint64_t str[2] = {(cuuint64_t)d.op_ld * eb,
                         (cuuint64_t)(q.seg_op_map ? d.op_seg : d.op_ld * d.M) * eb};
    // one operator row of a stage per box row: 128 B (TF32) or 64 B (16-bit)
    const int orow = b16 ? 2 * b16_ke(d.epilogue) : 128;
    cuuint32_t box[3] = {(cuuint32_t)(orow / eb), (cuuint32_t)q.Mtile, 1};
    const CUtensorMapDataType dt = prec == 2 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                   : b16     ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                             : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const CUtensorMapSwizzle sw =
        orow == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B;
    JFG_TRY(make_map(&maps[1], op_hi, 3, dims, str, box, dt, sw));
    if (lo) JFG_TRY(make_map(&maps[2], op_lo, 3, dims, str, box, dt, sw));
  }
  // output through TMA stores when its rows are 16-byte aligned and every
  // 32-column group of a tile is full (else plain coalesced stores)
  q.tma_store = 0;
  if (al16(out) && (d.out_ld & 3) == 0 && (d.out_seg & 3) == 0 && (d.out_batch & 3) == 0 &&
      q.Mtile % 32 == 0 && d.beta == 0.0) {
    cuuint64_t dims[4] = {(cuuint64_t)d.P, (cuuint64_t)d.M, (cuuint64_t)d.nseg,
                          (cuuint64_t)d.batch};
    cuuint64_t str[3] = {(cuuint64_t)d.out_ld * 4,
                         (cuuint64_t)(d.nseg > 1 ? d.out_seg : d.out_ld * d.M) * 4,
                         (cuuint64_t)(d.batch > 1 ? d.out_batch : d.out_ld * d.M) * 4};
    cuuint32_t box[4] = {32, 32, 1, 1};
    EncodeTiledFn fn = encode_fn();
    cuuint32_t estr[4] = {1, 1, 1, 1};
    if (fn && fn(&maps[3], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (void*)out, dims, str, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                 CU_TENSOR_MAP_L2_PROMOTION_NONE,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
      q.tma_store = 1;
  }
  return JFG_OK;
}

long long group_tiles(const TcGroup& q) {
  return (long long)((q.d.P + TILE_P - 1) / TILE_P) * ((q.d.M + q.Mtile - 1) / q.Mtile) *
         q.d.batch * q.d.nseg;
}

// One launch over ng <= G groups (same epilogue kind and beta != 0 for all).
// The scaled split-FP16 kernel exists for single-group launches only.
template <int E, bool BETA, int G>
void launch_h16(dim3 grid, size_t smem, cudaStream_t st, const TcLaunch<G>& L) {
  if constexpr (G == 1) k_contract_tc<E, BETA, 1, 2><<<grid, NTHREADS, smem, st>>>(L);
}
// ... and so does the plain BF16 kernel (the fast diagonalisation's passes:
// no beta, no field)
template <int E, bool BETA, int G>
void launch_b1(dim3 grid, size_t smem, cudaStream_t st, const TcLaunch<G>& L) {
  if constexpr (G == 1 && !BETA && E != JFG_EPI_MUL_FIELD)
    k_contract_tc<E, false, 1, 3><<<grid, NTHREADS, smem, st>>>(L);
}

// h16 (one group only): the scaled split-FP16 auxiliaries of that group.
struct H16Aux {
  const unsigned* in_max;
  unsigned* out_max;
  const float* op_inv;
  long long op_inv_seg;
};

template <int G>
int launch_groups(int ng, const jfg_contract_desc* const* ds, const void* const* op_hi,
                  const void* const* op_lo, const float* const* in, float* const* out,
                  const jfg_tc_config& cfg, int prec, cudaStream_t st,
                  const H16Aux* h16 = nullptr, const DotOut* dot = nullptr) {
  if (dot && dot->nb) *dot->nb = 0;
  const bool b16 = prec != 0;
  if (prec == 2 && (G != 1 || ng != 1 || !h16 || !h16->op_inv)) return JFG_ERR_ARG;
  if (prec == 3 && (G != 1 || ng != 1 || ds[0]->beta != 0.0 ||
                    ds[0]->epilogue == JFG_EPI_MUL_FIELD))
    return JFG_ERR_ARG;
  static_assert(sizeof(TcLaunch<G>) <= 32000, "kernel parameter block too large");
  TcLaunch<G> L;
  memset(&L, 0, sizeof(L));
  L.ngroups = ng;
  const int epi = ds[0]->epilogue;
  const bool hb = ds[0]->beta != 0.0;
  long long tiles = 0;
  int mt_max = 16, ostage = 0;
  for (int i = 0; i < ng; ++i) {
    if (ds[i]->epilogue != epi || (ds[i]->beta != 0.0) != hb) return JFG_ERR_ARG;
    JFG_TRY(fill_group(*ds[i], op_hi[i], op_lo[i], in[i], out[i], L.g[i], L.maps[i], prec,
                       cfg.mtile));
    if (h16) {
      L.g[i].in_max = h16->in_max;
      L.g[i].out_max = h16->out_max;
      L.g[i].op_inv = h16->op_inv;
      L.g[i].op_inv_seg = h16->op_inv_seg;
    }
    if (cfg.store == 2 || (cfg.store == 0 && !g_tma_store)) L.g[i].tma_store = 0;
    // single-group field-multiply launches fetch the field's 32 x 32 boxes
    // by TMA into the epilogue's staging boxes (16-byte aligned rows needed)
    TcGroup& q = L.g[i];
    const jfg_contract_desc& d = *ds[i];
    if (G == 1 && ng == 1 && d.epilogue == JFG_EPI_MUL_FIELD && q.tma_store && d.field &&
        ((uintptr_t)d.field & 15u) == 0 && (d.field_ld & 3) == 0 && (d.field_seg & 3) == 0 &&
        (d.field_batch & 3) == 0) {
      q.fld_seg = (d.nseg > 1 && d.field_seg != 0) ? 1 : 0;
      q.fld_bat = (d.batch > 1 && d.field_batch != 0) ? 1 : 0;
      const cuuint64_t plane = (cuuint64_t)d.field_ld * d.M;
      cuuint64_t dims[4] = {(cuuint64_t)d.P, (cuuint64_t)d.M,
                            (cuuint64_t)(q.fld_seg ? d.nseg : 1),
                            (cuuint64_t)(q.fld_bat ? d.batch : 1)};
      cuuint64_t str[3] = {(cuuint64_t)d.field_ld * 4,
                           (q.fld_seg ? (cuuint64_t)d.field_seg : plane) * 4,
                           (q.fld_bat ? (cuuint64_t)d.field_batch : plane) * 4};
      cuuint32_t box[4] = {32, 32, 1, 1};
      cuuint32_t estr[4] = {1, 1, 1, 1};
      EncodeTiledFn fn = encode_fn();
      q.tma_field = (fn && fn(&L.fmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (void*)d.field, dims,
                              str, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
                         ? 1
                         : 0;
    }
    tiles += group_tiles(L.g[i]);
    if (L.g[i].Mtile > mt_max) mt_max = L.g[i].Mtile;
    ostage |= L.g[i].tma_store;
  }
  if (tiles == 0) return JFG_OK;
  int dev = 0, nsm = 0;
  JFG_CUDA_TRY(cudaGetDevice(&dev));
  JFG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  int ctas = cfg.ctas > 0 && cfg.ctas < nsm ? cfg.ctas : nsm;
  const int ta = (b16 || cfg.operand_a_in_tmem) ? 1 : 0;
  // Operator-stationary schedule (16-bit operators, one group): each CTA keeps
  // its operator chunk (every K block, hi and lo) in shared memory and streams
  // only input tiles, halving the L2-to-SM traffic per tile.  Used when the
  // chunk leaves room for >= 2 input stages and every slot gets >= 2 tiles
  // per CTA.
  bool res = false;
  int nslots = 0;
  size_t res_bytes = 0;
  const int sched = cfg.schedule == 1 ? 0 : cfg.schedule == 2 ? 2 : g_op_resident;
  if (b16 && prec != 3 && ng == 1 && sched) {
    const TcGroup& q = L.g[0];
    const int mch = (q.d.M + q.Mtile - 1) / q.Mtile;
    nslots = q.d.nseg * mch;
    res_bytes = (size_t)((q.d.K + b16_ke(epi) - 1) / b16_ke(epi)) * 2 * (size_t)q.Mtile * 2 *
                b16_ke(epi);
    const long long per_slot = (long long)((q.d.P + TILE_P - 1) / TILE_P) * q.d.batch;
    const size_t room = (size_t)SMEM_MAX - 1024 - 64 * 8;
    res = nslots <= ctas && (sched == 2 || per_slot * nslots >= 2LL * ctas) &&
          res_bytes + 2 * (size_t)(b16_ke(epi) / KB) * XBYTES <= room;
  }
  const int ke16 = b16_ke(epi);
  const size_t xstage = (size_t)(ke16 / KB) * XBYTES;  // FP32 input of a 16-bit stage
  const size_t stage = res ? xstage
                           : b16 ? xstage + (prec == 3 ? 1 : 2) * (size_t)mt_max * 2 * ke16
                                 : (ta ? 1 : 2) * (size_t)XBYTES + 2 * (size_t)mt_max * 128;
  // field-multiply launches stage both of a warp's boxes of a tile (the
  // field of each fetched ahead), when two pipeline stages still fit
  int nbuf = ostage ? 1 : 0;
  if (!res && ng == 1 && L.g[0].tma_field &&
      (size_t)SMEM_MAX - 1024 - 64 * 8 - 16 * (size_t)STAGE_OUT >= 2 * stage)
    nbuf = 2;
  size_t ob = 8 * (size_t)STAGE_OUT * nbuf;
  const size_t fixed = 1024 + (res ? res_bytes : 0) + 64 * 8;
  int stages = (int)(((size_t)SMEM_MAX - fixed - ob) / stage);
  if (res && stages < 3 && ostage && ((size_t)SMEM_MAX - fixed) / stage > (size_t)stages) {
    // three input stages matter more than the TMA-store staging boxes
    ostage = 0;
    nbuf = 0;
    ob = 0;
    L.g[0].tma_store = 0;
    stages = (int)(((size_t)SMEM_MAX - fixed) / stage);
  }
  // operand A in TMEM: 256 accumulator columns plus one A slot per stage
  const int amax = ta ? 256 / (b16 ? ke16 : 2 * KB) : 6;
  if (stages > amax) stages = amax;  // <= 8: the kernel's per-stage tables hold 16
  if (cfg.stages >= 2 && cfg.stages < stages) stages = cfg.stages;
  if (stages < 2) return JFG_ERR_UNSUPPORTED;
  L.stages = stages;
  L.tmem_cols = 512;  // two accumulator buffers (+ operand A stages in TMEM mode)
  L.tmem_a = ta;
  L.mt_max = mt_max;
  L.out_stage = nbuf;
  L.op_res = res ? 1 : 0;
  L.nslots = res ? nslots : 0;
  if (dot && dot->part && ng == 1) {
    // fused dot: field or divide epilogue, <= DOT_NBMAX partials per problem;
    // split FP16 with the field loaded per element keeps the factors folded
    // and fuses none
    TcGroup& q = L.g[0];
    const int e = q.d.epilogue;
    const long long nb = (long long)q.d.nseg * ((q.d.M + q.Mtile - 1) / q.Mtile) *
                         ((q.d.P + TILE_P - 1) / TILE_P) * 8;
    if ((e == JFG_EPI_DIV_EIG || (e == JFG_EPI_MUL_FIELD && (prec != 2 || q.tma_field))) &&
        q.d.beta == 0.0 && nb <= DOT_NBMAX) {
      q.dot_part = dot->part;
      if (dot->nb) *dot->nb = (int)nb;
    }
  }
  const size_t smem = 1024 + res_bytes * (res ? 1 : 0) + stages * stage + ob +
                      (3 * stages + 23) * 8 + 16;
  if (smem > (size_t)SMEM_MAX) return JFG_ERR_UNSUPPORTED;
  long long nct = tiles < ctas ? tiles : ctas;
  if (res) nct = (long long)(ctas / nslots) * nslots;  // the same CTA count per slot
  dim3 grid((unsigned)nct);
  JFG_TRY(setup_kernel_attr());
#define JFG_LAUNCH(E)                                                          \
  do {                                                                         \
    if (prec == 2) {                                                           \
      if (hb)                                                                  \
        launch_h16<E, true, G>(grid, smem, st, L);                             \
      else                                                                     \
        launch_h16<E, false, G>(grid, smem, st, L);                            \
    } else if (prec == 3) {                                                    \
      launch_b1<E, false, G>(grid, smem, st, L);                               \
    } else if (b16) {                                                          \
      if (hb)                                                                  \
        k_contract_tc<E, true, G, 1><<<grid, NTHREADS, smem, st>>>(L);         \
      else                                                                     \
        k_contract_tc<E, false, G, 1><<<grid, NTHREADS, smem, st>>>(L);        \
    } else {                                                                   \
      if (hb)                                                                  \
        k_contract_tc<E, true, G, 0><<<grid, NTHREADS, smem, st>>>(L);         \
      else                                                                     \
        k_contract_tc<E, false, G, 0><<<grid, NTHREADS, smem, st>>>(L);        \
    }                                                                          \
  } while (0)
  switch (epi) {
    case JFG_EPI_NONE:
      JFG_LAUNCH(JFG_EPI_NONE);
      break;
    case JFG_EPI_MUL_FIELD:
      JFG_LAUNCH(JFG_EPI_MUL_FIELD);
      break;
    case JFG_EPI_DIV_EIG:
      JFG_LAUNCH(JFG_EPI_DIV_EIG);
      break;
    default:
      return JFG_ERR_ARG;
  }
#undef JFG_LAUNCH
  JFG_LAUNCHED();
  return JFG_OK;
}

}  // namespace

int tc_setup() {
  if (!encode_fn()) return JFG_ERR_UNSUPPORTED;
  return setup_kernel_attr();
}

jfg_tc_config tc_default_config() {
  jfg_tc_config c;
  c.operand_a_in_tmem = g_operand_a_in_tmem;
  c.order = 0;
  c.ctas = 0;
  c.stages = 0;
  c.mtile = 0;
  c.schedule = 0;
  c.store = 0;
  return c;
}

// ---- single-group launches: tuned configurations -------------------------

struct SingleTuned {
  jfg_tc_config cfg;
  float ms;
};
std::mutex g_single_mu;
std::map<std::string, SingleTuned> g_single;
int g_tune_single = 0;

std::string single_signature(int prec, const jfg_contract_desc& d) {
  int dev = 0;
  cudaGetDevice(&dev);
  char buf[200];
  snprintf(buf, sizeof buf, "d%d:p%d:b%d:s%d:M%d:P%d:K%d:e%d:beta%d", dev, prec, d.batch, d.nseg,
           d.M, d.P, d.K, d.epilogue, d.beta != 0.0 ? 1 : 0);
  return buf;
}

// Time every candidate configuration of this launch on its own operands and
// keep the fastest for its signature.
int tune_single(int prec, const jfg_contract_desc& d, const void* oh, const void* ol,
                const float* in, float* out, const H16Aux* aux, cudaStream_t st,
                const std::string& key, jfg_tc_config* best) {
  const jfg_contract_desc* dp = &d;
  std::vector<jfg_tc_config> cands;
  for (int ta : {1, 0})
    for (int sched : {1, 2})
      for (int sg : {0, 3, 2})
        for (int store : {1, 2})
          for (int mt : {0, 64}) {
            if ((prec != 0 && ta == 0) || ((prec == 0 || prec == 3) && sched == 2)) continue;
            // the operator-stationary schedule only where the chunk fits beside
            // two input stages (else the launch would stream anyway)
            if (sched == 2 && (size_t)((d.K + b16_ke(d.epilogue) - 1) / b16_ke(d.epilogue)) *
                                          2 * (mt ? mt : 128) * 2 * b16_ke(d.epilogue) +
                                      2 * (size_t)(b16_ke(d.epilogue) / KB) * XBYTES >
                                  (size_t)SMEM_MAX - 1024 - 64 * 8)
              continue;
            jfg_tc_config c = tc_default_config();
            c.operand_a_in_tmem = ta;
            c.schedule = sched;
            c.stages = sg;
            c.store = store;
            c.mtile = mt;
            cands.push_back(c);
          }
  cudaEvent_t e0, e1;
  JFG_CUDA_TRY(cudaEventCreate(&e0));
  JFG_CUDA_TRY(cudaEventCreate(&e1));
  const int reps = 3;
  float bt = -1.f;
  jfg_tc_config bc = tc_default_config();
  int status = JFG_OK;
  for (const jfg_tc_config& c : cands) {
    int s = launch_groups<1>(1, &dp, &oh, &ol, &in, &out, c, prec, st, aux);  // warm
    if (s == JFG_ERR_UNSUPPORTED) continue;  // does not fit: not a candidate
    if (s != JFG_OK) {
      status = s;
      break;
    }
    if (cudaEventRecord(e0, st) != cudaSuccess) {
      status = JFG_ERR_CUDA;
      break;
    }
    for (int r = 0; r < reps && s == JFG_OK; ++r)
      s = launch_groups<1>(1, &dp, &oh, &ol, &in, &out, c, prec, st, aux);
    float ms = 0.f;
    if (s != JFG_OK || cudaEventRecord(e1, st) != cudaSuccess ||
        cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      status = s != JFG_OK ? s : JFG_ERR_CUDA;
      break;
    }
    ms /= (float)reps;
    if (bt < 0.f || ms < bt) {
      bt = ms;
      bc = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (status != JFG_OK) return status;
  if (bt >= 0.f) {
    std::lock_guard<std::mutex> lk(g_single_mu);
    g_single[key] = SingleTuned{bc, bt};
  }
  *best = bc;
  return JFG_OK;
}

// One single-group launch with the tuned configuration of its signature (or
// the default); with autotuning on, an untuned signature launched outside
// stream capture is tuned first.
// jfg_tc_force_config: one configuration for every single-group launch
// (tests and tuning studies), instead of the tuned or default one
bool g_force_on = false;
jfg_tc_config g_force_cfg;

int launch_single(int prec, const jfg_contract_desc& d, const void* oh, const void* ol,
                  const float* in, float* out, const H16Aux* aux, cudaStream_t st,
                  const DotOut* dot = nullptr) {
  const jfg_contract_desc* dp = &d;
  jfg_tc_config cfg = tc_default_config();
  const std::string key = single_signature(prec, d);
  bool found = false;
  {
    std::lock_guard<std::mutex> lk(g_single_mu);
    if (g_force_on) {
      cfg = g_force_cfg;
      found = true;
    } else {
      auto it = g_single.find(key);
      if (it != g_single.end()) {
        cfg = it->second.cfg;
        found = true;
      }
    }
  }
  if (!found && g_tune_single) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    JFG_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
    if (cs == cudaStreamCaptureStatusNone)
      JFG_TRY(tune_single(prec, d, oh, ol, in, out, aux, st, key, &cfg));
  }
  return launch_groups<1>(1, &dp, &oh, &ol, &in, &out, cfg, prec, st, aux, dot);
}

int contract_tc(const jfg_contract_desc& d, const float* op_hi, const float* op_lo,
                const float* in, float* out, cudaStream_t st, const DotOut* dot) {
  if (dot && dot->nb) *dot->nb = 0;
  if (d.batch == 0 || d.M == 0 || d.P == 0) return validate_desc(d);
  return launch_single(0, d, op_hi, op_lo, in, out, nullptr, st, dot);
}

int contract_tc_b16(const jfg_contract_desc& d, const uint16_t* op_hi, const uint16_t* op_lo,
                    const float* in, float* out, cudaStream_t st, const DotOut* dot) {
  if (dot && dot->nb) *dot->nb = 0;
  if (d.batch == 0 || d.M == 0 || d.P == 0) return validate_desc(d);
  return launch_single(op_lo ? 1 : 3, d, op_hi, op_lo, in, out, nullptr, st, dot);
}

int contract_tc_h16(const jfg_contract_desc& d, const uint16_t* op_hi, const uint16_t* op_lo,
                    const float* op_inv, long long op_inv_seg, const unsigned* in_max,
                    unsigned* out_max, const float* in, float* out, cudaStream_t st,
                    const DotOut* dot) {
  if (dot && dot->nb) *dot->nb = 0;
  if (d.batch == 0 || d.M == 0 || d.P == 0) return validate_desc(d);
  if (!op_inv || !in_max) return JFG_ERR_ARG;
  const H16Aux aux{in_max, out_max, op_inv, op_inv_seg};
  return launch_single(2, d, op_hi, op_lo, in, out, &aux, st, dot);
}

void set_single_autotune(int on) { g_tune_single = on; }
int single_autotune() { return g_tune_single; }

int contract_tc_grouped(int ng, const jfg_contract_desc* ds, const float* const* op_hi,
                        const float* const* op_lo, const float* const* in, float* const* out,
                        const jfg_tc_config& cfg, cudaStream_t st) {
  if (ng < 0 || (ng > 0 && (!ds || !op_hi || !op_lo || !in || !out))) return JFG_ERR_ARG;
  if (cfg.order < 0 || cfg.order > 2 || cfg.stages < 0 || cfg.ctas < 0 ||
      (cfg.mtile != 0 && cfg.mtile != 64))
    return JFG_ERR_ARG;
  // launch order of the groups: as given, by operator-tile work (K * Mtile,
  // largest first), or by total work (largest first)
  std::vector<int> ord;
  ord.reserve(ng);
  for (int i = 0; i < ng; ++i)
    if (ds[i].batch > 0 && ds[i].M > 0 && ds[i].P > 0) ord.push_back(i);
    else JFG_TRY(validate_desc(ds[i]));
  auto work = [&](int i) {
    const double mt = ds[i].M < MT_MAX ? ds[i].M : MT_MAX;
    const double tile = (double)ds[i].K * mt;
    if (cfg.order == 1) return tile;
    return tile * (double)((ds[i].P + TILE_P - 1) / TILE_P) *
           (double)((ds[i].M + MT_MAX - 1) / MT_MAX) * ds[i].batch * ds[i].nseg;
  };
  if (cfg.order != 0)
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return work(a) > work(b); });
  for (size_t c0 = 0; c0 < ord.size(); c0 += GMAX) {
    const int n = (int)(ord.size() - c0 < (size_t)GMAX ? ord.size() - c0 : GMAX);
    const jfg_contract_desc* dp[GMAX];
    const void* oh[GMAX];
    const void* ol[GMAX];
    const float* ip[GMAX];
    float* op[GMAX];
    for (int k = 0; k < n; ++k) {
      const int i = ord[c0 + k];
      dp[k] = &ds[i];
      oh[k] = op_hi[i];
      ol[k] = op_lo[i];
      ip[k] = in[i];
      op[k] = out[i];
    }
    if (n == 1)
      JFG_TRY(launch_groups<1>(1, dp, oh, ol, ip, op, cfg, 0, st));
    else
      JFG_TRY(launch_groups<GMAX>(n, dp, oh, ol, ip, op, cfg, 0, st));
  }
  return JFG_OK;
}

int tc_status_take(int* status) {
  int zero = 0;
  JFG_CUDA_TRY(cudaMemcpyFromSymbol(status, g_tc_status, sizeof(int)));
  JFG_CUDA_TRY(cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(int)));
  return JFG_OK;
}

}  // namespace jfg

extern "C" int jfg_contract_tc(const jfg_contract_desc* d, const float* op_hi,
                               const float* op_lo, const float* in, float* out, void* stream) {
  if (!d) return JFG_ERR_ARG;
  return jfg::contract_tc(*d, op_hi, op_lo, in, out, (cudaStream_t)stream);
}

extern "C" int jfg_contract_tc_bf16x3(const jfg_contract_desc* d, const uint16_t* op_hi,
                                      const uint16_t* op_lo, const float* in, float* out,
                                      void* stream) {
  if (!d) return JFG_ERR_ARG;
  return jfg::contract_tc_b16(*d, op_hi, op_lo, in, out, (cudaStream_t)stream);
}

extern "C" int jfg_contract_tc_f16x3(const jfg_contract_desc* d, const uint16_t* op_hi,
                                     const uint16_t* op_lo, const float* op_inv,
                                     long long op_inv_seg, const unsigned* in_max,
                                     unsigned* out_max, const float* in, float* out,
                                     void* stream) {
  if (!d) return JFG_ERR_ARG;
  return jfg::contract_tc_h16(*d, op_hi, op_lo, op_inv, op_inv_seg, in_max, out_max, in, out,
                              (cudaStream_t)stream);
}

extern "C" void jfg_split_bf16_host(size_t n, const double* src, uint16_t* hi, uint16_t* lo) {
  auto bits = [](float f) -> uint32_t {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) return u >> 16;  // inf / nan: truncate
    return (u + 0x7FFFu + ((u >> 16) & 1u)) >> 16;         // round to nearest even
  };
  auto value = [](uint32_t b) -> float {
    const uint32_t u = b << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
  };
  for (size_t i = 0; i < n; ++i) {
    const uint32_t h = bits((float)src[i]);
    const uint32_t l = bits((float)(src[i] - (double)value(h)));
    hi[i] = (uint16_t)h;
    lo[i] = (uint16_t)l;
  }
}

extern "C" int jfg_tc_set_store_path(int tma_store) {
  if (tma_store != 0 && tma_store != 1) return JFG_ERR_ARG;
  jfg::g_tma_store = tma_store;
  return JFG_OK;
}

extern "C" int jfg_tc_set_wait_budget_ns(unsigned long long ns) {
  const unsigned long long v = ns == 0 ? jfg::WAIT_NS_DEFAULT : ns;
  JFG_CUDA_TRY(cudaMemcpyToSymbol(jfg::g_tc_wait_ns, &v, sizeof(v)));
  return JFG_OK;
}

extern "C" int jfg_tc_test_hold(int on) {
  if (on != 0 && on != 1) return JFG_ERR_ARG;
  JFG_CUDA_TRY(cudaMemcpyToSymbol(jfg::g_tc_test_hold, &on, sizeof(on)));
  return JFG_OK;
}

extern "C" int jfg_tc_force_config(const jfg_tc_config* cfg) {
  std::lock_guard<std::mutex> lk(jfg::g_single_mu);
  jfg::g_force_on = cfg != nullptr;
  if (cfg) jfg::g_force_cfg = *cfg;
  return JFG_OK;
}

extern "C" int jfg_tc_set_autotune(int on) {
  if (on != 0 && on != 1) return JFG_ERR_ARG;
  jfg::set_single_autotune(on);
  return JFG_OK;
}

extern "C" int jfg_tc_tuned_count(void) {
  std::lock_guard<std::mutex> lk(jfg::g_single_mu);
  return (int)jfg::g_single.size();
}

extern "C" int jfg_tc_tuned_entry(int i, char* signature, size_t signature_len,
                                  jfg_tc_config* cfg, float* ms) {
  std::lock_guard<std::mutex> lk(jfg::g_single_mu);
  if (i < 0 || i >= (int)jfg::g_single.size()) return JFG_ERR_ARG;
  auto it = jfg::g_single.begin();
  std::advance(it, i);
  if (signature && signature_len > 0) snprintf(signature, signature_len, "%s", it->first.c_str());
  if (cfg) *cfg = it->second.cfg;
  if (ms) *ms = it->second.ms;
  return JFG_OK;
}

extern "C" int jfg_tc_set_op_resident(int on) {
  if (on < 0 || on > 2) return JFG_ERR_ARG;
  jfg::g_op_resident = on;
  return JFG_OK;
}

extern "C" int jfg_tc_set_variant(int operand_a_in_tmem) {
  if (operand_a_in_tmem != 0 && operand_a_in_tmem != 1) return JFG_ERR_ARG;
  jfg::g_operand_a_in_tmem = operand_a_in_tmem;
  return JFG_OK;
}

namespace {

// Tuned configurations by launch signature (shapes, batch, epilogue of every group).
std::mutex g_tune_mu;
std::map<std::string, jfg_tc_config> g_tuned;

std::string signature(int ng, const jfg_contract_desc* ds) {
  std::string key;
  char buf[160];
  int dev = 0;
  cudaGetDevice(&dev);
  snprintf(buf, sizeof buf, "d%d:", dev);
  key += buf;
  for (int i = 0; i < ng; ++i) {
    const jfg_contract_desc& d = ds[i];
    snprintf(buf, sizeof buf, "%d,%d,%d,%d,%d,%d,%d;", d.batch, d.nseg, d.M, d.P, d.K,
             d.epilogue, d.beta != 0.0 ? 1 : 0);
    key += buf;
  }
  return key;
}

}  // namespace

extern "C" int jfg_contract_tc_grouped(int ngroups, const jfg_contract_desc* descs,
                                       const float* const* op_hi, const float* const* op_lo,
                                       const float* const* in, float* const* out,
                                       const jfg_tc_config* cfg, void* stream) {
  if (ngroups < 0 || (ngroups > 0 && !descs)) return JFG_ERR_ARG;
  jfg_tc_config c = jfg::tc_default_config();
  if (cfg) {
    c = *cfg;
  } else {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(signature(ngroups, descs));
    if (it != g_tuned.end()) c = it->second;
  }
  return jfg::contract_tc_grouped(ngroups, descs, op_hi, op_lo, in, out, c,
                                  (cudaStream_t)stream);
}

extern "C" int jfg_tc_autotune(int ngroups, const jfg_contract_desc* descs,
                               const float* const* op_hi, const float* const* op_lo,
                               const float* const* in, float* const* out, int reps,
                               jfg_tc_config* best, float* best_ms, void* stream) {
  if (ngroups < 1 || !descs || reps < 1) return JFG_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  JFG_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
  if (cap != cudaStreamCaptureStatusNone) return JFG_ERR_ARG;  // timing needs real launches
  std::vector<jfg_tc_config> cands;
  const int orders = ngroups > 1 ? 3 : 1;
  for (int ta = 1; ta >= 0; --ta)
    for (int o = 0; o < orders; ++o)
      for (int sg : {0, 3, 2})
        for (int mt : {0, 64}) {
          jfg_tc_config c;
          c.operand_a_in_tmem = ta;
          c.order = o;
          c.ctas = 0;
          c.stages = sg;
          c.mtile = mt;
          cands.push_back(c);
        }
  cudaEvent_t e0, e1;
  JFG_CUDA_TRY(cudaEventCreate(&e0));
  JFG_CUDA_TRY(cudaEventCreate(&e1));
  float bt = -1.f;
  jfg_tc_config bc = cands[0];
  int status = JFG_OK;
  for (const jfg_tc_config& c : cands) {
    status = jfg::contract_tc_grouped(ngroups, descs, op_hi, op_lo, in, out, c, st);  // warm
    if (status != JFG_OK) break;
    if (cudaEventRecord(e0, st) != cudaSuccess) { status = JFG_ERR_CUDA; break; }
    for (int r = 0; r < reps && status == JFG_OK; ++r)
      status = jfg::contract_tc_grouped(ngroups, descs, op_hi, op_lo, in, out, c, st);
    if (status != JFG_OK) break;
    float ms = 0.f;
    if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      status = JFG_ERR_CUDA;
      break;
    }
    ms /= (float)reps;
    if (bt < 0.f || ms < bt) {
      bt = ms;
      bc = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (status != JFG_OK) return status;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[signature(ngroups, descs)] = bc;
  }
  if (best) *best = bc;
  if (best_ms) *best_ms = bt;
  return JFG_OK;
}

extern "C" int jfg_device_status(void) {
  int s = 0, g = 0;
  int r = jfg::tc_status_take(&s);
  if (r != JFG_OK) return r;
  r = jfg::gemm_status_take(&g);
  if (r != JFG_OK) return r;
  return s != JFG_OK ? s : g;
}

extern "C" void jfg_split_tf32_host(size_t n, const double* src, float* hi, float* lo) {
  for (size_t i = 0; i < n; ++i) {
    const float f = (float)src[i];
    uint32_t u;
    memcpy(&u, &f, 4);
    // round-to-nearest onto the TF32 grid (10 explicit mantissa bits)
    uint32_t r = (u + 0x1000u) & 0xFFFFE000u;
    float h;
    memcpy(&h, &r, 4);
    if (!(h == h) || (h - h != 0.0f)) h = f;  // keep inf/nan as is
    hi[i] = h;
    lo[i] = (float)(src[i] - (double)h);
  }
}
