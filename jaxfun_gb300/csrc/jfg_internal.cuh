// Internal helpers shared by the jaxfun_gb300 CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "jaxfun_gb300.h"

namespace jfg {

// Last CUDA error observed on this host thread (reported by jfg_last_cuda_error).
void set_last_cuda_error(cudaError_t e);

// Kernel-launch accounting (jfg_launch_count): every launch site adds its
// launches; while a stream is being captured into a graph nothing is counted
// and each graph replay adds its kernel-node count instead.
void count_launches(long long n);
void set_capturing(bool on);

#define JFG_CUDA_TRY(expr)                              \
  do {                                                  \
    cudaError_t _e = (expr);                            \
    if (_e != cudaSuccess) {                            \
      ::jfg::set_last_cuda_error(_e);                   \
      return JFG_ERR_CUDA;                              \
    }                                                   \
  } while (0)

#define JFG_CHECK_LAUNCH()                              \
  do {                                                  \
    cudaError_t _e = cudaGetLastError();                \
    if (_e != cudaSuccess) {                            \
      ::jfg::set_last_cuda_error(_e);                   \
      return JFG_ERR_CUDA;                              \
    }                                                   \
  } while (0)

// after a <<<>>> launch: check it and count it
#define JFG_LAUNCHED()                                  \
  do {                                                  \
    JFG_CHECK_LAUNCH();                                 \
    ::jfg::count_launches(1);                           \
  } while (0)

#define JFG_TRY(expr)                                   \
  do {                                                  \
    int _s = (expr);                                    \
    if (_s != JFG_OK) return _s;                        \
  } while (0)

// A contraction operator: hi part (always) and, for the split-TF32 tensor-core
// path, the lo part with the same layout.
template <typename T>
struct OpRef {
  const T* hi;
  const T* lo;
  OpRef offset(long long o) const { return OpRef{hi + o, lo ? lo + o : nullptr}; }
};

// Dispatch of one contraction pass to an engine.
// DF: FP64 data, double-FP32 arithmetic (contract_df.cu).  TB: FP32 data on
// the tensor cores with a split-BF16 operator (OpRef<float> then points at
// BF16 arrays).  TH: FP32 data on the tensor cores as scaled split-FP16 pairs
// with a split-FP16 operator scaled per row (variable-coefficient apply only).
enum class Engine { F64, F32, TC, DF, TB, TH };

// Auxiliaries of the TH engine: the inverse row scales of the packed FP16
// operators and four per-problem max |x| slots (float bits, [4][batch]): the
// apply's input (slot 0) and the inputs of its passes 2-4 (slots 1-3).
struct H16Ops {
  const float* op_inv = nullptr;
  unsigned* slots = nullptr;  // [H16_SLOTS][batch]: max |x| of each pass's input
};
// per-problem max slots of a scaled split-FP16 operator apply (the 3-D one
// chains six)
constexpr int H16_SLOTS = 6;

// Fused dot product of a field-multiply or eigenvalue-divide pass: the
// epilogue writes, per problem b, partials part[b * DOT_NBMAX + i], i < *nb,
// of sum(acc * out) (acc the contraction before the epilogue factor, out the
// written value) -- p.Ap of the variable-coefficient operator in its field
// pass, r.M^-1 r of the fast diagonalisation in its divide pass.  The launch
// sets *nb (its tiles per problem x 8 epilogue warps), or 0 when the pass
// cannot produce it (then the caller computes the dot itself).
constexpr int DOT_NBMAX = 128;
struct DotOut {
  float* part = nullptr;
  int* nb = nullptr;
};

int contract_f64(const jfg_contract_desc& d, const double* op, const double* in, double* out,
                 cudaStream_t st);
int contract_f32(const jfg_contract_desc& d, const float* op, const float* in, float* out,
                 cudaStream_t st);
int contract_df64(const jfg_contract_desc& d, const double* op, const float2* op_pairs,
                  const double* in, double* out, cudaStream_t st, bool in_pairs = false,
                  bool out_pairs = false);
// dst[i] = (hi, lo) FP32 split of src[i] (the DF engine's pre-split operator)
int split_pairs_f64(const double* src, float2* dst, long long n, cudaStream_t st);
int contract_tc(const jfg_contract_desc& d, const float* op_hi, const float* op_lo,
                const float* in, float* out, cudaStream_t st, const DotOut* dot = nullptr);
// the same contraction with the operator as BF16 (hi, lo): three BF16 MMAs per product
int contract_tc_b16(const jfg_contract_desc& d, const uint16_t* op_hi, const uint16_t* op_lo,
                    const float* in, float* out, cudaStream_t st, const DotOut* dot = nullptr);
// the same contraction in scaled split FP16: operator (hi, lo) FP16 scaled per
// row with inverse scales op_inv[s * op_inv_seg + m]; the input of problem b
// is scaled by a power of two from in_max[b] (float bits of an upper bound on
// max |in[b]|); out_max[b] (optional, atomicMax) receives max |out[b]|
int contract_tc_h16(const jfg_contract_desc& d, const uint16_t* op_hi, const uint16_t* op_lo,
                    const float* op_inv, long long op_inv_seg, const unsigned* in_max,
                    unsigned* out_max, const float* in, float* out, cudaStream_t st,
                    const DotOut* dot = nullptr);
// ngroups contractions in persistent grouped launches (contract_tc.cu)
int contract_tc_grouped(int ng, const jfg_contract_desc* ds, const float* const* op_hi,
                        const float* const* op_lo, const float* const* in, float* const* out,
                        const jfg_tc_config& cfg, cudaStream_t st);
jfg_tc_config tc_default_config();
// Process-wide autotuning of single-group tensor-core launches (contract_tc.cu)
void set_single_autotune(int on);
int single_autotune();
// One-time per-device setup of the tensor-core kernels (shared-memory opt-in,
// tensor-map encoder); call before capturing their first launch into a graph.
int tc_setup();

inline int contract(Engine e, const jfg_contract_desc& d, OpRef<double> op, const double* in,
                    double* out, cudaStream_t st) {
  // DF: op.lo, when set, holds the operator pre-split into interleaved FP32
  // (hi, lo) pairs with the FP64 operator's element indexing (split_pairs_f64)
  if (e == Engine::DF) return contract_df64(d, op.hi, (const float2*)op.lo, in, out, st);
  return contract_f64(d, op.hi, in, out, st);
}
inline int contract(Engine e, const jfg_contract_desc& d, OpRef<float> op, const float* in,
                    float* out, cudaStream_t st, const DotOut* dot = nullptr) {
  if (e == Engine::TC) return contract_tc(d, op.hi, op.lo, in, out, st, dot);
  if (e == Engine::TB)
    return contract_tc_b16(d, (const uint16_t*)op.hi, (const uint16_t*)op.lo, in, out, st, dot);
  if (dot && dot->nb) *dot->nb = 0;  // CUDA-core engines do not fuse the dot
  return contract_f32(d, op.hi, in, out, st);
}

// Internal epilogues of the FP64 CUDA-core contraction (not part of the C
// ABI's jfg_contract_desc.epilogue values): the coefficient of a
// variable-coefficient form from the last pass of its backward transform.
constexpr int EPI_EXP_WEIGHT = 8;  // kw = exp(c1[b] (v - c0[b])) lam_m[m] lam_p[p]
constexpr int EPI_MOMENTS = 9;     // v, plus (count, mean, M2) per tile
int contract_f64_coef(const jfg_contract_desc& d, int kind, const double* op, const double* in,
                      double* out, double* aux, float* aux32, double* part, long long* tiles,
                      cudaStream_t st);

// Optional device-side active subset of a batch (jfg_contract_desc.batch_list).
struct Active {
  const int* list = nullptr;
  const int* count = nullptr;
};

// Problem index of slot j of a (possibly listed) batch, or -1 when the slot is
// past the active count or the entry is out of range.  n_active is *count
// (or batch without a list), read once by the caller.
__device__ __forceinline__ int active_problem(const int* list, int n_active, int batch, int j) {
  if (j >= n_active) return -1;
  const int b = list ? list[j] : j;
  return (b >= 0 && b < batch) ? b : -1;
}
__device__ __forceinline__ int active_count(const int* list, const int* count, int batch) {
  if (!list) return batch;
  const int c = *count;
  return c < 0 ? 0 : (c > batch ? batch : c);
}

// A zero-initialised descriptor for a single-segment pass with no epilogue.
inline jfg_contract_desc make_desc(int batch, int M, int P, int K, Active act = Active()) {
  jfg_contract_desc d = {};
  d.batch_list = act.list;
  d.batch_count = act.count;
  d.batch = batch;
  d.nseg = 1;
  d.M = M;
  d.P = P;
  d.K = K;
  d.op_ld = K;
  d.in_ld = K;
  d.in_batch = (long long)P * K;
  d.out_ld = P;
  d.out_batch = (long long)M * P;
  d.epilogue = JFG_EPI_NONE;
  d.alpha = 1.0;
  d.beta = 0.0;
  return d;
}

int validate_desc(const jfg_contract_desc& d);

// Higher-level sequences (ops.cu), shared by the FP64, FP32 and tensor-core paths.
template <typename T>
int tp_apply(Engine e, int ndim, const int* rows, const int* cols, int batch,
             const OpRef<T>* mats, const T* in, T* out, void* work, size_t work_bytes,
             cudaStream_t st, const T* shift = nullptr);
template <typename T>
int fd_solve(Engine e, int ndim, int n, int batch, OpRef<T> E, OpRef<T> W, const T* lam,
             const T* c0, const T* c1, const T* rhs, T* out, void* work, size_t work_bytes,
             cudaStream_t st, Active act = Active(), const DotOut* dot = nullptr);
template <typename T>
int varcoef_apply(Engine e, int ndim, int n, int nq, int batch, OpRef<T> ops, const T* kw,
                  const T* u, T* v, void* work, size_t work_bytes, cudaStream_t st,
                  Active act = Active(), const H16Ops* h16 = nullptr,
                  const DotOut* dot = nullptr);
// number of inverse row scales of the 2-D packed operators (TH engine)
inline long long varcoef_h16_rows(int n, int nq) { return 4LL * nq + 3LL * n; }
inline long long varcoef_h16_rows_nd(int ndim, int n, int nq) {
  return ndim == 3 ? 5LL * nq + 3LL * n : varcoef_h16_rows(n, nq);
}

// Read and clear the device status word of the BF16 GEMM kernel.
int gemm_status_take(int* status);

size_t tp_apply_ws(int ndim, const int* rows, const int* cols, int batch, int eb);
size_t fd_ws(int ndim, int n, int batch, int eb);
size_t varcoef_ws(int ndim, int n, int nq, int batch, int eb);

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace jfg
