// Pass sequences of the tensor-product operations on top of the per-axis
// contraction: separable transforms, fast-diagonalisation solve and the
// sum-factorised variable-coefficient operator.  The same sequences run on
// the FP64 / FP32 CUDA-core engines and on the split-TF32 tensor-core engine.
//
// Every pass contracts the LAST axis of its input and writes the result axis
// FIRST ("rotate"), so a d-dimensional field returns to its original axis
// order after d passes and every pass is the same strided GEMM shape with the
// contracted index contiguous in memory.
#include <math.h>
#include <string.h>

#include <type_traits>

#include "jfg_internal.cuh"

namespace jfg {

// ---------------------------------------------------------------------------
// separable transforms: out = (x_ax mats[ax]) in
// ---------------------------------------------------------------------------

// bytes of one intermediate buffer (the largest field between two passes)
static size_t tp_inter_bytes(int ndim, const int* rows, const int* cols, int batch, int eb) {
  int shape[3];
  int order[3];
  for (int i = 0; i < ndim; ++i) shape[i] = cols[i], order[i] = i;
  size_t mx = 0;
  for (int t = 0; t < ndim - 1; ++t) {
    const int ax = order[ndim - 1];
    for (int i = ndim - 1; i > 0; --i) shape[i] = shape[i - 1], order[i] = order[i - 1];
    shape[0] = rows[ax];
    order[0] = ax;
    size_t sz = (size_t)batch;
    for (int i = 0; i < ndim; ++i) sz *= (size_t)shape[i];
    if (sz > mx) mx = sz;
  }
  return align_up(mx * eb, 256);
}

// two intermediate buffers, then room for the operators split into FP32
// (hi, lo) pairs (used by the double-FP32 engine)
size_t tp_apply_ws(int ndim, const int* rows, const int* cols, int batch, int eb) {
  if (ndim < 1 || ndim > 3) return 0;
  size_t ops = 0;
  for (int i = 0; i < ndim; ++i) ops += (size_t)rows[i] * cols[i];
  return 2 * tp_inter_bytes(ndim, rows, cols, batch, eb) + align_up(ops * sizeof(float2), 256);
}

// out[i] = shift[i % per] for i < total: the constant field of an affine
// transform, written before the last pass accumulates into it (beta = 1)
template <typename T>
__global__ void k_bcast_fill(const T* __restrict__ shift, long long per, long long total,
                             T* __restrict__ out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride)
    out[i] = shift[i % per];
}

// shift (optional): out[b] = (x_ax mats[ax]) in[b] + shift, the same shift
// (shape rows[0] x ... x rows[ndim-1]) for every b; out must not overlap in
template <typename T>
int tp_apply(Engine e, int ndim, const int* rows, const int* cols, int batch,
             const OpRef<T>* mats, const T* in, T* out, void* work, size_t work_bytes,
             cudaStream_t st, const T* shift) {
  if (ndim < 1 || ndim > 3 || !rows || !cols || !mats || !in || !out || batch < 0)
    return JFG_ERR_ARG;
  for (int i = 0; i < ndim; ++i)
    if (rows[i] < 1 || cols[i] < 1 || !mats[i].hi) return JFG_ERR_ARG;
  const size_t need = tp_apply_ws(ndim, rows, cols, batch, (int)sizeof(T));
  if (ndim > 1 && (!work || work_bytes < need)) return JFG_ERR_WORKSPACE;
  const size_t inter = tp_inter_bytes(ndim, rows, cols, batch, (int)sizeof(T));
  T* buf[2] = {(T*)work, (T*)((char*)work + inter)};
  // Double-FP32: split every operator once into (hi, lo) pairs and keep the
  // intermediates split between the passes (no FP64 work in the tile loads)
  const bool dfp = std::is_same<T, double>::value && e == Engine::DF && work &&
                   work_bytes >= need && batch > 0;
  OpRef<T> opr[3];
  for (int i = 0; i < ndim; ++i) opr[i] = mats[i];
  if (dfp) {
    float2* pairs = (float2*)((char*)work + 2 * inter);
    for (int i = 0; i < ndim; ++i) {
      const long long cnt = (long long)rows[i] * cols[i];
      JFG_TRY(split_pairs_f64((const double*)mats[i].hi, pairs, cnt, st));
      opr[i] = OpRef<T>{mats[i].hi, (const T*)pairs};
      pairs += cnt;
    }
  }

  int shape[3], order[3];
  for (int i = 0; i < ndim; ++i) shape[i] = cols[i], order[i] = i;
  const T* src = in;
  for (int t = 0; t < ndim; ++t) {
    const int ax = order[ndim - 1];
    const int K = shape[ndim - 1];
    long long P = 1;
    for (int i = 0; i < ndim - 1; ++i) P *= shape[i];
    const int M = rows[ax];
    T* dst = (t == ndim - 1) ? out : buf[t & 1];
    jfg_contract_desc d = make_desc(batch, M, (int)P, K);
    if (shift && t == ndim - 1) {
      long long per = 1;
      for (int i = 0; i < ndim; ++i) per *= rows[i];
      const long long total = per * batch;
      long long blocks = (total + 255) / 256;
      if (blocks > 4 * 152) blocks = 4 * 152;
      if (total > 0) {
        k_bcast_fill<T><<<(int)blocks, 256, 0, st>>>(shift, per, total, out);
        JFG_CHECK_LAUNCH();
        count_launches(1);
      }
      d.beta = 1.0;
    }
    if (dfp)
      JFG_TRY(contract_df64(d, (const double*)opr[ax].hi, (const float2*)opr[ax].lo,
                            (const double*)src, (double*)dst, st, t > 0, t < ndim - 1));
    else
      JFG_TRY(contract(e, d, mats[ax], src, dst, st));
    for (int i = ndim - 1; i > 0; --i) shape[i] = shape[i - 1], order[i] = order[i - 1];
    shape[0] = M;
    order[0] = ax;
    src = dst;
  }
  return JFG_OK;
}

// ---------------------------------------------------------------------------
// fast diagonalisation: U = (x W) [(x E) F / (c0 + c1 * sum lam)]
// ---------------------------------------------------------------------------

template <typename T>
__global__ void k_lam_sum2(const T* __restrict__ lam, int n, T* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n * n) out[i] = lam[i / n] + lam[i % n];
}

size_t fd_ws(int ndim, int n, int batch, int eb) {
  size_t field = (size_t)batch;
  for (int i = 0; i < ndim; ++i) field *= (size_t)n;
  return 2 * align_up(field * eb, 256) + align_up((size_t)n * n * eb, 256);
}

template <typename T>
int fd_solve(Engine e, int ndim, int n, int batch, OpRef<T> E, OpRef<T> W, const T* lam,
             const T* c0, const T* c1, const T* rhs, T* out, void* work, size_t work_bytes,
             cudaStream_t st, Active act, const DotOut* dot) {
  if (dot && dot->nb) *dot->nb = 0;
  if ((ndim != 2 && ndim != 3) || n < 1 || batch < 0 || !E.hi || !W.hi || !lam || !rhs ||
      !out)
    return JFG_ERR_ARG;
  const size_t need = fd_ws(ndim, n, batch, (int)sizeof(T));
  if (!work || work_bytes < need) return JFG_ERR_WORKSPACE;
  size_t field = (size_t)batch;
  for (int i = 0; i < ndim; ++i) field *= (size_t)n;
  const size_t fb = align_up(field * sizeof(T), 256);
  T* buf[2] = {(T*)work, (T*)((char*)work + fb)};
  T* lam_p = (T*)((char*)work + 2 * fb);
  if (batch == 0) return JFG_OK;
  if (ndim == 3) {
    k_lam_sum2<T><<<(n * n + 255) / 256, 256, 0, st>>>(lam, n, lam_p);
    JFG_CHECK_LAUNCH();
    count_launches(1);
  }
  long long P = (long long)n * (ndim == 3 ? n : 1);
  const T* src = rhs;
  int b = 0;
  for (int t = 0; t < 2 * ndim; ++t) {
    jfg_contract_desc d = make_desc(batch, n, (int)P, n, act);
    if (t == ndim - 1) {
      d.epilogue = JFG_EPI_DIV_EIG;
      d.lam_m = lam;
      d.lam_p = (ndim == 3) ? lam_p : lam;
      d.c0 = c0;
      d.c1 = c1;
    }
    T* dst = (t == 2 * ndim - 1) ? out : buf[b];
    if constexpr (std::is_same<T, float>::value) {
      // the divide pass can fuse r.M^-1 r (sum of acc * out)
      JFG_TRY(contract(e, d, t < ndim ? E : W, src, dst, st, t == ndim - 1 ? dot : nullptr));
    } else {
      JFG_TRY(contract(e, d, t < ndim ? E : W, src, dst, st));
    }
    src = dst;
    b ^= 1;
  }
  return JFG_OK;
}

// ---------------------------------------------------------------------------
// variable-coefficient operator (kappa grad u, grad v), sum-factorised
// ---------------------------------------------------------------------------
//
// Packed operators (units of n*nq elements), B[q][k] = phi_k(x_q), D = phi_k':
//   2-D: [B;D] (2nq x n) | D, B (nq x n) | B^T, D^T (n x nq) | [D^T | B^T] (n x 2nq)
//   3-D: [B;D] (2nq x n) | D, B, B (nq x n) | B^T, B^T, D^T (n x nq)

size_t varcoef_ws(int ndim, int n, int nq, int batch, int eb) {
  size_t a, b;
  if (ndim == 2) {
    a = (size_t)2 * n * nq;
    b = (size_t)2 * nq * nq;
  } else {
    a = (size_t)3 * nq * nq * nq;
    b = (size_t)3 * nq * nq * n;
  }
  return align_up(a * batch * eb, 256) + align_up(b * batch * eb, 256);
}

template <typename T>
int varcoef_apply(Engine e, int ndim, int n, int nq, int batch, OpRef<T> ops, const T* kw,
                  const T* u, T* v, void* work, size_t work_bytes, cudaStream_t st,
                  Active act, const H16Ops* h16, const DotOut* dot) {
  if (dot && dot->nb) *dot->nb = 0;
  if ((ndim != 2 && ndim != 3) || n < 1 || nq < 1 || batch < 0 || !ops.hi || !kw || !u || !v)
    return JFG_ERR_ARG;
  const size_t need = varcoef_ws(ndim, n, nq, batch, (int)sizeof(T));
  if (!work || work_bytes < need) return JFG_ERR_WORKSPACE;
  if (batch == 0) return JFG_OK;
  const long long nn = (long long)n * nq;
  const size_t a_elems = ndim == 2 ? (size_t)2 * n * nq : (size_t)3 * nq * nq * nq;
  T* bufA = (T*)work;
  T* bufB = (T*)((char*)work + align_up(a_elems * batch * sizeof(T), 256));

  // Double-FP32 with a pre-split operator: u is split once into (hi, lo)
  // pairs (in bufB, free until the second pass) and the intermediates stay
  // split between the passes, so no tile load does FP64 work.
  const bool dfp = std::is_same<T, double>::value && e == Engine::DF && ops.lo != nullptr;
  auto pass = [&](const jfg_contract_desc& d, OpRef<T> op, const T* in, T* out, bool pin,
                  bool pout) -> int {
    if (dfp)
      return contract_df64(d, (const double*)op.hi, (const float2*)op.lo, (const double*)in,
                           (double*)out, st, pin, pout);
    return contract(e, d, op, in, out, st);
  };
  const T* u1 = u;
  if (dfp) {
    long long nu = batch;
    for (int i = 0; i < ndim; ++i) nu *= n;
    JFG_TRY(split_pairs_f64((const double*)u, (float2*)bufB, nu, st));
    u1 = bufB;
  }
  if (e == Engine::TH && (!h16 || !h16->op_inv || !h16->slots)) return JFG_ERR_ARG;
  if (ndim == 2) {
    // 1: T[b][r][j] = sum_l [B;D][r][l] U[b][j][l]            (M=2nq, P=n, K=n)
    jfg_contract_desc d1 = make_desc(batch, 2 * nq, n, n, act);
    if constexpr (std::is_same<T, float>::value) {
      if (e == Engine::TH) {
        // Scaled split FP16: the operators are FP16 (hi, lo) arrays with the
        // packed layout (offsets in 16-bit elements); each pass reads its
        // input's max from slot t and records its output's max in slot t+1.
        const uint16_t* oh = (const uint16_t*)ops.hi;
        const uint16_t* ol = (const uint16_t*)ops.lo;
        unsigned* sl = h16->slots;
        const float* inv = h16->op_inv;
        const long long B = batch;
        JFG_TRY(contract_tc_h16(d1, oh, ol, inv, 0, sl, sl + B, u, bufA, st));
        jfg_contract_desc d2 = make_desc(batch, nq, nq, n, act);
        d2.nseg = 2;
        d2.op_seg = nn;
        d2.in_seg = nn;
        d2.in_batch = 2 * nn;
        d2.out_seg = (long long)nq * nq;
        d2.out_batch = 2LL * nq * nq;
        d2.epilogue = JFG_EPI_MUL_FIELD;
        d2.field = kw;
        d2.field_ld = nq;
        d2.field_seg = 0;
        d2.field_batch = (long long)nq * nq;
        // the field pass can fuse p.Ap = sum over both gradient components of
        // kappa w (grad p)^2 (sum of acc * out)
        JFG_TRY(contract_tc_h16(d2, oh + 2 * nn, ol + 2 * nn, inv + 2LL * nq, nq, sl + B,
                                sl + 2 * B, bufA, bufB, st, dot));
        jfg_contract_desc d3 = make_desc(batch, n, nq, nq, act);
        d3.nseg = 2;
        d3.op_seg = nn;
        d3.in_seg = (long long)nq * nq;
        d3.in_batch = 2LL * nq * nq;
        d3.out_ld = 2LL * nq;
        d3.out_seg = nq;
        d3.out_batch = 2 * nn;
        JFG_TRY(contract_tc_h16(d3, oh + 4 * nn, ol + 4 * nn, inv + 4LL * nq, n, sl + 2 * B,
                                sl + 3 * B, bufB, bufA, st));
        jfg_contract_desc d4 = make_desc(batch, n, n, 2 * nq, act);
        JFG_TRY(contract_tc_h16(d4, oh + 6 * nn, ol + 6 * nn, inv + 4LL * nq + 2LL * n, 0,
                                sl + 3 * B, nullptr, bufA, v, st));
        return JFG_OK;
      }
    }
    JFG_TRY(pass(d1, ops, u1, bufA, dfp, dfp));
    // 2: G[b][s][p][q] = kw[b][p][q] * sum_j {D,B}[p][j] T[b][s][q][j]
    jfg_contract_desc d2 = make_desc(batch, nq, nq, n, act);
    d2.nseg = 2;
    d2.op_seg = nn;
    d2.in_seg = nn;
    d2.in_batch = 2 * nn;
    d2.out_seg = (long long)nq * nq;
    d2.out_batch = 2LL * nq * nq;
    d2.epilogue = JFG_EPI_MUL_FIELD;
    d2.field = kw;
    d2.field_ld = nq;
    d2.field_seg = 0;
    d2.field_batch = (long long)nq * nq;
    JFG_TRY(pass(d2, ops.offset(2 * nn), bufA, bufB, dfp, dfp));
    // 3: H[b][k][s][p] = sum_q {B^T,D^T}[k][q] G[b][s][p][q]   (M=n, P=nq, K=nq)
    jfg_contract_desc d3 = make_desc(batch, n, nq, nq, act);
    d3.nseg = 2;
    d3.op_seg = nn;
    d3.in_seg = (long long)nq * nq;
    d3.in_batch = 2LL * nq * nq;
    d3.out_ld = 2LL * nq;
    d3.out_seg = nq;
    d3.out_batch = 2 * nn;
    JFG_TRY(pass(d3, ops.offset(4 * nn), bufB, bufA, dfp, dfp));
    // 4: V[b][i][k] = sum_{s,p} [D^T|B^T][i][(s,p)] H[b][k][(s,p)]   (M=n, P=n, K=2nq)
    jfg_contract_desc d4 = make_desc(batch, n, n, 2 * nq, act);
    JFG_TRY(pass(d4, ops.offset(6 * nn), bufA, v, dfp, false));
    return JFG_OK;
  }

  // ---- 3-D ----
  const long long n2 = (long long)n * n, q2 = (long long)nq * nq;
  const OpRef<T> BD = ops;                   // [B;D]  (2nq x n)
  const OpRef<T> Q3 = ops.offset(2 * nn);    // D, B, B
  const OpRef<T> Q4 = ops.offset(5 * nn);    // B^T, B^T, D^T
  if constexpr (std::is_same<T, float>::value) {
    if (e == Engine::TH) {
      // Scaled split FP16: the passes below on the FP16 (hi, lo) operators.
      // Pass t reads its input's max from slot t and records its output's
      // max in slot t+1; a split output (bufB of passes 2a/2b, H2a and H2b
      // of pass 5) shares one slot, a bound over all of it.  Inverse row
      // scales: [B;D] 2nq | D,B,B 3nq | B^T,B^T,D^T 3n.
      const uint16_t* oh = (const uint16_t*)ops.hi;
      const uint16_t* ol = (const uint16_t*)ops.lo;
      const float* inv = h16->op_inv;
      unsigned* sl = h16->slots;
      const long long Bs = batch;
      auto hp = [&](const jfg_contract_desc& d, long long op_off, long long inv_off,
                    long long inv_seg, const float* in, float* out, int sin, int sout) -> int {
        return contract_tc_h16(d, oh + op_off, ol + op_off, inv + inv_off, inv_seg, sl + sin * Bs,
                               sout >= 0 ? sl + sout * Bs : nullptr, in, out, st);
      };
      const long long iq3 = 2LL * nq, iq4 = 5LL * nq;  // inverse-scale blocks
      jfg_contract_desc h1 = make_desc(batch, 2 * nq, (int)n2, n, act);
      JFG_TRY(hp(h1, 0, 0, 0, u, bufA, 0, 1));
      jfg_contract_desc h2 = make_desc(batch, 2 * nq, (int)nn, n, act);
      h2.in_batch = 2 * nq * n2;
      h2.out_batch = 3 * q2 * n;
      JFG_TRY(hp(h2, 0, 0, 0, bufA, bufB, 1, 2));
      jfg_contract_desc h2b = h2;
      h2b.M = nq;
      JFG_TRY(hp(h2b, 0, 0, 0, bufA + nq * n2, bufB + 2 * q2 * n, 1, 2));
      jfg_contract_desc h3 = make_desc(batch, nq, (int)q2, n, act);
      h3.nseg = 3;
      h3.op_seg = nn;
      h3.in_seg = q2 * n;
      h3.in_batch = 3 * q2 * n;
      h3.out_seg = q2 * nq;
      h3.out_batch = 3 * q2 * nq;
      h3.epilogue = JFG_EPI_MUL_FIELD;
      h3.field = kw;
      h3.field_ld = q2;
      h3.field_seg = 0;
      h3.field_batch = q2 * nq;
      JFG_TRY(hp(h3, 2 * nn, iq3, nq, bufB, bufA, 2, 3));
      jfg_contract_desc h4 = make_desc(batch, n, (int)q2, nq, act);
      h4.nseg = 3;
      h4.op_seg = nn;
      h4.in_seg = q2 * nq;
      h4.in_batch = 3 * q2 * nq;
      h4.out_seg = q2 * n;
      h4.out_batch = 3 * q2 * n;
      JFG_TRY(hp(h4, 5 * nn, iq4, n, bufA, bufB, 3, 4));
      float* G2a = bufA;
      float* G2b = bufA + (size_t)batch * n2 * nq;
      jfg_contract_desc h5 = make_desc(batch, n, (int)nn, nq, act);
      h5.in_batch = 3 * q2 * n;
      JFG_TRY(hp(h5, 5 * nn, iq4, 0, bufB, G2a, 4, 5));
      JFG_TRY(hp(h5, 7 * nn, iq4 + 2LL * n, 0, bufB + q2 * n, G2b, 4, 5));
      h5.beta = 1.0;
      JFG_TRY(hp(h5, 5 * nn, iq4, 0, bufB + 2 * q2 * n, G2b, 4, 5));
      jfg_contract_desc h6 = make_desc(batch, n, (int)n2, nq, act);
      JFG_TRY(hp(h6, 7 * nn, iq4 + 2LL * n, 0, G2a, v, 5, -1));
      h6.beta = 1.0;
      JFG_TRY(hp(h6, 5 * nn, iq4, 0, G2b, v, 5, -1));
      return JFG_OK;
    }
  }
  // 1: T1[b][(s2,q2)][(i0,i1)] = sum_i2 [B;D] U                 (M=2nq, P=n^2, K=n)
  jfg_contract_desc d1 = make_desc(batch, 2 * nq, (int)n2, n, act);
  JFG_TRY(pass(d1, BD, u1, bufA, dfp, dfp));
  // 2a: s2=0 rows with [B;D]: T2[b][(c,q1)][(q2,i0)], c in {0,1}  (M=2nq, P=nq*n, K=n)
  jfg_contract_desc d2 = make_desc(batch, 2 * nq, (int)nn, n, act);
  d2.in_batch = 2 * nq * n2;
  d2.out_batch = 3 * q2 * n;
  JFG_TRY(pass(d2, BD, bufA, bufB, dfp, dfp));
  // 2b: s2=1 rows with B -> c = 2
  jfg_contract_desc d2b = d2;
  d2b.M = nq;
  JFG_TRY(pass(d2b, BD, bufA + nq * n2, bufB + 2 * q2 * n, dfp, dfp));
  // 3: G[b][c][p0][(q1,q2)] = kw * sum_i0 {D,B,B}[p0][i0] T2[b][c][(q1,q2)][i0]
  jfg_contract_desc d3 = make_desc(batch, nq, (int)q2, n, act);
  d3.nseg = 3;
  d3.op_seg = nn;
  d3.in_seg = q2 * n;
  d3.in_batch = 3 * q2 * n;
  d3.out_seg = q2 * nq;
  d3.out_batch = 3 * q2 * nq;
  d3.epilogue = JFG_EPI_MUL_FIELD;
  d3.field = kw;
  d3.field_ld = q2;
  d3.field_seg = 0;
  d3.field_batch = q2 * nq;
  JFG_TRY(pass(d3, Q3, bufB, bufA, dfp, dfp));
  // 4: H1[b][c][k2][(p0,q1)] = sum_q2 {B^T,B^T,D^T}[k2][q2] G     (M=n, P=nq^2, K=nq)
  jfg_contract_desc d4 = make_desc(batch, n, (int)q2, nq, act);
  d4.nseg = 3;
  d4.op_seg = nn;
  d4.in_seg = q2 * nq;
  d4.in_batch = 3 * q2 * nq;
  d4.out_seg = q2 * n;
  d4.out_batch = 3 * q2 * n;
  JFG_TRY(pass(d4, Q4, bufA, bufB, dfp, dfp));
  // 5: H2a = B^T (c=0), H2b = D^T (c=1) + B^T (c=2)      (M=n, P=n*nq, K=nq)
  T* H2a = bufA;
  T* H2b = bufA + (size_t)batch * n2 * nq;
  jfg_contract_desc d5 = make_desc(batch, n, (int)nn, nq, act);
  d5.in_batch = 3 * q2 * n;
  JFG_TRY(pass(d5, Q4, bufB, H2a, dfp, dfp));
  JFG_TRY(pass(d5, Q4.offset(2 * nn), bufB + q2 * n, H2b, dfp, dfp));
  d5.beta = 1.0;
  JFG_TRY(pass(d5, Q4, bufB + 2 * q2 * n, H2b, dfp, dfp));
  // 6: V = D^T (x) on H2a + B^T (x) on H2b                 (M=n, P=n^2, K=nq)
  jfg_contract_desc d6 = make_desc(batch, n, (int)n2, nq, act);
  JFG_TRY(pass(d6, Q4.offset(2 * nn), H2a, v, dfp, false));
  d6.beta = 1.0;
  JFG_TRY(pass(d6, Q4, H2b, v, dfp, false));
  return JFG_OK;
}

template <typename T>
__global__ void k_weighted_field(int ndim, int nq, long long total, const T* __restrict__ kappa,
                                 const T* __restrict__ w, T* __restrict__ kw,
                                 float* __restrict__ kw32) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    T s = T(1);
    for (int a = 0; a < ndim; ++a) {
      s *= w[r % nq];
      r /= nq;
    }
    const T v = kappa[i] * s;
    kw[i] = v;
    if (kw32) kw32[i] = (float)v;
  }
}

// Per problem b (one block each): mean of g[b] and 1 / (population standard
// deviation), two passes over the grid values in FP64 (block tree reductions).
__global__ void k_field_moments(long long per, const double* __restrict__ g,
                                double* __restrict__ mean, double* __restrict__ inv_std) {
  __shared__ double red[256];
  const int b = blockIdx.x;
  const double* gb = g + (long long)b * per;
  auto block_sum = [&](double v) -> double {
    red[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
  };
  double s = 0.0;
  for (long long i = threadIdx.x; i < per; i += blockDim.x) s += gb[i];
  const double m = block_sum(s) / (double)per;
  double q = 0.0;
  for (long long i = threadIdx.x; i < per; i += blockDim.x) {
    const double d = gb[i] - m;
    q = fma(d, d, q);
  }
  const double var = block_sum(q) / (double)per;
  if (threadIdx.x == 0) {
    mean[b] = m;
    inv_std[b] = var > 0.0 ? 1.0 / sqrt(var) : 1.0;
  }
}

// kappa = exp(scale[b] (g - shift[b])) and kw = kappa * prod_ax w[i_ax] (FP64,
// plus an FP32 copy) in one pass over the grid.  g may be kw or kappa (in
// place: each element is read by the thread that then overwrites it), so
// those three are not restrict-qualified.
__global__ void k_exp_weighted_field(int ndim, int nq, long long per, long long total,
                                     const double* g, const double* __restrict__ scale,
                                     const double* __restrict__ shift,
                                     const double* __restrict__ w, double* kappa, double* kw,
                                     float* __restrict__ kw32) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / per;
    long long r = i;
    double wt = 1.0;
    for (int a = 0; a < ndim; ++a) {
      wt *= w[r % nq];
      r /= nq;
    }
    const double sc = scale ? scale[b] : 1.0;
    const double sh = shift ? shift[b] : 0.0;
    const double k = exp(sc * (g[i] - sh));
    if (kappa) kappa[i] = k;
    const double v = k * wt;
    kw[i] = v;
    if (kw32) kw32[i] = (float)v;
  }
}

// per-column weights of the last backward pass: wp[i] = prod of w over the
// base-nq digits of i (ndim - 1 of them)
__global__ void k_digit_weights(int digits, int nq, long long total, const double* __restrict__ w,
                                double* __restrict__ wp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    long long r = i;
    double v = 1.0;
    for (int a = 0; a < digits; ++a) {
      v *= w[r % nq];
      r /= nq;
    }
    wp[i] = v;
  }
}

// per problem: shift = mean, scale = 1 / population std from the tiles'
// (count, mean, M2) of the backward's last pass (Chan's pairwise update)
__global__ void k_moments_combine(const double* __restrict__ part, long long tiles, int batch,
                                  double* __restrict__ shift, double* __restrict__ scale) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  const double* pt = part + (long long)b * tiles * 3;
  double n = 0.0, mu = 0.0, m2 = 0.0;
  for (long long t = 0; t < tiles; ++t) {
    const double nb = pt[3 * t], mb = pt[3 * t + 1], qb = pt[3 * t + 2];
    if (nb <= 0.0) continue;
    const double nn = n + nb, dl = mb - mu;
    mu += dl * (nb / nn);
    m2 += qb + dl * dl * (n * nb / nn);
    n = nn;
  }
  const double var = n > 0.0 ? m2 / n : 0.0;
  shift[b] = mu;
  scale[b] = var > 0.0 ? 1.0 / sqrt(var) : 1.0;
}

template int tp_apply<double>(Engine, int, const int*, const int*, int, const OpRef<double>*,
                              const double*, double*, void*, size_t, cudaStream_t,
                              const double*);
template int tp_apply<float>(Engine, int, const int*, const int*, int, const OpRef<float>*,
                             const float*, float*, void*, size_t, cudaStream_t, const float*);
template int fd_solve<double>(Engine, int, int, int, OpRef<double>, OpRef<double>,
                              const double*, const double*, const double*, const double*,
                              double*, void*, size_t, cudaStream_t, Active, const DotOut*);
template int fd_solve<float>(Engine, int, int, int, OpRef<float>, OpRef<float>, const float*,
                             const float*, const float*, const float*, float*, void*, size_t,
                             cudaStream_t, Active, const DotOut*);
template int varcoef_apply<double>(Engine, int, int, int, int, OpRef<double>, const double*,
                                   const double*, double*, void*, size_t, cudaStream_t, Active,
                                   const H16Ops*, const DotOut*);
template int varcoef_apply<float>(Engine, int, int, int, int, OpRef<float>, const float*,
                                  const float*, float*, void*, size_t, cudaStream_t, Active,
                                  const H16Ops*, const DotOut*);

}  // namespace jfg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

using jfg::Engine;
using jfg::OpRef;

extern "C" int jfg_weighted_field_f64(int ndim, int nq, int batch, const double* kappa,
                                      const double* w, double* kw, float* kw32, void* stream) {
  if (ndim < 1 || ndim > 3 || nq < 1 || batch < 0 || !kappa || !w || !kw) return JFG_ERR_ARG;
  long long total = batch;
  for (int i = 0; i < ndim; ++i) total *= nq;
  if (total == 0) return JFG_OK;
  long long blocks = (total + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  jfg::k_weighted_field<double><<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(
      ndim, nq, total, kappa, w, kw, kw32);
  JFG_CHECK_LAUNCH();
  jfg::count_launches(1);
  return JFG_OK;
}

extern "C" int jfg_field_moments_f64(int ndim, int nq, int batch, const double* g,
                                     double* mean, double* inv_std, void* stream) {
  if (ndim < 1 || ndim > 3 || nq < 1 || batch < 0 || !g || !mean || !inv_std)
    return JFG_ERR_ARG;
  if (batch == 0) return JFG_OK;
  long long per = 1;
  for (int i = 0; i < ndim; ++i) per *= nq;
  jfg::k_field_moments<<<batch, 256, 0, (cudaStream_t)stream>>>(per, g, mean, inv_std);
  JFG_CHECK_LAUNCH();
  jfg::count_launches(1);
  return JFG_OK;
}

extern "C" int jfg_exp_weighted_field_f64(int ndim, int nq, int batch, const double* g,
                                          const double* scale, const double* shift,
                                          const double* w, double* kappa, double* kw,
                                          float* kw32, void* stream) {
  if (ndim < 1 || ndim > 3 || nq < 1 || batch < 0 || !g || !w || !kw) return JFG_ERR_ARG;
  long long per = 1;
  for (int i = 0; i < ndim; ++i) per *= nq;
  const long long total = per * batch;
  if (total == 0) return JFG_OK;
  long long blocks = (total + 255) / 256;
  if (blocks > 8 * 152) blocks = 8 * 152;
  jfg::k_exp_weighted_field<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(
      ndim, nq, per, total, g, scale, shift, w, kappa, kw, kw32);
  JFG_CHECK_LAUNCH();
  jfg::count_launches(1);
  return JFG_OK;
}

// ---- coefficient from its expansion: backward transform + exp + weights ----

namespace {
struct ExpBackwardLayout {
  size_t inter, wp, part, mom, total;
};
ExpBackwardLayout exp_backward_layout(int ndim, int n, int nq, int batch) {
  ExpBackwardLayout L;
  const int rows[3] = {nq, nq, nq}, cols[3] = {n, n, n};
  L.inter = ndim > 1 ? jfg::align_up(jfg::tp_apply_ws(ndim, rows, cols, batch, 8), 256) : 0;
  long long P = 1;
  for (int i = 1; i < ndim; ++i) P *= nq;
  L.wp = jfg::align_up((size_t)P * 8, 256);
  const long long tiles = ((P + 63) / 64) * ((nq + 63) / 64);
  L.part = jfg::align_up((size_t)batch * tiles * 3 * 8, 256);
  L.mom = jfg::align_up((size_t)batch * 2 * 8, 256);
  L.total = L.inter + L.wp + L.part + L.mom;
  return L;
}
}  // namespace

extern "C" size_t jfg_exp_weighted_backward_workspace_size(int ndim, int n, int nq, int batch) {
  if (ndim < 1 || ndim > 3 || n < 1 || nq < 1 || batch < 0) return 0;
  return exp_backward_layout(ndim, n, nq, batch).total;
}

extern "C" int jfg_exp_weighted_backward_f64(int ndim, int n, int nq, int batch, const double* V,
                                             const double* g_coef, int standardize,
                                             const double* w, double* kappa, double* kw,
                                             float* kw32, void* work, size_t work_bytes,
                                             void* stream) {
  using namespace jfg;
  if (ndim < 1 || ndim > 3 || n < 1 || nq < 1 || batch < 0 || !V || !g_coef || !w || !kw ||
      (standardize != 0 && standardize != 1))
    return JFG_ERR_ARG;
  const ExpBackwardLayout L = exp_backward_layout(ndim, n, nq, batch);
  if (!work || work_bytes < L.total) return JFG_ERR_WORKSPACE;
  if (batch == 0) return JFG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  char* wk = (char*)work;
  double* wp = (double*)(wk + L.inter);
  double* part = (double*)(wk + L.inter + L.wp);
  double* shift = (double*)(wk + L.inter + L.wp + L.part);
  double* scale = shift + batch;
  long long P = 1;
  for (int i = 1; i < ndim; ++i) P *= nq;
  {
    long long blocks = (P + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    k_digit_weights<<<(int)blocks, 256, 0, st>>>(ndim - 1, nq, P, w, wp);
    JFG_LAUNCHED();
  }
  // passes 1 .. ndim-1: the plain backward contraction (tp_apply's order:
  // contract the last axis, rotate it to the front)
  const int rows[3] = {nq, nq, nq}, cols[3] = {n, n, n};
  const size_t inter = ndim > 1 ? tp_inter_bytes(ndim, rows, cols, batch, 8) : 0;
  double* buf[2] = {(double*)wk, (double*)(wk + inter)};
  const double* src = g_coef;
  long long Pt = 1;
  for (int i = 0; i < ndim - 1; ++i) Pt *= n;  // leading axes still in coefficients
  for (int t = 0; t < ndim - 1; ++t) {
    jfg_contract_desc d = make_desc(batch, nq, (int)Pt, n);
    double* dst = buf[t & 1];
    JFG_TRY(contract_f64(d, V, src, dst, st));
    Pt = Pt / n * nq;
    src = dst;
  }
  // last pass: M = nq (axis 0 comes to the front), P = nq^(ndim-1)
  jfg_contract_desc d = make_desc(batch, nq, (int)P, n);
  if (!standardize) {
    d.lam_m = w;
    d.lam_p = wp;
    d.field_ld = P;
    d.field_batch = (long long)nq * P;
    return contract_f64_coef(d, EPI_EXP_WEIGHT, V, src, kw, kappa, kw32, nullptr, nullptr, st);
  }
  // standardised: g into kw with per-tile moments, then exp and weights in
  // place (each element is read before it is overwritten, by its own thread)
  long long tiles = 0;
  JFG_TRY(contract_f64_coef(d, EPI_MOMENTS, V, src, kw, nullptr, nullptr, part, &tiles, st));
  k_moments_combine<<<(batch + 127) / 128, 128, 0, st>>>(part, tiles, batch, shift, scale);
  JFG_LAUNCHED();
  const long long total = (long long)nq * P * batch;
  long long blocks = (total + 255) / 256;
  if (blocks > 8 * 152) blocks = 8 * 152;
  k_exp_weighted_field<<<(int)blocks, 256, 0, st>>>(ndim, nq, (long long)nq * P, total, kw,
                                                     scale, shift, w, kappa, kw, kw32);
  JFG_LAUNCHED();
  return JFG_OK;
}

extern "C" size_t jfg_tp_apply_workspace_size(int ndim, const int* rows, const int* cols,
                                              int batch, int elem_bytes) {
  if (!rows || !cols) return 0;
  return jfg::tp_apply_ws(ndim, rows, cols, batch, elem_bytes);
}

extern "C" int jfg_tp_apply_f64(int ndim, const int* rows, const int* cols, int batch,
                                const double* const* mats, const double* in, double* out,
                                void* work, size_t work_bytes, void* stream) {
  if (!mats || ndim < 1 || ndim > 3) return JFG_ERR_ARG;
  OpRef<double> m[3];
  for (int i = 0; i < ndim; ++i) m[i] = OpRef<double>{mats[i], nullptr};
  return jfg::tp_apply<double>(Engine::F64, ndim, rows, cols, batch, m, in, out, work,
                               work_bytes, (cudaStream_t)stream);
}

extern "C" int jfg_tp_apply_df64(int ndim, const int* rows, const int* cols, int batch,
                                 const double* const* mats, const double* in, double* out,
                                 void* work, size_t work_bytes, void* stream) {
  if (!mats || ndim < 1 || ndim > 3) return JFG_ERR_ARG;
  OpRef<double> m[3];
  for (int i = 0; i < ndim; ++i) m[i] = OpRef<double>{mats[i], nullptr};
  return jfg::tp_apply<double>(Engine::DF, ndim, rows, cols, batch, m, in, out, work,
                               work_bytes, (cudaStream_t)stream);
}

extern "C" int jfg_tp_apply_f32(int ndim, const int* rows, const int* cols, int batch,
                                const float* const* mats, const float* in, float* out,
                                void* work, size_t work_bytes, void* stream) {
  if (!mats || ndim < 1 || ndim > 3) return JFG_ERR_ARG;
  OpRef<float> m[3];
  for (int i = 0; i < ndim; ++i) m[i] = OpRef<float>{mats[i], nullptr};
  return jfg::tp_apply<float>(Engine::F32, ndim, rows, cols, batch, m, in, out, work,
                              work_bytes, (cudaStream_t)stream);
}

extern "C" int jfg_tp_apply_tc(int ndim, const int* rows, const int* cols, int batch,
                               const float* const* mats_hi, const float* const* mats_lo,
                               const float* in, float* out, void* work, size_t work_bytes,
                               void* stream) {
  if (!mats_hi || !mats_lo || ndim < 1 || ndim > 3) return JFG_ERR_ARG;
  OpRef<float> m[3];
  for (int i = 0; i < ndim; ++i) {
    if (!mats_lo[i]) return JFG_ERR_ARG;
    m[i] = OpRef<float>{mats_hi[i], mats_lo[i]};
  }
  return jfg::tp_apply<float>(Engine::TC, ndim, rows, cols, batch, m, in, out, work,
                              work_bytes, (cudaStream_t)stream);
}

extern "C" int jfg_tp_apply_tc_bf16x3(int ndim, const int* rows, const int* cols, int batch,
                                      const uint16_t* const* mats_hi,
                                      const uint16_t* const* mats_lo, const float* in,
                                      float* out, void* work, size_t work_bytes, void* stream) {
  if (!mats_hi || !mats_lo || ndim < 1 || ndim > 3) return JFG_ERR_ARG;
  OpRef<float> m[3];
  for (int i = 0; i < ndim; ++i) {
    if (!mats_hi[i] || !mats_lo[i]) return JFG_ERR_ARG;
    m[i] = OpRef<float>{(const float*)mats_hi[i], (const float*)mats_lo[i]};
  }
  return jfg::tp_apply<float>(Engine::TB, ndim, rows, cols, batch, m, in, out, work,
                              work_bytes, (cudaStream_t)stream);
}

extern "C" int jfg_tp_apply_affine_f64(int ndim, const int* rows, const int* cols, int batch,
                                       const double* const* mats, const double* in,
                                       const double* shift, double* out, void* work,
                                       size_t work_bytes, void* stream) {
  if (!mats || !shift || ndim < 1 || ndim > 3) return JFG_ERR_ARG;
  if (in == out) return JFG_ERR_ARG;
  OpRef<double> m[3];
  for (int i = 0; i < ndim; ++i) m[i] = OpRef<double>{mats[i], nullptr};
  return jfg::tp_apply<double>(Engine::F64, ndim, rows, cols, batch, m, in, out, work,
                               work_bytes, (cudaStream_t)stream, shift);
}

extern "C" size_t jfg_fd_solve_workspace_size(int ndim, int n, int batch, int elem_bytes) {
  return jfg::fd_ws(ndim, n, batch, elem_bytes);
}

extern "C" int jfg_fd_solve_f64(int ndim, int n, int batch, const double* E, const double* W,
                                const double* lam, const double* c0, const double* c1,
                                const double* rhs, double* out, void* work, size_t work_bytes,
                                void* stream) {
  return jfg::fd_solve<double>(Engine::F64, ndim, n, batch, OpRef<double>{E, nullptr},
                               OpRef<double>{W, nullptr}, lam, c0, c1, rhs, out, work,
                               work_bytes, (cudaStream_t)stream);
}

extern "C" int jfg_fd_solve_f32(int ndim, int n, int batch, const float* E, const float* W,
                                const float* lam, const float* c0, const float* c1,
                                const float* rhs, float* out, void* work, size_t work_bytes,
                                void* stream) {
  return jfg::fd_solve<float>(Engine::F32, ndim, n, batch, OpRef<float>{E, nullptr},
                              OpRef<float>{W, nullptr}, lam, c0, c1, rhs, out, work,
                              work_bytes, (cudaStream_t)stream);
}

extern "C" int jfg_fd_solve_tc(int ndim, int n, int batch, const float* E_hi, const float* E_lo,
                               const float* W_hi, const float* W_lo, const float* lam,
                               const float* c0, const float* c1, const float* rhs, float* out,
                               void* work, size_t work_bytes, void* stream) {
  if (!E_lo || !W_lo) return JFG_ERR_ARG;
  return jfg::fd_solve<float>(Engine::TC, ndim, n, batch, OpRef<float>{E_hi, E_lo},
                              OpRef<float>{W_hi, W_lo}, lam, c0, c1, rhs, out, work, work_bytes,
                              (cudaStream_t)stream);
}

extern "C" size_t jfg_varcoef_ops_count(int ndim, int n, int nq) {
  (void)ndim;
  return (size_t)8 * n * nq;
}

extern "C" void jfg_varcoef_pack_ops_host(int ndim, int n, int nq, const double* B,
                                          const double* D, double* o) {
  const size_t nn = (size_t)n * nq;
  // [B;D]
  for (int q = 0; q < nq; ++q)
    for (int k = 0; k < n; ++k) {
      o[(size_t)q * n + k] = B[(size_t)q * n + k];
      o[nn + (size_t)q * n + k] = D[(size_t)q * n + k];
    }
  if (ndim == 2) {
    for (int q = 0; q < nq; ++q)
      for (int k = 0; k < n; ++k) {
        o[2 * nn + (size_t)q * n + k] = D[(size_t)q * n + k];
        o[3 * nn + (size_t)q * n + k] = B[(size_t)q * n + k];
        o[4 * nn + (size_t)k * nq + q] = B[(size_t)q * n + k];
        o[5 * nn + (size_t)k * nq + q] = D[(size_t)q * n + k];
        o[6 * nn + (size_t)k * 2 * nq + q] = D[(size_t)q * n + k];
        o[6 * nn + (size_t)k * 2 * nq + nq + q] = B[(size_t)q * n + k];
      }
  } else {
    for (int q = 0; q < nq; ++q)
      for (int k = 0; k < n; ++k) {
        o[2 * nn + (size_t)q * n + k] = D[(size_t)q * n + k];
        o[3 * nn + (size_t)q * n + k] = B[(size_t)q * n + k];
        o[4 * nn + (size_t)q * n + k] = B[(size_t)q * n + k];
        o[5 * nn + (size_t)k * nq + q] = B[(size_t)q * n + k];
        o[6 * nn + (size_t)k * nq + q] = B[(size_t)q * n + k];
        o[7 * nn + (size_t)k * nq + q] = D[(size_t)q * n + k];
      }
  }
}

namespace {

// FP32 -> FP16 bit pattern, round to nearest even (normal, subnormal,
// overflow to infinity), in portable host code.
uint16_t f32_to_f16_rne(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const uint32_t ax = x & 0x7FFFFFFFu;
  if (ax >= 0x7F800000u) return (uint16_t)(sign | (ax > 0x7F800000u ? 0x7E00u : 0x7C00u));
  if (ax >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);  // >= 65520: infinity
  if (ax <= 0x33000000u) return (uint16_t)sign;              // <= 2^-25: zero (ties to even)
  const int e = (int)(ax >> 23) - 127;
  const uint32_t mant = (ax & 0x7FFFFFu) | 0x800000u;
  uint32_t h, rem, half;
  if (e >= -14) {  // normal: 10 of the 23 fraction bits kept
    h = ((uint32_t)(e + 15) << 10) | ((mant >> 13) & 0x3FFu);
    rem = mant & 0x1FFFu;
    half = 0x1000u;
  } else {         // subnormal: units of 2^-24
    const int sh = -e - 1;
    h = mant >> sh;
    rem = mant & ((1u << sh) - 1u);
    half = 1u << (sh - 1);
  }
  if (rem > half || (rem == half && (h & 1u))) h += 1u;  // a carry moves to the next binade
  return (uint16_t)(sign | h);
}

double f16_to_double(uint16_t h) {
  const int e = (h >> 10) & 0x1F;
  const int m = h & 0x3FF;
  double v = e == 0 ? ldexp((double)m, -24) : ldexp(1024.0 + m, e - 25);
  if (e == 31) v = m ? NAN : INFINITY;
  return (h & 0x8000u) ? -v : v;
}

}  // namespace

extern "C" size_t jfg_varcoef_f16_rows(int n, int nq) {
  return n < 1 || nq < 1 ? 0 : (size_t)jfg::varcoef_h16_rows(n, nq);
}

extern "C" size_t jfg_varcoef_f16_rows_nd(int ndim, int n, int nq) {
  return (ndim != 2 && ndim != 3) || n < 1 || nq < 1
             ? 0
             : (size_t)jfg::varcoef_h16_rows_nd(ndim, n, nq);
}

extern "C" void jfg_split_f16_rowscaled_host(size_t rows, size_t cols, const double* src,
                                              uint16_t* hi, uint16_t* lo, float* inv) {
  for (size_t r = 0; r < rows; ++r) {
    const double* row = src + r * cols;
    double mx = 0.0;
    for (size_t k = 0; k < cols; ++k) mx = fmax(mx, fabs(row[k]));
    int E = 0;
    if (mx > 0.0) frexp(mx, &E);  // mx < 2^E: the scaled row max lies in [2^14, 2^15)
    const int k2 = mx > 0.0 ? 15 - E : 0;
    inv[r] = (float)ldexp(1.0, -k2);
    for (size_t k = 0; k < cols; ++k) {
      const double v = ldexp(row[k], k2);
      const uint16_t h = f32_to_f16_rne((float)v);
      hi[r * cols + k] = h;
      lo[r * cols + k] = f32_to_f16_rne((float)(v - f16_to_double(h)));
    }
  }
}

extern "C" void jfg_split_f16_rows_host(int n, int nq, const double* ops, uint16_t* hi,
                                        uint16_t* lo, float* inv) {
  const size_t nn = (size_t)n * nq;
  // (first element, rows, row length) of the four blocks the passes read
  const size_t blk[4][3] = {{0, (size_t)2 * nq, (size_t)n},
                            {2 * nn, (size_t)2 * nq, (size_t)n},
                            {4 * nn, (size_t)2 * n, (size_t)nq},
                            {6 * nn, (size_t)n, (size_t)2 * nq}};
  size_t r_out = 0;
  for (const auto& bk : blk) {
    jfg_split_f16_rowscaled_host(bk[1], bk[2], ops + bk[0], hi + bk[0], lo + bk[0],
                                 inv + r_out);
    r_out += bk[1];
  }
}

extern "C" void jfg_split_f16_rows_nd_host(int ndim, int n, int nq, const double* ops,
                                           uint16_t* hi, uint16_t* lo, float* inv) {
  if (ndim != 3) {
    jfg_split_f16_rows_host(n, nq, ops, hi, lo, inv);
    return;
  }
  const size_t nn = (size_t)n * nq;
  // 3-D: [B;D] 2nq rows of n, then D,B,B 3nq rows of n, then B^T,B^T,D^T 3n
  // rows of nq
  const size_t blk[3][3] = {{0, (size_t)2 * nq, (size_t)n},
                            {2 * nn, (size_t)3 * nq, (size_t)n},
                            {5 * nn, (size_t)3 * n, (size_t)nq}};
  size_t r_out = 0;
  for (const auto& bk : blk) {
    jfg_split_f16_rowscaled_host(bk[1], bk[2], ops + bk[0], hi + bk[0], lo + bk[0],
                                 inv + r_out);
    r_out += bk[1];
  }
}

extern "C" size_t jfg_varcoef_workspace_size(int ndim, int n, int nq, int batch,
                                             int elem_bytes) {
  return jfg::varcoef_ws(ndim, n, nq, batch, elem_bytes);
}

extern "C" int jfg_varcoef_apply_f64(int ndim, int n, int nq, int batch, const double* ops,
                                     const double* kw, const double* u, double* v, void* work,
                                     size_t work_bytes, void* stream) {
  return jfg::varcoef_apply<double>(Engine::F64, ndim, n, nq, batch,
                                    OpRef<double>{ops, nullptr}, kw, u, v, work, work_bytes,
                                    (cudaStream_t)stream);
}

extern "C" int jfg_varcoef_apply_f32(int ndim, int n, int nq, int batch, const float* ops,
                                     const float* kw, const float* u, float* v, void* work,
                                     size_t work_bytes, void* stream) {
  return jfg::varcoef_apply<float>(Engine::F32, ndim, n, nq, batch, OpRef<float>{ops, nullptr},
                                   kw, u, v, work, work_bytes, (cudaStream_t)stream);
}
