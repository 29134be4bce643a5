/*
 * jaxfun_gb300 — C ABI of the GB300 (sm_103a) tensor-product spectral path.
 *
 * Every entry point takes plain device pointers, sizes and a cudaStream_t
 * (passed as void*), never allocates device memory unless it says so, never
 * throws, and returns an int status (JFG_OK == 0).  Arrays are C-order
 * (row-major), matching jaxfun's jax.Array layout.  The reference functions
 * each entry point replaces are cited as path:line of the jaxfun project.
 *
 * Layout conventions
 *   - A per-axis operator is a row-major matrix op[m][k]: row m of the result,
 *     k the contracted index.  Backward operators are (Nq x n) Vandermonde
 *     matrices with the Dirichlet stencil folded in, forward operators are
 *     (n x Nq) with the mass inverse folded in.
 *   - "Padded" solver layout: each spectral axis of length n (= N-2 for a
 *     Dirichlet composite) is stored in a buffer of length nq (the number of
 *     quadrature points), entries n..nq-1 equal to zero.
 */
#ifndef JAXFUN_GB300_H
#define JAXFUN_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  JFG_OK = 0,
  JFG_ERR_ARG = 1,            /* invalid shape / pointer / size (host check)   */
  JFG_ERR_CUDA = 2,           /* a CUDA runtime call failed                     */
  JFG_ERR_NOT_CONVERGED = 3,  /* iterative solver hit maxiter                   */
  JFG_ERR_DEVICE_TIMEOUT = 4, /* a bounded device wait gave up                  */
  JFG_ERR_UNSUPPORTED = 5,    /* device or configuration not supported          */
  JFG_ERR_WORKSPACE = 6       /* workspace smaller than *_workspace_size()      */
};

/* ---- epilogues of the per-axis contraction ----------------------------- */
enum {
  JFG_EPI_NONE = 0,      /* v = acc                                                  */
  JFG_EPI_MUL_FIELD = 1, /* v = acc * field[b][s][m][p]                              */
  JFG_EPI_DIV_EIG = 2    /* v = acc / (c0[b] + c1[b] * (lam_m[m] + lam_p[p]))        */
};

/*
 * One per-axis contraction pass ("contract the last axis, rotate it to the
 * front"):
 *   out[b][s][m][p] = alpha * epi( sum_k op[s][m][k] * in[b][s][p][k] )
 *                     + beta * out[b][s][m][p]
 * for b < batch, s < nseg, m < M, p < P, k < K.  Element (b,s,m,p) lives at
 *   op : s*op_seg + m*op_ld + k
 *   in : b*in_batch + s*in_seg + p*in_ld + k
 *   out: b*out_batch + s*out_seg + m*out_ld + p
 *   field (MUL): b*field_batch + s*field_seg + m*field_ld + p
 * Replaces the per-axis tensordot/moveaxis of TPMatrix._matmul_array
 * (src/jaxfun/la/tpmatrix.py:152-156), Matrix.matvec (src/jaxfun/la/
 * matrix.py:89-118) and the vmapped 1-D transforms of _build_local_apply_fn
 * (src/jaxfun/sharding.py:24-40).
 */
typedef struct {
  int batch, nseg, M, P, K;
  long long op_ld, op_seg;
  long long in_ld, in_seg, in_batch;
  long long out_ld, out_seg, out_batch;
  int epilogue;
  const void* field;
  long long field_ld, field_seg, field_batch;
  const void* lam_m; /* (M)      */
  const void* lam_p; /* (P)      */
  const void* c0;    /* (batch)  */
  const void* c1;    /* (batch)  */
  double alpha, beta;
  /* Optional active subset (device pointers; NULL = every problem): only
   * problems b = batch_list[j], j < *batch_count <= batch, are computed.  The
   * kernels read *batch_count and the list when they start, so a list that an
   * earlier kernel on the stream rebuilt (also inside a captured graph) takes
   * effect without the host.  Entries outside [0, batch) are skipped. */
  const int* batch_list;
  const int* batch_count;
} jfg_contract_desc;

/* ---- library ----------------------------------------------------------- */
const char* jfg_version(void);
const char* jfg_status_string(int status);
/* last CUDA error code seen by the library on this host thread (0 if none) */
int jfg_last_cuda_error(void);
/* 1 if the current device is sm_103 (GB300), else 0 */
int jfg_device_supported(void);
/* number of kernels this library has launched (graph replays count their
 * kernel nodes); reset with jfg_reset_launch_count */
long long jfg_launch_count(void);
void jfg_reset_launch_count(void);

/* kw[b][idx] = kappa[b][idx] * prod_ax w[i_ax]: the coefficient times the
 * tensor-product quadrature weights on the (nq)^ndim grid (the scale
 * evaluate_jaxfunction_expr_quad and the weights contribute in
 * src/jaxfun/galerkin/inner.py:445-490, 887-898); kw32 (optional, may be
 * NULL) receives the same values rounded to FP32 */
int jfg_weighted_field_f64(int ndim, int nq, int batch, const double* kappa, const double* w,
                           double* kw, float* kw32, void* stream);

/* The coefficient of a variable-coefficient form evaluated from its
 * logarithm on the quadrature grid: kappa = exp(scale[b] (g - shift[b])) and
 * kw = kappa * prod_ax w[i_ax] (kw32: FP32 copy, may be NULL; kappa: may be
 * NULL), one pass -- evaluate_jaxfunction_expr_quad for exp(g) of a
 * JAXFunction g (src/jaxfun/galerkin/arguments.py:928-990, the backward
 * transform of g being jfg_tp_apply_f64) fused with the weighting of
 * jfg_weighted_field_f64.  scale / shift: per problem, NULL for 1 / 0. */
int jfg_exp_weighted_field_f64(int ndim, int nq, int batch, const double* g,
                               const double* scale, const double* shift, const double* w,
                               double* kappa, double* kw, float* kw32, void* stream);
/* The same coefficient from the ORTHOGONAL-basis coefficients of g
 * ((batch, n, ..., n), a JAXFunction's coefficients) in one sequence: the
 * backward transform (V: the (nq, n) backward matrix of the orthogonal
 * space, every axis) whose last pass evaluates exp and the weights in its
 * epilogue, so g never crosses HBM on its own -- evaluate_jaxfunction_expr_quad
 * for exp(g) (src/jaxfun/galerkin/arguments.py:928-990) fused into the
 * backward transform of the coefficients (src/jaxfun/galerkin/
 * tensorproductspace.py:330-346).  standardize = 1: g is shifted and scaled
 * to mean 0 and population standard deviation 1 per problem; the last pass
 * then writes g with per-tile moments (count, mean, sum of squared
 * deviations, combined pairwise) and one more pass applies exp and the
 * weights.  kappa and kw32 may be NULL.  Workspace:
 * jfg_exp_weighted_backward_workspace_size. */
size_t jfg_exp_weighted_backward_workspace_size(int ndim, int n, int nq, int batch);
int jfg_exp_weighted_backward_f64(int ndim, int n, int nq, int batch, const double* V,
                                  const double* g_coef, int standardize, const double* w,
                                  double* kappa, double* kw, float* kw32, void* work,
                                  size_t work_bytes, void* stream);
/* Per problem: mean of g and 1 / population standard deviation (FP64, two
 * passes), for standardising g before exp (shift = mean, scale = 1 / std). */
int jfg_field_moments_f64(int ndim, int nq, int batch, const double* g, double* mean,
                          double* inv_std, void* stream);

/* ---- generic contraction (FP64 / FP32 CUDA cores) ---------------------- */
int jfg_contract_f64(const jfg_contract_desc* d, const double* op, const double* in,
                     double* out, void* stream);
int jfg_contract_f32(const jfg_contract_desc* d, const float* op, const float* in,
                     float* out, void* stream);
/* FP64 in/out, computed in double-FP32 arithmetic on the FP32 units: operands
 * split into hi + lo FP32 pairs, error-free products (FMA) and TwoSum
 * accumulation, ~2^-46 relative error per product (FP64: 2^-53).  Used for the
 * refinement residual, where GB300's FP64 rate would dominate. */
int jfg_contract_df64(const jfg_contract_desc* d, const double* op, const double* in,
                      double* out, void* stream);

/*
 * Tensor-core contraction (tcgen05, TMA, TMEM accumulators): three-term
 * split-TF32 products hi*hi + hi*lo + lo*hi with FP32 accumulation.
 * op_hi/op_lo are the TF32 split of the FP64 operator (op_hi has its low 13
 * mantissa bits cleared, op_lo = op - op_hi rounded to FP32).  Requires
 * K % 32 == 0, M % 16 == 0, M <= 256, P % 128 == 0, in_ld/op_ld % 4 == 0,
 * 16-byte aligned pointers.  Same semantics as jfg_contract_f32.
 */
int jfg_contract_tc(const jfg_contract_desc* d, const float* op_hi, const float* op_lo,
                    const float* in, float* out, void* stream);
/* The same contraction with the operator split into BF16 (hi, lo) pairs
 * (jfg_split_bf16_host) and the FP32 input split into BF16 pairs in the
 * kernel: three BF16 MMAs (hi*hi + hi*lo + lo*hi, FP32 accumulate) per
 * product at twice the TF32 rate; ~2^-16 relative per product.  For the
 * HBM-bound batched transforms.  op_ld, op_seg % 8 == 0.
 * op_lo NULL: plain BF16, one MMA per product (hi*hi: operator hi and the
 * input rounded to BF16, ~2^-8 relative; products exact in FP32), for the
 * inner preconditioner's passes; beta 0 and no field epilogue then (else
 * JFG_ERR_ARG). */
int jfg_contract_tc_bf16x3(const jfg_contract_desc* d, const uint16_t* op_hi,
                           const uint16_t* op_lo, const float* in, float* out, void* stream);
/* Split n FP64 values into BF16 hi (round to nearest even) and lo = x - hi
 * rounded to BF16 (host arrays of BF16 bit patterns). */
void jfg_split_bf16_host(size_t n, const double* src, uint16_t* hi, uint16_t* lo);
/* The same contraction in scaled split FP16 (kind::f16 with FP16 operands,
 * three MMAs per product at the BF16 rate, ~2^-22 relative to each row's
 * maximum like split TF32).  The operator is FP16 (hi, lo), each row m of
 * segment s scaled by a power of two (jfg_split_f16_rowscaled_host), with the
 * inverse scales at op_inv[s * op_inv_seg + m].  The input of problem b is
 * scaled in the kernel by the power of two that puts in_max[b] -- the float
 * bits of an upper bound on max |in[b]| -- in [2^14, 2^15) (a bound 0 means
 * no scaling; inputs beyond 65504 / 2 then overflow).  out_max (may be NULL)
 * receives, by atomicMax on the float bits, max |out[b]| of every written
 * problem; clear it before the call.  op_ld, op_seg % 8 == 0. */
int jfg_contract_tc_f16x3(const jfg_contract_desc* d, const uint16_t* op_hi,
                          const uint16_t* op_lo, const float* op_inv, long long op_inv_seg,
                          const unsigned* in_max, unsigned* out_max, const float* in,
                          float* out, void* stream);
/* rows x cols FP64 matrix -> FP16 hi / lo bit patterns with each row scaled
 * by the power of two that puts its max |entry| in [2^14, 2^15); inv[r] is
 * the inverse scale of row r.  Host arrays. */
void jfg_split_f16_rowscaled_host(size_t rows, size_t cols, const double* src, uint16_t* hi,
                                  uint16_t* lo, float* inv);
/* Kernel variant of jfg_contract_tc: 1 (default) keeps the split input tile
 * (MMA operand A) in TMEM, written by the split warps with tcgen05.st, so the
 * MMAs read only operand B from shared memory; 0 keeps A in shared memory. */
int jfg_tc_set_variant(int operand_a_in_tmem);
/* Epilogue output path of the tensor-core contractions: 1 (default) stages
 * 32 x 32 output boxes in shared memory and writes them with TMA bulk tensor
 * stores where the output rows are 16-byte aligned (and beta == 0); 0 uses
 * plain coalesced stores everywhere. */
int jfg_tc_set_store_path(int tma_store);
/* Schedule of single-group launches with 16-bit operators (split BF16, scaled
 * split FP16): 0 (default) streams operator and input tiles together; 1
 * operator-stationary -- each persistent CTA serves one (segment, operator
 * chunk) slot, keeps that chunk for all K blocks in shared memory and streams
 * only input tiles, used when the chunk fits beside >= 2 input stages
 * (K <= 256 at 128 operator rows) and there are >= 2 tiles per CTA; 2
 * whenever the chunk fits.  The autotuner tries both where the chunk fits. */
int jfg_tc_set_op_resident(int on);
/* Launch configuration of the tensor-core contraction. */
typedef struct {
  int operand_a_in_tmem; /* 1: split input tile in TMEM; 0: in shared memory          */
  int order;             /* grouped launches: 0 groups as given, 1 by operator-tile
                            work, 2 by total work (largest first)                    */
  int ctas;              /* persistent CTAs (0: one per SM)                          */
  int stages;            /* pipeline stages (0: as many as fit, else >= 2)           */
  int mtile;             /* operator rows per tile = MMA N (0: up to 128, else 64)   */
  int schedule;          /* single-group 16-bit launches: 0 the process setting
                            (jfg_tc_set_op_resident), 1 streaming, 2 operator-
                            stationary where the chunk fits                       */
  int store;             /* epilogue: 0 the process setting (jfg_tc_set_store_path),
                            1 TMA bulk-tensor stores where allowed, 2 plain stores */
} jfg_tc_config;
/*
 * Grouped tensor-core contraction: ngroups independent contractions (each a
 * jfg_contract_desc with its own shapes, batch and pointers; one epilogue kind
 * and beta != 0 either for all or for none) run in ONE persistent launch (per
 * 40 groups) whose CTAs walk the tiles of all groups -- e.g. the per-axis
 * passes of many fast-diagonalisation solves of uneven N.  cfg NULL: the
 * configuration jfg_tc_autotune chose for this signature, else the default.
 */
int jfg_contract_tc_grouped(int ngroups, const jfg_contract_desc* descs,
                            const float* const* op_hi, const float* const* op_lo,
                            const float* const* in, float* const* out,
                            const jfg_tc_config* cfg, void* stream);
/*
 * Autotuner: times every candidate configuration (operand A in TMEM or shared
 * memory x group order x pipeline depth x tile height) of the grouped contraction on the
 * given operands with CUDA events (reps launches each; the contraction runs,
 * so out is written), keeps the fastest for this launch signature (shapes,
 * batches, epilogue) and returns it with its time.  Not during stream capture.
 */
int jfg_tc_autotune(int ngroups, const jfg_contract_desc* descs, const float* const* op_hi,
                    const float* const* op_lo, const float* const* in, float* const* out,
                    int reps, jfg_tc_config* best, float* best_ms, void* stream);
/*
 * Autotuning of single-group launches (jfg_contract_tc, _bf16x3, _f16x3 and
 * the passes of the solvers built on them).  With on = 1, every launch whose
 * signature (device, precision, batch, segments, M, P, K, epilogue, beta) has
 * no tuned configuration yet and that is made outside stream capture first
 * times the candidates -- pipeline depth (as many as fit, 3, 2) x schedule
 * (streaming, operator-stationary for 16-bit operators) x epilogue store path
 * (TMA, plain) x tile height (128, 64) x operand A placement (split TF32) --
 * with CUDA events on its own operands (the launch runs, so out is written
 * repeatedly), keeps the fastest for that signature and launches with it;
 * tuned signatures always launch with their configuration.  Default 0.
 */
int jfg_tc_set_autotune(int on);
/* One configuration for every single-group tensor-core launch of the
 * process (NULL: back to the tuned or default one) -- for tests and tuning
 * studies; no counterpart in the reference. */
int jfg_tc_force_config(const jfg_tc_config* cfg);
/* Tuned single-group signatures: how many, and entry i (its signature as
 * text, its configuration and its time in ms per launch). */
int jfg_tc_tuned_count(void);
int jfg_tc_tuned_entry(int i, char* signature, size_t signature_len, jfg_tc_config* cfg,
                       float* ms);
/* Split n FP64 values into TF32 hi (round to nearest) and FP32 lo = x - hi
 * (host arrays), the operator format jfg_contract_tc expects. */
void jfg_split_tf32_host(size_t n, const double* src, float* hi, float* lo);
/* Reads and clears the device status word the tensor-core kernels set when a
 * bounded wait expires (JFG_OK or JFG_ERR_DEVICE_TIMEOUT); synchronous. */
int jfg_device_status(void);
/* Testing the bounded waits (no counterpart in the reference).  Budget of
 * every pipeline wait of the tcgen05 contraction kernels in ns (0 restores
 * the default 2 s); waits that drain the kernel's own copies and MMAs after
 * a timeout keep the default.  Affects launches made after the call. */
int jfg_tc_set_wait_budget_ns(unsigned long long ns);
/* Test hook (1 on, 0 off): the epilogue warps of the tcgen05 contraction
 * first wait on a barrier that nothing arrives on, so that wait runs out
 * after the wait budget, JFG_ERR_DEVICE_TIMEOUT is recorded for
 * jfg_device_status(), every other role's waits run out in turn and the
 * kernel drains its copies and MMAs, frees its TMEM and returns.  The output
 * of such a launch is not written completely. */
int jfg_tc_test_hold(int on);

/* ---- TensorProductSpace transforms -------------------------------------
 * out[b] = (x_ax mats[ax]) in[b]: mats[ax] is rows[ax] x cols[ax] row-major,
 * in is (batch, cols[0], ..., cols[ndim-1]), out (batch, rows[0], ...).
 * TensorProductSpace.backward / forward / scalar_product
 * (src/jaxfun/galerkin/tensorproductspace.py:330-417) with the 1-D
 * operators of OrthogonalSpace/Composite/Chebyshev (src/jaxfun/galerkin/
 * orthogonal.py:214-277, composite.py:205-349, Chebyshev.py:225-279).
 * ndim in {1,2,3}.  Workspace: jfg_tp_apply_workspace_size bytes.
 */
size_t jfg_tp_apply_workspace_size(int ndim, const int* rows, const int* cols, int batch,
                                   int elem_bytes);
int jfg_tp_apply_f64(int ndim, const int* rows, const int* cols, int batch,
                     const double* const* mats, const double* in, double* out,
                     void* work, size_t work_bytes, void* stream);
/* FP64 data in double-FP32 arithmetic (jfg_contract_df64 per pass, about
 * 1e-14 relative per contraction, ~3x the FP64 pipe's rate on GB300): for
 * FP64-class right-hand sides, e.g. the scalar product of a forcing. */
int jfg_tp_apply_df64(int ndim, const int* rows, const int* cols, int batch,
                      const double* const* mats, const double* in, double* out,
                      void* work, size_t work_bytes, void* stream);
int jfg_tp_apply_f32(int ndim, const int* rows, const int* cols, int batch,
                     const float* const* mats, const float* in, float* out,
                     void* work, size_t work_bytes, void* stream);
/* Same transforms on the tensor cores (jfg_contract_tc per pass): operators
 * given as TF32 (hi, lo) splits, FP32 data; rows/cols % 4 == 0 and 16-byte
 * aligned buffers (the TMA constraints of jfg_contract_tc). */
int jfg_tp_apply_tc(int ndim, const int* rows, const int* cols, int batch,
                    const float* const* mats_hi, const float* const* mats_lo, const float* in,
                    float* out, void* work, size_t work_bytes, void* stream);
/* ... and with split-BF16 operators (jfg_contract_tc_bf16x3 per pass; cols % 8
 * == 0 for the BF16 operator rows). */
int jfg_tp_apply_tc_bf16x3(int ndim, const int* rows, const int* cols, int batch,
                           const uint16_t* const* mats_hi, const uint16_t* const* mats_lo,
                           const float* in, float* out, void* work, size_t work_bytes,
                           void* stream);

/* ---- affine transforms (inhomogeneous boundary lifting) -----------------
 * out[b] = (x_ax mats[ax]) in[b] + shift, one shift array (rows[0] x ... x
 * rows[ndim-1]) for every b, added in the epilogue of the last pass (the pass
 * accumulates, beta = 1, into out pre-filled with shift).  The DirectSum
 * spaces' maps are affine in the coefficients: to_orthogonal adds the boundary
 * lift, from_orthogonal / forward subtract it, backward adds the lift's grid
 * values (DirectSum.to_orthogonal/from_orthogonal/backward/forward,
 * src/jaxfun/galerkin/composite.py:585-600, 617-621; DirectSumTPS,
 * src/jaxfun/galerkin/tensorproductspace.py:777-851).  out must not overlap
 * in; otherwise as jfg_tp_apply_f64 (same workspace size).
 */
int jfg_tp_apply_affine_f64(int ndim, const int* rows, const int* cols, int batch,
                            const double* const* mats, const double* in, const double* shift,
                            double* out, void* work, size_t work_bytes, void* stream);

/* ---- batched banded LU (wavenumber solver) ------------------------------
 * TPMatricesWavenumberSolver (src/jaxfun/la/tpmatrix.py:590-1013): one 1-D
 * banded system per Fourier wavenumber, factored without pivoting
 * (_lu_banded_no_pivot_kernel, src/jaxfun/la/diamatrix.py:1937-1973) and
 * solved by forward / backward substitution, one GPU thread per system.
 * data (nsys, ndiag, n) uses jaxfun's column-aligned DIA convention:
 * data[s][d][j] = A_s[j - offsets[d]][j]; offsets (host) distinct, one of them
 * 0.  p = max(0, -min offset), q = max(0, max offset); lu holds
 * jfg_banded_lu_size(nsys, n, p, q) bytes.  The solve reads element i of
 * system s at rhs[s*sys_stride + i*elem_stride] and writes x the same way
 * (x may equal rhs). */
size_t jfg_banded_lu_size(int nsys, int n, int p, int q);
int jfg_banded_lu_factor_f64(int nsys, int n, int ndiag, const int* offsets, const double* data,
                             double* lu, void* stream);
int jfg_banded_lu_solve_f64(int nsys, int n, int p, int q, const double* lu, const double* rhs,
                            double* x, long long sys_stride, long long elem_stride, void* stream);

/* ---- fast-diagonalisation solve ----------------------------------------
 * TPMatricesLUFactors.solve (src/jaxfun/la/tpmatrix.py:545-587), batched:
 *   U_b = (x_ax W) [ (x_ax E) F_b / (c0[b] + c1[b] * sum_ax lam[i_ax]) ]
 * Same n x n E (= W^{-1} M^{-1}; W^T for symmetric pairs), W and lam on
 * every axis (square tensor-product space, n per axis), rhs/out
 * (batch, n^ndim).  lam has length n.  ndim in {2,3}.
 */
size_t jfg_fd_solve_workspace_size(int ndim, int n, int batch, int elem_bytes);
int jfg_fd_solve_f64(int ndim, int n, int batch, const double* E, const double* W,
                     const double* lam, const double* c0, const double* c1,
                     const double* rhs, double* out, void* work, size_t work_bytes,
                     void* stream);
int jfg_fd_solve_f32(int ndim, int n, int batch, const float* E, const float* W,
                     const float* lam, const float* c0, const float* c1, const float* rhs,
                     float* out, void* work, size_t work_bytes, void* stream);

/* Tensor-core FD solve (split-TF32 tcgen05 passes, FP32 data): E/W given as
 * TF32 (hi, lo) pairs; n % 4 == 0 (pad with zero rows/columns and lam = 1). */
int jfg_fd_solve_tc(int ndim, int n, int batch, const float* E_hi, const float* E_lo,
                    const float* W_hi, const float* W_lo, const float* lam, const float* c0,
                    const float* c1, const float* rhs, float* out, void* work,
                    size_t work_bytes, void* stream);

/* v_b = alpha2[b] (M (x) M) u_b + (K (x) M) u_b + (M (x) K) u_b for 2-D
 * Dirichlet composites (family 0 Legendre, 1 Chebyshev; n = N - 2 per axis,
 * u/v (batch, n, n) FP64), computed in O(n^2) per problem from the closed
 * forms of M = S diag(h) S^T and K = -S D2 S^T (src/jaxfun/galerkin/
 * composite.py:330-333, Legendre.py:19-33, Chebyshev.py:21-35); with b != NULL
 * it returns v = b - A u (the FP64 refinement residual).  alpha2 may be NULL. */
size_t jfg_helmholtz_workspace_size(int n, int batch);
int jfg_helmholtz_apply_f64(int family, int n, int batch, const double* alpha2, const double* u,
                            const double* b, double* v, void* work, size_t work_bytes,
                            void* stream);

/* Mixed-precision batch of equal-size Dirichlet Helmholtz solves: FP64
 * iterative refinement x += ||r|| FD_tc(r / ||r||), r = b - A x (structured
 * FP64 apply above), until ||r_b|| <= tol ||b_b||.  The FD correction runs on
 * the tensor cores in the padded layout (nq >= n, nq % 4 == 0; E/W padded
 * with zeros, lam32 with ones) with D = alpha2_32[b] + lam_i + lam_j.
 * refinements (host, may be NULL) receives per-problem correction counts.
 * (jfg_helmholtz_solve_grouped solves uneven batches in one call.) */
size_t jfg_helmholtz_solve_workspace_size(int n, int nq, int batch);
int jfg_helmholtz_solve_mixed(int family, int n, int nq, int batch, const float* E_hi,
                              const float* E_lo, const float* W_hi, const float* W_lo,
                              const float* lam32, const double* alpha2, const float* alpha2_32,
                              const double* rhs, double* x, double tol, int max_refine,
                              int* refinements, void* work, size_t work_bytes, void* stream);

/*
 * The same refinement for an uneven batch in ONE call: ngroups size groups
 * (group g: batch[g] problems of n[g] = N_g - 2 unknowns per axis, padded
 * nq[g] % 4 == 0, its own FD factors E/W/lam32).  rhs, x (FP64) and alpha2,
 * alpha2_32 (per problem) are group-major and flat: problem k of group g
 * follows the earlier problems, n[g]^2 values each.  Each refinement step is
 * four grouped persistent tensor-core launches over all groups
 * (jfg_contract_tc_grouped with cfg, NULL = default), ragged FP32 pad/axpy
 * kernels and the structured FP64 residual over all lines; every per-problem
 * scalar stays on the device, the step is captured once into a CUDA graph and
 * replayed until no problem has ||r_b|| > tol ||b_b||.  Stands in for calling
 * TPMatrices.solve (src/jaxfun/la/tpmatrix.py:429-509) once per problem.
 */
size_t jfg_helmholtz_grouped_workspace_size(int ngroups, const int* n, const int* nq,
                                            const int* batch);
int jfg_helmholtz_solve_grouped(int family, int ngroups, const int* n, const int* nq,
                                const int* batch, const float* const* E_hi,
                                const float* const* E_lo, const float* const* W_hi,
                                const float* const* W_lo, const float* const* lam32,
                                const double* alpha2, const float* alpha2_32, const double* rhs,
                                double* x, double tol, int max_refine, int* refinements,
                                const jfg_tc_config* cfg, void* work, size_t work_bytes,
                                void* stream);

/*
 * jfg_fd_solve_f64 without a workspace argument: for callers that cannot
 * allocate device memory where they solve (inside a host runtime that owns
 * all device memory and offers no workspace, in a loop that must not block on
 * an allocator).  No counterpart in the
 * reference.  Scratch comes from a fixed 32 MiB device array inside the
 * library (jfg_fd_solve_noalloc_max_bytes()); every GPU that loads the library
 * holds it until exit.  A call whose scratch need (jfg_fd_solve_workspace_size)
 * exceeds it returns JFG_ERR_WORKSPACE and launches nothing.  All calls share
 * the array: calls whose kernels overlap on the GPU race; calls ordered on one
 * stream are safe.  The first call on a device resolves the array's device
 * address (with that device current) and caches it for the life of the
 * process; make it before any stream capture, and do not call again on a
 * device after cudaDeviceReset (the cached address is then stale).
 * Allocates nothing (no cudaMalloc/cudaFree, no allocating library call).
 */
size_t jfg_fd_solve_noalloc_max_bytes(void);
int jfg_fd_solve_f64_noalloc(int ndim, int n, int batch, const double* E, const double* W,
                             const double* lam, const double* c0, const double* c1,
                             const double* rhs, double* out, void* stream);

/* ---- variable-coefficient operator apply -------------------------------
 * v_b = A(kappa_b) u_b for the form (kappa grad u, grad v), sum-factorised:
 * the TensorMatrix jaxfun assembles for kappa*Dot(Grad(u), Grad(v))
 * (src/jaxfun/galerkin/inner.py:445-490, 991-1024) applied as
 * TensorMatrix._matmul_array (src/jaxfun/la/tensormatrix.py:54-56), without
 * forming the O(n^4) tensor.  ops is the packed operator set produced by
 * jfg_varcoef_pack_ops_host from B[q][k] = phi_k(x_q) and D[q][k] =
 * phi_k'(x_q) (nq x n); kw is (batch, nq^ndim) = kappa * w (x) w [(x) w];
 * u, v are (batch, n^ndim).  ndim in {2,3}.
 */
size_t jfg_varcoef_ops_count(int ndim, int n, int nq);
void jfg_varcoef_pack_ops_host(int ndim, int n, int nq, const double* B, const double* D,
                               double* ops_out);
size_t jfg_varcoef_workspace_size(int ndim, int n, int nq, int batch, int elem_bytes);
int jfg_varcoef_apply_f64(int ndim, int n, int nq, int batch, const double* ops,
                          const double* kw, const double* u, double* v, void* work,
                          size_t work_bytes, void* stream);
int jfg_varcoef_apply_f32(int ndim, int n, int nq, int batch, const float* ops,
                          const float* kw, const float* u, float* v, void* work,
                          size_t work_bytes, void* stream);

/* ---- preconditioned conjugate gradients --------------------------------
 * Batched PCG for A(kappa_b) x_b = rhs_b with the constant-coefficient
 * fast-diagonalisation preconditioner (E, W, lam; c0 = 0, c1 = fd_scale[b]).
 * No PCG exists on jaxfun's Galerkin path; this follows the textbook
 * algorithm of jax.scipy.sparse.linalg.cg (used at src/jaxfun/pinns/
 * hessoptimizer.py:97).  Problem b stops when sqrt(r.z / r0.z0) <= tol
 * (r0 = rhs - A x0).  If use_x0 is 0, x is zeroed first.  iters (host, may be
 * NULL) receives per-problem iteration counts.  Returns JFG_ERR_NOT_CONVERGED
 * when any problem reaches maxiter.
 */
size_t jfg_pcg_workspace_size(int ndim, int n, int nq, int batch, int elem_bytes);
int jfg_pcg_varcoef_f64(int ndim, int n, int nq, int batch, const double* ops,
                        const double* kw, const double* E, const double* W,
                        const double* lam, const double* fd_scale, const double* rhs,
                        double* x, int use_x0, double tol, int maxiter, int* iters,
                        void* work, size_t work_bytes, void* stream);

/* ---- BF16 tensor-core GEMM for the spectral neural operator ------------
 * D[b][m][n] = alpha * sum_k A[b][m][k] * B[b][n][k]   (BF16 in, FP32 accumulate)
 * then, in this order: + add[b][m][n] (FP32), + bias[n], * gelu'(gg[b][m][n]),
 * pre = value (FP32), value = gelu(value) if act == 1.  Outputs (each optional):
 * d32 (FP32 row-major; atomically added when ksplit > 1 or d32_accumulate),
 * dbf (BF16 row-major), dtbf (BF16 transposed: dtbf[b][n][m]).  A/B are K-major
 * with row strides lda/ldb (multiples of 8 elements) and batch strides
 * (0 = shared).  ksplit > 1 splits K across CTAs (d32 only, no add/bias/act).
 * tcgen05 kind::f16, 128 x N tiles (N <= 256), TMA 128-byte swizzle.  No
 * counterpart in the reference (the learned initial guess is new).
 */
typedef struct {
  int batch, M, N, K, ksplit;
  long long lda, a_batch, ldb, b_batch;
  float alpha;
  int act; /* 0 none, 1 GELU */
  const float* add;
  long long ld_add, add_batch;
  const float* bias;
  const float* gg;
  long long ld_gg, gg_batch;
  float* d32;
  long long ld_d32, d32_batch;
  int d32_accumulate;
  float* pre;
  long long ld_pre, pre_batch;
  void* dbf;
  long long ld_dbf, dbf_batch;
  void* dtbf;
  long long ld_dtbf, dtbf_batch;
} jfg_gemm_desc;

int jfg_gemm_bf16(const jfg_gemm_desc* d, const void* A, const void* B, void* stream);

/* ---- spectral neural operator helpers (CUDA cores) ---------------------
 * Mode mixing of a spectral convolution: for every mode q and sample b,
 *   out[b][co][q] = sum_ci R[q][co][ci] * x[b][q][ci]        (forward, BF16 out)
 * backward: dx[b][ci][q] = sum_co R[q][co][ci] * dy[b][q][co]  (BF16 out) and
 *           dR[q][co][ci] = sum_b dy[b][q][co] * x[b][q][ci]    (FP32, overwritten)
 * x, dy are FP32 [b][q][c]; R FP32 [q][co][ci]. */
int jfg_sno_modemix_fwd(int batch, int nmodes, int C, const float* R, const float* x,
                        void* out_bf16, void* stream);
int jfg_sno_modemix_bwd(int batch, int nmodes, int C, const float* R, const float* x,
                        const float* dy, void* dx_bf16, float* dR, void* stream);
/* colsum[n] (+)= sum_r src[r][n] for BF16 src (rows x n); accumulate 0/1 */
int jfg_colsum_bf16(long long rows, int n, const void* src, float* out, int accumulate,
                    void* stream);
/* Adam (decoupled from torch): p -= lr * mhat / (sqrt(vhat) + eps); optional
 * BF16 copies of p (row-major, and transposed when rows/cols > 0) */
int jfg_adam_step(long long n, float* p, const float* g, float* m, float* v, float lr,
                  float beta1, float beta2, float eps, int step, void* p_bf16,
                  void* pt_bf16, int rows, int cols, void* stream);
/* loss partials and dpred for 0.5*mean((pred - target)^2):
 * pred FP32 (rows, ld_pred) column 0; writes dq BF16 (rows x 16, col 0 used) and
 * its transpose dqt (16 x rows); loss_out[0] (+)= sum of squares (atomic). */
int jfg_sno_mse(long long rows, const float* pred, long long ld_pred, const float* target,
                void* dq_bf16, void* dqt_bf16, float* loss_out, void* stream);

/* ---- mixed-precision PCG with FP64 iterative refinement ----------------
 * Outer loop (FP64): r = rhs - A x with the FP64 operator (ops64, kw64 on the
 * unpadded (batch, n^ndim) layout); stop problem b when ||r_b|| <= tol ||rhs_b||.
 * Inner solve (tensor cores): PCG on A d = r / ||r|| in FP32 storage with
 * split-TF32 tcgen05 contractions, in the padded layout (nq per axis), to
 * sqrt(r.z / r0.z0) <= inner_tol; then x += ||r|| d.  The padded FP32
 * operators are the split (hi, lo) of the FP64 ones with zero rows/columns
 * beyond n (lam padded with ones).  Returns JFG_ERR_NOT_CONVERGED if any
 * problem misses tol after max_outer refinements.
 */
typedef struct {
  int ndim, n, nq, batch;
  const double* ops64;   /* jfg_varcoef_pack_ops_host(ndim, n, nq, ...)          */
  const double* kw64;    /* (batch, nq^ndim)                                       */
  const float* ops_hi;   /* packed padded operators (n -> nq), TF32 hi part        */
  const float* ops_lo;   /*                                      lo part           */
  const float* kw32;     /* (batch, nq^ndim)                                       */
  const float* E_hi;     /* (nq x nq) padded fast-diagonalisation factors          */
  const float* E_lo;
  const float* W_hi;
  const float* W_lo;
  const float* lam;      /* (nq), ones beyond n                                    */
  const float* fd_scale; /* (batch) or NULL                                        */
  const float* ops32;    /* packed padded operators rounded to FP32, or NULL: used for
                            r -= ||r|| A d once ||r|| <= 1e-4 ||rhs|| (else FP64 r = b - A x) */
  int residual;          /* arithmetic of r = b - A x: 0 FP64 (DFMA), 1 double-FP32
                            (jfg_contract_df64 passes)                                */
  int precond_bf16;      /* 1: the inner preconditioner's FD passes use split-BF16
                            operators (E/W_hi16, _lo16: jfg_split_bf16_host of the
                            padded factors), 2: plain BF16 (E/W_hi16 only; the
                            _lo16 pointers unused), 0: split-TF32 (E/W_hi, _lo).  The
                            operator passes stay split-TF32: with split-BF16 they
                            stall the inner solve near its 1e-5 tolerance           */
  const uint16_t* E_hi16;
  const uint16_t* E_lo16;
  const uint16_t* W_hi16;
  const uint16_t* W_lo16;
  int apply_f16;         /* 1 (nq % 8 == 0): the inner operator passes run as scaled
                            split FP16 (jfg_split_f16_rows_nd_host of the packed padded
                            operators, rows scaled by powers of two; the inputs of
                            each pass scaled per problem from a recorded max |x|):
                            the accuracy of split TF32 at the BF16 rate.  0: split
                            TF32 (ops_hi, ops_lo)                                   */
  const uint16_t* ops_hi16;  /* FP16 hi of the row-scaled packed padded operators   */
  const uint16_t* ops_lo16;  /* FP16 lo                                             */
  const float* ops_inv16;    /* inverse row scales, jfg_varcoef_f16_rows_nd(ndim, nq, nq)
                                of them; 2-D: [B;D] 2nq | D, B 2nq | B^T, D^T 2n |
                                [D^T|B^T] n; 3-D: [B;D] 2nq | D, B, B 3nq |
                                B^T, B^T, D^T 3n                                     */
  int fused_dots;        /* inner PCG scalars from the contraction epilogues instead of
                            separate dot kernels: bit 0 p.Ap = sum kappa w |grad p|^2 in
                            the operator's field pass; bit 1 r.M^-1 r = sum (E r)^2 / D
                            in the preconditioner's divide pass (valid only when
                            E = W^T, the symmetric (Legendre) factorisation)            */
  int schedule;          /* 0: every outer step waits for all problems' inner solves;
                            1: each problem takes its outer steps on its own (its
                            converged inner solve leaves for a ready list that takes
                            its outer step at the next 10-iteration boundary and
                            restarts while the others iterate), so the batch runs
                            about its slowest problem's total iteration count       */
} jfg_mixed_plan;

/* Rows of the 2-D packed operator set (jfg_varcoef_pack_ops_host(2, n, nq))
 * in the order their inverse scales are stored: 4 nq + 3 n. */
size_t jfg_varcoef_f16_rows(int n, int nq);
/* Split the 2-D packed operators (FP64, jfg_varcoef_pack_ops_host layout)
 * into FP16 hi / lo bit patterns, each operator row scaled by the power of
 * two that puts its max |entry| in [2^14, 2^15); inv receives the inverse
 * scales (jfg_varcoef_f16_rows(n, nq) floats).  Host arrays. */
void jfg_split_f16_rows_host(int n, int nq, const double* ops, uint16_t* hi, uint16_t* lo,
                             float* inv);
/* The same for the 2-D or 3-D packed operators (jfg_varcoef_pack_ops_host(ndim,
 * n, nq)); jfg_varcoef_f16_rows_nd gives the number of rows (2-D 4 nq + 3 n,
 * 3-D 5 nq + 3 n). */
size_t jfg_varcoef_f16_rows_nd(int ndim, int n, int nq);
void jfg_split_f16_rows_nd_host(int ndim, int n, int nq, const double* ops, uint16_t* hi,
                                uint16_t* lo, float* inv);

size_t jfg_pcg_mixed_workspace_size(int ndim, int n, int nq, int batch);
int jfg_pcg_varcoef_mixed(const jfg_mixed_plan* plan, const double* rhs, double* x, int use_x0,
                          double tol, double inner_tol, int max_outer, int maxiter_inner,
                          int* inner_iters, int* outer_iters, void* work, size_t work_bytes,
                          void* stream);
/* The same solve with a learned initial guess (batch, n^ndim) FP64 (may be
 * NULL): the first inner solve starts from guess / ||rhs|| and keeps it, per
 * problem, only where its preconditioned residual beats the zero start; the
 * inner tolerance is then measured relative to the right-hand side.  The
 * answer is always the converged solve judged by the outer residual. */
int jfg_pcg_varcoef_mixed_guess(const jfg_mixed_plan* plan, const double* rhs, double* x,
                                const double* guess, int use_x0, double tol, double inner_tol,
                                int max_outer, int maxiter_inner, int* inner_iters,
                                int* outer_iters, void* work, size_t work_bytes, void* stream);
/* Autotune the tensor-core passes of this plan's inner solve (no counterpart
 * in the reference): runs one operator apply and one preconditioner solve on
 * the (zeroed) workspace with jfg_tc_set_autotune's tuning on, so each
 * distinct pass signature keeps its fastest launch configuration for the
 * process.  Synchronous; call before solving (outside stream capture). */
int jfg_pcg_mixed_autotune(const jfg_mixed_plan* plan, void* work, size_t work_bytes,
                           void* stream);

#ifdef __cplusplus
}
#endif

#endif /* JAXFUN_GB300_H */
