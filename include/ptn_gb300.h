/*
 * ptn_gb300.h -- C ABI of the GB300 engine for PyTreeNet's TDVP local-update path.
 *
 * Every entry point takes caller-owned device pointers and a cudaStream_t (passed
 * as void*), allocates nothing, launches asynchronously on that stream, and
 * returns an int status (PTN_OK = 0). Complex numbers are interleaved
 * (re, im) pairs: complex128 = two doubles. All sizes and strides are in
 * elements of the operand's complex type.
 *
 * The reference (PyTreeNet) is pure Python/NumPy and has no FFI of its own; each
 * entry point below names the reference function whose NumPy call chain it
 * replaces. The Python layer (pytreenet_gb300) binds these with ctypes.
 */
#ifndef PTN_GB300_H
#define PTN_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PTN_OK = 0,
  PTN_ERR_ARG = 1,          /* bad shape / stride / null pointer          */
  PTN_ERR_LAUNCH = 2,       /* CUDA launch or runtime error               */
  PTN_ERR_NONFINITE = 3,    /* NaN or Inf found in an input               */
  PTN_ERR_BREAKDOWN = 4,    /* Krylov breakdown that cannot be continued  */
  PTN_ERR_NOCONVERGE = 5,   /* iterative decomposition did not converge   */
  PTN_ERR_UNSUPPORTED = 6,  /* configuration outside the kernel's limits  */
  PTN_ERR_TIMEOUT = 7       /* a bounded device-side wait ran out         */
};

#define PTN_MAX_MODES 8

/* A group of tensor modes that a contraction treats as one GEMM index.
 * n modes, row-major (mode 0 slowest); stride_x[i] is the element stride of
 * mode i inside operand x. */
typedef struct {
  int32_t n;
  int32_t pad_;
  int64_t dim[PTN_MAX_MODES];
  int64_t stride_a[PTN_MAX_MODES];
  int64_t stride_b[PTN_MAX_MODES];
  int64_t stride_c[PTN_MAX_MODES];
} ptn_modes;

/* C[m, n] = alpha * sum_k opA(A)[m, k] * opB(B)[k, n] + beta * C[m, n]
 * with m, n, k each a multi-mode index (ptn_modes). For the M group the
 * strides used are stride_a (A) and stride_c (C); for N: stride_b, stride_c;
 * for K: stride_a, stride_b. opX = conjugate when conj_x != 0.
 * This is np.tensordot without the transposes: the strides address the legs
 * in place, and C may be written in any leg order. Outputs of at most 38
 * 64 x 64 tiles with K >= 2048 split K over several CTAs that add into C with
 * atomics (C first scaled by beta), so their rounding can vary between runs;
 * C must not overlap A or B. */
typedef struct {
  const void* A;
  const void* B;
  void* C;
  double alpha_re, alpha_im;
  double beta_re, beta_im;
  int32_t conj_a, conj_b;
  ptn_modes m, n, k;
} ptn_contract_desc;

/* Complex128 tensor contraction in FP64 (plain path).
 * Replaces np.tensordot inside contract_ket_ham_with_envs
 * (contractions/state_operator_contraction.py:227-273), contract_any / contract_leaf /
 * contract_subtrees_using_dictionary (:407-694), contract_bond_tensor (:984-1040)
 * and contract_nodes (contractions/node_contraction.py:62-86). */
int ptn_zcontract(const ptn_contract_desc* d, void* stream);

/* The K split ptn_zcontract uses for an output of `tiles` 64 x 64 tiles and a
 * K range of K: returns the number of splits and sets *k_chunk (K indices per
 * split). Host-only arithmetic. No counterpart in the reference. */
int64_t ptn_zcontract_splits(int64_t tiles, int64_t K, int64_t* k_chunk);

/* ---- Krylov (Lanczos/Arnoldi) vector kernels, complex128 -------------------
 * Replace the np.vdot / np.linalg.norm / axpy loop of krylov_exp_action
 * (time_evolution/time_evolution.py:721-821). Vectors q_i are rows of a
 * matrix Q with leading dimension ldq (elements). partial buffers are
 * device scratch of at least ptn_krylov_partials(n) * (nq + 1) complex128. */
int64_t ptn_krylov_partials(int64_t n);

/* h[i] (+)= sum_x conj(Q[i, x]) w[x] for i < nq; h is device complex128[nq].
 * accumulate != 0 adds to h instead of overwriting. */
int ptn_zdot_multi(const void* Q, int64_t ldq, int32_t nq, const void* w, int64_t n,
                   void* h, int32_t accumulate, void* partial, void* stream);

/* w[x] -= sum_i h[i] * Q[i, x]. */
int ptn_zaxpy_multi(const void* Q, int64_t ldq, int32_t nq, const void* h,
                    void* w, int64_t n, void* stream);

/* out_norm[0] = ||w||_2 (double, device). */
int ptn_dznrm2(const void* w, int64_t n, void* out_norm, void* partial, void* stream);

/* y[x] = w[x] * (1 / scale[0]) with scale a device double. */
int ptn_zscal_inv(const void* w, const double* scale, void* y, int64_t n, void* stream);

/* y[x] = w[x] * (num[0] / den[0]) with num, den device doubles (den = 0: copy).
 * Restores the FP64 norm of a tensor after a reduced-precision contraction that
 * must preserve it (the orthogonality centre after an R absorption). No
 * counterpart in the reference, whose contractions run in FP64. */
int ptn_zscal_ratio(const void* w, const double* num, const double* den, void* y, int64_t n, void* stream);

/* out[x] = sum_i c[i] * Q[i, x], c device complex128[nq]. */
int ptn_zcombine(const void* Q, int64_t ldq, int32_t nq, const void* c,
                 void* out, int64_t n, void* stream);

/* ---- Householder QR (LAPACK zgeqrf/zungqr conventions) ----------------------
 * Replaces np.linalg.qr inside tensor_qr_decomposition(mode=KEEP)
 * (util/tensor_splitting.py:60-107). The m x k matrix lives inside a tensor:
 * element (i, c) is at A[rowoff[i] + c * colstride]; rowoff (device int64[m])
 * encodes the reference's row order. On return A holds Q (KEEP: columns past
 * min(m, k) are zero) and R (device complex128[k * k], row-major, rows past
 * min(m, k) zero) holds R. work: device scratch of ptn_zqr_work_bytes(m, k). */
int64_t ptn_zqr_work_bytes(int64_t m, int64_t k);
int ptn_zqr_keep(void* A, const int64_t* rowoff, int64_t m, int64_t k, int64_t colstride,
                 void* R, void* work, void* stream);

/* How ptn_zqr_keep runs an m x k problem on the current device: 1 = one
 * cooperative launch (m <= 2048 and the columns fit in shared memory; each
 * reflector is handed from CTA to CTA through a flag, no launch per step),
 * 0 = a launch sequence per Householder step. Both give the same bits. A
 * caller that records launch sequences into CUDA graphs uses this to record
 * only the sequences. No counterpart in the reference. */
int ptn_zqr_path(int64_t m, int64_t k);

/* ptn_zqr_keep, always as the launch sequence (path 0): the same result, for
 * callers that record the launches into a CUDA graph or compare the paths. */
int ptn_zqr_keep_steps(void* A, const int64_t* rowoff, int64_t m, int64_t k, int64_t colstride,
                       void* R, void* work, void* stream);

/* Same result as ptn_zqr_keep on the m x k matrix when its rows m_used..m-1
 * (in rowoff order) are exactly zero: the factorisation runs on the first
 * m_used rows with the kernel sequence of the m-row problem (so the same
 * rounding), and the steps that would meet a zero column are written directly
 * (R rows zero, Q column j = e_j for m_used <= j < min(m, k)). Replaces the
 * same np.linalg.qr call as ptn_zqr_keep; the zero rows are the padded bond
 * indices a KEEP split leaves behind, so near-leaf splits of a padded or
 * low-rank state skip most of their Householder steps. */
int ptn_zqr_keep_rows(void* A, const int64_t* rowoff, int64_t m, int64_t m_used, int64_t k, int64_t colstride,
                      void* R, void* work, void* stream);

/* out[0] (device int64) = 1 + the largest row index i (in rowoff order) with a
 * nonzero entry of the m x k matrix, 0 for a zero matrix: the m_used that
 * ptn_zqr_keep_rows may be given. No counterpart in the reference. */
int ptn_znonzero_rows(const void* A, const int64_t* rowoff, int64_t m, int64_t k, int64_t colstride,
                      int64_t* out, void* stream);

/* ---- CholeskyQR2 factors (mixed-precision QR split) ---------------------------
 * The mixed-precision path splits tall full-rank site matrices (the QR of
 * tensor_qr_decomposition, util/tensor_splitting.py:60-107) by CholeskyQR2:
 * Gram matrices and products with R^{-1} on the tensor cores, and these k x k
 * steps on the device, so no host round trip sits between them.
 *
 * G (k x k, row-major, leading dimension ldg, Hermitian up to rounding; its
 * Hermitian part is used) = R^H R with R upper triangular: writes R and R^{-1}
 * (k x k row-major, zero below the diagonal). Computed in FP32 on one CTA.
 * status (device int32) is set to PTN_ERR_NOCONVERGE when a pivot is not
 * positive or the smallest diagonal entry of R is not above pivot_ratio times
 * the largest (the matrix is not of full numerical rank; the caller falls back
 * to Householder). series != 0: when ||G - I||_F <= series_tol the first-order
 * factor R = I + U, R^{-1} = I - U (U = strict upper part of G - I plus half
 * its diagonal) is written instead (second pass of CholeskyQR2, whose Gram
 * matrix is the identity up to the first pass's rounding). work:
 * ptn_zchol_work_bytes(k) bytes (16-byte aligned); k <= ptn_zchol_max_k(). */
int64_t ptn_zchol_work_bytes(int64_t k);
int64_t ptn_zchol_max_k(void);
int ptn_zchol_upper(const void* G, int64_t ldg, int64_t k, void* R, void* Rinv, double pivot_ratio,
                    int32_t series, double series_tol, int32_t* status, void* work, void* stream);

/* C = A B for upper-triangular k x k row-major A, B (C must not alias them),
 * in FP64: X = R1^{-1} R2^{-1} and R2 R1 of CholeskyQR2. */
int ptn_ztri_mul_upper(const void* A, const void* B, void* C, int64_t k, void* stream);

/* R = R0 (2I - X R0) in FP64 for upper-triangular k x k X, R0 (one Newton step
 * toward X^{-1}; work: k x k complex128). CholeskyQR2 writes Q = A X and
 * returns this R, so that Q R reproduces A to FP64 rounding whatever the
 * FP32 error of the factors. No argument may alias another. */
int ptn_ztri_inv_newton(const void* X, const void* R0, void* R, void* work, int64_t k, void* stream);

/* ---- Mixed precision (tcgen05 tensor cores, BF16x3, FP32 accumulation) -------
 * C[m, n] = sum_k A[m, k] * B[n, k] over complex numbers; A and B are given as
 * `levels` BF16 pieces (2: ~16-bit mantissa, products i+j<2 = "BF16x3";
 * 3: ~24-bit, products i+j<3 = "BF16x6"). A: 2*levels planes (Re_0, Im_0,
 * Re_1, Im_1, ...), plane p at A + p * a_plane, row m at m * lda (a_plane a
 * multiple of 8, 16-byte aligned base; lda a multiple of 8 unless K <= 32 and
 * N <= 128, which run on a CUDA-core kernel that reads A without TMA, where
 * any lda >= K is taken). Bx: bf16 [levels][3 blocks
 * (-Im, Re, Im)][N][ldb] as written by ptn_expand_b. The result is written
 * through m_out / n_out (dims + stride_c): out_kind 0 = complex128 at C,
 * 1 = BF16 level planes at C with plane stride c_plane. status: device int32,
 * set on a device-side timeout.
 * Replaces the np.tensordot chain of contract_ket_ham_with_envs /
 * contract_any (contractions/state_operator_contraction.py:227-273, 407-694)
 * in the mixed-precision path. */
typedef struct {
  const void* A;
  int64_t lda, a_plane;
  int64_t M, K;
  const void* Bx;
  int64_t ldb, N;
  int32_t out_kind, levels;
  void* C;
  int64_t c_plane;
  ptn_modes m_out, n_out;
  int32_t* status;
  void* partial;            /* split-K scratch (8-byte aligned), or null   */
  int64_t partial_bytes;
} ptn_cgemm_desc;
int ptn_cgemm_bf16x3(const ptn_cgemm_desc* d, void* stream);
int ptn_cgemm_smem_bytes(int32_t levels);

/* Scratch that ptn_cgemm_bf16x3 uses to split the K range of an M x N x K
 * product whose output has too few 128 x 64 tiles to fill the GPU (0 when it
 * does not split). With at least this many bytes at d->partial, the K range
 * is cut into pieces whose FP32 partial sums a second kernel adds in FP64, in
 * a fixed order, before writing the output; with less (or null) the product
 * runs unsplit. No counterpart in the reference. */
int64_t ptn_cgemm_partial_bytes(int64_t M, int64_t N, int64_t K);

/* Gather a complex128 tensor into the split BF16 operand layouts above.
 * rows / cols: source mode groups (dims + stride_a); element (r, c) of the
 * operand is src[off_rows(r) + off_cols(c)], conjugated when conj != 0.
 * ptn_to_planes writes 2*levels planes of [rows][ld] with plane stride `plane`;
 * ptn_expand_b writes [levels][3][rows][ld] (rows = N). */
typedef struct {
  const void* src;
  void* dst;
  int64_t ld, plane;
  int32_t conj, levels;
  ptn_modes rows, cols;
} ptn_convert_desc;
int ptn_to_planes(const ptn_convert_desc* d, void* stream);
int ptn_expand_b(const ptn_convert_desc* d, void* stream);

/* Same as ptn_zqr_keep, but without a caller-provided work buffer. This entry
 * point has no counterpart in the reference. It is meant for callers that
 * cannot allocate device memory when they need a QR -- a host framework bound
 * through a plain C FFI with no CUDA allocator of its own, or code that must
 * not allocate while a stream is being captured. The scratch is a fixed 4 MiB
 * array inside the library (ptn_zqr_noalloc_max_bytes()); every GPU that loads
 * the library holds it until the process exits. Problems whose
 * ptn_zqr_work_bytes(m, k) exceeds it are rejected with PTN_ERR_UNSUPPORTED
 * before anything is launched. The first call on each device looks up the
 * array's device address (with that device current), so make one call on a
 * device before capturing a stream that uses it. The address is cached for the
 * life of the process: after cudaDeviceReset (or anything else that destroys
 * the device's primary context) it is stale, so do not call this entry point
 * on that device again in the same process. All calls share the one
 * array: calls that can overlap on the GPU (different streams, or different
 * host threads) race on it, so serialise them. Nothing in the scratch needs
 * to start at zero; each call writes every entry it later reads. */
int64_t ptn_zqr_noalloc_max_bytes(void);
int ptn_zqr_keep_noalloc(void* A, const int64_t* rowoff, int64_t m, int64_t k, int64_t colstride,
                         void* R, void* stream);

/* Number of kernel launches this library has issued since it was loaded
 * (host-side counter; used to report launches inside a timed region). */
/* ---- Singular value decomposition (FP64, one-sided Jacobi) ------------------
 * Replaces np.linalg.svd inside tensor_svd / truncated_tensor_svd
 * (util/tensor_splitting.py:122-177, 488-527), as called by split_node_svd
 * (core/ttn.py:1476-1497) in the two-site TDVP and TEBD splits. The truncation
 * rule itself (truncate_singular_values, :448-486) needs only S and is applied
 * by the caller. A (m x n, m >= n): element (i, j) at A[i * row_stride +
 * j * col_stride], read only. Outputs: U (m x n, column j at U + j * ldu), S
 * (device double[n], descending), V (n x n, column j at V + j * ldv) with
 * A = U diag(S) V^H; columns of U for zero singular values are zero.
 * work: ptn_zsvd_work_bytes(m, n) bytes of device scratch. status (device
 * int32, caller zeroes it): set to PTN_ERR_NOCONVERGE when the sweep limit is
 * reached, PTN_ERR_TIMEOUT when a bounded grid-barrier wait runs out. */
typedef struct {
  const void* A;
  int64_t m, n;
  int64_t row_stride, col_stride;
  void* U;
  int64_t ldu;
  double* S;
  void* V;
  int64_t ldv;
  void* work;
  int32_t* status;
} ptn_svd_desc;

int64_t ptn_zsvd_work_bytes(int64_t m, int64_t n);
int ptn_zsvd_jacobi(const ptn_svd_desc* d, void* stream);

/* dst[idx] = op(src[idx]) * (scale ? scale[idx_{scale_mode}] : 1) over an
 * n-mode index (mode n-1 fastest), op = conj when conj != 0. The strides
 * address both operands in place: this writes SVD factors straight into a
 * node's leg order (the transposes and np.diag(s) products of
 * contr_truncated_svd_splitting, util/tensor_splitting.py:541-572). */
typedef struct {
  const void* src;
  void* dst;
  int32_t n;
  int32_t conj;
  int64_t dim[PTN_MAX_MODES];
  int64_t stride_src[PTN_MAX_MODES];
  int64_t stride_dst[PTN_MAX_MODES];
  const double* scale;
  int32_t scale_mode;
  int32_t pad_;
} ptn_permute_desc;

int ptn_zpermute(const ptn_permute_desc* d, void* stream);

/* ---- Native executor ----------------------------------------------------------
 * A contraction chain (one matvec, one environment update) as a list of the
 * descriptors above whose operand pointers are filled in at run time from
 * ptrs[]: op.a / op.b / op.c index the table for A / B (Bx) / C of a
 * contraction or GEMM, and src (a) / dst (c) of a conversion (b = -1 when
 * unused). The descriptors stay in host memory and are copied, so one plan can
 * run with different vectors. Replaces the Python loop over np.tensordot calls
 * of contract_ket_ham_with_envs / contract_any
 * (contractions/state_operator_contraction.py:227-273, 407-694) with one call. */
enum { PTN_OP_ZCONTRACT = 0, PTN_OP_CGEMM = 1, PTN_OP_TO_PLANES = 2, PTN_OP_EXPAND_B = 3 };
typedef struct {
  int32_t kind;
  int32_t a, b, c;
  int32_t d;                /* PTN_OP_CGEMM: table index of the split-K scratch, or -1 */
  int32_t pad_;
  const void* desc;
} ptn_exec_op;
int ptn_exec_ops(const ptn_exec_op* ops, int32_t nops, void* const* ptrs, int32_t nptrs, void* stream);

/* One Gram-Schmidt step of krylov_exp_action (time_evolution/time_evolution.py:775-798):
 * norms[0] = |w|, two passes h = Q^H w, w -= Q h (coefficients in h[0:nq] and
 * h[nq:2nq]), norms[1] = |w|, and qnext = w / norms[1] when qnext is not null. */
int ptn_krylov_gs_step(const void* Q, int64_t ldq, int32_t nq, void* w, int64_t n, void* h,
                       void* partial, double* norms, void* qnext, void* stream);

unsigned long long ptn_launch_counter(void);

/* Wait until all work issued on `stream` has finished (cudaStreamSynchronize);
 * PTN_ERR_LAUNCH if an earlier asynchronous launch failed. The drivers call it
 * once per Krylov batch and per QR split to read a few scalars back. */
int ptn_stream_synchronize(void* stream);

/* Scan a complex128 buffer for NaN/Inf; flag (device int32) is set to 1 if found. */
int ptn_check_finite(const void* x, int64_t n, int32_t* flag, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PTN_GB300_H */
