/* hqrrp_gb300.h -- C ABI of libhqrrp_gb300.so, the GB300 (sm_103a) HQRRP.
 *
 * Householder QR with randomized column pivoting of Martinsson,
 * Quintana-Orti, Heavner and van de Geijn.  The first two entry points are
 * drop-in replacements, with identical signatures and argument meaning, for
 * the reference's C entry points:
 *
 *   lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.h:1-2   dgeqp4
 *   lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.h:4-6   NoFLA_HQRRP_WY_blk_var4
 *
 * All matrices are column-major FP64.  The host-pointer entry points copy A to
 * the GPU, factor it there and copy A, jpvt and tau back; every arithmetic
 * step runs in this library's CUDA kernels (no CPU LAPACK).  When A is in
 * page-locked host memory (cudaHostAlloc / cudaHostRegister), each block's
 * finished columns are copied back while later blocks are factored, so the
 * copy costs little beyond the factorization; pageable A is copied back once
 * at the end.  When the CUDA device or a kernel fails they report it (info /
 * return code, message from hqrrp_gb300_last_error()) instead of falling back
 * to the CPU; a page-locked A may then hold partial results.
 */
#ifndef HQRRP_GB300_H
#define HQRRP_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Drop-in entry points ------------------------------------------------ */

/* dgeqp3-plug-compatible pivoted QR.  Replaces dgeqp4 of
 * lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:127-300.
 *   jpvt in: jpvt[j] != 0 marks a fixed (leading) column; out: 1-based
 *   column permutation.  tau: min(m,n) reflector scalars.  work/lwork:
 *   lwork == -1 is a query (work[0] = 2n + (n+1)*32); otherwise lwork must be
 *   >= 3n+1 and work[0] returns the workspace LAPACK would report.  work is
 *   not used as scratch.
 *   info: 0 ok; -1/-2/-4/-8 as LAPACK (message names DGEQP3, like the
 *   reference); > 1000 a device error (info - 1000 is the error code, see
 *   hqrrp_gb300_last_error()).
 * min(m,n) < 250 follows dgeqpf, < 1000 dgeqp3 (both on the GPU here), larger
 * matrices HQRRP with nb = 64, pp = 10, panel pivoting on. */
void dgeqp4(int* m, int* n, double* A, int* lda, int* jpvt, double* tau, double* work,
            int* lwork, int* info);

/* Blocked HQRRP.  Replaces NoFLA_HQRRP_WY_blk_var4 of
 * lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:303-571.
 *   jpvt is carried: its incoming values are permuted like the columns.
 *   nb_alg: block size, pp: oversampling (nb_alg + pp <= 256),
 *   panel_pivoting: 1 = pivoted panel QR, 0 = unpivoted.
 * Returns 0 on success (always 0 in the reference).  Invalid m, n or lda
 * print the reference's messages and return 0 without touching A.  A device
 * error returns its positive code.  The sketch is drawn on the GPU by Philox
 * (seed hqrrp_gb300_set_seed, default 12), not by libc rand(); the reference's
 * srand(12) side effect on the caller's rand() state does not happen. */
int NoFLA_HQRRP_WY_blk_var4(int m_A, int n_A, double* buff_A, int ldim_A, int* buff_jpvt,
                            double* buff_tau, int nb_alg, int pp, int panel_pivoting);

/* ---- Extensions (no reference counterpart unless stated) ----------------- */

/* Precision of the block updates: 0 = plain FP64 (default), 1 = mixed: the
 * sketch Y = G A from two-digit BF16 operands; the trailing update (dlarfb:
 * U^T C, T^T W1, C -= U W2), the Gram matrix U^T U and the sketch downdate as
 * split-BF16 products on the tensor cores (seven digits per operand, exact
 * FP32 accumulation per level, recombined in FP64); pivot selection on the
 * sketch applies its reflectors in FP32 to a power-of-two-scaled copy of each
 * column.  The panel, its reflectors and tau, all column norms and their
 * downdating, and T stay FP64.  HQRRP_GB300_PRECISION=mixed in the
 * environment selects 1 at first use.  Returns the previous value, or -1 for
 * an unknown mode. */
int hqrrp_gb300_set_precision(int mode);

/* Block size of the HQRRP call inside dgeqp4 (and dgeqp4_device), with
 * oversampling 10.  The default is 128: the reference's 64
 * (NoFLA_HQRRP_WY_blk_var4.c:255-264, its "default values") is a CPU choice,
 * and on this GPU 128 runs the 16384^2 factorization about 1.5x faster.
 * With nb = 64 the block update's products have only 64 of their 128-row
 * tiles' rows, and the rank-64 trailing update is bound by its FP64 epilogue
 * instead of its tensor-core work.  The block size sets the block structure
 * of the randomized pivoting, not the interface or the output's form.
 * dgeqp4 with an explicit sketch (hqrrp_gb300_dgeqp4_sketch) always uses 64,
 * the reference's block structure.  Returns the previous value, or -1 if nb
 * is outside 1..246. */
int hqrrp_gb300_set_dgeqp4_block(int nb);

/* Seed of the device Philox sketch used when no sketch is supplied. */
void hqrrp_gb300_set_seed(unsigned long long seed);

/* Iteration cap of every spin-wait in the cooperative kernels (0 = default).
 * A wait that reaches it ends the kernel with an error code instead of
 * hanging; lowering it is how the timeout path is exercised. */
void hqrrp_gb300_set_spin_limit(unsigned limit);

/* NoFLA_HQRRP_WY_blk_var4 with an explicit host sketch G ((nb+pp) x m,
 * leading dimension ldg) used in place of the drawn one; with the
 * reference's own sketch this reproduces the reference run exactly up to
 * rounding (the oracle feeds it the reference's rand()-based G). */
int hqrrp_gb300_hqrrp_sketch(int m, int n, double* A, int lda, int* jpvt, double* tau,
                             int nb, int pp, int panel_pivoting, const double* G, int ldg);

/* dgeqp4 with an explicit host sketch for its HQRRP branch (min(m,n) >= 1000):
 * G is 74 x m ((64 + 10) rows, leading dimension ldg >= 74) and its first
 * m - nf columns (nf = number of fixed columns, at most m) replace the sketch
 * the reference draws inside NoFLA_HQRRP_WY_blk_var4 for the free block
 * (lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:257-265).  Everything
 * else is dgeqp4 above; the small-matrix branches do not read G.  With the
 * reference's own sketch of the free block this reproduces the reference's
 * dgeqp4 up to rounding.  info = 1003 if G is NULL or ldg < 74. */
void hqrrp_gb300_dgeqp4_sketch(int* m, int* n, double* A, int* lda, int* jpvt, double* tau,
                               double* work, int* lwork, int* info, const double* G, int ldg);

/* Device-pointer HQRRP on `stream` (a cudaStream_t, NULL = legacy default).
 * dA (ldda >= m), d_jpvt (n ints, carried), d_tau (min(m,n)).  dG: optional
 * device sketch ((nb+pp) x m, lddg); NULL draws Philox(seed).  Blocks until
 * the factorization is complete.  Returns 0 or a device error code. */
int hqrrp_gb300_hqrrp_device(int m, int n, double* dA, int ldda, int* d_jpvt, double* d_tau,
                             int nb, int pp, int panel_pivoting, const double* dG, int lddg,
                             unsigned long long seed, void* stream);

/* The Gaussian sketch the factorization draws when none is supplied: dG
 * (rows x cols, column-major, ldg >= rows) on the device, element e = c*rows + r
 * from Philox4x32-10 (Salmon et al., SC'11) of counter e / 2 under key =
 * seed, its 128 bits turned into two N(0,1) values by Box-Muller (even e the
 * cosine branch, odd e the sine branch).  Replaces the reference's polar
 * method over libc rand() (lapack_compatible_sources/
 * NoFLA_HQRRP_WY_blk_var4.c:575-614) as a counter-based generator.  Blocks
 * until done; returns 0 or an error code. */
int hqrrp_gb300_sketch_device(int rows, int cols, double* dG, int ldg, unsigned long long seed,
                              void* stream);

/* Device-pointer dgeqp4 (same semantics as dgeqp4; jpvt/tau on the device,
 * no work array).  Returns info. */
int hqrrp_gb300_dgeqp4_device(int m, int n, double* dA, int ldda, int* d_jpvt, double* d_tau,
                              void* stream);

/* Pivoted QR (LAPACK dgeqp3 results for free columns: R and reflectors in
 * dA, tau, 1-based jpvt) of an m x n device matrix with n <= 256, that
 * allocates NO device memory.  No counterpart in the reference.  For callers
 * that cannot allocate at this point: a process that has given all device
 * memory to its own arena, or a loop that cannot afford the device
 * synchronisation of cudaMalloc/cudaFree or their failure under memory
 * pressure.  Its scratch is a fixed 747 KiB __device__ array held by every GPU
 * that loads the library until exit, shared by all calls: calls that overlap
 * on the GPU race and must be serialised by the caller.  The first call on a
 * device does a one-time set-up (scratch address lookup) and should come
 * before any stream capture.  Returns 0, 3 for n > 256 or invalid sizes (see
 * hqrrp_gb300_last_error()), 2 if the kernel reported an error, 1 for a CUDA
 * error.  Blocks until done. */
int hqrrp_gb300_qrp_noalloc(int m, int n, double* dA, int ldda, int* d_jpvt, double* d_tau,
                            void* stream);

/* ---- The UT-transform variant (the reference's second implementation) --
 * Replaces FLA_HQRRP_UT_blk_var2(FLA_Obj A, FLA_Obj p, FLA_Obj s, int nb_alg,
 * int pp, int panel_pivoting) of libflame_sources/FLA_HQRRP_UT_blk_var2.h:3-4
 * (body FLA_HQRRP_UT_blk_var2.c:124-401).  libflame's FLA_Obj is not part of
 * this library; hqrrp_gb300_obj carries the fields of a view the variant
 * reads through FLA_Obj_datatype, _length, _width, _col_stride and
 * _buffer_at_view.  A: m x n double; p: n ints (an n x 1 view, or 1 x n with
 * col_stride as the element stride), carried like jpvt; s: min(m, n)
 * doubles, the UT scalars tau_UT of H_k = I - u_k u_k^T / tau_UT (tau_UT =
 * 1/tau of LAPACK's form; a reflector whose tail below the diagonal is zero
 * -- always the last one when m <= n -- is H = I - 2 e e^T with tau_UT = 1/2
 * and that row negated, where LAPACK's convention gives H = I).  Same
 * pivots, R and reflectors as NoFLA_HQRRP_WY_blk_var4 otherwise (same
 * algorithm, UT instead of compact-WY block transforms), on the GPU, with the
 * device Philox sketch; _sketch takes an explicit host sketch G ((nb + pp) x
 * m, ldg) instead.  Returns 0, or a positive error code (3 for a bad object
 * or shape) where libflame would abort. */
#define HQRRP_GB300_DOUBLE 1
#define HQRRP_GB300_INT 2
typedef struct hqrrp_gb300_obj {
  int datatype;   /* HQRRP_GB300_DOUBLE or HQRRP_GB300_INT */
  int m, n;       /* length (rows) and width (columns) of the view */
  int col_stride; /* distance between columns, in elements */
  void* buffer;   /* address of element (0, 0) of the view */
} hqrrp_gb300_obj;
int hqrrp_gb300_ut_blk_var2(hqrrp_gb300_obj A, hqrrp_gb300_obj p, hqrrp_gb300_obj s, int nb_alg,
                            int pp, int panel_pivoting);
int hqrrp_gb300_ut_blk_var2_sketch(hqrrp_gb300_obj A, hqrrp_gb300_obj p, hqrrp_gb300_obj s,
                                   int nb_alg, int pp, int panel_pivoting, const double* G,
                                   int ldg);

/* C = alpha * op(A) op(B) + beta * C in FP64 emulated on the BF16 tensor
 * cores: each operand row (of op(A)) / column (of op(B)) is scaled by a power
 * of two and cut into `slices` 8-bit digits (6 gives about 46 correct bits
 * relative to the row/column maxima); digit products accumulate exactly in
 * FP32 and are recombined in FP64.  Device pointers, column-major; alpha must
 * be +-1 and beta 0 or 1.  No counterpart in the reference: it is the
 * product kernel of the mixed-precision path, exposed for direct use. */
int hqrrp_gb300_ozaki_dgemm(char transa, char transb, int m, int n, int k, double alpha,
                            const double* dA, int lda, const double* dB, int ldb, double beta,
                            double* dC, int ldc, int slices, void* stream);

/* ---- Batched small pivoted QRs (no reference counterpart as an API; the
 * per-matrix result is that of the reference dgeqp4's small-matrix branch,
 * LAPACK dgeqpf/dgeqp3 with all columns free: ...var4.c:189-199) ---------
 * plan: host arrays of the batch's sizes; writes a largest-first schedule
 * into the device workspace (hqrrp_gb300_qrp_batched_workspace bytes) and,
 * with autotune != 0, times every launch shape on scratch matrices of these
 * sizes once per batch signature.  Synchronous; returns the launch-shape id
 * (>= 0) or minus an error code.
 * run: all arrays on the device (d_A[i] column-major m[i] x n[i] with leading
 * dimension d_lda[i], d_jpvt[i] n[i] ints, d_tau[i] min(m,n) doubles, d_info
 * may be NULL); max_n bounds every n[i].  One persistent launch with a device
 * work queue; asynchronous on `stream`, allocates nothing and does not
 * synchronise, so it can be captured in a CUDA graph.  Returns 0 or an error
 * code for the launch itself; d_info[i] != 0 flags a matrix it could not take. */
size_t hqrrp_gb300_qrp_batched_workspace(int batch);
int hqrrp_gb300_qrp_batched_plan(int batch, const int* h_m, const int* h_n, void* d_work,
                                 size_t work_bytes, int autotune, void* stream);
int hqrrp_gb300_qrp_batched_run(int batch, const int* d_m, const int* d_n, double* const* d_A,
                                const int* d_lda, int* const* d_jpvt, double* const* d_tau,
                                int* d_info, int max_n, int cfg, void* d_work, void* stream);
/* Launch shape of a plan id: threads per CTA, shared-memory staging budget
 * (KB), CTAs per SM.  Returns the number of shapes, or -1. */
int hqrrp_gb300_qrp_batched_config(int cfg, int* threads, int* stage_kb, int* ctas_per_sm);

/* ---- Truncated factorization and its adjoint (no reference counterpart) --
 * truncated: HQRRP of the device matrix dA stopped after k columns (its first
 * k pivots, rows and reflectors are those of the full run); d_jpvt must hold
 * 1..n on entry for the other entries below.
 * lowrank: dOut (m x n) = Q_k R_k P^T from a truncated factorization dF.
 * form_q: dQ (m x k) = the first k columns of Q, the reflector blocks of nb
 * columns rebuilt from dF (T recomputed per block, nothing stored).
 * adjoint: dG = dL/dA of L = <W, Q_k R_k P^T> with the pivots held fixed
 * (dA the original matrix, dF/d_jpvt/d_tau its truncated factorization);
 * the reflector blocks are recomputed, not stored.  All device pointers,
 * column-major; each returns 0 or an error code and blocks until done. */
int hqrrp_gb300_hqrrp_truncated_device(int m, int n, int k, double* dA, int ldda, int* d_jpvt,
                                       double* d_tau, int nb, int pp, unsigned long long seed,
                                       void* stream);
int hqrrp_gb300_lowrank_device(int m, int n, int k, const double* dF, int lddf, const int* d_jpvt,
                               const double* d_tau, double* dOut, int lddo, int nb, void* stream);
int hqrrp_gb300_form_q_device(int m, int k, const double* dF, int lddf, const double* d_tau,
                              double* dQ, int lddq, int nb, void* stream);
/* apply_q: dC (m x nc) := Q dC (trans 'N') or Q^T dC (trans 'T'), Q the
 * product of the first k reflectors of a factorization dF (LAPACK dormqr
 * with side 'L'); the reflector blocks of nb columns are rebuilt from dF. */
int hqrrp_gb300_apply_q_device(char trans, int m, int nc, int k, const double* dF, int lddf,
                               const double* d_tau, double* dC, int lddc, int nb, void* stream);
int hqrrp_gb300_hqrrp_adjoint_device(int m, int n, int k, const double* dA, int ldda,
                                     const double* dF, int lddf, const int* d_jpvt,
                                     const double* d_tau, const double* dW, int lddw, double* dG,
                                     int lddg, int nb, void* stream);

/* Per-phase profiler (off by default).  While enabled, every call records
 * CUDA events at phase boundaries on its stream; read returns the summed
 * milliseconds and flops per phase and resets them.  Phases: 0 sketch +
 * Y = G A, 1 pivot selection (sketch QRP + gathers), 2 panel QR + T, 3
 * trailing update (dlarfb), 4 sketch downdate, 5 other, and in mixed
 * precision 6 the tensor-core digit products (BF16 flops) and 7 the digit
 * splits (the FP64 parts of 3 and 4 stay in 3 and 4).  The reference's
 * libflame variant keeps the same buckets under #ifdef PROFILE
 * (libflame_sources/FLA_HQRRP_UT_blk_var2.c:165-167, :289-398).  Returns the
 * number of phases. */
void hqrrp_gb300_profile_enable(int on);
int hqrrp_gb300_profile_read(double* ms, double* flops, int n);
/* Intervals recorded per phase since the last call (for the tensor phase:
 * one per digit-product launch); resets them. */
int hqrrp_gb300_profile_counts(int* counts, int n);

/* Number of kernels this library has launched in this process. */
unsigned long long hqrrp_gb300_launch_count(void);

/* Number of device allocations this library has made from its memory pools
 * in this process (every entry point except hqrrp_gb300_qrp_noalloc draws its
 * workspace from a pool).  Setting HQRRP_GB300_FAIL_ALLOC=k in the
 * environment makes the k-th allocation of every later call fail as if the
 * device were out of memory (return code 4, dgeqp4 info 1004): host-side
 * fault injection for testing callers' error paths. */
unsigned long long hqrrp_gb300_pool_alloc_count(void);

/* Mixed precision's panels: of the last call that factored panels in mixed
 * precision, how many the Gram panel committed (Gram matrix, pivoted
 * CholeskyQR2, Householder reconstruction) and how many it passed on to the
 * column-by-column pivoted panel (a Cholesky or LU pivot that showed the
 * panel too ill-conditioned for it).  Synchronizes the device.  Setting
 * HQRRP_GB300_GRAM_PANEL=0 in the environment turns the Gram panel off. */
int hqrrp_gb300_gram_panel_counts(int* committed, int* fallback);

/* Message of the last failure on the calling thread ("" if none). */
const char* hqrrp_gb300_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
