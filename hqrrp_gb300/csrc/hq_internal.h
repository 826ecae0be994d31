/* hq_internal.h -- internal launcher interface between the C host driver
 * (hqrrp_driver.c) and the CUDA kernels (*.cu).  Plain C: no CUDA types beyond
 * cudaStream_t, no torch.  Every launcher enqueues work on `stream` and returns
 * a cudaError_t-compatible int (0 = success) for the launch itself; errors
 * found by the kernels are written to the device error word of the call.
 */
#ifndef HQ_INTERNAL_H
#define HQ_INTERNAL_H

#include <cuda_runtime_api.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Device error codes written by kernels (never collide with cudaError_t
 * values, which the driver reports separately). */
#define HQ_ERR_BARRIER_TIMEOUT 0x4801 /* a grid barrier or flag wait gave up */
#define HQ_ERR_BAD_SHAPE 0x4802       /* a kernel got a shape it cannot take */

/* Limits of the kernels. */
#define HQ_MAX_MY 256    /* nb + pp (rows of the sketch) */
#define HQ_MAX_PANEL 1024 /* columns of one pivoted panel kernel */
#define HQ_WIDE_MAX_ROWS 1024 /* rows of the wide pivoted QR kernel */

typedef struct hq_device_info {
  int device;
  int num_sms;
  size_t smem_optin; /* max dynamic shared memory per CTA */
} hq_device_info;

int hq_query_device(hq_device_info* info);

/* ---- FP64 GEMM: C = alpha * op(A) * op(B) + beta * C (column-major) ---- */
/* ws: scratch for split-K partial sums (ws_elems doubles; may be NULL). */
int hq_dgemm(cudaStream_t stream, const hq_device_info* dev, char transa, char transb, int M,
             int N, int K, double alpha, const double* A, int lda, const double* B, int ldb,
             double beta, double* Cm, int ldc, double* ws, size_t ws_elems);

/* ---- Gaussian sketch: G (rows x cols, ld) ~ N(0,1) from Philox4x32-10 ---- */
int hq_sketch_philox(cudaStream_t stream, int rows, int cols, double* G, int ldg,
                     unsigned long long seed);

/* ---- Pivot selection: b-stage pivoted QR of the mY x N sketch -----------
 * Reads Y (mY x N, ldy); when the columns do not fit in the shared memory of
 * the grid, V (same shape, ldv) is used as a working copy.  Writes the final
 * column permutation as (dst, src) pairs: pairs[2*i], pairs[2*i+1], count in
 * *npairs (zeroed by the launcher). */
int hq_skinny_qrp(cudaStream_t stream, const hq_device_info* dev, int mY, int N, int b,
                  const double* Y, int ldy, double* V, int ldv, int* pairs, int* npairs,
                  double* part, size_t part_elems, unsigned* bar, int* err,
                  unsigned spin_limit, int fp32);
size_t hq_skinny_part_elems(const hq_device_info* dev, int mY);

/* ---- Panel: pivoted (or plain) QR of the mp x nc block P (ldp) ---------
 * In place: R on and above the diagonal, Householder vectors below it.
 * ut != 0: a column whose tail below the diagonal is zero (or empty) gets
 * the UT transform's reflector H = I - 2 e e^T (tau = 2, beta = -alpha)
 * instead of LAPACK's H = I (tau = 0).
 * tau[0..nc), U (mp x nc, ldu) = explicit unit-lower copy of the vectors,
 * perm[k] = source column of final column k. */
int hq_panel_qrp(cudaStream_t stream, const hq_device_info* dev, int mp, int nc, int pivoting,
                 double* P, int ldp, double* tau, double* U, int ldu,
                 int* perm, double* part, size_t part_elems, double* rowbuf, unsigned* bar,
                 int* err, unsigned spin_limit,
                 int sqnorm, int ut);
/* The same, skipped (every CTA returns at once) when *gram_stat == 0: the
 * mixed path's Gram panel (qrp_gram.cu) already factored this panel. */
int hq_panel_qrp_fallback(cudaStream_t stream, const hq_device_info* dev, int mp, int nc,
                          int pivoting, double* P, int ldp, double* tau, double* U, int ldu,
                          int* perm, double* part, size_t part_elems, double* rowbuf,
                          unsigned* bar, int* err, unsigned spin_limit, int sqnorm, int ut,
                          const int* gram_stat);
size_t hq_panel_part_elems(const hq_device_info* dev, int nc);

/* ---- Gram panel (mixed path): the b x b kernels of qrp_gram.cu -----------
 * All matrices column-major, b <= HQ_GRAM_MAX.  Status bits go to *stat. */
#define HQ_GRAM_MAX 128
/* Pass 1: pivoted Cholesky of G (lower triangle read) scaled to unit
 * diagonal, in FP32: perm[k] = source column of position k, R (FP64, upper)
 * with R^T R ~ P^T G P; *stat := 0, or bit with R = I, perm = identity;
 * *alt, *emax := 0. */
int hq_gram_pchol32(cudaStream_t stream, int n, const double* G, int ldg, double* R, int ldr,
                    int* perm, int* stat, int bit, int* alt, unsigned long long* emax);
/* FP64 on a cluster of eight CTAs.  mode 0: Cholesky of the symmetric A
 * (lower triangle read), F := R upper.  mode 1: LU without pivoting of A - D
 * (Householder reconstruction), F := L strictly below the diagonal and U on
 * and above, dsgn := D, tau := -D U_kk.  A bad pivot sets bit in *stat and
 * gives identity factors.  gate (may be NULL): skipped when *gate == 0. */
int hq_cluster_fact(cudaStream_t stream, int n, int mode, const double* A, int lda, double* F,
                    int ldf, double* dsgn, double* tau, int* stat, int bit, const int* gate);
/* Second CholeskyQR pass for G = I + E near the identity (FP64, no
 * sequential factorization): R (= I + X, upper) and Rinv = R^{-1} by a fixed
 * number of fixed-point steps over b x b products; wX, wZ are b x b work
 * matrices (all with leading dimension ld); *emax receives max|E| (as the
 * bits of a double), which sets the number of steps.  Sets *alt when max|E|
 * is too large for the steps to converge (R and Rinv are then left to
 * kernels gated on *alt). */
int hq_nearid_chol(cudaStream_t stream, int n, const double* G, int ldg, double* R, double* Rinv,
                   double* wX, double* wZ, int ld, int* alt, unsigned long long* emax);
/* mode 0: X = A^{-1}; mode 1: X = diag(rs) A B (rs may be NULL); A, B upper.
 * gate (may be NULL): skipped when *gate == 0. */
int hq_tri(cudaStream_t stream, int n, int mode, const double* A, int lda, const double* B,
           int ldb, const double* rs, double* X, int ldx, const int* gate);
/* Two independent such jobs in one launch (mode1 = -1: the first only). */
int hq_tri2(cudaStream_t stream, int n, int mode0, const double* A0, int lda0, const double* B0,
            int ldb0, const double* rs0, double* X0, int ldx0, int mode1, const double* A1,
            int lda1, const double* B1, int ldb1, const double* rs1, double* X1, int ldx1);
/* The same, skipped when gate is not NULL and *gate == 0. */
int hq_tri2g(cudaStream_t stream, int n, int mode0, const double* A0, int lda0, const double* B0,
             int ldb0, const double* rs0, double* X0, int ldx0, int mode1, const double* A1,
             int lda1, const double* B1, int ldb1, const double* rs1, double* X1, int ldx1,
             const int* gate);
/* When *stat == 0: the panel P (mp x n) := R (RH's upper triangle) and the
 * Householder vectors (LU's strict lower part; U's rows >= n), U's top rows
 * := explicit unit-lower V1, tau := tau_in, perm := identity.  count (may be
 * NULL): count[0] += 1 if committed, count[1] += 1 if not. */
int hq_gram_commit(cudaStream_t stream, int mp, int n, double* P, int ldp, double* U, int ldu,
                   const double* RH, int ldr, const double* LU, int ldlu, const double* tau_in,
                   double* tau, int* perm, const int* stat, int* count);
/* Exchange area of the panel kernel for `ctas` CTAs and nc columns, in
 * doubles: [2][ps][ctas] FP64 partials (initial and recomputed norms), then
 * [3][ps][HQ_PANEL_FX_CS] 64-bit words of fixed-point stage sums (four used
 * per column; the stride spreads the columns' atomics over cache lines,
 * which measured 13 ms faster per 16384^2 factorization than packed words);
 * ps = nc rounded up to even (plus 2). */
#define HQ_PANEL_FX_CS 16 /* one 128-byte line per column: fewer atomics per line */
#define HQ_PANEL_PART_ELEMS(ctas, nc) \
  (2 * (size_t)(ctas) * (size_t)(((nc) + 2) & ~1) + \
   3 * (size_t)HQ_PANEL_FX_CS * (size_t)(((nc) + 2) & ~1))

/* ---- Wide pivoted QR: m <= HQ_WIDE_MAX_ROWS rows, any number of columns --
 * dgeqp3's result for an m x n matrix A (lda), in place except for the
 * column order: the final order is written as (dst, src) pairs (at most
 * 2 min(m, n) of them, count in *npairs) for hq_permute_pairs.  phys: n ints;
 * cand: hq_wide_cand_elems(dev) 64-bit words. */
size_t hq_wide_cand_elems(const hq_device_info* dev);
int hq_wide_qrp(cudaStream_t stream, const hq_device_info* dev, int m, int n, double* A, int lda,
                double* tau, int* phys, long long* cand, int* pairs, int* npairs, unsigned* bar,
                int* err, unsigned spin_limit);

/* ---- T factor of a forward columnwise block reflector (DLARFT) -----------
 * Z = U^T U (k x k, ldz) is given; writes T (k x k, ldt), zero below the
 * diagonal. */
int hq_larft_from_gram(cudaStream_t stream, int k, const double* Z, int ldz, const double* tau,
                       double* T, int ldt);

/* ---- Column permutation by (dst, src) pairs -----------------------------
 * For rows 0..rows-1 of X (ldx, ncols columns): X[:, dst] = X_old[:, src] for
 * each pair, via tmp (rows x max_pairs, ldt = rows).  Labels (int, may be
 * NULL) are permuted the same way. */
int hq_permute_pairs(cudaStream_t stream, int rows, double* X, int ldx, int ncols,
                     const int* pairs, const int* npairs, int max_pairs, double* tmp,
                     int* labels, int* label_tmp);

/* Apply a permutation of nc columns given as perm[k] = source column. */
int hq_permute_cols(cudaStream_t stream, int rows, double* X, int ldx, int nc, const int* perm,
                    double* tmp, int* labels, int* label_tmp);

/* ---- Split-BF16 (Ozaki) FP64 products on tcgen05 -------------------------
 * side 0 = M side (128-row tiles), 1 = N side (80-row tiles).  X element
 * (r, k) at X[r*rs + k*ks]; tiles sized by hq_ozk_tile_bytes; exps needs
 * rows rounded up to the tile height.  gemm: mode 0 writes sign * X Y^T to C,
 * mode 1 adds it; C element (r, c) at C[r*crs + c*ccs]; ws (optional) holds
 * split-K slices for mode 0. */
size_t hq_ozk_tile_bytes(int rows, int K, int S, int side);
/* raw (may be NULL): rows_total ints of scratch; when given, the two-pass
 * split of few long rows takes its row maxima with several CTAs per row. */
int hq_ozk_split(cudaStream_t stream, const double* X, long long rs, long long ks, int R, int K,
                 int S, int side, void* tiles, int* exps, int* raw);
/* Rows rounded up to the tile height of a side. */
int hq_ozk_split_rows(int R, int side);
/* raw[r] := largest FP64 exponent field of row r (r < R; 0 up to rows_total),
 * several CTAs per row: the row maxima hq_ozk_split_raw takes, computed once
 * when both operands of a product are the same matrix. */
int hq_ozk_rowmax_raw(cudaStream_t stream, const double* X, long long rs, long long ks, int R,
                      int K, int rows_total, int* raw);
/* The same split (S = 7) from each row's largest FP64 exponent field raw[r]
 * (rows < R), computed elsewhere: one streaming pass. */
int hq_ozk_split_raw(cudaStream_t stream, const double* X, long long rs, long long ks, int R,
                     int K, int S, int side, void* tiles, int* exps, const int* raw);
int hq_ozk_gemm(cudaStream_t stream, const hq_device_info* dev, int M, int N, int K, int S,
                const void* Atiles, const int* ea, const void* Btiles, const int* eb, int mode,
                double sign, double* C, long long crs, long long ccs, double* ws,
                size_t ws_elems, int* err, unsigned spin_limit);
/* mode 0 product whose N side is FP64: Y element (n, k) at Y[n*yld + k],
 * raw[n] its row's largest exponent field; digits are cut on the fly (S = 7).
 * cudaErrorNotSupported when Y's alignment does not allow tensor-map loads. */
int hq_ozk_gemm_c64(cudaStream_t stream, const hq_device_info* dev, int M, int N, int K,
                    const void* Atiles, const int* ea, const double* Y, long long yld,
                    const int* raw, double sign, double* C, long long crs, long long ccs,
                    double* ws, size_t ws_elems, int* err, unsigned spin_limit);
/* K <= 256: persistent kernel with double-buffered TMEM; the N side must be
 * split with side 2 (32-row tiles).  Mode 1 with colexp: colexp[c] (zeroed
 * before) receives the largest exponent field of the new C(r, c) over rows
 * r >= row_lo. */
int hq_ozk_short_ok(int K);
int hq_ozk_gemm_short(cudaStream_t stream, const hq_device_info* dev, int M, int N, int K, int S,
                      const void* Atiles, const int* ea, const void* Btiles, const int* eb,
                      int mode, double sign, double* C, long long crs, long long ccs,
                      int* colexp, int row_lo, int* err, unsigned spin_limit);

/* ---- Batched pivoted QR (one persistent launch, device work queue) -------
 * d_work: hq_qrp_batched_workspace(batch) bytes; ints [32..32+batch) hold the
 * schedule (matrix indices, largest first), int 0 the queue head. */
size_t hq_qrp_batched_workspace(int batch);
int hq_qrp_batched(cudaStream_t stream, const hq_device_info* dev, int batch, const int* d_m,
                   const int* d_n, double* const* d_A, const int* d_lda, int* const* d_jpvt,
                   double* const* d_tau, int* d_info, void* d_work, int max_n, int threads,
                   int stage_kb, int ctas_per_sm);

/* ---- Adjoint helpers (adjoint.cu) ---- */
int hq_unit_lower(cudaStream_t st, int rows, int b, const double* F, int ldf, double* U, int ldu);
int hq_eye(cudaStream_t st, int rows, int k, double* E, int lde);
int hq_copyltu(cudaStream_t st, int k, double* X, int ldx, double sign);
int hq_trsm_rt(cudaStream_t st, int rows, int k, const double* R, int ldr, double* Y, int ldy);
int hq_scatter_cols(cudaStream_t st, int rows, int ncols, const double* src, int lds,
                    const int* labels, double* dst, int ldd, int accumulate);
int hq_rk_unpermute(cudaStream_t st, int k, int n, const double* F, int ldf, const int* labels,
                    double* M, int ldm);

/* ---- Launch accounting: every launcher adds the kernels it enqueued ---- */
void hq_count_launches(int k);
unsigned long long hq_launches(void);

/* ---- Host driver services for launchers that are entry points ---------- */
void hq_set_error(const char* fmt, ...);
void hq_clear_error(void);
unsigned hq_spin_limit(void);

/* ---- Small kernels ---- */
int hq_fill_iota(cudaStream_t stream, int* x, int n, int base);
/* dst += alpha * src; A[i, i] = v; Z += L + L^T + I (L: strictly lower top
 * b x b block of U with its unit diagonal removed). */
int hq_add_matrix(cudaStream_t st, int rows, int cols, double alpha, const double* src, int lds,
                  double* dst, int ldd);
int hq_set_diag(cudaStream_t st, int n, double* A, int lda, double v);
int hq_gram_unit_fix(cudaStream_t st, int b, const double* Up, int ldu, double* Z, int ldz);
int hq_copy_matrix(cudaStream_t stream, int rows, int cols, const double* src, int lds,
                   double* dst, int ldd);

/* Programmatic dependent launch of this library's kernels: on unless
 * HQRRP_GB300_PDL=0 (read by each call's workspace setup). */
void hq_set_pdl(int on);
int hq_pdl(void);
/* Zero two word arrays (n1, n2 32-bit words; p2 may be NULL) in one launch
 * that keeps the programmatic-launch chain (a memset node breaks it). */
int hq_zero_words(cudaStream_t stream, void* p1, size_t n1, void* p2, size_t n2);

#ifdef __cplusplus
}
#endif
#endif
