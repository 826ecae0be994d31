/*
 * hqrrp_oracle.c -- CPU restatement of the reference HQRRP algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA library is compared
 * against.  It is loaded only by tests/, by __graft_entry__.smoke() and by the
 * CPU-baseline / reference arm of bench.py.  The product library
 * (libhqrrp_gb300.so) never links, loads or calls anything in this directory.
 *
 * What it restates (file:line in the reference project):
 *   lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c
 *     dgeqp4 front end ............................ :127-300
 *     NoFLA_HQRRP_WY_blk_var4 blocked driver ...... :303-571
 *     Gaussian sketch (polar method over rand()) .. :575-614
 *     Downdate_Y .................................. :617-708
 *     Apply_Q_WY_lhfc / rnfc (dlarfb wrappers) .... :711-771
 *     QRPmod_WY_unb_var4 (unblocked QRP) .......... :774-886
 *     compute_norms / Drmac downdate .............. :889-986
 *     pivot_G_B_C (column swap, norm copy) ........ :990-1036
 *
 * The arithmetic primitives (dgemm, dlarfb, dlarfg, ...) are the same LAPACK /
 * BLAS routines the reference calls, resolved at run time with dlopen from an
 * LP64 OpenBLAS (scipy's bundled libscipy_openblas, whose symbols carry a
 * "scipy_" prefix, or any unprefixed LP64 LAPACK).  The calls are issued in the
 * reference's order with the reference's arguments, so on the same library the
 * outputs are bit-identical to the compiled reference (checked by the golden
 * fixtures under tests/golden/).
 *
 * Deliberate differences, all on invalid input only:
 *   - NoFLA_HQRRP_WY_blk_var4 with m<0, n<0 or lda<max(1,m) prints the
 *     reference's messages and then returns 0 without touching A (the
 *     reference carries on into undefined behaviour).
 *   - dgeqp4 passes a real string to ilaenv's OPTS argument (the reference
 *     passes the character ' ' through a K&R prototype).
 */
#include <dlfcn.h>
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* LAPACK / BLAS table (Fortran calling convention, LP64, hidden lengths).   */

typedef size_t flen;
typedef void (*fn_dgemm)(const char*, const char*, const int*, const int*, const int*,
                         const double*, const double*, const int*, const double*,
                         const int*, const double*, double*, const int*, flen, flen);
typedef void (*fn_dlacpy)(const char*, const int*, const int*, const double*, const int*,
                          double*, const int*, flen);
typedef void (*fn_dlarfg)(const int*, double*, double*, const int*, double*);
typedef void (*fn_dlarf)(const char*, const int*, const int*, const double*, const int*,
                         const double*, double*, const int*, double*, flen);
typedef void (*fn_dlarft)(const char*, const char*, const int*, const int*, const double*,
                          const int*, const double*, double*, const int*, flen, flen);
typedef void (*fn_dlarfb)(const char*, const char*, const char*, const char*, const int*,
                          const int*, const int*, const double*, const int*, const double*,
                          const int*, double*, const int*, double*, const int*, flen, flen,
                          flen, flen);
typedef void (*fn_dtrmm)(const char*, const char*, const char*, const char*, const int*,
                         const int*, const double*, const double*, const int*, double*,
                         const int*, flen, flen, flen, flen);
typedef int (*fn_idamax)(const int*, const double*, const int*);
typedef void (*fn_dswap)(const int*, double*, const int*, double*, const int*);
typedef double (*fn_dnrm2)(const int*, const double*, const int*);
typedef double (*fn_dlamch)(const char*, flen);
typedef void (*fn_dgeqpf)(const int*, const int*, double*, const int*, int*, double*,
                          double*, int*);
typedef void (*fn_dgeqp3)(const int*, const int*, double*, const int*, int*, double*,
                          double*, const int*, int*);
typedef void (*fn_dgeqrf)(const int*, const int*, double*, const int*, double*, double*,
                          const int*, int*);
typedef void (*fn_dormqr)(const char*, const char*, const int*, const int*, const int*,
                          const double*, const int*, const double*, double*, const int*,
                          double*, const int*, int*, flen, flen);
typedef int (*fn_ilaenv)(const int*, const char*, const char*, const int*, const int*,
                         const int*, const int*, flen, flen);
typedef void (*fn_xerbla)(const char*, const int*, flen);
typedef void (*fn_setthreads)(int);
typedef void (*fn_dtrsm)(const char*, const char*, const char*, const char*, const int*,
                         const int*, const double*, const double*, const int*, double*,
                         const int*, flen, flen, flen, flen);
typedef void (*fn_dgemv)(const char*, const int*, const int*, const double*, const double*,
                         const int*, const double*, const int*, const double*, double*,
                         const int*, flen);
typedef void (*fn_dger)(const int*, const int*, const double*, const double*, const int*,
                        const double*, const int*, double*, const int*);
typedef void (*fn_dcopy)(const int*, const double*, const int*, double*, const int*);
typedef void (*fn_daxpy)(const int*, const double*, const double*, const int*, double*,
                         const int*);
typedef void (*fn_dscal)(const int*, const double*, double*, const int*);

static struct {
  void* handle;
  fn_dgemm dgemm;
  fn_dlacpy dlacpy;
  fn_dlarfg dlarfg;
  fn_dlarf dlarf;
  fn_dlarft dlarft;
  fn_dlarfb dlarfb;
  fn_dtrmm dtrmm;
  fn_idamax idamax;
  fn_dswap dswap;
  fn_dnrm2 dnrm2;
  fn_dlamch dlamch;
  fn_dgeqpf dgeqpf;
  fn_dgeqp3 dgeqp3;
  fn_dgeqrf dgeqrf;
  fn_dormqr dormqr;
  fn_ilaenv ilaenv;
  fn_xerbla xerbla;
  fn_setthreads set_threads;
  /* used by the UT-variant restatement */
  fn_dtrsm dtrsm;
  fn_dgemv dgemv;
  fn_dger dger;
  fn_dcopy dcopy;
  fn_daxpy daxpy;
  fn_dscal dscal;
} LA;

static void* find_sym(void* h, const char* prefix, const char* base) {
  char name[96];
  snprintf(name, sizeof name, "%s%s", prefix, base);
  return dlsym(h, name);
}

/* Open an LP64 LAPACK.  Returns 0 on success, -1 if the file will not open,
 * -2 if a routine is missing.  Tries the "scipy_" prefix first. */
int oracle_open(const char* path) {
  static const char* prefixes[] = {"scipy_", ""};
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return -1;
  for (int pi = 0; pi < 2; ++pi) {
    const char* p = prefixes[pi];
#define LOAD(field, sym) LA.field = (typeof(LA.field))find_sym(h, p, sym)
    LOAD(dgemm, "dgemm_");
    LOAD(dlacpy, "dlacpy_");
    LOAD(dlarfg, "dlarfg_");
    LOAD(dlarf, "dlarf_");
    LOAD(dlarft, "dlarft_");
    LOAD(dlarfb, "dlarfb_");
    LOAD(dtrmm, "dtrmm_");
    LOAD(idamax, "idamax_");
    LOAD(dswap, "dswap_");
    LOAD(dnrm2, "dnrm2_");
    LOAD(dlamch, "dlamch_");
    LOAD(dgeqpf, "dgeqpf_");
    LOAD(dgeqp3, "dgeqp3_");
    LOAD(dgeqrf, "dgeqrf_");
    LOAD(dormqr, "dormqr_");
    LOAD(ilaenv, "ilaenv_");
    LOAD(xerbla, "xerbla_");
    LOAD(dtrsm, "dtrsm_");
    LOAD(dgemv, "dgemv_");
    LOAD(dger, "dger_");
    LOAD(dcopy, "dcopy_");
    LOAD(daxpy, "daxpy_");
    LOAD(dscal, "dscal_");
#undef LOAD
    LA.set_threads = (fn_setthreads)find_sym(h, p, "openblas_set_num_threads");
    if (LA.dgemm && LA.dlacpy && LA.dlarfg && LA.dlarf && LA.dlarft && LA.dlarfb &&
        LA.dtrmm && LA.idamax && LA.dswap && LA.dnrm2 && LA.dlamch && LA.dgeqpf &&
        LA.dgeqp3 && LA.dgeqrf && LA.dormqr && LA.ilaenv && LA.xerbla && LA.dtrsm &&
        LA.dgemv && LA.dger && LA.dcopy && LA.daxpy && LA.dscal) {
      LA.handle = h;
      return 0;
    }
  }
  dlclose(h);
  memset(&LA, 0, sizeof LA);
  return -2;
}

int oracle_set_threads(int n) {
  if (!LA.set_threads) return -1;
  LA.set_threads(n);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Gaussian sketch.  Marsaglia's polar method over libc rand(), one spare    */
/* value carried between calls exactly as ...var4.c:593-614 carries it.     */

static struct {
  int have_spare;
  double spare;
} polar;

static double polar_normal(void) {
  if (polar.have_spare) {
    polar.have_spare = 0;
    return polar.spare;
  }
  double u, v, r;
  do {
    u = -1.0 + 2.0 * ((double)rand() / RAND_MAX);
    v = -1.0 + 2.0 * ((double)rand() / RAND_MAX);
    r = u * u + v * v;
  } while (r == 0 || r >= 1);
  double f = sqrt((-2 * log(r)) / r);
  polar.spare = v * f;
  polar.have_spare = 1;
  return u * f;
}

/* Fill a rows x cols column-major matrix (leading dim ld) column by column,
 * row index fastest (...var4.c:583-587). */
static void polar_fill(int rows, int cols, double* G, int ld) {
  for (int c = 0; c < cols; ++c)
    for (int r = 0; r < rows; ++r) G[r + (size_t)c * ld] = polar_normal();
}

/* The sketch the reference draws on entry to NoFLA_HQRRP_WY_blk_var4:
 * srand(12) (...var4.c:380) then the polar fill of an mY x m matrix. */
void oracle_sketch(int mY, int m, double* G) {
  srand(12);
  polar_fill(mY, m, G, mY);
}

/* ------------------------------------------------------------------------ */
/* Column norms (...var4.c:889-909) and the LAWN 176 downdate (:912-986).    */

static void colnorms(int rows, int cols, const double* A, int lda, double* d, double* e) {
  const int one = 1;
  for (int c = 0; c < cols; ++c) {
    d[c] = LA.dnrm2(&rows, A + (size_t)c * lda, &one);
    e[c] = d[c];
  }
}

/* rows_below: rows under the pivot row; wrow: the pivot row of the trailing
 * block (stride ldw); below: the trailing block under it (leading dim lda). */
static void colnorms_downdate(int rows_below, int cols, double* d, double* e,
                              const double* wrow, int ldw, const double* below, int lda) {
  const int one = 1;
  const double tol3z = sqrt(LA.dlamch("Epsilon", 7));
  for (int c = 0; c < cols; ++c) {
    if (d[c] == 0.0) continue;
    double t = fabs(wrow[(size_t)c * ldw]) / d[c];
    t = (1.0 + t) * (1 - t);
    if (0.0 > t) t = 0.0;
    double ratio = d[c] / e[c];
    double t2 = t * ratio * ratio;
    if (t2 <= tol3z) {
      d[c] = rows_below > 0 ? LA.dnrm2(&rows_below, below + (size_t)c * lda, &one) : 0.0;
      e[c] = d[c];
    } else {
      d[c] = d[c] * sqrt(t);
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Unblocked QR with optional column pivoting (...var4.c:774-886).          */

typedef struct {
  double* a;  /* companion matrix whose columns follow the pivots (or NULL) */
  int rows;
  int ld;
} companion;

static void swap_cols(int rows, double* x, double* y) {
  const int one = 1;
  LA.dswap(&rows, x, &one, y, &one);
}

/* Bring column k (relative to the front) to the front of the active part:
 * swap the factored matrix, the two companions and the labels; the norms of
 * the front column are copied into slot k (...var4.c:990-1036). */
static void bring_to_front(int k, int rows, double* a, int lda, companion* b, companion* c,
                           int* labels, double* d, double* e) {
  if (k == 0) return;
  swap_cols(rows, a, a + (size_t)k * lda);
  if (b) swap_cols(b->rows, b->a, b->a + (size_t)k * b->ld);
  if (c) swap_cols(c->rows, c->a, c->a + (size_t)k * c->ld);
  int t = labels[k];
  labels[k] = labels[0];
  labels[0] = t;
  d[k] = d[0];
  e[k] = e[0];
}

static void qrp_unblocked(int pivoting, int stages, int m, int n, double* A, int lda,
                          int* labels, double* tau, companion* B, companion* C, double* T,
                          int ldt) {
  const int one = 1;
  const int mn = m < n ? m : n;
  if (stages < 0) stages = mn;
  double* d = malloc(sizeof(double) * (n > 0 ? n : 1));
  double* e = malloc(sizeof(double) * (n > 0 ? n : 1));
  double* work = malloc(sizeof(double) * (n > 0 ? n : 1));
  if (pivoting == 1) colnorms(m, n, A, lda, d, e);

  for (int k = 0; k < stages; ++k) {
    double* akk = A + k + (size_t)k * lda;
    if (pivoting == 1) {
      int active = n - k;
      int best = LA.idamax(&active, d + k, &one) - 1;
      companion bk, ck, *pb = NULL, *pc = NULL;
      if (B) { bk = *B; bk.a = B->a + (size_t)k * B->ld; pb = &bk; }
      if (C) { ck = *C; ck.a = C->a + (size_t)k * C->ld; pc = &ck; }
      bring_to_front(best, m, A + (size_t)k * lda, lda, pb, pc, labels + k, d + k, e + k);
    }
    /* Reflector annihilating A[k+1:m, k]. */
    int len = m - k;
    int below = (k + 1 < m - 1 ? k + 1 : m - 1);
    LA.dlarfg(&len, akk, A + below + (size_t)k * lda, &one, tau + k);
    /* Apply it from the left to A[k:m, k+1:n] with the unit diagonal in place. */
    int rest = n - k - 1;
    double keep = *akk;
    *akk = 1.0;
    LA.dlarf("Left", &len, &rest, akk, &one, tau + k, akk + lda, &lda, work, 4);
    *akk = keep;
    if (pivoting == 1) {
      int next = (k + 1 < n - 1 ? k + 1 : n - 1);
      colnorms_downdate(m - k - 1, rest, d + k + 1, e + k + 1, akk + lda, lda,
                        A + (k + 1) + (size_t)next * lda, lda);
    }
  }
  if (T) LA.dlarft("Forward", "Columnwise", &m, &stages, A, &lda, tau, T, &ldt, 7, 10);
  free(d);
  free(e);
  free(work);
}

/* ------------------------------------------------------------------------ */
/* Block reflector application (...var4.c:711-771).                          */

/* B := Q^T B with Q = I - U T U^T, from the left. */
static void reflect_left_t(int mu, int k, const double* U, int ldu, const double* T, int ldt,
                           int mb, int nb, double* B, int ldb) {
  int ldw = nb > 1 ? nb : 1;
  double* W = malloc(sizeof(double) * ((size_t)nb * k + 1));
  (void)mu;
  LA.dlarfb("Left", "Transpose", "Forward", "Columnwise", &mb, &nb, &k, U, &ldu, T, &ldt, B,
            &ldb, W, &ldw, 4, 9, 7, 10);
  free(W);
}

/* B := B Q with Q = I - U T U^T, from the right. */
static void reflect_right_n(int mu, int k, const double* U, int ldu, const double* T, int ldt,
                            int mb, int nb, double* B, int ldb) {
  int ldw = mb > 1 ? mb : 1;
  double* W = malloc(sizeof(double) * ((size_t)mb * k + 1));
  (void)mu;
  LA.dlarfb("Right", "No transpose", "Forward", "Columnwise", &mb, &nb, &k, U, &ldu, T, &ldt,
            B, &ldb, W, &ldw, 5, 12, 7, 10);
  free(W);
}

/* ------------------------------------------------------------------------ */
/* Sketch downdate (...var4.c:617-708):                                      */
/*   Y2 := Y2 - (G1 - (G1 U11 + G2 U21) T U11^T) R12;  [G1 G2] := [G1 G2] Q  */

static void sketch_downdate(int b, const double* U11, int ldu, int m21, const double* U21,
                            int n12, const double* R12, int ldr, const double* T, int ldt,
                            int mY, double* Y2, int ldy, double* G1, const double* G2,
                            int n2, int ldg) {
  const double p1 = 1.0, m1 = -1.0;
  int ldb = mY;
  double* Bm = malloc(sizeof(double) * ((size_t)mY * b + 1));
  LA.dlacpy("All", &mY, &b, G1, &ldg, Bm, &ldb, 3);
  LA.dtrmm("Right", "Lower", "No transpose", "Unit", &mY, &b, &p1, U11, &ldu, Bm, &ldb, 5, 5,
           12, 4);
  LA.dgemm("No transpose", "No transpose", &mY, &b, &m21, &p1, G2, &ldg, U21, &ldu, &p1, Bm,
           &ldb, 12, 12);
  LA.dtrmm("Right", "Upper", "No transpose", "Non-unit", &mY, &b, &p1, T, &ldt, Bm, &ldb, 5, 5,
           12, 8);
  LA.dtrmm("Right", "Lower", "Conj_transpose", "Unit", &mY, &b, &m1, U11, &ldu, Bm, &ldb, 5,
           5, 14, 4);
  for (int c = 0; c < b; ++c)
    for (int r = 0; r < mY; ++r) Bm[r + (size_t)c * ldb] += G1[r + (size_t)c * ldg];
  LA.dgemm("No transpose", "No transpose", &mY, &n12, &b, &m1, Bm, &ldb, R12, &ldr, &p1, Y2,
           &ldy, 12, 12);
  reflect_right_n(b + m21, b, U11, ldu, T, ldt, mY, b + n2, G1, ldg);
  free(Bm);
}

/* ------------------------------------------------------------------------ */
/* Blocked HQRRP (...var4.c:303-571).  G_in == NULL draws the reference      */
/* sketch; otherwise the (nb+pp) x m matrix G_in (leading dim ldg_in) is     */
/* used in its place.                                                        */

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

int oracle_hqrrp_sketch(int m, int n, double* A, int lda, int* jpvt, double* tau, int nb,
                        int pp, int panel_piv, const double* G_in, int ldg_in) {
  int bad = 0;
  if (m < 0) { fprintf(stderr, "ERROR in NoFLA_HQRRP_WY_blk_var4: m_A is < 0.\n"); bad = 1; }
  if (n < 0) { fprintf(stderr, "ERROR in NoFLA_HQRRP_WY_blk_var4: n_A is < 0.\n"); bad = 1; }
  if (lda < imax(1, m)) {
    fprintf(stderr, "ERROR in NoFLA_HQRRP_WY_blk_var4: ldim_A is < max( 1, m_A ).\n");
    bad = 1;
  }
  if (bad) return 0;
  const int mn = imin(m, n);
  if (mn == 0) return 0;

  srand(12);
  const int mY = nb + pp;
  const int ldy = mY, ldv = mY, ldw = nb, ldg = mY;
  double* Y = malloc(sizeof(double) * (size_t)mY * n);
  double* V = malloc(sizeof(double) * (size_t)mY * n);
  double* W = malloc(sizeof(double) * (size_t)nb * n);
  double* G = malloc(sizeof(double) * (size_t)mY * m);
  if (G_in) {
    for (int c = 0; c < m; ++c)
      memcpy(G + (size_t)c * ldg, G_in + (size_t)c * ldg_in, sizeof(double) * mY);
  } else {
    polar_fill(mY, m, G, ldg);
  }
  {
    const double one = 1.0, zero = 0.0;
    LA.dgemm("No tranpose", "No transpose", &mY, &n, &m, &one, G, &ldg, A, &lda, &zero, Y,
             &ldy, 11, 12);
  }

  for (int j = 0; j < mn; j += nb) {
    const int b = imin(nb, imin(n - j, m - j));
    const int last = (j + nb >= m) || (j + nb >= n);
    double* AR = A + (size_t)j * lda;      /* all m rows, columns j: */
    double* ABR = A + j + (size_t)j * lda; /* rows j:, columns j: */
    double* YR = Y + (size_t)j * ldy;
    double* T1 = W + (size_t)j * ldw;

    if (!last) {
      /* Pivot selection: QRP of a copy of Y[:, j:], b stages, dragging the
       * columns of A (all rows) and of Y along. */
      int nvr = n - j;
      double* VR = V + (size_t)j * ldv;
      LA.dlacpy("All", &mY, &nvr, YR, &ldy, VR, &ldv, 3);
      companion ca = {AR, m, lda}, cy = {YR, mY, ldy};
      qrp_unblocked(1, b, mY, nvr, VR, ldv, jpvt + j, tau + j, &ca, &cy, NULL, 0);
    }

    /* Panel: QRP of A[j:, j:j+b] dragging A[0:j, j:j+b] and Y[:, j:j+b]; T. */
    {
      companion ca = {AR, j, lda}, cy = {YR, mY, ldy};
      qrp_unblocked(panel_piv, -1, m - j, b, ABR, lda, jpvt + j, tau + j, &ca, &cy, T1, ldw);
    }

    const int n12 = imax(0, n - j - b);
    const int m21 = imax(0, m - j - b);
    double* A12 = A + j + (size_t)imin(n - 1, j + b) * lda;
    if (j + b < n) reflect_left_t(m - j, b, ABR, lda, T1, ldw, m - j, n12, A12, lda);

    if (!last) {
      const double* U21 = A + imin(m - 1, j + nb) + (size_t)j * lda;
      double* Y2 = Y + (size_t)imin(n - 1, j + b) * ldy;
      double* G1 = G + (size_t)j * ldg;
      const double* G2 = G + (size_t)imin(m - 1, j + b) * ldg;
      sketch_downdate(b, ABR, lda, m21, U21, n12, A12, lda, T1, ldw, mY, Y2, ldy, G1, G2,
                      imax(0, m - j - b), ldg);
    }
  }
  free(G);
  free(Y);
  free(V);
  free(W);
  return 0;
}

int oracle_hqrrp(int m, int n, double* A, int lda, int* jpvt, double* tau, int nb, int pp,
                 int panel_piv) {
  return oracle_hqrrp_sketch(m, n, A, lda, jpvt, tau, nb, pp, panel_piv, NULL, 0);
}

/* ------------------------------------------------------------------------ */
/* dgeqp4: the dgeqp3-compatible front end (...var4.c:127-300).              */

#define SMALL_DGEQPF 250
#define SMALL_DGEQP3 1000

/* G_in (optional): the sketch of the HQRRP call on the free block, 74 x
 * (m - nf) with leading dimension ldg_in, in place of the one the reference
 * draws there (...var4.c:257-265). */
static void dgeqp4_impl(int* pm, int* pn, double* A, int* plda, int* jpvt, double* tau,
                        double* work, int* plwork, int* info, const double* G_in, int ldg_in) {
  const int m = *pm, n = *pn, lda = *plda, mn = imin(m, n);
  const int query = (*plwork == -1);
  int iws = 1;
  *info = 0;
  if (m < 0) *info = -1;
  else if (n < 0) *info = -2;
  else if (lda < imax(1, m)) *info = -4;

  if (*info == 0) {
    int lwkopt = 1;
    if (mn != 0) {
      const int ispec = 1, none = -1;
      iws = 3 * n + 1;
      int nbq = LA.ilaenv(&ispec, "DGEQRF", " ", &m, &n, &none, &none, 6, 1);
      lwkopt = 2 * n + (n + 1) * nbq;
    }
    work[0] = (double)lwkopt;
    if (*plwork < iws && !query) *info = -8;
  }
  if (*info != 0) {
    int arg = -*info;
    LA.xerbla("DGEQP3", &arg, 6);
    return;
  }
  if (query || mn == 0) return;

  if (mn < SMALL_DGEQPF) {
    LA.dgeqpf(pm, pn, A, plda, jpvt, tau, work, info);
    return;
  }
  if (mn < SMALL_DGEQP3) {
    LA.dgeqp3(pm, pn, A, plda, jpvt, tau, work, plwork, info);
    return;
  }

  /* Fixed columns (jpvt != 0) to the front; labels become 1-based. */
  int nfix = 0;
  for (int c = 0; c < n; ++c) {
    if (jpvt[c] != 0) {
      if (c != nfix) {
        swap_cols(m, A + (size_t)c * lda, A + (size_t)nfix * lda);
        jpvt[c] = jpvt[nfix];
        jpvt[nfix] = c + 1;
      } else {
        jpvt[c] = c + 1;
      }
      ++nfix;
    } else {
      jpvt[c] = c + 1;
    }
  }
  const int nf = imin(m, nfix);
  if (nf > 0) {
    LA.dgeqrf(&m, &nf, A, &lda, tau, work, plwork, info);
    if (*info != 0) fprintf(stderr, "ERROR in dgeqrf: Info: %d \n", *info);
    iws = imax(iws, (int)work[0]);
    if (nf < n) {
      int nrest = n - nf;
      LA.dormqr("Left", "Transpose", &m, &nrest, &nf, A, &lda, tau, A + (size_t)nf * lda, &lda,
                work, plwork, info, 4, 9);
      if (*info != 0) fprintf(stderr, "ERROR in dormqr: Info: %d \n", *info);
      iws = imax(iws, (int)work[0]);
    }
  }
  int* before = malloc(sizeof(int) * (size_t)n);
  if (nf > 0) memcpy(before, jpvt, sizeof(int) * (size_t)n);
  if (nf < mn)
    *info = oracle_hqrrp_sketch(m - nf, n - nf, A + nf + (size_t)nf * lda, lda, jpvt + nf,
                                tau + nf, 64, 10, 1, G_in, ldg_in);
  if (nf > 0) {
    /* Follow HQRRP's column order in the rows above the factored block. */
    for (int c = nf; c < n; ++c) {
      int k = c;
      while (k < n && jpvt[c] != before[k]) ++k;
      if (k != c && k < n) {
        int t = before[c];
        before[c] = before[k];
        before[k] = t;
        swap_cols(nf, A + (size_t)c * lda, A + (size_t)k * lda);
      }
    }
  }
  free(before);
  work[0] = iws;
}

void oracle_dgeqp4(int* pm, int* pn, double* A, int* plda, int* jpvt, double* tau,
                   double* work, int* plwork, int* info) {
  dgeqp4_impl(pm, pn, A, plda, jpvt, tau, work, plwork, info, NULL, 0);
}

void oracle_dgeqp4_sketch(int* pm, int* pn, double* A, int* plda, int* jpvt, double* tau,
                          double* work, int* plwork, int* info, const double* G, int ldg) {
  dgeqp4_impl(pm, pn, A, plda, jpvt, tau, work, plwork, info, G, ldg);
}

/* Plain LAPACK pass-throughs used as the threshold-path oracle. */
void oracle_dgeqp3(int* m, int* n, double* A, int* lda, int* jpvt, double* tau, double* work,
                   int* lwork, int* info) {
  LA.dgeqp3(m, n, A, lda, jpvt, tau, work, lwork, info);
}

void oracle_dgeqpf(int* m, int* n, double* A, int* lda, int* jpvt, double* tau, double* work,
                   int* info) {
  LA.dgeqpf(m, n, A, lda, jpvt, tau, work, info);
}

/* ======================================================================== */
/* The reference's second implementation: the UT-transform variant         */
/* libflame_sources/FLA_HQRRP_UT_blk_var2.c:124-401 (helpers :405-1166),    */
/* restated over plain column-major buffers (its libflame objects are views */
/* of such buffers).  libflame itself is not part of the reference tree and */
/* is not installed here, so this restatement is not pinned to a compiled   */
/* reference: it is checked against the WY restatement above (same pivots,  */
/* the same R up to the sign convention below, s = 1 / tau) in             */
/* tests/test_oracle.py.                                                    */
/*                                                                          */
/* Third-party routine restated: libflame's FLA_Househ2_UT_l_opd (libflame  */
/* 5.x, src/base/flamec/util/lapack/), called at :764.  For x = [chi_1; x2] */
/* it returns u2 = x2 / (chi_1 - alpha), alpha = -sign(chi_1) ||x||_2       */
/* written over chi_1, and tau = (1 + u2^T u2) / 2, so H = I - u u^T / tau, */
/* u = [1; u2]; when x2 = 0 it sets chi_1 = -chi_1 and tau = 1/2 (H         */
/* reflects e_1), where LAPACK's dlarfg returns tau = 0 (H = I).           */

static struct {
  int have_spare;
  double spare;
} polar_ut; /* MyFLA_Normal_random_number's own carried value (:443-465) */

static double polar_normal_ut(void) {
  if (polar_ut.have_spare) {
    polar_ut.have_spare = 0;
    return polar_ut.spare;
  }
  double u, v, r;
  do {
    u = -1.0 + 2.0 * ((double)rand() / RAND_MAX);
    v = -1.0 + 2.0 * ((double)rand() / RAND_MAX);
    r = u * u + v * v;
  } while (r == 0 || r >= 1);
  double f = sqrt((-2 * log(r)) / r);
  polar_ut.spare = v * f;
  polar_ut.have_spare = 1;
  return u * f;
}

static void househ2_ut(int m_x2, double* chi_1, double* x2, double* tau) {
  const int one = 1, two = 2;
  const double norm_x2 = m_x2 > 0 ? LA.dnrm2(&m_x2, x2, &one) : 0.0;
  if (norm_x2 == 0.0) {
    *chi_1 = -*chi_1;
    *tau = 0.5;
    return;
  }
  double v[2] = {fabs(*chi_1), norm_x2};
  const double norm_x = LA.dnrm2(&two, v, &one);
  const double alpha = (*chi_1 >= 0.0 ? -1.0 : 1.0) * norm_x;
  const double cma = *chi_1 - alpha;
  const double inv = 1.0 / cma;
  LA.dscal(&m_x2, &inv, x2, &one);
  const double nu = norm_x2 / fabs(cma); /* ||u2|| */
  *tau = (1.0 + nu * nu) / 2.0;
  *chi_1 = alpha;
}

/* MyFLA_Apply_H2_UT_l_opd_var2 (:824-930): w = (a1t + A2^T u2) / tau,
 * a1t -= w, A2 -= u2 w^T. */
static void apply_h2_ut(int m2, int n1, double tau, const double* u2, double* a1t, int inc_a1t,
                        double* A2, int lda2, double* w) {
  const int one = 1;
  const double d_one = 1.0, m_one = -1.0;
  if (n1 == 0) return;
  LA.dcopy(&n1, a1t, &inc_a1t, w, &one);
  LA.dgemv("Transpose", &m2, &n1, &d_one, A2, &lda2, u2, &one, &d_one, w, &one, 9);
  const double rtau = 1.0 / tau;
  LA.dscal(&n1, &rtau, w, &one);
  LA.daxpy(&n1, &m_one, w, &one, a1t, &inc_a1t);
  LA.dger(&m2, &n1, &m_one, u2, &one, w, &one, A2, &lda2);
}

/* NoFLA_my_idamax (:1123-1166): first index of the largest |d|, strict <. */
static int my_idamax(int n, const double* d) {
  if (n < 1) return -1;
  int r = 0;
  double dmax = fabs(d[0]);
  for (int i = 1; i < n; ++i)
    if (dmax < fabs(d[i])) {
      r = i;
      dmax = fabs(d[i]);
    }
  return r;
}

/* MyFLA_QRPmod_UT_unb_var2 (:640-822). */
static void qrp_ut_unblocked(int pivoting, int stages, int m, int n, double* A, int lda,
                             int* p, double* t, companion* B, companion* C, double* T,
                             int ldt) {
  const int one = 1;
  const double d_one = 1.0;
  const int mn = m < n ? m : n;
  if (stages < 0) stages = mn;
  double* d = malloc(sizeof(double) * (n > 0 ? n : 1));
  double* e = malloc(sizeof(double) * (n > 0 ? n : 1));
  double* work = malloc(sizeof(double) * (n > 0 ? n : 1));
  if (pivoting == 1) colnorms(m, n, A, lda, d, e);
  for (int j = 0; j < stages; ++j) {
    if (pivoting == 1) {
      const int idx = my_idamax(n - j, d + j);
      companion bk, ck, *pb = NULL, *pc = NULL;
      if (B) { bk = *B; bk.a = B->a + (size_t)j * B->ld; pb = &bk; }
      if (C) { ck = *C; ck.a = C->a + (size_t)j * C->ld; pc = &ck; }
      bring_to_front(idx, m, A + (size_t)j * lda, lda, pb, pc, p + j, d + j, e + j);
    }
    const int m21 = m - j - 1, n22 = n - j - 1;
    double* ajj = A + j + (size_t)j * lda;
    househ2_ut(m21, ajj, ajj + 1, t + j);
    apply_h2_ut(m21, n22, t[j], ajj + 1, ajj + lda, lda, ajj + 1 + lda, lda, work);
    if (T) {
      /* T[j, j] = tau_j; T[0:j, j] = A[j, 0:j]^T + A[j+1:, 0:j]^T u21. */
      T[j + (size_t)j * ldt] = t[j];
      LA.dcopy(&j, A + j, &lda, T + (size_t)j * ldt, &one);
      LA.dgemv("Transpose", &m21, &j, &d_one, A + j + 1, &lda, ajj + 1, &one, &d_one,
               T + (size_t)j * ldt, &one, 9);
    }
    if (pivoting == 1)
      colnorms_downdate(m21, n22, d + j + 1, e + j + 1, ajj + lda, lda, ajj + 1 + lda, lda);
  }
  free(d);
  free(e);
  free(work);
}

/* MyFLA_Apply_Q_UT_lhfc_blk_var2 (:532-582): [B1; B2] := Q^T [B1; B2] with
 * Q = I - U inv(T) U^T, U = [U11 (unit lower); U21]. */
static void apply_q_ut_lhfc(int b, int mr, int nc, const double* U11, const double* U21, int ldu,
                            const double* T, int ldt, double* B1, double* B2, int ldb) {
  if (nc <= 0) return;
  const double d_one = 1.0, m_one = -1.0;
  double* W = malloc(sizeof(double) * (size_t)b * nc);
  LA.dlacpy("All", &b, &nc, B1, &ldb, W, &b, 3);
  LA.dtrmm("Left", "Lower", "Transpose", "Unit", &b, &nc, &d_one, U11, &ldu, W, &b, 4, 5, 9, 4);
  if (mr > 0)
    LA.dgemm("Transpose", "No transpose", &b, &nc, &mr, &d_one, U21, &ldu, B2, &ldb, &d_one, W,
             &b, 9, 12);
  LA.dtrsm("Left", "Upper", "Transpose", "Non-unit", &b, &nc, &d_one, T, &ldt, W, &b, 4, 5, 9,
           8);
  if (mr > 0)
    LA.dgemm("No transpose", "No transpose", &mr, &nc, &b, &m_one, U21, &ldu, W, &b, &d_one, B2,
             &ldb, 12, 12);
  LA.dtrmm("Left", "Lower", "No transpose", "Unit", &b, &nc, &m_one, U11, &ldu, W, &b, 4, 5, 12,
           4);
  for (int c = 0; c < nc; ++c)
    for (int r = 0; r < b; ++r) B1[r + (size_t)c * ldb] += W[r + (size_t)c * b];
  free(W);
}

/* MyFLA_Apply_Q_UT_rnfc_blk_var2 (:585-637): [B1, B2] := [B1, B2] Q. */
static void apply_q_ut_rnfc(int b, int mr, int rows, const double* U11, const double* U21,
                            int ldu, const double* T, int ldt, double* B1, double* B2, int ldb) {
  const double d_one = 1.0, m_one = -1.0;
  double* W = malloc(sizeof(double) * (size_t)b * (rows > 0 ? rows : 1));
  for (int c = 0; c < b; ++c)
    for (int r = 0; r < rows; ++r) W[c + (size_t)r * b] = B1[r + (size_t)c * ldb];
  LA.dtrmm("Left", "Lower", "Transpose", "Unit", &b, &rows, &d_one, U11, &ldu, W, &b, 4, 5, 9,
           4);
  if (mr > 0)
    LA.dgemm("Transpose", "Transpose", &b, &rows, &mr, &d_one, U21, &ldu, B2, &ldb, &d_one, W, &b,
             9, 9);
  LA.dtrsm("Left", "Upper", "Transpose", "Non-unit", &b, &rows, &d_one, T, &ldt, W, &b, 4, 5, 9,
           8);
  if (mr > 0)
    LA.dgemm("Transpose", "Transpose", &rows, &mr, &b, &m_one, W, &b, U21, &ldu, &d_one, B2, &ldb,
             9, 9);
  LA.dtrmm("Left", "Lower", "No transpose", "Unit", &b, &rows, &m_one, U11, &ldu, W, &b, 4, 5,
           12, 4);
  for (int c = 0; c < b; ++c)
    for (int r = 0; r < rows; ++r) B1[r + (size_t)c * ldb] += W[c + (size_t)r * b];
  free(W);
}

/* MyFLA_Downdate_Y (:468-529):
 * Y2 -= (G1 - (G1 U11 + G2 U21) inv(T) U11^T) R12, then G := G Q. */
static void downdate_y_ut(int b, int mr, int mY, int n2, const double* U11, const double* U21,
                          int ldu, const double* A12, int lda, const double* T, int ldt,
                          double* Y2, int ldy, double* G1, double* G2, int ldg) {
  const double d_one = 1.0, m_one = -1.0;
  double* B = malloc(sizeof(double) * (size_t)mY * b);
  LA.dlacpy("All", &mY, &b, G1, &ldg, B, &mY, 3);
  LA.dtrmm("Right", "Lower", "No transpose", "Unit", &mY, &b, &d_one, U11, &ldu, B, &mY, 5, 5,
           12, 4);
  if (mr > 0)
    LA.dgemm("No transpose", "No transpose", &mY, &b, &mr, &d_one, G2, &ldg, U21, &ldu, &d_one,
             B, &mY, 12, 12);
  LA.dtrsm("Right", "Upper", "No transpose", "Non-unit", &mY, &b, &d_one, T, &ldt, B, &mY, 5, 5,
           12, 8);
  LA.dtrmm("Right", "Lower", "Transpose", "Unit", &mY, &b, &m_one, U11, &ldu, B, &mY, 5, 5, 9,
           4);
  for (int c = 0; c < b; ++c)
    for (int r = 0; r < mY; ++r) B[r + (size_t)c * mY] += G1[r + (size_t)c * ldg];
  if (n2 > 0)
    LA.dgemm("No transpose", "No transpose", &mY, &n2, &b, &m_one, B, &mY, A12, &lda, &d_one, Y2,
             &ldy, 12, 12);
  apply_q_ut_rnfc(b, mr, mY, U11, U21, ldu, T, ldt, G1, G2, ldg);
  free(B);
}

/* FLA_HQRRP_UT_blk_var2 (:124-401): p carried (permuted like the columns),
 * s[0..min(m,n)) the UT scalars tau_UT.  G_in (optional, (nb+pp) x m, ld
 * ldg_in) replaces the drawn sketch. */
int oracle_hqrrp_ut_sketch(int m, int n, double* A, int lda, int* p, double* s, int nb, int pp,
                           int panel_piv, const double* G_in, int ldg_in) {
  const int mn = imin(m, n);
  if (mn <= 0) return 0;
  srand(12);
  const int mY = nb + pp, ldg = mY, ldy = mY, ldw = nb;
  double* G = malloc(sizeof(double) * (size_t)mY * m);
  double* Y = malloc(sizeof(double) * (size_t)mY * n);
  double* V = malloc(sizeof(double) * (size_t)mY * n);
  double* W = calloc((size_t)nb * n, sizeof(double));
  if (G_in) {
    for (int c = 0; c < m; ++c)
      memcpy(G + (size_t)c * ldg, G_in + (size_t)c * ldg_in, sizeof(double) * mY);
  } else {
    for (int c = 0; c < m; ++c)
      for (int r = 0; r < mY; ++r) G[r + (size_t)c * ldg] = polar_normal_ut();
  }
  {
    const double one = 1.0, zero = 0.0;
    LA.dgemm("No transpose", "No transpose", &mY, &n, &m, &one, G, &ldg, A, &lda, &zero, Y, &ldy,
             12, 12);
  }
  for (int j = 0; j < mn;) {
    const int b = imin(imin(m - j, n - j), nb);
    const int last = imin(m - j - b, n - j - b) <= 0;
    double* AR = A + (size_t)j * lda;
    double* ABR = AR + j;
    double* YR = Y + (size_t)j * ldy;
    double* T1 = W + (size_t)j * ldw;
    if (!last) {
      const int nvr = n - j;
      double* VR = V + (size_t)j * ldy;
      LA.dlacpy("All", &mY, &nvr, YR, &ldy, VR, &ldy, 3);
      companion ca = {AR, m, lda}, cy = {YR, mY, ldy};
      qrp_ut_unblocked(1, b, mY, nvr, VR, ldy, p + j, s + j, &ca, &cy, NULL, 0);
    }
    {
      companion ca = {AR, j, lda}, cy = {YR, mY, ldy};
      qrp_ut_unblocked(panel_piv, -1, m - j, b, ABR, lda, p + j, s + j, &ca, &cy, T1, ldw);
    }
    const int n2 = n - j - b, mr = m - j - b;
    double* A12 = ABR + (size_t)b * lda;
    if (n2 > 0)
      apply_q_ut_lhfc(b, mr, n2, ABR, ABR + b, lda, T1, ldw, A12, A12 + b, lda);
    if (n2 > 0)
      downdate_y_ut(b, mr, mY, n2, ABR, ABR + b, lda, A12, lda, T1, ldw, YR + (size_t)b * ldy,
                    ldy, G + (size_t)j * ldg, G + (size_t)(j + b) * ldg, ldg);
    j += b;
  }
  free(G);
  free(Y);
  free(V);
  free(W);
  return 0;
}
