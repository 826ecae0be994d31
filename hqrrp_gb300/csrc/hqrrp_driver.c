/* hqrrp_driver.c -- host side of libhqrrp_gb300.so (C99).
 *
 * The host only validates arguments, moves data, allocates device workspace
 * from a library-owned stream-ordered pool and enqueues kernels; every
 * arithmetic step of the factorization runs on the GPU.  The block loop of
 * HQRRP (lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:412-558) is
 * enqueued without any host synchronisation: pivots, permutations and
 * reflectors stay on the device, and the host waits once at the end.
 */
#include <cuda_runtime_api.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <nvtx3/nvToolsExt.h>

#include "hq_internal.h"
#include "hqrrp_gb300.h"

/* NVTX ranges around the phases of every call (header-only NVTX v3: a no-op
 * unless a tool such as Nsight Systems is attached).  The ranges cover the
 * host's enqueueing; the tool attributes the kernels launched inside them. */
#define NV_PUSH(name) nvtxRangePushA(name)
#define NV_POP() nvtxRangePop()

#define HQ_API __attribute__((visibility("default")))

enum {
  HQ_OK = 0,
  HQ_E_CUDA = 1,        /* a CUDA call failed */
  HQ_E_DEVICE = 2,      /* a kernel reported an error (barrier timeout, ...) */
  HQ_E_UNSUPPORTED = 3, /* shape outside the kernels' limits */
  HQ_E_NOMEM = 4        /* device allocation failed */
};

#define DGEQP4_SMALL_DGEQP3 1000 /* ...var4.c:58 */
#define DGEQP4_NB 64 /* HQRRP block size and oversampling dgeqp4 uses (...var4.c:264) */
/* The block size dgeqp4's HQRRP call uses on this GPU by default: the
 * reference's 64 is a CPU default ("default values", ...var4.c:255-256); at
 * 64 the rank-64 trailing updates are bound by the split-BF16 products' FP64
 * epilogue, which 128 halves per output. */
#define DGEQP4_GPU_NB 128
static int g_dgeqp4_nb = DGEQP4_GPU_NB; /* hqrrp_gb300_set_dgeqp4_block */
#define DGEQP4_PP 10
#define LAPACK_NB_DGEQRF 32 /* ILAENV(1, 'DGEQRF') of reference LAPACK */
#define LAPACK_NX_DGEQRF 128 /* ILAENV(3, 'DGEQRF'): blocked-code crossover */
#define FIXED_BLOCK 128
#define DEFAULT_SPIN_LIMIT (1u << 22)
#define OZK_SLICES 7        /* digits per operand in the mixed block updates */
#define OZK_SKETCH_SLICES 2 /* the sketch Y = G A only steers pivots */

static __thread char g_err[512];
static int g_precision = -1;
static unsigned long long g_seed = 12ULL;
static unsigned g_spin_limit = 0;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

typedef struct {
  int ready;
  hq_device_info dev;
  cudaStream_t stream;
  cudaMemPool_t pool;
} dev_state;
static dev_state g_devs[64];

/* ---- Per-phase profiler ------------------------------------------------
 * The libflame variant of the reference accumulates wall-clock time in four
 * buckets under #ifdef PROFILE (libflame_sources/FLA_HQRRP_UT_blk_var2.c:165-167,
 * :289-398).  Here the buckets are CUDA-event intervals on the call's stream,
 * recorded only while profiling is enabled, together with the algorithmic
 * FP64 flops of the work in each interval. */
enum { PH_SKETCH = 0, PH_SELECT, PH_PANEL, PH_UPDATE, PH_DOWNDATE, PH_OTHER, PH_TENSOR,
       PH_SPLIT, PH_COUNT };
#define PROF_MAXEV 8192
static int g_prof_on = 0;
static double g_prof_ms[PH_COUNT], g_prof_flops[PH_COUNT];
static int g_prof_n[PH_COUNT];
static cudaEvent_t g_prof_ev[PROF_MAXEV];
static int g_prof_ev_ready = 0;

typedef struct {
  int n;
  int ph[PROF_MAXEV];
  double fl[PROF_MAXEV];
} prof_rec;

static void set_err(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

HQ_API const char* hqrrp_gb300_last_error(void) { return g_err; }

HQ_API int hqrrp_gb300_set_precision(int mode) {
  if (mode != 0 && mode != 1) return -1;
  int prev = g_precision < 0 ? 0 : g_precision;
  g_precision = mode;
  return prev;
}

HQ_API void hqrrp_gb300_set_seed(unsigned long long seed) { g_seed = seed; }

HQ_API int hqrrp_gb300_set_dgeqp4_block(int nb) {
  if (nb < 1 || nb + DGEQP4_PP > HQ_MAX_MY) return -1;
  const int prev = g_dgeqp4_nb;
  g_dgeqp4_nb = nb;
  return prev;
}

HQ_API void hqrrp_gb300_set_spin_limit(unsigned limit) { g_spin_limit = limit; }

static int precision(void) {
  if (g_precision < 0) {
    const char* e = getenv("HQRRP_GB300_PRECISION");
    g_precision = (e && strcmp(e, "mixed") == 0) ? 1 : 0;
  }
  return g_precision;
}

static unsigned spin_limit(void) { return g_spin_limit ? g_spin_limit : DEFAULT_SPIN_LIMIT; }

void hq_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

void hq_clear_error(void) { g_err[0] = 0; }

unsigned hq_spin_limit(void) { return spin_limit(); }

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }
static int round_up(int x, int q) { return (x + q - 1) / q * q; }

/* Library state of the current device: stream and memory pool. */
static dev_state* current_device(void) {
  int d = 0;
  cudaError_t e = cudaGetDevice(&d);
  if (e != cudaSuccess || d < 0 || d >= 64) {
    set_err("no CUDA device: %s", cudaGetErrorString(e));
    return NULL;
  }
  dev_state* s = &g_devs[d];
  pthread_mutex_lock(&g_lock);
  if (!s->ready) {
    int rc = hq_query_device(&s->dev);
    if (rc == 0) rc = (int)cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (rc == 0) {
      struct cudaMemPoolProps props;
      memset(&props, 0, sizeof props);
      props.allocType = cudaMemAllocationTypePinned;
      props.handleTypes = cudaMemHandleTypeNone;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = d;
      rc = (int)cudaMemPoolCreate(&s->pool, &props);
      if (rc == 0) {
        unsigned long long keep = ~0ULL;
        cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
      }
    }
    if (rc != 0) {
      set_err("device initialisation failed: %s", cudaGetErrorString((cudaError_t)rc));
      pthread_mutex_unlock(&g_lock);
      return NULL;
    }
    s->ready = 1;
  }
  pthread_mutex_unlock(&g_lock);
  return s;
}

/* ------------------------------------------------------------------------ */
/* Device workspace of one call.                                            */

#define MAX_ALLOCS 64
typedef struct {
  dev_state* ds;
  cudaStream_t st;
  void* ptrs[MAX_ALLOCS];
  int nptr;
  int nalloc; /* allocations attempted by this call */
  int failed;
  /* HQRRP buffers */
  double *G, *Y, *V, *U, *T, *Z, *W1, *W2, *Bm, *B2, *ws, *part, *rowbuf, *tmp;
  int *pairs, *npairs, *perm, *labels, *label_tmp, *err;
  unsigned* bar;
  int ldg, ldy, ldu, ldw, ldt, ldz, ldb, tmp_rows, tmp_cols;
  size_t ws_elems, part_elems;
  prof_rec* prof; /* non-NULL while profiling */
  int mixed;      /* split-BF16 tensor-core block updates */
  int ut;         /* UT-transform reflector convention in the panels */
  int dq_nb;      /* the HQRRP block size dgeqp4 uses in this call */
  void *ozA, *ozB; /* digit tiles of the two operands of a mixed product */
  int *ozea, *ozeb;
  int* ozraw; /* row maxima scratch of the splits (exponent fields) */
  /* Mixed mode: per global column, the largest FP64 exponent field of the
   * trailing matrix below the next block's diagonal, written by the epilogue
   * of the update that produced it (and permuted with the columns), so the
   * next block splits its trailing matrix in one streaming pass. */
  int* colexp;
  /* Mixed mode: U's digits, split once per block and shared by its products
   * (U^T as the M side: Gram, W1 = U^T C, the sketch's B^T = U^T G_R^T; U as
   * the M side: C -= U W2, G_R^T -= U B2^T). */
  void *ozUT, *ozU;
  int *ozUTe, *ozUe;
  /* Side stream (high priority) for the one-SM T factor, overlapped with
   * W1 = U^T C on st; created on first use, ordered by the two events. */
  cudaStream_t side;
  cudaEvent_t ev_gram, ev_t;
  /* Host-pointer calls on pinned host memory: each block's final columns go
   * back to the host on a copy stream while later blocks run (columns
   * [j, j + b) are never touched again once block j's panel is done). */
  double* drain_host;
  const double* drain_dev;
  int drain_lda, drain_ldda, drain_rows, drain_done;
  cudaStream_t cp;
  cudaEvent_t ev_cp;
  /* Mixed mode: the Gram panel (qrp_gram.cu).  gQ holds Q1, then Q (mp x b,
   * ldu); the b x b matrices (ld HQ_GRAM_MAX): G and G2, R1, R2, an inverse,
   * the LU of Q11 - D, and R; gstat is the panel's status word. */
  int gram;
  double *gQ, *gG, *gR1, *gR2, *gRi, *gLU, *gRH, *gsgn, *gtau;
  int *gperm, *gstat, *galt, *gcount; /* gcount: panels committed, panels passed on */
  unsigned long long* gemax;           /* the second pass's max|G2 - I| (double bits) */
  int ph_override; /* >= 0: charge split-product intervals to this phase */
} hq_ws;

/* Close the interval since the previous mark and charge it to `phase`. */
static void prof_mark(hq_ws* w, int phase, double flops) {
  prof_rec* p = w->prof;
  if (!p || p->n >= PROF_MAXEV) return;
  cudaEventRecord(g_prof_ev[p->n], w->st);
  p->ph[p->n] = phase;
  p->fl[p->n] = flops;
  p->n++;
}

static void prof_start(hq_ws* w) {
  if (!g_prof_on) return;
  pthread_mutex_lock(&g_lock);
  if (!g_prof_ev_ready) {
    for (int i = 0; i < PROF_MAXEV; ++i) cudaEventCreate(&g_prof_ev[i]);
    g_prof_ev_ready = 1;
  }
  pthread_mutex_unlock(&g_lock);
  w->prof = calloc(1, sizeof(prof_rec));
  prof_mark(w, -1, 0.0);
}

/* After the stream has been synchronised: accumulate the intervals. */
static void prof_finish(hq_ws* w) {
  prof_rec* p = w->prof;
  if (!p) return;
  for (int i = 1; i < p->n; ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, g_prof_ev[i - 1], g_prof_ev[i]) == cudaSuccess &&
        p->ph[i] >= 0 && p->ph[i] < PH_COUNT) {
      g_prof_ms[p->ph[i]] += ms;
      g_prof_flops[p->ph[i]] += p->fl[i];
      g_prof_n[p->ph[i]] += 1;
    }
  }
  free(p);
  w->prof = NULL;
}

HQ_API void hqrrp_gb300_profile_enable(int on) { g_prof_on = on ? 1 : 0; }

HQ_API int hqrrp_gb300_profile_read(double* ms, double* flops, int n) {
  for (int i = 0; i < PH_COUNT && i < n; ++i) {
    if (ms) ms[i] = g_prof_ms[i];
    if (flops) flops[i] = g_prof_flops[i];
  }
  memset(g_prof_ms, 0, sizeof g_prof_ms);
  memset(g_prof_flops, 0, sizeof g_prof_flops);
  return PH_COUNT;
}

HQ_API int hqrrp_gb300_profile_counts(int* counts, int n) {
  for (int i = 0; i < PH_COUNT && i < n; ++i) counts[i] = g_prof_n[i];
  memset(g_prof_n, 0, sizeof g_prof_n);
  return PH_COUNT;
}

HQ_API unsigned long long hqrrp_gb300_launch_count(void) { return hq_launches(); }

/* Device allocations made from the library's pools since the process
 * started. */
static unsigned long long g_pool_allocs = 0;

/* The Gram panel's counts of the last call that ran it (page-locked, written
 * by a copy on the call's stream when its workspace is released). */
static int* g_gram_counts = NULL;

HQ_API int hqrrp_gb300_gram_panel_counts(int* committed, int* fallback) {
  if (cudaDeviceSynchronize() != cudaSuccess) {
    set_err("cudaDeviceSynchronize failed: %s", cudaGetErrorString(cudaGetLastError()));
    return HQ_E_CUDA;
  }
  *committed = g_gram_counts ? g_gram_counts[0] : 0;
  *fallback = g_gram_counts ? g_gram_counts[1] : 0;
  return HQ_OK;
}

HQ_API unsigned long long hqrrp_gb300_pool_alloc_count(void) {
  return __atomic_load_n(&g_pool_allocs, __ATOMIC_RELAXED);
}

/* Host-side fault injection: HQRRP_GB300_FAIL_ALLOC=k (k >= 1) makes the k-th
 * device allocation of every call fail as if the pool were out of memory, so
 * the error path (return code / info 1000 + 4, message, workspace released)
 * can be exercised without a GPU fault.  Unset or 0: off. */
static int injected_alloc_failure(hq_ws* w) {
  const char* e = getenv("HQRRP_GB300_FAIL_ALLOC");
  if (!e || !*e) return 0;
  const long k = strtol(e, NULL, 10);
  return k > 0 && (long)w->nalloc == k;
}

static void* ws_alloc(hq_ws* w, size_t bytes) {
  void* p = NULL;
  if (w->failed) return NULL;
  if (bytes == 0) bytes = 16;
  w->nalloc++;
  if (injected_alloc_failure(w)) {
    set_err("device allocation of %zu bytes failed: injected by HQRRP_GB300_FAIL_ALLOC=%d",
            bytes, w->nalloc);
    w->failed = 1;
    return NULL;
  }
  cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, w->ds->pool, w->st);
  if (e != cudaSuccess || w->nptr >= MAX_ALLOCS) {
    set_err("device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    w->failed = 1;
    return NULL;
  }
  w->ptrs[w->nptr++] = p;
  __atomic_add_fetch(&g_pool_allocs, 1ULL, __ATOMIC_RELAXED);
  return p;
}

static void ws_release(hq_ws* w) {
  if (w->gcount) {
    if (!g_gram_counts && cudaHostAlloc((void**)&g_gram_counts, 2 * sizeof(int), 0) != cudaSuccess) {
      cudaGetLastError();
      g_gram_counts = NULL;
    }
    if (g_gram_counts)
      cudaMemcpyAsync(g_gram_counts, w->gcount, 2 * sizeof(int), cudaMemcpyDeviceToHost, w->st);
    w->gcount = NULL;
  }
  if (w->cp) {
    /* The copy stream reads the matrix: it finishes before anything is freed. */
    cudaEventRecord(w->ev_cp, w->cp);
    cudaStreamWaitEvent(w->st, w->ev_cp, 0);
    cudaStreamDestroy(w->cp);
    cudaEventDestroy(w->ev_cp);
    w->cp = NULL;
    w->drain_host = NULL;
  }
  if (w->side) {
    /* Nothing may be freed while the side stream could still use it. */
    cudaEventRecord(w->ev_t, w->side);
    cudaStreamWaitEvent(w->st, w->ev_t, 0);
  }
  for (int i = 0; i < w->nptr; ++i) cudaFreeAsync(w->ptrs[i], w->st);
  if (w->side) {
    cudaStreamDestroy(w->side);
    cudaEventDestroy(w->ev_gram);
    cudaEventDestroy(w->ev_t);
    w->side = NULL;
  }
  w->nptr = 0;
  if (w->prof) { /* an error path skipped ws_check */
    free(w->prof);
    w->prof = NULL;
  }
}

#define CK(call)                                                                  \
  do {                                                                            \
    int rc_ = (int)(call);                                                        \
    if (rc_ != 0) {                                                               \
      set_err("%s failed: %s", #call, cudaGetErrorString((cudaError_t)rc_));      \
      return HQ_E_CUDA;                                                           \
    }                                                                             \
  } while (0)

/* Workspace for HQRRP on an m x n matrix with block nb + oversampling pp,
 * and for the pivoted / unpivoted panels of dgeqp4 (panel width <= pw). */
/* N-side digit tiles: the larger of the two tile formats (general and
 * short-K kernels use different N tiles). */
static size_t ozk_b_bytes(int rows, int K, int S) {
  size_t b1 = hq_ozk_tile_bytes(rows, K, S, 1), b2 = hq_ozk_tile_bytes(rows, K, S, 2);
  return b1 > b2 ? b1 : b2;
}

static int ws_setup(hq_ws* w, int m, int n, int nb, int pp, int pw) {
  const hq_device_info* dev = &w->ds->dev;
  const int mY = nb + pp;
  const int kmax = imax(nb, pw);
  /* Programmatic dependent launch between this library's kernels, unless
   * HQRRP_GB300_PDL=0. */
  const char* pdl_env = getenv("HQRRP_GB300_PDL");
  hq_set_pdl(!(pdl_env && pdl_env[0] == '0'));
  w->ldg = round_up(imax(mY, 1), 2);
  w->ldy = w->ldg;
  w->ldb = w->ldg;
  w->ldu = round_up(imax(m, 1), 32);
  w->ldw = imax(kmax, 1);
  w->ldt = imax(kmax, 1);
  w->ldz = imax(kmax, 1);
  w->ws_elems = (size_t)16 << 20; /* split-K slices: 128 MB */
  size_t pe = hq_skinny_part_elems(dev, imin(imax(mY, 1), HQ_MAX_MY));
  size_t pe2 = hq_panel_part_elems(dev, imin(imax(kmax, 1), HQ_MAX_PANEL));
  w->part_elems = pe > pe2 ? pe : pe2;
  w->tmp_rows = imax(m, mY);
  w->tmp_cols = imax(2 * kmax, 1);
  if (mY > 0) {
    w->G = ws_alloc(w, sizeof(double) * (size_t)w->ldg * imax(m, 1));
    w->Y = ws_alloc(w, sizeof(double) * (size_t)w->ldy * imax(n, 1));
    w->V = ws_alloc(w, sizeof(double) * (size_t)w->ldy * imax(n, 1));
    w->Bm = ws_alloc(w, sizeof(double) * (size_t)w->ldb * kmax);
    w->B2 = ws_alloc(w, sizeof(double) * (size_t)w->ldb * kmax);
  }
  w->U = ws_alloc(w, sizeof(double) * (size_t)w->ldu * kmax);
  w->T = ws_alloc(w, sizeof(double) * (size_t)w->ldt * kmax);
  w->Z = ws_alloc(w, sizeof(double) * (size_t)w->ldz * kmax);
  w->W1 = ws_alloc(w, sizeof(double) * (size_t)w->ldw * imax(n, 1));
  w->W2 = ws_alloc(w, sizeof(double) * (size_t)w->ldw * imax(n, 1));
  w->ws = ws_alloc(w, sizeof(double) * w->ws_elems);
  w->part = ws_alloc(w, sizeof(double) * w->part_elems);
  w->rowbuf = ws_alloc(w, sizeof(double) * 2 * (size_t)imax(kmax, 1));
  w->tmp = ws_alloc(w, sizeof(double) * (size_t)w->tmp_rows * w->tmp_cols);
  w->pairs = ws_alloc(w, sizeof(int) * 4 * (size_t)kmax);
  w->npairs = ws_alloc(w, sizeof(int) * 2);
  w->perm = ws_alloc(w, sizeof(int) * (size_t)kmax);
  w->labels = ws_alloc(w, sizeof(int) * (size_t)imax(n, 1));
  w->label_tmp = ws_alloc(w, sizeof(int) * (size_t)imax(n, 2 * kmax));
  w->err = ws_alloc(w, sizeof(int) * 2);
  w->bar = ws_alloc(w, sizeof(unsigned) * 2);
  if (w->mixed) {
    /* Digit buffers of the split products: the sketch's (mY > 0) and those of
     * the block reflectors (HQRRP blocks and dgeqp4's fixed-column blocks). */
    const int S = OZK_SLICES, S2 = OZK_SKETCH_SLICES;
    size_t a = mY > 0 ? hq_ozk_tile_bytes(n, m, S2, 0) : 0, b = mY > 0 ? ozk_b_bytes(mY, m, S2) : 0;
    size_t t;
    if ((t = hq_ozk_tile_bytes(kmax, m, S, 0)) > a) a = t;
    if ((t = hq_ozk_tile_bytes(kmax, kmax, S, 0)) > a) a = t; /* W2 = T^T W1 */
    if ((t = hq_ozk_tile_bytes(m, kmax, S, 0)) > a) a = t;
    if ((t = hq_ozk_tile_bytes(n, kmax, S, 0)) > a) a = t;
    if ((t = ozk_b_bytes(n, m, S)) > b) b = t;
    if ((t = ozk_b_bytes(n, kmax, S)) > b) b = t;
    if ((t = ozk_b_bytes(mY, m, S)) > b) b = t;
    if ((t = ozk_b_bytes(mY, kmax, S)) > b) b = t;
    if ((t = hq_ozk_tile_bytes(mY, kmax, S, 0)) > a) a = t; /* B2 = Bm T */
    if ((t = ozk_b_bytes(kmax, kmax, S)) > b) b = t;
    if ((t = ozk_b_bytes(kmax, m, S)) > b) b = t;            /* Gram U'^T U' */
    const int rows = imax(imax(m, n), mY) + 128;
    w->ozA = ws_alloc(w, a);
    w->ozB = ws_alloc(w, b);
    w->ozea = ws_alloc(w, sizeof(int) * (size_t)rows);
    w->ozeb = ws_alloc(w, sizeof(int) * (size_t)rows);
    w->ozraw = ws_alloc(w, sizeof(int) * (size_t)rows);
    w->colexp = ws_alloc(w, sizeof(int) * (size_t)(imax(n, 1) + 64));
    w->ozUT = ws_alloc(w, hq_ozk_tile_bytes(kmax, m, S, 0));
    w->ozU = ws_alloc(w, hq_ozk_tile_bytes(m, kmax, S, 0));
    w->ozUTe = ws_alloc(w, sizeof(int) * (size_t)(kmax + 128));
    w->ozUe = ws_alloc(w, sizeof(int) * (size_t)(imax(m, 1) + 128));
    /* The Gram panel, unless HQRRP_GB300_GRAM_PANEL=0 (the cooperative
     * column-by-column panel only) or the UT convention is asked for. */
    const char* ge = getenv("HQRRP_GB300_GRAM_PANEL");
    w->gram = !(ge && ge[0] == '0');
    if (w->gram) {
      const size_t sq = (size_t)HQ_GRAM_MAX * HQ_GRAM_MAX;
      w->gQ = ws_alloc(w, sizeof(double) * (size_t)w->ldu * imin(kmax, HQ_GRAM_MAX));
      double* sm = ws_alloc(w, sizeof(double) * (6 * sq + 2 * HQ_GRAM_MAX + 1));
      w->gperm = ws_alloc(w, sizeof(int) * (HQ_GRAM_MAX + 4));
      if (sm && w->gperm) {
        w->gG = sm;
        w->gR1 = sm + sq;
        w->gR2 = sm + 2 * sq;
        w->gRi = sm + 3 * sq;
        w->gLU = sm + 4 * sq;
        w->gRH = sm + 5 * sq;
        w->gsgn = sm + 6 * sq;
        w->gtau = w->gsgn + HQ_GRAM_MAX;
        w->gemax = (unsigned long long*)(w->gtau + HQ_GRAM_MAX);
        w->gstat = w->gperm + HQ_GRAM_MAX;
        w->galt = w->gstat + 1;
        w->gcount = w->gstat + 2;
      }
    }
  }
  w->ph_override = -1;
  if (w->failed) return HQ_E_NOMEM;
  CK(cudaMemsetAsync(w->err, 0, sizeof(int) * 2, w->st));
  if (w->gcount) CK(cudaMemsetAsync(w->gcount, 0, sizeof(int) * 2, w->st));
  prof_start(w);
  return HQ_OK;
}

/* Read the device error word; 0 if clean. */
static int ws_check(hq_ws* w) {
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, w->err, sizeof(int), cudaMemcpyDeviceToHost, w->st));
  CK(cudaStreamSynchronize(w->st));
  prof_finish(w);
  if (herr != 0) {
    set_err("device kernel reported error 0x%x%s", herr,
            herr == HQ_ERR_BARRIER_TIMEOUT ? " (grid barrier wait gave up)" : "");
    return HQ_E_DEVICE;
  }
  return HQ_OK;
}

#define DG(ta, tb, M, N, K, al, A, lda, B, ldb, be, C, ldc)                              \
  CK(hq_dgemm(w->st, dev, ta, tb, M, N, K, al, A, lda, B, ldb, be, C, ldc, w->ws,       \
              w->ws_elems))

/* sign * X Y^T (mode 0: written to C; mode 1: added to C) with split-BF16
 * tensor-core products: X has M rows (element (r, k) at X[r*xrs + k*xks]),
 * Y has N rows, both K long; C element (r, c) at C[r*crs + c*ccs].
 * y_raw: Y's rows' largest exponent fields, when known (one-pass split);
 * c_exp: short products in mode 1 write C's columns' largest exponent fields
 * over rows >= c_row_lo there. */
static int ozk_product_x(hq_ws* w, int S, int M, int N, int K, const double* X, long long xrs,
                         long long xks, const double* Y, long long yrs, long long yks, int mode,
                         double sign, double* Cm, long long crs, long long ccs, const int* y_raw,
                         int* c_exp, int c_row_lo, const void* xt, const int* xe) {
  if (M <= 0 || N <= 0) return HQ_OK;
  const int short_k = hq_ozk_short_ok(K);
  /* xt / xe: X already split (M side), e.g. U's digits shared by a block's
   * products. */
  const void* at = xt ? xt : w->ozA;
  const int* ae = xt ? xe : w->ozea;
  const int ovr = w->ph_override;
  const int yside = short_k ? 2 : 1;
  if (!xt && X == Y && xrs == yrs && xks == yks && M == N && S == OZK_SLICES && K >= 512 &&
      (y_raw || w->ozraw)) {
    /* A Gram product (both operands the same matrix): one pass of row maxima
     * for both splits, or none when they are known (y_raw). */
    const int* raw = y_raw;
    if (!raw) {
      const int rt = imax(hq_ozk_split_rows(M, 0), hq_ozk_split_rows(N, yside));
      CK(hq_ozk_rowmax_raw(w->st, X, xrs, xks, M, K, rt, w->ozraw));
      raw = w->ozraw;
    }
    CK(hq_ozk_split_raw(w->st, X, xrs, xks, M, K, S, 0, w->ozA, w->ozea, raw));
    CK(hq_ozk_split_raw(w->st, Y, yrs, yks, N, K, S, yside, w->ozB, w->ozeb, raw));
  } else {
    if (!xt) CK(hq_ozk_split(w->st, X, xrs, xks, M, K, S, 0, w->ozA, w->ozea, w->ozraw));
    if (y_raw)
      CK(hq_ozk_split_raw(w->st, Y, yrs, yks, N, K, S, yside, w->ozB, w->ozeb, y_raw));
    else
      CK(hq_ozk_split(w->st, Y, yrs, yks, N, K, S, yside, w->ozB, w->ozeb, w->ozraw));
  }
  prof_mark(w, ovr >= 0 ? ovr : PH_SPLIT, 0.0);
  if (short_k)
    CK(hq_ozk_gemm_short(w->st, &w->ds->dev, M, N, K, S, at, ae, w->ozB, w->ozeb, mode, sign, Cm,
                         crs, ccs, c_exp, c_row_lo, w->err, spin_limit()));
  else
    CK(hq_ozk_gemm(w->st, &w->ds->dev, M, N, K, S, at, ae, w->ozB, w->ozeb, mode, sign, Cm, crs,
                   ccs, w->ws, w->ws_elems, w->err, spin_limit()));
  /* flops charged: the BF16 tensor work, S(S+1)/2 digit products (none
   * when the interval belongs to another phase, which charges its own) */
  if (ovr >= 0)
    prof_mark(w, ovr, 0.0);
  else
    prof_mark(w, PH_TENSOR, (double)S * (S + 1) * M * N * (double)K);
  return HQ_OK;
}

static int ozk_product(hq_ws* w, int S, int M, int N, int K, const double* X, long long xrs,
                       long long xks, const double* Y, long long yrs, long long yks, int mode,
                       double sign, double* Cm, long long crs, long long ccs) {
  return ozk_product_x(w, S, M, N, K, X, xrs, xks, Y, yrs, yks, mode, sign, Cm, crs, ccs, NULL,
                       NULL, 0, NULL, NULL);
}

/* Split U' (mp x b, w->U) once for the block: as U'^T (b rows, K = mp) and
 * as U' (mp rows, K = b), both M-side digit tiles. */
static int split_block_u(hq_ws* w, int mp, int b) {
  CK(hq_ozk_split(w->st, w->U, w->ldu, 1, b, mp, OZK_SLICES, 0, w->ozUT, w->ozUTe, w->ozraw));
  CK(hq_ozk_split(w->st, w->U, 1, w->ldu, mp, b, OZK_SLICES, 0, w->ozU, w->ozUe, w->ozraw));
  prof_mark(w, PH_SPLIT, 0.0);
  return HQ_OK;
}

static int side_stream(hq_ws* w) {
  if (w->side) return HQ_OK;
  int lo = 0, hi = 0;
  CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
  CK(cudaEventCreateWithFlags(&w->ev_gram, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&w->ev_t, cudaEventDisableTiming));
  CK(cudaStreamCreateWithPriority(&w->side, cudaStreamNonBlocking, hi));
  return HQ_OK;
}

/* Copy-back of finished columns for host-pointer calls.  drain_begin arms it
 * when the host matrix is page-locked (an asynchronous copy from pageable
 * memory would block the enqueueing thread); drain_cols sends columns
 * [drain_done, c1) once the work on st that finishes them is enqueued;
 * drain_finish sends the rest on st and orders st after the copy stream. */
static void drain_begin(hq_ws* w, double* host, int lda, const double* dev, int ldda, int rows) {
  struct cudaPointerAttributes at;
  w->drain_host = NULL;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError(); /* pageable memory on older runtimes: not an error */
    return;
  }
  if (at.type != cudaMemoryTypeHost) return;
  w->drain_host = host;
  w->drain_dev = dev;
  w->drain_lda = lda;
  w->drain_ldda = ldda;
  w->drain_rows = rows;
  w->drain_done = 0;
}

static int drain_cols(hq_ws* w, int c1) {
  if (!w->drain_host || c1 <= w->drain_done) return HQ_OK;
  if (!w->cp) {
    CK(cudaStreamCreateWithFlags(&w->cp, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&w->ev_cp, cudaEventDisableTiming));
  }
  const int c0 = w->drain_done;
  CK(cudaEventRecord(w->ev_cp, w->st));
  CK(cudaStreamWaitEvent(w->cp, w->ev_cp, 0));
  CK(cudaMemcpy2DAsync(w->drain_host + (size_t)c0 * w->drain_lda, sizeof(double) * w->drain_lda,
                       w->drain_dev + (size_t)c0 * w->drain_ldda, sizeof(double) * w->drain_ldda,
                       sizeof(double) * w->drain_rows, c1 - c0, cudaMemcpyDeviceToHost, w->cp));
  w->drain_done = c1;
  return HQ_OK;
}

/* The columns not yet sent (all of them when draining is off), on st. */
static int drain_finish(hq_ws* w, double* host, int lda, const double* dev, int ldda, int rows,
                        int n) {
  const int c0 = w->drain_host ? w->drain_done : 0;
  if (w->cp) {
    CK(cudaEventRecord(w->ev_cp, w->cp));
    CK(cudaStreamWaitEvent(w->st, w->ev_cp, 0));
  }
  if (c0 < n)
    CK(cudaMemcpy2DAsync(host + (size_t)c0 * lda, sizeof(double) * lda, dev + (size_t)c0 * ldda,
                         sizeof(double) * ldda, sizeof(double) * rows, n - c0,
                         cudaMemcpyDeviceToHost, w->st));
  return HQ_OK;
}

/* Build T for the b reflectors in U (mp rows) and apply Q^T from the left to
 * C (mp x nc2): the dlarfb('L','T','F','C') of ...var4.c:711-740.
 *
 * Mixed mode: w->U holds U' = U - [I_b; 0] (the unit diagonal removed).  A
 * split-digit product scales each operand row by its largest entry; with the
 * unit diagonal present that scale is 1 and the small entries below it lose
 * ~2^-47 over long dot products.  The identity's share is exact algebra added
 * in FP64: U^T U = U'^T U' + L + L^T + I, U^T C = U'^T C + C[0:b, :],
 * U W2 = U' W2 + [W2; 0]. */
/* Mixed mode: factor block j's panel [j, j + b) x [j, m) with the Gram panel
 * (qrp_gram.cu): Gram and CholeskyQR2 products on the tensor cores, the
 * b x b factorizations in small kernels (the pivoted first pass in FP32 on
 * one SM, the FP64 Cholesky and LU on a cluster), Householder
 * reconstruction.  The panel's
 * pivots are applied to all m rows of its columns and to jpvt before the
 * products; the factorization is written by the commit kernel only when
 * every step succeeded (*gstat == 0), and otherwise the cooperative panel
 * that follows on the stream factors the (permuted) panel itself. */
static int gram_panel(hq_ws* w, int m, int j, int b, int piv, double* AR, int ldda, int* jp,
                      double* tau, const int* raw) {
  const int mp = m - j, L = HQ_GRAM_MAX, S = OZK_SLICES;
  double* ABR = AR + j;
  int rc;
  w->ph_override = PH_PANEL;
  /* G = Ap^T Ap; R1, P (pivoted Cholesky); R1^{-1}.  raw: the panel
   * columns' largest exponent fields over rows >= j, when the previous
   * block's update recorded them (its product needs no row-maximum pass). */
  rc = ozk_product_x(w, S, b, b, mp, ABR, ldda, 1, ABR, ldda, 1, 0, 1.0, w->gG, 1, L, raw, NULL,
                     0, NULL, NULL);
  if (rc) return rc;
  if (piv) {
    CK(hq_gram_pchol32(w->st, b, w->gG, L, w->gR1, L, w->gperm, w->gstat, 1, w->galt,
                       w->gemax));
  } else {
    CK(hq_fill_iota(w->st, w->gperm, b, 0));
    CK(cudaMemsetAsync(w->gstat, 0, 2 * sizeof(int), w->st)); /* gstat, galt */
    CK(cudaMemsetAsync(w->gemax, 0, sizeof(unsigned long long), w->st));
    CK(hq_cluster_fact(w->st, b, 0, w->gG, L, w->gR1, L, NULL, NULL, w->gstat, 1, NULL));
  }
  CK(hq_tri(w->st, b, 0, w->gR1, L, NULL, 0, NULL, w->gRi, L, NULL));
  CK(hq_permute_cols(w->st, m, AR, ldda, b, w->gperm, w->tmp, jp, w->label_tmp));
  /* Q1 = Ap P R1^{-1}; G2 = Q1^T Q1; R2; Q = Q1 R2^{-1} (in place) */
  rc = ozk_product(w, S, mp, b, b, ABR, 1, ldda, w->gRi, L, 1, 0, 1.0, w->gQ, 1, w->ldu);
  if (!rc) rc = ozk_product(w, S, b, b, mp, w->gQ, w->ldu, 1, w->gQ, w->ldu, 1, 0, 1.0, w->gG, 1, L);
  if (rc) return rc;
  /* R2 and R2^{-1}: fixed-point steps when G2 is near the identity, else
   * (galt set by the first step) the cluster Cholesky and an inverse */
  CK(hq_nearid_chol(w->st, b, w->gG, L, w->gR2, w->gRi, w->gLU, w->gRH, L, w->galt,
                    w->gemax));
  CK(hq_cluster_fact(w->st, b, 0, w->gG, L, w->gR2, L, NULL, NULL, w->gstat, 2, w->galt));
  CK(hq_tri(w->st, b, 0, w->gR2, L, NULL, 0, NULL, w->gRi, L, w->galt));
  rc = ozk_product(w, S, mp, b, b, w->gQ, 1, w->ldu, w->gRi, L, 1, 0, 1.0, w->gQ, 1, w->ldu);
  if (rc) return rc;
  /* Q11 - D = L U; R = D R2 R1; V2 = Q2 U^{-1} (into U's rows >= b) */
  CK(hq_cluster_fact(w->st, b, 1, w->gQ, w->ldu, w->gLU, L, w->gsgn, w->gtau, w->gstat, 4, NULL));
  /* R_H = D R2 R1 and U^{-1}, one launch */
  CK(hq_tri2(w->st, b, 1, w->gR2, L, w->gR1, L, w->gsgn, w->gRH, L, mp > b ? 0 : -1, w->gLU, L,
             NULL, 0, NULL, w->gRi, L));
  if (mp > b) {
    rc = ozk_product(w, S, mp - b, b, b, w->gQ + b, 1, w->ldu, w->gRi, L, 1, 0, 1.0, w->U + b, 1,
                     w->ldu);
    if (rc) return rc;
  }
  CK(hq_gram_commit(w->st, mp, b, ABR, ldda, w->U, w->ldu, w->gRH, L, w->gLU, L, w->gtau, tau,
                    w->perm, w->gstat, w->gcount));
  w->ph_override = -1;
  return HQ_OK;
}

static int block_reflector(hq_ws* w, int mp, int b, const double* tau, double* Cm, int ldc,
                           int nc2, const int* cx_in, int* cx_out) {
  const hq_device_info* dev = &w->ds->dev;
  if (w->mixed) {
    int rc = split_block_u(w, mp, b);
    if (rc) return rc;
    rc = ozk_product_x(w, OZK_SLICES, b, b, mp, w->U, w->ldu, 1, w->U, w->ldu, 1, 0, 1.0, w->Z, 1,
                       w->ldz, NULL, NULL, 0, w->ozUT, w->ozUTe);
    if (rc) return rc;
    CK(hq_gram_unit_fix(w->st, b, w->U, w->ldu, w->Z, w->ldz));
  } else {
    DG('T', 'N', b, b, mp, 1.0, w->U, w->ldu, w->U, w->ldu, 0.0, w->Z, w->ldz);
  }
  /* T (one SM, a sequential recurrence) on the side stream, overlapped with
   * W1 = U^T C, which does not need it; st waits for T before W2. */
  int rs = side_stream(w);
  if (rs) return rs;
  CK(cudaEventRecord(w->ev_gram, w->st));
  CK(cudaStreamWaitEvent(w->side, w->ev_gram, 0));
  CK(hq_larft_from_gram(w->side, b, w->Z, w->ldz, tau, w->T, w->ldt));
  CK(cudaEventRecord(w->ev_t, w->side));
  prof_mark(w, PH_PANEL, w->mixed ? 0.0 : 2.0 * mp * b * b);
  if (nc2 > 0 && w->mixed) {
    /* W1 = U^T C, W2 = T^T W1 and C -= U W2 on the tensor cores. */
    /* cx_in: C's columns' largest exponent fields (from the previous update);
     * cx_out: the same for the next block, over rows >= b of the new C. */
    int rc = HQ_OK, done = 0;
    /* HQRRP_GB300_SPLIT_TRAILING=1 keeps the separate split pass (the same
     * digits; for verification). */
    const char* split_env = getenv("HQRRP_GB300_SPLIT_TRAILING");
    if (cx_in && !(split_env && split_env[0] == '1')) {
      /* C's column exponents are known: the product reads C as FP64 and cuts
       * it into digits on the fly (no split pass over the trailing matrix). */
      const int e = hq_ozk_gemm_c64(w->st, &w->ds->dev, b, nc2, mp, w->ozUT, w->ozUTe, Cm, ldc,
                                    cx_in, 1.0, w->W1, 1, w->ldw, w->ws, w->ws_elems, w->err,
                                    spin_limit());
      if (e != (int)cudaErrorNotSupported) {
        CK(e);
        prof_mark(w, PH_TENSOR, (double)OZK_SLICES * (OZK_SLICES + 1) * b * nc2 * (double)mp);
        done = 1;
      }
    }
    if (!done)
      rc = ozk_product_x(w, OZK_SLICES, b, nc2, mp, w->U, w->ldu, 1, Cm, ldc, 1, 0, 1.0, w->W1, 1,
                         w->ldw, cx_in, NULL, 0, w->ozUT, w->ozUTe);
    if (rc) return rc;
    CK(hq_add_matrix(w->st, b, nc2, 1.0, Cm, ldc, w->W1, w->ldw));
    CK(cudaStreamWaitEvent(w->st, w->ev_t, 0));
    rc = ozk_product(w, OZK_SLICES, b, nc2, b, w->T, w->ldt, 1, w->W1, w->ldw, 1, 0, 1.0, w->W2, 1,
                     w->ldw);
    if (rc) return rc;
    if (cx_out) CK(hq_zero_words(w->st, cx_out, (size_t)nc2, NULL, 0));
    rc = ozk_product_x(w, OZK_SLICES, mp, nc2, b, w->U, 1, w->ldu, w->W2, w->ldw, 1, 1, -1.0, Cm,
                       1, ldc, NULL, cx_out, b, w->ozU, w->ozUe);
    if (rc) return rc;
    CK(hq_add_matrix(w->st, b, nc2, -1.0, w->W2, w->ldw, Cm, ldc));
  } else if (nc2 > 0) {
    DG('T', 'N', b, nc2, mp, 1.0, w->U, w->ldu, Cm, ldc, 0.0, w->W1, w->ldw);
    CK(cudaStreamWaitEvent(w->st, w->ev_t, 0));
    DG('T', 'N', b, nc2, b, 1.0, w->T, w->ldt, w->W1, w->ldw, 0.0, w->W2, w->ldw);
    DG('N', 'N', mp, nc2, b, -1.0, w->U, w->ldu, w->W2, w->ldw, 1.0, Cm, ldc);
    prof_mark(w, PH_UPDATE, 4.0 * mp * b * nc2 + (double)b * b * nc2);
  }
  /* T is read after this call (the sketch downdate, the next block). */
  CK(cudaStreamWaitEvent(w->st, w->ev_t, 0));
  return HQ_OK;
}

/* ------------------------------------------------------------------------ */
/* HQRRP block loop (...var4.c:403-558) on device data.                      */

/* kmax < min(m, n) stops after the first kmax columns (the truncated
 * factorization: R's first kmax rows and their reflectors); the last block
 * then skips the sketch downdate nothing would read. */
static int core_hqrrp_k(hq_ws* w, int m, int n, double* dA, int ldda, int* djpvt, double* dtau,
                        int nb, int pp, int panel_piv, const double* dG, int lddg,
                        unsigned long long seed, int kmax) {
  const hq_device_info* dev = &w->ds->dev;
  const int mY = nb + pp, mn = imin(imin(m, n), kmax);
  const unsigned spin = spin_limit();
  if (mn == 0) return HQ_OK;

  /* Sketch G and Y = G A. */
  NV_PUSH("hqrrp.sketch");
  if (dG) CK(hq_copy_matrix(w->st, mY, m, dG, lddg, w->G, w->ldg));
  else CK(hq_sketch_philox(w->st, mY, m, w->G, w->ldg, seed));
  if (w->mixed) {
    /* Y^T = A^T G^T with two-digit BF16 operands: the sketch only steers pivots. */
    prof_mark(w, PH_SKETCH, 0.0);
    int rc = ozk_product(w, OZK_SKETCH_SLICES, n, mY, m, dA, ldda, 1, w->G, 1, w->ldg, 0, 1.0,
                         w->Y, w->ldy, 1);
    if (rc) return rc;
  } else {
    DG('N', 'N', mY, n, m, 1.0, w->G, w->ldg, dA, ldda, 0.0, w->Y, w->ldy);
    prof_mark(w, PH_SKETCH, 2.0 * mY * m * n);
  }
  NV_POP();

  int cx_ok = 0; /* w->colexp holds the trailing columns' exponent fields */
  /* HQRRP_GB300_SPLIT_TRAILING=1: the separate split and row-maximum passes
   * everywhere (the same digits; for verification). */
  const char* split_env = getenv("HQRRP_GB300_SPLIT_TRAILING");
  const int split_passes = split_env && split_env[0] == '1';
  for (int j = 0; j < mn; j += nb) {
    const int b = imin(imin(nb, mn - j), imin(n - j, m - j));
    const int last = (j + nb >= m) || (j + nb >= n);
    const int final_block = j + b >= mn;
    const int mp = m - j, nc2 = imax(0, n - j - b);
    double* AR = dA + (size_t)j * ldda;
    double* ABR = AR + j;
    double* YR = w->Y + (size_t)j * w->ldy;

    NV_PUSH("hqrrp.block");
    if (!last) {
      NV_PUSH("hqrrp.select");
      /* Pivot selection on the sketch, then one gather of A, Y and jpvt. */
      /* Mixed: the sketch's reflector applications in FP32 (it is formed from
       * two-digit BF16 operands and only steers pivots); norms stay FP64. */
      CK(hq_skinny_qrp(w->st, dev, mY, n - j, b, YR, w->ldy, w->V, w->ldy, w->pairs, w->npairs,
                       w->part, w->part_elems, w->bar, w->err, spin, w->mixed));
      CK(hq_permute_pairs(w->st, m, AR, ldda, n - j, w->pairs, w->npairs, 2 * b, w->tmp,
                          djpvt + j, w->label_tmp));
      CK(hq_permute_pairs(w->st, mY, YR, w->ldy, n - j, w->pairs, w->npairs, 2 * b, w->tmp,
                          cx_ok ? w->colexp + j : NULL, cx_ok ? w->label_tmp : NULL));
      double fl = 0.0;
      for (int s2 = 0; s2 < b; ++s2) fl += 4.0 * (mY - s2) * (n - j - s2 - 1);
      prof_mark(w, PH_SELECT, fl);
      NV_POP();
    }

    NV_PUSH("hqrrp.panel");
    /* Panel QR (pivoted within its b columns), U, tau. */
    /* Mixed: squared column norms in the panel's pivoting (division-free
     * LAWN 176 downdate); plain keeps LAPACK's formula. */
    const int use_gram = w->gram && w->gQ && !w->ut && b <= HQ_GRAM_MAX;
    if (use_gram) {
      int rc = gram_panel(w, m, j, b, panel_piv, AR, ldda, djpvt + j, dtau + j,
                          cx_ok && !split_passes ? w->colexp + j : NULL);
      if (rc) return rc;
    }
    CK(hq_panel_qrp_fallback(w->st, dev, mp, b, panel_piv, ABR, ldda, dtau + j, w->U, w->ldu,
                             w->perm, w->part, w->part_elems, w->rowbuf, w->bar + 1, w->err,
                             spin, w->mixed, w->ut, use_gram ? w->gstat : NULL));
    if (w->mixed) CK(hq_set_diag(w->st, b, w->U, w->ldu, 0.0)); /* U' for the digit products */
    /* The panel's swaps on the rows above it and on the labels. */
    CK(hq_permute_cols(w->st, j, AR, ldda, b, w->perm, w->tmp, djpvt + j, w->label_tmp));
    /* Columns [j, j + b) are final: later blocks touch only columns >= j + b. */
    if (w->drain_host) {
      int rc = drain_cols(w, j + b);
      if (rc) return rc;
    }
    {
      double fl = 0.0;
      for (int s2 = 0; s2 < b; ++s2) fl += 4.0 * (mp - s2) * (b - s2 - 1);
      prof_mark(w, PH_PANEL, fl);
    }
    NV_POP();

    /* T and the trailing update [A12; A22] := Q^T [A12; A22]. */
    int* cx_out = (w->mixed && w->colexp && nc2 > 0) ? w->colexp + j + b : NULL;
    NV_PUSH("hqrrp.update");
    int rc = block_reflector(w, mp, b, dtau + j, ABR + (size_t)b * ldda, ldda, nc2,
                             cx_ok ? w->colexp + j + b : NULL, cx_out);
    NV_POP();
    if (rc) return rc;
    cx_ok = cx_out != NULL;

    if (!last && !(final_block && mn < imin(m, n))) {
      NV_PUSH("hqrrp.downdate");
      /* Sketch downdate (...var4.c:617-708):
       *   G_R := G_R (I - U T U^T);  Y2 -= G_R[:, 0:b] R12. */
      double* GR = w->G + (size_t)j * w->ldg;
      if (w->mixed) {
        /* B^T = U^T G_R^T; G_R^T -= U B2^T; Y2^T -= R12^T G1^T (transposed so the
         * long dimension is the 128-row tile side). */
        /* U holds U' (unit diagonal removed): Bm = G_R U' + G_R[:, 0:b] and
         * G_R -= B2 U'^T + [B2, 0]. */
        int rc = ozk_product_x(w, OZK_SLICES, b, mY, mp, w->U, w->ldu, 1, GR, 1, w->ldg, 0, 1.0,
                               w->Bm, w->ldb, 1, NULL, NULL, 0, w->ozUT, w->ozUTe);
        if (rc) return rc;
        CK(hq_add_matrix(w->st, mY, b, 1.0, GR, w->ldg, w->Bm, w->ldb));
        /* B2 = Bm T (mY x b x b): too few tiles for the FP64 kernel to fill the GPU. */
        rc = ozk_product(w, OZK_SLICES, mY, b, b, w->Bm, 1, w->ldb, w->T, w->ldt, 1, 0, 1.0, w->B2,
                         1, w->ldb);
        if (rc) return rc;
        rc = ozk_product_x(w, OZK_SLICES, mp, mY, b, w->U, 1, w->ldu, w->B2, 1, w->ldb, 1, -1.0, GR,
                           w->ldg, 1, NULL, NULL, 0, w->ozU, w->ozUe);
        if (rc) return rc;
        CK(hq_add_matrix(w->st, mY, b, -1.0, w->B2, w->ldb, GR, w->ldg));
        rc = ozk_product(w, OZK_SLICES, nc2, mY, b, ABR + (size_t)b * ldda, ldda, 1, GR, 1, w->ldg,
                         1, -1.0, YR + (size_t)b * w->ldy, w->ldy, 1);
        if (rc) return rc;
      } else {
        DG('N', 'N', mY, b, mp, 1.0, GR, w->ldg, w->U, w->ldu, 0.0, w->Bm, w->ldb);
        DG('N', 'N', mY, b, b, 1.0, w->Bm, w->ldb, w->T, w->ldt, 0.0, w->B2, w->ldb);
        DG('N', 'T', mY, mp, b, -1.0, w->B2, w->ldb, w->U, w->ldu, 1.0, GR, w->ldg);
        DG('N', 'N', mY, nc2, b, -1.0, GR, w->ldg, ABR + (size_t)b * ldda, ldda, 1.0,
           YR + (size_t)b * w->ldy, w->ldy);
        prof_mark(w, PH_DOWNDATE, 4.0 * mY * mp * b + 2.0 * mY * b * b + 2.0 * mY * b * nc2);
      }
      NV_POP();
    }
    NV_POP();
  }
  return HQ_OK;
}

static int core_hqrrp(hq_ws* w, int m, int n, double* dA, int ldda, int* djpvt, double* dtau,
                      int nb, int pp, int panel_piv, const double* dG, int lddg,
                      unsigned long long seed) {
  return core_hqrrp_k(w, m, n, dA, ldda, djpvt, dtau, nb, pp, panel_piv, dG, lddg, seed,
                      imin(m, n));
}

static int check_hqrrp_shape(int nb, int pp) {
  if (nb < 1 || pp < 0 || nb + pp > HQ_MAX_MY) {
    set_err("unsupported block parameters nb=%d pp=%d (need nb >= 1, pp >= 0, nb+pp <= %d)", nb,
            pp, HQ_MAX_MY);
    return HQ_E_UNSUPPORTED;
  }
  return HQ_OK;
}

static int ws_begin(hq_ws* w, cudaStream_t user_stream, int use_user) {
  memset(w, 0, sizeof *w);
  w->ds = current_device();
  if (!w->ds) return HQ_E_CUDA;
  w->st = use_user ? user_stream : w->ds->stream;
  w->mixed = precision() == 1;
  return HQ_OK;
}

/* Host-pointer HQRRP: copy in, factor, copy out. */
static int hqrrp_host(int m, int n, double* A, int lda, int* jpvt, double* tau, int nb, int pp,
                      int panel_piv, const double* G, int ldg, int ut) {
  int rc = check_hqrrp_shape(nb, pp);
  if (rc) return rc;
  hq_ws w;
  if ((rc = ws_begin(&w, NULL, 0))) return rc;
  w.ut = ut;
  const int mn = imin(m, n), mY = nb + pp, ldda = round_up(m, 32);
  rc = ws_setup(&w, m, n, nb, pp, nb);
  double* dA = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)ldda * n);
  double* dtau = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)mn);
  int* djp = rc ? NULL : ws_alloc(&w, sizeof(int) * (size_t)n);
  double* dG = (rc || !G) ? NULL : ws_alloc(&w, sizeof(double) * (size_t)mY * m);
  if (w.failed) rc = HQ_E_NOMEM;
  cudaStream_t st = w.st;
#define CKF(call)                                                            \
  do {                                                                       \
    if (!rc) {                                                               \
      int e_ = (int)(call);                                                  \
      if (e_) {                                                              \
        set_err("%s failed: %s", #call, cudaGetErrorString((cudaError_t)e_)); \
        rc = HQ_E_CUDA;                                                      \
      }                                                                      \
    }                                                                        \
  } while (0)
  CKF(cudaMemcpy2DAsync(dA, sizeof(double) * ldda, A, sizeof(double) * lda, sizeof(double) * m, n,
                        cudaMemcpyHostToDevice, st));
  CKF(cudaMemcpyAsync(djp, jpvt, sizeof(int) * n, cudaMemcpyHostToDevice, st));
  if (G) CKF(cudaMemcpy2DAsync(dG, sizeof(double) * mY, G, sizeof(double) * ldg,
                               sizeof(double) * mY, m, cudaMemcpyHostToDevice, st));
  if (!rc) drain_begin(&w, A, lda, dA, ldda, m);
  if (!rc) rc = core_hqrrp(&w, m, n, dA, ldda, djp, dtau, nb, pp, panel_piv, dG, mY, g_seed);
  if (!rc) rc = drain_finish(&w, A, lda, dA, ldda, m, n);
  if (!rc) rc = ws_check(&w);
  CKF(cudaMemcpyAsync(jpvt, djp, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  CKF(cudaMemcpyAsync(tau, dtau, sizeof(double) * mn, cudaMemcpyDeviceToHost, st));
  ws_release(&w);
  CKF(cudaStreamSynchronize(st));
  return rc;
}

static int hqrrp_args_ok(int m, int n, int lda) {
  int bad = 0;
  if (m < 0) { fprintf(stderr, "ERROR in NoFLA_HQRRP_WY_blk_var4: m_A is < 0.\n"); bad = 1; }
  if (n < 0) { fprintf(stderr, "ERROR in NoFLA_HQRRP_WY_blk_var4: n_A is < 0.\n"); bad = 1; }
  if (lda < imax(1, m)) {
    fprintf(stderr, "ERROR in NoFLA_HQRRP_WY_blk_var4: ldim_A is < max( 1, m_A ).\n");
    bad = 1;
  }
  return !bad;
}

HQ_API int NoFLA_HQRRP_WY_blk_var4(int m_A, int n_A, double* buff_A, int ldim_A, int* buff_jpvt,
                                   double* buff_tau, int nb_alg, int pp, int panel_pivoting) {
  g_err[0] = 0;
  if (!hqrrp_args_ok(m_A, n_A, ldim_A)) return 0;
  if (imin(m_A, n_A) == 0) return 0;
  return hqrrp_host(m_A, n_A, buff_A, ldim_A, buff_jpvt, buff_tau, nb_alg, pp, panel_pivoting,
                    NULL, 0, 0);
}

HQ_API int hqrrp_gb300_hqrrp_sketch(int m, int n, double* A, int lda, int* jpvt, double* tau,
                                    int nb, int pp, int panel_pivoting, const double* G, int ldg) {
  g_err[0] = 0;
  if (!hqrrp_args_ok(m, n, lda)) return 0;
  if (imin(m, n) == 0) return 0;
  if (G == NULL || ldg < nb + pp) {
    set_err("explicit sketch missing or ldg < nb + pp");
    return HQ_E_UNSUPPORTED;
  }
  return hqrrp_host(m, n, A, lda, jpvt, tau, nb, pp, panel_pivoting, G, ldg, 0);
}

/* ---- The UT-transform variant behind a libflame-like object API -------- */

/* Element k of a vector view: an n x 1 view (stride 1) or a 1 x n view
 * (stride col_stride). */
static size_t obj_vec_stride(const hqrrp_gb300_obj* v) {
  return v->n == 1 ? 1u : (size_t)v->col_stride;
}

static int obj_vec_len(const hqrrp_gb300_obj* v) { return v->n == 1 ? v->m : (v->m == 1 ? v->n : -1); }

static int ut_entry(hqrrp_gb300_obj A, hqrrp_gb300_obj p, hqrrp_gb300_obj s, int nb_alg, int pp,
                    int panel_pivoting, const double* G, int ldg) {
  g_err[0] = 0;
  if (A.datatype != HQRRP_GB300_DOUBLE || p.datatype != HQRRP_GB300_INT ||
      s.datatype != HQRRP_GB300_DOUBLE) {
    set_err("FLA_HQRRP_UT_blk_var2: A and s must be double, p int objects");
    return HQ_E_UNSUPPORTED;
  }
  const int m = A.m, n = A.n, mn = imin(m, n);
  if (m < 0 || n < 0 || A.col_stride < imax(1, m) || (mn > 0 && !A.buffer)) {
    set_err("FLA_HQRRP_UT_blk_var2: invalid A view");
    return HQ_E_UNSUPPORTED;
  }
  if (mn == 0) return 0; /* :179-182 */
  if (obj_vec_len(&p) < n || obj_vec_len(&s) < mn || !p.buffer || !s.buffer ||
      (p.n != 1 && p.col_stride < 1) || (s.n != 1 && s.col_stride < 1)) {
    set_err("FLA_HQRRP_UT_blk_var2: p needs n, s min(m, n) elements (vector views)");
    return HQ_E_UNSUPPORTED;
  }
  int* jp = malloc(sizeof(int) * (size_t)n);
  double* tau = malloc(sizeof(double) * (size_t)mn);
  if (!jp || !tau) {
    free(jp);
    free(tau);
    set_err("host allocation failed");
    return HQ_E_NOMEM;
  }
  const size_t ps = obj_vec_stride(&p), ss = obj_vec_stride(&s);
  for (int k = 0; k < n; ++k) jp[k] = ((const int*)p.buffer)[k * ps];
  int rc = hqrrp_host(m, n, (double*)A.buffer, A.col_stride, jp, tau, nb_alg, pp, panel_pivoting,
                      G, ldg, 1);
  if (!rc) {
    for (int k = 0; k < n; ++k) ((int*)p.buffer)[k * ps] = jp[k];
    /* The UT transform's scalar of H = I - u u^T / tau_UT is 1 / tau. */
    for (int k = 0; k < mn; ++k) ((double*)s.buffer)[k * ss] = 1.0 / tau[k];
  }
  free(jp);
  free(tau);
  return rc;
}

HQ_API int hqrrp_gb300_ut_blk_var2(hqrrp_gb300_obj A, hqrrp_gb300_obj p, hqrrp_gb300_obj s,
                                   int nb_alg, int pp, int panel_pivoting) {
  return ut_entry(A, p, s, nb_alg, pp, panel_pivoting, NULL, 0);
}

HQ_API int hqrrp_gb300_ut_blk_var2_sketch(hqrrp_gb300_obj A, hqrrp_gb300_obj p,
                                          hqrrp_gb300_obj s, int nb_alg, int pp,
                                          int panel_pivoting, const double* G, int ldg) {
  if (G == NULL || ldg < nb_alg + pp) {
    g_err[0] = 0;
    set_err("explicit sketch missing or ldg < nb + pp");
    return HQ_E_UNSUPPORTED;
  }
  return ut_entry(A, p, s, nb_alg, pp, panel_pivoting, G, ldg);
}

HQ_API int hqrrp_gb300_hqrrp_device(int m, int n, double* dA, int ldda, int* d_jpvt,
                                    double* d_tau, int nb, int pp, int panel_pivoting,
                                    const double* dG, int lddg, unsigned long long seed,
                                    void* stream) {
  g_err[0] = 0;
  if (m < 0 || n < 0 || ldda < imax(1, m)) {
    set_err("invalid m, n or ldda");
    return HQ_E_UNSUPPORTED;
  }
  if (imin(m, n) == 0) return 0;
  int rc = check_hqrrp_shape(nb, pp);
  if (rc) return rc;
  if (dG && lddg < nb + pp) {
    set_err("lddg < nb + pp");
    return HQ_E_UNSUPPORTED;
  }
  hq_ws w;
  if ((rc = ws_begin(&w, (cudaStream_t)stream, 1))) return rc;
  rc = ws_setup(&w, m, n, nb, pp, nb);
  if (!rc) rc = core_hqrrp(&w, m, n, dA, ldda, d_jpvt, d_tau, nb, pp, panel_pivoting, dG, lddg, seed);
  if (!rc) rc = ws_check(&w);
  ws_release(&w);
  if (!rc) {
    int e = (int)cudaStreamSynchronize(w.st);
    if (e) {
      set_err("cudaStreamSynchronize failed: %s", cudaGetErrorString((cudaError_t)e));
      rc = HQ_E_CUDA;
    }
  }
  return rc;
}

HQ_API int hqrrp_gb300_sketch_device(int rows, int cols, double* dG, int ldg,
                                    unsigned long long seed, void* stream) {
  g_err[0] = 0;
  if (rows < 0 || cols < 0 || ldg < imax(1, rows)) {
    set_err("hqrrp_gb300_sketch_device: invalid rows, cols or ldg");
    return HQ_E_UNSUPPORTED;
  }
  if (rows == 0 || cols == 0) return 0;
  if (!current_device()) return HQ_E_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  int e = hq_sketch_philox(st, rows, cols, dG, ldg, seed);
  if (!e) e = (int)cudaStreamSynchronize(st);
  if (e) {
    set_err("hqrrp_gb300_sketch_device: %s", cudaGetErrorString((cudaError_t)e));
    return HQ_E_CUDA;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* dgeqp4 (...var4.c:127-300) on device data.                                */

/* Move the fixed columns (jpvt != 0) to the front exactly as the reference
 * does (...var4.c:201-218, the same loop as LAPACK dgeqp3/dgeqpf), returning
 * their count; hjp is updated in place to 1-based labels and src[k] receives
 * the original column now at position k. */
static int fixed_columns_front(int n, int* hjp, int* src) {
  int nfix = 0;
  for (int k = 0; k < n; ++k) src[k] = k;
  for (int c = 0; c < n; ++c) {
    if (hjp[c] != 0) {
      if (c != nfix) {
        int t = src[c];
        src[c] = src[nfix];
        src[nfix] = t;
        hjp[c] = hjp[nfix];
        hjp[nfix] = c + 1;
      } else {
        hjp[c] = c + 1;
      }
      ++nfix;
    } else {
      hjp[c] = c + 1;
    }
  }
  return nfix;
}

/* Everything of dgeqp4 after argument checking.  hjp: host copy of jpvt (in:
 * fixed marks; out: 1-based permutation).  Returns HQ_* and the LAPACK-style
 * workspace figure in *iws_out. */
/* dG (optional, lddg >= 74): the sketch of the HQRRP branch, 74 x (m - nf)
 * (its first m - nf columns are read); NULL draws Philox(seed). */
static int core_dgeqp4(hq_ws* w, int m, int n, double* dA, int ldda, int* hjp, int* djp,
                       double* dtau, int* iws_out, const double* dG, int lddg) {
  const hq_device_info* dev = &w->ds->dev;
  const int mn = imin(m, n);
  const int small = mn < DGEQP4_SMALL_DGEQP3;
  const unsigned spin = spin_limit();
  int iws = 3 * n + 1;

  /* 1. Fixed columns to the front (host bookkeeping, one device gather). */
  int* src = malloc(sizeof(int) * (size_t)n);
  int* hpairs = malloc(sizeof(int) * 2 * (size_t)n);
  if (!src || !hpairs) {
    free(src);
    free(hpairs);
    set_err("host allocation failed");
    return HQ_E_NOMEM;
  }
  const int nfix = fixed_columns_front(n, hjp, src);
  /* With fixed columns the rows above the free block are permuted at the
   * end, so no column is final early: copy back in one piece. */
  if (nfix > 0) w->drain_host = NULL;
  int np = 0;
  for (int k = 0; k < n; ++k)
    if (src[k] != k) {
      hpairs[2 * np] = k;
      hpairs[2 * np + 1] = src[k];
      ++np;
    }
  free(src);
  CK(cudaMemcpyAsync(djp, hjp, sizeof(int) * n, cudaMemcpyHostToDevice, w->st));
  if (np > 0) {
    int* dpairs = ws_alloc(w, sizeof(int) * 2 * (size_t)np);
    double* dtmp = ws_alloc(w, sizeof(double) * (size_t)m * np);
    if (w->failed) {
      free(hpairs);
      return HQ_E_NOMEM;
    }
    int rc0 = (int)cudaMemcpyAsync(dpairs, hpairs, sizeof(int) * 2 * np, cudaMemcpyHostToDevice,
                                   w->st);
    if (!rc0) rc0 = (int)cudaMemcpyAsync(w->npairs, &np, sizeof(int), cudaMemcpyHostToDevice, w->st);
    if (!rc0) rc0 = (int)cudaStreamSynchronize(w->st); /* hpairs / np are stack/heap */
    if (!rc0)
      rc0 = hq_permute_pairs(w->st, m, dA, ldda, n, dpairs, w->npairs, np, dtmp, NULL, NULL);
    if (rc0) {
      free(hpairs);
      set_err("fixed-column gather failed: %s", cudaGetErrorString((cudaError_t)rc0));
      return HQ_E_CUDA;
    }
  }
  free(hpairs);

  /* 2. Unpivoted blocked QR of the fixed columns, updating all columns to
   *    their right (dgeqrf + dormqr of ...var4.c:220-242). */
  const int nf = imin(m, nfix);
  for (int j = 0; j < nf; j += FIXED_BLOCK) {
    const int b = imin(FIXED_BLOCK, nf - j), mp = m - j;
    double* ABR = dA + j + (size_t)j * ldda;
    CK(hq_panel_qrp(w->st, dev, mp, b, 0, ABR, ldda, dtau + j, w->U, w->ldu, w->perm, w->part,
                    w->part_elems, w->rowbuf, w->bar + 1, w->err, spin, 0, 0));
    if (w->mixed) CK(hq_set_diag(w->st, b, w->U, w->ldu, 0.0)); /* U' for the digit products */
    int rc = block_reflector(w, mp, b, dtau + j, ABR + (size_t)b * ldda, ldda, n - j - b, NULL,
                             NULL);
    if (rc) return rc;
  }
  if (nf > 0) {
    /* The workspace LAPACK's dgeqrf and dormqr would report (reference
     * LAPACK 3.x: N*NB and NW*NB + 65*64). */
    iws = imax(iws, nf * LAPACK_NB_DGEQRF);
    if (nf < n) iws = imax(iws, (n - nf) * LAPACK_NB_DGEQRF + 65 * 64);
  }

  /* 3. The free columns: pivoted QR (small path) or HQRRP(64, 10, 1).  The
   *    permutation of the free block is tracked with position labels and
   *    then applied to the rows above it and to jpvt (...var4.c:267-292). */
  if (nf < mn) {
    const int mt = m - nf, nt = n - nf;
    double* At = dA + nf + (size_t)nf * ldda;
    CK(hq_fill_iota(w->st, w->labels, nt, 0));
    if (small && nt > HQ_MAX_PANEL) {
      /* Wide: min(m, n) < 1000 and more than HQ_MAX_PANEL free columns, so
       * mt < 1000 rows.  The column-partitioned kernel leaves the columns in
       * place and reports the final order as pairs, applied here to all m
       * rows of the free columns (the rows above them included) and to jpvt. */
      const int ns = imin(mt, nt);
      int* phys = ws_alloc(w, sizeof(int) * (size_t)nt);
      long long* cand = ws_alloc(w, sizeof(long long) * hq_wide_cand_elems(dev));
      int* wpairs = ws_alloc(w, sizeof(int) * 4 * (size_t)ns);
      int* wlab = ws_alloc(w, sizeof(int) * 2 * (size_t)ns);
      double* wtmp = ws_alloc(w, sizeof(double) * (size_t)m * 2 * ns);
      if (w->failed) return HQ_E_NOMEM;
      CK(hq_wide_qrp(w->st, dev, mt, nt, At, ldda, dtau + nf, phys, cand, wpairs, w->npairs,
                     w->bar + 1, w->err, spin));
      CK(hq_permute_pairs(w->st, m, dA + (size_t)nf * ldda, ldda, nt, wpairs, w->npairs, 2 * ns,
                          wtmp, djp + nf, wlab));
    } else if (small) {
      CK(hq_panel_qrp(w->st, dev, mt, nt, 1, At, ldda, dtau + nf, NULL, w->ldu, w->perm,
                      w->part, w->part_elems, w->rowbuf, w->bar + 1, w->err, spin, 0, 0));
      CK(hq_permute_cols(w->st, nf, dA + (size_t)nf * ldda, ldda, nt, w->perm, w->tmp,
                         djp + nf, w->label_tmp));
    } else {
      int rc = core_hqrrp(w, mt, nt, At, ldda, w->labels, dtau + nf, w->dq_nb, DGEQP4_PP, 1, dG,
                          lddg, g_seed);
      if (rc) return rc;
      double* t2 = w->tmp;
      if ((size_t)nf * nt > (size_t)w->tmp_rows * w->tmp_cols) {
        t2 = ws_alloc(w, sizeof(double) * (size_t)nf * nt);
        if (!t2) return HQ_E_NOMEM;
      }
      CK(hq_permute_cols(w->st, nf, dA + (size_t)nf * ldda, ldda, nt, w->labels, t2, djp + nf,
                         w->label_tmp));
    }
  }
  /* LAPACK's dgeqp3 also counts the blocked code's workspace for the free
   * block (SN = n - nfix columns), used when NB = 32 and the crossover
   * NX = 128 (ILAENV's DGEQRF values) are both below its min(m, n) - nfix. */
  if (small && nfix < mn) {
    const int sn = n - nfix, sminmn = mn - nfix;
    if (LAPACK_NB_DGEQRF < sminmn && LAPACK_NX_DGEQRF < sminmn)
      iws = imax(iws, 2 * sn + (sn + 1) * LAPACK_NB_DGEQRF);
  }
  *iws_out = iws;
  return HQ_OK;
}

static int dgeqp4_ws(hq_ws* w, int m, int n) {
  const int mn = imin(m, n);
  if (mn < DGEQP4_SMALL_DGEQP3) {
    /* pivoted panel of up to n - nf columns plus fixed blocks */
    int rc = ws_setup(w, m, n, 0, 0, imax(FIXED_BLOCK, imin(n, HQ_MAX_PANEL)));
    return rc;
  }
  return ws_setup(w, m, n, w->dq_nb, DGEQP4_PP, imax(FIXED_BLOCK, w->dq_nb));
}

static void xerbla_dgeqp3(int arg) {
  fprintf(stderr, " ** On entry to DGEQP3 parameter number %2d had an illegal value\n", arg);
}

/* Argument checks and the workspace query of ...var4.c:148-187.  Returns 1
 * when the caller should return immediately. */
static int dgeqp4_prologue(int m, int n, int lda, int lwork, double* work, int* info) {
  const int mn = imin(m, n), query = (lwork == -1);
  *info = 0;
  if (m < 0) *info = -1;
  else if (n < 0) *info = -2;
  else if (lda < imax(1, m)) *info = -4;
  if (*info == 0) {
    int iws = 1, lwkopt = 1;
    if (mn != 0) {
      iws = 3 * n + 1;
      lwkopt = 2 * n + (n + 1) * LAPACK_NB_DGEQRF;
    }
    if (work) work[0] = (double)lwkopt;
    if (work && lwork < iws && !query) *info = -8;
  }
  if (*info != 0) {
    xerbla_dgeqp3(-*info);
    return 1;
  }
  return query || mn == 0;
}

/* Host-pointer dgeqp4; G (optional, ldg >= 74, m columns of which the first
 * m - nf are read) replaces the drawn sketch of the HQRRP branch. */
static void dgeqp4_host(int* m, int* n, double* A, int* lda, int* jpvt, double* tau,
                        double* work, int* lwork, int* info, const double* G, int ldg) {
  g_err[0] = 0;
  if (dgeqp4_prologue(*m, *n, *lda, *lwork, work, info)) return;
  const int M = *m, N = *n, LDA = *lda, mn = imin(M, N), ldda = round_up(M, 32);
  const int mY = DGEQP4_NB + DGEQP4_PP;
  hq_ws w;
  int rc = ws_begin(&w, NULL, 0);
  if (rc) {
    *info = 1000 + rc;
    return;
  }
  /* With the reference's own sketch (74 rows), the reference's block size. */
  w.dq_nb = G ? DGEQP4_NB : g_dgeqp4_nb;
  int* hjp = malloc(sizeof(int) * (size_t)N);
  rc = hjp ? dgeqp4_ws(&w, M, N) : HQ_E_NOMEM;
  double* dA = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)ldda * N);
  double* dtau = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)mn);
  int* djp = rc ? NULL : ws_alloc(&w, sizeof(int) * (size_t)N);
  double* dG = (rc || !G || mn < DGEQP4_SMALL_DGEQP3) ? NULL
                                                      : ws_alloc(&w, sizeof(double) * (size_t)mY * M);
  if (!rc && w.failed) rc = HQ_E_NOMEM;
  cudaStream_t st = w.st;
  if (hjp) memcpy(hjp, jpvt, sizeof(int) * (size_t)N);
  CKF(cudaMemcpy2DAsync(dA, sizeof(double) * ldda, A, sizeof(double) * LDA, sizeof(double) * M, N,
                        cudaMemcpyHostToDevice, st));
  if (dG)
    CKF(cudaMemcpy2DAsync(dG, sizeof(double) * mY, G, sizeof(double) * ldg, sizeof(double) * mY,
                          M, cudaMemcpyHostToDevice, st));
  int iws = 3 * N + 1;
  if (!rc) drain_begin(&w, A, LDA, dA, ldda, M);
  if (!rc) rc = core_dgeqp4(&w, M, N, dA, ldda, hjp, djp, dtau, &iws, dG, mY);
  if (!rc) rc = drain_finish(&w, A, LDA, dA, ldda, M, N);
  if (!rc) rc = ws_check(&w);
  CKF(cudaMemcpyAsync(jpvt, djp, sizeof(int) * N, cudaMemcpyDeviceToHost, st));
  CKF(cudaMemcpyAsync(tau, dtau, sizeof(double) * mn, cudaMemcpyDeviceToHost, st));
  ws_release(&w);
  CKF(cudaStreamSynchronize(st));
  free(hjp);
  if (rc) {
    *info = 1000 + rc;
    return;
  }
  work[0] = (double)iws;
}

HQ_API void dgeqp4(int* m, int* n, double* A, int* lda, int* jpvt, double* tau, double* work,
                   int* lwork, int* info) {
  dgeqp4_host(m, n, A, lda, jpvt, tau, work, lwork, info, NULL, 0);
}

HQ_API void hqrrp_gb300_dgeqp4_sketch(int* m, int* n, double* A, int* lda, int* jpvt,
                                      double* tau, double* work, int* lwork, int* info,
                                      const double* G, int ldg) {
  if (G == NULL || ldg < DGEQP4_NB + DGEQP4_PP) {
    g_err[0] = 0;
    set_err("hqrrp_gb300_dgeqp4_sketch: sketch missing or ldg < %d", DGEQP4_NB + DGEQP4_PP);
    *info = 1000 + HQ_E_UNSUPPORTED;
    return;
  }
  dgeqp4_host(m, n, A, lda, jpvt, tau, work, lwork, info, G, ldg);
}

HQ_API int hqrrp_gb300_dgeqp4_device(int m, int n, double* dA, int ldda, int* d_jpvt,
                                     double* d_tau, void* stream) {
  g_err[0] = 0;
  int info = 0;
  int lw = 3 * (n > 0 ? n : 0) + 1;
  if (dgeqp4_prologue(m, n, ldda, lw, NULL, &info)) return info;
  hq_ws w;
  int rc = ws_begin(&w, (cudaStream_t)stream, 1);
  if (rc) return 1000 + rc;
  w.dq_nb = g_dgeqp4_nb;
  int* hjp = malloc(sizeof(int) * (size_t)n);
  rc = hjp ? dgeqp4_ws(&w, m, n) : HQ_E_NOMEM;
  cudaStream_t st = w.st;
  CKF(cudaMemcpyAsync(hjp, d_jpvt, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  CKF(cudaStreamSynchronize(st));
  int iws = 0;
  if (!rc) rc = core_dgeqp4(&w, m, n, dA, ldda, hjp, d_jpvt, d_tau, &iws, NULL, 0);
  if (!rc) rc = ws_check(&w);
  ws_release(&w);
  CKF(cudaStreamSynchronize(st));
  free(hjp);
  return rc ? 1000 + rc : 0;
}

/* ------------------------------------------------------------------------ */
/* FP64 GEMM on the BF16 tensor cores (split digits), device pointers.      */

HQ_API int hqrrp_gb300_ozaki_dgemm(char transa, char transb, int m, int n, int k, double alpha,
                                   const double* dA, int lda, const double* dB, int ldb,
                                   double beta, double* dC, int ldc, int slices, void* stream) {
  g_err[0] = 0;
  if (m < 0 || n < 0 || k < 0 || (alpha != 1.0 && alpha != -1.0) || (beta != 0.0 && beta != 1.0) ||
      slices < 1 || slices > 7) {
    set_err("hqrrp_gb300_ozaki_dgemm: need m, n, k >= 0, alpha = +-1, beta in {0, 1}, "
            "1 <= slices <= 7");
    return HQ_E_UNSUPPORTED;
  }
  if (m == 0 || n == 0) return 0;
  hq_ws w;
  int rc = ws_begin(&w, (cudaStream_t)stream, 1);
  if (rc) return rc;
  const int ta = (transa == 'T' || transa == 't'), tb = (transb == 'T' || transb == 't');
  w.ws_elems = (size_t)8 << 20;
  w.ws = ws_alloc(&w, sizeof(double) * w.ws_elems);
  w.ozA = ws_alloc(&w, hq_ozk_tile_bytes(m, k, slices, 0));
  w.ozB = ws_alloc(&w, ozk_b_bytes(n, k, slices));
  w.ozea = ws_alloc(&w, sizeof(int) * (size_t)(m + 128));
  w.ozeb = ws_alloc(&w, sizeof(int) * (size_t)(n + 128));
  w.err = ws_alloc(&w, sizeof(int) * 2);
  if (w.failed) rc = HQ_E_NOMEM;
  if (!rc) {
    int e = (int)cudaMemsetAsync(w.err, 0, sizeof(int) * 2, w.st);
    if (e) { set_err("cudaMemsetAsync failed"); rc = HQ_E_CUDA; }
  }
  if (!rc && k == 0 && beta == 0.0)
    rc = hq_dgemm(w.st, &w.ds->dev, 'N', 'N', m, n, 0, 0.0, dA, lda, dB, ldb, 0.0, dC, ldc, NULL,
                  0) ? HQ_E_CUDA : HQ_OK;
  else if (!rc && k > 0)
    /* op(A) rows are the M side; op(B) columns are the N side. */
    rc = ozk_product(&w, slices, m, n, k, dA, ta ? lda : 1, ta ? 1 : lda, dB, tb ? 1 : ldb,
                     tb ? ldb : 1, beta == 1.0 ? 1 : 0, alpha, dC, 1, ldc);
  if (!rc) rc = ws_check(&w);
  ws_release(&w);
  if (!rc) {
    int e = (int)cudaStreamSynchronize(w.st);
    if (e) { set_err("cudaStreamSynchronize failed: %s", cudaGetErrorString((cudaError_t)e)); rc = HQ_E_CUDA; }
  }
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Batched pivoted QR: plan (schedule + autotuned launch shape), then run.   */

typedef struct {
  int threads, stage_kb, ctas_per_sm;
} batched_cfg;

/* Launch shapes the autotuner tries: threads per CTA, shared-memory staging
 * budget for a matrix (KB; larger matrices are worked on in place in L2),
 * CTAs per SM. */
static const batched_cfg g_batched_cfgs[] = {
    {128, 0, 4},   {128, 48, 4}, {256, 0, 2},  {256, 96, 2},
    {256, 200, 1}, {512, 96, 2}, {512, 200, 1},
};
#define N_BATCHED_CFGS ((int)(sizeof g_batched_cfgs / sizeof g_batched_cfgs[0]))

typedef struct {
  int batch, max_n;
  double cost;
  int cfg;
} tune_entry;
static tune_entry g_tuned[32];
static int g_ntuned = 0;

HQ_API size_t hqrrp_gb300_qrp_batched_workspace(int batch) {
  return batch > 0 ? hq_qrp_batched_workspace(batch) : 0;
}

typedef struct {
  double cost;
  int idx;
} cost_idx;

static int cost_desc(const void* x, const void* y) {
  const cost_idx *a = (const cost_idx*)x, *b = (const cost_idx*)y;
  if (a->cost != b->cost) return a->cost < b->cost ? 1 : -1;
  return a->idx - b->idx;
}

/* Householder QR flops (2mn^2 - 2n^3/3 for m >= n) plus one pass over A. */
static double qr_cost(int m, int n) {
  const double M = m > n ? m : n, k = m < n ? m : n;
  return 2.0 * M * k * k - 2.0 * k * k * k / 3.0 + (double)m * n;
}

/* Time every launch shape on scratch matrices of the batch's sizes. */
static int autotune_batched(hq_ws* w, int batch, const int* h_m, const int* h_n, int max_n,
                            void* d_work) {
  size_t total = 0;
  for (int i = 0; i < batch; ++i) total += (size_t)(h_m[i] > 0 ? h_m[i] : 1) * (h_n[i] > 0 ? h_n[i] : 1);
  double* pool = ws_alloc(w, sizeof(double) * total);
  double** hA = malloc(sizeof(double*) * (size_t)batch);
  int** hJ = malloc(sizeof(int*) * (size_t)batch);
  double** hT = malloc(sizeof(double*) * (size_t)batch);
  int* jbuf = ws_alloc(w, sizeof(int) * (size_t)batch * max_n);
  double* tbuf = ws_alloc(w, sizeof(double) * (size_t)batch * max_n);
  int* dm = ws_alloc(w, sizeof(int) * (size_t)batch);
  int* dn = ws_alloc(w, sizeof(int) * (size_t)batch);
  int* dl = ws_alloc(w, sizeof(int) * (size_t)batch);
  void** dptr = ws_alloc(w, sizeof(void*) * 3 * (size_t)batch);
  int best = -1;
  if (!w->failed && hA && hJ && hT) {
    size_t off = 0;
    int* hl = malloc(sizeof(int) * (size_t)batch);
    for (int i = 0; i < batch; ++i) {
      hA[i] = pool + off;
      off += (size_t)(h_m[i] > 0 ? h_m[i] : 1) * (h_n[i] > 0 ? h_n[i] : 1);
      hJ[i] = jbuf + (size_t)i * max_n;
      hT[i] = tbuf + (size_t)i * max_n;
      hl[i] = h_m[i] > 1 ? h_m[i] : 1;
    }
    int ok = hl != NULL;
    ok = ok && hq_sketch_philox(w->st, 1, (int)(total < 2147483647 ? total : 2147483647), pool, 1,
                                2026ULL) == 0;
    ok = ok && cudaMemcpyAsync(dm, h_m, sizeof(int) * batch, cudaMemcpyHostToDevice, w->st) == 0;
    ok = ok && cudaMemcpyAsync(dn, h_n, sizeof(int) * batch, cudaMemcpyHostToDevice, w->st) == 0;
    ok = ok && cudaMemcpyAsync(dl, hl, sizeof(int) * batch, cudaMemcpyHostToDevice, w->st) == 0;
    ok = ok && cudaMemcpyAsync(dptr, hA, sizeof(void*) * batch, cudaMemcpyHostToDevice, w->st) == 0;
    ok = ok && cudaMemcpyAsync(dptr + batch, hJ, sizeof(void*) * batch, cudaMemcpyHostToDevice,
                               w->st) == 0;
    ok = ok && cudaMemcpyAsync(dptr + 2 * batch, hT, sizeof(void*) * batch,
                               cudaMemcpyHostToDevice, w->st) == 0;
    ok = ok && cudaStreamSynchronize(w->st) == 0;
    cudaEvent_t e0, e1;
    ok = ok && cudaEventCreate(&e0) == 0 && cudaEventCreate(&e1) == 0;
    float best_ms = 1e30f;
    for (int c = 0; ok && c < N_BATCHED_CFGS; ++c) {
      const batched_cfg* k = &g_batched_cfgs[c];
      float ms = 0.f;
      int rc = hq_qrp_batched(w->st, &w->ds->dev, batch, dm, dn, (double* const*)dptr, dl,
                              (int* const*)(dptr + batch), (double* const*)(dptr + 2 * batch),
                              NULL, d_work, max_n, k->threads, k->stage_kb, k->ctas_per_sm);
      if (rc) continue; /* shape does not fit this device: skip it */
      cudaEventRecord(e0, w->st);
      rc = hq_qrp_batched(w->st, &w->ds->dev, batch, dm, dn, (double* const*)dptr, dl,
                          (int* const*)(dptr + batch), (double* const*)(dptr + 2 * batch), NULL,
                          d_work, max_n, k->threads, k->stage_kb, k->ctas_per_sm);
      cudaEventRecord(e1, w->st);
      if (rc || cudaStreamSynchronize(w->st) != cudaSuccess) continue;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    if (ok) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
    }
    free(hl);
  }
  free(hA);
  free(hJ);
  free(hT);
  return best;
}

HQ_API int hqrrp_gb300_qrp_batched_plan(int batch, const int* h_m, const int* h_n, void* d_work,
                                        size_t work_bytes, int autotune, void* stream) {
  g_err[0] = 0;
  if (batch <= 0) return 0;
  if (work_bytes < hq_qrp_batched_workspace(batch) || !h_m || !h_n || !d_work) {
    set_err("hqrrp_gb300_qrp_batched_plan: missing sizes or workspace too small");
    return -HQ_E_UNSUPPORTED;
  }
  int max_n = 1;
  double total = 0.0;
  cost_idx* ord = malloc(sizeof(cost_idx) * (size_t)batch);
  int* hord = malloc(sizeof(int) * (size_t)batch);
  if (!ord || !hord) {
    free(ord);
    free(hord);
    set_err("host allocation failed");
    return -HQ_E_NOMEM;
  }
  for (int i = 0; i < batch; ++i) {
    if (h_m[i] < 0 || h_n[i] < 0) {
      free(ord);
      free(hord);
      set_err("hqrrp_gb300_qrp_batched_plan: negative size at %d", i);
      return -HQ_E_UNSUPPORTED;
    }
    ord[i].cost = qr_cost(h_m[i], h_n[i]);
    ord[i].idx = i;
    total += ord[i].cost;
    if (h_n[i] > max_n) max_n = h_n[i];
  }
  qsort(ord, (size_t)batch, sizeof(cost_idx), cost_desc);
  for (int i = 0; i < batch; ++i) hord[i] = ord[i].idx;
  free(ord);
  hq_ws w;
  int rc = ws_begin(&w, (cudaStream_t)stream, 1);
  if (!rc) {
    int e = (int)cudaMemcpyAsync((int*)d_work + 32, hord, sizeof(int) * batch,
                                 cudaMemcpyHostToDevice, w.st);
    if (!e) e = (int)cudaStreamSynchronize(w.st);
    if (e) {
      set_err("schedule upload failed: %s", cudaGetErrorString((cudaError_t)e));
      rc = HQ_E_CUDA;
    }
  }
  free(hord);
  if (rc) return -rc;
  int cfg = 3; /* 256 threads, 96 KB staging, 2 CTAs per SM */
  if (autotune) {
    for (int i = 0; i < g_ntuned; ++i)
      if (g_tuned[i].batch == batch && g_tuned[i].max_n == max_n && g_tuned[i].cost == total)
        return g_tuned[i].cfg;
    int best = autotune_batched(&w, batch, h_m, h_n, max_n, d_work);
    ws_release(&w);
    cudaStreamSynchronize(w.st);
    if (best >= 0) cfg = best;
    if (g_ntuned < 32) {
      g_tuned[g_ntuned].batch = batch;
      g_tuned[g_ntuned].max_n = max_n;
      g_tuned[g_ntuned].cost = total;
      g_tuned[g_ntuned].cfg = cfg;
      ++g_ntuned;
    }
  }
  return cfg;
}

HQ_API int hqrrp_gb300_qrp_batched_run(int batch, const int* d_m, const int* d_n,
                                       double* const* d_A, const int* d_lda, int* const* d_jpvt,
                                       double* const* d_tau, int* d_info, int max_n, int cfg,
                                       void* d_work, void* stream) {
  g_err[0] = 0;
  if (batch <= 0) return 0;
  if (cfg < 0 || cfg >= N_BATCHED_CFGS || max_n <= 0) {
    set_err("hqrrp_gb300_qrp_batched_run: bad configuration or max_n");
    return HQ_E_UNSUPPORTED;
  }
  dev_state* ds = current_device();
  if (!ds) return HQ_E_CUDA;
  const batched_cfg* k = &g_batched_cfgs[cfg];
  int rc = hq_qrp_batched((cudaStream_t)stream, &ds->dev, batch, d_m, d_n, d_A, d_lda, d_jpvt,
                          d_tau, d_info, d_work, max_n, k->threads, k->stage_kb, k->ctas_per_sm);
  if (rc) {
    set_err("batched launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    return HQ_E_CUDA;
  }
  return 0;
}

HQ_API int hqrrp_gb300_qrp_batched_config(int cfg, int* threads, int* stage_kb, int* ctas_per_sm) {
  if (cfg < 0 || cfg >= N_BATCHED_CFGS) return -1;
  if (threads) *threads = g_batched_cfgs[cfg].threads;
  if (stage_kb) *stage_kb = g_batched_cfgs[cfg].stage_kb;
  if (ctas_per_sm) *ctas_per_sm = g_batched_cfgs[cfg].ctas_per_sm;
  return N_BATCHED_CFGS;
}

/* ------------------------------------------------------------------------ */
/* Truncated factorization and its adjoint.                                 */

HQ_API int hqrrp_gb300_hqrrp_truncated_device(int m, int n, int k, double* dA, int ldda,
                                              int* d_jpvt, double* d_tau, int nb, int pp,
                                              unsigned long long seed, void* stream) {
  g_err[0] = 0;
  if (m < 0 || n < 0 || ldda < imax(1, m) || k < 0) {
    set_err("invalid m, n, k or ldda");
    return HQ_E_UNSUPPORTED;
  }
  const int kk = imin(k, imin(m, n));
  if (kk == 0) return 0;
  int rc = check_hqrrp_shape(nb, pp);
  if (rc) return rc;
  hq_ws w;
  if ((rc = ws_begin(&w, (cudaStream_t)stream, 1))) return rc;
  rc = ws_setup(&w, m, n, nb, pp, nb);
  if (!rc) rc = core_hqrrp_k(&w, m, n, dA, ldda, d_jpvt, d_tau, nb, pp, 1, NULL, 0, seed, kk);
  if (!rc) rc = ws_check(&w);
  ws_release(&w);
  if (!rc) {
    int e = (int)cudaStreamSynchronize(w.st);
    if (e) { set_err("cudaStreamSynchronize failed: %s", cudaGetErrorString((cudaError_t)e)); rc = HQ_E_CUDA; }
  }
  return rc;
}

/* C (m x nc, ldc) := Q C (trans 'N') or Q^T C (trans 'T'), Q = H_0 ... H_{k-1}
 * the product of the first k reflectors stored in F.  The reflector blocks
 * of nb columns are rebuilt (U, Gram, T) from F and applied one at a time:
 * from the last block to the first for Q C, first to last for Q^T C. */
static int apply_qk(hq_ws* w, char trans, int m, int nc, int k, int nb, const double* F, int ldf,
                    const double* tau, double* C, int ldc) {
  const hq_device_info* dev = &w->ds->dev;
  const int nblk = (k + nb - 1) / nb;
  const int tr = trans == 'T' || trans == 't';
  for (int step = 0; step < nblk; ++step) {
    const int bi = tr ? step : nblk - 1 - step;
    const int j = bi * nb, b = imin(nb, k - j), mp = m - j;
    CK(hq_unit_lower(w->st, mp, b, F + j + (size_t)j * ldf, ldf, w->U, w->ldu));
    DG('T', 'N', b, b, mp, 1.0, w->U, w->ldu, w->U, w->ldu, 0.0, w->Z, w->ldz);
    CK(hq_larft_from_gram(w->st, b, w->Z, w->ldz, tau + j, w->T, w->ldt));
    /* C[j:, :] -= U op(T) U^T C[j:, :] */
    DG('T', 'N', b, nc, mp, 1.0, w->U, w->ldu, C + j, ldc, 0.0, w->W1, w->ldw);
    DG(tr ? 'T' : 'N', 'N', b, nc, b, 1.0, w->T, w->ldt, w->W1, w->ldw, 0.0, w->W2, w->ldw);
    DG('N', 'N', mp, nc, b, -1.0, w->U, w->ldu, w->W2, w->ldw, 1.0, C + j, ldc);
  }
  return HQ_OK;
}

/* Q_k (m x k, ldq) = Q [I_k; 0]. */
static int form_qk(hq_ws* w, int m, int k, int nb, const double* F, int ldf, const double* tau,
                   double* Q, int ldq) {
  CK(hq_eye(w->st, m, k, Q, ldq));
  return apply_qk(w, 'N', m, k, k, nb, F, ldf, tau, Q, ldq);
}

HQ_API int hqrrp_gb300_apply_q_device(char trans, int m, int nc, int k, const double* dF,
                                      int lddf, const double* d_tau, double* dC, int lddc, int nb,
                                      void* stream) {
  g_err[0] = 0;
  if ((trans != 'N' && trans != 'n' && trans != 'T' && trans != 't') || m < 0 || nc < 0 ||
      k < 0 || k > m || lddf < imax(1, m) || lddc < imax(1, m) || nb < 1 || nb > HQ_MAX_MY) {
    set_err("hqrrp_gb300_apply_q_device: invalid arguments");
    return HQ_E_UNSUPPORTED;
  }
  if (m == 0 || nc == 0 || k == 0) return 0;
  hq_ws w;
  int rc = ws_begin(&w, (cudaStream_t)stream, 1);
  if (rc) return rc;
  rc = ws_setup(&w, m, imax(nc, k), 0, 0, nb);
  if (!rc) rc = apply_qk(&w, trans, m, nc, k, nb, dF, lddf, d_tau, dC, lddc);
  if (!rc) rc = ws_check(&w);
  ws_release(&w);
  if (!rc) {
    int e = (int)cudaStreamSynchronize(w.st);
    if (e) { set_err("cudaStreamSynchronize failed: %s", cudaGetErrorString((cudaError_t)e)); rc = HQ_E_CUDA; }
  }
  return rc;
}

HQ_API int hqrrp_gb300_hqrrp_adjoint_device(int m, int n, int k, const double* dA, int ldda,
                                            const double* dF, int lddf, const int* d_jpvt,
                                            const double* d_tau, const double* dW, int lddw,
                                            double* dG, int lddg, int nb, void* stream) {
  g_err[0] = 0;
  if (m < 0 || n < 0 || k < 0 || k > imin(m, n) || ldda < imax(1, m) || lddf < imax(1, m) ||
      lddw < imax(1, m) || lddg < imax(1, m) || nb < 1 || nb > HQ_MAX_MY) {
    set_err("hqrrp_gb300_hqrrp_adjoint_device: invalid sizes (need k <= min(m, n))");
    return HQ_E_UNSUPPORTED;
  }
  if (m == 0 || n == 0) return 0;
  hq_ws w;
  int rc = ws_begin(&w, (cudaStream_t)stream, 1);
  if (rc) return rc;
  const hq_device_info* dev;
  rc = ws_setup(&w, m, imax(n, k), 0, 0, nb);
  const int ldq = round_up(m, 32);
  double* Q = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)ldq * imax(k, 1));
  double* GQ = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)ldq * imax(k, 1));
  double* Mk = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)imax(k, 1) * n);
  double* Nk = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)imax(k, 1) * n);
  double* Mp = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)imax(k, 1) * imax(k, 1));
  if (!rc && w.failed) rc = HQ_E_NOMEM;
  if (!rc && k == 0) {
    int e = (int)cudaMemset2DAsync(dG, sizeof(double) * lddg, 0, sizeof(double) * m, n, w.st);
    if (e) { set_err("cudaMemset2DAsync failed"); rc = HQ_E_CUDA; }
  }
  if (!rc && k > 0) {
    hq_ws* wp = &w;
    dev = &wp->ds->dev;
#define DGW(ta, tb, M, N, K, al, A, lda, B, ldb, be, C, ldc)                                  \
  do {                                                                                       \
    int e_ = hq_dgemm(wp->st, dev, ta, tb, M, N, K, al, A, lda, B, ldb, be, C, ldc, wp->ws,  \
                      wp->ws_elems);                                                         \
    if (e_) { set_err("hq_dgemm failed: %s", cudaGetErrorString((cudaError_t)e_)); rc = HQ_E_CUDA; } \
  } while (0)
    rc = form_qk(&w, m, k, nb, dF, lddf, d_tau, Q, ldq);
    /* M = R_k P^T (k x n), N = Q^T W (k x n) */
    if (!rc && hq_rk_unpermute(w.st, k, n, dF, lddf, d_jpvt, Mk, k)) rc = HQ_E_CUDA;
    if (!rc) DGW('T', 'N', k, n, m, 1.0, Q, ldq, dW, lddw, 0.0, Nk, k);
    /* G_Q = W M^T + A N^T (m x k) */
    if (!rc) DGW('N', 'T', m, k, n, 1.0, dW, lddw, Mk, k, 0.0, GQ, ldq);
    if (!rc) DGW('N', 'T', m, k, n, 1.0, dA, ldda, Nk, k, 1.0, GQ, ldq);
    /* X = G_Q + Q copyltu(-G_Q^T Q) */
    if (!rc) DGW('T', 'N', k, k, m, 1.0, GQ, ldq, Q, ldq, 0.0, Mp, k);
    if (!rc && hq_copyltu(w.st, k, Mp, k, -1.0)) rc = HQ_E_CUDA;
    if (!rc) DGW('N', 'N', m, k, k, 1.0, Q, ldq, Mp, k, 1.0, GQ, ldq);
    /* Abar_1 = X R11^-T */
    if (!rc && hq_trsm_rt(w.st, m, k, dF, lddf, GQ, ldq)) rc = HQ_E_CUDA;
    /* dG = Q N, then dG[:, P_1] += Abar_1 */
    if (!rc) DGW('N', 'N', m, n, k, 1.0, Q, ldq, Nk, k, 0.0, dG, lddg);
    if (!rc && hq_scatter_cols(w.st, m, k, GQ, ldq, d_jpvt, dG, lddg, 1)) rc = HQ_E_CUDA;
#undef DGW
  }
  if (!rc) rc = ws_check(&w);
  ws_release(&w);
  if (!rc) {
    int e = (int)cudaStreamSynchronize(w.st);
    if (e) { set_err("cudaStreamSynchronize failed: %s", cudaGetErrorString((cudaError_t)e)); rc = HQ_E_CUDA; }
  }
  return rc;
}

HQ_API int hqrrp_gb300_form_q_device(int m, int k, const double* dF, int lddf,
                                     const double* d_tau, double* dQ, int lddq, int nb,
                                     void* stream) {
  g_err[0] = 0;
  if (m < 0 || k < 0 || k > m || lddf < imax(1, m) || lddq < imax(1, m) || nb < 1 ||
      nb > HQ_MAX_MY) {
    set_err("hqrrp_gb300_form_q_device: invalid sizes");
    return HQ_E_UNSUPPORTED;
  }
  if (m == 0 || k == 0) return 0;
  hq_ws w;
  int rc = ws_begin(&w, (cudaStream_t)stream, 1);
  if (rc) return rc;
  rc = ws_setup(&w, m, k, 0, 0, nb);
  if (!rc) rc = form_qk(&w, m, k, nb, dF, lddf, d_tau, dQ, lddq);
  if (!rc) rc = ws_check(&w);
  ws_release(&w);
  if (!rc) {
    int e = (int)cudaStreamSynchronize(w.st);
    if (e) { set_err("cudaStreamSynchronize failed: %s", cudaGetErrorString((cudaError_t)e)); rc = HQ_E_CUDA; }
  }
  return rc;
}

HQ_API int hqrrp_gb300_lowrank_device(int m, int n, int k, const double* dF, int lddf,
                                      const int* d_jpvt, const double* d_tau, double* dOut,
                                      int lddo, int nb, void* stream) {
  g_err[0] = 0;
  if (m < 0 || n < 0 || k < 0 || k > imin(m, n) || lddf < imax(1, m) || lddo < imax(1, m) ||
      nb < 1 || nb > HQ_MAX_MY) {
    set_err("hqrrp_gb300_lowrank_device: invalid sizes");
    return HQ_E_UNSUPPORTED;
  }
  if (m == 0 || n == 0) return 0;
  hq_ws w;
  int rc = ws_begin(&w, (cudaStream_t)stream, 1);
  if (rc) return rc;
  rc = ws_setup(&w, m, imax(n, k), 0, 0, nb);
  const int ldq = round_up(m, 32);
  double* Q = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)ldq * imax(k, 1));
  double* Mk = rc ? NULL : ws_alloc(&w, sizeof(double) * (size_t)imax(k, 1) * n);
  if (!rc && w.failed) rc = HQ_E_NOMEM;
  if (!rc && k > 0) rc = form_qk(&w, m, k, nb, dF, lddf, d_tau, Q, ldq);
  if (!rc && k > 0 && hq_rk_unpermute(w.st, k, n, dF, lddf, d_jpvt, Mk, k)) rc = HQ_E_CUDA;
  if (!rc) {
    int e = hq_dgemm(w.st, &w.ds->dev, 'N', 'N', m, n, k, 1.0, Q, ldq, Mk, imax(k, 1), 0.0, dOut,
                     lddo, w.ws, w.ws_elems);
    if (e) { set_err("hq_dgemm failed: %s", cudaGetErrorString((cudaError_t)e)); rc = HQ_E_CUDA; }
  }
  if (!rc) rc = ws_check(&w);
  ws_release(&w);
  if (!rc) {
    int e = (int)cudaStreamSynchronize(w.st);
    if (e) { set_err("cudaStreamSynchronize failed: %s", cudaGetErrorString((cudaError_t)e)); rc = HQ_E_CUDA; }
  }
  return rc;
}
