// qrp_panel.cu -- pivoted Householder QR of a tall panel, one cooperative
// kernel, plus the T factor of the resulting block reflector.
//
// Reference: lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:520-524 runs
// NoFLA_QRPmod_WY_unb_var4 (:774-886) on the (m-j) x b panel with
// num_stages = -1 and build_T = 1: per column, idamax of the partial norms,
// swap (columns, labels, copied norms: :990-1036), dlarfg, dlarf on the
// trailing panel columns, Drmac's norm downdate with recompute on
// cancellation (:912-986); then dlarft Forward/Columnwise (:875-878).  The
// same kernel, run over all columns, serves the small-matrix path of dgeqp4
// (:189-199): LAPACK's dgeqpf and dgeqp3 pick pivots by the same rule and
// downdate norms with the same LAWN 176 test.
//
// GB300 layout: the panel's rows are split into contiguous slabs, one per CTA
// (one CTA per SM), kept in shared memory when they fit (108 rows x 128
// columns = 110 KB at m = 16384) and otherwise worked on in place in L2.
// Column swaps are then local to every CTA.  Each stage needs one grid
// exchange: every CTA publishes, for its slab, the dot products of the pivot
// column with all not-yet-factored columns (the first of which is the pivot
// column's squared norm); the owner of the pivot row also publishes that row.
// The partials are summed as fixed-point integers: each CTA adds its partial
// of column k, exactly, as three 48-bit limbs of a 144-bit integer in units
// of 2^ue_k (ue_k from the two columns' norms, which bound every partial and
// their sum by Cauchy-Schwarz) to three 64-bit words with L2 atomics.
// Integer addition is associative, so the order of the atomics does not
// matter: the sums are the same in every run, and exact up to the truncation
// below 2^ue_k (2^-133 of the bound, far below FP64 rounding of the
// partials).  One grid barrier per stage then suffices: every CTA reads the
// words of all columns, converts them to FP64 and builds the reflector
// itself (identical inputs, identical results), with no reduce-scatter and
// no second barrier -- FP64 adds of 152 partials per column in every CTA
// would cost microseconds on this GPU's FP64 pipe, integer atomics do not.
// The slab is then updated without further communication.  The norm
// downdate of the trailing columns carries the warp-level argmax of the next
// pivot.  The rare norm recomputation costs one more barrier in the stages
// that need it (FP64 partials, summed in a fixed order in every CTA).
#include "hq_common.cuh"
#include "hq_fixedpoint.h"

namespace {

constexpr int NT = 256;
constexpr int NWARP = NT / 32;
constexpr int MAX_G = 160;          // CTAs (one per SM); partial loads per lane <= 5
constexpr int CB = (MAX_G + 31) / 32;
constexpr int QB = 8;               // columns reduced per warp per batch of loads

struct PnArgs {
  int mp, nc, ns, pivoting;
  double* P;
  int ldp;
  double* tau;
  double* U;
  int ldu;
  int* perm;
  double* part;  // [2][pstride][grid] partials (column q's contiguous)
  unsigned long long* acc;  // [3][pstride][FX_CS] fixed-point stage sums
  int pstride;
  double* rowbuf;  // [2][nc]
  unsigned* bar;
  int* err;
  unsigned spin_limit;
  int smem_mode, rloc_max, ldxs;
  int sqnorm;  // keep squared norms (d^2 <- d^2 - r^2, LAWN 176's test without divisions)
  int ut;      // UT-transform convention: a zero tail gives H = I - 2 e e^T (tau 2, beta -alpha)
  const int* gram_stat;  // non-null: skip when *gram_stat == 0 (the Gram panel succeeded)
};

// Fixed-point stage sums (hq_fixedpoint.h): words 0..2 of a column are the
// limbs' signed 64-bit accumulators, word 3 counts non-finite partials.
constexpr int FX_CS = HQ_PANEL_FX_CS;  // words between consecutive columns

__device__ __forceinline__ int fx_unit(double ep, double ek, int sqnorm) {
  return hq_fx_unit(ep, ek, sqnorm);
}

// Adds t / 2^ue, truncated to an integer, to the words w (L2 atomics).
__device__ __forceinline__ void fx_add(unsigned long long* w, double t, int ue) {
  unsigned long long p[3];
  int L = 0;
  const int rc = hq_fx_split(t, ue, p, &L);
  if (rc == 2) {
    atomicAdd(w + 3, 1ull);
  } else if (rc == 1) {
    if (p[0]) atomicAdd(w + L, p[0]);
    if (p[1] && L + 1 < 3) atomicAdd(w + L + 1, p[1]);
    if (p[2] && L + 2 < 3) atomicAdd(w + L + 2, p[2]);
  }
}

// The sum in the words w; all four words are loaded before any is used (one
// L2 round trip).
__device__ __forceinline__ double fx_value(const unsigned long long* w, int ue) {
  const unsigned long long nf = __ldcg(w + 3);
  const long long l0 = (long long)__ldcg(w), l1 = (long long)__ldcg(w + 1);
  const long long l2 = (long long)__ldcg(w + 2);
  if (nf != 0ull) return __longlong_as_double(0x7FF8000000000000LL);
  return hq_fx_combine(l0, l1, l2, ue);
}

// Candidate order for the pivot: larger norm, then lower column (idamax's
// first maximum); NaN never wins.
__device__ __forceinline__ void pick(long long key, int k, long long& bkey, int& bk) {
  if (key > bkey || (key == bkey && k < bk)) { bkey = key; bk = k; }
}

__global__ void __launch_bounds__(NT, 1) panel_qrp_kernel(PnArgs a) {
  HQ_PDL_WAIT();
  extern __shared__ __align__(16) double smem[];
  // Every CTA reads the same word, written before the launch.
  if (a.gram_stat != nullptr && *a.gram_stat == 0) return;
  const int G = gridDim.x, cta = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int nc = a.nc;
  const int r_lo = (int)((long long)cta * a.mp / G);
  const int r_hi = (int)((long long)(cta + 1) * a.mp / G);
  const int nloc = r_hi - r_lo;

  double* sX = smem;
  double* sd = sX + (a.smem_mode ? (size_t)a.ldxs * nc : 0);
  double* se = sd + nc;
  double* sw = se + nc;      // reduced dots of the stage
  double* srow = sw + nc;    // pivot row of the stage (old values)
  int* sperm = (int*)(srow + nc);
  int* sflag = sperm + nc;
  __shared__ int s_flag;
  __shared__ long long s_bd[NWARP];
  __shared__ int s_bk[NWARP];
  __shared__ double s_tau, s_scale, s_beta;

  double* X;
  int ldx;
  if (a.smem_mode) {
    X = sX;
    ldx = a.ldxs;
    for (int k = warp; k < nc; k += NWARP)
      for (int i = lane; i < nloc; i += 32) X[i + (size_t)k * ldx] = a.P[r_lo + i + (size_t)k * a.ldp];
  } else {
    X = a.P + r_lo;
    ldx = a.ldp;
  }
  for (int k = tid; k < nc; k += NT) {
    sperm[k] = k;
    sflag[k] = 0;
  }
  // A valid permutation is in place before any wait: if a barrier gives up
  // and the kernel returns early, the gathers that follow still read indices
  // within range.  Stage sums of stage s go to words buffer s % 3; buffers 0
  // and 1 start at zero (ordered before stage 0 by the first barrier), and
  // CTA 0 clears buffer (s + 1) % 3 during stage s: its last readers passed
  // the barrier of stage s - 1, its first writers come after that of stage s.
  if (cta == 0) {
    for (int k = tid; k < nc; k += NT) a.perm[k] = k;
    for (int i = tid; i < 2 * a.pstride * FX_CS; i += NT) a.acc[i] = 0ull;
  }
  __syncthreads();

  unsigned epoch = 0;
  auto part_w = [&](unsigned e) { return a.part + (size_t)(e & 1) * a.pstride * G + cta; };
  auto part_r = [&](unsigned e) { return a.part + (size_t)(e & 1) * a.pstride * G; };
  // The pivot row of stage s goes to buffer s & 1: it is read after the
  // stage's barrier, and the next write to the same buffer (stage s + 2)
  // comes after a barrier every reader has passed.
  auto rowbuf = [&](int s) { return a.rowbuf + (size_t)(s & 1) * nc; };
  auto fx_buf = [&](int s) { return a.acc + (size_t)(s % 3) * a.pstride * FX_CS; };

  // Slab-local sums over rows with global index > lo_row of x_i * X[i, k]
  // (x = column xs, or column k itself when xs < 0) for k in [k0, nc),
  // skipping columns without sflag when use_mask; column k's sum goes to
  // out[(k - k0) * G], or, when fx is given, is added to the fixed-point
  // words fx[(k - k0) * FX_CS..] in the units of columns xs and k (xs's norm
  // bound in sep).  Below NT columns, `groups` adjacent lanes share a column
  // and combine by shuffles.
  auto slab_dots = [&](int xs, int k0, int lo_row, bool use_mask, double* out,
                       unsigned long long* fx, double sep) {
    const int na = nc - k0;
    const int i0 = max(0, lo_row + 1 - r_lo);
    int groups = 1;
    if (na < NT) {
      groups = NT / na;
      groups = groups >= 32 ? 32 : (groups >= 16 ? 16 : (groups >= 8 ? 8 : (groups >= 4 ? 4 : (groups >= 2 ? 2 : 1))));
    }
    const int g = tid % groups, stride = NT / groups;
    // The trip count is the same for every thread, so whole warps take part
    // in the shuffles; columns past the end contribute zero.
    for (int q0 = 0; q0 < na; q0 += stride) {
      const int q = q0 + tid / groups;
      const int k = k0 + q;
      double t = 0.0;
      if (q < na && (!use_mask || sflag[k])) {
        const double* xk = X + (size_t)k * ldx;
        const double* xx = xs >= 0 ? X + (size_t)xs * ldx : xk;
        double t1 = 0.0;
        int i = i0 + g;
        for (; i + groups < nloc; i += 2 * groups) {
          t = fma(xx[i], xk[i], t);
          t1 = fma(xx[i + groups], xk[i + groups], t1);
        }
        if (i < nloc) t = fma(xx[i], xk[i], t);
        t += t1;
      }
      for (int o = groups >> 1; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (g == 0 && q < na) {
        if (fx) fx_add(fx + (size_t)q * FX_CS, t, fx_unit(sep, se[k], a.sqnorm));
        else out[(size_t)q * G] = t;
      }
    }
  };

  // sw[q] = sum over CTAs of the published column q (q < na), in a fixed
  // order, formed in every CTA (used for the one-off initial norms and the
  // rare norm recomputations).  Warp w takes columns w*QB.. in batches of QB,
  // lane l the CTAs l, l+32, ...; every load of a batch is issued before any
  // is used.
  auto reduce_parts = [&](unsigned e, int na) {
    const double* base = part_r(e);
    for (int q0 = warp * QB; q0 < na; q0 += NWARP * QB) {
      double v[QB][CB];
#pragma unroll
      for (int u = 0; u < QB; ++u) {
        const int q = q0 + u;
#pragma unroll
        for (int j = 0; j < CB; ++j) {
          const int c = lane + 32 * j;
          v[u][j] = (q < na && c < G) ? hq_ldcg(base + (size_t)q * G + c) : 0.0;
        }
      }
#pragma unroll
      for (int u = 0; u < QB; ++u) {
        double t = v[u][0];
#pragma unroll
        for (int j = 1; j < CB; ++j) t += v[u][j];
        t = hq_warp_sum(t);
        if (lane == u && q0 + u < na) sw[q0 + u] = t;
      }
    }
    __syncthreads();
  };

  // After the stage's barrier: the sums of all columns from the fixed-point
  // words, the pivot row, and the reflector (built by thread 0 of every CTA
  // from the same inputs).
  auto gather_sums = [&](int na, int s, double sep) {
    const unsigned long long* fx = fx_buf(s);
    const double* rb = rowbuf(s) + s;
    for (int q = tid; q < na; q += NT) {
      const double t = fx_value(fx + (size_t)q * FX_CS, fx_unit(sep, se[s + q], a.sqnorm));
      const double r = hq_ldcg(rb + q);
      sw[q] = t;
      srow[q] = r;
      if (q == 0) {
        const double tail = (a.mp - s > 1) ? t : 0.0;
        HqReflector h;
        if (a.ut && tail == 0.0) {  // libflame's Househ2_UT: chi_1 := -chi_1, tau_UT = 1/2
          h.tau = 2.0;
          h.beta = -r;
          h.scale = 1.0;
        } else {
          h = hq_make_reflector_sq(r, tail);
        }
        s_tau = h.tau;
        s_scale = h.scale;
        s_beta = h.beta;
      }
    }
    __syncthreads();
  };

  // Block argmax of (sd[k], k) over k in [k0, nc); every thread returns the
  // same index (k0 when no column qualifies, e.g. all norms NaN).
  auto block_argmax = [&](int k0) {
    long long bd = -2;
    int bk = 0x7fffffff;
    for (int k = k0 + tid; k < nc; k += NT) pick(hq_norm_key(sd[k]), k, bd, bk);
    for (int o = 16; o > 0; o >>= 1) {
      const long long od = __shfl_xor_sync(0xffffffffu, bd, o);
      const int ok = __shfl_xor_sync(0xffffffffu, bk, o);
      pick(od, ok, bd, bk);
    }
    if (lane == 0) { s_bd[warp] = bd; s_bk[warp] = bk; }
    __syncthreads();
    bd = s_bd[0];
    bk = s_bk[0];
    for (int w = 1; w < NWARP; ++w) pick(s_bd[w], s_bk[w], bd, bk);
    __syncthreads();  // s_bd is reused by the next call
    return (bk == 0x7fffffff || bd < 0) ? k0 : bk;
  };

  // Initial norms over the whole panel.
  slab_dots(-1, 0, -1, false, part_w(epoch + 1), nullptr, 0.0);
  ++epoch;
  if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;
  reduce_parts(epoch, nc);
  for (int k = tid; k < nc; k += NT) {
    sd[k] = a.sqnorm ? sw[k] : sqrt(sw[k]);
    se[k] = sd[k];
  }
  __syncthreads();
  int kp = a.pivoting ? block_argmax(0) : 0;

  for (int s = 0; s < a.ns; ++s) {
    const int na = nc - s;
    // 1. Swap the pivot column into place (columns, labels, copied norms;
    //    se[s] takes the pivot's own value, which bounds its stage sums --
    //    position s's norms are not read again otherwise).
    if (kp != s) {
      double* c1 = X + (size_t)s * ldx;
      double* c2 = X + (size_t)kp * ldx;
      for (int i = tid; i < nloc; i += NT) {
        const double t = c1[i];
        c1[i] = c2[i];
        c2[i] = t;
      }
      if (tid == 0) {
        const int t = sperm[s];
        sperm[s] = sperm[kp];
        sperm[kp] = t;
        const double pse = se[kp];
        sd[kp] = sd[s];
        se[kp] = se[s];
        se[s] = pse;
      }
      __syncthreads();
    }
    const double sep = se[s];

    // 2. Add the slab dots with the pivot column (rows > s) to the stage's
    //    fixed-point sums; the owner of row s publishes that row.  CTA 0
    //    clears the words of stage s + 1.
    if (cta == 0) {
      unsigned long long* nx = fx_buf(s + 1);
      for (int i = tid; i < na * FX_CS; i += NT) nx[i] = 0ull;
    }
    slab_dots(s, s, s, false, nullptr, fx_buf(s), sep);
    if (s >= r_lo && s < r_hi) {
      double* rb = rowbuf(s);
      for (int k = s + tid; k < nc; k += NT) rb[k] = X[(s - r_lo) + (size_t)k * ldx];
    }
    ++epoch;
    if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;

    // 3. Sums, pivot row and reflector in every CTA.
    gather_sums(na, s, sep);
    const double tau = s_tau, scale = s_scale;
    if (cta == 0 && tid == 0) a.tau[s] = tau;
    {
      // v = [1; scale * x] in place (rows > s), beta on the diagonal.
      double* xs = X + (size_t)s * ldx;
      for (int i = max(0, s + 1 - r_lo) + tid; i < nloc; i += NT) xs[i] *= scale;
      if (tid == 0 && s >= r_lo && s < r_hi) xs[s - r_lo] = s_beta;
    }
    __syncthreads();

    // 4. Update the slab: X[i,k] -= v_i * w_k for rows > s, with
    //    w_k = tau * v^T X[:, k] = tau * (scale * dot_k + row_k); the owner of
    //    row s stores the new row entries row_k - w_k.
    {
      const int nt = nc - s - 1;
      const int i0 = max(0, s + 1 - r_lo);
      const bool own = (s >= r_lo && s < r_hi);
      const double* v = X + (size_t)s * ldx;
      if (nt >= NT) {
        for (int q = tid; q < nt; q += NT) {
          const int k = s + 1 + q;
          const double wk = tau * fma(scale, sw[q + 1], srow[q + 1]);
          double* xk = X + (size_t)k * ldx;
          for (int i = i0; i < nloc; ++i) xk[i] = fma(-v[i], wk, xk[i]);
          if (own) xk[s - r_lo] = srow[q + 1] - wk;
        }
      } else if (nt > 0) {
        const int groups = NT / nt;
        const int q = tid % nt, g = tid / nt;
        if (g < groups) {
          const int k = s + 1 + q;
          const double wk = tau * fma(scale, sw[q + 1], srow[q + 1]);
          double* xk = X + (size_t)k * ldx;
          for (int i = i0 + g; i < nloc; i += groups) xk[i] = fma(-v[i], wk, xk[i]);
          if (own && g == 0) xk[s - r_lo] = srow[q + 1] - wk;
        }
      }
    }

    // 5. Norm downdate of the trailing columns with the next pivot's warp
    //    argmax; recompute flagged norms with one more barrier.
    if (!a.pivoting) {
      __syncthreads();
      kp = s + 1;
      continue;
    }
    int any = 0;
    long long bd = -2;
    int bk = 0x7fffffff;
    for (int k = s + 1 + tid; k < nc; k += NT) {
      const int q = k - s;
      const double wk = tau * fma(scale, sw[q], srow[q]);
      const double r = srow[q] - wk;  // the new entry of row s
      int flag = 0;
      double dk = sd[k];
      if (dk != 0.0) {
        if (a.sqnorm) {
          const double nd = fma(-r, r, dk);
          if (nd <= HQ_TOL3Z * se[k]) {
            flag = 1;
          } else {
            dk = nd;
            sd[k] = dk;
          }
        } else {
          double t1 = fabs(r) / dk;
          t1 = (1.0 + t1) * (1.0 - t1);
          if (0.0 > t1) t1 = 0.0;
          const double ratio = dk / se[k];
          const double t2 = t1 * ratio * ratio;
          if (t2 <= HQ_TOL3Z) {
            flag = 1;
          } else {
            dk *= sqrt(t1);
            sd[k] = dk;
          }
        }
      }
      sflag[k] = flag;
      any |= flag;
      pick(hq_norm_key(dk), k, bd, bk);
    }
    for (int o = 16; o > 0; o >>= 1) {
      const long long od = __shfl_xor_sync(0xffffffffu, bd, o);
      const int ok = __shfl_xor_sync(0xffffffffu, bk, o);
      pick(od, ok, bd, bk);
    }
    if (lane == 0) { s_bd[warp] = bd; s_bk[warp] = bk; }
    any = __syncthreads_or(any);
    if (!any) {
      bd = s_bd[0];
      bk = s_bk[0];
      for (int w = 1; w < NWARP; ++w) pick(s_bd[w], s_bk[w], bd, bk);
      kp = (bk == 0x7fffffff || bd < 0) ? s + 1 : bk;
      continue;  // s_bd is next written after the next stage's grid barrier
    }
    slab_dots(-1, s, s, true, part_w(epoch + 1), nullptr, 0.0);
    ++epoch;
    if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;
    reduce_parts(epoch, na);
    for (int k = s + 1 + tid; k < nc; k += NT) {
      if (sflag[k]) {
        const double nv = (a.mp - s - 1 > 0) ? (a.sqnorm ? sw[k - s] : sqrt(sw[k - s])) : 0.0;
        sd[k] = nv;
        se[k] = nv;
        sflag[k] = 0;
      }
    }
    __syncthreads();
    kp = block_argmax(s + 1);
  }

  // Write back, explicit unit-lower U, permutation.
  if (a.smem_mode) {
    for (int k = warp; k < nc; k += NWARP)
      for (int i = lane; i < nloc; i += 32) a.P[r_lo + i + (size_t)k * a.ldp] = X[i + (size_t)k * ldx];
  }
  if (a.U != nullptr) {
    for (int k = warp; k < nc; k += NWARP)
      for (int i = lane; i < nloc; i += 32) {
        const int gi = r_lo + i;
        a.U[gi + (size_t)k * a.ldu] = gi > k ? X[i + (size_t)k * ldx] : (gi == k ? 1.0 : 0.0);
      }
  }
  if (cta == 0)
    for (int k = tid; k < nc; k += NT) a.perm[k] = sperm[k];
}

// One CTA per 16 rows up to one per SM: a stage's FP64 work is spread over
// as many SMs as the panel has 16-row slabs (measured 7 ms faster per 16384^2
// mixed factorization than 64-row slabs, whose small late panels left SMs
// idle while the grid barrier costs about the same).
int panel_grid(const hq_device_info* dev, int mp) {
  int g = (mp + 15) / 16;
  if (g > dev->num_sms) g = dev->num_sms;
  if (g > MAX_G) g = MAX_G;
  return g < 1 ? 1 : g;
}

// DLARFT (Forward, Columnwise) from the Gram matrix Z = U^T U: for each i,
// T[0:i, i] = -tau_i T[0:i, 0:i] Z[0:i, i] and T[i, i] = tau_i (T[0:i, i] = 0
// when tau_i = 0).  One CTA; the columns are a sequential recurrence, so each
// step's triangular matrix-vector product is spread over the CTA with eight
// lanes per row (short FP64 dependency chains), combined by shuffles.  T is
// built in shared memory with an odd leading dimension (no bank conflicts
// between the eight lanes of a row) when it fits.
__global__ void larft_kernel(int k, const double* __restrict__ Z, int ldz,
                             const double* __restrict__ tau, double* __restrict__ T, int ldt,
                             int use_smem) {
  extern __shared__ double sT[];
  __shared__ double tmp[HQ_MAX_MY];
  double* Tm = use_smem ? sT : T;
  const int ld = use_smem ? (k | 1) : ldt;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int g = tid & 7, rows_per_pass = nt >> 3;
  for (int e = tid; e < k * k; e += nt) Tm[(e % k) + (size_t)(e / k) * ld] = 0.0;
  __syncthreads();
  for (int i = 0; i < k; ++i) {
    const double ti = tau[i];
    for (int r = tid; r < i; r += nt) tmp[r] = -ti * Z[r + (size_t)i * ldz];
    __syncthreads();
    if (ti != 0.0) {
      for (int r0 = 0; r0 < i; r0 += rows_per_pass) {
        const int r = r0 + (tid >> 3);
        double acc = 0.0;
        if (r < i)
          for (int c = r + g; c < i; c += 8) acc = fma(Tm[r + (size_t)c * ld], tmp[c], acc);
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        acc += __shfl_xor_sync(0xffffffffu, acc, 4);
        if (g == 0 && r < i) Tm[r + (size_t)i * ld] = acc;
      }
    }
    if (tid == 0) Tm[i + (size_t)i * ld] = ti;
    __syncthreads();
  }
  if (use_smem)
    for (int e = tid; e < k * k; e += nt)
      T[(e % k) + (size_t)(e / k) * ldt] = sT[(e % k) + (size_t)(e / k) * ld];
}

// The same T, one CTA per row.  Row r of T only involves row r itself:
// T[r, i] = -tau_i * sum_{c = r}^{i-1} T[r, c] Z[c, i] for i > r, T[r, r] =
// tau_r (zero when tau_i = 0), so the k rows are independent recurrences and
// run side by side on k SMs instead of one SM's FP64 pipe doing all of them.
// The CTA first stages the part of Z its row reads (Z[r:i, i], i > r: the
// upper triangle from row r) in shared memory with all its threads, then one
// warp runs the recurrence: per step a dot of length i - r over the lanes and
// a shuffle reduction, with the row kept in shared memory.
constexpr int LARFT_ROW_MAX = 128;  // k up to this: row and staged triangle fit (<= 66 KB)

__global__ void __launch_bounds__(128) larft_rows_kernel(int k, const double* __restrict__ Z,
                                                         int ldz, const double* __restrict__ tau,
                                                         double* __restrict__ T, int ldt) {
  extern __shared__ double lsm[];
  double* sT = lsm;      // [k] the row, from column r on
  double* sZ = lsm + k;  // [k (k - 1) / 2] the staged triangle
  const int r = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
  // Column i > r of the staged triangle holds Z[r:i, i] at offset
  // off(i) = (i - r - 1)(i - r) / 2.
  for (int i = r + 1; i < k; ++i) {
    const int off = (i - r - 1) * (i - r) / 2;
    for (int c = r + tid; c < i; c += blockDim.x) sZ[off + (c - r)] = Z[c + (size_t)i * ldz];
  }
  __syncthreads();
  if (tid < 32) {
    if (lane == 0) sT[0] = tau[r];
    __syncwarp();
    for (int i = r + 1; i < k; ++i) {
      const double ti = tau[i];
      const int off = (i - r - 1) * (i - r) / 2;
      double acc = 0.0;
      for (int c = lane; c < i - r; c += 32) acc = fma(sT[c], sZ[off + c], acc);
      acc = hq_warp_sum(acc);
      if (lane == 0) sT[i - r] = ti != 0.0 ? -ti * acc : 0.0;
      __syncwarp();
    }
    for (int i = lane; i < k; i += 32) T[r + (size_t)i * ldt] = i < r ? 0.0 : sT[i - r];
  }
}

}  // namespace

extern "C" size_t hq_panel_part_elems(const hq_device_info* dev, int nc) {
  return HQ_PANEL_PART_ELEMS(dev->num_sms, nc);
}

extern "C" int hq_panel_qrp(cudaStream_t stream, const hq_device_info* dev, int mp, int nc,
                            int pivoting, double* P, int ldp, double* tau,
                            double* U, int ldu, int* perm, double* part, size_t part_elems,
                            double* rowbuf, unsigned* bar, int* err, unsigned spin_limit,
                            int sqnorm, int ut) {
  return hq_panel_qrp_fallback(stream, dev, mp, nc, pivoting, P, ldp, tau, U, ldu, perm, part,
                               part_elems, rowbuf, bar, err, spin_limit, sqnorm, ut, nullptr);
}

extern "C" int hq_panel_qrp_fallback(cudaStream_t stream, const hq_device_info* dev, int mp,
                                     int nc, int pivoting, double* P, int ldp, double* tau,
                                     double* U, int ldu, int* perm, double* part,
                                     size_t part_elems, double* rowbuf, unsigned* bar, int* err,
                                     unsigned spin_limit, int sqnorm, int ut,
                                     const int* gram_stat) {
  if (nc <= 0 || mp <= 0) return 0;
  if (nc > HQ_MAX_PANEL) return (int)cudaErrorInvalidValue;
  PnArgs a;
  a.mp = mp;
  a.nc = nc;
  a.ns = mp < nc ? mp : nc;
  a.pivoting = pivoting;
  a.P = P;
  a.ldp = ldp;
  a.tau = tau;
  a.U = U;
  a.ldu = ldu;
  a.perm = perm;
  a.part = part;
  a.pstride = (nc + 2) & ~1;
  a.rowbuf = rowbuf;
  a.bar = bar;
  a.err = err;
  a.spin_limit = spin_limit;
  a.sqnorm = sqnorm;
  a.ut = ut;
  a.gram_stat = gram_stat;
  const int G = panel_grid(dev, mp);
  if (HQ_PANEL_PART_ELEMS(G, nc) > part_elems) return (int)cudaErrorInvalidValue;
  a.acc = reinterpret_cast<unsigned long long*>(part + (size_t)2 * G * a.pstride);
  a.rloc_max = (mp + G - 1) / G;
  a.ldxs = a.rloc_max | 1;
  const size_t fixed = sizeof(double) * (4 * (size_t)nc) + sizeof(int) * (2 * (size_t)nc + 2);
  const size_t with_x = fixed + sizeof(double) * (size_t)a.ldxs * nc;
  size_t smem;
  if (with_x <= dev->smem_optin) {
    a.smem_mode = 1;
    smem = with_x;
  } else {
    a.smem_mode = 0;
    smem = fixed;
    if (smem > dev->smem_optin) return (int)cudaErrorInvalidValue;
  }
  cudaError_t e = cudaFuncSetAttribute(panel_qrp_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  const int z = hq_zero_words(stream, bar, 1, nullptr, 0);
  if (z) return z;
  void* args[] = {&a};
  e = hq_launch_coop((const void*)panel_qrp_kernel, dim3(G), dim3(NT), args, smem, stream);
  hq_count_launches(1);
  return (int)e;
}

extern "C" int hq_larft_from_gram(cudaStream_t stream, int k, const double* Z, int ldz,
                                  const double* tau, double* T, int ldt) {
  if (k <= 0) return 0;
  if (k > HQ_MAX_MY) return (int)cudaErrorInvalidValue;
  if (k <= LARFT_ROW_MAX) {
    const size_t rsm = sizeof(double) * ((size_t)k + (size_t)k * (k - 1) / 2);
    cudaError_t e = cudaFuncSetAttribute(larft_rows_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm);
    if (e != cudaSuccess) return (int)e;
    larft_rows_kernel<<<k, 128, rsm, stream>>>(k, Z, ldz, tau, T, ldt);
    hq_count_launches(1);
    return (int)cudaGetLastError();
  }
  const size_t smem = sizeof(double) * (size_t)k * (k | 1);
  if (smem <= 160 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(larft_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return (int)e;
    larft_kernel<<<1, 256, smem, stream>>>(k, Z, ldz, tau, T, ldt, 1);
  } else {
    larft_kernel<<<1, 256, 0, stream>>>(k, Z, ldz, tau, T, ldt, 0);
  }
  hq_count_launches(1);
  return (int)cudaGetLastError();
}
