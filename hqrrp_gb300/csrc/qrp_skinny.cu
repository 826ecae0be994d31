// qrp_skinny.cu -- per-block pivot selection: b stages of pivoted Householder
// QR on the (nb+pp) x N sketch Y, in one cooperative kernel.
//
// Reference: lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:492-507 copies
// Y_R into V_R and runs NoFLA_QRPmod_WY_unb_var4 (:774-886) with num_stages =
// b, which per stage takes idamax of the partial column norms (:828), swaps
// the columns of V, A, Y and the labels (:831-837, :990-1036), generates and
// applies a Householder reflector (dlarfg/dlarf, :845-862) and downdates the
// norms with Drmac's LAWN 176 rule, recomputing them on cancellation
// (:864-871, :912-986).  Only the pivot sequence leaves this step: V is
// discarded and the swaps of A, Y and the labels are composed into one
// permutation that a gather kernel applies afterwards.
//
// GB300 layout: the N columns are split into contiguous ranges, one range per
// CTA (one CTA per SM), and a range stays in that CTA's shared memory for all
// b stages (138 x 108 doubles = 119 KB at N = 16384, nb = 128), falling back
// to an L2-resident global copy when it does not fit.  A column never changes
// owner, so swaps are bookkeeping: each CTA tracks the current position of
// each of its columns.  Per stage there is ONE grid barrier: each CTA publishes
// its best candidate (norm, position) together with that column's entries, and
// after the barrier every CTA picks the same winner (largest norm, lowest
// position on ties -- BLAS idamax's first-maximum rule) and builds the
// reflector from the published column itself, so no second exchange is needed.
#include "hq_common.cuh"

namespace {

constexpr int NT = 256;
constexpr int NWARP = NT / 32;
constexpr int HDR = 4;                // record header: norm, position, column, spare

struct SkArgs {
  int mY, N, b;
  const double* Y;
  int ldy;
  double* Xg;  // global working copy (global mode)
  int ldxg;
  int smem_mode;
  int nloc_max;
  int ldxs;
  int* pairs;
  int* npairs;
  int max_pairs;
  double* part;  // [2][P][rec]
  int rec;
  unsigned* bar;
  int* err;
  unsigned spin_limit;
};

// Candidate order: larger norm first, then lower position.
__device__ __forceinline__ bool better(double d1, int p1, double d2, int p2) {
  return d1 > d2 || (d1 == d2 && p1 < p2);
}

__global__ void __launch_bounds__(NT, 1) skinny_qrp_kernel(SkArgs a) {
  HQ_PDL_WAIT();
  extern __shared__ __align__(16) double smem[];
  const int P = gridDim.x, cta = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int mY = a.mY;
  const int c_lo = (int)((long long)cta * a.N / P);
  const int c_hi = (int)((long long)(cta + 1) * a.N / P);
  const int nloc = c_hi - c_lo;

  // Shared-memory carve-up.
  double* sX = smem;
  double* sd = sX + (a.smem_mode ? (size_t)a.nloc_max * a.ldxs : 0);
  double* se = sd + a.nloc_max;
  double* sv = se + a.nloc_max;       // reflector, HQ_MAX_MY
  double* sred = sv + HQ_MAX_MY;      // 2 * NT scratch
  int* spos = (int*)(sred + 2 * NT);  // nloc_max
  int* sint = spos + a.nloc_max;      // small ints
  __shared__ int s_flag;
  __shared__ double s_tau;
  __shared__ int s_win_pos, s_win_cta, s_win_col;

  double* X;
  int ldx;
  if (a.smem_mode) {
    X = sX;
    ldx = a.ldxs;
  } else {
    X = a.Xg + (size_t)c_lo * a.ldxg;
    ldx = a.ldxg;
  }

  // Load the range, initialise positions and full column norms.
  for (int c = warp; c < nloc; c += NWARP) {
    const double* src = a.Y + (size_t)(c_lo + c) * a.ldy;
    double* dst = X + (size_t)c * ldx;
    double q = 0.0;
    for (int r = lane; r < mY; r += 32) {
      const double v = src[r];
      dst[r] = v;
      q = fma(v, v, q);
    }
    q = hq_warp_sum(q);
    if (lane == 0) {
      sd[c] = sqrt(q);
      se[c] = sd[c];
      spos[c] = c_lo + c;
    }
  }
  __syncthreads();

  unsigned epoch = 0;
  // Publish this CTA's best candidate for stage s, entries from row s on.
  auto publish = [&](int s) {
    double bd = -2.0;
    int bp = 0x7fffffff, bc = -1;
    for (int c = tid; c < nloc; c += NT) {
      if (spos[c] < s) continue;
      double d = sd[c];
      if (d != d) d = -1.0;  // NaN never wins over a number
      if (better(d, spos[c], bd, bp)) { bd = d; bp = spos[c]; bc = c; }
    }
    // Block argmax.
    for (int o = 16; o > 0; o >>= 1) {
      const double od = __shfl_xor_sync(0xffffffffu, bd, o);
      const int op = __shfl_xor_sync(0xffffffffu, bp, o);
      const int oc = __shfl_xor_sync(0xffffffffu, bc, o);
      if (better(od, op, bd, bp)) { bd = od; bp = op; bc = oc; }
    }
    if (lane == 0) {
      sred[warp] = bd;
      sint[warp] = bp;
      sint[NWARP + warp] = bc;
    }
    __syncthreads();
    if (tid == 0) {
      for (int w = 1; w < NWARP; ++w)
        if (better(sred[w], sint[w], bd, bp)) { bd = sred[w]; bp = sint[w]; bc = sint[NWARP + w]; }
      sint[2 * NWARP] = bc;
      double* rec = a.part + ((size_t)((epoch + 1) & 1) * P + cta) * a.rec;
      rec[0] = bd;
      rec[1] = (double)bp;
      rec[2] = (double)(bc >= 0 ? c_lo + bc : -1);
    }
    __syncthreads();
    const int cbest = sint[2 * NWARP];
    if (cbest >= 0) {
      double* rec = a.part + ((size_t)((epoch + 1) & 1) * P + cta) * a.rec;
      const double* col = X + (size_t)cbest * ldx;
      for (int r = s + tid; r < mY; r += NT) rec[HDR + r] = col[r];
    }
  };

  publish(0);
  for (int s = 0; s < a.b; ++s) {
    ++epoch;
    if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;
    const double* recs = a.part + (size_t)(epoch & 1) * P * a.rec;

    // Winner: every CTA reduces the same records in the same way.
    if (warp == 0) {
      double bd = -3.0;
      int bp = 0x7fffffff, bcta = -1;
      for (int q = lane; q < P; q += 32) {
        const double d = hq_ldcg(recs + (size_t)q * a.rec);
        const int p = (int)hq_ldcg(recs + (size_t)q * a.rec + 1);
        if (d > -2.0 && better(d, p, bd, bp)) { bd = d; bp = p; bcta = q; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double od = __shfl_xor_sync(0xffffffffu, bd, o);
        const int op = __shfl_xor_sync(0xffffffffu, bp, o);
        const int oq = __shfl_xor_sync(0xffffffffu, bcta, o);
        if (better(od, op, bd, bp)) { bd = od; bp = op; bcta = oq; }
      }
      if (lane == 0) {
        s_win_pos = bp;
        s_win_cta = bcta;
        s_win_col = bcta >= 0 ? (int)hq_ldcg(recs + (size_t)bcta * a.rec + 2) : -1;
      }
    }
    __syncthreads();
    const int wpos = s_win_pos, wcta = s_win_cta, wcol = s_win_col;
    if (wcta < 0) {  // no active column anywhere: cannot happen for b <= N
      if (tid == 0) atomicCAS(a.err, 0, HQ_ERR_BAD_SHAPE);
      return;
    }
    // Position bookkeeping for the swap of positions s and wpos.
    if (wpos != s) {
      for (int c = tid; c < nloc; c += NT)
        if (spos[c] == s) spos[c] = wpos;
    }
    __syncthreads();
    if (cta == wcta && tid == 0) spos[wcol - c_lo] = s;

    // Reflector from the published winner column (rows s..mY-1).
    const double* wrec = recs + (size_t)wcta * a.rec + HDR;
    for (int r = s + tid; r < mY; r += NT) sv[r] = hq_ldcg(wrec + r);
    __syncthreads();
    if (warp == 0) {
      double q = 0.0;
      for (int r = s + 1 + lane; r < mY; r += 32) q = fma(sv[r], sv[r], q);
      q = hq_warp_sum(q);
      if (lane == 0) {
        const HqReflector h = hq_make_reflector_sq(sv[s], q);
        s_tau = h.tau;
        sred[0] = h.scale;
      }
      __syncwarp();
      const double scale = sred[0];
      for (int r = s + 1 + lane; r < mY; r += 32) sv[r] *= scale;
      if (lane == 0) sv[s] = 1.0;
    }
    __syncthreads();
    if (s + 1 == a.b) break;  // the pivots are complete; V is discarded

    // Apply H = I - tau v v^T to every other active column and downdate its
    // norm.  One thread per column: the column's dot product, update, norm
    // test and (rare) norm recomputation need no cross-lane reduction, and no
    // FP64 work is repeated across lanes.
    const double tau = s_tau;
    for (int c = tid; c < nloc; c += NT) {
      if (spos[c] <= s) continue;
      double* x = X + (size_t)c * ldx;
      double w0 = x[s], w1 = 0.0, w2 = 0.0, w3 = 0.0;
      int r = s + 1;
      for (; r + 3 < mY; r += 4) {
        w0 = fma(sv[r], x[r], w0);
        w1 = fma(sv[r + 1], x[r + 1], w1);
        w2 = fma(sv[r + 2], x[r + 2], w2);
        w3 = fma(sv[r + 3], x[r + 3], w3);
      }
      for (; r < mY; ++r) w0 = fma(sv[r], x[r], w0);
      const double g = -tau * ((w0 + w1) + (w2 + w3));
      const double rs = x[s] + g;
      x[s] = rs;
      for (r = s + 1; r < mY; ++r) x[r] = fma(g, sv[r], x[r]);
      double dc = sd[c];
      if (dc != 0.0) {
        double t1 = fabs(rs) / dc;
        t1 = (1.0 + t1) * (1.0 - t1);
        if (0.0 > t1) t1 = 0.0;
        const double ratio = dc / se[c];
        const double t2 = t1 * ratio * ratio;
        if (t2 <= HQ_TOL3Z) {
          double q0 = 0.0, q1 = 0.0;
          for (r = s + 1; r + 1 < mY; r += 2) {
            q0 = fma(x[r], x[r], q0);
            q1 = fma(x[r + 1], x[r + 1], q1);
          }
          if (r < mY) q0 = fma(x[r], x[r], q0);
          dc = (mY - s - 1 > 0) ? sqrt(q0 + q1) : 0.0;
          sd[c] = dc;
          se[c] = dc;
        } else {
          sd[c] = dc * sqrt(t1);
        }
      }
    }
    __syncthreads();
    publish(s + 1);
  }

  // Final permutation as (dst, src) pairs for the columns that moved.
  for (int c = tid; c < nloc; c += NT) {
    if (spos[c] != c_lo + c) {
      const int i = atomicAdd(a.npairs, 1);
      if (i < a.max_pairs) {
        a.pairs[2 * i] = spos[c];
        a.pairs[2 * i + 1] = c_lo + c;
      } else {
        atomicCAS(a.err, 0, HQ_ERR_BAD_SHAPE);  // only after an aborted run
      }
    }
  }
}

// Register-resident variant: two adjacent lanes hold one sketch column, rows
// interleaved (lane parity h holds rows 2i + h, i < RPT), so a stage reads its
// columns from registers instead of shared memory; the reflector is staged in
// shared memory (zero above the stage's row, so whole chunks of 16 rows above
// it are skipped).  FP64 issue is the scarce resource on this GPU, so scalar
// work is done once, not by every thread: one lane builds the reflector, one
// thread per column downdates its norm, and pivot candidates compare integer
// keys.  Used when a CTA's range has at most NT/2 columns and mY <= 2 * RPT;
// otherwise the shared-memory kernel above runs.  Record layout (as 64-bit
// integers): [0] norm key, [1] position, [2] column, then the column's entries.
//
// T is the arithmetic of the reflector applications (the bulk of the FP64
// work): double for the plain path, float for the mixed path, whose sketch is
// formed from two-digit BF16 operands (~16 significant bits) and only steers
// pivots.  Norms, their LAWN 176 downdate and recomputation, and the
// reflector scalars are FP64 in both.  The mixed path keeps squared norms:
// d^2 <- d^2 - r^2, recomputed when d^2 - r^2 <= tol3z e^2 -- LAPACK's test
// t2 = (d^2 - r^2) / e^2 <= tol3z without its two divisions and square root
// (~1.2k cycles of FP64 latency per stage on this GPU); the argmax of d^2 is
// the argmax of d.
__device__ __forceinline__ bool better_key(long long k1, int p1, long long k2, int p2) {
  return k1 > k2 || (k1 == k2 && p1 < p2);
}

template <int RPT, typename T>
__global__ void __launch_bounds__(NT, 1) skinny_qrp_reg_kernel(SkArgs a) {
  HQ_PDL_WAIT();
  constexpr int NCH = RPT / 8;  // chunks of 8 registers = 16 rows
  constexpr bool SQ = sizeof(T) == 4;  // mixed path: squared norms
  constexpr int NC = NT / 2;
  __shared__ __align__(16) T sv[2 * RPT];   // winner column (raw; scaled in FP32)
  __shared__ __align__(16) T sv2[2 * RPT];  // the reflector v
  __shared__ long long s_bk[NWARP];
  __shared__ int s_bp[NWARP], s_bc[NWARP];
  __shared__ int spos[NC], sflag[NC];
  __shared__ double sd[NC], se[NC], srs[NC];
  __shared__ int s_flag, s_win_pos, s_win_cta, s_win_col;
  __shared__ T s_tau, s_scale;
  const int P = gridDim.x, cta = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5, h = lane & 1;
  const unsigned pmask = 3u << (lane & 30);
  const int mY = a.mY;
  const int c_lo = (int)((long long)cta * a.N / P);
  const int c_hi = (int)((long long)(cta + 1) * a.N / P);
  const int nloc = c_hi - c_lo;
  const int c = tid >> 1;  // this pair's local column
  const bool have = c < nloc;

  T x[RPT];
  // FP32 registers hold the column times 2^-ec (ec from its norm), so FP32's
  // range never limits the input; unscale = 2^ec converts back (exact).
  double unscale = 1.0;
  {
    const double* src = a.Y + (size_t)(c_lo + (have ? c : 0)) * a.ldy;
    double q = 0.0;
    if constexpr (SQ) {
#pragma unroll 8
      for (int i = 0; i < RPT; ++i) {
        const int r = 2 * i + h;
        const double y = (have && r < mY) ? src[r] : 0.0;
        q = fma(y, y, q);
      }
      q += __shfl_xor_sync(0xffffffffu, q, 1);
      int eq = (int)((__double_as_longlong(q) >> 52) & 0x7FF) - 1023;  // q >= 0
      if (eq < -1022) eq = -1022;
      const int ec = eq / 2;
      const double sc = __longlong_as_double((long long)(1023 - ec) << 52);
      unscale = __longlong_as_double((long long)(1023 + ec) << 52);
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int r = 2 * i + h;
        x[i] = (have && r < mY) ? (T)(src[r] * sc) : (T)0;
      }
    } else {
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int r = 2 * i + h;
        x[i] = (have && r < mY) ? (T)src[r] : (T)0;
        q = fma((double)x[i], (double)x[i], q);
      }
      q += __shfl_xor_sync(0xffffffffu, q, 1);
    }
    if (have && h == 0) {
      sd[c] = SQ ? q : sqrt(q);
      se[c] = sd[c];
      spos[c] = c_lo + c;
    }
  }
  for (int r = tid; r < 2 * RPT; r += NT) sv2[r] = (T)0;
  __syncthreads();

  unsigned epoch = 0;
  // Publish this CTA's best candidate for stage s (entries from row s on).
  auto publish = [&](int s) {
    long long bk = -2;
    int bp = 0x7fffffff, bc = -1;
    if (tid < nloc && spos[tid] >= s) {
      bk = hq_norm_key(sd[tid]);
      bp = spos[tid];
      bc = tid;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const long long ok = __shfl_xor_sync(0xffffffffu, bk, o);
      const int op = __shfl_xor_sync(0xffffffffu, bp, o);
      const int oc = __shfl_xor_sync(0xffffffffu, bc, o);
      if (better_key(ok, op, bk, bp)) { bk = ok; bp = op; bc = oc; }
    }
    if (lane == 0) { s_bk[warp] = bk; s_bp[warp] = bp; s_bc[warp] = bc; }
    __syncthreads();
    bk = s_bk[0];
    bp = s_bp[0];
    bc = s_bc[0];
    for (int w = 1; w < NWARP; ++w)
      if (better_key(s_bk[w], s_bp[w], bk, bp)) { bk = s_bk[w]; bp = s_bp[w]; bc = s_bc[w]; }
    double* rec = a.part + ((size_t)((epoch + 1) & 1) * P + cta) * a.rec;
    if (tid == 0) {
      long long* hdr = reinterpret_cast<long long*>(rec);
      hdr[0] = bk;
      hdr[1] = bp;
      hdr[2] = bc >= 0 ? c_lo + bc : -1;
    }
    if (bc >= 0 && c == bc) {
      T* recd = reinterpret_cast<T*>(rec + HDR);
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int r = 2 * i + h;
        if (r >= s && r < mY) recd[r] = x[i];
      }
    }
  };

  publish(0);
  for (int s = 0; s < a.b; ++s) {
    ++epoch;
    if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;
    const double* recs = a.part + (size_t)(epoch & 1) * P * a.rec;

    // Winner: every CTA reduces the same records in the same way; all header
    // loads are issued before any is used.
    if (warp == 0) {
      constexpr int QL = 5;  // records per lane: P <= 160
      long long kk[QL];
      int pp[QL], cc[QL];
#pragma unroll
      for (int j = 0; j < QL; ++j) {
        const int q = lane + 32 * j;
        const long long* hdr = reinterpret_cast<const long long*>(recs + (size_t)q * a.rec);
        kk[j] = q < P ? hq_ldcg(hdr) : -3;
        pp[j] = q < P ? (int)hq_ldcg(hdr + 1) : 0x7fffffff;
        cc[j] = q < P ? (int)hq_ldcg(hdr + 2) : -1;
      }
      long long bk = -3;
      int bp = 0x7fffffff, bq = -1, bcol = -1;
#pragma unroll
      for (int j = 0; j < QL; ++j)
        if (kk[j] > -2 && better_key(kk[j], pp[j], bk, bp)) {
          bk = kk[j];
          bp = pp[j];
          bq = lane + 32 * j;
          bcol = cc[j];
        }
      for (int o = 16; o > 0; o >>= 1) {
        const long long ok = __shfl_xor_sync(0xffffffffu, bk, o);
        const int op = __shfl_xor_sync(0xffffffffu, bp, o);
        const int oq = __shfl_xor_sync(0xffffffffu, bq, o);
        const int ocol = __shfl_xor_sync(0xffffffffu, bcol, o);
        if (better_key(ok, op, bk, bp)) { bk = ok; bp = op; bq = oq; bcol = ocol; }
      }
      if (lane == 0) {
        s_win_pos = bp;
        s_win_cta = bq;
        s_win_col = bcol;
      }
    }
    __syncthreads();
    const int wpos = s_win_pos, wcta = s_win_cta, wcol = s_win_col;
    if (wcta < 0) {  // no active column anywhere: cannot happen for b <= N
      if (tid == 0) atomicCAS(a.err, 0, HQ_ERR_BAD_SHAPE);
      return;
    }
    // Position bookkeeping for the swap of positions s and wpos (columns are
    // never moved).
    if (tid < nloc) {
      if (wpos != s && spos[tid] == s) spos[tid] = wpos;
      if (cta == wcta && c_lo + tid == wcol) spos[tid] = s;
    }
    // Winner column, rows s..mY-1.
    const T* wrec = reinterpret_cast<const T*>(recs + (size_t)wcta * a.rec + HDR);
    for (int r = s + tid; r < mY; r += NT) sv[r] = __ldcg(wrec + r);
    __syncthreads();
    if (s + 1 == a.b) break;  // the pivots are complete; V is discarded
    // Warp 0: tail norm, reflector (one lane), v = [1; scale * tail].  In
    // FP32 the reflector of the scaled column is built directly (it does not
    // depend on the column's scale): beta = -sign(alpha) sqrt(alpha^2 + q),
    // tau = (beta - alpha) / beta, scale = 1 / (alpha - beta); tau = 0 when
    // the tail is zero.
    if (warp == 0) {
      T q = (T)0;
      for (int r = s + 1 + lane; r < mY; r += 32) q = fma(sv[r], sv[r], q);
      q = hq_warp_sum(q);
      if (lane == 0) {
        if constexpr (SQ) {
          const float alpha = sv[s];
          float tau = 0.f, scale = 0.f;
          if (q > 0.f) {
            const float beta = -copysignf(sqrtf(fmaf(alpha, alpha, q)), alpha);
            tau = (beta - alpha) / beta;
            scale = 1.f / (alpha - beta);
          }
          s_tau = tau;
          s_scale = scale;
        } else {
          const HqReflector hr = hq_make_reflector_sq(sv[s], q);
          s_tau = hr.tau;
          s_scale = hr.scale;
        }
      }
      __syncwarp();
      const T scale = s_scale;
      for (int r = s + 1 + lane; r < mY; r += 32) sv2[r] = scale * sv[r];
      if (lane == 0) {
        sv2[s] = (T)1;
        if (s > 0) sv2[s - 1] = (T)0;
      }
    }
    __syncthreads();

    // Apply H = I - tau v v^T to this pair's column (if still active); the
    // new entry of row s goes to srs for the downdate.
    const bool active = have && spos[c] > s;
    if (active) {
      const int sch = s >> 4;  // first chunk holding a row >= s
      T w = (T)0;
      if constexpr (SQ) {  // two chains: half the FP32 latency
        T w1 = (T)0;
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) {
          if (ch >= sch && 16 * ch < mY) {
#pragma unroll
            for (int j = 0; j < 8; j += 2) {
              w = fma(sv2[16 * ch + 2 * j + h], x[8 * ch + j], w);
              w1 = fma(sv2[16 * ch + 2 * j + 2 + h], x[8 * ch + j + 1], w1);
            }
          }
        }
        w += w1;
      } else {
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) {
          if (ch >= sch && 16 * ch < mY) {
#pragma unroll
            for (int j = 0; j < 8; ++j) w = fma(sv2[16 * ch + 2 * j + h], x[8 * ch + j], w);
          }
        }
      }
      w += __shfl_xor_sync(pmask, w, 1);
      const T g = (T)(-s_tau) * w;
      T xs_new = (T)0;
#pragma unroll
      for (int ch = 0; ch < NCH; ++ch) {
        if (ch >= sch && 16 * ch < mY) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            x[8 * ch + j] = fma(g, sv2[16 * ch + 2 * j + h], x[8 * ch + j]);
            if (16 * ch + 2 * j + h == s) xs_new = x[8 * ch + j];
          }
        }
      }
      if (h == (s & 1)) srs[c] = SQ ? (double)xs_new * unscale : (double)xs_new;
    }
    __syncthreads();
    // Norm downdate, one thread per column (LAWN 176); flagged norms are
    // recomputed from the pair's registers.
    int flag = 0;
    if (tid < nloc && spos[tid] > s) {
      double dc = sd[tid];
      if (dc != 0.0) {
        if (SQ) {
          const double r = srs[tid];
          const double nd = fma(-r, r, dc);
          if (nd <= HQ_TOL3Z * se[tid]) flag = 1;
          else sd[tid] = nd;
        } else {
          double t1 = fabs(srs[tid]) / dc;
          t1 = (1.0 + t1) * (1.0 - t1);
          if (0.0 > t1) t1 = 0.0;
          const double ratio = dc / se[tid];
          const double t2 = t1 * ratio * ratio;
          if (t2 <= HQ_TOL3Z) flag = 1;
          else sd[tid] = dc * sqrt(t1);
        }
      }
    }
    if (tid < NC) sflag[tid] = flag;
    if (__syncthreads_or(flag)) {
      if (active && sflag[c]) {
        double q2 = 0.0;
        if constexpr (SQ) {
          float f0 = 0.f, f1 = 0.f;
#pragma unroll
          for (int i = 0; i < RPT; i += 2) {
            if (2 * i + h > s) f0 = fmaf(x[i], x[i], f0);
            if (i + 1 < RPT && 2 * (i + 1) + h > s) f1 = fmaf(x[i + 1], x[i + 1], f1);
          }
          f0 += f1;
          f0 += __shfl_xor_sync(pmask, f0, 1);
          q2 = (double)f0 * (unscale * unscale);
        } else {
#pragma unroll
          for (int i = 0; i < RPT; ++i) {
            const int r = 2 * i + h;
            if (r > s) q2 = fma((double)x[i], (double)x[i], q2);
          }
          q2 += __shfl_xor_sync(pmask, q2, 1);
        }
        const double dc = (mY - s - 1 > 0) ? (SQ ? q2 : sqrt(q2)) : 0.0;
        if (h == 0) {
          sd[c] = dc;
          se[c] = dc;
        }
      }
      __syncthreads();
    }
    publish(s + 1);
  }

  // Final permutation as (dst, src) pairs for the columns that moved.
  for (int cc = tid; cc < nloc; cc += NT) {
    if (spos[cc] != c_lo + cc) {
      const int i = atomicAdd(a.npairs, 1);
      if (i < a.max_pairs) {
        a.pairs[2 * i] = spos[cc];
        a.pairs[2 * i + 1] = c_lo + cc;
      } else {
        atomicCAS(a.err, 0, HQ_ERR_BAD_SHAPE);  // only after an aborted run
      }
    }
  }
}

int skinny_grid(const hq_device_info* dev, int N) {
  int p = (N + 15) / 16;
  if (p > dev->num_sms) p = dev->num_sms;
  return p < 1 ? 1 : p;
}

}  // namespace

extern "C" size_t hq_skinny_part_elems(const hq_device_info* dev, int mY) {
  const int rec = HDR + ((mY + 1) & ~1);
  return (size_t)2 * dev->num_sms * rec;
}

extern "C" int hq_skinny_qrp(cudaStream_t stream, const hq_device_info* dev, int mY, int N,
                             int b, const double* Y, int ldy, double* V, int ldv, int* pairs,
                             int* npairs, double* part, size_t part_elems, unsigned* bar,
                             int* err, unsigned spin_limit, int fp32) {
  if (mY > HQ_MAX_MY || b > mY || b > N || b <= 0) return (int)cudaErrorInvalidValue;
  SkArgs a;
  a.mY = mY;
  a.N = N;
  a.b = b;
  a.Y = Y;
  a.ldy = ldy;
  a.Xg = V;
  a.ldxg = ldv;
  a.pairs = pairs;
  a.npairs = npairs;
  a.max_pairs = 2 * b;
  a.part = part;
  a.rec = HDR + ((mY + 1) & ~1);
  a.bar = bar;
  a.err = err;
  a.spin_limit = spin_limit;
  // The register kernel holds up to NT / 2 columns per CTA; with as few CTAs
  // as that allows, each stage's grid barrier has fewer arrivals to wait for
  // (the per-column arithmetic, and so the pivots, do not depend on the
  // partition).  The shared-memory kernel keeps one CTA per 16 columns up to
  // one per SM.
  const int p_reg = (N + NT / 2 - 1) / (NT / 2);
  const bool reg_fit = mY <= 2 * 72 && p_reg <= dev->num_sms && p_reg <= 160;
  const int P = reg_fit ? (p_reg < 1 ? 1 : p_reg) : skinny_grid(dev, N);
  if ((size_t)2 * P * a.rec > part_elems) return (int)cudaErrorInvalidValue;
  a.nloc_max = (N + P - 1) / P;
  a.ldxs = mY | 1;
  const size_t fixed = sizeof(double) * (2 * (size_t)a.nloc_max + HQ_MAX_MY + 2 * NT) +
                       sizeof(int) * ((size_t)a.nloc_max + 4 * NWARP + 8);
  const size_t with_x = fixed + sizeof(double) * (size_t)a.nloc_max * a.ldxs;
  size_t smem;
  if (with_x <= dev->smem_optin) {
    a.smem_mode = 1;
    smem = with_x;
  } else {
    a.smem_mode = 0;
    smem = fixed;
    if (V == nullptr || smem > dev->smem_optin) return (int)cudaErrorInvalidValue;
  }
  cudaError_t e;
  const int z = hq_zero_words(stream, bar, 1, npairs, 1);
  if (z) return z;
  void* args[] = {&a};
  const void* fn = nullptr;
  const bool reg_ok = a.nloc_max <= NT / 2 && P <= 160;  // 5 records per lane in the winner pick
  if (reg_ok && mY <= 2 * 40)
    fn = fp32 ? (const void*)skinny_qrp_reg_kernel<40, float> : (const void*)skinny_qrp_reg_kernel<40, double>;
  else if (reg_ok && mY <= 2 * 72)
    fn = fp32 ? (const void*)skinny_qrp_reg_kernel<72, float> : (const void*)skinny_qrp_reg_kernel<72, double>;
  if (fn != nullptr) {
    e = hq_launch_coop(fn, dim3(P), dim3(NT), args, 0, stream);
  } else {
    e = cudaFuncSetAttribute(skinny_qrp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return (int)e;
    e = hq_launch_coop((const void*)skinny_qrp_kernel, dim3(P), dim3(NT), args, smem, stream);
  }
  hq_count_launches(1);
  return (int)e;
}
