// qrp_wide.cu -- pivoted Householder QR of a short, wide matrix (m <= 1024
// rows, any number of columns), one cooperative kernel.
//
// Reference: the small-matrix branch of dgeqp4
// (lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:189-199) hands every
// matrix with min(m, n) < 1000 to LAPACK's dgeqpf or dgeqp3, whatever n is.
// Both pick, at stage s, the remaining column of largest partial norm (first
// maximum in column order, like idamax), swap it into position s (the norms
// follow their column), apply dlarfg/dlarf, and downdate the partial norms
// with the LAWN 176 test, recomputing a norm when cancellation is detected
// (the same rule as the reference's own QRPmod, :774-886 and :912-986).  The
// row-partitioned panel kernel (qrp_panel.cu) keeps per-column state of all
// columns in every CTA and so takes at most 1024 columns; this kernel takes
// the wide case.
//
// GB300 layout: the columns are split into contiguous ranges, one per CTA
// (one CTA per SM); a column never moves and never leaves its CTA.  Swaps are
// bookkeeping -- each CTA keeps the logical position of its own columns, and
// a device array maps logical positions to physical columns -- and the final
// order is applied afterwards by one gather of the displaced columns (at most
// two per stage).  Per stage there is one grid exchange: every CTA publishes
// its best candidate (norm order key, logical position, column) and, after
// the grid barrier, every CTA picks the same winner, reads the pivot column
// from L2 and builds the reflector itself (identical inputs and reduction
// order, so identical results).  Each warp then updates whole columns of its
// CTA with the column held in registers (m <= 1024: 32 rows per lane), so
// the norm downdate and the rare recomputation need no communication.  The
// pivot column's own new contents (v and beta) are written by its owner only
// after the next barrier, when no CTA reads the original values any more.
#include <climits>

#include "hq_common.cuh"

namespace {

constexpr int WT = 256;
constexpr int WW = WT / 32;
constexpr int RPL = HQ_WIDE_MAX_ROWS / 32;  // rows per lane of a register-held column

struct WdArgs {
  int m, n, ns;
  double* A;
  int lda;
  double* tau;
  int* phys;           // [n] logical position -> physical column
  long long* cand;     // [2][grid][2] candidates: order key; (position << 32) | column
  int* pairs;          // out: (dst, src) pairs of the final order
  int* npairs;         // out: their count (zeroed by the launcher)
  unsigned* bar;
  int* err;
  unsigned spin_limit;
  int cpc;             // most columns any CTA owns
};

// Candidate order: larger norm key, then lower logical position (idamax's
// first maximum).  (-2, INT_MAX, -1) is the empty candidate.
__device__ __forceinline__ void pick3(long long key, int lp, int ph, long long& bk, int& bl,
                                      int& bp) {
  if (key > bk || (key == bk && lp < bl)) {
    bk = key;
    bl = lp;
    bp = ph;
  }
}

__device__ __forceinline__ void warp_pick3(long long& bk, int& bl, int& bp) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long ok = __shfl_xor_sync(0xffffffffu, bk, o);
    const int ol = __shfl_xor_sync(0xffffffffu, bl, o);
    const int op = __shfl_xor_sync(0xffffffffu, bp, o);
    pick3(ok, ol, op, bk, bl, bp);
  }
}

__global__ void __launch_bounds__(WT, 1) wide_qrp_kernel(WdArgs a) {
  extern __shared__ __align__(16) double wsm[];
  const int G = gridDim.x, cta = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int m = a.m;
  const int c0 = (int)((long long)cta * a.n / G), c1 = (int)((long long)(cta + 1) * a.n / G);
  const int nl = c1 - c0;
  double* sv = wsm;            // [m] the stage's pivot column, then its reflector
  double* sd = sv + m;         // [cpc] partial norms of the CTA's columns
  double* se = sd + a.cpc;     // [cpc] norms at the last recomputation
  int* slp = (int*)(se + a.cpc);  // [cpc] logical positions (<= s: factored)
  __shared__ double s_red[WW];
  __shared__ long long s_k[WW];
  __shared__ int s_l[WW], s_p[WW];
  __shared__ int s_flag, s_pw, s_lpw, s_ps;
  __shared__ double s_tau, s_scale, s_beta;

  for (int p = cta * WT + tid; p < a.n; p += G * WT) a.phys[p] = p;
  for (int q = tid; q < nl; q += WT) slp[q] = c0 + q;
  // Initial norms, one warp per column.
  for (int q = warp; q < nl; q += WW) {
    const double* x = a.A + (size_t)(c0 + q) * a.lda;
    double t = 0.0;
    for (int i = lane; i < m; i += 32) t = fma(x[i], x[i], t);
    t = hq_warp_sum(t);
    if (lane == 0) {
      sd[q] = sqrt(t);
      se[q] = sd[q];
    }
  }
  __syncthreads();

  // The CTA's best not-yet-factored column (position >= s_next) goes to
  // candidate buffer s_next & 1; it is read after the next barrier and
  // rewritten two stages later, after a barrier every reader has passed.
  auto publish = [&](int s_next, long long bk, int bl, int bp) {
    warp_pick3(bk, bl, bp);
    if (lane == 0) {
      s_k[warp] = bk;
      s_l[warp] = bl;
      s_p[warp] = bp;
    }
    __syncthreads();
    if (tid == 0) {
      bk = s_k[0];
      bl = s_l[0];
      bp = s_p[0];
      for (int w = 1; w < WW; ++w) pick3(s_k[w], s_l[w], s_p[w], bk, bl, bp);
      long long* c = a.cand + ((size_t)(s_next & 1) * G + cta) * 2;
      c[0] = bk;
      c[1] = ((long long)bl << 32) | (long long)(unsigned)bp;
    }
  };
  {
    long long bk = -2;
    int bl = INT_MAX, bp = -1;
    for (int q = tid; q < nl; q += WT) pick3(hq_norm_key(sd[q]), slp[q], c0 + q, bk, bl, bp);
    publish(0, bk, bl, bp);
  }

  // Deferred writes: the owner's reflector (v = scale * x below row pend_s,
  // beta on it) and CTA 0's phys[pend_s] = pivot column, both applied after
  // the next barrier, when no CTA reads the old values any more.
  int pend_col = -1, pend_s = 0, pend_phys = -1;
  double pend_scale = 0.0, pend_beta = 0.0;
  auto flush = [&]() {
    if (pend_col >= 0) {
      double* x = a.A + (size_t)pend_col * a.lda;
      for (int i = pend_s + 1 + tid; i < m; i += WT) x[i] *= pend_scale;
      if (tid == 0) x[pend_s] = pend_beta;
      pend_col = -1;
    }
    if (pend_phys >= 0) {
      if (tid == 0) a.phys[pend_s] = pend_phys;
      pend_phys = -1;
    }
  };

  unsigned epoch = 0;
  for (int s = 0; s < a.ns; ++s) {
    ++epoch;
    if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;
    flush();

    // 1. The winner, in every CTA; CTA 0 records the swap.
    if (warp == 0) {
      long long bk = -2;
      int bl = INT_MAX, bp = -1;
      for (int c = lane; c < G; c += 32) {
        const long long* cp = a.cand + ((size_t)(s & 1) * G + c) * 2;
        const long long k = __ldcg(cp), v = __ldcg(cp + 1);
        pick3(k, (int)(v >> 32), (int)(v & 0xffffffffLL), bk, bl, bp);
      }
      warp_pick3(bk, bl, bp);
      if (lane == 0) {
        const int ps = __ldcg(a.phys + s);
        if (bp < 0 || bk < 0 || bl < s || bl >= a.n) {  // nothing valid (NaN norms): keep s
          bp = ps;
          bl = s;
        }
        s_pw = bp;
        s_lpw = bl;
        s_ps = ps;
        if (cta == 0 && bl != s) a.phys[bl] = ps;
      }
    }
    __syncthreads();
    const int pw = s_pw, lpw = s_lpw, ps = s_ps;
    if (cta == 0) {
      pend_phys = pw;
      pend_s = s;
    }
    if (tid == 0) {
      if (ps >= c0 && ps < c1) slp[ps - c0] = lpw;  // the column displaced from position s
      if (pw >= c0 && pw < c1) slp[pw - c0] = s;    // the pivot: factored from now on
    }

    // 2. The pivot column (rows >= s) and the reflector.
    {
      const double* xp = a.A + (size_t)pw * a.lda;
      double t = 0.0;
      for (int i = s + tid; i < m; i += WT) {
        const double v = __ldcg(xp + i);
        sv[i] = v;
        if (i > s) t = fma(v, v, t);
      }
      t = hq_warp_sum(t);
      if (lane == 0) s_red[warp] = t;
      __syncthreads();
      if (tid == 0) {
        double q = s_red[0];
        for (int w = 1; w < WW; ++w) q += s_red[w];
        const HqReflector h = hq_make_reflector_sq(sv[s], (m - s > 1) ? q : 0.0);
        s_tau = h.tau;
        s_scale = h.scale;
        s_beta = h.beta;
        if (cta == 0) a.tau[s] = h.tau;
      }
      __syncthreads();
    }
    const double tau = s_tau, scale = s_scale;
    for (int i = s + 1 + tid; i < m; i += WT) sv[i] *= scale;
    if (tid == 0) sv[s] = 1.0;
    if (pw >= c0 && pw < c1) {
      pend_col = pw;
      pend_s = s;
      pend_scale = scale;
      pend_beta = s_beta;
    }
    __syncthreads();

    // 3. Update the CTA's remaining columns, one warp per column held in
    //    registers; LAWN 176 norm downdate with recomputation; candidates.
    long long bk = -2;
    int bl = INT_MAX, bp = -1;
    for (int q = warp; q < nl; q += WW) {
      const int lp = slp[q];
      if (lp <= s) continue;  // factored (uniform across the warp)
      double* x = a.A + (size_t)(c0 + q) * a.lda;
      double xr[RPL];
      double dot = 0.0;
#pragma unroll
      for (int t = 0; t < RPL; ++t) {
        const int i = lane + 32 * t;
        const bool in = i >= s && i < m;
        xr[t] = in ? x[i] : 0.0;
        if (in) dot = fma(sv[i], xr[t], dot);
      }
      dot = hq_warp_sum(dot);
      const double wk = tau * dot;
      double rl = 0.0;
#pragma unroll
      for (int t = 0; t < RPL; ++t) {
        const int i = lane + 32 * t;
        if (i >= s && i < m) {
          xr[t] = fma(-sv[i], wk, xr[t]);
          x[i] = xr[t];
          if (i == s) rl = xr[t];
        }
      }
      const double r = __shfl_sync(0xffffffffu, rl, s & 31);  // the new entry of row s
      double dk = sd[q], ek = se[q];
      bool flag = false;
      if (dk != 0.0) {
        double t1 = fabs(r) / dk;
        t1 = (1.0 + t1) * (1.0 - t1);
        if (0.0 > t1) t1 = 0.0;
        const double ratio = dk / ek;
        if (t1 * ratio * ratio <= HQ_TOL3Z) flag = true;
        else dk *= sqrt(t1);
      }
      if (flag) {
        double ss = 0.0;
#pragma unroll
        for (int t = 0; t < RPL; ++t) {
          const int i = lane + 32 * t;
          if (i > s && i < m) ss = fma(xr[t], xr[t], ss);
        }
        ss = hq_warp_sum(ss);
        dk = (m - s - 1 > 0) ? sqrt(ss) : 0.0;
        ek = dk;
      }
      if (lane == 0) {
        sd[q] = dk;
        se[q] = ek;
      }
      pick3(hq_norm_key(dk), lp, c0 + q, bk, bl, bp);
    }
    publish(s + 1, bk, bl, bp);
  }

  // Every CTA is past its last read of the last pivot column and of phys[].
  ++epoch;
  if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;
  flush();
  ++epoch;
  if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;
  // The final order as (dst, src) pairs of the displaced positions.
  for (int p = cta * WT + tid; p < a.n; p += G * WT) {
    const int ph = __ldcg(a.phys + p);
    if (ph != p) {
      const int i = atomicAdd(a.npairs, 1);
      a.pairs[2 * i] = p;
      a.pairs[2 * i + 1] = ph;
    }
  }
}

int wide_grid(const hq_device_info* dev, int n) {
  int g = dev->num_sms;
  if (g > n) g = n;
  return g < 1 ? 1 : g;
}

}  // namespace

extern "C" size_t hq_wide_cand_elems(const hq_device_info* dev) {
  return 4 * (size_t)dev->num_sms;
}

extern "C" int hq_wide_qrp(cudaStream_t stream, const hq_device_info* dev, int m, int n,
                           double* A, int lda, double* tau, int* phys, long long* cand,
                           int* pairs, int* npairs, unsigned* bar, int* err,
                           unsigned spin_limit) {
  if (m <= 0 || n <= 0) return 0;
  if (m > HQ_WIDE_MAX_ROWS || lda < m) return (int)cudaErrorInvalidValue;
  WdArgs a;
  a.m = m;
  a.n = n;
  a.ns = m < n ? m : n;
  a.A = A;
  a.lda = lda;
  a.tau = tau;
  a.phys = phys;
  a.cand = cand;
  a.pairs = pairs;
  a.npairs = npairs;
  a.bar = bar;
  a.err = err;
  a.spin_limit = spin_limit;
  const int G = wide_grid(dev, n);
  a.cpc = (n + G - 1) / G;
  const size_t smem = sizeof(double) * ((size_t)m + 2 * (size_t)a.cpc) + sizeof(int) * (size_t)a.cpc;
  if (smem > dev->smem_optin) return (int)cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(wide_qrp_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  if ((e = cudaMemsetAsync(bar, 0, sizeof(unsigned), stream)) != cudaSuccess) return (int)e;
  if ((e = cudaMemsetAsync(npairs, 0, sizeof(int), stream)) != cudaSuccess) return (int)e;
  void* args[] = {&a};
  e = cudaLaunchCooperativeKernel((const void*)wide_qrp_kernel, dim3(G), dim3(WT), args, smem,
                                  stream);
  hq_count_launches(1);
  return (int)e;
}
