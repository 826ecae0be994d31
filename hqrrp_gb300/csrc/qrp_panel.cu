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
// barrier: every CTA publishes, for its slab, the dot products of the pivot
// column with all not-yet-factored columns (the first of which is the pivot
// column's squared norm); the owner of the pivot row also publishes that row.
// After the barrier all CTAs hold the same reduced values (summed in a fixed
// order, so results are reproducible) and apply the reflector to their slab
// without further communication.  The rare norm recomputation costs one more
// barrier in the stages that need it.
#include "hq_common.cuh"

namespace {

constexpr int NT = 256;
constexpr int NWARP = NT / 32;

struct PnArgs {
  int mp, nc, ns, pivoting;
  double* P;
  int ldp;
  double* tau;
  double* U;
  int ldu;
  int* perm;
  double* part;  // [2][grid][pstride]
  int pstride;
  double* rowbuf;  // [2][nc]
  unsigned* bar;
  int* err;
  unsigned spin_limit;
  int smem_mode, rloc_max, ldxs;
};

__global__ void __launch_bounds__(NT, 1) panel_qrp_kernel(PnArgs a) {
  extern __shared__ __align__(16) double smem[];
  const int G = gridDim.x, cta = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int nc = a.nc;
  const int r_lo = (int)((long long)cta * a.mp / G);
  const int r_hi = (int)((long long)(cta + 1) * a.mp / G);
  const int nloc = r_hi - r_lo;

  double* sX = smem;
  double* sd = sX + (a.smem_mode ? (size_t)a.ldxs * nc : 0);
  double* se = sd + nc;
  double* sw = se + nc;    // reduced dots, then w_k = tau * v^T X[:, k]
  double* snew = sw + nc;  // new pivot-row entries
  double* sred = snew + nc;  // NT scratch
  int* sperm = (int*)(sred + NT);
  int* sflag = sperm + nc;
  __shared__ int s_flag, s_any;
  __shared__ double s_tau, s_scale, s_beta;
  __shared__ double s_bd[NWARP];
  __shared__ int s_bk[NWARP];

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
  for (int k = tid; k < nc; k += NT) sperm[k] = k;
  // A valid permutation is in place before any wait: if a barrier gives up
  // and the kernel returns early, the gathers that follow still read indices
  // within range.
  if (cta == 0)
    for (int k = tid; k < nc; k += NT) a.perm[k] = k;
  __syncthreads();

  unsigned epoch = 0;
  auto part_w = [&](unsigned e) { return a.part + ((size_t)(e & 1) * G + cta) * a.pstride; };
  auto part_r = [&](unsigned e) { return a.part + (size_t)(e & 1) * G * a.pstride; };

  // Work split for na columns over NT threads: below NT columns, `groups`
  // threads share a column (each takes every groups-th item of the other
  // dimension) and their sums are combined in sred in a fixed order; from NT
  // columns up, each thread owns columns tid, tid + NT, ...

  // Sum over CTAs of the published values [0, na) into sw[0..na), in a
  // fixed order.  Loads are issued in batches of RB independent L2 reads per
  // thread so the reduction costs a few L2 round trips, not one per CTA.
  constexpr int RB = 32;
  auto reduce_parts = [&](unsigned e, int na) {
    const double* base = part_r(e);
    const int groups = na >= NT ? 1 : NT / na;
    for (int q0 = 0; q0 < na; q0 += NT) {
      const int q = q0 + tid % min(na, NT), g = tid / min(na, NT);
      double t = 0.0;
      if (g < groups && q < na) {
        for (int c0 = g; c0 < G; c0 += groups * RB) {
          double v[RB];
#pragma unroll
          for (int u = 0; u < RB; ++u) {
            const int c = c0 + u * groups;
            v[u] = c < G ? hq_ldcg(base + (size_t)c * a.pstride + q) : 0.0;
          }
#pragma unroll
          for (int u = 0; u < RB; ++u) t += v[u];
        }
      }
      if (groups == 1) {
        if (g == 0 && q < na) sw[q] = t;
      } else {
        sred[tid] = t;
        __syncthreads();
        if (tid < na) {
          double u = 0.0;
          for (int gg = 0; gg < groups; ++gg) u += sred[gg * na + tid];
          sw[tid] = u;
        }
      }
      __syncthreads();
    }
  };

  // Slab-local sums over rows with global index > lo_row of x_i * X[i, k]
  // (x = column xs, or column k itself when xs < 0) for k in [k0, nc),
  // skipping columns without sflag when use_mask; written to out[k - k0].
  auto slab_dots = [&](int xs, int k0, int lo_row, bool use_mask, double* out) {
    const int na = nc - k0;
    const int i0 = max(0, lo_row + 1 - r_lo);
    if (na >= NT) {
      for (int q = tid; q < na; q += NT) {
        const int k = k0 + q;
        double t = 0.0;
        if (!use_mask || sflag[k]) {
          const double* xk = X + (size_t)k * ldx;
          const double* xx = xs >= 0 ? X + (size_t)xs * ldx : xk;
          double t1 = 0.0;
          int i = i0;
          for (; i + 1 < nloc; i += 2) {
            t = fma(xx[i], xk[i], t);
            t1 = fma(xx[i + 1], xk[i + 1], t1);
          }
          if (i < nloc) t = fma(xx[i], xk[i], t);
          t += t1;
        }
        out[q] = t;
      }
      __syncthreads();
      return;
    }
    const int groups = NT / na;
    const int q = tid % na, g = tid / na;
    double t = 0.0;
    if (g < groups) {
      const int k = k0 + q;
      if (!use_mask || sflag[k]) {
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
    }
    sred[tid] = t;
    __syncthreads();
    if (tid < na) {
      double u = 0.0;
      for (int gg = 0; gg < groups; ++gg) u += sred[gg * na + tid];
      out[tid] = u;
    }
    __syncthreads();
  };

  // Initial norms over the whole panel.
  slab_dots(-1, 0, -1, false, part_w(epoch + 1));
  ++epoch;
  if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;
  reduce_parts(epoch, nc);
  for (int k = tid; k < nc; k += NT) {
    sd[k] = sqrt(sw[k]);
    se[k] = sd[k];
  }
  __syncthreads();

  for (int s = 0; s < a.ns; ++s) {
    const int na = nc - s;
    // 1. Pivot: first maximum of the partial norms (idamax).
    if (a.pivoting) {
      double bd = -1.0;
      int bk = 0x7fffffff;
      for (int k = s + tid; k < nc; k += NT) {
        const double d = sd[k];
        if (d > bd || (d == bd && k < bk)) { bd = d; bk = k; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double od = __shfl_xor_sync(0xffffffffu, bd, o);
        const int ok = __shfl_xor_sync(0xffffffffu, bk, o);
        if (od > bd || (od == bd && ok < bk)) { bd = od; bk = ok; }
      }
      if (lane == 0) { s_bd[warp] = bd; s_bk[warp] = bk; }
      __syncthreads();
      if (tid == 0) {
        for (int w = 1; w < NWARP; ++w)
          if (s_bd[w] > bd || (s_bd[w] == bd && s_bk[w] < bk)) { bd = s_bd[w]; bk = s_bk[w]; }
        if (bk == 0x7fffffff) bk = s;  // all norms NaN: keep the column in place
        s_any = bk;
      }
      __syncthreads();
      const int kp = s_any;
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
          sd[kp] = sd[s];
          se[kp] = se[s];
        }
      }
      __syncthreads();
    }

    // 2. Publish slab dots with the pivot column (rows > s) and, from the
    //    owner of row s, that row.
    slab_dots(s, s, s, false, part_w(epoch + 1));
    if (s >= r_lo && s < r_hi) {
      double* rb = a.rowbuf + (size_t)((epoch + 1) & 1) * nc;
      for (int k = s + tid; k < nc; k += NT) rb[k] = X[(s - r_lo) + (size_t)k * ldx];
    }
    ++epoch;
    if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;

    // 3. Reduce; build the reflector; w_k = tau * v^T X[:, k].
    reduce_parts(epoch, na);
    const double* rb = a.rowbuf + (size_t)(epoch & 1) * nc;
    if (tid == 0) {
      const double alpha = hq_ldcg(rb + s);
      const HqReflector h = hq_make_reflector(alpha, (a.mp - s > 1) ? sqrt(sw[0]) : 0.0);
      s_tau = h.tau;
      s_scale = h.scale;
      s_beta = h.beta;
      if (cta == 0) a.tau[s] = h.tau;
    }
    __syncthreads();
    const double tau = s_tau, scale = s_scale;
    // sw[k - s] (k > s) becomes w_k; snew[k] is the new pivot-row entry.
    for (int k = s + 1 + tid; k < nc; k += NT) {
      const double row = hq_ldcg(rb + k);
      const double w = tau * fma(scale, sw[k - s], row);
      sw[k - s] = w;
      snew[k] = row - w;
    }
    __syncthreads();
    // 4. Update the slab: X[i,k] -= (scale * x_i) * w_k for rows > s.
    {
      const int nt = nc - s - 1;
      const int i0 = max(0, s + 1 - r_lo);
      const bool own = (s >= r_lo && s < r_hi);
      const double* xs = X + (size_t)s * ldx;
      if (nt >= NT) {
        for (int q = tid; q < nt; q += NT) {
          const int k = s + 1 + q;
          const double wk = sw[q + 1];
          double* xk = X + (size_t)k * ldx;
          for (int i = i0; i < nloc; ++i) xk[i] = fma(-(scale * xs[i]), wk, xk[i]);
          if (own) xk[s - r_lo] = snew[k];
        }
      } else if (nt > 0) {
        const int groups = NT / nt;
        const int q = tid % nt, g = tid / nt;
        if (g < groups) {
          const int k = s + 1 + q;
          const double wk = sw[q + 1];
          double* xk = X + (size_t)k * ldx;
          for (int i = i0 + g; i < nloc; i += groups) xk[i] = fma(-(scale * xs[i]), wk, xk[i]);
          if (own && g == 0) xk[s - r_lo] = snew[k];
        }
      }
    }
    __syncthreads();
    {
      double* xs = X + (size_t)s * ldx;
      const int i0 = max(0, s + 1 - r_lo);
      for (int i = i0 + tid; i < nloc; i += NT) xs[i] *= scale;
      if (tid == 0 && s >= r_lo && s < r_hi) xs[s - r_lo] = s_beta;
    }

    // 5. Norm downdate; recompute flagged norms with one more barrier.
    if (a.pivoting) {
      int any = 0;
      for (int k = s + 1 + tid; k < nc; k += NT) {
        int flag = 0;
        double dk = sd[k];
        if (dk != 0.0) {
          const double r = snew[k];
          double t1 = fabs(r) / dk;
          t1 = (1.0 + t1) * (1.0 - t1);
          if (0.0 > t1) t1 = 0.0;
          const double ratio = dk / se[k];
          const double t2 = t1 * ratio * ratio;
          if (t2 <= HQ_TOL3Z) flag = 1;
          else sd[k] = dk * sqrt(t1);
        }
        sflag[k] = flag;
        any |= flag;
      }
      any = __syncthreads_or(any);
      if (any) {
        for (int k = tid; k <= s; k += NT) sflag[k] = 0;
        __syncthreads();
        slab_dots(-1, s, s, true, part_w(epoch + 1));
        ++epoch;
        if (!hq_grid_barrier(a.bar, a.err, epoch, a.spin_limit, &s_flag)) return;
        reduce_parts(epoch, na);
        for (int k = s + 1 + tid; k < nc; k += NT) {
          if (sflag[k]) {
            const double nv = (a.mp - s - 1 > 0) ? sqrt(sw[k - s]) : 0.0;
            sd[k] = nv;
            se[k] = nv;
          }
        }
      }
    }
    __syncthreads();
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

int panel_grid(const hq_device_info* dev, int mp) {
  int g = (mp + 63) / 64;
  if (g > dev->num_sms) g = dev->num_sms;
  return g < 1 ? 1 : g;
}

// DLARFT (Forward, Columnwise) from the Gram matrix Z = U^T U: for each i,
// T[0:i, i] = -tau_i T[0:i, 0:i] Z[0:i, i] and T[i, i] = tau_i (T[0:i, i] = 0
// when tau_i = 0).  One CTA; T is built in shared memory when it fits.
__global__ void larft_kernel(int k, const double* __restrict__ Z, int ldz,
                             const double* __restrict__ tau, double* __restrict__ T, int ldt,
                             int use_smem) {
  extern __shared__ double sT[];
  __shared__ double tmp[HQ_MAX_MY];
  double* Tm = use_smem ? sT : T;
  const int ld = use_smem ? k : ldt;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < k * k; e += nt) Tm[(e % k) + (size_t)(e / k) * ld] = 0.0;
  __syncthreads();
  for (int i = 0; i < k; ++i) {
    const double ti = tau[i];
    for (int r = tid; r < i; r += nt) tmp[r] = -ti * Z[r + (size_t)i * ldz];
    __syncthreads();
    if (ti != 0.0) {
      for (int r = tid; r < i; r += nt) {
        double s = 0.0;
        for (int c = r; c < i; ++c) s = fma(Tm[r + (size_t)c * ld], tmp[c], s);
        Tm[r + (size_t)i * ld] = s;
      }
    }
    if (tid == 0) Tm[i + (size_t)i * ld] = ti;
    __syncthreads();
  }
  if (use_smem)
    for (int e = tid; e < k * k; e += nt)
      T[(e % k) + (size_t)(e / k) * ldt] = sT[(e % k) + (size_t)(e / k) * k];
}

}  // namespace

extern "C" size_t hq_panel_part_elems(const hq_device_info* dev, int nc) {
  return (size_t)2 * dev->num_sms * (size_t)((nc + 2) & ~1);
}

extern "C" int hq_panel_qrp(cudaStream_t stream, const hq_device_info* dev, int mp, int nc,
                            int pivoting, double* P, int ldp, double* tau,
                            double* U, int ldu, int* perm, double* part, size_t part_elems,
                            double* rowbuf, unsigned* bar, int* err, unsigned spin_limit) {
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
  const int G = panel_grid(dev, mp);
  if ((size_t)2 * G * a.pstride > part_elems) return (int)cudaErrorInvalidValue;
  a.rloc_max = (mp + G - 1) / G;
  a.ldxs = a.rloc_max | 1;
  const size_t fixed = sizeof(double) * (4 * (size_t)nc + NT) + sizeof(int) * (2 * (size_t)nc + 2);
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
  if ((e = cudaMemsetAsync(bar, 0, sizeof(unsigned), stream)) != cudaSuccess) return (int)e;
  void* args[] = {&a};
  e = cudaLaunchCooperativeKernel((const void*)panel_qrp_kernel, dim3(G), dim3(NT), args, smem,
                                  stream);
  hq_count_launches(1);
  return (int)e;
}

extern "C" int hq_larft_from_gram(cudaStream_t stream, int k, const double* Z, int ldz,
                                  const double* tau, double* T, int ldt) {
  if (k <= 0) return 0;
  if (k > HQ_MAX_MY) return (int)cudaErrorInvalidValue;
  const size_t smem = sizeof(double) * (size_t)k * k;
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
