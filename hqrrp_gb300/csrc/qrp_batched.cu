// qrp_batched.cu -- thousands of independent small pivoted QRs in one
// persistent launch.
//
// dgeqp4 hands every matrix with min(m, n) < 1000 to LAPACK's dgeqpf / dgeqp3
// (lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:189-199); both produce
// the Businger-Golub column-pivoted Householder QR with LAWN 176 norm
// downdating, the algorithm restated per matrix here (one CTA per matrix).
// A batch is scheduled through a device work queue: the host orders the
// matrices by cost (largest first), and each resident CTA takes the next
// index with an atomic until the queue is empty, so uneven sizes balance
// across the SMs.  A matrix is staged in shared memory when it fits in the
// launch's staging budget and worked on in place (L2-resident) otherwise.
// The launch shape -- threads per CTA and the staging budget -- is chosen by
// the host autotuner (hqrrp_driver.c) per batch signature.
//
// All columns are free (LAPACK jpvt = 0 input); on return jpvt[k] is the
// 1-based original index of column k, tau[0..min(m,n)) the reflector scalars,
// R and the reflectors overwrite A.
#include "hq_common.cuh"

namespace {

struct BatchArgs {
  int batch;
  const int* m;
  const int* n;
  double* const* A;
  const int* lda;
  int* const* jpvt;
  double* const* tau;
  int* info;
  const int* order;  // schedule: matrix indices, largest first
  int* next;         // queue head (zeroed before the launch)
  int stage_bytes;   // dynamic shared memory available for staging a matrix
  int max_n;
};

template <int NT>
__global__ void __launch_bounds__(NT) qrp_batched_kernel(BatchArgs a) {
  extern __shared__ __align__(16) double smem[];
  constexpr int NW = NT / 32;
  __shared__ int s_item, s_kp;
  __shared__ double s_red[NW];
  __shared__ int s_bk[NW];
  __shared__ double s_tau, s_scale, s_beta;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double* sd = smem;                 // partial norms, max_n
  double* se = sd + a.max_n;         // norms at the last recomputation, max_n
  double* sw = se + a.max_n;         // spare, max_n
  int* sperm = (int*)(sw + a.max_n);  // max_n
  double* sX = (double*)(sperm + ((a.max_n + 1) & ~1));

  for (;;) {
    if (tid == 0) {
      const int q = atomicAdd(a.next, 1);
      s_item = q < a.batch ? a.order[q] : -1;
    }
    __syncthreads();
    const int item = s_item;
    __syncthreads();
    if (item < 0) break;
    const int m = a.m[item], n = a.n[item], lda = a.lda[item];
    double* Ag = a.A[item];
    // A size the kernel cannot take (negative, lda < max(1, m), more than
    // max_n columns) is flagged and left untouched; an empty matrix is done.
    const bool bad = m < 0 || n < 0 || n > a.max_n || lda < max(1, m);
    if (bad || m == 0 || n == 0) {
      if (tid == 0 && a.info) a.info[item] = bad ? HQ_ERR_BAD_SHAPE : 0;
      continue;
    }
    const int lds = m;
    const bool staged = (long long)lds * n * 8 <= a.stage_bytes;
    double* X = staged ? sX : Ag;
    const int ldx = staged ? lds : lda;
    if (staged)
      for (long long e = tid; e < (long long)m * n; e += NT) {
        const int i = (int)(e % m), k = (int)(e / m);
        sX[i + (long long)k * lds] = Ag[i + (long long)k * lda];
      }
    __syncthreads();
    // Initial norms (warp per column, fixed lane order).
    for (int k = warp; k < n; k += NW) {
      const double* x = X + (long long)k * ldx;
      double q = 0.0;
      for (int i = lane; i < m; i += 32) q = fma(x[i], x[i], q);
      q = hq_warp_sum(q);
      if (lane == 0) {
        sd[k] = sqrt(q);
        se[k] = sd[k];
        sperm[k] = k;
      }
    }
    __syncthreads();
    const int mn = min(m, n);
    for (int s = 0; s < mn; ++s) {
      // Pivot: first maximum of the partial norms (idamax).
      {
        double bd = -1.0;
        int bk = 0x7fffffff;
        for (int k = s + tid; k < n; k += NT) {
          const double d = sd[k];
          if (d > bd || (d == bd && k < bk)) { bd = d; bk = k; }
        }
        for (int o = 16; o > 0; o >>= 1) {
          const double od = __shfl_xor_sync(0xffffffffu, bd, o);
          const int ok = __shfl_xor_sync(0xffffffffu, bk, o);
          if (od > bd || (od == bd && ok < bk)) { bd = od; bk = ok; }
        }
        if (lane == 0) { s_red[warp] = bd; s_bk[warp] = bk; }
        __syncthreads();
        if (tid == 0) {
          for (int w = 1; w < NW; ++w)
            if (s_red[w] > bd || (s_red[w] == bd && s_bk[w] < bk)) { bd = s_red[w]; bk = s_bk[w]; }
          s_kp = bk == 0x7fffffff ? s : bk;
        }
        __syncthreads();
      }
      const int kp = s_kp;
      if (kp != s) {
        double* c1 = X + (long long)s * ldx;
        double* c2 = X + (long long)kp * ldx;
        for (int i = tid; i < m; i += NT) {
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
      // Reflector for column s (rows s..m-1).
      double* xs = X + (long long)s * ldx;
      {
        double q = 0.0;
        for (int i = s + 1 + tid; i < m; i += NT) q = fma(xs[i], xs[i], q);
        q = hq_warp_sum(q);
        if (lane == 0) s_red[warp] = q;
        __syncthreads();
        if (tid == 0) {
          double t = 0.0;
          for (int w = 0; w < NW; ++w) t += s_red[w];
          const HqReflector h = hq_make_reflector_sq(xs[s], m - s > 1 ? t : 0.0);
          s_tau = h.tau;
          s_scale = h.scale;
          s_beta = h.beta;
          a.tau[item][s] = h.tau;
        }
        __syncthreads();
        const double scale = s_scale;
        for (int i = s + 1 + tid; i < m; i += NT) xs[i] *= scale;
        __syncthreads();
        if (tid == 0) xs[s] = 1.0;  // v_s, restored to beta after the update
        __syncthreads();
      }
      // w_k = tau * v^T X[s:, k]; X[s:, k] -= v w_k, a warp per column.
      const double tau = s_tau;
      for (int k = s + 1 + warp; k < n; k += NW) {
        double* xk = X + (long long)k * ldx;
        double w = 0.0;
        for (int i = s + lane; i < m; i += 32) w = fma(xs[i], xk[i], w);
        w = hq_warp_sum(w) * tau;
        for (int i = s + lane; i < m; i += 32) xk[i] = fma(-xs[i], w, xk[i]);
      }
      __syncthreads();
      // LAWN 176 downdate of the partial norms, one thread per column, from
      // the new entries of row s (a warp per column would repeat its
      // divisions and square root on 32 lanes of the scarce FP64 pipe);
      // columns that need their norm recomputed are flagged and recomputed
      // below, a warp per column (rare).
      int* sflag = reinterpret_cast<int*>(sw);
      int any = 0;
      for (int k = s + 1 + tid; k < n; k += NT) {
        double dk = sd[k];
        int flag = 0;
        if (dk != 0.0) {
          double t1 = fabs(X[s + (long long)k * ldx]) / dk;
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
      if (__syncthreads_or(any)) {
        for (int k = s + 1 + warp; k < n; k += NW) {
          if (!sflag[k]) continue;  // uniform across the warp
          const double* xk = X + (long long)k * ldx;
          double q = 0.0;
          for (int i = s + 1 + lane; i < m; i += 32) q = fma(xk[i], xk[i], q);
          q = hq_warp_sum(q);
          if (lane == 0) {
            const double nv = m - s - 1 > 0 ? sqrt(q) : 0.0;
            sd[k] = nv;
            se[k] = nv;
          }
        }
        __syncthreads();
      }
      if (tid == 0) xs[s] = s_beta;
      __syncthreads();
    }
    if (staged)
      for (long long e = tid; e < (long long)m * n; e += NT) {
        const int i = (int)(e % m), k = (int)(e / m);
        Ag[i + (long long)k * lda] = sX[i + (long long)k * lds];
      }
    for (int k = tid; k < n; k += NT) a.jpvt[item][k] = sperm[k] + 1;
    if (tid == 0 && a.info) a.info[item] = 0;
    __syncthreads();
  }
}

template <int NT>
int launch_t(cudaStream_t st, const hq_device_info* dev, const BatchArgs& a, int ctas_per_sm) {
  const size_t fixed = sizeof(double) * 3 * (size_t)a.max_n + sizeof(int) * (size_t)((a.max_n + 1) & ~1);
  const size_t smem = fixed + (size_t)a.stage_bytes;
  if (smem > dev->smem_optin) return (int)cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(qrp_batched_kernel<NT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, qrp_batched_kernel<NT>, NT, smem);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  if (ctas_per_sm < per_sm) per_sm = ctas_per_sm;
  int grid = dev->num_sms * per_sm;
  if (grid > a.batch) grid = a.batch;
  qrp_batched_kernel<NT><<<grid, NT, smem, st>>>(a);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

}  // namespace

// Workspace: queue head + schedule.
extern "C" size_t hq_qrp_batched_workspace(int batch) {
  return sizeof(int) * (size_t)(batch + 64);
}

extern "C" int hq_qrp_batched(cudaStream_t stream, const hq_device_info* dev, int batch,
                              const int* d_m, const int* d_n, double* const* d_A,
                              const int* d_lda, int* const* d_jpvt, double* const* d_tau,
                              int* d_info, void* d_work, int max_n, int threads, int stage_kb,
                              int ctas_per_sm) {
  if (batch <= 0) return 0;
  if (max_n <= 0 || max_n > 4096) return (int)cudaErrorInvalidValue;
  BatchArgs a;
  a.batch = batch;
  a.m = d_m;
  a.n = d_n;
  a.A = d_A;
  a.lda = d_lda;
  a.jpvt = d_jpvt;
  a.tau = d_tau;
  a.info = d_info;
  a.next = static_cast<int*>(d_work);
  a.order = static_cast<const int*>(d_work) + 32;
  a.stage_bytes = stage_kb * 1024;
  a.max_n = max_n;
  cudaError_t e = cudaMemsetAsync(a.next, 0, sizeof(int), stream);
  if (e != cudaSuccess) return (int)e;
  switch (threads) {
    case 128: return launch_t<128>(stream, dev, a, ctas_per_sm);
    case 256: return launch_t<256>(stream, dev, a, ctas_per_sm);
    case 512: return launch_t<512>(stream, dev, a, ctas_per_sm);
    default: return (int)cudaErrorInvalidValue;
  }
}
