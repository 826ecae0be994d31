// gemm_f64.cu -- FP64 GEMM for the plain-precision path.
//
// C = alpha * op(A) * op(B) + beta * C, column-major, op in {N, T}.  GB300's
// FP64 rate (about 2 DFMA per clock per SM, the same for DMMA and the FP64
// pipe) bounds every FP64 product in HQRRP, so this kernel is written for the
// DFMA pipe: 64x64 tiles, 16-deep k slices staged in shared memory with a
// register prefetch of the next slice, 4x4 outputs per thread.  Products whose
// output is small next to their inner dimension (U^T C late in the
// factorization, G_R U, the Gram matrix of a panel) are split along K into
// slices summed in a fixed order by a second kernel, so results do not depend
// on scheduling.
#include "hq_common.cuh"

namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

template <bool TA, bool TB>
__global__ void __launch_bounds__(NT, 2)
    dgemm_tile(int M, int N, int K, int kchunk, double alpha, const double* __restrict__ A,
               int lda, const double* __restrict__ B, int ldb, double beta,
               double* __restrict__ Cm, int ldc, double* __restrict__ ws) {
  HQ_PDL_WAIT();
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int kbeg = blockIdx.z * kchunk;
  const int kend = min(K, kbeg + kchunk);

  double ra[4], rb[4];
  auto load_a = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + NT * q;
      int i, k;
      if (!TA) { i = idx & (BM - 1); k = idx >> 6; }
      else     { k = idx & (BK - 1); i = idx >> 4; }
      const int gi = m0 + i, gk = k0 + k;
      double v = 0.0;
      if (gi < M && gk < kend)
        v = TA ? A[gk + (size_t)gi * lda] : A[gi + (size_t)gk * lda];
      ra[q] = v;
    }
  };
  auto load_b = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + NT * q;
      int j, k;
      if (!TB) { k = idx & (BK - 1); j = idx >> 4; }
      else     { j = idx & (BN - 1); k = idx >> 6; }
      const int gj = n0 + j, gk = k0 + k;
      double v = 0.0;
      if (gj < N && gk < kend)
        v = TB ? B[gj + (size_t)gk * ldb] : B[gk + (size_t)gj * ldb];
      rb[q] = v;
    }
  };
  auto store_tiles = [&]() {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = tid + NT * q;
      if (!TA) As[idx >> 6][idx & (BM - 1)] = ra[q];
      else     As[idx & (BK - 1)][idx >> 4] = ra[q];
      if (!TB) Bs[idx & (BK - 1)][idx >> 4] = rb[q];
      else     Bs[idx >> 6][idx & (BN - 1)] = rb[q];
    }
  };

  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  if (kbeg < kend) {
    load_a(kbeg);
    load_b(kbeg);
    for (int k0 = kbeg; k0 < kend; k0 += BK) {
      __syncthreads();
      store_tiles();
      __syncthreads();
      if (k0 + BK < kend) {
        load_a(k0 + BK);
        load_b(k0 + BK);
      }
#pragma unroll
      for (int k = 0; k < BK; ++k) {
        double a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[k][tx + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[k][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
    }
  }

  if (ws != nullptr) {
    double* out = ws + (size_t)blockIdx.z * M * N;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gj = n0 + ty + 16 * j;
      if (gj >= N) continue;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int gi = m0 + tx + 16 * i;
        if (gi < M) out[gi + (size_t)gj * M] = acc[i][j];
      }
    }
    return;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gj = n0 + ty + 16 * j;
    if (gj >= N) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int gi = m0 + tx + 16 * i;
      if (gi >= M) continue;
      double* c = Cm + gi + (size_t)gj * ldc;
      *c = (beta == 0.0) ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *c);
    }
  }
}

__global__ void dgemm_splitk_sum(int M, int N, int splits, double alpha,
                                 const double* __restrict__ ws, double beta,
                                 double* __restrict__ Cm, int ldc) {
  HQ_PDL_WAIT();
  const size_t total = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < splits; ++z) s += ws[e + (size_t)z * total];
    const int i = (int)(e % M), j = (int)(e / M);
    double* c = Cm + i + (size_t)j * ldc;
    *c = (beta == 0.0) ? alpha * s : fma(alpha, s, beta * *c);
  }
}

__global__ void dgemm_scale(int M, int N, double beta, double* __restrict__ Cm, int ldc) {
  HQ_PDL_WAIT();
  const size_t total = (size_t)M * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % M), j = (int)(e / M);
    double* c = Cm + i + (size_t)j * ldc;
    *c = (beta == 0.0) ? 0.0 : beta * *c;
  }
}

}  // namespace

extern "C" int hq_dgemm(cudaStream_t stream, const hq_device_info* dev, char transa,
                        char transb, int M, int N, int K, double alpha, const double* A, int lda,
                        const double* B, int ldb, double beta, double* Cm, int ldc, double* ws,
                        size_t ws_elems) {
  if (M <= 0 || N <= 0) return 0;
  if (K <= 0 || alpha == 0.0) {
    if (beta == 1.0) return 0;
    hq_launch(dgemm_scale, dev->num_sms * 4, 256, 0, stream, M, N, beta, Cm, ldc);
    hq_count_launches(1);
    return (int)cudaGetLastError();
  }
  const bool ta = (transa == 'T' || transa == 't'), tb = (transb == 'T' || transb == 't');
  const int gm = (M + BM - 1) / BM, gn = (N + BN - 1) / BN;
  const long tiles = (long)gm * gn;
  // Split K when the tile grid cannot fill two waves of the SMs.
  int splits = 1;
  const long want = 2L * dev->num_sms;
  if (tiles < want && K >= 4 * BK * 8 && ws != nullptr) {
    long s = (want + tiles - 1) / tiles;
    long smax = K / (BK * 8);
    if (s > smax) s = smax;
    if (s > 64) s = 64;
    while (s > 1 && (size_t)s * M * N > ws_elems) --s;
    if (s > 1) splits = (int)s;
  }
  int kchunk = K;
  if (splits > 1) {
    kchunk = (K + splits - 1) / splits;
    kchunk = (kchunk + BK - 1) / BK * BK;
    splits = (K + kchunk - 1) / kchunk;
  }
  dim3 grid(gm, gn, splits);
  double* out_ws = splits > 1 ? ws : nullptr;
  if (!ta && !tb)
    hq_launch(dgemm_tile<false, false>, grid, NT, 0, stream, M, N, K, kchunk, alpha, A, lda, B, ldb,
                                                       beta, Cm, ldc, out_ws);
  else if (ta && !tb)
    hq_launch(dgemm_tile<true, false>, grid, NT, 0, stream, M, N, K, kchunk, alpha, A, lda, B, ldb,
                                                      beta, Cm, ldc, out_ws);
  else if (!ta && tb)
    hq_launch(dgemm_tile<false, true>, grid, NT, 0, stream, M, N, K, kchunk, alpha, A, lda, B, ldb,
                                                      beta, Cm, ldc, out_ws);
  else
    hq_launch(dgemm_tile<true, true>, grid, NT, 0, stream, M, N, K, kchunk, alpha, A, lda, B, ldb,
                                                     beta, Cm, ldc, out_ws);
  if (splits > 1) {
    long total = (long)M * N;
    int blocks = (int)((total + 255) / 256);
    if (blocks > dev->num_sms * 8) blocks = dev->num_sms * 8;
    hq_launch(dgemm_splitk_sum, blocks, 256, 0, stream, M, N, splits, alpha, ws, beta, Cm, ldc);
  }
  hq_count_launches(splits > 1 ? 2 : 1);
  return (int)cudaGetLastError();
}
