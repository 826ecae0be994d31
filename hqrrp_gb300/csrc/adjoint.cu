// adjoint.cu -- small kernels of the hand-written adjoint of the truncated
// factorization A P ~= Q_k R_k (no counterpart in the reference), and the
// element-wise pieces of the mixed path's unit-diagonal handling.
//
// For L = <W, Q_k R_k P^T> = <W, Q Q^T A> with the pivots P held fixed, Q
// depends only on A1 = A P[:, :k] = Q R11 (a thin Householder QR), and
//     dL/dA = Q (Q^T W) + scatter_P( (G + Q copyltu(-G^T Q)) R11^-T ),
//     G = W M^T + A N^T,  M = Q^T A = R_k P^T,  N = Q^T W,
// the standard reverse-mode rule of the thin QR (copyltu(X) = tril(X) +
// tril(X, -1)^T).  The GEMMs run on the library's product kernels; these are
// the element-wise and triangular pieces around them.
#include "hq_common.cuh"

namespace {

// U (rows x b, ldu) = unit-lower part of the reflector block stored in F.
__global__ void unit_lower_kernel(int rows, int b, const double* __restrict__ F, int ldf,
                                  double* __restrict__ U, int ldu) {
  HQ_PDL_WAIT();
  const long long total = (long long)rows * b;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % rows), k = (int)(e / rows);
    U[i + (long long)k * ldu] = i > k ? F[i + (long long)k * ldf] : (i == k ? 1.0 : 0.0);
  }
}

// E (rows x k) = [I_k; 0].
__global__ void eye_kernel(int rows, int k, double* __restrict__ E, int lde) {
  HQ_PDL_WAIT();
  const long long total = (long long)rows * k;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % rows), c = (int)(e / rows);
    E[i + (long long)c * lde] = i == c ? 1.0 : 0.0;
  }
}

// X (k x k) <- copyltu(X) * sign: lower triangle kept, mirrored to the upper.
__global__ void copyltu_kernel(int k, double* __restrict__ X, int ldx, double sign) {
  HQ_PDL_WAIT();
  const int total = k * k;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int i = e % k, j = e / k;
    if (i < j) continue;  // each thread owns a lower entry and its mirror
    const double v = sign * X[i + (long long)j * ldx];
    X[i + (long long)j * ldx] = v;
    if (i != j) X[j + (long long)i * ldx] = v;
  }
}

// Y (rows x k) <- Y R^-T for R upper triangular k x k (ldr): row-wise back
// substitution, Y[:, j] = (Y[:, j] - sum_{i>j} Y[:, i] R[j, i]) / R[j, j].
// One thread per row of Y; all threads of a warp read the same entry of R
// at the same time, so R is served from L1 as a broadcast.
__global__ void trsm_rt_kernel(int rows, int k, const double* __restrict__ R, int ldr,
                               double* __restrict__ Y, int ldy) {
  HQ_PDL_WAIT();
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
    double* y = Y + r;
    for (int j = k - 1; j >= 0; --j) {
      double v = y[(long long)j * ldy];
      for (int i = j + 1; i < k; ++i) v = fma(-y[(long long)i * ldy], __ldg(R + j + (long long)i * ldr), v);
      y[(long long)j * ldy] = v / __ldg(R + j + (long long)j * ldr);
    }
  }
}

// Columns: dst[:, labels[c] - 1] (+)= src[:, c] for c < ncols (1-based labels).
__global__ void scatter_cols_kernel(int rows, int ncols, const double* __restrict__ src, int lds,
                                    const int* __restrict__ labels, double* __restrict__ dst,
                                    int ldd, int accumulate) {
  HQ_PDL_WAIT();
  const long long total = (long long)rows * ncols;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % rows), c = (int)(e / rows);
    const int t = labels[c] - 1;
    double* p = dst + i + (long long)t * ldd;
    *p = accumulate ? *p + src[i + (long long)c * lds] : src[i + (long long)c * lds];
  }
}

// M (k x n) = triu(F[0:k, :]) with its columns moved to their original
// positions: M[:, labels[c] - 1] = triu part of column c.
__global__ void rk_unpermute_kernel(int k, int n, const double* __restrict__ F, int ldf,
                                    const int* __restrict__ labels, double* __restrict__ M,
                                    int ldm) {
  HQ_PDL_WAIT();
  const long long total = (long long)k * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % k), c = (int)(e / k);
    M[i + (long long)(labels[c] - 1) * ldm] = i <= c ? F[i + (long long)c * ldf] : 0.0;
  }
}

// dst (rows x cols) += alpha * src.
__global__ void add_matrix_kernel(int rows, int cols, double alpha, const double* __restrict__ src,
                                  int lds, double* __restrict__ dst, int ldd) {
  HQ_PDL_WAIT();
  const long long total = (long long)rows * cols;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % rows), j = (int)(e / rows);
    dst[i + (long long)j * ldd] = fma(alpha, src[i + (long long)j * lds], dst[i + (long long)j * ldd]);
  }
}

// A[i, i] = v for i < n.
__global__ void set_diag_kernel(int n, double* __restrict__ A, int lda, double v) {
  HQ_PDL_WAIT();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    A[i + (long long)i * lda] = v;
}

// Z (b x b) += L + L^T + I where L is the strictly lower b x b top block of
// U' (U with its unit diagonal removed): the terms of U^T U that involve the
// unit diagonal, U^T U = U'^T U' + L + L^T + I.
__global__ void gram_unit_fix_kernel(int b, const double* __restrict__ Up, int ldu,
                                     double* __restrict__ Z, int ldz) {
  HQ_PDL_WAIT();
  const int total = b * b;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int r = e % b, c = e / b;
    const double add = r == c ? 1.0 : (r > c ? Up[r + (long long)c * ldu] : Up[c + (long long)r * ldu]);
    Z[r + (long long)c * ldz] += add;
  }
}

inline unsigned grid_for(long long total) {
  long long b = (total + 255) / 256;
  if (b > 8192) b = 8192;
  return b < 1 ? 1u : (unsigned)b;
}

}  // namespace

extern "C" int hq_unit_lower(cudaStream_t st, int rows, int b, const double* F, int ldf, double* U,
                             int ldu) {
  if (rows <= 0 || b <= 0) return 0;
  hq_launch(unit_lower_kernel, grid_for((long long)rows * b), 256, 0, st, rows, b, F, ldf, U, ldu);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_eye(cudaStream_t st, int rows, int k, double* E, int lde) {
  if (rows <= 0 || k <= 0) return 0;
  hq_launch(eye_kernel, grid_for((long long)rows * k), 256, 0, st, rows, k, E, lde);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_copyltu(cudaStream_t st, int k, double* X, int ldx, double sign) {
  if (k <= 0) return 0;
  hq_launch(copyltu_kernel, grid_for((long long)k * k), 256, 0, st, k, X, ldx, sign);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_trsm_rt(cudaStream_t st, int rows, int k, const double* R, int ldr, double* Y,
                          int ldy) {
  if (rows <= 0 || k <= 0) return 0;
  const unsigned blocks = (unsigned)((rows + 63) / 64);
  hq_launch(trsm_rt_kernel, blocks, 64, 0, st, rows, k, R, ldr, Y, ldy);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_scatter_cols(cudaStream_t st, int rows, int ncols, const double* src, int lds,
                               const int* labels, double* dst, int ldd, int accumulate) {
  if (rows <= 0 || ncols <= 0) return 0;
  hq_launch(scatter_cols_kernel, grid_for((long long)rows * ncols), 256, 0, st,
      rows, ncols, src, lds, labels, dst, ldd, accumulate);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_rk_unpermute(cudaStream_t st, int k, int n, const double* F, int ldf,
                               const int* labels, double* M, int ldm) {
  if (k <= 0 || n <= 0) return 0;
  hq_launch(rk_unpermute_kernel, grid_for((long long)k * n), 256, 0, st, k, n, F, ldf, labels, M, ldm);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_add_matrix(cudaStream_t st, int rows, int cols, double alpha, const double* src,
                             int lds, double* dst, int ldd) {
  if (rows <= 0 || cols <= 0) return 0;
  hq_launch(add_matrix_kernel, grid_for((long long)rows * cols), 256, 0, st, rows, cols, alpha, src, lds,
                                                                      dst, ldd);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_set_diag(cudaStream_t st, int n, double* A, int lda, double v) {
  if (n <= 0) return 0;
  hq_launch(set_diag_kernel, (n + 255) / 256, 256, 0, st, n, A, lda, v);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_gram_unit_fix(cudaStream_t st, int b, const double* Up, int ldu, double* Z,
                                int ldz) {
  if (b <= 0) return 0;
  hq_launch(gram_unit_fix_kernel, grid_for((long long)b * b), 256, 0, st, b, Up, ldu, Z, ldz);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}
