// permute.cu -- column permutations and small utilities.
//
// The reference swaps whole columns one pivot at a time with dswap
// (lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:990-1036, called from
// :831-837 for A's m rows, Y and the labels).  Here the b swaps of a block are
// composed first (by the pivot-selection kernel, as (dst, src) pairs, or by the
// panel kernel, as perm[k] = src) and applied once: a gather of the moved
// columns into a scratch buffer, then a scatter to their destinations.  The
// copies are bit-exact; each moved column is read and written twice, at most
// 2b columns per block.
#include "hq_common.cuh"

namespace {

// Pair lists and permutations come from the pivoting kernels; an index
// outside [0, ncols) can only follow an aborted run (whose error word the host
// reports) and is skipped rather than followed.
__global__ void gather_pairs(int rows, const double* __restrict__ X, int ldx,
                             const int* __restrict__ pairs, const int* __restrict__ npairs,
                             int ncols, double* __restrict__ tmp,
                             const int* __restrict__ labels, int* __restrict__ label_tmp) {
  HQ_PDL_WAIT();
  const int p = blockIdx.y;
  if (p >= *npairs) return;
  const int src = pairs[2 * p + 1];
  if (src < 0 || src >= ncols || pairs[2 * p] < 0 || pairs[2 * p] >= ncols) return;
  const double* s = X + (size_t)src * ldx;
  double* t = tmp + (size_t)p * rows;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
    t[r] = s[r];
  if (labels && blockIdx.x == 0 && threadIdx.x == 0) label_tmp[p] = labels[src];
}

__global__ void scatter_pairs(int rows, double* __restrict__ X, int ldx,
                              const int* __restrict__ pairs, const int* __restrict__ npairs,
                              int ncols, const double* __restrict__ tmp,
                              int* __restrict__ labels, const int* __restrict__ label_tmp) {
  HQ_PDL_WAIT();
  const int p = blockIdx.y;
  if (p >= *npairs) return;
  const int dst = pairs[2 * p];
  if (dst < 0 || dst >= ncols || pairs[2 * p + 1] < 0 || pairs[2 * p + 1] >= ncols) return;
  double* d = X + (size_t)dst * ldx;
  const double* t = tmp + (size_t)p * rows;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
    d[r] = t[r];
  if (labels && blockIdx.x == 0 && threadIdx.x == 0) labels[dst] = label_tmp[p];
}

__global__ void gather_perm(int rows, const double* __restrict__ X, int ldx,
                            const int* __restrict__ perm, double* __restrict__ tmp,
                            const int* __restrict__ labels, int* __restrict__ label_tmp) {
  HQ_PDL_WAIT();
  const int k = blockIdx.y;
  const int src = perm[k];
  // A column that stays in place is neither gathered nor scattered.
  if (src < 0 || src >= (int)gridDim.y || src == k) return;
  const double* s = X + (size_t)src * ldx;
  double* t = tmp + (size_t)k * rows;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
    t[r] = s[r];
  if (labels && blockIdx.x == 0 && threadIdx.x == 0) label_tmp[k] = labels[src];
}

__global__ void scatter_perm(int rows, double* __restrict__ X, int ldx,
                             const int* __restrict__ perm, const double* __restrict__ tmp,
                             int* __restrict__ labels, const int* __restrict__ label_tmp) {
  HQ_PDL_WAIT();
  const int k = blockIdx.y;
  if (perm[k] < 0 || perm[k] >= (int)gridDim.y || perm[k] == k) return;
  double* d = X + (size_t)k * ldx;
  const double* t = tmp + (size_t)k * rows;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
    d[r] = t[r];
  if (labels && blockIdx.x == 0 && threadIdx.x == 0) labels[k] = label_tmp[k];
}

__global__ void zero_words_kernel(unsigned* __restrict__ p1, long long n1, unsigned* __restrict__ p2,
                                  long long n2) {
  HQ_PDL_WAIT();
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n1 + n2; i += stride) {
    if (i < n1) p1[i] = 0u;
    else p2[i - n1] = 0u;
  }
}

__global__ void iota_kernel(int* x, int n, int base) {
  HQ_PDL_WAIT();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] = base + i;
}

__global__ void copy_kernel(int rows, int cols, const double* __restrict__ src, int lds,
                            double* __restrict__ dst, int ldd) {
  HQ_PDL_WAIT();
  const size_t total = (size_t)rows * cols;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(e % rows), c = (int)(e / rows);
    dst[r + (size_t)c * ldd] = src[r + (size_t)c * lds];
  }
}

inline unsigned row_blocks(int rows) {
  int b = (rows + 255) / 256;
  if (b > 32) b = 32;
  return b < 1 ? 1u : (unsigned)b;
}

}  // namespace

extern "C" int hq_permute_pairs(cudaStream_t stream, int rows, double* X, int ldx, int ncols,
                                const int* pairs, const int* npairs, int max_pairs, double* tmp,
                                int* labels, int* label_tmp) {
  if (max_pairs <= 0 || (rows <= 0 && labels == nullptr)) return 0;
  const int r = rows > 0 ? rows : 0;
  dim3 grid(row_blocks(r), max_pairs);
  hq_launch(gather_pairs, grid, 256, 0, stream, r, X, ldx, pairs, npairs, ncols, tmp, labels, label_tmp);
  hq_launch(scatter_pairs, grid, 256, 0, stream, r, X, ldx, pairs, npairs, ncols, tmp, labels,
                                           label_tmp);
  hq_count_launches(2);
  return (int)cudaGetLastError();
}

extern "C" int hq_permute_cols(cudaStream_t stream, int rows, double* X, int ldx, int nc,
                               const int* perm, double* tmp, int* labels, int* label_tmp) {
  if (nc <= 0 || (rows <= 0 && labels == nullptr)) return 0;
  const int r = rows > 0 ? rows : 0;
  dim3 grid(row_blocks(r), nc);
  hq_launch(gather_perm, grid, 256, 0, stream, r, X, ldx, perm, tmp, labels, label_tmp);
  hq_launch(scatter_perm, grid, 256, 0, stream, r, X, ldx, perm, tmp, labels, label_tmp);
  hq_count_launches(2);
  return (int)cudaGetLastError();
}

extern "C" int hq_zero_words(cudaStream_t stream, void* p1, size_t n1, void* p2, size_t n2) {
  if (p2 == nullptr) n2 = 0;
  const size_t total = n1 + n2;
  if (total == 0) return 0;
  size_t blocks = (total + 255) / 256;
  if (blocks > 1024) blocks = 1024;
  hq_launch(zero_words_kernel, (unsigned)blocks, 256, 0, stream, static_cast<unsigned*>(p1),
            (long long)n1, static_cast<unsigned*>(p2), (long long)n2);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_fill_iota(cudaStream_t stream, int* x, int n, int base) {
  if (n <= 0) return 0;
  hq_launch(iota_kernel, (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, stream, x, n, base);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_copy_matrix(cudaStream_t stream, int rows, int cols, const double* src,
                              int lds, double* dst, int ldd) {
  if (rows <= 0 || cols <= 0) return 0;
  size_t total = (size_t)rows * cols;
  size_t blocks = (total + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  hq_launch(copy_kernel, (unsigned)blocks, 256, 0, stream, rows, cols, src, lds, dst, ldd);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

static unsigned long long g_launches = 0;

extern "C" void hq_count_launches(int k) { __atomic_add_fetch(&g_launches, (unsigned long long)k, __ATOMIC_RELAXED); }

extern "C" unsigned long long hq_launches(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

static int g_pdl = 1;

extern "C" void hq_set_pdl(int on) { __atomic_store_n(&g_pdl, on ? 1 : 0, __ATOMIC_RELAXED); }

extern "C" int hq_pdl(void) { return __atomic_load_n(&g_pdl, __ATOMIC_RELAXED); }

extern "C" int hq_query_device(hq_device_info* info) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  int sms = 0, smem = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return (int)e;
  if ((e = cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) !=
      cudaSuccess)
    return (int)e;
  info->device = dev;
  info->num_sms = sms;
  // Leave room for the static shared variables of the kernels.
  info->smem_optin = (size_t)smem - 2048;
  return 0;
}
