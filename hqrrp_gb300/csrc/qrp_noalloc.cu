// qrp_noalloc.cu -- pivoted QR of a device matrix of at most 256 columns that
// allocates no device memory.
//
// Who needs this: a caller that has already handed all of the GPU's memory to
// its own arena (a serving process that reserves HBM up front), or that runs
// where a device allocation is not allowed or not affordable -- cudaMalloc and
// cudaFree synchronise the device and can fail under memory pressure, and a
// latency-critical loop cannot take either.  Every other entry point of this
// library draws its workspace from a memory pool, which allocates on first
// use; this one does not.
//
// Its scratch (the cooperative kernel's exchange buffers, barrier counter,
// error word and the column permutation) is one file-scope __device__ array
// of fixed size, present on every GPU that loads the library until the
// process exits.  Limits: n <= 256 columns, at most 160 CTAs; any m.  All
// calls on a device share the array and it keeps the previous call's
// contents, so the call clears what must start at zero (error word, barrier
// counter); calls that overlap on the GPU (other streams, other threads)
// race on it and must be serialised by the caller.
#include <mutex>

#include "hq_common.cuh"

#define NOALLOC_MAX_N 256
#define NOALLOC_MAX_CTAS 160

namespace {

constexpr size_t kPartElems = HQ_PANEL_PART_ELEMS(NOALLOC_MAX_CTAS, NOALLOC_MAX_N);
constexpr size_t kRowbufElems = 2ull * NOALLOC_MAX_N;
constexpr size_t kPermElems = NOALLOC_MAX_N / 2;  // NOALLOC_MAX_N ints
constexpr size_t kFlagElems = 2;                  // barrier counter, error word
constexpr size_t kScratchElems = kPartElems + kRowbufElems + kPermElems + kFlagElems;

// Return codes, the same values as the rest of the library's entry points.
constexpr int kRcCuda = 1, kRcDevice = 2, kRcUnsupported = 3;

}  // namespace

// 2 x 160 x 258 + 48 x 258 + 512 + 128 + 2 doubles = 764,688 bytes (747 KiB)
// per GPU.
static __device__ __align__(256) double hq_noalloc_scratch[kScratchElems];

namespace {

std::mutex g_setup_mu;
double* g_scratch[64];

// Device address of the scratch array for `dev`.  The first call on a device
// looks the symbol up (which loads this module on that device if needed);
// later calls reuse the address.
int scratch_for(int dev, double** out) {
  if (dev < 0 || dev >= 64) return (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (g_scratch[dev] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, hq_noalloc_scratch);
    if (e != cudaSuccess) return (int)e;
    g_scratch[dev] = static_cast<double*>(p);
  }
  *out = g_scratch[dev];
  return 0;
}

__global__ void labels_from_perm(const int* __restrict__ perm, int n, int* __restrict__ jpvt) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    jpvt[k] = perm[k] + 1;
}

}  // namespace

// Pivoted Householder QR of the m x n device matrix dA (column-major, ldda),
// in place, with the result conventions of LAPACK dgeqp3 for free columns:
// R on and above the diagonal, reflectors below it, tau[0..min(m,n)), and
// d_jpvt[k] = 1-based original index of column k.  n <= 256.  Runs on
// `stream` (a cudaStream_t) and returns when the factorization is complete:
// 0 on success, 3 for shapes beyond the limits, 2 if the kernel reported an
// error, 1 for a CUDA error; the message is in hqrrp_gb300_last_error().
// The first call on a device performs its one-time set-up (the scratch
// address lookup) and should come before any stream capture.
extern "C" __attribute__((visibility("default"))) int hqrrp_gb300_qrp_noalloc(
    int m, int n, double* dA, int ldda, int* d_jpvt, double* d_tau, void* stream) {
  hq_clear_error();
  if (m < 0 || n < 0 || ldda < (m > 1 ? m : 1)) {
    hq_set_error("hqrrp_gb300_qrp_noalloc: invalid m, n or ldda");
    return kRcUnsupported;
  }
  if (n > NOALLOC_MAX_N) {
    hq_set_error("hqrrp_gb300_qrp_noalloc: n = %d exceeds its limit of %d columns", n,
                 NOALLOC_MAX_N);
    return kRcUnsupported;
  }
  if (m == 0 || n == 0) return 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  hq_device_info dev;
  int rc = hq_query_device(&dev);
  if (rc == 0 && dev.num_sms > NOALLOC_MAX_CTAS) dev.num_sms = NOALLOC_MAX_CTAS;
  double* base = nullptr;
  if (rc == 0) rc = scratch_for(dev.device, &base);
  if (rc != 0) {
    hq_set_error("hqrrp_gb300_qrp_noalloc: set-up failed: %s",
                 cudaGetErrorString((cudaError_t)rc));
    return kRcCuda;
  }
  double* part = base;
  double* rowbuf = part + kPartElems;
  int* perm = reinterpret_cast<int*>(rowbuf + kRowbufElems);
  unsigned* bar = reinterpret_cast<unsigned*>(rowbuf + kRowbufElems + kPermElems);
  int* err = reinterpret_cast<int*>(bar + 1);

  rc = (int)cudaMemsetAsync(err, 0, sizeof(int), st);
  if (rc == 0)
    rc = hq_panel_qrp(st, &dev, m, n, 1, dA, ldda, d_tau, nullptr, 1, perm, part, kPartElems,
                      rowbuf, bar, err, hq_spin_limit(), 0, 0);
  if (rc == 0) {
    labels_from_perm<<<(n + 255) / 256, 256, 0, st>>>(perm, n, d_jpvt);
    hq_count_launches(1);
    rc = (int)cudaGetLastError();
  }
  int herr = 0;
  if (rc == 0) rc = (int)cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (rc == 0) rc = (int)cudaStreamSynchronize(st);
  if (rc != 0) {
    hq_set_error("hqrrp_gb300_qrp_noalloc: %s", cudaGetErrorString((cudaError_t)rc));
    return kRcCuda;
  }
  if (herr != 0) {
    hq_set_error("hqrrp_gb300_qrp_noalloc: kernel reported error 0x%x", herr);
    return kRcDevice;
  }
  return 0;
}
