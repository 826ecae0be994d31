// hq_common.cuh -- device helpers shared by the HQRRP kernels (sm_103a).
//
// Grid-wide barriers here are bounded: every spin has an iteration cap, after
// which the waiting CTA records an error code in the call's error word and
// returns, so a barrier that can never complete ends the kernel instead of
// hanging the GPU.  The host reads the error word after the call.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hq_internal.h"

#define HQ_WARP 32

// Launch with programmatic dependent launch.  The grid may then be scheduled
// while the previous kernel on the stream is still finishing; every kernel
// launched this way begins with HQ_PDL_WAIT(), which holds each thread until
// that kernel has completed and its writes are visible.  Nothing is read or
// written before the wait, so the stream order is kept exactly; what is saved
// is the latency between the end of one kernel and the start of the next
// (about 4.1 against 1.4 microseconds per launch for a chain of small
// dependent kernels on GB300).  The wait returns at once in a grid launched
// without the attribute (HQRRP_GB300_PDL=0).  Launch errors are left to the
// caller's cudaGetLastError(), as with <<<>>>.
#define HQ_PDL_WAIT() asm volatile("griddepcontrol.wait;" ::: "memory")

template <typename... KArgs, typename... Args>
static inline void hq_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                             cudaStream_t stream, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = hq_pdl() ? 1 : 0;
  (void)cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// Cooperative launch (every CTA co-resident, as the grid barriers need), with
// programmatic dependent launch as above; the kernel begins with
// HQ_PDL_WAIT().  Should the runtime refuse the two attributes together, the
// launch is repeated as a plain cooperative launch.
static inline cudaError_t hq_launch_coop(const void* kernel, dim3 grid, dim3 block, void** args,
                                         size_t smem, cudaStream_t stream) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = hq_pdl() ? 2 : 1;
  cudaError_t e = cudaLaunchKernelExC(&cfg, kernel, args);
  if (e != cudaSuccess && cfg.numAttrs == 2) {
    (void)cudaGetLastError();
    cfg.numAttrs = 1;
    e = cudaLaunchKernelExC(&cfg, kernel, args);
  }
  return e;
}

__device__ __forceinline__ unsigned hq_ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void hq_red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int hq_ld_volatile(const int* p) {
  return *(const volatile int*)p;
}

// Loads that bypass L1: data written by other CTAs during this kernel.
__device__ __forceinline__ double hq_ldcg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ int hq_ldcg(const int* p) { return __ldcg(p); }
__device__ __forceinline__ long long hq_ldcg(const long long* p) { return __ldcg(p); }

// Order key of a column norm for pivot comparisons on the integer pipe: for
// d >= 0 the IEEE bit pattern orders like the value; NaN maps below every
// number (it never wins a comparison).
__device__ __forceinline__ long long hq_norm_key(double d) {
  const long long b = __double_as_longlong(d);
  const long long mag = b & 0x7fffffffffffffffLL;
  if (mag > 0x7ff0000000000000LL) return -1LL;  // NaN
  return b < 0 ? (mag == 0 ? 0LL : -1LL) : b;  // -0 is 0; a norm is never negative
}

// Bounded grid barrier.  `counter` is zeroed before the launch; barrier number
// `epoch` (1-based) completes when the counter reaches epoch * nctas.  Returns
// false (in every thread of the CTA) if the wait gave up or another CTA
// reported an error; the caller must then leave the kernel.  Ordering: the
// CTA's writes before the barrier reach thread 0 through __syncthreads, and
// its release add at GPU scope carries them (release is cumulative) to every
// CTA whose acquire load reads the completed count; __syncthreads passes them
// on to that CTA's threads.  No sequentially consistent fence is needed.
__device__ __forceinline__ bool hq_grid_barrier(unsigned* counter, int* err, unsigned epoch,
                                                unsigned spin_limit, int* s_flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    hq_red_release_add(counter, 1u);
    const unsigned target = epoch * gridDim.x;
    unsigned spins = 0;
    int ok = 1;
    while (hq_ld_acquire(counter) < target) {
      if (hq_ld_volatile(err) != 0) {
        ok = 0;
        break;
      }
      if (++spins > spin_limit) {
        atomicCAS(err, 0, HQ_ERR_BARRIER_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    *s_flag = ok;
  }
  __syncthreads();
  return *s_flag != 0;
}

template <typename T>
__device__ __forceinline__ T hq_warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sqrt(a^2 + b^2) without destructive overflow (LAPACK DLAPY2's formula).
__device__ __forceinline__ double hq_lapy2(double a, double b) {
  double x = fabs(a), y = fabs(b);
  double w = fmax(x, y), z = fmin(x, y);
  if (z == 0.0 || isnan(a) || isnan(b)) return (isnan(a) || isnan(b)) ? a + b : w;
  double q = z / w;
  return w * sqrt(1.0 + q * q);
}

// Householder generation in the convention of LAPACK DLARFG: given alpha and
// the norm of the tail x, returns tau, beta (the new alpha) and the factor
// the tail is scaled by so that v = [1; scale * x].  tau == 0 means H = I.
// The safe-minimum rescaling loop of DLARFG only changes results for columns
// whose norm is below ~1e-292; it is reproduced by scaling beta and alpha.
struct HqReflector {
  double tau, beta, scale;
};

__device__ __forceinline__ HqReflector hq_make_reflector(double alpha, double xnorm) {
  HqReflector r;
  if (xnorm == 0.0) {
    r.tau = 0.0;
    r.beta = alpha;
    r.scale = 1.0;
    return r;
  }
  const double safmin = 2.2250738585072014e-308 / 1.1102230246251565e-16;  // dlamch S / E
  const double rsafmn = 1.0 / safmin;
  double beta = -copysign(hq_lapy2(alpha, xnorm), alpha);
  int knt = 0;
  double a = alpha, xn = xnorm, mul = 1.0;
  while (fabs(beta) < safmin && knt < 20) {
    ++knt;
    mul *= rsafmn;
    a *= rsafmn;
    xn *= rsafmn;
    beta = -copysign(hq_lapy2(a, xn), a);
  }
  r.tau = (beta - a) / beta;
  r.scale = mul / (a - beta);
  for (int k = 0; k < knt; ++k) beta *= safmin;
  r.beta = beta;
  return r;
}

// The same reflector from alpha and q = ||x||^2 (the tail's sum of squares).
// Away from under/overflow, beta = -sign(alpha) sqrt(alpha^2 + q) takes one
// square root and tau and the scale are two independent divisions -- a short
// dependency chain, which matters where FP64 latency sits on a critical path;
// beta agrees with DLAPY2's value to an ulp.  Near the range limits it falls
// back to the careful form above.
__device__ __forceinline__ HqReflector hq_make_reflector_sq(double alpha, double q) {
  if (q == 0.0) return hq_make_reflector(alpha, 0.0);
  const double t = fma(alpha, alpha, q);
  if (t >= 1e-280 && t <= 1e280) {
    HqReflector r;
    const double beta = -copysign(sqrt(t), alpha);
    r.tau = (beta - alpha) / beta;
    r.scale = 1.0 / (alpha - beta);
    r.beta = beta;
    return r;
  }
  return hq_make_reflector(alpha, sqrt(q));
}

// LAPACK's tol3z = sqrt(dlamch('Epsilon')) with eps = 2^-53.
#define HQ_TOL3Z 1.0536712127723509e-08
