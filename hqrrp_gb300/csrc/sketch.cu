// sketch.cu -- the Gaussian sketch G on the device.
//
// Replaces the reference's Marsaglia polar method over libc rand()
// (lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:575-614, seeded by
// srand(12) at :380).  A counter-based generator needs no sequential state,
// so every element is produced independently: element e = c * rows + r of the
// column-major rows x cols sketch takes Philox4x32-10 of counter e / 2 under
// the 64-bit seed, and a Box-Muller pair turns its 128 random bits into two
// N(0,1) values (even e takes the cosine branch, odd e the sine branch).
//
// Philox4x32-10 is the published generator of Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3" (SC'11): ten rounds of two
// 32x32->64 multiplies with Weyl-sequence key bumps.
#include "hq_common.cuh"

namespace {

__device__ __forceinline__ void philox_round(uint32_t& c0, uint32_t& c1, uint32_t& c2,
                                             uint32_t& c3, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t lo0 = M0 * c0, hi0 = __umulhi(M0, c0);
  const uint32_t lo1 = M1 * c2, hi1 = __umulhi(M1, c2);
  const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
  c0 = n0;
  c1 = lo1;
  c2 = n2;
  c3 = lo0;
}

__device__ __forceinline__ void philox4x32_10(uint64_t counter, uint64_t seed, uint32_t out[4]) {
  uint32_t c0 = (uint32_t)counter, c1 = (uint32_t)(counter >> 32), c2 = 0u, c3 = 0u;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    philox_round(c0, c1, c2, c3, k0, k1);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

__global__ void sketch_philox_kernel(int rows, int cols, double* __restrict__ G, int ldg,
                                     uint64_t seed) {
  HQ_PDL_WAIT();
  const uint64_t total = (uint64_t)rows * cols;
  const uint64_t pairs = (total + 1) / 2;
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < pairs;
       p += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x[4];
    philox4x32_10(p, seed, x);
    const uint64_t a = ((uint64_t)x[1] << 32) | x[0];
    const uint64_t b = ((uint64_t)x[3] << 32) | x[2];
    // u1 in (0, 1], u2 in [0, 1): 53-bit uniforms.
    const double u1 = ((double)(a >> 11) + 1.0) * 0x1.0p-53;
    const double u2 = (double)(b >> 11) * 0x1.0p-53;
    const double rad = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    const uint64_t e0 = 2 * p;
    {
      const int r = (int)(e0 % rows), col = (int)(e0 / rows);
      G[r + (size_t)col * ldg] = rad * c;
    }
    if (e0 + 1 < total) {
      const uint64_t e1 = e0 + 1;
      const int r = (int)(e1 % rows), col = (int)(e1 / rows);
      G[r + (size_t)col * ldg] = rad * s;
    }
  }
}

}  // namespace

extern "C" int hq_sketch_philox(cudaStream_t stream, int rows, int cols, double* G, int ldg,
                                unsigned long long seed) {
  if (rows <= 0 || cols <= 0) return 0;
  const uint64_t pairs = ((uint64_t)rows * cols + 1) / 2;
  uint64_t blocks = (pairs + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  hq_launch(sketch_philox_kernel, (unsigned)blocks, 256, 0, stream, rows, cols, G, ldg, seed);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}
