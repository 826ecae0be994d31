// ozaki.cu -- FP64 products on the BF16 tensor cores (tcgen05), split-digit
// ("Ozaki scheme I") emulation, for the mixed-precision block updates.
//
// Each operand row r (a row of the M-side matrix, or a column of the output
// on the N side) gets a power-of-two scale 2^e_r >= max |x|, and every entry
// is written as S balanced base-256 digits:
//     x = 2^e_r * sum_s d_s * 2^(-7-8s) (+ a remainder below 2^(e_r - 8S)),
// with integer digits |d_s| <= 128, each exact in BF16.  The product of a
// digit pair is an integer of at most 2^14 in the pair's unit, so a tensor-
// core FP32 accumulation of up to 2^24 / (2^14 * pairs) terms is exact.  Pairs
// are grouped by level L = s + t (same unit 2^(-14-8L)), one TMEM accumulator
// per level, and only pairs with L <= S-1 are formed (the rest are below the
// dropped remainder).  Levels 0..3 are exact per 256-deep slice of K and are
// drained every 256 K into float-float running sums (FP32 pairs, ~48 bits);
// levels 4 and up are small enough that FP32 rounding there is below the
// result's precision.  The result is recombined in FP64.  With S = 6 the
// product is accurate to about 2^-46 relative to |A| |B| row/column-wise.
//
// Layout: operands are pre-split by ozk_split_kernel into K-major BF16 tiles
// already in the 64-byte-swizzled shared-memory order the MMA reads (rows of
// 32 K-elements = 64 B, 8-row atoms of 512 B), grouped so that the S digit
// tiles of one (row tile, K block) are contiguous: each pipeline stage is two
// cp.async.bulk copies.  M tile 128 rows, N tile 64, K block 32.
//
// The GEMM kernel is warp-specialised: warp 4 issues the bulk copies into a
// 3-stage (2 for seven digits) ring, one thread of warp 5 issues tcgen05.mma (cta_group::1,
// kind::f16, 128 x 64 x 16) into TMEM, warps 0-3 drain TMEM (tcgen05.ld,
// 32 lanes each) and write the output.  Every wait is bounded; on expiry the
// kernel records an error, waits (bounded) for its in-flight copies and MMAs,
// frees its TMEM and returns.
#include <cuda_bf16.h>

#include "hq_common.cuh"

namespace {

constexpr int TM = 128, TN = 64, TK = 32;
constexpr int MAX_STAGES = 3;
constexpr int KB_PER_DRAIN = 8;  // 256 K elements
constexpr int EXACT_LEVELS = 4;
constexpr int NT = 192;  // warps 0-3 epilogue, 4 producer, 5 MMA
constexpr int A_TILE = TM * TK * 2;  // 8 KB per digit tile
constexpr int B_TILE = TN * TK * 2;  // 4 KB per digit tile

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// ---------------------------------------------------------------------------
// Split

// Byte offset of element (row rr, k-in-block kk) inside a 64B-swizzled tile.
__device__ __forceinline__ int swz64(int rr, int kk) {
  const int c = kk >> 3;
  return rr * 64 + ((c ^ ((rr >> 1) & 3)) << 4) + (kk & 7) * 2;
}

// The fixed-point integer V = round(x * 2^(8S - 1 - e)) of one FP64 entry,
// computed from its bits (no FP64 arithmetic); |V| <= 2^(8S-1).
__device__ __forceinline__ long long fixed_point(double x, int shift_base) {
  const long long bits = __double_as_longlong(x);
  const int ex = (int)((bits >> 52) & 0x7FF);
  if (ex == 0 || ex == 0x7FF) return 0;  // zeros and subnormals -> 0
  const long long mant = (bits & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
  const int sh = ex + shift_base;
  long long V = 0;
  if (sh >= 0) V = mant << sh;
  else if (sh > -63) V = (mant + (1LL << (-sh - 1))) >> (-sh);
  return bits < 0 ? -V : V;
}

// Rows r < R of X (element (r, k) at X[r*rs + k*ks], k < K) -> S digit tiles.
// One warp per row; each lane takes 8-element chunks (one 16-byte group of a
// tile row), so every digit is written with one 16-byte store.  Rows
// R..RT*TR-1 and k >= K are written as zeros.
__global__ void ozk_split_kernel(const double* __restrict__ X, long long rs, long long ks, int R,
                                 int K, int S, int TR, int KB, int rows_total,
                                 uint8_t* __restrict__ tiles, int* __restrict__ exps) {
  const int lane = threadIdx.x & 31;
  const int warps = blockDim.x >> 5;
  const int nchunk = KB * (TK / 8);
  const long long tile_bytes = (long long)TR * TK * 2;
  for (int r = blockIdx.x * warps + (threadIdx.x >> 5); r < rows_total;
       r += gridDim.x * warps) {
    const bool live = r < R;
    const double* xr = X + (live ? (long long)r * rs : 0);
    double mx = 0.0;
    if (live)
      for (int k = lane; k < K; k += 32) mx = fmax(mx, fabs(xr[(long long)k * ks]));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if (mx > 0.0) frexp(mx, &e);  // mx < 2^e
    if (lane == 0) exps[r] = e;
    const int rt = r / TR, rr = r % TR;
    const int shift_base = 8 * S - 1076 - e;
    for (int ch = lane; ch < nchunk; ch += 32) {
      const int k0 = ch * 8;
      long long V[8];
#pragma unroll
      for (int j = 0; j < 8; ++j)
        V[j] = (live && k0 + j < K) ? fixed_point(xr[(long long)(k0 + j) * ks], shift_base) : 0;
      const int kb = k0 / TK, c = (k0 % TK) >> 3;
      uint8_t* base = tiles + ((long long)(rt * KB + kb) * S) * tile_bytes + rr * 64 +
                      ((c ^ ((rr >> 1) & 3)) << 4);
      // Balanced base-256 digits from the bottom; the top digit takes what is
      // left, which lies in [-128, 128].
      for (int s = S - 1; s >= 0; --s) {
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          const int d0 = s > 0 ? (int)(((V[j] + 128) & 255) - 128) : (int)V[j];
          const int d1 = s > 0 ? (int)(((V[j + 1] + 128) & 255) - 128) : (int)V[j + 1];
          V[j] = (V[j] - d0) >> 8;
          V[j + 1] = (V[j + 1] - d1) >> 8;
          const __nv_bfloat162 h = __floats2bfloat162_rn((float)d0, (float)d1);
          w[j >> 1] = *reinterpret_cast<const uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(base + (long long)s * tile_bytes) =
            make_uint4(w[0], w[1], w[2], w[3]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// GEMM

struct OzkArgs {
  const uint8_t* A;  // M-side tiles [MT][KB][S][TM x TK]
  const uint8_t* B;  // N-side tiles [NTL][KB][S][TN x TK]
  const int* ea;
  const int* eb;
  int M, N, S, KB;
  int kb_per_z;  // K blocks per grid.z slice (multiple of KB_PER_DRAIN)
  int mode;      // 0: out = sign * A B^T (per z slice); 1: C += sign * A B^T
  double* C;
  long long crs, ccs;  // element (r, c) at C[r*crs + c*ccs]
  long long zstride;   // mode 0, gridDim.z > 1: slice z writes at C + z*zstride
  double sign;
  int stages;  // 2 or 3, whatever fits in shared memory
  int* err;
  unsigned spin_limit;
};

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}

__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity, unsigned limit,
                                          volatile int* abort_flag) {
  for (unsigned it = 0; it < limit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    if (ok) return true;
    if (abort_flag && *abort_flag) return false;
  }
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;               // LBO, unused for swizzled K-major
  d |= (uint64_t)(512 >> 4) << 32;      // SBO: 8 rows x 64 B
  d |= (uint64_t)1 << 46;               // descriptor version for tcgen05
  d |= (uint64_t)4 << 61;               // 64-byte swizzle
  return d;
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t ad, uint64_t bd, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(b))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// (hi, lo) += x in FP32 pairs (TwoSum, then renormalise).
__device__ __forceinline__ void ff_add(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
  const float l = __fadd_rn(lo, e);
  const float h = __fadd_rn(s, l);
  lo = __fsub_rn(l, __fsub_rn(h, s));
  hi = h;
}

__global__ void __launch_bounds__(NT, 1) ozk_gemm_kernel(OzkArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[MAX_STAGES], empty_bar[MAX_STAGES];
  __shared__ __align__(8) uint64_t drain_full, drain_empty, done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int S = a.S;
  const int a_stage = S * A_TILE, b_stage = S * B_TILE;
  // One TN-column accumulator per level, rounded up to a power of two.
  const uint32_t tmem_cols = S * TN <= 64 ? 64u : (S * TN <= 128 ? 128u : (S * TN <= 256 ? 256u : 512u));
  uint8_t* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  uint8_t* sA = smem;
  const int STAGES = a.stages;
  uint8_t* sB = smem + STAGES * a_stage;
  const int mt = blockIdx.x, nt = blockIdx.y, z = blockIdx.z;
  const int kb0 = z * a.kb_per_z;
  const int nkb = min(a.KB - kb0, a.kb_per_z);
  const int ndrain = nkb > 0 ? (nkb - 1) / KB_PER_DRAIN : 0;  // drains before the final one

  if (tid == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&full_bar[i], 1);
      mbar_init(&empty_bar[i], 1);
    }
    mbar_init(&drain_full, 1);
    mbar_init(&drain_empty, 128);
    mbar_init(&done_bar, 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tbase = tmem_base;
  const unsigned lim = a.spin_limit;
  int mma_issued = 0;  // MMA thread: any tcgen05.mma issued
  int copies_issued = 0;

  if (warp == 4) {
    // Producer: one elected lane streams the digit tiles through the ring.
    if (lane == 0) {
      const uint8_t* Ab = a.A + ((long long)mt * a.KB) * a_stage;
      const uint8_t* Bb = a.B + ((long long)nt * a.KB) * b_stage;
      for (int i = 0; i < nkb; ++i) {
        const int st = i % STAGES;
        if (!mbar_wait(&empty_bar[st], ((i / STAGES) & 1) ^ 1, lim, &s_abort)) {
          s_abort = 1;
          break;
        }
        mbar_expect_tx(&full_bar[st], (unsigned)(a_stage + b_stage));
        bulk_g2s(sA + st * a_stage, Ab + (long long)(kb0 + i) * a_stage, a_stage, &full_bar[st]);
        bulk_g2s(sB + st * b_stage, Bb + (long long)(kb0 + i) * b_stage, b_stage, &full_bar[st]);
        ++copies_issued;
      }
    }
  } else if (warp == 5) {
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                             ((uint32_t)(TM >> 4) << 24);
      unsigned fresh = 0xFFu;  // bit L: the next MMA into level L overwrites
      int d = 0;
      for (int i = 0; i < nkb; ++i) {
        const int st = i % STAGES;
        if (!mbar_wait(&full_bar[st], (i / STAGES) & 1, lim, &s_abort)) {
          s_abort = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t abase = smem_u32(sA + st * a_stage), bbase = smem_u32(sB + st * b_stage);
        for (int s = 0; s < S; ++s) {
          for (int t = 0; s + t < S; ++t) {
            const int L = s + t;
            const uint32_t dt = tbase + (uint32_t)(L * TN);
#pragma unroll
            for (int kk = 0; kk < TK / 16; ++kk) {
              mma_bf16(dt, sw64_desc(abase + s * A_TILE + kk * 32),
                       sw64_desc(bbase + t * B_TILE + kk * 32), idesc, ((fresh >> L) & 1u) ^ 1u);
              fresh &= ~(1u << L);
              mma_issued = 1;
            }
          }
        }
        mma_commit(&empty_bar[st]);
        if ((i + 1) % KB_PER_DRAIN == 0 && i + 1 < nkb) {
          mma_commit(&drain_full);
          if (!mbar_wait(&drain_empty, d & 1, lim, &s_abort)) {
            s_abort = 1;
            break;
          }
          ++d;
          fresh |= (1u << EXACT_LEVELS) - 1u;
        }
      }
      mma_commit(&done_bar);
    }
  } else {
    // Epilogue warps 0-3: TMEM lanes 32*warp .. 32*warp+31 = tile rows.
    float hi[TN], lo[TN];
#pragma unroll
    for (int c = 0; c < TN; ++c) {
      hi[c] = 0.f;
      lo[c] = 0.f;
    }
    const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
    bool ok = true;
    for (int d = 0; d < ndrain && ok; ++d) {
      ok = mbar_wait(&drain_full, d & 1, lim, &s_abort);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int nl = min(S, EXACT_LEVELS);
#pragma unroll
      for (int c0 = 0; c0 < TN; c0 += 16) {
        for (int L = 0; L < nl; ++L) {
          float v[16];
          tmem_ld16(tbase + lane_off + (uint32_t)(L * TN + c0), v);
          const float w = __int_as_float((127 - 8 * L) << 23);  // 2^(-8L)
#pragma unroll
          for (int j = 0; j < 16; ++j) ff_add(hi[c0 + j], lo[c0 + j], __fmul_rn(v[j], w));
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(&drain_empty);
    }
    if (ok) ok = mbar_wait(&done_bar, 0, lim, &s_abort);
    if (!ok) {
      s_abort = 1;
    } else {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int c0 = 0; c0 < TN; c0 += 16) {
        for (int L = 0; L < S; ++L) {
          float v[16];
          tmem_ld16(tbase + lane_off + (uint32_t)(L * TN + c0), v);
          const float w = __int_as_float((127 - 8 * L) << 23);
#pragma unroll
          for (int j = 0; j < 16; ++j) ff_add(hi[c0 + j], lo[c0 + j], __fmul_rn(v[j], w));
        }
      }
      const int r = mt * TM + warp * 32 + lane;
      if (r < a.M) {
        // Output in chunks of 16 columns: every load (column scales, and C in
        // update mode) of a chunk is issued before any store, so the loads of
        // a chunk overlap instead of each waiting behind the previous store.
        const int* __restrict__ ebp = a.eb;
        double* __restrict__ crow = a.C + (long long)r * a.crs + (long long)z * a.zstride;
        const int er = a.ea[r] - 14;
#pragma unroll
        for (int c0 = 0; c0 < TN; c0 += 16) {
          int ek[16];
          double cv[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int n = nt * TN + c0 + j;
            ek[j] = n < a.N ? er + ebp[n] : 0;
            cv[j] = (a.mode == 1 && n < a.N) ? crow[(long long)n * a.ccs] : 0.0;
          }
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int n = nt * TN + c0 + j;
            if (n >= a.N) continue;
            // hi + lo is exact in FP64; scaling by a power of two is exact.
            const double v = ldexp(a.sign * ((double)hi[c0 + j] + (double)lo[c0 + j]), ek[j]);
            crow[(long long)n * a.ccs] = a.mode == 0 ? v : cv[j] + v;
          }
        }
      }
    }
  }

  // Teardown: on abort, wait (bounded) for in-flight copies and MMAs first.
  __syncthreads();
  if (s_abort) {
    if (tid == 0) atomicCAS(a.err, 0, HQ_ERR_BARRIER_TIMEOUT);
    if (warp == 4 && lane == 0) {
      // The last copy issued into each stage is the only one that can still
      // be in flight.
      for (int i = copies_issued > STAGES ? copies_issued - STAGES : 0; i < copies_issued; ++i)
        mbar_wait(&full_bar[i % STAGES], (i / STAGES) & 1, lim, nullptr);
    }
    if (warp == 5 && lane == 0 && mma_issued) {
      // done_bar was committed after the loop; its completion covers all MMAs.
      mbar_wait(&done_bar, 0, lim, nullptr);
    }
    __syncthreads();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase),
                 "r"(tmem_cols)
                 : "memory");
}

__global__ void ozk_sum_slices(int M, int N, int Z, const double* __restrict__ ws,
                               double* __restrict__ C, long long crs, long long ccs, int accumulate) {
  const long long total = (long long)M * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e % M), c = (int)(e / M);
    double s = 0.0;
    for (int zz = 0; zz < Z; ++zz) s += ws[e + (long long)zz * total];
    double* p = C + (long long)r * crs + (long long)c * ccs;
    *p = accumulate ? *p + s : s;
  }
}

}  // namespace

extern "C" size_t hq_ozk_tile_bytes(int rows, int K, int S, int side) {
  const int TR = side == 0 ? TM : TN;
  const long long RT = (rows + TR - 1) / TR, KB = (K + TK - 1) / TK;
  return (size_t)(RT * KB * S) * (size_t)(TR * TK * 2);
}

extern "C" int hq_ozk_split(cudaStream_t stream, const double* X, long long rs, long long ks,
                            int R, int K, int S, int side, void* tiles, int* exps) {
  if (R <= 0 || K <= 0) return 0;
  if (S < 1 || S > 7) return (int)cudaErrorInvalidValue;
  const int TR = side == 0 ? TM : TN;
  const int RT = (R + TR - 1) / TR, KB = (K + TK - 1) / TK;
  const int rows_total = RT * TR;
  int blocks = (rows_total + 7) / 8;
  if (blocks > 4096) blocks = 4096;
  ozk_split_kernel<<<blocks, 256, 0, stream>>>(X, rs, ks, R, K, S, TR, KB, rows_total,
                                               static_cast<uint8_t*>(tiles), exps);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_ozk_gemm(cudaStream_t stream, const hq_device_info* dev, int M, int N, int K,
                           int S, const void* Atiles, const int* ea, const void* Btiles,
                           const int* eb, int mode, double sign, double* C, long long crs,
                           long long ccs, double* ws, size_t ws_elems, int* err,
                           unsigned spin_limit) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  if (S < 1 || S > 7) return (int)cudaErrorInvalidValue;
  const int MT = (M + TM - 1) / TM, NTL = (N + TN - 1) / TN, KB = (K + TK - 1) / TK;
  // Split K across grid.z (mode 0 only) when the tile grid is short of the SMs.
  int Z = 1;
  if (mode == 0 && ws != nullptr) {
    const long long tiles = (long long)MT * NTL;
    const int max_z = (KB + KB_PER_DRAIN - 1) / KB_PER_DRAIN;
    while (Z < max_z && tiles * Z < 2LL * dev->num_sms &&
           (size_t)(Z + 1) * M * N <= ws_elems)
      ++Z;
  }
  int kb_per_z = (KB + Z - 1) / Z;
  kb_per_z = (kb_per_z + KB_PER_DRAIN - 1) / KB_PER_DRAIN * KB_PER_DRAIN;
  Z = (KB + kb_per_z - 1) / kb_per_z;
  OzkArgs a;
  a.A = static_cast<const uint8_t*>(Atiles);
  a.B = static_cast<const uint8_t*>(Btiles);
  a.ea = ea;
  a.eb = eb;
  a.M = M;
  a.N = N;
  a.S = S;
  a.KB = KB;
  a.kb_per_z = kb_per_z;
  a.mode = mode;
  a.sign = sign;
  a.err = err;
  a.spin_limit = spin_limit;
  if (Z > 1) {
    a.C = ws;
    a.crs = 1;
    a.ccs = M;
    a.zstride = (long long)M * N;
  } else {
    a.C = C;
    a.crs = crs;
    a.ccs = ccs;
    a.zstride = 0;
  }
  int stages = MAX_STAGES;
  size_t smem = (size_t)stages * S * (A_TILE + B_TILE) + 1024;
  if (smem > dev->smem_optin) {
    stages = 2;
    smem = (size_t)stages * S * (A_TILE + B_TILE) + 1024;
  }
  if (smem > dev->smem_optin) return (int)cudaErrorInvalidValue;
  a.stages = stages;
  cudaError_t e =
      cudaFuncSetAttribute(ozk_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  ozk_gemm_kernel<<<dim3(MT, NTL, Z), NT, smem, stream>>>(a);
  hq_count_launches(1);
  if (Z > 1) {
    long long total = (long long)M * N;
    int blocks = (int)((total + 255) / 256);
    if (blocks > dev->num_sms * 8) blocks = dev->num_sms * 8;
    ozk_sum_slices<<<blocks, 256, 0, stream>>>(M, N, Z, ws, C, crs, ccs, 0);
    hq_count_launches(1);
  }
  return (int)cudaGetLastError();
}
