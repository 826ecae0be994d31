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
// are grouped by level L = s + t (unit 2^(-14-8L)), and only pairs with
// L <= S-1 are formed (the rest are below the dropped remainder).  Digit s is
// stored pre-scaled by 2^(-8s) (exact in BF16), so every product already
// carries its level's weight.  Levels 0..3 each get a TMEM accumulator, exact
// per 256-deep slice of K (integers below 2^24 in their unit); level 4 gets its
// own; levels 5 and 6 need at most 2^-12 relative precision and share one.
// All are drained every 256 K into float-float running sums (FP32 pairs, ~48
// bits).  (Folding level 4 in as well measured 2^-47.5 instead of 2^-52: the
// tensor core's FP32 accumulation loses more than IEEE rounding when products
// of very different magnitude meet in one accumulator.)  Six accumulators
// instead of seven leave TMEM room for 80-column tiles in the short-K kernel --
// a tcgen05 BF16 MMA takes the same time for N = 64 as for N = 128.  The
// result is recombined in FP64.  With S = 7 the product is accurate to about
// 2^-52 relative to |A| |B| row/column-wise.
//
// Layout: the split writes each operand as S plain K-major BF16 digit
// matrices D[s][row][k] (rows padded to the tile height, K to 32).  The GEMM
// kernels read them with tensor-map TMA loads (cp.async.bulk.tensor.3d): one
// load per operand per pipeline stage brings a box of 32 K x tile rows x S
// digits into shared memory, swizzled by the copy engine into the 64-byte
// pattern the MMA descriptors name (rows of 64 B, 8-row atoms of 512 B).
// M tile 128 rows, N tile 80, K block 32.
//
// The GEMM kernels are warp-specialised: warp 20 issues the bulk copies into a
// 3-stage (2 for seven digits) ring, one thread of warp 21 issues tcgen05.mma
// (cta_group::1, kind::f16, 128 x 80 x 16) into TMEM, warps 0-19 drain TMEM
// (tcgen05.ld, five warps per 32-lane quadrant, 16 columns each) and write
// the output.  Every wait is bounded; on expiry the
// kernel records an error, waits (bounded) for its in-flight copies and MMAs,
// frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "hq_common.cuh"

namespace {

constexpr int TM = 128, TN = 80, TK = 32;  // six accumulators x 80 = 480 TMEM columns
constexpr int TN_SHORT = TN;  // the short-K kernel uses the same N tiles
constexpr int MAX_STAGES = 3;
constexpr int KB_PER_DRAIN = 8;  // 256 K elements
constexpr int MAX_ACC = 6;  // levels 0..4 alone (0..3 exact), 5 and 6 shared

__host__ __device__ constexpr int n_acc(int S) { return S < MAX_ACC ? S : MAX_ACC; }
__device__ __forceinline__ int acc_of_level(int L) { return L < MAX_ACC - 1 ? L : MAX_ACC - 1; }
__host__ __device__ inline uint32_t tmem_pow2(uint32_t c) {
  return c <= 32 ? 32u : (c <= 64 ? 64u : (c <= 128 ? 128u : (c <= 256 ? 256u : 512u)));
}
// Warps 0-19 epilogue (five per TMEM lane quadrant, each a fifth of the
// tile's columns), warp 20 producer, warp 21 MMA.  The epilogue is latency-
// bound (FP64 adds, C loads, TMEM loads): five warps per quadrant instead of
// two hide it -- 257 -> 206 ms of tensor-phase time per 16384^2 mixed
// factorization -- at 80 registers per thread.
constexpr int NT = 704;
constexpr int NEPI = 640;
constexpr int PRODUCER_WARP = 20, MMA_WARP = 21;
constexpr int EPI_COLS = TN / 5;  // columns per epilogue thread (a multiple of 8)
static_assert(TN % 5 == 0 && EPI_COLS % 8 == 0, "epilogue columns come in TMEM loads of 8");
constexpr int A_TILE = TM * TK * 2;  // 8 KB per digit tile
constexpr int B_TILE = TN * TK * 2;  // 5 KB per digit tile

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// ---------------------------------------------------------------------------
// Split

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

// The same digit times 2^(-8s) for slice s, so that products carry their
// level's weight: the FP32 pattern with exponent 23 - 8s and mantissa u is
// 2^(23-8s) + u 2^(-8s) exactly, and subtracting 2^(23-8s) + 128 2^(-8s)
// (exact in FP32) leaves (u - 128) 2^(-8s) in one add.
__device__ __forceinline__ uint32_t digit_scaled(uint32_t u, int s) {
  const float base = __uint_as_float(((uint32_t)(150 - 8 * s) << 23) | u);
  const float off = __uint_as_float(((uint32_t)(150 - 8 * s) << 23) | 128u);
  return __float_as_uint(__fsub_rn(base, off));
}

// Rows r < R of X (element (r, k) at X[r*rs + k*ks], k < K) -> S digit tiles.
// One warp per row; each lane takes 8-element chunks (one 16-byte group of a
// tile row), so every digit is written with one 16-byte store.  Rows
// R..RT*TR-1 and k >= K are written as zeros.  Balanced base-256 digits come
// from W = V + 128 * sum_p 256^p: digit p < S-1 is byte p of W minus 128, the
// top digit W >> 8(S-1) minus 128 (the same digits as peeling them from the
// bottom); slice s holds digit p = S-1-s, the most significant first.
template <int S>
__global__ void ozk_split_kernel(const double* __restrict__ X, long long rs, long long ks, int R,
                                 int K, int TR, int KB, int rows_total,
                                 uint8_t* __restrict__ tiles, int* __restrict__ exps) {
  HQ_PDL_WAIT();
  constexpr unsigned long long BIAS = 0x8080808080808080ULL >> (8 * (8 - S));
  const int lane = threadIdx.x & 31;
  const int warps = blockDim.x >> 5;
  const int nchunk = KB * (TK / 8);
  const long long kp = (long long)KB * TK;
  const long long slice_bytes = (long long)rows_total * kp * 2;
  for (int r = blockIdx.x * warps + (threadIdx.x >> 5); r < rows_total;
       r += gridDim.x * warps) {
    const bool live = r < R;
    const double* xr = X + (live ? (long long)r * rs : 0);
    // Largest magnitude from the bit patterns (integer compares).
    long long mb = 0;
    if (live)
      for (int k = lane; k < K; k += 32) {
        const long long bb = __double_as_longlong(xr[(long long)k * ks]) & 0x7FFFFFFFFFFFFFFFLL;
        mb = bb > mb ? bb : mb;
      }
    for (int o = 16; o > 0; o >>= 1) {
      const long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
      mb = ob > mb ? ob : mb;
    }
    // 2^e > max |x| >= 2^(e-1); 0 for zero or subnormal rows.
    const int bexp = (int)(mb >> 52);
    const int e = bexp == 0 ? 0 : bexp - 1022;
    if (lane == 0) exps[r] = e;
    const int shift_base = 8 * S - 1076 - e;
    for (int ch = lane; ch < nchunk; ch += 32) {
      const int k0 = ch * 8;
      unsigned long long W[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const long long V =
            (live && k0 + j < K) ? fixed_point(xr[(long long)(k0 + j) * ks], shift_base) : 0;
        W[j] = (unsigned long long)V + BIAS;
      }
      uint8_t* base = tiles + ((long long)r * kp + k0) * 2;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        // Slice s holds digit position p = S-1-s (slice 0 the most significant).
        const int p = S - 1 - s;
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          uint32_t u0, u1;
          if (p == S - 1) {
            u0 = (uint32_t)(W[j] >> (8 * p));
            u1 = (uint32_t)(W[j + 1] >> (8 * p));
          } else {
            u0 = (uint32_t)(W[j] >> (8 * p)) & 255u;
            u1 = (uint32_t)(W[j + 1] >> (8 * p)) & 255u;
          }
          w[j >> 1] = __byte_perm(digit_scaled(u0, s), digit_scaled(u1, s), 0x7632);
        }
        *reinterpret_cast<uint4*>(base + (long long)s * slice_bytes) =
            make_uint4(w[0], w[1], w[2], w[3]);
      }
    }
  }
}

// Column-major operand with short rows (row stride 1, K <= CM_KMAX, e.g. a
// panel's rows with K = its columns): reading a row walks a column stride
// per entry, so a CTA first stages 32 consecutive rows x K in shared memory
// with coalesced loads (one warp load = 32 consecutive rows of one column),
// then splits each row exactly as ozk_split_kernel does (same digits and
// exponents), one warp per row.
constexpr int CM_KMAX = 128;
template <int S>
__global__ void __launch_bounds__(256) ozk_split_cm_kernel(const double* __restrict__ X,
                                                           long long ks, int R, int K, int KB,
                                                           int rows_total,
                                                           uint8_t* __restrict__ tiles,
                                                           int* __restrict__ exps) {
  HQ_PDL_WAIT();
  constexpr unsigned long long BIAS = 0x8080808080808080ULL >> (8 * (8 - S));
  __shared__ double tile[CM_KMAX][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nchunk = KB * (TK / 8);
  const long long kp = (long long)KB * TK;
  const long long slice_bytes = (long long)rows_total * kp * 2;
  const int r0 = blockIdx.x * 32;
  for (int k = warp; k < K; k += 8) {
    const int r = r0 + lane;
    tile[k][lane] = r < R ? X[(long long)r + (long long)k * ks] : 0.0;
  }
  __syncthreads();
  for (int rr = warp; rr < 32; rr += 8) {
    const int r = r0 + rr;
    if (r >= rows_total) break;
    const bool live = r < R;
    long long mb = 0;
    if (live)
      for (int k = lane; k < K; k += 32) {
        const long long bb = __double_as_longlong(tile[k][rr]) & 0x7FFFFFFFFFFFFFFFLL;
        mb = bb > mb ? bb : mb;
      }
    for (int o = 16; o > 0; o >>= 1) {
      const long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
      mb = ob > mb ? ob : mb;
    }
    const int bexp = (int)(mb >> 52);
    const int e = bexp == 0 ? 0 : bexp - 1022;
    if (lane == 0) exps[r] = e;
    const int shift_base = 8 * S - 1076 - e;
    for (int ch = lane; ch < nchunk; ch += 32) {
      const int k0 = ch * 8;
      unsigned long long W[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const long long V = (live && k0 + j < K) ? fixed_point(tile[k0 + j][rr], shift_base) : 0;
        W[j] = (unsigned long long)V + BIAS;
      }
      uint8_t* base = tiles + ((long long)r * kp + k0) * 2;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int p = S - 1 - s;
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          uint32_t u0, u1;
          if (p == S - 1) {
            u0 = (uint32_t)(W[j] >> (8 * p));
            u1 = (uint32_t)(W[j + 1] >> (8 * p));
          } else {
            u0 = (uint32_t)(W[j] >> (8 * p)) & 255u;
            u1 = (uint32_t)(W[j + 1] >> (8 * p)) & 255u;
          }
          w[j >> 1] = __byte_perm(digit_scaled(u0, s), digit_scaled(u1, s), 0x7632);
        }
        *reinterpret_cast<uint4*>(base + (long long)s * slice_bytes) =
            make_uint4(w[0], w[1], w[2], w[3]);
      }
    }
  }
}

// Largest exponent field of each row, several CTAs per row (ROWMAX_SPAN
// entries each, eight loads in flight per thread) raising raw[r] -- zeroed
// before -- with an integer atomicMax: the first pass of the two-pass split
// for few long rows, which one CTA per row left latency-bound.
constexpr int ROWMAX_SPAN = 2048;
__global__ void __launch_bounds__(256) ozk_rowmax_atomic_kernel(const double* __restrict__ X,
                                                                long long rs, long long ks, int K,
                                                                int* __restrict__ raw) {
  HQ_PDL_WAIT();
  __shared__ long long s_max[8];
  const int r = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int k0 = blockIdx.y * ROWMAX_SPAN;
  const double* xr = X + (long long)r * rs;
  long long v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int k = k0 + tid + 256 * i;
    v[i] = k < K ? (__double_as_longlong(xr[(long long)k * ks]) & 0x7FFFFFFFFFFFFFFFLL) : 0;
  }
  long long mb = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) mb = v[i] > mb ? v[i] : mb;
  for (int o = 16; o > 0; o >>= 1) {
    const long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
    mb = ob > mb ? ob : mb;
  }
  if (lane == 0) s_max[warp] = mb;
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < 8; ++w) mb = s_max[w] > mb ? s_max[w] : mb;
    mb = s_max[0] > mb ? s_max[0] : mb;
    if (mb != 0) atomicMax(raw + r, (int)(mb >> 52));
  }
}

// One-pass variant for long rows (4096 <= K <= 16384 with 512 threads): one
// CTA per row holds the row in registers (CPT chunks of 8 per thread), takes
// the block maximum and writes the digits, so every entry is read from
// memory once (the two-pass kernel above re-reads each row, which misses L2
// when many long rows are in flight).  Same output as the kernel above.
template <int S, int CPT>
__global__ void __launch_bounds__(512) ozk_split_row_kernel(
    const double* __restrict__ X, long long rs, long long ks, int R, int K, int TR, int KB,
    int rows_total, uint8_t* __restrict__ tiles, int* __restrict__ exps) {
  HQ_PDL_WAIT();
  constexpr unsigned long long BIAS = 0x8080808080808080ULL >> (8 * (8 - S));
  constexpr int NTH = 512;
  __shared__ long long s_max[NTH / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nchunk = KB * (TK / 8);
  const long long kp = (long long)KB * TK;
  const long long slice_bytes = (long long)rows_total * kp * 2;
  for (int r = blockIdx.x; r < rows_total; r += gridDim.x) {
    const bool live = r < R;
    const double* xr = X + (live ? (long long)r * rs : 0);
    double v[CPT][8];
    long long mb = 0;
    // Contiguous, 16-byte aligned rows are read with 16-byte loads.
    const bool vec = ks == 1 && ((reinterpret_cast<uintptr_t>(xr) & 15) == 0);
#pragma unroll
    for (int i = 0; i < CPT; ++i) {
      const int k0 = (tid + i * NTH) * 8;
      if (vec && live && k0 + 8 <= K) {
        const double2* p2 = reinterpret_cast<const double2*>(xr + k0);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const double2 d = p2[j];
          v[i][2 * j] = d.x;
          v[i][2 * j + 1] = d.y;
        }
      } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) v[i][j] = (live && k0 + j < K) ? xr[(long long)(k0 + j) * ks] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const long long bb = __double_as_longlong(v[i][j]) & 0x7FFFFFFFFFFFFFFFLL;
        mb = bb > mb ? bb : mb;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
      mb = ob > mb ? ob : mb;
    }
    if (lane == 0) s_max[warp] = mb;
    __syncthreads();
    mb = s_max[0];
#pragma unroll
    for (int w = 1; w < NTH / 32; ++w) mb = s_max[w] > mb ? s_max[w] : mb;
    __syncthreads();  // s_max is rewritten for the next row
    const int bexp = (int)(mb >> 52);
    const int e = bexp == 0 ? 0 : bexp - 1022;
    if (tid == 0) exps[r] = e;
    const int shift_base = 8 * S - 1076 - e;
#pragma unroll
    for (int i = 0; i < CPT; ++i) {
      const int ch = tid + i * NTH;
      if (ch >= nchunk) continue;
      unsigned long long W[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) W[j] = (unsigned long long)fixed_point(v[i][j], shift_base) + BIAS;
      const int k0 = ch * 8;
      uint8_t* base = tiles + ((long long)r * kp + k0) * 2;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int p = S - 1 - s;
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          uint32_t u0, u1;
          if (p == S - 1) {
            u0 = (uint32_t)(W[j] >> (8 * p));
            u1 = (uint32_t)(W[j + 1] >> (8 * p));
          } else {
            u0 = (uint32_t)(W[j] >> (8 * p)) & 255u;
            u1 = (uint32_t)(W[j + 1] >> (8 * p)) & 255u;
          }
          w[j >> 1] = __byte_perm(digit_scaled(u0, s), digit_scaled(u1, s), 0x7632);
        }
        *reinterpret_cast<uint4*>(base + (long long)s * slice_bytes) =
            make_uint4(w[0], w[1], w[2], w[3]);
      }
    }
  }
}

// Long rows (K > 16384): the row does not fit the registers of one CTA, so
// the split takes two streaming passes -- the per-row scale exponent first,
// then every 8-element chunk of every row independently (consecutive threads
// take consecutive chunks of a row: coalesced 64-byte loads, 512-byte digit
// stores per warp and slice).  Same output as the kernels above.
__global__ void __launch_bounds__(256) ozk_rowmax_kernel(const double* __restrict__ X,
                                                         long long rs, long long ks, int R, int K,
                                                         int rows_total, int* __restrict__ exps) {
  HQ_PDL_WAIT();
  __shared__ long long s_max[8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int r = blockIdx.x; r < rows_total; r += gridDim.x) {
    long long mb = 0;
    if (r < R) {
      const double* xr = X + (long long)r * rs;
      for (int k = tid; k < K; k += 256) {
        const long long bb = __double_as_longlong(xr[(long long)k * ks]) & 0x7FFFFFFFFFFFFFFFLL;
        mb = bb > mb ? bb : mb;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const long long ob = __shfl_xor_sync(0xffffffffu, mb, o);
      mb = ob > mb ? ob : mb;
    }
    if (lane == 0) s_max[warp] = mb;
    __syncthreads();
    if (tid == 0) {
      for (int w = 1; w < 8; ++w) mb = s_max[w] > mb ? s_max[w] : mb;
      mb = s_max[0] > mb ? s_max[0] : mb;
      const int bexp = (int)(mb >> 52);
      exps[r] = bexp == 0 ? 0 : bexp - 1022;
    }
    __syncthreads();
  }
}

template <int S>
__global__ void __launch_bounds__(256) ozk_split_chunk_kernel(
    const double* __restrict__ X, long long rs, long long ks, int R, int K, int KB, int rows_total,
    uint8_t* __restrict__ tiles, int* __restrict__ exps, const int* __restrict__ raw) {
  HQ_PDL_WAIT();
  constexpr unsigned long long BIAS = 0x8080808080808080ULL >> (8 * (8 - S));
  const int nchunk = KB * (TK / 8);
  const long long kp = (long long)KB * TK;
  const long long slice_bytes = (long long)rows_total * kp * 2;
  const long long total = (long long)rows_total * nchunk;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(idx / nchunk), ch = (int)(idx % nchunk);
    const int k0 = ch * 8;
    const bool live = r < R;
    const double* xr = X + (live ? (long long)r * rs : 0);
    int e;
    if (raw != nullptr) {  // the rows' largest exponent fields, known in advance
      const int bexp = live ? raw[r] : 0;
      e = bexp == 0 ? 0 : bexp - 1022;
      if (ch == 0) exps[r] = e;
    } else {
      e = exps[r];
    }
    const int shift_base = 8 * S - 1076 - e;
    double v[8];
    if (live && ks == 1 && k0 + 8 <= K && ((reinterpret_cast<uintptr_t>(xr + k0) & 15) == 0)) {
      const double2* p2 = reinterpret_cast<const double2*>(xr + k0);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const double2 d = p2[j];
        v[2 * j] = d.x;
        v[2 * j + 1] = d.y;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = (live && k0 + j < K) ? xr[(long long)(k0 + j) * ks] : 0.0;
    }
    unsigned long long W[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) W[j] = (unsigned long long)fixed_point(v[j], shift_base) + BIAS;
    uint8_t* base = tiles + ((long long)r * kp + k0) * 2;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const int p = S - 1 - s;
      uint32_t w[4];
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        uint32_t u0, u1;
        if (p == S - 1) {
          u0 = (uint32_t)(W[j] >> (8 * p));
          u1 = (uint32_t)(W[j + 1] >> (8 * p));
        } else {
          u0 = (uint32_t)(W[j] >> (8 * p)) & 255u;
          u1 = (uint32_t)(W[j + 1] >> (8 * p)) & 255u;
        }
        w[j >> 1] = __byte_perm(digit_scaled(u0, s), digit_scaled(u1, s), 0x7632);
      }
      *reinterpret_cast<uint4*>(base + (long long)s * slice_bytes) = make_uint4(w[0], w[1], w[2], w[3]);
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
  // Short kernel, mode 1: when set, colexp[c] gets the largest exponent field
  // of the new C over rows >= row_lo of column c (atomicMax; zeroed before).
  int* colexp;
  int row_lo;
  // FP64 N-side operand (ozk_gemm_c64_kernel): eb_raw[n] is column n's
  // largest exponent field, from which its scale exponent follows (eb unused).
  const int* eb_raw;
};

// The scale exponent of a row whose largest exponent field is raw: 2^e >
// max |x| >= 2^(e-1), 0 for a zero row.
__device__ __forceinline__ int scale_of_raw(int raw) { return raw == 0 ? 0 : raw - 1022; }

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

// One box of a 3-D tensor map (k, row, digit) into shared memory, completing
// on the mbarrier; x = k must be a multiple of 8 (16 bytes of BF16).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
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

// An FP32 value times 2^ek (negated when neg) as an FP64, assembled from the
// bits on the integer pipe -- the FP64 pipe is this GPU's scarce resource and
// the epilogue of a short-K product would otherwise be bound by it.  Exact for
// FP32 normals; zero and FP32 subnormals give 0, and so do results below the
// FP64 normal range (negligible next to the rest of the sum).
__device__ __forceinline__ double f32_scaled(float f, int ek, unsigned neg) {
  const unsigned b = __float_as_uint(f);
  const int ex = (int)((b >> 23) & 0xFF);
  const int e64 = ex - 127 + 1023 + ek;
  const unsigned long long bits = ((unsigned long long)((b >> 31) ^ neg) << 63) |
                                  ((unsigned long long)(e64 & 0x7FF) << 52) |
                                  ((unsigned long long)(b & 0x7FFFFF) << 29);
  return (ex == 0 || e64 <= 0) ? 0.0 : __longlong_as_double(bits);
}

// Epilogue thread's share of a tile: TMEM lanes of its quadrant (one output
// row each), EPI_COLS columns starting at col0.  Adds the nacc accumulators
// of those columns into the float-float running sums.
// 16 consecutive TMEM columns of this warp's 32 lanes (one load, one wait).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// One 16-column TMEM load per accumulator (EPI_COLS = 16): half the
// load-and-wait round trips of 8-column loads, on the path the MMAs wait for.
__device__ __forceinline__ void drain_tmem(uint32_t tacc, int nacc, float* hi, float* lo) {
  static_assert(EPI_COLS == 16, "one 16-column load per accumulator");
  for (int q = 0; q < nacc; ++q) {
    float v[16];
    tmem_ld16(tacc + (uint32_t)(q * TN), v);
#pragma unroll
    for (int j = 0; j < 16; ++j) ff_add(hi[j], lo[j], v[j]);
  }
}

// Output of one row's EPI_COLS columns: out = sign * (hi + lo) * 2^(ea + eb - 14)
// (mode 0) or C += that (mode 1).  In update mode the row's C entries are
// first prefetched into L2 (no registers held), then read in batches of 8
// with every load of a batch issued before its stores.
__device__ __forceinline__ void write_row(const OzkArgs& a, int r, int n0, double* crow,
                                          const float* hi, const float* lo, bool live) {
  const unsigned neg = a.sign < 0.0 ? 1u : 0u;
  const int er = live ? a.ea[r] - 14 : 0;
  const bool counted = live && r >= a.row_lo;
  if (a.mode == 1 && live) {
#pragma unroll
    for (int j = 0; j < EPI_COLS; ++j)
      if (n0 + j < a.N)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(crow + (long long)(n0 + j) * a.ccs));
  }
#pragma unroll
  for (int c8 = 0; c8 < EPI_COLS; c8 += 8) {
    double cv[8];
    int ek[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int n = n0 + c8 + j;
      ek[j] = (live && n < a.N) ? er + (a.eb_raw ? scale_of_raw(a.eb_raw[n]) : a.eb[n]) : 0;
      cv[j] = (a.mode == 1 && live && n < a.N) ? crow[(long long)n * a.ccs] : 0.0;
    }
    unsigned fx[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int n = n0 + c8 + j;
      fx[j] = 0u;
      if (live && n < a.N) {
        // sign * (hi + lo) * 2^ek: the two exact conversions take no FP64
        // instruction, their sum one (exact: hi + lo fits in FP64).
        const double v = f32_scaled(hi[c8 + j], ek[j], neg) + f32_scaled(lo[c8 + j], ek[j], neg);
        const double out = a.mode == 0 ? v : cv[j] + v;
        crow[(long long)n * a.ccs] = out;
        if (counted) fx[j] = (unsigned)((__double_as_longlong(out) >> 52) & 0x7FF);
      }
    }
    if (a.colexp != nullptr) {  // kernel-uniform; every lane of the warp is here
      const int lane = threadIdx.x & 31;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const unsigned m = __reduce_max_sync(0xffffffffu, fx[j]);
        if (lane == j && m != 0u) atomicMax(a.colexp + n0 + c8 + j, (int)m);
      }
    }
  }
}

// Digit-pair MMAs of one K block into the accumulators at tb: pair (s, t) into
// acc_of_level(s + t).  fresh: bit q set = the next MMA into q overwrites.
__device__ __forceinline__ void issue_block(uint32_t tb, uint64_t da0, uint64_t db0, int S,
                                            uint32_t idesc, unsigned& fresh) {
  for (int s = 0; s < S; ++s) {
    const uint64_t da = da0 + (uint64_t)((s * A_TILE) >> 4);  // start address advances by bytes >> 4
    for (int t = 0; s + t < S; ++t) {
      const int q = acc_of_level(s + t);
      const uint64_t db = db0 + (uint64_t)((t * B_TILE) >> 4);
#pragma unroll
      for (int kk = 0; kk < TK / 16; ++kk) {
        mma_bf16(tb + (uint32_t)(q * TN), da + 2 * kk, db + 2 * kk, idesc, ((fresh >> q) & 1u) ^ 1u);
        fresh &= ~(1u << q);
      }
    }
  }
}

// The same for seven digits, fully unrolled: every descriptor offset, TMEM
// column and accumulate flag is a constant, so the single issuing thread
// spends its time on tcgen05.mma instead of loop and index arithmetic.
// FIRST: the first K block after a drain (the first MMA into each
// accumulator overwrites it; with seven digits every accumulator's first
// pair has s = 0).
template <bool FIRST>
__device__ __forceinline__ void issue_block7(uint32_t tb, uint64_t da0, uint64_t db0,
                                             uint32_t idesc) {
  constexpr int S = 7;
#pragma unroll
  for (int s = 0; s < S; ++s) {
#pragma unroll
    for (int t = 0; t < S - s; ++t) {
      const int L = s + t;
      const int q = L < MAX_ACC - 1 ? L : MAX_ACC - 1;
#pragma unroll
      for (int kk = 0; kk < TK / 16; ++kk) {
        const bool overwrite = FIRST && s == 0 && kk == 0 && t <= MAX_ACC - 1;
        mma_bf16(tb + (uint32_t)(q * TN), da0 + (uint64_t)((s * A_TILE) >> 4) + 2 * kk,
                 db0 + (uint64_t)((t * B_TILE) >> 4) + 2 * kk, idesc, overwrite ? 0u : 1u);
      }
    }
  }
}

__device__ __forceinline__ void issue_any(uint32_t tb, uint64_t da0, uint64_t db0, int S,
                                          uint32_t idesc, unsigned& fresh) {
  if (S == 7) {
    if (fresh == 0xFFu) issue_block7<true>(tb, da0, db0, idesc);
    else issue_block7<false>(tb, da0, db0, idesc);
    fresh = 0u;
  } else {
    issue_block(tb, da0, db0, S, idesc, fresh);
  }
}

__global__ void __launch_bounds__(NT, 1) ozk_gemm_kernel(OzkArgs a,
                                                        const __grid_constant__ CUtensorMap tmA,
                                                        const __grid_constant__ CUtensorMap tmB) {
  HQ_PDL_WAIT();
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[MAX_STAGES], empty_bar[MAX_STAGES];
  __shared__ __align__(8) uint64_t drain_full, drain_empty, done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int S = a.S;
  const int a_stage = S * A_TILE, b_stage = S * B_TILE;
  const int nacc = n_acc(S);
  const uint32_t tmem_cols = tmem_pow2((uint32_t)(nacc * TN));
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
    mbar_init(&drain_empty, NEPI);
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

  if (warp == PRODUCER_WARP) {
    // Producer: one elected lane streams the digit tiles through the ring.
    if (lane == 0) {
      for (int i = 0; i < nkb; ++i) {
        const int st = i % STAGES;
        if (!mbar_wait(&empty_bar[st], ((i / STAGES) & 1) ^ 1, lim, &s_abort)) {
          s_abort = 1;
          break;
        }
        mbar_expect_tx(&full_bar[st], (unsigned)(a_stage + b_stage));
        const int k0 = (kb0 + i) * TK;
        tma_load_3d(sA + st * a_stage, &tmA, k0, mt * TM, 0, &full_bar[st]);
        tma_load_3d(sB + st * b_stage, &tmB, k0, nt * TN, 0, &full_bar[st]);
        ++copies_issued;
      }
    }
  } else if (warp == MMA_WARP) {
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                             ((uint32_t)(TM >> 4) << 24);
      unsigned fresh = 0xFFu;
      int d = 0;
      for (int i = 0; i < nkb; ++i) {
        const int st = i % STAGES;
        if (!mbar_wait(&full_bar[st], (i / STAGES) & 1, lim, &s_abort)) {
          s_abort = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        issue_any(tbase, sw64_desc(smem_u32(sA + st * a_stage)),
                  sw64_desc(smem_u32(sB + st * b_stage)), S, idesc, fresh);
        mma_issued = 1;
        mma_commit(&empty_bar[st]);
        if ((i + 1) % KB_PER_DRAIN == 0 && i + 1 < nkb) {
          mma_commit(&drain_full);
          if (!mbar_wait(&drain_empty, d & 1, lim, &s_abort)) {
            s_abort = 1;
            break;
          }
          ++d;
          fresh = 0xFFu;  // every accumulator restarts after a drain
        }
      }
      mma_commit(&done_bar);
    }
  } else {
    // Epilogue warps 0-19: TMEM lanes 32*(warp&3).. = tile rows, columns
    // (warp>>2)*EPI_COLS.. of the tile.
    float hi[EPI_COLS], lo[EPI_COLS];
#pragma unroll
    for (int c = 0; c < EPI_COLS; ++c) {
      hi[c] = 0.f;
      lo[c] = 0.f;
    }
    const int col0 = (warp >> 2) * EPI_COLS;
    const uint32_t tacc = tbase + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)col0;
    bool ok = true;
    for (int d = 0; d < ndrain && ok; ++d) {
      ok = mbar_wait(&drain_full, d & 1, lim, &s_abort);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      drain_tmem(tacc, nacc, hi, lo);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(&drain_empty);
    }
    if (ok) ok = mbar_wait(&done_bar, 0, lim, &s_abort);
    if (!ok) {
      s_abort = 1;
    } else {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      drain_tmem(tacc, nacc, hi, lo);
      const int r = mt * TM + (warp & 3) * 32 + lane;
      if (r < a.M)
        write_row(a, r, nt * TN + col0, a.C + (long long)r * a.crs + (long long)z * a.zstride, hi,
                  lo, true);
    }
  }

  // Teardown: on abort, wait (bounded) for in-flight copies and MMAs first.
  __syncthreads();
  if (s_abort) {
    if (tid == 0) atomicCAS(a.err, 0, HQ_ERR_BARRIER_TIMEOUT);
    if (warp == PRODUCER_WARP && lane == 0) {
      // The last copy issued into each stage is the only one that can still
      // be in flight.
      for (int i = copies_issued > STAGES ? copies_issued - STAGES : 0; i < copies_issued; ++i)
        mbar_wait(&full_bar[i % STAGES], (i / STAGES) & 1, lim, nullptr);
    }
    if (warp == MMA_WARP && lane == 0 && mma_issued) {
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

// Long-K product whose N-side operand is read as FP64 (C in the block update
// W1 = U'^T C): the producer brings each K block of C (80 columns x 32 rows,
// 20 KB) with a 2-D tensor-map load next to the M side's digit tiles, and the
// epilogue warps -- idle between drains -- cut it into the seven digit planes
// in shared memory, in the 64-byte-swizzled layout the MMA descriptors read
// (16-byte chunk c of row r of a 64-byte row at chunk c ^ ((r >> 1) & 3)).
// The column scales come from eb_raw (each column's largest exponent field,
// recorded by the epilogue of the update that wrote C), so nothing is read
// twice: the trailing matrix is read once as FP64 instead of being split to
// 14 bytes of digits per entry and read back.  The digits are those
// ozk_split_chunk_kernel writes.  A conversion barrier per stage orders the
// digit writes (generic proxy, fenced to the async proxy) before the MMAs.
constexpr int C64_TILE = TN * TK * 8;  // 20 KB of FP64 per stage

// One thread's share of a block's conversion: 4 consecutive K entries (h-th
// quarter of the 32) of tile column c, read as two 16-byte loads, written as
// 8 bytes of each digit plane.
template <int S>
__device__ __forceinline__ void convert_quarter(const double* __restrict__ sC, uint8_t* sBst, int c,
                                                int h, int shift_base) {
  constexpr unsigned long long BIAS = 0x8080808080808080ULL >> (8 * (8 - S));
  const double2* x2 = reinterpret_cast<const double2*>(sC + c * TK + h * 4);
  const double2 p0 = x2[0], p1 = x2[1];
  const double x[4] = {p0.x, p0.y, p1.x, p1.y};
  unsigned long long W[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) W[j] = (unsigned long long)fixed_point(x[j], shift_base) + BIAS;
  const int phys = (h >> 1) ^ ((c >> 1) & 3);  // 64-byte swizzle of the 16-byte chunk
  uint8_t* dst = sBst + c * (TK * 2) + phys * 16 + (h & 1) * 8;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int p = S - 1 - s;
    uint32_t w[2];
#pragma unroll
    for (int j = 0; j < 4; j += 2) {
      uint32_t u0, u1;
      if (p == S - 1) {
        u0 = (uint32_t)(W[j] >> (8 * p));
        u1 = (uint32_t)(W[j + 1] >> (8 * p));
      } else {
        u0 = (uint32_t)(W[j] >> (8 * p)) & 255u;
        u1 = (uint32_t)(W[j + 1] >> (8 * p)) & 255u;
      }
      w[j >> 1] = __byte_perm(digit_scaled(u0, s), digit_scaled(u1, s), 0x7632);
    }
    *reinterpret_cast<uint2*>(dst + s * B_TILE) = make_uint2(w[0], w[1]);
  }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__global__ void __launch_bounds__(NT, 1) ozk_gemm_c64_kernel(
    OzkArgs a, const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmC) {
  HQ_PDL_WAIT();
  constexpr int S = 7;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // a_full: the M side's digits of a block landed; c_full: its FP64 N-side
  // tile landed; c_empty: the converters are done with that FP64 tile;
  // conv_bar: its digits are in the B stage; empty_bar: the MMAs are done
  // with the A and B stages.  The FP64 tile of block i is fetched as soon as
  // block i - 2's was converted, so its load never waits for the MMAs.
  __shared__ __align__(8) uint64_t a_full[MAX_STAGES], c_full[MAX_STAGES], c_empty[MAX_STAGES],
      empty_bar[MAX_STAGES], conv_bar[MAX_STAGES];
  __shared__ __align__(8) uint64_t drain_full, drain_empty, done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int a_stage = S * A_TILE, b_stage = S * B_TILE;
  const int nacc = n_acc(S);
  const uint32_t tmem_cols = tmem_pow2((uint32_t)(nacc * TN));
  uint8_t* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  const int STAGES = a.stages;
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * a_stage;
  uint8_t* sC = sB + STAGES * b_stage;  // FP64 staging, C64_TILE per stage
  const int mt = blockIdx.x, nt = blockIdx.y, z = blockIdx.z;
  const int kb0 = z * a.kb_per_z;
  const int nkb = min(a.KB - kb0, a.kb_per_z);
  const int ndrain = nkb > 0 ? (nkb - 1) / KB_PER_DRAIN : 0;

  if (tid == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&a_full[i], 1);
      mbar_init(&c_full[i], 1);
      mbar_init(&c_empty[i], NEPI);
      mbar_init(&empty_bar[i], 1);
      mbar_init(&conv_bar[i], NEPI);
    }
    mbar_init(&drain_full, 1);
    mbar_init(&drain_empty, NEPI);
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
  int mma_issued = 0;
  int a_issued = 0, c_issued = 0;  // producer lanes 0 and 1

  if (warp == PRODUCER_WARP) {
    if (lane == 0) {  // the M side's digit tiles, as the MMAs free the stages
      for (int i = 0; i < nkb; ++i) {
        const int st = i % STAGES;
        if (!mbar_wait(&empty_bar[st], ((i / STAGES) & 1) ^ 1, lim, &s_abort)) {
          s_abort = 1;
          break;
        }
        mbar_expect_tx(&a_full[st], (unsigned)a_stage);
        tma_load_3d(sA + st * a_stage, &tmA, (kb0 + i) * TK, mt * TM, 0, &a_full[st]);
        ++a_issued;
      }
    } else if (lane == 1) {  // the FP64 tiles, as the converters free them
      for (int i = 0; i < nkb; ++i) {
        const int st = i % STAGES;
        if (!mbar_wait(&c_empty[st], ((i / STAGES) & 1) ^ 1, lim, &s_abort)) {
          s_abort = 1;
          break;
        }
        mbar_expect_tx(&c_full[st], (unsigned)C64_TILE);
        tma_load_2d(sC + st * C64_TILE, &tmC, (kb0 + i) * TK, nt * TN, &c_full[st]);
        ++c_issued;
      }
    }
  } else if (warp == MMA_WARP) {
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                             ((uint32_t)(TM >> 4) << 24);
      unsigned fresh = 0xFFu;
      int d = 0;
      for (int i = 0; i < nkb; ++i) {
        const int st = i % STAGES;
        if (!mbar_wait(&a_full[st], (i / STAGES) & 1, lim, &s_abort) ||
            !mbar_wait(&conv_bar[st], (i / STAGES) & 1, lim, &s_abort)) {
          s_abort = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        issue_any(tbase, sw64_desc(smem_u32(sA + st * a_stage)),
                  sw64_desc(smem_u32(sB + st * b_stage)), S, idesc, fresh);
        mma_issued = 1;
        mma_commit(&empty_bar[st]);
        if ((i + 1) % KB_PER_DRAIN == 0 && i + 1 < nkb) {
          mma_commit(&drain_full);
          if (!mbar_wait(&drain_empty, d & 1, lim, &s_abort)) {
            s_abort = 1;
            break;
          }
          ++d;
          fresh = 0xFFu;
        }
      }
      mma_commit(&done_bar);
    }
  } else {
    // Epilogue warps 0-19: convert every K block, drain every 256 K, write.
    float hi[EPI_COLS], lo[EPI_COLS];
#pragma unroll
    for (int c = 0; c < EPI_COLS; ++c) {
      hi[c] = 0.f;
      lo[c] = 0.f;
    }
    const int col0 = (warp >> 2) * EPI_COLS;
    const uint32_t tacc = tbase + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)col0;
    // Conversion task of this thread: column cc of the tile, quarter cq
    // (4 K entries) of the block's 32 -- 80 x 8 tasks, one per epilogue thread.
    static_assert(TN * (TK / 4) == NEPI, "one conversion task per epilogue thread");
    const int cc = tid >> 3, cq = tid & 7;
    int shift_base = 0;
    {
      const int n = nt * TN + cc;
      shift_base = 8 * S - 1076 - (n < a.N ? scale_of_raw(a.eb_raw[n]) : 0);
    }
    bool ok = true;
    int d = 0;
    for (int i = 0; i < nkb && ok; ++i) {
      const int st = i % STAGES;
      // The FP64 tile is here, and the MMAs of block i - STAGES are done with
      // the B stage the digits go to.
      ok = mbar_wait(&c_full[st], (i / STAGES) & 1, lim, &s_abort) &&
           mbar_wait(&empty_bar[st], ((i / STAGES) & 1) ^ 1, lim, &s_abort);
      if (!ok) break;
      convert_quarter<S>(reinterpret_cast<const double*>(sC + st * C64_TILE), sB + st * b_stage,
                         cc, cq, shift_base);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(&conv_bar[st]);
      mbar_arrive(&c_empty[st]);
      if ((i + 1) % KB_PER_DRAIN == 0 && i + 1 < nkb && d < ndrain) {
        ok = mbar_wait(&drain_full, d & 1, lim, &s_abort);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        drain_tmem(tacc, nacc, hi, lo);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        mbar_arrive(&drain_empty);
        ++d;
      }
    }
    if (ok) ok = mbar_wait(&done_bar, 0, lim, &s_abort);
    if (!ok) {
      s_abort = 1;
    } else {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      drain_tmem(tacc, nacc, hi, lo);
      const int r = mt * TM + (warp & 3) * 32 + lane;
      if (r < a.M)
        write_row(a, r, nt * TN + col0, a.C + (long long)r * a.crs + (long long)z * a.zstride, hi,
                  lo, true);
    }
  }

  // Teardown: on abort, wait (bounded) for in-flight copies and MMAs first.
  __syncthreads();
  if (s_abort) {
    if (tid == 0) atomicCAS(a.err, 0, HQ_ERR_BARRIER_TIMEOUT);
    if (warp == PRODUCER_WARP && lane == 0) {
      for (int i = a_issued > STAGES ? a_issued - STAGES : 0; i < a_issued; ++i)
        mbar_wait(&a_full[i % STAGES], (i / STAGES) & 1, lim, nullptr);
    }
    if (warp == PRODUCER_WARP && lane == 1) {
      for (int i = c_issued > STAGES ? c_issued - STAGES : 0; i < c_issued; ++i)
        mbar_wait(&c_full[i % STAGES], (i / STAGES) & 1, lim, nullptr);
    }
    if (warp == MMA_WARP && lane == 0 && mma_issued) mbar_wait(&done_bar, 0, lim, nullptr);
    __syncthreads();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase),
                 "r"(tmem_cols)
                 : "memory");
}

// Persistent variant for short products (K <= 256, so no intermediate drain
// of the exact levels): one CTA per SM walks the output tiles (TM x TN), and
// the producer streams operand stages ahead across tile boundaries.  The
// epilogue warps first drain a tile's accumulators into registers and hand
// the TMEM back, then do the FP64 output (the part bound by the FP64 pipe and
// by C's memory traffic) while the MMAs of the next tile run.  Mode 1
// (C += sign * A B^T) or 0 (C = sign * A B^T), no grid.z split.
__global__ void __launch_bounds__(NT, 1) ozk_gemm_short_kernel(
    OzkArgs a, const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB) {
  HQ_PDL_WAIT();
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[MAX_STAGES], empty_bar[MAX_STAGES];
  __shared__ __align__(8) uint64_t tfull, tempty, done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int S = a.S;
  const int a_stage = S * A_TILE, b_stage = S * B_TILE;
  const int nacc = n_acc(S);
  const uint32_t tmem_cols = tmem_pow2((uint32_t)(nacc * TN));
  uint8_t* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  const int STAGES = a.stages;
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * a_stage;
  const int MT = (a.M + TM - 1) / TM, NTL = (a.N + TN - 1) / TN;
  const int ntiles = MT * NTL, nkb = a.KB;

  if (tid == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&full_bar[i], 1);
      mbar_init(&empty_bar[i], 1);
    }
    mbar_init(&tfull, 1);
    mbar_init(&tempty, NEPI);
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
  int mma_issued = 0;
  int copies_issued = 0;

  if (warp == PRODUCER_WARP) {
    if (lane == 0) {
      int i = 0;  // stage counter across tiles
      for (int t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x) {
        const int mt = t / NTL, nt = t % NTL;
        for (int kb = 0; kb < nkb; ++kb, ++i) {
          const int st = i % STAGES;
          if (!mbar_wait(&empty_bar[st], ((i / STAGES) & 1) ^ 1, lim, &s_abort)) {
            s_abort = 1;
            break;
          }
          mbar_expect_tx(&full_bar[st], (unsigned)(a_stage + b_stage));
          tma_load_3d(sA + st * a_stage, &tmA, kb * TK, mt * TM, 0, &full_bar[st]);
          tma_load_3d(sB + st * b_stage, &tmB, kb * TK, nt * TN, 0, &full_bar[st]);
          ++copies_issued;
        }
      }
    }
  } else if (warp == MMA_WARP) {
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                             ((uint32_t)(TM >> 4) << 24);
      int i = 0, lt = 0;
      for (int t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x, ++lt) {
        if (!mbar_wait(&tempty, (lt & 1) ^ 1, lim, &s_abort)) {
          s_abort = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        unsigned fresh = 0xFFu;
        bool ok = true;
        for (int kb = 0; kb < nkb; ++kb, ++i) {
          const int st = i % STAGES;
          if (!mbar_wait(&full_bar[st], (i / STAGES) & 1, lim, &s_abort)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          issue_any(tbase, sw64_desc(smem_u32(sA + st * a_stage)),
                    sw64_desc(smem_u32(sB + st * b_stage)), S, idesc, fresh);
          mma_issued = 1;
          mma_commit(&empty_bar[st]);
        }
        if (!ok) {
          s_abort = 1;
          break;
        }
        mma_commit(&tfull);
      }
      mma_commit(&done_bar);
    }
  } else {
    const int col0 = (warp >> 2) * EPI_COLS;
    const uint32_t tacc = tbase + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)col0;
    int lt = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
      // One outcome per warp: the TMEM loads and the exponent reduction
      // below are warp-wide, so no lane may leave the loop alone.
      if (!__all_sync(0xffffffffu, mbar_wait(&tfull, lt & 1, lim, &s_abort))) {
        s_abort = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      float hi[EPI_COLS], lo[EPI_COLS];
#pragma unroll
      for (int c = 0; c < EPI_COLS; ++c) {
        hi[c] = 0.f;
        lo[c] = 0.f;
      }
      drain_tmem(tacc, nacc, hi, lo);
      // The sums are in registers: hand the TMEM back for the next tile.
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(&tempty);
      const int mt = t / NTL, nt = t % NTL;
      const int r = mt * TM + (warp & 3) * 32 + lane;
      // Every lane takes part (the column-exponent reduction is warp-wide);
      // rows past M only skip their loads and stores.
      write_row(a, r, nt * TN + col0, a.C + (long long)(r < a.M ? r : 0) * a.crs, hi, lo,
                r < a.M);
    }
  }

  // Teardown: on abort, wait (bounded) for in-flight copies and MMAs first.
  __syncthreads();
  if (s_abort) {
    if (tid == 0) atomicCAS(a.err, 0, HQ_ERR_BARRIER_TIMEOUT);
    if (warp == PRODUCER_WARP && lane == 0) {
      for (int i = copies_issued > STAGES ? copies_issued - STAGES : 0; i < copies_issued; ++i)
        mbar_wait(&full_bar[i % STAGES], (i / STAGES) & 1, lim, nullptr);
    }
    if (warp == MMA_WARP && lane == 0 && mma_issued) mbar_wait(&done_bar, 0, lim, nullptr);
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
  HQ_PDL_WAIT();
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

// side 0: M-side tiles (TM rows); 1: N-side tiles (TN rows) for the general
// kernel; 2: N-side tiles of TN_SHORT rows for the short-K kernel.
extern "C" size_t hq_ozk_tile_bytes(int rows, int K, int S, int side) {
  const int TR = side == 0 ? TM : (side == 2 ? TN_SHORT : TN);
  const long long RT = (rows + TR - 1) / TR, KB = (K + TK - 1) / TK;
  return (size_t)(RT * KB * S) * (size_t)(TR * TK * 2);
}

extern "C" int hq_ozk_rowmax_raw(cudaStream_t stream, const double* X, long long rs,
                                 long long ks, int R, int K, int rows_total, int* raw) {
  if (R <= 0 || K <= 0) return 0;
  const int e = hq_zero_words(stream, raw, (size_t)rows_total, nullptr, 0);
  if (e) return e;
  hq_launch(ozk_rowmax_atomic_kernel, dim3(R, (K + ROWMAX_SPAN - 1) / ROWMAX_SPAN), 256, 0, stream,
      X, rs, ks, K, raw);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_ozk_split_rows(int R, int side) {
  const int TR = side == 0 ? TM : (side == 2 ? TN_SHORT : TN);
  return (R + TR - 1) / TR * TR;
}

extern "C" int hq_ozk_split(cudaStream_t stream, const double* X, long long rs, long long ks,
                            int R, int K, int S, int side, void* tiles, int* exps, int* raw) {
  if (R <= 0 || K <= 0) return 0;
  if (S < 1 || S > 7) return (int)cudaErrorInvalidValue;
  const int TR = side == 0 ? TM : (side == 2 ? TN_SHORT : TN);
  const int RT = (R + TR - 1) / TR, KB = (K + TK - 1) / TK;
  const int rows_total = RT * TR;
  int blocks = (rows_total + 7) / 8;
  if (blocks > 4096) blocks = 4096;
  uint8_t* t = static_cast<uint8_t*>(tiles);
  constexpr int ROW_CPT = 4;
  // Long rows (K > 16384), or fewer than FEW_ROWS rows of 512 or more (the
  // one-pass kernel's 8-row CTAs would then number fewer than a GB300's 152
  // SMs, each warp walking a long row), take the two-pass split, which
  // spreads every row over CTAs.
  constexpr int FEW_ROWS = 8 * 152;
  if (S == 7 && (K > 512 * 8 * ROW_CPT || (K >= 512 && rows_total < FEW_ROWS))) {
    const long long chunks = (long long)rows_total * KB * (TK / 8);
    long long cblocks = (chunks + 255) / 256;
    if (cblocks > 65536) cblocks = 65536;
    if (raw != nullptr) {  // row maxima with several CTAs per row (scratch given)
      const int e = hq_ozk_rowmax_raw(stream, X, rs, ks, R, K, rows_total, raw);
      if (e) return e;
      hq_launch(ozk_split_chunk_kernel<7>, (unsigned)cblocks, 256, 0, stream, X, rs, ks, R, K, KB,
                                                                        rows_total, t, exps, raw);
      hq_count_launches(1);
      return (int)cudaGetLastError();
    }
    int mblocks = rows_total < 8192 ? rows_total : 8192;
    hq_launch(ozk_rowmax_kernel, mblocks, 256, 0, stream, X, rs, ks, R, K, rows_total, exps);
    hq_launch(ozk_split_chunk_kernel<7>, (unsigned)cblocks, 256, 0, stream, X, rs, ks, R, K, KB,
                                                                      rows_total, t, exps, nullptr);
    hq_count_launches(2);
    return (int)cudaGetLastError();
  }
  if (rs == 1 && ks != 1 && K <= CM_KMAX) {  // column-major rows of a short operand
    const int cb = (rows_total + 31) / 32;
    switch (S) {
#define HQ_SPLIT_CM_CASE(SS)                                                            \
  case SS:                                                                              \
    hq_launch(ozk_split_cm_kernel<SS>, cb, 256, 0, stream, X, ks, R, K, KB, rows_total, t, exps); \
    break;
      HQ_SPLIT_CM_CASE(1) HQ_SPLIT_CM_CASE(2) HQ_SPLIT_CM_CASE(3) HQ_SPLIT_CM_CASE(4)
      HQ_SPLIT_CM_CASE(5) HQ_SPLIT_CM_CASE(6) HQ_SPLIT_CM_CASE(7)
#undef HQ_SPLIT_CM_CASE
    }
    hq_count_launches(1);
    return (int)cudaGetLastError();
  }
  if (K >= 4096 && K <= 512 * 8 * ROW_CPT && S == 7) {
    int rblocks = rows_total < 16384 ? rows_total : 16384;
    hq_launch(ozk_split_row_kernel<7, ROW_CPT>, rblocks, 512, 0, stream, X, rs, ks, R, K, TR, KB,
                                                                 rows_total, t, exps);
    hq_count_launches(1);
    return (int)cudaGetLastError();
  }
  switch (S) {
#define HQ_SPLIT_CASE(SS)                                                                  \
  case SS:                                                                                 \
    hq_launch(ozk_split_kernel<SS>, blocks, 256, 0, stream, X, rs, ks, R, K, TR, KB, rows_total, t, \
                                                     exps);                                \
    break;
    HQ_SPLIT_CASE(1) HQ_SPLIT_CASE(2) HQ_SPLIT_CASE(3) HQ_SPLIT_CASE(4) HQ_SPLIT_CASE(5)
    HQ_SPLIT_CASE(6) HQ_SPLIT_CASE(7)
#undef HQ_SPLIT_CASE
  }
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

// The split with each row's largest exponent field already known (raw[r],
// e.g. produced by the epilogue of the update that wrote X): one streaming
// pass, no row maximum.  exps receives the scale exponents as hq_ozk_split
// writes them.
extern "C" int hq_ozk_split_raw(cudaStream_t stream, const double* X, long long rs, long long ks,
                                int R, int K, int S, int side, void* tiles, int* exps,
                                const int* raw) {
  if (R <= 0 || K <= 0) return 0;
  if (S != 7) return (int)cudaErrorInvalidValue;
  const int TR = side == 0 ? TM : (side == 2 ? TN_SHORT : TN);
  const int RT = (R + TR - 1) / TR, KB = (K + TK - 1) / TK;
  const int rows_total = RT * TR;
  const long long chunks = (long long)rows_total * KB * (TK / 8);
  long long cblocks = (chunks + 255) / 256;
  if (cblocks > 65536) cblocks = 65536;
  hq_launch(ozk_split_chunk_kernel<7>, (unsigned)cblocks, 256, 0, stream,
      X, rs, ks, R, K, KB, rows_total, static_cast<uint8_t*>(tiles), exps, raw);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

// Tensor map of a split operand: D[s][row][k], BF16, dims (k, row, digit) =
// (kp, rows_p, S); box 32 x tile_rows x S, 64-byte swizzle.
static int make_digit_map(CUtensorMap* map, const void* tiles, int rows, int K, int S,
                          int tile_rows) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (encode == nullptr) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || fn == nullptr)
      return (int)cudaErrorNotSupported;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const cuuint64_t rp = (cuuint64_t)((rows + tile_rows - 1) / tile_rows) * tile_rows;
  const cuuint64_t kp = (cuuint64_t)((K + TK - 1) / TK) * TK;
  const cuuint64_t dims[3] = {kp, rp, (cuuint64_t)S};
  const cuuint64_t strides[2] = {kp * 2, rp * kp * 2};  // bytes, dims 1 and 2
  const cuuint32_t box[3] = {(cuuint32_t)TK, (cuuint32_t)tile_rows, (cuuint32_t)S};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(tiles), dims,
                      strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : (int)cudaErrorInvalidValue;
}

// Split K of the long products (one CTA per SM): the time is about (waves)
// x (K blocks per CTA + a fixed cost of ~2 per tile) plus the slices' sum.
// Taking the split that minimizes it, instead of the first one past two
// waves, keeps the last wave from running mostly empty (modelled 16 % less
// W1 time over a 16384^2 factorization's blocks).  Both long kernels use it,
// so they sum the same slices in the same order.
static int choose_split(long long tiles, int KB, int M, int N, size_t ws_elems, int num_sms) {
  const int max_z = (KB + KB_PER_DRAIN - 1) / KB_PER_DRAIN;
  int Z = 1;
  double best = 1e300;
  for (int z = 1; z <= max_z; ++z) {
    if (z > 1 && (size_t)(z + 1) * M * N > ws_elems) break;
    int kz = (KB + z - 1) / z;
    kz = (kz + KB_PER_DRAIN - 1) / KB_PER_DRAIN * KB_PER_DRAIN;
    const int zz = (KB + kz - 1) / kz;
    const long long waves = (tiles * zz + num_sms - 1) / num_sms;
    const double sum = zz > 1 ? (double)zz * M * N / (6000.0 * num_sms) : 0.0;
    const double cost = (double)waves * (kz + 2.0) + sum;
    if (cost < best) {
      best = cost;
      Z = zz;
    }
  }
  return Z;
}

extern "C" int hq_ozk_gemm(cudaStream_t stream, const hq_device_info* dev, int M, int N, int K,
                           int S, const void* Atiles, const int* ea, const void* Btiles,
                           const int* eb, int mode, double sign, double* C, long long crs,
                           long long ccs, double* ws, size_t ws_elems, int* err,
                           unsigned spin_limit) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  if (S < 1 || S > 7) return (int)cudaErrorInvalidValue;
  const int MT = (M + TM - 1) / TM, NTL = (N + TN - 1) / TN, KB = (K + TK - 1) / TK;
  // Split K across grid.z (mode 0 only).
  int Z = 1;
  if (mode == 0 && ws != nullptr)
    Z = choose_split((long long)MT * NTL, KB, M, N, ws_elems, dev->num_sms);
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
  a.colexp = nullptr;
  a.row_lo = 0;
  a.eb_raw = nullptr;
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
  CUtensorMap tmA, tmB;
  int rc = make_digit_map(&tmA, Atiles, M, K, S, TM);
  if (rc == 0) rc = make_digit_map(&tmB, Btiles, N, K, S, TN);
  if (rc) return rc;
  cudaError_t e =
      cudaFuncSetAttribute(ozk_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  hq_launch(ozk_gemm_kernel, dim3(MT, NTL, Z), NT, smem, stream, a, tmA, tmB);
  hq_count_launches(1);
  if (Z > 1) {
    long long total = (long long)M * N;
    int blocks = (int)((total + 255) / 256);
    if (blocks > dev->num_sms * 8) blocks = dev->num_sms * 8;
    hq_launch(ozk_sum_slices, blocks, 256, 0, stream, M, N, Z, ws, C, crs, ccs, 0);
    hq_count_launches(1);
  }
  return (int)cudaGetLastError();
}

// W1-style product with an FP64 N-side operand: Y element (n, k) at
// Y[n * yld + k] (k contiguous), n < N, k < K; raw[n] = row n's largest
// exponent field.  Mode 0 only (C = sign * A Y^T, split K through ws as in
// hq_ozk_gemm).  Returns cudaErrorNotSupported when Y's layout does not meet
// the tensor-map rules (16-byte aligned base and stride), so the caller can
// split Y instead.
extern "C" int hq_ozk_gemm_c64(cudaStream_t stream, const hq_device_info* dev, int M, int N,
                               int K, const void* Atiles, const int* ea, const double* Y,
                               long long yld, const int* raw, double sign, double* C,
                               long long crs, long long ccs, double* ws, size_t ws_elems,
                               int* err, unsigned spin_limit) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  constexpr int S = 7;
  if ((reinterpret_cast<uintptr_t>(Y) & 15) != 0 || ((yld * 8) & 15) != 0 || yld < K)
    return (int)cudaErrorNotSupported;
  const size_t smem = (size_t)2 * (S * (A_TILE + B_TILE) + C64_TILE) + 1024;
  if (smem > dev->smem_optin) return (int)cudaErrorNotSupported;
  const int MT = (M + TM - 1) / TM, NTL = (N + TN - 1) / TN, KB = (K + TK - 1) / TK;
  int Z = 1;
  if (ws != nullptr) Z = choose_split((long long)MT * NTL, KB, M, N, ws_elems, dev->num_sms);
  int kb_per_z = (KB + Z - 1) / Z;
  kb_per_z = (kb_per_z + KB_PER_DRAIN - 1) / KB_PER_DRAIN * KB_PER_DRAIN;
  Z = (KB + kb_per_z - 1) / kb_per_z;
  OzkArgs a;
  a.A = static_cast<const uint8_t*>(Atiles);
  a.B = nullptr;
  a.ea = ea;
  a.eb = nullptr;
  a.eb_raw = raw;
  a.M = M;
  a.N = N;
  a.S = S;
  a.KB = KB;
  a.kb_per_z = kb_per_z;
  a.mode = 0;
  a.sign = sign;
  a.err = err;
  a.spin_limit = spin_limit;
  a.colexp = nullptr;
  a.row_lo = 0;
  a.stages = 2;
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
  CUtensorMap tmA, tmC;
  int rc = make_digit_map(&tmA, Atiles, M, K, S, TM);
  if (rc) return rc;
  {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (encode == nullptr) {
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult q;
      cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                       cudaEnableDefault, &q);
      if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || fn == nullptr)
        return (int)cudaErrorNotSupported;
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)N};
    const cuuint64_t strides[1] = {(cuuint64_t)yld * 8};
    const cuuint32_t box[2] = {(cuuint32_t)TK, (cuuint32_t)TN};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(&tmC, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(Y), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return (int)cudaErrorNotSupported;
  }
  cudaError_t e = cudaFuncSetAttribute(ozk_gemm_c64_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  hq_launch(ozk_gemm_c64_kernel, dim3(MT, NTL, Z), NT, smem, stream, a, tmA, tmC);
  hq_count_launches(1);
  if (Z > 1) {
    long long total = (long long)M * N;
    int blocks = (int)((total + 255) / 256);
    if (blocks > dev->num_sms * 8) blocks = dev->num_sms * 8;
    hq_launch(ozk_sum_slices, blocks, 256, 0, stream, M, N, Z, ws, C, crs, ccs, 0);
    hq_count_launches(1);
  }
  return (int)cudaGetLastError();
}

// Short products (K <= 256): the persistent kernel; B must be split with side
// 2 (TN_SHORT-row tiles).
extern "C" int hq_ozk_short_ok(int K) { return K > 0 && K <= KB_PER_DRAIN * TK; }

extern "C" int hq_ozk_gemm_short(cudaStream_t stream, const hq_device_info* dev, int M, int N,
                                 int K, int S, const void* Atiles, const int* ea,
                                 const void* Btiles, const int* eb, int mode, double sign,
                                 double* C, long long crs, long long ccs, int* colexp, int row_lo,
                                 int* err, unsigned spin_limit) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  if (S < 1 || S > 7 || !hq_ozk_short_ok(K)) return (int)cudaErrorInvalidValue;
  constexpr int TNV = TN_SHORT;
  OzkArgs a;
  a.A = static_cast<const uint8_t*>(Atiles);
  a.B = static_cast<const uint8_t*>(Btiles);
  a.ea = ea;
  a.eb = eb;
  a.M = M;
  a.N = N;
  a.S = S;
  a.KB = (K + TK - 1) / TK;
  a.kb_per_z = a.KB;
  a.mode = mode;
  a.sign = sign;
  a.err = err;
  a.spin_limit = spin_limit;
  a.C = C;
  a.crs = crs;
  a.ccs = ccs;
  a.zstride = 0;
  a.colexp = mode == 1 ? colexp : nullptr;
  a.row_lo = row_lo;
  a.eb_raw = nullptr;
  const size_t per_stage = (size_t)S * (A_TILE + B_TILE);
  int stages = MAX_STAGES;
  while (stages > 2 && (size_t)stages * per_stage + 1024 > dev->smem_optin) --stages;
  const size_t smem = (size_t)stages * per_stage + 1024;
  if (smem > dev->smem_optin) return (int)cudaErrorInvalidValue;
  a.stages = stages;
  CUtensorMap tmA, tmB;
  int rc = make_digit_map(&tmA, Atiles, M, K, S, TM);
  if (rc == 0) rc = make_digit_map(&tmB, Btiles, N, K, S, TNV);
  if (rc) return rc;
  cudaError_t e = cudaFuncSetAttribute(ozk_gemm_short_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  const long long tiles = (long long)((M + TM - 1) / TM) * ((N + TNV - 1) / TNV);
  const int grid = (int)(tiles < dev->num_sms ? tiles : dev->num_sms);
  hq_launch(ozk_gemm_short_kernel, grid, NT, smem, stream, a, tmA, tmB);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}
