// qrp_gram.cu -- the mixed-precision path's panel without a grid-wide
// reduction per column (sm_103a).
//
// The reference factors each block's panel column by column
// (NoFLA_QRPmod_WY_unb_var4, NoFLA_HQRRP_WY_blk_var4.c:774-886): every column
// needs the norms and dot products of the whole panel, which on a GPU is one
// grid-wide reduction and barrier per column.  Here a panel Ap (mp x b,
// b <= 128), pivoted within its b columns, is factored as
//   1. G = Ap^T Ap, a split-BF16 tensor-core product (FP64-accurate);
//   2. pivoted Cholesky of G, column-scaled to unit diagonal, in FP32 on one
//      SM: P and a preconditioner R1 with (Ap P)^T (Ap P) ~ R1^T R1.  The
//      Schur complement's diagonal holds the squared norms of the columns'
//      residuals, so taking the largest (first on ties) is the pivot rule of
//      column-pivoted Householder QR;
//   3. CholeskyQR2 (Fukaya, Nakatsukasa, Yanagisawa, Yamamoto, 2014), the
//      first pass preconditioned in FP32 (Yamazaki, Tomov, Dongarra, 2015):
//      Q1 = Ap P R1^{-1}, G2 = Q1^T Q1 = R2^T R2 with R2 in FP64,
//      Q = Q1 R2^{-1}, R = R2 R1; the FP64 second pass restores
//      orthogonality to working precision;
//   4. Householder reconstruction (Ballard, Demmel, Grigori, Jacquelin,
//      Nguyen, Solomonik, IPDPS 2014): the LU factorization without pivoting
//      Q - [D; 0] = V U, with D_kk = -sign of the k-th Schur pivot, gives the
//      unit lower trapezoidal V of Householder QR with LAPACK's sign choice
//      (beta = -sign(alpha) ||x||), tau_k = -D_kk U_kk, and R_H = D R.
// The steps over the panel's rows (G, Q1, G2, Q, V2 = Q2 U^{-1}) are
// tensor-core products issued by the host driver; the b x b steps are the
// kernels of this file.  FP64 runs at about two lanes per clock on a GB300
// SM, so one SM is slow for them: the FP64 Cholesky and LU run on a cluster
// of eight CTAs (each owns every eighth column; the pivot column travels
// through distributed shared memory), the triangular inverses and products
// with one CTA per column, and only the pivoted first pass on one SM, in
// FP32.
//
// A step that meets a panel it cannot factor accurately sets a bit in a
// status word: a first-pass pivot below 1e-5 of the column's own squared
// norm (the column lies within about 0.3 % of the span of the earlier ones:
// the panel is too ill-conditioned for an FP32 preconditioner), a
// second-pass pivot below 1e-10 of its diagonal entry (G2 far from the
// identity), or an LU pivot outside [0.5, 2.5] (|U_kk| = tau_k lies in
// [1, 2] for an orthonormal Q).  The commit kernel then leaves
// the panel untouched, and the cooperative pivoted panel kernel, which reads
// the same word, factors it instead.

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math.h>

#include "hq_common.cuh"
#include "hq_internal.h"

namespace cg = cooperative_groups;

namespace {

constexpr int GN = HQ_GRAM_MAX;  // widest panel
constexpr int LDS = GN + 1;      // shared-memory column stride of the b x b kernels
constexpr int CT = 512;          // threads of the one-SM kernels
constexpr int CW = CT / 32;
constexpr int TW = 4;            // warps per CTA of the triangular kernel (one column per CTA)
constexpr float PIVOT32_REL_MIN = 1e-5f;  // first pass: scaled pivot floor
constexpr double CHOL2_REL_MIN = 1e-10;   // cluster Cholesky: pivot floor, relative to the diagonal
constexpr double NEARID_MAX = 2e-4;       // second pass: largest max|G2 - I| it converges from
constexpr int NEARID_ITERS = 4;           // second pass: fixed-point steps
constexpr int CL = 8;                     // CTAs of the cluster kernels
constexpr int CLT = 256;                  // threads per CTA of the cluster kernels
constexpr int CLW = CLT / 32;
constexpr int OWN = GN / CL;              // columns per CTA (column j lives in CTA j % CL)
static_assert(OWN == 2 * CLW, "each warp of a cluster CTA updates two own columns");

// Pass 1: pivoted Cholesky of the n x n Gram matrix G (ldg) scaled to unit
// diagonal, in FP32 on one SM, the matrix held in registers.  Thread (warp
// w, lane t) holds the 32 entries (i, j) with i = t + 32 a (a < 4) and
// j = w + 16 c (c < 8) of the full symmetric matrix.  Columns are not moved:
// step k picks the active column p with the largest residual norm (scaled
// Schur diagonal times the column's original squared norm relative to the
// largest; the lowest index among residuals equal to 2^-15), the warp holding column p publishes
// l = S[:, p] / sqrt(S[p][p]) over the active rows (0 elsewhere), and every
// thread updates its entries by S_ij -= l_i l_j -- a no-op on eliminated
// rows and columns, so the update needs no masks.  Every warp finds the
// pivot itself (one warp maximum), so a step takes two barriers.
// Writes perm[k] (source column of position k) and R = Rs diag(sqrt(G_pp))
// in FP64 (upper, zeros below), Rs the scaled factor; *stat = 0, or `bit`
// with R = I and perm = identity when a scaled pivot is not above
// PIVOT32_REL_MIN; *alt (the second pass's choice of method) and *emax
// (its max|E|) := 0.
__global__ void __launch_bounds__(CT, 1)
    gram_pchol32_kernel(int n, const double* __restrict__ G, int ldg, double* __restrict__ R,
                        int ldr, int* __restrict__ perm, int* __restrict__ stat, int bit,
                        int* __restrict__ alt, unsigned long long* __restrict__ emax) {
  HQ_PDL_WAIT();
  extern __shared__ float s_Rp[];  // GN * GN: s_Rp[k * GN + i] = row k of Rs at source column i
  __shared__ double s_sc[GN], s_rt[GN];
  __shared__ float s_key[GN], s_d[GN], s_l[GN], s_r[GN], s_wmax[CW];
  __shared__ int s_ord[GN];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  static_assert(CT == 512 && GN == 128, "register layout: 16 warps x 32 lanes, 4 x 8 entries");
  for (int j = tid; j < GN; j += CT) {
    double d = 0.0;
    if (j < n) d = G[j + (size_t)j * ldg];
    const int ok = j < n && d > 0.0 && d <= 1.7e308;
    const double rt = ok ? sqrt(d) : 0.0;
    s_rt[j] = rt;
    s_sc[j] = ok ? 1.0 / rt : 0.0;
    s_key[j] = ok ? (float)log2(d) : -4096.0f;  // squared norm, scaled below
  }
  __syncthreads();
  if (warp == 0) {
    float m = -4096.0f;
    for (int j = lane; j < n; j += 32) m = fmaxf(m, s_key[j]);
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) s_wmax[0] = m;
  }
  __syncthreads();
  const float kmax = s_wmax[0];
  for (int j = tid; j < n; j += CT) s_key[j] = exp2f(s_key[j] - kmax);  // d_j / max d
  float S[4][8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int j = warp + 16 * c;
    double v[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int i = lane + 32 * a;
      v[a] = (i < n && j < n) ? G[i + (size_t)j * ldg] : 0.0;
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int i = lane + 32 * a;
      S[a][c] = (i < n && j < n) ? (float)(v[a] * s_sc[i] * s_sc[j]) : 0.0f;
      if (i == j) s_d[j] = S[a][c];
    }
  }
  __syncthreads();

  // Per lane: the keys and active flags of columns lane + 32 q.
  float keyr[4];
  int actr[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int j = lane + 32 * q;
    keyr[q] = j < n ? s_key[j] : 0.0f;
    actr[q] = j < n;
  }
  int fail = 0;
  for (int k = 0; k < n; ++k) {
    // Every warp finds the pivot: one 32-bit key per column, the residual's
    // FP32 bits above the low 8 (positive floats order like their bits) and
    // 255 - j below them, so one warp maximum gives the largest residual
    // and, among residuals equal to 2^-15, the lowest column.
    float dq[4];
    unsigned best = 0u;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = lane + 32 * q;
      dq[q] = s_d[j];
      if (actr[q]) {
        const float v = keyr[q] * dq[q];
        const unsigned vb = v > 0.0f ? __float_as_uint(v) : 0u;  // NaN and v <= 0: lowest
        best = max(best, (vb & ~255u) | (unsigned)(255 - j));
      }
    }
    best = __reduce_max_sync(0xffffffffu, best);
    const int p = best ? 255 - (int)(best & 255u) : 0;
    const int pq = p >> 5;
    float dsel = dq[0];
#pragma unroll
    for (int q = 1; q < 4; ++q)
      if (q == pq) dsel = dq[q];
    const float dp = __shfl_sync(0xffffffffu, dsel, p & 31);
    if (best == 0u || !(dp > PIVOT32_REL_MIN)) {  // also NaN and a zero column
      fail = 1;
      break;
    }
    if ((p & 31) == lane) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q == pq) actr[q] = 0;
    }
    const float r = sqrtf(dp);
    if (tid == 0) {
      s_r[k] = r;
      s_ord[k] = p;
    }
    // The warp holding column p publishes l over the active rows (row
    // lane + 32 a is this lane's column slot a: its flag is actr[a]).
    if (warp == (p & 15)) {
      const int cp = p >> 4;
      const float rinv = 1.0f / r;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        float v = S[a][0];
#pragma unroll
        for (int c = 1; c < 8; ++c)
          if (c == cp) v = S[a][c];
        const int i = lane + 32 * a;
        const float l = actr[a] ? v * rinv : 0.0f;
        s_l[i] = l;
        s_Rp[k * GN + i] = l;
      }
    }
    __syncthreads();
    float li[4], lj[8];
#pragma unroll
    for (int a = 0; a < 4; ++a) li[a] = s_l[lane + 32 * a];
#pragma unroll
    for (int c = 0; c < 8; ++c) lj[c] = s_l[warp + 16 * c];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 8; ++c) S[a][c] = fmaf(-li[a], lj[c], S[a][c]);
    // Diagonal entries: lane w + 16 h of warp w holds (i, i) for
    // i = lane + 32 a in slot c = 2 a + h.
    if ((lane & 15) == warp) {
      const int h = lane >> 4;
#pragma unroll
      for (int a = 0; a < 4; ++a) s_d[lane + 32 * a] = h ? S[a][2 * a + 1] : S[a][2 * a];
    }
    __syncthreads();
  }
  // R[k][m] = Rs[k][m] sqrt(G_pp), p = perm[m]: row k of Rs at source column p.
  for (int m = warp; m < n; m += CW)
    for (int k = lane; k < n; k += 32) {
      double v;
      if (fail)
        v = k == m ? 1.0 : 0.0;
      else if (k < m)
        v = (double)s_Rp[k * GN + s_ord[m]] * s_rt[s_ord[m]];
      else
        v = k == m ? (double)s_r[m] * s_rt[s_ord[m]] : 0.0;
      R[k + (size_t)m * ldr] = v;
    }
  for (int k = tid; k < n; k += CT) perm[k] = fail ? k : s_ord[k];
  if (tid == 0) {
    *stat = fail ? bit : 0;
    *alt = 0;
    *emax = 0ull;
  }
}

// Pivot scalars of a cluster factorization step, from the updated diagonal
// entry q of the pivot column (one thread): Cholesky (mode 0) r = sqrt(q),
// bad when q <= 1e-10 d0; LU (mode 1) D = -1 if q >= 0 else +1, u = q - D,
// bad when |u| is outside [0.5, 2.5].  A bad pivot is replaced by 1.
__device__ __forceinline__ void cluster_scalars(int mode, double q, double d0, double* out) {
  double piv, D = 0.0;
  int bad;
  if (mode == 0) {
    bad = !(q > CHOL2_REL_MIN * d0);
    piv = bad ? 1.0 : sqrt(q);
  } else {
    D = q >= 0.0 ? -1.0 : 1.0;
    const double u = q - D;
    const double au = fabs(u);
    bad = !(au >= 0.5 && au <= 2.5);
    piv = bad ? 1.0 : u;
  }
  out[0] = piv;
  // 1 / piv: an FP32 quotient refined by two Newton steps y += y (1 - piv y)
  // (2^-24 -> 2^-48 -> FP64 rounding), four dependent FMAs instead of the
  // longer FP64 division sequence on this critical path; piv lies in
  // [0.5, 2.5] (LU) or is a square root of a diagonal entry well inside
  // FP32's range (Cholesky of a scaled Gram matrix).
  double y = (double)(1.0f / (float)piv);
  y = fma(y, fma(-piv, y, 1.0), y);
  y = fma(y, fma(-piv, y, 1.0), y);
  out[1] = y;
  out[2] = D;
  out[3] = bad ? 1.0 : 0.0;
}

// Unpivoted FP64 factorization of an n x n matrix A (lda) on a cluster of CL
// CTAs:
//   mode 0: Cholesky of the symmetric A (lower triangle read); F := R (upper,
//           zeros below) with R^T R = A;
//   mode 1: LU of A - D, D_kk = -1 if the k-th Schur pivot is >= 0 else +1
//           (Householder reconstruction); F := L strictly below the diagonal
//           and U on and above it, dsgn := D, tau := -D U_kk.
// Column j lives in the shared memory of CTA j % CL.  Step k: every CTA
// updates its columns right of k from the published, scaled column k; the
// owner of column k + 1 updates that column first, takes its pivot scalars,
// scales it and writes it into every CTA's receive buffer (distributed
// shared memory, double-buffered by the parity of the step).  One cluster
// barrier per step, split into arrive and wait around the update of the
// remaining own columns; it also orders the receive buffers' reuse.  A bad
// pivot is recorded and replaced by 1, so every CTA takes the same barriers;
// the output is then the identity (and tau 0) and `bit` is set in *stat.
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(CLT, 1)
    cluster_fact_kernel(int n, int mode, const double* __restrict__ A, int lda,
                        double* __restrict__ F, int ldf, double* __restrict__ dsgn,
                        double* __restrict__ tau, int* __restrict__ stat, int bit,
                        const int* __restrict__ gate) {
  HQ_PDL_WAIT();
  if (gate != nullptr && *gate == 0) return;  // every CTA of the cluster reads the same word
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  __shared__ double Xc[OWN * LDS];
  __shared__ double colbuf[2][GN];
  __shared__ double scal[2][4];  // pivot, 1 / pivot, D, bad
  __shared__ double s_pub[4];
  __shared__ double s_d0[OWN], s_D[OWN];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nown = rank < n ? (n - 1 - rank) / CL + 1 : 0;
  for (int c = warp; c < nown; c += CLW) {
    const int j = rank + CL * c;
    double v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = lane + 32 * q;
      v[q] = (i < n && (mode == 1 || i >= j)) ? A[i + (size_t)j * lda] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = lane + 32 * q;
      if (i < n) Xc[i + c * LDS] = v[q];
    }
  }
  __syncthreads();
  for (int c = tid; c < nown; c += CLT) s_d0[c] = Xc[(rank + CL * c) + c * LDS];

  // Publish own column kk (local c): scalars, final diagonal, scaled rows
  // below it, into every CTA's buffers of parity par.  Thread 0 wrote the
  // column's diagonal entry itself (it updates row kk), so it takes the
  // scalars before the barrier that orders the other rows' updates.
  auto publish = [&](int kk, int par) {
    const int c = kk / CL;
    if (tid == 0) {
      cluster_scalars(mode, Xc[kk + c * LDS], s_d0[c], s_pub);
      Xc[kk + c * LDS] = s_pub[0];
      s_D[c] = s_pub[2];
    }
    __syncthreads();
    const double inv = s_pub[1];
    for (int i = kk + 1 + tid; i < n; i += CLT) {
      const double l = Xc[i + c * LDS] * inv;
      Xc[i + c * LDS] = l;
#pragma unroll
      for (int r = 0; r < CL; ++r) *cl.map_shared_rank(&colbuf[par][i], r) = l;
    }
    if (tid < CL) {
      double* d = cl.map_shared_rank(&scal[par][0], tid);
      d[0] = s_pub[0];
      d[1] = s_pub[1];
      d[2] = s_pub[2];
      d[3] = s_pub[3];
    }
  };

  if (rank == 0 && n > 0) publish(0, 0);
  cl.sync();
  int bad = 0;
  for (int k = 0; k < n; ++k) {
    const int b = k & 1;
    const int nx = k + 1;
    if (nx < n && nx % CL == rank) {
      const int c1 = nx / CL;
      if (mode == 1) {
        const double ukj = Xc[k + c1 * LDS];
        for (int i = k + 1 + tid; i < n; i += CLT) Xc[i + c1 * LDS] -= colbuf[b][i] * ukj;
      } else {
        const double lj = colbuf[b][nx];
        for (int i = nx + tid; i < n; i += CLT) Xc[i + c1 * LDS] -= colbuf[b][i] * lj;
      }
      publish(nx, b ^ 1);
    }
    // The other own columns right of k: warp w takes local columns w and
    // w + CLW together, their four row chunks unrolled.  Everything read
    // from the receive buffer is in registers before this CTA arrives at the
    // step's barrier (after which the buffer may be refilled two steps on),
    // so the barrier's latency overlaps the update; the wait comes last.
    {
      double xa[2][4], lb[2][4], mult[2];
      int act[2], base[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int c = warp + CLW * u, j = rank + CL * c;
        act[u] = c < nown && j > k && j != nx;
        mult[u] = act[u] ? (mode == 1 ? Xc[k + c * LDS] : colbuf[b][j]) : 0.0;
        base[u] = mode == 1 ? k + 1 : j;
      }
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int c = warp + CLW * u, i = base[u] + lane + 32 * q;
          const int live = act[u] && i < n;
          xa[u][q] = live ? Xc[i + c * LDS] : 0.0;
          lb[u][q] = live ? colbuf[b][i] : 0.0;
        }
      bad |= scal[b][3] != 0.0;
      cl.barrier_arrive();
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int c = warp + CLW * u, i = base[u] + lane + 32 * q;
          if (act[u] && i < n) Xc[i + c * LDS] = xa[u][q] - lb[u][q] * mult[u];
        }
    }
    __syncthreads();  // the CTA's own updates (after its arrive) before the next step reads them
    cl.barrier_wait();
  }
  // Output of the own columns.
  for (int c = warp; c < nown; c += CLW) {
    const int g = rank + CL * c;
    for (int i = lane; i < n; i += 32) {
      const double x = Xc[i + c * LDS];
      if (mode == 1) {
        F[i + (size_t)g * ldf] = bad ? (i == g ? 1.0 : 0.0) : x;
      } else if (i >= g) {
        // R[g][i] = L[i][g]; R[i][g] = 0 below the diagonal
        F[g + (size_t)i * ldf] = bad ? (i == g ? 1.0 : 0.0) : x;
        if (i > g) F[i + (size_t)g * ldf] = 0.0;
      }
    }
  }
  if (mode == 1)
    for (int c = tid; c < nown; c += CLT) {
      const int g = rank + CL * c;
      dsgn[g] = bad ? -1.0 : s_D[c];
      tau[g] = bad ? 0.0 : -s_D[c] * Xc[g + c * LDS];
    }
  if (bad && rank == 0 && tid == 0) atomicOr(stat, bit);
}

// E_ij (i <= j) of G = I + E, read from G's upper triangle (column j is
// contiguous: coalesced loads).
__device__ __forceinline__ double e_upper(const double* __restrict__ G, int ldg, int i, int j) {
  const double g = G[i + (size_t)j * ldg];
  return i < j ? g : g - 1.0;
}

// Fixed-point steps the second pass needs from max|E|: the error of R^{-1}
// after m steps is about max|E|^(m+1) (measured on FP32-preconditioned
// panels), below 2^-53 after 2 steps up to 4e-6, 3 up to 5e-5, 4 up to
// NEARID_MAX.
__device__ __forceinline__ int nearid_steps(double emax) {
  return emax <= 4e-6 ? 2 : (emax <= 5e-5 ? 3 : NEARID_ITERS);
}

// One step of the second CholeskyQR pass for G = I + E near the identity:
// R2 = I + X (X upper with its diagonal) and R2^{-1} = I + Z are the fixed
// points of
//   X <- Uh(E - X^T X),   Z <- -X (I + Z),
// Uh = strict upper part plus half the diagonal (X + X^T + X^T X = E is
// R2^T R2 = G).  Both converge linearly at a rate of about ||E||_2, so
// NEARID_ITERS steps from X = Uh(E), Z = -X reach working precision when
// max|E| <= NEARID_MAX (first pass in FP32: max|E| ~ 1e-6 .. 1e-4 for
// panels with condition numbers 10 .. 300); fewer suffice for smaller
// max|E| (nearid_steps), and the later launches then only copy.  Every product is a column of a
// b x b product, so the pass needs no sequential factorization: one CTA per
// column c stages X's columns 0..c and each thread accumulates one row.
// Step 0: X, Z are Uh(E), -Uh(E) (Xin, Zin unused), and the CTA checks its
// column of E against NEARID_MAX, setting *alt when it is exceeded (the
// later steps then return at once and the cluster Cholesky and a triangular
// inverse, gated on *alt, take the pass) and raising *emax; the last step
// writes I + X and I + Z.
__global__ void __launch_bounds__(TW * 32)
    nearid_kernel(int n, const double* __restrict__ G, int ldg, const double* __restrict__ Xin,
                  const double* __restrict__ Zin, int ld, double* __restrict__ Xout,
                  double* __restrict__ Zout, int it, int* __restrict__ alt,
                  unsigned long long* __restrict__ emax) {
  HQ_PDL_WAIT();
  extern __shared__ double sX[];  // LDS * n: X's columns 0..c, rows <= column
  __shared__ double s_z[GN];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c = blockIdx.x;
  const int first = it == 0, last = it == NEARID_ITERS - 1;
  if (!first) {
    if (*alt != 0) return;  // too far from the identity: the cluster Cholesky runs
    if (it >= nearid_steps(__longlong_as_double((long long)*emax))) {
      // converged: pass X and Z through (adding I after the last step)
      for (int i = tid; i < n; i += TW * 32) {
        const double d = (last && i == c) ? 1.0 : 0.0;
        Xout[i + (size_t)c * ld] = Xin[i + (size_t)c * ld] + d;
        Zout[i + (size_t)c * ld] = Zin[i + (size_t)c * ld] + d;
      }
      return;
    }
  }
  for (int j0 = 4 * warp; j0 <= c; j0 += 4 * TW) {
    double v[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = j0 + a, i = lane + 32 * q;
        double x = 0.0;
        if (j <= c && i <= j) {
          if (first) {
            const double e = e_upper(G, ldg, i, j);
            x = i < j ? e : 0.5 * e;
          } else {
            x = Xin[i + (size_t)j * ld];
          }
        }
        v[a][q] = x;
      }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = j0 + a, i = lane + 32 * q;
        if (j <= c && i <= j) sX[i + j * LDS] = v[a][q];
      }
  }
  for (int k = tid; k <= c; k += TW * 32) {
    if (first) {
      const double e = e_upper(G, ldg, k, c);
      s_z[k] = -(k < c ? e : 0.5 * e);
      const double ae = fabs(e);
      if (!(ae <= NEARID_MAX)) atomicOr(alt, 1);  // also NaN
      // non-negative doubles order like their bits
      else atomicMax(emax, (unsigned long long)__double_as_longlong(ae));
    } else {
      s_z[k] = Zin[k + (size_t)c * ld];
    }
  }
  __syncthreads();
  for (int i = tid; i < n; i += TW * 32) {
    double xn = 0.0, zn = 0.0;
    if (i <= c) {
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      int k = 0;
      for (; k + 3 <= i; k += 4) {
        a0 = fma(sX[k + i * LDS], sX[k + c * LDS], a0);
        a1 = fma(sX[k + 1 + i * LDS], sX[k + 1 + c * LDS], a1);
        a2 = fma(sX[k + 2 + i * LDS], sX[k + 2 + c * LDS], a2);
        a3 = fma(sX[k + 3 + i * LDS], sX[k + 3 + c * LDS], a3);
      }
      for (; k <= i; ++k) a0 = fma(sX[k + i * LDS], sX[k + c * LDS], a0);
      const double e = e_upper(G, ldg, i, c);
      const double r = e - ((a0 + a1) + (a2 + a3));
      xn = i < c ? r : 0.5 * r;
      double b0 = 0.0, b1 = 0.0, b2 = 0.0, b3 = 0.0;
      k = i;
      for (; k + 3 <= c; k += 4) {
        b0 = fma(sX[i + k * LDS], s_z[k], b0);
        b1 = fma(sX[i + (k + 1) * LDS], s_z[k + 1], b1);
        b2 = fma(sX[i + (k + 2) * LDS], s_z[k + 2], b2);
        b3 = fma(sX[i + (k + 3) * LDS], s_z[k + 3], b3);
      }
      for (; k <= c; ++k) b0 = fma(sX[i + k * LDS], s_z[k], b0);
      zn = -sX[i + c * LDS] - ((b0 + b1) + (b2 + b3));
      if (last && i == c) {
        xn += 1.0;
        zn += 1.0;
      }
    }
    Xout[i + (size_t)c * ld] = xn;
    Zout[i + (size_t)c * ld] = zn;
  }
}

// One triangular job: X = A^{-1} (mode 0) or X = diag(rs) A B (mode 1; rs
// may be null), A and B upper triangular n x n (only their upper triangles
// are read), X upper triangular with zeros below.
struct TriJob {
  int mode;
  const double* A;
  int lda;
  const double* B;
  int ldb;
  const double* rs;
  double* X;
  int ldx;
};

// One CTA per column c of X (and per job: blocks [0, n) run j0, [n, 2n)
// j1): its warps stage A's columns 0..c in shared memory, then warp 0
// computes the column with its entries in four registers per lane (rows
// lane + 32 q) -- the inverse as a back substitution of axpys, the product
// as rank-1 column updates.  One column per SM keeps each SM's narrow FP64
// pipe on one dependent chain.
__global__ void __launch_bounds__(TW * 32)
    tri_kernel(int n, TriJob j0, TriJob j1, const int* __restrict__ gate) {
  HQ_PDL_WAIT();
  extern __shared__ double sA[];  // LDS * n
  __shared__ double s_dinv[GN];
  if (gate != nullptr && *gate == 0) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const TriJob J = blockIdx.x < (unsigned)n ? j0 : j1;
  const int c = (int)(blockIdx.x % (unsigned)n);
  const int mode = J.mode, lda = J.lda, ldb = J.ldb, ldx = J.ldx;
  const double* __restrict__ A = J.A;
  const double* __restrict__ B = J.B;
  const double* __restrict__ rs = J.rs;
  double* __restrict__ X = J.X;
  // Stage A's columns 0..c, four columns per warp at a time (16 loads in
  // flight per lane).
  for (int j0 = 4 * warp; j0 <= c; j0 += 4 * TW) {
    double v[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = j0 + a, i = lane + 32 * q;
        v[a][q] = (j <= c && i <= j) ? A[i + (size_t)j * lda] : 0.0;
      }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = j0 + a, i = lane + 32 * q;
        if (j <= c && i <= j) sA[i + j * LDS] = v[a][q];
      }
  }
  if (mode == 0)
    for (int i = tid; i <= c; i += TW * 32) s_dinv[i] = 1.0 / A[i + (size_t)i * lda];
  __syncthreads();
  if (warp != 0) return;
  double t[4];
  if (mode == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) t[q] = (lane + 32 * q == c) ? 1.0 : 0.0;
    for (int k = c; k >= 0; --k) {
      const int sq = k >> 5, sl = k & 31;
      double tk = t[0];
#pragma unroll
      for (int q = 1; q < 4; ++q)
        if (q == sq) tk = t[q];
      const double xk = __shfl_sync(0xffffffffu, tk, sl) * s_dinv[k];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = lane + 32 * q;
        if (q == sq && lane == sl)
          t[q] = xk;
        else if (32 * q < k && i < k)
          t[q] -= sA[i + k * LDS] * xk;
      }
    }
  } else {
    double bc[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = lane + 32 * q;
      bc[q] = (i <= c) ? B[i + (size_t)c * ldb] : 0.0;
      t[q] = 0.0;
    }
    for (int k = 0; k <= c; ++k) {
      const int sq = k >> 5, sl = k & 31;
      double bk = bc[0];
#pragma unroll
      for (int q = 1; q < 4; ++q)
        if (q == sq) bk = bc[q];
      bk = __shfl_sync(0xffffffffu, bk, sl);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = lane + 32 * q;
        if (32 * q <= k && i <= k) t[q] += sA[i + k * LDS] * bk;
      }
    }
    if (rs) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = lane + 32 * q;
        if (i <= c) t[q] *= rs[i];
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = lane + 32 * q;
    if (i < n) X[i + (size_t)c * ldx] = (i <= c) ? t[q] : 0.0;
  }
}

// When *stat == 0: the panel P (mp x n, ldp) gets R on and above the
// diagonal and the Householder vectors below it (L's strict lower part in
// the top n rows, V2 below from U's rows >= n, where the V2 product wrote
// them); U's top n rows become the explicit unit-lower V1; tau and the
// panel permutation (identity: the Gram path's pivots were applied to the
// columns before the products) are written.  Otherwise nothing.
__global__ void gram_commit_kernel(int mp, int n, double* __restrict__ P, int ldp,
                                   double* __restrict__ U, int ldu, const double* __restrict__ RH,
                                   int ldr, const double* __restrict__ LU, int ldlu,
                                   const double* __restrict__ tau_in, double* __restrict__ tau,
                                   int* __restrict__ perm, const int* __restrict__ stat,
                                   int* __restrict__ count) {
  HQ_PDL_WAIT();
  const int st = *stat;
  if (count != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0)
    atomicAdd(&count[st != 0 ? 1 : 0], 1);
  if (st != 0) return;
  const int k = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < mp; i += gridDim.x * blockDim.x) {
    double pv;
    if (i < n) {
      double uv;
      if (i < k) {
        pv = RH[i + (size_t)k * ldr];
        uv = 0.0;
      } else if (i == k) {
        pv = RH[i + (size_t)k * ldr];
        uv = 1.0;
      } else {
        pv = LU[i + (size_t)k * ldlu];
        uv = pv;
      }
      U[i + (size_t)k * ldu] = uv;
    } else {
      pv = U[i + (size_t)k * ldu];
    }
    P[i + (size_t)k * ldp] = pv;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    tau[k] = tau_in[k];
    perm[k] = k;
  }
}

}  // namespace

extern "C" int hq_gram_pchol32(cudaStream_t stream, int n, const double* G, int ldg, double* R,
                               int ldr, int* perm, int* stat, int bit, int* alt,
                               unsigned long long* emax) {
  if (n <= 0 || n > GN) return (int)cudaErrorInvalidValue;
  const size_t smem = sizeof(float) * (size_t)GN * GN;
  cudaError_t e = cudaFuncSetAttribute(gram_pchol32_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  hq_launch(gram_pchol32_kernel, 1, CT, smem, stream, n, G, ldg, R, ldr, perm, stat, bit, alt,
                                                emax);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_cluster_fact(cudaStream_t stream, int n, int mode, const double* A, int lda,
                               double* F, int ldf, double* dsgn, double* tau, int* stat, int bit,
                               const int* gate) {
  if (n <= 0 || n > GN || mode < 0 || mode > 1) return (int)cudaErrorInvalidValue;
  hq_launch(cluster_fact_kernel, CL, CLT, 0, stream, n, mode, A, lda, F, ldf, dsgn, tau, stat, bit,
                                              gate);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_nearid_chol(cudaStream_t stream, int n, const double* G, int ldg, double* R,
                              double* Rinv, double* wX, double* wZ, int ld, int* alt,
                              unsigned long long* emax) {
  if (n <= 0 || n > GN) return (int)cudaErrorInvalidValue;
  const size_t smem = sizeof(double) * (size_t)LDS * (size_t)n;
  cudaError_t e =
      cudaFuncSetAttribute(nearid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  static_assert(NEARID_ITERS % 2 == 0, "the last step writes R and Rinv");
  for (int it = 0; it < NEARID_ITERS; ++it) {
    // ping-pong: odd steps write the work pair, even steps the output pair
    const double* xi = (it & 1) ? wX : R;
    const double* zi = (it & 1) ? wZ : Rinv;
    double* xo = (it & 1) ? R : wX;
    double* zo = (it & 1) ? Rinv : wZ;
    hq_launch(nearid_kernel, n, TW * 32, smem, stream, n, G, ldg, xi, zi, ld, xo, zo, it, alt, emax);
  }
  hq_count_launches(NEARID_ITERS);
  return (int)cudaGetLastError();
}

extern "C" int hq_tri(cudaStream_t stream, int n, int mode, const double* A, int lda,
                      const double* B, int ldb, const double* rs, double* X, int ldx,
                      const int* gate) {
  return hq_tri2g(stream, n, mode, A, lda, B, ldb, rs, X, ldx, -1, nullptr, 0, nullptr, 0,
                  nullptr, nullptr, 0, gate);
}

extern "C" int hq_tri2(cudaStream_t stream, int n, int mode0, const double* A0, int lda0,
                       const double* B0, int ldb0, const double* rs0, double* X0, int ldx0,
                       int mode1, const double* A1, int lda1, const double* B1, int ldb1,
                       const double* rs1, double* X1, int ldx1) {
  return hq_tri2g(stream, n, mode0, A0, lda0, B0, ldb0, rs0, X0, ldx0, mode1, A1, lda1, B1, ldb1,
                  rs1, X1, ldx1, nullptr);
}

extern "C" int hq_tri2g(cudaStream_t stream, int n, int mode0, const double* A0, int lda0,
                        const double* B0, int ldb0, const double* rs0, double* X0, int ldx0,
                        int mode1, const double* A1, int lda1, const double* B1, int ldb1,
                        const double* rs1, double* X1, int ldx1, const int* gate) {
  if (n <= 0) return 0;
  if (n > GN || mode0 < 0 || mode0 > 1 || mode1 < -1 || mode1 > 1)
    return (int)cudaErrorInvalidValue;
  const size_t smem = sizeof(double) * (size_t)LDS * (size_t)n;
  cudaError_t e =
      cudaFuncSetAttribute(tri_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  const TriJob j0 = {mode0, A0, lda0, B0, ldb0, rs0, X0, ldx0};
  const TriJob j1 = {mode1 < 0 ? 0 : mode1, A1, lda1, B1, ldb1, rs1, X1, ldx1};
  hq_launch(tri_kernel, mode1 < 0 ? n : 2 * n, TW * 32, smem, stream, n, j0, j1, gate);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int hq_gram_commit(cudaStream_t stream, int mp, int n, double* P, int ldp, double* U,
                              int ldu, const double* RH, int ldr, const double* LU, int ldlu,
                              const double* tau_in, double* tau, int* perm, const int* stat,
                              int* count) {
  if (mp <= 0 || n <= 0) return 0;
  int bx = (mp + 255) / 256;
  if (bx > 64) bx = 64;
  hq_launch(gram_commit_kernel, dim3(bx, n), 256, 0, stream, mp, n, P, ldp, U, ldu, RH, ldr, LU, ldlu,
                                                      tau_in, tau, perm, stat, count);
  hq_count_launches(1);
  return (int)cudaGetLastError();
}
