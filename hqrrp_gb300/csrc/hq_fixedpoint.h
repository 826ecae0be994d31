/* hq_fixedpoint.h -- exact fixed-point sums of FP64 partials (host + device).
 *
 * The pivoted panel kernel sums, per column and stage, one FP64 partial dot
 * product from every CTA.  Each partial t becomes the integer V = t / 2^ue
 * (truncated), split into three 48-bit limbs that are added to three signed
 * 64-bit words; the 16 spare bits of each word absorb the carries of up to
 * 2^15 addends.  Integer addition is associative, so the words end up the
 * same whatever order the addends arrive in, and the sum is exact up to the
 * truncation of each addend below 2^ue.
 *
 * ue comes from a bound B on the sum's magnitude (for dot products, the two
 * columns' norms: Cauchy-Schwarz bounds every CTA's partial and their sum)
 * with 2^8 of slack: |V| < 2^133, so a single addend spans at most 53 bits
 * at bit positions below 134, and the truncation is 2^-133 of B.
 *
 * The functions here are pure arithmetic; the kernel adds the limbs with L2
 * atomics and reads the words back.  A CPU test drives the same code.
 */
#ifndef HQ_FIXEDPOINT_H
#define HQ_FIXEDPOINT_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define HQ_FX_HD __host__ __device__ __forceinline__
#else
#define HQ_FX_HD static inline
#endif

#define HQ_FX_MARGIN 8 /* bound slack 2^8 */
#define HQ_FX_MASK ((1ull << 48) - 1)

HQ_FX_HD long long hq_fx_bits(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  long long b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}

HQ_FX_HD double hq_fx_double(long long b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}

/* e(x) with 0 <= x < 2^e(x) for finite x >= 0 (zero and subnormals: 2^-1022). */
HQ_FX_HD int hq_fx_exp(double x) {
  const int b = (int)((hq_fx_bits(x) >> 52) & 0x7FF);
  return b == 0 ? -1022 : b - 1022;
}

/* Unit exponent for a sum bounded by sqrt(ep * ek) (sq != 0: ep, ek are
 * squared norms) or by ep * ek (norms). */
HQ_FX_HD int hq_fx_unit(double ep, double ek, int sq) {
  const int e = sq ? (hq_fx_exp(ep) + hq_fx_exp(ek) + 1) >> 1 : hq_fx_exp(ep) + hq_fx_exp(ek);
  return e + HQ_FX_MARGIN - 141;
}

/* The limbs of t / 2^ue: returns 0 (nothing to add: zero, subnormal or below
 * the unit), 1 (add p[0..2] to words *first .. *first + 2; limbs past word 2
 * are zero) or 2 (non-finite, or beyond the bound: count it as non-finite). */
HQ_FX_HD int hq_fx_split(double t, int ue, unsigned long long p[3], int* first) {
  const long long bits = hq_fx_bits(t);
  const int ex = (int)((bits >> 52) & 0x7FF);
  if (ex == 0x7FF) return 2;
  if (ex == 0) return 0;
  const unsigned long long mant = (unsigned long long)(bits & 0xFFFFFFFFFFFFFLL) | (1ull << 52);
  const int sh = ex - 1075 - ue; /* t = mant * 2^sh units */
  unsigned long long M;
  int s0;
  if (sh >= 0) {
    M = mant;
    s0 = sh;
  } else if (sh > -53) {
    M = mant >> (-sh);
    s0 = 0;
  } else {
    return 0;
  }
  if (s0 > 91) return 2; /* beyond the bound: only from non-finite norms */
  const int L = s0 / 48, off = s0 - 48 * L; /* M * 2^off spans limbs L..L+2 */
  p[0] = (M << off) & HQ_FX_MASK;
  p[1] = (M >> (48 - off)) & HQ_FX_MASK;
  p[2] = (96 - off) < 64 ? (M >> (96 - off)) : 0ull;
  if (bits < 0) {
    p[0] = 0ull - p[0];
    p[1] = 0ull - p[1];
    p[2] = 0ull - p[2];
  }
  *first = L;
  return 1;
}

/* The value of the summed words (carries normalised in integers, then two
 * FMAs: within an ulp of the exact sum). */
HQ_FX_HD double hq_fx_combine(long long l0, long long l1, long long l2, int ue) {
  long long c = l0 >> 48; /* arithmetic shift: floor */
  l0 -= c * (1LL << 48);
  l1 += c;
  c = l1 >> 48;
  l1 -= c * (1LL << 48);
  l2 += c;
  const double two48 = 281474976710656.0;
  const double hi = fma((double)l2, two48, (double)l1);
  return scalbn(fma(hi, two48, (double)l0), ue);
}

#endif /* HQ_FIXEDPOINT_H */
