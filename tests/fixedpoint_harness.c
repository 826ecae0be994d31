/* CPU driver of hqrrp_gb300/csrc/hq_fixedpoint.h for tests/test_fixedpoint.py:
 * the fixed-point sum the panel kernel forms with L2 atomics, formed here by
 * plain 64-bit additions of the same limbs (integer addition, so the order
 * of the addends does not matter). */
#include "hq_fixedpoint.h"

double hq_test_fx_sum(const double* parts, int n, double ep, double ek, int sq) {
  unsigned long long w[4] = {0, 0, 0, 0};
  const int ue = hq_fx_unit(ep, ek, sq);
  for (int i = 0; i < n; ++i) {
    unsigned long long p[3];
    int L = 0;
    const int rc = hq_fx_split(parts[i], ue, p, &L);
    if (rc == 2) {
      w[3] += 1;
    } else if (rc == 1) {
      for (int q = 0; q < 3; ++q)
        if (L + q < 3) w[L + q] += p[q];
    }
  }
  if (w[3]) return hq_fx_double(0x7FF8000000000000LL);
  return hq_fx_combine((long long)w[0], (long long)w[1], (long long)w[2], ue);
}
