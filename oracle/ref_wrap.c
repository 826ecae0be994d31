/*
 * ref_wrap.c -- compiles the UNMODIFIED reference source into oracle/_ref/.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle/build.py).  The reference file is found
 * on the include path (-I<reference>/lapack_compatible_sources); its LAPACK /
 * BLAS calls are mapped onto scipy's prefixed OpenBLAS with -D<name>_=scipy_<name>_.
 * One helper is added: the sketch the reference draws on entry, which is a
 * file-static function in the reference and so cannot be called from outside.
 */
#include "NoFLA_HQRRP_WY_blk_var4.c"

void oracle_reference_sketch(int mY, int m, double* G) {
  srand(12);
  NoFLA_Normal_random_matrix(mY, m, G, mY);
}
