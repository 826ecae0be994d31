"""The UT-transform variant (FLA_HQRRP_UT_blk_var2, the reference's libflame
implementation: libflame_sources/FLA_HQRRP_UT_blk_var2.c:124-401) on the GPU,
through its object API (hqrrp_gb300_ut_blk_var2), against the oracle's
restatement of that variant fed the same sketch: p identical, the factored
matrix within 1e-12 relative per column, s (the UT scalars) within 1e-12.
The restatement is itself checked against the reference-pinned WY
restatement in tests/test_oracle.py (libflame is not available to compile
the variant directly)."""
import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _col_rel(X, Xref):
    den = np.linalg.norm(Xref, axis=0)
    den[den == 0] = 1.0
    return float(np.max(np.linalg.norm(X - Xref, axis=0) / den))


def _check(got, want):
    Ag, pg, sg = got
    Ao, po, so = want
    np.testing.assert_array_equal(pg, po)
    assert np.max(np.abs(sg - so) / np.abs(so)) <= TOL
    assert _col_rel(Ag, Ao) <= TOL


@pytest.mark.parametrize("m,n,nb,pp,ppiv,seed", [
    (2000, 2000, 64, 10, 1, 1),   # square: the last reflector has an empty tail
    (1500, 700, 128, 10, 1, 2),   # tall
    (600, 1000, 64, 10, 1, 3),    # wide
    (777, 555, 50, 6, 1, 4),      # nb does not divide n
    (500, 400, 32, 10, 0, 5),     # unpivoted panels
    (40, 20, 64, 10, 1, 6),       # one block
])
def test_ut_variant_matches_oracle(hq, oracle_lib, m, n, nb, pp, ppiv, seed):
    A = oracle.gaussian(m, n, seed)
    G = oracle_lib.sketch(nb + pp, m)
    want = oracle_lib.hqrrp_ut(A, nb, pp, ppiv, G=G)
    got = hq.hqrrp_ut(A, nb, pp, ppiv, G=G)
    _check(got, want)


def test_ut_variant_zero_tail_reflectors(hq, oracle_lib):
    """Zero columns: when one becomes the pivot its tail is zero, and the UT
    transform's H = I - 2 e e^T applies (tau_UT = 1/2), not H = I."""
    m, n = 300, 260
    A = oracle.gaussian(m, n, 7)
    A[:, [5, 77, 140]] = 0.0
    G = oracle_lib.sketch(42, m)
    want = oracle_lib.hqrrp_ut(A, 32, 10, 1, G=G)
    got = hq.hqrrp_ut(A, 32, 10, 1, G=G)
    _check(got, want)
    assert np.sum(got[2] == 0.5) >= 3


def test_ut_variant_carries_labels_and_row_vector_views(hq, oracle_lib):
    """p carried like jpvt; p and s given as 1 x n row views with a stride."""
    m, n = 400, 300
    A = oracle.gaussian(m, n, 8)
    G = oracle_lib.sketch(42, m)
    labels = (np.arange(n, dtype=np.int32) * 7 + 3)[::-1].copy()
    want = oracle_lib.hqrrp_ut(A, 32, 10, 1, p=labels, G=G)
    L = hq.load()
    Af = np.array(A, order="F")
    pbuf = np.zeros(2 * n, np.int32)
    pbuf[::2] = labels
    sbuf = np.zeros(3 * min(m, n))
    oA = hq.Obj(hq.DOUBLE, m, n, m, Af.ctypes.data)
    op = hq.Obj(hq.INT, 1, n, 2, pbuf.ctypes.data)
    os_ = hq.Obj(hq.DOUBLE, 1, min(m, n), 3, sbuf.ctypes.data)
    Gf = np.array(G, order="F")
    rc = L.hqrrp_gb300_ut_blk_var2_sketch(oA, op, os_, 32, 10, 1,
                                          Gf.ctypes.data_as(C.POINTER(C.c_double)), 42)
    assert rc == 0, hq.last_error()
    assert np.all(pbuf[1::2] == 0) and np.all(sbuf[1::3] == 0) and np.all(sbuf[2::3] == 0)
    _check((Af, pbuf[::2], sbuf[::3]), want)


def test_ut_variant_rejects_bad_objects(hq):
    L = hq.load()
    A = np.zeros((10, 8), order="F")
    p = np.zeros(8, np.int32)
    s = np.zeros(8)
    oA = hq.Obj(hq.DOUBLE, 10, 8, 10, A.ctypes.data)
    bad_p = hq.Obj(hq.DOUBLE, 8, 1, 8, p.ctypes.data)   # wrong datatype
    os_ = hq.Obj(hq.DOUBLE, 8, 1, 8, s.ctypes.data)
    assert L.hqrrp_gb300_ut_blk_var2(oA, bad_p, os_, 4, 2, 1) == 3
    short_p = hq.Obj(hq.INT, 5, 1, 5, p.ctypes.data)    # fewer than n elements
    assert L.hqrrp_gb300_ut_blk_var2(oA, short_p, os_, 4, 2, 1) == 3


def test_ut_variant_mixed_precision_quality(hq):
    m = n = 1200
    sigma = 10.0 ** (-12.0 * np.arange(n) / n)
    A = oracle.with_spectrum(m, n, sigma, 9)
    prev = hq.set_precision(hq.MIXED)
    try:
        Af, p, s = hq.hqrrp_ut(A, 128, 10, 1)
    finally:
        hq.set_precision(prev)
    tau = 1.0 / s
    tau[s == 0.5] = 2.0
    res, orth, d = oracle.quality(A, Af, p, tau)
    assert res <= 1e-13 and orth <= 1e-12, (res, orth)
