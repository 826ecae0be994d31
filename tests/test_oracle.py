"""The oracle (CPU restatement of the reference) is pinned to the reference.

Two pins: (1) against the golden fixtures, which hold what the unmodified
reference returned for seeded inputs (tests/golden/make_golden.py); (2) where
the reference tree is present, against the reference compiled here, bit for
bit.  Only after these pass is the oracle used to check the GPU library.
"""
import numpy as np
import pytest

import oracle
import golden_cases as gc

# Same LAPACK here: results are bit-identical.  On another build of
# OpenBLAS (the aarch64 GPU host) only rounding may differ.
RTOL = 1e-12


@pytest.mark.parametrize("name", sorted(gc.CASES))
def test_oracle_matches_reference_golden(oracle_lib, name):
    kind, m, n, seed, nb, pp, ppiv, fixed, full = gc.CASES[name]
    A, jp, same_input = gc.case_input(name)
    if not same_input:
        pytest.skip("numpy's generator no longer reproduces the fixture input")
    g = gc.load(name)
    if kind == "hqrrp":
        Af, jpvt, tau = oracle_lib.hqrrp(A, nb, pp, ppiv)
    else:
        Af, jpvt, tau, info, work0 = oracle_lib.dgeqp4(A, jp)
        assert info == int(g["info"])
        if min(m, n) >= 250:  # dgeqpf leaves a norm in work[0]
            assert work0 == float(g["work0"])
    s = gc.summary(Af, jpvt, tau, m, n)
    np.testing.assert_array_equal(s["jpvt"], g["jpvt"])
    for key in ("tau", "diag", "aw", "atu"):
        assert gc.rel(s[key], g[key]) <= RTOL, key
    if "af" in g:
        assert gc.rel(Af, g["af"]) <= RTOL


def test_oracle_demo_7x5(oracle_lib):
    g = gc.load("dgeqp4_demo_7x5")
    Af, jpvt, tau, info, _ = oracle_lib.dgeqp4(g["a"], g["jpvt_in"])
    assert info == 0
    np.testing.assert_array_equal(jpvt, g["jpvt"])
    assert gc.rel(tau, g["tau"]) <= RTOL and gc.rel(Af, g["af"]) <= RTOL


def test_oracle_sketch_is_the_reference_sketch(oracle_lib):
    g = gc.load("sketch_74x2000")
    G = oracle_lib.sketch(74, 2000)
    assert gc.rel(G[:, :4], g["head"]) <= 1e-15
    assert gc.rel(G.sum(axis=0), g["colsum"]) <= 1e-14
    np.testing.assert_allclose(G[0:3, 0], [1.4365379616796561, -0.30089934168138049,
                                           0.39098155517110622], rtol=1e-15)


def test_oracle_explicit_sketch_equals_drawn_sketch(oracle_lib):
    A = oracle.gaussian(300, 280, 5)
    G = oracle_lib.sketch(42, 300)
    a1 = oracle_lib.hqrrp(A, 32, 10, 1)
    a2 = oracle_lib.hqrrp_sketch(A, G, 32, 10, 1)
    for x, y in zip(a1, a2):
        np.testing.assert_array_equal(x, y)


def _nfix(jp, m):
    return 0 if jp is None else min(m, int(np.count_nonzero(jp)))


@pytest.mark.parametrize("m,n,fixed", [(1200, 1100, None), (1100, 1200, 97), (1100, 1050, 9),
                                       (1030, 1000, 3)])
def test_oracle_dgeqp4_explicit_sketch_equals_drawn_sketch(oracle_lib, m, n, fixed):
    """dgeqp4's HQRRP branch fed the reference's own sketch of the free block
    (74 x (m - nf), srand(12) + polar method) is the drawn-sketch run, bit for
    bit: the sketch is the only input the explicit form replaces."""
    A = oracle.gaussian(m, n, m + 3 * n)
    jp = None if fixed is None else np.array([i % fixed == 0 for i in range(n)], np.int32)
    G = oracle_lib.sketch(74, m - _nfix(jp, m))
    a = oracle_lib.dgeqp4(A, jp)
    b = oracle_lib.dgeqp4_sketch(A, G, jp)
    for x, y in zip(a[:4], b[:4]):
        np.testing.assert_array_equal(x, y)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference tree not on this host")
@pytest.mark.parametrize("m,n,nb,pp,ppiv", [(500, 400, 32, 10, 1), (260, 390, 24, 8, 1),
                                            (333, 333, 40, 10, 0), (1000, 1000, 64, 10, 1)])
def test_oracle_bitexact_vs_compiled_reference(oracle_lib, m, n, nb, pp, ppiv):
    ref = oracle.Reference()
    A = oracle.gaussian(m, n, m * 7 + n)
    r = ref.hqrrp(A, nb, pp, ppiv)
    o = oracle_lib.hqrrp(A, nb, pp, ppiv)
    for x, y in zip(r, o):
        np.testing.assert_array_equal(x, y)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference tree not on this host")
@pytest.mark.parametrize("m,n,fixed", [(1050, 1000, None), (1000, 1040, 31), (520, 400, 5),
                                       (120, 90, 4), (0, 5, None), (5, 0, None)])
def test_oracle_dgeqp4_bitexact_vs_compiled_reference(oracle_lib, m, n, fixed):
    ref = oracle.Reference()
    A = oracle.gaussian(m, n, 99) if m * n else np.zeros((m, n), order="F")
    jp = None if fixed is None else np.array([i % fixed == 0 for i in range(n)], np.int32)
    r = ref.dgeqp4(A, jp)
    o = oracle_lib.dgeqp4(A, jp)
    for x, y in zip(r[:4], o[:4]):
        np.testing.assert_array_equal(x, y)


def test_oracle_quality(oracle_lib):
    sigma = np.logspace(0, -12, 500)
    A = oracle.with_spectrum(600, 500, sigma, 3)
    Af, jpvt, tau = oracle_lib.hqrrp(A, 64, 10, 1)
    res, orth, d = oracle.quality(A, Af, jpvt, tau)
    assert res < 1e-14 and orth < 1e-13
    ratio = d / sigma  # rank-revealing: |R_kk| tracks sigma_k
    assert 0.05 < ratio.min() and ratio.max() < 20


@pytest.mark.parametrize("m,n,nb,pp,ppiv", [(300, 280, 32, 10, 1), (150, 260, 32, 10, 1),
                                            (400, 300, 32, 8, 0), (257, 257, 64, 10, 1),
                                            (700, 350, 48, 10, 1)])
def test_ut_restatement_agrees_with_wy(oracle_lib, m, n, nb, pp, ppiv):
    """The UT-variant restatement (FLA_HQRRP_UT_blk_var2; libflame is absent,
    so it cannot be compiled) against the WY restatement pinned to the
    reference: on the same sketch the same pivots, the same factored matrix up
    to rounding, s = 1 / tau -- except where the UT transform's convention
    differs: a reflector with an empty or zero tail is H = I - 2 e e^T (tau_UT
    = 1/2, the row negated) where LAPACK's is H = I.  In a matrix with
    m <= n that is the last row (stage m - 1)."""
    A = oracle.gaussian(m, n, m + n + nb)
    G = oracle_lib.sketch(nb + pp, m)
    Aw, jw, tw = oracle_lib.hqrrp_sketch(A, G, nb, pp, ppiv)
    Au, ju, su = oracle_lib.hqrrp_ut(A, nb, pp, ppiv, G=G)
    np.testing.assert_array_equal(ju, jw)
    k = min(m, n)
    Aw = Aw.copy()
    tw = tw.copy()
    if m <= n:  # the empty-tail reflector of the last row
        assert tw[k - 1] == 0.0 and su[k - 1] == 0.5
        Aw[k - 1, k - 1:] *= -1.0
        tw[k - 1] = 2.0
    assert np.max(np.abs(su * tw - 1.0)) <= 1e-12
    den = np.linalg.norm(Aw, axis=0)
    assert np.max(np.linalg.norm(Au - Aw, axis=0) / den) <= 1e-12


def test_ut_restatement_drawn_sketch_is_the_reference_sketch(oracle_lib):
    """MyFLA_Normal_random_matrix draws the same polar-method stream after
    srand(12) as the WY variant's generator (for an even count)."""
    A = oracle.gaussian(200, 150, 3)
    G = oracle_lib.sketch(42, 200)
    a = oracle_lib.hqrrp_ut(A, 32, 10, 1)
    b = oracle_lib.hqrrp_ut(A, 32, 10, 1, G=G)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
