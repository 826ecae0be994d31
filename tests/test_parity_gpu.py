"""GPU parity: libhqrrp_gb300.so against the oracle on the same inputs.

The oracle is the CPU restatement of the reference, itself pinned to the
reference by tests/test_oracle.py.  Both runs use the same sketch G (the
reference's own rand()-based one, passed explicitly to the GPU).  The parity bar
for the plain path: jpvt identical; tau and R within 1e-12 relative.  The
Householder vectors below the diagonal are compared at the same tolerance.
"""
import numpy as np
import pytest

import oracle
import golden_cases as gc

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, tau / R / V (FP64 plain path)


def col_rel_err(X, Xref):
    num = np.linalg.norm(X - Xref, axis=0)
    den = np.linalg.norm(Xref, axis=0)
    den[den == 0] = 1.0
    return float(np.max(num / den)) if X.size else 0.0


def assert_parity(got, want, tol=TOL):
    Af, jp, tau = got
    Ao, jo, to = want
    m, n = Ao.shape
    k = min(m, n)
    np.testing.assert_array_equal(jp, jo)
    terr = float(np.max(np.abs(tau - to) / np.maximum(np.abs(to), 1e-300))) if k else 0.0
    R, Ro = np.triu(Af[:k, :]), np.triu(Ao[:k, :])
    V, Vo = np.tril(Af[:, :k], -1), np.tril(Ao[:, :k], -1)
    rerr, verr = col_rel_err(R, Ro), col_rel_err(V, Vo)
    assert terr <= tol and rerr <= tol and verr <= tol, (terr, rerr, verr)
    return terr, rerr, verr


HQRRP_CASES = [
    # m, n, nb, pp, panel_pivoting, seed
    (2000, 2000, 64, 10, 1, 20261203),   # config 1
    (1500, 1200, 128, 10, 1, 1),
    (600, 1000, 64, 10, 1, 2),           # wide: last block pivots within its columns
    (3000, 400, 32, 8, 1, 3),            # tall
    (777, 555, 50, 6, 1, 4),             # nb does not divide n
    (500, 400, 32, 10, 0, 5),            # unpivoted panels
    (40, 20, 64, 10, 1, 6),              # nb > n: one block, no sketch step
    (2, 3, 2, 2, 1, 7),
    (3, 2, 1, 1, 1, 8),
    (1, 1, 1, 1, 1, 9),
]


@pytest.mark.parametrize("m,n,nb,pp,ppiv,seed", HQRRP_CASES)
def test_hqrrp_matches_oracle(hq, oracle_lib, m, n, nb, pp, ppiv, seed):
    A = oracle.gaussian(m, n, seed)
    G = oracle_lib.sketch(nb + pp, m)
    want = oracle_lib.hqrrp_sketch(A, G, nb, pp, ppiv)
    got = hq.hqrrp(A, nb, pp, ppiv, G=G)
    assert_parity(got, want)


def test_config1_against_reference_golden(hq, oracle_lib):
    """Config 1 straight against what the reference returned (fixture)."""
    name = "hqrrp_2000x2000_nb64"
    A, _, same = gc.case_input(name)
    if not same:
        pytest.skip("fixture input not reproducible by this numpy")
    g = gc.load(name)
    G = oracle_lib.sketch(74, 2000)
    Af, jp, tau = hq.hqrrp(A, 64, 10, 1, G=G)
    s = gc.summary(Af, jp, tau, 2000, 2000)
    np.testing.assert_array_equal(s["jpvt"], g["jpvt"])
    for key in ("tau", "diag", "aw", "atu"):
        assert gc.rel(s[key], g[key]) <= TOL, key


def test_hqrrp_full_output_golden(hq, oracle_lib):
    name = "hqrrp_160x120_nb16"
    A, _, same = gc.case_input(name)
    if not same:
        pytest.skip("fixture input not reproducible by this numpy")
    g = gc.load(name)
    G = oracle_lib.sketch(20, 160)
    Af, jp, tau = hq.hqrrp(A, 16, 4, 1, G=G)
    np.testing.assert_array_equal(jp, g["jpvt"])
    assert col_rel_err(Af, g["af"]) <= TOL


def test_hqrrp_quality_geometric_spectrum(hq):
    m = n = 1200
    sigma = 10.0 ** (-12.0 * np.arange(n) / n)
    A = oracle.with_spectrum(m, n, sigma, 11)
    Af, jp, tau = hq.hqrrp(A, 128, 10, 1)
    res, orth, d = oracle.quality(A, Af, jp, tau)
    assert res < 1e-14 and orth < 1e-13, (res, orth)
    ratio = d / sigma
    assert 0.05 < ratio.min() and ratio.max() < 20


def test_hqrrp_carries_incoming_labels(hq, oracle_lib):
    A = oracle.gaussian(300, 250, 12)
    labels = np.arange(250, dtype=np.int32)[::-1] * 3 + 7
    G = oracle_lib.sketch(42, 300)
    want = oracle_lib.hqrrp_sketch(A, G, 32, 10, 1, jpvt=labels)
    got = hq.hqrrp(A, 32, 10, 1, jpvt=labels, G=G)
    assert_parity(got, want)


def test_hqrrp_deterministic(hq):
    A = oracle.gaussian(900, 700, 13)
    a = hq.hqrrp(A, 64, 10, 1)
    b = hq.hqrrp(A, 64, 10, 1)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_hqrrp_lda_larger_than_m(hq, oracle_lib):
    """A sub-matrix view with lda > m: only the m x n block is read and written."""
    big = oracle.gaussian(700, 300, 14)
    import ctypes as C
    L = hq.load()
    m, n, lda = 500, 300, 700
    G = oracle_lib.sketch(42, m)
    want = oracle_lib.hqrrp_sketch(big[:m], G, 32, 10, 1)
    buf = np.array(big, order="F")
    jp = np.arange(1, n + 1, dtype=np.int32)
    tau = np.zeros(n)
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    Gf = np.array(G, order="F")
    rc = L.hqrrp_gb300_hqrrp_sketch(m, n, buf.ctypes.data_as(dp), lda, jp.ctypes.data_as(ip),
                                    tau.ctypes.data_as(dp), 32, 10, 1, Gf.ctypes.data_as(dp), 42)
    assert rc == 0
    np.testing.assert_array_equal(buf[m:], big[m:])
    assert_parity((buf[:m], jp, tau), want)


@pytest.mark.parametrize("m,n,lda,nb,fixed", [
    (1300, 1100, 1333, 64, None),   # tall, lda > m
    (1000, 1300, 1000, 64, None),   # wide: the columns past min(m, n) go back at the end
    (1024, 1024, 1024, 128, None),
    (1100, 1050, 1100, 64, 9),      # dgeqp4 with fixed columns: one copy at the end
])
def test_pinned_host_buffers_match_pageable(hq, m, n, lda, nb, fixed):
    """Page-locked host matrices are copied back column block by column block
    while later blocks run; the result is bit-identical to the pageable-buffer
    call (one copy at the end), for both reference entry points, and rows
    m..lda-1 are left alone."""
    import ctypes as C
    import torch
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    L = hq.load()
    big = oracle.gaussian(lda, n, 31 + m)
    ref = hq.hqrrp(big[:m], nb, 10, 1)
    pin = torch.from_numpy(np.array(big.T)).pin_memory()   # (n, lda) = column-major lda x n
    jp = np.arange(1, n + 1, dtype=np.int32)
    tau = np.zeros(min(m, n))
    rc = L.NoFLA_HQRRP_WY_blk_var4(m, n, C.cast(pin.data_ptr(), dp), lda, jp.ctypes.data_as(ip),
                                   tau.ctypes.data_as(dp), nb, 10, 1)
    assert rc == 0, hq.last_error()
    got = pin.numpy().T
    np.testing.assert_array_equal(got[:m], ref[0])
    np.testing.assert_array_equal(got[m:], big[m:])
    np.testing.assert_array_equal(jp, ref[1])
    np.testing.assert_array_equal(tau, ref[2])

    jin = None if fixed is None else np.array([i % fixed == 0 for i in range(n)], np.int32)
    ref4 = hq.dgeqp4(big[:m], jin)
    pin = torch.from_numpy(np.array(big.T)).pin_memory()
    jp = np.zeros(n, np.int32) if jin is None else jin.copy()
    tau = np.zeros(min(m, n))
    lwork = max(3 * n + 1, 2 * n + (n + 1) * 32)
    work = np.zeros(lwork)
    mi, ni, li, lw, info = C.c_int(m), C.c_int(n), C.c_int(lda), C.c_int(lwork), C.c_int(0)
    L.dgeqp4(C.byref(mi), C.byref(ni), C.cast(pin.data_ptr(), dp), C.byref(li),
             jp.ctypes.data_as(ip), tau.ctypes.data_as(dp), work.ctypes.data_as(dp), C.byref(lw),
             C.byref(info))
    assert info.value == 0, hq.last_error()
    got = pin.numpy().T
    np.testing.assert_array_equal(got[:m], ref4[0])
    np.testing.assert_array_equal(got[m:], big[m:])
    np.testing.assert_array_equal(jp, ref4[1])
    np.testing.assert_array_equal(tau, ref4[2])


def test_device_pointer_entry(hq, oracle_lib):
    import torch
    m, n, nb, pp = 1000, 800, 64, 10
    A = oracle.gaussian(m, n, 15)
    G = oracle_lib.sketch(nb + pp, m)
    want = oracle_lib.hqrrp_sketch(A, G, nb, pp, 1)
    At = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    Gt = torch.from_numpy(np.ascontiguousarray(G.T)).cuda()
    jp = torch.arange(1, n + 1, dtype=torch.int32, device="cuda")
    tau = torch.zeros(min(m, n), dtype=torch.float64, device="cuda")
    hq.hqrrp_device(At, jp, tau, nb, pp, 1, Gt=Gt)
    got = (At.cpu().numpy().T, jp.cpu().numpy(), tau.cpu().numpy())
    assert_parity(got, want)


# ---- dgeqp4 -----------------------------------------------------------------

DGEQP4_CASES = [
    # m, n, seed, fixed-column rule (every k-th column fixed) or None
    (200, 300, 19, None),     # dgeqpf branch
    (249, 249, 20, None),     # last dgeqpf size
    (250, 250, 21, None),     # first dgeqp3 size
    (600, 500, 17, None),     # dgeqp3 branch
    (300, 260, 18, 7),        # dgeqp3 branch with fixed columns
    (999, 999, 22, None),     # last dgeqp3 size
    (120, 90, 23, 4),         # dgeqpf branch with fixed columns
    # more than 1024 free columns: the column-partitioned wide kernel
    (300, 2000, 24, None),    # dgeqp3 branch
    (200, 3000, 25, None),    # dgeqpf branch
    (999, 5000, 26, None),    # last dgeqp3 size, five times as many columns
    (400, 1500, 27, 9),       # fixed columns, then 1333 free ones
    (64, 1025, 28, None),     # one column past the panel kernel's limit
]


@pytest.mark.parametrize("m,n,seed,fixed", DGEQP4_CASES)
def test_dgeqp4_small_paths_match_lapack(hq, oracle_lib, m, n, seed, fixed):
    A = oracle.gaussian(m, n, seed)
    jp = None if fixed is None else np.array([i % fixed == 0 for i in range(n)], np.int32)
    Ao, jo, to, io, wo = oracle_lib.dgeqp4(A, jp)
    Ag, jg, tg, ig, wg = hq.dgeqp4(A, jp)
    assert ig == io == 0
    assert_parity((Ag, jg, tg), (Ao, jo, to))
    if min(m, n) >= 250:
        assert wg == wo


def test_dgeqp4_demo_7x5(hq):
    g = gc.load("dgeqp4_demo_7x5")
    Af, jp, tau, info, _ = hq.dgeqp4(g["a"], g["jpvt_in"])
    assert info == 0
    np.testing.assert_array_equal(jp, g["jpvt"])
    assert col_rel_err(Af, g["af"]) <= TOL and gc.rel(tau, g["tau"]) <= TOL


# ---- dgeqp4's HQRRP branch (min(m, n) >= 1000) on the reference's sketch ------

def _fixed_marks(n, fixed):
    return None if fixed is None else np.array([i % fixed == 0 for i in range(n)], np.int32)


def _nfix(jp, m):
    return 0 if jp is None else min(m, int(np.count_nonzero(jp)))


DGEQP4_HQRRP_CASES = [
    # m, n, seed, fixed-column rule (every k-th column fixed) or None
    (1200, 1100, 41, None),
    (1100, 1200, 42, 7),      # wide, fixed columns: unpivoted QR + update, then HQRRP
    (1100, 1050, 43, 9),      # m > n with fixed columns
    (1000, 1000, 44, None),   # the first size dgeqp4 gives to HQRRP
    (1500, 1030, 45, 3),      # a third of the columns fixed: HQRRP on 1156 x 686
]


@pytest.mark.parametrize("m,n,seed,fixed", DGEQP4_HQRRP_CASES)
def test_dgeqp4_hqrrp_branch_matches_oracle(hq, oracle_lib, m, n, seed, fixed):
    """dgeqp4 (...var4.c:127-300) through the C ABI, its HQRRP(64, 10, 1) call
    fed the reference's own sketch of the free block: the oracle draws that
    sketch itself (srand(12) + polar method, as the reference does), the GPU
    is given the same matrix.  jpvt identical, tau/R/V within 1e-12, and the
    same LAPACK workspace figure."""
    A = oracle.gaussian(m, n, seed)
    jp = _fixed_marks(n, fixed)
    G = oracle_lib.sketch(74, m - _nfix(jp, m))
    Ao, jo, to, io, wo = oracle_lib.dgeqp4(A, jp)
    Ag, jg, tg, ig, wg = hq.dgeqp4(A, jp, G=G)
    assert ig == io == 0
    assert_parity((Ag, jg, tg), (Ao, jo, to))
    assert wg == wo


@pytest.mark.parametrize("name", ["dgeqp4_1200x1100", "dgeqp4_1100x1200_fixed"])
def test_dgeqp4_hqrrp_branch_against_reference_golden(hq, oracle_lib, name):
    """The GPU dgeqp4 straight against what the reference's dgeqp4 returned
    (fixtures made by tests/golden/make_golden.py from the compiled reference)."""
    A, jp, same = gc.case_input(name)
    if not same:
        pytest.skip("fixture input not reproducible by this numpy")
    g = gc.load(name)
    m, n = A.shape
    G = oracle_lib.sketch(74, m - _nfix(jp, m))
    Af, jpv, tau, info, work0 = hq.dgeqp4(A, jp, G=G)
    assert info == int(g["info"]) and work0 == float(g["work0"])
    s = gc.summary(Af, jpv, tau, m, n)
    np.testing.assert_array_equal(s["jpvt"], g["jpvt"])
    for key in ("tau", "diag", "aw", "atu"):
        assert gc.rel(s[key], g[key]) <= TOL, key


def test_dgeqp4_rows_above_follow_hqrrp_bit_exact(hq, oracle_lib):
    """The re-pivot of the rows above the free block (...var4.c:267-292) is a
    pure column permutation.  With unit vectors e_0, e_1, ... as the fixed
    columns, every fixed-column reflector is the identity (tau = 0), so rows
    0..nf-1 of the free columns must come out as the input's rows, in HQRRP's
    column order, bit for bit -- on the GPU and in the oracle alike."""
    m, n, every = 1100, 1200, 50
    A = oracle.gaussian(m, n, 46)
    jp = _fixed_marks(n, every)
    pos = np.flatnonzero(jp)
    nf = len(pos)
    for t, c in enumerate(pos):
        A[:, c] = 0.0
        A[t, c] = 1.0
    G = oracle_lib.sketch(74, m - nf)
    Ag, jg, tg, ig, _ = hq.dgeqp4(A, jp, G=G)
    Ao, jo, to, io, _ = oracle_lib.dgeqp4(A, jp)
    assert ig == io == 0
    assert np.all(tg[:nf] == 0.0) and np.all(to[:nf] == 0.0)
    np.testing.assert_array_equal(Ag[:nf, nf:], A[:nf, jg[nf:] - 1])
    np.testing.assert_array_equal(Ao[:nf, nf:], A[:nf, jo[nf:] - 1])
    assert_parity((Ag, jg, tg), (Ao, jo, to))


@pytest.mark.parametrize("nb", [128, 64])
def test_dgeqp4_block_size(hq, oracle_lib, nb):
    """dgeqp4 with HQRRP block 128 (the GPU default) and 64 (the reference's,
    through hqrrp_gb300_set_dgeqp4_block): each block structure has its own
    pivots but the same quality, fixed columns still first, and an explicit
    reference sketch still gets the reference's block size 64 (parity with the
    oracle unchanged)."""
    m, n = 1500, 1400
    A = oracle.gaussian(m, n, 47)
    jp = _fixed_marks(n, 11)
    prev = hq.set_dgeqp4_block(nb)
    try:
        Af, jpv, tau, info, _ = hq.dgeqp4(A, jp)
        G = oracle_lib.sketch(74, m - _nfix(jp, m))
        got = hq.dgeqp4(A, jp, G=G)
    finally:
        hq.set_dgeqp4_block(prev)
    assert info == 0
    nf = _nfix(jp, m)
    assert sorted(jpv[:nf]) == [i + 1 for i in range(0, n, 11)]
    res, orth, _ = oracle.quality(A, Af, jpv, tau)
    assert res <= 1e-14 and orth <= 1e-13, (res, orth)
    Ao, jo, to, io, _ = oracle_lib.dgeqp4(A, jp)
    assert got[3] == io == 0
    assert_parity(got[:3], (Ao, jo, to))
