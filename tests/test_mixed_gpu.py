"""Mixed precision: the split-BF16 tensor-core FP64 products and HQRRP with them.

Tolerances (stated here, checked per element or normwise):
* hqrrp_gb300_ozaki_dgemm with s digits: |C - AB| <= tol(s) * (|A| |B|) per
  element, tol(6) = 2^-42, tol(7) = 2^-49 (design accuracy 2^-45 / 2^-52).
* mixed HQRRP (the mixed form's target): ||AP - QR||_F / ||A||_F <= 1e-13 and
  |R_kk| / sigma_k within a factor 2 of the plain FP64 path.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = {4: 2.0 ** -27, 6: 2.0 ** -42, 7: 2.0 ** -49}


def _col(X):
    import torch
    return torch.from_numpy(np.ascontiguousarray(X.T)).cuda()


@pytest.mark.parametrize("m,n,k,ta,tb,s", [
    (128, 64, 32, "N", "N", 6),     # one tile, one K block
    (200, 100, 300, "N", "N", 6),   # partial tiles, one drain
    (300, 250, 1000, "T", "N", 7),  # several drains
    (128, 1000, 4000, "T", "N", 7),  # the W1 = U^T C shape (split K)
    (1000, 777, 128, "N", "T", 7),  # the C -= U W2 shape
    (513, 65, 2049, "N", "N", 7),
    (128, 200, 20000, "T", "N", 7),  # rows longer than 16384: two-pass split
    (640, 640, 640, "N", "N", 4),
])
def test_ozaki_dgemm_accuracy(hq, m, n, k, ta, tb, s):
    import torch
    rng = np.random.default_rng(m + n + k)
    A = rng.standard_normal((k, m) if ta == "T" else (m, k)) * 3.0 ** rng.integers(-5, 5)
    B = rng.standard_normal((n, k) if tb == "T" else (k, n))
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    C = torch.zeros((n, m), dtype=torch.float64, device="cuda")
    hq.ozaki_dgemm(ta, tb, 1.0, _col(A), _col(B), 0.0, C, slices=s)
    got = C.cpu().numpy().T
    err = np.abs(got - opA @ opB) / (np.abs(opA) @ np.abs(opB))
    assert err.max() <= TOL[s], err.max()


def test_ozaki_dgemm_update_mode(hq):
    rng = np.random.default_rng(3)
    A = rng.standard_normal((700, 128))
    B = rng.standard_normal((128, 900))
    C0 = rng.standard_normal((700, 900))
    C = _col(C0)
    hq.ozaki_dgemm("N", "N", -1.0, _col(A), _col(B), 1.0, C, slices=7)
    got = C.cpu().numpy().T
    err = np.abs(got - (C0 - A @ B)) / (np.abs(A) @ np.abs(B) + np.abs(C0))
    assert err.max() <= TOL[7]


def test_ozaki_dgemm_rejects_unsupported_scalars(hq):
    import torch
    C = torch.zeros((4, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(hq.HQRRPError):
        hq.ozaki_dgemm("N", "N", 2.0, C, C, 0.0, C)


@pytest.fixture
def mixed(hq):
    prev = hq.set_precision(hq.MIXED)
    yield hq
    hq.set_precision(prev)


@pytest.mark.parametrize("m,n,nb", [(2000, 2000, 64), (1500, 1200, 128), (900, 1400, 64)])
def test_mixed_hqrrp_residual_and_rank_revealing(hq, m, n, nb):
    k = min(m, n)
    sigma = 10.0 ** (-12.0 * np.arange(k) / k)
    A = oracle.with_spectrum(m, n, sigma, m + n)
    hq.set_precision(hq.PLAIN)
    plain = hq.hqrrp(A, nb, 10, 1)
    hq.set_precision(hq.MIXED)
    try:
        got = hq.hqrrp(A, nb, 10, 1)
    finally:
        hq.set_precision(hq.PLAIN)
    res, orth, d = oracle.quality(A, *got)
    _, _, dp = oracle.quality(A, *plain)
    assert res <= 1e-13 and orth <= 1e-12, (res, orth)
    # |R_kk| / sigma_k within 2x of the plain path: per k before the last two
    # blocks (a wide matrix's last block pivots only within itself, where a
    # different sketch reorders near-equal columns), and for the extremes.
    kk = k - 2 * nb
    ratio = d[:kk] / dp[:kk]
    assert 0.5 <= ratio.min() and ratio.max() <= 2.0
    r, rp = d / sigma, dp / sigma  # no worse than 2x at either extreme
    assert r.min() >= 0.5 * rp.min() and r.max() <= 2.0 * rp.max()


def test_mixed_dgeqp4_fixed_columns(mixed):
    A = oracle.gaussian(1100, 1050, 41)
    jp = np.array([1 if i % 50 == 0 else 0 for i in range(1050)], np.int32)
    Af, jpvt, tau, info, _ = mixed.dgeqp4(A, jp)
    assert info == 0
    assert sorted(jpvt[:21]) == [i + 1 for i in range(0, 1050, 50)]
    res, orth, _ = oracle.quality(A, Af, jpvt, tau)
    assert res <= 1e-13 and orth <= 1e-12


@pytest.mark.parametrize("m,n,every", [(400, 300, 7), (300, 520, 9), (120, 90, 4)])
def test_mixed_dgeqp4_small_path_fixed_columns(mixed, m, n, every):
    """Below dgeqp4's dgeqp3 threshold, with fixed columns: the fixed block's
    trailing update runs as split-BF16 products, the rest as the pivoted
    FP64 panel kernel."""
    A = oracle.gaussian(m, n, m + 3 * n)
    jp = np.array([1 if i % every == 0 else 0 for i in range(n)], np.int32)
    nf = int(jp.sum())
    Af, jpvt, tau, info, _ = mixed.dgeqp4(A, jp)
    assert info == 0
    assert sorted(jpvt[:nf]) == [i + 1 for i in range(0, n, every)]
    res, orth, _ = oracle.quality(A, Af, jpvt, tau)
    assert res <= 1e-13 and orth <= 1e-12, (res, orth)


@pytest.mark.parametrize("m,n,nb", [(2000, 1800, 128), (1500, 1500, 64)])
def test_trailing_digits_cut_on_the_fly_are_the_split_digits(hq, m, n, nb):
    """From the second block on, W1 = U'^T C reads C as FP64 and cuts its
    digits in shared memory (scales from the previous update's column
    exponents) instead of a separate split pass, and the Gram panel's
    G = Ap^T Ap takes the same recorded exponents instead of a row-maximum
    pass: the digits are the same, so the factorization is bit-identical to
    the separate passes' (HQRRP_GB300_SPLIT_TRAILING=1)."""
    import os
    A = oracle.gaussian(m, n, m + 2 * n)
    prev = hq.set_precision(hq.MIXED)
    try:
        a = hq.hqrrp(A, nb, 10, 1)
        os.environ["HQRRP_GB300_SPLIT_TRAILING"] = "1"
        try:
            b = hq.hqrrp(A, nb, 10, 1)
        finally:
            os.environ.pop("HQRRP_GB300_SPLIT_TRAILING", None)
    finally:
        hq.set_precision(prev)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
