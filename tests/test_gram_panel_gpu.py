"""The mixed path's Gram panel (hqrrp_gb300/csrc/qrp_gram.cu).

Each block's panel is factored from its Gram matrix (pivoted Cholesky,
CholeskyQR2, Householder reconstruction) instead of column by column, and
falls back to the column-by-column pivoted panel when a Cholesky or LU pivot
shows the panel too ill-conditioned for it.

Bars (stated here): ||AP - QR||_F / ||A||_F <= 1e-13 and ||Q^T Q - I||_F <=
1e-12, the mixed path's own; |R_kk| of the Gram-panel run within a factor 2
of the column-by-column run on the same sketch (the block pivots come from
the same sketch and the Gram panel pivots by the same greedy largest-residual
rule, so the two differ only where near-equal residual norms are ordered
differently).
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _run(hq, A, nb, gram, G=None):
    prev = hq.set_precision(hq.MIXED)
    if not gram:
        os.environ["HQRRP_GB300_GRAM_PANEL"] = "0"
    try:
        out = hq.hqrrp(A, nb, 10, 1, G=G)
        counts = hq.gram_panel_counts()
    finally:
        os.environ.pop("HQRRP_GB300_GRAM_PANEL", None)
        hq.set_precision(prev)
    return out, counts


@pytest.mark.parametrize("m,n,nb", [(2000, 2000, 128), (1500, 1200, 64), (900, 1400, 64),
                                    (3000, 700, 128), (1000, 1000, 100)])
def test_gram_panel_matches_column_panel(hq, m, n, nb):
    k = min(m, n)
    sigma = 10.0 ** (-12.0 * np.arange(k) / k)
    A = oracle.with_spectrum(m, n, sigma, m + 7 * n)
    G = np.random.default_rng(m + n).standard_normal((nb + 10, m))
    got, (com, fb) = _run(hq, A, nb, True, G)
    ref, (com0, fb0) = _run(hq, A, nb, False, G)
    nblocks = (k + nb - 1) // nb
    assert (com, fb) == (nblocks, 0), (com, fb, nblocks)
    res, orth, d = oracle.quality(A, *got)
    res0, orth0, d0 = oracle.quality(A, *ref)
    assert res <= 1e-13 and orth <= 1e-12, (res, orth)
    assert res0 <= 1e-13 and orth0 <= 1e-12, (res0, orth0)
    ratio = d / d0
    assert 0.5 <= ratio.min() and ratio.max() <= 2.0, (ratio.min(), ratio.max())


def test_gram_panel_falls_back_at_the_rank(hq):
    """Exact rank 300 in a 1200 x 1000 matrix: the panel across column 300
    holds columns within rounding of the span of the earlier ones, so its
    Cholesky pivot falls below 1e-10 of the column's squared norm and the
    column-by-column panel takes it; the factorization still meets the bars
    and reveals the rank."""
    m, n, r, nb = 1200, 1000, 300, 128
    rng = np.random.default_rng(11)
    A = rng.standard_normal((m, r)) @ rng.standard_normal((r, n))
    (Af, jp, tau), (com, fb) = _run(hq, A, nb, True)
    assert fb >= 1 and com + fb == (n + nb - 1) // nb, (com, fb)
    res, orth, d = oracle.quality(A, Af, jp, tau)
    assert res <= 1e-13 and orth <= 1e-12, (res, orth)
    assert d[r - 1] > 1e-8 * d[0] and d[r] < 1e-12 * d[0], (d[r - 1], d[r], d[0])


def test_gram_panel_duplicate_and_zero_columns(hq):
    """Exactly repeated columns (a zero residual after the first copy) and
    all-zero columns (a zero Gram diagonal) are handed to the
    column-by-column panel, which factors them as LAPACK does."""
    m, n, nb = 800, 600, 64
    rng = np.random.default_rng(12)
    A = rng.standard_normal((m, n))
    A[:, 10:40] = A[:, 40:70]
    A[:, 200:230] = 0.0
    (Af, jp, tau), (com, fb) = _run(hq, A, nb, True)
    assert fb >= 1 and com + fb == (n + nb - 1) // nb, (com, fb)
    res, orth, _ = oracle.quality(A, Af, jp, tau)
    assert res <= 1e-13 and orth <= 1e-12, (res, orth)
    assert np.all(np.isfinite(Af))


def test_gram_panel_all_zero_matrix(hq):
    A = np.zeros((300, 200))
    (Af, jp, tau), (com, fb) = _run(hq, A, 64, True)
    assert (com, fb) == (0, 4)
    assert np.all(Af == 0.0) and np.all(tau == 0.0)
    assert sorted(jp) == list(range(1, 201))
