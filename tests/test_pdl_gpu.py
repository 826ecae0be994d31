"""Programmatic dependent launch (hqrrp_gb300/csrc/hq_common.cuh, hq_launch).

The library's kernels are launched with the programmatic-serialization
attribute and wait (griddepcontrol.wait) before touching memory, so the order
of their reads and writes is the stream's.  The bar (stated here): with the
attribute (the default) and without it (HQRRP_GB300_PDL=0) every output array
is bit-identical, on both precision paths, through the rank-revealing Gram
panel fallback, and through dgeqp4.
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _both(hq, fn):
    a = fn()
    os.environ["HQRRP_GB300_PDL"] = "0"
    try:
        b = fn()
    finally:
        os.environ.pop("HQRRP_GB300_PDL", None)
    c = fn()
    return a, b, c


def _same(a, b):
    for x, y in zip(a, b):
        np.testing.assert_array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("m,n,nb", [(1500, 1300, 128), (900, 1400, 64)])
def test_pdl_bit_identical(hq, precision, m, n, nb):
    A = oracle.gaussian(m, n, 3 * m + n)
    prev = hq.set_precision(hq.MIXED if precision == "mixed" else hq.PLAIN)
    try:
        a, b, c = _both(hq, lambda: hq.hqrrp(A, nb, 10, 1))
    finally:
        hq.set_precision(prev)
    _same(a, b)
    _same(a, c)
    res, orth, _ = oracle.quality(A, *a)
    assert res <= 1e-13 and orth <= 1e-12, (res, orth)


def test_pdl_bit_identical_rank_deficient_mixed(hq):
    """Rank 300: some Gram panels fall back to the column-by-column panel,
    whose kernels are gated on the Gram panel's status word."""
    m, n, r = 1200, 1000, 300
    rng = np.random.default_rng(21)
    A = rng.standard_normal((m, r)) @ rng.standard_normal((r, n))
    prev = hq.set_precision(hq.MIXED)
    try:
        a, b, _ = _both(hq, lambda: hq.hqrrp(A, 128, 10, 1))
    finally:
        hq.set_precision(prev)
    _same(a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pdl_bit_identical_dgeqp4(hq, precision):
    m, n = 1100, 900
    A = oracle.gaussian(m, n, 77)
    prev = hq.set_precision(hq.MIXED if precision == "mixed" else hq.PLAIN)
    try:
        a, b, _ = _both(hq, lambda: hq.dgeqp4(A))
    finally:
        hq.set_precision(prev)
    _same(a, b)
