"""CPU checks of the panel kernel's fixed-point stage sums.

hqrrp_gb300/csrc/hq_fixedpoint.h holds the arithmetic the pivoted panel
kernel uses to sum one FP64 partial dot product per CTA: each partial becomes
an integer in units of 2^ue (ue from the columns' norms) split into 48-bit
limbs, the limbs are added as 64-bit integers, and the words are converted
back to FP64.  Here the same header is compiled for the host and its sums are
compared with exact rational sums of the same partials.
"""
import ctypes as C
import math
import os
import random
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def fx(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("fx") / "libfx.so")
    src = os.path.join(ROOT, "tests", "fixedpoint_harness.c")
    inc = os.path.join(ROOT, "hqrrp_gb300", "csrc")
    subprocess.run(["gcc", "-O2", "-std=c11", "-shared", "-fPIC", "-I", inc, src, "-o", out,
                    "-lm"], check=True)
    lib = C.CDLL(out)
    lib.hq_test_fx_sum.restype = C.c_double
    lib.hq_test_fx_sum.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_double, C.c_double,
                                   C.c_int]

    def fsum(parts, ep, ek, sq):
        a = np.ascontiguousarray(parts, dtype=np.float64)
        return lib.hq_test_fx_sum(a.ctypes.data_as(C.POINTER(C.c_double)), len(a), ep, ek, sq)
    return fsum


def partials(x, y, ctas):
    """Per-CTA partial dot products of x and y over contiguous row slabs, each
    summed with FMAs in order (as a CTA's lanes do, up to order)."""
    n = len(x)
    out = []
    for c in range(ctas):
        lo, hi = c * n // ctas, (c + 1) * n // ctas
        out.append(float(np.dot(x[lo:hi], y[lo:hi])) if hi > lo else 0.0)
    return out


def check(fsum, parts, x, y, sq):
    nx, ny = float(np.dot(x, x)), float(np.dot(y, y))
    ep, ek = (nx, ny) if sq else (math.sqrt(nx), math.sqrt(ny))
    got = fsum(parts, ep, ek, int(sq))
    exact = sum(Fraction(p) for p in parts)
    bound = Fraction(math.sqrt(nx)) * Fraction(math.sqrt(ny))
    err = abs(Fraction(got) - exact)
    # Within an ulp of the exact sum of the partials, or negligible next to
    # the bound (truncation below 2^ue, 2^-133 of it).
    assert err <= abs(exact) * Fraction(2) ** -52 or err <= bound * Fraction(2) ** -120, (
        got, float(exact), float(bound))
    return got


@pytest.mark.parametrize("sq", [0, 1])
def test_sums_match_exact_rational_sums(fx, sq):
    rng = np.random.default_rng(20261203 + sq)
    for trial in range(400):
        n = int(rng.integers(1, 600))
        ctas = int(rng.choice([1, 2, 7, 96, 152, 160]))
        scale = 10.0 ** rng.uniform(-120, 120)
        x = rng.standard_normal(n) * scale
        y = rng.standard_normal(n) * scale * float(rng.choice([1.0, 1e-6, 1e6]))
        if trial % 5 == 0:
            y = x + 1e-9 * y  # near-parallel columns: large sums
        if trial % 7 == 0:
            y = np.where(np.arange(n) % 2 == 0, 1.0, -1.0) * np.abs(x)  # cancellation
        check(fx, partials(x, y, ctas), x, y, sq)


def test_order_does_not_change_the_bits(fx):
    rng = np.random.default_rng(7)
    x, y = rng.standard_normal(5000), rng.standard_normal(5000)
    parts = partials(x, y, 152)
    ep, ek = float(np.dot(x, x)), float(np.dot(y, y))
    ref = fx(parts, ep, ek, 1)
    for _ in range(20):
        random.Random(_).shuffle(parts)
        assert fx(parts, ep, ek, 1) == ref  # bit-identical in any order


def test_self_dot_is_the_squared_norm(fx):
    rng = np.random.default_rng(11)
    x = rng.standard_normal(16384) * 3.0
    parts = partials(x, x, 152)
    got = fx(parts, float(np.dot(x, x)), float(np.dot(x, x)), 1)
    assert got == pytest.approx(float(sum(Fraction(p) for p in parts)), rel=2.0 ** -52)


def test_zero_and_non_finite(fx):
    assert fx([0.0] * 10, 1.0, 1.0, 1) == 0.0
    assert math.isnan(fx([1.0, float("nan"), 2.0], 9.0, 9.0, 1))
    assert math.isnan(fx([1.0, float("inf")], 9.0, 9.0, 1))
    # A partial far beyond its bound (impossible for true norms) is flagged,
    # not wrapped around.
    assert math.isnan(fx([1e40], 1.0, 1.0, 1))
    # Subnormal partials lie below every unit in use and add nothing.
    assert fx([5e-324, 1.0], 4.0, 4.0, 1) == 1.0
