"""Access to the golden fixtures made by tests/golden/make_golden.py."""
import hashlib
import importlib.util
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
make_golden = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(make_golden)

CASES = make_golden.CASES


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def case_input(name):
    """(A, jpvt_in, input_matches_fixture)."""
    A, jp = make_golden.case_input(name)
    g = load(name)
    sha = np.frombuffer(hashlib.sha256(A.tobytes(order="F")).digest(), np.uint8)
    return A, jp, bool(np.array_equal(sha, g["sha"]))


def projections(m, n):
    return make_golden.projections(m, n)


def summary(Af, jpvt, tau, m, n):
    w, u = projections(m, n)
    k = min(m, n)
    return dict(jpvt=jpvt, tau=tau, diag=np.abs(np.diag(Af[:k, :k])), aw=Af @ w, atu=Af.T @ u)


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (d if d > 0 else 1.0)
