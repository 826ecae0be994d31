"""Generate the golden fixtures in this directory from the REFERENCE itself.

Run here, where the reference tree is mounted:  python tests/golden/make_golden.py

Each case factors a seeded matrix with the unmodified reference
(lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c compiled by oracle/build.py
into oracle/_ref/) and stores what the reference returned: jpvt, tau, |diag R|
and projections of the factored matrix (A_out @ w, A_out^T @ u with fixed
vectors w, u), plus full outputs for the small cases.  The SHA-256 of the input
bytes is stored so a test can tell when numpy's generator no longer reproduces
the input.  The sketch of each HQRRP run is the reference's own (srand(12) +
polar method); every case keeps (nb + pp) * m even, so the reference's carried
spare normal is empty on entry and the sketch does not depend on call order.
"""
import hashlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def demo_7x5():
    """The integer matrix of the reference's lapack_compatible_sources/simple_test.c
    (7 x 5, column j filled from row j mod m downward with a running counter,
    A[0,0] = 1.2), with columns 1, 2, 4 marked fixed."""
    m, n = 7, 5
    A = np.zeros((m, n), order="F")
    num = 1
    for j in range(n):
        for i in list(range(j % m, m)) + list(range(0, j % m)):
            A[i, j] = num
            num += 1
    A[0, 0] = 1.2
    return A, np.array([0, 1, 1, 0, 1], dtype=np.int32)


# name: (kind, m, n, seed, nb, pp, panel_pivoting, fixed-column rule, full outputs)
CASES = {
    "hqrrp_2000x2000_nb64": ("hqrrp", 2000, 2000, 20261203, 64, 10, 1, None, False),
    "hqrrp_160x120_nb16": ("hqrrp", 160, 120, 11, 16, 4, 1, None, True),
    "hqrrp_150x260_nb32_wide": ("hqrrp", 150, 260, 12, 32, 10, 1, None, False),
    "hqrrp_400x300_nb32_nopanelpiv": ("hqrrp", 400, 300, 13, 32, 8, 0, None, False),
    "hqrrp_700x350_nb48": ("hqrrp", 700, 350, 14, 48, 10, 1, None, False),
    "dgeqp4_1100x1200_fixed": ("dgeqp4", 1100, 1200, 15, 0, 0, 0, 97, False),
    "dgeqp4_1200x1100": ("dgeqp4", 1200, 1100, 16, 0, 0, 0, None, False),
    "dgeqp4_600x500_dgeqp3": ("dgeqp4", 600, 500, 17, 0, 0, 0, None, False),
    "dgeqp4_300x260_dgeqp3_fixed": ("dgeqp4", 300, 260, 18, 0, 0, 0, 7, False),
    "dgeqp4_200x300_dgeqpf": ("dgeqp4", 200, 300, 19, 0, 0, 0, None, False),
}


def case_input(name):
    import oracle
    kind, m, n, seed, nb, pp, ppiv, fixed, full = CASES[name]
    A = oracle.gaussian(m, n, seed)
    jp = None
    if fixed is not None:
        jp = np.array([1 if i % fixed == 0 else 0 for i in range(n)], dtype=np.int32)
    return A, jp


def projections(m, n):
    rng = np.random.default_rng(7)
    return rng.standard_normal(n), rng.standard_normal(m)


def run_case(name):
    import oracle
    ref = oracle.Reference()
    ref.set_threads(1)
    kind, m, n, seed, nb, pp, ppiv, fixed, full = CASES[name]
    A, jp = case_input(name)
    if kind == "hqrrp":
        Af, jpvt, tau = ref.hqrrp(A, nb, pp, ppiv)
        info, work0 = 0, 0.0
    else:
        Af, jpvt, tau, info, work0 = ref.dgeqp4(A, jp)
    w, u = projections(m, n)
    k = min(m, n)
    out = dict(sha=np.frombuffer(hashlib.sha256(A.tobytes(order="F")).digest(), np.uint8),
               jpvt=jpvt, tau=tau, diag=np.abs(np.diag(Af[:k, :k])), aw=Af @ w, atu=Af.T @ u,
               info=np.int32(info), work0=np.float64(work0))
    if full:
        out["af"] = Af
    return out


def main():
    if len(sys.argv) > 2 and sys.argv[1] == "--one":
        name = sys.argv[2]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **run_case(name))
        return
    import oracle
    if not oracle.reference_available():
        sys.exit("the reference must be buildable here (oracle/build.py)")
    # One process per case: the reference keeps static RNG state.
    for name in CASES:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--one", name], check=True)
    demo, jp = demo_7x5()
    ref = oracle.Reference()
    Af, jpvt, tau, info, work0 = ref.dgeqp4(demo, jp)
    np.savez_compressed(os.path.join(HERE, "dgeqp4_demo_7x5.npz"), a=demo, jpvt_in=jp, af=Af,
                        jpvt=jpvt, tau=tau, info=np.int32(info))
    G = ref.sketch(74, 2000)
    np.savez_compressed(os.path.join(HERE, "sketch_74x2000.npz"), head=G[:, :4].copy(),
                        colsum=G.sum(axis=0))


if __name__ == "__main__":
    main()
