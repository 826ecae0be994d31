"""Q formation and application on the GPU (LAPACK dorgqr / dormqr side 'L').

The reflectors come from the GPU factorization; the check is LAPACK's dorgqr
on the same reflectors (scipy), to 1e-13, and Q^T Q = I.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _factor(hq, m, n, nb, seed):
    import torch
    A = oracle.gaussian(m, n, seed)
    At = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    jp = torch.arange(1, n + 1, dtype=torch.int32, device="cuda")
    tau = torch.zeros(max(1, min(m, n)), dtype=torch.float64, device="cuda")
    hq.hqrrp_device(At, jp, tau, nb, 10, 1)
    return A, At, jp, tau


@pytest.mark.parametrize("m,n,nb", [(300, 200, 32), (257, 257, 64), (200, 330, 16), (1000, 64, 64)])
def test_form_q_matches_dorgqr(hq, m, n, nb):
    A, Ft, jp, tau = _factor(hq, m, n, nb, m * 7 + n)
    k = min(m, n)
    Q = hq.form_q(Ft, tau, k, nb).cpu().numpy().T
    Qref = oracle.form_q(Ft.cpu().numpy().T, tau.cpu().numpy())
    assert np.max(np.abs(Q - Qref)) <= 1e-13
    assert np.linalg.norm(Q.T @ Q - np.eye(k)) <= 1e-13 * k


@pytest.mark.parametrize("trans", ["N", "T"])
def test_apply_q_matches_dense(hq, trans):
    import torch
    m, n, nb, nc = 400, 300, 32, 37
    A, Ft, jp, tau = _factor(hq, m, n, nb, 3)
    k = min(m, n)
    Qfull = oracle.form_q(np.hstack([Ft.cpu().numpy().T, np.zeros((m, m - n))]),
                          np.concatenate([tau.cpu().numpy(), np.zeros(m - n)]))
    C = np.random.default_rng(4).standard_normal((m, nc))
    Ct = torch.from_numpy(np.ascontiguousarray(C.T)).cuda()
    hq.apply_q(Ft, tau, Ct, trans, k, nb)
    ref = (Qfull if trans == "N" else Qfull.T) @ C
    assert np.max(np.abs(Ct.cpu().numpy().T - ref)) <= 1e-13 * np.abs(ref).max()


def test_apply_q_round_trip_and_reconstruction(hq):
    import torch
    m, n, nb = 520, 520, 64
    A, Ft, jp, tau = _factor(hq, m, n, nb, 8)
    X = torch.randn(5, m, dtype=torch.float64, device="cuda")
    Y = X.clone()
    hq.apply_q(Ft, tau, Y, "T", None, nb)
    hq.apply_q(Ft, tau, Y, "N", None, nb)
    assert float((Y - X).norm() / X.norm()) <= 1e-14
    # Q R = A P column by column
    R = torch.triu(Ft.T)  # m x n
    QR = R.T.contiguous()  # (n, m) = column-major R
    hq.apply_q(Ft, tau, QR, "N", None, nb)
    AP = torch.from_numpy(np.ascontiguousarray(A[:, jp.cpu().numpy() - 1].T)).cuda()
    assert float((QR - AP).norm() / AP.norm()) <= 1e-14
