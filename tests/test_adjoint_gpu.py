"""The hand-written adjoint of the truncated factorization A P ~= Q_k R_k.

L = <W, Q_k R_k P^T> with the pivots fixed.  Checked (FP64) against
* central finite differences (h = 1e-6) of L through the GPU forward, which
  recomputes the pivots (they do not move for steps this small): relative
  error <= 1e-6 in each random direction;
* torch's FP64 autograd gradient of an unpivoted QR of A P (CPU):
  relative error <= 1e-10 normwise.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _t(A):
    import torch
    return torch.from_numpy(np.ascontiguousarray(A.T)).cuda()


def _problem(m, n, seed):
    rng = np.random.default_rng(seed)
    k = min(m, n)
    A = oracle.with_spectrum(m, n, (1.0 + np.arange(k)) ** -2.0, seed)
    W = rng.standard_normal((m, n))
    return A, W


def _loss_gpu(hq, A, W, k, nb):
    Ft, jp, tau = hq.truncated_factor(_t(A), k, nb)
    Ahat = hq.lowrank(Ft, jp, tau, k, nb).cpu().numpy().T
    return float(np.sum(W * Ahat)), jp.cpu().numpy()


@pytest.mark.parametrize("m,n,k,nb", [(300, 200, 64, 32), (256, 320, 48, 16), (500, 400, 100, 32)])
def test_adjoint_matches_unpivoted_qr_autograd(hq, m, n, k, nb):
    import torch
    A, W = _problem(m, n, m + n)
    At = _t(A)
    Ft, jp, tau = hq.truncated_factor(At, k, nb)
    G = hq.adjoint(At, Ft, jp, tau, _t(W), k, nb).cpu().numpy().T
    perm = jp.cpu().numpy() - 1
    At_cpu = torch.tensor(A, dtype=torch.float64, requires_grad=True)
    Q, _ = torch.linalg.qr(At_cpu[:, perm[:k]])
    L = (torch.tensor(W) * (Q @ (Q.T @ At_cpu))).sum()
    L.backward()
    ref = At_cpu.grad.numpy()
    assert np.linalg.norm(G - ref) <= 1e-10 * np.linalg.norm(ref)


def test_adjoint_matches_central_differences(hq):
    m, n, k, nb = 240, 180, 40, 16
    A, W = _problem(m, n, 5)
    At = _t(A)
    Ft, jp, tau = hq.truncated_factor(At, k, nb)
    G = hq.adjoint(At, Ft, jp, tau, _t(W), k, nb).cpu().numpy().T
    jp0 = jp.cpu().numpy()
    rng = np.random.default_rng(6)
    h = 1e-6
    for _ in range(3):
        E = rng.standard_normal((m, n))
        E /= np.linalg.norm(E)
        lp, jpp = _loss_gpu(hq, A + h * E, W, k, nb)
        lm, jpm = _loss_gpu(hq, A - h * E, W, k, nb)
        np.testing.assert_array_equal(jpp[:k], jp0[:k])
        np.testing.assert_array_equal(jpm[:k], jp0[:k])
        fd = (lp - lm) / (2 * h)
        an = float(np.sum(G * E))
        assert abs(fd - an) <= 1e-6 * max(abs(an), np.linalg.norm(G) * 1e-3), (fd, an)


def test_truncated_prefix_equals_full_run(hq):
    import torch
    m, n, k, nb = 400, 300, 96, 32
    A = oracle.gaussian(m, n, 9)
    Ft, jp, tau = hq.truncated_factor(_t(A), k, nb)
    Af = _t(A)
    jf = torch.arange(1, n + 1, dtype=torch.int32, device="cuda")
    tf = torch.zeros(n, dtype=torch.float64, device="cuda")
    hq.hqrrp_device(Af, jf, tf, nb, 10, 1)
    np.testing.assert_array_equal(jp.cpu().numpy()[:k], jf.cpu().numpy()[:k])
    # R_k P^T: the full run goes on permuting the trailing columns, so compare
    # the first k rows with their columns back in their original places.
    def rk_pt(F, j):
        M = np.zeros((k, n))
        M[:, j - 1] = np.triu(F.cpu().numpy().T[:k])
        return M
    R1, R2 = rk_pt(Ft, jp.cpu().numpy()), rk_pt(Af, jf.cpu().numpy())
    assert np.max(np.abs(R1 - R2)) <= 1e-13 * np.max(np.abs(R2))


def test_autograd_function(hq):
    import torch
    m, n, k = 200, 150, 32
    A, W = _problem(m, n, 12)
    Ad = torch.tensor(A, device="cuda", requires_grad=True)
    Ahat = hq.truncated_hqrrp(Ad, k, 32)
    L = (torch.tensor(W, device="cuda") * Ahat).sum()
    L.backward()
    At = _t(A)
    Ft, jp, tau = hq.truncated_factor(At, k, 32)
    G = hq.adjoint(At, Ft, jp, tau, _t(W), k, 32).cpu().numpy().T
    assert np.allclose(Ad.grad.cpu().numpy(), G, rtol=0, atol=1e-12 * np.abs(G).max())
    # the forward is the rank-k approximation: residual ~ sigma_{k+1}
    err = np.linalg.norm(Ahat.detach().cpu().numpy() - A, 2)
    assert err <= 3.0 * (k + 1.0) ** -2.0 * 10
