"""The measured workloads at their own sizes, checked for correctness.

* Mixed precision, 32768 x 8192, sigma geometric from 1 to 1e-10 plus 64
  equal values at 1e-4 (Haar U, V): ||AP - QR||_F / ||A||_F <= 1e-13,
  ||Q^T Q - I||_F <= 1e-12, and |R_kk| within a factor 2 of the plain FP64
  path's.  Q is formed by torch's householder_product (cuSOLVER) from the
  returned reflectors, so the check does not use the library's own Q code.
* Batched: the 4096-matrix workload (m log-uniform in [64, 1024], n
  log-uniform in [32, min(m, 512)], A = U diag(i^-2) V^T) in one persistent
  launch; every matrix reports info 0, and a strided sample of 256 matrices
  has jpvt identical to LAPACK dgeqp3 (the reference dgeqp4's branch for these
  sizes) and ||AP - QR|| / ||A|| <= 1e-14.
* Adjoint: the truncated rank-256 factorization of a 4096 x 2048 matrix with
  sigma_i = i^-2: the gradient of L = <W, Q_k R_k P^T> (pivots fixed) against
  torch's FP64 autograd of an unpivoted QR of A P (relative 1e-10 normwise)
  and against a central difference (h = 1e-6) of that fixed-pivot loss.  The
  difference quotient itself carries a rounding error of about
  kappa(R_11) * eps * |L| / h: the loss goes through a QR of A P's first 256
  columns, whose condition is sigma_1 / sigma_256 ~ 6.5e4, so |L| ~ 1 is known
  to ~1e-11 and the quotient to ~1e-5.  Its bar is therefore 3e-4 relative
  (the small cases in test_adjoint_gpu.py keep 1e-6).
"""
import numpy as np
import pytest

import bench
import oracle

pytestmark = pytest.mark.gpu


def _quality_torch(At0, Ft, jp, tau):
    """Exact ||AP - QR||_F / ||A||_F, ||Q^T Q - I||_F and |diag R| on the GPU."""
    import torch
    n, m = At0.shape
    k = min(m, n)
    F = Ft.T
    Q = torch.linalg.householder_product(F[:, :k].contiguous(), tau[:k])
    R = torch.triu(F[:k, :])
    AP = At0.T[:, jp.long() - 1]
    res = float(torch.linalg.norm(AP - Q @ R) / torch.linalg.norm(At0))
    orth = float(torch.linalg.norm(Q.T @ Q - torch.eye(k, dtype=Q.dtype, device=Q.device)))
    return res, orth, torch.abs(torch.diagonal(R)).cpu().numpy()


def test_mixed_tall_workload_full_size(hq):
    import torch
    m, n, nb, pp = 32768, 8192, 128, 10
    sigma = bench.spectrum_tall(n)
    At0 = bench.make_matrix_gpu(m, n, sigma, 2026, torch.device("cuda"))
    out = {}
    for prec in (hq.PLAIN, hq.MIXED):
        hq.set_precision(prec)
        try:
            At = At0.clone()
            jp = torch.arange(1, n + 1, dtype=torch.int32, device="cuda")
            tau = torch.zeros(n, dtype=torch.float64, device="cuda")
            hq.hqrrp_device(At, jp, tau, nb, pp, 1)
            torch.cuda.synchronize()
        finally:
            hq.set_precision(hq.PLAIN)
        out[prec] = _quality_torch(At0, At, jp, tau)
        del At
    res, orth, d = out[hq.MIXED]
    _, _, dp = out[hq.PLAIN]
    assert res <= 1e-13 and orth <= 1e-12, (res, orth)
    ratio = d / dp
    assert 0.5 <= ratio.min() and ratio.max() <= 2.0, (ratio.min(), ratio.max())
    # rank revealing through the 64-value cluster at 1e-4
    r = d / sigma
    assert r.min() > 0.05 and r.max() < 20, (r.min(), r.max())


def test_batched_workload_full_size(hq, oracle_lib):
    import torch
    shapes = bench.batched_shapes(4096, 2026)
    flat0, offs = bench.make_batched_gpu(shapes, 2026, torch.device("cuda"))
    flat = flat0.clone()
    mats = [flat[offs[i]:offs[i + 1]].view(n, m) for i, (m, n) in enumerate(shapes)]
    bq = hq.BatchedQRP(shapes, autotune=True)
    jpvt, tau, info = bq.run(mats)
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    for i in range(0, len(shapes), 16):  # 256 matrices
        m, n = shapes[i]
        A = np.asfortranarray(flat0[offs[i]:offs[i + 1]].view(n, m).cpu().numpy().T)
        Ao, jo, to, io = oracle_lib.dgeqp3(A)
        assert io == 0
        jg = jpvt[i].cpu().numpy()
        np.testing.assert_array_equal(jg, jo, err_msg="matrix %d (%d x %d)" % (i, m, n))
        Af = mats[i].cpu().numpy().T
        res, orth, _ = oracle.quality(A, Af, jg, tau[i].cpu().numpy())
        assert res <= 1e-14 and orth <= 1e-13, (i, res, orth)


def test_adjoint_workload_full_size(hq):
    import torch
    m, n, k, nb = 4096, 2048, 256, 64
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(7)
    U, V = bench._orth(m, n, g, dev), bench._orth(n, n, g, dev)
    sig = (1.0 + torch.arange(n, dtype=torch.float64, device=dev)) ** -2.0
    At = ((V * sig[None, :]) @ U.T).contiguous()  # column-major A
    Wt = torch.randn(n, m, dtype=torch.float64, device=dev, generator=g)
    del U, V
    Ft, jp, tau = hq.truncated_factor(At, k, nb)
    Gt = hq.adjoint(At, Ft, jp, tau, Wt, k, nb)
    torch.cuda.synchronize()
    perm = jp.long() - 1
    A = At.T.detach().clone().requires_grad_(True)
    W = Wt.T

    def loss(X):
        Q, _ = torch.linalg.qr(X[:, perm[:k]])
        return (W * (Q @ (Q.T @ X))).sum()

    L = loss(A)
    L.backward()
    ref = A.grad
    G = Gt.T
    assert float(torch.linalg.norm(G - ref) / torch.linalg.norm(ref)) <= 1e-10
    # the forward of the library is that loss at A (pivots of the same run)
    Ahat = hq.lowrank(Ft, jp, tau, k, nb).T
    Lv = float(L.detach())
    assert abs(float((W * Ahat).sum()) - Lv) <= 1e-10 * abs(Lv)
    # central difference of the fixed-pivot loss in one random direction
    E = torch.randn(m, n, dtype=torch.float64, device=dev, generator=g)
    E /= torch.linalg.norm(E)
    h = 1e-6
    with torch.no_grad():
        fd = (float(loss(At.T + h * E)) - float(loss(At.T - h * E))) / (2 * h)
    an = float((G * E).sum())
    assert abs(fd - an) <= 3e-4 * abs(an), (fd, an)
