"""Batched pivoted QR: one persistent launch over many uneven matrices.

Each matrix must match LAPACK dgeqp3 (the reference dgeqp4's branch for
min(m, n) < 1000, ...var4.c:189-199) from the oracle's LAPACK: on Gaussian
inputs jpvt identical and tau / R / reflectors within 1e-12 relative per
column.  On the batched workload's spectrum (sigma_i = i^-2, condition up to
~2.6e5) the pivots must still be identical and each factorization must have
||AP - QR|| / ||A|| <= 1e-14 (its R differs from LAPACK's by ~cond * eps).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _shapes(count, seed, mmax=1024, nmax=512):
    rng = np.random.default_rng(seed)
    m = np.exp(rng.uniform(np.log(64), np.log(mmax), count)).astype(int)
    n = [int(np.exp(rng.uniform(np.log(32), np.log(min(mi, nmax))))) for mi in m]
    return [(int(a), int(b)) for a, b in zip(m, n)]


def _mats(shapes, seed, spectrum=False):
    """Gaussian matrices (well conditioned: the strict parity inputs), or the
    batched workload's A = U diag(i^-2) V^T with Haar U, V."""
    rng = np.random.default_rng(seed)
    out = []
    for m, n in shapes:
        k = min(m, n)
        if spectrum:
            out.append(oracle.with_spectrum(m, n, (1.0 + np.arange(k)) ** -2.0,
                                            int(rng.integers(1 << 30))))
        else:
            out.append(oracle.gaussian(m, n, int(rng.integers(1 << 30))))
    return out


def _device(A):
    import torch
    return torch.from_numpy(np.ascontiguousarray(A.T)).cuda()


def _check(A, Af, jp, tau, want):
    Ao, jo, to, _ = want
    np.testing.assert_array_equal(jp, jo)
    k = min(A.shape)
    assert np.max(np.abs(tau[:k] - to) / np.maximum(np.abs(to), 1e-300)) <= TOL
    den = np.linalg.norm(Ao, axis=0)
    den[den == 0] = 1
    assert np.max(np.linalg.norm(Af - Ao, axis=0) / den) <= TOL


def test_batched_matches_lapack_dgeqp3(hq, oracle_lib):
    import torch
    shapes = _shapes(48, 1) + [(7, 5), (64, 100), (300, 300), (1024, 512), (5, 1), (1, 4)]
    As = _mats(shapes, 2)
    bq = hq.BatchedQRP(shapes, autotune=False)
    mats = [_device(A) for A in As]
    jp, tau, info = bq.run(mats)
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    for A, t, j, ta in zip(As, mats, jp, tau):
        _check(A, t.cpu().numpy().T, j.cpu().numpy(), ta.cpu().numpy(), oracle_lib.dgeqp3(A))


def test_batched_every_launch_shape_agrees(hq):
    import torch
    shapes = _shapes(40, 3)
    As = _mats(shapes, 4)
    ref = None
    L = hq.load()
    nshapes = L.hqrrp_gb300_qrp_batched_config(0, None, None, None)
    for cfg in range(nshapes):
        bq = hq.BatchedQRP(shapes, autotune=False)
        bq.cfg = cfg
        mats = [_device(A) for A in As]
        try:
            jp, tau, info = bq.run(mats)
        except hq.HQRRPError:
            continue  # a shape this device cannot launch
        torch.cuda.synchronize()
        got = [(t.cpu().numpy().T, j.cpu().numpy(), ta.cpu().numpy()) for t, j, ta in
               zip(mats, jp, tau)]
        if ref is None:
            ref = got
            continue
        for (a, j, t), (a0, j0, t0) in zip(got, ref):
            np.testing.assert_array_equal(j, j0)
            assert np.max(np.abs(a - a0)) <= 1e-12 * max(1.0, np.max(np.abs(a0)))
    assert ref is not None


def test_batched_workload_spectrum_quality(hq, oracle_lib):
    import torch
    shapes = _shapes(40, 7)
    As = _mats(shapes, 8, spectrum=True)
    bq = hq.BatchedQRP(shapes, autotune=False)
    mats = [_device(A) for A in As]
    jp, tau, info = bq.run(mats)
    torch.cuda.synchronize()
    for A, t, j, ta in zip(As, mats, jp, tau):
        Af, jj, tt = t.cpu().numpy().T, j.cpu().numpy(), ta.cpu().numpy()
        np.testing.assert_array_equal(jj, oracle_lib.dgeqp3(A)[1])
        res, orth, _ = oracle.quality(A, Af, jj, tt[:min(A.shape)])
        assert res <= 1e-14 and orth <= 1e-13


def test_batched_autotune_and_cuda_graph(hq, oracle_lib):
    import torch
    shapes = _shapes(64, 5)
    As = _mats(shapes, 6)
    bq = hq.BatchedQRP(shapes, autotune=True)
    assert 0 <= bq.cfg and bq.config()["threads"] in (128, 256, 512)
    mats = [_device(A) for A in As]
    originals = [m.clone() for m in mats]
    bq.bind(mats)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        bq.run(stream=s)  # warm-up outside capture
    torch.cuda.synchronize()
    for m, o in zip(mats, originals):
        m.copy_(o)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        bq.run(stream=s)
    for _ in range(2):  # replay twice on fresh inputs
        for m, o in zip(mats, originals):
            m.copy_(o)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        for A, t, j, ta in zip(As, mats, bq.jpvt, bq.tau):
            _check(A, t.cpu().numpy().T, j.cpu().numpy(), ta.cpu().numpy(),
                   oracle_lib.dgeqp3(A))
