"""Failure paths, exercised without faulting or hanging the GPU.

* Bounded waits: every grid barrier of the cooperative kernels gives up after
  an iteration cap (hqrrp_gb300_set_spin_limit).  With the cap at 1 the
  barriers of the plain FP64 path run out: the kernels record
  HQ_ERR_BARRIER_TIMEOUT in the call's error word and return, the call
  reports it (return code 2 / dgeqp4 info 1002, message), and the next call
  on the same context runs normally.  Only the plain path is used here: its
  kernels have no bulk copies or tensor-core operations in flight when a
  wait gives up.
* Allocation failure, injected on the host (HQRRP_GB300_FAIL_ALLOC=k fails the
  k-th device allocation of each call): return code 4 / info 1004 with a
  message, no partial result is reported as success, and the next call
  without the injection succeeds.
* A batched item with a size the kernel cannot take (lda < m) is flagged in
  its info word and left untouched; the other items are factored.
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture
def plain(hq):
    prev = hq.set_precision(hq.PLAIN)
    yield hq
    hq.set_precision(prev)
    hq.set_spin_limit(0)
    os.environ.pop("HQRRP_GB300_FAIL_ALLOC", None)


def test_barrier_timeout_is_reported_and_context_survives(plain):
    hq = plain
    A = oracle.gaussian(1000, 800, 71)
    ref = hq.hqrrp(A, 64, 10, 1)
    hq.set_spin_limit(1)
    try:
        with pytest.raises(hq.HQRRPError) as ei:
            hq.hqrrp(A, 64, 10, 1)
    finally:
        hq.set_spin_limit(0)
    msg = str(ei.value)
    assert "(2)" in msg and "barrier" in msg, msg
    again = hq.hqrrp(A, 64, 10, 1)
    for x, y in zip(again, ref):
        np.testing.assert_array_equal(x, y)


def test_barrier_timeout_in_dgeqp4_small_path(plain):
    hq = plain
    A = oracle.gaussian(600, 500, 72)
    ref = hq.dgeqp4(A)
    hq.set_spin_limit(1)
    try:
        with pytest.raises(hq.HQRRPError) as ei:
            hq.dgeqp4(A)
    finally:
        hq.set_spin_limit(0)
    assert "info=1002" in str(ei.value), str(ei.value)
    again = hq.dgeqp4(A)
    for x, y in zip(again[:3], ref[:3]):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("k", [1, 5])
def test_injected_allocation_failure(plain, k):
    hq = plain
    A = oracle.gaussian(1200, 1100, 73)
    ref = hq.dgeqp4(A)
    before = hq.pool_alloc_count()
    os.environ["HQRRP_GB300_FAIL_ALLOC"] = str(k)
    try:
        with pytest.raises(hq.HQRRPError) as e1:
            hq.dgeqp4(A)
        with pytest.raises(hq.HQRRPError) as e2:
            hq.hqrrp(A, 64, 10, 1)
    finally:
        os.environ.pop("HQRRP_GB300_FAIL_ALLOC", None)
    assert "info=1004" in str(e1.value) and "injected" in str(e1.value), str(e1.value)
    assert "(4)" in str(e2.value) and "injected" in str(e2.value), str(e2.value)
    assert hq.pool_alloc_count() - before == 2 * (k - 1)  # the successful ones only
    again = hq.dgeqp4(A)
    for x, y in zip(again[:3], ref[:3]):
        np.testing.assert_array_equal(x, y)


def test_batched_bad_lda_is_flagged(hq, oracle_lib):
    import torch
    shapes = [(300, 200), (150, 120), (400, 90)]
    As = [oracle.gaussian(m, n, 80 + i) for i, (m, n) in enumerate(shapes)]
    bq = hq.BatchedQRP(shapes, autotune=False)
    bq.d_lda[1] = shapes[1][0] - 1  # lda < m for item 1
    mats = [torch.from_numpy(np.ascontiguousarray(A.T)).cuda() for A in As]
    before = mats[1].clone()
    jp, tau, info = bq.run(mats)
    torch.cuda.synchronize()
    info = info.cpu().numpy()
    assert info[0] == 0 and info[2] == 0 and info[1] == 0x4802, info
    assert torch.equal(mats[1], before)
    for i in (0, 2):
        np.testing.assert_array_equal(jp[i].cpu().numpy(), oracle_lib.dgeqp3(As[i])[1])
