"""The no-allocation entry point, hqrrp_gb300_qrp_noalloc, through the C ABI.

It exists for callers that cannot allocate device memory when they need a
pivoted QR -- a process whose device memory is all owned by its own arena, or
a loop that cannot take the device synchronisation or the failure modes of
cudaMalloc/cudaFree.  It must give the same factorization as the library's
allocating entry point for the same work (hqrrp_gb300_dgeqp4_device on a
matrix below dgeqp4's small-matrix threshold, all columns free), call after
call: its scratch is one shared device array that keeps the previous call's
contents.  This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the tolerance of the GPU parity tests


def _bind(L):
    f = L.hqrrp_gb300_qrp_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    g = L.hqrrp_gb300_dgeqp4_device
    g.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    g.restype = C.c_int
    return f, g


def _buffers(A):
    import torch
    m, n = A.shape
    At = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    jp = torch.zeros(n, dtype=torch.int32, device="cuda")
    tau = torch.zeros(min(m, n), dtype=torch.float64, device="cuda")
    return At, jp, tau


def _run(fn, A, bufs, stream):
    import torch
    m, n = A.shape
    At, jp, tau = bufs
    torch.cuda.synchronize()
    rc = fn(m, n, At.data_ptr(), m, jp.data_ptr(), tau.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc, At.cpu().numpy().T, jp.cpu().numpy(), tau.cpu().numpy()


def _same(a, b):
    """a, b = (A_out, jpvt, tau): jpvt identical, the rest within TOL."""
    np.testing.assert_array_equal(a[1], b[1])
    den = np.linalg.norm(b[0], axis=0)
    den[den == 0] = 1.0
    assert np.max(np.linalg.norm(a[0] - b[0], axis=0) / den) <= TOL
    assert np.max(np.abs(a[2] - b[2]) / np.maximum(np.abs(b[2]), 1e-300)) <= TOL


def test_noalloc_matches_allocating_entry_two_calls_in_a_row(hq):
    import torch
    noalloc, alloc = _bind(hq.load())
    stream = torch.cuda.current_stream().cuda_stream
    cases = [(700, 200, 31), (300, 256, 32)]  # two consecutive calls, different shapes
    inputs = [oracle.gaussian(m, n, seed) for m, n, seed in cases]
    want = []
    for A in inputs:
        rc, *out = _run(alloc, A, _buffers(A), stream)
        assert rc == 0, hq.last_error()
        want.append(out)
    bufs = [_buffers(A) for A in inputs]  # every device buffer exists before the calls
    free_before = None
    pool_before = hq.pool_alloc_count()
    for i, A in enumerate(inputs):
        if i == 1:  # after the one-time set-up done by the first call
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
        rc, *got = _run(noalloc, A, bufs[i], stream)
        assert rc == 0, hq.last_error()
        _same(got, want[i])
        assert oracle.quality(A, got[0], got[1], got[2])[0] < 1e-14
    torch.cuda.synchronize()
    assert hq.pool_alloc_count() == pool_before  # no allocation from the library's pools
    assert torch.cuda.mem_get_info()[0] == free_before  # the second call took no device memory


def test_noalloc_tall_matrix_in_place_panel(hq):
    """20000 x 256: a CTA's rows no longer fit its shared memory, so the
    kernel works on the matrix in place (global memory) -- the same results
    as the allocating entry point, again with no pool allocation."""
    import torch
    noalloc, alloc = _bind(hq.load())
    stream = torch.cuda.current_stream().cuda_stream
    A = oracle.gaussian(20000, 256, 34)
    rc, *want = _run(alloc, A, _buffers(A), stream)
    assert rc == 0, hq.last_error()
    bufs = _buffers(A)
    pool_before = hq.pool_alloc_count()
    rc, *got = _run(noalloc, A, bufs, stream)
    assert rc == 0, hq.last_error()
    assert hq.pool_alloc_count() == pool_before
    _same(got, want)
    assert oracle.quality(A, got[0], got[1], got[2])[0] < 1e-14


def test_noalloc_rejects_sizes_beyond_its_limit(hq):
    import torch
    noalloc, _ = _bind(hq.load())
    At = torch.zeros((257, 300), dtype=torch.float64, device="cuda")
    jp = torch.zeros(257, dtype=torch.int32, device="cuda")
    tau = torch.zeros(257, dtype=torch.float64, device="cuda")
    rc = noalloc(300, 257, At.data_ptr(), 300, jp.data_ptr(), tau.data_ptr(),
                 torch.cuda.current_stream().cuda_stream)
    assert rc == 3
    assert "exceeds" in hq.last_error()
    assert float(At.abs().sum()) == 0.0
