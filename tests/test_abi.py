"""The C-ABI library: builds, loads, exports every declared symbol, and
handles the argument paths that never reach the device exactly like the
reference (lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c:148-187,
:357-377)."""
import ctypes as C

import numpy as np
import pytest

from conftest import HAS_GPU


def test_library_exports_every_declared_symbol(hq):
    names = hq.declared_symbols()
    assert {"dgeqp4", "NoFLA_HQRRP_WY_blk_var4"} <= set(names)
    lib = C.CDLL(hq.LIB_PATH)
    for name in names:
        assert hasattr(lib, name), name


def test_library_exports_nothing_else(hq):
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", hq.LIB_PATH], capture_output=True,
                         text=True).stdout
    funcs = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert funcs == set(hq.declared_symbols())


def _dgeqp4_raw(hq, m, n, lda, lwork, jpvt=None):
    L = hq.load()
    A = np.zeros(max(1, lda * max(n, 1)))
    jp = np.zeros(max(1, n), np.int32) if jpvt is None else jpvt
    tau = np.zeros(max(1, min(m, n)))
    work = np.zeros(max(1, lwork, 1))
    mi, ni, ldi, lw, info = C.c_int(m), C.c_int(n), C.c_int(lda), C.c_int(lwork), C.c_int(7)
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    L.dgeqp4(C.byref(mi), C.byref(ni), A.ctypes.data_as(dp), C.byref(ldi),
             jp.ctypes.data_as(ip), tau.ctypes.data_as(dp), work.ctypes.data_as(dp),
             C.byref(lw), C.byref(info))
    return info.value, work[0]


@pytest.mark.parametrize("m,n,lda,lwork,expect", [(-1, 5, 1, 100, -1), (5, -1, 5, 100, -2),
                                                  (5, 4, 4, 100, -4), (10, 8, 10, 24, -8),
                                                  (0, 5, 1, 100, 0), (5, 0, 5, 100, 0)])
def test_dgeqp4_argument_errors_match_oracle(hq, oracle_lib, m, n, lda, lwork, expect):
    info, _ = _dgeqp4_raw(hq, m, n, lda, lwork)
    assert info == expect
    # the oracle (LAPACK-backed restatement) reports the same code
    L = oracle_lib.lib
    A = np.zeros(max(1, lda * max(n, 1)))
    jp = np.zeros(max(1, n), np.int32)
    tau = np.zeros(max(1, min(m, n)))
    work = np.zeros(max(1, lwork))
    mi, ni, ldi, lw, oinfo = C.c_int(m), C.c_int(n), C.c_int(lda), C.c_int(lwork), C.c_int(7)
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    L.oracle_dgeqp4(C.byref(mi), C.byref(ni), A.ctypes.data_as(dp), C.byref(ldi),
                    jp.ctypes.data_as(ip), tau.ctypes.data_as(dp), work.ctypes.data_as(dp),
                    C.byref(lw), C.byref(oinfo))
    assert oinfo.value == expect


@pytest.mark.parametrize("m,n", [(100, 80), (2000, 1500), (7, 5)])
def test_dgeqp4_workspace_query_matches_oracle(hq, oracle_lib, m, n):
    info, work0 = _dgeqp4_raw(hq, m, n, m, -1)
    assert info == 0
    _, _, _, oinfo, owork0 = oracle_lib.dgeqp4(np.zeros((m, n), order="F"), lwork=-1)
    assert oinfo == 0 and work0 == owork0 == 2 * n + (n + 1) * 32


def test_hqrrp_invalid_arguments_return_zero_untouched(hq):
    L = hq.load()
    A = np.arange(12, dtype=np.float64)
    jp = np.arange(1, 5, dtype=np.int32)
    tau = np.zeros(4)
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    for m, n, lda in [(-1, 4, 3), (3, -4, 3), (3, 4, 2)]:
        rc = L.NoFLA_HQRRP_WY_blk_var4(m, n, A.ctypes.data_as(dp), lda, jp.ctypes.data_as(ip),
                                       tau.ctypes.data_as(dp), 2, 1, 1)
        assert rc == 0
    np.testing.assert_array_equal(A, np.arange(12, dtype=np.float64))
    rc = L.NoFLA_HQRRP_WY_blk_var4(0, 4, A.ctypes.data_as(dp), 1, jp.ctypes.data_as(ip),
                                   tau.ctypes.data_as(dp), 2, 1, 1)
    assert rc == 0


@pytest.mark.skipif(HAS_GPU, reason="checks the no-GPU behaviour")
def test_no_gpu_fails_loudly(hq):
    """Without a device the library reports an error; it never computes on the CPU."""
    with pytest.raises(hq.HQRRPError):
        hq.hqrrp(np.eye(40), 8, 2)
    with pytest.raises(hq.HQRRPError):
        hq.dgeqp4(np.eye(40))


@pytest.mark.skipif(HAS_GPU, reason="checks the no-GPU behaviour")
def test_no_gpu_error_codes(hq):
    """Host-side failure: without a device, dgeqp4 returns info = 1000 + 1
    (a CUDA error) with a message, and the HQRRP entry its positive code."""
    info, _ = _dgeqp4_raw(hq, 40, 30, 40, 200)
    assert info == 1001
    assert "device" in hq.last_error()
    L = hq.load()
    A = np.eye(40)
    jp = np.arange(1, 41, dtype=np.int32)
    tau = np.zeros(40)
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    rc = L.NoFLA_HQRRP_WY_blk_var4(40, 40, A.ctypes.data_as(dp), 40, jp.ctypes.data_as(ip),
                                   tau.ctypes.data_as(dp), 8, 2, 1)
    assert rc == 1 and hq.last_error()
    np.testing.assert_array_equal(A, np.eye(40))


def test_dgeqp4_block_setter(hq):
    """Host-side state only: the previous value comes back, invalid sizes are
    refused and leave it unchanged."""
    assert hq.set_dgeqp4_block(64) == 128  # the GPU default
    with pytest.raises(ValueError):
        hq.set_dgeqp4_block(0)
    with pytest.raises(ValueError):
        hq.set_dgeqp4_block(247)
    assert hq.set_dgeqp4_block(128) == 64
