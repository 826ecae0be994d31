"""CPU oracle for HQRRP -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline /
reference arm of ``bench.py`` import this package, and only as the checker
(or, in bench.py, as the timed CPU baseline).  The product library never
imports it.

Two implementations sit behind the same Python interface:

* :class:`Oracle` -- ``hqrrp_oracle.c``, a restatement of the reference
  algorithm (``lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c``) that
  calls the same LAPACK/BLAS routines in the same order.  It builds on any
  host, including the aarch64 GPU host.
* :class:`Reference` -- the unmodified reference source compiled by
  ``oracle/build.py`` into ``oracle/_ref/``; present only where the
  reference tree is.

All matrices are Fortran-ordered float64 numpy arrays; pivots are int32.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _dptr(a):
    return a.ctypes.data_as(_dp)


def _iptr(a):
    return a.ctypes.data_as(_ip)


def _fortran(A):
    A = np.asarray(A, dtype=np.float64)
    return np.array(A, order="F", copy=True)


class _Base:
    """Shared numpy-facing calls; subclasses bind the symbol names."""

    lib = None
    _hqrrp_name = None
    _dgeqp4_name = None
    _sketch_name = None

    def _bind(self):
        L = self.lib
        f = getattr(L, self._hqrrp_name)
        f.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip, _dp, C.c_int, C.c_int, C.c_int]
        f.restype = C.c_int
        self._hqrrp = f
        g = getattr(L, self._dgeqp4_name)
        g.argtypes = [_ip, _ip, _dp, _ip, _ip, _dp, _dp, _ip, _ip]
        g.restype = None
        self._dgeqp4 = g
        s = getattr(L, self._sketch_name)
        s.argtypes = [C.c_int, C.c_int, _dp]
        s.restype = None
        self._sketch = s

    # -- the two reference entry points ------------------------------------
    def hqrrp(self, A, nb=64, pp=10, panel_pivoting=1, jpvt=None):
        """NoFLA_HQRRP_WY_blk_var4 on a copy of A; returns (A_out, jpvt, tau).

        jpvt defaults to 1..n (the reference carries incoming labels)."""
        A = _fortran(A)
        m, n = A.shape
        jp = (np.arange(1, n + 1, dtype=np.int32) if jpvt is None
              else np.array(jpvt, dtype=np.int32, copy=True))
        tau = np.zeros(max(1, min(m, n)), dtype=np.float64)
        self._hqrrp(m, n, _dptr(A), max(1, m), _iptr(jp), _dptr(tau), nb, pp, panel_pivoting)
        return A, jp, tau[:min(m, n)]

    def dgeqp4(self, A, jpvt=None, lwork=None):
        """dgeqp4 on a copy of A; returns (A_out, jpvt, tau, info, work0)."""
        A = _fortran(A)
        m, n = A.shape
        jp = (np.zeros(n, dtype=np.int32) if jpvt is None
              else np.array(jpvt, dtype=np.int32, copy=True))
        tau = np.zeros(max(1, min(m, n)), dtype=np.float64)
        if lwork is None:
            lwork = max(1, 3 * n + 1, 2 * n + (n + 1) * 64)
        work = np.zeros(max(1, lwork), dtype=np.float64)
        mi, ni, ldi, lw, info = (C.c_int(m), C.c_int(n), C.c_int(max(1, m)), C.c_int(lwork),
                                 C.c_int(0))
        self._dgeqp4(C.byref(mi), C.byref(ni), _dptr(A), C.byref(ldi), _iptr(jp), _dptr(tau),
                     _dptr(work), C.byref(lw), C.byref(info))
        return A, jp, tau[:min(m, n)], info.value, work[0]

    def timed_dgeqp4(self, A):
        """dgeqp4 in place on the Fortran-ordered float64 array A, all columns
        free; returns the seconds spent in the call (for the CPU baselines)."""
        import time
        assert A.flags.f_contiguous and A.dtype == np.float64
        m, n = A.shape
        jp = np.zeros(max(1, n), dtype=np.int32)
        tau = np.zeros(max(1, min(m, n)))
        lwork = max(1, 3 * n + 1, 2 * n + (n + 1) * 64)
        work = np.zeros(lwork)
        mi, ni, ldi, lw, info = (C.c_int(m), C.c_int(n), C.c_int(max(1, m)), C.c_int(lwork),
                                 C.c_int(0))
        t0 = time.perf_counter()
        self._dgeqp4(C.byref(mi), C.byref(ni), _dptr(A), C.byref(ldi), _iptr(jp), _dptr(tau),
                     _dptr(work), C.byref(lw), C.byref(info))
        dt = time.perf_counter() - t0
        if info.value != 0:
            raise RuntimeError("dgeqp4 info %d" % info.value)
        return dt

    def timed_hqrrp(self, A, nb, pp, panel_pivoting=1):
        """NoFLA_HQRRP_WY_blk_var4 in place on A; returns the seconds of the call."""
        import time
        assert A.flags.f_contiguous and A.dtype == np.float64
        m, n = A.shape
        jp = np.arange(1, n + 1, dtype=np.int32)
        tau = np.zeros(max(1, min(m, n)))
        t0 = time.perf_counter()
        self._hqrrp(m, n, _dptr(A), max(1, m), _iptr(jp), _dptr(tau), nb, pp, panel_pivoting)
        return time.perf_counter() - t0

    def sketch(self, mY, m):
        """The (mY x m) Gaussian sketch the reference draws on entry."""
        G = np.zeros((mY, m), dtype=np.float64, order="F")
        self._sketch(mY, m, _dptr(G))
        return G


class Oracle(_Base):
    """The restatement (oracle/hqrrp_oracle.c) over a run-time LAPACK."""

    _hqrrp_name = "oracle_hqrrp"
    _dgeqp4_name = "oracle_dgeqp4"
    _sketch_name = "oracle_sketch"

    def __init__(self, lapack_path=None):
        so = _build.build_oracle()
        self.lib = C.CDLL(so, mode=C.RTLD_LOCAL)
        self.lapack_path = lapack_path or _build.find_openblas()
        if self.lapack_path is None:
            raise RuntimeError("no LP64 LAPACK (scipy's bundled OpenBLAS) found for the oracle")
        self.lib.oracle_open.argtypes = [C.c_char_p]
        rc = self.lib.oracle_open(self.lapack_path.encode())
        if rc != 0:
            raise RuntimeError("oracle_open(%s) failed: %d" % (self.lapack_path, rc))
        self._bind()
        f = self.lib.oracle_hqrrp_sketch
        f.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip, _dp, C.c_int, C.c_int, C.c_int, _dp,
                      C.c_int]
        f.restype = C.c_int
        self._hqrrp_sketch = f
        f = self.lib.oracle_hqrrp_ut_sketch
        f.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip, _dp, C.c_int, C.c_int, C.c_int, _dp,
                      C.c_int]
        f.restype = C.c_int
        self._hqrrp_ut = f
        for name in ("oracle_dgeqp3",):
            g = getattr(self.lib, name)
            g.argtypes = [_ip, _ip, _dp, _ip, _ip, _dp, _dp, _ip, _ip]
        self.lib.oracle_dgeqpf.argtypes = [_ip, _ip, _dp, _ip, _ip, _dp, _dp, _ip]
        self.lib.oracle_dgeqp4_sketch.argtypes = [_ip, _ip, _dp, _ip, _ip, _dp, _dp, _ip, _ip,
                                                  _dp, C.c_int]
        self.lib.oracle_dgeqp4_sketch.restype = None
        self.lib.oracle_set_threads.argtypes = [C.c_int]

    def set_threads(self, n):
        return self.lib.oracle_set_threads(int(n))

    def hqrrp_sketch(self, A, G, nb=64, pp=10, panel_pivoting=1, jpvt=None):
        """HQRRP with an explicit sketch G ((nb+pp) x m) in place of the drawn one."""
        A = _fortran(A)
        G = _fortran(G)
        m, n = A.shape
        assert G.shape == (nb + pp, m)
        jp = (np.arange(1, n + 1, dtype=np.int32) if jpvt is None
              else np.array(jpvt, dtype=np.int32, copy=True))
        tau = np.zeros(max(1, min(m, n)), dtype=np.float64)
        self._hqrrp_sketch(m, n, _dptr(A), max(1, m), _iptr(jp), _dptr(tau), nb, pp,
                           panel_pivoting, _dptr(G), nb + pp)
        return A, jp, tau[:min(m, n)]

    def hqrrp_ut(self, A, nb=64, pp=10, panel_pivoting=1, p=None, G=None):
        """The UT-transform variant (FLA_HQRRP_UT_blk_var2) on a copy of A;
        returns (A_out, p, s) with s the UT scalars.  G: optional explicit sketch."""
        A = _fortran(A)
        m, n = A.shape
        pv = (np.arange(1, n + 1, dtype=np.int32) if p is None
              else np.array(p, dtype=np.int32, copy=True))
        s = np.zeros(max(1, min(m, n)), dtype=np.float64)
        if G is None:
            self._hqrrp_ut(m, n, _dptr(A), max(1, m), _iptr(pv), _dptr(s), nb, pp,
                           panel_pivoting, None, 0)
        else:
            G = _fortran(G)
            assert G.shape == (nb + pp, m)
            self._hqrrp_ut(m, n, _dptr(A), max(1, m), _iptr(pv), _dptr(s), nb, pp,
                           panel_pivoting, _dptr(G), nb + pp)
        return A, pv, s[:min(m, n)]

    def dgeqp4_sketch(self, A, G, jpvt=None):
        """dgeqp4 whose HQRRP branch uses the sketch G (74 x (m - nf)) in place of
        the drawn one; returns (A_out, jpvt, tau, info, work0)."""
        A = _fortran(A)
        G = _fortran(G)
        m, n = A.shape
        assert G.shape[0] == 74
        jp = (np.zeros(n, dtype=np.int32) if jpvt is None
              else np.array(jpvt, dtype=np.int32, copy=True))
        tau = np.zeros(max(1, min(m, n)), dtype=np.float64)
        lwork = max(1, 3 * n + 1, 2 * n + (n + 1) * 64)
        work = np.zeros(lwork, dtype=np.float64)
        mi, ni, ldi, lw, info = (C.c_int(m), C.c_int(n), C.c_int(max(1, m)), C.c_int(lwork),
                                 C.c_int(0))
        self.lib.oracle_dgeqp4_sketch(C.byref(mi), C.byref(ni), _dptr(A), C.byref(ldi),
                                      _iptr(jp), _dptr(tau), _dptr(work), C.byref(lw),
                                      C.byref(info), _dptr(G), 74)
        return A, jp, tau[:min(m, n)], info.value, work[0]

    def timed_dgeqp3(self, A):
        """LAPACK dgeqp3 in place on A (all columns free); returns seconds."""
        import time
        assert A.flags.f_contiguous and A.dtype == np.float64
        m, n = A.shape
        jp = np.zeros(max(1, n), dtype=np.int32)
        tau = np.zeros(max(1, min(m, n)))
        lwork = max(1, 3 * n + 1 + (n + 1) * 64)
        work = np.zeros(lwork)
        mi, ni, ldi, lw, info = C.c_int(m), C.c_int(n), C.c_int(max(1, m)), C.c_int(lwork), C.c_int(0)
        t0 = time.perf_counter()
        self.lib.oracle_dgeqp3(C.byref(mi), C.byref(ni), _dptr(A), C.byref(ldi), _iptr(jp),
                               _dptr(tau), _dptr(work), C.byref(lw), C.byref(info))
        return time.perf_counter() - t0

    def dgeqp3(self, A, jpvt=None):
        A = _fortran(A)
        m, n = A.shape
        jp = (np.zeros(n, dtype=np.int32) if jpvt is None
              else np.array(jpvt, dtype=np.int32, copy=True))
        tau = np.zeros(max(1, min(m, n)))
        lwork = max(1, 3 * n + 1 + (n + 1) * 64)
        work = np.zeros(lwork)
        mi, ni, ldi, lw, info = C.c_int(m), C.c_int(n), C.c_int(max(1, m)), C.c_int(lwork), C.c_int(0)
        self.lib.oracle_dgeqp3(C.byref(mi), C.byref(ni), _dptr(A), C.byref(ldi), _iptr(jp),
                               _dptr(tau), _dptr(work), C.byref(lw), C.byref(info))
        return A, jp, tau[:min(m, n)], info.value

    def dgeqpf(self, A, jpvt=None):
        A = _fortran(A)
        m, n = A.shape
        jp = (np.zeros(n, dtype=np.int32) if jpvt is None
              else np.array(jpvt, dtype=np.int32, copy=True))
        tau = np.zeros(max(1, min(m, n)))
        work = np.zeros(max(1, 3 * n))
        mi, ni, ldi, info = C.c_int(m), C.c_int(n), C.c_int(max(1, m)), C.c_int(0)
        self.lib.oracle_dgeqpf(C.byref(mi), C.byref(ni), _dptr(A), C.byref(ldi), _iptr(jp),
                               _dptr(tau), _dptr(work), C.byref(info))
        return A, jp, tau[:min(m, n)], info.value


class Reference(_Base):
    """The unmodified reference compiled into oracle/_ref/libhqrrp_ref.so."""

    _hqrrp_name = "NoFLA_HQRRP_WY_blk_var4"
    _dgeqp4_name = "dgeqp4"
    _sketch_name = "oracle_reference_sketch"

    def __init__(self):
        so = _build.build_reference()
        if so is None or not os.path.exists(so):
            raise RuntimeError("reference library not available on this host")
        self.lib = C.CDLL(so, mode=C.RTLD_LOCAL)
        self._bind()

    def set_threads(self, n):
        f = getattr(self.lib, "scipy_openblas_set_num_threads", None)
        if f is None:
            return -1
        f.argtypes = [C.c_int]
        f(int(n))
        return 0


def reference_available():
    try:
        return _build.build_reference() is not None
    except RuntimeError:
        return False


# -- matrix generators and quality metrics shared by tests and bench -------

def gaussian(m, n, seed):
    """i.i.d. N(0,1), Fortran order, from numpy's PCG64 stream."""
    return np.asfortranarray(np.random.default_rng(seed).standard_normal((m, n)))


def haar_orthogonal(n, rng):
    """Haar-distributed orthogonal matrix: QR of a Gaussian with sign fix."""
    Z = rng.standard_normal((n, n))
    Q, R = np.linalg.qr(Z)
    return Q * np.sign(np.diag(R))[None, :]


def with_spectrum(m, n, sigma, seed):
    """A = U diag(sigma) V^T with Haar U (m x k), V (n x k), k = len(sigma)."""
    rng = np.random.default_rng(seed)
    k = len(sigma)
    U = haar_orthogonal(m, rng)[:, :k]
    V = haar_orthogonal(n, rng)[:, :k]
    return np.asfortranarray((U * np.asarray(sigma)[None, :]) @ V.T)


def form_q(Af, tau):
    """Explicit thin Q from the Householder vectors under the diagonal."""
    import scipy.linalg.lapack as la
    m, n = Af.shape
    k = min(m, n)
    Q, _, info = la.dorgqr(np.array(Af[:, :k], order="F"), tau[:k])
    assert info == 0
    return Q


def quality(A0, Af, jpvt, tau):
    """(||AP - QR||_F / ||A||_F, ||Q^T Q - I||_F, |diag R|)."""
    m, n = A0.shape
    k = min(m, n)
    Q = form_q(Af, tau)
    R = np.triu(Af[:k, :])
    AP = A0[:, np.asarray(jpvt) - 1]
    res = np.linalg.norm(AP - Q @ R) / np.linalg.norm(A0)
    orth = np.linalg.norm(Q.T @ Q - np.eye(k))
    return res, orth, np.abs(np.diag(R))
