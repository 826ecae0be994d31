"""GB300-native HQRRP: Python mirror of the C ABI in include/hqrrp_gb300.h.

The product is ``libhqrrp_gb300.so`` (C host driver + sm_103a CUDA kernels).
This module only loads it with ctypes and offers numpy / torch-facing calls
that mirror the reference's two entry points
(``lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c``: ``dgeqp4`` :127-300,
``NoFLA_HQRRP_WY_blk_var4`` :303-571) with the same argument meaning and error
behaviour.  There is no CPU fallback: if the library is missing or the GPU
fails, calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhqrrp_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "hqrrp_gb300.h")

PLAIN, MIXED = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None

DOUBLE, INT = 1, 2  # hqrrp_gb300_obj datatypes


class Obj(C.Structure):
    """hqrrp_gb300_obj: a view (the fields libflame's FLA_Obj exposes)."""
    _fields_ = [("datatype", C.c_int), ("m", C.c_int), ("n", C.c_int),
                ("col_stride", C.c_int), ("buffer", C.c_void_p)]


class HQRRPError(RuntimeError):
    """A device or shape error reported by libhqrrp_gb300.so."""


def build(force=False):
    """Compile libhqrrp_gb300.so for sm_103a (nvcc); returns its path."""
    from . import buildlib as _b
    return _b.build(force=force)


def load():
    """Load libhqrrp_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise HQRRPError("libhqrrp_gb300.so not built (run hqrrp_gb300.build() / "
                         "__graft_entry__.build())")
    L = C.CDLL(LIB_PATH, mode=C.RTLD_LOCAL)
    L.dgeqp4.argtypes = [_ip, _ip, _dp, _ip, _ip, _dp, _dp, _ip, _ip]
    L.dgeqp4.restype = None
    L.hqrrp_gb300_dgeqp4_sketch.argtypes = [_ip, _ip, _dp, _ip, _ip, _dp, _dp, _ip, _ip, _dp,
                                            C.c_int]
    L.hqrrp_gb300_dgeqp4_sketch.restype = None
    L.hqrrp_gb300_ut_blk_var2.argtypes = [Obj, Obj, Obj, C.c_int, C.c_int, C.c_int]
    L.hqrrp_gb300_ut_blk_var2.restype = C.c_int
    L.hqrrp_gb300_ut_blk_var2_sketch.argtypes = [Obj, Obj, Obj, C.c_int, C.c_int, C.c_int, _dp,
                                                 C.c_int]
    L.hqrrp_gb300_ut_blk_var2_sketch.restype = C.c_int
    L.NoFLA_HQRRP_WY_blk_var4.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip, _dp, C.c_int,
                                          C.c_int, C.c_int]
    L.NoFLA_HQRRP_WY_blk_var4.restype = C.c_int
    L.hqrrp_gb300_set_precision.argtypes = [C.c_int]
    L.hqrrp_gb300_set_precision.restype = C.c_int
    L.hqrrp_gb300_set_dgeqp4_block.argtypes = [C.c_int]
    L.hqrrp_gb300_set_dgeqp4_block.restype = C.c_int
    L.hqrrp_gb300_set_seed.argtypes = [C.c_ulonglong]
    L.hqrrp_gb300_set_seed.restype = None
    L.hqrrp_gb300_set_spin_limit.argtypes = [C.c_uint]
    L.hqrrp_gb300_set_spin_limit.restype = None
    L.hqrrp_gb300_hqrrp_sketch.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip, _dp, C.c_int,
                                           C.c_int, C.c_int, _dp, C.c_int]
    L.hqrrp_gb300_hqrrp_sketch.restype = C.c_int
    L.hqrrp_gb300_hqrrp_device.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                           C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                           C.c_int, C.c_ulonglong, C.c_void_p]
    L.hqrrp_gb300_hqrrp_device.restype = C.c_int
    L.hqrrp_gb300_dgeqp4_device.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                            C.c_void_p, C.c_void_p]
    L.hqrrp_gb300_dgeqp4_device.restype = C.c_int
    L.hqrrp_gb300_sketch_device.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int,
                                            C.c_ulonglong, C.c_void_p]
    L.hqrrp_gb300_sketch_device.restype = C.c_int
    L.hqrrp_gb300_profile_enable.argtypes = [C.c_int]
    L.hqrrp_gb300_profile_enable.restype = None
    L.hqrrp_gb300_profile_read.argtypes = [_dp, _dp, C.c_int]
    L.hqrrp_gb300_profile_read.restype = C.c_int
    L.hqrrp_gb300_launch_count.argtypes = []
    L.hqrrp_gb300_launch_count.restype = C.c_ulonglong
    L.hqrrp_gb300_pool_alloc_count.argtypes = []
    L.hqrrp_gb300_pool_alloc_count.restype = C.c_ulonglong
    L.hqrrp_gb300_gram_panel_counts.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.hqrrp_gb300_gram_panel_counts.restype = C.c_int
    L.hqrrp_gb300_ozaki_dgemm.argtypes = [C.c_char, C.c_char, C.c_int, C.c_int, C.c_int,
                                          C.c_double, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                          C.c_double, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.hqrrp_gb300_ozaki_dgemm.restype = C.c_int
    L.hqrrp_gb300_qrp_batched_workspace.argtypes = [C.c_int]
    L.hqrrp_gb300_qrp_batched_workspace.restype = C.c_size_t
    L.hqrrp_gb300_qrp_batched_plan.argtypes = [C.c_int, _ip, _ip, C.c_void_p, C.c_size_t,
                                               C.c_int, C.c_void_p]
    L.hqrrp_gb300_qrp_batched_plan.restype = C.c_int
    L.hqrrp_gb300_qrp_batched_run.argtypes = [C.c_int] + [C.c_void_p] * 7 + [C.c_int, C.c_int,
                                                                              C.c_void_p, C.c_void_p]
    L.hqrrp_gb300_qrp_batched_run.restype = C.c_int
    L.hqrrp_gb300_qrp_batched_config.argtypes = [C.c_int, _ip, _ip, _ip]
    L.hqrrp_gb300_qrp_batched_config.restype = C.c_int
    L.hqrrp_gb300_hqrrp_truncated_device.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p,
                                                      C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                                      C.c_int, C.c_ulonglong, C.c_void_p]
    L.hqrrp_gb300_lowrank_device.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                             C.c_void_p]
    L.hqrrp_gb300_form_q_device.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                            C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.hqrrp_gb300_hqrrp_adjoint_device.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p,
                                                   C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                                   C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                                   C.c_int, C.c_int, C.c_void_p]
    L.hqrrp_gb300_apply_q_device.argtypes = [C.c_char, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                             C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                             C.c_void_p]
    for f in ("hqrrp_gb300_hqrrp_truncated_device", "hqrrp_gb300_lowrank_device",
              "hqrrp_gb300_apply_q_device",
              "hqrrp_gb300_form_q_device", "hqrrp_gb300_hqrrp_adjoint_device"):
        getattr(L, f).restype = C.c_int
    L.hqrrp_gb300_profile_counts.argtypes = [_ip, C.c_int]
    L.hqrrp_gb300_profile_counts.restype = C.c_int
    L.hqrrp_gb300_last_error.argtypes = []
    L.hqrrp_gb300_last_error.restype = C.c_char_p
    _lib = L
    return L


def declared_symbols(header=HEADER):
    """Function names declared in include/hqrrp_gb300.h."""
    import re
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text.split("extern \"C\" {", 1)[-1])


def last_error():
    return load().hqrrp_gb300_last_error().decode()


def set_precision(mode):
    return load().hqrrp_gb300_set_precision(int(mode))


def set_dgeqp4_block(nb):
    """Block size of dgeqp4's HQRRP call (default 64, the reference's);
    returns the previous value."""
    prev = load().hqrrp_gb300_set_dgeqp4_block(int(nb))
    if prev < 0:
        raise ValueError("dgeqp4 block size must be in 1..246")
    return prev


def set_seed(seed):
    load().hqrrp_gb300_set_seed(int(seed))


def set_spin_limit(limit):
    load().hqrrp_gb300_set_spin_limit(int(limit))


PHASES = ("sketch", "select", "panel", "update", "downdate", "other", "tensor", "split")


def profile_enable(on=True):
    load().hqrrp_gb300_profile_enable(1 if on else 0)


def profile_read():
    """{phase: (ms, algorithmic FP64 flops)} since the last read; resets."""
    ms = np.zeros(16)
    fl = np.zeros(16)
    n = load().hqrrp_gb300_profile_read(ms.ctypes.data_as(_dp), fl.ctypes.data_as(_dp), 16)
    return {PHASES[i]: (float(ms[i]), float(fl[i])) for i in range(n)}


def profile_counts():
    """{phase: intervals recorded} since the last call; resets."""
    c = np.zeros(16, dtype=np.int32)
    n = load().hqrrp_gb300_profile_counts(c.ctypes.data_as(_ip), 16)
    return {PHASES[i]: int(c[i]) for i in range(n)}


def launch_count():
    return int(load().hqrrp_gb300_launch_count())


def gram_panel_counts():
    """(committed, fallback): the mixed path's Gram panels of the last call
    that ran any, committed and passed on to the column-by-column panel."""
    L = load()
    a, b = C.c_int(0), C.c_int(0)
    rc = L.hqrrp_gb300_gram_panel_counts(C.byref(a), C.byref(b))
    if rc != 0:
        raise HQRRPError("gram_panel_counts failed (%d): %s" % (rc, last_error()))
    return a.value, b.value


def pool_alloc_count():
    """Device allocations the library has made from its memory pools."""
    return int(load().hqrrp_gb300_pool_alloc_count())


def _fortran(A):
    return np.array(np.asarray(A, dtype=np.float64), order="F", copy=True)


def hqrrp(A, nb=64, pp=10, panel_pivoting=1, jpvt=None, G=None):
    """NoFLA_HQRRP_WY_blk_var4 on a copy of A (host arrays through the C ABI).

    Returns (A_out, jpvt, tau).  jpvt defaults to 1..n and is carried like the
    reference carries it.  G: optional explicit sketch ((nb+pp) x m)."""
    L = load()
    A = _fortran(A)
    m, n = A.shape
    jp = (np.arange(1, n + 1, dtype=np.int32) if jpvt is None
          else np.array(jpvt, dtype=np.int32, copy=True))
    tau = np.zeros(max(1, min(m, n)), dtype=np.float64)
    if G is None:
        rc = L.NoFLA_HQRRP_WY_blk_var4(m, n, A.ctypes.data_as(_dp), max(1, m),
                                       jp.ctypes.data_as(_ip), tau.ctypes.data_as(_dp),
                                       nb, pp, panel_pivoting)
    else:
        G = _fortran(G)
        rc = L.hqrrp_gb300_hqrrp_sketch(m, n, A.ctypes.data_as(_dp), max(1, m),
                                        jp.ctypes.data_as(_ip), tau.ctypes.data_as(_dp), nb, pp,
                                        panel_pivoting, G.ctypes.data_as(_dp), G.shape[0])
    if rc != 0:
        raise HQRRPError("hqrrp failed (%d): %s" % (rc, last_error()))
    return A, jp, tau[:min(m, n)]


def hqrrp_ut(A, nb=64, pp=10, panel_pivoting=1, p=None, G=None):
    """FLA_HQRRP_UT_blk_var2 (the UT-transform variant) on a copy of A through
    hqrrp_gb300_ut_blk_var2; returns (A_out, p, s), s the UT scalars
    (tau_UT = 1 / tau).  p defaults to 1..n and is carried.  G: optional
    explicit sketch ((nb + pp) x m)."""
    L = load()
    A = _fortran(A)
    m, n = A.shape
    pv = (np.arange(1, n + 1, dtype=np.int32) if p is None
          else np.array(p, dtype=np.int32, copy=True))
    s = np.zeros(max(1, min(m, n)), dtype=np.float64)
    oA = Obj(DOUBLE, m, n, max(1, m), A.ctypes.data)
    op = Obj(INT, n, 1, max(1, n), pv.ctypes.data)
    os_ = Obj(DOUBLE, s.size, 1, s.size, s.ctypes.data)
    if G is None:
        rc = L.hqrrp_gb300_ut_blk_var2(oA, op, os_, nb, pp, panel_pivoting)
    else:
        Gf = _fortran(G)
        rc = L.hqrrp_gb300_ut_blk_var2_sketch(oA, op, os_, nb, pp, panel_pivoting,
                                              Gf.ctypes.data_as(_dp), Gf.shape[0])
    if rc != 0:
        raise HQRRPError("hqrrp_ut failed (%d): %s" % (rc, last_error()))
    return A, pv, s[:min(m, n)]


def dgeqp4(A, jpvt=None, lwork=None, G=None):
    """dgeqp4 on a copy of A; returns (A_out, jpvt, tau, info, work0).

    G: optional explicit sketch of the HQRRP branch (74 x m, the first m - nf
    columns read; hqrrp_gb300_dgeqp4_sketch).  info < 0 is an argument error
    (as LAPACK); info > 1000 raises."""
    L = load()
    A = _fortran(A)
    m, n = A.shape
    jp = (np.zeros(n, dtype=np.int32) if jpvt is None
          else np.array(jpvt, dtype=np.int32, copy=True))
    tau = np.zeros(max(1, min(m, n)), dtype=np.float64)
    if lwork is None:
        lwork = max(1, 3 * n + 1, 2 * n + (n + 1) * 32)
    work = np.zeros(max(1, lwork), dtype=np.float64)
    mi, ni, ldi, lw, info = (C.c_int(m), C.c_int(n), C.c_int(max(1, m)), C.c_int(lwork),
                             C.c_int(0))
    args = (C.byref(mi), C.byref(ni), A.ctypes.data_as(_dp), C.byref(ldi),
            jp.ctypes.data_as(_ip), tau.ctypes.data_as(_dp), work.ctypes.data_as(_dp),
            C.byref(lw), C.byref(info))
    if G is None:
        L.dgeqp4(*args)
    else:
        Gf = np.zeros((74, max(1, m)), order="F")
        g = np.asarray(G, dtype=np.float64)
        assert g.shape[0] == 74 and g.shape[1] <= m
        Gf[:, :g.shape[1]] = g
        L.hqrrp_gb300_dgeqp4_sketch(*args, Gf.ctypes.data_as(_dp), 74)
    if info.value > 1000:
        raise HQRRPError("dgeqp4 failed (info=%d): %s" % (info.value, last_error()))
    return A, jp, tau[:min(m, n)], info.value, work[0]


def _stream_ptr(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return int(getattr(stream, "cuda_stream", stream))


def hqrrp_device(At, jpvt, tau, nb=64, pp=10, panel_pivoting=1, Gt=None, seed=12, stream=None):
    """HQRRP on torch CUDA tensors, in place.

    At: (n, m) contiguous float64 = column-major m x n A (ld = m).
    jpvt: int32 (n,), carried.  tau: float64 (min(m,n),).
    Gt: optional (m, nb+pp) contiguous float64 = column-major sketch."""
    L = load()
    n, m = At.shape
    assert At.is_contiguous() and At.dtype.is_floating_point
    gptr = Gt.data_ptr() if Gt is not None else None
    rc = L.hqrrp_gb300_hqrrp_device(m, n, At.data_ptr(), max(1, m), jpvt.data_ptr(),
                                    tau.data_ptr(), nb, pp, panel_pivoting, gptr,
                                    nb + pp, int(seed), _stream_ptr(stream))
    if rc != 0:
        raise HQRRPError("hqrrp_device failed (%d): %s" % (rc, last_error()))


def sketch_device(rows, cols, seed=12, stream=None):
    """The device Philox sketch ((cols, rows) contiguous = column-major rows x cols)."""
    import torch
    Gt = torch.empty((cols, rows), dtype=torch.float64, device="cuda")
    rc = load().hqrrp_gb300_sketch_device(rows, cols, Gt.data_ptr(), rows, int(seed),
                                          _stream_ptr(stream))
    if rc != 0:
        raise HQRRPError("sketch_device failed (%d): %s" % (rc, last_error()))
    return Gt


def dgeqp4_device(At, jpvt, tau, stream=None):
    """dgeqp4 on torch CUDA tensors (At: (n, m) contiguous = column-major A)."""
    L = load()
    n, m = At.shape
    info = L.hqrrp_gb300_dgeqp4_device(m, n, At.data_ptr(), max(1, m), jpvt.data_ptr(),
                                       tau.data_ptr(), _stream_ptr(stream))
    if info > 1000:
        raise HQRRPError("dgeqp4_device failed (info=%d): %s" % (info, last_error()))
    return info


def ozaki_dgemm(transa, transb, alpha, At, Bt, beta, Ct, slices=6, stream=None):
    """C = alpha op(A) op(B) + beta C on torch CUDA tensors holding column-major
    matrices as their transposes (At: (cols, rows) contiguous, and so on).
    alpha = +-1, beta in {0, 1}."""
    L = load()
    m = Ct.shape[1]
    n = Ct.shape[0]
    k = (At.shape[1] if transa in ("T", b"T") else At.shape[0])
    ta = transa.encode() if isinstance(transa, str) else transa
    tb = transb.encode() if isinstance(transb, str) else transb
    rc = L.hqrrp_gb300_ozaki_dgemm(ta, tb, m, n, k, float(alpha), At.data_ptr(), At.shape[1],
                                   Bt.data_ptr(), Bt.shape[1], float(beta), Ct.data_ptr(),
                                   Ct.shape[1], int(slices), _stream_ptr(stream))
    if rc != 0:
        raise HQRRPError("ozaki_dgemm failed (%d): %s" % (rc, last_error()))


class BatchedQRP:
    """Pivoted QR of many small matrices in one persistent launch.

    ``shapes``: list of (m, n).  ``plan`` (at construction) uploads a
    largest-first schedule and, with ``autotune``, picks the launch shape by
    timing.  ``run(mats)`` factors torch CUDA tensors in place -- mats[i] is
    (n_i, m_i) contiguous, i.e. column-major A_i -- and returns (jpvt, tau,
    info) tensors; ``run`` only enqueues work, so it can be captured in a CUDA
    graph once the pointer tables are built (``bind``)."""

    def __init__(self, shapes, autotune=True, stream=None):
        import torch
        L = load()
        self.shapes = [(int(m), int(n)) for m, n in shapes]
        self.batch = len(self.shapes)
        self.max_n = max([n for _, n in self.shapes] + [1])
        hm = np.array([m for m, _ in self.shapes], np.int32)
        hn = np.array([n for _, n in self.shapes], np.int32)
        dev = torch.device("cuda")
        self.d_m = torch.from_numpy(hm).to(dev)
        self.d_n = torch.from_numpy(hn).to(dev)
        self.d_lda = torch.from_numpy(np.maximum(hm, 1)).to(dev)
        nbytes = L.hqrrp_gb300_qrp_batched_workspace(self.batch)
        self.work = torch.zeros(max(16, nbytes), dtype=torch.uint8, device=dev)
        torch.cuda.synchronize()
        cfg = L.hqrrp_gb300_qrp_batched_plan(self.batch, hm.ctypes.data_as(_ip),
                                             hn.ctypes.data_as(_ip), self.work.data_ptr(),
                                             self.work.numel(), 1 if autotune else 0,
                                             _stream_ptr(stream))
        if cfg < 0:
            raise HQRRPError("batched plan failed (%d): %s" % (cfg, last_error()))
        self.cfg = cfg
        # Outputs: one flat buffer each (so a caller can copy them in one
        # transfer), handed out as per-matrix views.
        nj = [n for _, n in self.shapes]
        nt = [max(1, min(m, n)) for m, n in self.shapes]
        self.jpvt_flat = torch.zeros(max(1, sum(nj)), dtype=torch.int32, device=dev)
        self.tau_flat = torch.zeros(max(1, sum(nt)), dtype=torch.float64, device=dev)
        oj = np.concatenate([[0], np.cumsum(nj)]).astype(int)
        ot = np.concatenate([[0], np.cumsum(nt)]).astype(int)
        self.jpvt = [self.jpvt_flat[oj[i]:oj[i + 1]] for i in range(self.batch)]
        self.tau = [self.tau_flat[ot[i]:ot[i + 1]] for i in range(self.batch)]
        self.info = torch.zeros(self.batch, dtype=torch.int32, device=dev)
        self._ptrs = None

    def config(self):
        t, s, c = C.c_int(), C.c_int(), C.c_int()
        load().hqrrp_gb300_qrp_batched_config(self.cfg, C.byref(t), C.byref(s), C.byref(c))
        return {"threads": t.value, "stage_kb": s.value, "ctas_per_sm": c.value}

    def bind(self, mats):
        """Build the device pointer tables for these matrices."""
        import torch
        assert len(mats) == self.batch
        for t, (m, n) in zip(mats, self.shapes):
            assert tuple(t.shape) == (n, m) and t.is_contiguous() and t.dtype == torch.float64
        mk = lambda xs: torch.tensor([x.data_ptr() for x in xs], dtype=torch.int64,
                                     device="cuda")
        self._mats = mats
        self._ptrs = (mk(mats), mk(self.jpvt), mk(self.tau))

    def run(self, mats=None, stream=None):
        if mats is not None:
            self.bind(mats)
        pa, pj, pt = self._ptrs
        rc = load().hqrrp_gb300_qrp_batched_run(
            self.batch, self.d_m.data_ptr(), self.d_n.data_ptr(), pa.data_ptr(),
            self.d_lda.data_ptr(), pj.data_ptr(), pt.data_ptr(), self.info.data_ptr(),
            self.max_n, self.cfg, self.work.data_ptr(), _stream_ptr(stream))
        if rc != 0:
            raise HQRRPError("batched run failed (%d): %s" % (rc, last_error()))
        return self.jpvt, self.tau, self.info


# ---- Truncated factorization, its low-rank reconstruction and adjoint -------

def _check(rc, what):
    if rc != 0:
        raise HQRRPError("%s failed (%d): %s" % (what, rc, last_error()))


def truncated_factor(At, k, nb=64, pp=10, seed=12, stream=None):
    """Truncated HQRRP of column-major A (At: (n, m) contiguous CUDA float64).
    Returns (Ft, jpvt, tau): Ft the factored copy, jpvt 1-based int32."""
    import torch
    n, m = At.shape
    Ft = At.clone()
    jp = torch.arange(1, n + 1, dtype=torch.int32, device=At.device)
    tau = torch.zeros(max(1, min(m, n)), dtype=torch.float64, device=At.device)
    _check(load().hqrrp_gb300_hqrrp_truncated_device(m, n, k, Ft.data_ptr(), m, jp.data_ptr(),
                                                     tau.data_ptr(), nb, pp, int(seed),
                                                     _stream_ptr(stream)), "truncated HQRRP")
    return Ft, jp, tau


def lowrank(Ft, jpvt, tau, k, nb=64, stream=None):
    """Q_k R_k P^T (returned transposed: (n, m) contiguous = column-major)."""
    import torch
    n, m = Ft.shape
    Out = torch.empty_like(Ft)
    _check(load().hqrrp_gb300_lowrank_device(m, n, k, Ft.data_ptr(), m, jpvt.data_ptr(),
                                             tau.data_ptr(), Out.data_ptr(), m, nb,
                                             _stream_ptr(stream)), "lowrank")
    return Out


def form_q(Ft, tau, k, nb=64, stream=None):
    """First k columns of Q ((k, m) contiguous = column-major m x k)."""
    import torch
    n, m = Ft.shape
    Qt = torch.empty((k, m), dtype=torch.float64, device=Ft.device)
    _check(load().hqrrp_gb300_form_q_device(m, k, Ft.data_ptr(), m, tau.data_ptr(),
                                            Qt.data_ptr(), m, nb, _stream_ptr(stream)), "form_q")
    return Qt


def apply_q(Ft, tau, Ct, trans="N", k=None, nb=64, stream=None):
    """In place: C := Q C (trans 'N') or Q^T C ('T'); Ft (n, m) and Ct (nc, m)
    contiguous = column-major; Q = product of the first k reflectors (default
    min(m, n)) of the factorization Ft, tau."""
    n, m = Ft.shape
    nc = Ct.shape[0]
    if Ct.shape[1] != m or not Ct.is_contiguous():
        raise ValueError("Ct must be (nc, m) contiguous")
    k = min(m, n) if k is None else k
    _check(load().hqrrp_gb300_apply_q_device(trans.encode(), m, nc, k, Ft.data_ptr(), m,
                                             tau.data_ptr(), Ct.data_ptr(), m, nb,
                                             _stream_ptr(stream)), "apply_q")
    return Ct


def adjoint(At, Ft, jpvt, tau, Wt, k, nb=64, stream=None):
    """dL/dA for L = <W, Q_k R_k P^T>, pivots fixed (all (n, m) column-major)."""
    import torch
    n, m = At.shape
    Gt = torch.empty_like(At)
    _check(load().hqrrp_gb300_hqrrp_adjoint_device(
        m, n, k, At.data_ptr(), m, Ft.data_ptr(), m, jpvt.data_ptr(), tau.data_ptr(),
        Wt.data_ptr(), m, Gt.data_ptr(), m, nb, _stream_ptr(stream)), "adjoint")
    return Gt


def _autograd_function():
    import torch

    class TruncatedHQRRP(torch.autograd.Function):
        """A (m x n, CUDA float64) -> Q_k R_k P^T, the rank-k HQRRP
        approximation.  Backward: the library's adjoint with the forward's
        pivots held fixed; only A and the factored matrix (reflectors in its
        lower part) are kept, Q and the T factors are recomputed."""

        @staticmethod
        def forward(ctx, A, k, nb=64, pp=10, seed=12):
            At = A.detach().t().contiguous()
            Ft, jp, tau = truncated_factor(At, k, nb, pp, seed)
            ctx.save_for_backward(At, Ft, jp, tau)
            ctx.k, ctx.nb = k, nb
            return lowrank(Ft, jp, tau, k, nb).t()

        @staticmethod
        def backward(ctx, grad):
            At, Ft, jp, tau = ctx.saved_tensors
            Gt = adjoint(At, Ft, jp, tau, grad.t().contiguous(), ctx.k, ctx.nb)
            return Gt.t(), None, None, None, None

    return TruncatedHQRRP


_TRUNC = None


def truncated_hqrrp(A, k, nb=64, pp=10, seed=12):
    """Differentiable rank-k HQRRP approximation Q_k R_k P^T of A."""
    global _TRUNC
    if _TRUNC is None:
        _TRUNC = _autograd_function()
    return _TRUNC.apply(A, k, nb, pp, seed)
