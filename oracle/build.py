"""Build recipe for the oracle (test infrastructure only).

Two shared libraries come out of this recipe:

* ``oracle/_lib/libhqrrp_oracle.so`` -- the CPU restatement in
  ``hqrrp_oracle.c``.  It loads LAPACK/BLAS at run time, so it builds on any
  host with gcc (x86_64 here, aarch64 on the GPU host).
* ``oracle/_ref/libhqrrp_ref.so`` -- the unmodified reference source
  ``lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4.c`` compiled through
  ``ref_wrap.c`` and linked to scipy's bundled OpenBLAS.  Built only where the
  reference tree is found: the ``reference`` argument, else the
  ``HQRRP_REFERENCE_DIR`` environment variable, else DEFAULT_REFERENCE (where
  this recipe's build container mounts it); elsewhere the restatement alone
  is the oracle.

Nothing here is imported by the product package.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_lib")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(LIB_DIR, "libhqrrp_oracle.so")
REF_SO = os.path.join(REF_DIR, "libhqrrp_ref.so")
# Where the build container mounts the reference project; the argument and
# HQRRP_REFERENCE_DIR take precedence.
DEFAULT_REFERENCE = "/root/reference"

# LAPACK/BLAS symbols the reference calls; each is mapped onto scipy_<name>_.
_REF_SYMBOLS = ["dgemm", "dgeqp3", "dgeqpf", "dgeqrf", "dlacpy", "dlamch", "dlarf",
                "dlarfb", "dlarfg", "dlarft", "dnrm2", "dorgqr", "dormqr", "dswap",
                "dtrmm", "idamax", "ilaenv", "xerbla"]

CFLAGS = ["-O2", "-fPIC", "-shared", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math"]


def find_openblas():
    """Path of an LP64 OpenBLAS with LAPACK: scipy's bundled copy.

    numpy's copy is ILP64 (64-bit integers, ``64_`` suffix) and is never used.
    """
    try:
        import scipy
    except ImportError:
        return None
    base = os.path.dirname(os.path.dirname(scipy.__file__))
    cands = sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")))
    cands = [c for c in cands if "openblas64" not in os.path.basename(c)]
    if not cands:
        cands = sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__), ".dylibs",
                                              "libscipy_openblas*")))
    return cands[0] if cands else None


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle(force=False):
    src = os.path.join(HERE, "hqrrp_oracle.c")
    os.makedirs(LIB_DIR, exist_ok=True)
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        _run(["gcc"] + CFLAGS + [src, "-o", ORACLE_SO, "-ldl", "-lm"])
    return ORACLE_SO


def reference_dir(reference=None):
    """The reference project's root, or None where its source is absent."""
    d = reference or os.environ.get("HQRRP_REFERENCE_DIR") or DEFAULT_REFERENCE
    src = os.path.join(d, "lapack_compatible_sources", "NoFLA_HQRRP_WY_blk_var4.c")
    return d if os.path.exists(src) else None


def build_reference(force=False, reference=None):
    """Compile the unmodified reference; returns the .so path or None."""
    d = reference_dir(reference)
    blas = find_openblas()
    if d is None or blas is None:
        return REF_SO if os.path.exists(REF_SO) else None
    os.makedirs(REF_DIR, exist_ok=True)
    wrap = os.path.join(HERE, "ref_wrap.c")
    if force or not os.path.exists(REF_SO) or os.path.getmtime(REF_SO) < os.path.getmtime(wrap):
        defs = ["-D%s_=scipy_%s_" % (s, s) for s in _REF_SYMBOLS]
        _run(["gcc"] + CFLAGS + ["-w", "-I", os.path.join(d, "lapack_compatible_sources")] + defs
             + [wrap, "-o", REF_SO, "-L", os.path.dirname(blas), "-l:" + os.path.basename(blas),
                "-Wl,-rpath," + os.path.dirname(blas), "-lm"])
    return REF_SO


def build(force=False, reference=None):
    out = {"oracle": build_oracle(force)}
    try:
        out["reference"] = build_reference(force, reference)
    except RuntimeError as exc:  # the reference is optional
        print(exc, file=sys.stderr)
        out["reference"] = None
    return out


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    print(build(force="--force" in sys.argv, reference=args[0] if args else None))
