"""Build libhqrrp_gb300.so in-tree for sm_103a.

nvcc compiles each CUDA translation unit (in parallel) with
``-gencode arch=compute_103a,code=sm_103a``; gcc compiles the C host driver;
the shared library links the CUDA runtime statically and exports only the
symbols declared in ``include/hqrrp_gb300.h``.  Objects go to
``hqrrp_gb300/_build/`` and the library to ``hqrrp_gb300/libhqrrp_gb300.so``
(both git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhqrrp_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

CUDA_SOURCES = ["gemm_f64.cu", "sketch.cu", "qrp_skinny.cu", "qrp_panel.cu", "permute.cu",
                "qrp_noalloc.cu", "qrp_wide.cu", "qrp_gram.cu", "ozaki.cu", "qrp_batched.cu",
                "adjoint.cu"]
C_SOURCES = ["hqrrp_driver.c"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_nvcc=()):
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "hqrrp_gb300.h"))
    jobs = []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                         "-Xcompiler", "-fvisibility=hidden", "-I", CSRC, "-I",
                                         INCLUDE] + list(extra_nvcc) + ["-c", src, "-o", obj])
    for s in C_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        if force or _stale(obj, [src] + headers):
            jobs.append(["gcc", "-O2", "-std=gnu11", "-fPIC", "-fvisibility=hidden", "-Wall",
                         "-Wno-unused-function", "-I", CSRC, "-I", INCLUDE, "-I",
                         os.path.join(cuda, "include"), "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [os.path.join(BUILD, s + ".o") for s in CUDA_SOURCES + C_SOURCES]
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs +
             ["-Xlinker", "--exclude-libs,ALL", "-lpthread", "-ldl", "-lrt"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra_nvcc=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
