#!/usr/bin/env python
"""HQRRP throughput on one GB300 (TFLOP/s, 2mn^2 - 2n^3/3 for m >= n).

Workloads (``--workload``):
  square (default; the configuration the metric is quoted on): m = n = 16384,
      A = U diag(sigma) V^T with Haar U, V (QR of seeded Gaussians,
      sign-fixed), sigma_i = 10^(-12 i / n), nb = 128, pp = 10, panel
      pivoting on.  Also reports bwd_ms, the adjoint of the truncated rank-256
      factorization of a 4096 x 2048 matrix.
  tall: m = 32768, n = 8192, sigma geometric from 1 to 1e-10 with a cluster of
      64 equal values at 1e-4, same nb/pp.
  batched: 4096 matrices, m log-uniform in [64, 1024], n log-uniform in
      [32, min(m, 512)], A_i = U diag(i^-2) V^T, full pivoted QR of each in
      one persistent launch replayed from a captured CUDA graph.
All inputs are synthetic and seeded, generated on the GPU before the timed
region.

One step = one full factorization of a fresh copy of the input (larger than
L2 in every workload, so nothing carries over between steps).  For square and
tall the headline is the mixed-precision path (split-BF16 tensor-core block
updates); the plain FP64 path is timed the same way in the same run and
reported beside it, with both residuals.  ``value`` is timed with CUDA events
on the factorization's stream with the input already in HBM; ``e2e`` goes
through the reference-facing C entry points (NoFLA_HQRRP_WY_blk_var4, and
dgeqp4 beside it) with host (pinned) buffers, so both copies are inside its
timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload square|tall|batched]
                  [--precision both|mixed|plain]
  python bench.py --impl reference ...   # the reference algorithm on host cores

Under torchrun (N > 1) every rank factors its own matrix (replicas: a single
factorization does not shard) or its cost-balanced shard of the batch, and
value is the whole-job aggregate.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "dgeqp4 TFLOP/s at n=16384, mixed vs plain FP64 at equal residual; bwd ms"
# DRAM bytes per algorithmic flop of the dominant kernels, from ncu captures at
# m = n = 6144 (committed summaries under profiles/): the split-BF16 products
# -- W1 = U'^T C reading C as FP64 (302.1 MB per 2.43e11 BF16 flops,
# ozk_gemm_c64_n6144.md) and C -= U'W2 (556.1 MB per 2.649e11, ozk_gemm_n6144.md)
# -- and the FP64 update GEMMs of the plain path (W1, C -= U W2).
TENSOR_BYTES_PER_FLOP = (302.1e6 + 556.1e6) / (2.43e11 + 2.649e11)
FP64_UPDATE_BYTES_PER_FLOP = (314.4e6 + 546.3e6) / (2 * 9.462e9)


def flops_qr(m, n):
    k = min(m, n)
    return 2.0 * m * n * k - 2.0 * k ** 3 / 3.0 if m >= n else 2.0 * n * m * m - 2.0 * m ** 3 / 3.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="square", choices=["square", "tall", "batched"])
    p.add_argument("--batch", type=int, default=4096)
    p.add_argument("--precision", default="both", choices=["both", "mixed", "plain"],
                   help="both (default): headline = mixed, plain timed alongside")
    p.add_argument("--n", type=int, default=None, help="columns (square: also rows)")
    p.add_argument("--m", type=int, default=None, help="rows (tall workload)")
    p.add_argument("--nb", type=int, default=128)
    p.add_argument("--pp", type=int, default=10)
    p.add_argument("--seed", type=int, default=2026)
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--cpu-dgeqp3-n", type=int, default=6144,
                   help="size of the LAPACK dgeqp3 CPU sample")
    p.add_argument("--cpu-1t-n", type=int, default=3072,
                   help="size of the one-thread CPU sample")
    p.add_argument("--ref-n", type=int, default=16384, help="reference-arm matrix size")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-adjoint", action="store_true", help="skip the bwd_ms measurement")
    p.add_argument("--single", action="store_true",
                   help="one untimed factorization of the workload's matrix (for profilers)")
    p.add_argument("--no-extras", action="store_true",
                   help="square workload only: skip the nested tall and batched lines")
    return p.parse_args()


# ---------------------------------------------------------------------------
# Inputs

def spectrum(n):
    return 10.0 ** (-12.0 * np.arange(n) / n)


def spectrum_tall(n, cluster=64):
    """Geometric from 1 to 1e-10 over n - cluster values, plus cluster equal
    values at 1e-4, in descending order."""
    g = 10.0 ** (-10.0 * np.arange(n - cluster) / max(1, n - cluster - 1))
    return np.sort(np.concatenate([g, np.full(cluster, 1e-4)]))[::-1].copy()


def _preload_linalg():
    import ctypes
    import torch
    # torch loads its CUDA linear-algebra library lazily by bare name; load it by
    # path first so the lookup also succeeds under a profiler's injection.
    linalg = os.path.join(os.path.dirname(torch.__file__), "lib", "libtorch_cuda_linalg.so")
    if os.path.exists(linalg):
        ctypes.CDLL(linalg, mode=ctypes.RTLD_GLOBAL)


def _orth(r, c, g, device):
    """r x c with Haar-distributed orthonormal columns (QR of a Gaussian, sign-fixed)."""
    import torch
    Q, R = torch.linalg.qr(torch.randn(r, c, dtype=torch.float64, device=device, generator=g))
    return Q * torch.sign(torch.diagonal(R))[None, :]


def make_matrix_gpu(m, n, sigma, seed, device):
    """A^T (n x m, contiguous) = column-major A = U diag(sigma) V^T, FP64;
    U m x k, V n x k, k = len(sigma) = min(m, n)."""
    import torch
    _preload_linalg()
    g = torch.Generator(device=device).manual_seed(seed)
    k = len(sigma)
    U = _orth(m, k, g, device)
    V = _orth(n, k, g, device)
    sig = torch.from_numpy(np.asarray(sigma, np.float64)).to(device)
    At = (V * sig[None, :]) @ U.T  # (A)^T = V diag(sigma) U^T
    del U, V
    return At.contiguous()


def make_matrix_cpu(n, seed):
    import oracle
    return oracle.with_spectrum(n, n, spectrum(n), seed)


def make_batched_gpu(shapes, seed, device):
    """The batched workload's matrices A_i = U diag(i^-2) V^T (Haar U, V),
    column-major, back to back in one flat FP64 buffer; returns (flat, offsets)."""
    import torch
    _preload_linalg()
    sizes = [m * n for m, n in shapes]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(int)
    flat = torch.empty(max(1, int(offs[-1])), dtype=torch.float64, device=device)
    g = torch.Generator(device=device).manual_seed(seed)
    for i, (m, n) in enumerate(shapes):
        k = min(m, n)
        U, V = _orth(m, k, g, device), _orth(n, k, g, device)
        sig = (1.0 + torch.arange(k, dtype=torch.float64, device=device)) ** -2.0
        flat[offs[i]:offs[i + 1]].view(n, m).copy_((V * sig[None, :]) @ U.T)
    return flat, offs


def batched_shapes(count, seed):
    """m log-uniform in [64, 1024], n log-uniform in [32, min(m, 512)]."""
    rng = np.random.default_rng(seed)
    m = np.exp(rng.uniform(np.log(64), np.log(1024), count)).astype(int)
    return [(int(a), int(np.exp(rng.uniform(np.log(32), np.log(min(a, 512)))))) for a in m]


# ---------------------------------------------------------------------------
# Quality (measurement infrastructure): ||AP - QR||_F / ||A||_F estimated with
# r Gaussian probes, and |R_kk| / sigma_k.

def quality_gpu(hq, At0, Atf, jp, tau, nb, r=8, seed=1):
    """(||AP - QR||_F / ||AP||_F and ||Q^T Q - I||_F, each estimated with r
    Gaussian probes X: ||E X||_F / sqrt(r) for E = Q^T Q - I; |diag R|).  Q is
    applied by the library's blocked reflector application (dormqr)."""
    import torch
    n, m = At0.shape
    k = min(m, n)
    g = torch.Generator(device=At0.device).manual_seed(seed)
    X = torch.randn(n, r, dtype=torch.float64, device=At0.device, generator=g)
    A = At0.T  # m x n view
    APX = A[:, jp.long() - 1] @ X
    F = Atf.T  # factored, m x n view
    R = torch.triu(F[:k, :])
    Yt = torch.zeros(r, m, dtype=torch.float64, device=At0.device)
    Yt[:, :k] = (R @ X).T
    hq.apply_q(Atf, tau, Yt, "N", k, nb)
    res = float(torch.linalg.norm(APX - Yt.T) / torch.linalg.norm(APX))
    Zt = torch.randn(r, m, dtype=torch.float64, device=At0.device, generator=g)
    Wt = Zt.clone()
    hq.apply_q(Atf, tau, Wt, "N", k, nb)
    hq.apply_q(Atf, tau, Wt, "T", k, nb)
    orth = float(torch.linalg.norm(Wt - Zt)) / r ** 0.5
    d = torch.abs(torch.diagonal(R)).cpu().numpy()
    return res, d, orth


# ---------------------------------------------------------------------------
# Clocks sampled during the timed region.

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.index)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (restatement of the reference, LAPACK/BLAS from
# scipy's OpenBLAS) on the host cores.

def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the
    cpu_baseline record; 'unknown' if neither says."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_impl(threads):
    """The compiled reference where its tree is present, else the oracle's
    restatement of it (bit-identical on the same LAPACK, tests/test_oracle.py)."""
    import oracle
    try:
        impl, kind = oracle.Reference(), "reference"
    except RuntimeError:
        impl, kind = oracle.Oracle(), "port"
    impl.set_threads(threads)
    return impl, kind


def host_square_matrix(n, seed):
    """The square workload's matrix on the host (column-major numpy), made on
    the GPU exactly as the GPU arm makes it when a GPU is present."""
    try:
        import torch
        if torch.cuda.is_available():
            At = make_matrix_gpu(n, n, spectrum(n), seed, torch.device("cuda", 0))
            A = np.asfortranarray(At.cpu().numpy().T)
            del At
            torch.cuda.empty_cache()
            return A
    except ImportError:
        pass
    return make_matrix_cpu(n, seed)


def cpu_baseline_run(A, args):
    """Bounded CPU sample beside the GPU arm (about half a minute on the GPU
    host's 16 cores): the reference dgeqp4 once on the headline matrix itself,
    LAPACK dgeqp3 once on its leading args.cpu_dgeqp3_n block, and dgeqp4 on
    one thread on its leading args.cpu_1t_n block."""
    import oracle
    cores = os.cpu_count() or 1
    impl, kind = cpu_impl(cores)
    n = A.shape[1]
    t4 = impl.timed_dgeqp4(np.array(A, order="F"))
    n3 = min(n, args.cpu_dgeqp3_n)
    lap = oracle.Oracle()
    lap.set_threads(cores)
    t3 = lap.timed_dgeqp3(np.array(A[:n3, :n3], order="F"))
    n1 = min(n, args.cpu_1t_n)
    impl.set_threads(1)
    t1 = impl.timed_dgeqp4(np.array(A[:n1, :n1], order="F"))
    impl.set_threads(cores)
    return {"value": flops_qr(n, n) / t4 / 1e12, "unit": "TFLOP/s", "cores": cores,
            "kind": kind, "cpu_model": cpu_model(),
            "sample": "reference dgeqp4 (HQRRP nb=64, pp=10 inside) on the headline's own m=n=%d "
                      "matrix, once: %.1f s" % (n, t4),
            "lapack_dgeqp3": {"value": flops_qr(n3, n3) / t3 / 1e12, "unit": "TFLOP/s",
                              "cores": cores, "seconds": t3,
                              "sample": "LAPACK dgeqp3 (scipy OpenBLAS) on the leading m=n=%d "
                                        "block of the same matrix, once" % n3},
            "one_thread": {"value": flops_qr(n1, n1) / t1 / 1e12, "unit": "TFLOP/s", "cores": 1,
                           "seconds": t1,
                           "sample": "reference dgeqp4 on one thread, leading m=n=%d block, "
                                     "once" % n1}}


def run_reference_arm(args):
    """The reference's dgeqp4 (HQRRP nb=64, pp=10 inside, as the reference
    hard-codes) on the host cores, on the square workload's own matrix: each
    timed step factors a fresh copy of it.  Warm-up steps factor a 4096^2
    block (they only wake the BLAS threads).  HQRRP nb=128 on the same matrix
    is timed once beside it (the block size of the GPU headline)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.ref_n
    cores = os.cpu_count() or 1
    impl, kind = cpu_impl(cores)
    A = host_square_matrix(n, args.seed)
    nw = min(n, 4096)
    for _ in range(args.warmup):
        impl.timed_dgeqp4(np.array(A[:nw, :nw], order="F"))
    times = []
    for _ in range(args.steps):
        B = np.array(A, order="F")
        times.append(impl.timed_dgeqp4(B))
        del B
    sec = sum(times)
    value = flops_qr(n, n) * len(times) / sec / 1e12
    th = impl.timed_hqrrp(np.array(A, order="F"), args.nb, args.pp)
    sample = ("reference dgeqp4 (HQRRP nb=64 pp=10 inside) on m=n=%d, A=U diag(10^(-12 i/n)) "
              "V^T (the GPU arm's matrix), one factorization per step; warm-up steps on its "
              "leading %d^2 block" % (n, nw))
    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": len(times), "warmup": args.warmup,
            "ms_per_step": sec / len(times) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "pivoted QR of m=n=%d, A=U diag(10^(-12 i/n)) V^T, Haar U,V; "
                                   "reference dgeqp4 on host cores" % n,
                       "name": "square", "m": n, "n": n, "api": "dgeqp4"},
            "hqrrp_nb128": {"value": flops_qr(n, n) / th / 1e12, "unit": "TFLOP/s", "seconds": th,
                            "api": "NoFLA_HQRRP_WY_blk_var4(nb=%d, pp=%d), once"
                                   % (args.nb, args.pp)},
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": cores, "kind": kind,
                             "sample": sample, "cpu_model": cpu_model()},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------

def fp64_peak_tflops(device):
    """cuBLAS DGEMM 8192^3, best of 3: the FP64 denominator of the roofline."""
    import torch
    a = torch.randn(8192, 8192, dtype=torch.float64, device=device)
    b = torch.randn_like(a)
    a @ b
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * 8192 ** 3 / (best * 1e-3) / 1e12


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def run_arm(hq, precision, At0, At, jp, iota, tau, nb, pp, sigma, steps, warmup, device, dist,
            local):
    """Warm up, then time exactly `steps` factorizations (one arm)."""
    import torch
    hq.set_precision(hq.MIXED if precision == "mixed" else hq.PLAIN)
    stream = torch.cuda.current_stream()

    def step():
        At.copy_(At0)
        jp.copy_(iota)
        hq.hqrrp_device(At, jp, tau, nb, pp, 1, stream=stream)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = hq.launch_count()
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    launches = hq.launch_count() - l0
    ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
    res, diag, orth = quality_gpu(hq, At0, At, jp, tau, nb)
    ratio = diag / sigma
    # One more (untimed) factorization under the phase profiler.
    hq.profile_enable(True)
    hq.profile_read()
    hq.profile_counts()
    step()
    torch.cuda.synchronize()
    prof = hq.profile_read()
    counts = hq.profile_counts()
    hq.profile_enable(False)
    return {"ms_per_step": ms / steps, "steps": steps, "warmup": warmup, "launches": launches,
            "clocks": clocks,
            "quality": {"residual_est": res, "orthogonality_est": orth,
                        "rkk_over_sigma_min": float(ratio.min()),
                        "rkk_over_sigma_max": float(ratio.max())},
            "ratio": ratio, "prof": prof, "counts": counts}


def phase_table(prof):
    return ({k: round(v[0], 3) for k, v in prof.items()},
            {k: (round(v[1] / (v[0] * 1e-3) / 1e12, 4) if v[0] > 0 and v[1] > 0 else None)
             for k, v in prof.items()})


def measure_adjoint(hq, device, m=4096, n=2048, k=256, nb=64, reps=5, seed=7):
    """Forward (truncated rank-k HQRRP + Q_k R_k P^T) and backward (the
    adjoint dL/dA of L = <W, Q_k R_k P^T>, pivots fixed) on A = U diag(i^-2) V^T
    with Haar U (m x n orthonormal columns) and V; CUDA events, 3 warm-ups."""
    import torch
    g = torch.Generator(device=device).manual_seed(seed)

    U, V = _orth(m, n, g, device), _orth(n, n, g, device)
    sig = (1.0 + torch.arange(n, dtype=torch.float64, device=device)) ** -2.0
    At = ((V * sig[None, :]) @ U.T).contiguous()  # column-major A (m x n)
    Wt = torch.randn(n, m, dtype=torch.float64, device=device, generator=g)
    del U, V
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fwd, bwd = [], []
    for it in range(3 + reps):
        torch.cuda.synchronize()
        ev[0].record()
        Ft, jp, tau = hq.truncated_factor(At, k, nb)
        hq.lowrank(Ft, jp, tau, k, nb)
        ev[1].record()
        hq.adjoint(At, Ft, jp, tau, Wt, k, nb)
        ev[2].record()
        torch.cuda.synchronize()
        if it >= 3:
            fwd.append(ev[0].elapsed_time(ev[1]))
            bwd.append(ev[1].elapsed_time(ev[2]))
    fwd.sort()
    bwd.sort()
    return {"bwd_ms": bwd[len(bwd) // 2], "fwd_ms": fwd[len(fwd) // 2],
            "config": "m=%d n=%d k=%d nb=%d, sigma_i=i^-2, Haar U,V; median of %d after 3 "
                      "warm-ups; fwd = truncated HQRRP + Q_k R_k P^T, bwd = adjoint "
                      "(Q_k and T rebuilt from the reflectors)" % (m, n, k, nb, reps)}


def run_batched(hq, args, device, dist, rank, world, local, steps, warmup):
    """Config: args.batch matrices of random shape, A_i = U diag(i^-2) V^T; one
    step = restore the inputs and replay the captured graph of one persistent
    launch over this rank's cost-balanced shard of the batch.  Returns rank
    0's line (None on other ranks)."""
    import torch
    from hqrrp_gb300 import shard
    _preload_linalg()
    shapes_all = batched_shapes(args.batch, args.seed)
    mine = shard.partition_by_cost(shapes_all, world)[rank] if world > 1 else list(
        range(len(shapes_all)))
    shapes = [shapes_all[i] for i in mine]
    flat0, offs = make_batched_gpu(shapes, args.seed + 1000 * rank, device)
    flat = flat0.clone()
    mats = [flat[offs[i]:offs[i + 1]].view(n, m) for i, (m, n) in enumerate(shapes)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bq = hq.BatchedQRP(shapes, autotune=True)
    plan_s = time.perf_counter() - t0
    bq.bind(mats)
    s = torch.cuda.Stream(device=device)
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        flat.copy_(flat0)
        bq.run(stream=s)
    torch.cuda.synchronize()
    l0 = hq.launch_count()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        bq.run(stream=s)
    per_replay = hq.launch_count() - l0

    def step():
        flat.copy_(flat0)
        graph.replay()

    with torch.cuda.stream(s):
        for _ in range(warmup):
            step()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(local)
        sampler.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(steps):
            step()
        e1.record(s)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / steps
    info = bq.info.cpu().numpy()
    if (info != 0).any():
        raise RuntimeError("batched QR reported info %s" % info[info != 0][:4])
    # Quality on a sample: ||A P - Q R||_F / ||A||_F with Q applied by the library.
    worst = 0.0
    for i in range(0, len(shapes), max(1, len(shapes) // 16)):
        m, n = shapes[i]
        k = min(m, n)
        F, A0 = mats[i], flat0[offs[i]:offs[i + 1]].view(n, m)
        QR = torch.zeros(n, m, dtype=torch.float64, device=device)
        QR[:, :k] = torch.triu(F.T[:k, :]).T
        hq.apply_q(F, bq.tau[i], QR, "N", k, 32)
        AP = A0[bq.jpvt[i].long() - 1]
        worst = max(worst, float((QR - AP).norm() / A0.norm()))

    # End to end: pinned host buffers in, factored matrices + jpvt + tau out.
    hflat0 = flat0.cpu().pin_memory()
    hflat = torch.empty_like(hflat0).pin_memory()
    hjp = torch.empty_like(bq.jpvt_flat, device="cpu").pin_memory()
    htau = torch.empty_like(bq.tau_flat, device="cpu").pin_memory()
    etimes = []
    with torch.cuda.stream(s):
        for it in range(1 + args.e2e_steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            flat.copy_(hflat0, non_blocking=True)
            graph.replay()
            hflat.copy_(flat, non_blocking=True)
            hjp.copy_(bq.jpvt_flat, non_blocking=True)
            htau.copy_(bq.tau_flat, non_blocking=True)
            s.synchronize()
            if it > 0:
                etimes.append(time.perf_counter() - t0)
    esec = sum(etimes) / len(etimes)
    tms = torch.tensor([ms, esec], dtype=torch.float64, device=device)
    if dist:
        dist.all_reduce(tms, op=dist.ReduceOp.MAX)
    ms, esec = float(tms[0]), float(tms[1])
    flops_all = sum(flops_qr(m, n) for m, n in shapes_all)
    value = flops_all / (ms * 1e-3) / 1e12

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_batched_run(shapes, offs, flat0)
    if rank == 0:
        h2d = 8 * int(offs[-1])
        d2h = h2d + 4 * bq.jpvt_flat.numel() + 8 * bq.tau_flat.numel()
        line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
                "steps": steps, "warmup": warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak" if world == 1 else "strong",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "batched pivoted QR of %d matrices, m log-uniform in "
                                       "[64,1024], n log-uniform in [32,min(m,512)], "
                                       "A_i=U diag(i^-2) V^T, Haar U,V; one persistent launch "
                                       "in a captured CUDA graph" % len(shapes_all),
                           "name": "batched", "batch": len(shapes_all),
                           "api": "hqrrp_gb300_qrp_batched_run",
                           "launch_shape": bq.config(), "autotune_s": plan_s,
                           "parallelism": "cost-balanced shards x%d" % world,
                           "l2": "inputs larger than L2 (%.2f GB per step, restored each step)"
                                 % (8 * offs[-1] * world / 1e9)},
                "matrices_per_s": len(shapes_all) / (ms * 1e-3),
                "quality": {"residual_max_sample": worst},
                "roofline": {"bound": "tensor", "pipe": "fp64", "achieved": value,
                             "peak": fp64_peak_tflops(device), "unit": "TFLOP/s",
                             "kernel": "qrp_batched_kernel (whole step)",
                             "peak_source": "cuBLAS DGEMM 8192^3 measured in this run",
                             "traffic": None},
                "cpu_baseline": cpu,
                "e2e": {"value": flops_all / esec / 1e12, "unit": "TFLOP/s",
                        "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "ms_per_step": esec * 1e3,
                        "api": "graph replay of hqrrp_gb300_qrp_batched_run, pinned host "
                               "buffers"},
                "gpu_launches": per_replay * steps, "clocks": clocks}
        line["roofline"]["frac"] = value / line["roofline"]["peak"]
        return line
    return None


def cpu_batched_run(shapes, offs, flat0, stride=1, reps=3):
    """The reference's dgeqp4 (which hands these sizes to LAPACK dgeqpf /
    dgeqp3) on every stride-th matrix, one matrix per host thread, one BLAS
    thread each (ctypes releases the GIL around each call); best of reps."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    try:
        impl, kind = oracle.Reference(), "reference"
    except RuntimeError:
        impl, kind = oracle.Oracle(), "port"
    impl.set_threads(1)
    idx = list(range(0, len(shapes), stride))
    As = []
    for i in idx:
        m, n = shapes[i]
        As.append(np.asfortranarray(flat0[offs[i]:offs[i + 1]].view(n, m).cpu().numpy().T))
    cores = os.cpu_count() or 1
    sec = 1e30
    with ThreadPoolExecutor(cores) as ex:
        for _ in range(reps):
            t0 = time.perf_counter()
            list(ex.map(lambda A: impl.dgeqp4(A), As))
            sec = min(sec, time.perf_counter() - t0)
    fl = sum(flops_qr(*shapes[i]) for i in idx)
    return {"value": fl / sec / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": kind,
            "cpu_model": cpu_model(),
            "sample": "dgeqp4 (-> LAPACK dgeqpf/dgeqp3) on %d of the %d matrices, %d threads "
                      "x 1 BLAS thread, best of %d: %.2f s" % (len(idx), len(shapes), cores,
                                                              reps, sec)}


def roofline_of(H, head, peaks, device):
    """Roofline of the dominant kernel of an arm, from its live phase profile:
    mixed -> the split-BF16 products (BF16 tensor work), plain -> dgemm_tile."""
    if head == "mixed":
        t_ms, t_fl = H["prof"]["tensor"]
        n_t = max(1, H["counts"].get("tensor", 0))
        peak = peaks.get("bf16_tflops_sustained") or 1700.0
        achieved = t_fl / (t_ms * 1e-3) / 1e12 if t_ms > 0 else None
        roofline = {"bound": "tensor", "pipe": "bf16 tcgen05",
                    "kernel": "ozk_gemm_kernel + ozk_gemm_short_kernel (split-BF16 digit "
                              "products of the block update, Gram, T^T W1 and sketch downdate)",
                    "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak if achieved else None,
                    "peak_source": "bf16_tflops_sustained of measured (MEASURED_PEAKS.json)"
                    if peaks.get("bf16_tflops_sustained") else "fallback 1.7 PFLOP/s sustained",
                    "launches": n_t, "flops_per_launch": t_fl / n_t,
                    "traffic": TENSOR_BYTES_PER_FLOP * t_fl / n_t,
                    "traffic_source": "ncu dram__bytes_read+write of W1 and C -= U'W2 at "
                                      "6144^2, scaled by flops per launch"}
    else:
        u_ms, u_fl = H["prof"]["update"]
        peak = fp64_peak_tflops(device)
        achieved = u_fl / (u_ms * 1e-3) / 1e12 if u_ms > 0 else None
        n_u = 3 * max(1, H["counts"].get("update", 0))  # W1, W2, U3 per block
        roofline = {"bound": "tensor", "pipe": "fp64",
                    "kernel": "dgemm_tile (trailing dlarfb update)",
                    "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak if achieved else None,
                    "peak_source": "cuBLAS DGEMM 8192^3 measured in this run (MEASURED_PEAKS.json "
                                   "has no FP64 figure)",
                    "launches": n_u, "flops_per_launch": u_fl / n_u,
                    "traffic": FP64_UPDATE_BYTES_PER_FLOP * u_fl / n_u,
                    "traffic_source": "ncu dram__bytes_read+write at 6144^2 scaled by flops "
                                      "per launch"}
    roofline["phases_ms"], roofline["phases_tflops"] = phase_table(H["prof"])
    return roofline


def e2e_host(hq, At0, m, n, nb, pp, steps, head, world, dist, device):
    """The same factorization end to end through the reference-facing C entry
    points, host buffers in and out inside the timed region:
    NoFLA_HQRRP_WY_blk_var4 and dgeqp4 (HQRRP nb=64, pp=10 inside) on
    page-locked buffers, and NoFLA_HQRRP_WY_blk_var4 on pageable memory (what a
    drop-in caller's malloc gives)."""
    import ctypes as C
    import torch
    L = hq.load()
    hq.set_precision(hq.MIXED if head == "mixed" else hq.PLAIN)
    host0 = At0.cpu().pin_memory()
    hA = torch.empty_like(host0).pin_memory()
    hjp = torch.empty(n, dtype=torch.int32).pin_memory()
    htau = torch.empty(min(m, n), dtype=torch.float64).pin_memory()
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)

    def hqrrp_call(A_ptr, jp_ptr, tau_ptr):
        rc = L.NoFLA_HQRRP_WY_blk_var4(m, n, C.cast(A_ptr, dp), m, C.cast(jp_ptr, ip),
                                       C.cast(tau_ptr, dp), nb, pp, 1)
        if rc != 0:
            raise RuntimeError("e2e call failed: %s" % hq.last_error())

    times = []
    for it in range(1 + steps):
        hA.copy_(host0)
        hjp.copy_(torch.arange(1, n + 1, dtype=torch.int32))
        t0 = time.perf_counter()
        hqrrp_call(hA.data_ptr(), hjp.data_ptr(), htau.data_ptr())
        if it > 0:
            times.append(time.perf_counter() - t0)
    sec = sum(times) / len(times)
    # dgeqp4 on the same page-locked buffers; all columns free.
    ltimes = []
    mi, ni, ldi, info = C.c_int(m), C.c_int(n), C.c_int(m), C.c_int(0)
    lwork = C.c_int(-1)
    wq = (C.c_double * 1)()
    L.dgeqp4(C.byref(mi), C.byref(ni), C.cast(hA.data_ptr(), dp), C.byref(ldi),
             C.cast(hjp.data_ptr(), ip), C.cast(htau.data_ptr(), dp), wq, C.byref(lwork),
             C.byref(info))
    work = (C.c_double * max(1, int(wq[0])))()
    lwork = C.c_int(max(1, int(wq[0])))
    for it in range(1 + steps):
        hA.copy_(host0)
        hjp.zero_()
        t0 = time.perf_counter()
        L.dgeqp4(C.byref(mi), C.byref(ni), C.cast(hA.data_ptr(), dp), C.byref(ldi),
                 C.cast(hjp.data_ptr(), ip), C.cast(htau.data_ptr(), dp), work,
                 C.byref(lwork), C.byref(info))
        dt = time.perf_counter() - t0
        if info.value != 0:
            raise RuntimeError("dgeqp4 failed: info %d %s" % (info.value, hq.last_error()))
        if it > 0:
            ltimes.append(dt)
    lsec = sum(ltimes) / len(ltimes)
    # dgeqp4 with the reference's CPU block size 64 for its HQRRP call
    # (hqrrp_gb300_set_dgeqp4_block; the GPU default is 128): one untimed call
    # under the phase profiler (where nb = 64 loses against 128), then timed.
    prev_nb = hq.set_dgeqp4_block(64)
    qtimes = []
    try:
        hA.copy_(host0)
        hjp.zero_()
        hq.profile_enable(True)
        hq.profile_read()
        L.dgeqp4(C.byref(mi), C.byref(ni), C.cast(hA.data_ptr(), dp), C.byref(ldi),
                 C.cast(hjp.data_ptr(), ip), C.cast(htau.data_ptr(), dp), work,
                 C.byref(lwork), C.byref(info))
        dprof = phase_table(hq.profile_read())
        hq.profile_enable(False)
        for it in range(1 + steps):
            hA.copy_(host0)
            hjp.zero_()
            t0 = time.perf_counter()
            L.dgeqp4(C.byref(mi), C.byref(ni), C.cast(hA.data_ptr(), dp), C.byref(ldi),
                     C.cast(hjp.data_ptr(), ip), C.cast(htau.data_ptr(), dp), work,
                     C.byref(lwork), C.byref(info))
            dt = time.perf_counter() - t0
            if info.value != 0:
                raise RuntimeError("dgeqp4 failed: info %d %s" % (info.value, hq.last_error()))
            if it > 0:
                qtimes.append(dt)
    finally:
        hq.set_dgeqp4_block(prev_nb)
    qsec = sum(qtimes) / len(qtimes)
    del hA
    # pageable host memory (numpy)
    pA0 = host0.numpy().copy()
    pA = np.empty_like(pA0)
    pjp = np.empty(n, np.int32)
    ptau = np.empty(min(m, n))
    ptimes = []
    for it in range(1 + steps):
        np.copyto(pA, pA0)
        pjp[:] = np.arange(1, n + 1, dtype=np.int32)
        t0 = time.perf_counter()
        hqrrp_call(pA.ctypes.data, pjp.ctypes.data, ptau.ctypes.data)
        if it > 0:
            ptimes.append(time.perf_counter() - t0)
    psec = sum(ptimes) / len(ptimes)
    del pA, pA0
    if dist:
        t = torch.tensor([sec, lsec, psec, qsec], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        sec, lsec, psec, qsec = float(t[0]), float(t[1]), float(t[2]), float(t[3])
    fl = world * flops_qr(m, n)
    return {"value": fl / sec / 1e12, "unit": "TFLOP/s",
            "h2d_bytes_per_step": 8 * m * n + 4 * n,
            "d2h_bytes_per_step": 8 * m * n + 4 * n + 8 * min(m, n),
            "ms_per_step": sec * 1e3, "precision": head,
            "api": "NoFLA_HQRRP_WY_blk_var4(nb=%d, pp=%d), host page-locked buffers" % (nb, pp),
            "dgeqp4": {"value": fl / lsec / 1e12, "unit": "TFLOP/s", "ms_per_step": lsec * 1e3,
                       "api": "dgeqp4 (HQRRP nb=128 inside: the GPU default block size; "
                              "pp=10), host page-locked buffers"},
            "dgeqp4_block64": {"value": fl / qsec / 1e12, "unit": "TFLOP/s",
                               "ms_per_step": qsec * 1e3,
                               "api": "dgeqp4 after hqrrp_gb300_set_dgeqp4_block(64), the "
                                      "reference's block size, host page-locked buffers",
                               "phases_ms": dprof[0], "phases_tflops": dprof[1]},
            "pageable": {"value": fl / psec / 1e12, "unit": "TFLOP/s", "ms_per_step": psec * 1e3,
                         "api": "NoFLA_HQRRP_WY_blk_var4(nb=%d, pp=%d), host pageable (numpy) "
                                "buffers" % (nb, pp)}}


def run_factorization(hq, args, name, device, dist, rank, world, local, steps, warmup,
                      plain_steps, plain_warmup, e2e_steps, precision):
    """Square or tall workload: time the arms, then the roofline and the end to
    end figures; returns (line, At0) with At0 the input on the device."""
    import torch
    nb, pp = args.nb, args.pp
    if name == "tall":
        n = args.n or 8192
        m = args.m or 4 * n
        sigma = spectrum_tall(min(m, n))
        wl = ("HQRRP m=%d n=%d nb=%d pp=%d panel_pivoting=1, A=U diag(sigma) V^T, Haar U,V, "
              "sigma geometric 1..1e-10 with 64 equal values at 1e-4" % (m, n, nb, pp))
    else:
        n = m = args.n or 16384
        sigma = spectrum(n)
        wl = ("HQRRP m=n=%d nb=%d pp=%d panel_pivoting=1, A=U diag(10^(-12 i/n)) V^T, "
              "Haar U,V" % (n, nb, pp))
    At0 = make_matrix_gpu(m, n, sigma, args.seed + rank, device)
    At = torch.empty_like(At0)
    iota = torch.arange(1, n + 1, dtype=torch.int32, device=device)
    jp = iota.clone()
    tau = torch.zeros(min(m, n), dtype=torch.float64, device=device)
    arms = ["mixed", "plain"] if precision == "both" else [precision]
    res = {}
    for p in arms:
        k, w = (plain_steps, plain_warmup) if (p == "plain" and len(arms) > 1) else (steps, warmup)
        res[p] = run_arm(hq, p, At0, At, jp, iota, tau, nb, pp, sigma, k, w, device, dist, local)
    del At
    head = arms[0]
    H = res[head]
    value = world * flops_qr(m, n) / (H["ms_per_step"] * 1e-3) / 1e12
    peaks = measured_peaks()
    roofline = roofline_of(H, head, peaks, device)
    e2e = None
    if e2e_steps > 0:
        e2e = e2e_host(hq, At0, m, n, nb, pp, e2e_steps, head, world, dist, device)
    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": H["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if head == "plain" else "f64 (split-bf16 tensor products)",
            "data": "synthetic",
            "config": {"workload": wl, "name": name, "m": m, "n": n, "nb": nb, "pp": pp,
                       "precision": head, "api": "hqrrp_gb300_hqrrp_device",
                       "parallelism": "replicas%d" % world,
                       "l2": "inputs larger than L2 (%.1f GB matrix per step)" % (8 * m * n / 1e9)},
            "quality": H["quality"], "roofline": roofline, "e2e": e2e,
            "gpu_launches": H["launches"], "clocks": H["clocks"],
            "measured_peaks": {k: peaks.get(k) for k in ("hbm_gbs", "bf16_tflops",
                                                          "bf16_tflops_sustained")}}
    if "plain" in res and head != "plain":
        P = res["plain"]
        pv = world * flops_qr(m, n) / (P["ms_per_step"] * 1e-3) / 1e12
        pm, pt = phase_table(P["prof"])
        line["plain"] = {"value": pv, "ms_per_step": P["ms_per_step"], "steps": P["steps"],
                         "warmup": P["warmup"], "quality": P["quality"],
                         "gpu_launches": P["launches"], "clocks": P["clocks"],
                         "phases_ms": pm, "phases_tflops": pt}
        line["mixed_over_plain"] = value / pv
        r = H["ratio"] / P["ratio"]
        line["quality"]["rkk_ratio_mixed_over_plain"] = [float(r.min()), float(r.max())]
    return line, At0


def run_single(hq, args, device):
    """One factorization of the square (or tall) workload's matrix, untimed:
    the command the ncu launch lists and captures run."""
    import torch
    if args.workload == "batched":
        shapes = batched_shapes(args.batch, args.seed)
        flat, offs = make_batched_gpu(shapes, args.seed, device)
        mats = [flat[offs[i]:offs[i + 1]].view(n, m) for i, (m, n) in enumerate(shapes)]
        bq = hq.BatchedQRP(shapes, autotune=False)
        bq.cfg = 3  # 256 threads, 96 KB staging, 2 CTAs per SM
        torch.cuda.synchronize()
        _, _, info = bq.run(mats)
        torch.cuda.synchronize()
        if int(info.abs().sum()) != 0:
            raise RuntimeError("batched QR reported errors")
        print("factored %d matrices" % len(shapes))
        return
    if args.workload == "tall":
        n = args.n or 8192
        m = args.m or 4 * n
        sigma = spectrum_tall(min(m, n))
    else:
        n = m = args.n or 16384
        sigma = spectrum(n)
    At = make_matrix_gpu(m, n, sigma, args.seed, device)
    jp = torch.arange(1, n + 1, dtype=torch.int32, device=device)
    tau = torch.zeros(min(m, n), dtype=torch.float64, device=device)
    hq.set_precision(hq.PLAIN if args.precision == "plain" else hq.MIXED)
    torch.cuda.synchronize()
    hq.hqrrp_device(At, jp, tau, args.nb, args.pp, 1)
    torch.cuda.synchronize()
    print("factored %d x %d (%s)" % (m, n, "plain" if args.precision == "plain" else "mixed"))


def sub_line(d, keep=("value", "unit", "ms_per_step", "steps", "warmup", "config", "quality",
                      "roofline", "e2e", "plain", "mixed_over_plain", "gpu_launches", "clocks",
                      "matrices_per_s", "cpu_baseline")):
    """A workload's own line, nested under the headline's."""
    return None if d is None else {k: d[k] for k in keep if k in d}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args)
        return

    import torch
    import hqrrp_gb300 as hq
    hq.load()
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)

    if args.single:
        run_single(hq, args, device)
        return
    if args.workload == "batched":
        line = run_batched(hq, args, device, dist, rank, world, local, args.steps, args.warmup)
        if line is not None:
            print(json.dumps(line), flush=True)
        if dist:
            dist.destroy_process_group()
        return

    # The plain FP64 arm beside the mixed headline: at most 5 timed steps after
    # 3 warm-ups (it is ~12x slower and only the comparison needs it).
    line, At0 = run_factorization(hq, args, args.workload, device, dist, rank, world, local,
                                  args.steps, args.warmup, min(args.steps, 5), 3,
                                  args.e2e_steps, args.precision)
    A_host = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.workload == "square":
        A_host = np.asfortranarray(At0.cpu().numpy().T)
    del At0
    torch.cuda.empty_cache()

    extras = args.workload == "square" and world == 1 and not args.no_extras
    if rank == 0 and not args.no_adjoint and args.workload == "square":
        hq.set_precision(hq.PLAIN)
        adj = measure_adjoint(hq, device)
        line["bwd_ms"], line["adjoint"] = adj["bwd_ms"], adj
    if extras:
        # The other measured workloads, each with its own figures, nested.
        targs = argparse.Namespace(**vars(args))
        targs.n, targs.m = 8192, 32768
        tall, tA = run_factorization(hq, targs, "tall", device, None, 0, 1, local,
                                     min(args.steps, 5), 3, 2, 1, 1, "both")
        del tA
        torch.cuda.empty_cache()
        line["tall"] = sub_line(tall)
        b = run_batched(hq, args, device, None, 0, 1, local, min(args.steps, 10), 3)
        line["batched"] = sub_line(b)
        torch.cuda.empty_cache()
    if A_host is not None:
        line["cpu_baseline"] = cpu_baseline_run(A_host, args)
    else:
        line["cpu_baseline"] = None
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
