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
# (W1 and the rank-b update) and the FP64 update GEMMs (W1, C -= U W2).
TENSOR_BYTES_PER_FLOP = (550.2e6 + 556.1e6) / (2 * 2.649e11)
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
    p.add_argument("--cpu-n", type=int, default=6144, help="CPU baseline sample size")
    p.add_argument("--ref-n", type=int, default=8192, help="reference-arm sample size")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-adjoint", action="store_true", help="skip the bwd_ms measurement")
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


def cpu_oracle_run(n, nb, pp, reps, seed):
    import oracle
    try:
        impl = oracle.Reference()
        kind = "reference"
    except RuntimeError:
        impl = oracle.Oracle()
        kind = "port"
    cores = os.cpu_count() or 1
    impl.set_threads(cores)
    A = make_matrix_cpu(n, seed)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        impl.hqrrp(A, nb, pp, 1)
        times.append(time.perf_counter() - t0)
    return kind, cores, times


def cpu_dgeqp3_run(n, seed):
    import oracle
    o = oracle.Oracle()
    o.set_threads(os.cpu_count() or 1)
    A = make_matrix_cpu(n, seed)
    t0 = time.perf_counter()
    o.dgeqp3(A)
    return time.perf_counter() - t0


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.ref_n
    kind, cores, times = cpu_oracle_run(n, args.nb, args.pp, args.warmup + args.steps, args.seed)
    timed = times[args.warmup:] or times
    sec = sum(timed)
    value = flops_qr(n, n) * len(timed) / sec / 1e12
    sample = ("HQRRP nb=%d pp=%d on m=n=%d (same spectrum as the GPU workload), one "
              "factorization per step" % (args.nb, args.pp, n))
    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": len(timed), "warmup": args.warmup,
            "ms_per_step": sec / len(timed) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "HQRRP m=n=%d nb=%d pp=%d, reference algorithm on host cores"
                       % (n, args.nb, args.pp), "m": n, "n": n, "nb": args.nb, "pp": args.pp},
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


def run_arm(hq, precision, At0, At, jp, iota, tau, nb, pp, sigma, args, device, dist, local):
    """Warm up, then time exactly args.steps factorizations (one arm)."""
    import torch
    hq.set_precision(hq.MIXED if precision == "mixed" else hq.PLAIN)
    stream = torch.cuda.current_stream()

    def step():
        At.copy_(At0)
        jp.copy_(iota)
        hq.hqrrp_device(At, jp, tau, nb, pp, 1, stream=stream)

    for _ in range(args.warmup):
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
    for _ in range(args.steps):
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
    return {"ms_per_step": ms / args.steps, "launches": launches, "clocks": clocks,
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


def run_batched(hq, args, device, dist, rank, world, local):
    """Config: args.batch matrices of random shape, A_i = U diag(i^-2) V^T; one
    step = restore the inputs and replay the captured graph of one persistent
    launch over this rank's cost-balanced shard of the batch."""
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
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(local)
        sampler.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(args.steps):
            step()
        e1.record(s)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
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
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
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
                "gpu_launches": per_replay * args.steps, "clocks": clocks}
        line["roofline"]["frac"] = value / line["roofline"]["peak"]
        print(json.dumps(line), flush=True)


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

    if args.workload == "batched":
        run_batched(hq, args, device, dist, rank, world, local)
        if dist:
            dist.destroy_process_group()
        return
    nb, pp = args.nb, args.pp
    if args.workload == "tall":
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

    arms = ["mixed", "plain"] if args.precision == "both" else [args.precision]
    res = {p: run_arm(hq, p, At0, At, jp, iota, tau, nb, pp, sigma, args, device, dist, local)
           for p in arms}
    head = arms[0]
    H = res[head]
    value = world * flops_qr(m, n) / (H["ms_per_step"] * 1e-3) / 1e12
    peaks = measured_peaks()

    # Roofline of the dominant kernel of the headline arm, from the live phase
    # profile: mixed -> ozk_gemm_kernel (BF16 tensor work), plain -> dgemm_tile.
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
                    # DRAM bytes per BF16 flop of the two large products of a block,
                    # ncu at 6144^2 (W1 550.2 MB, C -= U'W2 556.1 MB per 2.649e11
                    # flops each), times this run's flops per launch.
                    "traffic": TENSOR_BYTES_PER_FLOP * t_fl / n_t,
                    "traffic_source": "ncu dram__bytes_read+write at 6144^2 scaled by flops "
                                      "per launch"}
    else:
        u_ms, u_fl = H["prof"]["update"]
        peak = fp64_peak_tflops(device)
        achieved = u_fl / (u_ms * 1e-3) / 1e12 if u_ms > 0 else None
        n_u = 3 * max(1, H["counts"].get("update", 0))  # W1, W2, U3 per block
        roofline = {"bound": "tensor", "pipe": "fp64", "kernel": "dgemm_tile (trailing dlarfb update)",
                    "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak if achieved else None,
                    "peak_source": "cuBLAS DGEMM 8192^3 measured in this run (MEASURED_PEAKS.json "
                                   "has no FP64 figure)",
                    "launches": n_u, "flops_per_launch": u_fl / n_u,
                    "traffic": FP64_UPDATE_BYTES_PER_FLOP * u_fl / n_u,
                    "traffic_source": "ncu dram__bytes_read+write at 6144^2 scaled by flops "
                                      "per launch"}
    roofline["phases_ms"], roofline["phases_tflops"] = phase_table(H["prof"])

    # End to end through the reference-facing C entry point, host buffers.
    e2e = None
    if args.e2e_steps > 0:
        import ctypes as C
        L = hq.load()
        hq.set_precision(hq.MIXED if head == "mixed" else hq.PLAIN)
        host0 = At0.cpu().pin_memory()
        hA = torch.empty_like(host0).pin_memory()
        hjp = torch.empty(n, dtype=torch.int32).pin_memory()
        htau = torch.empty(min(m, n), dtype=torch.float64).pin_memory()
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        times = []
        for it in range(1 + args.e2e_steps):
            hA.copy_(host0)
            hjp.copy_(torch.arange(1, n + 1, dtype=torch.int32))
            t0 = time.perf_counter()
            rc = L.NoFLA_HQRRP_WY_blk_var4(m, n, C.cast(hA.data_ptr(), dp), m,
                                           C.cast(hjp.data_ptr(), ip), C.cast(htau.data_ptr(), dp),
                                           nb, pp, 1)
            dt = time.perf_counter() - t0
            if rc != 0:
                raise RuntimeError("e2e call failed: %s" % hq.last_error())
            if it > 0:
                times.append(dt)
        sec = sum(times) / len(times)
        # dgeqp4 (HQRRP with nb = 64, pp = 10 inside, as the reference's) on
        # the same host buffers; all columns free.
        ltimes = []
        mi, ni, ldi, info = C.c_int(m), C.c_int(n), C.c_int(m), C.c_int(0)
        lwork = C.c_int(-1)
        wq = (C.c_double * 1)()
        L.dgeqp4(C.byref(mi), C.byref(ni), C.cast(hA.data_ptr(), dp), C.byref(ldi),
                 C.cast(hjp.data_ptr(), ip), C.cast(htau.data_ptr(), dp), wq, C.byref(lwork),
                 C.byref(info))
        work = (C.c_double * max(1, int(wq[0])))()
        lwork = C.c_int(max(1, int(wq[0])))
        for it in range(1 + args.e2e_steps):
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
        if dist:
            t = torch.tensor([sec, lsec], dtype=torch.float64, device=device)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            sec, lsec = float(t[0]), float(t[1])
        e2e = {"value": world * flops_qr(m, n) / sec / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": 8 * m * n + 4 * n,
               "d2h_bytes_per_step": 8 * m * n + 4 * n + 8 * min(m, n),
               "ms_per_step": sec * 1e3, "precision": head,
               "api": "NoFLA_HQRRP_WY_blk_var4(nb=%d, pp=%d), host pinned buffers" % (nb, pp),
               "dgeqp4": {"value": world * flops_qr(m, n) / lsec / 1e12, "unit": "TFLOP/s",
                          "ms_per_step": lsec * 1e3,
                          "api": "dgeqp4 (HQRRP nb=64, pp=10 inside), host pinned buffers"}}

    adj = None
    if rank == 0 and not args.no_adjoint and args.workload == "square":
        hq.set_precision(hq.PLAIN)
        adj = measure_adjoint(hq, device)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        kind, cores, times = cpu_oracle_run(args.cpu_n, nb, pp, 2, args.seed)
        t = min(times)
        t3 = cpu_dgeqp3_run(args.cpu_n, args.seed)
        cpu = {"value": flops_qr(args.cpu_n, args.cpu_n) / t / 1e12, "unit": "TFLOP/s",
               "cores": cores, "kind": kind, "cpu_model": cpu_model(),
               "sample": "HQRRP nb=%d pp=%d on m=n=%d, same spectrum as the square workload, "
                         "best of 2, %.1f s each" % (nb, pp, args.cpu_n, t),
               "lapack_dgeqp3": {"value": flops_qr(args.cpu_n, args.cpu_n) / t3 / 1e12,
                                 "unit": "TFLOP/s", "cores": cores, "seconds": t3,
                                 "sample": "LAPACK dgeqp3 (scipy OpenBLAS) on the same m=n=%d "
                                           "matrix, once" % args.cpu_n}}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": H["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if head == "plain" else "f64 (split-bf16 tensor products)",
                "data": "synthetic",
                "config": {"workload": wl, "name": args.workload, "m": m, "n": n, "nb": nb, "pp": pp, "precision": head,
                           "api": "hqrrp_gb300_hqrrp_device", "parallelism": "replicas%d" % world,
                           "l2": "inputs larger than L2 (%.1f GB matrix per step)"
                                 % (8 * m * n / 1e9)},
                "quality": H["quality"], "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": H["launches"], "clocks": H["clocks"],
                "bwd_ms": adj["bwd_ms"] if adj else None, "adjoint": adj,
                "measured_peaks": {k: peaks.get(k) for k in ("hbm_gbs", "bf16_tflops",
                                                              "bf16_tflops_sustained")}}
        if "plain" in res and head != "plain":
            P = res["plain"]
            pv = world * flops_qr(m, n) / (P["ms_per_step"] * 1e-3) / 1e12
            pm, pt = phase_table(P["prof"])
            line["plain"] = {"value": pv, "ms_per_step": P["ms_per_step"],
                             "quality": P["quality"], "gpu_launches": P["launches"],
                             "clocks": P["clocks"], "phases_ms": pm, "phases_tflops": pt}
            line["mixed_over_plain"] = value / pv
            r = H["ratio"] / P["ratio"]
            line["quality"]["rkk_ratio_mixed_over_plain"] = [float(r.min()), float(r.max())]
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
