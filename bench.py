#!/usr/bin/env python
"""Headline benchmark: HQRRP throughput on one GB300 (TFLOP/s, 2mn^2 - 2n^3/3).

Workload (the configuration the metric is quoted on): m = n = 16384,
A = U diag(sigma) V^T with Haar U, V (QR of seeded Gaussians, sign-fixed) and
sigma_i = 10^(-12 i / n), nb = 128, pp = 10, panel pivoting on.  Synthetic,
seeded; generated on the GPU before the timed region.

One step = one full factorization of a fresh copy of A (the 2.1 GB matrix is
larger than L2, so nothing carries over between steps).  The headline is the
mixed-precision path (split-BF16 tensor-core block updates); the plain FP64
path is timed the same way in the same run and reported beside it, with both
residuals.  ``value`` is timed
with CUDA events on the factorization's stream with A already in HBM;
``e2e`` goes through the reference-facing C entry point
NoFLA_HQRRP_WY_blk_var4 with host (pinned) buffers, so both copies are inside
its timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision both|mixed|plain]
  python bench.py --impl reference ...   # the reference algorithm on host cores

Under torchrun (N > 1) every rank factors its own matrix (replicas: a single
factorization does not shard), and value is the whole-job aggregate.
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


def flops_qr(m, n):
    k = min(m, n)
    return 2.0 * m * n * k - 2.0 * k ** 3 / 3.0 if m >= n else 2.0 * n * m * m - 2.0 * m ** 3 / 3.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default="both", choices=["both", "mixed", "plain"],
                   help="both (default): headline = mixed, plain timed alongside")
    p.add_argument("--n", type=int, default=16384)
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


def make_matrix_gpu(n, seed, device):
    """A^T (n x m, contiguous) = column-major A = U diag(sigma) V^T, FP64."""
    import ctypes
    import torch
    # torch loads its CUDA linear-algebra library lazily by bare name; load it by
    # path first so the lookup also succeeds under a profiler's injection.
    linalg = os.path.join(os.path.dirname(torch.__file__), "lib", "libtorch_cuda_linalg.so")
    if os.path.exists(linalg):
        ctypes.CDLL(linalg, mode=ctypes.RTLD_GLOBAL)
    g = torch.Generator(device=device).manual_seed(seed)

    def haar(k):
        Z = torch.randn(k, k, dtype=torch.float64, device=device, generator=g)
        Q, R = torch.linalg.qr(Z)
        Q *= torch.sign(torch.diagonal(R))[None, :]
        return Q

    U = haar(n)
    V = haar(n)
    sig = torch.from_numpy(spectrum(n)).to(device)
    At = (V * sig[None, :]) @ U.T  # (A)^T = V diag(sigma) U^T
    del U, V
    return At.contiguous()


def make_matrix_cpu(n, seed):
    import oracle
    return oracle.with_spectrum(n, n, spectrum(n), seed)


# ---------------------------------------------------------------------------
# Quality (measurement infrastructure): ||AP - QR||_F / ||A||_F estimated with
# r Gaussian probes, and |R_kk| / sigma_k.

def quality_gpu(At0, Atf, jp, tau, r=8, seed=1):
    import torch
    n, m = At0.shape
    k = min(m, n)
    g = torch.Generator(device=At0.device).manual_seed(seed)
    X = torch.randn(n, r, dtype=torch.float64, device=At0.device, generator=g)
    A = At0.T  # m x n view
    perm = jp.long() - 1
    APX = A[:, perm] @ X
    F = Atf.T  # factored, m x n view
    R = torch.triu(F[:k, :])
    Y = torch.zeros(m, r, dtype=torch.float64, device=At0.device)
    Y[:k] = R @ X
    taus = tau.cpu().numpy()
    for i in range(k - 1, -1, -1):  # Q Y = H_0 ... H_{k-1} Y
        t = float(taus[i])
        if t == 0.0:
            continue
        v = F[i:, i].clone()
        v[0] = 1.0
        Y[i:] -= t * torch.outer(v, v @ Y[i:])
    res = float(torch.linalg.norm(APX - Y) / torch.linalg.norm(APX))
    d = torch.abs(torch.diagonal(R)).cpu().numpy()
    return res, d


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
                             "sample": sample},
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


def run_arm(hq, precision, At0, At, jp, iota, tau, nb, pp, args, device, dist, local):
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
    res, diag = quality_gpu(At0, At, jp, tau)
    ratio = diag / spectrum(At0.shape[0])
    # One more (untimed) factorization under the phase profiler.
    hq.profile_enable(True)
    hq.profile_read()
    step()
    torch.cuda.synchronize()
    prof = hq.profile_read()
    hq.profile_enable(False)
    return {"ms_per_step": ms / args.steps, "launches": launches, "clocks": clocks,
            "quality": {"residual_est": res, "rkk_over_sigma_min": float(ratio.min()),
                        "rkk_over_sigma_max": float(ratio.max())},
            "ratio": ratio, "prof": prof}


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

    def orth(r, c):
        Q, R = torch.linalg.qr(torch.randn(r, c, dtype=torch.float64, device=device, generator=g))
        return Q * torch.sign(torch.diagonal(R))[None, :]

    U, V = orth(m, n), orth(n, n)
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

    n = m = args.n
    nb, pp = args.nb, args.pp
    At0 = make_matrix_gpu(n, args.seed + rank, device)
    At = torch.empty_like(At0)
    iota = torch.arange(1, n + 1, dtype=torch.int32, device=device)
    jp = iota.clone()
    tau = torch.zeros(min(m, n), dtype=torch.float64, device=device)

    arms = ["mixed", "plain"] if args.precision == "both" else [args.precision]
    res = {p: run_arm(hq, p, At0, At, jp, iota, tau, nb, pp, args, device, dist, local)
           for p in arms}
    head = arms[0]
    H = res[head]
    value = world * flops_qr(m, n) / (H["ms_per_step"] * 1e-3) / 1e12
    peaks = measured_peaks()

    # Roofline of the dominant kernel of the headline arm, from the live phase
    # profile: mixed -> ozk_gemm_kernel (BF16 tensor work), plain -> dgemm_tile.
    if head == "mixed":
        t_ms, t_fl = H["prof"]["tensor"]
        peak = peaks.get("bf16_tflops_sustained") or 1700.0
        achieved = t_fl / (t_ms * 1e-3) / 1e12 if t_ms > 0 else None
        roofline = {"bound": "tensor", "pipe": "bf16 tcgen05", "kernel": "ozk_gemm_kernel "
                    "(split-BF16 digit products of the block update and sketch downdate)",
                    "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak if achieved else None,
                    "peak_source": "bf16_tflops_sustained of measured (MEASURED_PEAKS.json)"
                    if peaks.get("bf16_tflops_sustained") else "fallback 1.7 PFLOP/s sustained",
                    "traffic": None}
    else:
        u_ms, u_fl = H["prof"]["update"]
        peak = fp64_peak_tflops(device)
        achieved = u_fl / (u_ms * 1e-3) / 1e12 if u_ms > 0 else None
        roofline = {"bound": "tensor", "pipe": "fp64", "kernel": "dgemm_tile (trailing dlarfb update)",
                    "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak if achieved else None,
                    "peak_source": "cuBLAS DGEMM 8192^3 measured in this run (MEASURED_PEAKS.json "
                                   "has no FP64 figure)", "traffic": None}
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
        if dist:
            t = torch.tensor([sec], dtype=torch.float64, device=device)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            sec = float(t)
        e2e = {"value": world * flops_qr(m, n) / sec / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": 8 * m * n + 4 * n,
               "d2h_bytes_per_step": 8 * m * n + 4 * n + 8 * min(m, n),
               "ms_per_step": sec * 1e3, "precision": head,
               "api": "NoFLA_HQRRP_WY_blk_var4 (host pinned buffers)"}

    adj = None
    if rank == 0 and not args.no_adjoint:
        hq.set_precision(hq.PLAIN)
        adj = measure_adjoint(hq, device)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        kind, cores, times = cpu_oracle_run(args.cpu_n, nb, pp, 2, args.seed)
        t = min(times)
        cpu = {"value": flops_qr(args.cpu_n, args.cpu_n) / t / 1e12, "unit": "TFLOP/s",
               "cores": cores, "kind": kind,
               "sample": "HQRRP nb=%d pp=%d on m=n=%d, same spectrum, best of 2, %.1f s each"
                         % (nb, pp, args.cpu_n, t)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": H["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if head == "plain" else "f64 (split-bf16 tensor products)",
                "data": "synthetic",
                "config": {"workload": "HQRRP m=n=%d nb=%d pp=%d panel_pivoting=1, "
                                       "A=U diag(10^(-12 i/n)) V^T, Haar U,V" % (n, nb, pp),
                           "m": m, "n": n, "nb": nb, "pp": pp, "precision": head,
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
