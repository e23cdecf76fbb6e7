#!/usr/bin/env python3
"""Benchmark of the one-rank GEMM path on GB300.

Workload (the precision configuration): C = A*B with m = n = k = 16384, FP64,
column-major, entries u*2^e (u ~ U[-1, 1], integer e ~ U{-phi..phi}, phi = 0
for the headline, 8 and 32 as variants), seeded synthetic data.  One step is
one FP64-accurate GEMM through the Ozaki-split path (integer slices on the
FP8 tensor cores, exact accumulation, FP64 recombination) with the inputs
resident in HBM; `e2e` runs the same GEMM through the Tiled-MM C-ABI entry
point (cosma_gpu_tmm_gemm_d) from pinned host buffers, copies included.
Beside it: the native FP64 (DMMA) kernel on the same inputs, the accuracy of
both against a double-double oracle on sampled entries, the roofline of the
dominant kernel, and the reference's CPU path (OpenBLAS DGEMM, the arithmetic
cblas_dgemm performs at P = 1) timed on the host cores.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "FP64-accurate GEMM TFLOP/s: INT8-split vs native FP64 at <=1e-15 rel err"
UNIT = "TFLOP/s"
KERNELS_PER_STEP = 6  # A scale (2), B scale (1), A split, B split, slice-product GEMM


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--size", type=int, default=16384)
    p.add_argument("--phi", type=int, default=0)
    p.add_argument("--no-native", action="store_true", help="skip the native FP64 comparison run")
    p.add_argument("--no-variants", action="store_true", help="skip the phi = 8 / 32 variants")
    p.add_argument("--count", type=int, default=10000,
                   help="problems in the grouped configuration (10,000; fewer for profiler captures)")
    p.add_argument("--config", default="precision",
                   choices=["precision", "plain", "pdgemm", "sgemm", "grouped", "stream"],
                   help="precision: the headline line; pdgemm: the 1x1 ScaLAPACK configuration; "
                        "sgemm: the FP32 3xBF16 variant of the precision configuration; "
                        "grouped: the batching configuration")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_max_ms(ms, world, device=None):
    """Max over the ranks of one rank's time per step: the replicas run the
    same step independently, so the job takes as long as its slowest rank."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms


def job_tflops(flops_per_rank, world, ms):
    """Whole-job rate: every rank's flops over the slowest rank's time."""
    return flops_per_rank * world / (ms * 1e-3) / 1e12


def config(n, phi):
    return {"workload": f"precision: FP64-accurate DGEMM NN m=n=k={n}, u*2^e entries phi={phi}",
            "m": n, "n": n, "k": n, "phi": phi, "layout": "column-major", "alpha": 1.0, "beta": 0.0,
            "l2": "inputs larger than L2 (2 GiB per operand vs 129 MB)", "parallelism": "replicas"}


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        under = sorted(sm)[len(sm) // 4:] if sm else []  # drop idle edges of the window
        return {"sm_mhz": float(np.median(under)) if under else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_dgemm_sample(A, B, budget_s=12.0):
    """OpenBLAS DGEMM (numpy) on a K-slab of the workload, sized to ~budget_s."""
    n = A.shape[0]
    kb = 512
    t = time.perf_counter()
    np.matmul(A[:, :kb], B[:kb, :])
    dt = time.perf_counter() - t
    rate = 2.0 * n * n * kb / max(dt, 1e-6)
    kb = int(min(A.shape[1], max(512, (budget_s * rate) / (2.0 * n * n))))
    kb -= kb % 256
    t = time.perf_counter()
    np.matmul(A[:, :kb], B[:kb, :])
    dt = time.perf_counter() - t
    return 2.0 * n * n * kb / dt / 1e12, kb, dt


def run_reference(args):
    """The reference's CPU path on the host cores: at P = 1 cosma::multiply is
    one cblas_dgemm(ColMajor, N, N) (src/cosma/blas.cpp:35-48); the reference
    cannot be built here (MPI, ScaLAPACK, COSTA and Tiled-MM are absent), so
    its arithmetic runs through numpy's OpenBLAS on every host thread."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    n = args.size
    A = oracle.exp_spread((n, n), 1, args.phi)
    B = oracle.exp_spread((n, n), 2, args.phi)
    kb = min(1024, n)
    for _ in range(max(1, args.warmup)):
        np.matmul(A[:, :kb], B[:kb, :])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        np.matmul(A[:, :kb], B[:kb, :])
    dt = time.perf_counter() - t0
    flops = 2.0 * n * n * kb * args.steps
    val = flops / dt / 1e12
    cores = int(os.environ.get("OPENBLAS_NUM_THREADS", os.cpu_count() or 1))
    out = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": config(n, args.phi),
           "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": f"OpenBLAS DGEMM NN {n}x{n}x{kb} K-slab of the workload per step"},
           "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_pdgemm(args):
    """pdgemm on a 1x1 grid: C = 1.5 * A^T * B + 0.5 * C, m = n = 4096, k = 65536,
    128 x 128 blocks, N(0,1) entries.  Device phases (COSTA pack of A with
    transpose, pack of B, GEMM, alpha/beta unpack) are timed with CUDA events on
    the launching stream; e2e is the pdgemm_ symbol called with host arrays."""
    import torch

    import cosma_gb300 as cg
    import oracle

    dev = torch.device("cuda", 0)
    m = n = 4096
    k = 65536
    alpha, beta = 1.5, 0.5
    A = oracle.normal((k, m), 1)  # stored k x m, op(A) = A^T
    B = oracle.normal((k, n), 2)
    C0 = oracle.normal((m, n), 3)
    dAsc = torch.from_numpy(A.reshape(-1, order="F")).to(dev)
    dBsc = torch.from_numpy(B.reshape(-1, order="F")).to(dev)
    dCsc = torch.from_numpy(C0.reshape(-1, order="F")).to(dev)
    dA = torch.empty(m * k, dtype=torch.float64, device=dev)
    dB = torch.empty(k * n, dtype=torch.float64, device=dev)
    dCc = torch.empty(m * n, dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream(dev)
    method = "ozaki"

    def phases():
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev[0].record(s)
        cg.pack("T", m, k, dAsc, k, dA, m, stream=s)
        ev[1].record(s)
        cg.pack("N", k, n, dBsc, k, dB, k, stream=s)
        ev[2].record(s)
        if method == "ozaki":
            cg.dgemm_ozaki_device("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, dCc, m, stream=s)
        else:
            cg.gemm_device("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, dCc, m, method=method, stream=s)
        ev[3].record(s)
        cg.unpack(m, n, alpha, dCc, m, beta, dCsc, m, stream=s)
        ev[4].record(s)
        torch.cuda.synchronize()
        return [ev[i].elapsed_time(ev[i + 1]) for i in range(4)]

    for _ in range(max(args.warmup, 3)):
        dCsc.copy_(torch.from_numpy(C0.reshape(-1, order="F")))
        phases()
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    times = []
    for _ in range(args.steps):
        times.append(phases())
    clocks = sampler.stop()
    t = np.median(np.array(times), axis=0)
    total = float(t.sum())
    flops = 2.0 * m * n * k
    pk, pk_kind = peaks()
    pack_a_bytes = 2.0 * m * k * 8
    pack_b_bytes = 2.0 * k * n * 8
    unpack_bytes = 3.0 * m * n * 8
    gbs = lambda b, ms: b / (ms * 1e-3) / 1e9
    # e2e: the ScaLAPACK symbol with host arrays
    desca = cg.descinit(k, m, 128, 128, 0, 0, 0, k)
    descb = cg.descinit(k, n, 128, 128, 0, 0, 0, k)
    descc = cg.descinit(m, n, 128, 128, 0, 0, 0, m)
    cg.pxgemm_set_method(method)
    Ch = C0.copy(order="F")
    cg.pxgemm("T", "N", m, n, k, alpha, A, 1, 1, desca, B, 1, 1, descb, beta, Ch, 1, 1, descc)
    e2e = []
    for _ in range(max(1, min(args.steps, 3))):
        Ch = C0.copy(order="F")
        t0 = time.perf_counter()
        cg.pxgemm("T", "N", m, n, k, alpha, A, 1, 1, desca, B, 1, 1, descb, beta, Ch, 1, 1, descc)
        e2e.append(time.perf_counter() - t0)
    cg.pxgemm_set_method("native")
    e2e_s = float(np.median(e2e))
    # accuracy of the host result on sampled entries (double-double oracle)
    rng = np.random.default_rng(7)
    rows, cols = rng.integers(0, m, 1024), rng.integers(0, n, 1024)
    hi, lo, ab = oracle.gemm_dd_sampled("T", "N", A, B, rows, cols)
    exact = alpha * (hi + lo) + beta * C0[rows, cols]
    rel = np.abs(Ch[rows, cols] - exact) / np.maximum(np.abs(exact), 1e-300)
    out = {"metric": "pdgemm 1x1 TFLOP/s (COSTA pack + FP64-accurate GEMM + unpack)",
           "value": flops / (total * 1e-3) / 1e12, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": max(args.warmup, 3), "ms_per_step": total, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic N(0,1), seeded",
           "config": {"workload": "pdgemm 1x1 grid C = 1.5*A^T*B + 0.5*C, m=n=4096, k=65536, 128x128 blocks",
                      "gemm_method": method},
           "phases_ms": {"pack_A_transpose": t[0], "pack_B": t[1], "gemm": t[2], "unpack_alpha_beta": t[3]},
           "pack_GBs": {"A_transpose": gbs(pack_a_bytes, t[0]), "B_copy": gbs(pack_b_bytes, t[1]),
                        "unpack": gbs(unpack_bytes, t[3])},
           "roofline": {"bound": "hbm", "achieved": gbs(pack_a_bytes, t[0]), "peak": pk["hbm_gbs"], "unit": "GB/s",
                        "frac": gbs(pack_a_bytes, t[0]) / pk["hbm_gbs"], "traffic": None,
                        "kernel": "transpose_kernel (COSTA pack, op T)", "peak_note": pk_kind},
           "accuracy": {"max_rel_err": float(rel.max()), "mean_rel_err": float(rel.mean()), "samples": 1024},
           "e2e": {"value": flops / e2e_s / 1e12, "unit": UNIT, "h2d_bytes_per_step": (m * k + k * n + m * n) * 8,
                   "d2h_bytes_per_step": m * n * 8, "entry": "pdgemm_ (ScaLAPACK symbol), host arrays",
                   "host_copy_route": cg.host_copy_route(A),
                   "ms_per_step": e2e_s * 1e3},
           "clocks": clocks, "gpu_launches": 4 * args.steps}
    print(json.dumps(out), flush=True)


def run_sgemm(args):
    """FP32 GEMM m = n = k = 16384, N(0,1) entries, through the 3xBF16 path;
    cuBLAS SGEMM (FP32 SIMT, TF32 off) timed beside it for context."""
    import torch

    import cosma_gb300 as cg
    import oracle

    dev = torch.device("cuda", 0)
    n = args.size
    A = oracle.normal((n, n), 1, dtype=np.float32)
    B = oracle.normal((n, n), 2, dtype=np.float32)
    dA = torch.from_numpy(A.reshape(-1, order="F")).to(dev)
    dB = torch.from_numpy(B.reshape(-1, order="F")).to(dev)
    dC = torch.empty(n * n, dtype=torch.float32, device=dev)
    s = torch.cuda.current_stream(dev)

    def step():
        cg.gemm_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, method="bf16x3", stream=s, scalar="s")

    for _ in range(max(args.warmup, 3)):
        step()
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        step()
    e1.record(s)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    flops = 2.0 * n * n * n
    rng = np.random.default_rng(5)
    rows, cols = rng.integers(0, n, 2048), rng.integers(0, n, 2048)
    Cg = dC.cpu().numpy().reshape(n, n).T
    exact = np.einsum("ij,ji->i", A[rows, :].astype(np.float64), B[:, cols].astype(np.float64))
    absab = np.einsum("ij,ji->i", np.abs(A[rows, :]).astype(np.float64), np.abs(B[:, cols]).astype(np.float64))
    err = np.abs(Cg[rows, cols] - exact)
    # cuBLAS SGEMM on the same data (row-major view: C^T = B^T A^T)
    torch.backends.cuda.matmul.allow_tf32 = False
    At = dA.view(n, n)  # = A^T row-major
    Bt = dB.view(n, n)
    Ct = torch.matmul(Bt, At)
    torch.cuda.synchronize()
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record()
    Ct = torch.matmul(Bt, At)
    c1.record()
    torch.cuda.synchronize()
    cublas_ms = c0.elapsed_time(c1)
    Cc = Ct.cpu().numpy().T  # column-major C
    err_cublas = np.abs(Cc[rows, cols] - exact)
    pk, pk_kind = peaks()
    out = {"metric": "FP32 GEMM TFLOP/s (3xBF16 split on BF16 tensor cores)", "value": flops / (ms * 1e-3) / 1e12,
           "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic N(0,1), seeded",
           "config": {"workload": f"precision: SGEMM NN m=n=k={n}, N(0,1), 3xBF16 (6 BF16 products)"},
           "accuracy": {"max_err_over_absab": float((err / absab).max()), "max_abs_err": float(err.max()),
                        "cublas_sgemm_max_err_over_absab": float((err_cublas / absab).max())},
           "cublas_sgemm_tflops": flops / (cublas_ms * 1e-3) / 1e12,
           "roofline": {"bound": "tensor", "achieved": 6 * flops / (ms * 1e-3) / 1e12, "peak": pk["bf16_tflops"],
                        "unit": "TFLOP/s", "frac": 6 * flops / (ms * 1e-3) / 1e12 / pk["bf16_tflops"],
                        "traffic": None, "kernel": "bf16x3_gemm_kernel (tcgen05 kind::f16), step incl. slicing",
                        "peak_note": f"{pk_kind} BF16 burst"},
           "clocks": clocks, "gpu_launches": 3 * args.steps}
    print(json.dumps(out), flush=True)


def run_grouped(args):
    """10,000 independent FP64 GEMMs, m, n, k log-uniform integers in [16, 1024],
    transa/transb uniform in {N, T}, U[-1, 1] entries: one persistent grouped
    launch (autotuned, CUDA graph) against a loop of per-problem drop-in calls."""
    import torch

    import cosma_gb300 as cg

    dev = torch.device("cuda", 0)
    count = args.count
    rng = np.random.default_rng(2024)
    draw = lambda: np.clip(np.round(np.exp(rng.uniform(np.log(16), np.log(1024), count))), 16, 1024).astype(np.int64)
    m, n, k = draw(), draw(), draw()
    ta = rng.choice(["N", "T"], count)
    tb = rng.choice(["N", "T"], count)
    align = lambda x: (x + 31) // 32 * 32
    sa, sb, sc = np.cumsum([0] + [align(x) for x in m * k]), np.cumsum([0] + [align(x) for x in k * n]), \
        np.cumsum([0] + [align(x) for x in m * n])
    g = torch.Generator(device=dev).manual_seed(7)
    dA = torch.rand(int(sa[-1]), dtype=torch.float64, device=dev, generator=g) * 2 - 1
    dB = torch.rand(int(sb[-1]), dtype=torch.float64, device=dev, generator=g) * 2 - 1
    dC = torch.zeros(int(sc[-1]), dtype=torch.float64, device=dev)
    pa, pb, pc = dA.data_ptr(), dB.data_ptr(), dC.data_ptr()
    probs = []
    for i in range(count):
        lda = int(m[i] if ta[i] == "N" else k[i])
        ldb = int(k[i] if tb[i] == "N" else n[i])
        probs.append((str(ta[i]), str(tb[i]), int(m[i]), int(n[i]), int(k[i]), 1.0, pa + 8 * int(sa[i]), lda,
                      pb + 8 * int(sb[i]), ldb, 0.0, pc + 8 * int(sc[i]), int(m[i])))
    useful = float((2 * m * n * k).sum())
    t0 = time.perf_counter()
    plan = cg.GroupedPlan(probs, method="native", autotune=True)
    plan_s = time.perf_counter() - t0
    s = torch.cuda.current_stream(dev)
    for _ in range(max(args.warmup, 3)):
        plan.run(stream=s)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        plan.run(stream=s)
    e1.record(s)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    info = plan.info()
    # accuracy on sampled problems against FP64 numpy (OpenBLAS)
    worst = 0.0
    for i in rng.choice(count, 24, replace=False):
        A = dA[int(sa[i]):int(sa[i]) + int(m[i] * k[i])].cpu().numpy()
        B = dB[int(sb[i]):int(sb[i]) + int(k[i] * n[i])].cpu().numpy()
        Cg = dC[int(sc[i]):int(sc[i]) + int(m[i] * n[i])].cpu().numpy().reshape(int(n[i]), int(m[i])).T
        # column-major storage: a rows x cols matrix is flat.reshape(cols, rows).T
        Am = A.reshape(int(k[i]), int(m[i])).T if ta[i] == "N" else A.reshape(int(m[i]), int(k[i]))
        Bm = B.reshape(int(n[i]), int(k[i])).T if tb[i] == "N" else B.reshape(int(k[i]), int(n[i]))
        ref = Am @ Bm
        worst = max(worst, float(np.max(np.abs(Cg - ref) / (np.abs(Am) @ np.abs(Bm)))))
    plan.close()
    # the same batch in the INT8-split (Ozaki) arithmetic: one graph of
    # grouped scale / check / split launches and one persistent FP8 GEMM
    t0 = time.perf_counter()
    oplan = cg.GroupedPlan(probs, method="ozaki", autotune=True)
    oplan_s = time.perf_counter() - t0
    for _ in range(max(args.warmup, 3)):
        oplan.run(stream=s)
    torch.cuda.synchronize()
    o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    o0.record(s)
    for _ in range(args.steps):
        oplan.run(stream=s)
    o1.record(s)
    torch.cuda.synchronize()
    oms = o0.elapsed_time(o1) / args.steps
    oinfo = oplan.info()
    oslices = oplan.slices()
    oworst = 0.0
    for i in rng.choice(count, 24, replace=False):
        A = dA[int(sa[i]):int(sa[i]) + int(m[i] * k[i])].cpu().numpy()
        B = dB[int(sb[i]):int(sb[i]) + int(k[i] * n[i])].cpu().numpy()
        Cg = dC[int(sc[i]):int(sc[i]) + int(m[i] * n[i])].cpu().numpy().reshape(int(n[i]), int(m[i])).T
        Am = A.reshape(int(k[i]), int(m[i])).T if ta[i] == "N" else A.reshape(int(m[i]), int(k[i]))
        Bm = B.reshape(int(n[i]), int(k[i])).T if tb[i] == "N" else B.reshape(int(k[i]), int(n[i]))
        oworst = max(oworst, float(np.max(np.abs(Cg - Am @ Bm) / (np.abs(Am) @ np.abs(Bm)))))
    oplan.close()
    ozaki = {"tflops": useful / (oms * 1e-3) / 1e12, "ms": oms, "plan_build_s": oplan_s,
             "speedup_vs_native_grouped": ms / oms, "tiles": oinfo["tiles"],
             "fp8_flops_issued": oinfo["padded_flops"], "slices_min_max": [min(oslices), max(oslices)],
             "accuracy": {"max_err_over_absab_24_problems_vs_fp64_blas": oworst},
             "kernels_per_run": "scale (2) + check + split (one per slice count and memory order) + GEMM"}
    # loop of per-problem drop-in calls (the reference's way of running a batch)
    torch.cuda.synchronize()
    l0 = time.perf_counter()
    for (pta, ptb, pm, pn, pk, al, A, lda, B, ldb, be, Cm, ldc) in probs:
        cg.gemm_device(pta, ptb, pm, pn, pk, al, A, lda, B, ldb, be, Cm, ldc, method="native", stream=s, scalar="d")
    torch.cuda.synchronize()
    loop_s = time.perf_counter() - l0
    # native FP64 peak reference: one large native DGEMM
    big = 4096
    X = torch.rand(big * big, dtype=torch.float64, device=dev)
    Y = torch.empty_like(X)
    cg.gemm_device("N", "N", big, big, big, 1.0, X, big, X, big, 0.0, Y, big, method="native", stream=s)
    torch.cuda.synchronize()
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b0.record(s)
    cg.gemm_device("N", "N", big, big, big, 1.0, X, big, X, big, 0.0, Y, big, method="native", stream=s)
    b1.record(s)
    torch.cuda.synchronize()
    native_peak = 2.0 * big ** 3 / (b0.elapsed_time(b1) * 1e-3) / 1e12
    value = useful / (ms * 1e-3) / 1e12
    out = {"metric": f"grouped FP64 GEMM TFLOP/s ({count:,} uneven problems, one launch)", "value": value, "unit": UNIT,
           "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic U[-1,1], seeded",
           "config": {"workload": f"batching: {count:,} FP64 GEMMs, m,n,k log-uniform in [16,1024], random N/T",
                      "useful_gflop": useful / 1e9},
           "plan": info, "plan_build_s": plan_s,
           "frac_of_native_fp64": value / native_peak, "native_fp64_tflops_4096": native_peak,
           "loop_of_dropin_calls": {"tflops": useful / loop_s / 1e12, "s": loop_s},
           "ozaki_split_form": ozaki,
           "accuracy": {"max_err_over_absab_24_problems": worst},
           "roofline": {"bound": "fp64", "achieved": value, "peak": native_peak, "unit": "TFLOP/s",
                        "frac": value / native_peak, "traffic": None, "kernel": "grouped_dmma_kernel",
                        "peak_note": "measured: this library's native DGEMM at 4096^3 on the same GPU"},
           "clocks": clocks, "gpu_launches": args.steps}
    print(json.dumps(out), flush=True)


def run_plain(args):
    """The plain small configuration: DGEMM C = A*B, m = n = k = 2048, NN, alpha = 1,
    beta = 0, A and B U[-1,1] from seeds 1 and 2.  The native FP64 drop-in on
    device-resident data (value), the same call end to end through
    cosma_gpu_local_multiply_d from host buffers (e2e, the one-rank
    cosma::multiply), the error bound c*k*u*(|A||B|) against OpenBLAS on the
    host, the Ozaki form beside it, and OpenBLAS itself timed on the host cores."""
    import torch

    import cosma_gb300 as cg
    import oracle

    n = 2048 if args.size == 16384 else args.size
    dev = torch.device("cuda", 0)
    A = oracle.uniform((n, n), 1)
    B = oracle.uniform((n, n), 2)
    dA = torch.from_numpy(A.reshape(-1, order="F")).to(dev)
    dB = torch.from_numpy(B.reshape(-1, order="F")).to(dev)
    dC = torch.empty(n * n, dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream(dev)
    flops = 2.0 * n ** 3

    def timed(method):
        for _ in range(max(args.warmup, 3)):
            cg.gemm_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, method=method, stream=s)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(args.steps):
            cg.gemm_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, method=method, stream=s)
        e1.record(s)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps, dC.cpu().numpy().reshape(n, n).T

    sampler = ClockSampler(0)
    sampler.start()
    ms, Cn = timed("native")
    clocks = sampler.stop()
    oms, Co = timed("ozaki")
    # host reference (the reference's CPU arithmetic) and its timing
    t0 = time.perf_counter()
    reps = 0
    while True:
        ref = A @ B
        reps += 1
        if time.perf_counter() - t0 > 10.0:
            break
    cpu_s = (time.perf_counter() - t0) / reps
    absab = np.abs(A) @ np.abs(B)
    bound = 2.0 * (n + 2) * 2.0 ** -53 * absab
    within = bool(np.all(np.abs(Cn - ref) <= bound))
    # end to end: cosma::local_multiply on a one-rank strategy, host buffers
    hA = torch.from_numpy(A.reshape(-1, order="F")).pin_memory()
    hB = torch.from_numpy(B.reshape(-1, order="F")).pin_memory()
    hC = torch.empty(n * n, dtype=torch.float64).pin_memory()
    cg.local_multiply(hA, hB, hC, n, n, n, 1.0, 0.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cg.local_multiply(hA, hB, hC, n, n, n, 1.0, 0.0)
    e2e_s = (time.perf_counter() - t0) / args.steps
    value = flops / (ms * 1e-3) / 1e12
    out = {"metric": "plain FP64 DGEMM TFLOP/s (native drop-in)", "value": value, "unit": UNIT, "n_gpus": 1,
           "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic U[-1,1], seeds 1 and 2",
           "config": {"workload": f"plain: DGEMM NN m=n=k={n}, alpha=1, beta=0, column-major",
                      "l2": "operands 32 MiB each, inside L2; dmma kernel re-reads tiles from L2"},
           "within_ckuAB_bound": within, "bound": "2 (k+2) u (|A||B|) elementwise vs OpenBLAS",
           "max_err_over_absab": float(np.max(np.abs(Cn - ref) / absab)),
           "ozaki_form": {"tflops": flops / (oms * 1e-3) / 1e12, "ms": oms,
                          "max_err_over_absab": float(np.max(np.abs(Co - ref) / absab))},
           "e2e": {"value": flops / e2e_s / 1e12, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * n * n,
                   "d2h_bytes_per_step": 8 * n * n, "entry": "cosma_gpu_local_multiply_d, pinned host buffers"},
           "cpu_baseline": {"value": flops / cpu_s / 1e12, "unit": UNIT, "cores": oracle.openblas_threads(),
                            "kind": "port", "sample": f"OpenBLAS DGEMM NN {n}^3, {reps} repetitions"},
           "clocks": clocks, "gpu_launches": args.steps}
    print(json.dumps(out), flush=True)


def run_stream(args):
    """Out-of-HBM streaming through the Tiled-MM entry point from pinned host
    memory, with tile limits far below the problem so every operand streams:
      * FP64-accurate (Ozaki) DGEMM, m = n = k = 32768, tiles 8192^3;
      * the configuration's own operation, ZGEMM C = A * B^H, native FP64
        (m = n = k = 8192, 4096^3 tiles) and Ozaki-split (m = n = k = 16384,
        8192^3 tiles; the headline value).
    The full configuration (65536^3 complex, 206 GB of host matrices) exceeds
    this box's 214 GB of host memory, and native FP64 would need ~35 minutes
    for it; link behaviour is measured at these sizes instead."""
    import torch

    import cosma_gb300 as cg

    link_h2d = 211.0  # GB/s, pinned H2D measured on this machine's GB300 (probe of torch copies)
    out_runs = {}
    # 1. Ozaki DGEMM streamed
    n = 32768 if args.size == 16384 else args.size
    tile = n // 4
    g = torch.Generator().manual_seed(3)
    hA = (torch.rand(n * n, dtype=torch.float64, generator=g) * 2 - 1).pin_memory()
    hB = (torch.rand(n * n, dtype=torch.float64, generator=g) * 2 - 1).pin_memory()
    hC = torch.empty(n * n, dtype=torch.float64).pin_memory()
    h = cg.make_context("d", 3, tile, tile, tile)
    h.set_method("ozaki", 0)
    cg.gemm(h, "N", "N", n, n, n, 1.0, hA, n, hB, n, 0.0, hC, n)  # warm-up: allocates the rings
    times = []
    for _ in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        cg.gemm(h, "N", "N", n, n, n, 1.0, hA, n, hB, n, 0.0, hC, n)
        times.append(time.perf_counter() - t0)
    h2d, d2h = h.transfer_bytes()
    info = h.ozaki_info()
    wall = float(np.median(times))
    flops = 2.0 * n ** 3
    # compute alone on one device-resident tile step, scaled by the number of steps
    steps = (n // tile) ** 3
    dA = torch.empty(tile * tile, dtype=torch.float64, device="cuda").uniform_(-1, 1)
    dC = torch.empty_like(dA)
    cg.dgemm_ozaki_device("N", "N", tile, tile, tile, 1.0, dA, tile, dA, tile, 0.0, dC, tile)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cg.dgemm_ozaki_device("N", "N", tile, tile, tile, 1.0, dA, tile, dA, tile, 0.0, dC, tile)
    torch.cuda.synchronize()
    compute_s = (time.perf_counter() - t0) * steps
    link_s = (h2d + d2h) / (link_h2d * 1e9)
    # spot-check 256 entries against FP64 on the host
    rng = np.random.default_rng(1)
    rows, cols = rng.integers(0, n, 256), rng.integers(0, n, 256)
    An = hA.numpy().reshape(n, n).T
    Bn = hB.numpy().reshape(n, n).T
    Cn = hC.numpy().reshape(n, n).T
    exact = np.einsum("ij,ji->i", An[rows, :], Bn[:, cols])
    absab = np.einsum("ij,ji->i", np.abs(An[rows, :]), np.abs(Bn[:, cols]))
    out_runs["ozaki_dgemm"] = {
        "m": n, "tile": tile, "tflops": flops / wall / 1e12, "wall_s": wall, "h2d_bytes": h2d, "d2h_bytes": d2h,
        "link_GBs_achieved": (h2d + d2h) / wall / 1e9, "link_GBs_measured_peak": link_h2d,
        "compute_alone_s": compute_s, "link_alone_s": link_s,
        "overlap_efficiency": max(compute_s, link_s) / wall, "slices": info["slices"],
        "max_err_over_absab_256": float((np.abs(Cn[rows, cols] - exact) / absab).max())}
    h.close()
    del hA, hB, hC, dA, dC
    # 2. ZGEMM C = A * B^H, native FP64, streamed
    nz, tz = 8192, 4096
    hA = torch.complex(torch.rand(nz * nz, dtype=torch.float64, generator=g) * 2 - 1,
                       torch.rand(nz * nz, dtype=torch.float64, generator=g) * 2 - 1).pin_memory()
    hB = torch.complex(torch.rand(nz * nz, dtype=torch.float64, generator=g) * 2 - 1,
                       torch.rand(nz * nz, dtype=torch.float64, generator=g) * 2 - 1).pin_memory()
    hC = torch.empty(nz * nz, dtype=torch.complex128).pin_memory()
    hz = cg.make_context("z", 3, tz, tz, tz)
    t0 = time.perf_counter()
    cg.gemm(hz, "N", "C", nz, nz, nz, 1.0, hA, nz, hB, nz, 0.0, hC, nz)
    zwall = time.perf_counter() - t0
    zh2d, zd2h = hz.transfer_bytes()
    Az = hA.numpy().reshape(nz, nz).T
    Bz = hB.numpy().reshape(nz, nz).T
    Cz = hC.numpy().reshape(nz, nz).T
    r2, c2 = rng.integers(0, nz, 64), rng.integers(0, nz, 64)
    exact = np.einsum("ij,ij->i", Az[r2, :], Bz[c2, :].conj())
    out_runs["zgemm_a_bh_native"] = {
        "m": nz, "tile": tz, "tflops": 8.0 * nz ** 3 / zwall / 1e12, "wall_s": zwall, "h2d_bytes": zh2d,
        "d2h_bytes": zd2h, "link_GBs_achieved": (zh2d + zd2h) / zwall / 1e9,
        "max_rel_err_64": float((np.abs(Cz[r2, c2] - exact) / np.abs(exact)).max())}
    hz.close()
    del hA, hB, hC
    # 3. the configuration's operation in the precision form: ZGEMM C = A * B^H
    #    split into digit slices (four real products per complex one), streamed
    n3, t3 = 16384, 8192
    hA = torch.complex(torch.rand(n3 * n3, dtype=torch.float64, generator=g) * 2 - 1,
                       torch.rand(n3 * n3, dtype=torch.float64, generator=g) * 2 - 1).pin_memory()
    hB = torch.complex(torch.rand(n3 * n3, dtype=torch.float64, generator=g) * 2 - 1,
                       torch.rand(n3 * n3, dtype=torch.float64, generator=g) * 2 - 1).pin_memory()
    hC = torch.empty(n3 * n3, dtype=torch.complex128).pin_memory()
    h3 = cg.make_context("z", 3, t3, t3, t3)
    h3.set_method("ozaki", 0)
    cg.gemm(h3, "N", "C", n3, n3, n3, 1.0, hA, n3, hB, n3, 0.0, hC, n3)  # warm-up: allocates the rings
    ztimes = []
    for _ in range(max(1, min(args.steps, 2))):
        t0 = time.perf_counter()
        cg.gemm(h3, "N", "C", n3, n3, n3, 1.0, hA, n3, hB, n3, 0.0, hC, n3)
        ztimes.append(time.perf_counter() - t0)
    z3h2d, z3d2h = h3.transfer_bytes()
    z3info = h3.ozaki_info()
    z3wall = float(np.median(ztimes))
    dA = torch.complex(torch.rand(t3 * t3, dtype=torch.float64, device="cuda") * 2 - 1,
                       torch.rand(t3 * t3, dtype=torch.float64, device="cuda") * 2 - 1)
    dC = torch.empty_like(dA)
    cg.zgemm_ozaki_device("N", "C", t3, t3, t3, 1.0, dA, t3, dA, t3, 0.0, dC, t3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cg.zgemm_ozaki_device("N", "C", t3, t3, t3, 1.0, dA, t3, dA, t3, 0.0, dC, t3)
    torch.cuda.synchronize()
    z3compute = (time.perf_counter() - t0) * (n3 // t3) ** 3
    z3link = (z3h2d + z3d2h) / (link_h2d * 1e9)
    Az = hA.numpy().reshape(n3, n3).T
    Bz = hB.numpy().reshape(n3, n3).T
    Cz = hC.numpy().reshape(n3, n3).T
    r3, c3 = rng.integers(0, n3, 64), rng.integers(0, n3, 64)
    exact = np.einsum("ij,ij->i", Az[r3, :], Bz[c3, :].conj())
    absab = np.einsum("ij,ij->i", np.abs(Az[r3, :]), np.abs(Bz[c3, :]))
    out_runs["zgemm_a_bh_ozaki"] = {
        "m": n3, "tile": t3, "tflops": 8.0 * n3 ** 3 / z3wall / 1e12, "wall_s": z3wall, "h2d_bytes": z3h2d,
        "d2h_bytes": z3d2h, "link_GBs_achieved": (z3h2d + z3d2h) / z3wall / 1e9,
        "compute_alone_s": z3compute, "link_alone_s": z3link,
        "overlap_efficiency": max(z3compute, z3link) / z3wall, "slices": z3info["slices"],
        "max_err_over_absab_64": float((np.abs(Cz[r3, c3] - exact) / absab).max()),
        "speedup_vs_native_zgemm": (8.0 * n3 ** 3 / z3wall) / (8.0 * nz ** 3 / zwall)}
    h3.close()
    del hA, hB, hC, dA, dC
    o = out_runs["zgemm_a_bh_ozaki"]
    out = {"metric": "out-of-HBM streamed GEMM TFLOP/s (host-resident operands, tiles << problem)",
           "value": o["tflops"], "unit": UNIT, "n_gpus": 1, "steps": len(ztimes), "warmup": 1,
           "ms_per_step": o["wall_s"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic U[-1,1], seeded",
           "config": {"workload": "out-of-HBM: ZGEMM C = A*B^H (Ozaki split, 4 real products per complex) "
                                  "streamed through the Tiled-MM entry from pinned host memory, m=n=k=16384, "
                                  "8192^3 tiles (the 65536^3 configuration does not fit the host memory)"},
           "runs": out_runs,
           "roofline": {"bound": "host-link", "achieved": o["link_GBs_achieved"], "peak": link_h2d, "unit": "GB/s",
                        "frac": o["link_GBs_achieved"] / link_h2d, "traffic": o["h2d_bytes"] + o["d2h_bytes"],
                        "kernel": "streamer copies (cudaMemcpy2DAsync on the H2D/D2H streams)",
                        "peak_note": "pinned H2D copy measured on this pool's GB300"},
           "e2e": {"value": o["tflops"], "unit": UNIT, "h2d_bytes_per_step": o["h2d_bytes"],
                   "d2h_bytes_per_step": o["d2h_bytes"]},
           "gpu_launches": None}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "plain":
        return run_plain(args)
    if args.config == "pdgemm":
        return run_pdgemm(args)
    if args.config == "grouped":
        return run_grouped(args)
    if args.config == "stream":
        return run_stream(args)
    if args.config == "sgemm":
        return run_sgemm(args)
    import torch

    import cosma_gb300 as cg
    import oracle

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    cg.load()
    n, phi = args.size, args.phi
    A = oracle.exp_spread((n, n), 1 + 10 * rank, phi)
    B = oracle.exp_spread((n, n), 2 + 10 * rank, phi)
    dA = torch.from_numpy(A.reshape(-1, order="F")).to(dev)
    dB = torch.from_numpy(B.reshape(-1, order="F")).to(dev)
    dC = torch.empty(n * n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        return cg.dgemm_ozaki_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, stream=stream)

    for _ in range(max(args.warmup, 3)):
        info = step()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    gemm_ms = []
    for _ in range(args.steps):
        info = step()
        gemm_ms.append(info["gemm_ms"])
    ev1.record(stream)
    barrier()
    clocks = sampler.stop()
    ms = replica_max_ms(ev0.elapsed_time(ev1) / args.steps, world, dev)
    flops = 2.0 * n * n * n
    value = job_tflops(flops, world, ms)

    # accuracy against the double-double oracle on sampled entries
    rng = np.random.default_rng(1234)
    ns = 4096
    rows, cols = rng.integers(0, n, ns), rng.integers(0, n, ns)
    Cg = dC.cpu().numpy().reshape(n, n).T  # column-major view
    hi, lo, ab = oracle.gemm_dd_sampled("N", "N", A, B, rows, cols)
    acc = oracle.error_stats(Cg[rows, cols], hi, lo, ab)

    # native FP64 on the same inputs (one run)
    native = None
    if not args.no_native:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        cg.gemm_device("N", "N", n, n, 256, 1.0, dA, n, dB, n, 0.0, dC, n, method="native", stream=stream)
        torch.cuda.synchronize()
        e0.record(stream)
        cg.gemm_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, method="native", stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        nms = e0.elapsed_time(e1)
        Cn = dC.cpu().numpy().reshape(n, n).T
        native = {"tflops": flops / (nms * 1e-3) / 1e12, "ms": nms,
                  "accuracy": oracle.error_stats(Cn[rows, cols], hi, lo, ab)}

    # end to end through the Tiled-MM C-ABI entry point, pinned host buffers
    hA = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    hB = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    hC = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    hA.numpy()[:] = A.reshape(-1, order="F")
    hB.numpy()[:] = B.reshape(-1, order="F")
    del dA, dB, dC
    torch.cuda.empty_cache()
    h = cg.make_context("d", 2, 0, 0, 0)
    h.set_method("ozaki", 0)
    cg.gemm(h, "N", "N", n, n, n, 1.0, hA, n, hB, n, 0.0, hC, n)  # warm-up (allocates tile buffers)
    barrier()
    e2e_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        cg.gemm(h, "N", "N", n, n, n, 1.0, hA, n, hB, n, 0.0, hC, n)
    barrier()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_val = flops * world / e2e_s / 1e12
    # the same call on the caller's pageable arrays (no pinned copies made)
    del hA, hB, hC
    pA, pB = np.asfortranarray(A), np.asfortranarray(B)
    pC = np.empty((n, n), order="F")
    t0 = time.perf_counter()
    cg.gemm(h, "N", "N", n, n, n, 1.0, pA, n, pB, n, 0.0, pC, n)  # first use of these allocations
    first_s = time.perf_counter() - t0
    cg.gemm(h, "N", "N", n, n, n, 1.0, pA, n, pB, n, 0.0, pC, n)
    barrier()
    t0 = time.perf_counter()
    for _ in range(3):
        cg.gemm(h, "N", "N", n, n, n, 1.0, pA, n, pB, n, 0.0, pC, n)
    barrier()
    pageable_s = (time.perf_counter() - t0) / 3
    pageable_route = cg.host_copy_route(pA)
    del pA, pB, pC
    h.close()

    # exponent-spread variants (one step each)
    variants = []
    if not args.no_variants:
        for vphi in (8, 32):
            Av = oracle.exp_spread((n, n), 101 + vphi, vphi)
            Bv = oracle.exp_spread((n, n), 202 + vphi, vphi)
            dA = torch.from_numpy(Av.reshape(-1, order="F")).to(dev)
            dB = torch.from_numpy(Bv.reshape(-1, order="F")).to(dev)
            dC = torch.empty(n * n, dtype=torch.float64, device=dev)
            cg.dgemm_ozaki_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, stream=stream)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            vinfo = cg.dgemm_ozaki_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            vms = e0.elapsed_time(e1)
            Cv = dC.cpu().numpy().reshape(n, n).T
            vhi, vlo, vab = oracle.gemm_dd_sampled("N", "N", Av, Bv, rows, cols)
            variants.append({"phi": vphi, "tflops": flops / (vms * 1e-3) / 1e12, "slices": vinfo["slices"],
                             "products": vinfo["products"], "spread_bits": vinfo["spread_bits"],
                             "accuracy": oracle.error_stats(Cv[rows, cols], vhi, vlo, vab)})
            del dA, dB, dC
            torch.cuda.empty_cache()

    # roofline of the dominant kernel (slice-product GEMM on the FP8 tensor pipe)
    pk, pk_kind = peaks()
    fp8_peak = 2.0 * pk["bf16_tflops"]
    kms = float(np.median(gemm_ms))
    achieved = info["products"] * flops / (kms * 1e-3) / 1e12
    traffic = None
    # DRAM bytes (read + write) of one full-size launch, from the ncu capture
    # summarised in profiles/ (a line "bytes_per_launch_full_size: N")
    tf = ROOT / "profiles" / "ozaki_gemm_pair_16384_dram.md"
    if tf.exists() and n == 16384 and args.phi == 0:
        for line in tf.read_text().splitlines():
            if line.strip().startswith("bytes_per_launch_full_size:"):
                try:
                    traffic = int(line.split(":", 1)[1].strip())
                except ValueError:
                    traffic = None
    roofline = {"bound": "tensor", "achieved": achieved, "peak": fp8_peak, "unit": "TFLOP/s",
                "frac": achieved / fp8_peak, "traffic": traffic,
                "kernel": "ozaki_gemm_pair_kernel (tcgen05.mma.cta_group::2 kind::f8f6f4, 256x256 tiles)",
                "peak_note": f"FP8 dense peak taken as 2x the {pk_kind} BF16 burst figure "
                             f"({pk['bf16_tflops']} TFLOP/s)",
                "kernel_ms": kms, "prep_ms": info["prep_ms"]}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded u*2^e)", "config": config(n, phi),
           "ozaki": {"slices": info["slices"], "products": info["products"], "groups": info["groups"],
                     "spread_bits": info["spread_bits"], "accuracy": acc,
                     "accuracy_note": "4096 sampled entries vs double-double; max_rel_err is elementwise "
                                      "|C-C_dd|/|C_dd|, max_err_over_absab normalises by (|A||B|)_ij"},
           "native_fp64": native,
           "speedup_vs_native": (value / world / native["tflops"]) if native else None,
           "variants": variants, "roofline": roofline, "clocks": clocks,
           "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 2 * n * n * 8, "d2h_bytes_per_step": n * n * 8,
                   "entry": "cosma_gpu_tmm_gemm_d (Tiled-MM gpu::gemm drop-in), pinned host A/B/C",
                   "ms_per_step": e2e_s * 1e3,
                   "pageable": {"value": flops * world / pageable_s / 1e12, "ms_per_step": pageable_s * 1e3,
                                "first_call_ms": first_s * 1e3, "host_copy_route": pageable_route,
                                "note": "same call on the caller's pageable numpy arrays: 2 warm-up calls "
                                        "(the first one on fresh allocations timed apart), mean of 3"}},
           "gpu_launches": KERNELS_PER_STEP * args.steps}
    if rank == 0:
        tflops_cpu, kb, cdt = cpu_dgemm_sample(A, B)
        out["cpu_baseline"] = {"value": tflops_cpu, "unit": UNIT,
                               "cores": int(os.environ.get("OPENBLAS_NUM_THREADS", os.cpu_count() or 1)),
                               "kind": "port",
                               "sample": f"OpenBLAS DGEMM NN {n}x{n}x{kb} K-slab of the workload ({cdt:.1f} s)"}
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
