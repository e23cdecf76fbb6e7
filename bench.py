#!/usr/bin/env python3
"""Benchmark of the one-rank GEMM path on GB300.

Headline workload (the precision configuration): C = A*B with m = n = k =
16384, FP64, column-major, entries u*2^e (u ~ U[-1, 1], integer e ~
U{-phi..phi}, phi = 0 for the headline, 8 and 32 as variants), seeded
synthetic data.  One step is one FP64-accurate GEMM through the
Chinese-remainder (Ozaki scheme II) path - 8-bit integer residues of the
scaled operands multiplied exactly on the BF16 tensor cores, one GEMM per
modulus, the exact product rebuilt and rounded once - with the inputs resident
in HBM; `e2e` runs the same GEMM through the Tiled-MM C-ABI entry point
(cosma_gpu_tmm_gemm_d) from pinned host buffers, copies included.  Beside it:
the native FP64 (DMMA) kernel and the digit-slice Ozaki form on the same
inputs, the accuracy of each over every entry of C against the exact product,
the roofline of the dominant kernel, and the reference's CPU path (OpenBLAS
DGEMM, the arithmetic cblas_dgemm performs at P = 1) timed on the host cores.

The default run (one GPU) adds one object per other configuration under
"configs": plain (2048^3 native drop-in), pdgemm (1x1 ScaLAPACK wrapper),
grouped (10,000 uneven problems), sgemm (3xBF16) and stream (host-resident
operands streamed through the Tiled-MM entry), each with its own roofline,
e2e, CPU baseline and clock record.  --config NAME prints one of them alone.

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
# kernels of one headline step: A exponents (partial + combine), B exponents,
# A residues, B residues, modular GEMM, reconstruction
KERNELS_PER_STEP = 7
# DRAM bytes of one launch of the modular GEMM kernel on the headline
# workload itself (m = n = k = 16384, u*2^e inputs with phi = 0, 16 moduli):
# dram__bytes_read.sum + dram__bytes_write.sum from a one-pass ncu capture
# of that launch (the command is in profiles/ozaki2_gemm_pair_16384_dram.md)
TRAFFIC_BYTES_16384 = {16: 137_887_403_520 + 4_843_662_848}
CONFIG_NAMES = ("plain", "pdgemm", "grouped", "sgemm", "stream")
FP64_NOMINAL_TFLOPS = 1.25  # GB300 FP64 (no FP64 figure is measured on this machine)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--size", type=int, default=16384)
    p.add_argument("--phi", type=int, default=0)
    p.add_argument("--moduli", type=int, default=0, help="moduli of the headline GEMM (0: chosen from the inputs)")
    p.add_argument("--no-native", action="store_true", help="skip the native FP64 comparison run")
    p.add_argument("--no-variants", action="store_true", help="skip the phi = 8 / 32 variants")
    p.add_argument("--no-configs", action="store_true", help="headline line only")
    p.add_argument("--count", type=int, default=10000,
                   help="problems in the grouped configuration (10,000; fewer for profiler captures)")
    p.add_argument("--config", default="precision", choices=("precision",) + CONFIG_NAMES + ("grouped_crt",),
                   help="precision: the headline line (with the other configurations under 'configs'); "
                        "otherwise one configuration alone (grouped_crt: the grouped batch in the "
                        "Chinese-remainder form only, for profiler captures)")
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
        time.sleep(0.3)

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


def cpu_dgemm_sample(A, B, budget_s=10.0):
    """OpenBLAS DGEMM (numpy) on a K-slab of the workload, sized to ~budget_s."""
    n = A.shape[0]
    kb = 512
    t = time.perf_counter()
    np.matmul(A[:, :kb], B[:kb, :])
    dt = time.perf_counter() - t
    rate = 2.0 * n * B.shape[1] * kb / max(dt, 1e-6)
    kb = int(min(A.shape[1], max(512, (budget_s * rate) / (2.0 * n * B.shape[1]))))
    kb -= kb % 256
    t = time.perf_counter()
    np.matmul(A[:, :kb], B[:kb, :])
    dt = time.perf_counter() - t
    return 2.0 * n * B.shape[1] * kb / dt / 1e12, kb, dt


def cuda_ms(fn, stream, reps=1, warm=True):
    """Mean milliseconds of fn() by CUDA events on `stream` (after one warm-up call if `warm`)."""
    import torch
    if warm:
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    out = None
    for _ in range(reps):
        out = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps, out


def full_accuracy(cg, dA, dB, dC, absab, E, R, n, stream):
    """Error of every entry of C against the exact product: the residual mode
    of the Chinese-remainder form at 28 moduli (every input bit kept for these
    inputs) gives E = AB - C exactly before one rounding, and R = AB rounded."""
    import torch
    info = cg.dgemm_ozaki2_residual("N", "N", n, n, n, dA, n, dB, n, dC, n, E, R, n, moduli=28, stream=stream)
    torch.cuda.synchronize()
    nz = R != 0
    aE = E.abs()
    rel = aE[nz] / R.abs()[nz]
    nw = aE / absab
    out = {"entries": int(n) * int(n), "entries_nonzero": int(nz.sum()), "nan": int(torch.isnan(E).sum()),
           "max_rel_err": float(rel.max()), "mean_rel_err": float(rel.mean()),
           "count_rel_err_gt_1e-15": int((rel > 1e-15).sum()),
           "max_err_over_absab": float(nw.max()), "mean_err_over_absab": float(nw.mean()),
           "reference": f"exact product (Chinese-remainder residual mode, 28 moduli, P = {info['fraction_bits']})"}
    del rel, nw, aE, nz
    return out


def absab_of(cg, dA, dB, n, out, stream):
    """(|A||B|)_ij, the normaliser of the componentwise error (8 moduli: ~2^-23 relative)."""
    cg.dgemm_ozaki2_device("N", "N", n, n, n, 1.0, dA.abs(), n, dB.abs(), n, 0.0, out, n, moduli=8, stream=stream)


# --------------------------------------------------------------- reference arm
def run_reference(args):
    """The reference's CPU path on the host cores: at P = 1 cosma::multiply is
    one cblas_dgemm(ColMajor, N, N) (src/cosma/blas.cpp:35-48); the reference
    as a whole cannot be built here (MPI, ScaLAPACK, COSTA and Tiled-MM are
    absent), so its arithmetic runs through numpy's OpenBLAS on every host
    thread, a bounded K-slab of the workload per step."""
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
    ms = dt / args.steps * 1e3
    out = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms,
           "ms_per_step_covers": f"a K-slab of {kb} of the {n}-deep product ({kb / n:.4f} of one workload step)",
           "ms_per_full_step_equivalent": ms * n / kb,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded)", "config": config(n, args.phi),
           "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": f"OpenBLAS DGEMM NN {n}x{n}x{kb} K-slab of the workload per step"},
           "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ----------------------------------------------------------- configurations
def cfg_pdgemm(steps, warmup):
    """pdgemm on a 1x1 grid: C = 1.5 * A^T * B + 0.5 * C, m = n = 4096, k = 65536,
    128 x 128 blocks, N(0,1) entries.  Device phases (COSTA pack of A with
    transpose, pack of B, FP64-accurate GEMM, alpha/beta unpack) are timed with
    CUDA events on the launching stream; e2e is the pdgemm_ symbol called with
    the caller's host arrays."""
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
    method = "ozaki2"

    def phases():
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev[0].record(s)
        cg.pack("T", m, k, dAsc, k, dA, m, stream=s)
        ev[1].record(s)
        cg.pack("N", k, n, dBsc, k, dB, k, stream=s)
        ev[2].record(s)
        cg.gemm_device("N", "N", m, n, k, 1.0, dA, m, dB, k, 0.0, dCc, m, method=method, stream=s)
        ev[3].record(s)
        cg.unpack(m, n, alpha, dCc, m, beta, dCsc, m, stream=s)
        ev[4].record(s)
        torch.cuda.synchronize()
        return [ev[i].elapsed_time(ev[i + 1]) for i in range(4)]

    for _ in range(max(warmup, 3)):
        dCsc.copy_(torch.from_numpy(C0.reshape(-1, order="F")))
        phases()
    sampler = ClockSampler(0)
    sampler.start()
    times = [phases() for _ in range(steps)]
    clocks = sampler.stop()
    t = np.median(np.array(times), axis=0)
    total = float(t.sum())
    flops = 2.0 * m * n * k
    pk, pk_kind = peaks()
    pack_a_bytes = 2.0 * m * k * 8
    pack_b_bytes = 2.0 * k * n * 8
    unpack_bytes = 3.0 * m * n * 8
    gbs = lambda b, ms: b / (ms * 1e-3) / 1e9
    del dAsc, dBsc, dCsc, dA, dB, dCc
    torch.cuda.empty_cache()
    # e2e: the ScaLAPACK symbol with host arrays
    desca = cg.descinit(k, m, 128, 128, 0, 0, 0, k)
    descb = cg.descinit(k, n, 128, 128, 0, 0, 0, k)
    descc = cg.descinit(m, n, 128, 128, 0, 0, 0, m)
    cg.pxgemm_set_method(method)
    Ch = C0.copy(order="F")
    cg.pxgemm("T", "N", m, n, k, alpha, A, 1, 1, desca, B, 1, 1, descb, beta, Ch, 1, 1, descc)
    e2e = []
    for _ in range(3):
        Ch = C0.copy(order="F")
        t0 = time.perf_counter()
        cg.pxgemm("T", "N", m, n, k, alpha, A, 1, 1, desca, B, 1, 1, descb, beta, Ch, 1, 1, descc)
        e2e.append(time.perf_counter() - t0)
    h2d_px, d2h_px, overlapped = cg.pxgemm_last_transfers()
    cg.pxgemm_set_method("native")
    e2e_s = float(np.median(e2e))
    # accuracy of the host result on sampled entries (double-double oracle)
    rng = np.random.default_rng(7)
    rows, cols = rng.integers(0, m, 1024), rng.integers(0, n, 1024)
    hi, lo, ab = oracle.gemm_dd_sampled("T", "N", A, B, rows, cols)
    exact = alpha * (hi + lo) + beta * C0[rows, cols]
    rel = np.abs(Ch[rows, cols] - exact) / np.maximum(np.abs(exact), 1e-300)
    # the reference's CPU arithmetic for the same call: pack A^T, OpenBLAS
    # DGEMM on a K-slab, alpha/beta unpack (cosma_pxgemm.cpp:338-364 at P = 1)
    kb = 4096
    t0 = time.perf_counter()
    At = np.ascontiguousarray(A[:kb].T)
    P = At @ B[:kb]
    _ = alpha * P + beta * C0
    cpu_s = time.perf_counter() - t0
    return {"metric": "pdgemm 1x1 TFLOP/s (COSTA pack + FP64-accurate GEMM + unpack)",
            "value": flops / (total * 1e-3) / 1e12, "unit": UNIT, "steps": steps, "ms_per_step": total,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic N(0,1), seeded",
            "config": {"workload": "pdgemm 1x1 grid C = 1.5*A^T*B + 0.5*C, m=n=4096, k=65536, 128x128 blocks",
                       "gemm_method": method},
            "phases_ms": {"pack_A_transpose": t[0], "pack_B": t[1], "gemm": t[2], "unpack_alpha_beta": t[3]},
            "pack_GBs": {"A_transpose": gbs(pack_a_bytes, t[0]), "B_copy": gbs(pack_b_bytes, t[1]),
                         "unpack": gbs(unpack_bytes, t[3])},
            "roofline": {"bound": "hbm", "achieved": gbs(pack_a_bytes, t[0]), "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": gbs(pack_a_bytes, t[0]) / pk["hbm_gbs"], "traffic": None,
                         "kernel": "transpose_kernel (COSTA pack, op T), 2 x 8 bytes per element",
                         "peak_note": f"{pk_kind} HBM copy bandwidth",
                         "unpack_frac": gbs(unpack_bytes, t[3]) / pk["hbm_gbs"],
                         "pack_B_frac": gbs(pack_b_bytes, t[1]) / pk["hbm_gbs"]},
            "accuracy": {"max_rel_err": float(rel.max()), "mean_rel_err": float(rel.mean()), "samples": 1024,
                         "reference": "double-double (oracle) on sampled entries"},
            "e2e": {"value": flops / e2e_s / 1e12, "unit": UNIT, "h2d_bytes_per_step": h2d_px,
                    "d2h_bytes_per_step": d2h_px, "entry": "pdgemm_ (ScaLAPACK symbol), pageable host arrays",
                    "form": ("overlapped one-step: op(A) / op(B) panels and C blocks on the copy engines, issued "
                             "by a copy thread, beside the modular GEMMs") if overlapped else
                            "staged: whole arrays copied in, pack, GEMM, unpack, C copied out",
                    "host_copy_route": cg.host_copy_route(A), "ms_per_step": e2e_s * 1e3,
                    "calls_ms": [round(x * 1e3, 2) for x in e2e]},
            "cpu_baseline": {"value": 2.0 * m * n * kb / cpu_s / 1e12, "unit": UNIT, "cores": oracle.openblas_threads(),
                             "kind": "port",
                             "sample": f"numpy pack of A^T, OpenBLAS DGEMM {m}x{n}x{kb} K-slab, alpha/beta ({cpu_s:.1f} s)"},
            "clocks": clocks, "gpu_launches": 4 * steps}


def cfg_sgemm(steps, warmup, n=16384):
    """FP32 GEMM m = n = k = 16384, N(0,1) entries, through the 3xBF16 path;
    cuBLAS SGEMM (FP32 SIMT, TF32 off) timed beside it for context."""
    import torch

    import cosma_gb300 as cg
    import oracle

    dev = torch.device("cuda", 0)
    A = oracle.normal((n, n), 1, dtype=np.float32)
    B = oracle.normal((n, n), 2, dtype=np.float32)
    dA = torch.from_numpy(A.reshape(-1, order="F")).to(dev)
    dB = torch.from_numpy(B.reshape(-1, order="F")).to(dev)
    dC = torch.empty(n * n, dtype=torch.float32, device=dev)
    s = torch.cuda.current_stream(dev)

    def step():
        cg.gemm_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, method="bf16x3", stream=s, scalar="s")

    for _ in range(max(warmup, 3)):
        step()
    sampler = ClockSampler(0)
    sampler.start()
    ms, _ = cuda_ms(step, s, steps)
    clocks = sampler.stop()
    flops = 2.0 * n * n * n
    rng = np.random.default_rng(5)
    rows, cols = rng.integers(0, n, 2048), rng.integers(0, n, 2048)
    Cg = dC.cpu().numpy().reshape(n, n).T
    exact = np.einsum("ij,ji->i", A[rows, :].astype(np.float64), B[:, cols].astype(np.float64))
    absab = np.einsum("ij,ji->i", np.abs(A[rows, :]).astype(np.float64), np.abs(B[:, cols]).astype(np.float64))
    err = np.abs(Cg[rows, cols] - exact)
    torch.backends.cuda.matmul.allow_tf32 = False
    At, Bt = dA.view(n, n), dB.view(n, n)  # row-major views: C^T = B^T A^T
    cublas_ms, Ct = cuda_ms(lambda: torch.matmul(Bt, At), s, 1)
    Cc = Ct.cpu().numpy().T
    err_cublas = np.abs(Cc[rows, cols] - exact)
    # e2e: the Tiled-MM entry (AUTO = 3xBF16 for float) from pinned host buffers
    hA = torch.from_numpy(A.reshape(-1, order="F")).pin_memory()
    hB = torch.from_numpy(B.reshape(-1, order="F")).pin_memory()
    hC = torch.empty(n * n, dtype=torch.float32).pin_memory()
    h = cg.make_context("s", 2, 0, 0, 0)
    for _ in range(max(1, warmup)):
        cg.gemm(h, "N", "N", n, n, n, 1.0, hA, n, hB, n, 0.0, hC, n)
    t0 = time.perf_counter()
    for _ in range(3):
        cg.gemm(h, "N", "N", n, n, n, 1.0, hA, n, hB, n, 0.0, hC, n)
    e2e_s = (time.perf_counter() - t0) / 3
    e2e_overlapped = h.last_overlapped()
    h.close()
    del dA, dB, dC, Ct, hA, hB, hC
    torch.cuda.empty_cache()
    cpu_val, kb, cdt = cpu_dgemm_sample(A, B, budget_s=4.0)
    pk, pk_kind = peaks()
    ach = 6 * flops / (ms * 1e-3) / 1e12
    return {"metric": "FP32 GEMM TFLOP/s (3xBF16 split on BF16 tensor cores)", "value": flops / (ms * 1e-3) / 1e12,
            "unit": UNIT, "steps": steps, "ms_per_step": ms, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic N(0,1), seeded",
            "config": {"workload": f"precision: SGEMM NN m=n=k={n}, N(0,1), 3xBF16 (6 BF16 products)"},
            "accuracy": {"max_err_over_absab": float((err / absab).max()), "max_abs_err": float(err.max()),
                         "cublas_sgemm_max_err_over_absab": float((err_cublas / absab).max()), "samples": 2048},
            "cublas_sgemm_tflops": flops / (cublas_ms * 1e-3) / 1e12,
            "roofline": {"bound": "tensor", "achieved": ach, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                         "frac": ach / pk["bf16_tflops"], "traffic": None,
                         "kernel": "bf16x3_gemm_kernel (tcgen05 kind::f16), step incl. slicing",
                         "peak_note": f"{pk_kind} BF16 burst"},
            "e2e": {"value": flops / e2e_s / 1e12, "unit": UNIT, "h2d_bytes_per_step": 2 * 4 * n * n,
                    "d2h_bytes_per_step": 4 * n * n, "entry": "cosma_gpu_tmm_gemm_s, pinned host buffers",
                    "form": ("overlapped one-step: op(A) / op(B) panels split as they land, block GEMMs, C blocks "
                             "copied out while later ones compute") if e2e_overlapped else "one step",
                    "ms_per_step": e2e_s * 1e3},
            "cpu_baseline": {"value": cpu_val, "unit": UNIT, "cores": oracle.openblas_threads(), "kind": "port",
                             "sample": f"OpenBLAS SGEMM NN {n}x{n}x{kb} K-slab ({cdt:.1f} s)"},
            "clocks": clocks, "gpu_launches": 3 * steps}


def grouped_batch(count, dev):
    """The batching configuration's batch on `dev`: m, n, k log-uniform integers
    in [16, 1024] (seed 2024), transa / transb uniform in {N, T}, U[-1, 1]
    entries (torch generator seed 7), alpha = 1, beta = 0, packed one after
    another (32-element aligned) in three device arrays."""
    import torch

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
    return rng, (m, n, k, ta, tb), (sa, sb, sc), (dA, dB, dC), probs


def cfg_grouped_crt(steps, warmup, count=10000):
    """The batching configuration's batch in the Chinese-remainder form alone
    (plan, warm-up runs, timed runs): the command behind the grouped launch
    lists and kernel captures."""
    import torch

    import cosma_gb300 as cg

    dev = torch.device("cuda", 0)
    _, (m, n, k, _, _), _, bufs, probs = grouped_batch(count, dev)
    useful = float((2 * m * n * k).sum())
    s = torch.cuda.current_stream(dev)
    plan = cg.GroupedPlan(probs, method="ozaki2", autotune=False)
    for _ in range(warmup):
        plan.run(stream=s)
    ms, _ = cuda_ms(lambda: plan.run(stream=s), s, max(steps, 1))
    info = plan.info()
    plan.close()
    return {"metric": f"grouped FP64-accurate GEMM TFLOP/s ({count:,} uneven problems, Chinese-remainder form)",
            "value": useful / (ms * 1e-3) / 1e12, "unit": UNIT, "steps": steps, "ms_per_step": ms,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic U[-1,1], seeded",
            "config": {"workload": f"batching: {count:,} FP64 GEMMs, m,n,k log-uniform in [16,1024], random N/T"},
            "plan": info}


def cfg_grouped(steps, warmup, count=10000):
    """10,000 independent FP64 GEMMs, m, n, k log-uniform integers in [16, 1024],
    transa/transb uniform in {N, T}, U[-1, 1] entries: one persistent grouped
    launch (autotuned, CUDA graph) in native FP64 and in the digit-slice Ozaki
    form and in the Chinese-remainder form, against a loop of per-problem
    drop-in calls."""
    import torch

    import cosma_gb300 as cg
    import oracle

    dev = torch.device("cuda", 0)
    rng, (m, n, k, ta, tb), (sa, sb, sc), (dA, dB, dC), probs = grouped_batch(count, dev)
    useful = float((2 * m * n * k).sum())
    s = torch.cuda.current_stream(dev)

    def host_problem(i):
        A = dA[int(sa[i]):int(sa[i]) + int(m[i] * k[i])].cpu().numpy()
        B = dB[int(sb[i]):int(sb[i]) + int(k[i] * n[i])].cpu().numpy()
        Cg = dC[int(sc[i]):int(sc[i]) + int(m[i] * n[i])].cpu().numpy().reshape(int(n[i]), int(m[i])).T
        # column-major storage: a rows x cols matrix is flat.reshape(cols, rows).T
        Am = A.reshape(int(k[i]), int(m[i])).T if ta[i] == "N" else A.reshape(int(m[i]), int(k[i]))
        Bm = B.reshape(int(n[i]), int(k[i])).T if tb[i] == "N" else B.reshape(int(k[i]), int(n[i]))
        return np.asfortranarray(Am), np.asfortranarray(Bm), Cg

    def accuracy(picks):
        """Double-double oracle on up to 256 entries of each picked problem."""
        worst_rel, worst_nw, entries = 0.0, 0.0, 0
        arng = np.random.default_rng(11)
        for i in picks:
            Am, Bm, Cg = host_problem(i)
            ns = min(256, Cg.size)
            rr, cc = arng.integers(0, Cg.shape[0], ns), arng.integers(0, Cg.shape[1], ns)
            hi, lo, ab = oracle.gemm_dd_sampled("N", "N", Am, Bm, rr, cc)
            st = oracle.error_stats(Cg[rr, cc], hi, lo, ab)
            worst_rel = max(worst_rel, st["max_rel_err"])
            worst_nw = max(worst_nw, st["max_err_over_absab"])
            entries += ns
        return {"max_rel_err": worst_rel, "max_err_over_absab": worst_nw, "problems": len(picks), "entries": entries,
                "reference": "double-double (oracle), up to 256 entries of each sampled problem"}

    picks = [int(i) for i in rng.choice(count, 24, replace=False)]
    t0 = time.perf_counter()
    plan = cg.GroupedPlan(probs, method="native", autotune=True)
    plan_s = time.perf_counter() - t0
    for _ in range(max(warmup, 3)):
        plan.run(stream=s)
    sampler = ClockSampler(0)
    sampler.start()
    ms, _ = cuda_ms(lambda: plan.run(stream=s), s, steps)
    clocks = sampler.stop()
    info = plan.info()
    acc_native = accuracy(picks)
    plan.close()
    t0 = time.perf_counter()
    oplan = cg.GroupedPlan(probs, method="ozaki", autotune=True)
    oplan_s = time.perf_counter() - t0
    for _ in range(max(warmup, 3)):
        oplan.run(stream=s)
    oms, _ = cuda_ms(lambda: oplan.run(stream=s), s, steps)
    oinfo = oplan.info()
    oslices = oplan.slices()
    acc_oz = accuracy(picks)
    oplan.close()
    # the Chinese-remainder form: one modulus count for the batch
    t0 = time.perf_counter()
    cplan = cg.GroupedPlan(probs, method="ozaki2", autotune=True)
    cplan_s = time.perf_counter() - t0
    for _ in range(max(warmup, 3)):
        cplan.run(stream=s)
    cms, _ = cuda_ms(lambda: cplan.run(stream=s), s, steps)
    cinfo = cplan.info()
    cmods = [x for x in cplan.slices() if x]
    acc_crt = accuracy(picks)
    cplan.close()
    # loop of per-problem drop-in calls (the reference's way of running a batch)
    torch.cuda.synchronize()
    l0 = time.perf_counter()
    for (pta, ptb, pm, pn, pk_, al, A, lda, B, ldb, be, Cm, ldc) in probs:
        cg.gemm_device(pta, ptb, pm, pn, pk_, al, A, lda, B, ldb, be, Cm, ldc, method="native", stream=s, scalar="d")
    torch.cuda.synchronize()
    loop_s = time.perf_counter() - l0
    # native FP64 reference rate: one large native DGEMM
    big = 4096
    X = torch.rand(big * big, dtype=torch.float64, device=dev)
    Y = torch.empty_like(X)
    bms, _ = cuda_ms(lambda: cg.gemm_device("N", "N", big, big, big, 1.0, X, big, X, big, 0.0, Y, big,
                                            method="native", stream=s), s, 1)
    native_peak = 2.0 * big ** 3 / (bms * 1e-3) / 1e12
    # e2e: the batch from host memory - inputs copied in, the grouped launch, C
    # copied out, the copies by the library's copy kernel (COSTA pack, op N)
    # reading and writing the pinned host arrays in place
    hA, hB = dA.cpu().pin_memory(), dB.cpu().pin_memory()
    hC = torch.empty(dC.numel(), dtype=torch.float64).pin_memory()
    route = cg.host_copy_route(hA)

    def flat_copy(dst, src, count_):
        rows = 1 << 20
        main = count_ // rows * rows
        if main:
            cg.pack("N", rows, main // rows, src, rows, dst, rows, stream=s)
        if count_ - main:
            cg.pack("N", count_ - main, 1, src.data_ptr() + 8 * main, count_ - main, dst.data_ptr() + 8 * main,
                    count_ - main, stream=s)

    plan = cg.GroupedPlan(probs, method="ozaki2", autotune=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        if route == 2:
            flat_copy(dA, hA, dA.numel())
            flat_copy(dB, hB, dB.numel())
        else:
            dA.copy_(hA, non_blocking=True)
            dB.copy_(hB, non_blocking=True)
        plan.run(stream=s)
        if route == 2:
            flat_copy(hC, dC, dC.numel())
        else:
            hC.copy_(dC, non_blocking=True)
        torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / 3
    plan.close()
    # the reference's CPU arithmetic: OpenBLAS per problem on a sample of the batch
    cpu_picks = [int(i) for i in rng.choice(count, 500, replace=False)]
    hostp = [host_problem(i)[:2] for i in cpu_picks]
    t0 = time.perf_counter()
    for Am, Bm in hostp:
        Am @ Bm
    cpu_s = time.perf_counter() - t0
    cpu_flops = float(sum(2.0 * Am.shape[0] * Am.shape[1] * Bm.shape[1] for Am, Bm in hostp))
    del dA, dB, dC, X, Y, hA, hB, hC
    torch.cuda.empty_cache()
    value = useful / (ms * 1e-3) / 1e12
    oval = useful / (oms * 1e-3) / 1e12
    cval = useful / (cms * 1e-3) / 1e12
    pk, pk_kind = peaks()
    return {"metric": f"grouped FP64 GEMM TFLOP/s ({count:,} uneven problems, one launch)", "value": value,
            "unit": UNIT, "steps": steps, "ms_per_step": ms, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic U[-1,1], seeded",
            "config": {"workload": f"batching: {count:,} FP64 GEMMs, m,n,k log-uniform in [16,1024], random N/T",
                       "useful_gflop": useful / 1e9},
            "plan": info, "plan_build_s": plan_s,
            "frac_of_native_fp64": value / native_peak, "native_fp64_tflops_4096": native_peak,
            "loop_of_dropin_calls": {"tflops": useful / loop_s / 1e12, "s": loop_s},
            "ozaki_split_form": {"tflops": oval, "ms": oms, "plan_build_s": oplan_s,
                                 "speedup_vs_native_grouped": ms / oms, "tiles": oinfo["tiles"],
                                 "fp8_flops_issued": oinfo["padded_flops"],
                                 "slices_min_max": [min(oslices), max(oslices)], "accuracy": acc_oz},
            "crt_form": {"tflops": cval, "ms": cms, "plan_build_s": cplan_s, "speedup_vs_native_grouped": ms / cms,
                         "speedup_vs_split_form": oms / cms, "tiles": cinfo["tiles"], "moduli": max(cmods),
                         "bf16_flops_issued": cinfo["padded_flops"],
                         "bf16_tflops_issued": cinfo["padded_flops"] / (cms * 1e-3) / 1e12,
                         "bf16_frac_of_sustained": cinfo["padded_flops"] / (cms * 1e-3) / 1e12
                         / pk["bf16_tflops_sustained"],
                         "peak_kind": pk_kind, "accuracy": acc_crt},
            "accuracy": acc_native,
            "roofline": {"bound": "fp64", "achieved": value, "peak": native_peak, "unit": "TFLOP/s",
                         "frac": value / native_peak, "traffic": None, "kernel": "grouped_dmma_kernel",
                         "peak_note": "measured: this library's native DGEMM at 4096^3 on the same GPU",
                         "frac_of_nominal_fp64": value / FP64_NOMINAL_TFLOPS},
            "e2e": {"value": useful / e2e_s / 1e12, "unit": UNIT,
                    "h2d_bytes_per_step": int(8 * (sa[-1] + sb[-1])), "d2h_bytes_per_step": int(8 * sc[-1]),
                    "entry": "grouped plan (Chinese-remainder form) with the batch copied in from and out to pinned "
                             "host memory" + (" by the library's in-place copy kernel (costa_gpu_pack reading / "
                                              "writing host memory)" if route == 2 else " (cudaMemcpyAsync)"),
                    "ms_per_step": e2e_s * 1e3},
            "cpu_baseline": {"value": cpu_flops / cpu_s / 1e12, "unit": UNIT, "cores": oracle.openblas_threads(),
                             "kind": "port", "sample": f"OpenBLAS DGEMM per problem on 500 of the {count:,} problems"},
            "clocks": clocks, "gpu_launches": steps}


def cfg_plain(steps, warmup, n=2048):
    """The plain small configuration: DGEMM C = A*B, m = n = k = 2048, NN, alpha = 1,
    beta = 0, A and B U[-1,1] from seeds 1 and 2.  The native FP64 drop-in on
    device-resident data (value), the same call end to end through
    cosma_gpu_local_multiply_d from host buffers (e2e, the one-rank
    cosma::multiply), the error bound c*k*u*(|A||B|) against OpenBLAS on the
    host, the FP64-accurate form beside it, and OpenBLAS timed on the host cores."""
    import torch

    import cosma_gb300 as cg
    import oracle

    dev = torch.device("cuda", 0)
    A = oracle.uniform((n, n), 1)
    B = oracle.uniform((n, n), 2)
    dA = torch.from_numpy(A.reshape(-1, order="F")).to(dev)
    dB = torch.from_numpy(B.reshape(-1, order="F")).to(dev)
    dC = torch.empty(n * n, dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream(dev)
    flops = 2.0 * n ** 3

    def timed(method):
        for _ in range(max(warmup, 3)):
            cg.gemm_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, method=method, stream=s)
        ms, _ = cuda_ms(lambda: cg.gemm_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, method=method,
                                               stream=s), s, steps)
        return ms, dC.cpu().numpy().reshape(n, n).T

    sampler = ClockSampler(0)
    sampler.start()
    ms, Cn = timed("native")
    clocks = sampler.stop()
    oms, Co = timed("ozaki2")
    t0 = time.perf_counter()
    reps = 0
    while True:
        ref = A @ B
        reps += 1
        if time.perf_counter() - t0 > 3.0:
            break
    cpu_s = (time.perf_counter() - t0) / reps
    absab = np.abs(A) @ np.abs(B)
    bound = 2.0 * (n + 2) * 2.0 ** -53 * absab
    within = bool(np.all(np.abs(Cn - ref) <= bound))
    hA = torch.from_numpy(A.reshape(-1, order="F")).pin_memory()
    hB = torch.from_numpy(B.reshape(-1, order="F")).pin_memory()
    hC = torch.empty(n * n, dtype=torch.float64).pin_memory()
    cg.local_multiply(hA, hB, hC, n, n, n, 1.0, 0.0)
    t0 = time.perf_counter()
    for _ in range(steps):
        cg.local_multiply(hA, hB, hC, n, n, n, 1.0, 0.0)
    e2e_s = (time.perf_counter() - t0) / steps
    value = flops / (ms * 1e-3) / 1e12
    del dA, dB, dC
    torch.cuda.empty_cache()
    return {"metric": "plain FP64 DGEMM TFLOP/s (native drop-in)", "value": value, "unit": UNIT,
            "steps": steps, "ms_per_step": ms, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic U[-1,1], seeds 1 and 2",
            "config": {"workload": f"plain: DGEMM NN m=n=k={n}, alpha=1, beta=0, column-major",
                       "l2": "operands 32 MiB each, inside L2; the kernel re-reads tiles from L2"},
            "within_ckuAB_bound": within, "bound": "2 (k+2) u (|A||B|) elementwise vs OpenBLAS",
            "max_err_over_absab": float(np.max(np.abs(Cn - ref) / absab)),
            "fp64_accurate_form": {"tflops": flops / (oms * 1e-3) / 1e12, "ms": oms,
                                   "max_err_over_absab": float(np.max(np.abs(Co - ref) / absab))},
            "roofline": {"bound": "fp64", "achieved": value, "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                         "frac": value / FP64_NOMINAL_TFLOPS, "traffic": None,
                         "kernel": "dmma_gemm_kernel (mma.sync m16n8k4 f64)",
                         "peak_note": "nominal GB300 FP64 rate (no measured FP64 figure exists for this pool)"},
            "e2e": {"value": flops / e2e_s / 1e12, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * n * n,
                    "d2h_bytes_per_step": 8 * n * n, "entry": "cosma_gpu_local_multiply_d, pinned host buffers",
                    "ms_per_step": e2e_s * 1e3},
            "cpu_baseline": {"value": flops / cpu_s / 1e12, "unit": UNIT, "cores": oracle.openblas_threads(),
                             "kind": "port", "sample": f"OpenBLAS DGEMM NN {n}^3, {reps} repetitions"},
            "clocks": clocks, "gpu_launches": steps}


def link_rates(nbytes=4 << 30):
    """Host-link copy rates (GB/s) measured now: pinned H2D and D2H, 4 GiB, CUDA events."""
    import torch
    h = torch.empty(nbytes // 8, dtype=torch.float64).pin_memory()
    d = torch.empty_like(h, device="cuda")
    s = torch.cuda.current_stream()
    d.copy_(h, non_blocking=True)
    torch.cuda.synchronize()
    h2d, _ = cuda_ms(lambda: d.copy_(h, non_blocking=True), s, 3)
    d2h, _ = cuda_ms(lambda: h.copy_(d, non_blocking=True), s, 3)
    del h, d
    torch.cuda.empty_cache()
    return nbytes / (h2d * 1e-3) / 1e9, nbytes / (d2h * 1e-3) / 1e9


def cfg_stream(steps, warmup, n=16384, tile=8192):
    """Out-of-HBM streaming through the Tiled-MM entry point: ZGEMM C = A * B^H
    (the configuration's operation) with A, B, C in pinned host memory and
    tile limits below the problem, so every operand streams; FP64-accurate
    (Chinese-remainder form, four real products per complex one).  The full
    configuration (65536^3 complex, 206 GB of host matrices) exceeds the GPU
    host's 214 GB; the streamer's behaviour is measured at 16384^3 with
    8192^3 tiles, the same tile-to-problem ratio in each dimension as 65536^3
    with 32768^3 tiles."""
    import torch

    import cosma_gb300 as cg
    import oracle

    h2d_gbs, d2h_gbs = link_rates()
    g = torch.Generator().manual_seed(3)
    cplx = lambda: torch.complex(torch.rand(n * n, dtype=torch.float64, generator=g) * 2 - 1,
                                 torch.rand(n * n, dtype=torch.float64, generator=g) * 2 - 1).pin_memory()
    hA, hB = cplx(), cplx()
    hC = torch.empty(n * n, dtype=torch.complex128).pin_memory()
    h = cg.make_context("z", 3, tile, tile, tile)
    h.set_method("ozaki2", 0)
    cg.gemm(h, "N", "C", n, n, n, 1.0, hA, n, hB, n, 0.0, hC, n)  # warm-up: allocates the rings
    sampler = ClockSampler(0)
    sampler.start()
    times = []
    for _ in range(max(1, min(steps, 2))):
        t0 = time.perf_counter()
        cg.gemm(h, "N", "C", n, n, n, 1.0, hA, n, hB, n, 0.0, hC, n)
        times.append(time.perf_counter() - t0)
    clocks = sampler.stop()
    h2d, d2h = h.transfer_bytes()
    zinfo = h.ozaki_info()
    wall = float(np.median(times))
    route = cg.host_copy_route(hA)
    h.close()
    # the same tile GEMM on device-resident data, times the tile steps: compute alone
    dA = torch.complex(torch.rand(tile * tile, dtype=torch.float64, device="cuda") * 2 - 1,
                       torch.rand(tile * tile, dtype=torch.float64, device="cuda") * 2 - 1)
    dC = torch.empty_like(dA)
    s = torch.cuda.current_stream()
    tms, _ = cuda_ms(lambda: cg.zgemm_ozaki2_device("N", "C", tile, tile, tile, 1.0, dA, tile, dA, tile, 0.0, dC,
                                                     tile, stream=s), s, 1)
    compute_s = tms * 1e-3 * (n // tile) ** 3
    del dA, dC
    torch.cuda.empty_cache()
    link_s = h2d / (h2d_gbs * 1e9) + d2h / (d2h_gbs * 1e9)
    # accuracy on sampled entries (double-double)
    rng = np.random.default_rng(1)
    r3, c3 = rng.integers(0, n, 64), rng.integers(0, n, 64)
    Az = hA.numpy().reshape(n, n).T
    Bz = hB.numpy().reshape(n, n).T
    Cz = hC.numpy().reshape(n, n).T
    rel = []
    for i, j in zip(r3, c3):
        a = np.asfortranarray(Az[i:i + 1, :])
        b = np.asfortranarray(Bz[j:j + 1, :].conj().T)  # column j of B^H
        hre, lre, _ = oracle.gemm_dd("N", "N", np.asfortranarray(a.real), np.asfortranarray(b.real))
        hii, lii, _ = oracle.gemm_dd("N", "N", np.asfortranarray(a.imag), np.asfortranarray(b.imag))
        hri, lri, _ = oracle.gemm_dd("N", "N", np.asfortranarray(a.real), np.asfortranarray(b.imag))
        hir, lir, _ = oracle.gemm_dd("N", "N", np.asfortranarray(a.imag), np.asfortranarray(b.real))
        ex = complex((hre + lre - hii - lii)[0, 0], (hri + lri + hir + lir)[0, 0])
        rel.append(abs(Cz[i, j] - ex) / abs(ex))
    # the reference's CPU arithmetic: OpenBLAS ZGEMM on a K-slab sample
    kb = 512
    As, Bs = np.ascontiguousarray(Az[:4096, :kb]), np.ascontiguousarray(Bz[:4096, :kb].conj().T)
    t0 = time.perf_counter()
    As @ Bs
    cpu_s = time.perf_counter() - t0
    del hA, hB, hC
    flops = 8.0 * n ** 3
    pk, pk_kind = peaks()
    nmod = zinfo["slices"]
    tensor_s = nmod * flops / (pk["bf16_tflops_sustained"] * 1e12)  # one BF16 GEMM per modulus, 8mnk real flops
    bound_s = max(tensor_s, link_s)
    return {"metric": "out-of-HBM streamed GEMM TFLOP/s (host-resident operands, tiles << problem)",
            "value": flops / wall / 1e12, "unit": UNIT, "steps": len(times), "ms_per_step": wall * 1e3,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic U[-1,1], seeded",
            "config": {"workload": f"out-of-HBM: ZGEMM C = A*B^H, m=n=k={n}, {tile}^3 tiles, FP64-accurate "
                                   f"(Chinese-remainder form), streamed from pinned host memory",
                       "scaled_down_from": "65536^3 (206 GB of host matrices, beyond the host's memory)"},
            "moduli": nmod, "h2d_bytes": h2d, "d2h_bytes": d2h,
            "link": {"h2d_GBs_measured": h2d_gbs, "d2h_GBs_measured": d2h_gbs,
                     "tile_copies": "copy engines (page-locked host buffers; the in-place copy kernel, route "
                                    f"{route} for standalone copies, would hold SMs the tile GEMMs wait for)",
                     "link_GBs_achieved": (h2d + d2h) / wall / 1e9},
            "compute_alone_s": compute_s, "link_alone_s": link_s, "overlap_efficiency": max(compute_s, link_s) / wall,
            "accuracy": {"max_rel_err": float(max(rel)), "samples": len(rel),
                         "reference": "double-double (oracle) on sampled entries"},
            "roofline": {"bound": "tensor" if tensor_s >= link_s else "host-link",
                         "achieved": flops / wall / 1e12, "unit": "TFLOP/s",
                         "peak": flops / bound_s / 1e12, "frac": bound_s / wall, "traffic": h2d + d2h,
                         "kernel": "streamer: tile copies by the copy engines on two streams overlapped with "
                                   "the Chinese-remainder GEMM",
                         "peak_note": f"the slower of tensor time ({nmod} BF16 GEMMs of 8mnk flops at the {pk_kind} "
                                      f"sustained BF16 rate) and link time (bytes at the link rates measured in "
                                      f"this run)"},
            "e2e": {"value": flops / wall / 1e12, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "entry": "cosma_gpu_tmm_gemm_z, pinned host A, B, C"},
            "cpu_baseline": {"value": 8.0 * 4096 * 4096 * kb / cpu_s / 1e12, "unit": UNIT,
                             "cores": oracle.openblas_threads(), "kind": "port",
                             "sample": f"OpenBLAS ZGEMM 4096x4096x{kb} sample of the workload ({cpu_s:.2f} s)"},
            "clocks": clocks, "gpu_launches": None}


CONFIGS = {"plain": cfg_plain, "pdgemm": cfg_pdgemm, "grouped": cfg_grouped, "sgemm": cfg_sgemm,
           "stream": cfg_stream, "grouped_crt": cfg_grouped_crt}


# ----------------------------------------------------------------- headline
def headline(args):
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
        return cg.dgemm_ozaki2_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, moduli=args.moduli,
                                      stream=stream)

    for _ in range(max(args.warmup, 3)):
        info = step()
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    gemm_ms, prep_ms = [], []
    for _ in range(args.steps):
        info = step()
        gemm_ms.append(info["gemm_ms"])
        prep_ms.append(info["prep_ms"])
    ev1.record(stream)
    barrier()
    clocks = sampler.stop()
    ms = replica_max_ms(ev0.elapsed_time(ev1) / args.steps, world, dev)
    flops = 2.0 * n * n * n
    value = job_tflops(flops, world, ms)

    # accuracy of every entry against the exact product
    absab = torch.empty_like(dC)
    absab_of(cg, dA, dB, n, absab, stream)
    E, R = torch.empty_like(dC), torch.empty_like(dC)
    acc = full_accuracy(cg, dA, dB, dC, absab, E, R, n, stream)
    rng = np.random.default_rng(1234)
    rows, cols = rng.integers(0, n, 512), rng.integers(0, n, 512)
    Cg = dC.cpu().numpy().reshape(n, n).T
    hi, lo, ab = oracle.gemm_dd_sampled("N", "N", A, B, rows, cols)
    acc["cross_check_double_double_512"] = oracle.error_stats(Cg[rows, cols], hi, lo, ab)
    del Cg

    # the other two arithmetics on the same inputs (one run each, same accuracy check)
    native = None
    if not args.no_native:
        nms, _ = cuda_ms(lambda: cg.gemm_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n, method="native",
                                                stream=stream), stream, 1, warm=False)
        native = {"tflops": flops / (nms * 1e-3) / 1e12, "ms": nms,
                  "accuracy": full_accuracy(cg, dA, dB, dC, absab, E, R, n, stream)}
    sms, sinfo = cuda_ms(lambda: cg.dgemm_ozaki_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n,
                                                       stream=stream), stream, 1)
    slice_form = {"tflops": flops / (sms * 1e-3) / 1e12, "ms": sms, "slices": sinfo["slices"],
                  "products": sinfo["products"], "kernel_ms": sinfo["gemm_ms"],
                  "accuracy": full_accuracy(cg, dA, dB, dC, absab, E, R, n, stream)}

    # end to end through the Tiled-MM C-ABI entry point, pinned host buffers
    hA = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    hB = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    hC = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    hA.numpy()[:] = A.reshape(-1, order="F")
    hB.numpy()[:] = B.reshape(-1, order="F")
    del dA, dB, dC, E, R, absab
    torch.cuda.empty_cache()
    h = cg.make_context("d", 2, 0, 0, 0)
    h.set_method("ozaki2", args.moduli)
    # W untimed warm-up calls: the first allocates the workspaces, and the first
    # transfers over freshly page-locked buffers ran slower than later ones
    for _ in range(max(1, args.warmup)):
        cg.gemm(h, "N", "N", n, n, n, 1.0, hA, n, hB, n, 0.0, hC, n)
    barrier()
    e2e_steps = max(3, min(args.steps, 8))
    calls = []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        c0 = time.perf_counter()
        cg.gemm(h, "N", "N", n, n, n, 1.0, hA, n, hB, n, 0.0, hC, n)
        calls.append(time.perf_counter() - c0)
    barrier()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_val = flops * world / e2e_s / 1e12
    e2e_calls_ms = [round(c * 1e3, 2) for c in calls]
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

    # exponent-spread variants (one step each, every entry checked)
    variants = []
    if not args.no_variants and rank == 0:
        for vphi in (8, 32):
            Av = oracle.exp_spread((n, n), 101 + vphi, vphi)
            Bv = oracle.exp_spread((n, n), 202 + vphi, vphi)
            dA = torch.from_numpy(Av.reshape(-1, order="F")).to(dev)
            dB = torch.from_numpy(Bv.reshape(-1, order="F")).to(dev)
            del Av, Bv
            dC = torch.empty(n * n, dtype=torch.float64, device=dev)
            vms, vinfo = cuda_ms(lambda: cg.dgemm_ozaki2_device("N", "N", n, n, n, 1.0, dA, n, dB, n, 0.0, dC, n,
                                                                stream=stream), stream, 1)
            absab = torch.empty_like(dC)
            absab_of(cg, dA, dB, n, absab, stream)
            E, R = torch.empty_like(dC), torch.empty_like(dC)
            variants.append({"phi": vphi, "tflops": flops / (vms * 1e-3) / 1e12, "moduli": vinfo["slices"],
                             "fraction_bits": vinfo["fraction_bits"], "spread_bits": vinfo["spread_bits"],
                             "accuracy": full_accuracy(cg, dA, dB, dC, absab, E, R, n, stream)})
            del dA, dB, dC, absab, E, R
            torch.cuda.empty_cache()

    # roofline of the dominant kernel: the modular GEMM on the BF16 tensor pipe
    pk, pk_kind = peaks()
    kms = float(np.median(gemm_ms))
    achieved = info["slices"] * flops / (kms * 1e-3) / 1e12
    peak = pk["bf16_tflops_sustained"]
    traffic = None
    if n == 16384 and args.phi == 0 and info["slices"] in TRAFFIC_BYTES_16384:
        traffic = {"bytes": TRAFFIC_BYTES_16384[info["slices"]],
                   "scaled_from": "one-pass ncu capture of this launch on this workload (dram__bytes_read.sum + "
                                  "dram__bytes_write.sum); algorithmic: residues read once "
                                  f"{2 * info['slices'] * n * n * 2 / 1e9:.1f} GB, residue bytes written "
                                  f"{info['slices'] * n * n / 1e9:.1f} GB"}
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "frac_of_burst": achieved / pk["bf16_tflops"], "traffic": traffic["bytes"] if traffic else None,
                "traffic_note": traffic["scaled_from"] if traffic else None,
                "kernel": "oz2::gemm_pair_kernel (tcgen05.mma.cta_group::2 kind::f16, BF16 residues, 256x256 tiles)",
                "work": f"{info['slices']} moduli x 2mnk BF16 flops per launch",
                "peak_note": f"{pk_kind} sustained BF16 dense rate (the kernel runs inside a timed region of "
                             f"{ms * args.steps / 1e3:.1f} s); frac_of_burst against the {pk_kind} burst figure",
                "kernel_ms": kms, "prep_ms": float(np.median(prep_ms)),
                "reconstruct_ms": ms - kms - float(np.median(prep_ms))}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded u*2^e)", "config": config(n, phi),
           "method": "Chinese-remainder form of the Ozaki scheme (Ozaki scheme II): 8-bit integer residues "
                     "(|r| <= 127) on the BF16 tensor cores, exact 1024-deep FP32 accumulations, exact "
                     "reconstruction, one rounding",
           "ozaki2": {"moduli": info["slices"], "fraction_bits": info["fraction_bits"],
                      "spread_bits": info["spread_bits"], "accuracy": acc,
                      "accuracy_target": "max elementwise |C - AB| / |AB| over every nonzero entry of C "
                                         "(max_rel_err) <= 1e-15; max_err_over_absab normalises by (|A||B|)_ij"},
           "native_fp64": native,
           "speedup_vs_native": (value / world / native["tflops"]) if native else None,
           "slice_form": slice_form,
           "variants": variants, "roofline": roofline, "clocks": clocks,
           "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 2 * n * n * 8, "d2h_bytes_per_step": n * n * 8,
                   "entry": "cosma_gpu_tmm_gemm_d (Tiled-MM gpu::gemm drop-in, method ozaki2), pinned host A/B/C: "
                            "the overlapped one-step form (operand panels copied by the copy engines while "
                            "earlier blocks compute, C blocks copied out while later ones do)",
                   "ms_per_step": e2e_s * 1e3, "calls_ms": e2e_calls_ms,
                   "median_ms": float(np.median(calls)) * 1e3, "warmup_calls": max(1, args.warmup),
                   "value_is": "mean over the timed calls (whole timed region / calls)",
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
    del A, B
    return out, rank, world


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config != "precision":
        if args.config in ("grouped", "grouped_crt"):
            out = CONFIGS[args.config](args.steps, args.warmup, count=args.count)
        else:
            out = CONFIGS[args.config](args.steps, args.warmup)
        out.update({"n_gpus": 1, "warmup": max(args.warmup, 3), "scaling": "weak", "vs_baseline": None})
        print(json.dumps(out), flush=True)
        return
    out, rank, world = headline(args)
    if world == 1 and not args.no_configs:
        import torch
        configs = {}
        for name in CONFIG_NAMES:
            t0 = time.perf_counter()
            try:
                configs[name] = CONFIGS[name](min(args.steps, 5), 3)
            except Exception as e:  # one configuration failing must not lose the headline line
                configs[name] = {"error": f"{type(e).__name__}: {e}"}
            configs[name]["wall_s"] = time.perf_counter() - t0
            torch.cuda.empty_cache()
        out["configs"] = configs
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
