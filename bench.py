"""Benchmark of the GB300 dense Cholesky (LLT) path.

Default workload (the configuration the metric is quoted on): n = 32768, 64 right-hand sides,
A = Q diag(lambda) Q^T with Q a product of 8 Householder reflectors and lambda log-spaced over
[1e-6, 1] and randomly permuted (kappa = 1e6), B ~ N(0,1).  One step = one solve of that system
to normwise backward error <= 1e-14, by two arms on the same device-resident inputs: the plain
FP64 factor + solve, and the mixed-precision factorisation + FP64 iterative refinement.  The
8.6 GB matrix is larger than the 129 MB L2, so no flush is needed between steps.  The same line
carries the other configurations as extra keys: the kappa / right-hand-side sweep at n = 32768,
n = 1024 with 16 RHS, the batch of 20000 uneven small systems and the 64 GP-likelihood matrices.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config ...]

--impl reference times the CPU restatement of Eigen's LLT (the oracle; Eigen's own headers do
not exist on the GPU host) on the host cores, on a bounded sample of the same workload.
Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "eigen-git-mirror_gb300"))

METRIC = "LLT solve s & TFLOP/s: FP64 vs mixed+refinement at backward err ≤1e-14"

CONFIGS = {
    "c3": dict(workload="LLT solve to backward error <= 1e-14, n=32768, 64 RHS, Householder spectrum "
                        "kappa=1e6: plain FP64 factor+solve vs mixed-precision factor + FP64 refinement",
               n=32768, nrhs=64, kappa=1e6),
    "c2": dict(workload="LLT solve to backward error <= 1e-14, n=16384, 64 RHS, Householder spectrum kappa=1e6",
               n=16384, nrhs=64, kappa=1e6),
    "c1": dict(workload="LLT solve to backward error <= 1e-14, n=1024, 16 RHS, A=G G^T/n+I", n=1024, nrhs=16,
               kappa=None),
}
DEFAULT_CONFIG = "c3"
CPU_SAMPLE_N = 8192
# split products per algorithmic product of each mixed precision (tc_update's profiled flops count them all)
SPLIT_PRODUCTS = {"fp32": 1, "tf32": 1, "bf16": 1, "tf32x3": 3, "bf16x3": 3, "bf16x6": 6}


def llt_flops(n: int, k: int) -> float:
    return n ** 3 / 3.0 + 2.0 * n * n * k


# ---- clocks during the timed region -----------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = [l.split(",") for l in Path(self.file.name).read_text().splitlines() if l.count(",") >= 8]
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---- distributed plumbing ---------------------------------------------------------------------

def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("GBLLT_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v: float) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---- inputs -----------------------------------------------------------------------------------

def make_inputs_gpu(cfg, seed: int = 1):
    """Synthetic inputs generated on the GPU with torch's seeded generator (same construction as
    the oracle's generators: G G^T/n + I, or 8 Householder reflectors around a log-spaced,
    randomly permuted spectrum)."""
    import torch
    n, k = cfg["n"], cfg["nrhs"]
    g = torch.Generator(device="cuda").manual_seed(seed)
    f64 = torch.float64
    if cfg["kappa"] is None:
        G = torch.randn(n, n, generator=g, dtype=f64, device="cuda")
        A = G @ G.T / n + torch.eye(n, dtype=f64, device="cuda")
        del G
    else:
        j = torch.arange(n, dtype=f64, device="cuda")
        lam = cfg["kappa"] ** (-1.0 + j / max(n - 1, 1))
        lam = lam[torch.randperm(n, generator=g, device="cuda")]
        A = torch.diag(lam)
        for _ in range(8):
            v = torch.randn(n, generator=g, dtype=f64, device="cuda")
            beta = 2.0 / torch.dot(v, v)
            p = beta * (A @ v)
            w = p - 0.5 * beta * torch.dot(v, p) * v
            A.addr_(v, w, alpha=-1.0)
            A.addr_(w, v, alpha=-1.0)
    B = torch.randn(k, n, generator=g, dtype=f64, device="cuda")  # row-major k x n = column-major n x k
    torch.cuda.synchronize()
    return A.contiguous(), B.contiguous()


def fp64_peak_tflops() -> float:
    """cuBLAS DGEMM 4096^3 throughput (best of 3): the FP64 roofline denominator."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    a @ b
    best = 1e9
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        e0.record()
        a @ b
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


# ---- CPU legs (oracle: test infrastructure, used only here and in the tests) -------------------

def cpu_sample(reps_max: int = 3, min_seconds: float = 10.0) -> dict:
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    if not O.LIB_PATH.exists():
        O.build(ref=False)
    n, k = CPU_SAMPLE_N, 64
    a = O.gen_householder(n, 1e6)
    b = np.asfortranarray(O.normal(12, n * k).reshape(k, n).T)
    times = []
    t_start = time.perf_counter()
    be = None
    while len(times) < reps_max and (time.perf_counter() - t_start < min_seconds or not times):
        f = np.array(a, order="F", copy=True)
        x = np.array(b, order="F", copy=True)
        t0 = time.perf_counter()
        info = O.potrf(f)
        O.potrs(f, x)
        times.append(time.perf_counter() - t0)
        assert info == 0
        if be is None:
            be = O.backward_error(a, np.asfortranarray(x[:, :2]), np.asfortranarray(b[:, :2]))
    t = statistics.median(times)
    return {"value": llt_flops(n, k) / t / 1e12, "unit": "TFLOP/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"n={n}, 64 RHS, same Householder construction (kappa=1e6), FP64 factor+solve, "
                      f"median of {len(times)} wall-clock runs ({t:.2f} s each); OpenMP over SYRK/TRSM rows",
            "seconds": t, "backward_error": be}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    if not O.LIB_PATH.exists():
        O.build(ref=False)
    cfg = CONFIGS[args.config]
    n, k = min(cfg["n"], CPU_SAMPLE_N), cfg["nrhs"]
    a = O.gen_householder(n, 1e6) if cfg["kappa"] else O.gen_gram(n)
    b = np.asfortranarray(O.normal(12, n * k).reshape(k, n).T)

    def step():
        f = np.array(a, order="F", copy=True)
        x = np.array(b, order="F", copy=True)
        t0 = time.perf_counter()
        info = O.potrf(f)
        O.potrs(f, x)
        dt = time.perf_counter() - t0
        assert info == 0
        return dt

    for _ in range(args.warmup):
        step()
    ts = [step() for _ in range(args.steps)]
    total = sum(ts)
    value = llt_flops(n, k) * len(ts) / total / 1e12
    sample = (f"n={n}, {k} RHS, same construction as the workload, FP64 factor+solve per step "
              f"(CPU restatement of Eigen's blocked LLT; OpenMP over SYRK/TRSM rows)")
    # config.n is the order actually timed; the workload it samples is named beside it
    out = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": total / len(ts) * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"LLT factor+solve FP64 on the CPU, n={n}, {k} RHS: a bounded sample of "
                                  f"the n={cfg['n']} workload", "n": n, "nrhs": k, "kappa": cfg["kappa"],
                      "sample_of": {"workload": cfg["workload"], "n": cfg["n"]}},
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": O.num_threads(), "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ---- GPU arm ------------------------------------------------------------------------------------

def measured_peaks() -> dict:
    """Roofline denominators: HBM and BF16 from MEASURED_PEAKS.json (measured on this machine),
    FP64 and TF32 measured here with cuBLAS (they are not in that file)."""
    import torch
    out = {"fp64_tflops": fp64_peak_tflops(), "source": {}}
    out["source"]["fp64_tflops"] = "cuBLAS DGEMM 4096^3, best of 3, this run"
    n = 8192
    a = torch.randn(n, n, device="cuda")
    b = torch.randn(n, n, device="cuda")
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    a @ b
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e9
    for _ in range(3):
        e0.record()
        a @ b
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    torch.backends.cuda.matmul.allow_tf32 = old
    out["tf32_tflops"] = 2.0 * n ** 3 / (best * 1e-3) / 1e12
    out["source"]["tf32_tflops"] = "cuBLAS TF32 GEMM 8192^3, best of 3, this run"
    mp = ROOT / "MEASURED_PEAKS.json"
    if mp.exists():
        d = json.loads(mp.read_text())
        out["hbm_gbs"], out["bf16_tflops"] = d["hbm_gbs"], d["bf16_tflops"]
        out["source"]["hbm_gbs"] = out["source"]["bf16_tflops"] = "of measured (MEASURED_PEAKS.json)"
    else:
        out["hbm_gbs"], out["bf16_tflops"] = 6800.0, 1900.0
        out["source"]["hbm_gbs"] = out["source"]["bf16_tflops"] = "of fallback"
    return out


# DRAM bytes (read + write) per launch from ncu captures of the kernel on a smaller case, and the
# law that scales them to this run's launch (profiles/ holds the summaries with the commands):
#   symm_residual_f64 (NR = 16 kernel): 1.628 GB at n = 8192, 64 RHS; A's stored tiles are read
#     once per 16-column chunk of right-hand sides, so traffic grows as n^2 * ceil(k / 16).
#   sweep_f32 (chains of 32 columns): 578 MB at n = 16384, 64 RHS (mean of the forward and backward
#     launch); the triangle of L is read about once whatever k is, so traffic grows as n^2.
#   tc_update_bf16: the look-ahead launch at n = 8192 moved 0.75 of its algorithmic bytes with BF16x6
#     and 0.755 with BF16x3 (C read and written once in FP32, the operand parts once; part of C stays
#     in L2): the launch's algorithmic bytes times that ratio.
NCU_TRAFFIC = {"symm_residual_f64": (8192, 64, 1.628e9, "n2_kchunks"),
               "sweep_f32": (16384, 64, 5.78e8, "n2"),
               "tc_update_bf16": (8192, 64, 0.75, "ratio")}
TRAFFIC_SOURCE = {"n2_kchunks": "ncu dram__bytes_read.sum + dram__bytes_write.sum at n={n0}, {k0} RHS, scaled by "
                                "n^2 ceil(k/16)",
                  "n2": "ncu dram__bytes_read.sum + dram__bytes_write.sum at n={n0}, {k0} RHS, scaled by n^2",
                  "ratio": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a look-ahead launch at n={n0}: "
                           "{by} of its algorithmic bytes, applied to this launch's algorithmic bytes"}


def ncu_traffic(name: str, n: int, k: int, per_launch_bytes: float | None = None):
    if name not in NCU_TRAFFIC or k < 16:
        return None
    n0, k0, by, law = NCU_TRAFFIC[name]
    if law == "ratio":
        return by * per_launch_bytes if per_launch_bytes else None
    scale = (n / n0) ** 2
    if law == "n2_kchunks":
        scale *= (-(-k // 16)) / (-(-k0 // 16))
    return by * scale


# The FP64-exact products on the tensor cores (ozaki.cu) run 36 BF16 products per FP64 product
# (8 slices per operand, the slice pairs p + q <= 9); the split-precision trailing updates run 3 or 6.
# `achieved` counts the algorithmic work only (one product); the products the tensor cores actually
# execute are reported under `split_products`.
OZAKI_KERNELS = ("syrk_tc_f64", "residual_tc")
OZAKI_PRODUCTS = 36


def roofline_for(name: str, st: dict, peaks: dict, n: int = 0, k: int = 0, nseg: int = 1) -> dict:
    """Achieved = algorithmic work of the kernel's launches / their summed device time, against the
    peak of the unit the kernel runs on.  st["flops"] is the profiled work: for tc_update_* it counts
    every split product (nseg per algorithmic product); for the ozaki kernels it is the FP64 product."""
    ms = max(st["ms"], 1e-9)
    products = 1
    if name in OZAKI_KERNELS:
        bound, unit, peak, src = "tensor", "TFLOP/s", peaks["bf16_tflops"], peaks["source"]["bf16_tflops"]
        ach = st["flops"] / ms / 1e9
        products = OZAKI_PRODUCTS
    elif name.startswith("tc_update_tf32") or name.startswith("tc_update_bf16"):
        key = "tf32_tflops" if name.startswith("tc_update_tf32") else "bf16_tflops"
        bound, unit, peak, src = "tensor", "TFLOP/s", peaks[key], peaks["source"][key]
        products = max(int(nseg), 1)
        ach = st["flops"] / products / ms / 1e9
    elif name.endswith("_f64") and st["flops"] > 0 and not name.startswith(("trsv", "split", "transpose")):
        bound, unit, peak, src = "tensor", "TFLOP/s", peaks["fp64_tflops"], peaks["source"]["fp64_tflops"] + \
            " (FP64 pipe: DFMA and DMMA run at the same rate on GB300)"
        ach = st["flops"] / ms / 1e9
    else:
        bound, unit, peak, src = "hbm", "GB/s", peaks["hbm_gbs"], peaks["source"]["hbm_gbs"]
        ach = st["bytes"] / ms / 1e6
    traffic = ncu_traffic(name, n, k, st["bytes"] / st["launches"])
    per_launch = st["flops"] / st["launches"] / (products if name not in OZAKI_KERNELS else 1)
    src_fmt = NCU_TRAFFIC[name] if name in NCU_TRAFFIC else None
    out = {"kernel": name, "bound": bound, "achieved": ach, "peak": peak, "unit": unit, "frac": ach / peak,
           "work": "algorithmic flops (one product per output and depth step)" if unit == "TFLOP/s"
           else "algorithmic bytes",
           "traffic": traffic,
           "traffic_source": TRAFFIC_SOURCE[src_fmt[3]].format(n0=src_fmt[0], k0=src_fmt[1], by=src_fmt[2])
           if traffic else None, "launches": st["launches"],
           "per_launch_flops": per_launch, "per_launch_bytes": st["bytes"] / st["launches"],
           "peak_source": src,
           "timing": "CUDA events around each launch of the kernel, on its stream, in a repeat of the timed steps"}
    if products > 1:
        out["split_products"] = {"products_per_algorithmic_product": products, "tensor_achieved": ach * products,
                                 "tensor_frac": ach * products / peak,
                                 "note": "the tensor cores' executed work, all split products counted"}
    return out


def measure_config(args, cfg, ws, rank, local, peaks, steps, warmup, profile_steps, e2e_calls,
                   clocks_on=True) -> dict:
    """Both arms of one configuration on the same device-resident inputs: the plain FP64 factor +
    solve and the mixed-precision solve with FP64 refinement.  Returns the arms, the headline (the
    faster arm whose solution an independent torch FP64 residual puts at backward error <= 1e-14)
    and the end-to-end figure through the host-pointer C ABI."""
    import ctypes
    import torch
    import gbllt as G

    n, k = cfg["n"], cfg["nrhs"]
    flops = llt_flops(n, k)
    A0, B0 = make_inputs_gpu(cfg, seed=1 + rank)
    A = torch.empty_like(A0)
    B = torch.empty_like(B0)
    X = torch.zeros_like(B0)
    info = torch.zeros(1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    opts = G.mixed_opts(args.mixed_precision, 10, 1e-14, fallback=False, panel=args.panel,
                        reserve_sms=args.reserve_sms)
    nseg = SPLIT_PRODUCTS[args.mixed_precision]
    reports = []

    def step_fp64():
        with torch.cuda.stream(stream):
            A.copy_(A0)
            B.copy_(B0)
            G.potrf_dev(A, n, n, info, "L", sp)
            G.potrs_dev(A, n, n, B, k, n, "L", sp)

    def step_mixed():
        with torch.cuda.stream(stream):
            rc, rep = G.posv_mixed_dev(A0, n, n, B0, n, X, n, k, opts, "L", sp, raise_on_error=False)
            reports.append((rc, rep))

    # L2 hygiene: a matrix smaller than 4 x L2 (129 MB) gets a 512 MB write between timed steps
    l2_bytes = 129 << 20
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda") if n * n * 8 < 4 * l2_bytes else None
    l2_note = (f"inputs larger than L2 (matrix {n * n * 8 / 1e9:.1f} GB vs 129 MB L2)" if flush is None else
               f"L2 flushed before each timed step (512 MB write; matrix {n * n * 8 / 1e6:.0f} MB)")

    def timed(step_fn, nprof):
        for _ in range(max(warmup, 0)):
            step_fn()
        stream.synchronize()
        clocks = ClockSampler(local) if clocks_on else None
        barrier(ws)
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if flush is None:  # inputs larger than L2: one timed region over all steps
            e0.record(stream)
            for _ in range(steps):
                step_fn()
            e1.record(stream)
            e1.synchronize()
            total_ms = e0.elapsed_time(e1)
        else:  # small inputs: L2 flushed (a write larger than L2) before each step, outside its timing
            total_ms = 0.0
            for _ in range(steps):
                with torch.cuda.stream(stream):
                    flush.zero_()
                e0.record(stream)
                step_fn()
                e1.record(stream)
                e1.synchronize()
                total_ms += e0.elapsed_time(e1)
        torch.cuda.synchronize()
        barrier(ws)
        ck = clocks.stop() if clocks else None
        # per-kernel device times (roofline, shares) from a repeat of nprof steps with CUDA events
        # around every launch; the events cost a few percent, so they stay out of the timed region
        prof = {}
        if nprof > 0:
            G.profile_enable(True)
            for _ in range(nprof):
                if flush is not None:
                    with torch.cuda.stream(stream):
                        flush.zero_()
                step_fn()
            torch.cuda.synchronize()
            prof = G.profile_read()
            G.profile_enable(False)
        return max_over_ranks(ws, total_ms), prof, ck

    def backward_error(Xs):  # torch FP64 GEMM as an independent check of the returned solution
        R = A0 @ Xs.T - B0.T
        return float(torch.linalg.norm(R) / (torch.linalg.norm(A0) * torch.linalg.norm(Xs)))

    # --arms fp64 / mixed (profiling a smaller case) times one arm only; that arm is then the headline
    run64, runmx = args.arms != "mixed", args.arms != "fp64"
    ms64 = prof64 = ck64 = be64 = msmx = profmx = ckmx = bemx = None
    mixed_ok = False
    if run64:
        ms64, prof64, ck64 = timed(step_fp64, profile_steps[0])
        assert int(info.item()) == 0, f"factorisation failed, info={int(info.item())}"
        be64 = backward_error(B)
    if runmx:
        reports.clear()
        msmx, profmx, ckmx = timed(step_mixed, profile_steps[1])
        rcs = {rc for rc, _ in reports}
        rep = reports[-1][1]
        bemx = backward_error(X)
        mixed_ok = rcs == {G.SUCCESS} and rep["converged"] and bemx <= 1e-14

    def arm(ms, prof, be, nprof, extra, seg=1):
        d = {"seconds_per_solve": ms / steps / 1e3, "tflops": ws * flops * steps / (ms * 1e-3) / 1e12,
             "backward_error": be, "reached_1e-14": be <= 1e-14}
        if prof:
            top = max(prof.items(), key=lambda kv: kv[1]["ms"])
            total = sum(v["ms"] for v in prof.values())
            d["gpu_launches"] = int(round(sum(v["launches"] for v in prof.values()) * steps / nprof))
            d["roofline"] = dict(roofline_for(top[0], top[1], peaks, n, k,
                                              seg if top[0].startswith("tc_update") else 1),
                                 kernel_share_of_device_time=top[1]["ms"] / total)
            d["kernels"] = {kn: {"launches": v["launches"], "ms": v["ms"]} for kn, v in prof.items()}
            d["kernels_note"] = f"launches and device ms summed over {nprof} profiled steps"
        d.update(extra)
        return d

    fp64 = mixed = None
    if run64:
        fp64 = arm(ms64, prof64, be64, profile_steps[0],
                   {"path": "plain FP64: gbllt_dpotrf_dev + gbllt_dpotrs_dev"})
    if runmx:
        mixed = arm(msmx, profmx, bemx, profile_steps[1],
                    {"path": f"gbllt_dposv_mixed_dev precision={args.mixed_precision}, FP64 residuals, tol 1e-14, "
                             f"no fallback", "precision": args.mixed_precision, "reached_1e-14": mixed_ok,
                     "steps": rep["steps"], "history": rep["history"], "factor_ms": rep["factor_ms"],
                     "refine_ms": rep["refine_ms"]}, nseg)
    use_mixed = mixed_ok and (fp64 is None or mixed["seconds_per_solve"] < fp64["seconds_per_solve"])
    head = mixed if use_mixed else fp64
    assert head is not None, "the mixed arm alone did not reach backward error 1e-14"
    del A, B
    torch.cuda.empty_cache()

    # end to end through the host-pointer C ABI (pinned host buffers; the copies are inside the call)
    e2e = None
    if e2e_calls > 0:
        hA = torch.empty(A0.shape, dtype=A0.dtype, pin_memory=True)
        hA.copy_(A0)
        hB0 = B0.cpu().pin_memory()
        hB = torch.empty(hB0.shape, dtype=hB0.dtype).pin_memory()
        hX = torch.zeros(hB0.shape, dtype=hB0.dtype).pin_memory()
        hA0 = None
        if not use_mixed:  # the FP64 entry overwrites A with its factor: keep a pristine copy
            hA0 = torch.empty(A0.shape, dtype=A0.dtype, pin_memory=True)
            hA0.copy_(A0)
        a_np, b_np, x_np = hA.numpy(), hB.numpy(), hX.numpy()
        tt = []
        for i in range(1 + e2e_calls):
            if hA0 is not None:
                hA.copy_(hA0)
            hB.copy_(hB0)
            inf = ctypes.c_int64(0)
            t0 = time.perf_counter()
            if use_mixed:
                r = G.MixedReport()
                rc = G.lib().gbllt_dposv_mixed(G.COL_MAJOR, b"L", n, k, a_np.ctypes.data, n, b_np.ctypes.data, n,
                                               x_np.ctypes.data, n, ctypes.byref(opts), ctypes.byref(r))
            else:
                rc = G.lib().gbllt_dposv(G.COL_MAJOR, b"L", n, k, a_np.ctypes.data, n, b_np.ctypes.data, n,
                                         ctypes.byref(inf))
            dt = time.perf_counter() - t0
            G.check("e2e", rc)
            if i > 0:  # the first call warms up
                tt.append(dt)
        e2e_s = max_over_ranks(ws, sum(tt) / len(tt))
        # the library copies A's stored triangle in 256-column blocks, each from its diagonal row down
        # (and the FP64 entry copies the factor's back)
        tri = sum((n - j0) * min(256, n - j0) for j0 in range(0, n, 256)) * 8
        bytes_io = tri + int(n * k * 8)
        e2e = {"value": ws * flops / e2e_s / 1e12, "unit": "TFLOP/s", "seconds_per_step": e2e_s,
               "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": int(n * k * 8) if use_mixed else bytes_io,
               "calls_timed": len(tt),
               "path": ("gbllt_dposv_mixed" if use_mixed else "gbllt_dposv") + " (host pointers, pinned), wall clock"}
        del hA, hA0, hB, hB0, hX
    res = {"n": n, "nrhs": k, "kappa": cfg["kappa"], "fp64": fp64, "mixed": mixed, "use_mixed": use_mixed,
           "head": head, "ms_head": msmx if use_mixed else ms64, "clocks": ckmx if use_mixed else ck64,
           "clocks_fp64_arm": ck64, "e2e": e2e, "l2": l2_note, "flops": flops,
           "mixed_over_fp64_speedup": (fp64["seconds_per_solve"] / mixed["seconds_per_solve"]
                                       if mixed_ok and fp64 is not None else None)}
    del A0, B0, X
    torch.cuda.empty_cache()
    return res


def c3_sweep(args, n: int, fp64_k64_s: float | None) -> dict:
    """The rest of the n = 32768 configuration: kappa in {1e2, 1e4, 1e6} and 1 or 64 right-hand
    sides, the mixed solve (the headline precision) after one warm-up call, and the plain FP64
    factor + solve with 1 right-hand side, each checked by an independent torch FP64 residual."""
    import torch
    import gbllt as G
    s = torch.cuda.current_stream().cuda_stream
    opts = G.mixed_opts(args.mixed_precision, 10, 1e-14, False)
    rows = []
    fp64_s = {64: fp64_k64_s}
    for kappa in (1e2, 1e4, 1e6):
        A0, B64 = make_inputs_gpu({"n": n, "nrhs": 64, "kappa": kappa}, seed=3)
        for k in (1, 64):
            B0 = B64[:k].contiguous()
            if k == 1 and kappa == 1e6:  # the FP64 time does not depend on kappa
                A = A0.clone()
                B = B0.clone()
                info = torch.zeros(1, dtype=torch.int64, device="cuda")
                for it in range(2):  # the first pass warms up
                    A.copy_(A0)
                    B.copy_(B0)
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    G.potrf_dev(A, n, n, info, "L", s)
                    G.potrs_dev(A, n, n, B, k, n, "L", s)
                    torch.cuda.synchronize()
                    fp64_s[1] = time.perf_counter() - t0
                R = A0 @ B.T - B0.T
                be = float(torch.linalg.norm(R) / (torch.linalg.norm(A0) * torch.linalg.norm(B)))
                rows.append({"path": "fp64", "nrhs": k, "kappa": kappa, "seconds": fp64_s[1], "backward_error": be})
                del A, B
            X = torch.zeros_like(B0)
            G.posv_mixed_dev(A0, n, n, B0, n, X, n, k, opts, "L", s, raise_on_error=False)  # warm-up
            X.zero_()  # a failed low-precision factorisation leaves X untouched
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc, rep = G.posv_mixed_dev(A0, n, n, B0, n, X, n, k, opts, "L", s, raise_on_error=False)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            R = A0 @ X.T - B0.T
            be = float(torch.linalg.norm(R) / (torch.linalg.norm(A0) * torch.linalg.norm(X)))
            rows.append({"path": "mixed", "precision": args.mixed_precision, "nrhs": k, "kappa": kappa,
                         "seconds": dt, "reached_1e-14": bool(rc == 0 and rep["info"] == 0 and rep["converged"]
                                                              and be <= 1e-14),
                         "steps": rep["steps"], "backward_error": be, "factor_ms": rep["factor_ms"],
                         "refine_ms": rep["refine_ms"]})
        del A0, B64
        torch.cuda.empty_cache()
    for r in rows:
        if r["path"] == "mixed" and fp64_s.get(r["nrhs"]):
            r["speedup_vs_fp64"] = fp64_s[r["nrhs"]] / r["seconds"]
    return {"n": n, "timing": "wall clock around one call after one warm-up call (64-RHS FP64 time: the "
                              "headline arm's device-timed mean)", "rows": rows}


def run_ours(args, ws, rank, local):
    import torch

    torch.cuda.set_device(local)
    cfg = dict(CONFIGS[args.config])
    if args.n:
        cfg["n"] = args.n
        cfg["workload"] += f" (n overridden to {args.n})"
    peaks = measured_peaks()
    K, W = args.steps, args.warmup
    # the FP64 arm's per-kernel profile repeats a few steps (its steps take a second at n = 32768)
    main = measure_config(args, cfg, ws, rank, local, peaks, K, W, (min(K, 5), K), max(3, min(K, 10)))
    head = main["head"]
    extras = {}
    if args.config == DEFAULT_CONFIG and not args.no_extras and args.arms == "both":
        extras["c3_sweep"] = c3_sweep(args, cfg["n"], main["fp64"]["seconds_per_solve"])
        c1 = measure_config(args, CONFIGS["c1"], ws, rank, local, peaks, max(K, 10), max(W, 3), (0, 0), 5,
                            clocks_on=False)
        extras["c1"] = {"workload": CONFIGS["c1"]["workload"], "l2": c1["l2"], "e2e": c1["e2e"],
                        "headline": "mixed+refinement" if c1["use_mixed"] else "plain FP64",
                        "fp64": c1["fp64"], "mixed": c1["mixed"]}
        extras["c4"] = run_c4(args, ws, rank, steps=max(3, min(K, 10)))
        extras["c5"] = run_c5(args, passes=2)
    if rank != 0:
        return
    cpu = None if args.no_cpu_baseline or ws > 1 else cpu_sample()
    n, k = main["n"], main["nrhs"]
    use_mixed = main["use_mixed"]
    out = {
        "metric": METRIC, "value": ws * main["flops"] * K / (main["ms_head"] * 1e-3) / 1e12, "unit": "TFLOP/s",
        "n_gpus": ws, "steps": K, "warmup": W, "ms_per_step": main["ms_head"] / K,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": f"{args.mixed_precision}+f64" if use_mixed else "f64", "data": "synthetic",
        "config": {"workload": cfg["workload"], "n": n, "nrhs": k, "kappa": cfg["kappa"],
                   "headline": "mixed+refinement" if use_mixed else "plain FP64",
                   "work_per_step_flops": main["flops"], "work": "n^3/3 + 2 n^2 k FP64-equivalent flop per solve",
                   "accuracy": "normwise backward error <= 1e-14 (checked with a torch FP64 residual of the "
                               "returned X)", "l2": main["l2"]},
        "seconds_per_solve": head["seconds_per_solve"], "backward_error": head["backward_error"],
        "mixed_over_fp64_speedup": main["mixed_over_fp64_speedup"],
        "roofline": head["roofline"], "gpu_launches": head["gpu_launches"],
        "fp64": main["fp64"], "mixed": main["mixed"], "peaks": peaks,
        "e2e": main["e2e"], "cpu_baseline": cpu, "clocks": main["clocks"], "clocks_fp64_arm": main["clocks_fp64_arm"],
    }
    out.update(extras)
    print(json.dumps(out), flush=True)


# ---- other configurations (one JSON line each; the default run is the one above) -------------------

def run_c4(args, ws: int = 1, rank: int = 0, steps: int | None = None) -> dict:
    """20000 SPD systems, n_i ~ U{4..256}, one RHS each, FP64 and FP32, one graph-replayed launch.
    With N ranks the systems are sharded by cost (shard.partition, no data-path collective): each
    rank solves its share, the step time is the maximum over ranks, and the value counts all
    20000 systems (fixed total work: strong scaling)."""
    import torch
    import gbllt as G
    import shard
    count_all = 20000
    steps = steps or args.steps
    rng = torch.Generator(device="cpu").manual_seed(21)
    sizes_all = torch.randint(4, 257, (count_all,), generator=rng).numpy().astype(np.int64)
    sizes = sizes_all[shard.partition(sizes_all, ws)[rank]] if ws > 1 else sizes_all
    count = len(sizes)
    out = {"metric": "batched LLT solves/s and fraction of HBM", "config": {
        "workload": "C4: 20000 SPD systems, n_i uniform in [4,256], A_i = G_i G_i^T/n_i + 0.1 I, 1 RHS each",
        "count": count_all, "ranks": ws}, "unit": "solves/s", "higher_is_better": True, "data": "synthetic",
        "n_gpus": ws, "scaling": "strong", "results": []}
    peaks = {"hbm_gbs": json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"]
             if (ROOT / "MEASURED_PEAKS.json").exists() else 6800.0, "fp64_tflops": fp64_peak_tflops()}
    s = torch.cuda.current_stream().cuda_stream
    for dt, tdt, name in ((np.float64, torch.float64, "f64"), (np.float32, torch.float32, "f32")):
        plan = G.BatchPlan(sizes, dt)
        variant = plan.tune(str(ROOT / "eigen-git-mirror_gb300" / "lib" / "batched_tune.json"), s)
        # A_i = G_i G_i^T / n_i + 0.1 I built on the device, system by system into the packed array
        a0 = torch.empty(plan.a_elems, dtype=tdt, device="cuda")
        g = torch.Generator(device="cuda").manual_seed(22)
        for i, nn in enumerate(sizes):
            nn = int(nn)
            Gm = torch.randn(nn, nn, generator=g, dtype=torch.float64, device="cuda")
            Ai = Gm @ Gm.T / nn + 0.1 * torch.eye(nn, dtype=torch.float64, device="cuda")
            a0[int(plan.aoff[i]):int(plan.aoff[i]) + nn * nn] = Ai.T.reshape(-1).to(tdt)
        b0 = torch.randn(plan.b_elems, generator=g, dtype=torch.float64, device="cuda").to(tdt)
        a = torch.empty_like(a0)
        b = torch.empty_like(b0)
        info = torch.zeros(count, dtype=torch.int64, device="cuda")
        for _ in range(max(args.warmup, 3)):
            a.copy_(a0)
            b.copy_(b0)
            plan.solve_dev(a, b, info, s)
        torch.cuda.synchronize()
        G.profile_enable(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        tot = 0.0
        for _ in range(steps):
            a.copy_(a0)
            b.copy_(b0)
            barrier(ws)
            torch.cuda.synchronize()
            e0.record()
            plan.solve_dev(a, b, info, s)
            e1.record()
            e1.synchronize()
            tot += max_over_ranks(ws, e0.elapsed_time(e1))
        prof = G.profile_read()
        G.profile_enable(False)
        assert int(info.max()) == 0
        st = prof[f"batched_posv_{name}"]
        ms = tot / steps
        gbs = st["bytes"] / st["ms"] / 1e6
        tfs = st["flops"] / st["ms"] / 1e9
        out["results"].append({"dtype": name, "ms": ms, "solves_per_s": count_all / (ms * 1e-3),
                               "achieved_gbs": gbs, "hbm_frac": gbs / peaks["hbm_gbs"], "achieved_tflops": tfs,
                               "fp64_frac": tfs / peaks["fp64_tflops"] if name == "f64" else None,
                               "variant": plan.variant(), "launches_per_step": 1,
                               "per_rank_note": "achieved_* are rank 0's kernel on its shard" if ws > 1 else None})
        if name == "f64":
            # the same FP64 systems to FP64 accuracy with FP32 factors and FP64 refinement
            # (gbllt_batch_dposv_mixed_dev; A and b read only, x separate)
            x = torch.empty_like(b0)
            opts = G.mixed_opts("fp32", 10, 1e-14, fallback=True)
            rep = plan.solve_mixed_dev(a0, b0, x, info, opts, s)  # warm-up: tunes the FP32 plan once
            torch.cuda.synchronize()
            tot = 0.0
            for _ in range(steps):
                barrier(ws)
                torch.cuda.synchronize()
                e0.record()
                rep = plan.solve_mixed_dev(a0, b0, x, info, opts, s)
                e1.record()
                e1.synchronize()
                tot += max_over_ranks(ws, e0.elapsed_time(e1))
            assert int(info.max()) == 0 and int(info.min()) == 0
            ms = tot / steps
            fl = sum(float(v) ** 3 / 3.0 + 2.0 * float(v) ** 2 for v in sizes)
            by = sum((float(v) * (v + 1) + 2.0 * v) * 8.0 for v in sizes)
            out["results"].append({
                "dtype": "f64 (FP32 factors + FP64 refinement)", "ms": ms, "solves_per_s": count_all / (ms * 1e-3),
                "achieved_tflops_fp64_equivalent": fl / ms / 1e9, "fp64_frac": fl / ms / 1e9 / peaks["fp64_tflops"],
                "achieved_gbs_fp64_bytes": by / ms / 1e6, "hbm_frac": by / ms / 1e6 / peaks["hbm_gbs"],
                "refinement": rep, "speedup_vs_fp64": out["results"][-1]["ms"] / ms,
                "path": "gbllt_batch_dposv_mixed_dev, tol 1e-14, FP64 fallback on; every system converged "
                        "(info 0); the time includes one host read per refinement step"})
    out["peaks"] = peaks
    out["steps"] = steps
    out["timing"] = "CUDA events around each graph-replayed launch (max over ranks), inputs restored between steps"
    return out


def run_c5(args, passes: int = 2) -> dict:
    """64 RBF kernel matrices, n = 2048 (x ~ U[0,1]^3, lengthscale 0.2, variance 1, noise 1e-2),
    y ~ N(0,1): f = logdet A + y^T A^{-1} y forward and the hand-written adjoint (dA, dy) in FP64 and
    in mixed precision, each gradient's error against the closed form stated; the mixed-precision
    forward solves A alpha = y with the tensor-core factorisation + refinement."""
    import torch
    import gbllt as G
    nmat, n = 64, args.n or 2048
    s = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device="cuda").manual_seed(31)
    X = torch.rand(nmat, n, 3, generator=g, dtype=torch.float64, device="cuda")
    Y = torch.randn(nmat, n, generator=g, dtype=torch.float64, device="cuda")
    d2 = ((X[:, :, None, :] - X[:, None, :, :]) ** 2).sum(-1)
    A = torch.exp(-d2 / (2 * 0.2 ** 2)) + 1e-2 * torch.eye(n, dtype=torch.float64, device="cuda")
    del d2
    # the 64 independent problems run on NSTREAM concurrent streams (matrix m on stream m % NSTREAM)
    nstream = 8
    streams = [torch.cuda.Stream() for _ in range(nstream)]
    infos = [torch.zeros(1, dtype=torch.int64, device="cuda") for _ in range(nstream)]
    res = {}
    for it in range(max(passes, 2)):  # the first pass warms up, the last one is reported
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Ls, alphas, fs = [None] * nmat, [None] * nmat, [None] * nmat
        for m in range(nmat):
            st = streams[m % nstream]
            with torch.cuda.stream(st):
                L = A[m].clone()  # symmetric: row-major storage = column-major A
                G.potrf_dev(L, n, n, infos[m % nstream], "L", st.cuda_stream)
                al = Y[m].clone().reshape(1, n)
                G.potrs_dev(L, n, n, al, 1, n, "L", st.cuda_stream)
                fs[m] = 2.0 * torch.log(torch.diagonal(L)).sum() + torch.dot(Y[m], al.reshape(n))
                Ls[m], alphas[m] = L, al
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0

        def backward(mixed):
            t0 = time.perf_counter()
            grads = [None] * nmat
            for m in range(nmat):
                st = streams[m % nstream]
                with torch.cuda.stream(st):
                    M = torch.zeros_like(Ls[m])
                    M.diagonal().copy_(2.0 / torch.diagonal(Ls[m]))
                    G.potrf_adjoint_dev(Ls[m], n, n, M, n, st.cuda_stream, mixed=mixed)
                    bbar = torch.empty_like(alphas[m])
                    G.potrs_adjoint_dev(Ls[m], n, n, alphas[m], n, Y[m].reshape(1, n), n, bbar, n, 1, M, n,
                                        st.cuda_stream)
                    grads[m] = M
            torch.cuda.synchronize()
            return time.perf_counter() - t0, grads

        t_bwd, grads = backward(False)
        t_bwd_mx, grads_mx = backward(True)
        res = {"forward_s": t_fwd, "backward_s": t_bwd, "backward_mixed_s": t_bwd_mx, "streams": nstream}
    # gradient check of the first matrix against the closed form A^{-1} - a a^T (cuSOLVER FP64)
    Ainv = torch.cholesky_inverse(torch.linalg.cholesky(A[0]))
    a0 = alphas[0].reshape(n)
    want = torch.tril(Ainv - torch.outer(a0, a0))
    for key, gr in (("grad_rel_err_vs_closed_form", grads), ("grad_mixed_rel_err_vs_closed_form", grads_mx)):
        got = gr[0].T.tril()
        res[key] = float(torch.linalg.norm(got - want) / torch.linalg.norm(want))
    res["backward_paths"] = {"backward_s": "gbllt_dpotrf_adjoint_dev (FP64-exact panel products)",
                             "backward_mixed_s": "gbllt_dpotrf_adjoint_mixed_dev (28-bit panel products)"}
    # mixed-precision forward solve of the same systems
    opts = G.mixed_opts(args.mixed_precision, 10, 1e-14, True)
    torch.cuda.synchronize()
    Xs = [torch.zeros(1, n, dtype=torch.float64, device="cuda") for _ in range(nmat)]
    # each mixed solve reads its convergence test on the host, so the streams are driven by one host
    # thread each (ctypes releases the GIL during the call)
    from concurrent.futures import ThreadPoolExecutor

    def mixed_chain(t):
        st = streams[t]
        torch.cuda.set_device(0)
        got = []
        with torch.cuda.stream(st):
            for m in range(t, nmat, nstream):
                rc, rep = G.posv_mixed_dev(A[m], n, n, Y[m].reshape(1, n), n, Xs[m], n, 1, opts, "L",
                                           st.cuda_stream, raise_on_error=False)
                got.append((rc, rep["steps"]))
        return got

    t0 = time.perf_counter()
    with ThreadPoolExecutor(nstream) as pool:
        got = [v for chain in pool.map(mixed_chain, range(nstream)) for v in chain]
    torch.cuda.synchronize()
    res["mixed_solve_s"] = time.perf_counter() - t0
    steps = [st_ for _, st_ in got]
    res["mixed_steps"] = [min(steps), max(steps)]
    res["mixed_return_codes"] = sorted({rc for rc, _ in got})
    fl_fwd = nmat * (n ** 3 / 3 + 2 * n * n)
    out = {"metric": "GP likelihood logdet+quad forward and adjoint (s)", "config": {
        "workload": "C5: 64 RBF matrices n=2048, lengthscale 0.2, noise 1e-2", "nmat": nmat, "n": n},
        "unit": "s", "higher_is_better": False, "data": "synthetic", "results": res,
        "forward_tflops": fl_fwd / res["forward_s"] / 1e12, "backward_tflops_equiv": fl_fwd / res["backward_s"] / 1e12,
        "timing": "wall clock around all 64 problems on 8 streams, after a warm-up pass"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(CONFIGS) + ["c3-sweep", "c4", "c5"], default=DEFAULT_CONFIG)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="the default configuration's line without the "
                    "kappa sweep and the C1 / C4 / C5 keys")
    ap.add_argument("--mixed-precision", default="bf16x3", choices=sorted(SPLIT_PRODUCTS),
                    help="split of the mixed factorisation's tensor-core products (bf16x3: two BF16 parts, "
                    "three products; bf16x6: three parts, six products)")
    ap.add_argument("--n", type=int, default=0, help="override the order n (profiling a smaller case)")
    ap.add_argument("--arms", choices=["both", "fp64", "mixed"], default="both",
                    help="time one arm only (profiling); that arm is then the line's headline, without extras")
    ap.add_argument("--reserve-sms", type=int, default=0, help="SMs left to the panel factorisation while the "
                    "look-ahead update runs (0: the library's default)")
    ap.add_argument("--panel", type=int, default=0, help="outer panel width of the mixed factorisation "
                    "(0: the library default)")
    args = ap.parse_args()
    if args.impl == "reference":
        # CPU only: under torchrun rank 0 alone runs it, the other ranks exit without work
        run_reference(args, int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")))
        return
    ws, rank, local = dist_setup()
    if args.config in ("c3-sweep", "c4", "c5"):
        import torch
        torch.cuda.set_device(local)
        if args.config == "c4":
            out = run_c4(args, ws, rank)
        elif args.config == "c5":
            out = run_c5(args)
        else:
            out = {"metric": METRIC, "config": {"workload": "n=32768 sweep: kappa in {1e2,1e4,1e6}, 1 and 64 RHS"},
                   **c3_sweep(args, args.n or CONFIGS["c3"]["n"], None)}
        if rank == 0:
            print(json.dumps(out), flush=True)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
