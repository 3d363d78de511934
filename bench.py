"""Benchmark of the GB300 dense Cholesky (LLT) path.

Default workload: n = 16384, 64 right-hand sides, A = Q diag(lambda) Q^T with Q a product of 8
Householder reflectors and lambda log-spaced over [1e-6, 1] (kappa = 1e6), B ~ N(0,1); FP64
factor + solve (the large plain-FP64 LLT configuration).  One step = one factor + solve of that
system.  Inputs are synthetic and seeded; the 2.1 GB matrix is larger than the 129 MB L2, so
no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

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
    "c2": dict(workload="LLT factor+solve FP64, n=16384, 64 RHS, Householder spectrum kappa=1e6",
               n=16384, nrhs=64, kappa=1e6),
    "c1": dict(workload="LLT factor+solve FP64, n=1024, 16 RHS, A=G G^T/n+I", n=1024, nrhs=16, kappa=None),
}
CPU_SAMPLE_N = 8192


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
    out = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": total / len(ts) * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": cfg["workload"], "n": cfg["n"], "nrhs": k, "kappa": cfg["kappa"]},
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": O.num_threads(), "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ---- GPU arm ------------------------------------------------------------------------------------

def run_ours(args, ws, rank, local):
    import torch
    import gbllt as G

    torch.cuda.set_device(local)
    cfg = CONFIGS[args.config]
    n, k = cfg["n"], cfg["nrhs"]
    A0, B0 = make_inputs_gpu(cfg, seed=1 + rank)
    A = torch.empty_like(A0)
    B = torch.empty_like(B0)
    info = torch.zeros(1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream

    def step():
        with torch.cuda.stream(stream):
            A.copy_(A0)
            B.copy_(B0)
            G.potrf_dev(A, n, n, info, "L", sp)
            G.potrs_dev(A, n, n, B, k, n, "L", sp)

    for _ in range(max(args.warmup, 0)):
        step()
    stream.synchronize()
    peak = fp64_peak_tflops()

    clocks = ClockSampler(local)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    G.profile_enable(True)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    ck = clocks.stop()
    prof = G.profile_read()
    G.profile_enable(False)
    ms = e0.elapsed_time(e1)
    ms_max = max_over_ranks(ws, ms)
    assert int(info.item()) == 0, f"factorisation failed, info={int(info.item())}"

    # backward error of the last step's solution (torch FP64 GEMM as a plain reference computation)
    X = B.T  # n x k
    R = A0 @ X - B0.T
    be = float(torch.linalg.norm(R) / (torch.linalg.norm(A0) * torch.linalg.norm(X)))

    flops = llt_flops(n, k)
    value = ws * flops * args.steps / (ms_max * 1e-3) / 1e12
    launches = sum(v["launches"] for v in prof.values())
    top = max(prof.items(), key=lambda kv: kv[1]["ms"])
    top_name, top_s = top
    achieved = top_s["flops"] / (top_s["ms"] * 1e-3) / 1e12
    per_launch_flops = top_s["flops"] / top_s["launches"]
    total_kernel_ms = sum(v["ms"] for v in prof.values())

    # end to end through the host-pointer C ABI (pinned host buffers; copies inside the timed call)
    e2e = None
    if rank == 0 or ws > 1:
        hA0 = A0.cpu().pin_memory()
        hB0 = B0.cpu().pin_memory()
        hA = torch.empty_like(hA0).pin_memory()
        hB = torch.empty_like(hB0).pin_memory()
        a_np, b_np = hA.numpy(), hB.numpy()
        import ctypes
        e2e_steps = max(1, min(args.steps, 3))
        tt = []
        for i in range(1 + e2e_steps):
            hA.copy_(hA0)
            hB.copy_(hB0)
            inf = ctypes.c_int64(0)
            t0 = time.perf_counter()
            rc = G.lib().gbllt_dposv(G.COL_MAJOR, b"L", n, k, a_np.ctypes.data, n, b_np.ctypes.data, n,
                                     ctypes.byref(inf))
            dt = time.perf_counter() - t0
            G.check("gbllt_dposv", rc)
            assert inf.value == 0
            if i > 0:
                tt.append(dt)
        e2e_s = max_over_ranks(ws, sum(tt) / len(tt))
        e2e = {"value": ws * flops / e2e_s / 1e12, "unit": "TFLOP/s", "seconds_per_step": e2e_s,
               "h2d_bytes_per_step": int(n * n * 8 + n * k * 8), "d2h_bytes_per_step": int(n * n * 8 + n * k * 8),
               "path": "gbllt_dposv (host pointers, pinned), wall clock"}

    if rank != 0:
        return
    cpu = None if args.no_cpu_baseline or ws > 1 else cpu_sample()
    out = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": cfg["workload"], "n": n, "nrhs": k, "kappa": cfg["kappa"],
                   "path": "plain FP64 (gbllt_dpotrf_dev + gbllt_dpotrs_dev)",
                   "l2": "inputs larger than L2 (matrix 2.1 GB vs 129 MB L2); each step restores A and B "
                         "from a pristine device copy (included in the timed step)"},
        "seconds_per_solve": ms_max / args.steps / 1e3,
        "backward_error": be,
        "roofline": {"kernel": top_name, "bound": "tensor", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                     "per_launch_flops": per_launch_flops, "launches": top_s["launches"],
                     "kernel_share_of_device_time": top_s["ms"] / total_kernel_ms,
                     "peak_source": "measured in this run: cuBLAS DGEMM 4096^3 (FP64 peak; not in MEASURED_PEAKS.json)"},
        "kernels": {kn: {"launches": v["launches"], "ms": v["ms"],
                         "tflops": v["flops"] / max(v["ms"], 1e-9) / 1e9} for kn, v in prof.items()},
        "gpu_launches": launches,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "clocks": ck,
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(CONFIGS), default="c2")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        # CPU only: under torchrun rank 0 alone runs it, the other ranks exit without work
        run_reference(args, int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")))
        return
    ws, rank, local = dist_setup()
    run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
