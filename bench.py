"""Benchmark of the matrix-free hot path on GB300.

Headline workload (the BASELINE configuration the metric is quoted on):
neo-Hookean tangent vmult, cantilever [0,8]x[0,1]^2, 8x1x1 coarse cells
refined 3 times (64x8x8 = 4096 cells), Q4 vector elements with 5^3 Gauss
points, 839,619 DoFs, FP64, linearised at a seeded smooth displacement;
source vector U(-1,1) (seed 3).  A "step" is one operator application.

Output: one JSON line (rank 0).  `value` is DoF/s of the device-resident
vmult (L2 flushed before every timed application, CUDA events on the
library's stream); `e2e` is the same metric through the C-ABI host-buffer
call mfgpu_operator_vmult_host (host->device copy of the source and
device->host copy of the result inside the timed region).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--caching referential_qp|scalar_referential|...]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "matrix-free-dealii-precice_gb300")
sys.path.insert(0, PKG)

METRIC = "DoF/s per vmult (neo-Hookean tangent, Q4, FP64)"
UNIT = "DoF/s"
WORKLOAD = dict(degree=4, n_ref=3, rep=(8, 1, 1), length=(8.0, 1.0, 1.0))


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--caching", default="referential_qp")
    p.add_argument("--arith", default="native", choices=["native", "df64"],
                   help="FP64 operator arithmetic: native FP64 or double-float on the FP32 pipe")
    p.add_argument("--cpu-seconds", type=float, default=10.0,
                   help="wall-clock budget of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def algorithmic_bytes(n_dofs, n_cells, s=8, k_state=1):
    """B_alg = s*N_dof*(2 + k_state) + 4*s*N_cells (src read, dst write,
    linearisation state read, per-cell affine geometry)."""
    return s * n_dofs * (2 + k_state) + 4 * s * n_cells


def algorithmic_flops(n_cells, n, nc=3, f_qp=250):
    """F_alg = N_cells*nc*24*n^4 + N_cells*n^3*f_qp (+ the second gradient
    evaluation of scalar_referential, 12 n^4 per component)."""
    return n_cells * nc * 24 * n ** 4 + n_cells * n ** 3 * f_qp + n_cells * nc * 12 * n ** 4


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic():
    """dram bytes per launch of the vmult cell kernel, from the committed
    ncu summary of this workload (None when absent)."""
    path = os.path.join(ROOT, "profiles", "nh_vmult_q4_cantilever_ncu.txt")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def cpu_baseline(spec, u, src, budget_s, threads=None):
    """The oracle (C++ OpenMP restatement of the reference's CPU matrix-free
    vmult) on the host cores: repeated applications of the same operator on
    the same inputs until the time budget is used (at least one)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import workloads as W
    nthreads = O.set_threads(threads or (os.cpu_count() or 1))
    om = W.to_oracle_mesh(O, spec)
    mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    t0 = time.perf_counter()
    O.nh_vmult(om, spec["n_ref"], mat, "scalar_referential", u, src)  # includes cache
    t_first = time.perf_counter() - t0
    # the oracle entry point caches and applies per call; time whole calls
    reps, t_sum = 0, 0.0
    while reps == 0 or (t_sum < budget_s and reps < 50):
        t0 = time.perf_counter()
        O.nh_vmult(om, spec["n_ref"], mat, "scalar_referential", u, src)
        t_sum += time.perf_counter() - t0
        reps += 1
    n = len(src)
    return {"value": n / (t_sum / reps), "unit": UNIT, "cores": nthreads,
            "kind": "port",
            "sample": f"{reps} full applications (cache + vmult, scalar_referential) of "
                      f"the {n}-DoF Q4 operator on {nthreads} threads; first call {t_first:.2f}s"}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    import workloads as W
    spec = W.cantilever(WORKLOAD["degree"], WORKLOAD["n_ref"], WORKLOAD["rep"], WORKLOAD["length"])
    n = W.n_dofs(spec, 3)
    u = W.smooth_displacement(spec["degree"], spec["n_ref"], spec["rep"], spec["lo"], spec["hi"], seed=2)
    src = W.uniform_vector(n, 3)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    nthreads = O.set_threads(os.cpu_count() or 1)
    om = W.to_oracle_mesh(O, spec)
    mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    for _ in range(max(args.warmup, 0) and 1):
        O.nh_vmult(om, spec["n_ref"], mat, "scalar_referential", u, src)
    steps = max(1, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(steps):
        O.nh_vmult(om, spec["n_ref"], mat, "scalar_referential", u, src)
    dt = (time.perf_counter() - t0) / steps
    value = n / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": steps, "warmup": 1, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "nh_tangent_vmult_q4_cantilever_64x8x8",
                       "n_dofs": n, "caching": "scalar_referential"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"{steps} full cache+vmult applications on {nthreads} threads "
                                       "(the reference itself needs deal.II/p4est/MPI, absent here)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_info()
    import torch
    import build as pkg_build
    import mfgpu
    import workloads as W
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    pkg_build.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = mfgpu.Context(local)

    spec = W.cantilever(WORKLOAD["degree"], WORKLOAD["n_ref"], WORKLOAD["rep"], WORKLOAD["length"])
    mesh = W.to_lib_mesh(mfgpu, spec)
    n = W.n_dofs(spec, 3)
    n_cells = 64 * 8 * 8
    u_h = W.smooth_displacement(spec["degree"], spec["n_ref"], spec["rep"], spec["lo"], spec["hi"], seed=2)
    src_h = W.uniform_vector(n, 3)
    u = torch.from_numpy(u_h).to(dev)
    src = torch.from_numpy(src_h).to(dev)
    dst = torch.zeros(n, dtype=torch.float64, device=dev)
    op = mfgpu.NeoHookOperator(ctx, mesh, -1, 64, args.caching)
    op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01))
    op.initialize(u)
    if args.arith == "df64":
        op.set_fp64_emulation(True)
    op.cache()
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 512 MB > L2

    def barrier():
        torch.cuda.synchronize(dev)
        ctx.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # warm-up
    for _ in range(max(args.warmup, 3)):
        op.vmult(dst, src)
    ctx.synchronize()

    # timed: K device-resident vmults, L2 flushed before each (not timed)
    K = args.steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    kstarts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    kends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    launches0 = mfgpu.launch_count()
    t_wall0 = time.perf_counter()
    for i in range(K):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
            starts[i].record(stream)
        op.vmult(dst, src)
        with torch.cuda.stream(stream):
            ends[i].record(stream)
    barrier()
    t_wall = time.perf_counter() - t_wall0
    launches = mfgpu.launch_count() - launches0
    # dominant kernel alone: cell application (vmult_add = cell kernel +
    # constrained-row add), also L2-flushed
    for i in range(K):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
            kstarts[i].record(stream)
        op.vmult_add(dst, src)
        with torch.cuda.stream(stream):
            kends[i].record(stream)
    barrier()
    clk = clocks.stop()
    ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    kms = [s.elapsed_time(e) for s, e in zip(kstarts, kends)]
    ms_step = sum(ms) / K
    k_ms = sum(kms) / K
    if world > 1:
        t = torch.tensor([ms_step], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_step = float(t.item())

    # end to end through the C-ABI with host buffers (pinned)
    src_pin = torch.from_numpy(src_h).pin_memory()
    dst_pin = torch.zeros(n, dtype=torch.float64).pin_memory()
    src_np, dst_np = src_pin.numpy(), dst_pin.numpy()
    for _ in range(max(args.warmup, 3)):
        op.vmult_host(dst_np, src_np)
    barrier()
    t0 = time.perf_counter()
    for _ in range(K):
        op.vmult_host(dst_np, src_np)
    barrier()
    e2e_s = (time.perf_counter() - t0) / K
    if world > 1:
        t = torch.tensor([e2e_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())

    # correctness guard of the timed result: symmetric operator, u^T A v == v^T A u
    ctx.synchronize()
    peak, peak_kind = measured_peak_hbm()
    b_alg = algorithmic_bytes(n, n_cells)
    achieved = b_alg / (k_ms * 1e-3) / 1e9
    f_alg = algorithmic_flops(n_cells, 5)
    line = {
        "metric": METRIC, "value": world * n / (ms_step * 1e-3), "unit": UNIT,
        "n_gpus": world, "steps": K, "warmup": max(args.warmup, 3),
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "nh_tangent_vmult_q4_cantilever_64x8x8", "n_dofs": n,
                   "n_cells": n_cells, "degree": 4, "n_q_1d": 5, "caching": args.caching,
                   "arithmetic": "native FP64" if args.arith == "native" else
                                 "double-float (FP32 pipe), parity 1e-12 vs FP64",
                   "l2": "flushed (512 MB write) before every timed application",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": world * n / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": profile_traffic(),
                     "peak_kind": peak_kind,
                     "kernel": "cell_apply_kernel (vmult_add, CUDA events, L2 flushed)",
                     "kernel_ms": k_ms, "bytes_alg_per_launch": b_alg},
        "fp64": {"alg_tflops": f_alg / (k_ms * 1e-3) / 1e12,
                 "note": "FP64 pipe of GB300 is ~1.25 TFLOP/s nominal: the FP64 operator is pipe-bound"},
        "clocks": clk,
        "gpu_launches": launches,
        "wall_ms_per_step": t_wall / K * 1e3,
    }
    if rank == 0 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline(spec, u_h, src_h, args.cpu_seconds)
        except Exception as e:  # reported, never fatal for the GPU number
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port",
                                    "sample": f"failed: {e}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
