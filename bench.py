"""Benchmark of the matrix-free hot path on GB300.

Headline workload: neo-Hookean tangent vmult, cantilever [0,8]x[0,1]^2,
8x1x1 coarse cells refined 3 times (64x8x8 = 4096 cells), Q4 vector
elements with 5^3 Gauss points, 839,619 DoFs, native FP64 arithmetic,
linearised at a seeded smooth displacement; source vector U(-1,1) (seed 3).
A "step" is one operator application.

Output: one JSON line (rank 0).  `value` is DoF/s of the device-resident
vmult (L2 flushed before every timed application, CUDA events on the
library's stream); `e2e` is the same metric through the C-ABI host-buffer
call mfgpu_operator_vmult_host (host->device copy of the source and
device->host copy of the result inside the timed region).  The key `df64`
reports the same operator in double-float arithmetic (FP32 pipe), with its
own roofline and e2e figures.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--arith native|df64] [--caching referential_qp|...]
    python bench.py --kernel-case NAME --steps K   # one operator, for ncu
    python bench.py --solver-case NAME             # one solver workload, for ncu launch lists
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
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--caching", default="referential_qp")
    p.add_argument("--arith", default="native", choices=["native", "df64"],
                   help="arithmetic of the headline FP64 operator: native FP64 (the reference's) or "
                        "double-float on the FP32 pipe")
    p.add_argument("--kernel-case", default=None, choices=sorted(KERNEL_CASES),
                   help="apply one operator `--steps` times on its workload and exit (the cases the "
                        "ncu summaries under profiles/ were taken on)")
    p.add_argument("--solver-case", default=None, choices=sorted(SOLVER_CASES),
                   help="run one solver workload twice, the second between cudaProfilerStart and "
                        "cudaProfilerStop (ncu --profile-from-start off), and exit")
    p.add_argument("--cpu-seconds", type=float, default=10.0,
                   help="wall-clock budget of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the secondary measurements (solves, degree sweep)")
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device=None):
    """Max of a per-rank time over all replicas (identity on one rank).
    Every rank gets the max, whichever process-group backend is initialised."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, seconds_max, world):
    """Whole-job throughput of `world` independent replicas that each
    processed `units_per_rank` units, timed by the slowest replica."""
    return world * units_per_rank / seconds_max


def algorithmic_bytes(n_dofs, n_cells, s=8, k_state=1):
    """B_alg = s*N_dof*(2 + k_state) + 4*s*N_cells (src read, dst write,
    linearisation state read, per-cell affine geometry)."""
    return s * n_dofs * (2 + k_state) + 4 * s * n_cells


def algorithmic_flops(n_cells, n, nc=3, f_qp=250):
    """F_alg = N_cells*nc*24*n^4 + N_cells*n^3*f_qp (+ the second gradient
    evaluation of scalar_referential, 12 n^4 per component)."""
    return n_cells * nc * 24 * n ** 4 + n_cells * n ** 3 * f_qp + n_cells * nc * 12 * n ** 4


class ClockSampler:
    """nvidia-smi clocks / throttle reasons, sampled every 100 ms from
    start() to stop(); stop() keeps the samples read inside mark()ed windows
    (the timed regions), or all of them when no window holds one."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []
        self.windows = []

    def start(self, settle_s=1.0):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return
        # nvidia-smi takes a moment to print its first sample
        t0 = time.perf_counter()
        while not self.lines and time.perf_counter() - t0 < settle_s:
            time.sleep(0.02)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def mark(self, t0, t1):
        self.windows.append((t0, t1))

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"],
                    "samples": 0}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        inside = [ln for t, ln in self.lines if any(a <= t <= b + 0.1 for a, b in self.windows)]
        scope = "timed regions" if inside else "whole run"
        rows = inside or [ln for _, ln in self.lines]
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in rows:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "reasons": sorted(reasons), "samples": len(sm), "scope": scope,
                "timed_window_s": sum(b - a for a, b in self.windows)}


class NvmlSampler:
    """SM clock, power and clock-event reasons read through NVML (ctypes on
    libnvidia-ml.so.1, read-only queries) every 2 ms from start() to stop(),
    so that even a timed region of a few milliseconds holds samples;
    stop() keeps the samples inside the mark()ed windows.  Falls back to
    nvidia-smi polling (ClockSampler) when NVML cannot be loaded."""

    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
               0x4: "sw_power_cap"}

    def __init__(self, device, torch_device=None):
        import ctypes
        self.C = ctypes
        self.samples = []
        self.windows = []
        self.running = False
        self.nv = ctypes.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        uuid = None
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(torch_device).uuid)
        except Exception:
            uuid = None
        ok = False
        if uuid:
            key = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
            ok = self.nv.nvmlDeviceGetHandleByUUID(key.encode(), ctypes.byref(self.h)) == 0
        if not ok and self.nv.nvmlDeviceGetHandleByIndex_v2(device, ctypes.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        mx = ctypes.c_uint()
        self.max_mhz = None
        if self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(mx)) == 0:
            self.max_mhz = float(mx.value)
        self.get_reasons = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nv.nvmlDeviceGetCurrentClocksThrottleReasons

    def _loop(self):
        C = self.C
        mhz, mw, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        while self.running:
            t = time.perf_counter()
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) == 0:
                p = mw.value if self.nv.nvmlDeviceGetPowerUsage(self.h, C.byref(mw)) == 0 else 0
                r = rs.value if self.get_reasons(self.h, C.byref(rs)) == 0 else 0
                self.samples.append((t, float(mhz.value), p / 1000.0, r))
            time.sleep(0.002)

    def start(self):
        self.running = True
        self.t = threading.Thread(target=self._loop, daemon=True)
        self.t.start()

    def mark(self, t0, t1):
        self.windows.append((t0, t1))

    def stop(self):
        self.running = False
        self.t.join(timeout=2)
        inside = [x for x in self.samples if any(a <= x[0] <= b for a, b in self.windows)]
        rows = inside or self.samples
        reasons = sorted({nm for _, _, _, r in rows for bit, nm in self.REASONS.items() if r & bit})
        sm = [x[1] for x in rows]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.max_mhz,
                "sm_mhz_min": min(sm) if sm else None,
                "power_w_max": max(x[2] for x in rows) if rows else None,
                "reasons": reasons, "samples": len(sm),
                "scope": "timed regions" if inside else "whole run", "source": "NVML, every 2 ms",
                "timed_window_s": sum(b - a for a, b in self.windows)}


def clock_sampler(device, torch_device=None):
    try:
        return NvmlSampler(device, torch_device)
    except (OSError, AttributeError):
        return ClockSampler(device)


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


HEADLINE_PROFILE = {"native": "nh_vmult_q4_cantilever_native_fp64_ncu.txt",
                    "df64": "nh_vmult_q4_cantilever_df64_ncu.txt"}


def profile_summary(name):
    """Figures of a committed ncu summary under profiles/ (None when absent):
    pipe and DRAM fractions, and the DRAM bytes per launch."""
    path = os.path.join(ROOT, "profiles", name)
    out = {}
    try:
        for line in open(path):
            for key in ("pipe_fma_pct", "issue_active_pct", "pipe_fp64_pct", "dram_throughput_pct_of_peak"):
                if line.startswith(key + ":"):
                    out[key[:-4] + "_frac"] = float(line.split(":", 1)[1].split()[0]) / 100.0
            if line.startswith("traffic_bytes_per_launch:"):
                out["traffic_bytes_per_launch"] = float(line.split(":", 1)[1])
            if line.startswith("duration"):
                out["ncu_duration"] = line.split(":", 1)[1].strip()
    except OSError:
        return None
    return out or None


def measured_fp64_peak(torch, dev):
    """FP64 throughput of cuBLAS DGEMM (4096^3, best of 3) on this GPU, in
    TFLOP/s: the measured FP64 roof of the native-FP64 operator."""
    n = 4096
    a = torch.rand(n, n, dtype=torch.float64, device=dev)
    b = torch.rand(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize(dev)
    best = float("inf")
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize(dev)
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    del a, b
    return 2 * n ** 3 / best / 1e12


# device solutions kept by the secondary measurements for the oracle's check
SOLUTIONS = {}
CPU_FLAGS = "g++ -O3 -fopenmp (portable: no -march/-mcpu=native)"

CPU_CACHINGS = ("scalar_referential", "tensor2", "tensor4", "tensor4_ns")
# the throughput form (oracle/oracle_fast.hpp): cell batches across SIMD
# lanes, compile-time degree, even-odd collocation sweeps, as deal.II runs
# the reference's vmult
CPU_FAST = tuple((c, w) for c in CPU_CACHINGS for w in (2, 4, 8))


def oracle_vmult_rates(spec, u, src, budget_s, threads=None):
    """The reference's CPU matrix-free vmult restated in C++/OpenMP, on the
    host cores: each caching variant of the reference in the oracle's plain
    form, and the variants the throughput form covers at each lane count;
    every one cached once and then applied repeatedly, the applications timed
    without the cache (as the GPU vmult is).  The throughput form's result is
    checked against the plain form's before it is timed.  Returns
    ({variant: DoF/s}, threads, applications per variant, {variant:
    timer(reps, warmup) -> (dst, seconds)})."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import workloads as W
    O.build()
    nthreads = O.set_threads(threads or (os.cpu_count() or 1))
    om = W.to_oracle_mesh(O, spec)
    mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    n = len(src)
    level = spec["n_ref"]
    plain = {c: (lambda reps, warmup=1, c=c: O.nh_vmult_timed(om, level, mat, c, u, src, reps, warmup))
             for c in CPU_CACHINGS}
    fast = {f"{c}/simd{w}": (lambda reps, warmup=1, c=c, w=w:
                             O.nh_vmult_fast_timed(om, level, mat, c, u, src, reps, lanes=w, warmup=warmup))
            for c, w in CPU_FAST}
    # one timed application per variant sizes the rest of the budget
    first, ref = {}, {}
    for name, fn in plain.items():
        ref[name], first[name] = fn(1)
    skipped = {}
    for name, fn in list(fast.items()):
        try:
            out, first[name] = fn(1)
            base = ref[name.split("/")[0]]
            err = np.linalg.norm(out - base) / np.linalg.norm(base)
            if not err < 1e-12:
                raise RuntimeError(f"differs from the oracle: {err:.2e}")
        except Exception as e:  # a variant that fails its check is not timed
            skipped[name] = str(e)
            fast.pop(name)
            first.pop(name, None)
    reps = max(1, min(20, int(budget_s / max(sum(first.values()), 1e-9))))
    rates = {}
    for name, fn in {**plain, **fast}.items():
        _, secs = fn(reps)
        rates[name] = n / (secs / reps)
    if skipped:
        print(f"CPU variants not timed: {skipped}", file=sys.stderr, flush=True)
    return rates, nthreads, reps, {**plain, **fast}


def cpu_baseline(spec, u, src, budget_s, threads=None):
    rates, nthreads, reps, _ = oracle_vmult_rates(spec, u, src, budget_s, threads)
    best = max(rates, key=rates.get)
    return {"value": rates[best], "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{reps} applications per variant of the {len(src)}-DoF Q4 operator, cached once, "
                      f"vmult timed alone, on {nthreads} threads, built {CPU_FLAGS}; variants: each "
                      f"caching of the reference "
                      f"in plain loops, and the cell-batched SIMD form (/simdW: W cells per batch); the "
                      f"fastest ({best}) is reported; all: " +
                      ", ".join(f"{c} {v / 1e6:.1f}" for c, v in rates.items()) + " MDoF/s"}


def cpu_heat_step():
    """The heat workload beside the GPU's (unit cube, 16^3 cells, Q2, 35,937
    DoFs) on the host cores: one backward-Euler step by GMG-CG to 1e-10 (FP32
    levels, as on the GPU), setup included, with every operator in the
    cell-batched form; and 100 FP64 vmults on U(-1,1), the fastest of the
    plain loops and the cell-batched form at 2, 4 and 8 lanes."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import workloads as W
    spec = W.unit_cube_heat(2, 4)
    om = W.to_oracle_mesh(O, spec)
    c, w, a = W.gaussian_source(0)
    p = O.HeatParams()
    p.mesh = om
    p.dt, p.n_steps, p.tol_rel, p.precond, p.mg_float, p.fast = 0.1, 1, 1e-10, 2, 1, 1
    p.n_gauss = 8
    for i in range(8):
        for d in range(3):
            p.g_center[i][d] = c[i, d]
        p.g_width[i] = w[i]
        p.g_amp[i] = a[i]
    r = O.heat_run(p)
    n = W.n_dofs(spec, 1)
    x = W.uniform_vector(n, 1)
    ref, secs = O.heat_vmult_timed(om, spec["n_ref"], 0.1, x, 100)
    rates = {"plain": 100 * n / secs}
    for w in (2, 4, 8):
        out, secs = O.heat_vmult_fast_timed(om, spec["n_ref"], 0.1, x, 100, lanes=w)
        if not np.linalg.norm(out - ref) <= 1e-12 * np.linalg.norm(ref):
            raise RuntimeError(f"throughput heat form ({w} lanes) differs from the oracle")
        rates[f"simd{w}"] = 100 * n / secs
    best = max(rates, key=rates.get)
    return {"workload": "heat unit cube 16^3 Q2, 35,937 DoFs",
            "step_s": r.seconds, "step_form": "cell-batched", "cg_its": int(r.cg_its[0]),
            "vmult_100_s": 100 * n / rates[best], "vmult_dofs_per_s": rates[best], "vmult_form": best,
            "vmult_all_dofs_per_s": rates}


def cpu_mixed_solve():
    """The config-2 system on the host cores (128x16x16-cell Q3 cantilever,
    2,773,155 DoFs; first Newton system from rest, traction (0,-100,0) on
    x = 8) set up and solved to a 1e-8 relative residual by FP64 CG with an
    FP32 V-cycle and with an all-FP64 V-cycle, every operator, level operator
    and diagonal in the cell-batched form (tensor2 caching, the fastest CPU
    variant of the vmult)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import workloads as W
    spec = W.cantilever(3, 4)
    out = {"workload": "cantilever 128x16x16 cells Q3, 2,773,155 DoFs, first Newton system",
           "tolerance": 1e-8, "form": "cell-batched, tensor2"}
    for name, mg_float in (("mixed_fp32_vcycle", 1), ("fp64_vcycle", 0)):
        p = O.SolidParams()
        p.mesh = W.to_oracle_mesh(O, spec)
        p.mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
        p.caching = O.CACHING["tensor2"]
        p.precond, p.dt, p.n_steps, p.max_newton, p.max_it_mult = 2, 0.01, 1, 10, 1
        p.relaxation, p.tol_lin = 0.65, 1e-8
        p.traction_id = W.TRACTION_ID
        p.traction[:] = [0.0, -100.0, 0.0]
        p.cheb_degree, p.cheb_range, p.cheb_eig_its, p.coarse_accurate = 5, 20.0, 30, 1
        p.mg_float, p.fast = mg_float, 1
        its, setup_s, solve_s, _ = O.solid_first_solve(p, 1e-8)
        out[name] = {"cg_iterations": its, "setup_s": setup_s, "solve_s": solve_s,
                     "setup_plus_solve_s": setup_s + solve_s}
    # the device solutions (FP32 and FP64 V-cycles, to 1e-8) against the
    # oracle's FP64-everywhere solve to 1e-12
    dev_sol = SOLUTIONS.get("time_to_solve_1e-8")
    if dev_sol:
        p.mg_float = 0
        _, _, _, du_ref = O.solid_first_solve(p, 1e-12)
        out["device_error_vs_oracle_fp64"] = {
            name: {"l2_rel": float(np.linalg.norm(du - du_ref) / np.linalg.norm(du_ref)),
                   "max_rel": float(np.max(np.abs(du - du_ref)) / np.max(np.abs(du_ref)))}
            for name, du in dev_sol.items()}
        out["device_error_vs_oracle_fp64"]["oracle"] = (
            "FP64 CG + FP64 V-cycle, cell-batched form, relative residual 1e-12")
    return out


def cpu_solid_first_step():
    """The first Newmark step of the 64x8x8-cell Q4 cantilever (839,619
    DoFs, traction (0,-100,0) on x = 8, Newton to 1e-9 / 1e-6, GMG-CG to
    1e-6 with an FP32 V-cycle) on the host cores, every operator in the
    cell-batched form (tensor2 caching)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import workloads as W
    spec = W.cantilever(4, 3)
    p = O.SolidParams()
    p.mesh = W.to_oracle_mesh(O, spec)
    p.mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    p.caching = O.CACHING["tensor2"]
    p.precond = 2
    p.relaxation, p.tol_lin, p.max_it_mult, p.max_newton = 0.65, 1e-6, 1, 10
    p.tol_f, p.tol_f_abs, p.tol_u, p.tol_u_abs = 1e-9, 0.0, 1e-6, 0.0
    p.dt, p.n_steps = 0.01, 1
    p.traction_id = W.TRACTION_ID
    p.traction[:] = [0.0, -100.0, 0.0]
    p.watch[:] = [8.0, 0.5, 0.5]
    p.cheb_degree, p.cheb_range, p.cheb_eig_its, p.coarse_accurate = 5, 20.0, 30, 1
    p.mg_float, p.fast = 1, 1
    r = O.solid_run(p)
    return {"workload": "cantilever 64x8x8 cells Q4, 839,619 DoFs, first Newmark step",
            "form": "cell-batched, tensor2", "newton_its": int(r.newton_its[0]),
            "cg_iterations": int(r.total_cg), "linear_solves": int(r.n_solves), "seconds": r.seconds,
            "watch_displacement": list(r.watch_disp[0][:3])}


def cpu_heat_sweep(reps=3):
    """The degree sweep's heat operator (unit cube, 64^3 cells, Q1..Q6, FP64)
    on the host cores in the cell-batched form, the fastest of 2, 4 and 8
    lanes per degree; each degree's form is first checked against the
    oracle's plain loops on a 2x1x1-cell mesh.  Returns {degree: DoF/s}."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import workloads as W
    out = {}
    for deg in range(1, 7):
        small = W.unit_cube_heat(deg, 0, rep=(2, 1, 1))
        om = W.to_oracle_mesh(O, small)
        x = W.uniform_vector(W.n_dofs(small, 1), 5)
        ref = O.heat_vmult(om, 0, 0.1, x)
        spec = W.unit_cube_heat(deg, 6)
        n = W.n_dofs(spec, 1)
        big = W.to_oracle_mesh(O, spec)
        src = W.uniform_vector(n, 1)
        best = 0.0
        for w in (2, 4, 8):
            got, _ = O.heat_vmult_fast_timed(om, 0, 0.1, x, 1, lanes=w)
            if not np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref):
                raise RuntimeError(f"throughput heat form, degree {deg}, {w} lanes, differs from the oracle")
            _, secs = O.heat_vmult_fast_timed(big, spec["n_ref"], 0.1, src, reps, lanes=w)
            best = max(best, n * reps / secs)
        out[str(deg)] = best
    return out


def _timed_vmults(torch, op, dst, src, flush, stream, reps):
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(reps)]
    for i in range(reps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
            ev[i][0].record(stream)
        op.vmult(dst, src)
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / reps * 1e-3


def extra_mixed_precision_solve(torch, mfgpu, W, ctx, dev):
    """128x16x16-cell Q3 cantilever (2.77M DoFs): the first Newton linear
    system (linearised at rest, traction (0,-100,0) on x = 8) solved to a
    1e-8 relative residual by FP64 CG with an FP32 V-cycle (FP64 coarse
    solve) and with an all-FP64 V-cycle; error against an FP64-everywhere
    solve to 1e-12."""
    spec = W.cantilever(3, 4)
    n = W.n_dofs(spec, 3)
    zero = torch.zeros(n, dtype=torch.float64, device=dev)
    rhs = torch.zeros(n, dtype=torch.float64, device=dev)

    def params(mgp, c64, tol, emul=False):
        p = mfgpu.SolidParams()
        p.mesh = W.to_lib_mesh(mfgpu, spec)
        p.material = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
        p.caching = b"referential_qp"
        p.solver = mfgpu.solver_params("gmg", tol=tol, mg_precision=mgp, coarse_fp64=c64,
                                       fp64_emulation=emul)
        p.dt, p.n_steps, p.max_newton = 0.01, 1, 10
        p.traction_id = W.TRACTION_ID
        p.traction[:] = [0.0, -100.0, 0.0]
        return p

    out_solutions = SOLUTIONS.setdefault("time_to_solve_1e-8", {})
    ref_solver = mfgpu.Solid(ctx, params(64, False, 1e-12))
    ref_solver.residual(zero, zero, rhs)
    du_ref = torch.zeros_like(rhs)
    ref_solver.linear_solve(zero, rhs, du_ref)
    ref_solver.close()
    out = {"workload": "cantilever 128x16x16 cells Q3, 2,773,155 DoFs, first Newton system",
           "tolerance": 1e-8}
    for name, mgp, c64, emul in (("mixed_fp32_vcycle", 32, True, False),
                                 ("mixed_fp32_vcycle_df64", 32, True, True),
                                 ("fp64_vcycle", 64, False, False),
                                 ("fp64_vcycle_df64", 64, False, True)):
        s = mfgpu.Solid(ctx, params(mgp, c64, 1e-8, emul))
        du = torch.zeros_like(rhs)
        s.linear_solve(zero, rhs, du)  # warm-up (setup + solve)
        du.zero_()
        t0 = time.perf_counter()
        its, secs = s.linear_solve(zero, rhs, du)
        total = time.perf_counter() - t0
        err = (du - du_ref)
        out[name] = {"cg_iterations": its, "solve_s": secs, "setup_plus_solve_s": total,
                     "l2_rel_error_vs_device_fp64_1e-12": float(err.norm() / du_ref.norm()),
                     "max_rel_error_vs_device_fp64_1e-12": float(err.abs().max() / du_ref.abs().max())}
        out_solutions[name] = du.cpu().numpy()
        s.close()
    out["speedup_mixed_vs_fp64"] = out["fp64_vcycle"]["solve_s"] / out["mixed_fp32_vcycle"]["solve_s"]
    out["speedup_mixed_df64_vs_fp64"] = out["fp64_vcycle"]["solve_s"] / out["mixed_fp32_vcycle_df64"]["solve_s"]
    out["note"] = ("mixed: FP64 outer CG + FP32 V-cycle + FP64 coarse solve; _df64: the FP64 operators "
                   "(fine level, coarse level) in double-float arithmetic; the errors against the "
                   "oracle's FP64-everywhere solve are in cpu_baseline.time_to_solve_1e-8")
    return out


def _config1_solid_params(mfgpu, W, n_steps):
    spec = W.cantilever(4, 3)
    p = mfgpu.SolidParams()
    p.mesh = W.to_lib_mesh(mfgpu, spec)
    p.material = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
    p.caching = b"referential_qp"
    p.solver = mfgpu.solver_params("gmg", tol=1e-6, mg_precision=32)
    p.max_newton = 10
    p.tol_f, p.tol_f_abs, p.tol_u, p.tol_u_abs = 1e-9, 0.0, 1e-6, 0.0
    p.dt, p.n_steps = 0.01, n_steps
    p.traction_id = W.TRACTION_ID
    p.traction[:] = [0.0, -100.0, 0.0]
    p.watch[:] = [8.0, 0.5, 0.5]
    return p


def extra_solid_newton(mfgpu, W, ctx):
    """The 64x8x8-cell Q4 cantilever (839,619 DoFs): Newmark steps of
    dt = 0.01 under the traction (0,-100,0) on x = 8, Newton to 1e-9
    (residual) and 1e-6 (update), each system by GMG-CG to 1e-6 (FP32
    V-cycle, native FP64 fine operator): the first step alone and five
    steps, each from rest on a fresh solver."""
    out = {"workload": "cantilever 64x8x8 cells Q4, 839,619 DoFs, Newton-Newmark"}
    for key, steps in (("first_step", 1), ("five_steps", 5)):
        s = mfgpu.Solid(ctx, _config1_solid_params(mfgpu, W, steps))
        r = s.run()
        s.close()
        out[key] = {"newton_its": list(r.newton_its[:steps]), "cg_iterations": int(r.total_cg),
                    "linear_solves": int(r.n_solves), "seconds": r.seconds,
                    "watch_displacement": list(r.watch_disp[steps - 1][:3])}
    return out


def extra_degree_sweep(torch, mfgpu, W, ctx, dev, stream, flush, peak):
    """Heat operator on the unit cube with 64^3 cells, Q1..Q6: vmult DoF/s
    and achieved GB/s (B_alg = 2 s N_dof + 4 s N_cells) in FP64 (native and
    double-float) and FP32, with the default cell kernel (the tensor-product
    form: 1D mass and stiffness matrices, 7 sweeps per cell), the
    sum-factorization kernel through the Gauss points beside it
    (`*_sumfact`), and for FP32 Q1..Q5 the element-matrix product on the
    tensor cores; FP32-GMG vs FP64-GMG CG to 1e-8 with the seeded Gaussian
    source."""
    res = []
    c, w, a = W.gaussian_source(0)
    for deg in range(1, 7):
        spec = W.unit_cube_heat(deg, 6)
        mesh = W.to_lib_mesh(mfgpu, spec)
        n = W.n_dofs(spec, 1)
        cells = 64 ** 3
        row = {"degree": deg, "n_dofs": n}
        for label, prec, emul in (("fp64", 64, False), ("fp64_sumfact", 64, False), ("fp64_df64", 64, True),
                                  ("fp32", 32, False), ("fp32_sumfact", 32, False), ("fp32_tensor", 32, False)):
            if label == "fp32_tensor" and deg > 5:
                continue
            dt = torch.float64 if prec == 64 else torch.float32
            op = mfgpu.LaplaceOperator(ctx, mesh, -1, prec, True, delta_t=0.1)
            if emul:
                op.set_fp64_emulation(True)
            if label == "fp32_tensor":
                op.set_cell_kernel("tensor")
            if label.endswith("_sumfact"):
                op.set_cell_kernel("line")
            src = torch.rand(n, dtype=dt, device=dev) * 2 - 1
            dst = torch.zeros_like(src)
            op.vmult(dst, src)
            t = _timed_vmults(torch, op, dst, src, flush, stream, 5)
            s = 8 if prec == 64 else 4
            gbs = (2 * s * n + 4 * s * cells) / t / 1e9
            row[label] = {"dofs_per_s": n / t, "ms": t * 1e3, "gbs": gbs, "hbm_frac": gbs / peak}
            op.close()
            del src, dst
        for label, mgp in (("gmg_fp32_solve_s", 32), ("gmg_fp64_solve_s", 64)):
            hp = mfgpu.HeatParams()
            hp.mesh = mesh
            hp.dt, hp.n_steps = 0.1, 1
            hp.solver = mfgpu.solver_params("gmg", tol=1e-8, cheb_range=15.0, cheb_eig_its=10,
                                            mg_precision=mgp, coarse_fp64=(mgp == 32))
            hp.n_gauss = 8
            for i in range(8):
                for d in range(3):
                    hp.g_center[i][d] = c[i, d]
                hp.g_width[i] = w[i]
                hp.g_amp[i] = a[i]
            h = mfgpu.Heat(ctx, hp)
            r = h.run()
            row[label] = r.seconds
            row[label[:-2] + "_its"] = r.cg_its[0]
            h.close()
        res.append(row)
        torch.cuda.empty_cache()
    return res


def extra_design_choices(torch, mfgpu, W, ctx, dev, stream, flush, mesh, u, src, n, op, src_np, dst_np,
                         arith="native"):
    """Measurements behind the kernel choices on the headline workload (Q4
    cantilever 64x8x8, 839,619 DoFs), L2 flushed before every application:
    * scatter: atomic adds vs 8 parity colours with plain adds (the heat
      operator with the sum-factorization kernel in both modes);
    * quadrature data: each caching variant of the tangent in native FP64
      (streamed bytes vs recomputation), referential_qp also in FP32, and
      both referential cachings on the FP32 Q3 level of the mixed solve;
    * host-buffer vmult: number of overlapped z-slabs (1 = no overlap)."""
    out = {"scatter": {}, "caching_fp64": {}, "host_slabs": {}}
    dst = torch.zeros(n, dtype=torch.float64, device=dev)
    for mode in ("atomic", "colored"):
        op.set_scatter(mode)
        t = _timed_vmults(torch, op, dst, src, flush, stream, 10)
        out["scatter"]["nh_q4_" + arith + "_" + mode] = {"ms": t * 1e3, "dofs_per_s": n / t}
    op.set_scatter("atomic")
    heat = W.unit_cube_heat(2, 6)
    hm = W.to_lib_mesh(mfgpu, heat)
    hn = W.n_dofs(heat, 1)
    for prec in (64, 32):
        dt = torch.float64 if prec == 64 else torch.float32
        hop = mfgpu.LaplaceOperator(ctx, hm, -1, prec, True, delta_t=0.1)
        # both scatter modes with the sum-factorization kernel (the
        # tensor-product kernel, the default, scatters by atomics only)
        hop.set_cell_kernel("line")
        hs = torch.rand(hn, dtype=dt, device=dev) * 2 - 1
        hd = torch.zeros_like(hs)
        for mode in ("atomic", "colored"):
            hop.set_scatter(mode)
            hop.vmult(hd, hs)
            t = _timed_vmults(torch, hop, hd, hs, flush, stream, 10)
            out["scatter"][f"heat_64cube_q2_fp{prec}_{mode}"] = {"ms": t * 1e3, "dofs_per_s": hn / t}
        hop.close()
        del hs, hd
    mat = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
    for caching in ("scalar_referential", "tensor2", "tensor4", "tensor4_ns", "referential_qp"):
        for prec in ((64, 32) if caching in ("scalar_referential", "referential_qp") else (64,)):
            dt = torch.float64 if prec == 64 else torch.float32
            cop = mfgpu.NeoHookOperator(ctx, mesh, -1, prec, caching)
            cop.set_material(mat)
            uu = u if prec == 64 else u.to(torch.float32)
            cop.initialize(uu)
            cop.cache()
            s2 = src.to(dt)
            d2 = torch.zeros_like(s2)
            cop.vmult(d2, s2)
            t = _timed_vmults(torch, cop, d2, s2, flush, stream, 10)
            out["caching_fp64" if prec == 64 else "caching_fp32"] = out.get(
                "caching_fp64" if prec == 64 else "caching_fp32", {})
            out["caching_fp64" if prec == 64 else "caching_fp32"][caching] = {
                "ms": t * 1e3, "dofs_per_s": n / t, "cache_mb": cop.memory_consumption() / 1e6}
            cop.close()
            del s2, d2, uu
    # the finest multigrid level of the mixed solve (cantilever 128x16x16 cells
    # Q3, 2,773,155 DoFs, FP32): streamed referential_qp cache (10 values per
    # quadrature point) against scalar_referential (1 value per quadrature
    # point, the second gradient recomputed from the cell's displacement)
    q3 = W.cantilever(3, 4)
    q3m = W.to_lib_mesh(mfgpu, q3)
    nq3 = W.n_dofs(q3, 3)
    uq3 = torch.from_numpy(W.smooth_displacement(3, 4, q3["rep"], q3["lo"], q3["hi"], seed=2)).to(dev).float()
    sq3 = torch.rand(nq3, dtype=torch.float32, device=dev) * 2 - 1
    dq3 = torch.zeros_like(sq3)
    out["caching_fp32_q3_level"] = {}
    for caching in ("referential_qp", "scalar_referential"):
        cop = mfgpu.NeoHookOperator(ctx, q3m, -1, 32, caching)
        cop.set_material(mat)
        cop.initialize(uq3)
        cop.cache()
        cop.vmult(dq3, sq3)
        t = _timed_vmults(torch, cop, dq3, sq3, flush, stream, 10)
        out["caching_fp32_q3_level"][caching] = {"ms": t * 1e3, "dofs_per_s": nq3 / t,
                                                 "cache_mb": cop.memory_consumption() / 1e6}
        cop.close()
    del uq3, sq3, dq3
    K = 20
    for chunks in (1, 2, 4, 8):
        op.set_host_chunks(chunks)
        for _ in range(3):
            op.vmult_host(dst_np, src_np)
        t0 = time.perf_counter()
        for _ in range(K):
            op.vmult_host(dst_np, src_np)
        t = (time.perf_counter() - t0) / K
        out["host_slabs"][str(chunks)] = {"ms": t * 1e3, "dofs_per_s": n / t}
    op.set_host_chunks(0)
    torch.cuda.empty_cache()
    return out


def extra_heat_step(torch, mfgpu, W, ctx, dev, stream, flush):
    """Unit cube 16^3 cells Q2 (35,937 DoFs): one backward-Euler step solved
    by GMG-CG to 1e-10, and 100 FP64 vmults."""
    spec = W.unit_cube_heat(2, 4)
    mesh = W.to_lib_mesh(mfgpu, spec)
    c, w, a = W.gaussian_source(0)
    hp = mfgpu.HeatParams()
    hp.mesh = mesh
    hp.dt, hp.n_steps = 0.1, 1
    hp.solver = mfgpu.solver_params("gmg", tol=1e-10, cheb_range=15.0, cheb_eig_its=10,
                                    mg_precision=32)
    hp.n_gauss = 8
    for i in range(8):
        for d in range(3):
            hp.g_center[i][d] = c[i, d]
        hp.g_width[i] = w[i]
        hp.g_amp[i] = a[i]
    h = mfgpu.Heat(ctx, hp)
    h.run()
    r = h.run()
    h.close()
    n = W.n_dofs(spec, 1)
    op = mfgpu.LaplaceOperator(ctx, mesh, -1, 64, True, delta_t=0.1)
    src = torch.rand(n, dtype=torch.float64, device=dev)
    dst = torch.zeros_like(src)
    op.vmult(dst, src)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(100):
        op.vmult(dst, src)
    ctx.synchronize()
    t100 = time.perf_counter() - t0
    return {"workload": "heat unit cube 16^3 Q2, 35,937 DoFs", "step_s": r.seconds,
            "cg_iterations": r.cg_its[0], "vmult_100_s": t100}


def extra_serving(mfgpu, W, n_requests=300, workers=4, load=0.8, seed=7):
    """300 independent requests (60 % heat on 8^3..64^3 cells, 40 %
    neo-Hookean cantilevers 8k x k x k, k in {2,4,8}; degree U{1..4}; seeded
    sources / tractions), Poisson arrivals at `load` times the server's
    measured capacity, FP32-GMG preconditioned FP64 CG to 1e-8 (native FP64
    operators; the first 100 also with double-float FP64 operators) served
    by `workers` concurrent solves; against the same requests one at a time
    with the plain FP64 solver (all-FP64 V-cycle)."""
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    reqs = W.serving_requests(mfgpu, n_requests, seed=seed, mg_precision=32)
    # capacity: closed loop over the first 40 requests
    srv = mfgpu.Server(0, workers, 0.8)
    t0 = time.perf_counter()
    ids = [srv.submit(r) for r in reqs[:40]]
    for i in ids:
        srv.wait(i)
    capacity = 40 / (time.perf_counter() - t0)
    rate = load * capacity
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    t0 = time.perf_counter()
    ids = []
    for r, ta in zip(reqs, arrivals):
        dt = ta - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        ids.append(srv.submit(r))
    res = [srv.wait(i) for i in ids]
    span = time.perf_counter() - t0
    max_running, budget = srv.stats()
    reused, built = srv.pool_stats()
    batched, largest = srv.batch_stats()
    srv.close()
    lat = np.array([r.latency_seconds for r in res])
    errors = sum(1 for r in res if r.status != 0)
    # the same mixed-precision requests one at a time (first 100), closed loop:
    # what the concurrent solves on per-worker streams add
    # closed loop over the first 100 requests, then the same 100 again on
    # the same server (their problems resident: no construction, whose
    # allocations synchronise the whole device)
    def closed_loop(nw):
        srv = mfgpu.Server(0, nw, 0.8)
        rates = []
        for _ in range(2):
            t0 = time.perf_counter()
            ids = [srv.submit(r) for r in reqs[:100]]
            for i in ids:
                srv.wait(i)
            rates.append(100 / (time.perf_counter() - t0))
        nb = srv.batch_stats()[0]
        srv.close()
        return rates[0], rates[1], nb

    one, one_res, one_batched = closed_loop(1)
    many, many_res, many_batched = closed_loop(workers)
    # the same mixed-precision requests with the FP64 operators in
    # double-float instead of native FP64, closed loop, first 100
    df_reqs = W.serving_requests(mfgpu, 100, seed=seed, mg_precision=32, fp64_emulation=True)
    srv = mfgpu.Server(0, workers, 0.8)
    t0 = time.perf_counter()
    ids = [srv.submit(r) for r in df_reqs]
    dres = [srv.wait(i) for i in ids]
    dfrate = 100 / (time.perf_counter() - t0)
    srv.close()
    # baseline: one at a time, plain FP64 solver
    base_reqs = W.serving_requests(mfgpu, n_requests, seed=seed, mg_precision=64)
    srv = mfgpu.Server(0, 1, 0.8)
    t0 = time.perf_counter()
    ids = [srv.submit(r) for r in base_reqs]
    bres = [srv.wait(i) for i in ids]
    bspan = time.perf_counter() - t0
    srv.close()
    brun = np.array([r.run_seconds for r in bres])
    return {"requests": n_requests, "workers": workers, "arrival_rate_per_s": rate,
            "capacity_closed_loop_per_s": capacity,
            "solves_per_s": n_requests / span, "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)), "max_concurrent": max_running,
            "resident_problems": {"reused": reused, "built": built},
            "batching": {"requests_in_batches": batched, "largest_batch": largest,
                         "rule": "queued heat requests of the same shape and step count join the one a worker "
                                 "takes (one operator, V-cycle and CG for all), up to 4"},
            "errors": errors,
            "closed_loop_first100_df64_operators_per_s": {
                f"{workers}_workers": dfrate, "errors": sum(1 for r in dres if r.status != 0)},
            "closed_loop_first100_per_s": {"1_worker": one, f"{workers}_workers": many},
            "closed_loop_first100_resident_per_s": {"1_worker": one_res, f"{workers}_workers": many_res},
            "closed_loop_requests_in_batches": {"1_worker": one_batched, f"{workers}_workers": many_batched},
            "baseline_fp64_one_at_a_time": {"solves_per_s": n_requests / bspan,
                                            "service_p50_s": float(np.percentile(brun, 50)),
                                            "service_p99_s": float(np.percentile(brun, 99)),
                                            "errors": sum(1 for r in bres if r.status != 0)}}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    import workloads as W
    spec = W.cantilever(WORKLOAD["degree"], WORKLOAD["n_ref"], WORKLOAD["rep"], WORKLOAD["length"])
    n = W.n_dofs(spec, 3)
    u = W.smooth_displacement(spec["degree"], spec["n_ref"], spec["rep"], spec["lo"], spec["hi"], seed=2)
    src = W.uniform_vector(n, 3)
    # every caching variant of the reference (plain loops) and the
    # cell-batched SIMD form, cached once, vmults timed alone: the fastest
    # is the reference arm; it then runs W untimed and K timed applications
    budget = max(2.0, min(30.0, 3.0 * max(args.steps, 1)))
    rates, nthreads, reps, timers = oracle_vmult_rates(spec, u, src, budget)
    best = max(rates, key=rates.get)
    K, Wu = max(args.steps, 1), max(args.warmup, 1)
    _, secs = timers[best](K, Wu)
    value = n * K / secs
    dt = secs / K
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": K, "warmup": Wu, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "nh_tangent_vmult_q4_cantilever_64x8x8",
                       "n_dofs": n, "caching": best},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"{reps} applications per variant (each caching of the reference in "
                                       f"plain loops, and the cell-batched SIMD form /simdW), cached once, "
                                       f"vmult timed alone, on {nthreads} threads, built {CPU_FLAGS}; the "
                                       f"fastest, {best}, then "
                                       f"timed over {K} steps after {Wu} untimed; all: " +
                                       ", ".join(f"{c} {v / 1e6:.1f}" for c, v in rates.items()) +
                                       " MDoF/s (the reference itself needs deal.II/p4est/MPI, absent here)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


KERNEL_CASES = {
    # name: (operator, degree, refinements, precision, arithmetic)
    "nh_fp64_q4": ("nh", 4, 3, 64, "native"),   # the headline: 64x8x8 cells, 839,619 DoFs
    "nh_df64_q4": ("nh", 4, 3, 64, "df64"),
    "nh_fp64_q4_line": ("nh", 4, 3, 64, "line"),  # the line-parallel kernel on the headline case
    "nh_fp32_q3": ("nh", 3, 4, 32, "native"),   # finest level of the mixed solve, 2,773,155 DoFs
    "nh_fp32_q3_scalar_ref": ("nh_sr", 3, 4, 32, "native"),
    "heat_fp32_q1": ("heat", 1, 6, 32, "native"),  # unit cube 64^3 cells (tensor-product kernel)
    "heat_fp32_q2": ("heat", 2, 6, 32, "native"),
    "heat_fp32_q3": ("heat", 3, 6, 32, "native"),
    "heat_fp32_q4": ("heat", 4, 6, 32, "native"),
    "heat_fp32_q6": ("heat", 6, 6, 32, "native"),
    "heat_fp64_q2": ("heat", 2, 6, 64, "native"),
    "heat_fp64_q4": ("heat", 4, 6, 64, "native"),
    "heat_fp32_q2_sumfact": ("heat", 2, 6, 32, "line"),  # sum factorization through the Gauss points
    "heat_fp32_q6_sumfact": ("heat", 6, 6, 32, "line"),
    "heat_fp64_q2_sumfact": ("heat", 2, 6, 64, "line"),
    "heat_fp32_q2_tensor": ("heat", 2, 6, 32, "tensor"),  # element matrix on the tensor cores
    "heat_fp32_q3_tensor": ("heat", 3, 6, 32, "tensor"),
    "heat_fp32_q4_tensor": ("heat", 4, 6, 32, "tensor"),
}


SOLVER_CASES = {
    # the first Newton-Newmark step of the 64x8x8-cell Q4 cantilever (839,619 DoFs)
    "solid_step_64x8x8_q4": "solid",
    # the first Newton system of the 128x16x16-cell Q3 cantilever (2,773,155 DoFs) to 1e-8,
    # FP32 V-cycle, native FP64 fine and coarse operators
    "mixed_solve_q3": "mixed",
}


def run_solver_case(args):
    """One solver workload, run twice; the second run is the profiled one."""
    import torch
    import build as pkg_build
    import mfgpu
    import workloads as W
    pkg_build.build()
    dev = torch.device("cuda", 0)
    ctx = mfgpu.Context(0)
    kind = SOLVER_CASES[args.solver_case]

    def once():
        if kind == "solid":
            s = mfgpu.Solid(ctx, _config1_solid_params(mfgpu, W, 1))
            r = s.run()
            s.close()
            return {"seconds": r.seconds, "newton_its": list(r.newton_its[:1]), "cg_iterations": r.total_cg}
        spec = W.cantilever(3, 4)
        n = W.n_dofs(spec, 3)
        p = mfgpu.SolidParams()
        p.mesh = W.to_lib_mesh(mfgpu, spec)
        p.material = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
        p.caching = b"referential_qp"
        p.solver = mfgpu.solver_params("gmg", tol=1e-8, mg_precision=32, coarse_fp64=True)
        p.dt, p.n_steps, p.max_newton = 0.01, 1, 10
        p.traction_id = W.TRACTION_ID
        p.traction[:] = [0.0, -100.0, 0.0]
        s = mfgpu.Solid(ctx, p)
        zero = torch.zeros(n, dtype=torch.float64, device=dev)
        rhs = torch.zeros_like(zero)
        du = torch.zeros_like(zero)
        s.residual(zero, zero, rhs)
        its, secs = s.linear_solve(zero, rhs, du)
        s.close()
        return {"seconds": secs, "cg_iterations": its}

    once()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    out = once()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    print(json.dumps({"solver_case": args.solver_case, **out}))
    ctx.close()
    return 0


def run_kernel_case(args):
    """One operator applied `--steps` times on its workload (for ncu)."""
    import torch
    import build as pkg_build
    import mfgpu
    import workloads as W
    kind, deg, nref, prec, arith = KERNEL_CASES[args.kernel_case]
    pkg_build.build()
    dev = torch.device("cuda", 0)
    ctx = mfgpu.Context(0)
    dt = torch.float32 if prec == 32 else torch.float64
    if kind.startswith("nh"):
        spec = W.cantilever(deg, nref)
        n = W.n_dofs(spec, 3)
        u = torch.from_numpy(W.smooth_displacement(deg, nref, spec["rep"], spec["lo"], spec["hi"],
                                                   seed=2)).to(dev).to(dt)
        caching = "scalar_referential" if kind == "nh_sr" else "referential_qp"
        op = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, prec, caching)
        op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01))
        op.initialize(u)
        if arith == "df64":
            op.set_fp64_emulation(True)
        if arith == "line":
            op.set_cell_kernel("line")
        op.cache()
    else:
        spec = W.unit_cube_heat(deg, nref)
        n = W.n_dofs(spec, 1)
        op = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, prec, True, delta_t=0.1)
        if arith in ("tensor", "line"):
            op.set_cell_kernel(arith)
    src = torch.from_numpy(W.uniform_vector(n, 3)).to(dev).to(dt)
    dst = torch.zeros_like(src)
    for _ in range(max(args.steps, 1)):
        op.vmult(dst, src)
    ctx.synchronize()
    print(json.dumps({"kernel_case": args.kernel_case, "n_dofs": n, "vmults": max(args.steps, 1)}))
    op.close()
    ctx.close()
    return 0


def time_operator(torch, op, dst, src, flush, stream, K, warmup, clocks=None):
    """K device-resident vmults (L2 flushed before each, CUDA events on the
    library's stream) and K vmult_adds (the cell kernel and the constrained-
    row add, the dominant launch): per-step ms, kernel ms, launches."""
    import mfgpu
    for _ in range(warmup):
        op.vmult(dst, src)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    kstarts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    kends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    launches0 = mfgpu.launch_count()
    t0 = time.perf_counter()
    for i in range(K):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
            starts[i].record(stream)
        op.vmult(dst, src)
        with torch.cuda.stream(stream):
            ends[i].record(stream)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    launches = mfgpu.launch_count() - launches0
    for i in range(K):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
            kstarts[i].record(stream)
        op.vmult_add(dst, src)
        with torch.cuda.stream(stream):
            kends[i].record(stream)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    if clocks is not None:
        clocks.mark(t0, t2)
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / K
    kms = sum(s.elapsed_time(e) for s, e in zip(kstarts, kends)) / K
    return ms, kms, launches, t1 - t0


def time_host_vmult(op, dst_np, src_np, K, warmup, clocks=None):
    """K host-buffer vmults through the C-ABI (pinned source and result):
    seconds per call, with the z-slab overlap and without it."""
    for _ in range(warmup):
        op.vmult_host(dst_np, src_np)
    t0 = time.perf_counter()
    for _ in range(K):
        op.vmult_host(dst_np, src_np)
    t1 = time.perf_counter()
    if clocks is not None:
        clocks.mark(t0, t1)
    op.set_host_chunks(1)
    for _ in range(2):
        op.vmult_host(dst_np, src_np)
    t2 = time.perf_counter()
    for _ in range(K):
        op.vmult_host(dst_np, src_np)
    serial = (time.perf_counter() - t2) / K
    op.set_host_chunks(0)
    return (t1 - t0) / K, serial


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.kernel_case:
        return run_kernel_case(args)
    if args.solver_case:
        return run_solver_case(args)
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
    src_pin = torch.from_numpy(src_h).pin_memory()
    dst_pin = torch.zeros(n, dtype=torch.float64).pin_memory()
    src_np, dst_np = src_pin.numpy(), dst_pin.numpy()

    def barrier():
        torch.cuda.synchronize(dev)
        ctx.synchronize()
        if world > 1:
            torch.distributed.barrier()

    K = args.steps
    Wu = max(args.warmup, 3)
    clocks = clock_sampler(local, dev)
    clocks.start()
    barrier()
    ms_step, k_ms, launches, t_wall = time_operator(torch, op, dst, src, flush, stream, K, Wu, clocks)
    barrier()
    ms_step = max_over_ranks(ms_step, world, dev)
    k_ms = max_over_ranks(k_ms, world, dev)
    # end to end through the C-ABI with host buffers (pinned)
    e2e_s, e2e_serial_s = time_host_vmult(op, dst_np, src_np, K, Wu, clocks)
    barrier()
    e2e_s = max_over_ranks(e2e_s, world, dev)
    e2e_serial_s = max_over_ranks(e2e_serial_s, world, dev)

    # the other arithmetic of the same operator, reported beside the headline
    other = "df64" if args.arith == "native" else "native"
    op.set_fp64_emulation(other == "df64")
    op.cache()
    o_ms, o_kms, _, _ = time_operator(torch, op, dst, src, flush, stream, K, Wu, clocks)
    o_e2e, _ = time_host_vmult(op, dst_np, src_np, K, Wu, clocks)
    o_ms, o_kms, o_e2e = (max_over_ranks(x, world, dev) for x in (o_ms, o_kms, o_e2e))
    op.set_fp64_emulation(args.arith == "df64")
    op.cache()
    clk = clocks.stop()
    ctx.synchronize()

    peak, peak_kind = measured_peak_hbm()
    b_alg = algorithmic_bytes(n, n_cells)
    achieved = b_alg / (k_ms * 1e-3) / 1e9
    f_alg = algorithmic_flops(n_cells, 5)
    fp64_peak = measured_fp64_peak(torch, dev)
    prof = profile_summary(HEADLINE_PROFILE[args.arith])
    oprof = profile_summary(HEADLINE_PROFILE[other])
    o_block = {
        "arithmetic": ("double-float: each FP64 value carried as a pair of FP32 (48-bit significand, "
                       "FP32 exponent range) on the FP32 pipe; agrees with the FP64 oracle within "
                       "1e-12 relative l2 (tests/test_gpu_operators.py)") if other == "df64" else
                      "native FP64",
        "value": replica_throughput(n, o_ms * 1e-3, world), "unit": UNIT, "ms_per_step": o_ms,
        "kernel_ms": o_kms,
        "roofline": {"bound": "hbm", "achieved": b_alg / (o_kms * 1e-3) / 1e9, "peak": peak,
                     "unit": "GB/s", "frac": b_alg / (o_kms * 1e-3) / 1e9 / peak,
                     "traffic": (oprof or {}).get("traffic_bytes_per_launch"),
                     "traffic_source": "ncu, profiles/" + HEADLINE_PROFILE[other]},
        "e2e": {"value": replica_throughput(n, o_e2e, world), "unit": UNIT,
                "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8, "ms_per_step": o_e2e * 1e3},
    }
    line = {
        "metric": METRIC, "value": replica_throughput(n, ms_step * 1e-3, world), "unit": UNIT,
        "n_gpus": world, "steps": K, "warmup": Wu,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "df64" if args.arith == "df64" else "f64",
        "dtype_note": "native FP64 arithmetic, the reference's" if args.arith == "native" else
                      ("FP64 vectors in and out; arithmetic in double-float (a pair of FP32, 48-bit "
                       "significand) on the FP32 pipe"),
        "data": "synthetic",
        "config": {"workload": "nh_tangent_vmult_q4_cantilever_64x8x8", "n_dofs": n,
                   "n_cells": n_cells, "degree": 4, "n_q_1d": 5, "caching": args.caching,
                   "arithmetic": "native FP64" if args.arith == "native" else
                                 "double-float (FP32 pipe), parity 1e-12 vs FP64",
                   "l2": "flushed (512 MB write) before every timed application",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": replica_throughput(n, e2e_s, world), "unit": UNIT,
                "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8,
                "ms_per_step": e2e_s * 1e3,
                "overlap": "z-slabs: copy-in, cell launches and copy-out overlapped, replayed as a CUDA graph",
                "no_overlap": {"value": replica_throughput(n, e2e_serial_s, world),
                               "ms_per_step": e2e_serial_s * 1e3}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": (prof or {}).get("traffic_bytes_per_launch"),
                     "traffic_source": "ncu, profiles/" + HEADLINE_PROFILE[args.arith] +
                                       " (dram__bytes_read.sum + dram__bytes_write.sum of one launch)",
                     "peak_kind": peak_kind,
                     "kernel": "cell kernel of vmult_add (CUDA events, L2 flushed)",
                     "kernel_ms": k_ms, "bytes_alg_per_launch": b_alg},
        "compute_roofline": {
            "bound": "FP64 pipe" if args.arith == "native" else "FP32 pipe issue (double-float)",
            "fp64_peak_tflops_measured": fp64_peak,
            "fp64_peak_source": "cuBLAS DGEMM 4096^3 on this GPU, best of 3",
            "alg_tflops": f_alg / (k_ms * 1e-3) / 1e12,
            "alg_flop_per_launch": f_alg,
            "ncu": prof, "source": "profiles/" + HEADLINE_PROFILE[args.arith],
            "note": "the roof that binds this kernel; the HBM fraction above is the fixed "
                    "algorithmic-bytes convention"},
        other: o_block,
        "clocks": clk,
        "gpu_launches": launches,
        "wall_ms_per_step": t_wall / K * 1e3,
    }
    if not args.no_extras and world == 1:  # secondary measurements: one GPU only
        extras = {}
        for key, fn in (("time_to_solve_1e-8", lambda: extra_mixed_precision_solve(torch, mfgpu, W, ctx, dev)),
                        ("heat_step_16cube_q2", lambda: extra_heat_step(torch, mfgpu, W, ctx, dev, stream, flush)),
                        ("solid_newton_64x8x8_q4", lambda: extra_solid_newton(mfgpu, W, ctx)),
                        ("design_choices", lambda: extra_design_choices(torch, mfgpu, W, ctx, dev, stream, flush,
                                                                         mesh, u, src, n, op, src_np, dst_np,
                                                                         args.arith)),
                        ("degree_sweep_heat_64cube", lambda: extra_degree_sweep(torch, mfgpu, W, ctx, dev,
                                                                               stream, flush, peak)),
                        ("serving_300_requests", lambda: extra_serving(mfgpu, W))):
            try:
                t0 = time.perf_counter()
                extras[key] = fn()
                extras[key + "_wall_s"] = time.perf_counter() - t0
            except Exception as e:
                extras[key] = {"error": str(e)}
        line["extras"] = extras
    if rank == 0 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline(spec, u_h, src_h, args.cpu_seconds)
        except Exception as e:  # reported, never fatal for the GPU number
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port",
                                    "sample": f"failed: {e}"}
        try:
            line["cpu_baseline"]["heat_step_16cube_q2"] = cpu_heat_step()
        except Exception as e:
            line["cpu_baseline"]["heat_step_16cube_q2"] = {"error": str(e)}
        if not args.no_extras:
            for key, fn in (("heat_vmult_64cube_dofs_per_s", cpu_heat_sweep),
                            ("time_to_solve_1e-8", cpu_mixed_solve),
                            ("solid_newton_first_step", cpu_solid_first_step)):
                try:
                    line["cpu_baseline"][key] = fn()
                except Exception as e:
                    line["cpu_baseline"][key] = {"error": str(e)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
