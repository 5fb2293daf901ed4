"""Named single-kernel cases for profiling (ncu) the operator kernels.

    python matrix-free-dealii-precice_gb300/kernel_cases.py <case> [vmults]

Each case builds one operator on its workload and applies it `vmults`
times (default 5) on a seeded U(-1,1) vector:

* nh_fp32_q3   FP32 referential_qp tangent on the Q3 cantilever 128x16x16
               (2,773,155 DoFs): the finest multigrid level of the
               mixed-precision solve;
* nh_df64_q4   FP64 referential_qp tangent in double-float arithmetic on the
               Q4 cantilever 64x8x8 (839,619 DoFs), the benchmark workload;
* heat_fp32_q6 FP32 heat operator on the unit cube 64^3 cells, Q6
               (57,066,625 DoFs);
* heat_fp32_q2 FP32 heat operator on the unit cube 64^3 cells, Q2.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def main(argv):
    import torch
    import build
    import mfgpu
    import workloads as W
    case = argv[1] if len(argv) > 1 else "nh_fp32_q3"
    reps = int(argv[2]) if len(argv) > 2 else 5
    build.build()
    dev = torch.device("cuda", 0)
    ctx = mfgpu.Context(0)
    if case.startswith("nh"):
        deg, nref = (3, 4) if case == "nh_fp32_q3" else (4, 3)
        prec = 32 if "fp32" in case else 64
        dt = torch.float32 if prec == 32 else torch.float64
        spec = W.cantilever(deg, nref)
        n = W.n_dofs(spec, 3)
        u = torch.from_numpy(W.smooth_displacement(deg, nref, spec["rep"], spec["lo"], spec["hi"],
                                                   seed=2)).to(dev).to(dt)
        op = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, prec, "referential_qp")
        op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01))
        op.initialize(u)
        if "df64" in case:
            op.set_fp64_emulation(True)
        op.cache()
    elif case.startswith("heat"):
        deg = int(case[-1])
        dt = torch.float32
        spec = W.unit_cube_heat(deg, 6)
        n = W.n_dofs(spec, 1)
        op = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 32, True, delta_t=0.1)
    else:
        raise SystemExit(f"unknown case {case}")
    g = torch.Generator(device=dev)
    g.manual_seed(1)
    src = (torch.rand(n, dtype=dt, device=dev, generator=g) * 2 - 1)
    dst = torch.zeros_like(src)
    for _ in range(reps):
        op.vmult(dst, src)
    ctx.synchronize()
    print(f"{case}: {n} DoFs, {reps} vmults")
    op.close()
    ctx.close()


if __name__ == "__main__":
    main(sys.argv)
