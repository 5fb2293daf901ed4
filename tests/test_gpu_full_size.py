"""Parity at the benchmark's full sizes, through the C-ABI.

The headline workload (Q4 neo-Hookean tangent on the 64x8x8-cell cantilever,
839,619 DoFs, the bench's seeded linearisation and source vector) is applied
on the device in double-float and in native FP64 and compared with the
oracle's FP64 vmult (mf_nh_operator.h:545-625) at the FP64 bar, 1e-12
relative l2; likewise the heat operator on 64^3 cells at Q2 (2,146,689
DoFs).  Size-independent properties complete the check: vmult is linear in
the source and vmult_add adds.
"""
import numpy as np
import pytest

import mfgpu
import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_headline_tangent_full_size(ctx):
    spec = W.cantilever(4, 3)
    n = W.n_dofs(spec, 3)
    assert n == 839619
    u = W.smooth_displacement(4, 3, spec["rep"], spec["lo"], spec["hi"], seed=2)
    src = W.uniform_vector(n, 3)
    ref = O.nh_vmult(W.to_oracle_mesh(O, spec), 3, O.material(0.5e6, 0.4, 1000.0, 0.01),
                     "scalar_referential", u, src)
    d_u, d_src, d_src2 = dev(u), dev(src), dev(2.0 * src)
    for emulate in (True, False):
        op = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 64, "referential_qp")
        op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01))
        op.initialize(d_u)
        op.set_fp64_emulation(emulate)
        op.cache()
        d_dst = dev(np.zeros(n))
        op.vmult(d_dst, d_src)
        got = host(d_dst)
        assert rel(got, ref) < TOL64, ("df64" if emulate else "f64", rel(got, ref))
        # linearity and vmult_add at full size
        op.vmult(d_dst, d_src2)
        assert rel(host(d_dst), 2.0 * got) < TOL64
        op.vmult_add(d_dst, d_src)
        assert rel(host(d_dst), 3.0 * got) < TOL64
        op.close()


def test_heat_64cube_q2_full_size(ctx):
    spec = W.unit_cube_heat(2, 6)
    n = W.n_dofs(spec, 1)
    assert n == 2146689
    src = W.uniform_vector(n, 1)
    ref = O.heat_vmult(W.to_oracle_mesh(O, spec), 6, 0.1, src)
    d_src = dev(src)
    for emulate in (True, False):
        op = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 64, True, delta_t=0.1)
        op.set_fp64_emulation(emulate)
        d_dst = dev(np.zeros(n))
        op.vmult(d_dst, d_src)
        assert rel(host(d_dst), ref) < TOL64, "df64" if emulate else "f64"
        op.close()
