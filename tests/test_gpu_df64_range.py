"""Range limits of the double-float ("df64") FP64 operators against the
oracle's FP64 vmult, next to native FP64.

A df64 value is an unevaluated sum of two FP32 numbers: 48 significand bits
and FP32's exponent range.  On inputs scaled by s (the operator is linear,
so the exact result scales by s) the df64 operators keep the 1e-12 relative
l2 bar from s = 1e-30 up to 1e36 (heat) and 1e28 (the referential_qp
tangent with the shear modulus raised to 0.5e9, whose quadrature-point
terms reach mu/h^2 times the gradients); past the FP32 exponent range the
results overflow (non-finite), and below about 1e-35 the low halves become
FP32 subnormals and the accuracy falls off.  Native FP64, the default, keeps
1e-12 over the whole range.  The heat operator is
heat_transfer.h:236-250, the tangent mf_nh_operator.h:848-943.
"""
import numpy as np
import pytest

import mfgpu
import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu
TOL64 = 1e-12


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _heat(ctx, arith):
    spec = W.unit_cube_heat(3, 1, rep=(2, 1, 1))
    op = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 64, True, delta_t=0.1)
    if arith == "df64":
        op.set_fp64_emulation(True)
    return spec, op


def _apply(op, src):
    d = dev(np.zeros_like(src))
    op.vmult(d, dev(src))
    return host(d)


def test_df64_heat_range(ctx):
    spec, op = _heat(ctx, "df64")
    _, nat = _heat(ctx, "native")
    n = W.n_dofs(spec, 1)
    src = W.uniform_vector(n, 1)
    ref = O.heat_vmult(W.to_oracle_mesh(O, spec), 1, 0.1, src)
    for s in (1e-30, 1e-20, 1.0, 1e20, 1e30, 1e36):
        assert rel(_apply(op, src * s), ref * s) < TOL64, s
    # FP32 exponent range exceeded: non-finite in df64, exact in FP64
    big = _apply(op, src * 1e38)
    assert not np.isfinite(big).all()
    assert rel(_apply(nat, src * 1e38), ref * 1e38) < TOL64
    # FP32 subnormal low halves: the 1e-12 bar is lost, FP64 keeps it
    tiny = _apply(op, src * 1e-38)
    assert rel(tiny, ref * 1e-38) > TOL64
    assert rel(_apply(nat, src * 1e-38), ref * 1e-38) < TOL64


@pytest.mark.parametrize("mu,top", [(0.5e6, 1e30), (0.5e9, 1e28)])
def test_df64_tangent_range(ctx, mu, top):
    spec = W.cantilever(2, 1, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    n = W.n_dofs(spec, 3)
    u = W.smooth_displacement(2, 1, spec["rep"], spec["lo"], spec["hi"], seed=2)
    src = W.uniform_vector(n, 3)
    ref = O.nh_vmult(W.to_oracle_mesh(O, spec), 1, O.material(mu=mu, dt=0.01),
                     "scalar_referential", u, src)
    d_u = dev(u)
    ops = {}
    for arith in ("df64", "native"):
        op = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 64, "referential_qp")
        op.set_material(mfgpu.material(mu=mu, dt=0.01))
        op.initialize(d_u)
        if arith == "df64":
            op.set_fp64_emulation(True)
        op.cache()
        ops[arith] = op
    for s in (1e-30, 1e-20, 1.0, 1e20, top):
        assert rel(_apply(ops["df64"], src * s), ref * s) < TOL64, s
    over = top * 1e4
    assert not np.isfinite(_apply(ops["df64"], src * over)).all()
    assert rel(_apply(ops["native"], src * over), ref * over) < TOL64
    assert rel(_apply(ops["df64"], src * 1e-40), ref * 1e-40) > TOL64
    assert rel(_apply(ops["native"], src * 1e-40), ref * 1e-40) < TOL64
