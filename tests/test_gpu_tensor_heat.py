"""The FP32 heat operator on the tensor cores (cell kernel 3: the cells'
common element matrix applied to batches of 128 cells by tcgen05.mma in
TF32 with a three-term split) against the oracle's FP32 and FP64 vmult and
against the sum-factorization kernel: FP32 tolerance 5e-5 relative l2, as
the other FP32 operator tests (heat_transfer.h:236-250)."""
import numpy as np
import pytest

import mfgpu
import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu
TOL32 = 5e-5


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _spec(degree, rep, n_ref, hi=(1.0, 1.0, 1.0), dirichlet=True):
    spec = dict(degree=degree, n_ref=n_ref, rep=rep, lo=(0.0, 0.0, 0.0), hi=hi,
                boundary_id=(1, 0, 2, 0, 0, 2), dirichlet=[(1, 0b1), (2, 0b1)] if dirichlet else [])
    return spec


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("constrained", [True, False])
def test_tensor_core_heat_vmult(ctx, degree, constrained):
    # anisotropic cells; 3 x 2 x 5 coarse cells, one refinement: 240 cells,
    # so the last batch of 128 is partial
    spec = _spec(degree, (3, 2, 5), 1, hi=(1.5, 0.7, 2.0))
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    n = W.n_dofs(spec, 1)
    src = W.uniform_vector(n, 7, np.float32)
    ref64 = O.heat_vmult(om, 1, 0.1, src.astype(np.float64), constrained=constrained)
    op = mfgpu.LaplaceOperator(ctx, m, -1, 32, constrained, delta_t=0.1)
    d_src = dev(src)
    d_sf, d_tc = dev(np.zeros_like(src)), dev(np.zeros_like(src))
    op.vmult(d_sf, d_src)
    op.set_cell_kernel("tensor")
    op.vmult(d_tc, d_src)
    tc, sf = host(d_tc).astype(np.float64), host(d_sf).astype(np.float64)
    assert rel(tc, ref64) < TOL32, rel(tc, ref64)
    assert rel(tc, sf) < TOL32
    # vmult_add adds; a second application gives the same result
    op.vmult_add(d_tc, d_src)
    assert rel(host(d_tc).astype(np.float64), 2 * ref64) < TOL32


def test_tensor_core_heat_full_level_and_delta_t_change(ctx):
    """A 64^3-cell Q2 level (2.1M DoFs): against the sum-factorization
    kernel; after set_delta_t the element matrix is rebuilt."""
    spec = W.unit_cube_heat(2, 6)
    m = W.to_lib_mesh(mfgpu, spec)
    n = W.n_dofs(spec, 1)
    op = mfgpu.LaplaceOperator(ctx, m, -1, 32, True, delta_t=0.1)
    src = dev(W.uniform_vector(n, 3, np.float32))
    a, b = dev(np.zeros(n, np.float32)), dev(np.zeros(n, np.float32))
    for dt in (0.1, 0.37):
        op.set_delta_t(dt)
        op.set_cell_kernel("auto")
        op.vmult(a, src)
        op.set_cell_kernel("tensor")
        op.vmult(b, src)
        assert rel(host(b).astype(np.float64), host(a).astype(np.float64)) < TOL32


def test_tensor_core_kernel_is_refused_where_it_does_not_apply(ctx):
    spec = W.unit_cube_heat(2, 1)
    m = W.to_lib_mesh(mfgpu, spec)
    op64 = mfgpu.LaplaceOperator(ctx, m, -1, 64, True, delta_t=0.1)
    with pytest.raises(mfgpu.MfgpuError) as e:
        op64.set_cell_kernel("tensor")
    assert e.value.code == 8
    nh = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, W.cantilever(2, 0, rep=(2, 1, 1))), -1, 32,
                               "referential_qp")
    with pytest.raises(mfgpu.MfgpuError) as e:
        nh.set_cell_kernel("tensor")
    assert e.value.code == 8
    q6 = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, W.unit_cube_heat(6, 0)), -1, 32, True,
                               delta_t=0.1)
    with pytest.raises(mfgpu.MfgpuError):
        q6.set_cell_kernel("tensor")
