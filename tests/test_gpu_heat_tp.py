"""The heat operator in its tensor-product form (cell kernel 4: the element
operator as sums of products of the 1D mass and stiffness matrices, one
thread per cell column segment in registers) against the oracle's vmult
(heat_transfer.h:236-250) and against the sum-factorization kernel.

Degrees 1-6: one thread per cell in registers at Q1 on levels of 16384
cells or more, the shared-memory block form otherwise (and always in
double-float).  Tolerances: FP64 1e-12 relative l2
(the operator parity bar), FP32 5e-5 as the other FP32 operator tests.  The meshes exercise what the kernel's
work split depends on: rows of cells shorter and longer than a warp (the
x-neighbour exchange by shuffles across warp ends), column segments that do
not divide the z extent (the z-carry of results between the cells of a
segment), anisotropic cells, constrained faces on every side
and none, and cell ranges (the z-slabs of the host-buffer vmult)."""
import numpy as np
import pytest

import mfgpu
import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu
TOL = {32: 5e-5, 64: 1e-12}
DEGREES = [1, 2, 3, 4, 5, 6]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy().astype(np.float64)


def _spec(degree, rep, n_ref, hi, boundary_id, dirichlet):
    return dict(degree=degree, n_ref=n_ref, rep=rep, lo=(0.0, 0.0, 0.0), hi=hi,
                boundary_id=boundary_id, dirichlet=dirichlet)


# (repetitions, refinements, upper corner, boundary ids, dirichlet)
MESHES = {
    # 6 x 4 x 10 cells: rows shorter than a warp, anisotropic cells, two
    # clamped faces
    "short_rows": ((3, 2, 5), 1, (1.5, 0.7, 2.0), (1, 0, 2, 0, 0, 2), [(1, 1), (2, 1)]),
    # 40 x 30 x 14 cells (16,800: the register kernel at Q1-Q2): rows
    # across warp ends, every face clamped
    "long_rows": ((40, 30, 14), 0, (4.0, 3.0, 0.7), (1, 1, 1, 1, 1, 1), [(1, 1)]),
    # 33 x 25 x 20 cells (16,500), no constraint
    "free": ((33, 25, 20), 0, (1.0, 0.8, 0.9), (0, 0, 0, 0, 0, 0), []),
    # 64 x 64 x 39 cells: column segments of 4 cells (enough columns for the
    # launch heuristic), the last one of 3
    "segments": ((64, 64, 39), 0, (1.0, 1.0, 0.6), (1, 0, 2, 0, 0, 2), [(1, 1), (2, 1)]),
}


@pytest.mark.parametrize("precision", [32, 64, "df64"])
@pytest.mark.parametrize("mesh", sorted(MESHES))
def test_tensor_product_heat_vmult(ctx, precision, mesh):
    """FP32, native FP64 and double-float (FP64 vectors, the block form in
    float-pair arithmetic: the FP64 bar of 1e-12)."""
    df64 = precision == "df64"
    precision = 64 if df64 else precision
    rep, nref, hi, bid, dirichlet = MESHES[mesh]
    # the 64 x 64 x 39 mesh tests the column segments of the register
    # kernel (degrees 1-2); the others every degree
    for degree in DEGREES if mesh != "segments" else [1, 2]:
        spec = _spec(degree, rep, nref, hi, bid, dirichlet)
        m = W.to_lib_mesh(mfgpu, spec)
        n = W.n_dofs(spec, 1)
        dt = np.float32 if precision == 32 else np.float64
        src = W.uniform_vector(n, 11 + degree, dt)
        constrained = bool(dirichlet)
        ref = O.heat_vmult(W.to_oracle_mesh(O, spec), nref, 0.1, src.astype(np.float64),
                           constrained=constrained)
        op = mfgpu.LaplaceOperator(ctx, m, -1, precision, constrained, delta_t=0.1)
        if df64:
            op.set_fp64_emulation(True)
        d_src = dev(src)
        d_sf, d_tp = dev(np.zeros_like(src)), dev(np.zeros_like(src))
        op.set_cell_kernel("line")
        op.vmult(d_sf, d_src)
        sf = host(d_sf)
        # "tp": registers; "tp_tma": FP32 Q1-Q2 bricks staged by TMA,
        # registers otherwise
        for mode in ("tp", "tp_tma"):
            op.set_cell_kernel(mode)
            op.vmult(d_tp, d_src)
            tp = host(d_tp)
            assert rel(tp, ref) < TOL[precision], (mode, degree, rel(tp, ref))
            assert rel(tp, sf) < TOL[precision], (mode, degree, rel(tp, sf))
            # vmult_add adds
            op.vmult_add(d_tp, d_src)
            assert rel(host(d_tp), 2 * ref) < TOL[precision]


@pytest.mark.parametrize("precision", [32, 64])
def test_tensor_product_heat_default_and_host_buffers(ctx, precision):
    """A 16^3-cell Q2 level takes kernel 4 by default (4096 cells, the block
    form); the overlapped host-buffer vmult (z-slabs of cells) gives the same
    result."""
    spec = W.unit_cube_heat(2, 4)
    m = W.to_lib_mesh(mfgpu, spec)
    n = W.n_dofs(spec, 1)
    dt = np.float32 if precision == 32 else np.float64
    src = W.uniform_vector(n, 5, dt)
    ref = O.heat_vmult(W.to_oracle_mesh(O, spec), 4, 0.1, src.astype(np.float64))
    op = mfgpu.LaplaceOperator(ctx, m, -1, precision, True, delta_t=0.1)
    d = dev(np.zeros_like(src))
    before = mfgpu.launch_count()
    op.vmult(d, dev(src))
    assert mfgpu.launch_count() - before == 1
    assert rel(host(d), ref) < TOL[precision]
    if precision == 64:
        out = np.zeros_like(src)
        for chunks in (1, 4):
            op.set_host_chunks(chunks)
            op.vmult_host(out, src)
            assert rel(out, ref) < TOL[64], chunks


def test_tensor_product_heat_rejects_unsupported(ctx):
    """Two-dimensional meshes and the neo-Hookean operator keep their own
    kernels."""
    spec = W.cantilever(2, 1, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    op = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 64, "referential_qp")
    with pytest.raises(mfgpu.MfgpuError):
        op.set_cell_kernel("tp")
    m2 = mfgpu.make_mesh(2, 2, (1, 1), (0.0, 0.0), (1.0, 1.0), boundary_id=(1, 0, 0, 0),
                         dirichlet=[(1, 1)])
    op = mfgpu.LaplaceOperator(ctx, m2, -1, 32, True, delta_t=0.1)
    with pytest.raises(mfgpu.MfgpuError):
        op.set_cell_kernel("tp")


def test_tensor_product_heat_unaligned_vectors(ctx):
    """Vectors that do not start on 16 bytes (views at an offset of one
    float) cannot be staged by TMA: the register kernel serves them."""
    import torch
    spec = _spec(2, (40, 30, 14), 0, (4.0, 3.0, 0.7), (1, 1, 1, 1, 1, 1), [(1, 1)])
    n = W.n_dofs(spec, 1)
    src = W.uniform_vector(n, 21, np.float32)
    ref = O.heat_vmult(W.to_oracle_mesh(O, spec), 0, 0.1, src.astype(np.float64))
    op = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 32, True, delta_t=0.1)
    op.set_cell_kernel("tp_tma")
    big_src = torch.zeros(n + 1, dtype=torch.float32, device="cuda")
    big_src[1:] = dev(src)
    big_dst = torch.zeros(n + 1, dtype=torch.float32, device="cuda")
    op.vmult(big_dst[1:], big_src[1:])
    assert rel(host(big_dst[1:]), ref) < TOL[32]
    assert float(big_dst[0]) == 0.0
