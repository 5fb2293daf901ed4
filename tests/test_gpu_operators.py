"""Device operators through the C-ABI against the CPU oracle.

Tolerances: FP64 operator applications agree with the oracle within 1e-12
relative l2 (the FP64 parity bar); FP32 within 2e-5 relative l2; FP64
diagonals within 1e-11 (the device uses the tensor-product diagonal, the
oracle applies the cell operator to local unit vectors).
"""
import numpy as np
import pytest

import mfgpu
import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def small_heat(degree):
    return W.unit_cube_heat(degree, 1, rep=(2, 1, 1))


def small_cantilever(degree):
    return W.cantilever(degree, 1, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("precision", [64, 32])
def test_heat_vmult(ctx, degree, precision):
    spec = small_heat(degree)
    dt = np.float64 if precision == 64 else np.float32
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    n = W.n_dofs(spec, 1)
    src = W.uniform_vector(n, 1, dt)
    ref = O.heat_vmult(om, 1, 0.1, src, precision=precision)
    op = mfgpu.LaplaceOperator(ctx, m, -1, precision, True, delta_t=0.1)
    d_src, d_dst = dev(src), dev(np.zeros_like(src))
    op.vmult(d_dst, d_src)
    assert rel(host(d_dst), ref) < (TOL64 if precision == 64 else TOL32)
    # vmult_add adds; Tvmult == vmult (symmetric)
    op.vmult_add(d_dst, d_src)
    assert rel(host(d_dst), 2 * ref) < (TOL64 if precision == 64 else TOL32)
    op.Tvmult(d_dst, d_src)
    assert rel(host(d_dst), ref) < (TOL64 if precision == 64 else TOL32)


@pytest.mark.parametrize("degree", [1, 2, 4])
def test_heat_unconstrained_and_diagonal(ctx, degree):
    spec = small_heat(degree)
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    n = W.n_dofs(spec, 1)
    src = W.uniform_vector(n, 3)
    ref = O.heat_vmult(om, 1, 0.1, src, constrained=False)
    op = mfgpu.LaplaceOperator(ctx, m, -1, 64, False, delta_t=0.1)
    d_dst = dev(np.zeros(n))
    op.vmult(d_dst, dev(src))
    assert rel(host(d_dst), ref) < TOL64
    opc = mfgpu.LaplaceOperator(ctx, m, -1, 64, True, delta_t=0.1)
    opc.compute_diagonal()
    ptr = opc.get_matrix_diagonal_inverse()
    d_inv = dev(np.zeros(n))
    # copy through the Jacobi preconditioner: dst = 1.0 * Dinv * ones
    opc.precondition_Jacobi(d_inv, dev(np.ones(n)), 1.0)
    ref_inv = O.heat_inv_diagonal(om, 1, 0.1)
    assert rel(host(d_inv), ref_inv) < 1e-11
    assert ptr
    # el(i,i) is the diagonal entry
    i = n // 2
    assert abs(opc.el(i, i) - 1.0 / ref_inv[i]) < 1e-10 * abs(1.0 / ref_inv[i])


CACHINGS = ["scalar_referential", "tensor2", "tensor4", "tensor4_ns",
            "referential_qp"]


def nh_setup(degree, seed=2):
    spec = small_cantilever(degree)
    u = W.smooth_displacement(degree, spec["n_ref"], spec["rep"], spec["lo"],
                              spec["hi"], seed=seed)
    return spec, u


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("caching", CACHINGS)
def test_nh_vmult_fp64(ctx, degree, caching):
    spec, u = nh_setup(degree)
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    n = W.n_dofs(spec, 3)
    mat_o = O.material(0.5e6, 0.4, 1000.0, 0.01)
    mat_l = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
    src = W.uniform_vector(n, 3)
    oracle_caching = "scalar_referential" if caching == "referential_qp" else caching
    ref = O.nh_vmult(om, 1, mat_o, oracle_caching, u, src)
    op = mfgpu.NeoHookOperator(ctx, m, -1, 64, caching)
    op.set_material(mat_l)
    d_u = dev(u)
    op.initialize(d_u)
    op.cache()
    d_dst = dev(np.zeros(n))
    op.vmult(d_dst, dev(src))
    assert rel(host(d_dst), ref) < TOL64, caching


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("arith", ["f64", "df64", "f32"])
def test_qp10_anisotropic_cells(ctx, degree, arith):
    """referential_qp works with reference-cell gradients and folds the
    per-direction Jacobian into its cache and constants: checked on cells
    with three different edge lengths (1.5 x 0.5 x 0.35)."""
    spec = W.cantilever(degree, 1, rep=(2, 1, 1), length=(3.0, 0.5, 0.35))
    spec["lo"] = (0.0, -0.25, 0.1)
    spec["hi"] = (3.0, 0.25, 0.45)
    u = W.smooth_displacement(degree, 1, spec["rep"], spec["lo"], spec["hi"], seed=6,
                              amplitude=0.02)
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    n = W.n_dofs(spec, 3)
    src = W.uniform_vector(n, 8)
    ref = O.nh_vmult(om, 1, O.material(0.5e6, 0.4, 1000.0, 0.01), "scalar_referential", u, src)
    prec = 32 if arith == "f32" else 64
    dt = np.float32 if prec == 32 else np.float64
    op = mfgpu.NeoHookOperator(ctx, m, -1, prec, "referential_qp")
    op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01))
    d_u = dev(u.astype(dt))
    op.initialize(d_u)
    if arith == "df64":
        op.set_fp64_emulation(True)
    op.cache()
    d_dst = dev(np.zeros(n, dt))
    op.vmult(d_dst, dev(src.astype(dt)))
    assert rel(host(d_dst).astype(np.float64), ref) < (TOL64 if prec == 64 else 5e-5)


@pytest.mark.parametrize("degree", [1, 3, 5])
def test_nh_vmult_fp32(ctx, degree):
    spec, u = nh_setup(degree)
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    n = W.n_dofs(spec, 3)
    src = W.uniform_vector(n, 3)
    ref = O.nh_vmult(om, 1, O.material(dt=0.01), "scalar_referential", u, src)
    for caching in ("scalar_referential", "referential_qp"):
        op = mfgpu.NeoHookOperator(ctx, m, -1, 32, caching)
        op.set_material(mfgpu.material(dt=0.01))
        d_u = dev(u.astype(np.float32))
        op.initialize(d_u)
        op.cache()
        d_dst = dev(np.zeros(n, np.float32))
        op.vmult(d_dst, dev(src.astype(np.float32)))
        assert rel(host(d_dst).astype(np.float64), ref) < 5e-5, caching


@pytest.mark.parametrize("degree", [1, 2, 4])
def test_nh_formulation0(ctx, degree):
    spec, u = nh_setup(degree)
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    n = W.n_dofs(spec, 3)
    src = W.uniform_vector(n, 5)
    ref = O.nh_vmult(om, 1, O.material(dt=0.01, formulation=0), "tensor2", u, src)
    op = mfgpu.NeoHookOperator(ctx, m, -1, 64, "tensor2")
    op.set_material(mfgpu.material(dt=0.01, formulation=0))
    d_u = dev(u)
    op.initialize(d_u)
    op.cache()
    d_dst = dev(np.zeros(n))
    op.vmult(d_dst, dev(src))
    assert rel(host(d_dst), ref) < TOL64
    # the diagonal of formulation 0 (column-wise tangent blocks)
    op.compute_diagonal()
    d_inv = dev(np.zeros(n))
    op.precondition_Jacobi(d_inv, dev(np.ones(n)), 1.0)
    ref_inv = O.nh_inv_diagonal(om, 1, O.material(dt=0.01, formulation=0), "tensor2", u)
    assert rel(host(d_inv), ref_inv) < 1e-11


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("precision", [64, 32])
def test_nh_diagonal(ctx, degree, precision):
    spec, u = nh_setup(degree)
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    n = W.n_dofs(spec, 3)
    npdt = np.float64 if precision == 64 else np.float32
    ref_inv = O.nh_inv_diagonal(om, 1, O.material(dt=0.01), "scalar_referential", u)
    op = mfgpu.NeoHookOperator(ctx, m, -1, precision, "scalar_referential")
    op.set_material(mfgpu.material(dt=0.01))
    d_u = dev(u.astype(npdt))
    op.initialize(d_u)
    op.cache()
    op.compute_diagonal()
    d_inv = dev(np.zeros(n, npdt))
    op.precondition_Jacobi(d_inv, dev(np.ones(n, npdt)), 1.0)
    tol = 1e-11 if precision == 64 else 5e-5
    assert rel(host(d_inv).astype(np.float64), ref_inv) < tol


def test_nh_det_f_error_status(ctx):
    """A linearisation with det F <= 0 is reported as MFGPU_ERR_DET_F (the
    kernel sets an error word; no device fault)."""
    spec, u = nh_setup(2)
    m = W.to_lib_mesh(mfgpu, spec)
    op = mfgpu.NeoHookOperator(ctx, m, -1, 64, "scalar_referential")
    op.set_material(mfgpu.material(dt=0.01))
    X, Y, Z = W.node_coords(2, spec["n_ref"], spec["rep"], spec["lo"], spec["hi"])
    bad = np.concatenate([-2.0 * X, np.zeros_like(Y), np.zeros_like(Z)])  # F_xx = -1
    d_u = dev(bad)
    op.initialize(d_u)
    with pytest.raises(mfgpu.MfgpuError) as e:
        op.cache()
    assert e.value.code == 7
    # the context stays usable
    op.initialize(dev(u))
    op.cache()


def test_state_errors(ctx):
    spec, _ = nh_setup(1)
    m = W.to_lib_mesh(mfgpu, spec)
    op = mfgpu.NeoHookOperator(ctx, m, -1, 64, "tensor2")
    n = op.m()
    with pytest.raises(mfgpu.MfgpuError) as e:
        op.vmult(dev(np.zeros(n)), dev(np.zeros(n)))
    assert e.value.code == 6
    with pytest.raises(mfgpu.MfgpuError):
        mfgpu.NeoHookOperator(ctx, m, -1, 64, "no_such_caching")


@pytest.mark.parametrize("degree", [1, 2, 3, 5])
def test_vmult_host_buffers(ctx, degree):
    spec, u = nh_setup(degree)
    m = W.to_lib_mesh(mfgpu, spec)
    n = W.n_dofs(spec, 3)
    op = mfgpu.NeoHookOperator(ctx, m, -1, 64, "referential_qp")
    op.set_material(mfgpu.material(dt=0.01))
    d_u = dev(u)
    op.initialize(d_u)
    op.cache()
    src = W.uniform_vector(n, 9)
    out = np.zeros(n)
    op.vmult_host(out, src)
    d_dst = dev(np.zeros(n))
    op.vmult(d_dst, dev(src))
    # same operator, same inputs; the scatter's atomic adds may differ in
    # the order of summation, so compare to round-off
    assert rel(out, host(d_dst)) < 1e-14


def _pinned(n, dtype):
    import torch
    t = torch.zeros(n, dtype=torch.float64 if dtype == np.float64 else torch.float32).pin_memory()
    return t, t.numpy()


@pytest.mark.parametrize("chunks", [1, 2, 4, 5, 8])
@pytest.mark.parametrize("kind", ["nh_df64", "nh_f64", "nh_f32", "heat_f64", "heat_df64"])
def test_vmult_host_overlapped(ctx, kind, chunks):
    """The z-slab pipelined host-buffer vmult equals the oracle and the
    device vmult, for slab counts that do and do not divide the 6 cell
    layers in z (8 is clamped to 6)."""
    degree = 3
    if kind.startswith("nh"):
        spec = W.cantilever(degree, 1, rep=(2, 1, 3), length=(2.0, 1.0, 3.0))
        nc = 3
    else:
        spec = W.unit_cube_heat(degree, 1, rep=(1, 2, 3))
        nc = 1
    precision = 32 if kind.endswith("f32") else 64
    dt = np.float32 if precision == 32 else np.float64
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    n = W.n_dofs(spec, nc)
    src = W.uniform_vector(n, 21, dt)
    if nc == 3:
        u = W.smooth_displacement(degree, spec["n_ref"], spec["rep"], spec["lo"], spec["hi"], seed=4)
        op = mfgpu.NeoHookOperator(ctx, m, -1, precision, "referential_qp")
        op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01))
        d_u = dev(u if precision == 64 else u.astype(np.float32))
        op.initialize(d_u)
        ref = O.nh_vmult(om, spec["n_ref"], O.material(0.5e6, 0.4, 1000.0, 0.01),
                         "scalar_referential", u, src.astype(np.float64))
    else:
        op = mfgpu.LaplaceOperator(ctx, m, -1, precision, True, delta_t=0.1)
        ref = O.heat_vmult(om, spec["n_ref"], 0.1, src, precision=precision)
    if kind.endswith("df64"):
        op.set_fp64_emulation(True)
    if nc == 3:
        op.cache()
    op.set_host_chunks(chunks)
    src_t, src_p = _pinned(n, dt)
    dst_t, dst_p = _pinned(n, dt)
    src_p[:] = src
    tol = TOL64 if precision == 64 else 5e-5
    # first call eager, second captured into a CUDA graph, then replays
    for _ in range(4):
        dst_p[:] = np.nan
        op.vmult_host(dst_p, src_p)
        assert rel(dst_p.astype(np.float64), np.asarray(ref, np.float64)) < tol
    d_dst = dev(np.zeros(n, dt))
    op.vmult(d_dst, dev(src))
    # (the whole-grid and the per-slab launches may take different cell
    # kernels on this small mesh: summation orders differ)
    assert rel(dst_p, host(d_dst)) < (1e-13 if precision == 64 else 1e-6)
    # a new source in the same pinned buffer is picked up by the replay
    src_p[:] = -2.0 * src
    op.vmult_host(dst_p, src_p)
    assert rel(dst_p.astype(np.float64), -2.0 * np.asarray(ref, np.float64)) < tol
    # pageable buffers in between (another path through the same staging
    # buffers), then pinned again
    out_pg = np.zeros(n, dt)
    op.vmult_host(out_pg, src)
    assert rel(out_pg.astype(np.float64), np.asarray(ref, np.float64)) < tol
    op.vmult_host(dst_p, src_p)
    assert rel(dst_p.astype(np.float64), -2.0 * np.asarray(ref, np.float64)) < tol
    if nc == 1:
        # operator state that the kernels take as parameters invalidates the graph
        op.set_delta_t(0.2)
        ref2 = O.heat_vmult(om, spec["n_ref"], 0.2, -2.0 * src, precision=precision)
        for _ in range(3):
            op.vmult_host(dst_p, src_p)
            assert rel(dst_p.astype(np.float64), np.asarray(ref2, np.float64)) < tol


@pytest.mark.parametrize("kind", ["heat_f64", "heat_f32", "nh_f64", "nh_df64", "nh_f32"])
@pytest.mark.parametrize("degree,n_ref,rep", [(1, 0, (3, 3, 1)), (2, 1, (3, 1, 1)), (4, 0, (3, 2, 1))])
def test_colored_scatter(ctx, kind, degree, n_ref, rep):
    """Parity-coloured plain scatter: equal to the oracle, bitwise equal from
    run to run, equal to the atomic scatter to round-off; odd cell counts
    and empty colours included."""
    nc = 3 if kind.startswith("nh") else 1
    precision = 32 if kind.endswith("f32") else 64
    dt = np.float32 if precision == 32 else np.float64
    length = tuple(float(r) for r in rep)
    spec = W.cantilever(degree, n_ref, rep=rep, length=length) if nc == 3 \
        else W.unit_cube_heat(degree, n_ref, rep=rep)
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    n = W.n_dofs(spec, nc)
    src = W.uniform_vector(n, 31, dt)
    if nc == 3:
        u = W.smooth_displacement(degree, n_ref, spec["rep"], spec["lo"], spec["hi"], seed=5)
        op = mfgpu.NeoHookOperator(ctx, m, -1, precision, "referential_qp")
        op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01))
        d_u = dev(u if precision == 64 else u.astype(np.float32))
        op.initialize(d_u)
        if kind.endswith("df64"):
            op.set_fp64_emulation(True)
        op.cache()
        ref = O.nh_vmult(om, n_ref, O.material(0.5e6, 0.4, 1000.0, 0.01), "scalar_referential",
                         u, src.astype(np.float64))
        tol = TOL64 if precision == 64 else 5e-5
    else:
        op = mfgpu.LaplaceOperator(ctx, m, -1, precision, True, delta_t=0.1)
        ref = O.heat_vmult(om, n_ref, 0.1, src, precision=precision)
        tol = TOL64 if precision == 64 else TOL32
    d_src = dev(src)
    d_at = dev(np.zeros(n, dt))
    # the coloured scatter is a mode of the line-parallel kernel: compare
    # with the atomic scatter of the same kernel
    op.set_cell_kernel("line")
    op.vmult(d_at, d_src)
    op.set_scatter("colored")
    outs = []
    for _ in range(2):
        d = dev(np.zeros(n, dt))
        op.vmult(d, d_src)
        outs.append(host(d))
    assert rel(outs[0].astype(np.float64), np.asarray(ref, np.float64)) < tol
    assert np.array_equal(outs[0], outs[1])
    assert rel(outs[0], host(d_at)) < (1e-14 if precision == 64 else 1e-6)
    # the host-buffer call takes the same coloured path
    out_h = np.zeros(n, dt)
    op.vmult_host(out_h, src)
    assert np.array_equal(out_h, outs[0])


def test_context_outlives_its_operators():
    """A context with live operators refuses to be destroyed (ERR_STATE);
    the Python wrapper releases its operators first."""
    c = mfgpu.Context(0)
    spec = small_heat(1)
    op = mfgpu.LaplaceOperator(c, W.to_lib_mesh(mfgpu, spec), -1, 64, True, delta_t=0.1)
    assert mfgpu.lib().mfgpu_context_destroy(c.h) == 6
    c.close()
    assert op.h is None and c.h is None


def test_set_host_chunks_rejects(ctx):
    spec = small_heat(2)
    op = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 64, True, delta_t=0.1)
    with pytest.raises(mfgpu.MfgpuError):
        op.set_host_chunks(9)
    with pytest.raises(mfgpu.MfgpuError):
        op.set_host_chunks(-1)


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("nc", [1, 3])
def test_transfer(ctx, degree, nc):
    spec = W.cantilever(degree, 2, rep=(2, 1, 1), length=(2.0, 1.0, 1.0)) if nc == 3 \
        else W.unit_cube_heat(degree, 2, rep=(2, 1, 1))
    m = W.to_lib_mesh(mfgpu, spec)
    om = W.to_oracle_mesh(O, spec)
    nco = mfgpu.n_nodes(m, 0) * nc
    nf = mfgpu.n_nodes(m, 1) * nc
    coarse = W.uniform_vector(nco, 11)
    fine = W.uniform_vector(nf, 12)
    # prolongate
    ref_f = np.zeros(nf)
    O.transfer(om, 0, nc, "prolongate", coarse.copy(), ref_f)
    d_f = dev(np.zeros(nf))
    mfgpu.prolongate(ctx, m, 0, nc, dev(coarse), d_f)
    assert rel(host(d_f), ref_f) < 1e-13
    # restrict (adds into coarse)
    ref_c = coarse.copy()
    O.transfer(om, 0, nc, "restrict", ref_c, fine.copy())
    d_c = dev(coarse)
    mfgpu.restrict_add(ctx, m, 0, nc, d_c, dev(fine))
    assert rel(host(d_c), ref_c) < 1e-13
    # interpolate
    ref_i = np.zeros(nco)
    O.transfer(om, 0, nc, "interpolate", ref_i, fine.copy())
    d_i = dev(np.zeros(nco))
    mfgpu.interpolate(ctx, m, 0, nc, d_i, dev(fine))
    assert rel(host(d_i), ref_i) < 1e-13


def test_prolongation_reproduces_polynomials(ctx):
    """P interpolates: a polynomial of degree p is transferred exactly."""
    spec = W.unit_cube_heat(3, 2, rep=(2, 1, 1))
    spec["dirichlet"] = []
    m = W.to_lib_mesh(mfgpu, spec)
    f = lambda X, Y, Z: 1 + X ** 3 - 2 * X * Y ** 2 + Z ** 3 * Y ** 2
    Xc, Yc, Zc = W.node_coords(3, 0, spec["rep"], spec["lo"], spec["hi"])
    Xf, Yf, Zf = W.node_coords(3, 1, spec["rep"], spec["lo"], spec["hi"])
    d_f = dev(np.zeros(len(Xf)))
    mfgpu.prolongate(ctx, m, 0, 1, dev(f(Xc, Yc, Zc)), d_f)
    assert np.max(np.abs(host(d_f) - f(Xf, Yf, Zf))) < 1e-12


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
def test_fp64_emulation_parity(ctx, degree):
    """Double-float arithmetic on the FP32 pipe keeps the FP64 operator
    within the 1e-12 relative l2 bar against the oracle (heat and the
    referential_qp tangent)."""
    spec = small_heat(degree)
    n = W.n_dofs(spec, 1)
    src = W.uniform_vector(n, 1)
    ref = O.heat_vmult(W.to_oracle_mesh(O, spec), 1, 0.1, src)
    op = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 64, True, delta_t=0.1)
    op.set_fp64_emulation(True)
    d_dst = dev(np.zeros(n))
    op.vmult(d_dst, dev(src))
    assert rel(host(d_dst), ref) < TOL64

    spec, u = nh_setup(degree)
    n = W.n_dofs(spec, 3)
    src = W.uniform_vector(n, 3)
    ref = O.nh_vmult(W.to_oracle_mesh(O, spec), 1, O.material(dt=0.01),
                     "scalar_referential", u, src)
    op = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 64, "referential_qp")
    op.set_material(mfgpu.material(dt=0.01))
    d_u = dev(u)
    op.initialize(d_u)
    op.set_fp64_emulation(True)
    op.cache()
    d_dst = dev(np.zeros(n))
    op.vmult(d_dst, dev(src))
    assert rel(host(d_dst), ref) < TOL64
    # vmult_add on the same path
    op.vmult_add(d_dst, dev(src))
    assert rel(host(d_dst), 2 * ref) < TOL64


def test_fp64_emulation_rejects_unsupported(ctx):
    spec, _ = nh_setup(2)
    op = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 64, "tensor4")
    op.set_material(mfgpu.material(dt=0.01))
    with pytest.raises(mfgpu.MfgpuError) as e:
        op.set_fp64_emulation(True)
    assert e.value.code == 8
    op32 = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, small_heat(2)), -1, 32, True,
                                 delta_t=0.1)
    with pytest.raises(mfgpu.MfgpuError):
        op32.set_fp64_emulation(True)


DENSE_CASES = [("heat", 64, False, None), ("heat", 32, False, None), ("heat", 64, True, None),
               ("nh", 64, False, "scalar_referential"), ("nh", 64, False, "tensor4"),
               ("nh", 64, False, "tensor4_ns"), ("nh", 32, False, "tensor2"),
               ("nh", 64, True, "referential_qp"), ("nh0", 64, False, "tensor2")]


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 6])
@pytest.mark.parametrize("kind,precision,df64,caching", DENSE_CASES)
def test_dense_copy_matches_matrix_free(ctx, degree, kind, precision, df64, caching):
    """The dense copy of a coarse-level operator (element columns from unit
    vectors, constrained rows and columns as the identity) multiplies like
    the matrix-free operator, is symmetric, and is not used once the
    operator's state has changed."""
    import torch
    dt = np.float64 if precision == 64 else np.float32
    tol = 1e-13 if precision == 64 else 2e-6
    if kind == "heat":
        spec = W.unit_cube_heat(degree, 0, rep=(2, 1, 1))
        n = W.n_dofs(spec, 1)
        op = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, precision, True, delta_t=0.1)
    else:
        spec = W.cantilever(degree, 0, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
        n = W.n_dofs(spec, 3)
        u1 = W.smooth_displacement(degree, 0, spec["rep"], spec["lo"], spec["hi"], seed=2)
        op = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, precision, caching)
        op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01, 0 if kind == "nh0" else 1))
        d_u = dev(u1.astype(dt))
        op.initialize(d_u)
    if df64:
        op.set_fp64_emulation(True)
    if kind != "heat":
        op.cache()
    x = dev(W.uniform_vector(n, 5, dt))
    y = dev(W.uniform_vector(n, 6, dt))
    mf_x, dn_x, dn_y = (torch.zeros_like(x) for _ in range(3))
    op.vmult(mf_x, x)
    op.set_dense(True)
    op.vmult(dn_x, x)
    op.vmult(dn_y, y)
    ref = host(mf_x).astype(np.float64)
    assert rel(host(dn_x).astype(np.float64), ref) < tol
    # symmetric: y . A x == x . A y
    xa, ya = host(x).astype(np.float64), host(y).astype(np.float64)
    assert abs(ya @ host(dn_x) - xa @ host(dn_y)) <= tol * np.linalg.norm(ya) * np.linalg.norm(ref)
    # vmult_add on the dense copy
    op.vmult_add(dn_x, x)
    assert rel(host(dn_x).astype(np.float64), 2 * ref) < tol
    if kind != "heat":
        # a new linearisation: the stale dense copy is bypassed
        u2 = W.smooth_displacement(degree, 0, spec["rep"], spec["lo"], spec["hi"], seed=7)
        d_u.copy_(dev(u2.astype(dt)))
        op.cache()
        op.vmult(dn_x, x)
        op.set_dense(False)
        op.vmult(mf_x, x)
        assert rel(host(dn_x), host(mf_x)) == 0.0
    else:
        op.set_delta_t(0.05)
        op.vmult(dn_x, x)
        op.set_dense(False)
        op.vmult(mf_x, x)
        assert rel(host(dn_x), host(mf_x)) == 0.0
    op.close()


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("rep", [(1, 1, 1), (2, 1, 1), (3, 1, 1)])
def test_dense_copy_row_splits(ctx, precision, rep):
    """Dense copies of 1029, 1911 and 2793 rows (Q6 cantilevers of one to
    three cells) run the dense kernels with 256, 128 and 64 threads per row
    in FP32 and half as many in FP64, on rows padded to 16-byte boundaries;
    each multiplies like the matrix-free operator, also on an input vector
    that is not 16-byte aligned (read in scalars)."""
    dt = np.float64 if precision == 64 else np.float32
    tol = 1e-13 if precision == 64 else 2e-6
    spec = W.cantilever(6, 0, rep=rep, length=(float(rep[0]), 1.0, 1.0))
    n = W.n_dofs(spec, 3)
    u1 = W.smooth_displacement(6, 0, spec["rep"], spec["lo"], spec["hi"], seed=2)
    op = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, precision, "referential_qp")
    op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01))
    d_u = dev(u1.astype(dt))
    op.initialize(d_u)
    op.cache()
    x = dev(W.uniform_vector(n, 5, dt))
    mf_x, dn_x = dev(np.zeros(n, dt)), dev(np.zeros(n, dt))
    op.vmult(mf_x, x)
    op.set_dense(True)
    op.vmult(dn_x, x)
    assert rel(host(dn_x).astype(np.float64), host(mf_x).astype(np.float64)) < tol
    # the same input one element into a larger buffer: not 16-byte aligned
    xs = dev(np.concatenate([[0.0], W.uniform_vector(n, 5, dt)]).astype(dt))[1:]
    assert xs.data_ptr() % 16 != 0
    dn_xs = dev(np.zeros(n, dt))
    op.vmult(dn_xs, xs)
    assert rel(host(dn_xs).astype(np.float64), host(mf_x).astype(np.float64)) < tol
    op.close()


def test_dense_copy_rejects_large_operators(ctx):
    spec = W.unit_cube_heat(4, 2)
    op = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, 64, True, delta_t=0.1)
    with pytest.raises(mfgpu.MfgpuError, match="dense copy"):
        op.set_dense(True)
    op.close()


KERNEL_CASES = [("heat", 64, False, None), ("heat", 32, False, None), ("heat", 64, True, None),
                ("nh", 64, False, "scalar_referential"), ("nh", 32, False, "scalar_referential"),
                ("nh", 64, False, "tensor2"), ("nh", 64, False, "tensor4"), ("nh", 32, False, "tensor4_ns"),
                ("nh", 64, False, "referential_qp"), ("nh", 32, False, "referential_qp"),
                ("nh", 64, True, "referential_qp"), ("nh0", 64, False, "tensor2")]


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("kind,precision,df64,caching", KERNEL_CASES)
def test_line_and_point_kernels_agree(ctx, degree, kind, precision, df64, caching):
    """The line-parallel and the point-parallel cell kernels apply the same
    operator (constrained rows included) to round-off."""
    import torch
    dt = np.float64 if precision == 64 else np.float32
    tol = 1e-13 if precision == 64 else 3e-6
    if kind == "heat":
        spec = small_heat(degree)
        n = W.n_dofs(spec, 1)
        op = mfgpu.LaplaceOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, precision, True, delta_t=0.1)
    else:
        spec, u = nh_setup(degree)
        n = W.n_dofs(spec, 3)
        op = mfgpu.NeoHookOperator(ctx, W.to_lib_mesh(mfgpu, spec), -1, precision, caching)
        op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01, 0 if kind == "nh0" else 1))
        d_u = dev(u.astype(dt))
        op.initialize(d_u)
    if df64:
        op.set_fp64_emulation(True)
    if kind != "heat":
        op.cache()
    x = dev(W.uniform_vector(n, 9, dt))
    out = {}
    for mode in ("line", "point"):
        op.set_cell_kernel(mode)
        y = torch.zeros_like(x)
        op.vmult(y, x)
        out[mode] = host(y).astype(np.float64)
    assert rel(out["point"], out["line"]) < tol
    op.close()
