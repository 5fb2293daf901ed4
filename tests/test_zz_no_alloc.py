"""The prolongation entry point that allocates no device memory.

Some callers of this library may not allocate GPU memory while they run: a
coupled solver whose partner code's memory pool already holds the device,
a time loop that must not stall on cudaMalloc/cudaFree, or a deployment
that forbids allocation after start-up.  mfgpu_transfer_prolongate_noalloc
serves them with a static 4 MiB device scratch.  These tests call it
through the C-ABI and check, on two calls in a row, that:
  * it gives the same fine vector as mfgpu_transfer_prolongate (the same
    1e-13 relative tolerance as the other transfer tests; 1e-6 in FP32);
  * it leaves the device's free memory unchanged;
  * it rejects levels larger than the scratch with MFGPU_ERR_ARG.
Meshes are three- and two-dimensional (a single node plane in z).
This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

import mfgpu
import workloads as W

pytestmark = pytest.mark.gpu


def _call_noalloc(mesh, coarse_level, nc, precision, coarse, fine):
    return mfgpu.lib().mfgpu_transfer_prolongate_noalloc(
        ctypes.byref(mesh), coarse_level, nc, precision,
        ctypes.c_void_p(coarse.data_ptr()), ctypes.c_void_p(fine.data_ptr()), None)


def _mesh(kind, degree):
    if kind == "cantilever":
        return W.to_lib_mesh(mfgpu, W.cantilever(degree, 2, rep=(2, 1, 1),
                                                 length=(2.0, 1.0, 1.0)))
    if kind == "heat":
        return W.to_lib_mesh(mfgpu, W.unit_cube_heat(degree, 2, rep=(2, 1, 1)))
    if kind == "heat2d":
        # two-dimensional box, Dirichlet on x = 0 (one component)
        return mfgpu.make_mesh(degree, 2, (3, 2), (0.0, 0.0), (1.2, 0.5),
                               boundary_id=(1, 0, 0, 0), dirichlet=[(1, 1)])
    # "beam2d": the 2D flap shape, both components clamped at x = 0
    return mfgpu.make_mesh(degree, 2, (5, 1), (0.24899, 0.19), (0.6, 0.21),
                           boundary_id=(1, 11, 11, 11), dirichlet=[(1, 0b11)])


@pytest.mark.parametrize("kind,degree,nc,precision", [
    ("cantilever", 2, 3, 64),
    ("cantilever", 3, 3, 32),
    ("heat", 4, 1, 64),
    ("heat2d", 2, 1, 64),
    ("heat2d", 2, 1, 32),
    ("beam2d", 2, 2, 64),
    ("beam2d", 2, 2, 32),
])
def test_noalloc_prolongation_matches_allocating_entry_point(ctx, kind, degree, nc,
                                                             precision):
    import torch
    mesh = _mesh(kind, degree)
    dt = torch.float64 if precision == 64 else torch.float32
    tol = 1e-13 if precision == 64 else 1e-6
    nco = mfgpu.n_nodes(mesh, 0) * nc
    nf = mfgpu.n_nodes(mesh, 1) * nc
    free_before = None
    for call, seed in enumerate((21, 22)):
        coarse = torch.from_numpy(W.uniform_vector(nco, seed)).to("cuda", dt)
        ref = torch.zeros(nf, dtype=dt, device="cuda")
        mfgpu.prolongate(ctx, mesh, 0, nc, coarse, ref, precision=precision)
        out = torch.full((nf,), float("nan"), dtype=dt, device="cuda")
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        rc = _call_noalloc(mesh, 0, nc, precision, coarse, out)
        assert rc == 0, mfgpu.lib().mfgpu_last_error()
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        a = out.double().cpu().numpy()
        b = ref.double().cpu().numpy()
        assert np.all(np.isfinite(a))
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < tol, (call, seed)


def test_noalloc_rejects_levels_beyond_the_scratch(ctx):
    import torch
    spec = W.cantilever(4, 3)  # fine level 64x8x8 cells, Q4: far beyond 4 MiB
    mesh = W.to_lib_mesh(mfgpu, spec)
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = _call_noalloc(mesh, 2, 3, 64, dummy, dummy)
    assert rc == 1  # MFGPU_ERR_ARG
    assert b"static scratch" in mfgpu.lib().mfgpu_last_error()
