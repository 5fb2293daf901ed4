"""The map between a caller's DoF numbering and the library's
(mfgpu_dof_permutation): deal.II numbers the reference's solid DoFs by
Cuthill-McKee (mf_elasticity.h:669) with components interleaved per support
point; the library numbers them component-blocked on the lexicographic
Gauss-Lobatto node grid.  Host-only checks here; the device map and an
operator applied in the caller's numbering are in tests/test_gpu_boundary.py."""
import ctypes

import numpy as np
import pytest

import mfgpu
import workloads as W


def caller_numbering(spec, nc, seed=5, dim=3):
    """Support points and components of a shuffled, component-interleaved
    numbering of the library's DoFs, and the library index of each."""
    if dim == 3:
        X, Y, Z = W.node_coords(spec["degree"], spec["n_ref"], spec["rep"], spec["lo"], spec["hi"])
    else:
        xs = W.axis_coords(spec["rep"][0] << spec["n_ref"], spec["lo"][0], spec["hi"][0], spec["degree"])
        ys = W.axis_coords(spec["rep"][1] << spec["n_ref"], spec["lo"][1], spec["hi"][1], spec["degree"])
        Yg, Xg = np.meshgrid(ys, xs, indexing="ij")
        X, Y, Z = Xg.ravel(), Yg.ravel(), np.zeros(Xg.size)
    nn = len(X)
    node = np.repeat(np.arange(nn), nc)          # interleaved: (node, comp) pairs
    comp = np.tile(np.arange(nc), nn)
    order = np.random.Generator(np.random.PCG64(seed)).permutation(nn * nc)
    node, comp = node[order], comp[order]
    pts = np.stack([X[node], Y[node], Z[node]], axis=1)
    return pts, comp.astype(np.uint32), comp * nn + node


@pytest.mark.parametrize("nc,degree", [(1, 2), (3, 3), (3, 1)])
def test_permutation_recovers_a_shuffled_numbering(nc, degree):
    spec = W.cantilever(degree, 1, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    mesh = W.to_lib_mesh(mfgpu, spec)
    pts, comp, expected = caller_numbering(spec, nc)
    got = mfgpu.dof_permutation(mesh, -1, pts, comp if nc > 1 else None)
    assert np.array_equal(got, expected)


def test_permutation_two_dimensional():
    spec = dict(degree=2, n_ref=1, rep=(3, 2), lo=(0.0, 0.0), hi=(1.2, 0.5))
    mesh = mfgpu.make_mesh(2, 1, (3, 2), (0.0, 0.0), (1.2, 0.5))
    pts, comp, expected = caller_numbering(spec, 2, dim=2)
    assert np.array_equal(mfgpu.dof_permutation(mesh, -1, pts, comp), expected)


def test_permutation_rejects_bad_input():
    spec = W.cantilever(2, 0, rep=(1, 1, 1), length=(1.0, 1.0, 1.0))
    mesh = W.to_lib_mesh(mfgpu, spec)
    pts, comp, _ = caller_numbering(spec, 1)
    bad = pts.copy()
    bad[3] = bad[4]  # two DoFs at one point
    with pytest.raises(mfgpu.MfgpuError, match="map to library DoF"):
        mfgpu.dof_permutation(mesh, -1, bad)
    off = pts.copy()
    off[0, 0] += 0.13  # between two nodes
    with pytest.raises(mfgpu.MfgpuError, match="not a node"):
        mfgpu.dof_permutation(mesh, -1, off)
    with pytest.raises(mfgpu.MfgpuError, match="n_dofs"):
        mfgpu.dof_permutation(mesh, -1, pts[:-1])
    with pytest.raises(mfgpu.MfgpuError, match="component"):
        mfgpu.dof_permutation(mesh, -1, pts, np.full(len(pts), 2, dtype=np.uint32))
