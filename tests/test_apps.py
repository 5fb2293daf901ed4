"""The prm-driven executables `solid` and `heat`: parameter-file handling
(CPU) and full runs on the device compared with the oracle (GPU)."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

import build as pkg_build
import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
PRM = os.path.join(HERE, "golden", "prm")
PKG = os.path.dirname(pkg_build.__file__)


def run_app(app, prm, cwd):
    pkg_build.build()
    return subprocess.run([os.path.join(PKG, app), prm], capture_output=True, text=True,
                          cwd=cwd, timeout=600)


def test_unknown_entry_is_rejected(tmp_path):
    prm = tmp_path / "bad.prm"
    prm.write_text("subsection Geometry\n  set Dimension = 3\n  set No such key = 1\nend\n")
    r = run_app("solid", str(prm), tmp_path)
    assert r.returncode == 1
    assert "unknown entry 'No such key'" in r.stderr and "Aborting!" in r.stderr


def test_invalid_dimension_is_rejected_before_device_work(tmp_path):
    txt = open(os.path.join(PRM, "turek3d_gmg_tensor4.prm")).read()
    txt = txt.replace("set Dimension          = 3", "set Dimension          = 4")
    prm = tmp_path / "t4d.prm"
    prm.write_text(txt)
    r = run_app("solid", str(prm), tmp_path)
    assert r.returncode == 1 and "Dimension must be 2 or 3" in r.stderr
    r = run_app("heat", os.path.join(PRM, "heat3d_analytic_q2.prm").replace(".prm", "_missing.prm"),
                tmp_path)
    assert r.returncode == 1 and "cannot open" in r.stderr


def turek3d_oracle(degree, n_ref, caching):
    p = O.SolidParams()
    p.mesh = O.make_mesh(3, degree, degree + 1, n_ref, (5, 1, 1), (0.24899, 0.19, -0.005),
                         (0.6, 0.21, 0.005), boundary_id=(1, 11, 11, 11, 2, 2),
                         dirichlet=[(1, 0b111), (2, 0b100)])
    p.mat = O.material(0.5e6, 0.4, 1000.0, 0.1, 1)
    p.caching = O.CACHING[caching]
    p.precond, p.relaxation, p.tol_lin, p.max_it_mult, p.max_newton = 2, 0.65, 1e-6, 1, 10
    p.tol_f, p.tol_f_abs, p.tol_u, p.tol_u_abs = 1e-9, 2e-9, 1e-6, 5e-15
    p.dt, p.n_steps = 0.1, 2
    p.body_force[:] = [0.0, -0.5, 0.0]
    p.traction_id = 11
    p.traction[:] = [0.0, -4.0, 0.0]
    p.watch[:] = [0.6, 0.2, 0.0]
    p.cheb_degree, p.cheb_range, p.cheb_eig_its, p.coarse_accurate, p.mg_float = 5, 20.0, 30, 1, 1
    return O.solid_run(p)


def parse_output(txt):
    newton = [int(x) for x in re.findall(r"Converged in (\d+) Newton", txt)]
    disp = [[float(v) for v in m.split()] for m in re.findall(r"displacement: (.+)", txt)]
    avg = int(re.search(r"Average CG iter = (\d+)", txt).group(1))
    return newton, disp, avg


@pytest.mark.gpu
@pytest.mark.parametrize("prm,degree,n_ref,caching", [
    ("turek3d_gmg_tensor4.prm", 1, 2, "tensor4"),
    ("turek3d_q2_scalar_referential.prm", 2, 1, "scalar_referential"),
])
def test_solid_executable_matches_oracle(tmp_path, prm, degree, n_ref, caching):
    r = run_app("solid", os.path.join(PRM, prm), tmp_path)
    assert r.returncode == 0, r.stderr
    folder = "turek3d_out" if degree == 1 else "turek3d_q2_out"
    newton, disp, avg = parse_output((tmp_path / folder / "output").read_text())
    ro = turek3d_oracle(degree, n_ref, caching)
    assert newton == list(ro.newton_its[:2])
    for s in range(2):
        wo = np.array(ro.watch_disp[s][:3])
        # the output file prints 6 significant digits
        assert np.allclose(disp[s], wo, rtol=1e-5, atol=1e-12), (disp[s], wo)
    assert abs(avg - ro.total_cg // ro.n_solves) <= 1
    # the last written solution: order-p Lagrange hexahedra on the displaced
    # mesh; points minus displacements lie on the equispaced sub-grid
    v = read_vtu(tmp_path / folder / "solution_000.vtu")
    cells = 5 * 8 ** n_ref
    assert v["cells"] == cells and v["points"] == cells * (degree + 1) ** 3 and set(v["types"]) == {72}
    ref = v["Points"] - v["displacement"]
    lo, hi = np.array([0.24899, 0.19, -0.005]), np.array([0.6, 0.21, 0.005])
    steps = (hi - lo) / (np.array([5, 1, 1]) * 2 ** n_ref * degree)
    g = (ref - lo) / steps
    assert np.allclose(g, np.round(g), atol=1e-8)
    assert np.abs(v["displacement"]).max() > 0


@pytest.mark.gpu
def test_heat_executable_reproduces_analytic_solution(tmp_path):
    r = run_app("heat", os.path.join(PRM, "heat3d_analytic_q2.prm"), tmp_path)
    assert r.returncode == 0, r.stderr
    errs = [float(x) for x in re.findall(r"Error: (\S+)", r.stdout)]
    assert len(errs) == 11
    assert max(errs) < 1e-11, errs


@pytest.mark.gpu
def test_solid_executable_2d_matches_reference_golden(tmp_path):
    """The reference's own 2D turek_hron case (tests/solid/turek_gmg_tensor4:
    Q1, 320 cells, 738 DoFs) through the prm-driven executable."""
    g = json.load(open(os.path.join(HERE, "golden", "reference_goldens.json")))["solid"]["turek_gmg_tensor4"]
    r = run_app("solid", os.path.join(PRM, "turek2d_gmg_tensor4.prm"), tmp_path)
    assert r.returncode == 0, r.stderr
    assert "Number of degrees of freedom: %d" % g["n_dofs"] in r.stdout, r.stdout
    newton, disp, avg = parse_output((tmp_path / "turek2d_out" / "output").read_text())
    assert newton == g["newton_its"]
    for s in range(2):
        assert len(disp[s]) == 2
        assert np.allclose(disp[s], g["watch_disp"][s], rtol=6e-6, atol=0), (disp[s], g["watch_disp"][s])
    assert abs(avg - g["avg_cg"]) <= 1


@pytest.mark.gpu
def test_heat_executable_2d_reproduces_analytic_solution(tmp_path):
    r = run_app("heat", os.path.join(PRM, "heat2d_analytic_q2.prm"), tmp_path)
    assert r.returncode == 0, r.stderr
    assert "dim       = 2" in r.stdout and "Number of active cells: 64" in r.stdout
    errs = [float(x) for x in re.findall(r"Error: (\S+)", r.stdout)]
    assert len(errs) == 11
    assert max(errs) < 1e-11, errs


def read_vtu(path):
    """Arrays of a VTK XML UnstructuredGrid file with raw appended data
    (UInt64 block headers): {name: numpy array}, plus NumberOfPoints/Cells."""
    data = open(path, "rb").read()
    head, _, tail = data.partition(b'<AppendedData encoding="raw">')
    raw = tail[tail.index(b"_") + 1:]
    text = head.decode()
    out = {"points": int(re.search(r'NumberOfPoints="(\d+)"', text).group(1)),
           "cells": int(re.search(r'NumberOfCells="(\d+)"', text).group(1))}
    dtypes = {"Float64": np.float64, "Float32": np.float32, "Int64": np.int64, "UInt8": np.uint8}
    for m in re.finditer(r'<DataArray ([^>]*)/>', text):
        attrs = dict(re.findall(r'(\w+)="([^"]*)"', m.group(1)))
        off = int(attrs["offset"])
        nbytes = int(np.frombuffer(raw[off:off + 8], dtype=np.uint64)[0])
        arr = np.frombuffer(raw[off + 8:off + 8 + nbytes], dtype=dtypes[attrs["type"]])
        ncomp = int(attrs.get("NumberOfComponents", "1"))
        out[attrs.get("Name", "Points")] = arr.reshape(-1, ncomp) if ncomp > 1 else arr
    return out


@pytest.mark.gpu
def test_heat_executable_writes_vtu(tmp_path):
    """Output solution = true: solution_000.vtu .. solution_010.vtu (every
    0.1 of the 1 s run) hold the Q2 field on order-2 Lagrange quadrilaterals;
    the analytic solution 1 + x^2 + 3 y^2 + 1.3 t is quadratic, so every
    written point value equals it."""
    txt = open(os.path.join(PRM, "heat2d_analytic_q2.prm")).read()
    txt = txt.replace("set Output solution = false", "set Output solution = true")
    prm = tmp_path / "h.prm"
    prm.write_text(txt)
    r = run_app("heat", str(prm), tmp_path)
    assert r.returncode == 0, r.stderr
    for k in (0, 5, 10):
        v = read_vtu(tmp_path / "heat2d_out" / ("solution_%03d.vtu" % k))
        assert v["cells"] == 64 and v["points"] == 64 * 9
        assert set(v["types"]) == {70} and list(v["offsets"][:2]) == [9, 18]
        x, y = v["Points"][:, 0], v["Points"][:, 1]
        exact = 1 + x ** 2 + 3 * y ** 2 + 1.3 * 0.1 * k
        assert np.max(np.abs(v["solution"] - exact)) < 1e-10, k
        assert np.all(v["owner"] == 0)


@pytest.mark.gpu
def test_solid_executable_writes_vtu(tmp_path):
    """The solid executable writes the displacement on the displaced mesh:
    every point is its reference position plus its displacement, and the
    point at the watch vertex carries the displacement of the output file."""
    txt = open(os.path.join(PRM, "turek2d_gmg_tensor4.prm")).read()
    txt = txt.replace("set Output tick     = 1", "set Output tick     = 0.1")
    prm = tmp_path / "t.prm"
    prm.write_text(txt)
    r = run_app("solid", str(prm), tmp_path)
    assert r.returncode == 0, r.stderr
    newton, disp, avg = parse_output((tmp_path / "turek2d_out" / "output").read_text())
    for k in (0, 1, 2):
        v = read_vtu(tmp_path / "turek2d_out" / ("solution_%03d.vtu" % k))
        assert v["cells"] == 320 and v["points"] == 320 * 4 and set(v["types"]) == {70}
        d = v["displacement"]
        ref = v["Points"] - d  # reference positions
        # Q1: the points are the cell vertices of the 40 x 8 grid on [0.24899, 0.6] x [0.19, 0.21]
        ix = (ref[:, 0] - 0.24899) / ((0.6 - 0.24899) / 40)
        iy = (ref[:, 1] - 0.19) / (0.02 / 8)
        assert np.allclose(ix, np.round(ix), atol=1e-9) and np.allclose(iy, np.round(iy), atol=1e-9)
        assert np.all(d[:, 2] == 0) and np.all(v["manifold_id"] == np.float32(4294967295.0))
        if k == 0:
            assert np.all(d == 0)
        else:
            at = np.where((np.abs(ref[:, 0] - 0.6) < 1e-9) & (np.abs(ref[:, 1] - 0.2) < 1e-9))[0]
            assert len(at) >= 1
            assert np.allclose(d[at[0], :2], disp[k - 1], rtol=1e-5, atol=0), (d[at[0]], disp[k - 1])


def test_vtk_lagrange_point_orders_are_permutations(tmp_path):
    """The VTK point orders of the written Lagrange cells (app/vtu.h) are
    permutations of the (p+1)^3 / (p+1)^2 cell points, with the corners
    first in VTK's vertex order."""
    src = tmp_path / "idx.cc"
    src.write_text('''
#include "vtu.h"
#include <cstdio>
#include <set>
int main()
{
  for (int p = 1; p <= 6; ++p)
    {
      std::set<int> h, q;
      for (int k = 0; k <= p; ++k)
        for (int j = 0; j <= p; ++j)
          for (int i = 0; i <= p; ++i)
            h.insert(mfapp::vtk_hex_index(i, j, k, p));
      for (int j = 0; j <= p; ++j)
        for (int i = 0; i <= p; ++i)
          q.insert(mfapp::vtk_quad_index(i, j, p));
      const int n3 = (p + 1) * (p + 1) * (p + 1), n2 = (p + 1) * (p + 1);
      const bool ok = int(h.size()) == n3 && *h.rbegin() == n3 - 1 && int(q.size()) == n2 &&
                      *q.rbegin() == n2 - 1 && mfapp::vtk_hex_index(p, p, 0, p) == 2 &&
                      mfapp::vtk_hex_index(0, p, p, p) == 7 && mfapp::vtk_quad_index(0, p, p) == 3;
      std::printf("%d %d\\n", p, ok ? 1 : 0);
    }
}
''')
    exe = tmp_path / "idx"
    app = os.path.join(PKG, "app")
    r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(os.path.dirname(PKG), "include"), "-I", app,
                        str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()
    assert out == [str(v) for p in range(1, 7) for v in (p, 1)]


def test_gpu_entries_are_checked_before_device_work(tmp_path):
    """The GPU section's entries (here the dense coarse operator switch)
    are parsed with the rest of the file: a bad value stops the run before
    any device work."""
    txt = open(os.path.join(PRM, "turek3d_gmg_tensor4.prm")).read()
    txt += "\nsubsection GPU\n  set Dense coarse operator = maybe\nend\n"
    prm = tmp_path / "g.prm"
    prm.write_text(txt)
    r = run_app("solid", str(prm), tmp_path)
    assert r.returncode == 1
    assert "Dense coarse operator is not a bool: maybe" in r.stderr


def test_timing_table_parser():
    """mfgpu.timing_table reads the drivers' section table."""
    import mfgpu
    text = """+------------------------------+-----------+------------+------------+
| Total wallclock time elapsed |           |    0.0436s |            |
+------------------------------+-----------+------------+------------+
| Section                      | no. calls |  wall time | % of total |
+------------------------------+-----------+------------+------------+
| Setup MF: cache()            |         2 |  0.000953s |       2.2% |
| Linear solver                |         1 |    0.0275s |        63% |
+------------------------------+-----------+------------+------------+
"""
    assert mfgpu.timing_table(text) == {"Setup MF: cache()": (2, 0.000953), "Linear solver": (1, 0.0275)}
