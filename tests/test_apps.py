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
