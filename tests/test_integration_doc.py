"""The C++ binding sketches in INTEGRATION.md compile against include/mfgpu.h
(syntax and template instantiation only; deal.II's Subscriptor, AssertThrow
and ExcMessage are stood in for by minimal definitions)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PRELUDE = r"""
#include <stdexcept>
#include <string>
#include <vector>
struct Subscriptor {};
inline std::runtime_error ExcMessage(const char *m) { return std::runtime_error(m); }
#define AssertThrow(cond, exc) do { if (!(cond)) throw exc; } while (0)
"""


def cpp_blocks():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```cpp\n(.*?)```", text, flags=re.S)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integration_sketches_compile(tmp_path):
    blocks = cpp_blocks()
    assert len(blocks) == 4
    perm, mg, wrapper, loop = blocks
    src = (PRELUDE + wrapper +
           "\ntemplate class NeoHookOperatorGPU<3, double>;\n"
           "template class NeoHookOperatorGPU<2, float>;\n"
           "static void check(int rc) { AssertThrow(rc == MFGPU_OK, ExcMessage(mfgpu_last_error())); }\n"
           "void solid_driver(mfgpu_context *ctx, const mfgpu_solid_params &params)\n{\n" + loop + "}\n"
           "void numbering(mfgpu_context *ctx, const mfgpu_mesh &mesh, size_t n_dofs, double *d_dealii,\n"
           "               double *d_lib)\n{\n" + perm + "mfgpu_permutation_destroy(perm);\n}\n"
           "void own_cg(mfgpu_context *ctx, const mfgpu_mesh &mesh, const mfgpu_material &mat,\n"
           "            const mfgpu_solver_params &solver_params, mfgpu_operator *op, const double *u_dev,\n"
           "            double *du_dev, const double *rhs_dev, double tol, int max_it)\n{\n" + mg + "(void)its;\n"
           "(void)res;\n}\n")
    f = tmp_path / "integration_sketch.cc"
    f.write_text(src)
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror",
                        "-I", os.path.join(ROOT, "include"), str(f)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-3000:]
