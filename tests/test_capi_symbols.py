"""The C-ABI library builds, loads without a GPU, and exports every entry
point declared in include/mfgpu.h (no compute calls here)."""
import ctypes
import os
import re

import build as pkg_build
import mfgpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "mfgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mfgpu_[A-Za-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_function():
    path = pkg_build.build()
    lib = ctypes.CDLL(path)
    names = declared_functions()
    assert len(names) >= 59
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_without_gpu_call_paths():
    lib = mfgpu.lib()
    assert lib.mfgpu_version() == 100
    # argument validation happens before any device work
    n = ctypes.c_size_t()
    m = mfgpu.make_mesh(2, 1, (1, 1, 1), (0, 0, 0), (1, 1, 1))
    assert lib.mfgpu_mesh_n_nodes(ctypes.byref(m), -1, ctypes.byref(n)) == 0
    assert n.value == 5 ** 3
    bad = mfgpu.make_mesh(9, 1, (1, 1, 1), (0, 0, 0), (1, 1, 1))
    rc = lib.mfgpu_mesh_n_nodes(ctypes.byref(bad), -1, ctypes.byref(n))
    assert rc == 8  # MFGPU_ERR_UNSUPPORTED
    assert b"degree" in lib.mfgpu_last_error()
    assert lib.mfgpu_operator_vmult(None, None, None) == 1


_NULL_CHECK = r'''
import ctypes, re, sys
sys.path[:0] = sys.argv[2:]
import mfgpu
lib = mfgpu.lib()
lib.mfgpu_last_error.restype = ctypes.c_char_p
src = open(sys.argv[1]).read()
src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
src = re.sub(r"//[^\n]*", "", src)
kinds = {"int": ctypes.c_int, "double": ctypes.c_double, "size_t": ctypes.c_size_t,
         "long long": ctypes.c_longlong}
for m in re.finditer(r"\b(mfgpu_[A-Za-z0-9_]+)\s*\(([^)]*)\)\s*;", src):
    name = m.group(1)
    params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
    if not any("*" in p for p in params):
        continue
    types = [ctypes.c_void_p if "*" in p else kinds[p.rsplit(" ", 1)[0]] for p in params]
    f = getattr(lib, name)
    f.restype, f.argtypes = ctypes.c_int, types
    lib.mfgpu_mesh_n_nodes(None, 0, None)  # leaves a different message behind
    rc = f(*[None if t is ctypes.c_void_p else t(0) for t in types])
    print(name, rc, (lib.mfgpu_last_error() or b"").decode())
'''


def test_every_entry_rejects_null_handles():
    """Every entry point that takes a pointer, called with null pointers and
    zero scalars, returns MFGPU_ERR_ARG with a message (destroy functions
    accept null and return MFGPU_OK); none dereferences a null handle. Run in
    a child process so that a crash fails the test instead of the session."""
    import subprocess
    import sys

    r = subprocess.run(
        [sys.executable, "-c", _NULL_CHECK, os.path.join(ROOT, "include", "mfgpu.h"),
         os.path.join(ROOT, "matrix-free-dealii-precice_gb300"), ROOT],
        capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = [line.split(" ", 2) for line in r.stdout.splitlines()]
    assert len(rows) >= 56
    for row in rows:
        name, rc = row[0], int(row[1])
        msg = row[2] if len(row) > 2 else ""
        if name.endswith("_destroy"):
            assert rc == 0, name
        else:
            assert rc == 1, (name, rc)
            assert msg and (name == "mfgpu_mesh_n_nodes" or "mesh" not in msg), (name, msg)


def test_mesh_validation_edge_cases():
    """Degenerate and out-of-range meshes are rejected with a reason before
    any device work: no cells, inverted boxes, degrees outside 1..6,
    refinement counts out of range, unknown dimensions, levels beyond the
    hierarchy, too many Dirichlet entries."""
    lib = mfgpu.lib()
    lib.mfgpu_last_error.restype = ctypes.c_char_p
    n = ctypes.c_size_t()

    def rc_of(m, level=-1):
        return lib.mfgpu_mesh_n_nodes(ctypes.byref(m), level, ctypes.byref(n))

    bad = [mfgpu.make_mesh(2, 0, (0, 1, 1), (0, 0, 0), (1, 1, 1)),
           mfgpu.make_mesh(2, 0, (-1, 1, 1), (0, 0, 0), (1, 1, 1)),
           mfgpu.make_mesh(2, 0, (1, 1, 1), (0, 0, 0), (-1, 1, 1)),
           mfgpu.make_mesh(2, -1, (1, 1, 1), (0, 0, 0), (1, 1, 1)),
           mfgpu.make_mesh(2, 40, (1, 1, 1), (0, 0, 0), (1, 1, 1))]
    for m in bad:
        assert rc_of(m) == 1 and lib.mfgpu_last_error()
    for degree in (0, 7):
        assert rc_of(mfgpu.make_mesh(degree, 0, (1, 1, 1), (0, 0, 0), (1, 1, 1))) == 8
    m = mfgpu.make_mesh(2, 0, (1, 1, 1), (0, 0, 0), (1, 1, 1))
    m.dim = 4
    assert rc_of(m) == 1 and b"dim" in lib.mfgpu_last_error()
    m = mfgpu.make_mesh(2, 1, (1, 1, 1), (0, 0, 0), (1, 1, 1))
    assert rc_of(m, 5) == 1 and b"level" in lib.mfgpu_last_error()
    m.n_dirichlet = 9
    assert rc_of(m) == 1 and b"n_dirichlet" in lib.mfgpu_last_error()
    # the largest degree on one cell, and a 2D mesh
    assert rc_of(mfgpu.make_mesh(6, 0, (1, 1, 1), (0, 0, 0), (1, 1, 1))) == 0 and n.value == 7 ** 3
    assert rc_of(mfgpu.make_mesh(3, 1, (2, 1), (0, 0), (1, 1))) == 0 and n.value == 13 * 7
