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
    return sorted(set(re.findall(r"\b(mfgpu_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_function():
    path = pkg_build.build()
    lib = ctypes.CDLL(path)
    names = declared_functions()
    assert len(names) >= 35
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
