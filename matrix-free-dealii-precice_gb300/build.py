"""Build libmfgpu.so in-tree with nvcc for sm_103a.

The cell kernels are instantiated once per degree (N = p+1 = 2..7) in
separate translation units so that they compile in parallel; the host
layer is four more translation units.  Output: <package>/libmfgpu.so.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmfgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
         "-diag-suppress", "550,177"]
HOST_TUS = ["mf_ops", "mf_solvers", "mf_drivers", "mf_capi", "mf_capi_solvers", "mf_noalloc", "mf_serve",
            "mf_kernels2d", "mf_heat_em", "mf_heat_tp"]
DEGREE_NS = [2, 3, 4, 5, 6, 7]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    app = os.path.join(HERE, "app")
    if os.path.isdir(app):
        files += [os.path.join(app, f) for f in os.listdir(app)]
    return max(os.path.getmtime(f) for f in files)


def _header_mtime():
    inc = os.path.join(os.path.dirname(HERE), "include", "mfgpu.h")
    return os.path.getmtime(inc) if os.path.exists(inc) else 0.0


def build(force=False, verbose=False, jobs=None):
    """Compile (if stale) and return the path of libmfgpu.so."""
    newest = max(_sources_mtime(), _header_mtime(), os.path.getmtime(__file__))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    jobs_list = []
    for tu in HOST_TUS:
        jobs_list.append(([nvcc] + FLAGS + ARCH + ["-c", os.path.join(CSRC, tu + ".cu"),
                                                   "-o", os.path.join(BUILD, tu + ".o")],
                          os.path.join(BUILD, tu + ".o")))
    for n in DEGREE_NS:
        obj = os.path.join(BUILD, f"mf_kernels_N{n}.o")
        jobs_list.append(([nvcc] + FLAGS + ARCH + [f"-DMF_N={n}", "-c",
                                                   os.path.join(CSRC, "mf_kernels.cu"),
                                                   "-o", obj], obj))
    njobs = jobs or min(len(jobs_list), max(2, os.cpu_count() or 2))

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(njobs) as ex:
        list(ex.map(run, [c for c, _ in jobs_list]))
    objs = [o for _, o in jobs_list]
    tmp = LIB + ".tmp"
    run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    build_apps(verbose=verbose)
    return LIB


APPS = ["solid", "heat"]


def build_apps(verbose=False):
    """The prm-driven executables `solid` and `heat` (host C++ over the
    C-ABI, linked against libmfgpu.so with an $ORIGIN rpath)."""
    inc = os.path.join(os.path.dirname(HERE), "include")
    for app in APPS:
        out = os.path.join(HERE, app)
        cmd = ["g++", "-O2", "-std=c++17", "-I", inc, os.path.join(HERE, "app", app + ".cc"),
               "-L", HERE, "-lmfgpu", "-Wl,-rpath,$ORIGIN", "-o", out + ".tmp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("g++ failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        os.replace(out + ".tmp", out)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
