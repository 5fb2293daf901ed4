"""CPU ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes binding of the oracle library (the C++ CPU restatement of the
reference's matrix-free path, built from oracle/*.cpp into
oracle/_build/liboracle.so).  Imported only by tests/, by
__graft_entry__.smoke() and by the CPU-baseline leg of bench.py, always as
the CPU computation the device results are compared with; the product never
imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
SOURCES = ["oracle_capi.cpp", "oracle_fast.cpp", "oracle_core.hpp", "oracle_ops.hpp",
           "oracle_fast.hpp", "oracle_fast_api.hpp", "oracle_solvers.hpp", "oracle_problems.hpp"]
FAST_LANES = (2, 4, 8)
FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-fPIC", "-Wno-psabi"]


def build(force=False):
    """Compile the oracle with g++ (portable flags: no -march=native): the
    main unit and one unit per lane count and scalar type of the throughput
    form, compiled in parallel, then linked."""
    bdir = os.path.join(HERE, "_build")
    os.makedirs(bdir, exist_ok=True)
    newest = max(os.path.getmtime(os.path.join(HERE, s)) for s in SOURCES)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    units = [(os.path.join(HERE, "oracle_capi.cpp"), os.path.join(bdir, "capi.o"), [])]
    units += [(os.path.join(HERE, "oracle_fast.cpp"), os.path.join(bdir, f"fast_w{w}d.o"), [f"-DORC_FAST_W={w}"])
              for w in FAST_LANES]
    units += [(os.path.join(HERE, "oracle_fast.cpp"), os.path.join(bdir, "fast_w4f.o"),
               ["-DORC_FAST_W=4", "-DORC_FAST_T=float", "-DORC_FAST_TS=f"])]
    procs = [(subprocess.Popen(["g++", *FLAGS, *d, "-c", src, "-o", obj]), src) for src, obj, d in units]
    failed = [src for p, src in procs if p.wait() != 0]
    if failed:
        raise subprocess.CalledProcessError(1, f"g++ {' '.join(failed)}")
    subprocess.check_call(["g++", "-shared", "-fopenmp", *[obj for _, obj, _ in units], "-o", LIB_PATH + ".tmp"])
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


class Mesh(C.Structure):
    _fields_ = [("dim", C.c_int), ("degree", C.c_int), ("n_q", C.c_int),
                ("n_ref", C.c_int), ("rep", C.c_int * 3),
                ("lo", C.c_double * 3), ("hi", C.c_double * 3),
                ("boundary_id", C.c_int * 6), ("n_dirichlet", C.c_int),
                ("dirichlet_id", C.c_int * 8),
                ("dirichlet_mask", C.c_uint * 8)]


class Material(C.Structure):
    _fields_ = [("mu", C.c_double), ("nu", C.c_double), ("rho", C.c_double),
                ("alpha_1", C.c_double), ("formulation", C.c_int)]


class SolidParams(C.Structure):
    _fields_ = [("mesh", Mesh), ("mat", Material), ("caching", C.c_int),
                ("precond", C.c_int), ("relaxation", C.c_double),
                ("tol_lin", C.c_double), ("max_it_mult", C.c_int),
                ("max_newton", C.c_int), ("tol_f", C.c_double),
                ("tol_f_abs", C.c_double), ("tol_u", C.c_double),
                ("tol_u_abs", C.c_double), ("dt", C.c_double),
                ("n_steps", C.c_int), ("body_force", C.c_double * 3),
                ("traction_id", C.c_int), ("traction", C.c_double * 3),
                ("watch", C.c_double * 3), ("cheb_degree", C.c_int),
                ("cheb_range", C.c_double), ("cheb_eig_its", C.c_int),
                ("coarse_accurate", C.c_int), ("mg_float", C.c_int), ("fast", C.c_int)]


class SolidResult(C.Structure):
    _fields_ = [("newton_its", C.c_int * 64),
                ("watch_disp", (C.c_double * 3) * 64),
                ("total_cg", C.c_long), ("n_solves", C.c_int),
                ("n_steps", C.c_int), ("ok", C.c_int),
                ("seconds", C.c_double)]


class HeatParams(C.Structure):
    _fields_ = [("mesh", Mesh), ("dt", C.c_double), ("n_steps", C.c_int),
                ("tol_rel", C.c_double), ("precond", C.c_int),
                ("analytic", C.c_int), ("alpha", C.c_double),
                ("beta", C.c_double), ("n_gauss", C.c_int),
                ("g_center", (C.c_double * 3) * 8),
                ("g_width", C.c_double * 8), ("g_amp", C.c_double * 8),
                ("mg_float", C.c_int), ("fast", C.c_int)]


class HeatResult(C.Structure):
    _fields_ = [("l2_error", C.c_double * 64), ("cg_its", C.c_int * 64),
                ("n_steps", C.c_int), ("seconds", C.c_double)]


CACHING = {"scalar_referential": 0, "tensor2": 1, "tensor4": 2,
           "tensor4_ns": 3}

_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _lib.or_n_nodes.restype = C.c_long
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def make_mesh(dim, degree, n_q, n_ref, rep, lo, hi, boundary_id=(0,) * 6,
              dirichlet=()):
    """dirichlet: iterable of (boundary_id, component_mask)."""
    m = Mesh()
    m.dim, m.degree, m.n_q, m.n_ref = dim, degree, n_q, n_ref
    for d in range(3):
        m.rep[d] = rep[d] if d < len(rep) else 1
        m.lo[d] = lo[d] if d < len(lo) else 0.0
        m.hi[d] = hi[d] if d < len(hi) else 1.0
    for f in range(6):
        m.boundary_id[f] = boundary_id[f] if f < len(boundary_id) else -1
    m.n_dirichlet = len(dirichlet)
    for i, (bid, mask) in enumerate(dirichlet):
        m.dirichlet_id[i] = bid
        m.dirichlet_mask[i] = mask
    return m


def n_nodes(mesh, level):
    return int(lib().or_n_nodes(C.byref(mesh), level))


def basis(degree, n_q):
    N = degree + 1
    S = np.zeros((n_q, N)); G = np.zeros((n_q, N))
    nodes = np.zeros(N); xq = np.zeros(n_q); wq = np.zeros(n_q)
    lib().or_basis(degree, n_q, _ptr(S), _ptr(G), _ptr(nodes), _ptr(xq), _ptr(wq))
    return dict(S=S, G=G, nodes=nodes, xq=xq, wq=wq)


def _dt(precision):
    return np.float32 if precision == 32 else np.float64


def heat_vmult(mesh, level, k_dt, src, precision=64, constrained=True):
    src = np.ascontiguousarray(src, dtype=_dt(precision))
    dst = np.zeros_like(src)
    lib().or_heat_vmult(C.byref(mesh), level, C.c_double(k_dt),
                        int(constrained), precision, _ptr(src), _ptr(dst))
    return dst


def heat_vmult_timed(mesh, level, k_dt, src, reps):
    """(dst, seconds) of `reps` FP64 heat vmults after one untimed one."""
    src = np.ascontiguousarray(src, dtype=np.float64)
    dst = np.zeros_like(src)
    secs = C.c_double()
    lib().or_heat_vmult_timed(C.byref(mesh), level, C.c_double(k_dt), _ptr(src), _ptr(dst), int(reps),
                              C.byref(secs))
    return dst, secs.value


def heat_vmult_fast_timed(mesh, level, k_dt, src, reps, lanes=2):
    """(dst, seconds) of the throughput form of the FP64 heat vmult (cell
    batches of `lanes` cells across SIMD lanes, compile-time degree, even-odd
    collocation sweeps; 3D, n_q = p + 1): one untimed application, then
    `reps` timed."""
    src = np.ascontiguousarray(src, dtype=np.float64)
    dst = np.zeros_like(src)
    secs = C.c_double()
    rc = lib().or_heat_vmult_fast_timed(C.byref(mesh), level, C.c_double(k_dt), int(lanes), _ptr(src),
                                        _ptr(dst), int(reps), C.byref(secs))
    if rc != 0:
        raise RuntimeError(f"oracle heat_vmult_fast_timed failed: {rc}")
    return dst, secs.value


def heat_inv_diagonal(mesh, level, k_dt, precision=64):
    out = np.zeros(n_nodes(mesh, level), dtype=_dt(precision))
    lib().or_heat_inv_diagonal(C.byref(mesh), level, C.c_double(k_dt),
                               precision, _ptr(out))
    return out


def material(mu=0.5e6, nu=0.4, rho=1000.0, dt=0.01, formulation=1,
             beta=0.25):
    m = Material()
    m.mu, m.nu, m.rho = mu, nu, rho
    m.alpha_1 = 1.0 / (beta * dt * dt)
    m.formulation = formulation
    return m


def nh_vmult(mesh, level, mat, caching, u, src, precision=64):
    dt = _dt(precision)
    u = np.ascontiguousarray(u, dtype=dt)
    src = np.ascontiguousarray(src, dtype=dt)
    dst = np.zeros_like(src)
    rc = lib().or_nh_vmult(C.byref(mesh), level, C.byref(mat),
                           CACHING.get(caching, caching), precision, _ptr(u),
                           _ptr(src), _ptr(dst))
    if rc != 0:
        raise RuntimeError(f"oracle nh_vmult failed: {rc}")
    return dst


def nh_vmult_timed(mesh, level, mat, caching, u, src, reps, warmup=1):
    """(dst, seconds): the tangent cached once, `warmup` untimed FP64
    applications, then `reps` applications timed without the cache."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    src = np.ascontiguousarray(src, dtype=np.float64)
    dst = np.zeros_like(src)
    secs = C.c_double()
    rc = lib().or_nh_vmult_timed(C.byref(mesh), level, C.byref(mat), CACHING.get(caching, caching),
                                 _ptr(u), _ptr(src), _ptr(dst), int(warmup), int(reps), C.byref(secs))
    if rc != 0:
        raise RuntimeError(f"oracle nh_vmult_timed failed: {rc}")
    return dst, secs.value


def nh_vmult_fast_timed(mesh, level, mat, caching, u, src, reps, lanes=8, warmup=1):
    """(dst, seconds) of the throughput form of the FP64 tangent vmult
    (cell batches of `lanes` = 2, 4 or 8 cells across SIMD lanes, compile-time
    degree, even-odd collocation sweeps; 3D, n_q = p + 1, formulation 1, any
    caching variant): cached once, applied `warmup` times untimed, then
    `reps` applications timed."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    src = np.ascontiguousarray(src, dtype=np.float64)
    dst = np.zeros_like(src)
    secs = C.c_double()
    rc = lib().or_nh_vmult_fast_timed(C.byref(mesh), level, C.byref(mat), CACHING.get(caching, caching),
                                      int(lanes), _ptr(u), _ptr(src), _ptr(dst), int(warmup), int(reps),
                                      C.byref(secs))
    if rc != 0:
        raise RuntimeError(f"oracle nh_vmult_fast_timed failed: {rc}")
    return dst, secs.value


def nh_residual(mesh, level, mat, u, acc):
    """-int P(F(u)):grad v - rho int acc.v on the unconstrained rows (FP64)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    acc = np.ascontiguousarray(acc, dtype=np.float64)
    out = np.zeros_like(u)
    rc = lib().or_nh_residual(C.byref(mesh), level, C.byref(mat), _ptr(u), _ptr(acc), _ptr(out))
    if rc != 0:
        raise RuntimeError(f"or_nh_residual failed ({rc})")
    return out


def nh_inv_diagonal(mesh, level, mat, caching, u, precision=64):
    dt = _dt(precision)
    u = np.ascontiguousarray(u, dtype=dt)
    out = np.zeros_like(u)
    rc = lib().or_nh_inv_diagonal(C.byref(mesh), level, C.byref(mat),
                                  CACHING.get(caching, caching), precision,
                                  _ptr(u), _ptr(out))
    if rc != 0:
        raise RuntimeError(f"oracle nh_inv_diagonal failed: {rc}")
    return out


def transfer(mesh, coarse_level, nc, op, coarse, fine):
    """op: 'prolongate' (fine = P coarse), 'restrict' (coarse += P^T fine),
    'interpolate' (coarse = fine at coarse nodes). Arrays modified in place."""
    code = {"prolongate": 0, "restrict": 1, "interpolate": 2}[op]
    assert coarse.dtype == np.float64 and fine.dtype == np.float64
    lib().or_transfer(C.byref(mesh), coarse_level, nc, code, _ptr(coarse),
                      _ptr(fine))


def solid_run(params, return_u=False):
    res = SolidResult()
    n = n_nodes(params.mesh, params.mesh.n_ref) * params.mesh.dim
    u = np.zeros(n) if return_u else None
    rc = lib().or_solid_run(C.byref(params), C.byref(res),
                            _ptr(u) if return_u else None)
    if rc != 0:
        raise RuntimeError(f"oracle solid_run failed: {rc}")
    return (res, u) if return_u else res


def solid_first_solve(params, tol):
    """The first Newton system from rest, set up and solved to tol * |rhs|:
    (cg_iterations, setup_seconds, solve_seconds, du).  params.fast = 1
    routes every operator through the throughput form."""
    n = params.mesh.dim * n_nodes(params.mesh, params.mesh.n_ref)
    du = np.zeros(n)
    its, t_setup, t_solve = C.c_int(), C.c_double(), C.c_double()
    rc = lib().or_solid_first_solve(C.byref(params), C.c_double(tol), C.byref(its), C.byref(t_setup),
                                    C.byref(t_solve), _ptr(du))
    if rc != 0:
        raise RuntimeError(f"oracle solid_first_solve failed: {rc}")
    return its.value, t_setup.value, t_solve.value, du


def heat_run(params, return_u=False):
    res = HeatResult()
    n = n_nodes(params.mesh, params.mesh.n_ref)
    u = np.zeros(n) if return_u else None
    rc = lib().or_heat_run(C.byref(params), C.byref(res),
                           _ptr(u) if return_u else None)
    if rc != 0:
        raise RuntimeError(f"oracle heat_run failed: {rc}")
    return (res, u) if return_u else res


def set_threads(n):
    return int(lib().or_set_threads(int(n)))


# ---------------------------------------------------------------------------
# reference test cases restated as parameter sets
# ---------------------------------------------------------------------------

def turek_params(caching="tensor4", precond="gmg", formulation=1):
    """2D turek_hron beam of tests/solid/*/ *.prm: Q1, QGauss(2), 3
    refinements of a 5x1 box [0.24899,0.6]x[0.19,0.21]; clamped short side
    (boundary id 1 = x-), interface id 11 on the other sides carrying the
    dummy tester's constant traction (0,-4); body force (0,-0.5);
    dt 0.1, 2 steps; watchpoint (0.6, 0.2)."""
    p = SolidParams()
    # colorized ids: x-=0 -> clamped (1); x+=1, y-=2, y+=3 -> interface 11
    p.mesh = make_mesh(2, 1, 2, 3, (5, 1), (0.24899, 0.19), (0.6, 0.21),
                       boundary_id=(1, 11, 11, 11), dirichlet=[(1, 0b11)])
    p.mat = material(0.5e6, 0.4, 1000.0, 0.1, formulation)
    p.caching = CACHING[caching]
    p.precond = {"none": 0, "jacobi": 1, "gmg": 2}[precond]
    p.relaxation = 0.65
    p.tol_lin = 1e-6
    p.max_it_mult = 1
    p.max_newton = 10
    p.tol_f, p.tol_f_abs, p.tol_u, p.tol_u_abs = 1e-9, 2e-9, 1e-6, 5e-15
    p.dt = 0.1
    p.n_steps = 2
    p.body_force[:] = [0.0, -0.5, 0.0]
    p.traction_id = 11
    p.traction[:] = [0.0, -4.0, 0.0]
    p.watch[:] = [0.6, 0.2, 0.0]
    p.cheb_degree, p.cheb_range, p.cheb_eig_its = 5, 20.0, 30
    p.coarse_accurate = 1
    p.mg_float = 1
    return p
