"""Python host binding of libmfgpu.so (ctypes over the C-ABI of include/mfgpu.h).

Mirrors the reference's operator interface for the matrix-free path:
``NeoHookOperator`` (include/solid_mechanics/mf_nh_operator.h:103-173) and
``LaplaceOperator`` (include/heat_transfer/heat_transfer.h:81-127) with
``vmult / vmult_add / Tvmult / compute_diagonal / get_matrix_diagonal_inverse
/ el / m / precondition_Jacobi / memory_consumption``, the multigrid
transfer, and the solid / heat drivers.  Vectors are CUDA tensors (torch is
used only for device memory); every call goes through the C-ABI and raises
``MfgpuError`` when the library returns a non-zero status.  There is no CPU
fallback: without the built library or a GPU the calls fail.
"""
import ctypes as C
import os
import weakref

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmfgpu.so")

OK = 0
STATUS = {1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_OOM", 4: "ERR_NONFINITE",
          5: "ERR_NOT_CONVERGED", 6: "ERR_STATE", 7: "ERR_DET_F",
          8: "ERR_UNSUPPORTED", 9: "ERR_TIMEOUT"}


class MfgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Mesh(C.Structure):
    _fields_ = [("degree", C.c_int), ("n_q_1d", C.c_int),
                ("n_refinements", C.c_int), ("repetitions", C.c_int * 3),
                ("lower", C.c_double * 3), ("upper", C.c_double * 3),
                ("boundary_id", C.c_int * 6), ("n_dirichlet", C.c_int),
                ("dirichlet_id", C.c_int * 8),
                ("dirichlet_mask", C.c_uint * 8), ("dim", C.c_int)]


class Material(C.Structure):
    _fields_ = [("mu", C.c_double), ("nu", C.c_double), ("rho", C.c_double),
                ("alpha_1", C.c_double), ("formulation", C.c_int)]


class SolverParams(C.Structure):
    _fields_ = [("preconditioner", C.c_int), ("relaxation", C.c_double),
                ("tol", C.c_double), ("max_it_mult", C.c_int),
                ("cheb_degree", C.c_int), ("cheb_range", C.c_double),
                ("cheb_eig_its", C.c_int), ("coarse_accurate", C.c_int),
                ("mg_precision", C.c_int), ("coarse_fp64", C.c_int),
                ("fp64_emulation", C.c_int),
                ("cuda_graphs", C.c_int), ("coarse_dense", C.c_int),
                ("estimate_condition", C.c_int), ("cond_cg_iterations", C.c_int)]


class MGParams(C.Structure):
    _fields_ = [("kind", C.c_int), ("delta_t", C.c_double), ("caching", C.c_char_p),
                ("material", Material), ("solver", SolverParams)]


class SolidParams(C.Structure):
    _fields_ = [("mesh", Mesh), ("material", Material),
                ("caching", C.c_char_p), ("solver", SolverParams),
                ("max_newton", C.c_int), ("tol_f", C.c_double),
                ("tol_f_abs", C.c_double), ("tol_u", C.c_double),
                ("tol_u_abs", C.c_double), ("dt", C.c_double),
                ("n_steps", C.c_int), ("body_force", C.c_double * 3),
                ("traction_id", C.c_int), ("traction", C.c_double * 3),
                ("watch", C.c_double * 3)]


class SolidResult(C.Structure):
    _fields_ = [("newton_its", C.c_int * 64),
                ("watch_disp", (C.c_double * 3) * 64),
                ("total_cg", C.c_long), ("n_solves", C.c_int),
                ("n_steps", C.c_int), ("seconds", C.c_double)]


class HeatParams(C.Structure):
    _fields_ = [("mesh", Mesh), ("dt", C.c_double), ("n_steps", C.c_int),
                ("solver", SolverParams), ("analytic", C.c_int),
                ("alpha", C.c_double), ("beta", C.c_double),
                ("n_gauss", C.c_int), ("g_center", (C.c_double * 3) * 8),
                ("g_width", C.c_double * 8), ("g_amp", C.c_double * 8)]


class HeatResult(C.Structure):
    _fields_ = [("cg_its", C.c_int * 64), ("n_steps", C.c_int),
                ("seconds", C.c_double)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_int), ("heat", HeatParams), ("solid", SolidParams)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("message", C.c_char * 128),
                ("cg_iterations", C.c_int), ("newton_iterations", C.c_int),
                ("watch", C.c_double * 3), ("solution_norm", C.c_double),
                ("n_dofs", C.c_double), ("queue_seconds", C.c_double),
                ("run_seconds", C.c_double), ("latency_seconds", C.c_double)]


_lib = None


def lib():
    """Load libmfgpu.so (built by build.py); fails loudly when missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MfgpuError(-1, f"{LIB_PATH} not built (run build.py)")
        _lib = C.CDLL(LIB_PATH)
        _lib.mfgpu_last_error.restype = C.c_char_p
        _lib.mfgpu_launch_count.restype = C.c_longlong
    return _lib


def _check(rc):
    if rc != OK:
        raise MfgpuError(rc, lib().mfgpu_last_error().decode())


def _text(call, size=1 << 16):
    buf = C.create_string_buffer(size)
    _check(call(buf, C.c_size_t(size)))
    return buf.value.decode()


def timing_table(text):
    """{section: (calls, seconds)} from a timing summary."""
    out = {}
    for line in text.splitlines():
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cells) == 4 and cells[1].isdigit():
            out[cells[0]] = (int(cells[1]), float(cells[2].rstrip("s")))
    return out


def launch_count():
    return int(lib().mfgpu_launch_count())


def _ptr(t):
    if t is None:
        return None
    if isinstance(t, int):
        return C.c_void_p(t)
    return C.c_void_p(t.data_ptr())


def make_mesh(degree, n_refinements, repetitions, lower, upper,
              boundary_id=(0, 0, 0, 0, 0, 0), dirichlet=(), n_q_1d=None, dim=None):
    """Box mesh (2D when repetitions/lower/upper have two entries, or dim=2);
    dirichlet: iterable of (boundary_id, component_mask)."""
    dim = dim or len(repetitions)
    repetitions = tuple(repetitions) + (1,) * (3 - len(repetitions))
    lower = tuple(lower) + (0.0,) * (3 - len(lower))
    upper = tuple(upper) + (1.0,) * (3 - len(upper))
    boundary_id = tuple(boundary_id) + (0,) * (6 - len(boundary_id))
    m = Mesh()
    m.dim = dim
    m.degree = degree
    m.n_q_1d = degree + 1 if n_q_1d is None else n_q_1d
    m.n_refinements = n_refinements
    for d in range(3):
        m.repetitions[d] = repetitions[d]
        m.lower[d] = lower[d]
        m.upper[d] = upper[d]
    for f in range(6):
        m.boundary_id[f] = boundary_id[f]
    m.n_dirichlet = len(dirichlet)
    for i, (bid, mask) in enumerate(dirichlet):
        m.dirichlet_id[i] = bid
        m.dirichlet_mask[i] = mask
    return m


def n_nodes(mesh, level=-1):
    n = C.c_size_t()
    _check(lib().mfgpu_mesh_n_nodes(C.byref(mesh), level, C.byref(n)))
    return n.value


def material(mu=0.5e6, nu=0.4, rho=1000.0, dt=0.01, formulation=1, beta=0.25):
    m = Material()
    m.mu, m.nu, m.rho = mu, nu, rho
    m.alpha_1 = 1.0 / (beta * dt * dt)
    m.formulation = formulation
    return m


class Context:
    """One CUDA device + stream (mfgpu_context)."""

    def __init__(self, device=0):
        self.h = C.c_void_p()
        self._children = weakref.WeakSet()  # objects to release before the context
        _check(lib().mfgpu_context_create(device, C.byref(self.h)))

    def _adopt(self, obj):
        self._children.add(obj)

    def synchronize(self):
        _check(lib().mfgpu_context_synchronize(self.h))

    def copy(self, dst, src, nbytes):
        """Copy nbytes between device/host pointers or tensors."""
        _check(lib().mfgpu_copy(self.h, _ptr(dst), _ptr(src), C.c_size_t(nbytes)))

    def stream(self):
        s = C.c_void_p()
        _check(lib().mfgpu_context_stream(self.h, C.byref(s)))
        return s.value

    def close(self):
        """Release the context; operators and drivers created on it first."""
        if self.h:
            for child in list(self._children):
                child.close()
            lib().mfgpu_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Operator:
    def __init__(self, ctx):
        self.ctx = ctx
        self.h = C.c_void_p()
        ctx._adopt(self)

    def m(self):
        v = C.c_size_t()
        _check(lib().mfgpu_operator_m(self.h, C.byref(v)))
        return v.value

    n = m

    def vmult(self, dst, src):
        _check(lib().mfgpu_operator_vmult(self.h, _ptr(dst), _ptr(src)))

    def vmult_add(self, dst, src):
        _check(lib().mfgpu_operator_vmult_add(self.h, _ptr(dst), _ptr(src)))

    def Tvmult(self, dst, src):
        _check(lib().mfgpu_operator_Tvmult(self.h, _ptr(dst), _ptr(src)))

    def Tvmult_add(self, dst, src):
        _check(lib().mfgpu_operator_Tvmult_add(self.h, _ptr(dst), _ptr(src)))

    def vmult_host(self, dst_np, src_np):
        """dst = A src with host numpy buffers (copies inside the call)."""
        _check(lib().mfgpu_operator_vmult_host(
            self.h, dst_np.ctypes.data_as(C.c_void_p),
            src_np.ctypes.data_as(C.c_void_p)))

    def set_scatter(self, mode):
        """0: atomic scatter; 1: parity-coloured plain scatter (deterministic)."""
        _check(lib().mfgpu_operator_set_scatter(self.h, {"atomic": 0, "colored": 1}.get(mode, mode)))

    def set_cell_kernel(self, mode):
        """0 by grid size, 1 line-parallel, 2 point-parallel, 3 tensor cores
        (FP32 heat operators, element matrix), 4 tensor product (heat
        operators of low degree, 1D mass and stiffness matrices, registers),
        5 tensor product with FP32 Q1-Q2 bricks staged by TMA."""
        _check(lib().mfgpu_operator_set_cell_kernel(
            self.h, {"auto": 0, "line": 1, "point": 2, "tensor": 3, "tp": 4, "tp_tma": 5}.get(mode, mode)))

    def set_dense(self, enable=True):
        """Dense copy of a small operator (assembled now; used while the
        operator's state is unchanged)."""
        _check(lib().mfgpu_operator_set_dense(self.h, int(enable)))

    def set_host_chunks(self, n_chunks):
        """z-slabs of the overlapped vmult_host (0 auto, 1 no overlap)."""
        _check(lib().mfgpu_operator_set_host_chunks(self.h, int(n_chunks)))

    def set_fp64_emulation(self, enable=True):
        """Double-float arithmetic on the FP32 pipe for an FP64 operator."""
        _check(lib().mfgpu_operator_set_fp64_emulation(self.h, int(enable)))

    def compute_diagonal(self):
        _check(lib().mfgpu_operator_compute_diagonal(self.h))

    def get_matrix_diagonal_inverse(self):
        p = C.c_void_p()
        _check(lib().mfgpu_operator_get_matrix_diagonal_inverse(self.h, C.byref(p)))
        return p.value

    def el(self, row, col):
        v = C.c_double()
        _check(lib().mfgpu_operator_el(self.h, C.c_size_t(row), C.c_size_t(col),
                                       C.byref(v)))
        return v.value

    def precondition_Jacobi(self, dst, src, omega):
        _check(lib().mfgpu_operator_precondition_jacobi(
            self.h, _ptr(dst), _ptr(src), C.c_double(omega)))

    def memory_consumption(self):
        v = C.c_size_t()
        _check(lib().mfgpu_operator_memory_consumption(self.h, C.byref(v)))
        return v.value

    def clear(self):
        _check(lib().mfgpu_operator_clear(self.h))

    def close(self):
        if self.h:
            lib().mfgpu_operator_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LaplaceOperator(_Operator):
    """Heat operator M + dt k K on one level (heat_transfer.h:81-250)."""

    def __init__(self, ctx, mesh, level=-1, precision=64, constrained=True,
                 delta_t=None, coefficient=1.0):
        super().__init__(ctx)
        _check(lib().mfgpu_heat_operator_create(ctx.h, C.byref(mesh), level,
                                                precision, int(constrained),
                                                C.byref(self.h)))
        if delta_t is not None:
            self.set_delta_t(delta_t)
        self.evaluate_coefficient(coefficient)

    def set_delta_t(self, dt):
        _check(lib().mfgpu_heat_operator_set_delta_t(self.h, C.c_double(dt)))

    def evaluate_coefficient(self, k=1.0):
        _check(lib().mfgpu_heat_operator_evaluate_coefficient(self.h, C.c_double(k)))


class NeoHookOperator(_Operator):
    """Linearised neo-Hookean tangent on one level (mf_nh_operator.h)."""

    def __init__(self, ctx, mesh, level=-1, precision=64,
                 caching="scalar_referential"):
        super().__init__(ctx)
        _check(lib().mfgpu_nh_operator_create(ctx.h, C.byref(mesh), level,
                                              precision, caching.encode(),
                                              C.byref(self.h)))
        self._u = None

    def set_material(self, mat, inclusion=None):
        _check(lib().mfgpu_nh_operator_set_material(
            self.h, C.byref(mat), C.byref(inclusion) if inclusion else None))

    def set_cell_material_ids(self, ids):
        import numpy as np
        a = np.ascontiguousarray(ids, dtype=np.uint8)
        _check(lib().mfgpu_nh_operator_set_cell_material_ids(self.h, a.ctypes.data_as(C.c_void_p),
                                                               C.c_size_t(a.size)))

    def initialize(self, displacement):
        self._u = displacement  # keep the linearisation alive
        _check(lib().mfgpu_nh_operator_initialize(self.h, _ptr(displacement)))

    def cache(self):
        _check(lib().mfgpu_nh_operator_cache(self.h))


def _transfer(fn, ctx, mesh, coarse_level, nc, precision, a, b):
    _check(getattr(lib(), fn)(ctx.h, C.byref(mesh), coarse_level, nc, precision,
                              _ptr(a), _ptr(b)))


def prolongate(ctx, mesh, coarse_level, nc, coarse, fine, precision=64):
    _transfer("mfgpu_transfer_prolongate", ctx, mesh, coarse_level, nc, precision,
              coarse, fine)


def restrict_add(ctx, mesh, coarse_level, nc, coarse, fine, precision=64):
    _transfer("mfgpu_transfer_restrict_add", ctx, mesh, coarse_level, nc, precision,
              coarse, fine)


def interpolate(ctx, mesh, coarse_level, nc, coarse, fine, precision=64):
    _transfer("mfgpu_transfer_interpolate", ctx, mesh, coarse_level, nc, precision,
              coarse, fine)


def prolongate_noalloc(mesh, coarse_level, nc, coarse, fine, precision=64,
                       stream=None):
    """fine = P coarse with no device allocation (static 4 MiB scratch);
    asynchronous on `stream` (None: the default stream)."""
    _check(lib().mfgpu_transfer_prolongate_noalloc(
        C.byref(mesh), coarse_level, nc, precision, _ptr(coarse), _ptr(fine),
        C.c_void_p(stream) if stream else None))


def solver_params(preconditioner="gmg", tol=1e-6, relaxation=0.65,
                  cheb_degree=5, cheb_range=20.0, cheb_eig_its=30,
                  coarse_accurate=True, mg_precision=32, coarse_fp64=False,
                  max_it_mult=1, fp64_emulation=False, cuda_graphs=True, coarse_dense=True,
                  estimate_condition=False, cond_cg_iterations=20):
    s = SolverParams()
    s.preconditioner = {"none": 0, "jacobi": 1, "gmg": 2}[preconditioner]
    s.relaxation = relaxation
    s.tol = tol
    s.max_it_mult = max_it_mult
    s.cheb_degree = cheb_degree
    s.cheb_range = cheb_range
    s.cheb_eig_its = cheb_eig_its
    s.coarse_accurate = int(coarse_accurate)
    s.mg_precision = mg_precision
    s.coarse_fp64 = int(coarse_fp64)
    s.fp64_emulation = int(fp64_emulation)
    s.cuda_graphs = int(cuda_graphs)
    s.coarse_dense = int(coarse_dense)
    s.estimate_condition = int(estimate_condition)
    s.cond_cg_iterations = cond_cg_iterations
    return s


class Multigrid:
    """PreconditionMG over the level hierarchy of a mesh (mfgpu_mg):
    kind "heat" (LaplaceOperator levels, delta_t) or "nh" (NeoHookOperator
    levels, caching and material)."""

    def __init__(self, ctx, mesh, kind="nh", delta_t=0.1, caching="referential_qp",
                 material=None, solver=None):
        p = MGParams()
        p.kind = {"heat": 0, "nh": 1}[kind]
        p.delta_t = delta_t
        self._caching = caching.encode()
        p.caching = self._caching
        p.material = material if material is not None else globals()["material"]()
        p.solver = solver if solver is not None else solver_params("gmg")
        self.ctx = ctx
        self.h = C.c_void_p()
        _check(lib().mfgpu_mg_create(ctx.h, C.byref(mesh), C.byref(p), C.byref(self.h)))
        ctx._adopt(self)

    def setup(self, linearisation=None):
        _check(lib().mfgpu_mg_setup(self.h, _ptr(linearisation) if linearisation is not None else None))

    def vmult(self, dst, src):
        _check(lib().mfgpu_mg_vmult(self.h, _ptr(dst), _ptr(src)))

    def info(self):
        nl, nd = C.c_int(), C.c_size_t()
        _check(lib().mfgpu_mg_info(self.h, C.byref(nl), C.byref(nd)))
        return nl.value, nd.value

    def close(self):
        if self.h:
            _check(lib().mfgpu_mg_destroy(self.h))
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pcg_solve(op, x, b, tol, max_iterations, mg=None, jacobi_omega=0.0):
    """SolverCG::solve under SolverControl(max_iterations, tol): (iterations,
    final residual); x holds the initial guess."""
    its, res = C.c_int(), C.c_double()
    _check(lib().mfgpu_pcg_solve(op.h, mg.h if mg is not None else None, C.c_double(jacobi_omega),
                                 _ptr(x), _ptr(b), C.c_double(tol), int(max_iterations),
                                 C.byref(its), C.byref(res)))
    return its.value, res.value


def estimate_condition_number(op, b, n_iterations=20, tol=0.0):
    c = C.c_double()
    _check(lib().mfgpu_estimate_condition_number(op.h, _ptr(b), int(n_iterations), C.c_double(tol),
                                                 C.byref(c)))
    return c.value


def dof_permutation(mesh, level, support_points, components=None, tol=1e-6):
    """library_dof[i] of the caller's DoF i (host; numpy arrays)."""
    import numpy as np
    pts = np.ascontiguousarray(support_points, dtype=np.float64).reshape(-1, 3)
    n = pts.shape[0]
    comps = None if components is None else np.ascontiguousarray(components, dtype=np.uint32)
    out = np.zeros(n, dtype=np.uint64)
    _check(lib().mfgpu_dof_permutation(C.byref(mesh), level, C.c_size_t(n),
                                       pts.ctypes.data_as(C.c_void_p),
                                       comps.ctypes.data_as(C.c_void_p) if comps is not None else None,
                                       C.c_double(tol), out.ctypes.data_as(C.c_void_p)))
    return out


class Permutation:
    """The DoF map on the device (mfgpu_permutation)."""

    def __init__(self, ctx, mesh, level, support_points, components=None, tol=1e-6):
        import numpy as np
        pts = np.ascontiguousarray(support_points, dtype=np.float64).reshape(-1, 3)
        comps = None if components is None else np.ascontiguousarray(components, dtype=np.uint32)
        self.ctx = ctx
        self.h = C.c_void_p()
        _check(lib().mfgpu_permutation_create(ctx.h, C.byref(mesh), level, C.c_size_t(pts.shape[0]),
                                              pts.ctypes.data_as(C.c_void_p),
                                              comps.ctypes.data_as(C.c_void_p) if comps is not None else None,
                                              C.c_double(tol), C.byref(self.h)))
        ctx._adopt(self)

    def to_library(self, src, dst, precision=64):
        _check(lib().mfgpu_permutation_to_library(self.h, precision, _ptr(src), _ptr(dst)))

    def from_library(self, src, dst, precision=64):
        _check(lib().mfgpu_permutation_from_library(self.h, precision, _ptr(src), _ptr(dst)))

    def close(self):
        if self.h:
            _check(lib().mfgpu_permutation_destroy(self.h))
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solid:
    """Newton-Newmark driver (mf_elasticity.h:555-628) on the device."""

    def __init__(self, ctx, params):
        self.ctx = ctx
        self.params = params
        self.h = C.c_void_p()
        ctx._adopt(self)
        _check(lib().mfgpu_solid_create(ctx.h, C.byref(params), C.byref(self.h)))

    def run(self):
        r = SolidResult()
        _check(lib().mfgpu_solid_run(self.h, C.byref(r)))
        return r

    def displacement_ptr(self):
        p = C.c_void_p()
        _check(lib().mfgpu_solid_displacement(self.h, C.byref(p)))
        return p.value

    def step(self):
        """One time step: (Newton iterations, CG iterations, linear solves,
        watchpoint displacement)."""
        nits, cg, solves = C.c_int(), C.c_long(), C.c_int()
        w = (C.c_double * 3)()
        _check(lib().mfgpu_solid_step(self.h, C.byref(nits), C.byref(cg), C.byref(solves), w))
        return nits.value, cg.value, solves.value, list(w)

    def residual(self, u, acc, rhs):
        nrm = C.c_double()
        _check(lib().mfgpu_solid_residual(self.h, _ptr(u), _ptr(acc), _ptr(rhs),
                                          C.byref(nrm)))
        return nrm.value

    def linear_solve(self, u, rhs, du):
        its = C.c_int()
        secs = C.c_double()
        _check(lib().mfgpu_solid_linear_solve(self.h, _ptr(u), _ptr(rhs), _ptr(du),
                                              C.byref(its), C.byref(secs)))
        return its.value, secs.value

    def set_timing(self, enable=True):
        """Per-section wall times (the reference's TimerOutput); clears the table."""
        _check(lib().mfgpu_solid_set_timing(self.h, int(enable)))

    def timing_summary(self):
        return _text(lambda buf, n: lib().mfgpu_solid_timing_summary(self.h, buf, n))

    def convergence_table(self):
        """The Newton convergence table of the last time step."""
        return _text(lambda buf, n: lib().mfgpu_solid_convergence_table(self.h, buf, n))

    def close(self):
        if self.h:
            lib().mfgpu_solid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Heat:
    """Backward-Euler heat driver (heat_transfer.h:972-1037) on the device."""

    def __init__(self, ctx, params):
        self.ctx = ctx
        self.params = params
        self.h = C.c_void_p()
        ctx._adopt(self)
        _check(lib().mfgpu_heat_create(ctx.h, C.byref(params), C.byref(self.h)))

    def run(self):
        r = HeatResult()
        _check(lib().mfgpu_heat_run(self.h, C.byref(r)))
        return r

    def solution_ptr(self):
        p = C.c_void_p()
        _check(lib().mfgpu_heat_solution(self.h, C.byref(p)))
        return p.value

    def step(self):
        its = C.c_int()
        _check(lib().mfgpu_heat_step(self.h, C.byref(its)))
        return its.value

    def set_timing(self, enable=True):
        _check(lib().mfgpu_heat_set_timing(self.h, int(enable)))

    def timing_summary(self):
        return _text(lambda buf, n: lib().mfgpu_heat_timing_summary(self.h, buf, n))

    def close(self):
        if self.h:
            lib().mfgpu_heat_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Concurrent solve server (mfgpu_server): submit heat / solid requests,
    wait for their results."""

    def __init__(self, device=0, max_concurrent=4, memory_fraction=0.8):
        self.h = C.c_void_p()
        _check(lib().mfgpu_server_create(device, max_concurrent,
                                         C.c_double(memory_fraction), C.byref(self.h)))
        self._keep = {}

    def submit(self, request):
        rid = C.c_longlong()
        _check(lib().mfgpu_server_submit(self.h, C.byref(request), C.byref(rid)))
        self._keep[rid.value] = request
        return rid.value

    def wait(self, rid):
        r = RequestResult()
        _check(lib().mfgpu_server_wait(self.h, C.c_longlong(rid), C.byref(r)))
        self._keep.pop(rid, None)
        return r

    def stats(self):
        mr = C.c_int()
        b = C.c_size_t()
        _check(lib().mfgpu_server_stats(self.h, C.byref(mr), C.byref(b)))
        return mr.value, b.value

    def set_max_batch(self, k):
        """Heat requests of one shape solved together, at most (1: no batching)."""
        _check(lib().mfgpu_server_set_max_batch(self.h, int(k)))

    def batch_stats(self):
        """(requests that ran in a batch of two or more, largest batch)"""
        n, k = C.c_longlong(), C.c_int()
        _check(lib().mfgpu_server_batch_stats(self.h, C.byref(n), C.byref(k)))
        return n.value, k.value

    def pool_stats(self):
        """(requests that reused a resident problem, requests that built one)"""
        reused, built = C.c_longlong(), C.c_longlong()
        _check(lib().mfgpu_server_pool_stats(self.h, C.byref(reused), C.byref(built)))
        return reused.value, built.value

    def close(self):
        if self.h:
            lib().mfgpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
