"""Synthetic, seeded workloads of the benchmark configurations.

The reference publishes no dataset; these generators build the meshes and
fields the benchmark configurations describe:

* heat on the unit cube, zero Dirichlet on x = 0, source = sum of 8
  Gaussians (centres U[0.2,0.8]^3, widths U(0.05,0.15), amplitudes U(0.5,2));
* neo-Hookean cantilever [0,8]x[0,1]^2 (8x1x1 coarse cells), clamped at
  x = 0, uniform traction on x = 8 (boundary id 11), mu = 0.5e6, nu = 0.4,
  rho = 1000, Newmark dt = 0.01;
* a smooth linearisation state u = sum of 6 sine modes per component,
  scaled to max |u| = 0.05 with det(I + grad u) kept in [0.85, 1.15].

Node numbering and vector layout are those of the library: lexicographic
Gauss-Lobatto node grid, component-blocked vectors.
"""
import numpy as np

CLAMPED_ID = 1
TRACTION_ID = 11


def gauss_lobatto(p):
    """FE_Q(p) support points on [0,1] (end points + roots of P'_p)."""
    if p == 1:
        return np.array([0.0, 1.0])
    c = np.zeros(p + 1)
    c[p] = 1.0
    dP = np.polynomial.legendre.legder(c)
    r = np.sort(np.polynomial.legendre.legroots(dP).real)
    return np.concatenate([[0.0], (r + 1) / 2, [1.0]])


def axis_coords(n_cells, lo, hi, p):
    """Coordinates of the Q_p nodes along one axis."""
    gl = gauss_lobatto(p)
    h = (hi - lo) / n_cells
    x = np.empty(n_cells * p + 1)
    for c in range(n_cells):
        x[c * p:(c + 1) * p + 1] = lo + (c + gl) * h
    return x


def node_coords(degree, n_ref, rep, lo, hi):
    """(X, Y, Z) node coordinate arrays in lexicographic node order."""
    axes = [axis_coords(rep[d] << n_ref, lo[d], hi[d], degree) for d in range(3)]
    Z, Y, X = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return X.ravel(), Y.ravel(), Z.ravel()


def smooth_displacement(degree, n_ref, rep, lo, hi, seed=2, amplitude=0.05,
                        j_range=(0.85, 1.15)):
    """u_c(x) = sum_m a_m sin(k_m . x + phi_m), 6 modes per component, scaled
    to max |u| = amplitude; the amplitude is reduced if det(I + grad u) at
    the nodes leaves j_range.  Returns a component-blocked float64 vector."""
    rng = np.random.Generator(np.random.PCG64(seed))
    X, Y, Z = node_coords(degree, n_ref, rep, lo, hi)
    pts = np.stack([X, Y, Z], axis=1)
    ext = np.array(hi, float) - np.array(lo, float)
    u = np.zeros((3, len(X)))
    g = np.zeros((3, 3, len(X)))
    for c in range(3):
        for _ in range(6):
            k = rng.uniform(-1.0, 1.0, 3) * (2 * np.pi / ext) * np.array([2.0, 1.0, 1.0])
            phi = rng.uniform(0, 2 * np.pi)
            a = rng.uniform(0.5, 1.0)
            arg = pts @ k + phi
            u[c] += a * np.sin(arg)
            g[c] += a * np.cos(arg)[None, :] * k[:, None]
    scale = amplitude / np.abs(u).max()
    for _ in range(30):
        F = np.eye(3)[:, :, None] + scale * g
        J = np.linalg.det(np.moveaxis(F, 2, 0))
        if J.min() >= j_range[0] and J.max() <= j_range[1]:
            break
        scale *= 0.8
    return (scale * u).ravel()


def gaussian_source(seed=0, n=8):
    """8 Gaussians with centres U[0.2,0.8]^3, widths U(0.05,0.15),
    amplitudes U(0.5,2)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centers = rng.uniform(0.2, 0.8, (n, 3))
    widths = rng.uniform(0.05, 0.15, n)
    amps = rng.uniform(0.5, 2.0, n)
    return centers, widths, amps


def uniform_vector(n, seed, dtype=np.float64):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(-1.0, 1.0, n).astype(dtype)


# --- mesh descriptions (tuples usable with both the library and the oracle)

def cantilever(degree, n_ref, rep=(8, 1, 1), length=(8.0, 1.0, 1.0)):
    """Clamped (all components) at x = 0, traction boundary at x = 8."""
    return dict(degree=degree, n_ref=n_ref, rep=tuple(rep), lo=(0.0, 0.0, 0.0),
                hi=tuple(length),
                boundary_id=(CLAMPED_ID, TRACTION_ID, 0, 0, 0, 0),
                dirichlet=[(CLAMPED_ID, 0b111)])


def unit_cube_heat(degree, n_ref, rep=(1, 1, 1)):
    """Zero Dirichlet on x = 0, natural elsewhere."""
    return dict(degree=degree, n_ref=n_ref, rep=tuple(rep), lo=(0.0, 0.0, 0.0),
                hi=(1.0, 1.0, 1.0), boundary_id=(1, 0, 0, 0, 0, 0),
                dirichlet=[(1, 0b1)])


def to_lib_mesh(mfgpu, spec):
    return mfgpu.make_mesh(spec["degree"], spec["n_ref"], spec["rep"], spec["lo"],
                           spec["hi"], boundary_id=spec["boundary_id"],
                           dirichlet=spec["dirichlet"])


def to_oracle_mesh(oracle, spec):
    return oracle.make_mesh(3, spec["degree"], spec["degree"] + 1, spec["n_ref"],
                            spec["rep"], spec["lo"], spec["hi"],
                            boundary_id=spec["boundary_id"],
                            dirichlet=spec["dirichlet"])


def n_dofs(spec, n_components):
    n = 1
    for d in range(3):
        n *= (spec["rep"][d] << spec["n_ref"]) * spec["degree"] + 1
    return n * n_components


def serving_requests(mfgpu, n, seed=7, max_heat_ref=6, solid_k=(2, 4, 8), degrees=(1, 2, 3, 4),
                     mg_precision=32, tol=1e-8, fp64_emulation=None):
    """The serving mix: 60 % heat / 40 % neo-Hookean requests.  Heat: unit
    cube with 8^3..(2^max_heat_ref)^3 cells (uniform random refinement 3..),
    zero Dirichlet on x = 0, a seeded Gaussian source, one backward-Euler
    step.  Solid: cantilever 8k x k x k cells, k in solid_k, clamped at x = 0,
    a seeded traction of magnitude U(50, 150) on x = 8, one Newton-Newmark
    step.  Degree uniform in `degrees`.  FP32-GMG preconditioned FP64 CG
    with the FP64 operators (fine and coarse level) in native FP64
    (mg_precision=32; fp64_emulation=True runs them in double-float), or the
    plain FP64 solver (mg_precision=64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    emul = bool(fp64_emulation) and mg_precision == 32
    reqs = []
    for i in range(n):
        r = mfgpu.Request()
        deg = int(rng.choice(degrees))
        if rng.uniform() < 0.6:
            r.kind = 0
            nref = int(rng.integers(3, max_heat_ref + 1))
            spec = unit_cube_heat(deg, nref)
            hp = r.heat
            hp.mesh = to_lib_mesh(mfgpu, spec)
            hp.dt, hp.n_steps = 0.1, 1
            hp.solver = mfgpu.solver_params("gmg", tol=tol, cheb_range=15.0, cheb_eig_its=10,
                                            mg_precision=mg_precision,
                                            coarse_fp64=(mg_precision == 32),
                                            fp64_emulation=emul)
            c, w, a = gaussian_source(int(rng.integers(1 << 30)))
            hp.n_gauss = 8
            for j in range(8):
                for d in range(3):
                    hp.g_center[j][d] = c[j, d]
                hp.g_width[j] = w[j]
                hp.g_amp[j] = a[j]
        else:
            r.kind = 1
            k = int(rng.choice(solid_k))
            nref = {2: 1, 4: 2, 8: 3, 16: 4}[k]
            spec = cantilever(deg, nref)
            sp = r.solid
            sp.mesh = to_lib_mesh(mfgpu, spec)
            sp.material = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
            sp.caching = b"referential_qp"
            sp.solver = mfgpu.solver_params("gmg", tol=tol, mg_precision=mg_precision,
                                            coarse_fp64=(mg_precision == 32),
                                            fp64_emulation=emul)
            sp.max_newton = 10
            sp.tol_f, sp.tol_f_abs, sp.tol_u, sp.tol_u_abs = 1e-9, 0.0, 1e-6, 0.0
            sp.dt, sp.n_steps = 0.01, 1
            sp.traction_id = TRACTION_ID
            sp.traction[:] = [0.0, -float(rng.uniform(50, 150)), 0.0]
            sp.watch[:] = [8.0, 0.5, 0.5]
        reqs.append(r)
    return reqs
