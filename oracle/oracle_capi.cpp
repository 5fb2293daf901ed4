// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle_core.hpp).
//
// C entry points of the oracle library (oracle/_build/liboracle.so), called
// through ctypes by the tests, by __graft_entry__.smoke() and by the CPU
// baseline leg of bench.py.  Never linked into the product.
#include "oracle_fast_api.hpp"
#include "oracle_problems.hpp"

#include <chrono>

using namespace orc;


extern "C"
{
  struct or_mesh_t
  {
    int      dim, degree, n_q, n_ref;
    int      rep[3];
    double   lo[3], hi[3];
    int      boundary_id[6];
    int      n_dirichlet;
    int      dirichlet_id[8];
    unsigned dirichlet_mask[8];
  };

  struct or_material_t
  {
    double mu, nu, rho, alpha_1;
    int    formulation;
  };

  static MeshSpec
  to_spec(const or_mesh_t *m)
  {
    MeshSpec s;
    s.dim    = m->dim;
    s.degree = m->degree;
    s.n_q    = m->n_q;
    s.n_ref  = m->n_ref;
    for (int d = 0; d < 3; ++d)
      {
        s.rep[d] = m->rep[d];
        s.lo[d]  = m->lo[d];
        s.hi[d]  = m->hi[d];
      }
    for (int f = 0; f < 6; ++f)
      s.boundary_id[f] = m->boundary_id[f];
    s.n_dirichlet = m->n_dirichlet;
    for (int i = 0; i < 8; ++i)
      {
        s.dirichlet_id[i]   = m->dirichlet_id[i];
        s.dirichlet_mask[i] = m->dirichlet_mask[i];
      }
    return s;
  }

  static Material
  to_mat(const or_material_t *m)
  {
    Material r;
    r.mu          = m->mu;
    r.nu          = m->nu;
    r.rho         = m->rho;
    r.alpha_1     = m->alpha_1;
    r.formulation = m->formulation;
    return r;
  }

  int
  or_set_threads(int n)
  {
#ifdef _OPENMP
    if (n > 0)
      omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
  }

  long
  or_n_nodes(const or_mesh_t *m, int level)
  {
    return long(to_spec(m).box(level).n_nodes);
  }

  // basis matrices (for tests of the 1D machinery): S, G of size Q x N,
  // nodes (N), points (Q), weights (Q)
  int
  or_basis(int degree, int nq, double *S, double *G, double *nodes,
           double *xq, double *wq)
  {
    Basis1D b(degree, nq);
    std::copy(b.S.begin(), b.S.end(), S);
    std::copy(b.G.begin(), b.G.end(), G);
    std::copy(b.nodes.begin(), b.nodes.end(), nodes);
    std::copy(b.xq.begin(), b.xq.end(), xq);
    std::copy(b.wq.begin(), b.wq.end(), wq);
    return 0;
  }

  extern "C++"
  {
  template <typename T>
  static int
  heat_vmult_t(const or_mesh_t *m, int level, double k_dt, int constrained,
               const T *src, T *dst)
  {
    MeshSpec   s = to_spec(m);
    Basis1D    b(s.degree, s.n_q);
    LevelOp<T> op;
    op.box         = s.box(level);
    op.basis       = &b;
    op.nc          = 1;
    op.kind        = op_heat;
    op.k_dt        = k_dt;
    op.constrained = constrained != 0;
    op.vmult(dst, src);
    return 0;
  }
  }

  int
  or_heat_vmult(const or_mesh_t *m, int level, double k_dt, int constrained,
                int precision, const void *src, void *dst)
  {
    if (precision == 32)
      return heat_vmult_t(m, level, k_dt, constrained, (const float *)src,
                          (float *)dst);
    return heat_vmult_t(m, level, k_dt, constrained, (const double *)src,
                        (double *)dst);
  }

  extern "C++"
  {
  template <typename T>
  static int
  heat_invdiag_t(const or_mesh_t *m, int level, double k_dt, T *out)
  {
    MeshSpec   s = to_spec(m);
    Basis1D    b(s.degree, s.n_q);
    LevelOp<T> op;
    op.box   = s.box(level);
    op.basis = &b;
    op.nc    = 1;
    op.kind  = op_heat;
    op.k_dt  = k_dt;
    op.compute_diagonal();
    std::copy(op.inv_diag.begin(), op.inv_diag.end(), out);
    return 0;
  }
  }

  int
  or_heat_inv_diagonal(const or_mesh_t *m, int level, double k_dt,
                       int precision, void *out)
  {
    if (precision == 32)
      return heat_invdiag_t(m, level, k_dt, (float *)out);
    return heat_invdiag_t(m, level, k_dt, (double *)out);
  }

  // mode: 0 vmult, 1 inverse diagonal (src ignored)
  extern "C++"
  {
  template <typename T>
  static int
  nh_apply_t(const or_mesh_t *m, int level, const or_material_t *mat,
             int caching, const T *u, const T *src, T *dst, int mode)
  {
    MeshSpec   s = to_spec(m);
    Basis1D    b(s.degree, s.n_q);
    LevelOp<T> op;
    op.box        = s.box(level);
    op.basis      = &b;
    op.nc         = s.dim;
    op.kind       = op_nh;
    op.nh.mat     = to_mat(mat);
    op.nh.caching = Caching(caching);
    try
      {
        nh_cache(op.nh, op.box, b, u);
      }
    catch (...)
      {
        return -2;
      }
    if (!op.nh.positive_J)
      return -3;
    if (mode == 0)
      op.vmult(dst, src);
    else
      {
        op.compute_diagonal();
        std::copy(op.inv_diag.begin(), op.inv_diag.end(), dst);
      }
    return 0;
  }
  }

  int
  or_nh_vmult(const or_mesh_t *m, int level, const or_material_t *mat,
              int caching, int precision, const void *u, const void *src,
              void *dst)
  {
    if (precision == 32)
      return nh_apply_t(m, level, mat, caching, (const float *)u,
                        (const float *)src, (float *)dst, 0);
    return nh_apply_t(m, level, mat, caching, (const double *)u,
                      (const double *)src, (double *)dst, 0);
  }

  // the CPU timing of the matrix-free tangent: cache once, then `reps`
  // applications, *seconds = their wall time (the cache excluded)
  int
  or_nh_vmult_timed(const or_mesh_t *m, int level, const or_material_t *mat, int caching, const double *u,
                    const double *src, double *dst, int warmup, int reps, double *seconds)
  {
    MeshSpec        s = to_spec(m);
    Basis1D         b(s.degree, s.n_q);
    LevelOp<double> op;
    op.box        = s.box(level);
    op.basis      = &b;
    op.nc         = s.dim;
    op.kind       = op_nh;
    op.nh.mat     = to_mat(mat);
    op.nh.caching = Caching(caching);
    try
      {
        nh_cache(op.nh, op.box, b, u);
      }
    catch (...)
      {
        return -2;
      }
    if (!op.nh.positive_J)
      return -3;
    for (int w = 0; w < std::max(warmup, 1); ++w)
      op.vmult(dst, src); // first touch of the caches and vectors, not timed
    const auto t0 = std::chrono::steady_clock::now();
    for (int r = 0; r < reps; ++r)
      op.vmult(dst, src);
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
  }

  // the throughput form (oracle_fast.hpp) of the same vmult, 3D, n_q = p + 1,
  // formulation 1, any caching variant, cell batches of `lanes` = 2, 4 or 8:
  // cached once, applied once untimed, then `reps` applications timed (dst
  // holds the result); returns 0, -2 when the case is outside the fast form,
  // -3 when det F <= 0
  int
  or_nh_vmult_fast_timed(const or_mesh_t *m, int level, const or_material_t *mat, int caching, int lanes,
                         const double *u, const double *src, double *dst, int warmup, int reps,
                         double *seconds)
  {
    MeshSpec s = to_spec(m);
    if (s.dim != 3 || s.n_q != s.degree + 1 || mat->formulation != 1 || caching < 0 || caching > 3)
      return -2;
    Basis1D  b(s.degree, s.n_q);
    Box      box = s.box(level);
    Material mt  = to_mat(mat);
    try
      {
        switch (lanes)
          {
            case 2: return nh_vmult_fast_timed_w2d(box, b, mt, Caching(caching), u, src, dst, warmup, reps, seconds);
            case 4: return nh_vmult_fast_timed_w4d(box, b, mt, Caching(caching), u, src, dst, warmup, reps, seconds);
            case 8: return nh_vmult_fast_timed_w8d(box, b, mt, Caching(caching), u, src, dst, warmup, reps, seconds);
            default: return -2;
          }
      }
    catch (...)
      {
        return -2;
      }
  }

  // heat vmult (M + k dt K, constrained) applied once untimed, then `reps`
  // applications timed; dst holds the result
  int
  or_heat_vmult_timed(const or_mesh_t *m, int level, double k_dt, const double *src, double *dst, int reps,
                      double *seconds)
  {
    MeshSpec        s = to_spec(m);
    Basis1D         b(s.degree, s.n_q);
    LevelOp<double> op;
    op.box   = s.box(level);
    op.basis = &b;
    op.nc    = 1;
    op.kind  = op_heat;
    op.k_dt  = k_dt;
    op.vmult(dst, src);
    const auto t0 = std::chrono::steady_clock::now();
    for (int r = 0; r < reps; ++r)
      op.vmult(dst, src);
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
  }

  // the throughput form of the heat vmult (3D, n_q = p + 1, `lanes` = 2, 4
  // or 8), applied once untimed, then `reps` applications timed
  int
  or_heat_vmult_fast_timed(const or_mesh_t *m, int level, double k_dt, int lanes, const double *src, double *dst,
                           int reps, double *seconds)
  {
    MeshSpec s = to_spec(m);
    if (s.dim != 3 || s.n_q != s.degree + 1)
      return -2;
    Basis1D b(s.degree, s.n_q);
    Box     box = s.box(level);
    switch (lanes)
      {
        case 2: return heat_vmult_fast_timed_w2d(box, b, k_dt, src, dst, reps, seconds);
        case 4: return heat_vmult_fast_timed_w4d(box, b, k_dt, src, dst, reps, seconds);
        case 8: return heat_vmult_fast_timed_w8d(box, b, k_dt, src, dst, reps, seconds);
        default: return -2;
      }
  }

  int
  or_nh_inv_diagonal(const or_mesh_t *m, int level, const or_material_t *mat,
                     int caching, int precision, const void *u, void *out)
  {
    if (precision == 32)
      return nh_apply_t(m, level, mat, caching, (const float *)u,
                        (const float *)nullptr, (float *)out, 1);
    return nh_apply_t(m, level, mat, caching, (const double *)u,
                      (const double *)nullptr, (double *)out, 1);
  }

  // internal-force + inertia residual (assemble_residual without the
  // traction term): out = -int P(F(u)) : grad v - rho int acc . v, with the
  // constrained rows zero (mf_elasticity.h:1649-1908).  With acc = alpha_1 u
  // its derivative along v is minus the tangent vmult (mf_nh_operator.h:
  // 545-625) on the unconstrained rows.
  int
  or_nh_residual(const or_mesh_t *m, int level, const or_material_t *mat,
                 const double *u, const double *acc, double *out)
  {
    MeshSpec          s    = to_spec(m);
    Basis1D           b(s.degree, s.n_q);
    const Box         box  = s.box(level);
    const Material    M    = to_mat(mat);
    const double      body[3] = {0, 0, 0};
    std::fill(out, out + size_t(s.dim) * box.n_nodes, 0.0);
    ResidualQ<double> q{&M, &box, &b, acc, body};
    cell_loop(box, b, s.dim, u, out, q, false);
    set_constrained_zero(box, s.dim, out);
    return 0;
  }

  // transfer between level (coarse) and level+1; op: 0 prolongate
  // (fine = P coarse), 1 restrict (coarse += P^T fine), 2 interpolate
  // (coarse = fine at coarse nodes)
  int
  or_transfer(const or_mesh_t *m, int coarse_level, int nc, int op,
              double *coarse, double *fine)
  {
    MeshSpec              s = to_spec(m);
    Basis1D               b(s.degree, s.n_q);
    Box                   bc = s.box(coarse_level), bf = s.box(coarse_level + 1);
    LevelTransfer<double> t(b, bc, bf, nc);
    if (op == 0)
      t.prolongate(fine, coarse);
    else if (op == 1)
      t.restrict_add(coarse, fine);
    else
      t.interpolate(coarse, fine);
    return 0;
  }

  struct or_solid_params_t
  {
    or_mesh_t     mesh;
    or_material_t mat;
    int           caching, precond;
    double        relaxation, tol_lin;
    int           max_it_mult, max_newton;
    double        tol_f, tol_f_abs, tol_u, tol_u_abs;
    double        dt;
    int           n_steps;
    double        body_force[3];
    int           traction_id;
    double        traction[3];
    double        watch[3];
    int           cheb_degree;
    double        cheb_range;
    int           cheb_eig_its, coarse_accurate, mg_float;
    int           fast;
  };

  struct or_solid_result_t
  {
    int    newton_its[64];
    double watch_disp[64][3];
    long   total_cg;
    int    n_solves, n_steps, ok;
    double seconds;
  };

  static SolidParams
  to_solid(const or_solid_params_t *p)
  {
    SolidParams P;
    P.mesh            = to_spec(&p->mesh);
    P.mat             = to_mat(&p->mat);
    P.caching         = p->caching;
    P.precond         = p->precond;
    P.relaxation      = p->relaxation;
    P.tol_lin         = p->tol_lin;
    P.max_it_mult     = p->max_it_mult;
    P.max_newton      = p->max_newton;
    P.tol_f           = p->tol_f;
    P.tol_f_abs       = p->tol_f_abs;
    P.tol_u           = p->tol_u;
    P.tol_u_abs       = p->tol_u_abs;
    P.dt              = p->dt;
    P.n_steps         = p->n_steps;
    P.traction_id     = p->traction_id;
    P.cheb_degree     = p->cheb_degree;
    P.cheb_range      = p->cheb_range;
    P.cheb_eig_its    = p->cheb_eig_its;
    P.coarse_accurate = p->coarse_accurate;
    P.mg_float        = p->mg_float;
    P.fast            = p->fast;
    for (int d = 0; d < 3; ++d)
      {
        P.body_force[d] = p->body_force[d];
        P.traction[d]   = p->traction[d];
        P.watch[d]      = p->watch[d];
      }
    return P;
  }

  // the first Newton system of a time step from rest (u = 0, zero
  // acceleration; the right-hand side is the traction term), set up and
  // solved to tol * |rhs| as Solid::update_matrix_free + solve_linear_system
  // do (mf_elasticity.h:1291-1353, 1983-2070); setup and solve timed apart.
  // du (may be null) receives the update.  Returns 0, -1 on an exception,
  // -3 when det F <= 0.
  extern "C++"
  {
  template <typename LT>
  static int
  solid_first_solve_t(const SolidParams &P, double tol, int *its, double *setup_s, double *solve_s, double *du_out)
  {
    SolidDriver<LT>     drv(P);
    const size_t        n = drv.fine.m();
    std::vector<double> u(n, 0.0), acc(n, 0.0), rhs(n, 0.0), du(n, 0.0);
    drv.assemble_residual(u, acc, rhs);
    const auto t0 = std::chrono::steady_clock::now();
    drv.update_operators(u);
    if (!drv.fine.nh.positive_J)
      return -3;
    const auto t1 = std::chrono::steady_clock::now();
    *its          = drv.solve_linear(rhs, du, tol * norm(n, rhs.data()));
    const auto t2 = std::chrono::steady_clock::now();
    *setup_s      = std::chrono::duration<double>(t1 - t0).count();
    *solve_s      = std::chrono::duration<double>(t2 - t1).count();
    if (du_out)
      std::copy(du.begin(), du.end(), du_out);
    return 0;
  }
  }

  int
  or_solid_first_solve(const or_solid_params_t *p, double tol, int *its, double *setup_s, double *solve_s,
                       double *du_out)
  {
    try
      {
        const SolidParams P = to_solid(p);
        return P.mg_float ? solid_first_solve_t<float>(P, tol, its, setup_s, solve_s, du_out) :
                            solid_first_solve_t<double>(P, tol, its, setup_s, solve_s, du_out);
      }
    catch (...)
      {
        return -1;
      }
  }

  int
  or_solid_run(const or_solid_params_t *p, or_solid_result_t *r,
               double *u_out)
  {
    SolidParams P;
    try
      {
        P = to_solid(p);
      }
    catch (...)
      {
        return -1;
      }
    SolidResult R;
    auto        t0 = std::chrono::steady_clock::now();
    try
      {
        if (P.mg_float)
          {
            SolidDriver<float> drv(P);
            drv.run(R);
            if (u_out)
              std::copy(drv.last_u.begin(), drv.last_u.end(), u_out);
          }
        else
          {
            SolidDriver<double> drv(P);
            drv.run(R);
            if (u_out)
              std::copy(drv.last_u.begin(), drv.last_u.end(), u_out);
          }
      }
    catch (...)
      {
        return -1;
      }
    auto t1 = std::chrono::steady_clock::now();
    std::memset(r, 0, sizeof(*r));
    for (int i = 0; i < 64; ++i)
      {
        r->newton_its[i] = R.newton_its[i];
        for (int d = 0; d < 3; ++d)
          r->watch_disp[i][d] = R.watch_disp[i][d];
      }
    r->total_cg = R.total_cg;
    r->n_solves = R.n_solves;
    r->n_steps  = R.n_steps;
    r->ok       = R.ok;
    r->seconds  = std::chrono::duration<double>(t1 - t0).count();
    return R.ok ? 0 : -3;
  }

  struct or_heat_params_t
  {
    or_mesh_t mesh;
    double    dt;
    int       n_steps;
    double    tol_rel;
    int       precond, analytic;
    double    alpha, beta;
    int       n_gauss;
    double    g_center[8][3];
    double    g_width[8];
    double    g_amp[8];
    int       mg_float;
    int       fast;
  };

  struct or_heat_result_t
  {
    double l2_error[64];
    int    cg_its[64];
    int    n_steps;
    double seconds;
  };

  int
  or_heat_run(const or_heat_params_t *p, or_heat_result_t *r, double *u_out)
  {
    HeatParams P;
    P.mesh     = to_spec(&p->mesh);
    P.dt       = p->dt;
    P.n_steps  = p->n_steps;
    P.tol_rel  = p->tol_rel;
    P.precond  = p->precond;
    P.analytic = p->analytic;
    P.alpha    = p->alpha;
    P.beta     = p->beta;
    P.n_gauss  = p->n_gauss;
    P.mg_float = p->mg_float;
    P.fast     = p->fast;
    for (int i = 0; i < 8; ++i)
      {
        for (int d = 0; d < 3; ++d)
          P.g_center[i][d] = p->g_center[i][d];
        P.g_width[i] = p->g_width[i];
        P.g_amp[i]   = p->g_amp[i];
      }
    HeatResult R;
    auto       t0 = std::chrono::steady_clock::now();
    try
      {
        if (P.mg_float)
          {
            HeatDriver<float> drv(P);
            drv.run(R);
            if (u_out)
              std::copy(drv.solution.begin(), drv.solution.end(), u_out);
          }
        else
          {
            HeatDriver<double> drv(P);
            drv.run(R);
            if (u_out)
              std::copy(drv.solution.begin(), drv.solution.end(), u_out);
          }
      }
    catch (...)
      {
        return -1;
      }
    auto t1 = std::chrono::steady_clock::now();
    std::memset(r, 0, sizeof(*r));
    for (int i = 0; i < 64; ++i)
      {
        r->l2_error[i] = R.l2_error[i];
        r->cg_its[i]   = R.cg_its[i];
      }
    r->n_steps = R.n_steps;
    r->seconds = std::chrono::duration<double>(t1 - t0).count();
    return 0;
  }
}
