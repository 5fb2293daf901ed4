// Solid (Newton-Newmark) and heat (backward Euler) drivers on the device,
// restating Solid::solve_nonlinear_timestep / assemble_residual /
// solve_linear_system (include/solid_mechanics/mf_elasticity.h:1402-1491,
// 1649-1908, 1983-2070) and LaplaceProblem::assemble_rhs / solve
// (include/heat_transfer/heat_transfer.h:579-655, 715-812), with preCICE
// replaced by a constant boundary traction / analytic Dirichlet data.
#include <chrono>
#include <cstdio>
#include <cmath>
#include <cstring>

#include "../../include/mfgpu.h"
#include "mf_drivers.h"
#include "mf_vec.cuh"

namespace mfgpu
{
  static cudaError_t
  dispatch_residual(int N, const HostBasis &b, const LevelGeom &g, int form, const NHMatD &m,
                    double rho, const double *body, const double *u, const double *acc,
                    double *rhs, cudaStream_t s)
  {
    switch (N)
      {
        case 2: return launch_residual<2>(b, g, form, m, rho, body, u, acc, rhs, s);
        case 3: return launch_residual<3>(b, g, form, m, rho, body, u, acc, rhs, s);
        case 4: return launch_residual<4>(b, g, form, m, rho, body, u, acc, rhs, s);
        case 5: return launch_residual<5>(b, g, form, m, rho, body, u, acc, rhs, s);
        case 6: return launch_residual<6>(b, g, form, m, rho, body, u, acc, rhs, s);
        case 7: return launch_residual<7>(b, g, form, m, rho, body, u, acc, rhs, s);
      }
    return cudaErrorInvalidValue;
  }

  static cudaError_t
  dispatch_heat_rhs(int N, const HostBasis &b, const LevelGeom &g, double dt,
                    const SourceDesc &f, const double *u_old, double *rhs, double *tab, cudaStream_t s)
  {
    switch (N)
      {
        case 2: return launch_heat_rhs<2>(b, g, dt, f, u_old, rhs, tab, s);
        case 3: return launch_heat_rhs<3>(b, g, dt, f, u_old, rhs, tab, s);
        case 4: return launch_heat_rhs<4>(b, g, dt, f, u_old, rhs, tab, s);
        case 5: return launch_heat_rhs<5>(b, g, dt, f, u_old, rhs, tab, s);
        case 6: return launch_heat_rhs<6>(b, g, dt, f, u_old, rhs, tab, s);
        case 7: return launch_heat_rhs<7>(b, g, dt, f, u_old, rhs, tab, s);
      }
    return cudaErrorInvalidValue;
  }

  Mesh
  to_mesh(const mfgpu_mesh &m)
  {
    Mesh r;
    r.dim    = m.dim == 0 ? 3 : m.dim;
    if (r.dim != 2 && r.dim != 3)
      throw Error(ERR_ARG, "mesh: dim must be 2 or 3");
    r.degree = m.degree;
    r.n_q    = m.n_q_1d;
    r.n_ref  = m.n_refinements;
    for (int d = 0; d < r.dim; ++d)
      {
        r.rep[d] = m.repetitions[d];
        r.lo[d]  = m.lower[d];
        r.hi[d]  = m.upper[d];
        if (m.repetitions[d] < 1 || !(m.upper[d] > m.lower[d]))
          throw Error(ERR_ARG, "mesh: repetitions must be >= 1 and upper > lower");
      }
    if (r.dim == 2)
      {
        r.rep[2] = 1;
        r.lo[2]  = 0;
        r.hi[2]  = 1;
      }
    if (m.degree < 1 || m.degree > 6)
      throw Error(ERR_UNSUPPORTED, "mesh: degree must be 1..6");
    if (m.n_refinements < 0 || m.n_refinements > 12)
      throw Error(ERR_ARG, "mesh: n_refinements out of range");
    if (m.n_dirichlet < 0 || m.n_dirichlet > 8)
      throw Error(ERR_ARG, "mesh: n_dirichlet out of range");
    for (int f = 0; f < 6; ++f)
      r.boundary_id[f] = m.boundary_id[f];
    r.n_dirichlet = m.n_dirichlet;
    for (int i = 0; i < 8; ++i)
      {
        r.dirichlet_id[i]   = m.dirichlet_id[i];
        r.dirichlet_mask[i] = m.dirichlet_mask[i];
      }
    return r;
  }

  double
  estimate_condition_number(Operator &A, const double *b, int n_its, double tol)
  {
    DevBuf        y, ws;
    const size_t  n = A.m();
    y.alloc(n * sizeof(double));
    MF_CK(cudaMemsetAsync(y.ptr, 0, n * sizeof(double), A.ctx->stream));
    OpRef<double> L(&A);
    const CGStats st = cg_solve<double>(*A.ctx, L, nullptr, y.as<double>(), b, tol, n_its, true, false, &ws);
    const auto    ev = lanczos_extreme_eigenvalues(st);
    return ev.first > 0 ? ev.second / ev.first : 1.0;
  }

  // ---------------------------------------------------------------------
  // preconditioner wrappers
  // ---------------------------------------------------------------------
  struct IdentityPre : Precond<double>
  {
    Context *ctx;
    size_t   n;
    void vmult(double *d, const double *s) override { vec_copy<double>(*ctx, n, s, d); }
  };

  struct JacobiPre64 : Precond<double>
  {
    Context  *ctx;
    Operator *A;
    double    omega;
    void
    vmult(double *d, const double *s) override
    {
      vec_scale<double>(*ctx, A->m(), omega, A->inv_diag.as<double>(), s, d);
    }
  };

  // ---------------------------------------------------------------------
  // multigrid hierarchy
  // ---------------------------------------------------------------------
  std::unique_ptr<GMGHierarchy>
  GMGHierarchy::heat(Context *c, const Mesh &m, const mfgpu_solver_params &s, double delta_t, int batch)
  {
    std::unique_ptr<GMGHierarchy> h(new GMGHierarchy());
    h->mesh  = m;
    h->S     = s;
    h->kind  = 0;
    h->nc    = batch; // the transfers move every problem of a batch
    h->batch = batch;
    h->lprec = s.mg_precision == 64 ? 64 : 32;
    // LaplaceProblem::setup_gmg (heat_transfer.h:515-573): Chebyshev degree
    // 5, smoothing range 15, 10 eigenvalue-estimate iterations; the coarse
    // level's estimate runs m() iterations
    h->range      = 15.;
    h->degree     = 5;
    h->eig_its    = 10;
    h->coarse_its = -1;
    const bool emul = s.fp64_emulation != 0;
    for (int l = 0; l <= m.n_ref; ++l)
      {
        auto lo     = make_heat(c, m, l, h->lprec, true, batch);
        lo->delta_t = delta_t;
        lo->arith   = (emul && h->lprec == 64) ? 1 : 0;
        h->lops.push_back(std::move(lo));
      }
    if (s.coarse_fp64 && h->lprec == 32)
      {
        auto co     = make_heat(c, m, 0, 64, true, batch);
        co->delta_t = delta_t;
        co->arith   = emul ? 1 : 0;
        h->coarse64 = std::move(co);
      }
    h->finish(c);
    return h;
  }

  std::unique_ptr<GMGHierarchy>
  GMGHierarchy::solid(Context *c, const Mesh &m, const mfgpu_solver_params &s, const NHMatD &mat,
                      int formulation, int variant)
  {
    std::unique_ptr<GMGHierarchy> h(new GMGHierarchy());
    h->mesh       = m;
    h->S          = s;
    h->kind       = 1;
    h->nc         = m.dim;
    h->lprec      = s.mg_precision == 64 ? 64 : 32;
    h->range      = s.cheb_range;
    h->degree     = unsigned(s.cheb_degree);
    h->eig_its    = s.cheb_eig_its;
    h->coarse_its = s.coarse_accurate ? -1 : s.cheb_eig_its;
    const bool emul = s.fp64_emulation != 0;
    auto       nh   = [&](int l, int prec, int arith) {
      auto op           = make_nh(c, m, l, prec, variant);
      op->mat           = mat;
      op->formulation   = formulation;
      op->have_material = true;
      op->arith         = arith;
      return op;
    };
    for (int l = 0; l <= m.n_ref; ++l)
      {
        h->lops.push_back(nh(l, h->lprec, (emul && h->lprec == 64) ? 1 : 0));
        h->u_levels.emplace_back(h->lops.back()->m() * (h->lprec == 32 ? 4 : 8));
      }
    if (s.coarse_fp64 && h->lprec == 32)
      {
        h->coarse64 = nh(0, 64, emul ? 1 : 0);
        h->u0_64.alloc(h->coarse64->m() * sizeof(double));
      }
    h->finish(c);
    return h;
  }

  void
  GMGHierarchy::finish(Context *c)
  {
    ctx = c;
    L   = mesh.n_ref;
    make_host_basis(mesh.degree, basis);
    auto fill = [&](auto &mg) {
      mg.ctx = ctx;
      for (int l = 0; l <= L; ++l)
        {
          mg.ops.push_back(lops[l].get());
          if (l == 0)
            mg.transfers.emplace_back(nullptr);
          else
            mg.transfers.emplace_back(new Transfer(ctx, basis, lops[l - 1]->geom, lops[l]->geom, nc, lprec));
        }
      mg.coarse64   = coarse64.get();
      mg.use_graphs = S.cuda_graphs != 0;
    };
    if (lprec == 32)
      {
        mgf.reset(new Multigrid<float>());
        fill(*mgf);
      }
    else
      {
        mgd.reset(new Multigrid<double>());
        fill(*mgd);
      }
  }

  void
  GMGHierarchy::set_linearisation(const double *ulin, PhaseTimer &timer)
  {
    if (kind != 1)
      throw Error(ERR_STATE, "only neo-Hookean levels take a linearisation");
    {
      PhaseTimer::Scope ts(timer, ctx, "Setup MF: interpolate_to_mg");
      const size_t      nf = lops[L]->m();
      if (lprec == 32)
        vec_convert<float, double>(*ctx, nf, ulin, u_levels[L].as<float>());
      else
        vec_copy<double>(*ctx, nf, ulin, u_levels[L].as<double>());
      for (int l = L; l > 0; --l)
        {
          Transfer *t = lprec == 32 ? mgf->transfers[l].get() : mgd->transfers[l].get();
          t->interpolate(u_levels[l - 1].ptr, u_levels[l].ptr);
        }
      if (coarse64)
        vec_convert<double, float>(*ctx, coarse64->m(), u_levels[0].as<float>(), u0_64.as<double>());
    }
    PhaseTimer::Scope ts(timer, ctx, "Setup MF: cache()");
    for (int l = 0; l <= L; ++l)
      {
        auto *op = static_cast<NHOperator *>(lops[l].get());
        op->u    = u_levels[l].ptr;
        op->do_cache();
      }
    if (coarse64)
      {
        auto *op = static_cast<NHOperator *>(coarse64.get());
        op->u    = u0_64.ptr;
        op->do_cache();
      }
  }

  void
  GMGHierarchy::update_diagonals(PhaseTimer &timer)
  {
    size_t key = 1469598103934665603ull;
    for (auto &op : lops)
      key = (key ^ op->value_state()) * 1099511628211ull;
    if (coarse64)
      key = (key ^ coarse64->value_state()) * 1099511628211ull;
    if (key == diag_key)
      return;
    {
      PhaseTimer::Scope ts(timer, ctx, "Setup MF: diagonal()");
      for (auto &op : lops)
        op->compute_diagonal();
      if (coarse64)
        coarse64->compute_diagonal();
    }
    Operator *co = coarse64 ? coarse64.get() : lops[0].get();
    if (S.coarse_dense && co->dense_fits())
      {
        PhaseTimer::Scope ts(timer, ctx, "Setup MF: coarse matrix");
        co->assemble_dense();
      }
    diag_key = key;
  }

  void
  GMGHierarchy::setup_smoothers(PhaseTimer &timer)
  {
    PhaseTimer::Scope ts(timer, ctx, kind == 1 ? "Setup MF: GMG setup" : "GMG setup");
    // the coarse estimate runs m() iterations of one problem (a batch's
    // problems are identical)
    const int         cits = coarse_its < 0 ? int(lops[0]->m() / size_t(batch)) : coarse_its;
    if (lprec == 32)
      mgf->setup(range, degree, eig_its, cits);
    else
      mgd->setup(range, degree, eig_its, cits);
  }

  Precond<double> *
  GMGHierarchy::precond()
  {
    return lprec == 32 ? static_cast<Precond<double> *>(mgf.get()) : static_cast<Precond<double> *>(mgd.get());
  }

  // ---------------------------------------------------------------------
  // solid
  // ---------------------------------------------------------------------
  SolidDriver::SolidDriver(Context *c, const mfgpu_solid_params &p)
    : ctx(c)
    , P(p)
  {
    mesh = to_mesh(P.mesh);
    L    = mesh.n_ref;
    make_host_basis(mesh.degree, basis);
    const double beta = 0.25;
    const double a1   = 1. / (beta * P.dt * P.dt);
    P.material.alpha_1 = a1;
    mat      = make_material(P.material.mu, P.material.nu, P.material.rho, a1);
    variant  = parse_caching(P.caching);
    P.caching = nullptr; // parsed into variant; the caller's string need not outlive the driver
    if (P.material.formulation != 0 && P.material.formulation != 1)
      throw Error(ERR_ARG, "formulation must be 0 or 1");
    fine                = make_nh(ctx, mesh, -1, 64, variant);
    fine->mat           = mat;
    fine->formulation   = P.material.formulation;
    fine->have_material = true;
    const bool emul     = P.solver.fp64_emulation != 0;
    if (emul && (variant != V_QP10 || P.material.formulation != 1))
      throw Error(ERR_UNSUPPORTED, "fp64_emulation needs referential_qp caching and formulation 1");
    fine->arith = emul ? 1 : 0;
    const size_t n      = fine->m();
    for (DevBuf *b : {&u, &delta, &v_old, &a_old, &acc, &rhs, &du})
      {
        b->alloc(n * sizeof(double));
        MF_CK(cudaMemsetAsync(b->ptr, 0, n * sizeof(double), ctx->stream));
      }
    if (P.solver.preconditioner == 2)
      {
        gmg   = GMGHierarchy::solid(ctx, mesh, P.solver, mat, P.material.formulation, variant);
        lprec = gmg->lprec;
      }
  }

  void
  SolidDriver::update_operators(const double *ulin)
  {
    {
      PhaseTimer::Scope ts(timer, ctx, "Setup MF: cache()");
      fine->u = ulin;
      fine->do_cache();
    }
    if (P.solver.preconditioner == 1)
      {
        PhaseTimer::Scope ts(timer, ctx, "Setup MF: diagonal()");
        fine->compute_diagonal();
      }
    if (P.solver.preconditioner != 2)
      return;
    gmg->set_linearisation(ulin, timer);
    gmg->update_diagonals(timer);
    gmg->setup_smoothers(timer);
  }

  double
  SolidDriver::assemble_residual()
  {
    PhaseTimer::Scope ts(timer, ctx, "Assemble residual");
    const size_t      n = fine->m();
    MF_CK(cudaMemsetAsync(rhs.ptr, 0, n * sizeof(double), ctx->stream));
    if (mesh.dim == 2)
      MF_CK(launch_residual2d(basis.N, basis, fine->geom, P.material.formulation, mat, P.material.rho,
                              P.body_force, u.as<double>(), acc.as<double>(), rhs.as<double>(), ctx->stream));
    else
      MF_CK(dispatch_residual(basis.N, basis, fine->geom, P.material.formulation, mat, P.material.rho,
                              P.body_force, u.as<double>(), acc.as<double>(), rhs.as<double>(),
                              ctx->stream));
    count_launch();
    // traction faces
    for (int f = 0; f < 2 * mesh.dim; ++f)
      {
        if (mesh.boundary_id[f] != P.traction_id)
          continue;
        TractionArgs A;
        std::memset(&A, 0, sizeof(A));
        const LevelGeom &g = fine->geom;
        for (int d = 0; d < 3; ++d)
          {
            A.C[d]  = g.C[d];
            A.Nn[d] = g.Nn[d];
            A.h[d]  = g.h[d];
            A.t[d]  = P.traction[d];
          }
        A.p       = g.p;
        A.N       = basis.N;
        A.n_nodes = g.n_nodes;
        A.face    = f;
        for (int i = 0; i < basis.N * basis.N; ++i)
          {
            A.S[i] = basis.S[i];
            A.G[i] = basis.G[i];
          }
        for (int i = 0; i < basis.N; ++i)
          {
            A.Ge[0][i] = basis.Ge[0][i];
            A.Ge[1][i] = basis.Ge[1][i];
            A.w[i]     = basis.w[i];
          }
        const int nd = f / 2, d1 = nd == 0 ? 1 : 0, d2 = nd == 2 ? 1 : 2;
        if (mesh.dim == 2)
          k_traction2d<<<unsigned(g.C[1 - nd]), 64, 0, ctx->stream>>>(A, u.as<double>(), rhs.as<double>());
        else
          k_traction<<<unsigned(g.C[d1] * g.C[d2]), 128, 0, ctx->stream>>>(A, u.as<double>(), rhs.as<double>());
        count_launch();
        MF_CK(cudaGetLastError());
      }
    constrained_op<double>(*ctx, fine->geom, fine->nc, 2, nullptr, rhs.as<double>());
    return std::sqrt(vec_dot<double>(*ctx, n, rhs.as<double>(), rhs.as<double>()));
  }

  double
  SolidDriver::residual_at(const double *uu, const double *aa, double *r)
  {
    const size_t n = fine->m();
    vec_copy<double>(*ctx, n, uu, u.as<double>());
    vec_copy<double>(*ctx, n, aa, acc.as<double>());
    const double nrm = assemble_residual();
    vec_copy<double>(*ctx, n, rhs.as<double>(), r);
    ctx->sync();
    return nrm;
  }

  struct FineOp : LinOp<double>
  {
    Operator *op;
    size_t size() const override { return op->m(); }
    void   vmult(double *d, const double *s) override { op->vmult(d, s); }
  };

  int
  SolidDriver::solve_linear(const double *b, double *x, double tol)
  {
    // "Estimate condition number" (mf_elasticity.h:1998-2013): a dummy CG
    // before the solve, whose result only enters the convergence table
    last_cond = P.solver.estimate_condition
                  ? estimate_condition_number(*fine, b, std::max(P.solver.cond_cg_iterations, 1), tol)
                  : 1.0;
    PhaseTimer::Scope ts(timer, ctx, "Linear solver");
    const size_t      n = fine->m();
    MF_CK(cudaMemsetAsync(x, 0, n * sizeof(double), ctx->stream));
    FineOp A;
    A.op            = fine.get();
    const int maxit = int(std::min<size_t>(n * size_t(std::max(P.solver.max_it_mult, 1)), 1000000000));
    CGStats   st;
    if (P.solver.preconditioner == 1)
      {
        JacobiPre64 J;
        J.ctx   = ctx;
        J.A     = fine.get();
        J.omega = P.solver.relaxation;
        st      = cg_solve<double>(*ctx, A, &J, x, b, tol, maxit, false, false, &cg_ws);
      }
    else if (P.solver.preconditioner == 2)
      {
        st = cg_solve<double>(*ctx, A, gmg->precond(), x, b, tol, maxit, false, false, &cg_ws);
      }
    else
      st = cg_solve<double>(*ctx, A, nullptr, x, b, tol, maxit, false, false, &cg_ws);
    constrained_op<double>(*ctx, fine->geom, fine->nc, 2, nullptr, x);
    if (!st.converged)
      throw Error(ERR_NOT_CONVERGED, "CG did not converge");
    last_lin_res = st.res;
    return st.its;
  }

  std::string
  SolidDriver::convergence_table() const
  {
    // Solid::print_conv_header / solve_nonlinear_timestep / print_conv_footer
    // (mf_elasticity.h:1402-1491, 1498-1530)
    const std::string rule(98, '_');
    std::string       out = "\nTimestep " + std::to_string(table_step) + "\n" + rule + "\n" +
                      "    SOLVER STEP     |  LIN_IT    LIN_RES   COND_NUM   RES_NORM      RES_U      NU_NORM"
                      "       NU_U\n" +
                      rule + "\n";
    char line[256];
    for (const NewtonRow &r : table)
      {
        std::snprintf(line, sizeof(line), " %2d  | %7d  %.3e  %.3e  %.3e  %.3e    %.3e  %.3e\n", r.it,
                      r.lin_its, r.lin_res, r.cond, r.res_norm, r.res, r.upd_norm, r.upd);
        out += line;
      }
    std::snprintf(line, sizeof(line), " %2d  CONVERGED! \n", int(table.size()));
    out += line;
    return out + rule + "\n";
  }

  // the displacement at a point of a cell: sum over the cell's nodes of
  // the tensor-product Lagrange weights times the nodal values, one thread
  // per component, in a fixed order
  struct PointArgs
  {
    size_t n_nodes, base;
    int    N, nz, nc, Nn0, Nn1;
    double lx[MAX_N], ly[MAX_N], lz[MAX_N];
  };

  __global__ void
  k_point_value(const __grid_constant__ PointArgs a, const double *__restrict__ u, double *__restrict__ out)
  {
    const int c = threadIdx.x;
    if (c >= a.nc)
      return;
    double r = 0;
    for (int k = 0; k < a.nz; ++k)
      for (int j = 0; j < a.N; ++j)
        for (int i = 0; i < a.N; ++i)
          r += a.lx[i] * a.ly[j] * a.lz[k] *
               u[size_t(c) * a.n_nodes + a.base + size_t(i) + size_t(a.Nn0) * (size_t(j) + size_t(a.Nn1) * k)];
    out[c] = r;
  }

  std::vector<double>
  SolidDriver::point_value(const double *x)
  {
    // evaluated on the device: only the three values cross to the host
    const LevelGeom &g = fine->geom;
    int              cc[3] = {0, 0, 0};
    double           xi[3] = {0, 0, 0};
    for (int d = 0; d < mesh.dim; ++d)
      {
        const double t = (x[d] - g.lo[d]) / g.h[d];
        int          c = int(std::floor(t));
        c              = std::min(std::max(c, 0), g.C[d] - 1);
        cc[d]          = c;
        xi[d]          = t - c;
      }
    auto lag = [&](int i, double t) {
      double v = 1;
      for (int j = 0; j < basis.N; ++j)
        if (j != i)
          v *= (t - basis.nodes[j]) / (basis.nodes[i] - basis.nodes[j]);
      return v;
    };
    PointArgs a{};
    a.n_nodes = g.n_nodes;
    a.base    = size_t(cc[0] * g.p) + size_t(g.Nn[0]) * (size_t(cc[1] * g.p) + size_t(g.Nn[1]) * (cc[2] * g.p));
    a.N       = basis.N;
    a.nz      = mesh.dim == 2 ? 1 : basis.N;
    a.nc      = fine->nc;
    a.Nn0     = g.Nn[0];
    a.Nn1     = g.Nn[1];
    for (int i = 0; i < basis.N; ++i)
      {
        a.lx[i] = lag(i, xi[0]);
        a.ly[i] = lag(i, xi[1]);
        a.lz[i] = mesh.dim == 2 ? 1.0 : lag(i, xi[2]);
      }
    point_dev.ensure(4 * sizeof(double));
    point_host.ensure(4);
    k_point_value<<<1, 32, 0, ctx->stream>>>(a, u.as<double>(), point_dev.as<double>());
    count_launch();
    MF_CK(cudaGetLastError());
    MF_CK(cudaMemcpyAsync(point_host.p, point_dev.ptr, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    std::vector<double> r(3, 0.0);
    for (int c = 0; c < fine->nc; ++c)
      r[c] = point_host.p[c];
    return r;
  }

  void
  SolidDriver::reset(const mfgpu_solid_params &p)
  {
    const double a1 = P.material.alpha_1;
    P               = p;
    P.material.alpha_1 = a1;
    P.caching          = nullptr;
    const size_t n     = fine->m();
    for (DevBuf *b : {&u, &delta, &v_old, &a_old, &acc, &rhs, &du})
      MF_CK(cudaMemsetAsync(b->ptr, 0, n * sizeof(double), ctx->stream));
    step_no = 0;
    table.clear();
  }

  void
  SolidDriver::run(mfgpu_solid_result &res)
  {
    auto t0 = std::chrono::steady_clock::now();
    std::memset(&res, 0, sizeof(res));
    if (P.n_steps > 64)
      throw Error(ERR_ARG, "at most 64 time steps per run");
    res.n_steps = P.n_steps;
    for (int s = 0; s < P.n_steps; ++s)
      {
        long cg = 0;
        int  solves = 0;
        step(res.newton_its[s], cg, solves, res.watch_disp[s]);
        res.total_cg += cg;
        res.n_solves += solves;
      }
    ctx->sync();
    res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  void
  SolidDriver::step(int &newton_its, long &total_cg, int &n_solves, double *watch)
  {
    const size_t n  = fine->m();
    const double dt = P.dt, beta = 0.25, gamma = 0.5;
    const double a1 = 1. / (beta * dt * dt), a2 = 1. / (beta * dt), a3 = (1 - 2 * beta) / (2 * beta),
                 a4 = gamma / (beta * dt), a5 = 1 - gamma / beta, a6 = (1 - gamma / (2 * beta)) * dt;
    double *U = u.as<double>(), *Dl = delta.as<double>(), *V = v_old.as<double>(),
           *Ao = a_old.as<double>(), *Ac = acc.as<double>(), *R = rhs.as<double>(), *DU = du.as<double>();
    total_cg = 0;
    n_solves = 0;
    table.clear();
    table_step = step_no + 1;
    MF_CK(cudaMemsetAsync(Dl, 0, n * sizeof(double), ctx->stream));
    double err_res0 = 0, err_upd = 0, err_upd0 = 0, err_upd_norm = 0;
    int    it       = 0;
    for (; it < P.max_newton; ++it)
      {
        // update_acceleration (mf_elasticity.h:1616-1620)
        vec_axpbyz<double>(*ctx, n, a1, Dl, -a2, V, Ac);
        vec_axpby<double>(*ctx, n, -a3, Ao, 1.0, Ac);
        const double err_res = assemble_residual();
        if (!std::isfinite(err_res))
          throw Error(ERR_NONFINITE, "non-finite residual");
        if (it == 0)
          err_res0 = err_res;
        const double err_res_norm = err_res0 != 0 ? err_res / err_res0 : err_res;
        if (it > 2)
          {
            bool conv = (err_res <= P.tol_f_abs || err_upd <= P.tol_u_abs);
            if (err_res_norm <= P.tol_f && err_upd_norm <= P.tol_u)
              conv = true;
            if (conv)
              break;
          }
        update_operators(U);
        const int its = solve_linear(R, DU, P.solver.tol * err_res);
        total_cg += its;
        n_solves++;
        err_upd = std::sqrt(vec_dot<double>(*ctx, n, DU, DU));
        if (it == 0)
          err_upd0 = err_upd;
        err_upd_norm = err_upd0 != 0 ? err_upd / err_upd0 : err_upd;
        table.push_back({it, its, last_lin_res, last_cond, err_res_norm, err_res, err_upd_norm, err_upd});
        vec_axpby<double>(*ctx, n, 1.0, DU, 1.0, Dl);
        vec_axpby<double>(*ctx, n, 1.0, DU, 1.0, U);
      }
    if (it >= P.max_newton)
      throw Error(ERR_NOT_CONVERGED, "no convergence in nonlinear solver");
    newton_its = it;
    // update_velocity (mf_elasticity.h:1602-1610): v = a4 delta + a5 v_old + a6 a_old
    vec_axpby<double>(*ctx, n, a6, Ao, a5, V);
    vec_axpby<double>(*ctx, n, a4, Dl, 1.0, V);
    vec_copy<double>(*ctx, n, Ac, Ao);
    const std::vector<double> w = point_value(P.watch);
    for (int d = 0; d < 3; ++d)
      watch[d] = w[d];
    ++step_no;
  }

  // ---------------------------------------------------------------------
  // heat
  // ---------------------------------------------------------------------
  HeatDriver::HeatDriver(Context *c, const mfgpu_heat_params &p, int batch)
    : ctx(c)
    , P(p)
    , nb(batch)
    , Pb(size_t(batch), p)
  {
    mesh = to_mesh(P.mesh);
    L    = mesh.n_ref;
    make_host_basis(mesh.degree, basis);
    if (nb < 1 || nb > 6 || (nb > 1 && mesh.dim != 3))
      throw Error(ERR_ARG, "heat batches: 1..6 three-dimensional problems");
    op          = make_heat(ctx, mesh, -1, 64, true, nb);
    op->delta_t = P.dt;
    op_u        = make_heat(ctx, mesh, -1, 64, false, nb);
    op_u->delta_t = P.dt;
    const bool emul = P.solver.fp64_emulation != 0;
    op->arith       = emul ? 1 : 0;
    op_u->arith     = emul ? 1 : 0;
    const size_t n = op->m();
    for (DevBuf *b : {&sol, &sol_old, &rhs, &du, &uD})
      {
        b->alloc(n * sizeof(double));
        MF_CK(cudaMemsetAsync(b->ptr, 0, n * sizeof(double), ctx->stream));
      }
    if (P.solver.preconditioner == 2)
      {
        gmg   = GMGHierarchy::heat(ctx, mesh, P.solver, P.dt, nb);
        lprec = gmg->lprec;
      }
  }

  void
  HeatDriver::node_x(size_t g, double *x) const
  {
    const LevelGeom &G = op->geom;
    int              ii[3];
    ii[0] = int(g % G.Nn[0]);
    g /= G.Nn[0];
    ii[1] = int(g % G.Nn[1]);
    ii[2] = int(g / G.Nn[1]);
    for (int d = 0; d < 3; ++d)
      {
        const int c  = std::min(ii[d] / G.p, G.C[d] - 1);
        const int li = ii[d] - c * G.p;
        x[d]         = G.lo[d] + (c + basis.nodes[li]) * G.h[d];
      }
  }

  void
  HeatDriver::start()
  {
    const size_t n  = op->m();
    const size_t n0 = op->geom.n_nodes; // one problem
    for (int b = 0; b < nb; ++b)
      if (Pb[b].analytic)
        {
          std::vector<double> h(n0);
          for (size_t g = 0; g < n0; ++g)
            {
              double x[3];
              node_x(g, x);
              h[g] = 1 + x[0] * x[0] + Pb[b].alpha * x[1] * x[1];
            }
          MF_CK(cudaMemcpyAsync(sol.as<double>() + b * n0, h.data(), n0 * sizeof(double), cudaMemcpyHostToDevice,
                                ctx->stream));
          ctx->sync();
        }
    vec_copy<double>(*ctx, n, sol.as<double>(), sol_old.as<double>());
    // the level operators stay fixed over the time steps: their diagonals
    // and the dense coarse operator are made once
    if (P.solver.preconditioner == 2)
      gmg->update_diagonals(timer);
    if (P.solver.preconditioner == 1)
      op->compute_diagonal();
    srcs.assign(size_t(nb), SourceDesc{});
    for (int b = 0; b < nb; ++b)
      {
        const mfgpu_heat_params &q  = Pb[b];
        SourceDesc              &sd = srcs[b];
        std::memset(&sd, 0, sizeof(sd));
        sd.constant = q.analytic ? q.beta - 2 - 2 * q.alpha : 0.0;
        sd.n_gauss  = q.analytic ? 0 : q.n_gauss;
        for (int i = 0; i < 8; ++i)
          {
            for (int d = 0; d < 3; ++d)
              sd.center[i][d] = q.g_center[i][d];
            sd.width[i] = q.g_width[i];
            sd.amp[i]   = q.g_amp[i];
          }
      }
    src     = srcs[0];
    t       = 0;
    step_no = 0;
    started = true;
  }

  int
  HeatDriver::step()
  {
    return step_batch()[0];
  }

  std::vector<int>
  HeatDriver::step_batch()
  {
    if (!started)
      start();
    const size_t     n  = op->m();
    const size_t     n0 = op->geom.n_nodes;
    const LevelGeom &G  = op->geom;
    t += P.dt;
    ++step_no;
    std::unique_ptr<PhaseTimer::Scope> ts(new PhaseTimer::Scope(timer, ctx, "assemble rhs"));
    // inhomogeneous Dirichlet values on the constrained nodes at time t
    MF_CK(cudaMemsetAsync(uD.ptr, 0, n * sizeof(double), ctx->stream));
    for (int b = 0; b < nb; ++b)
      if (Pb[b].analytic)
        {
          std::vector<double> hd(n0, 0.0);
          for (size_t g = 0; g < n0; ++g)
            {
              int    ii[3];
              size_t gg = g;
              ii[0]     = int(gg % G.Nn[0]);
              gg /= G.Nn[0];
              ii[1] = int(gg % G.Nn[1]);
              ii[2] = int(gg / G.Nn[1]);
              if (node_mask(G.face_mask, G.Nn, ii[0], ii[1], ii[2]) & 1u)
                {
                  double x[3];
                  node_x(g, x);
                  hd[g] = 1 + x[0] * x[0] + Pb[b].alpha * x[1] * x[1] + Pb[b].beta * t;
                }
            }
          MF_CK(cudaMemcpyAsync(uD.as<double>() + b * n0, hd.data(), n0 * sizeof(double), cudaMemcpyHostToDevice,
                                ctx->stream));
          ctx->sync();
        }
    // rhs = -A_unconstrained uD + int (u_old + dt f) v; without Dirichlet
    // data (uD = 0, the homogeneous problems) the first term is zero
    bool any_lift = false;
    for (int b = 0; b < nb; ++b)
      any_lift = any_lift || Pb[b].analytic;
    if (any_lift)
      {
        op_u->vmult(rhs.ptr, uD.ptr);
        vec_axpby<double>(*ctx, n, 0.0, rhs.as<double>(), -1.0, rhs.as<double>());
      }
    else
      MF_CK(cudaMemsetAsync(rhs.ptr, 0, n * sizeof(double), ctx->stream));
    std::vector<double> tol(static_cast<size_t>(nb), 0.0);
    for (int b = 0; b < nb; ++b)
      {
        double *rb = rhs.as<double>() + b * n0;
        if (G.dim == 2)
          MF_CK(launch_heat_rhs2d(basis.N, basis, G, P.dt, srcs[b], sol_old.as<double>() + b * n0, rb, ctx->stream));
        else
          {
            src_tab.ensure(heat_rhs_table_size(G, basis.N) * sizeof(double));
            MF_CK(dispatch_heat_rhs(basis.N, basis, G, P.dt, srcs[b], sol_old.as<double>() + b * n0, rb,
                                    src_tab.as<double>(), ctx->stream));
            if (srcs[b].n_gauss > 0)
              count_launch(); // the source table
          }
        count_launch();
        tol[b] = P.solver.tol * std::sqrt(vec_dot<double>(*ctx, n0, rb, rb));
      }
    ts.reset();
    FineOp A;
    A.op = op.get();
    JacobiPre64      J;
    Precond<double> *M = nullptr;
    if (P.solver.preconditioner == 2)
      {
        gmg->setup_smoothers(timer);
        M = gmg->precond();
      }
    else if (P.solver.preconditioner == 1)
      {
        J.ctx   = ctx;
        J.A     = op.get();
        J.omega = 0.7;
        M       = &J;
      }
    std::vector<int> its(size_t(nb), 0);
    {
      PhaseTimer::Scope tsol(timer, ctx, "solve system");
      if (nb == 1)
        {
          const CGStats st = cg_solve<double>(*ctx, A, M, du.as<double>(), rhs.as<double>(), tol[0], int(n), false,
                                              false, &cg_ws);
          if (!st.converged)
            throw Error(ERR_NOT_CONVERGED, "CG did not converge");
          its[0] = st.its;
        }
      else if (!cg_solve_batched(*ctx, A, M, du.as<double>(), rhs.as<double>(), nb, n0, tol, int(n0), its, &cg_ws))
        throw Error(ERR_NOT_CONVERGED, "CG did not converge");
    }
    constrained_op<double>(*ctx, G, nb, 2, nullptr, du.as<double>());
    vec_axpbyz<double>(*ctx, n, 1.0, uD.as<double>(), 1.0, du.as<double>(), sol.as<double>());
    vec_copy<double>(*ctx, n, sol.as<double>(), sol_old.as<double>());
    return its;
  }

  void
  HeatDriver::reset(const mfgpu_heat_params &p)
  {
    reset_batch(std::vector<mfgpu_heat_params>(size_t(nb), p));
  }

  void
  HeatDriver::reset_batch(const std::vector<mfgpu_heat_params> &ps)
  {
    if (int(ps.size()) != nb)
      throw Error(ERR_ARG, "reset_batch: one parameter set per problem of the batch");
    Pb             = ps;
    P              = ps[0];
    const size_t n = op->m();
    for (DevBuf *b : {&sol, &sol_old, &rhs, &du, &uD})
      MF_CK(cudaMemsetAsync(b->ptr, 0, n * sizeof(double), ctx->stream));
    started = false;
    step_no = 0;
    t       = 0;
  }

  void
  HeatDriver::run(mfgpu_heat_result &res)
  {
    auto t0 = std::chrono::steady_clock::now();
    std::memset(&res, 0, sizeof(res));
    if (P.n_steps > 64)
      throw Error(ERR_ARG, "at most 64 time steps per run");
    res.n_steps = P.n_steps;
    start();
    for (int s = 0; s < P.n_steps; ++s)
      res.cg_its[s] = step();
    ctx->sync();
    res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
} // namespace mfgpu
