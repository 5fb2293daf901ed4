// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle_core.hpp).
//
// End-to-end drivers: the solid Newton-Newmark time loop
// (Solid::run / solve_nonlinear_timestep / assemble_residual,
// include/solid_mechanics/mf_elasticity.h:555-628, 1402-1491, 1649-1908) and
// the backward-Euler heat step (LaplaceProblem::assemble_rhs / solve,
// include/heat_transfer/heat_transfer.h:579-655, 715-812), with the
// preCICE coupling replaced by a constant boundary traction / analytic
// Dirichlet data.
#pragma once

#include "oracle_fast_api.hpp"
#include "oracle_solvers.hpp"

namespace orc
{
  struct MeshSpec
  {
    int      dim = 3, degree = 1, n_q = 2, n_ref = 0;
    int      rep[3]{1, 1, 1};
    double   lo[3]{0, 0, 0}, hi[3]{1, 1, 1};
    int      boundary_id[6]{0, 0, 0, 0, 0, 0};
    int      n_dirichlet = 0;
    int      dirichlet_id[8]{};
    unsigned dirichlet_mask[8]{};

    void
    face_masks(unsigned *m) const
    {
      for (int f = 0; f < 6; ++f)
        {
          m[f] = 0;
          if (f >= 2 * dim)
            continue;
          for (int i = 0; i < n_dirichlet; ++i)
            if (boundary_id[f] == dirichlet_id[i])
              m[f] |= dirichlet_mask[i];
        }
    }

    Box
    box(int level) const
    {
      unsigned m[6];
      face_masks(m);
      return Box(dim, degree, rep, lo, hi, level, m);
    }
  };

  // Real coordinates of the quadrature points of a cell
  inline void
  qp_coords(const Box &box, const Basis1D &b, size_t e, int q, double *x)
  {
    int cc[3];
    box.cell_coords(e, cc);
    for (int d = 0; d < box.dim; ++d)
      {
        x[d] = box.lo[d] + (cc[d] + b.xq[q % b.Q]) * box.h[d];
        q /= b.Q;
      }
  }

  // ---------------------------------------------------------------------
  // Solid
  // ---------------------------------------------------------------------
  struct SolidParams
  {
    MeshSpec mesh;
    Material mat; // alpha_1 filled by the driver from dt
    int      caching        = 0;
    int      precond        = 2; // 0 none, 1 jacobi, 2 gmg
    double   relaxation     = 0.65;
    double   tol_lin        = 1e-6;
    int      max_it_mult    = 1;
    int      max_newton     = 10;
    double   tol_f = 1e-9, tol_f_abs = 0, tol_u = 1e-6, tol_u_abs = 0;
    double   dt             = 0.1;
    int      n_steps        = 2;
    double   body_force[3]{0, 0, 0};
    int      traction_id    = 11;
    double   traction[3]{0, 0, 0};
    double   watch[3]{0, 0, 0};
    int      cheb_degree    = 5;
    double   cheb_range     = 20;
    int      cheb_eig_its   = 30;
    int      coarse_accurate = 1;
    int      mg_float       = 1; // level operators in FP32 (reference)
    int      fast           = 0; // operators in the throughput form (oracle_fast.hpp)
  };

  struct SolidResult
  {
    int    newton_its[64]{};
    double watch_disp[64][3]{};
    long   total_cg = 0;
    int    n_solves = 0;
    int    n_steps  = 0;
    int    ok       = 1;
  };

  template <typename T>
  struct ResidualQ
  {
    static constexpr bool has_val  = true;
    static constexpr bool has_grad = true;
    const Material       *mat;
    const Box            *box;
    const Basis1D        *basis;
    const double         *acc;
    const double         *body;
    void
    cell(size_t e, int nc, int Qp, T *val, T *grad)
    {
      const int dim = box->dim;
      thread_local CellScratch<T> s;
      thread_local std::vector<T> av;
      thread_local int            key = -1;
      const int k = dim * 1000 + basis->N * 10 + basis->Q;
      if (key != k)
        {
          s.init(dim, dim, basis->N, basis->Q);
          av.resize(size_t(dim) * Qp);
          key = k;
        }
      // acceleration values at the qp (read_dof_values_plain + evaluate)
      const int Nd = ipow(basis->N, dim);
      box->cell_nodes(e, s.nodes.data());
      const DirMats m = cell_mats(*basis);
      for (int c = 0; c < nc; ++c)
        {
          for (int l = 0; l < Nd; ++l)
            s.u[l] = T(acc[size_t(c) * box->n_nodes + s.nodes[l]]);
          evaluate_scalar(dim, basis->N, m, s.u.data(), av.data() + size_t(c) * Qp,
                          (T *)nullptr, s.w0.data(), s.w1.data(), s.w2.data(),
                          s.w3.data());
        }
      for (int q = 0; q < Qp; ++q)
        {
          T H[9], F[9], Fi[9], tau[9];
          for (int c = 0; c < dim; ++c)
            for (int d = 0; d < dim; ++d)
              {
                H[c * dim + d] = grad[(size_t(c) * dim + d) * Qp + q];
                F[c * dim + d] = H[c * dim + d] + (c == d ? T(1) : T(0));
              }
          get_tau(*mat, dim, H, tau);
          invert(dim, F, Fi);
          for (int i = 0; i < dim; ++i)
            for (int j = 0; j < dim; ++j)
              {
                T sum = T(0);
                for (int k2 = 0; k2 < dim; ++k2)
                  sum += tau[i * dim + k2] * Fi[j * dim + k2];
                grad[(size_t(i) * dim + j) * Qp + q] = -sum;
              }
          for (int c = 0; c < dim; ++c)
            val[size_t(c) * Qp + q] =
              (-av[size_t(c) * Qp + q] + T(body[c])) * T(mat->rho);
        }
    }
  };

  // Traction face term (mf_elasticity.h:1849-1897): pulled-back traction
  // t |det F F^{-T} N| on the faces with the interface boundary id.
  inline void
  traction_term(const Box &box, const Basis1D &b, const MeshSpec &ms,
                int traction_id, const double *t, const double *u, double *rhs)
  {
    const int dim = box.dim;
    const int N   = b.N;
    const int Nd  = ipow(N, dim);
    CellScratch<double> s;
    s.init(dim, dim, N, b.Q);
    for (int f = 0; f < 2 * dim; ++f)
      {
        if (ms.boundary_id[f] != traction_id)
          continue;
        const int     nd   = f / 2;
        const int     side = f % 2;
        const DirMats m    = face_mats(b, nd, side);
        int           Qf   = 1;
        for (int d = 0; d < dim; ++d)
          Qf *= m.Q[d];
        double Nvec[3] = {0, 0, 0};
        Nvec[nd]       = side ? 1.0 : -1.0;
        std::vector<double> grad(size_t(dim) * dim * Qf), val(size_t(dim) * Qf);
        for (size_t e = 0; e < box.n_cells; ++e)
          {
            int cc[3];
            box.cell_coords(e, cc);
            if (cc[nd] != (side ? box.C[nd] - 1 : 0))
              continue;
            box.cell_nodes(e, s.nodes.data());
            for (int c = 0; c < dim; ++c)
              {
                for (int l = 0; l < Nd; ++l)
                  s.u[l] = u[size_t(c) * box.n_nodes + s.nodes[l]];
                evaluate_scalar(dim, N, m, s.u.data(), (double *)nullptr,
                                grad.data() + size_t(c) * dim * Qf, s.w0.data(),
                                s.w1.data(), s.w2.data(), s.w3.data());
                for (int d = 0; d < dim; ++d)
                  for (int q = 0; q < Qf; ++q)
                    grad[(size_t(c) * dim + d) * Qf + q] /= box.h[d];
              }
            for (int q = 0; q < Qf; ++q)
              {
                double F[9], Fi[9];
                for (int c = 0; c < dim; ++c)
                  for (int d = 0; d < dim; ++d)
                    F[c * dim + d] = grad[(size_t(c) * dim + d) * Qf + q] +
                                     (c == d ? 1.0 : 0.0);
                const double J = det(dim, F);
                invert(dim, F, Fi);
                double ns = 0;
                for (int i = 0; i < dim; ++i)
                  {
                    double v = 0;
                    for (int k = 0; k < dim; ++k)
                      v += Fi[k * dim + i] * Nvec[k]; // (F^{-T} N)_i
                    ns += (J * v) * (J * v);
                  }
                ns = std::sqrt(ns);
                // face JxW
                double w = 1;
                int    qq = q;
                for (int d = 0; d < dim; ++d)
                  {
                    const int qd = qq % m.Q[d];
                    qq /= m.Q[d];
                    if (d != nd)
                      w *= b.wq[qd] * box.h[d];
                  }
                for (int c = 0; c < dim; ++c)
                  val[size_t(c) * Qf + q] = t[c] * ns * w;
              }
            for (int c = 0; c < dim; ++c)
              {
                integrate_scalar(dim, N, m, val.data() + size_t(c) * Qf,
                                 (const double *)nullptr, s.out.data(),
                                 s.w0.data(), s.w1.data(), s.w2.data(),
                                 s.w3.data());
                for (int l = 0; l < Nd; ++l)
                  rhs[size_t(c) * box.n_nodes + s.nodes[l]] += s.out[l];
              }
          }
      }
  }

  template <typename LT>
  struct SolidDriver
  {
    SolidParams                 P;
    Basis1D                     basis;
    int                         L = 0; // finest level
    std::vector<Box>            boxes;
    LevelOp<double>             fine;
    std::vector<LevelOp<LT>>    lops;
    Multigrid<LT>               mg;
    std::vector<std::vector<LT>> u_levels;

    explicit SolidDriver(const SolidParams &p)
      : P(p)
      , basis(p.mesh.degree, p.mesh.n_q)
    {
      L = P.mesh.n_ref;
      for (int l = 0; l <= L; ++l)
        boxes.push_back(P.mesh.box(l));
      const double beta = 0.25;
      P.mat.alpha_1     = 1. / (beta * P.dt * P.dt);
      fine.box          = boxes[L];
      fine.basis        = &basis;
      fine.nc           = P.mesh.dim;
      fine.kind         = op_nh;
      fine.nh.mat       = P.mat;
      fine.nh.caching   = Caching(P.caching);
      if (P.precond == 2)
        {
          lops.resize(L + 1);
          u_levels.resize(L + 1);
          for (int l = 0; l <= L; ++l)
            {
              lops[l].box        = boxes[l];
              lops[l].basis      = &basis;
              lops[l].nc         = P.mesh.dim;
              lops[l].kind       = op_nh;
              lops[l].nh.mat     = P.mat;
              lops[l].nh.caching = Caching(P.caching);
            }
          mg.ops.clear();
          mg.transfers.clear();
          for (int l = 0; l <= L; ++l)
            {
              mg.ops.push_back(&lops[l]);
              if (l == 0)
                mg.transfers.emplace_back(nullptr);
              else
                mg.transfers.emplace_back(new LevelTransfer<LT>(
                  basis, lops[l - 1].box, lops[l].box, P.mesh.dim));
            }
        }
    }

    // update_matrix_free: cache + diagonal on the fine level and every level
    void
    update_operators(const std::vector<double> &u)
    {
      if (P.fast)
        {
          bool ok = true;
          fine.fast = make_fast_nh(fine.box, basis, P.mat, Caching(P.caching), u.data(), ok);
          fine.nh.positive_J = ok;
        }
      else
        nh_cache(fine.nh, fine.box, basis, u.data());
      if (P.precond == 1)
        fine.compute_diagonal();
      if (P.precond != 2)
        return;
      const size_t nf = lops[L].m();
      u_levels[L].resize(nf);
      for (size_t i = 0; i < nf; ++i)
        u_levels[L][i] = LT(u[i]);
      for (int l = L; l > 0; --l)
        {
          u_levels[l - 1].assign(lops[l - 1].m(), LT(0));
          mg.transfers[l]->interpolate(u_levels[l - 1].data(),
                                       u_levels[l].data());
        }
      for (int l = 0; l <= L; ++l)
        {
          if (P.fast)
            {
              bool ok = true;
              lops[l].fast = make_fast_nh(lops[l].box, basis, P.mat, Caching(P.caching), u_levels[l].data(), ok);
            }
          else
            nh_cache(lops[l].nh, lops[l].box, basis, u_levels[l].data());
          lops[l].compute_diagonal();
        }
      mg.setup(P.cheb_range, P.cheb_degree, P.cheb_eig_its,
               P.coarse_accurate ? int(lops[0].m()) : P.cheb_eig_its);
    }

    void
    assemble_residual(const std::vector<double> &u,
                      const std::vector<double> &acc, std::vector<double> &rhs)
    {
      std::fill(rhs.begin(), rhs.end(), 0.0);
      ResidualQ<double> q{&P.mat, &fine.box, &basis, acc.data(), P.body_force};
      cell_loop(fine.box, basis, P.mesh.dim, u.data(), rhs.data(), q, false);
      traction_term(fine.box, basis, P.mesh, P.traction_id, P.traction,
                    u.data(), rhs.data());
      set_constrained_zero(fine.box, P.mesh.dim, rhs.data());
    }

    // one linear solve; returns CG iterations
    int
    solve_linear(const std::vector<double> &rhs, std::vector<double> &du,
                 double tol)
    {
      const size_t n = fine.m();
      std::fill(du.begin(), du.end(), 0.0);
      auto A = [&](double *d, const double *s) { fine.vmult(d, s); };
      CGResult R;
      const int maxit = int(n) * P.max_it_mult;
      if (P.precond == 1)
        {
          auto Pj = [&](double *d, const double *s) {
            for (size_t i = 0; i < n; ++i)
              d[i] = P.relaxation * fine.inv_diag[i] * s[i];
          };
          R = cg_solve<double>(n, A, Pj, du.data(), rhs.data(), tol, maxit);
        }
      else if (P.precond == 2)
        {
          auto Pm = [&](double *d, const double *s) { mg.vmult(d, s); };
          R = cg_solve<double>(n, A, Pm, du.data(), rhs.data(), tol, maxit);
        }
      else
        {
          auto Pi = [&](double *d, const double *s) { std::copy(s, s + n, d); };
          R = cg_solve<double>(n, A, Pi, du.data(), rhs.data(), tol, maxit);
        }
      set_constrained_zero(fine.box, P.mesh.dim, du.data());
      return R.its;
    }

    void
    run(SolidResult &res)
    {
      const size_t n  = fine.m();
      const double dt = P.dt, beta = 0.25, gamma = 0.5;
      const double a1 = 1. / (beta * dt * dt), a2 = 1. / (beta * dt),
                   a3 = (1 - 2 * beta) / (2 * beta), a4 = gamma / (beta * dt),
                   a5 = 1 - gamma / beta, a6 = (1 - gamma / (2 * beta)) * dt;
      std::vector<double> u(n, 0.), delta(n, 0.), v_old(n, 0.), a_old(n, 0.),
        acc(n, 0.), rhs(n, 0.), du(n, 0.);
      res.n_steps = P.n_steps;
      for (int step = 0; step < P.n_steps; ++step)
        {
          std::fill(delta.begin(), delta.end(), 0.0);
          double err_res0 = 0, err_upd = 0, err_upd0 = 0, err_upd_norm = 0;
          int    it       = 0;
          for (; it < P.max_newton; ++it)
            {
              for (size_t i = 0; i < n; ++i)
                acc[i] = a1 * delta[i] - a2 * v_old[i] - a3 * a_old[i];
              assemble_residual(u, acc, rhs);
              const double err_res = norm(n, rhs.data());
              if (it == 0)
                err_res0 = err_res;
              const double err_res_norm =
                err_res0 != 0 ? err_res / err_res0 : err_res;
              if (it > 2)
                {
                  bool conv = (err_res <= P.tol_f_abs || err_upd <= P.tol_u_abs);
                  if (err_res_norm <= P.tol_f && err_upd_norm <= P.tol_u)
                    conv = true;
                  if (conv)
                    break;
                }
              update_operators(u);
              if (!fine.nh.positive_J)
                {
                  res.ok = 0;
                  return;
                }
              const int its = solve_linear(rhs, du, P.tol_lin * err_res);
              res.total_cg += its;
              res.n_solves++;
              err_upd = norm(n, du.data());
              if (it == 0)
                err_upd0 = err_upd;
              err_upd_norm = err_upd0 != 0 ? err_upd / err_upd0 : err_upd;
              for (size_t i = 0; i < n; ++i)
                {
                  delta[i] += du[i];
                  u[i] += du[i];
                }
            }
          res.newton_its[step] = it;
          // update_velocity (mf_elasticity.h:1602-1610)
          for (size_t i = 0; i < n; ++i)
            {
              const double v = a4 * delta[i] + a5 * v_old[i] + a6 * a_old[i];
              v_old[i]       = v;
              a_old[i]       = acc[i];
            }
          std::vector<double> w =
            point_value(fine.box, basis, P.mesh.dim, u.data(), P.watch);
          for (int d = 0; d < P.mesh.dim; ++d)
            res.watch_disp[step][d] = w[d];
        }
      last_u = u;
    }

    std::vector<double> last_u;
  };

  // ---------------------------------------------------------------------
  // Heat
  // ---------------------------------------------------------------------
  struct HeatParams
  {
    MeshSpec mesh;
    double   dt       = 0.1;
    int      n_steps  = 1;
    double   tol_rel  = 1e-12;
    int      precond  = 2; // 0 none, 1 jacobi (relaxation .7), 2 gmg
    int      analytic = 0; // 1: u = 1 + x^2 + alpha y^2 + beta t
    double   alpha = 3, beta = 1.3;
    int      n_gauss  = 0; // Gaussian source terms
    double   g_center[8][3]{};
    double   g_width[8]{};
    double   g_amp[8]{};
    int      mg_float = 1;
    int      fast     = 0; // operators in the throughput form (oracle_fast.hpp)
  };

  struct HeatResult
  {
    double l2_error[64]{};
    int    cg_its[64]{};
    int    n_steps = 0;
  };

  template <typename LT>
  struct HeatDriver
  {
    HeatParams                 P;
    Basis1D                    basis;
    int                        L = 0;
    std::vector<Box>           boxes;
    LevelOp<double>            op;   // constrained
    LevelOp<double>            op_u; // unconstrained
    std::vector<LevelOp<LT>>   lops;
    Multigrid<LT>              mg;
    std::vector<double>        solution;

    explicit HeatDriver(const HeatParams &p)
      : P(p)
      , basis(p.mesh.degree, p.mesh.n_q)
    {
      L = P.mesh.n_ref;
      for (int l = 0; l <= L; ++l)
        boxes.push_back(P.mesh.box(l));
      op.box   = boxes[L];
      op.basis = &basis;
      op.nc    = 1;
      op.kind  = op_heat;
      op.k_dt  = P.dt;
      op_u     = op;
      op_u.constrained = false;
      if (P.precond == 2)
        {
          lops.resize(L + 1);
          for (int l = 0; l <= L; ++l)
            {
              lops[l].box   = boxes[l];
              lops[l].basis = &basis;
              lops[l].nc    = 1;
              lops[l].kind  = op_heat;
              lops[l].k_dt  = P.dt;
            }
          for (int l = 0; l <= L; ++l)
            {
              mg.ops.push_back(&lops[l]);
              if (l == 0)
                mg.transfers.emplace_back(nullptr);
              else
                mg.transfers.emplace_back(
                  new LevelTransfer<LT>(basis, lops[l - 1].box, lops[l].box, 1));
            }
        }
      if (P.fast)
        {
          op.fast = make_fast_heat<double>(op.box, basis, P.dt);
          for (auto &lo : lops)
            lo.fast = make_fast_heat<LT>(lo.box, basis, P.dt);
        }
    }

    double
    exact(const double *x, double t) const
    {
      return 1 + x[0] * x[0] + P.alpha * x[1] * x[1] + P.beta * t;
    }

    double
    source(const double *x) const
    {
      if (P.analytic)
        return P.beta - 2 - 2 * P.alpha;
      double f = 0;
      for (int i = 0; i < P.n_gauss; ++i)
        {
          double r2 = 0;
          for (int d = 0; d < P.mesh.dim; ++d)
            {
              const double dx = x[d] - P.g_center[i][d];
              r2 += dx * dx;
            }
          f += P.g_amp[i] *
               std::exp(-r2 / (2 * P.g_width[i] * P.g_width[i]));
        }
      return f;
    }

    // node coordinates
    void
    node_x(const Box &box, size_t g, double *x) const
    {
      int ii[3];
      box.node_coords(g, ii);
      for (int d = 0; d < box.dim; ++d)
        {
          const int c  = std::min(ii[d] / box.p, box.C[d] - 1);
          const int li = ii[d] - c * box.p;
          x[d]         = box.lo[d] + (c + basis.nodes[li]) * box.h[d];
        }
    }

    double
    l2_error(const std::vector<double> &u, double t) const
    {
      const Box &box = op.box;
      const int  Qp  = ipow(basis.Q, box.dim);
      CellScratch<double> s;
      s.init(box.dim, 1, basis.N, basis.Q);
      const DirMats m  = cell_mats(basis);
      const int     Nd = ipow(basis.N, box.dim);
      double        err = 0;
      for (size_t e = 0; e < box.n_cells; ++e)
        {
          box.cell_nodes(e, s.nodes.data());
          for (int l = 0; l < Nd; ++l)
            s.u[l] = u[s.nodes[l]];
          evaluate_scalar(box.dim, basis.N, m, s.u.data(), s.val.data(),
                          (double *)nullptr, s.w0.data(), s.w1.data(),
                          s.w2.data(), s.w3.data());
          for (int q = 0; q < Qp; ++q)
            {
              double x[3];
              qp_coords(box, basis, e, q, x);
              const double d = exact(x, t) - s.val[q];
              err += d * d * qweight(basis, box.dim, q) * box.cell_volume();
            }
        }
      return std::sqrt(err);
    }

    struct RhsQ
    {
      static constexpr bool has_val  = true;
      static constexpr bool has_grad = false;
      const HeatDriver     *drv;
      void
      cell(size_t e, int, int Qp, double *val, double *)
      {
        for (int q = 0; q < Qp; ++q)
          {
            double x[3];
            qp_coords(drv->op.box, drv->basis, e, q, x);
            val[q] = val[q] + drv->P.dt * drv->source(x);
          }
      }
    };

    void
    run(HeatResult &res)
    {
      const Box   &box = op.box;
      const size_t n   = box.n_nodes;
      solution.assign(n, 0.0);
      std::vector<double> sol_old(n), rhs(n), du(n, 0.0), uD(n);
      double              t = 0;
      if (P.analytic)
        for (size_t g = 0; g < n; ++g)
          {
            double x[3];
            node_x(box, g, x);
            solution[g] = exact(x, 0.0);
          }
      sol_old = solution;
      if (P.precond == 2)
        for (int l = 0; l <= L; ++l)
          lops[l].compute_diagonal();
      if (P.precond == 1)
        op.compute_diagonal();
      res.n_steps = P.n_steps;
      for (int step = 0; step < P.n_steps; ++step)
        {
          t += P.dt;
          // inhomogeneous Dirichlet values at time t
          std::fill(uD.begin(), uD.end(), 0.0);
          if (P.analytic)
            for (size_t g = 0; g < n; ++g)
              if (box.constrained(g, 0))
                {
                  double x[3];
                  node_x(box, g, x);
                  uD[g] = exact(x, t);
                }
          // rhs = -A_unconstrained uD + (u_old + dt f, v)
          op_u.vmult(rhs.data(), uD.data());
          for (auto &r : rhs)
            r = -r;
          RhsQ q{this};
          cell_loop(box, basis, 1, sol_old.data(), rhs.data(), q, false, true,
                    false);
          const double tol = P.tol_rel * norm(n, rhs.data());
          auto A = [&](double *d, const double *s) { op.vmult(d, s); };
          CGResult R;
          if (P.precond == 2)
            {
              mg.setup(15., 5, 10, int(lops[0].m()));
              auto Pm = [&](double *d, const double *s) { mg.vmult(d, s); };
              R = cg_solve<double>(n, A, Pm, du.data(), rhs.data(), tol, int(n));
            }
          else if (P.precond == 1)
            {
              auto Pj = [&](double *d, const double *s) {
                for (size_t i = 0; i < n; ++i)
                  d[i] = 0.7 * op.inv_diag[i] * s[i];
              };
              R = cg_solve<double>(n, A, Pj, du.data(), rhs.data(), tol, int(n));
            }
          else
            {
              auto Pi = [&](double *d, const double *s) { std::copy(s, s + n, d); };
              R = cg_solve<double>(n, A, Pi, du.data(), rhs.data(), tol, int(n));
            }
          res.cg_its[step] = R.its;
          set_constrained_zero(box, 1, du.data());
          for (size_t i = 0; i < n; ++i)
            solution[i] = uD[i] + du[i];
          if (P.analytic)
            res.l2_error[step] = l2_error(solution, t);
          sol_old = solution;
        }
    }
  };
} // namespace orc
