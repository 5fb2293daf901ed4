// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle_core.hpp).
//
// Solver layer restated from the reference and from the deal.II classes it
// configures:
//   * level operators, inverse diagonals (mf_nh_operator.h:1025-1060,
//     heat_transfer.h:205-230);
//   * MGTransferMatrixFree prolongation / restriction / interpolate_to_mg for
//     continuous FE_Q on uniformly refined meshes (mf_elasticity.h:865-929,
//     heat_transfer.h:761-762);
//   * PreconditionChebyshev with CG-Lanczos eigenvalue estimates, used as the
//     smoother and (degree = invalid, smoothing range 1e-3) as the coarse
//     solver (mf_elasticity.h:1142-1198, heat_transfer.h:764-791);
//   * Multigrid V-cycle + PreconditionMG (mf_elasticity.h:1207-1276,
//     heat_transfer.h:793-808);
//   * SolverCG (mf_elasticity.h:1983-2070, heat_transfer.h:715-754);
//   * Newton-Newmark time stepping of the solid (mf_elasticity.h:237-245,
//     1359-1491, 1602-1620, 1649-1908) and the backward-Euler heat step
//     (heat_transfer.h:579-655, 715-754).
#pragma once

#include <functional>
#include <memory>

#include "oracle_ops.hpp"

namespace orc
{
  template <typename T>
  double
  dot(size_t n, const T *a, const T *b)
  {
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long i = 0; i < long(n); ++i)
      s += double(a[i]) * double(b[i]);
    return s;
  }

  template <typename T>
  double
  norm(size_t n, const T *a)
  {
    return std::sqrt(dot(n, a, a));
  }

  // ---------------------------------------------------------------------
  // Operator on one level (or the active level) in precision T.
  // ---------------------------------------------------------------------
  enum OpKind
  {
    op_heat = 0,
    op_nh   = 1
  };

  template <typename T>
  struct LevelOp
  {
    Box            box;
    const Basis1D *basis = nullptr;
    int            nc    = 1;
    OpKind         kind  = op_heat;
    double         k_dt  = 0;
    bool           constrained = true;
    NHState<T>     nh;
    std::vector<T> inv_diag;
    // when set, the throughput form (oracle_fast.hpp) applies the operator
    // and its cell diagonal in place of the loops below
    FastLevel<T>   fast;

    size_t
    m() const
    {
      return size_t(nc) * box.n_nodes;
    }

    void
    vmult(T *dst, const T *src)
    {
      if (fast.vmult && constrained)
        {
          fast.vmult(dst, src);
          return;
        }
      std::fill(dst, dst + m(), T(0));
      vmult_add(dst, src);
    }

    void
    vmult_add(T *dst, const T *src)
    {
      if (fast.vmult && constrained)
        {
          std::vector<T> t(m());
          fast.vmult(t.data(), src);
          for (size_t i = 0; i < m(); ++i)
            dst[i] += t[i];
          return;
        }
      if (kind == op_heat)
        {
          HeatQ<T> q{box.dim, k_dt};
          cell_loop(box, *basis, nc, src, dst, q, constrained);
        }
      else
        {
          NHQ<T> q{&nh};
          cell_loop(box, *basis, nc, src, dst, q, constrained);
        }
      if (constrained)
        constrained_identity(box, nc, src, dst);
    }

    // diagonal -> constrained entries 1 -> invert
    void
    compute_diagonal()
    {
      std::vector<T> diag(m(), T(0));
      if (fast.cell_diagonal)
        fast.cell_diagonal(diag.data());
      else if (kind == op_heat)
        {
          HeatQ<T> q{box.dim, k_dt};
          cell_diagonal(box, *basis, nc, diag.data(), q);
        }
      else
        {
          NHQ<T> q{&nh};
          cell_diagonal(box, *basis, nc, diag.data(), q);
        }
      for (size_t g = 0; g < box.n_nodes; ++g)
        for (int c = 0; c < nc; ++c)
          if (box.constrained(g, c))
            diag[size_t(c) * box.n_nodes + g] = T(1);
      inv_diag.resize(m());
      for (size_t i = 0; i < m(); ++i)
        inv_diag[i] = T(1) / diag[i];
    }
  };

  // ---------------------------------------------------------------------
  // 1D transfer matrices between level l (C cells) and level l+1 (2C cells)
  // ---------------------------------------------------------------------
  struct Transfer1D
  {
    int                 nf = 0, ncr = 0, p = 1;
    // prolongation: fine row f has (p+1) entries starting at coarse col c0
    std::vector<int>    P_col;
    std::vector<double> P_val;
    // interpolation fine -> coarse: coarse row i has (p+1) entries at fine cols
    std::vector<int>    R_col;
    std::vector<double> R_val;

    Transfer1D(const Basis1D &b, int C)
    {
      p   = b.p;
      nf  = 2 * C * p + 1;
      ncr = C * p + 1;
      P_col.resize(nf);
      P_val.resize(size_t(nf) * (p + 1));
      for (int f = 0; f < nf; ++f)
        {
          const int    fc = std::min(f / p, 2 * C - 1);
          const int    lf = f - fc * p;
          const int    c  = fc / 2;
          const double xi = 0.5 * (fc % 2) + 0.5 * b.nodes[lf];
          P_col[f]        = c * p;
          for (int i = 0; i <= p; ++i)
            P_val[size_t(f) * (p + 1) + i] = lagrange(b.nodes, i, xi);
        }
      R_col.resize(ncr);
      R_val.resize(size_t(ncr) * (p + 1));
      for (int i = 0; i < ncr; ++i)
        {
          const int    c  = std::min(i / p, C - 1);
          const int    li = i - c * p;
          const double xi = b.nodes[li];
          const int    child = xi < 0.5 ? 0 : 1;
          const double xl    = child == 0 ? 2 * xi : 2 * xi - 1;
          const int    fc    = 2 * c + child;
          R_col[i]           = fc * p;
          for (int j = 0; j <= p; ++j)
            R_val[size_t(i) * (p + 1) + j] = lagrange(b.nodes, j, xl);
        }
    }
  };

  // Apply a banded 1D operator (rows x (p+1) entries starting at col[r])
  // along direction dir of a lexicographic array.
  template <typename T>
  void
  apply_banded(int dim, const int *ext_in, int dir, int rows, int p,
               const int *col, const double *val, bool transposed, const T *in,
               T *out)
  {
    int stride = 1;
    for (int d = 0; d < dir; ++d)
      stride *= ext_in[d];
    int outer = 1;
    for (int d = dir + 1; d < dim; ++d)
      outer *= ext_in[d];
    const int Kin  = ext_in[dir];
    const int Kout = transposed ? /* cols */ 0 : rows;
    (void)Kout;
    if (!transposed)
      {
#pragma omp parallel for collapse(2) schedule(static)
        for (int o = 0; o < outer; ++o)
          for (int s = 0; s < stride; ++s)
            for (int r = 0; r < rows; ++r)
              {
                T acc = T(0);
                for (int i = 0; i <= p; ++i)
                  acc += T(val[size_t(r) * (p + 1) + i]) *
                         in[(size_t(o) * Kin + col[r] + i) * stride + s];
                out[(size_t(o) * rows + r) * stride + s] = acc;
              }
      }
    else
      {
        // out has extent `ncols` along dir; input extent Kin == rows
        // caller zero-initialises out
        int ncols = 0;
        for (int r = 0; r < rows; ++r)
          ncols = std::max(ncols, col[r] + p + 1);
        // each (o, s) line is written by one thread
#pragma omp parallel for collapse(2) schedule(static)
        for (int o = 0; o < outer; ++o)
          for (int s = 0; s < stride; ++s)
            for (int r = 0; r < rows; ++r)
              {
                const T x = in[(size_t(o) * Kin + r) * stride + s];
                for (int i = 0; i <= p; ++i)
                  out[(size_t(o) * ncols + col[r] + i) * stride + s] +=
                    T(val[size_t(r) * (p + 1) + i]) * x;
              }
      }
  }

  template <typename T>
  struct LevelTransfer
  {
    // from level l (coarse box) to l+1 (fine box)
    const Box *coarse = nullptr, *fine = nullptr;
    int        nc     = 1;
    std::vector<std::unique_ptr<Transfer1D>> t1d; // per direction

    LevelTransfer(const Basis1D &b, const Box &c, const Box &f, int nc_)
      : coarse(&c)
      , fine(&f)
      , nc(nc_)
    {
      for (int d = 0; d < c.dim; ++d)
        t1d.emplace_back(new Transfer1D(b, c.C[d]));
    }

    // fine = P coarse (coarse constrained entries read as zero)
    void
    prolongate(T *fine_v, const T *coarse_v) const
    {
      const int dim = coarse->dim;
      const int p   = coarse->p;
      std::vector<T> a, bbuf;
      for (int c = 0; c < nc; ++c)
        {
          a.assign(coarse_v + size_t(c) * coarse->n_nodes,
                   coarse_v + size_t(c + 1) * coarse->n_nodes);
#pragma omp parallel for schedule(static)
          for (size_t g = 0; g < coarse->n_nodes; ++g)
            if (coarse->constrained(g, c))
              a[g] = T(0);
          int ext[3] = {coarse->Nn[0], coarse->Nn[1], coarse->Nn[2]};
          for (int d = 0; d < dim; ++d)
            {
              int ext_out[3] = {ext[0], ext[1], ext[2]};
              ext_out[d]     = fine->Nn[d];
              bbuf.assign(size_t(ext_out[0]) * ext_out[1] * ext_out[2], T(0));
              apply_banded(dim, ext, d, t1d[d]->nf, p, t1d[d]->P_col.data(),
                           t1d[d]->P_val.data(), false, a.data(), bbuf.data());
              a.swap(bbuf);
              ext[d] = ext_out[d];
            }
#pragma omp parallel for schedule(static)
          for (size_t g = 0; g < fine->n_nodes; ++g)
            fine_v[size_t(c) * fine->n_nodes + g] =
              fine->constrained(g, c) ? T(0) : a[g];
        }
    }

    // coarse += P^T fine (coarse constrained entries zeroed)
    void
    restrict_add(T *coarse_v, const T *fine_v) const
    {
      const int dim = coarse->dim;
      const int p   = coarse->p;
      std::vector<T> a, bbuf;
      for (int c = 0; c < nc; ++c)
        {
          a.assign(fine_v + size_t(c) * fine->n_nodes,
                   fine_v + size_t(c + 1) * fine->n_nodes);
#pragma omp parallel for schedule(static)
          for (size_t g = 0; g < fine->n_nodes; ++g)
            if (fine->constrained(g, c))
              a[g] = T(0);
          int ext[3] = {fine->Nn[0], fine->Nn[1], fine->Nn[2]};
          for (int d = 0; d < dim; ++d)
            {
              int ext_out[3] = {ext[0], ext[1], ext[2]};
              ext_out[d]     = coarse->Nn[d];
              bbuf.assign(size_t(ext_out[0]) * ext_out[1] * ext_out[2], T(0));
              apply_banded(dim, ext, d, t1d[d]->nf, p, t1d[d]->P_col.data(),
                           t1d[d]->P_val.data(), true, a.data(), bbuf.data());
              a.swap(bbuf);
              ext[d] = ext_out[d];
            }
#pragma omp parallel for schedule(static)
          for (size_t g = 0; g < coarse->n_nodes; ++g)
            if (!coarse->constrained(g, c))
              coarse_v[size_t(c) * coarse->n_nodes + g] += a[g];
        }
    }

    // coarse = fine field evaluated at the coarse nodes (interpolate_to_mg)
    template <typename TF>
    void
    interpolate(T *coarse_v, const TF *fine_v) const
    {
      const int dim = coarse->dim;
      const int p   = coarse->p;
      std::vector<T> a, bbuf;
      for (int c = 0; c < nc; ++c)
        {
          a.resize(fine->n_nodes);
          for (size_t g = 0; g < fine->n_nodes; ++g)
            a[g] = T(fine_v[size_t(c) * fine->n_nodes + g]);
          int ext[3] = {fine->Nn[0], fine->Nn[1], fine->Nn[2]};
          for (int d = 0; d < dim; ++d)
            {
              int ext_out[3] = {ext[0], ext[1], ext[2]};
              ext_out[d]     = coarse->Nn[d];
              bbuf.assign(size_t(ext_out[0]) * ext_out[1] * ext_out[2], T(0));
              apply_banded(dim, ext, d, t1d[d]->ncr, p, t1d[d]->R_col.data(),
                           t1d[d]->R_val.data(), false, a.data(), bbuf.data());
              a.swap(bbuf);
              ext[d] = ext_out[d];
            }
          for (size_t g = 0; g < coarse->n_nodes; ++g)
            coarse_v[size_t(c) * coarse->n_nodes + g] = a[g];
        }
    }
  };

  // ---------------------------------------------------------------------
  // Extreme eigenvalues of a symmetric tridiagonal matrix (bisection on the
  // Sturm count).
  // ---------------------------------------------------------------------
  inline int
  sturm_count(const std::vector<double> &d, const std::vector<double> &e,
              double x)
  {
    int    cnt = 0;
    double q   = 1;
    for (size_t i = 0; i < d.size(); ++i)
      {
        const double ee = i ? e[i - 1] * e[i - 1] : 0.0;
        q               = d[i] - x - (i ? ee / q : 0.0);
        if (q == 0)
          q = 1e-300;
        if (q < 0)
          ++cnt;
      }
    return cnt;
  }

  inline double
  tridiag_eig(const std::vector<double> &d, const std::vector<double> &e,
              int k /* k-th smallest, 0-based */)
  {
    double lo = 1e300, hi = -1e300;
    for (size_t i = 0; i < d.size(); ++i)
      {
        double r = (i ? std::fabs(e[i - 1]) : 0.0) +
                   (i + 1 < d.size() ? std::fabs(e[i]) : 0.0);
        lo = std::min(lo, d[i] - r);
        hi = std::max(hi, d[i] + r);
      }
    for (int it = 0; it < 200; ++it)
      {
        const double mid = 0.5 * (lo + hi);
        if (sturm_count(d, e, mid) > k)
          hi = mid;
        else
          lo = mid;
      }
    return 0.5 * (lo + hi);
  }

  // ---------------------------------------------------------------------
  // Preconditioned CG with deal.II SolverCG semantics.  Returns the number
  // of iterations; optionally records the Lanczos tridiagonal.
  // ---------------------------------------------------------------------
  struct CGResult
  {
    int    its       = 0;
    double res       = 0;
    bool   converged = false;
    std::vector<double> diag, offdiag;
  };

  template <typename T, typename AOp, typename POp>
  CGResult
  cg_solve(size_t n, AOp &&A, POp &&P, T *x, const T *b, double tol, int maxit,
           bool lanczos = false, bool fixed_its = false)
  {
    CGResult       R;
    std::vector<T> r(n), z(n), p(n), q(n);
    A(q.data(), x);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i)
      r[i] = b[i] - q[i];
    double res = norm(n, r.data());
    R.res      = res;
    if (res <= tol && !fixed_its)
      {
        R.converged = true;
        return R;
      }
    P(z.data(), r.data());
    double rz = dot(n, r.data(), z.data());
    std::copy(z.begin(), z.end(), p.begin());
    double alpha_old = 0, beta_old = 0;
    for (int it = 1; it <= maxit; ++it)
      {
        A(q.data(), p.data());
        const double pq    = dot(n, p.data(), q.data());
        const double alpha = rz / pq;
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n; ++i)
          {
            x[i] += T(alpha) * p[i];
            r[i] -= T(alpha) * q[i];
          }
        res    = norm(n, r.data());
        R.its  = it;
        R.res  = res;
        if (lanczos)
          {
            R.diag.push_back(1. / alpha + (it > 1 ? beta_old / alpha_old : 0.));
            if (it > 1)
              R.offdiag.push_back(std::sqrt(beta_old) / alpha_old);
          }
        if (res <= tol)
          {
            R.converged = true;
            break;
          }
        P(z.data(), r.data());
        const double rz_new = dot(n, r.data(), z.data());
        const double beta   = rz_new / rz;
        rz                  = rz_new;
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n; ++i)
          p[i] = z[i] + T(beta) * p[i];
        alpha_old = alpha;
        beta_old  = beta;
      }
    return R;
  }

  // ---------------------------------------------------------------------
  // Chebyshev smoother (deal.II PreconditionChebyshev semantics).
  // ---------------------------------------------------------------------
  template <typename T>
  struct Chebyshev
  {
    LevelOp<T> *A                 = nullptr;
    double      smoothing_range   = 20;
    unsigned    degree            = 5; // 0 == "invalid": choose from range
    int         eig_cg_iterations = 30;
    bool        initialized       = false;
    double      theta = 0, delta = 0, lambda_max = 0, lambda_min = 0;
    std::vector<T> x_old, t1, t2;

    void
    estimate()
    {
      const size_t   n = A->m();
      std::vector<T> rhs(n), sol(n, T(0));
      // initial guess with high-frequency content and the constant mode
      for (size_t i = 0; i < n; ++i)
        rhs[i] = (i % 11 == 0) ? T(0) : T(1);
      double mean = 0;
      for (size_t i = 0; i < n; ++i)
        mean += double(rhs[i]);
      mean /= double(n);
      for (size_t i = 0; i < n; ++i)
        rhs[i] -= T(mean);
      auto Aop = [&](T *d, const T *s) { A->vmult(d, s); };
      auto Pop = [&](T *d, const T *s) {
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n; ++i)
          d[i] = A->inv_diag[i] * s[i];
      };
      CGResult R = cg_solve<T>(n, Aop, Pop, sol.data(), rhs.data(), 1e-10,
                               eig_cg_iterations, true, false);
      if (R.diag.empty())
        lambda_min = lambda_max = 1.0;
      else
        {
          std::vector<double> off(R.offdiag.begin(),
                                  R.offdiag.begin() + (R.diag.size() - 1));
          lambda_min = tridiag_eig(R.diag, off, 0);
          lambda_max = 1.2 * tridiag_eig(R.diag, off, int(R.diag.size()) - 1);
        }
      const double alpha = smoothing_range > 1. ?
                             lambda_max / smoothing_range :
                             std::min(0.9 * lambda_max, lambda_min);
      if (degree == 0)
        {
          const double actual_range = lambda_max / alpha;
          const double sigma = (1. - std::sqrt(1. / actual_range)) /
                               (1. + std::sqrt(1. / actual_range));
          const double eps = smoothing_range;
          degree           = 1 + unsigned(std::log(1. / eps + std::sqrt(1. / eps / eps - 1.)) /
                                std::log(1. / sigma));
        }
      delta       = (lambda_max - alpha) * 0.5;
      theta       = (lambda_max + alpha) * 0.5;
      initialized = true;
      x_old.resize(n);
      t1.resize(n);
      t2.resize(n);
    }

    // x_{k+1} = x_k + f1 (x_k - x_{k-1}) + f2 D^{-1} (b - A x_k)
    void
    update(const T *b, T *x, double f1, double f2, bool first)
    {
      const size_t n = A->m();
#pragma omp parallel for schedule(static)
      for (size_t i = 0; i < n; ++i)
        {
          const T t  = A->inv_diag[i] * (b[i] - t1[i]);
          const T xn = first ? T(1 + f1) * x[i] + T(f2) * t :
                               x[i] + T(f1) * (x[i] - x_old[i]) + T(f2) * t;
          x_old[i] = x[i];
          x[i]     = xn;
        }
    }

    // zero initial guess (PreconditionChebyshev::vmult)
    void
    vmult(T *x, const T *b)
    {
      if (!initialized)
        estimate();
      const size_t n = A->m();
#pragma omp parallel for schedule(static)
      for (size_t i = 0; i < n; ++i)
        {
          x[i]     = T(1. / theta) * A->inv_diag[i] * b[i];
          x_old[i] = T(0);
        }
      if (degree < 2)
        return;
      double rhok = delta / theta, sigma = theta / delta;
      for (unsigned k = 0; k + 1 < degree; ++k)
        {
          A->vmult(t1.data(), x);
          const double rhokp = 1. / (2. * sigma - rhok);
          const double f1 = rhokp * rhok, f2 = 2. * rhokp / delta;
          rhok = rhokp;
          update(b, x, f1, f2, k == 0);
        }
    }

    // nonzero initial guess (PreconditionChebyshev::step)
    void
    step(T *x, const T *b)
    {
      if (!initialized)
        estimate();
      A->vmult(t1.data(), x);
      update(b, x, 0., 1. / theta, true);
      if (degree < 2)
        return;
      double rhok = delta / theta, sigma = theta / delta;
      for (unsigned k = 0; k + 1 < degree; ++k)
        {
          A->vmult(t1.data(), x);
          const double rhokp = 1. / (2. * sigma - rhok);
          const double f1 = rhokp * rhok, f2 = 2. * rhokp / delta;
          rhok = rhokp;
          update(b, x, f1, f2, false);
        }
    }
  };

  // ---------------------------------------------------------------------
  // Multigrid V-cycle (deal.II Multigrid::level_v_step) + PreconditionMG
  // ---------------------------------------------------------------------
  template <typename T>
  struct Multigrid
  {
    std::vector<LevelOp<T> *>                        ops;
    std::vector<std::unique_ptr<LevelTransfer<T>>>   transfers; // [l]: l-1 -> l
    std::vector<Chebyshev<T>>                        smoothers;
    std::vector<std::vector<T>>                      sol, def, tmp;

    void
    setup(double range, int degree, int eig_its, int coarse_eig_its)
    {
      const size_t L = ops.size();
      smoothers.resize(L);
      sol.resize(L);
      def.resize(L);
      tmp.resize(L);
      for (size_t l = 0; l < L; ++l)
        {
          smoothers[l].A = ops[l];
          if (l == 0)
            {
              smoothers[l].smoothing_range   = 1e-3;
              smoothers[l].degree            = 0;
              smoothers[l].eig_cg_iterations = coarse_eig_its;
            }
          else
            {
              smoothers[l].smoothing_range   = range;
              smoothers[l].degree            = degree;
              smoothers[l].eig_cg_iterations = eig_its;
            }
          smoothers[l].initialized = false;
          sol[l].assign(ops[l]->m(), T(0));
          def[l].assign(ops[l]->m(), T(0));
          tmp[l].assign(ops[l]->m(), T(0));
        }
    }

    void
    level_v_step(size_t l)
    {
      if (l == 0)
        {
          smoothers[0].vmult(sol[0].data(), def[0].data());
          return;
        }
      const size_t n = ops[l]->m();
      smoothers[l].vmult(sol[l].data(), def[l].data());
      ops[l]->vmult(tmp[l].data(), sol[l].data());
#pragma omp parallel for schedule(static)
      for (size_t i = 0; i < n; ++i)
        tmp[l][i] = def[l][i] - tmp[l][i];
      std::fill(def[l - 1].begin(), def[l - 1].end(), T(0));
      transfers[l]->restrict_add(def[l - 1].data(), tmp[l].data());
      std::fill(sol[l - 1].begin(), sol[l - 1].end(), T(0));
      level_v_step(l - 1);
      transfers[l]->prolongate(tmp[l].data(), sol[l - 1].data());
#pragma omp parallel for schedule(static)
      for (size_t i = 0; i < n; ++i)
        sol[l][i] += tmp[l][i];
      smoothers[l].step(sol[l].data(), def[l].data());
    }

    // PreconditionMG::vmult: copy_to_mg, V-cycle, copy_from_mg
    template <typename TF>
    void
    vmult(TF *dst, const TF *src)
    {
      const size_t L = ops.size() - 1;
      const size_t n = ops[L]->m();
      for (size_t i = 0; i < n; ++i)
        def[L][i] = T(src[i]);
      for (auto &s : sol)
        std::fill(s.begin(), s.end(), T(0));
      level_v_step(L);
      for (size_t i = 0; i < n; ++i)
        dst[i] = TF(sol[L][i]);
    }
  };

  // Point evaluation of a field at a point in the box (undeformed frame)
  inline std::vector<double>
  point_value(const Box &box, const Basis1D &b, int nc, const double *u,
              const double *x)
  {
    int    cc[3]  = {0, 0, 0};
    double xi[3]  = {0, 0, 0};
    for (int d = 0; d < box.dim; ++d)
      {
        double t = (x[d] - box.lo[d]) / box.h[d];
        int    c = int(std::floor(t));
        c        = std::min(std::max(c, 0), box.C[d] - 1);
        cc[d]    = c;
        xi[d]    = t - c;
      }
    std::vector<double> res(nc, 0.0);
    const int           N = b.N;
    for (int c = 0; c < nc; ++c)
      {
        double s = 0;
        for (int k = 0; k < (box.dim == 3 ? N : 1); ++k)
          for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i)
              {
                double w = lagrange(b.nodes, i, xi[0]) * lagrange(b.nodes, j, xi[1]);
                if (box.dim == 3)
                  w *= lagrange(b.nodes, k, xi[2]);
                const size_t g = box.node(cc[0] * box.p + i, cc[1] * box.p + j,
                                          box.dim == 3 ? cc[2] * box.p + k : 0);
                s += w * u[size_t(c) * box.n_nodes + g];
              }
        res[c] = s;
      }
    return res;
  }
} // namespace orc
