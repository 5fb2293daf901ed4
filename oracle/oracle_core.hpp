// CPU ORACLE — TEST INFRASTRUCTURE ONLY.
//
// This file is part of the CPU restatement of the reference's matrix-free
// hot path (davidscn/matrix-free-dealii-precice).  It is used only by the
// tests, by the smoke check and by the CPU-baseline leg of the benchmark, as
// the CPU computation the device results are compared with.  The product (the
// CUDA library) never includes, links or calls anything in this directory.
//
// What is restated here:
//   * deal.II FE_Q(p) on Gauss-Lobatto support points and QGauss(n_q)
//     (the reference uses FE_Q / FESystem(FE_Q, dim) with QGauss(quad_order):
//     include/solid_mechanics/mf_elasticity.h:369-377, heat_transfer.h:359-360);
//   * subdivided_hyper_rectangle + refine_global box meshes
//     (include/cases/elasticity/turek_hron.h:23-45);
//   * FEEvaluation read_dof_values / evaluate / integrate /
//     distribute_local_to_global (include/base/fe_integrator.h:9-22, call
//     sites include/solid_mechanics/mf_nh_operator.h:640-646,
//     include/heat_transfer/heat_transfer.h:185-188).  The oracle evaluates
//     gradients with the direct 9-sweep tensor product (S/G matrices), not the
//     collocation form, so it is an independent check of the device kernels.
//
// Parity at the operator level is unpinned by reference tests (they pin only
// end-to-end Newton/CG counts and watchpoint displacements); the oracle is
// pinned end to end against those goldens by tests/test_oracle_golden.py.
#pragma once

#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc
{
  // ---------------------------------------------------------------------
  // 1D polynomial machinery
  // ---------------------------------------------------------------------

  // Legendre polynomial P_n and its derivative at x in [-1,1].
  inline void
  legendre(int n, long double x, long double &p, long double &dp)
  {
    long double p0 = 1, p1 = x;
    if (n == 0)
      {
        p  = 1;
        dp = 0;
        return;
      }
    for (int k = 2; k <= n; ++k)
      {
        long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0             = p1;
        p1             = p2;
      }
    p  = p1;
    dp = n * (x * p1 - p0) / (x * x - 1);
  }

  // Gauss-Legendre points and weights on [0,1] (QGauss<1>(n)).
  inline void
  gauss_points(int n, std::vector<double> &x, std::vector<double> &w)
  {
    x.resize(n);
    w.resize(n);
    const long double pi = 3.14159265358979323846264338327950288L;
    for (int i = 0; i < n; ++i)
      {
        long double z = std::cos(pi * (i + 0.75L) / (n + 0.5L));
        long double p, dp;
        for (int it = 0; it < 100; ++it)
          {
            legendre(n, z, p, dp);
            long double dz = p / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-19L)
              break;
          }
        legendre(n, z, p, dp);
        // ascending order on [0,1]
        x[n - 1 - i] = double((1.0L + z) / 2.0L);
        w[n - 1 - i] = double(1.0L / ((1.0L - z * z) * dp * dp));
      }
  }

  // Gauss-Lobatto support points of FE_Q(p) on [0,1]: end points plus the
  // roots of P'_p.
  inline std::vector<double>
  gauss_lobatto_points(int p)
  {
    std::vector<double> x(p + 1);
    x[0] = 0.0;
    x[p] = 1.0;
    const long double pi = 3.14159265358979323846264338327950288L;
    for (int i = 1; i < p; ++i)
      {
        // roots of P'_p: Newton on P'_p using P''_p from the Legendre ODE
        long double z = -std::cos(pi * i / p);
        for (int it = 0; it < 100; ++it)
          {
            long double pn, dpn;
            legendre(p, z, pn, dpn);
            // (1-z^2) P'' = 2 z P' - p(p+1) P
            long double d2 = (2 * z * dpn - p * (p + 1) * pn) / (1 - z * z);
            long double dz = dpn / d2;
            z -= dz;
            if (std::fabs(dz) < 1e-19L)
              break;
          }
        x[i] = double((1.0L + z) / 2.0L);
      }
    return x;
  }

  // Lagrange polynomial i on the nodes, and its derivative, at x.
  inline double
  lagrange(const std::vector<double> &nodes, int i, double x)
  {
    long double v = 1;
    for (size_t j = 0; j < nodes.size(); ++j)
      if (int(j) != i)
        v *= (long double)(x - nodes[j]) / (nodes[i] - nodes[j]);
    return double(v);
  }

  inline double
  lagrange_deriv(const std::vector<double> &nodes, int i, double x)
  {
    long double s = 0;
    for (size_t k = 0; k < nodes.size(); ++k)
      {
        if (int(k) == i)
          continue;
        long double t = 1.0L / (nodes[i] - nodes[k]);
        for (size_t j = 0; j < nodes.size(); ++j)
          if (int(j) != i && j != k)
            t *= (long double)(x - nodes[j]) / (nodes[i] - nodes[j]);
        s += t;
      }
    return double(s);
  }

  // Shape values/derivatives of FE_Q(p) at QGauss(nq) on [0,1].
  struct Basis1D
  {
    int                 p = 1, N = 2, Q = 2;
    std::vector<double> nodes, xq, wq;
    std::vector<double> S, G; // [q][i], Q x N
    // point evaluations at 0 and 1 (for faces)
    std::vector<double> S0, G0, S1, G1; // [i]

    Basis1D() = default;
    Basis1D(int degree, int nq)
      : p(degree)
      , N(degree + 1)
      , Q(nq)
    {
      nodes = gauss_lobatto_points(p);
      gauss_points(Q, xq, wq);
      S.resize(Q * N);
      G.resize(Q * N);
      for (int q = 0; q < Q; ++q)
        for (int i = 0; i < N; ++i)
          {
            S[q * N + i] = lagrange(nodes, i, xq[q]);
            G[q * N + i] = lagrange_deriv(nodes, i, xq[q]);
          }
      S0.resize(N);
      G0.resize(N);
      S1.resize(N);
      G1.resize(N);
      for (int i = 0; i < N; ++i)
        {
          S0[i] = lagrange(nodes, i, 0.0);
          G0[i] = lagrange_deriv(nodes, i, 0.0);
          S1[i] = lagrange(nodes, i, 1.0);
          G1[i] = lagrange_deriv(nodes, i, 1.0);
        }
    }
  };

  // ---------------------------------------------------------------------
  // Structured box mesh on one multigrid level.
  //
  // Nodes are numbered lexicographically (x fastest) on the global Q_p node
  // grid; a vector field with nc components is stored component-blocked:
  // index = c * n_nodes + node.  Box faces are numbered (x-,x+,y-,y+,z-,z+),
  // matching deal.II's colorize numbering of subdivided_hyper_rectangle.
  // ---------------------------------------------------------------------
  struct Box
  {
    int      dim = 3;
    int      p   = 1;
    int      C[3]{1, 1, 1};  // cells per direction
    int      Nn[3]{2, 2, 2}; // nodes per direction
    double   lo[3]{0, 0, 0};
    double   h[3]{1, 1, 1};
    unsigned face_mask[6]{0, 0, 0, 0, 0, 0}; // Dirichlet component bitmask per face
    size_t   n_nodes = 0;
    size_t   n_cells = 0;

    Box() = default;
    Box(int dim_, int p_, const int *rep, const double *lo_, const double *hi_,
        int level, const unsigned *masks)
      : dim(dim_)
      , p(p_)
    {
      n_nodes = 1;
      n_cells = 1;
      for (int d = 0; d < 3; ++d)
        {
          if (d < dim)
            {
              C[d]  = rep[d] << level;
              Nn[d] = C[d] * p + 1;
              lo[d] = lo_[d];
              h[d]  = (hi_[d] - lo_[d]) / C[d];
            }
          else
            {
              C[d]  = 1;
              Nn[d] = 1;
              lo[d] = 0;
              h[d]  = 1;
            }
          n_nodes *= Nn[d];
          n_cells *= C[d];
        }
      for (int f = 0; f < 6; ++f)
        face_mask[f] = (f < 2 * dim) ? masks[f] : 0u;
    }

    size_t
    node(int ix, int iy, int iz) const
    {
      return size_t(ix) + size_t(Nn[0]) * (size_t(iy) + size_t(Nn[1]) * iz);
    }

    void
    node_coords(size_t g, int *ii) const
    {
      ii[0] = int(g % Nn[0]);
      g /= Nn[0];
      ii[1] = int(g % Nn[1]);
      ii[2] = int(g / Nn[1]);
    }

    // component mask of the Dirichlet constraints acting on a node
    unsigned
    node_mask(const int *ii) const
    {
      unsigned m = 0;
      for (int d = 0; d < dim; ++d)
        {
          if (ii[d] == 0)
            m |= face_mask[2 * d];
          if (ii[d] == Nn[d] - 1)
            m |= face_mask[2 * d + 1];
        }
      return m;
    }

    bool
    constrained(size_t node_index, int comp) const
    {
      int ii[3];
      node_coords(node_index, ii);
      return (node_mask(ii) >> comp) & 1u;
    }

    void
    cell_coords(size_t e, int *cc) const
    {
      cc[0] = int(e % C[0]);
      e /= C[0];
      cc[1] = int(e % C[1]);
      cc[2] = int(e / C[1]);
    }

    // global node indices of the (p+1)^dim local nodes, lexicographic
    void
    cell_nodes(size_t e, size_t *out) const
    {
      int cc[3];
      cell_coords(e, cc);
      const int N  = p + 1;
      const int Nz = dim == 3 ? N : 1;
      int       l  = 0;
      for (int k = 0; k < Nz; ++k)
        for (int j = 0; j < N; ++j)
          for (int i = 0; i < N; ++i)
            out[l++] = node(cc[0] * p + i, cc[1] * p + j,
                            dim == 3 ? cc[2] * p + k : 0);
    }

    double
    cell_volume() const
    {
      double v = 1;
      for (int d = 0; d < dim; ++d)
        v *= h[d];
      return v;
    }
  };

  inline int
  ipow(int b, int e)
  {
    int r = 1;
    for (int i = 0; i < e; ++i)
      r *= b;
    return r;
  }

  // ---------------------------------------------------------------------
  // Tensor-product sweeps.  Arrays are lexicographic with x fastest.
  // apply_dir: along direction `dir`, out_r = sum_k M[r][k] in_k where M is
  // given as the Q x N matrix; forward maps N -> Q, transposed maps Q -> N.
  // ---------------------------------------------------------------------
  template <typename T>
  void
  apply_dir(int dim, const int *ext_in, int dir, const double *M, int Q, int N,
            bool transposed, const T *in, T *out, bool add)
  {
    const int K = transposed ? Q : N; // input extent along dir
    const int R = transposed ? N : Q; // output extent along dir
    (void)K;
    int stride = 1;
    for (int d = 0; d < dir; ++d)
      stride *= ext_in[d];
    int outer = 1;
    for (int d = dir + 1; d < dim; ++d)
      outer *= ext_in[d];
    const int Kin = ext_in[dir];
    for (int o = 0; o < outer; ++o)
      for (int s = 0; s < stride; ++s)
        {
          const T *ip = in + size_t(o) * Kin * stride + s;
          T       *op = out + size_t(o) * R * stride + s;
          for (int r = 0; r < R; ++r)
            {
              T acc = T(0);
              for (int k = 0; k < Kin; ++k)
                {
                  const double m = transposed ? M[k * N + r] : M[r * N + k];
                  acc += T(m) * ip[size_t(k) * stride];
                }
              if (add)
                op[size_t(r) * stride] += acc;
              else
                op[size_t(r) * stride] = acc;
            }
        }
  }

  // Per-direction 1D matrices: values matrix, derivative matrix, number of
  // points (cells use QGauss in every direction, faces use a single point in
  // the normal direction).
  struct DirMats
  {
    const double *S[3];
    const double *G[3];
    int           Q[3];
  };

  inline DirMats
  cell_mats(const Basis1D &b)
  {
    DirMats m;
    for (int d = 0; d < 3; ++d)
      {
        m.S[d] = b.S.data();
        m.G[d] = b.G.data();
        m.Q[d] = b.Q;
      }
    return m;
  }

  // face with normal direction `nd` on side `side` (0: lower, 1: upper)
  inline DirMats
  face_mats(const Basis1D &b, int nd, int side)
  {
    DirMats m = cell_mats(b);
    m.S[nd]   = side == 0 ? b.S0.data() : b.S1.data();
    m.G[nd]   = side == 0 ? b.G0.data() : b.G1.data();
    m.Q[nd]   = 1;
    return m;
  }

  // Evaluate values and reference gradients of one scalar field:
  //   u[N^dim] -> val[Qp], grad[d][Qp], Qp = prod Q[d].
  // Work arrays must hold max(N,Q)^dim entries each.
  template <typename T>
  void
  evaluate_scalar(int dim, int N, const DirMats &m, const T *u, T *val, T *grad,
                  T *w0, T *w1, T *w2, T *w3)
  {
    const size_t Qp = size_t(m.Q[0]) * m.Q[1] * (dim == 3 ? m.Q[2] : 1);
    if (dim == 2)
      {
        int e0[2] = {N, N};
        apply_dir(2, e0, 0, m.S[0], m.Q[0], N, false, u, w0, false); // S_x u
        apply_dir(2, e0, 0, m.G[0], m.Q[0], N, false, u, w1, false); // G_x u
        int e1[2] = {m.Q[0], N};
        if (val)
          apply_dir(2, e1, 1, m.S[1], m.Q[1], N, false, w0, val, false);
        if (grad)
          {
            apply_dir(2, e1, 1, m.S[1], m.Q[1], N, false, w1, grad, false);
            apply_dir(2, e1, 1, m.G[1], m.Q[1], N, false, w0, grad + Qp, false);
          }
        return;
      }
    int e0[3] = {N, N, N};
    apply_dir(3, e0, 0, m.S[0], m.Q[0], N, false, u, w0, false); // a = S_x u
    apply_dir(3, e0, 0, m.G[0], m.Q[0], N, false, u, w1, false); // b = G_x u
    int e1[3] = {m.Q[0], N, N};
    apply_dir(3, e1, 1, m.S[1], m.Q[1], N, false, w0, w2, false); // aa
    int e2[3] = {m.Q[0], m.Q[1], N};
    if (val)
      apply_dir(3, e2, 2, m.S[2], m.Q[2], N, false, w2, val, false);
    if (grad)
      {
        apply_dir(3, e2, 2, m.G[2], m.Q[2], N, false, w2, grad + 2 * Qp, false); // dz
        apply_dir(3, e1, 1, m.G[1], m.Q[1], N, false, w0, w3, false); // ab
        apply_dir(3, e2, 2, m.S[2], m.Q[2], N, false, w3, grad + Qp, false); // dy
        apply_dir(3, e1, 1, m.S[1], m.Q[1], N, false, w1, w3, false); // ba
        apply_dir(3, e2, 2, m.S[2], m.Q[2], N, false, w3, grad, false); // dx
      }
  }

  // Transposed: out[N^dim] = S^T val + sum_d (grad-matrix)^T grad[d].
  template <typename T>
  void
  integrate_scalar(int dim, int N, const DirMats &m, const T *val, const T *grad,
                   T *out, T *w0, T *w1, T *w2, T *w3)
  {
    const size_t Qp = size_t(m.Q[0]) * m.Q[1] * (dim == 3 ? m.Q[2] : 1);
    if (dim == 2)
      {
        int e1[2] = {m.Q[0], m.Q[1]};
        // a = S_y^T val + G_y^T gy ; b = S_y^T gx
        bool have_a = false;
        if (val)
          {
            apply_dir(2, e1, 1, m.S[1], m.Q[1], N, true, val, w0, false);
            have_a = true;
          }
        if (grad)
          {
            apply_dir(2, e1, 1, m.G[1], m.Q[1], N, true, grad + Qp, w0, have_a);
            have_a = true;
            apply_dir(2, e1, 1, m.S[1], m.Q[1], N, true, grad, w1, false);
          }
        int e0[2] = {m.Q[0], N};
        apply_dir(2, e0, 0, m.S[0], m.Q[0], N, true, w0, out, false);
        if (grad)
          apply_dir(2, e0, 0, m.G[0], m.Q[0], N, true, w1, out, true);
        return;
      }
    int  e2[3] = {m.Q[0], m.Q[1], m.Q[2]};
    bool have  = false;
    // aa = S_z^T val + G_z^T gz
    if (val)
      {
        apply_dir(3, e2, 2, m.S[2], m.Q[2], N, true, val, w2, false);
        have = true;
      }
    if (grad)
      apply_dir(3, e2, 2, m.G[2], m.Q[2], N, true, grad + 2 * Qp, w2, have);
    int e1[3] = {m.Q[0], m.Q[1], N};
    // a = S_y^T aa (+ G_y^T ab)
    apply_dir(3, e1, 1, m.S[1], m.Q[1], N, true, w2, w0, false);
    if (grad)
      {
        apply_dir(3, e2, 2, m.S[2], m.Q[2], N, true, grad + Qp, w3, false); // ab
        apply_dir(3, e1, 1, m.G[1], m.Q[1], N, true, w3, w0, true);
        apply_dir(3, e2, 2, m.S[2], m.Q[2], N, true, grad, w3, false); // ba
        apply_dir(3, e1, 1, m.S[1], m.Q[1], N, true, w3, w1, false);   // b
      }
    int e0[3] = {m.Q[0], N, N};
    apply_dir(3, e0, 0, m.S[0], m.Q[0], N, true, w0, out, false);
    if (grad)
      apply_dir(3, e0, 0, m.G[0], m.Q[0], N, true, w1, out, true);
  }

  // quadrature weight product of cell qp q (lexicographic)
  inline double
  qweight(const Basis1D &b, int dim, int q)
  {
    double w = 1;
    for (int d = 0; d < dim; ++d)
      {
        w *= b.wq[q % b.Q];
        q /= b.Q;
      }
    return w;
  }

  // ---------------------------------------------------------------------
  // Generic matrix-free cell loop (the restatement of
  // MatrixFree::cell_loop + FEEvaluation gather/evaluate/integrate/scatter).
  //
  // QOp::cell(e, nc, Qp, val[c][q], grad[c][d][q]) receives values and REAL
  // gradients at the quadrature points and overwrites them in place with the
  // submitted values and gradients (before JxW); the loop multiplies by JxW,
  // maps the gradients back to reference derivatives and integrates.
  // Constrained DoFs are zeroed on read and skipped on write, like
  // read_dof_values / distribute_local_to_global with homogeneous
  // constraints.  Parallel over cells with a 2^dim parity colouring.
  // ---------------------------------------------------------------------
  template <typename T>
  struct CellScratch
  {
    std::vector<T>      u, val, grad, out, w0, w1, w2, w3;
    std::vector<size_t> nodes;
    void
    init(int dim, int nc, int N, int Q)
    {
      const int    M   = std::max(N, Q);
      const size_t big = size_t(ipow(M, dim));
      u.assign(size_t(nc) * big, T(0));
      val.assign(size_t(nc) * big, T(0));
      grad.assign(size_t(nc) * dim * big, T(0));
      out.assign(size_t(nc) * big, T(0));
      w0.assign(big, T(0));
      w1.assign(big, T(0));
      w2.assign(big, T(0));
      w3.assign(big, T(0));
      nodes.assign(size_t(ipow(N, dim)), 0);
    }
  };

  // Apply the cell pipeline evaluate -> QOp -> integrate to the local DoF
  // values in s.u (component-blocked [c][l]); result in s.out.
  template <typename T, typename QOp>
  void
  process_cell(const Box &box, const Basis1D &b, int nc, size_t e,
               CellScratch<T> &s, QOp &qop, bool want_val, bool want_grad)
  {
    const int     dim = box.dim;
    const int     N   = b.N;
    const int     Qp  = ipow(b.Q, dim);
    const int     Nd  = ipow(N, dim);
    const DirMats m   = cell_mats(b);
    const double  vol = box.cell_volume();
    for (int c = 0; c < nc; ++c)
      evaluate_scalar(dim, N, m, s.u.data() + size_t(c) * Nd,
                      want_val ? s.val.data() + size_t(c) * Qp : nullptr,
                      want_grad ? s.grad.data() + size_t(c) * dim * Qp :
                                  nullptr,
                      s.w0.data(), s.w1.data(), s.w2.data(), s.w3.data());
    if (want_grad)
      for (int c = 0; c < nc; ++c)
        for (int d = 0; d < dim; ++d)
          for (int q = 0; q < Qp; ++q)
            s.grad[(size_t(c) * dim + d) * Qp + q] /= T(box.h[d]);
    qop.cell(e, nc, Qp, s.val.data(), s.grad.data());
    for (int q = 0; q < Qp; ++q)
      {
        const T jxw = T(qweight(b, dim, q) * vol);
        for (int c = 0; c < nc; ++c)
          {
            if (qop.has_val)
              s.val[size_t(c) * Qp + q] *= jxw;
            if (qop.has_grad)
              for (int d = 0; d < dim; ++d)
                s.grad[(size_t(c) * dim + d) * Qp + q] *= jxw / T(box.h[d]);
          }
      }
    for (int c = 0; c < nc; ++c)
      integrate_scalar(dim, N, m,
                       qop.has_val ? s.val.data() + size_t(c) * Qp : nullptr,
                       qop.has_grad ? s.grad.data() + size_t(c) * dim * Qp :
                                      nullptr,
                       s.out.data() + size_t(c) * Nd, s.w0.data(), s.w1.data(),
                       s.w2.data(), s.w3.data());
  }

  // cells of one parity colour (cells of equal colour share no DoF)
  inline std::vector<size_t>
  colour_cells(const Box &box, int colour)
  {
    std::vector<size_t> cells;
    for (size_t e = 0; e < box.n_cells; ++e)
      {
        int cc[3];
        box.cell_coords(e, cc);
        int col = 0;
        for (int d = 0; d < box.dim; ++d)
          col |= (cc[d] & 1) << d;
        if (col == colour)
          cells.push_back(e);
      }
    return cells;
  }

  template <typename T, typename QOp>
  void
  cell_loop(const Box &box, const Basis1D &b, int nc, const T *src, T *dst,
            QOp &qop, bool use_constraints, bool want_val = true,
            bool want_grad = true)
  {
    const int dim = box.dim;
    const int Nd  = ipow(b.N, dim);
    for (int colour = 0; colour < (1 << dim); ++colour)
      {
        const std::vector<size_t> cells = colour_cells(box, colour);
#pragma omp parallel
        {
          CellScratch<T> s;
          s.init(dim, nc, b.N, b.Q);
#pragma omp for schedule(static)
          for (long ci = 0; ci < long(cells.size()); ++ci)
            {
              const size_t e = cells[ci];
              box.cell_nodes(e, s.nodes.data());
              for (int c = 0; c < nc; ++c)
                for (int l = 0; l < Nd; ++l)
                  {
                    const size_t g = s.nodes[l];
                    s.u[size_t(c) * Nd + l] =
                      (use_constraints && box.constrained(g, c)) ?
                        T(0) :
                        src[size_t(c) * box.n_nodes + g];
                  }
              process_cell(box, b, nc, e, s, qop, want_val, want_grad);
              for (int c = 0; c < nc; ++c)
                for (int l = 0; l < Nd; ++l)
                  {
                    const size_t g = s.nodes[l];
                    if (use_constraints && box.constrained(g, c))
                      continue;
                    dst[size_t(c) * box.n_nodes + g] +=
                      s.out[size_t(c) * Nd + l];
                  }
            }
        }
      }
  }

  // Diagonal of the constrained operator by local unit vectors, like
  // MatrixFreeTools::compute_diagonal (mf_nh_operator.h:1033-1036,
  // heat_transfer.h:215-218): for every cell and every unconstrained local
  // DoF, apply the cell operator to the unit vector and keep the diagonal
  // entry.  Constrained entries are left at zero here.
  template <typename T, typename QOp>
  void
  cell_diagonal(const Box &box, const Basis1D &b, int nc, T *diag, QOp &qop)
  {
    const int dim = box.dim;
    const int Nd  = ipow(b.N, dim);
    for (int colour = 0; colour < (1 << dim); ++colour)
      {
        const std::vector<size_t> cells = colour_cells(box, colour);
#pragma omp parallel
        {
          CellScratch<T> s;
          s.init(dim, nc, b.N, b.Q);
#pragma omp for schedule(static)
          for (long ci = 0; ci < long(cells.size()); ++ci)
            {
              const size_t e = cells[ci];
              box.cell_nodes(e, s.nodes.data());
              for (int c = 0; c < nc; ++c)
                for (int l = 0; l < Nd; ++l)
                  {
                    const size_t g = s.nodes[l];
                    if (box.constrained(g, c))
                      continue;
                    std::fill(s.u.begin(), s.u.end(), T(0));
                    s.u[size_t(c) * Nd + l] = T(1);
                    process_cell(box, b, nc, e, s, qop, true, true);
                    diag[size_t(c) * box.n_nodes + g] +=
                      s.out[size_t(c) * Nd + l];
                  }
            }
        }
      }
  }

  // dst[c] += src[c] on constrained rows (mf_nh_operator.h:622-624 and
  // MatrixFreeOperators::Base::vmult_add)
  template <typename T>
  void
  constrained_identity(const Box &box, int nc, const T *src, T *dst)
  {
    for (size_t g = 0; g < box.n_nodes; ++g)
      {
        int ii[3];
        box.node_coords(g, ii);
        const unsigned m = box.node_mask(ii);
        if (!m)
          continue;
        for (int c = 0; c < nc; ++c)
          if ((m >> c) & 1u)
            dst[size_t(c) * box.n_nodes + g] += src[size_t(c) * box.n_nodes + g];
      }
  }

  template <typename T>
  void
  set_constrained_zero(const Box &box, int nc, T *v)
  {
    for (size_t g = 0; g < box.n_nodes; ++g)
      {
        int ii[3];
        box.node_coords(g, ii);
        const unsigned m = box.node_mask(ii);
        if (!m)
          continue;
        for (int c = 0; c < nc; ++c)
          if ((m >> c) & 1u)
            v[size_t(c) * box.n_nodes + g] = T(0);
      }
  }

  // ---------------------------------------------------------------------
  // Small dense 2nd-order tensor helpers (row-major dim x dim)
  // ---------------------------------------------------------------------
  template <typename T>
  T
  det(int dim, const T *F)
  {
    if (dim == 2)
      return F[0] * F[3] - F[1] * F[2];
    return F[0] * (F[4] * F[8] - F[5] * F[7]) -
           F[1] * (F[3] * F[8] - F[5] * F[6]) +
           F[2] * (F[3] * F[7] - F[4] * F[6]);
  }

  // det(I + H) - 1 from the displacement gradient H (row-major dim x dim)
  // by the principal invariants of H: tr H + (sum of principal 2x2 minors)
  // + det H.  The reference takes std::log(determinant(F))
  // (mf_nh_operator.h:448,457; material.h:116-161); the two agree in exact
  // arithmetic, and this form keeps the relative accuracy of J - 1 and of
  // ln J = log1p(J - 1) at small strains, where det F - 1 cancels.
  template <typename T>
  T
  jm1_from_grad(int dim, const T *H)
  {
    if (dim == 2)
      return (H[0] + H[3]) + (H[0] * H[3] - H[1] * H[2]);
    const T i1 = H[0] + H[4] + H[8];
    const T i2 = (H[0] * H[4] - H[1] * H[3]) + (H[0] * H[8] - H[2] * H[6]) +
                 (H[4] * H[8] - H[5] * H[7]);
    return i1 + (i2 + det(3, H));
  }

  template <typename T>
  void
  invert(int dim, const T *F, T *Fi)
  {
    const T d = det(dim, F);
    if (dim == 2)
      {
        Fi[0] = F[3] / d;
        Fi[1] = -F[1] / d;
        Fi[2] = -F[2] / d;
        Fi[3] = F[0] / d;
        return;
      }
    Fi[0] = (F[4] * F[8] - F[5] * F[7]) / d;
    Fi[1] = (F[2] * F[7] - F[1] * F[8]) / d;
    Fi[2] = (F[1] * F[5] - F[2] * F[4]) / d;
    Fi[3] = (F[5] * F[6] - F[3] * F[8]) / d;
    Fi[4] = (F[0] * F[8] - F[2] * F[6]) / d;
    Fi[5] = (F[2] * F[3] - F[0] * F[5]) / d;
    Fi[6] = (F[3] * F[7] - F[4] * F[6]) / d;
    Fi[7] = (F[1] * F[6] - F[0] * F[7]) / d;
    Fi[8] = (F[0] * F[4] - F[1] * F[3]) / d;
  }

  // C = A * B
  template <typename T>
  void
  matmul(int dim, const T *A, const T *B, T *C)
  {
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j)
        {
          T s = T(0);
          for (int k = 0; k < dim; ++k)
            s += A[i * dim + k] * B[k * dim + j];
          C[i * dim + j] = s;
        }
  }
} // namespace orc
