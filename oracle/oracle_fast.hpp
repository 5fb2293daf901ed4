// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle_core.hpp).
//
// Throughput form of the neo-Hookean tangent and of the heat operator for
// the timed CPU baseline.  It restates how deal.II executes the reference's
// CPU path, rather than the plain loops of oracle_ops.hpp, so that the
// baseline is not slowed by the oracle's generality:
//   * cells are processed in batches of W lanes, one cell per lane, as
//     deal.II's VectorizedArray<double> does (FEEvaluation over a cell batch,
//     NeoHookOperator::local_apply_cell, mf_nh_operator.h:631-647); the lanes
//     use GCC's portable vector extension, no target intrinsics;
//   * polynomial degree and dimension are compile-time constants
//     (FEEvaluation<dim, degree, n_q_points_1d, ...>, include/base/
//     fe_integrator.h:14-15, precompiled degrees 1-6);
//   * evaluate/integrate use the collocation scheme for FE_Q on Gauss-Lobatto
//     points with n_q = p + 1: S-sweeps from the nodes to the Gauss points,
//     then derivative sweeps on the Gauss points, each 1D product in even-odd
//     form (deal.II's EvaluatorTensorProduct<evaluate_evenodd>);
//   * the quadrature-point operations are those of oracle_ops.hpp (NHQ) for
//     every caching variant of formulation 1: scalar_referential
//     (mf_nh_operator.h:848-943, with the second gradient evaluation of the
//     cached linearisation values, :865-867), tensor2 and tensor4 (deformed
//     frame, :945-994; tensor4 stored on symmetric index pairs like
//     SymmetricTensor<4,3>) and tensor4_ns (:996-1010);
//   * cells are coloured by parity (cells of one colour share no DoF), so
//     threads scatter without atomics; constrained DoFs read as zero and are
//     skipped on the scatter, and the constrained rows get dst += src;
//   * diagonals apply every local unit vector of a batch to the cell
//     operator (MatrixFreeTools::compute_diagonal), and make_*_level hands
//     vmult and diagonal to the oracle's solvers (LevelOp::fast), in FP64 or,
//     for the multigrid levels, FP32 lanes.
// Results equal the oracle's to round-off (tests/test_oracle_fast.py).
// oracle_fast.cpp instantiates this file once per lane count ORC_FAST_W and
// scalar type ORC_FAST_T.
#include "oracle_ops.hpp"

#include <array>
#include <chrono>
#include <memory>

#ifndef ORC_FAST_W
#define ORC_FAST_W 4
#endif
// scalar type of the lanes (double, or float for FP32 multigrid levels) and
// its namespace suffix
#ifndef ORC_FAST_T
#define ORC_FAST_T double
#define ORC_FAST_TS d
#endif
#define ORC_FAST_CAT2(a, b) a##b
#define ORC_FAST_CAT(a, b) ORC_FAST_CAT2(a, b)
#define ORC_FAST_CAT3(a, b, c) ORC_FAST_CAT(ORC_FAST_CAT(a, b), c)
#define ORC_FAST_NS ORC_FAST_CAT3(fast_w, ORC_FAST_W, ORC_FAST_TS)

namespace orc
{
  // one namespace per lane count and scalar type, so that several link together
  namespace ORC_FAST_NS
  {
    constexpr int W = ORC_FAST_W; // lanes per cell batch

    typedef ORC_FAST_T real;
    typedef real       vd __attribute__((vector_size(W * sizeof(real))));

    inline vd
    splat(real x)
    {
      vd r;
      for (int l = 0; l < W; ++l)
        r[l] = x;
      return r;
    }

    // 1D matrix (N x N, row-major, out[q] = sum_i M[q][i] in[i]) in even-odd
    // form; SIG = +1 for M[N-1-q][N-1-i] == M[q][i], -1 for == -M[q][i]
    template <int N, int SIG>
    struct EvenOdd
    {
      static constexpr int H  = N / 2;
      static constexpr int HR = (N + 1) / 2;
      real                 e[HR][HR]; // even part; column H holds the middle column (N odd)
      real                 o[HR][H > 0 ? H : 1];

      void
      set(const double *M)
      {
        for (int q = 0; q < HR; ++q)
          {
            for (int i = 0; i < H; ++i)
              {
                e[q][i] = 0.5 * (M[q * N + i] + M[q * N + N - 1 - i]);
                o[q][i] = 0.5 * (M[q * N + i] - M[q * N + N - 1 - i]);
              }
            if (N % 2 == 1)
              e[q][H] = M[q * N + H];
          }
      }

      // out[q * STRIDE] (+)= sum_i M[q][i] in[i * STRIDE]
      template <int STRIDE, bool ADD>
      inline void
      apply(const vd *in, vd *out) const
      {
        vd ev[HR], od[H > 0 ? H : 1];
        for (int i = 0; i < H; ++i)
          {
            ev[i] = in[i * STRIDE] + in[(N - 1 - i) * STRIDE];
            od[i] = in[i * STRIDE] - in[(N - 1 - i) * STRIDE];
          }
        if (N % 2 == 1)
          ev[H] = in[H * STRIDE];
        for (int q = 0; q < HR; ++q)
          {
            vd se = splat(0.0), so = splat(0.0);
            for (int i = 0; i < HR; ++i)
              se += e[q][i] * ev[i];
            for (int i = 0; i < H; ++i)
              so += o[q][i] * od[i];
            if (N % 2 == 1 && q == H)
              {
                // middle row: the exact row is even + odd parts
                if (ADD)
                  out[q * STRIDE] += se + so;
                else
                  out[q * STRIDE] = se + so;
                continue;
              }
            const vd lo = se + so;
            const vd hi = SIG > 0 ? se - so : so - se;
            if (ADD)
              {
                out[q * STRIDE] += lo;
                out[(N - 1 - q) * STRIDE] += hi;
              }
            else
              {
                out[q * STRIDE]           = lo;
                out[(N - 1 - q) * STRIDE] = hi;
              }
          }
      }
    };

    // apply a 1D matrix along direction D of an N^3 array (x fastest)
    template <int N, int D, bool ADD, int SIG>
    inline void
    sweep(const EvenOdd<N, SIG> &m, const vd *in, vd *out)
    {
      constexpr int stride = D == 0 ? 1 : (D == 1 ? N : N * N);
      for (int a = 0; a < N; ++a)
        for (int b = 0; b < N; ++b)
          {
            int base;
            if (D == 0)
              base = (a * N + b) * N;
            else if (D == 1)
              base = a * N * N + b;
            else
              base = a * N + b;
            m.template apply<stride, ADD>(in + base, out + base);
          }
    }

    template <int N>
    struct Shape
    {
      EvenOdd<N, 1>  S, St;           // nodes -> Gauss points, and transpose
      EvenOdd<N, -1> D[3], Dt[3];     // collocation derivative / h_d, and transpose
      real           jxw[N * N * N];  // quadrature weight times cell volume

      Shape(const Basis1D &b, const Box &box)
      {
        std::vector<double> M(N * N), Mt(N * N);
        for (int q = 0; q < N; ++q)
          for (int i = 0; i < N; ++i)
            {
              M[q * N + i]  = b.S[q * N + i];
              Mt[i * N + q] = b.S[q * N + i];
            }
        S.set(M.data());
        St.set(Mt.data());
        // derivative of the Lagrange basis on the Gauss points, at the Gauss
        // points (deal.II's collocation gradient)
        for (int d = 0; d < 3; ++d)
          {
            for (int q = 0; q < N; ++q)
              for (int r = 0; r < N; ++r)
                {
                  const double v = lagrange_deriv(b.xq, r, b.xq[q]) / box.h[d];
                  M[q * N + r]   = v;
                  Mt[r * N + q]  = v;
                }
            D[d].set(M.data());
            Dt[d].set(Mt.data());
          }
        const double vol = box.h[0] * box.h[1] * box.h[2];
        for (int k = 0; k < N; ++k)
          for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i)
              jxw[(k * N + j) * N + i] = b.wq[i] * b.wq[j] * b.wq[k] * vol;
      }

      // values and gradients at the Gauss points of one scalar field
      inline void
      evaluate(const vd *u, vd *val, vd *gx, vd *gy, vd *gz, vd *t0, vd *t1) const
      {
        sweep<N, 0, false>(S, u, t0);
        sweep<N, 1, false>(S, t0, t1);
        sweep<N, 2, false>(S, t1, val);
        sweep<N, 0, false>(D[0], val, gx);
        sweep<N, 1, false>(D[1], val, gy);
        sweep<N, 2, false>(D[2], val, gz);
      }

      // gradients only (evaluate(gradients)); the collocation scheme passes
      // through the values, which land in the scratch array val
      inline void
      gradients(const vd *u, vd *gx, vd *gy, vd *gz, vd *t0, vd *t1, vd *val) const
      {
        evaluate(u, val, gx, gy, gz, t0, t1);
      }

      // nodal test-function integrals of values val and fluxes (fx, fy, fz);
      // val is overwritten
      inline void
      integrate(vd *val, const vd *fx, const vd *fy, const vd *fz, vd *out, vd *t0) const
      {
        sweep<N, 0, true>(Dt[0], fx, val);
        sweep<N, 1, true>(Dt[1], fy, val);
        sweep<N, 2, true>(Dt[2], fz, val);
        sweep<N, 2, false>(St, val, t0);
        sweep<N, 1, false>(St, t0, val);
        sweep<N, 0, false>(St, val, out);
      }
    };

    inline void
    inv3(const vd *F, vd *Fi, vd &J)
    {
      Fi[0] = F[4] * F[8] - F[5] * F[7];
      Fi[1] = F[2] * F[7] - F[1] * F[8];
      Fi[2] = F[1] * F[5] - F[2] * F[4];
      Fi[3] = F[5] * F[6] - F[3] * F[8];
      Fi[4] = F[0] * F[8] - F[2] * F[6];
      Fi[5] = F[2] * F[3] - F[0] * F[5];
      Fi[6] = F[3] * F[7] - F[4] * F[6];
      Fi[7] = F[1] * F[6] - F[0] * F[7];
      Fi[8] = F[0] * F[4] - F[1] * F[3];
      J          = F[0] * Fi[0] + F[1] * Fi[3] + F[2] * Fi[6];
      const vd r = splat(real(1)) / J;
      for (int i = 0; i < 9; ++i)
        Fi[i] *= r;
    }

    // cell batches of one level: cells of one parity colour in groups of W
    // (a partly filled last group repeats its last cell in the spare lanes,
    // which are never scattered), lane-interleaved gather and scatter of NC
    // component-blocked fields
    template <int N, int NC>
    struct CellBatches
    {
      static constexpr int                Nd = N * N * N;
      const Box                          &box;
      std::vector<std::array<size_t, W>> cells;
      std::vector<int>                   lanes;      // filled lanes per batch
      std::vector<unsigned char>         touches;    // batch has a constrained node
      std::vector<size_t>                colour_end; // batches of colour c end here
      std::vector<size_t>                constrained_rows; // c * n_nodes + node

      explicit CellBatches(const Box &bx)
        : box(bx)
      {
        for (int colour = 0; colour < 8; ++colour)
          {
            const std::vector<size_t> cs = colour_cells(box, colour);
            for (size_t i = 0; i < cs.size(); i += W)
              {
                std::array<size_t, W> bt;
                const int             n = int(std::min<size_t>(W, cs.size() - i));
                bool                  t = false;
                for (int l = 0; l < W; ++l)
                  {
                    bt[l] = cs[i + std::min(l, n - 1)];
                    t     = t || cell_touches(bt[l]);
                  }
                cells.push_back(bt);
                lanes.push_back(n);
                touches.push_back(t);
              }
            colour_end.push_back(cells.size());
          }
        for (int c = 0; c < NC; ++c)
          for (size_t g = 0; g < box.n_nodes; ++g)
            if (box.constrained(g, c))
              constrained_rows.push_back(size_t(c) * box.n_nodes + g);
      }

      bool
      cell_touches(size_t e) const
      {
        int cc[3];
        box.cell_coords(e, cc);
        for (int d = 0; d < 3; ++d)
          if ((cc[d] == 0 && box.face_mask[2 * d]) || (cc[d] == box.C[d] - 1 && box.face_mask[2 * d + 1]))
            return true;
        return false;
      }

      size_t
      first_node(size_t e) const
      {
        int cc[3];
        box.cell_coords(e, cc);
        return box.node(cc[0] * box.p, cc[1] * box.p, cc[2] * box.p);
      }

      // read the NC components of the batch's cells into lane-interleaved form
      void
      gather(size_t bt, const real *src, vd *u, bool constrained) const
      {
        const size_t plane = size_t(box.Nn[0]) * box.Nn[1];
        for (int l = 0; l < W; ++l)
          {
            const size_t e  = cells[bt][l];
            const size_t g0 = first_node(e);
            for (int c = 0; c < NC; ++c)
              {
                const real   *s = src + size_t(c) * box.n_nodes + g0;
                vd           *o = u + c * Nd;
                for (int k = 0; k < N; ++k)
                  for (int j = 0; j < N; ++j)
                    for (int i = 0; i < N; ++i)
                      o[(k * N + j) * N + i][l] = s[k * plane + size_t(j) * box.Nn[0] + i];
              }
            if (constrained && touches[bt])
              {
                size_t nodes[Nd];
                box.cell_nodes(e, nodes);
                for (int c = 0; c < NC; ++c)
                  for (int n = 0; n < Nd; ++n)
                    if (box.constrained(nodes[n], c))
                      u[c * Nd + n][l] = 0.0;
              }
          }
      }

      void
      scatter(size_t bt, const vd *out, real *dst) const
      {
        const size_t plane = size_t(box.Nn[0]) * box.Nn[1];
        for (int l = 0; l < lanes[bt]; ++l)
          {
            const size_t e  = cells[bt][l];
            const size_t g0 = first_node(e);
            if (touches[bt])
              {
                size_t nodes[Nd];
                box.cell_nodes(e, nodes);
                for (int c = 0; c < NC; ++c)
                  for (int n = 0; n < Nd; ++n)
                    if (!box.constrained(nodes[n], c))
                      dst[size_t(c) * box.n_nodes + nodes[n]] += out[c * Nd + n][l];
                continue;
              }
            for (int c = 0; c < NC; ++c)
              {
                real     *d = dst + size_t(c) * box.n_nodes + g0;
                const vd *o = out + c * Nd;
                for (int k = 0; k < N; ++k)
                  for (int j = 0; j < N; ++j)
                    for (int i = 0; i < N; ++i)
                      d[k * plane + size_t(j) * box.Nn[0] + i] += o[(k * N + j) * N + i][l];
              }
          }
      }

      // dst = A src with A given cell batch by cell batch: dst zeroed, the
      // colours in turn (the loop's closing barrier orders them), then the
      // identity on the constrained rows (skipped when src is null).
      // apply(bt, scratch) handles a batch.
      template <typename Apply>
      void
      run(real *dst, const real *src, size_t scratch, const Apply &apply) const
      {
        const size_t n = size_t(NC) * box.n_nodes;
#pragma omp parallel
        {
          std::vector<vd> w(scratch);
#pragma omp for schedule(static)
          for (long i = 0; i < long(n); ++i)
            dst[i] = 0.0;
          size_t b0 = 0;
          for (size_t colour = 0; colour < colour_end.size(); ++colour)
            {
              const size_t b1 = colour_end[colour];
#pragma omp for schedule(static)
              for (long bl = long(b0); bl < long(b1); ++bl)
                apply(size_t(bl), w.data());
              b0 = b1;
            }
          if (src)
            {
#pragma omp for schedule(static)
              for (long i = 0; i < long(constrained_rows.size()); ++i)
                dst[constrained_rows[i]] += src[constrained_rows[i]];
            }
        }
      }
    };

    // the tangent on one level, cached for one linearisation point
    template <int N>
    struct NHFast
    {
      static constexpr int Nd = N * N * N;
      const Box           &box;
      CellBatches<N, 3>    cb;
      Shape<N>             sh;
      Caching              caching;
      double               mu, lambda, ra;
      std::vector<vd>      A; // tensor4_ns: [batch][q][81]
      // tensor2 / tensor4 (deformed frame): per qp F^{-1} (9), det F, tau / J
      // (9), then tensor2: 2c / J, 1 / J; tensor4: 1 / J and the symmetric
      // 4th-order tensor as a 6 x 6 matrix on (00, 11, 22, 01, 02, 12)
      std::vector<vd> E;
      int             es = 0; // entries of E per qp
      std::vector<vd> cscal;  // scalar_referential: [batch][q]
      std::vector<vd> ucell;  // scalar_referential: [batch][c][Nd]

      NHFast(const Box &bx, const Basis1D &b, const Material &mat, Caching cach)
        : box(bx)
        , cb(bx)
        , sh(b, bx)
        , caching(cach)
        , mu(mat.mu)
        , lambda(mat.lambda())
        , ra(mat.rho_alpha())
      {
        if (mat.formulation != 1)
          throw std::runtime_error("fast form: formulation 1 only");
        es = cach == tensor2 ? 21 : (cach == tensor4 ? 56 : 0);
      }

      // NeoHookOperator::cache (mf_nh_operator.h:394-523), from the
      // linearisation u read without constraints
      bool
      cache(const real *u)
      {
        const size_t nb = cb.cells.size();
        if (caching == tensor4_ns)
          A.assign(nb * Nd * 81, splat(0.0));
        else if (es > 0)
          E.assign(nb * Nd * es, splat(0.0));
        else
          {
            cscal.assign(nb * Nd, splat(0.0));
            ucell.assign(nb * 3 * Nd, splat(0.0));
          }
        bool ok = true;
#pragma omp parallel reduction(&& : ok)
        {
          std::vector<vd> w(16 * Nd);
          vd             *uu = w.data(), *g = uu + 3 * Nd, *val = g + 9 * Nd, *t0 = val + Nd, *t1 = t0 + Nd;
#pragma omp for schedule(static)
          for (long bl = 0; bl < long(nb); ++bl)
            {
              const size_t bt = size_t(bl);
              cb.gather(bt, u, uu, false);
              for (int c = 0; c < 3; ++c)
                sh.gradients(uu + c * Nd, g + (3 * c) * Nd, g + (3 * c + 1) * Nd, g + (3 * c + 2) * Nd, t0, t1,
                             val);
              if (caching == scalar_referential)
                std::copy(uu, uu + 3 * Nd, ucell.begin() + bt * 3 * Nd);
              for (int q = 0; q < Nd; ++q)
                for (int l = 0; l < W; ++l)
                  {
                    double H[9], F[9], Fi[9];
                    for (int c = 0; c < 3; ++c)
                      for (int d = 0; d < 3; ++d)
                        {
                          H[c * 3 + d] = g[(3 * c + d) * Nd + q][l];
                          F[c * 3 + d] = H[c * 3 + d] + (c == d ? 1.0 : 0.0);
                        }
                    const double Jm1 = jm1_from_grad(3, H);
                    const double J   = 1.0 + Jm1;
                    if (!(J > 0.0))
                      {
                        ok = false;
                        continue;
                      }
                    const double lnJ = std::log1p(Jm1);
                    if (caching == scalar_referential)
                      {
                        cscal[bt * Nd + q][l] = mu - 2.0 * lambda * lnJ;
                        continue;
                      }
                    invert(3, F, Fi);
                    if (es > 0)
                      {
                        const double c = mu - 2.0 * lambda * lnJ;
                        vd          *x = &E[(bt * Nd + q) * es];
                        for (int i = 0; i < 9; ++i)
                          x[i][l] = Fi[i];
                        x[9][l] = J;
                        for (int i = 0; i < 3; ++i)
                          for (int j = 0; j < 3; ++j)
                            {
                              // tau = mu (H + H^T + H H^T) + 2 lambda ln J I
                              const double hh = H[i * 3] * H[j * 3] + H[i * 3 + 1] * H[j * 3 + 1] +
                                                H[i * 3 + 2] * H[j * 3 + 2];
                              x[10 + i * 3 + j][l] =
                                (mu * (H[i * 3 + j] + H[j * 3 + i] + hh) + (i == j ? 2.0 * lambda * lnJ : 0.0)) / J;
                            }
                        if (caching == tensor2)
                          {
                            x[19][l] = c * 2.0 / J;
                            x[20][l] = 1.0 / J;
                            continue;
                          }
                        x[19][l] = 1.0 / J;
                        // (2c / J) S + (2 lambda / J) I x I on the symmetric
                        // pairs (mf_nh_operator.h:490-494)
                        static const int vi[6] = {0, 1, 2, 0, 0, 1}, vj[6] = {0, 1, 2, 1, 2, 2};
                        const double     a = c * 2.0 / J, bl = lambda * 2.0 / J;
                        for (int r = 0; r < 6; ++r)
                          for (int t = 0; t < 6; ++t)
                            {
                              const int i = vi[r], j = vj[r], k = vi[t], m = vj[t];
                              x[20 + r * 6 + t][l] =
                                a * 0.5 * (double(i == k && j == m) + double(i == m && j == k)) +
                                bl * double(i == j && k == m);
                            }
                        continue;
                      }
                    vd *a = &A[(bt * Nd + q) * 81];
                    for (int i = 0; i < 3; ++i)
                      for (int j = 0; j < 3; ++j)
                        for (int k = 0; k < 3; ++k)
                          for (int m = 0; m < 3; ++m)
                            a[((i * 3 + j) * 3 + k) * 3 + m][l] =
                              2.0 * lambda * Fi[j * 3 + i] * Fi[m * 3 + k] +
                              (mu - 2.0 * lambda * lnJ) * Fi[m * 3 + i] * Fi[j * 3 + k] +
                              mu * double(i == k && j == m);
                  }
            }
        }
        return ok;
      }

      // dst = A src (cell part + constrained identity), dst zeroed here
      void
      vmult(real *dst, const real *src) const
      {
        cb.run(dst, src, 32 * Nd, [&](size_t bt, vd *w) {
          vd *u = w, *val = u + 3 * Nd, *g = val + 3 * Nd, *gu = g + 9 * Nd, *t0 = gu + 9 * Nd, *t1 = t0 + Nd,
             *t2 = t1 + Nd, *out = t2 + Nd;
          apply_batch(bt, src, dst, u, val, g, gu, t0, t1, t2, out);
        });
      }

      void
      apply_batch(size_t bt, const real *src, real *dst, vd *u, vd *val, vd *g, vd *gu, vd *t0, vd *t1,
                  vd *t2, vd *out) const
      {
        cb.gather(bt, src, u, true);
        cell_op(bt, u, val, g, gu, t0, t1, t2, out);
        cb.scatter(bt, out, dst);
      }

      // diagonal of the cell part (MatrixFreeTools::compute_diagonal,
      // mf_nh_operator.h:1025-1060): every local unit vector of a batch
      // through the cell operator; the constrained rows stay zero
      void
      cell_diagonal(real *diag) const
      {
        cb.run(diag, nullptr, 36 * Nd, [&](size_t bt, vd *w) {
          vd *u = w, *val = u + 3 * Nd, *g = val + 3 * Nd, *gu = g + 9 * Nd, *t0 = gu + 9 * Nd, *t1 = t0 + Nd,
             *t2 = t1 + Nd, *out = t2 + Nd, *dg = out + 3 * Nd;
          for (int i = 0; i < 3 * Nd; ++i)
            u[i] = splat(real(0));
          for (int i = 0; i < 3 * Nd; ++i)
            {
              u[i] = splat(real(1));
              cell_op(bt, u, val, g, gu, t0, t1, t2, out);
              dg[i] = out[i];
              u[i] = splat(real(0));
            }
          cb.scatter(bt, dg, diag);
        });
      }

      // the cell operator of batch bt on its 3-component values u, into out
      void
      cell_op(size_t bt, const vd *u, vd *val, vd *g, vd *gu, vd *t0, vd *t1, vd *t2, vd *out) const
      {
        for (int c = 0; c < 3; ++c)
          sh.evaluate(u + c * Nd, val + c * Nd, g + (3 * c) * Nd, g + (3 * c + 1) * Nd, g + (3 * c + 2) * Nd, t0,
                      t1);
        if (caching == scalar_referential)
          {
            const vd *uc = &ucell[bt * 3 * Nd];
            for (int c = 0; c < 3; ++c)
              sh.gradients(uc + c * Nd, gu + (3 * c) * Nd, gu + (3 * c + 1) * Nd, gu + (3 * c + 2) * Nd, t0, t1,
                           t2);
          }
        const vd rav = splat(ra), lam2 = splat(2.0 * lambda), muv = splat(mu);
        for (int q = 0; q < Nd; ++q)
          {
            vd H[9], P[9], vs = rav;
            for (int i = 0; i < 9; ++i)
              H[i] = g[i * Nd + q];
            if (es > 0)
              {
                // deformed frame (mf_nh_operator.h:945-994), pulled back:
                // P = J Pc F^{-T}
                const vd *x  = &E[(bt * Nd + q) * es];
                const vd *Fi = x, *T2 = x + 10;
                const vd  J  = x[9];
                vd        gg[9], Pc[9];
                for (int i = 0; i < 3; ++i)
                  for (int j = 0; j < 3; ++j)
                    gg[i * 3 + j] = H[i * 3] * Fi[j] + H[i * 3 + 1] * Fi[3 + j] + H[i * 3 + 2] * Fi[6 + j];
                for (int i = 0; i < 3; ++i)
                  for (int j = 0; j < 3; ++j)
                    Pc[i * 3 + j] = gg[i * 3] * T2[j] + gg[i * 3 + 1] * T2[3 + j] + gg[i * 3 + 2] * T2[6 + j];
                if (caching == tensor2)
                  {
                    const vd sc = x[19], tmp = lam2 * x[20] * (gg[0] + gg[4] + gg[8]);
                    for (int i = 0; i < 3; ++i)
                      for (int j = 0; j < 3; ++j)
                        Pc[i * 3 + j] += sc * real(0.5) * (gg[i * 3 + j] + gg[j * 3 + i]);
                    Pc[0] += tmp;
                    Pc[4] += tmp;
                    Pc[8] += tmp;
                    vs = rav * x[20] * J;
                  }
                else
                  {
                    const vd *C = x + 20;
                    const vd  e[6] = {gg[0], gg[4], gg[8], gg[1] + gg[3], gg[2] + gg[6], gg[5] + gg[7]};
                    vd        r[6];
                    for (int a = 0; a < 6; ++a)
                      {
                        // off-diagonal pairs count twice: 2 * 0.5 (g_kl + g_lk)
                        vd t = C[a * 6] * e[0] + C[a * 6 + 1] * e[1] + C[a * 6 + 2] * e[2];
                        t += C[a * 6 + 3] * e[3] + C[a * 6 + 4] * e[4] + C[a * 6 + 5] * e[5];
                        r[a] = t;
                      }
                    Pc[0] += r[0];
                    Pc[4] += r[1];
                    Pc[8] += r[2];
                    Pc[1] += r[3];
                    Pc[3] += r[3];
                    Pc[2] += r[4];
                    Pc[6] += r[4];
                    Pc[5] += r[5];
                    Pc[7] += r[5];
                    vs = rav * x[19] * J;
                  }
                for (int i = 0; i < 3; ++i)
                  for (int j = 0; j < 3; ++j)
                    P[i * 3 + j] = J * (Pc[i * 3] * Fi[j * 3] + Pc[i * 3 + 1] * Fi[j * 3 + 1] + Pc[i * 3 + 2] * Fi[j * 3 + 2]);
              }
            else if (caching == tensor4_ns)
              {
                // P = A : H (mf_nh_operator.h:996-1010)
                const vd *a = &A[(bt * Nd + q) * 81];
                for (int i = 0; i < 9; ++i)
                  {
                    vd s = a[i * 9] * H[0];
                    for (int k = 1; k < 9; ++k)
                      s += a[i * 9 + k] * H[k];
                    P[i] = s;
                  }
              }
            else
              {
                // mf_nh_operator.h:848-943
                vd F[9], Fi[9], J, tau[9], gg[9], q9[9];
                for (int i = 0; i < 9; ++i)
                  F[i] = gu[i * Nd + q];
                F[0] += real(1);
                F[4] += real(1);
                F[8] += real(1);
                const vd c = cscal[bt * Nd + q];
                for (int i = 0; i < 3; ++i)
                  for (int j = 0; j < 3; ++j)
                    tau[i * 3 + j] = muv * (F[i * 3] * F[j * 3] + F[i * 3 + 1] * F[j * 3 + 1] + F[i * 3 + 2] * F[j * 3 + 2]);
                tau[0] -= c;
                tau[4] -= c;
                tau[8] -= c;
                inv3(F, Fi, J);
                for (int i = 0; i < 3; ++i)
                  for (int j = 0; j < 3; ++j)
                    gg[i * 3 + j] = H[i * 3] * Fi[j] + H[i * 3 + 1] * Fi[3 + j] + H[i * 3 + 2] * Fi[6 + j];
                const vd tr = lam2 * (gg[0] + gg[4] + gg[8]);
                for (int i = 0; i < 3; ++i)
                  for (int j = 0; j < 3; ++j)
                    q9[i * 3 + j] = c * (gg[i * 3 + j] + gg[j * 3 + i]) + gg[i * 3] * tau[j] +
                                    gg[i * 3 + 1] * tau[3 + j] + gg[i * 3 + 2] * tau[6 + j];
                q9[0] += tr;
                q9[4] += tr;
                q9[8] += tr;
                for (int i = 0; i < 3; ++i)
                  for (int j = 0; j < 3; ++j)
                    P[i * 3 + j] = q9[i * 3] * Fi[j * 3] + q9[i * 3 + 1] * Fi[j * 3 + 1] + q9[i * 3 + 2] * Fi[j * 3 + 2];
              }
            const vd jw = splat(sh.jxw[q]);
            for (int c = 0; c < 3; ++c)
              {
                val[c * Nd + q] *= vs * jw;
                for (int d = 0; d < 3; ++d)
                  g[(3 * c + d) * Nd + q] = P[c * 3 + d] * jw;
              }
          }
        for (int c = 0; c < 3; ++c)
          sh.integrate(val + c * Nd, g + (3 * c) * Nd, g + (3 * c + 1) * Nd, g + (3 * c + 2) * Nd, out + c * Nd, t0);
      }
    };

    // the heat operator M + k dt K (heat_transfer.h:236-250: submit_value(u),
    // submit_gradient(k dt grad u), k == 1)
    template <int N>
    struct HeatFast
    {
      static constexpr int Nd = N * N * N;
      CellBatches<N, 1>    cb;
      Shape<N>             sh;
      double               kdt;

      HeatFast(const Box &bx, const Basis1D &b, double k_dt)
        : cb(bx)
        , sh(b, bx)
        , kdt(k_dt)
      {}

      void
      vmult(real *dst, const real *src) const
      {
        cb.run(dst, src, 8 * Nd, [&](size_t bt, vd *w) {
          cb.gather(bt, src, w, true);
          cell_op(w, w + Nd, w + 7 * Nd);
          cb.scatter(bt, w + 7 * Nd, dst);
        });
      }

      // diagonal of the cell part (heat_transfer.h:205-230), constrained
      // rows zero
      void
      cell_diagonal(real *diag) const
      {
        cb.run(diag, nullptr, 10 * Nd, [&](size_t bt, vd *w) {
          vd *u = w, *out = w + 7 * Nd, *dg = out + Nd;
          for (int i = 0; i < Nd; ++i)
            u[i] = splat(real(0));
          for (int i = 0; i < Nd; ++i)
            {
              u[i] = splat(real(1));
              cell_op(u, w + Nd, out);
              dg[i] = out[i];
              u[i] = splat(real(0));
            }
          cb.scatter(bt, dg, diag);
        });
      }

      // cell operator on values u into out; s holds 6 Nd of scratch
      void
      cell_op(const vd *u, vd *s, vd *out) const
      {
        vd *val = s, *gx = val + Nd, *gy = gx + Nd, *gz = gy + Nd, *t0 = gz + Nd, *t1 = t0 + Nd;
        sh.evaluate(u, val, gx, gy, gz, t0, t1);
        for (int q = 0; q < Nd; ++q)
          {
            const vd jw = splat(sh.jxw[q]), kj = splat(kdt * sh.jxw[q]);
            val[q] *= jw;
            gx[q] *= kj;
            gy[q] *= kj;
            gz[q] *= kj;
          }
        sh.integrate(val, gx, gy, gz, out, t0);
      }
    };

    // level operators for a driver (oracle_solvers.hpp LevelOp::fast)
    template <int N>
    FastLevel<real>
    make_nh_level(const Box &box, const Basis1D &b, const Material &mat, Caching caching, const real *u, bool &ok)
    {
      auto            op = std::make_shared<NHFast<N>>(box, b, mat, caching);
      FastLevel<real> f;
      ok              = op->cache(u);
      f.vmult         = [op](real *d, const real *s) { op->vmult(d, s); };
      f.cell_diagonal = [op](real *d) { op->cell_diagonal(d); };
      return f;
    }

    template <int N>
    FastLevel<real>
    make_heat_level(const Box &box, const Basis1D &b, double k_dt)
    {
      auto            op = std::make_shared<HeatFast<N>>(box, b, k_dt);
      FastLevel<real> f;
      f.vmult         = [op](real *d, const real *s) { op->vmult(d, s); };
      f.cell_diagonal = [op](real *d) { op->cell_diagonal(d); };
      return f;
    }

    template <int N>
    int
    heat_vmult_timed(const Box &box, const Basis1D &b, double k_dt, const real *src, real *dst, int reps,
                     double *seconds)
    {
      HeatFast<N> op(box, b, k_dt);
      op.vmult(dst, src);
      const auto t0 = std::chrono::steady_clock::now();
      for (int r = 0; r < reps; ++r)
        op.vmult(dst, src);
      *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      return 0;
    }

    // build, cache, apply once (untimed: first touch), then time `reps`
    // applications; returns 0, -2 (unsupported), -3 (det F <= 0)
    template <int N>
    int
    nh_vmult_timed(const Box &box, const Basis1D &b, const Material &mat, Caching caching, const real *u,
                   const real *src, real *dst, int warmup, int reps, double *seconds)
    {
      NHFast<N> op(box, b, mat, caching);
      if (!op.cache(u))
        return -3;
      for (int w = 0; w < std::max(warmup, 1); ++w)
        op.vmult(dst, src);
      const auto t0 = std::chrono::steady_clock::now();
      for (int r = 0; r < reps; ++r)
        op.vmult(dst, src);
      *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      return 0;
    }
  } // namespace ORC_FAST_NS
} // namespace orc
