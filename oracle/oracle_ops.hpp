// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle_core.hpp).
//
// Quadrature-point kernels of the two operators on the path:
//   * heat: LaplaceOperator::do_operation_on_cell
//     (include/heat_transfer/heat_transfer.h:234-250): submit_value(u),
//     submit_gradient(k * dt * grad u), k == 1 (heat_transfer.h:63-71);
//   * neo-Hookean tangent: NeoHookOperator::cache / do_operation_on_cell
//     (include/solid_mechanics/mf_nh_operator.h:394-523, 653-1019) for the
//     caching variants scalar_referential, tensor2, tensor4, tensor4_ns and
//     the formulation-0 (isochoric/volumetric) tensor2 path, with the material
//     constants of Material_Compressible_Neo_Hook_One_Field
//     (include/solid_mechanics/material.h:78-94) and its Kirchhoff stress
//     get_tau (material.h:116-161).
// The Eulerian variants (tensor2, tensor4, formulation 0) integrate on the
// current configuration given by MappingQEulerian of the displacement
// (mf_elasticity.h:739-742).  Because the Eulerian mapping of degree p
// reproduces x = X + u_h(X) exactly, its Jacobian at a quadrature point is
// F * J_ref; the oracle therefore integrates the current-frame flux P_cur as
// the referential flux det(F) P_cur F^{-T} (and values times det F), which is
// the same integral.
#pragma once

#include "oracle_core.hpp"

#include <functional>

namespace orc
{
  // a level operator in the throughput form (oracle_fast.hpp), as a driver
  // holds it: vmult = A with the constrained identity; cell_diagonal = the
  // cell part of diag(A), constrained rows left zero
  template <typename T>
  struct FastLevel
  {
    std::function<void(T *, const T *)> vmult;
    std::function<void(T *)>            cell_diagonal;
  };

  struct Material
  {
    double mu = 0, nu = 0, rho = 0, alpha_1 = 0;
    int    formulation = 1;
    // material.h:78-94
    double kappa() const { return (2.0 * mu * (1.0 + nu)) / (3.0 * (1.0 - 2.0 * nu)); }
    double c_1() const { return mu / 2.0; }
    double lambda() const { return (2.0 * mu * nu) / (1.0 - 2.0 * nu); }
    double rho_alpha() const { return rho * alpha_1; }
  };

  enum Caching
  {
    scalar_referential = 0,
    tensor2            = 1,
    tensor4            = 2,
    tensor4_ns         = 3
  };

  // ---------------------------------------------------------------------
  // heat
  // ---------------------------------------------------------------------
  template <typename T>
  struct HeatQ
  {
    static constexpr bool has_val  = true;
    static constexpr bool has_grad = true;
    int                   dim;
    double                k_dt; // coefficient * delta_t
    void
    cell(size_t, int nc, int Qp, T *val, T *grad)
    {
      (void)val;
      for (size_t i = 0; i < size_t(nc) * dim * Qp; ++i)
        grad[i] *= T(k_dt);
    }
  };

  // ---------------------------------------------------------------------
  // neo-Hookean
  // ---------------------------------------------------------------------

  // Kirchhoff stress tau (material.h:116-161) as a full dim x dim tensor,
  // from the displacement gradient H (F = I + H).  Formulation 1 is
  // evaluated as mu (H + H^T + H H^T) + 2 lambda ln J I, which equals the
  // reference's mu b - (mu - 2 lambda ln J) I, with ln J = log1p(J - 1) and
  // J - 1 from the invariants of H (jm1_from_grad).
  template <typename T>
  void
  get_tau(const Material &mat, int dim, const T *H, T *tau)
  {
    const T Jm1 = jm1_from_grad(dim, H);
    const T J   = T(1) + Jm1;
    const T lnJ = std::log1p(Jm1);
    if (mat.formulation == 1)
      {
        for (int i = 0; i < dim; ++i)
          for (int j = 0; j < dim; ++j)
            {
              T s = T(0);
              for (int k = 0; k < dim; ++k)
                s += H[i * dim + k] * H[j * dim + k];
              tau[i * dim + j] = T(mat.mu) * (H[i * dim + j] + H[j * dim + i] + s);
            }
        for (int d = 0; d < dim; ++d)
          tau[d * dim + d] += T(2.0 * mat.lambda()) * lnJ;
      }
    else
      {
        // tau = tau_vol + P : tau_bar, tau_bar = 2 c1 b_bar
        const T f = std::exp(lnJ * T(-1.0 / dim));
        T       F[9], tau_bar[9];
        for (int i = 0; i < dim; ++i)
          for (int j = 0; j < dim; ++j)
            F[i * dim + j] = H[i * dim + j] + (i == j ? T(1) : T(0));
        for (int i = 0; i < dim; ++i)
          for (int j = 0; j < dim; ++j)
            {
              T s = T(0);
              for (int k = 0; k < dim; ++k)
                s += F[i * dim + k] * F[j * dim + k];
              tau_bar[i * dim + j] = T(2.0 * mat.c_1()) * s * f * f;
            }
        T tr = T(0);
        for (int d = 0; d < dim; ++d)
          tr += tau_bar[d * dim + d];
        // (kappa / 2) (J - 1/J) J = (kappa / 2) (J - 1)(J + 1)
        const T tmp = T(mat.kappa() / 2.0) * Jm1 * (T(2) + Jm1);
        (void)J;
        for (int i = 0; i < dim * dim; ++i)
          tau[i] = tau_bar[i];
        for (int d = 0; d < dim; ++d)
          tau[d * dim + d] += tmp - tr / T(dim);
      }
  }

  // Per-quadrature-point state of the neo-Hookean tangent (the fields the
  // reference caches, plus the Eulerian mapping data F^{-1}, det F for the
  // deformed-frame variants).
  template <typename T>
  struct NHState
  {
    int            dim = 3, Qp = 0;
    Caching        caching = scalar_referential;
    Material       mat;
    size_t         n_cells = 0;
    std::vector<T> scalar;        // cached_scalar            [cell][q]
    std::vector<T> second_scalar; // cached_second_scalar     [cell][q]
    std::vector<T> t2;            // cached_tensor2           [cell][q][dim*dim]
    std::vector<T> t4;            // cached_tensor4 (full)    [cell][q][dim^4]
    std::vector<T> t4ns;          // cached_tensor4_ns        [cell][q][dim^4]
    std::vector<T> map_Finv;      // Eulerian mapping F^{-1}  [cell][q][dim*dim]
    std::vector<T> map_J;         // Eulerian mapping det F   [cell][q]
    std::vector<T> u;             // linearisation (plain), for scalar_referential
    const Box     *box   = nullptr;
    const Basis1D *basis = nullptr;
    bool           positive_J = true;
  };

  // Gradient of the linearisation field at the qp of a cell (real coords),
  // read without constraints (read_dof_values_plain, mf_nh_operator.h:410).
  template <typename T>
  void
  cell_gradients_plain(const Box &box, const Basis1D &b, const T *u, size_t e,
                       CellScratch<T> &s, T *grad_out)
  {
    const int dim = box.dim;
    const int Nd  = ipow(b.N, dim);
    const int Qp  = ipow(b.Q, dim);
    box.cell_nodes(e, s.nodes.data());
    const DirMats m = cell_mats(b);
    for (int c = 0; c < dim; ++c)
      {
        for (int l = 0; l < Nd; ++l)
          s.u[l] = u[size_t(c) * box.n_nodes + s.nodes[l]];
        evaluate_scalar(dim, b.N, m, s.u.data(), (T *)nullptr,
                        grad_out + size_t(c) * dim * Qp, s.w0.data(),
                        s.w1.data(), s.w2.data(), s.w3.data());
        for (int d = 0; d < dim; ++d)
          for (int q = 0; q < Qp; ++q)
            grad_out[(size_t(c) * dim + d) * Qp + q] /= T(box.h[d]);
      }
  }

  // NeoHookOperator::cache (mf_nh_operator.h:394-523)
  template <typename T>
  void
  nh_cache(NHState<T> &st, const Box &box, const Basis1D &b, const T *u)
  {
    const int dim = box.dim;
    const int Qp  = ipow(b.Q, dim);
    const int d2  = dim * dim;
    const int d4  = d2 * d2;
    st.dim        = dim;
    st.Qp         = Qp;
    st.n_cells    = box.n_cells;
    st.box        = &box;
    st.basis      = &b;
    st.positive_J = true;
    const size_t nq = box.n_cells * size_t(Qp);
    st.scalar.assign(nq, T(0));
    st.second_scalar.assign(nq, T(0));
    st.t2.assign(nq * d2, T(0));
    st.map_Finv.assign(nq * d2, T(0));
    st.map_J.assign(nq, T(0));
    if (st.caching == tensor4)
      st.t4.assign(nq * d4, T(0));
    if (st.caching == tensor4_ns)
      st.t4ns.assign(nq * d4, T(0));
    st.u.assign(u, u + size_t(dim) * box.n_nodes);
    const Material &mat    = st.mat;
    const T         mu     = T(mat.mu);
    const T         lambda = T(mat.lambda());
    if (mat.formulation == 0 && st.caching != tensor2)
      throw std::runtime_error("formulation 0 requires tensor2 caching");
    bool ok = true;
#pragma omp parallel reduction(&& : ok)
    {
      CellScratch<T> s;
      s.init(dim, dim, b.N, b.Q);
      std::vector<T> grad(size_t(dim) * dim * Qp);
#pragma omp for schedule(static)
      for (long el = 0; el < long(box.n_cells); ++el)
        {
          const size_t e = size_t(el);
          cell_gradients_plain(box, b, u, e, s, grad.data());
          for (int q = 0; q < Qp; ++q)
            {
              T H[9], F[9], Fi[9];
              for (int c = 0; c < dim; ++c)
                for (int d = 0; d < dim; ++d)
                  {
                    H[c * dim + d] = grad[(size_t(c) * dim + d) * Qp + q];
                    F[c * dim + d] = H[c * dim + d] + (c == d ? T(1) : T(0));
                  }
              const T Jm1 = jm1_from_grad(dim, H);
              const T J   = T(1) + Jm1;
              const T lnJ = std::log1p(Jm1);
              if (!(J > T(0)))
                {
                  ok = false;
                  continue;
                }
              invert(dim, F, Fi);
              const size_t iq = e * Qp + q;
              for (int i = 0; i < d2; ++i)
                st.map_Finv[iq * d2 + i] = Fi[i];
              st.map_J[iq] = J;
              if (mat.formulation == 0)
                {
                  st.scalar[iq] = std::exp(lnJ * T(-1.0 / dim));
                  for (int i = 0; i < d2; ++i)
                    st.t2[iq * d2 + i] = F[i];
                  continue;
                }
              const T scalar = mu - T(2.0) * lambda * lnJ;
              T       tau[9];
              get_tau(mat, dim, H, tau);
              switch (st.caching)
                {
                  case scalar_referential:
                    st.scalar[iq] = scalar;
                    break;
                  case tensor2:
                    st.scalar[iq]        = scalar * T(2.) / J;
                    st.second_scalar[iq] = T(1.) / J;
                    for (int i = 0; i < d2; ++i)
                      st.t2[iq * d2 + i] = tau[i] / J;
                    break;
                  case tensor4:
                    {
                      st.second_scalar[iq] = T(1.) / J;
                      for (int i = 0; i < d2; ++i)
                        st.t2[iq * d2 + i] = tau[i] / J;
                      // (2 scalar / J) S + (2 lambda / J) I x I, S the
                      // symmetric identity on symmetric tensors
                      const T a  = scalar * T(2.) / J;
                      const T bl = lambda * T(2.) / J;
                      T      *C  = &st.t4[iq * d4];
                      for (int i = 0; i < dim; ++i)
                        for (int j = 0; j < dim; ++j)
                          for (int k = 0; k < dim; ++k)
                            for (int l = 0; l < dim; ++l)
                              C[((i * dim + j) * dim + k) * dim + l] =
                                a * T(0.5) *
                                  (T(i == k && j == l) + T(i == l && j == k)) +
                                bl * T(i == j && k == l);
                      break;
                    }
                  case tensor4_ns:
                    {
                      // 2 lambda F^{-T} (x) F^{-T} + (mu - 2 lambda ln J)
                      // [F^{-T}]_il [F^{-1}]_jk + mu delta_ik delta_jl
                      T *A = &st.t4ns[iq * d4];
                      for (int i = 0; i < dim; ++i)
                        for (int j = 0; j < dim; ++j)
                          for (int k = 0; k < dim; ++k)
                            for (int l = 0; l < dim; ++l)
                              {
                                const T FiT_ij = Fi[j * dim + i];
                                const T FiT_kl = Fi[l * dim + k];
                                const T FiT_il = Fi[l * dim + i];
                                const T Fi_jk  = Fi[j * dim + k];
                                A[((i * dim + j) * dim + k) * dim + l] =
                                  T(2.) * lambda * FiT_ij * FiT_kl +
                                  (mu - T(2.0) * lambda * lnJ) * FiT_il * Fi_jk +
                                  mu * T(i == k && j == l);
                              }
                      break;
                    }
                }
            }
        }
    }
    st.positive_J = ok;
  }

  // Formulation-0 tangent flux in the current frame (mf_nh_operator.h:701-840)
  template <typename T>
  void
  form0_flux(const Material &mat, int dim, const T *F, T jscale, const T *g,
             T *P)
  {
    const T kappa = T(mat.kappa());
    const T c_1   = T(mat.c_1());
    const T J     = det(dim, F);
    T       Fb[9], b_bar[9], sg[9];
    for (int i = 0; i < dim * dim; ++i)
      Fb[i] = F[i] * jscale;
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j)
        {
          T s = T(0);
          for (int k = 0; k < dim; ++k)
            s += Fb[i * dim + k] * Fb[j * dim + k];
          b_bar[i * dim + j] = s;
          sg[i * dim + j]    = T(0.5) * (g[i * dim + j] + g[j * dim + i]);
        }
    const T inv_dim = T(1.0 / dim), two_over_dim = T(2.0 / dim);
    T       tau_bar[9];
    for (int i = 0; i < dim * dim; ++i)
      tau_bar[i] = b_bar[i] * (T(2.0) * c_1);
    T tr_tau_bar = T(0);
    for (int d = 0; d < dim; ++d)
      tr_tau_bar += tau_bar[d * dim + d];
    const T tr_tau_bar_dim = tr_tau_bar * inv_dim;
    const T dPsi           = (kappa / T(2.0)) * (J - T(1.0) / J);
    const T dPsi_J         = dPsi * J;
    const T d2Psi          = (kappa / T(2.0)) * (T(1.0) + T(1.0) / (J * J));
    T       tau[9];
    for (int i = 0; i < dim * dim; ++i)
      tau[i] = tau_bar[i];
    for (int d = 0; d < dim; ++d)
      tau[d * dim + d] += dPsi_J - tr_tau_bar_dim;
    T tr = T(0);
    for (int d = 0; d < dim; ++d)
      tr += sg[d * dim + d];
    T jc[9], dev[9], tau_iso[9];
    for (int i = 0; i < dim * dim; ++i)
      {
        dev[i]     = sg[i];
        tau_iso[i] = tau_bar[i];
        jc[i]      = sg[i] * (-dPsi_J * T(2.0));
      }
    for (int d = 0; d < dim; ++d)
      {
        dev[d * dim + d] -= tr * inv_dim;
        tau_iso[d * dim + d] -= tr_tau_bar_dim;
        jc[d * dim + d] += J * (dPsi + J * d2Psi) * tr;
      }
    T tau_iso_src = T(0);
    for (int i = 0; i < dim * dim; ++i)
      {
        jc[i] += (two_over_dim * tr_tau_bar) * dev[i];
        jc[i] -= (two_over_dim * tr) * tau_iso[i];
        tau_iso_src += tau_iso[i] * sg[i];
      }
    for (int d = 0; d < dim; ++d)
      jc[d * dim + d] -= two_over_dim * tau_iso_src;
    const T inv_J = T(1.0) / J;
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j)
        {
          T geo = T(0);
          for (int k = 0; k < dim; ++k)
            geo += g[i * dim + k] * tau[k * dim + j];
          P[i * dim + j] = (jc[i * dim + j] + geo) * inv_J;
        }
  }

  // Quadrature-point operation of the tangent, all variants.
  template <typename T>
  struct NHQ
  {
    static constexpr bool has_val  = true;
    static constexpr bool has_grad = true;
    NHState<T>           *st;
    void
    cell(size_t e, int nc, int Qp, T *val, T *grad)
    {
      (void)nc;
      NHState<T>     &S      = *st;
      const int       dim    = S.dim;
      const int       d2     = dim * dim;
      const Material &mat    = S.mat;
      const T         mu     = T(mat.mu);
      const T         lambda = T(mat.lambda());
      const T         ra     = T(mat.rho_alpha());
      thread_local std::vector<T>              gu;
      thread_local CellScratch<T>              s;
      thread_local int                         init_key = -1;
      const int key = dim * 1000 + S.basis->N * 10 + S.basis->Q;
      if (init_key != key)
        {
          s.init(dim, dim, S.basis->N, S.basis->Q);
          gu.resize(size_t(dim) * dim * Qp);
          init_key = key;
        }
      if (mat.formulation == 1 && S.caching == scalar_referential)
        cell_gradients_plain(*S.box, *S.basis, S.u.data(), e, s, gu.data());
      for (int q = 0; q < Qp; ++q)
        {
          const size_t iq = e * Qp + q;
          T            H[9], P[9], v[3];
          for (int c = 0; c < dim; ++c)
            {
              v[c] = val[size_t(c) * Qp + q];
              for (int d = 0; d < dim; ++d)
                H[c * dim + d] = grad[(size_t(c) * dim + d) * Qp + q];
            }
          T out_v[3];
          if (mat.formulation == 0)
            {
              const T *F  = &S.t2[iq * d2];
              const T *Fi = &S.map_Finv[iq * d2];
              const T  J  = S.map_J[iq];
              T        g[9], Pc[9];
              matmul(dim, H, Fi, g); // grad_x v = grad_X v F^{-1}
              form0_flux(mat, dim, F, S.scalar[iq], g, Pc);
              // current -> referential: J Pc F^{-T}
              for (int i = 0; i < dim; ++i)
                for (int j = 0; j < dim; ++j)
                  {
                    T sum = T(0);
                    for (int k = 0; k < dim; ++k)
                      sum += Pc[i * dim + k] * Fi[j * dim + k];
                    P[i * dim + j] = J * sum;
                  }
              for (int c = 0; c < dim; ++c)
                out_v[c] = v[c] * ra / J * J;
            }
          else
            switch (S.caching)
              {
                case scalar_referential:
                  {
                    // mf_nh_operator.h:848-943
                    T F[9], Fi[9], g[9], tau[9], q9[9];
                    for (int c = 0; c < dim; ++c)
                      for (int d = 0; d < dim; ++d)
                        F[c * dim + d] = gu[(size_t(c) * dim + d) * Qp + q] +
                                         (c == d ? T(1) : T(0));
                    for (int i = 0; i < dim; ++i)
                      for (int j = 0; j < dim; ++j)
                        {
                          T sum = T(0);
                          for (int k = 0; k < dim; ++k)
                            sum += F[i * dim + k] * F[j * dim + k];
                          tau[i * dim + j] = mu * sum;
                        }
                    const T c = S.scalar[iq];
                    for (int d = 0; d < dim; ++d)
                      tau[d * dim + d] -= c;
                    invert(dim, F, Fi);
                    matmul(dim, H, Fi, g);
                    T tr = T(0);
                    for (int d = 0; d < dim; ++d)
                      tr += g[d * dim + d];
                    for (int i = 0; i < dim; ++i)
                      for (int j = 0; j < dim; ++j)
                        {
                          T gt = T(0);
                          for (int k = 0; k < dim; ++k)
                            gt += g[i * dim + k] * tau[k * dim + j];
                          q9[i * dim + j] =
                            (T(2.0) * c) * T(0.5) * (g[i * dim + j] + g[j * dim + i]) +
                            (i == j ? T(2.0) * lambda * tr : T(0)) + gt;
                        }
                    for (int i = 0; i < dim; ++i)
                      for (int j = 0; j < dim; ++j)
                        {
                          T sum = T(0);
                          for (int k = 0; k < dim; ++k)
                            sum += q9[i * dim + k] * Fi[j * dim + k];
                          P[i * dim + j] = sum;
                        }
                    for (int c2 = 0; c2 < dim; ++c2)
                      out_v[c2] = v[c2] * ra;
                    break;
                  }
                case tensor2:
                case tensor4:
                  {
                    // mf_nh_operator.h:945-994 (deformed frame)
                    const T *Fi = &S.map_Finv[iq * d2];
                    const T  J  = S.map_J[iq];
                    const T *T2 = &S.t2[iq * d2];
                    T        g[9], Pc[9];
                    matmul(dim, H, Fi, g);
                    if (S.caching == tensor2)
                      {
                        T tr = T(0);
                        for (int d = 0; d < dim; ++d)
                          tr += g[d * dim + d];
                        const T tmp = T(2) * lambda * S.second_scalar[iq] * tr;
                        for (int i = 0; i < dim; ++i)
                          for (int j = 0; j < dim; ++j)
                            {
                              T gt = T(0);
                              for (int k = 0; k < dim; ++k)
                                gt += g[i * dim + k] * T2[k * dim + j];
                              Pc[i * dim + j] =
                                S.scalar[iq] * T(0.5) *
                                  (g[i * dim + j] + g[j * dim + i]) +
                                (i == j ? tmp : T(0)) + gt;
                            }
                      }
                    else
                      {
                        const T *C = &S.t4[iq * d2 * d2];
                        for (int i = 0; i < dim; ++i)
                          for (int j = 0; j < dim; ++j)
                            {
                              T gt = T(0);
                              for (int k = 0; k < dim; ++k)
                                gt += g[i * dim + k] * T2[k * dim + j];
                              T cs = T(0);
                              for (int k = 0; k < dim; ++k)
                                for (int l = 0; l < dim; ++l)
                                  cs += C[((i * dim + j) * dim + k) * dim + l] *
                                        T(0.5) * (g[k * dim + l] + g[l * dim + k]);
                              Pc[i * dim + j] = gt + cs;
                            }
                      }
                    for (int i = 0; i < dim; ++i)
                      for (int j = 0; j < dim; ++j)
                        {
                          T sum = T(0);
                          for (int k = 0; k < dim; ++k)
                            sum += Pc[i * dim + k] * Fi[j * dim + k];
                          P[i * dim + j] = J * sum;
                        }
                    for (int c = 0; c < dim; ++c)
                      out_v[c] = v[c] * ra * S.second_scalar[iq] * J;
                    break;
                  }
                case tensor4_ns:
                  {
                    // mf_nh_operator.h:996-1010
                    const T *A = &S.t4ns[iq * d2 * d2];
                    for (int i = 0; i < dim; ++i)
                      for (int j = 0; j < dim; ++j)
                        {
                          T sum = T(0);
                          for (int k = 0; k < dim; ++k)
                            for (int l = 0; l < dim; ++l)
                              sum += A[((i * dim + j) * dim + k) * dim + l] *
                                     H[k * dim + l];
                          P[i * dim + j] = sum;
                        }
                    for (int c = 0; c < dim; ++c)
                      out_v[c] = v[c] * ra;
                    break;
                  }
              }
          for (int c = 0; c < dim; ++c)
            {
              val[size_t(c) * Qp + q] = out_v[c];
              for (int d = 0; d < dim; ++d)
                grad[(size_t(c) * dim + d) * Qp + q] = P[c * dim + d];
            }
        }
    }
  };
} // namespace orc
