// CG (SolverCG), Chebyshev smoother (PreconditionChebyshev) and the
// multigrid V-cycle (Multigrid::level_v_step + PreconditionMG) on the
// device.  The host only sequences kernel launches; vectors never leave
// HBM.  Per CG iteration one 8-byte residual norm is read back for the
// convergence test.
#include <algorithm>
#include <cmath>
#include <functional>

#include "mf_solvers.h"

namespace mfgpu
{
  // ---------------------------------------------------------------------
  // CG
  // ---------------------------------------------------------------------
  template <typename T>
  CGStats
  cg_solve(Context &c, LinOp<T> &A, Precond<T> *P, T *x, const T *b, double tol,
           int maxit, bool record, bool fixed_iterations, DevBuf *ws)
  {
    CGStats      st;
    const size_t n  = A.size();
    const size_t vb = (n * sizeof(T) + 255) / 256 * 256;
    DevBuf       own;
    DevBuf      &W = ws ? *ws : own;
    if (W.bytes < 4 * vb)
      W.alloc(4 * vb);
    char *base = static_cast<char *>(W.ptr);
    T    *r = reinterpret_cast<T *>(base), *z = reinterpret_cast<T *>(base + vb);
    T    *p = reinterpret_cast<T *>(base + 2 * vb), *q = reinterpret_cast<T *>(base + 3 * vb);
    // r = b - A x
    A.vmult(r, x);
    vec_axpby<T>(c, n, T(1), b, T(-1), r);
    vec_dot_dev<T>(c, n, r, r, S_RR);
    read_scalars(c, S_RR + 1);
    double res = std::sqrt(c.host_scalars[S_RR]);
    st.res0    = res;
    st.res     = res;
    if (!std::isfinite(res))
      throw Error(ERR_NONFINITE, "CG: non-finite residual");
    if (res <= tol && !fixed_iterations)
      {
        st.converged = true;
        return st;
      }
    if (P)
      P->vmult(z, r);
    else
      vec_copy<T>(c, n, r, z);
    vec_dot_dev<T>(c, n, r, z, S_RZ);
    vec_copy<T>(c, n, z, p);
    int rz = S_RZ, rzn = S_RZN;
    for (int it = 1; it <= maxit; ++it)
      {
        A.vmult(q, p);
        vec_dot_dev<T>(c, n, p, q, S_PQ);
        cg_update<T>(c, n, rz, S_PQ, x, p, r, q, S_RR);
        read_scalars(c, 5);
        res    = std::sqrt(c.host_scalars[S_RR]);
        st.its = it;
        st.res = res;
        if (record)
          st.alpha.push_back(c.host_scalars[rz] / c.host_scalars[S_PQ]);
        if (!std::isfinite(res))
          throw Error(ERR_NONFINITE, "CG: non-finite residual");
        if (res <= tol)
          {
            st.converged = true;
            break;
          }
        if (P)
          P->vmult(z, r);
        else
          vec_copy<T>(c, n, r, z);
        vec_dot_dev<T>(c, n, r, z, rzn);
        cg_direction<T>(c, n, rzn, rz, z, p);
        if (record)
          {
            read_scalars(c, 5);
            st.beta.push_back(c.host_scalars[rzn] / c.host_scalars[rz]);
          }
        std::swap(rz, rzn);
      }
    return st;
  }

  bool
  cg_solve_batched(Context &c, LinOp<double> &A, Precond<double> *P, double *x, const double *b, int nb, size_t n,
                   const std::vector<double> &tol, int maxit, std::vector<int> &its, DevBuf *ws)
  {
    if (nb < 1 || nb > 6 || A.size() != size_t(nb) * n || int(tol.size()) != nb)
      throw Error(ERR_ARG, "cg_solve_batched: 1..6 systems of n unknowns");
    const size_t N  = size_t(nb) * n;
    const size_t vb = (N * sizeof(double) + 255) / 256 * 256;
    DevBuf       own;
    DevBuf      &W = ws ? *ws : own;
    if (W.bytes < 4 * vb)
      W.alloc(4 * vb);
    char   *base = static_cast<char *>(W.ptr);
    double *r = reinterpret_cast<double *>(base), *z = reinterpret_cast<double *>(base + vb);
    double *p = reinterpret_cast<double *>(base + 2 * vb), *q = reinterpret_cast<double *>(base + 3 * vb);
    // slots of system i: 5 i + {RR, RZ, RZN, PQ}
    auto slot = [](int i, int s) { return 5 * i + s; };
    std::vector<int>  rz(nb, S_RZ), rzn(nb, S_RZN);
    std::vector<char> active(nb, 1);
    its.assign(nb, 0);
    A.vmult(r, x);
    vec_axpby<double>(c, N, 1.0, b, -1.0, r);
    for (int i = 0; i < nb; ++i)
      vec_dot_dev<double>(c, n, r + i * n, r + i * n, slot(i, S_RR));
    read_scalars(c, 5 * nb);
    int n_active = 0;
    for (int i = 0; i < nb; ++i)
      {
        const double res = std::sqrt(c.host_scalars[slot(i, S_RR)]);
        if (!std::isfinite(res))
          throw Error(ERR_NONFINITE, "CG: non-finite residual");
        active[i] = res > tol[i];
        n_active += active[i];
      }
    if (n_active == 0)
      return true;
    if (P)
      P->vmult(z, r);
    else
      vec_copy<double>(c, N, r, z);
    for (int i = 0; i < nb; ++i)
      if (active[i])
        {
          vec_dot_dev<double>(c, n, r + i * n, z + i * n, slot(i, rz[i]));
          vec_copy<double>(c, n, z + i * n, p + i * n);
        }
    for (int it = 1; it <= maxit && n_active > 0; ++it)
      {
        A.vmult(q, p);
        for (int i = 0; i < nb; ++i)
          if (active[i])
            {
              vec_dot_dev<double>(c, n, p + i * n, q + i * n, slot(i, S_PQ));
              cg_update<double>(c, n, slot(i, rz[i]), slot(i, S_PQ), x + i * n, p + i * n, r + i * n, q + i * n,
                                slot(i, S_RR));
            }
        read_scalars(c, 5 * nb);
        for (int i = 0; i < nb; ++i)
          if (active[i])
            {
              const double res = std::sqrt(c.host_scalars[slot(i, S_RR)]);
              its[i]           = it;
              if (!std::isfinite(res))
                throw Error(ERR_NONFINITE, "CG: non-finite residual");
              if (res <= tol[i])
                {
                  active[i] = 0;
                  --n_active;
                }
            }
        if (n_active == 0)
          break;
        if (P)
          P->vmult(z, r);
        else
          vec_copy<double>(c, N, r, z);
        for (int i = 0; i < nb; ++i)
          if (active[i])
            {
              vec_dot_dev<double>(c, n, r + i * n, z + i * n, slot(i, rzn[i]));
              cg_direction<double>(c, n, slot(i, rzn[i]), slot(i, rz[i]), z + i * n, p + i * n);
              std::swap(rz[i], rzn[i]);
            }
      }
    return n_active == 0;
  }

  template <typename T>
  CGStats
  cg_lanczos(Context &c, LinOp<T> &A, Precond<T> *P, T *x, const T *b, double tol, int maxit,
             int check, DevBuf *ws, double *host_rec)
  {
    CGStats      st;
    const size_t n = A.size();
    // r, z, p, q, the Lanczos records and the record counter in one
    // allocation (256-byte aligned parts)
    const size_t vb    = (n * sizeof(T) + 255) / 256 * 256;
    const size_t recb  = (sizeof(double) * 3 * size_t(std::max(maxit, 1)) + 255) / 256 * 256;
    const size_t total = 4 * vb + recb + 256;
    DevBuf       own;
    DevBuf      &W = ws ? *ws : own;
    if (W.bytes < total)
      W.alloc(total);
    char   *base = static_cast<char *>(W.ptr);
    T      *r = reinterpret_cast<T *>(base), *z = reinterpret_cast<T *>(base + vb);
    T      *p = reinterpret_cast<T *>(base + 2 * vb), *q = reinterpret_cast<T *>(base + 3 * vb);
    double *rec     = reinterpret_cast<double *>(base + 4 * vb);
    int    *counter = reinterpret_cast<int *>(base + 4 * vb + recb);
    A.vmult(r, x);
    vec_axpby<T>(c, n, T(1), b, T(-1), r);
    vec_dot_dev<T>(c, n, r, r, S_RR);
    double res = 0;
    if (!host_rec)
      {
        read_scalars(c, S_RR + 1);
        res     = std::sqrt(c.host_scalars[S_RR]);
        st.res0 = res;
        st.res  = res;
        if (!std::isfinite(res))
          throw Error(ERR_NONFINITE, "CG: non-finite residual");
        if (res <= tol)
          {
            st.converged = true;
            return st;
          }
      }
    if (P)
      P->vmult(z, r);
    else
      vec_copy<T>(c, n, r, z);
    vec_dot_dev<T>(c, n, r, z, S_RZ);
    vec_copy<T>(c, n, z, p);
    int                 rz = S_RZ, rzn = S_RZN;
    std::vector<double> h;
    MF_CK(cudaMemsetAsync(counter, 0, sizeof(int), c.stream));
    // point-Jacobi preconditioner and an operator that adds: four launches
    // per iteration (q = A p into a zero q; p.q; x, r, z with |r|^2 and
    // r.z; p and the record).  The direction kernel zeroes q for the next
    // iteration on small vectors, a memset on large ones
    // (ZERO_IN_KERNEL_BYTES).
    const T   *jd     = P ? P->jacobi_diagonal() : nullptr;
    const bool q_kern = n * sizeof(T) <= ZERO_IN_KERNEL_BYTES;
    if (jd && A.can_add() && q_kern)
      MF_CK(cudaMemsetAsync(q, 0, n * sizeof(T), c.stream));
    auto iteration = [&]() {
      if (jd && A.can_add())
        {
          if (!q_kern)
            MF_CK(cudaMemsetAsync(q, 0, n * sizeof(T), c.stream));
          A.vmult_add(q, p);
          vec_dot_dev<T>(c, n, p, q, S_PQ);
          cg_update_jacobi<T>(c, n, rz, S_PQ, x, p, r, q, jd, z, S_RR, rzn);
          cg_direction_rec<T>(c, n, rz, rzn, S_PQ, S_RR, z, p, q_kern ? q : nullptr, rec, counter);
          std::swap(rz, rzn);
          return;
        }
      A.vmult(q, p);
      vec_dot_dev<T>(c, n, p, q, S_PQ);
      cg_update<T>(c, n, rz, S_PQ, x, p, r, q, S_RR);
      if (P)
        P->vmult(z, r);
      else
        vec_copy<T>(c, n, r, z);
      vec_dot_dev<T>(c, n, r, z, rzn);
      cg_direction<T>(c, n, rzn, rz, z, p);
      lanczos_record(c, rz, rzn, S_PQ, S_RR, rec, counter);
      std::swap(rz, rzn);
    };
    if (host_rec)
      {
        for (int j = 0; j < maxit; ++j)
          iteration();
        MF_CK(cudaMemcpyAsync(host_rec, rec, sizeof(double) * 3 * size_t(maxit), cudaMemcpyDeviceToHost,
                              c.stream));
        return st;
      }
    // a full batch (an even number of iterations, so the slot roles repeat)
    // is the same work every time: the second one is captured into a CUDA
    // graph and the later ones replay it
    cudaGraphExec_t gx      = nullptr;
    long long       gx_lnch = 0;
    int             batch   = 0;
    struct GraphGuard
    {
      cudaGraphExec_t &g;
      ~GraphGuard()
      {
        if (g)
          cudaGraphExecDestroy(g);
      }
    } guard{gx};
    for (int it0 = 1; it0 <= maxit; it0 += check, ++batch)
      {
        const int it1  = std::min(maxit, it0 + check - 1);
        const int cnt  = it1 - it0 + 1;
        const bool full = cnt == check && check % 2 == 0;
        if (full && gx)
          {
            MF_CK(cudaGraphLaunch(gx, c.stream));
            count_launch(int(gx_lnch));
          }
        else if (full && batch == 1)
          {
            const long long l0 = launch_count();
            MF_CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            cudaGraph_t g = nullptr;
            try
              {
                for (int j = 0; j < cnt; ++j)
                  iteration();
              }
            catch (...)
              {
                cudaStreamEndCapture(c.stream, &g);
                if (g)
                  cudaGraphDestroy(g);
                throw;
              }
            MF_CK(cudaStreamEndCapture(c.stream, &g));
            const cudaError_t e = cudaGraphInstantiate(&gx, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess)
              {
                gx = nullptr;
                MF_CK(e);
              }
            gx_lnch = launch_count() - l0;
            MF_CK(cudaGraphLaunch(gx, c.stream));
          }
        else
          for (int j = 0; j < cnt; ++j)
            iteration();
        h.resize(3 * size_t(cnt));
        MF_CK(cudaMemcpyAsync(h.data(), rec + 3 * size_t(it0 - 1), sizeof(double) * h.size(),
                              cudaMemcpyDeviceToHost, c.stream));
        MF_CK(cudaStreamSynchronize(c.stream));
        for (int j = 0; j < cnt; ++j)
          {
            res    = std::sqrt(h[3 * j + 1]);
            st.its = it0 + j;
            st.res = res;
            st.alpha.push_back(h[3 * j]);
            if (!std::isfinite(res))
              throw Error(ERR_NONFINITE, "CG: non-finite residual");
            if (res <= tol)
              {
                st.converged = true;
                return st;
              }
            st.beta.push_back(h[3 * j + 2]);
          }
      }
    return st;
  }

  template CGStats cg_lanczos<double>(Context &, LinOp<double> &, Precond<double> *, double *, const double *, double, int,
                                      int, DevBuf *, double *);
  template CGStats cg_lanczos<float>(Context &, LinOp<float> &, Precond<float> *, float *, const float *, double, int, int,
                                     DevBuf *, double *);

  CGStats
  lanczos_collect(const double *h, int maxit, double tol)
  {
    CGStats st;
    for (int j = 0; j < maxit; ++j)
      {
        const double res = std::sqrt(h[3 * j + 1]);
        st.its           = j + 1;
        st.res           = res;
        st.alpha.push_back(h[3 * j]);
        if (!std::isfinite(res))
          throw Error(ERR_NONFINITE, "CG: non-finite residual");
        if (res <= tol)
          {
            st.converged = true;
            return st;
          }
        st.beta.push_back(h[3 * j + 2]);
      }
    return st;
  }

  template CGStats cg_solve<double>(Context &, LinOp<double> &, Precond<double> *, double *, const double *, double, int,
                                    bool, bool, DevBuf *);
  template CGStats cg_solve<float>(Context &, LinOp<float> &, Precond<float> *, float *, const float *, double, int, bool,
                                   bool, DevBuf *);

  // ---------------------------------------------------------------------
  // symmetric tridiagonal extreme eigenvalues (bisection, Sturm counts)
  // ---------------------------------------------------------------------
  static int
  sturm(const std::vector<double> &d, const std::vector<double> &e, double x)
  {
    int    cnt = 0;
    double q   = 1;
    for (size_t i = 0; i < d.size(); ++i)
      {
        q = d[i] - x - (i ? e[i - 1] * e[i - 1] / q : 0.0);
        if (q == 0)
          q = 1e-300;
        if (q < 0)
          ++cnt;
      }
    return cnt;
  }

  static double
  tridiag_eig(const std::vector<double> &d, const std::vector<double> &e, int k)
  {
    double lo = 1e300, hi = -1e300;
    for (size_t i = 0; i < d.size(); ++i)
      {
        const double r = (i ? std::fabs(e[i - 1]) : 0.0) + (i + 1 < d.size() ? std::fabs(e[i]) : 0.0);
        lo             = std::min(lo, d[i] - r);
        hi             = std::max(hi, d[i] + r);
      }
    for (int it = 0; it < 200; ++it)
      {
        const double mid = 0.5 * (lo + hi);
        if (sturm(d, e, mid) > k)
          hi = mid;
        else
          lo = mid;
      }
    return 0.5 * (lo + hi);
  }

  std::pair<double, double>
  lanczos_extreme_eigenvalues(const CGStats &st)
  {
    const size_t k = st.alpha.size();
    if (k == 0)
      return {1.0, 1.0};
    std::vector<double> d(k), e(k - 1);
    for (size_t i = 0; i < k; ++i)
      d[i] = 1. / st.alpha[i] + (i > 0 ? st.beta[i - 1] / st.alpha[i - 1] : 0.);
    for (size_t i = 0; i + 1 < k; ++i)
      e[i] = std::sqrt(st.beta[i]) / st.alpha[i];
    return {tridiag_eig(d, e, 0), tridiag_eig(d, e, int(k) - 1)};
  }

  // ---------------------------------------------------------------------
  // Chebyshev
  // ---------------------------------------------------------------------
  template <typename T>
  struct JacobiPre : Precond<T>
  {
    Context  *ctx;
    Operator *A;
    void
    vmult(T *dst, const T *src) override
    {
      vec_scale<T>(*ctx, A->m(), T(1), A->inv_diag.as<T>(), src, dst);
    }
    const T *jacobi_diagonal() const override { return A->inv_diag.as<T>(); }
  };

  template <typename T>
  void
  Chebyshev<T>::estimate()
  {
    const size_t n = A->m();
    xold.ensure(n * sizeof(T));
    if (t1.bytes != n * sizeof(T))
      t1_zero = false;
    t1.ensure(n * sizeof(T));
    w0.ensure(n * sizeof(T));
    w1.ensure(n * sizeof(T));
    // initial guess with high-frequency content and the constant mode:
    // entries 1 except every 11th, mean removed
    vec_estimate_start<T>(*ctx, n, w0.as<T>(), start_period());
    MF_CK(cudaMemsetAsync(w1.ptr, 0, n * sizeof(T), ctx->stream));
    OpRef<T>     Aop(A);
    JacobiPre<T> P;
    P.ctx      = ctx;
    P.A        = A;
    CGStats st = cg_lanczos<T>(*ctx, Aop, &P, w1.as<T>(), w0.as<T>(), estimate_tol(), eig_cg_iterations, 8,
                               &cg_ws);
    set_bounds(st);
  }

  template <typename T>
  void
  Chebyshev<T>::estimate_begin(Context *ec)
  {
    const size_t n = A->m();
    xold.ensure(n * sizeof(T));
    if (t1.bytes != n * sizeof(T))
      t1_zero = false;
    t1.ensure(n * sizeof(T));
    w0.ensure(n * sizeof(T));
    w1.ensure(n * sizeof(T));
    host_rec.ensure(3 * size_t(std::max(eig_cg_iterations, 1)));
    // the operator launches on ec's stream until the work is enqueued
    struct Restore
    {
      Operator *op;
      Context  *c;
      ~Restore() { op->ctx = c; }
    } restore{A, A->ctx};
    A->ctx = ec;
    vec_estimate_start<T>(*ec, n, w0.as<T>(), start_period());
    MF_CK(cudaMemsetAsync(w1.ptr, 0, n * sizeof(T), ec->stream));
    OpRef<T>     Aop(A);
    JacobiPre<T> P;
    P.ctx = ec;
    P.A   = A;
    cg_lanczos<T>(*ec, Aop, &P, w1.as<T>(), w0.as<T>(), estimate_tol(), eig_cg_iterations, 8, &cg_ws,
                  host_rec.p);
    est_ctx = ec;
  }

  template <typename T>
  void
  Chebyshev<T>::estimate_end()
  {
    if (!est_ctx)
      throw Error(ERR_STATE, "Chebyshev: estimate_end without estimate_begin");
    Context *ec = est_ctx;
    est_ctx     = nullptr;
    MF_CK(cudaStreamSynchronize(ec->stream));
    set_bounds(lanczos_collect(host_rec.p, eig_cg_iterations, estimate_tol()));
  }

  template <typename T>
  void
  Chebyshev<T>::set_bounds(const CGStats &st)
  {
    const auto ev = lanczos_extreme_eigenvalues(st);
    lambda_min    = ev.first;
    lambda_max    = st.alpha.empty() ? 1.0 : 1.2 * ev.second;
    const double alpha = smoothing_range > 1. ? lambda_max / smoothing_range :
                                                std::min(0.9 * lambda_max, lambda_min);
    if (degree == 0)
      {
        const double actual_range = lambda_max / alpha;
        const double sigma        = (1. - std::sqrt(1. / actual_range)) / (1. + std::sqrt(1. / actual_range));
        const double eps          = smoothing_range;
        degree = 1 + unsigned(std::log(1. / eps + std::sqrt(1. / eps / eps - 1.)) / std::log(1. / sigma));
      }
    delta       = (lambda_max - alpha) * 0.5;
    theta       = (lambda_max + alpha) * 0.5;
    initialized = true;
  }

  template <typename T>
  void
  Chebyshev<T>::vmult(T *x, const T *b)
  {
    if (!initialized)
      estimate();
    const size_t n    = A->m();
    const T     *dinv = A->inv_diag.as<T>();
    cheby_start<T>(*ctx, n, T(1. / theta), b, dinv, x, xold.as<T>());
    if (degree < 2)
      return;
    double rhok = delta / theta, sigma = theta / delta;
    if (A->use_dense())
      {
        // dense operator: each step is one kernel (row products and the
        // update); the new iterate goes into the older buffer, then the two
        // swap
        const T *Ad  = A->dense.as<T>();
        T       *cur = x, *old = xold.as<T>();
        for (unsigned k = 0; k + 1 < degree; ++k)
          {
            const double rhokp = 1. / (2. * sigma - rhok);
            const double f1 = rhokp * rhok, f2 = 2. * rhokp / delta;
            rhok = rhokp;
            cheby_dense_step<T>(*ctx, n, Ad, T(f1), T(f2), k == 0, b, dinv, cur, old);
            std::swap(cur, old);
          }
        if (cur != x)
          vec_copy<T>(*ctx, n, cur, x);
        return;
      }
    // small levels (launch-bound): t1 = A x accumulates into a zero t1,
    // which every update leaves zero again, so no memset per step; large
    // levels zero t1 before every application (measured faster there)
    const bool keep_zero = small_level();
    if (!t1_zero || !keep_zero)
      MF_CK(cudaMemsetAsync(t1.ptr, 0, n * sizeof(T), ctx->stream));
    t1_zero = false;
    for (unsigned k = 0; k + 1 < degree; ++k)
      {
        if (k > 0 && !keep_zero)
          MF_CK(cudaMemsetAsync(t1.ptr, 0, n * sizeof(T), ctx->stream));
        A->vmult_add(t1.ptr, x);
        const double rhokp = 1. / (2. * sigma - rhok);
        const double f1 = rhokp * rhok, f2 = 2. * rhokp / delta;
        rhok = rhokp;
        cheby_update<T>(*ctx, n, T(f1), T(f2), k == 0, keep_zero, b, t1.as<T>(), dinv, x, xold.as<T>());
      }
    t1_zero = keep_zero;
  }

  template <typename T>
  void
  Chebyshev<T>::step(T *x, const T *b)
  {
    if (!initialized)
      estimate();
    const size_t n    = A->m();
    const T     *dinv = A->inv_diag.as<T>();
    // t1 as in vmult()
    const bool keep_zero = small_level();
    if (!t1_zero || !keep_zero)
      MF_CK(cudaMemsetAsync(t1.ptr, 0, n * sizeof(T), ctx->stream));
    t1_zero = false;
    A->vmult_add(t1.ptr, x);
    cheby_update<T>(*ctx, n, T(0), T(1. / theta), true, keep_zero, b, t1.as<T>(), dinv, x, xold.as<T>());
    if (degree >= 2)
      {
        double rhok = delta / theta, sigma = theta / delta;
        for (unsigned k = 0; k + 1 < degree; ++k)
          {
            if (!keep_zero)
              MF_CK(cudaMemsetAsync(t1.ptr, 0, n * sizeof(T), ctx->stream));
            A->vmult_add(t1.ptr, x);
            const double rhokp = 1. / (2. * sigma - rhok);
            const double f1 = rhokp * rhok, f2 = 2. * rhokp / delta;
            rhok = rhokp;
            cheby_update<T>(*ctx, n, T(f1), T(f2), false, keep_zero, b, t1.as<T>(), dinv, x, xold.as<T>());
          }
      }
    t1_zero = keep_zero;
  }

  template struct Chebyshev<float>;
  template struct Chebyshev<double>;

  // ---------------------------------------------------------------------
  // Multigrid
  // ---------------------------------------------------------------------
  template <typename T>
  void
  Multigrid<T>::drop_graph()
  {
    if (gexec)
      {
        // a replay may still be running on the context's stream
        if (ctx)
          cudaStreamSynchronize(ctx->stream);
        cudaGraphExecDestroy(gexec);
      }
    gexec      = nullptr;
    g_dst      = nullptr;
    g_src      = nullptr;
    eager_done = false;
  }

  namespace
  {
    size_t
    key_mix(size_t h, size_t v)
    {
      return h ^ (v + size_t(0x9e3779b97f4a7c15ULL) + (h << 6) + (h >> 2));
    }
  } // namespace

  template <typename T>
  void
  Multigrid<T>::setup(double range, unsigned degree, int eig_its, int coarse_eig_its)
  {
    // unchanged operators and parameters: the eigenvalue bounds, the
    // Chebyshev coefficients and the captured V-cycle stay valid (they are
    // functions of the operators; the reference rebuilds them every solve)
    size_t key = key_mix(std::hash<double>()(range), size_t(degree));
    key        = key_mix(key_mix(key, size_t(eig_its)), size_t(coarse_eig_its));
    for (Operator *op : ops)
      key = key_mix(key_mix(key, op->value_state()), reinterpret_cast<uintptr_t>(op->inv_diag.ptr));
    if (coarse64)
      key = key_mix(key_mix(key, coarse64->value_state()), reinterpret_cast<uintptr_t>(coarse64->inv_diag.ptr));
    if (setup_done && key == setup_key)
      return;
    setup_done = false;
    drop_graph();
    const int L = int(ops.size());
    // the smoothers keep their work buffers across setups (same level sizes)
    if (int(smoothers.size()) != L)
      {
        smoothers.clear();
        smoothers.resize(L);
      }
    sol.resize(L);
    def.resize(L);
    tmp.resize(L);
    for (int l = 0; l < L; ++l)
      {
        Chebyshev<T> &s = smoothers[l];
        s.ctx           = ctx;
        s.A             = ops[l];
        if (l == 0)
          {
            s.smoothing_range   = 1e-3;
            s.degree            = 0;
            s.eig_cg_iterations = coarse_eig_its;
          }
        else
          {
            s.smoothing_range   = range;
            s.degree            = degree;
            s.eig_cg_iterations = eig_its;
          }
        s.initialized = false;
        const size_t bytes = ops[l]->m() * sizeof(T);
        if (sol[l].bytes != bytes)
          {
            sol[l].alloc(bytes);
            def[l].alloc(bytes);
            tmp[l].alloc(bytes);
          }
      }
    if (coarse64)
      {
        coarse_cheb64.ctx               = ctx;
        coarse_cheb64.A                 = coarse64;
        coarse_cheb64.smoothing_range   = 1e-3;
        coarse_cheb64.degree            = 0;
        coarse_cheb64.eig_cg_iterations = coarse_eig_its;
        coarse_cheb64.initialized       = false;
        c64_sol.ensure(coarse64->m() * sizeof(double));
        c64_def.ensure(coarse64->m() * sizeof(double));
      }
    // eigenvalue bounds of every smoother now (PreconditionChebyshev
    // estimates on its first vmult; here setup carries that cost)
    // The level estimates are independent: the ones with a fixed, small
    // iteration count are enqueued on their own contexts (finest first,
    // no host wait), the coarse one with m() iterations and convergence
    // checks runs on the main stream meanwhile; the small, launch-bound
    // levels then overlap instead of adding up.
    std::vector<int> deferred;
    for (int l = L - 1; l >= 0; --l)
      if ((l > 0 || !coarse64) && smoothers[l].eig_cg_iterations <= 64)
        deferred.push_back(l);
    if (!deferred.empty())
      {
        if (int(aux.size()) < L)
          aux.resize(L);
        if (!setup_ev)
          MF_CK(cudaEventCreateWithFlags(&setup_ev, cudaEventDisableTiming));
        // the diagonals and caches were written on the main stream
        MF_CK(cudaEventRecord(setup_ev, ctx->stream));
        for (int l : deferred)
          {
            if (!aux[l])
              aux[l].reset(new Context(ctx->device));
            MF_CK(cudaStreamWaitEvent(aux[l]->stream, setup_ev, 0));
            smoothers[l].estimate_begin(aux[l].get());
          }
      }
    for (int l = 0; l < L; ++l)
      if ((l > 0 || !coarse64) && smoothers[l].eig_cg_iterations > 64)
        smoothers[l].estimate();
    if (coarse64)
      coarse_cheb64.estimate();
    for (int l : deferred)
      smoothers[l].estimate_end();
    setup_key  = key;
    setup_done = true;
  }

  template <typename T>
  Multigrid<T>::~Multigrid()
  {
    drop_graph();
    aux.clear(); // synchronises their streams
    if (setup_ev)
      cudaEventDestroy(setup_ev);
  }

  template <typename T>
  void
  Multigrid<T>::level_v_step(int l)
  {
    const size_t n = ops[l]->m();
    if (l == 0)
      {
        if (coarse64)
          {
            vec_convert<double, T>(*ctx, n, def[0].template as<T>(), c64_def.as<double>());
            coarse_cheb64.vmult(c64_sol.as<double>(), c64_def.as<double>());
            vec_convert<T, double>(*ctx, n, c64_sol.as<double>(), sol[0].template as<T>());
          }
        else
          smoothers[0].vmult(sol[0].template as<T>(), def[0].template as<T>());
        return;
      }
    T *s = sol[l].template as<T>(), *d = def[l].template as<T>(), *t = tmp[l].template as<T>();
    smoothers[l].vmult(s, d);
    ops[l]->vmult(t, s);
    vec_axpby<T>(*ctx, n, T(1), d, T(-1), t); // t = d - A s
    MF_CK(cudaMemsetAsync(def[l - 1].ptr, 0, def[l - 1].bytes, ctx->stream));
    transfers[l]->restrict_add(def[l - 1].ptr, t);
    MF_CK(cudaMemsetAsync(sol[l - 1].ptr, 0, sol[l - 1].bytes, ctx->stream));
    level_v_step(l - 1);
    transfers[l]->prolongate_add(s, sol[l - 1].ptr);
    smoothers[l].step(s, d);
  }

  template <typename T>
  void
  Multigrid<T>::vmult(double *dst, const double *src)
  {
    if (use_graphs)
      {
        if (gexec && dst == g_dst && src == g_src)
          {
            MF_CK(cudaGraphLaunch(gexec, ctx->stream));
            count_launch(int(g_launches));
            ++graph_replays;
            ++vcycles;
            return;
          }
        if (eager_done)
          {
            // the smoothers' eigenvalue estimates ran in the eager V-cycle,
            // so the captured work is launches, copies and memsets only
            drop_graph();
            const long long l0 = launch_count();
            MF_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            cudaGraph_t g = nullptr;
            try
              {
                vcycle(dst, src);
              }
            catch (...)
              {
                cudaStreamEndCapture(ctx->stream, &g);
                if (g)
                  cudaGraphDestroy(g);
                throw;
              }
            MF_CK(cudaStreamEndCapture(ctx->stream, &g));
            const cudaError_t e = cudaGraphInstantiate(&gexec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess)
              {
                gexec = nullptr;
                MF_CK(e);
              }
            g_launches = launch_count() - l0;
            g_dst      = dst;
            g_src      = src;
            eager_done = true;
            MF_CK(cudaGraphLaunch(gexec, ctx->stream)); // vcycle() counted it
            return;
          }
        eager_done = true;
      }
    vcycle(dst, src);
  }

  template <typename T>
  void
  Multigrid<T>::vcycle(double *dst, const double *src)
  {
    const int    L = int(ops.size()) - 1;
    const size_t n = ops[L]->m();
    if constexpr (std::is_same<T, double>::value)
      vec_copy<double>(*ctx, n, src, def[L].template as<double>());
    else
      vec_convert<T, double>(*ctx, n, src, def[L].template as<T>());
    MF_CK(cudaMemsetAsync(sol[L].ptr, 0, sol[L].bytes, ctx->stream));
    level_v_step(L);
    if constexpr (std::is_same<T, double>::value)
      vec_copy<double>(*ctx, n, sol[L].template as<double>(), dst);
    else
      vec_convert<double, T>(*ctx, n, sol[L].template as<T>(), dst);
    ++vcycles;
  }

  template struct Multigrid<float>;
  template struct Multigrid<double>;
} // namespace mfgpu
