// extern "C" entry points of the multigrid preconditioner (PreconditionMG),
// the CG solver (SolverCG), the condition-number estimate and the maps
// between a caller's DoF numbering and the library's (declared in
// include/mfgpu.h).
#include <cmath>

#include "mf_capi.h"

struct mfgpu_mg
{
  std::unique_ptr<GMGHierarchy> h;
  mfgpu_context                *ctx   = nullptr;
  bool                          ready = false;
  PhaseTimer                    timer; // disabled: no section timing
};

struct mfgpu_permutation
{
  mfgpu_context *ctx = nullptr;
  DevBuf         idx; // library_dof[i], size_t
  size_t         n   = 0;
};

namespace
{
  // the library DoF of each of the caller's DoFs (support point, component)
  std::vector<size_t>
  build_permutation(const mfgpu_mesh &mm, int level, size_t n, const double *pts, const unsigned *comps,
                    double tol)
  {
    const Mesh      m = to_mesh(mm);
    const LevelGeom g = m.level(level);
    HostBasis       b;
    make_host_basis(m.degree, b);
    if (g.n_nodes == 0 || n % g.n_nodes != 0 || n / g.n_nodes < 1 || n / g.n_nodes > 3)
      throw Error(ERR_ARG, "n_dofs must be 1, 2 or 3 times the number of nodes of the level (" +
                             std::to_string(g.n_nodes) + ")");
    if (!(tol > 0) || tol >= 0.5)
      throw Error(ERR_ARG, "tol must be in (0, 0.5)");
    const unsigned nc = unsigned(n / g.n_nodes);
    std::vector<size_t> out(n);
    std::vector<char>   hit(n, 0);
    for (size_t i = 0; i < n; ++i)
      {
        int idx[3] = {0, 0, 0};
        for (int d = 0; d < m.dim; ++d)
          {
            const double t = (pts[3 * i + d] - g.lo[d]) / g.h[d];
            if (!(t > -tol && t < g.C[d] + tol))
              throw Error(ERR_ARG, "support point " + std::to_string(i) + " lies outside the mesh");
            const int    c  = std::min(std::max(int(std::floor(t)), 0), g.C[d] - 1);
            const double lc = t - c;
            int          best = 0;
            for (int k = 1; k < b.N; ++k)
              if (std::fabs(b.nodes[k] - lc) < std::fabs(b.nodes[best] - lc))
                best = k;
            if (std::fabs(b.nodes[best] - lc) > tol)
              throw Error(ERR_ARG, "support point " + std::to_string(i) + " is not a node of the level");
            idx[d] = c * g.p + best;
          }
        const unsigned comp = comps ? comps[i] : 0u;
        if (comp >= nc)
          throw Error(ERR_ARG, "component of DoF " + std::to_string(i) + " out of range");
        const size_t node = size_t(idx[0]) + size_t(g.Nn[0]) * (size_t(idx[1]) + size_t(g.Nn[1]) * idx[2]);
        const size_t lib  = size_t(comp) * g.n_nodes + node;
        if (hit[lib])
          throw Error(ERR_ARG, "two DoFs map to library DoF " + std::to_string(lib));
        hit[lib] = 1;
        out[i]   = lib;
      }
    return out;
  }

  template <typename T>
  __global__ void
  k_permute(size_t n, const size_t *__restrict__ idx, const T *__restrict__ src, T *__restrict__ dst,
            int to_library)
  {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
      {
        const size_t j = idx[i];
        if (to_library)
          dst[j] = src[i];
        else
          dst[i] = src[j];
      }
  }

  void
  permute(mfgpu_permutation *p, int precision, const void *src, void *dst, int to_library)
  {
    need(p, "perm");
    need(src, "src");
    need(dst, "dst");
    if (src == dst)
      throw Error(ERR_ARG, "src and dst must differ");
    if (precision != 32 && precision != 64)
      throw Error(ERR_ARG, "precision must be 32 or 64");
    Context       &c    = *p->ctx->c;
    const unsigned grid = unsigned(std::min<size_t>((p->n + 255) / 256, size_t(c.n_sm) * 8));
    if (precision == 64)
      k_permute<double><<<std::max(grid, 1u), 256, 0, c.stream>>>(
        p->n, p->idx.as<size_t>(), static_cast<const double *>(src), static_cast<double *>(dst), to_library);
    else
      k_permute<float><<<std::max(grid, 1u), 256, 0, c.stream>>>(
        p->n, p->idx.as<size_t>(), static_cast<const float *>(src), static_cast<float *>(dst), to_library);
    count_launch();
    MF_CK(cudaGetLastError());
  }

  Operator *
  fp64_operator(mfgpu_operator *A)
  {
    need(A, "A");
    Operator *o = A->op.get();
    if (o->precision != 64)
      throw Error(ERR_ARG, "CG runs on FP64 operators");
    return o;
  }

  struct JacobiOmega : Precond<double>
  {
    Operator *A     = nullptr;
    double    omega = 1;
    void
    vmult(double *d, const double *s) override
    {
      vec_scale<double>(*A->ctx, A->m(), omega, A->inv_diag.as<double>(), s, d);
    }
  };
} // namespace

extern "C"
{
  int
  mfgpu_mg_create(mfgpu_context *ctx, const mfgpu_mesh *mesh, const mfgpu_mg_params *params, mfgpu_mg **mg)
  {
    return guarded([&] {
      need(ctx, "ctx");
      need(mesh, "mesh");
      need(params, "params");
      need(mg, "mg");
      const Mesh m = to_mesh(*mesh);
      auto      *o = new mfgpu_mg();
      try
        {
          if (params->kind == 0)
            {
              if (!(params->delta_t > 0))
                throw Error(ERR_ARG, "delta_t must be positive");
              o->h = GMGHierarchy::heat(ctx->c.get(), m, params->solver, params->delta_t);
            }
          else if (params->kind == 1)
            {
              const mfgpu_material &mt = params->material;
              if (mt.formulation != 0 && mt.formulation != 1)
                throw Error(ERR_ARG, "Unknown material formulation");
              const int var = parse_caching(params->caching);
              if (params->solver.fp64_emulation && (var != V_QP10 || mt.formulation != 1))
                throw Error(ERR_UNSUPPORTED, "fp64_emulation needs referential_qp caching and formulation 1");
              o->h = GMGHierarchy::solid(ctx->c.get(), m, params->solver,
                                         make_material(mt.mu, mt.nu, mt.rho, mt.alpha_1), mt.formulation, var);
            }
          else
            throw Error(ERR_ARG, "kind must be 0 (heat) or 1 (neo-Hookean)");
          o->ctx = ctx;
          ++ctx->live;
        }
      catch (...)
        {
          delete o;
          throw;
        }
      *mg = o;
    });
  }

  int
  mfgpu_mg_setup(mfgpu_mg *mg, const double *linearisation)
  {
    return guarded([&] {
      need(mg, "mg");
      GMGHierarchy &h = *mg->h;
      if (h.kind == 1)
        {
          need(linearisation, "linearisation");
          h.set_linearisation(linearisation, mg->timer);
        }
      else if (linearisation)
        throw Error(ERR_ARG, "heat levels take no linearisation");
      h.update_diagonals(mg->timer);
      h.setup_smoothers(mg->timer);
      mg->ready = true;
    });
  }

  int
  mfgpu_mg_vmult(mfgpu_mg *mg, double *dst, const double *src)
  {
    return guarded([&] {
      need(mg, "mg");
      need(dst, "dst");
      need(src, "src");
      if (!mg->ready)
        throw Error(ERR_STATE, "mfgpu_mg_setup() first");
      if (dst == src)
        throw Error(ERR_ARG, "dst and src must differ");
      mg->h->precond()->vmult(dst, src);
    });
  }

  int
  mfgpu_mg_info(mfgpu_mg *mg, int *n_levels, size_t *n_dofs)
  {
    return guarded([&] {
      need(mg, "mg");
      if (n_levels)
        *n_levels = int(mg->h->lops.size());
      if (n_dofs)
        *n_dofs = mg->h->n_dofs();
    });
  }

  int
  mfgpu_mg_destroy(mfgpu_mg *mg)
  {
    return guarded([&] {
      if (!mg)
        return;
      mfgpu_context *c = mg->ctx;
      c->c->sync();
      delete mg;
      --c->live;
    });
  }

  int
  mfgpu_pcg_solve(mfgpu_operator *A, mfgpu_mg *mg, double jacobi_omega, double *x, const double *b, double tol,
                  int max_iterations, int *iterations, double *residual)
  {
    return guarded([&] {
      Operator *op = fp64_operator(A);
      need(x, "x");
      need(b, "b");
      if (max_iterations < 0)
        throw Error(ERR_ARG, "max_iterations must be >= 0");
      if (!(tol >= 0))
        throw Error(ERR_ARG, "tol must be >= 0");
      OpRef<double>    L(op);
      JacobiOmega      J;
      Precond<double> *P = nullptr;
      if (mg)
        {
          if (mg->ctx != A->ctx)
            throw Error(ERR_ARG, "operator and multigrid belong to different contexts");
          if (!mg->ready)
            throw Error(ERR_STATE, "mfgpu_mg_setup() first");
          if (mg->h->n_dofs() != op->m())
            throw Error(ERR_ARG, "multigrid and operator sizes differ");
          P = mg->h->precond();
        }
      else if (jacobi_omega > 0)
        {
          if (!op->diag_ready)
            throw Error(ERR_STATE, "compute_diagonal() first");
          J.A     = op;
          J.omega = jacobi_omega;
          P       = &J;
        }
      const CGStats st = cg_solve<double>(*op->ctx, L, P, x, b, tol, max_iterations);
      if (iterations)
        *iterations = st.its;
      if (residual)
        *residual = st.res;
      if (!st.converged)
        throw Error(ERR_NOT_CONVERGED, "CG did not reach the tolerance in " + std::to_string(max_iterations) +
                                         " iterations");
    });
  }

  int
  mfgpu_estimate_condition_number(mfgpu_operator *A, const double *b, int n_iterations, double tol,
                                  double *condition_number)
  {
    return guarded([&] {
      Operator *op = fp64_operator(A);
      need(b, "b");
      need(condition_number, "condition_number");
      if (n_iterations < 1)
        throw Error(ERR_ARG, "n_iterations must be >= 1");
      *condition_number = estimate_condition_number(*op, b, n_iterations, tol);
    });
  }

  int
  mfgpu_dof_permutation(const mfgpu_mesh *mesh, int level, size_t n_dofs, const double *support_points,
                        const unsigned *components, double tol, size_t *library_dof)
  {
    return guarded([&] {
      need(library_dof, "library_dof");
      need(support_points, "support_points");
      need(mesh, "mesh");
      const std::vector<size_t> p = build_permutation(*mesh, level, n_dofs, support_points, components, tol);
      std::copy(p.begin(), p.end(), library_dof);
    });
  }

  int
  mfgpu_permutation_create(mfgpu_context *ctx, const mfgpu_mesh *mesh, int level, size_t n_dofs,
                           const double *support_points, const unsigned *components, double tol,
                           mfgpu_permutation **perm)
  {
    return guarded([&] {
      need(ctx, "ctx");
      need(mesh, "mesh");
      need(support_points, "support_points");
      need(perm, "perm");
      const std::vector<size_t> p = build_permutation(*mesh, level, n_dofs, support_points, components, tol);
      auto                     *o = new mfgpu_permutation();
      try
        {
          o->ctx = ctx;
          o->n   = p.size();
          o->idx.alloc(p.size() * sizeof(size_t));
          MF_CK(cudaMemcpyAsync(o->idx.ptr, p.data(), p.size() * sizeof(size_t), cudaMemcpyHostToDevice,
                                ctx->c->stream));
          ctx->c->sync();
          ++ctx->live;
        }
      catch (...)
        {
          delete o;
          throw;
        }
      *perm = o;
    });
  }

  int
  mfgpu_permutation_to_library(mfgpu_permutation *perm, int precision, const void *src, void *dst)
  {
    return guarded([&] { permute(perm, precision, src, dst, 1); });
  }

  int
  mfgpu_permutation_from_library(mfgpu_permutation *perm, int precision, const void *src, void *dst)
  {
    return guarded([&] { permute(perm, precision, src, dst, 0); });
  }

  int
  mfgpu_permutation_destroy(mfgpu_permutation *perm)
  {
    return guarded([&] {
      if (!perm)
        return;
      mfgpu_context *c = perm->ctx;
      c->c->sync();
      delete perm;
      --c->live;
    });
  }
}
