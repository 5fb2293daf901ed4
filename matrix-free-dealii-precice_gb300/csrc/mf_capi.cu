// extern "C" entry points of libmfgpu.so (declared in include/mfgpu.h).
// Every entry point converts exceptions into a status code and a
// per-thread error message.
#include <chrono>

#include "mf_capi.h"

static thread_local std::string g_last_error;

void
mfgpu::set_last_error(const char *msg)
{
  g_last_error = msg ? msg : "";
}

extern "C"
{
  const char *
  mfgpu_last_error(void)
  {
    return g_last_error.c_str();
  }

  int
  mfgpu_version(void)
  {
    return 100;
  }

  long long
  mfgpu_launch_count(void)
  {
    return launch_count();
  }

  int
  mfgpu_context_create(int device, mfgpu_context **ctx)
  {
    return guarded([&] {
      need(ctx, "ctx");
      auto *c = new mfgpu_context();
      try
        {
          c->c.reset(new Context(device));
        }
      catch (...)
        {
          delete c;
          throw;
        }
      *ctx = c;
    });
  }

  int
  mfgpu_context_destroy(mfgpu_context *ctx)
  {
    return guarded([&] {
      if (ctx && ctx->live.load() > 0)
        throw Error(ERR_STATE, "context still has " + std::to_string(ctx->live.load()) +
                                 " operators/drivers: destroy them first");
      delete ctx;
    });
  }

  int
  mfgpu_context_synchronize(mfgpu_context *ctx)
  {
    return guarded([&] {
      need(ctx, "ctx");
      ctx->c->sync();
    });
  }

  int
  mfgpu_context_stream(mfgpu_context *ctx, void **stream)
  {
    return guarded([&] {
      need(ctx, "ctx");
      need(stream, "stream");
      *stream = (void *)ctx->c->stream;
    });
  }

  int
  mfgpu_copy(mfgpu_context *ctx, void *dst, const void *src, size_t bytes)
  {
    return guarded([&] {
      need(ctx, "ctx");
      if (bytes == 0)
        return;
      need(dst, "dst");
      need(src, "src");
      MF_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->c->stream));
      ctx->c->sync();
    });
  }

  int
  mfgpu_mesh_n_nodes(const mfgpu_mesh *mesh, int level, size_t *n_nodes)
  {
    return guarded([&] {
      need(mesh, "mesh");
      need(n_nodes, "n_nodes");
      *n_nodes = to_mesh(*mesh).level(level).n_nodes;
    });
  }

  int
  mfgpu_heat_operator_create(mfgpu_context *ctx, const mfgpu_mesh *mesh, int level,
                             int precision, int constrained, mfgpu_operator **op)
  {
    return guarded([&] {
      need(ctx, "ctx");
      need(mesh, "mesh");
      need(op, "op");
      auto *o = new mfgpu_operator();
      try
        {
          o->op  = make_heat(ctx->c.get(), to_mesh(*mesh), level, precision, constrained != 0);
          o->ctx = ctx;
          ++ctx->live;
        }
      catch (...)
        {
          delete o;
          throw;
        }
      *op = o;
    });
  }

  static HeatOperator *
  as_heat(mfgpu_operator *op)
  {
    need(op, "op");
    auto *h = dynamic_cast<HeatOperator *>(op->op.get());
    if (!h)
      throw Error(ERR_ARG, "not a heat operator");
    return h;
  }

  static NHOperator *
  as_nh(mfgpu_operator *op)
  {
    need(op, "op");
    auto *h = dynamic_cast<NHOperator *>(op->op.get());
    if (!h)
      throw Error(ERR_ARG, "not a neo-Hookean operator");
    return h;
  }

  int
  mfgpu_heat_operator_set_delta_t(mfgpu_operator *op, double delta_t)
  {
    return guarded([&] {
      if (!(delta_t > 0))
        throw Error(ERR_ARG, "delta_t must be positive");
      as_heat(op)->delta_t = delta_t;
    });
  }

  int
  mfgpu_heat_operator_evaluate_coefficient(mfgpu_operator *op, double coefficient)
  {
    return guarded([&] { as_heat(op)->coefficient = coefficient; });
  }

  int
  mfgpu_nh_operator_create(mfgpu_context *ctx, const mfgpu_mesh *mesh, int level,
                           int precision, const char *caching, mfgpu_operator **op)
  {
    return guarded([&] {
      need(ctx, "ctx");
      need(mesh, "mesh");
      need(op, "op");
      const int var = parse_caching(caching);
      auto     *o   = new mfgpu_operator();
      try
        {
          o->op  = make_nh(ctx->c.get(), to_mesh(*mesh), level, precision, var);
          o->ctx = ctx;
          ++ctx->live;
        }
      catch (...)
        {
          delete o;
          throw;
        }
      *op = o;
    });
  }

  int
  mfgpu_nh_operator_set_material(mfgpu_operator *op, const mfgpu_material *material,
                                 const mfgpu_material *inclusion)
  {
    return guarded([&] {
      need(material, "material");
      if (inclusion && inclusion->formulation != material->formulation)
        throw Error(ERR_UNSUPPORTED, "the inclusion material must use the formulation of the material");
      if (inclusion && !(inclusion->mu > 0 && inclusion->nu > -1 && inclusion->nu < 0.5))
        throw Error(ERR_ARG, "inclusion material: mu > 0 and -1 < nu < 0.5 required");
      NHOperator *h    = as_nh(op);
      h->mat           = make_material(material->mu, material->nu, material->rho, material->alpha_1);
      h->formulation   = material->formulation;
      if (h->formulation != 0 && h->formulation != 1)
        throw Error(ERR_ARG, "Unknown material formulation");
      h->have_material = true;
      h->cached        = false;
    });
  }

  int
  mfgpu_nh_operator_set_cell_material_ids(mfgpu_operator *op, const unsigned char *ids, size_t n_cells)
  {
    return guarded([&] {
      NHOperator *h = as_nh(op);
      need(ids, "ids");
      if (n_cells != h->geom.n_cells)
        throw Error(ERR_ARG, "n_cells must be the level's cell count (" + std::to_string(h->geom.n_cells) + ")");
      for (size_t c = 0; c < n_cells; ++c)
        if (ids[c] != 0)
          throw Error(ERR_UNSUPPORTED, "cell " + std::to_string(c) +
                                         " carries a nonzero material id (the inclusion material): the device "
                                         "cell kernels apply one material to all cells");
    });
  }

  int
  mfgpu_nh_operator_initialize(mfgpu_operator *op, const void *displacement)
  {
    return guarded([&] {
      need(displacement, "displacement");
      NHOperator *h = as_nh(op);
      h->u          = displacement;
      h->cached     = false;
    });
  }

  int
  mfgpu_nh_operator_cache(mfgpu_operator *op)
  {
    return guarded([&] { as_nh(op)->do_cache(); });
  }

  int
  mfgpu_operator_set_fp64_emulation(mfgpu_operator *op, int enable)
  {
    return guarded([&] {
      need(op, "op");
      Operator *o = op->op.get();
      if (enable && o->precision != 64)
        throw Error(ERR_UNSUPPORTED, "double-float arithmetic applies to FP64 operators");
      if (enable)
        {
          auto *nh = dynamic_cast<NHOperator *>(o);
          if (nh && (nh->variant != V_QP10 || nh->formulation != 1))
            throw Error(ERR_UNSUPPORTED,
                        "double-float arithmetic supports heat and referential_qp (formulation 1)");
          if (nh)
            nh->cached = false;
        }
      o->arith = enable ? 1 : 0;
    });
  }

  int
  mfgpu_operator_vmult(mfgpu_operator *op, void *dst, const void *src)
  {
    return guarded([&] {
      need(op, "op");
      need(dst, "dst");
      need(src, "src");
      op->op->vmult(dst, src);
    });
  }

  int
  mfgpu_operator_vmult_add(mfgpu_operator *op, void *dst, const void *src)
  {
    return guarded([&] {
      need(op, "op");
      need(dst, "dst");
      need(src, "src");
      op->op->vmult_add(dst, src);
    });
  }

  int
  mfgpu_operator_Tvmult(mfgpu_operator *op, void *dst, const void *src)
  {
    return mfgpu_operator_vmult(op, dst, src);
  }

  int
  mfgpu_operator_Tvmult_add(mfgpu_operator *op, void *dst, const void *src)
  {
    return mfgpu_operator_vmult_add(op, dst, src);
  }

  int
  mfgpu_operator_vmult_host(mfgpu_operator *op, void *dst_host, const void *src_host)
  {
    return guarded([&] {
      need(op, "op");
      need(dst_host, "dst");
      need(src_host, "src");
      Operator    *o     = op->op.get();
      const size_t bytes = o->m() * o->elem_size();
      if (op->hsrc.bytes != bytes)
        {
          op->hsrc.alloc(bytes);
          op->hdst.alloc(bytes);
        }
      o->vmult_host(dst_host, src_host, op->hdst.ptr, op->hsrc.ptr, op->pipe);
    });
  }

  int
  mfgpu_operator_set_scatter(mfgpu_operator *op, int mode)
  {
    return guarded([&] {
      need(op, "op");
      if (mode != 0 && mode != 1)
        throw Error(ERR_ARG, "scatter mode must be 0 (atomic) or 1 (coloured)");
      op->op->scatter = mode;
    });
  }

  int
  mfgpu_operator_set_cell_kernel(mfgpu_operator *op, int mode)
  {
    return guarded([&] {
      need(op, "op");
      if (mode < 0 || mode > 5)
        throw Error(ERR_ARG, "cell kernel must be 0 (by grid size), 1 (line), 2 (point), 3 (tensor cores), "
                             "4 (tensor product) or 5 (tensor product, TMA-staged bricks)");
      if (mode >= 4)
        {
          Operator *o = op->op.get();
          if (!dynamic_cast<HeatOperator *>(o) || o->geom.dim != 3 || !heat_tp_supported(o->basis.N, o->precision))
            throw Error(ERR_UNSUPPORTED, "the tensor-product cell kernel applies to three-dimensional heat operators");
        }
      if (mode == 3)
        {
          Operator *o = op->op.get();
          if (!dynamic_cast<HeatOperator *>(o) || o->precision != 32 || o->geom.dim != 3 ||
              !heat_em_supported(o->basis.N))
            throw Error(ERR_UNSUPPORTED,
                        "the tensor-core cell kernel applies to three-dimensional FP32 heat operators of degree 1..5");
        }
      op->op->cell_kernel = mode;
    });
  }

  int
  mfgpu_operator_set_dense(mfgpu_operator *op, int enable)
  {
    return guarded([&] {
      need(op, "op");
      if (enable)
        op->op->assemble_dense();
      else
        op->op->drop_dense();
    });
  }

  int
  mfgpu_operator_set_host_chunks(mfgpu_operator *op, int n_chunks)
  {
    return guarded([&] {
      need(op, "op");
      if (n_chunks < 0 || n_chunks > HostPipe::MAXC)
        throw Error(ERR_ARG, "n_chunks must be in [0, 8]");
      op->pipe.chunks = n_chunks;
    });
  }

  int
  mfgpu_operator_compute_diagonal(mfgpu_operator *op)
  {
    return guarded([&] {
      need(op, "op");
      op->op->compute_diagonal();
    });
  }

  int
  mfgpu_operator_get_matrix_diagonal_inverse(mfgpu_operator *op, const void **inv_diag)
  {
    return guarded([&] {
      need(op, "op");
      need(inv_diag, "inv_diag");
      if (!op->op->diag_ready)
        throw Error(ERR_STATE, "compute_diagonal() first");
      *inv_diag = op->op->inv_diag.ptr;
    });
  }

  int
  mfgpu_operator_el(mfgpu_operator *op, size_t row, size_t col, double *value)
  {
    return guarded([&] {
      need(op, "op");
      need(value, "value");
      if (row != col)
        throw Error(ERR_UNSUPPORTED, "el(): only diagonal entries are available");
      Operator *o = op->op.get();
      if (!o->diag_ready)
        throw Error(ERR_STATE, "compute_diagonal() first");
      if (row >= o->m())
        throw Error(ERR_ARG, "row out of range");
      if (o->precision == 32)
        {
          float v;
          MF_CK(cudaMemcpyAsync(&v, o->diag.as<float>() + row, 4, cudaMemcpyDeviceToHost, o->ctx->stream));
          o->ctx->sync();
          *value = v;
        }
      else
        {
          MF_CK(cudaMemcpyAsync(value, o->diag.as<double>() + row, 8, cudaMemcpyDeviceToHost, o->ctx->stream));
          o->ctx->sync();
        }
    });
  }

  int
  mfgpu_operator_precondition_jacobi(mfgpu_operator *op, void *dst, const void *src, double omega)
  {
    return guarded([&] {
      need(op, "op");
      need(dst, "dst");
      need(src, "src");
      Operator *o = op->op.get();
      if (!o->diag_ready)
        throw Error(ERR_STATE, "compute_diagonal() first");
      if (o->precision == 32)
        vec_scale<float>(*o->ctx, o->m(), float(omega), o->inv_diag.as<float>(), (const float *)src, (float *)dst);
      else
        vec_scale<double>(*o->ctx, o->m(), omega, o->inv_diag.as<double>(), (const double *)src, (double *)dst);
    });
  }

  int
  mfgpu_operator_m(mfgpu_operator *op, size_t *m)
  {
    return guarded([&] {
      need(op, "op");
      need(m, "m");
      *m = op->op->m();
    });
  }

  int
  mfgpu_operator_memory_consumption(mfgpu_operator *op, size_t *bytes)
  {
    return guarded([&] {
      need(op, "op");
      need(bytes, "bytes");
      *bytes = op->op->memory_consumption();
    });
  }

  int
  mfgpu_operator_clear(mfgpu_operator *op)
  {
    return guarded([&] {
      need(op, "op");
      op->op->clear();
    });
  }

  int
  mfgpu_operator_destroy(mfgpu_operator *op)
  {
    return guarded([&] {
      if (op && op->op)
        op->op->ctx->sync();
      if (op && op->ctx)
        --op->ctx->live;
      delete op;
    });
  }

  static int
  transfer_call(mfgpu_context *ctx, const mfgpu_mesh *mesh, int coarse_level, int nc,
                int precision, const void *in, void *out, int mode)
  {
    return guarded([&] {
      need(ctx, "ctx");
      need(mesh, "mesh");
      need(in, "input");
      need(out, "output");
      const Mesh m = to_mesh(*mesh);
      if (coarse_level < 0 || coarse_level + 1 > m.n_ref)
        throw Error(ERR_ARG, "coarse_level must be in [0, n_refinements)");
      if (precision != 32 && precision != 64)
        throw Error(ERR_ARG, "precision must be 32 or 64");
      HostBasis b;
      make_host_basis(m.degree, b);
      Transfer t(ctx->c.get(), b, m.level(coarse_level), m.level(coarse_level + 1), nc, precision);
      if (mode == 0)
        t.prolongate(out, in);
      else if (mode == 1)
        t.restrict_add(out, in);
      else
        t.interpolate(out, in);
      ctx->c->sync();
    });
  }

  int
  mfgpu_transfer_prolongate(mfgpu_context *ctx, const mfgpu_mesh *mesh, int coarse_level,
                            int n_components, int precision, const void *coarse, void *fine)
  {
    return transfer_call(ctx, mesh, coarse_level, n_components, precision, coarse, fine, 0);
  }

  int
  mfgpu_transfer_restrict_add(mfgpu_context *ctx, const mfgpu_mesh *mesh, int coarse_level,
                              int n_components, int precision, void *coarse, const void *fine)
  {
    return transfer_call(ctx, mesh, coarse_level, n_components, precision, fine, coarse, 1);
  }

  int
  mfgpu_transfer_interpolate(mfgpu_context *ctx, const mfgpu_mesh *mesh, int coarse_level,
                             int n_components, int precision, void *coarse, const void *fine)
  {
    return transfer_call(ctx, mesh, coarse_level, n_components, precision, fine, coarse, 2);
  }

  int
  mfgpu_solid_create(mfgpu_context *ctx, const mfgpu_solid_params *p, mfgpu_solid **s)
  {
    return guarded([&] {
      need(ctx, "ctx");
      need(p, "params");
      need(s, "solid");
      auto *o = new mfgpu_solid();
      try
        {
          o->d.reset(new SolidDriver(ctx->c.get(), *p));
        }
      catch (...)
        {
          delete o;
          throw;
        }
      o->ctx = ctx;
      ++ctx->live;
      *s = o;
    });
  }

  int
  mfgpu_solid_run(mfgpu_solid *s, mfgpu_solid_result *r)
  {
    return guarded([&] {
      need(s, "solid");
      need(r, "result");
      s->d->run(*r);
    });
  }

  int
  mfgpu_solid_step(mfgpu_solid *s, int *newton_iterations, long *cg_iterations, int *linear_solves,
                   double *watch_displacement)
  {
    return guarded([&] {
      need(s, "solid");
      int    nits = 0, solves = 0;
      long   cg   = 0;
      double w[3] = {0, 0, 0};
      s->d->step(nits, cg, solves, w);
      if (newton_iterations)
        *newton_iterations = nits;
      if (cg_iterations)
        *cg_iterations = cg;
      if (linear_solves)
        *linear_solves = solves;
      if (watch_displacement)
        for (int d = 0; d < 3; ++d)
          watch_displacement[d] = w[d];
    });
  }

  int
  mfgpu_solid_residual(mfgpu_solid *s, const double *u, const double *acceleration,
                       double *rhs, double *l2_norm)
  {
    return guarded([&] {
      need(s, "solid");
      need(u, "u");
      need(acceleration, "acceleration");
      need(rhs, "rhs");
      const double nrm = s->d->residual_at(u, acceleration, rhs);
      if (l2_norm)
        *l2_norm = nrm;
    });
  }

  int
  mfgpu_solid_set_timing(mfgpu_solid *s, int enable)
  {
    return guarded([&] {
      need(s, "solid");
      s->d->timer.reset();
      s->d->timer.enabled = enable != 0;
    });
  }

  int
  mfgpu_solid_timing_summary(mfgpu_solid *s, char *buf, size_t len)
  {
    return guarded([&] {
      need(s, "solid");
      need(buf, "buf");
      copy_text(s->d->timer.summary(), buf, len);
    });
  }

  int
  mfgpu_solid_displacement(mfgpu_solid *s, const double **u)
  {
    return guarded([&] {
      need(s, "solid");
      need(u, "u");
      *u = s->d->u.as<double>();
    });
  }

  int
  mfgpu_solid_linear_solve(mfgpu_solid *s, const double *u, const double *rhs, double *du,
                           int *iterations, double *seconds)
  {
    return guarded([&] {
      need(s, "solid");
      need(u, "u");
      need(rhs, "rhs");
      need(du, "du");
      SolidDriver *d = s->d.get();
      d->update_operators(u);
      const size_t n  = d->fine->m();
      const double nb = std::sqrt(vec_dot<double>(*d->ctx, n, rhs, rhs));
      d->ctx->sync();
      auto      t0  = std::chrono::steady_clock::now();
      const int its = d->solve_linear(rhs, du, d->P.solver.tol * nb);
      d->ctx->sync();
      if (iterations)
        *iterations = its;
      if (seconds)
        *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    });
  }

  int
  mfgpu_solid_convergence_table(mfgpu_solid *s, char *buf, size_t len)
  {
    return guarded([&] {
      need(s, "solid");
      need(buf, "buf");
      copy_text(s->d->convergence_table(), buf, len);
    });
  }

  int
  mfgpu_solid_destroy(mfgpu_solid *s)
  {
    return guarded([&] {
      if (s && s->ctx)
        --s->ctx->live;
      delete s;
    });
  }

  int
  mfgpu_heat_create(mfgpu_context *ctx, const mfgpu_heat_params *p, mfgpu_heat **h)
  {
    return guarded([&] {
      need(ctx, "ctx");
      need(p, "params");
      need(h, "heat");
      auto *o = new mfgpu_heat();
      try
        {
          o->d.reset(new HeatDriver(ctx->c.get(), *p));
        }
      catch (...)
        {
          delete o;
          throw;
        }
      o->ctx = ctx;
      ++ctx->live;
      *h = o;
    });
  }

  int
  mfgpu_heat_run(mfgpu_heat *h, mfgpu_heat_result *r)
  {
    return guarded([&] {
      need(h, "heat");
      need(r, "result");
      h->d->run(*r);
    });
  }

  int
  mfgpu_heat_step(mfgpu_heat *h, int *cg_iterations)
  {
    return guarded([&] {
      need(h, "heat");
      const int its = h->d->step();
      h->d->ctx->sync();
      if (cg_iterations)
        *cg_iterations = its;
    });
  }

  int
  mfgpu_heat_solution(mfgpu_heat *h, const double **u)
  {
    return guarded([&] {
      need(h, "heat");
      need(u, "u");
      *u = h->d->sol.as<double>();
    });
  }

  int
  mfgpu_heat_set_timing(mfgpu_heat *h, int enable)
  {
    return guarded([&] {
      need(h, "heat");
      h->d->timer.reset();
      h->d->timer.enabled = enable != 0;
    });
  }

  int
  mfgpu_heat_timing_summary(mfgpu_heat *h, char *buf, size_t len)
  {
    return guarded([&] {
      need(h, "heat");
      need(buf, "buf");
      copy_text(h->d->timer.summary(), buf, len);
    });
  }

  int
  mfgpu_heat_destroy(mfgpu_heat *h)
  {
    return guarded([&] {
      if (h && h->ctx)
        --h->ctx->live;
      delete h;
    });
  }
}
