// Request server: independent heat and neo-Hookean solves on one GPU.
//
// Requests are queued FIFO.  A request is admitted when its estimated
// device memory fits in the remaining budget (half of the memory fraction
// of the free HBM at server start) and a worker is free.  Every worker owns
// a context with its own CUDA stream, so admitted solves run concurrently
// and their kernels overlap on the device.  A solve keeps its geometry,
// multigrid hierarchy and vectors resident in HBM for its lifetime.
//
// Problems stay resident after they finish: a resident problem is a driver
// together with its own context (CUDA stream, reduction buffers), kept in
// one pool shared by the workers with its own memory cap (the other half of
// the budget; least recently used first out).  A request of a pooled shape
// (mesh, degree, material, solver parameters, time step) checks that
// problem out, resets its loads and state and runs it on its stream: no
// allocation, no operator or transfer construction, and for the heat
// problem no diagonal, no eigenvalue estimate and no V-cycle capture.
// Workers are host threads; concurrency on the device comes from the
// problems' streams.  A free worker prefers, among the first queued
// requests, one whose shape is resident and free.  Latency = completion
// time - submit time.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <string>
#include <thread>

#include "../../include/mfgpu.h"
#include "mf_drivers.h"

namespace mfgpu
{
  using clock_t_ = std::chrono::steady_clock;

  struct ServerJob
  {
    long long            id;
    mfgpu_request        req;
    std::string          caching; // keeps req.solid.caching alive
    std::string          shape;   // pool key
    size_t               bytes = 0;
    clock_t_::time_point t_submit, t_start, t_end;
    mfgpu_request_result res{};
    bool                 done = false;
  };

  // device memory a request will hold (vectors, caches, level hierarchy),
  // from the DoF and quadrature-point counts of its finest level
  size_t
  estimate_request_bytes(const mfgpu_request &r)
  {
    const mfgpu_mesh &mm = r.kind == 0 ? r.heat.mesh : r.solid.mesh;
    const Mesh        m  = to_mesh(mm);
    const LevelGeom   g  = m.level(-1);
    const double      nq = double(g.n_cells) * (m.degree + 1) * (m.degree + 1) * (m.degree + 1);
    const double      ml = 8.0 / 7.0; // geometric level hierarchy
    if (r.kind == 0)
      {
        const double nd = double(g.n_nodes);
        // 5 driver vectors + 2 operators' diagonals + CG (4) + MG (3 per level,
        // FP32) + transfers (2 fine-sized temporaries)
        return size_t(nd * 8 * 13 + nd * ml * 4 * 8 + (64 << 20));
      }
    const double nd = 3.0 * double(g.n_nodes);
    // 7 driver vectors + CG (4) + diag (2) + cache (10 words per qp) + MG
    return size_t(nd * 8 * 15 + nq * 80 * ml + nd * ml * 4 * 10 + (64 << 20));
  }

  // the shape of a request: everything but its loads (heat source or
  // analytic data, solid traction and body force), watchpoint and step
  // count; requests of one shape share operators and multigrid setups
  template <typename V>
  void
  put(std::string &k, const V &v)
  {
    k.append(reinterpret_cast<const char *>(&v), sizeof(V));
  }

  void
  put_mesh(std::string &k, const mfgpu_mesh &m)
  {
    put(k, m.degree), put(k, m.n_q_1d), put(k, m.n_refinements), put(k, m.dim), put(k, m.n_dirichlet);
    for (int d = 0; d < 3; ++d)
      put(k, m.repetitions[d]), put(k, m.lower[d]), put(k, m.upper[d]);
    for (int f = 0; f < 6; ++f)
      put(k, m.boundary_id[f]);
    for (int i = 0; i < m.n_dirichlet && i < 8; ++i)
      put(k, m.dirichlet_id[i]), put(k, m.dirichlet_mask[i]);
  }

  void
  put_solver(std::string &k, const mfgpu_solver_params &s)
  {
    put(k, s.preconditioner), put(k, s.relaxation), put(k, s.tol), put(k, s.max_it_mult);
    put(k, s.cheb_degree), put(k, s.cheb_range), put(k, s.cheb_eig_its), put(k, s.coarse_accurate);
    put(k, s.mg_precision), put(k, s.coarse_fp64), put(k, s.fp64_emulation), put(k, s.cuda_graphs);
    put(k, s.coarse_dense), put(k, s.estimate_condition), put(k, s.cond_cg_iterations);
  }

  std::string
  request_shape(const mfgpu_request &r, const std::string &caching)
  {
    std::string k;
    put(k, r.kind);
    if (r.kind == 0)
      {
        put_mesh(k, r.heat.mesh);
        put(k, r.heat.dt);
        put_solver(k, r.heat.solver);
      }
    else
      {
        const mfgpu_solid_params &p = r.solid;
        put_mesh(k, p.mesh);
        put(k, p.material.mu), put(k, p.material.nu), put(k, p.material.rho), put(k, p.material.formulation);
        k += caching;
        k.push_back('\0');
        put_solver(k, p.solver);
        put(k, p.max_newton), put(k, p.tol_f), put(k, p.tol_f_abs), put(k, p.tol_u), put(k, p.tol_u_abs);
        put(k, p.dt), put(k, p.traction_id);
      }
    return k;
  }

  // a resident problem kept between requests: the driver and the context
  // it runs on (members in this order: the driver goes first)
  struct PoolEntry
  {
    std::unique_ptr<Context>     ctx;
    std::string                  shape;
    std::string                  caching; // the solid driver's caching string
    std::unique_ptr<HeatDriver>  heat;
    std::unique_ptr<SolidDriver> solid;
    size_t                       bytes = 0;
    ~PoolEntry()
    {
      heat.reset();
      solid.reset();
    }
    PoolEntry() = default;
    PoolEntry(PoolEntry &&) = default;
    PoolEntry &operator=(PoolEntry &&) = default;
  };

  struct Server
  {
    int                                   device;
    size_t                                budget = 0, reserved = 0;
    int                                   n_workers;
    std::deque<ServerJob *>               queue;
    std::map<long long, std::unique_ptr<ServerJob>> jobs;
    std::mutex                            mu;
    std::condition_variable               cv_work, cv_done;
    std::vector<std::thread>              workers;
    bool                                  stop = false;
    long long                             next_id = 1;
    int                                   running = 0, max_running = 0;
    size_t                                pool_cap = 0;
    std::list<PoolEntry>                  pool; // resident problems, most recent first
    size_t                                pool_bytes = 0;
    long long                             reused = 0, built = 0;
    int                                   max_batch      = 4; // heat requests solved together, at most
    int                                   max_batch_seen = 1;
    long long                             batched        = 0; // requests that ran in a batch of two or more
    // how far down the queue a free worker looks for a resident shape
    static constexpr int                  LOOKAHEAD = 16;

    Server(int dev, int nw, double fraction)
      : device(dev)
      , n_workers(nw)
    {
      MF_CK(cudaSetDevice(dev));
      size_t free_b = 0, total_b = 0;
      MF_CK(cudaMemGetInfo(&free_b, &total_b));
      const size_t all = size_t(double(free_b) * fraction);
      budget           = all / 2;
      pool_cap         = all / 2;
      for (int i = 0; i < nw; ++i)
        workers.emplace_back([this] { loop(); });
    }

    ~Server()
    {
      {
        std::lock_guard<std::mutex> l(mu);
        stop = true;
      }
      cv_work.notify_all();
      for (auto &t : workers)
        t.join();
      pool.clear();
    }

    bool
    resident(const std::string &shape) const
    {
      for (const PoolEntry &e : pool)
        if (e.shape == shape)
          return true;
      return false;
    }

    void
    loop()
    {
      cudaSetDevice(device);
      for (;;)
        {
          std::vector<ServerJob *> batch;
          {
            std::unique_lock<std::mutex> l(mu);
            auto fits = [&](const ServerJob *j) {
              return reserved + j->bytes <= budget || running == 0; // a job larger than the budget runs alone
            };
            cv_work.wait(l, [&] { return stop || (!queue.empty() && fits(queue.front())); });
            if (stop && queue.empty())
              return;
            if (queue.empty())
              continue;
            auto pick = queue.begin();
            int  look = 0;
            for (auto it = queue.begin(); it != queue.end() && look < LOOKAHEAD; ++it, ++look)
              if (fits(*it) && resident((*it)->shape))
                {
                  pick = it;
                  break;
                }
            ServerJob *job = *pick;
            queue.erase(pick);
            batch.push_back(job);
            reserved += job->bytes;
            // continuous batching: queued heat requests of the same shape and
            // step count join this one, one solve for all of them
            if (job->req.kind == 0 && max_batch > 1)
              {
                look = 0;
                for (auto it = queue.begin(); it != queue.end() && look < LOOKAHEAD && int(batch.size()) < max_batch;
                     ++look)
                  if ((*it)->shape == job->shape && (*it)->req.heat.n_steps == job->req.heat.n_steps &&
                      reserved + (*it)->bytes <= budget)
                    {
                      reserved += (*it)->bytes;
                      batch.push_back(*it);
                      it = queue.erase(it);
                    }
                  else
                    ++it;
              }
            running += int(batch.size());
            max_running = std::max(max_running, running);
            max_batch_seen = std::max(max_batch_seen, int(batch.size()));
            if (batch.size() > 1)
              batched += static_cast<long long>(batch.size());
            for (ServerJob *j : batch)
              j->t_start = clock_t_::now();
          }
          if (batch.size() == 1)
            run(*batch[0]);
          else
            run_batch(batch);
          {
            std::lock_guard<std::mutex> l(mu);
            const auto t_end = clock_t_::now();
            for (ServerJob *job : batch)
              {
                job->t_end = t_end;
                reserved -= job->bytes;
                --running;
                job->done                = true;
                job->res.queue_seconds   = std::chrono::duration<double>(job->t_start - job->t_submit).count();
                job->res.run_seconds     = std::chrono::duration<double>(job->t_end - job->t_start).count();
                job->res.latency_seconds = std::chrono::duration<double>(job->t_end - job->t_submit).count();
              }
          }
          cv_done.notify_all();
          cv_work.notify_all();
        }
    }

    // check out the resident problem of a pool key (null entry if none)
    PoolEntry
    checkout(const std::string &key)
    {
      PoolEntry                   e;
      std::lock_guard<std::mutex> l(mu);
      for (auto it = pool.begin(); it != pool.end(); ++it)
        if (it->shape == key)
          {
            e = std::move(*it);
            pool.erase(it);
            pool_bytes -= e.bytes;
            break;
          }
      return e;
    }

    // return a problem to the pool, within its cap; evicted problems are
    // released outside the lock
    void
    checkin(PoolEntry &&e, bool reuse)
    {
      std::list<PoolEntry> evicted;
      std::lock_guard<std::mutex> l(mu);
      (reuse ? reused : built) += 1;
      if (e.bytes <= pool_cap)
        {
          pool_bytes += e.bytes;
          pool.push_front(std::move(e));
          while (pool_bytes > pool_cap && pool.size() > 1)
            {
              pool_bytes -= pool.back().bytes;
              evicted.splice(evicted.begin(), pool, std::prev(pool.end()));
            }
        }
    }

    // heat requests of one shape solved together: one batched driver (one
    // operator, one V-cycle, one CG for all), resident under its own key
    void
    run_batch(std::vector<ServerJob *> &batch)
    {
      const int         nb  = int(batch.size());
      const std::string key = batch[0]->shape + "|batch" + std::to_string(nb);
      PoolEntry         e   = checkout(key);
      const bool        reuse = bool(e.heat);
      try
        {
          std::vector<mfgpu_heat_params> ps;
          for (ServerJob *j : batch)
            ps.push_back(j->req.heat);
          if (!reuse)
            {
              e.ctx.reset(new Context(device));
              e.heat.reset(new HeatDriver(e.ctx.get(), ps[0], nb));
            }
          HeatDriver &d = *e.heat;
          d.reset_batch(ps);
          d.start();
          std::vector<int> its(size_t(nb), 0);
          for (int s = 0; s < ps[0].n_steps; ++s)
            {
              const std::vector<int> st = d.step_batch();
              for (int b = 0; b < nb; ++b)
                its[b] += st[b];
            }
          const size_t n0 = d.op->geom.n_nodes;
          for (int b = 0; b < nb; ++b)
            {
              mfgpu_request_result &r = batch[b]->res;
              const double         *x = d.sol.as<double>() + b * n0;
              r.cg_iterations         = its[b];
              r.solution_norm         = std::sqrt(vec_dot<double>(*e.ctx, n0, x, x));
              r.n_dofs                = double(n0);
              r.status                = MFGPU_OK;
            }
          e.ctx->sync();
          e.shape = key;
          e.bytes = 0;
          for (ServerJob *j : batch)
            e.bytes += j->bytes;
          checkin(std::move(e), reuse);
        }
      catch (const std::exception &x)
        {
          const Error *err = dynamic_cast<const Error *>(&x);
          for (ServerJob *j : batch)
            {
              j->res.status = err ? err->code : MFGPU_ERR_ARG;
              std::strncpy(j->res.message, x.what(), sizeof(j->res.message) - 1);
            }
        }
    }

    void
    run(ServerJob &job)
    {
      mfgpu_request_result &r = job.res;
      // check out the resident problem of this shape, or make a new one
      PoolEntry  e     = checkout(job.shape);
      const bool reuse = e.heat || e.solid;
      try
        {
          if (!reuse)
            e.ctx.reset(new Context(device));
          Context &ctx = *e.ctx;
          if (job.req.kind == 0)
            {
              if (reuse)
                e.heat->reset(job.req.heat);
              else
                e.heat.reset(new HeatDriver(&ctx, job.req.heat));
              HeatDriver       &d = *e.heat;
              mfgpu_heat_result hr;
              d.run(hr);
              int its = 0;
              for (int s = 0; s < hr.n_steps; ++s)
                its += hr.cg_its[s];
              r.cg_iterations = its;
              const size_t n  = d.op->m();
              r.solution_norm = std::sqrt(vec_dot<double>(ctx, n, d.sol.as<double>(), d.sol.as<double>()));
              r.n_dofs        = double(n);
            }
          else
            {
              mfgpu_solid_params p = job.req.solid;
              if (reuse)
                e.solid->reset(p);
              else
                {
                  e.caching = job.caching;
                  p.caching = e.caching.c_str();
                  e.solid.reset(new SolidDriver(&ctx, p));
                }
              SolidDriver       &d = *e.solid;
              mfgpu_solid_result sr;
              d.run(sr);
              r.cg_iterations     = int(sr.total_cg);
              r.newton_iterations = 0;
              for (int s = 0; s < sr.n_steps; ++s)
                r.newton_iterations += sr.newton_its[s];
              for (int k = 0; k < 3; ++k)
                r.watch[k] = sr.watch_disp[sr.n_steps - 1][k];
              const size_t n  = d.fine->m();
              r.solution_norm = std::sqrt(vec_dot<double>(ctx, n, d.u.as<double>(), d.u.as<double>()));
              r.n_dofs        = double(n);
            }
          r.status = MFGPU_OK;
          ctx.sync();
          // keep the problem resident
          e.shape = job.shape;
          e.bytes = job.bytes;
          checkin(std::move(e), reuse);
        }
      catch (const Error &e2)
        {
          r.status = e2.code;
          std::strncpy(r.message, e2.what(), sizeof(r.message) - 1);
        }
      catch (const std::exception &e2)
        {
          r.status = MFGPU_ERR_ARG;
          std::strncpy(r.message, e2.what(), sizeof(r.message) - 1);
        }
    }

    long long
    submit(const mfgpu_request &req)
    {
      std::unique_ptr<ServerJob> j(new ServerJob());
      j->req = req;
      if (req.kind == 1)
        {
          j->caching     = req.solid.caching ? req.solid.caching : "scalar_referential";
          j->req.solid.caching = nullptr;
        }
      else if (req.kind != 0)
        throw Error(ERR_ARG, "request kind must be 0 (heat) or 1 (solid)");
      j->bytes    = estimate_request_bytes(req);
      j->shape    = request_shape(req, j->caching);
      j->t_submit = clock_t_::now();
      std::lock_guard<std::mutex> l(mu);
      const long long id = next_id++;
      j->id              = id;
      queue.push_back(j.get());
      jobs[id] = std::move(j);
      cv_work.notify_one();
      return id;
    }

    mfgpu_request_result
    wait(long long id, bool remove)
    {
      std::unique_lock<std::mutex> l(mu);
      auto                         it = jobs.find(id);
      if (it == jobs.end())
        throw Error(ERR_ARG, "unknown request id");
      ServerJob *j = it->second.get();
      cv_done.wait(l, [&] { return j->done; });
      mfgpu_request_result r = j->res;
      if (remove)
        jobs.erase(it);
      return r;
    }
  };
} // namespace mfgpu

using namespace mfgpu;

struct mfgpu_server
{
  std::unique_ptr<Server> s;
};

extern "C"
{
  int
  mfgpu_server_create(int device, int max_concurrent, double memory_fraction, mfgpu_server **server)
  {
    try
      {
        if (!server || max_concurrent < 1 || max_concurrent > 64 || !(memory_fraction > 0) ||
            memory_fraction > 1)
          throw Error(ERR_ARG, "server: invalid arguments");
        auto *o = new mfgpu_server();
        try
          {
            o->s.reset(new Server(device, max_concurrent, memory_fraction));
          }
        catch (...)
          {
            delete o;
            throw;
          }
        *server = o;
        return MFGPU_OK;
      }
    catch (const Error &e)
      {
        set_last_error(e.what());
        return e.code;
      }
  }

  int
  mfgpu_server_submit(mfgpu_server *server, const mfgpu_request *request, long long *id)
  {
    try
      {
        if (!server || !request || !id)
          throw Error(ERR_ARG, "server_submit: null argument");
        *id = server->s->submit(*request);
        return MFGPU_OK;
      }
    catch (const Error &e)
      {
        set_last_error(e.what());
        return e.code;
      }
  }

  int
  mfgpu_server_wait(mfgpu_server *server, long long id, mfgpu_request_result *result)
  {
    try
      {
        if (!server || !result)
          throw Error(ERR_ARG, "server_wait: null argument");
        *result = server->s->wait(id, true);
        return MFGPU_OK;
      }
    catch (const Error &e)
      {
        set_last_error(e.what());
        return e.code;
      }
  }

  int
  mfgpu_server_stats(mfgpu_server *server, int *max_running, size_t *budget_bytes)
  {
    if (!server)
      {
        set_last_error("server_stats: null argument");
        return MFGPU_ERR_ARG;
      }
    std::lock_guard<std::mutex> l(server->s->mu);
    if (max_running)
      *max_running = server->s->max_running;
    if (budget_bytes)
      *budget_bytes = server->s->budget;
    return MFGPU_OK;
  }

  int
  mfgpu_server_pool_stats(mfgpu_server *server, long long *reused, long long *built)
  {
    if (!server)
      {
        set_last_error("server_pool_stats: null argument");
        return MFGPU_ERR_ARG;
      }
    std::lock_guard<std::mutex> l(server->s->mu);
    if (reused)
      *reused = server->s->reused;
    if (built)
      *built = server->s->built;
    return MFGPU_OK;
  }

  int
  mfgpu_server_set_max_batch(mfgpu_server *server, int max_batch)
  {
    if (!server || max_batch < 1 || max_batch > 6)
      {
        set_last_error("server_set_max_batch: null server or max_batch outside 1..6");
        return MFGPU_ERR_ARG;
      }
    std::lock_guard<std::mutex> l(server->s->mu);
    server->s->max_batch = max_batch;
    return MFGPU_OK;
  }

  int
  mfgpu_server_batch_stats(mfgpu_server *server, long long *batched_requests, int *largest_batch)
  {
    if (!server)
      {
        set_last_error("server_batch_stats: null argument");
        return MFGPU_ERR_ARG;
      }
    std::lock_guard<std::mutex> l(server->s->mu);
    if (batched_requests)
      *batched_requests = server->s->batched;
    if (largest_batch)
      *largest_batch = server->s->max_batch_seen;
    return MFGPU_OK;
  }

  int
  mfgpu_server_destroy(mfgpu_server *server)
  {
    delete server;
    return MFGPU_OK;
  }
}
