// Solver layer on the device: CG, Chebyshev smoother, multigrid V-cycle,
// and the solid (Newton-Newmark) and heat (backward Euler) drivers.
#pragma once

#include <cmath>

#include "mf_host.h"

namespace mfgpu
{
  // A vector that atomic scatters accumulate into is zeroed for the next
  // application either by the kernel that consumes it or by a memset.  The
  // kernel's stores are slow on lines that the scatter's atomics have just
  // updated (measured on GB300, FP32 vectors, memset + scatter + update:
  // 839,619 entries 31.1 us zeroed in the update against 23.3 us with a
  // memset; 420,000: 21.1 / 17.6; 105,000: 12.1 / 13.1; 14,000: 9.1 / 12.4),
  // so the kernel zeroes vectors up to this size, where it saves the
  // memset's launch, and larger ones take a memset.
  constexpr size_t ZERO_IN_KERNEL_BYTES = size_t(512) << 10;

  // scalar slots of the context used by the solvers
  enum Slot
  {
    S_RR  = 0,
    S_RZ  = 1,
    S_RZN = 2,
    S_PQ  = 3,
    S_TMP = 4
  };

  // typed view of an operator application (any precision)
  template <typename T>
  struct LinOp
  {
    virtual ~LinOp() = default;
    virtual size_t size() const = 0;
    virtual void   vmult(T *dst, const T *src) = 0;
    // dst += A src, where the operator offers it (can_add())
    virtual bool can_add() const { return false; }
    virtual void vmult_add(T *, const T *) {}
  };

  template <typename T>
  struct OpRef : LinOp<T>
  {
    Operator *op;
    explicit OpRef(Operator *o)
      : op(o)
    {}
    size_t size() const override { return op->m(); }
    void   vmult(T *dst, const T *src) override { op->vmult(dst, src); }
    bool   can_add() const override { return true; }
    void   vmult_add(T *dst, const T *src) override { op->vmult_add(dst, src); }
  };

  template <typename T>
  struct Precond
  {
    virtual ~Precond() = default;
    virtual void vmult(T *dst, const T *src) = 0;
    // the inverse diagonal of a point-Jacobi preconditioner (omega = 1), so
    // that CG can fuse it into its vector update; null otherwise
    virtual const T *jacobi_diagonal() const { return nullptr; }
  };

  struct CGStats
  {
    int    its       = 0;
    double res0      = 0;
    double res       = 0;
    bool   converged = false;
    std::vector<double> alpha, beta; // for Lanczos
  };

  // deal.II SolverCG semantics: stops when |r| <= tol (absolute), counts
  // iterations; x is the initial guess
  // (ws: optional workspace kept by the caller across solves, so that the
  // preconditioner sees the same vectors every time; grown to fit)
  template <typename T>
  CGStats cg_solve(Context &c, LinOp<T> &A, Precond<T> *P, T *x, const T *b,
                   double tol, int maxit, bool record = false,
                   bool fixed_iterations = false, DevBuf *ws = nullptr);

  // nb independent systems of n unknowns each, stacked in x and b, solved
  // together: every operator and preconditioner application covers all of
  // them (one launch per stage), the scalars are per system, and each
  // system's iterates are those cg_solve gives it alone; a system stops
  // updating when it has converged.  its[i]: system i's iterations;
  // returns false if a system did not converge in maxit.  nb <= 6 (the
  // context's scalar slots).
  bool cg_solve_batched(Context &c, LinOp<double> &A, Precond<double> *P, double *x, const double *b, int nb,
                        size_t n, const std::vector<double> &tol, int maxit, std::vector<int> &its, DevBuf *ws);

  // CG as used for the Chebyshev eigenvalue estimate: the same iterates as
  // cg_solve(record = true), with the Lanczos coefficients recorded on the
  // device and the convergence test made every `check` iterations (the
  // coefficients of iterations past convergence are discarded), so the
  // host waits once per `check` iterations instead of twice per iteration
  // (ws: optional workspace kept by the caller across calls; grown to fit)
  // host_rec (pinned, >= 3 maxit doubles): deferred mode.  All maxit
  // iterations are enqueued without a host wait and the records are copied
  // to host_rec on the context's stream; after the stream has finished,
  // lanczos_collect turns them into the statistics (iterations past
  // convergence discarded as above).
  template <typename T>
  CGStats cg_lanczos(Context &c, LinOp<T> &A, Precond<T> *P, T *x, const T *b, double tol,
                     int maxit, int check = 8, DevBuf *ws = nullptr, double *host_rec = nullptr);
  CGStats lanczos_collect(const double *host_rec, int maxit, double tol);
  // extreme eigenvalues of the Lanczos tridiagonal matrix of a recorded CG
  // (the CG coefficients alpha, beta): {lambda_min, lambda_max}
  std::pair<double, double> lanczos_extreme_eigenvalues(const CGStats &st);

  template <typename T>
  struct Chebyshev
  {
    Context  *ctx = nullptr;
    Operator *A   = nullptr;
    double    smoothing_range   = 20;
    unsigned  degree            = 5; // 0: choose from the range (coarse solver)
    int       eig_cg_iterations = 30;
    bool      initialized       = false;
    double    theta = 0, delta = 0, lambda_max = 0, lambda_min = 0;
    DevBuf     xold, t1, w0, w1;
    bool       t1_zero = false; // t1 is all zero between applications
    // levels of at most ZERO_IN_KERNEL_BYTES per vector skip the memset
    // before each application: the update kernel leaves the product vector
    // zero (launch-bound there)
    bool small_level() const { return A->m() * sizeof(T) <= ZERO_IN_KERNEL_BYTES; }
    DevBuf     cg_ws;    // work vectors of the eigenvalue-estimate CG, kept across setups
    HostPinned host_rec; // Lanczos records of a deferred estimate
    Context   *est_ctx = nullptr;
    void estimate();
    // a batch of identical problems (a batched heat operator) starts every
    // block from the single problem's vector and stops at the single
    // problem's residual, so its bounds equal the single problem's
    size_t
    start_period() const
    {
      return A->heat_batch ? A->geom.n_nodes : 0;
    }
    double
    estimate_tol() const
    {
      return A->heat_batch ? 1e-10 * std::sqrt(double(A->nc)) : 1e-10;
    }
    // the same estimate enqueued on another context's stream (the operator
    // launches there meanwhile), finished by estimate_end()
    void estimate_begin(Context *ec);
    void estimate_end();
    void set_bounds(const CGStats &st);
    void vmult(T *x, const T *b); // zero initial guess
    void step(T *x, const T *b);  // nonzero initial guess
  };

  template <typename T>
  struct Multigrid : Precond<double>
  {
    Context                               *ctx = nullptr;
    std::vector<Operator *>                ops; // level operators (precision T)
    std::vector<std::unique_ptr<Transfer>> transfers; // [l]: l-1 -> l
    std::vector<Chebyshev<T>>              smoothers;
    std::vector<DevBuf>                    sol, def, tmp;
    // optional FP64 coarse level
    Operator          *coarse64 = nullptr;
    Chebyshev<double>  coarse_cheb64;
    DevBuf             c64_sol, c64_def;
    int                vcycles = 0;
    // CUDA-graph replay of the V-cycle: the first application after setup()
    // runs eagerly, the second is captured into a graph (for its dst/src
    // pair) and later applications with the same pair replay it.  setup()
    // drops the graph (new eigenvalue bounds and diagonals).
    bool               use_graphs = false;
    // contexts (streams, scalar slots, reduction buffers) of the level
    // eigenvalue estimates, which run concurrently in setup()
    std::vector<std::unique_ptr<Context>> aux;
    cudaEvent_t                           setup_ev = nullptr;
    // what the last setup() was made for: the level operators' value
    // states and the smoother parameters (a setup with the same key, e.g.
    // every heat time step, keeps the smoothers and the captured V-cycle)
    size_t setup_key  = 0;
    bool   setup_done = false;
    ~Multigrid();
    cudaGraphExec_t    gexec      = nullptr;
    double            *g_dst      = nullptr;
    const double      *g_src      = nullptr;
    long long          g_launches = 0;
    bool               eager_done = false;
    int                graph_replays = 0;
    void setup(double range, unsigned degree, int eig_its, int coarse_eig_its);
    void level_v_step(int l);
    void vmult(double *dst, const double *src) override;
    void drop_graph();
  private:
    void vcycle(double *dst, const double *src);
  };
} // namespace mfgpu
