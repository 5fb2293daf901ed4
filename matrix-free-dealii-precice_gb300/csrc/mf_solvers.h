// Solver layer on the device: CG, Chebyshev smoother, multigrid V-cycle,
// and the solid (Newton-Newmark) and heat (backward Euler) drivers.
#pragma once

#include "mf_host.h"

namespace mfgpu
{
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
  };

  template <typename T>
  struct Precond
  {
    virtual ~Precond() = default;
    virtual void vmult(T *dst, const T *src) = 0;
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
  template <typename T>
  CGStats cg_solve(Context &c, LinOp<T> &A, Precond<T> *P, T *x, const T *b,
                   double tol, int maxit, bool record = false,
                   bool fixed_iterations = false);

  // CG as used for the Chebyshev eigenvalue estimate: the same iterates as
  // cg_solve(record = true), with the Lanczos coefficients recorded on the
  // device and the convergence test made every `check` iterations (the
  // coefficients of iterations past convergence are discarded), so the
  // host waits once per `check` iterations instead of twice per iteration
  template <typename T>
  CGStats cg_lanczos(Context &c, LinOp<T> &A, Precond<T> *P, T *x, const T *b, double tol,
                     int maxit, int check = 8);

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
    DevBuf    xold, t1, w0, w1;
    void estimate();
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
    cudaGraphExec_t    gexec      = nullptr;
    double            *g_dst      = nullptr;
    const double      *g_src      = nullptr;
    long long          g_launches = 0;
    bool               eager_done = false;
    int                graph_replays = 0;
    ~Multigrid() { drop_graph(); }
    void setup(double range, unsigned degree, int eig_its, int coarse_eig_its);
    void level_v_step(int l);
    void vmult(double *dst, const double *src) override;
    void drop_graph();
  private:
    void vcycle(double *dst, const double *src);
  };
} // namespace mfgpu
