// Solid and heat drivers (device-resident Newton-Newmark / backward Euler).
#pragma once

#include "../../include/mfgpu.h"
#include "mf_solvers.h"

namespace mfgpu
{
  Mesh to_mesh(const mfgpu_mesh &m);

  // SolverCG::connect_condition_number_slot under IterationNumberControl
  // (mf_elasticity.h:1998-2013): up to n_its unpreconditioned CG iterations
  // on A y = b from y = 0 (stopping early at |r| <= tol), then the ratio of
  // the extreme eigenvalues of the Lanczos tridiagonal matrix (FP64 A)
  double estimate_condition_number(Operator &A, const double *b, int n_its, double tol);

  // The geometric-multigrid preconditioner over the level hierarchy of a
  // box mesh: level operators (FP32 or FP64), an optional FP64 coarse
  // operator, the transfers, the Chebyshev smoothers and the V-cycle.
  // Restates Solid::setup_gmg with the level part of update_matrix_free
  // (mf_elasticity.h:1142-1279, 1291-1353) and LaplaceProblem::setup_gmg /
  // solve_gmg_preconditioner (heat_transfer.h:515-573, 759-812).  Used by
  // the drivers and by the mfgpu_mg object of the C-ABI.
  struct GMGHierarchy
  {
    Context                               *ctx = nullptr;
    Mesh                                   mesh;
    int                                    L = 0;
    int                                    kind = 0; // 0 heat (LaplaceOperator), 1 neo-Hookean
    int                                    nc = 1;
    int                                    batch = 1;
    int                                    lprec = 32;
    mfgpu_solver_params                    S{};
    HostBasis                              basis;
    std::vector<std::unique_ptr<Operator>> lops;
    std::unique_ptr<Operator>              coarse64;
    std::unique_ptr<Multigrid<float>>      mgf;
    std::unique_ptr<Multigrid<double>>     mgd;
    std::vector<DevBuf>                    u_levels;
    DevBuf                                 u0_64;
    // smoother parameters: range, degree, eigenvalue-estimate iterations on
    // levels > 0; coarse_its < 0 means m() of level 0
    double   range      = 20;
    unsigned degree     = 5;
    int      eig_its    = 30;
    int      coarse_its = -1;
    size_t   diag_key   = 0; // value states the level diagonals were made for
    // heat levels: M + delta_t K
    // batch > 1: the levels of a batch of identical heat problems
    static std::unique_ptr<GMGHierarchy> heat(Context *c, const Mesh &m, const mfgpu_solver_params &s,
                                              double delta_t, int batch = 1);
    // neo-Hookean levels of caching `variant`
    static std::unique_ptr<GMGHierarchy> solid(Context *c, const Mesh &m, const mfgpu_solver_params &s,
                                               const NHMatD &mat, int formulation, int variant);
    // neo-Hookean: the FP64 finest-level linearisation interpolated to every
    // level (interpolate_to_mg) and cached there
    void set_linearisation(const double *ulin, PhaseTimer &t);
    // level diagonals (and the dense coarse operator) for the current level
    // states; nothing is recomputed while they are unchanged
    void update_diagonals(PhaseTimer &t);
    // Chebyshev eigenvalue estimates and coefficients (Multigrid::setup)
    void             setup_smoothers(PhaseTimer &t);
    Precond<double> *precond();
    size_t           n_dofs() const { return lops.back()->m(); }
  private:
    void finish(Context *c);
  };

  struct SolidDriver
  {
    Context                                  *ctx;
    mfgpu_solid_params                        P;
    Mesh                                      mesh;
    int                                       L = 0;
    HostBasis                                 basis;
    NHMatD                                    mat{};
    int                                       variant = 0;
    int                                       lprec   = 32;
    std::unique_ptr<NHOperator>               fine;
    std::unique_ptr<GMGHierarchy>             gmg;
    DevBuf                                    u, delta, v_old, a_old, acc, rhs, du;
    DevBuf                                    cg_ws; // vectors of the outer CG, kept across solves
    PhaseTimer                                timer;
    DevBuf                                    point_dev; // the watchpoint value
    HostPinned                                point_host;
    // the convergence table of the current / last time step (one row per
    // Newton iteration with a linear solve, as the reference prints it)
    struct NewtonRow
    {
      int    it, lin_its;
      double lin_res, cond, res_norm, res, upd_norm, upd;
    };
    std::vector<NewtonRow> table;
    int                    table_step = 0;
    double                 last_lin_res = 0, last_cond = 1;
    std::string            convergence_table() const;
    SolidDriver(Context *c, const mfgpu_solid_params &p);
    void                update_operators(const double *ulin);
    double              assemble_residual();
    double              residual_at(const double *u, const double *acc, double *rhs);
    int                 solve_linear(const double *b, double *x, double tol);
    std::vector<double> point_value(const double *x);
    void                run(mfgpu_solid_result &res);
    // one time step: Newton-Newmark iterations, velocity update, watchpoint
    void step(int &newton_its, long &total_cg, int &n_solves, double *watch);
    int  step_no = 0;
    // a new problem of the same shape (mesh, material, caching, solver and
    // Newton parameters, time step): the state starts from rest again and
    // the loads, watchpoint and step count are p's; the operators, the
    // multigrid hierarchy and every device buffer are kept
    void reset(const mfgpu_solid_params &p);
  };

  struct HeatDriver
  {
    Context                                   *ctx;
    mfgpu_heat_params                          P;
    Mesh                                       mesh;
    int                                        L = 0;
    HostBasis                                  basis;
    int                                        lprec = 32;
    std::unique_ptr<HeatOperator>              op, op_u;
    std::unique_ptr<GMGHierarchy>              gmg;
    DevBuf                                     sol, sol_old, rhs, du, uD;
    bool                                       started = false;
    int                                        step_no = 0;
    double                                     t       = 0;
    SourceDesc                                 src{};
    DevBuf                                     cg_ws; // vectors of the outer CG, kept across steps
    DevBuf                                     src_tab; // per-direction factors of the source's Gaussians
    PhaseTimer                                 timer;
    // a batch of nb problems of one shape (mesh, time step, solver) with
    // their own loads: one operator, one multigrid hierarchy and one CG
    // for all of them, every application one launch (make_heat(..., nb),
    // cg_solve_batched); problem i's vectors are block i of sol, rhs, ...
    int                                        nb = 1;
    std::vector<mfgpu_heat_params>             Pb;   // per problem (Pb[0] == P)
    std::vector<SourceDesc>                    srcs; // per problem
    HeatDriver(Context *c, const mfgpu_heat_params &p, int batch = 1);
    void node_x(size_t g, double *x) const;
    void start();          // initial condition, diagonals
    int  step();           // one backward-Euler step; returns CG iterations
    // one step of every problem of the batch; CG iterations per problem
    std::vector<int> step_batch();
    void run(mfgpu_heat_result &res);
    // new loads for the nb problems (same shape as the driver's)
    void reset_batch(const std::vector<mfgpu_heat_params> &ps);
    // a new problem of the same shape (mesh, time step, solver parameters):
    // the source / analytic data and step count are p's and the solution
    // starts from zero; operators, diagonals, smoothers and the captured
    // V-cycle are kept
    void reset(const mfgpu_heat_params &p);
  };
} // namespace mfgpu
