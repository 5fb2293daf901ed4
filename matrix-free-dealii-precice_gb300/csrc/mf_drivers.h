// Solid and heat drivers (device-resident Newton-Newmark / backward Euler).
#pragma once

#include "../../include/mfgpu.h"
#include "mf_solvers.h"

namespace mfgpu
{
  Mesh to_mesh(const mfgpu_mesh &m);

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
    std::vector<std::unique_ptr<NHOperator>>  lops;
    std::unique_ptr<NHOperator>               coarse64;
    std::unique_ptr<Multigrid<float>>         mgf;
    std::unique_ptr<Multigrid<double>>        mgd;
    std::vector<DevBuf>                       u_levels;
    DevBuf                                    u0_64;
    DevBuf                                    u, delta, v_old, a_old, acc, rhs, du;
    DevBuf                                    cg_ws; // vectors of the outer CG, kept across solves
    PhaseTimer                                timer;
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
  };

  struct HeatDriver
  {
    Context                                   *ctx;
    mfgpu_heat_params                          P;
    Mesh                                       mesh;
    int                                        L = 0;
    HostBasis                                  basis;
    int                                        lprec = 32;
    std::unique_ptr<HeatOperator>              op, op_u, coarse64;
    std::vector<std::unique_ptr<HeatOperator>> lops;
    std::unique_ptr<Multigrid<float>>          mgf;
    std::unique_ptr<Multigrid<double>>         mgd;
    DevBuf                                     sol, sol_old, rhs, du, uD;
    bool                                       started = false;
    int                                        step_no = 0;
    double                                     t       = 0;
    SourceDesc                                 src{};
    DevBuf                                     cg_ws; // vectors of the outer CG, kept across steps
    PhaseTimer                                 timer;
    HeatDriver(Context *c, const mfgpu_heat_params &p);
    void node_x(size_t g, double *x) const;
    void start();          // initial condition, diagonals
    int  step();           // one backward-Euler step; returns CG iterations
    void run(mfgpu_heat_result &res);
  };
} // namespace mfgpu
