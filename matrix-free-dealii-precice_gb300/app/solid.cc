// `solid <prm>`: the Newton-Newmark neo-Hookean solver of the reference
// (src/solid.cc, include/solid_mechanics/mf_elasticity.h:555-628) on the
// device path.  Reads the reference's parameter file format, runs
// End time / Time step size steps, and writes the reference's blessed
// `output` file (reference volume, problem size, Newton iterations per
// step, the displacement at the first output point, average CG
// iterations; mf_elasticity.h:625-627,1389-1390,1591-1592) into the output
// folder.  Exceptions print the reference's message and return 1
// (src/solid.cc:64-89).
#include <sys/stat.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <sstream>
#include <vector>

#include "cases.h"
#include "prm.h"
#include "vtu.h"

using namespace mfapp;

static void
check(int rc)
{
  if (rc != MFGPU_OK)
    throw std::runtime_error(mfgpu_last_error());
}

int
main(int argc, char *argv[])
{
  try
    {
      const std::string file = argc > 1 ? argv[1] : "parameters.prm";
      Prm               prm;
      declare_solid(prm);
      prm.parse(file);
      const int dim = prm.get_int("Geometry", "Dimension");
      if (dim != 2 && dim != 3)
        throw std::runtime_error("Dimension must be 2 or 3, not " + std::to_string(dim));
      const int degree = prm.get_int("Finite element system", "Polynomial degree");
      const int nq     = prm.get_int("Finite element system", "Quadrature order");
      if (degree < 1)
        throw std::runtime_error("polynomial degree must be positive");

      mfgpu_solid_params P;
      std::memset(&P, 0, sizeof(P));
      P.mesh.degree        = degree;
      P.mesh.n_q_1d        = nq;
      P.mesh.n_refinements = prm.get_int("Geometry", "Global refinement");
      const SolidCase sc   = make_solid_case(prm.get("Geometry", "Testcase"), P.mesh, dim);
      P.material.mu          = prm.get_double("Material properties", "Shear modulus");
      P.material.nu          = prm.get_double("Material properties", "Poisson's ratio");
      P.material.rho         = prm.get_double("Material properties", "Density");
      P.material.formulation = prm.get_int("Material properties", "Formulation");
      const std::string caching = prm.get("Linear solver", "MF caching");
      P.caching                 = caching.c_str();
      const std::string pt      = prm.get("Linear solver", "Preconditioner type");
      P.solver.preconditioner   = pt == "gmg" ? 2 : (pt == "jacobi" ? 1 : (pt == "none" ? 0 : -1));
      if (P.solver.preconditioner < 0)
        throw std::runtime_error("Preconditioner type must be jacobi|gmg|none");
      P.solver.relaxation      = prm.get_double("Linear solver", "Preconditioner relaxation");
      P.solver.tol             = prm.get_double("Linear solver", "Residual");
      P.solver.max_it_mult     = prm.get_int("Linear solver", "Max iteration multiplier");
      P.solver.cheb_degree     = 5;
      P.solver.cheb_range      = 20;
      P.solver.cheb_eig_its    = prm.get_int("Linear solver", "MF Chebyshev number CG iterations");
      P.solver.coarse_accurate = prm.get_bool("Linear solver", "MF Chebyshev coarse accurate eigenvalues");
      // the level-0 solver: Chebyshev (the default); the alternative CG
      // coarse solver of mf_elasticity.h:1183-1198 is not built
      if (P.solver.preconditioner == 2 && !prm.get_bool("Linear solver", "MF Chebyshev coarse"))
        throw std::runtime_error("MF Chebyshev coarse = false (CG coarse-grid solver) is not supported");
      P.solver.estimate_condition = prm.get_bool("Linear solver", "Estimate condition number");
      P.solver.cond_cg_iterations = prm.get_int("Linear solver", "Condition number CG iterations");
      P.solver.mg_precision    = prm.get_int("GPU", "MG precision");
      P.solver.coarse_fp64     = prm.get_bool("GPU", "FP64 coarse solve");
      P.solver.fp64_emulation  = prm.get_bool("GPU", "FP64 emulation");
      P.solver.cuda_graphs     = prm.get_bool("GPU", "CUDA graphs");
      P.solver.coarse_dense    = prm.get_bool("GPU", "Dense coarse operator");
      P.max_newton             = prm.get_int("Nonlinear solver", "Max iterations Newton-Raphson");
      P.tol_f                  = prm.get_double("Nonlinear solver", "Tolerance force");
      P.tol_f_abs              = prm.get_double("Nonlinear solver", "Absolute tolerance force");
      P.tol_u                  = prm.get_double("Nonlinear solver", "Tolerance displacement");
      P.tol_u_abs              = prm.get_double("Nonlinear solver", "Absolute tolerance displacement");
      P.dt                     = prm.get_double("Time", "Time step size");
      const double end_time    = prm.get_double("Time", "End time");
      P.n_steps                = int(std::lround(end_time / P.dt));
      if (P.n_steps < 1 || P.n_steps > 64)
        throw std::runtime_error("End time / Time step size must give 1..64 steps");
      for (int d = 0; d < 3; ++d)
        {
          P.body_force[d] = sc.body[d];
          P.traction[d]   = sc.traction[d];
        }
      const std::vector<double> tr = prm.get_list("GPU", "Traction");
      if (tr.size() == 3)
        for (int d = 0; d < 3; ++d)
          P.traction[d] = tr[d];
      P.traction_id                = 11;
      const std::vector<double> pt3 = prm.get_list("Output", "Output points");
      if (int(pt3.size()) != dim)
        throw std::runtime_error("Output points must give one point with " + std::to_string(dim) +
                                 " coordinates");
      for (int d = 0; d < dim; ++d)
        P.watch[d] = pt3[d];

      mfgpu_context *ctx = nullptr;
      check(mfgpu_context_create(prm.get_int("GPU", "Device"), &ctx));
      mfgpu_solid *solid = nullptr;
      check(mfgpu_solid_create(ctx, &P, &solid));
      // wall-clock sections, printed at the end as the reference's
      // TimerOutput summary
      check(mfgpu_solid_set_timing(solid, 1));

      // time loop of Solid::run (mf_elasticity.h:555-613): the solution is
      // written at t = 0, at every output tick and at the end
      const bool   write_sol = prm.get_bool("Output", "Output solution");
      const double tick      = prm.get_double("Output", "Output tick");
      std::string  folder    = prm.get("Output", "Output folder");
      if (!folder.empty() && folder.back() != '/')
        folder += '/';
      if (!folder.empty())
        make_dirs(folder);
      size_t nn = 0;
      check(mfgpu_mesh_n_nodes(&P.mesh, -1, &nn));
      std::vector<double> uh(size_t(dim) * nn, 0.0);
      // cell data of the reference's output: MPI subdomain, material id and
      // manifold id (flat_manifold_id of the box cells)
      const std::vector<std::pair<std::string, double>> cell_data = {
        {"subdomain", 0.0}, {"material_id", 0.0}, {"manifold_id", 4294967295.0}};
      auto write_solution = [&](int number) {
        const double *ud = nullptr;
        check(mfgpu_solid_displacement(solid, &ud));
        check(mfgpu_copy(ctx, uh.data(), ud, uh.size() * sizeof(double)));
        write_vtu(vtu_name(folder, number), P.mesh, dim, dim, uh, "displacement", true, cell_data);
      };
      mfgpu_solid_result R;
      std::memset(&R, 0, sizeof(R));
      R.n_steps = P.n_steps;
      if (write_sol)
        write_solution(0);
      double tt = 0;
      for (int s = 0; s < P.n_steps; ++s)
        {
          long cg     = 0;
          int  solves = 0;
          check(mfgpu_solid_step(solid, &R.newton_its[s], &cg, &solves, R.watch_disp[s]));
          // the Newton convergence table the reference prints per step
          std::vector<char> conv(1 << 14);
          check(mfgpu_solid_convergence_table(solid, conv.data(), conv.size()));
          std::cout << conv.data();
          R.total_cg += cg;
          R.n_solves += solves;
          tt += P.dt;
          const bool crossed = int(std::round(tt / tick * 1e12) / 1e12) !=
                                 int(std::round((tt - P.dt) / tick * 1e12) / 1e12) ||
                               s == P.n_steps - 1;
          if (write_sol && crossed)
            write_solution(int(std::lround(tt / tick)));
        }
      long cells = 1;
      double vol = 1;
      for (int d = 0; d < dim; ++d)
        {
          cells *= long(P.mesh.repetitions[d]) << P.mesh.n_refinements;
          vol *= P.mesh.upper[d] - P.mesh.lower[d];
        }
      std::ostringstream out;
      out << "--     . Reference volume: " << vol << "\n"
          << "--     . dim       = " << dim << "\n"
          << "--     . fe_degree = " << degree << "\n"
          << "--     . 1d_quad   = " << nq << "\n"
          << "--     . Number of active cells: " << cells << "\n"
          << "--     . Number of degrees of freedom: " << dim * nn << "\n"
          << "\n";
      double t = 0;
      for (int s = 0; s < R.n_steps; ++s)
        {
          t += P.dt;
          out << "\nTimestep " << s + 1 << " @ " << t << "s\n"
              << "Converged in " << R.newton_its[s] << " Newton iterations\n"
              << "Solution @";
          for (int d = 0; d < dim; ++d)
            out << " " << P.watch[d];
          out << "\n  displacement:";
          for (int d = 0; d < dim; ++d)
            out << " " << R.watch_disp[s][d];
          out << "\n";
        }
      out << "\nAverage CG iter = " << (R.n_solves ? R.total_cg / R.n_solves : 0) << "\n";
      std::cout << out.str();
      if (write_sol)
        {
          std::FILE *f = std::fopen((folder + "output").c_str(), "w");
          if (!f)
            throw std::runtime_error("can't create: " + folder + "output");
          std::fputs(out.str().c_str(), f);
          std::fclose(f);
        }
      std::vector<char> table(1 << 16);
      check(mfgpu_solid_timing_summary(solid, table.data(), table.size()));
      std::cout << "\n" << table.data() << std::flush;
      mfgpu_solid_destroy(solid);
      mfgpu_context_destroy(ctx);
    }
  catch (std::exception &exc)
    {
      std::cerr << std::endl
                << std::endl
                << "----------------------------------------------------" << std::endl;
      std::cerr << "Exception on processing: " << std::endl
                << exc.what() << std::endl
                << "Aborting!" << std::endl
                << "----------------------------------------------------" << std::endl;
      return 1;
    }
  return 0;
}
