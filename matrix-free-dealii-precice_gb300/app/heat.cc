// `heat <prm>`: the backward-Euler heat solver of the reference
// (src/heat.cc, include/heat_transfer/heat_transfer.h:972-1037) on the
// device path.  Reads the reference's parameter file format, runs
// End time / Time step size steps with GMG-preconditioned CG to
// 1e-12 |rhs| (heat_transfer.h:719-720), prints the L2 error against the
// analytic solution at every output tick for the analytic case
// (heat_transfer.h:888-893) and the CG statistics (:1030-1034).
#include <cmath>
#include <cstdio>
#include <iostream>
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

// L2 error of the nodal field u against 1 + x^2 + alpha y^2 + beta t with
// QGauss(p+1) on every cell
static double
l2_error(const mfgpu_mesh &m, const std::vector<double> &u, double alpha, double beta, double t)
{
  const int p = m.degree, N = p + 1;
  const std::vector<double> gl = lobatto(p);
  std::vector<double>       xq(N), wq(N);
  for (int i = 0; i < N; ++i)
    {
      long double z = std::cos(3.14159265358979323846L * (i + 0.75L) / (N + 0.5L)), dp = 0;
      for (int it = 0; it < 100; ++it)
        {
          long double p0 = 1, p1 = z;
          for (int k = 2; k <= N; ++k)
            {
              long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
              p0             = p1;
              p1             = p2;
            }
          dp = N * (z * p1 - p0) / (z * z - 1);
          z -= p1 / dp;
        }
      xq[N - 1 - i] = double((1 + z) / 2);
      wq[N - 1 - i] = double(1 / ((1 - z * z) * dp * dp));
    }
  std::vector<double> S(N * N);
  for (int q = 0; q < N; ++q)
    for (int i = 0; i < N; ++i)
      {
        double v = 1;
        for (int j = 0; j < N; ++j)
          if (j != i)
            v *= (xq[q] - gl[j]) / (gl[i] - gl[j]);
        S[q * N + i] = v;
      }
  // 2D: one node plane, one "quadrature point" of weight 1 along z
  const bool two = m.dim == 2;
  const int  Nz  = two ? 1 : N;
  int        C[3], Nn[3];
  double     h[3];
  for (int d = 0; d < 3; ++d)
    {
      C[d]  = (two && d == 2) ? 1 : (m.repetitions[d] << m.n_refinements);
      Nn[d] = (two && d == 2) ? 1 : C[d] * p + 1;
      h[d]  = (two && d == 2) ? 1.0 : (m.upper[d] - m.lower[d]) / C[d];
    }
  auto Sz = [&](int q, int k) { return two ? 1.0 : S[q * N + k]; };
  auto wz = [&](int q) { return two ? 1.0 : wq[q]; };
  double err = 0;
  for (int cz = 0; cz < C[2]; ++cz)
    for (int cy = 0; cy < C[1]; ++cy)
      for (int cx = 0; cx < C[0]; ++cx)
        for (int qz = 0; qz < Nz; ++qz)
          for (int qy = 0; qy < N; ++qy)
            for (int qx = 0; qx < N; ++qx)
              {
                double v = 0;
                for (int k = 0; k < Nz; ++k)
                  for (int j = 0; j < N; ++j)
                    for (int i = 0; i < N; ++i)
                      v += S[qx * N + i] * S[qy * N + j] * Sz(qz, k) *
                           u[size_t(cx * p + i) + size_t(Nn[0]) * (size_t(cy * p + j) + size_t(Nn[1]) * (cz * p + k))];
                const double x = m.lower[0] + (cx + xq[qx]) * h[0];
                const double y = m.lower[1] + (cy + xq[qy]) * h[1];
                const double e = 1 + x * x + alpha * y * y + beta * t - v;
                err += e * e * wq[qx] * wq[qy] * wz(qz) * h[0] * h[1] * h[2];
              }
  return std::sqrt(err);
}

int
main(int argc, char *argv[])
{
  try
    {
      const std::string file = argc > 1 ? argv[1] : "parameters.prm";
      Prm               prm;
      declare_common(prm);
      prm.parse(file);
      const int dim = prm.get_int("Geometry", "Dimension");
      if (dim != 2 && dim != 3)
        throw std::runtime_error("Dimension must be 2 or 3, not " + std::to_string(dim));
      mfgpu_heat_params P;
      std::memset(&P, 0, sizeof(P));
      P.mesh.degree        = prm.get_int("Finite element system", "Polynomial degree");
      P.mesh.n_q_1d        = prm.get_int("Finite element system", "Quadrature order");
      P.mesh.n_refinements = prm.get_int("Geometry", "Global refinement");
      make_heat_case(prm.get("Geometry", "Testcase"), P, dim);
      P.dt                     = prm.get_double("Time", "Time step size");
      const double end_time    = prm.get_double("Time", "End time");
      const int    n_steps     = int(std::lround(end_time / P.dt));
      P.n_steps                = 1;
      P.solver.preconditioner  = 2; // heat_transfer.h:386
      P.solver.tol             = 1e-12;
      P.solver.cheb_degree     = 5;
      P.solver.cheb_range      = 15;
      P.solver.cheb_eig_its    = 10;
      P.solver.coarse_accurate = 1;
      P.solver.max_it_mult     = 1;
      P.solver.mg_precision    = prm.get_int("GPU", "MG precision");
      P.solver.coarse_fp64     = prm.get_bool("GPU", "FP64 coarse solve");
      P.solver.fp64_emulation  = prm.get_bool("GPU", "FP64 emulation");
      P.solver.cuda_graphs     = prm.get_bool("GPU", "CUDA graphs");
      P.solver.coarse_dense    = prm.get_bool("GPU", "Dense coarse operator");
      const double tick        = prm.get_double("Output", "Output tick");

      mfgpu_context *ctx = nullptr;
      check(mfgpu_context_create(prm.get_int("GPU", "Device"), &ctx));
      mfgpu_heat *heat = nullptr;
      check(mfgpu_heat_create(ctx, &P, &heat));
      size_t nn = 0;
      check(mfgpu_mesh_n_nodes(&P.mesh, -1, &nn));
      std::vector<double> u(nn);
      long                cells = 1;
      for (int d = 0; d < dim; ++d)
        cells *= long(P.mesh.repetitions[d]) << P.mesh.n_refinements;
      std::cout << "--     . dim       = " << dim << "\n"
                << "--     . fe_degree = " << P.mesh.degree << "\n"
                << "--     . 1d_quad   = " << P.mesh.n_q_1d << "\n"
                << "--     . Number of active cells: " << cells << "\n"
                << "--     . Number of degrees of freedom: " << nn << "\n\n";
      const bool report    = P.analytic && cells <= 32768;
      const bool write_sol = prm.get_bool("Output", "Output solution");
      std::string folder   = prm.get("Output", "Output folder");
      if (!folder.empty() && folder.back() != '/')
        folder += '/';
      if (write_sol && !folder.empty())
        make_dirs(folder);
      // output_results (heat_transfer.h:854-880): the solution and the MPI
      // owner of every cell, at t = 0, every output tick and the end
      const std::vector<std::pair<std::string, double>> cell_data = {{"owner", 0.0}};
      std::vector<double> u0(nn, 0.0);
      if (report || (write_sol && P.analytic))
        {
          // initial condition
          const std::vector<double> gl = lobatto(P.mesh.degree);
          int Nn[3], C[3];
          for (int d = 0; d < 3; ++d)
            {
              C[d]  = P.mesh.repetitions[d] << P.mesh.n_refinements;
              Nn[d] = C[d] * P.mesh.degree + 1;
            }
          for (size_t g = 0; g < nn; ++g)
            {
              const int ix = int(g % Nn[0]), iy = int((g / Nn[0]) % Nn[1]);
              auto      coord = [&](int i, int d) {
                const int c = std::min(i / P.mesh.degree, C[d] - 1);
                return P.mesh.lower[d] + (c + gl[i - c * P.mesh.degree]) *
                                           (P.mesh.upper[d] - P.mesh.lower[d]) / C[d];
              };
              const double x = coord(ix, 0), y = coord(iy, 1);
              u0[g]          = 1 + x * x + P.alpha * y * y;
            }
        }
      if (report)
        std::cout << "Error: " << l2_error(P.mesh, u0, P.alpha, P.beta, 0.0) << "\n\n";
      if (write_sol)
        write_vtu(vtu_name(folder, 0), P.mesh, dim, 1, u0, "solution", false, cell_data);
      long total_its = 0;
      double t = 0;
      for (int s = 0; s < n_steps; ++s)
        {
          int its = 0;
          check(mfgpu_heat_step(heat, &its));
          total_its += its;
          t += P.dt;
          const bool tick_crossed = int(std::round(t / tick * 1e12) / 1e12) !=
                                      int(std::round((t - P.dt) / tick * 1e12) / 1e12) ||
                                    s == n_steps - 1;
          if ((report || write_sol) && tick_crossed)
            {
              const double *dptr = nullptr;
              check(mfgpu_heat_solution(heat, &dptr));
              check(mfgpu_copy(ctx, u.data(), dptr, nn * sizeof(double)));
              if (report)
                std::cout << "Error: " << l2_error(P.mesh, u, P.alpha, P.beta, t) << "\n\n";
              if (write_sol)
                write_vtu(vtu_name(folder, int(std::lround(t / tick))), P.mesh, dim, 1, u, "solution", false,
                          cell_data);
            }
        }
      std::cout << "\nAverage CG iter = " << (n_steps ? total_its / n_steps : 0) << "\n"
                << "Total CG iter = " << total_its << "\n"
                << "Total CG solve = " << n_steps << "\n";
      mfgpu_heat_destroy(heat);
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
