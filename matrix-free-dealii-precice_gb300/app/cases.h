// Test cases of the executables, restating the reference's case registry
// (include/cases/case_selector.h:31-49) for the three-dimensional device
// path.  The preCICE coupling data become constant boundary data:
//   * turek_hron (include/cases/elasticity/turek_hron.h:23-90): flap
//     [0.24899,0.6]x[0.19,0.21]x[-0.005,0.005], 5x1x1 coarse cells, clamped
//     short side (x-, id 1), out-of-plane faces clamped in z (id 2), the
//     remaining faces are the interface (id 11) carrying the dummy tester's
//     constant stress (0,-4,0) (tests/solid/dummy_tester.cpp:193-197); body
//     force (0,-0.5,0);
//   * cantilever: [0,8]x[0,1]^2, 8x1x1 coarse cells, clamped at x = 0,
//     traction (0,-100,0) on x = 8 (id 11), no body force;
//   * partitioned_heat_dirichlet (include/cases/heat_transfer/
//     partitioned_heat.h:36-133): u = 1 + x^2 + 3 y^2 + 1.3 t on the unit
//     cube with its Dirichlet data on every face (the coupled interface
//     receives the same analytic values from the Neumann partner);
//   * unit_cube_gaussians: unit cube, zero Dirichlet on x = 0, source = 8
//     seeded Gaussians.
#pragma once

#include <cmath>
#include <cstring>
#include <random>
#include <stdexcept>
#include <string>

#include "../../include/mfgpu.h"

namespace mfapp
{
  inline void
  set_box(mfgpu_mesh &m, const double *lo, const double *hi, const int *rep)
  {
    for (int d = 0; d < 3; ++d)
      {
        m.lower[d]       = lo[d];
        m.upper[d]       = hi[d];
        m.repetitions[d] = rep[d];
      }
  }

  struct SolidCase
  {
    double body[3]     = {0, 0, 0};
    double traction[3] = {0, 0, 0};
  };

  inline SolidCase
  make_solid_case(const std::string &name, mfgpu_mesh &m, int dim = 3)
  {
    SolidCase c;
    m.dim = dim;
    if (name == "turek_hron" && dim == 2)
      {
        // the reference's 2D flap: clamped short side (id 1), interface (id
        // 11) on the other three sides
        const double lo[3] = {0.24899, 0.19, 0.0}, hi[3] = {0.6, 0.21, 1.0};
        const int    rep[3] = {5, 1, 1};
        set_box(m, lo, hi, rep);
        const int ids[6] = {1, 11, 11, 11, -1, -1};
        std::memcpy(m.boundary_id, ids, sizeof(ids));
        m.n_dirichlet       = 1;
        m.dirichlet_id[0]   = 1;
        m.dirichlet_mask[0] = 0b11;
        c.body[1]           = -0.5;
        c.traction[1]       = -4.0;
        return c;
      }
    if (dim == 2)
      throw std::runtime_error("unknown two-dimensional elasticity test case '" + name +
                               "' (available: turek_hron)");
    if (name == "turek_hron")
      {
        const double lo[3] = {0.24899, 0.19, -0.005}, hi[3] = {0.6, 0.21, 0.005};
        const int    rep[3] = {5, 1, 1};
        set_box(m, lo, hi, rep);
        const int ids[6] = {1, 11, 11, 11, 2, 2};
        std::memcpy(m.boundary_id, ids, sizeof(ids));
        m.n_dirichlet       = 2;
        m.dirichlet_id[0]   = 1;
        m.dirichlet_mask[0] = 0b111;
        m.dirichlet_id[1]   = 2;
        m.dirichlet_mask[1] = 0b100;
        c.body[1]           = -0.5;
        c.traction[1]       = -4.0;
        return c;
      }
    if (name == "cantilever")
      {
        const double lo[3] = {0, 0, 0}, hi[3] = {8, 1, 1};
        const int    rep[3] = {8, 1, 1};
        set_box(m, lo, hi, rep);
        const int ids[6] = {1, 11, 0, 0, 0, 0};
        std::memcpy(m.boundary_id, ids, sizeof(ids));
        m.n_dirichlet       = 1;
        m.dirichlet_id[0]   = 1;
        m.dirichlet_mask[0] = 0b111;
        c.traction[1]       = -100.0;
        return c;
      }
    throw std::runtime_error("unknown elasticity test case '" + name +
                             "' (available on the device path: turek_hron, cantilever)");
  }

  inline void
  make_heat_case(const std::string &name, mfgpu_heat_params &p, int dim = 3)
  {
    const double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    const int    rep[3] = {1, 1, 1};
    set_box(p.mesh, lo, hi, rep);
    p.mesh.dim = dim;
    if (name == "partitioned_heat_dirichlet")
      {
        for (int f = 0; f < 2 * dim; ++f)
          p.mesh.boundary_id[f] = 1;
        p.mesh.n_dirichlet       = 1;
        p.mesh.dirichlet_id[0]   = 1;
        p.mesh.dirichlet_mask[0] = 1;
        p.analytic               = 1;
        p.alpha                  = 3;
        p.beta                   = 1.3;
        return;
      }
    if (name == "unit_cube_gaussians")
      {
        const int ids[6] = {1, 0, 0, 0, 0, 0};
        std::memcpy(p.mesh.boundary_id, ids, sizeof(ids));
        p.mesh.n_dirichlet       = 1;
        p.mesh.dirichlet_id[0]   = 1;
        p.mesh.dirichlet_mask[0] = 1;
        p.analytic               = 0;
        std::mt19937_64                        rng(0);
        std::uniform_real_distribution<double> u01(0.0, 1.0);
        p.n_gauss = 8;
        for (int i = 0; i < 8; ++i)
          {
            for (int d = 0; d < 3; ++d)
              p.g_center[i][d] = 0.2 + 0.6 * u01(rng);
            p.g_width[i] = 0.05 + 0.1 * u01(rng);
            p.g_amp[i]   = 0.5 + 1.5 * u01(rng);
          }
        return;
      }
    throw std::runtime_error("unknown heat transfer test case '" + name +
                             "' (available on the device path: partitioned_heat_dirichlet, "
                             "unit_cube_gaussians)");
  }
} // namespace mfapp
