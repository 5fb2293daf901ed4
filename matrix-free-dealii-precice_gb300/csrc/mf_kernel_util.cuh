// Host-side helpers shared by the kernel instantiation units: shape data
// in the compute precision, material constants, launch ranges and the
// one-time shared-memory attribute of a kernel.
#pragma once

#include <cmath>
#include <cstring>
#include <mutex>
#include <set>
#include <tuple>

#include "mf_cell.cuh"
#include "mf_launch.h"

namespace mfgpu
{
  namespace detail
  {
    template <int N, typename T>
    Shape<N, T>
    make_shape(const HostBasis &b)
    {
      Shape<N, T> s;
      for (int i = 0; i < N * N; ++i)
        {
          s.S[i] = conv_host<T>(b.S[i]);
          s.D[i] = conv_host<T>(b.D[i]);
        }
      for (int i = 0; i < N; ++i)
        s.w[i] = conv_host<T>(b.w[i]);
      return s;
    }

    // even-odd form of the row-major N x N matrix scale * M (FP64 on the
    // host, then rounded to the compute type)
    template <int N, typename T, int SIG>
    EO<N, T, SIG>
    make_eo(const double *M, double scale)
    {
      using E = EO<N, T, SIG>;
      E r;
      for (int i = 0; i < E::HR; ++i)
        {
          for (int k = 0; k < E::H; ++k)
            {
              r.e[i * E::HR + k] = conv_host<T>(0.5 * scale * (M[i * N + k] + M[i * N + N - 1 - k]));
              r.o[i * E::H + k]  = conv_host<T>(0.5 * scale * (M[i * N + k] - M[i * N + N - 1 - k]));
            }
          if (N % 2 == 1)
            r.e[i * E::HR + E::H] = conv_host<T>(scale * M[i * N + E::H]);
        }
      return r;
    }

    template <int N, typename T>
    ShapeA<N, T>
    make_shape_apply(const HostBasis &b, const LevelGeom &g)
    {
      ShapeA<N, T> s;
      for (int i = 0; i < N * N; ++i)
        {
          s.S[i]  = conv_host<T>(b.S[i]);
          s.Du[i] = conv_host<T>(b.D[i]);
          for (int d = 0; d < 3; ++d)
            s.D[d][i] = conv_host<T>(b.D[i] / g.h[d]);
        }
      for (int i = 0; i < N; ++i)
        s.w[i] = conv_host<T>(b.w[i]);
      s.Se  = make_eo<N, T, 1>(b.S, 1.0);
      s.Due = make_eo<N, T, -1>(b.D, 1.0);
      for (int d = 0; d < 3; ++d)
        s.De[d] = make_eo<N, T, -1>(b.D, 1.0 / g.h[d]);
      return s;
    }

    template <typename T>
    NHMat<T>
    to_mat(const NHMatD &m)
    {
      NHMat<T> r;
      r.mu         = conv_host<T>(m.mu);
      r.lambda     = conv_host<T>(m.lambda);
      r.rho_alpha  = conv_host<T>(m.rho_alpha);
      r.kappa      = conv_host<T>(m.kappa);
      r.c_1        = conv_host<T>(m.c_1);
      r.two_lambda = conv_host<T>(2.0 * m.lambda);
      return r;
    }

    // restrict an application launch to the cells [a.cell_begin, a.cell_end)
    template <typename T>
    CellGeom<T>
    apply_range(CellGeom<T> c, const ApplyArgs &a)
    {
      c.batch   = unsigned(a.batch > 1 ? a.batch : 1);
      c.bstride = a.batch > 1 ? a.bstride : 0;
      c.unit_ld = a.unit_ld;
      if (a.cell_end > a.cell_begin)
        {
          c.cell_begin = unsigned(a.cell_begin);
          c.cell_end   = unsigned(a.cell_end < c.n_cells ? a.cell_end : c.n_cells);
        }
      else if (a.colored)
        c.color = 8; // all colours, one launch each
      return c;
    }

    // raise a kernel's dynamic shared memory limit once per (kernel,
    // device, size): the launch path then makes no attribute call
    template <typename K>
    cudaError_t
    prepare(K kernel, size_t smem)
    {
      if (smem <= 48 * 1024)
        return cudaSuccess;
      static std::mutex                                    mu;
      static std::set<std::tuple<const void *, int, size_t>> done;
      int                                                  dev = 0;
      cudaError_t                                          e   = cudaGetDevice(&dev);
      if (e != cudaSuccess)
        return e;
      const auto                  key = std::make_tuple(reinterpret_cast<const void *>(kernel), dev, smem);
      std::lock_guard<std::mutex> l(mu);
      if (done.count(key))
        return cudaSuccess;
      e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (e == cudaSuccess)
        done.insert(key);
      return e;
    }

  } // namespace detail
} // namespace mfgpu
