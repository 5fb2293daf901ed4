// Launches of the two-dimensional kernels (all degrees in one unit: the 2D
// kernels are small).
#include "mf_kernel_util.cuh"
#include "mf_setup.cuh"
#include "mf_cell2d.cuh"

namespace mfgpu
{
  using namespace detail;

  namespace
  {
    template <int N, typename T, int NC, class Op>
    cudaError_t
    run2(const ShapeA<N, T> &sh, const CellGeom<T> &cg, const Op &op, bool con, const T *src, T *dst,
         cudaStream_t s)
    {
      constexpr int  CPB   = cpb2d<N>();
      const size_t   smem  = size_t(CPB) * NC * 3 * N * N * sizeof(T);
      const unsigned cells = cg.cell_end - cg.cell_begin;
      const unsigned grid  = (cells + CPB - 1) / CPB;
      if (grid == 0)
        return cudaSuccess;
      auto        k = con ? cell_apply2d_kernel<N, T, NC, Op, true> : cell_apply2d_kernel<N, T, NC, Op, false>;
      cudaError_t e = prepare(k, smem);
      if (e != cudaSuccess)
        return e;
      k<<<grid, CPB * N, smem, s>>>(sh, cg, op, src, dst);
      return cudaGetLastError();
    }

    template <int N, typename T>
    cudaError_t
    apply2(const HostBasis &b, const LevelGeom &g, const ApplyArgs &a, cudaStream_t s)
    {
      if (a.colored)
        return cudaErrorNotSupported;
      const ShapeA<N, T> sh  = make_shape_apply<N, T>(b, g);
      const CellGeom<T>  cg  = apply_range(make_cell_geom<T>(g), a);
      const T           *src = static_cast<const T *>(a.src);
      T                 *dst = static_cast<T *>(a.dst);
      if (a.kind == 0)
        {
          Heat2QOp<T> op{conv_host<T>(a.kdt)};
          return run2<N, T, 1>(sh, cg, op, a.constrained, src, dst, s);
        }
      if (a.var == V_FORM0)
        {
          NH2Form0QOp<T> op{static_cast<const T *>(a.cache), to_mat<T>(a.mat), N * N};
          return run2<N, T, 2>(sh, cg, op, a.constrained, src, dst, s);
        }
      NH2Form1QOp<T> op{static_cast<const T *>(a.cache), to_mat<T>(a.mat), N * N};
      return run2<N, T, 2>(sh, cg, op, a.constrained, src, dst, s);
    }

    template <int N, typename T>
    cudaError_t
    cache2(const HostBasis &b, const LevelGeom &g, int form, const NHMatD &md, const void *u, void *cache,
           int *err, cudaStream_t s)
    {
      const ShapeA<N, T> sh   = make_shape_apply<N, T>(b, g);
      const CellGeom<T>  cg   = make_cell_geom<T>(g);
      constexpr int      CPB  = cpb2d<N>();
      const size_t       smem = size_t(CPB) * 6 * N * N * sizeof(T);
      const unsigned     grid = (cg.n_cells + CPB - 1) / CPB;
      auto               k    = form == 0 ? nh_cache2d_kernel<N, T, 0> : nh_cache2d_kernel<N, T, 1>;
      cudaError_t        e    = prepare(k, smem);
      if (e != cudaSuccess)
        return e;
      k<<<grid, CPB * N, smem, s>>>(sh, cg, to_mat<T>(md), static_cast<const T *>(u), static_cast<T *>(cache),
                                    err);
      return cudaGetLastError();
    }

    template <int N, typename T>
    cudaError_t
    diag2(const HostBasis &b, const LevelGeom &g, int kind, const NHMatD &md, double kdt, const void *cache,
          void *diag, cudaStream_t s)
    {
      const ShapeA<N, T> sh = make_shape_apply<N, T>(b, g);
      const CellGeom<T>  cg = make_cell_geom<T>(g);
      T                 *d  = static_cast<T *>(diag);
      if (kind == 0)
        {
          Heat2QOp<T> op{conv_host<T>(kdt)};
          diag2d_kernel<N, T, 1><<<cg.n_cells, N * N, 0, s>>>(sh, cg, op, d);
        }
      else if (kind == 2)
        {
          NH2Form0QOp<T> op{static_cast<const T *>(cache), to_mat<T>(md), N * N};
          diag2d_kernel<N, T, 2><<<cg.n_cells, 2 * N * N, 0, s>>>(sh, cg, op, d);
        }
      else
        {
          NH2Form1QOp<T> op{static_cast<const T *>(cache), to_mat<T>(md), N * N};
          diag2d_kernel<N, T, 2><<<cg.n_cells, 2 * N * N, 0, s>>>(sh, cg, op, d);
        }
      return cudaGetLastError();
    }

    template <int N>
    cudaError_t
    residual2(const HostBasis &b, const LevelGeom &g, int form, const NHMatD &md, double rho,
              const double *body, const double *u, const double *acc, double *rhs, cudaStream_t s)
    {
      const ShapeA<N, double> sh   = make_shape_apply<N, double>(b, g);
      const CellGeom<double>  cg   = make_cell_geom<double>(g);
      constexpr int           CPB  = cpb2d<N>();
      const size_t            smem = size_t(CPB) * 8 * N * N * sizeof(double);
      const unsigned          grid = (cg.n_cells + CPB - 1) / CPB;
      auto                    k    = form == 0 ? residual2d_kernel<N, 0> : residual2d_kernel<N, 1>;
      cudaError_t             e    = prepare(k, smem);
      if (e != cudaSuccess)
        return e;
      k<<<grid, CPB * N, smem, s>>>(sh, cg, to_mat<double>(md), rho, body[0], body[1], u, acc, rhs);
      return cudaGetLastError();
    }

    template <int N>
    cudaError_t
    heat_rhs2(const HostBasis &b, const LevelGeom &g, double dt, const SourceDesc &f, const double *u_old,
              double *rhs, cudaStream_t s)
    {
      const ShapeA<N, double> sh = make_shape_apply<N, double>(b, g);
      const CellGeom<double>  cg = make_cell_geom<double>(g);
      SourceDev               sd;
      std::memset(&sd, 0, sizeof(sd));
      sd.constant = f.constant;
      sd.n_gauss  = f.n_gauss;
      for (int i = 0; i < 8; ++i)
        {
          for (int d = 0; d < 3; ++d)
            sd.center[i][d] = f.center[i][d];
          sd.width[i] = f.width[i];
          sd.amp[i]   = f.amp[i];
        }
      for (int d = 0; d < 3; ++d)
        {
          sd.lo[d] = g.lo[d];
          sd.h[d]  = g.h[d];
        }
      for (int i = 0; i < N; ++i)
        sd.xq[i] = b.xq[i];
      constexpr int  CPB  = cpb2d<N>();
      const size_t   smem = size_t(CPB) * 2 * N * N * sizeof(double);
      const unsigned grid = (cg.n_cells + CPB - 1) / CPB;
      heat_rhs2d_kernel<N><<<grid, CPB * N, smem, s>>>(sh, cg, sd, dt, u_old, rhs);
      return cudaGetLastError();
    }
  } // namespace

#define MF_SWITCH_N(N, CALL)                                                                                      \
  switch (N)                                                                                                      \
    {                                                                                                             \
      case 2: return CALL(2);                                                                                     \
      case 3: return CALL(3);                                                                                     \
      case 4: return CALL(4);                                                                                     \
      case 5: return CALL(5);                                                                                     \
      case 6: return CALL(6);                                                                                     \
      case 7: return CALL(7);                                                                                     \
    }                                                                                                             \
  return cudaErrorInvalidValue

  cudaError_t
  launch_apply2d(int N, int precision, const HostBasis &b, const LevelGeom &g, const ApplyArgs &a,
                 cudaStream_t s)
  {
#define MF_CALL(n) (precision == 32 ? apply2<n, float>(b, g, a, s) : apply2<n, double>(b, g, a, s))
    MF_SWITCH_N(N, MF_CALL);
#undef MF_CALL
  }

  cudaError_t
  launch_nh_cache2d(int N, int precision, const HostBasis &b, const LevelGeom &g, int form, const NHMatD &m,
                    const void *u, void *cache, int *err, cudaStream_t s)
  {
#define MF_CALL(n)                                                                                                \
  (precision == 32 ? cache2<n, float>(b, g, form, m, u, cache, err, s) : cache2<n, double>(b, g, form, m, u, cache, err, s))
    MF_SWITCH_N(N, MF_CALL);
#undef MF_CALL
  }

  cudaError_t
  launch_diag2d(int N, int precision, const HostBasis &b, const LevelGeom &g, int kind, const NHMatD &m,
                double kdt, const void *cache, void *diag, cudaStream_t s)
  {
#define MF_CALL(n)                                                                                                \
  (precision == 32 ? diag2<n, float>(b, g, kind, m, kdt, cache, diag, s) :                                         \
                     diag2<n, double>(b, g, kind, m, kdt, cache, diag, s))
    MF_SWITCH_N(N, MF_CALL);
#undef MF_CALL
  }

  cudaError_t
  launch_residual2d(int N, const HostBasis &b, const LevelGeom &g, int form, const NHMatD &m, double rho,
                    const double *body, const double *u, const double *acc, double *rhs, cudaStream_t s)
  {
#define MF_CALL(n) residual2<n>(b, g, form, m, rho, body, u, acc, rhs, s)
    MF_SWITCH_N(N, MF_CALL);
#undef MF_CALL
  }

  cudaError_t
  launch_heat_rhs2d(int N, const HostBasis &b, const LevelGeom &g, double dt, const SourceDesc &f,
                    const double *u_old, double *rhs, cudaStream_t s)
  {
#define MF_CALL(n) heat_rhs2<n>(b, g, dt, f, u_old, rhs, s)
    MF_SWITCH_N(N, MF_CALL);
#undef MF_CALL
  }
#undef MF_SWITCH_N
} // namespace mfgpu
