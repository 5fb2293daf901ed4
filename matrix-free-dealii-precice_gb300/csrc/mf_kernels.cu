// Instantiation of the cell kernels for one degree.  Compiled once per
// N = p+1 in {2..7} with -DMF_N=<N>, so the per-degree builds run in
// parallel.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <set>
#include <tuple>

#include "mf_kernel_util.cuh"
#include "mf_setup.cuh"

#ifndef MF_N
#error "MF_N must be defined (2..7)"
#endif

namespace mfgpu
{
  using namespace detail;
  namespace
  {
    // launches of fewer cells than this (the SM count of GB300) take the
    // one-cell-per-block kernel
    constexpr unsigned SMALL_GRID = 152;

    template <int N, typename TS, typename T, int NC, class Op, bool CON>
    cudaError_t
    run_apply(const ShapeA<N, T> &sh, const CellGeom<T> &cg, const Op &op,
              const TS *src, TS *dst, bool unit, int kernel, cudaStream_t s)
    {
      constexpr int CPB  = apply_cells_per_block<N, NC, TS, Op::eval_u>();
      const size_t  smem = size_t(CPB) * apply_smem_per_cell<N, NC, Op::eval_u, T>() * sizeof(T);
      cudaError_t   e    = cudaSuccess;
      if (unit)
        {
          // element columns: one block per (cell, local DoF), constrained
          // operators only (the coarse levels)
          if constexpr (CON)
            {
              auto         ku    = cell_apply_kernel<N, TS, T, NC, Op, true, true, true>;
              const size_t smemu = apply_smem_per_cell<N, NC, Op::eval_u, T>() * sizeof(T);
              if ((e = prepare(ku, smemu)) != cudaSuccess)
                return e;
              const size_t blocks = size_t(cg.cell_end - cg.cell_begin) * NC * N * N * N;
              if (blocks == 0)
                return cudaSuccess;
              if (blocks > 0x7fffffffu || cg.color >= 0)
                return cudaErrorInvalidValue;
              ku<<<unsigned(blocks), N * N, smemu, s>>>(sh, cg, op, src, dst);
              return cudaGetLastError();
            }
          return cudaErrorInvalidValue;
        }
      const unsigned n_cells = cg.cell_end - cg.cell_begin;
      // native FP64 keeps the point-parallel kernel up to 4096 cells, and the
      // referential_qp tangent at every size but Q2 (measured, CUDA events,
      // L2 flushed: 4096 cells Q3 122 against 154 us, Q4 257 / 289, Q5
      // 498 / 580; 32768 cells Q3 881 / 951, Q4 1995 / 2004, Q6 863 / 873;
      // Q2 at 32768 cells 384 / 345, where the line kernel's even-odd sweeps
      // win)
      // (the FP32 referential_qp tangent at Q2 up to 4096 cells as well:
      // 13.0 against 17.0 us there)
      const unsigned point_below = !std::is_same<T, double>::value ?
                                     ((std::is_same<T, float>::value && N == 3 && Op::prefetch) ? 4097u :
                                                                                                 POINT_CELLS) :
                                   (Op::prefetch && N != 3) ? 0xffffffffu :
                                                              4097u;
      if (cg.color < 0 && n_cells > 0 && (kernel == 2 || (kernel == 0 && n_cells < point_below)))
        {
          // few cells: one block per cell, one thread per point
          auto         kp    = cell_apply_point_kernel<N, TS, T, NC, Op, CON>;
          const size_t smemp = point_smem_elems<N, NC, Op::eval_u>() * sizeof(T);
          if ((e = prepare(kp, smemp)) != cudaSuccess)
            return e;
          kp<<<dim3(n_cells, cg.batch), N * N * N, smemp, s>>>(sh, cg, op, src, dst);
          return cudaGetLastError();
        }
      auto k = cell_apply_kernel<N, TS, T, NC, Op, CON>;
      if ((e = prepare(k, smem)) != cudaSuccess)
        return e;
      if (cg.color == 8)
        {
          // coloured scatter: one launch per non-empty parity colour, in order
          for (int color = 0; color < 8; ++color)
            {
              CellGeom<T> c = cg;
              c.color       = color;
              c.color_n     = color_cells(cg.C, color, c.hc);
              if (c.color_n == 0)
                continue;
              k<<<dim3((c.color_n + CPB - 1) / CPB, cg.batch), CPB * N * N, smem, s>>>(sh, c, op, src, dst);
              if ((e = cudaGetLastError()) != cudaSuccess)
                return e;
            }
          return cudaSuccess;
        }
      const unsigned cells = cg.cell_end - cg.cell_begin;
      const unsigned grid  = (cells + CPB - 1) / CPB;
      if (grid == 0)
        return cudaSuccess;
      if constexpr (Op::ref_grad && CPB > 1)
        if (cells < SMALL_GRID)
          {
            // fewer cells than SMs: one cell per block, on as many SMs
            auto         k1    = cell_apply_kernel<N, TS, T, NC, Op, CON, true>;
            const size_t smem1 = apply_smem_per_cell<N, NC, Op::eval_u, T>() * sizeof(T);
            if ((e = prepare(k1, smem1)) != cudaSuccess)
              return e;
            k1<<<dim3(cells, cg.batch), N * N, smem1, s>>>(sh, cg, op, src, dst);
            return cudaGetLastError();
          }
      k<<<dim3(grid, cg.batch), CPB * N * N, smem, s>>>(sh, cg, op, src, dst);
      return cudaGetLastError();
    }

    template <int N, typename TS, typename T, int NC, class Op>
    cudaError_t
    run_apply_c(const ApplyArgs &a, const ShapeA<N, T> &sh, const CellGeom<T> &cg,
                const Op &op, const TS *src, TS *dst, cudaStream_t s)
    {
      return a.constrained ? run_apply<N, TS, T, NC, Op, true>(sh, cg, op, src, dst, a.unit, a.kernel, s) :
                             run_apply<N, TS, T, NC, Op, false>(sh, cg, op, src, dst, a.unit, a.kernel, s);
    }
  } // namespace

  template <int N, typename T>
  cudaError_t
  launch_apply(const HostBasis &b, const LevelGeom &g, const ApplyArgs &a,
               cudaStream_t s)
  {
    const ShapeA<N, T>   sh  = make_shape_apply<N, T>(b, g);
    const CellGeom<T>    cg  = apply_range(make_cell_geom<T>(g), a);
    const T             *src = static_cast<const T *>(a.src);
    T                   *dst = static_cast<T *>(a.dst);
    constexpr int        N3  = N * N * N;
    if (a.kind == 0)
      {
        HeatQOp<T> op;
        for (int d = 0; d < 3; ++d)
          op.kd[d] = conv_host<T>(a.kdt / (g.h[d] * g.h[d]));
        return run_apply_c<N, T, T, 1>(a, sh, cg, op, src, dst, s);
      }
    const NHMat<T> m     = to_mat<T>(a.mat);
    const T       *cache = static_cast<const T *>(a.cache);
    switch (a.var)
      {
        case V_SCALAR_REF:
          {
            NHScalarRefQOp<T> op;
            op.ucell  = static_cast<const T *>(a.ucell);
            op.scalar = cache;
            op.m      = m;
            op.n3     = N3;
            return run_apply_c<N, T, T, 3>(a, sh, cg, op, src, dst, s);
          }
        case V_QP10:
          {
            NHQp10QOp<T> op;
            op.cache = cache;
            op.m     = m;
            op.n3    = N3;
            for (int d = 0; d < 3; ++d)
              op.mu_d[d] = conv_host<T>(a.mat.mu / (g.h[d] * g.h[d]));
            return run_apply_c<N, T, T, 3>(a, sh, cg, op, src, dst, s);
          }
        case V_TENSOR2:
          {
            NHCachedQOp<T, V_TENSOR2> op;
            op.cache = cache;
            op.m     = m;
            op.n3    = N3;
            return run_apply_c<N, T, T, 3>(a, sh, cg, op, src, dst, s);
          }
        case V_TENSOR4:
          {
            NHCachedQOp<T, V_TENSOR4> op;
            op.cache = cache;
            op.m     = m;
            op.n3    = N3;
            return run_apply_c<N, T, T, 3>(a, sh, cg, op, src, dst, s);
          }
        case V_TENSOR4_NS:
          {
            NHCachedQOp<T, V_TENSOR4_NS> op;
            op.cache = cache;
            op.m     = m;
            op.n3    = N3;
            return run_apply_c<N, T, T, 3>(a, sh, cg, op, src, dst, s);
          }
        case V_FORM0:
          {
            NHCachedQOp<T, V_FORM0> op;
            op.cache = cache;
            op.m     = m;
            op.n3    = N3;
            return run_apply_c<N, T, T, 3>(a, sh, cg, op, src, dst, s);
          }
      }
    return cudaErrorInvalidValue;
  }

  template <int N, typename T>
  cudaError_t
  launch_nh_cache(const HostBasis &b, const LevelGeom &g, int var,
                  const NHMatD &md, const void *u, void *cache, void *ucell,
                  int *err, cudaStream_t s)
  {
    const Shape<N, T>  sh   = make_shape<N, T>(b);
    const CellGeom<T>  cg   = make_cell_geom<T>(g);
    const NHMat<T>     m    = to_mat<T>(md);
    constexpr int      CPB  = cells_per_block<N, 3, T>();
    const size_t       smem = size_t(CPB) * smem_per_cell<N, 3, false>() * sizeof(T);
    const unsigned     grid = (cg.n_cells + CPB - 1) / CPB;
    const T           *uu   = static_cast<const T *>(u);
    T                 *cp   = static_cast<T *>(cache);
    T                 *uc   = static_cast<T *>(ucell);
    cudaError_t        e    = cudaSuccess;
#define MF_CACHE_CASE(V)                                                      \
  case V:                                                                     \
    {                                                                         \
      auto k = nh_cache_kernel<N, T, V>;                                      \
      if ((e = prepare(k, smem)) != cudaSuccess)                              \
        return e;                                                             \
      k<<<grid, CPB * N * N, smem, s>>>(sh, cg, m, uu, cp, uc, err);          \
      return cudaGetLastError();                                              \
    }
    switch (var)
      {
        MF_CACHE_CASE(V_SCALAR_REF)
        MF_CACHE_CASE(V_TENSOR2)
        MF_CACHE_CASE(V_TENSOR4)
        MF_CACHE_CASE(V_TENSOR4_NS)
        MF_CACHE_CASE(V_QP10)
        MF_CACHE_CASE(V_FORM0)
      }
#undef MF_CACHE_CASE
    return cudaErrorInvalidValue;
  }

  template <int N, typename T>
  cudaError_t
  launch_diag(const HostBasis &b, const LevelGeom &g, int kind,
              const NHMatD &md, double kdt, const void *u, void *diag,
              cudaStream_t s)
  {
    const Shape<N, T>  sh = make_shape<N, T>(b);
    DiagShape<N, T>    ds;
    for (int q = 0; q < N; ++q)
      for (int i = 0; i < N; ++i)
        {
          const double sv = b.S[q * N + i], gv = b.G[q * N + i];
          ds.SS[q * N + i] = T(sv * sv);
          ds.SG[q * N + i] = T(sv * gv);
          ds.GG[q * N + i] = T(gv * gv);
        }
    for (int i = 0; i < N; ++i)
      ds.w[i] = T(b.w[i]);
    const CellGeom<T> cg   = make_cell_geom<T>(g);
    const NHMat<T>    m    = to_mat<T>(md);
    constexpr int     CPB  = cells_per_block<N, 3, T>();
    constexpr int     N3   = N * N * N;
    const unsigned    grid = (cg.n_cells + CPB - 1) / CPB;
    const T          *uu   = static_cast<const T *>(u);
    T                *dg   = static_cast<T *>(diag);
    cudaError_t       e;
#define MF_DIAG_CASE(K)                                                       \
  case K:                                                                     \
    {                                                                         \
      const size_t smem = size_t(CPB) * ((K == 0 ? 0 : 12 * N3) + 9 * N3) * sizeof(T); \
      auto         k    = diag_kernel<N, T, K>;                               \
      if ((e = prepare(k, smem)) != cudaSuccess)                              \
        return e;                                                             \
      k<<<grid, CPB * N * N, smem, s>>>(sh, ds, cg, m, T(kdt), uu, dg);      \
      return cudaGetLastError();                                              \
    }
    switch (kind)
      {
        MF_DIAG_CASE(0)
        MF_DIAG_CASE(1)
        MF_DIAG_CASE(2)
      }
#undef MF_DIAG_CASE
    return cudaErrorInvalidValue;
  }

  template <int N>
  cudaError_t
  launch_residual(const HostBasis &b, const LevelGeom &g, int form,
                  const NHMatD &md, double rho, const double *body,
                  const double *u, const double *acc, double *rhs,
                  cudaStream_t s)
  {
    const Shape<N, double>    sh   = make_shape<N, double>(b);
    const CellGeom<double>    cg   = make_cell_geom<double>(g);
    const NHMat<double>       m    = to_mat<double>(md);
    constexpr int             CPB  = cells_per_block<N, 3, double>();
    constexpr int             N3   = N * N * N;
    const size_t              smem = size_t(CPB) * (smem_per_cell<N, 3, false>() + 3 * N3) * sizeof(double);
    const unsigned            grid = (cg.n_cells + CPB - 1) / CPB;
    cudaError_t               e;
    if (form == 1)
      {
        auto k = residual_kernel<N, double, 1>;
        if ((e = prepare(k, smem)) != cudaSuccess)
          return e;
        k<<<grid, CPB * N * N, smem, s>>>(sh, cg, m, rho, body[0], body[1], body[2], u, acc, rhs);
      }
    else
      {
        auto k = residual_kernel<N, double, 0>;
        if ((e = prepare(k, smem)) != cudaSuccess)
          return e;
        k<<<grid, CPB * N * N, smem, s>>>(sh, cg, m, rho, body[0], body[1], body[2], u, acc, rhs);
      }
    return cudaGetLastError();
  }

  template <int N>
  cudaError_t
  launch_heat_rhs(const HostBasis &b, const LevelGeom &g, double dt,
                  const SourceDesc &f, const double *u_old, double *rhs,
                  double *tab, cudaStream_t s)
  {
    const Shape<N, double>  sh = make_shape<N, double>(b);
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
    sd.N = N;
    sd.J = 0;
    for (int d = 0; d < 3; ++d)
      {
        sd.C[d] = g.C[d];
        sd.J    = std::max(sd.J, g.C[d] * N);
      }
    if (sd.n_gauss < 0 || sd.n_gauss > 8 || !tab)
      return cudaErrorInvalidValue;
    if (sd.n_gauss > 0)
      {
        const int total = sd.n_gauss * 3 * sd.J;
        heat_source_table_kernel<<<(total + 255) / 256, 256, 0, s>>>(sd, tab);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
          return e;
      }
    constexpr int  CPB  = cells_per_block<N, 1, double>();
    const size_t   smem = size_t(CPB) * smem_per_cell<N, 1, false>() * sizeof(double);
    const unsigned grid = (cg.n_cells + CPB - 1) / CPB;
    auto           k    = heat_rhs_kernel<N>;
    cudaError_t    e    = prepare(k, smem);
    if (e != cudaSuccess)
      return e;
    k<<<grid, CPB * N * N, smem, s>>>(sh, cg, sd, dt, u_old, rhs, tab);
    return cudaGetLastError();
  }

  template cudaError_t launch_apply<MF_N, double>(const HostBasis &, const LevelGeom &, const ApplyArgs &, cudaStream_t);
  template cudaError_t launch_apply<MF_N, float>(const HostBasis &, const LevelGeom &, const ApplyArgs &, cudaStream_t);
  template cudaError_t launch_nh_cache<MF_N, double>(const HostBasis &, const LevelGeom &, int, const NHMatD &, const void *, void *, void *, int *, cudaStream_t);
  template cudaError_t launch_nh_cache<MF_N, float>(const HostBasis &, const LevelGeom &, int, const NHMatD &, const void *, void *, void *, int *, cudaStream_t);
  template cudaError_t launch_diag<MF_N, double>(const HostBasis &, const LevelGeom &, int, const NHMatD &, double, const void *, void *, cudaStream_t);
  template cudaError_t launch_diag<MF_N, float>(const HostBasis &, const LevelGeom &, int, const NHMatD &, double, const void *, void *, cudaStream_t);
  template cudaError_t launch_residual<MF_N>(const HostBasis &, const LevelGeom &, int, const NHMatD &, double, const double *, const double *, const double *, double *, cudaStream_t);
  template cudaError_t launch_heat_rhs<MF_N>(const HostBasis &, const LevelGeom &, double, const SourceDesc &, const double *, double *, double *, cudaStream_t);
  template <int N>
  cudaError_t
  launch_apply_df(const HostBasis &b, const LevelGeom &g, const ApplyArgs &a,
                  cudaStream_t s)
  {
    const ShapeA<N, df64>   sh  = make_shape_apply<N, df64>(b, g);
    const CellGeom<df64>    cg  = apply_range(make_cell_geom<df64>(g), a);
    const double           *src = static_cast<const double *>(a.src);
    double                 *dst = static_cast<double *>(a.dst);
    constexpr int           N3  = N * N * N;
    if (a.kind == 0)
      {
        HeatQOp<df64> op;
        for (int d = 0; d < 3; ++d)
          op.kd[d] = conv_host<df64>(a.kdt / (g.h[d] * g.h[d]));
        return run_apply_c<N, double, df64, 1>(a, sh, cg, op, src, dst, s);
      }
    if (a.var != V_QP10)
      return cudaErrorInvalidValue;
    NHQp10QOp<df64> op;
    op.cache = static_cast<const df64 *>(a.cache);
    op.m     = to_mat<df64>(a.mat);
    op.n3    = N3;
    for (int d = 0; d < 3; ++d)
      op.mu_d[d] = conv_host<df64>(a.mat.mu / (g.h[d] * g.h[d]));
    return run_apply_c<N, double, df64, 3>(a, sh, cg, op, src, dst, s);
  }

  template <int N>
  cudaError_t
  launch_nh_cache_df(const HostBasis &b, const LevelGeom &g, const NHMatD &md,
                     const double *u, void *cache, int *err, cudaStream_t s)
  {
    const Shape<N, double>  sh   = make_shape<N, double>(b);
    const CellGeom<double>  cg   = make_cell_geom<double>(g);
    const NHMat<double>     m    = to_mat<double>(md);
    constexpr int           CPB  = cells_per_block<N, 3, double>();
    const size_t            smem = size_t(CPB) * smem_per_cell<N, 3, false>() * sizeof(double);
    const unsigned          grid = (cg.n_cells + CPB - 1) / CPB;
    auto                    k    = nh_cache_kernel<N, double, V_QP10, df64>;
    cudaError_t             e    = prepare(k, smem);
    if (e != cudaSuccess)
      return e;
    k<<<grid, CPB * N * N, smem, s>>>(sh, cg, m, u, static_cast<df64 *>(cache), nullptr, err);
    return cudaGetLastError();
  }

  template cudaError_t launch_apply_df<MF_N>(const HostBasis &, const LevelGeom &, const ApplyArgs &, cudaStream_t);
  template cudaError_t launch_nh_cache_df<MF_N>(const HostBasis &, const LevelGeom &, const NHMatD &, const double *, void *, int *, cudaStream_t);
} // namespace mfgpu
