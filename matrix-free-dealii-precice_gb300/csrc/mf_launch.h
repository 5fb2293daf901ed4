// Host-side launch interface of the cell kernels (instantiated per degree
// in mf_kernels.cu, one translation unit per N = p+1).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "mf_common.cuh"

namespace mfgpu
{
  // 1D data of one degree on the host, double precision
  struct HostBasis
  {
    int    N = 0;
    double nodes[MAX_N];      // Gauss-Lobatto support points on [0,1]
    double xq[MAX_N];         // Gauss points on [0,1]
    double w[MAX_N];          // Gauss weights
    double S[MAX_N * MAX_N];  // [q][i] nodal basis at Gauss points
    double D[MAX_N * MAX_N];  // [q][r] collocation derivative on Gauss points
    double G[MAX_N * MAX_N];  // [q][i] derivative of nodal basis at Gauss points
    double Ge[2][MAX_N];      // derivative of nodal basis at 0 and 1
  };

  void make_host_basis(int degree, HostBasis &b);

  struct NHMatD
  {
    double mu, lambda, rho_alpha, kappa, c_1;
  };

  // operator application: dst += A src (cell part only)
  //   kind 0: heat (param kdt); kind 1: neo-Hookean with variant var
  struct ApplyArgs
  {
    int         kind;
    int         var;
    bool        constrained;
    double      kdt;
    NHMatD      mat;
    const void *cache;
    const void *ucell;
    const void *src;
    void       *dst;
    size_t      cell_begin = 0, cell_end = 0; // cell range; empty = all cells
    bool        colored = false; // all cells by parity colour, plain (non-atomic) scatter
    // element columns: dst is the dense row-major matrix of m = NC n_nodes
    // rows (row stride unit_ld, zeroed by the caller) and receives the
    // operator's entries of the unconstrained rows and columns; src is not
    // read
    bool        unit = false;
    // row stride of that matrix in elements (0: m); padded so that every
    // row starts on a 16-byte boundary
    size_t      unit_ld = 0;
    // cell kernel: 0 by grid size (point-parallel below POINT_CELLS cells),
    // 1 line-parallel (cell_apply_kernel), 2 point-parallel
    int         kernel = 0;
    // a batch of problems sharing the operator: vectors of `batch` blocks of
    // `bstride` entries, all blocks in one launch (grid.y = batch)
    int         batch   = 1;
    size_t      bstride = 0;
  };

  // the heat operator as a batched-cell product with its element matrix on
  // the tensor cores (FP32, three-dimensional, N = 2..6; mf_heat_em.cu):
  // the matrix in the kernel's layout, and dst += A src over all cells
  bool        heat_em_supported(int N);
  size_t      heat_em_matrix(const HostBasis &b, const LevelGeom &g, double kdt, std::vector<unsigned char> &out);
  cudaError_t launch_heat_em(const HostBasis &b, const LevelGeom &g, bool constrained, const void *bmat,
                             const float *src, float *dst, int *err, cudaStream_t s);

  // the heat operator in its tensor-product form (1D mass and stiffness
  // matrices, 7 sweeps per cell; mf_heat_tp.cu), N = 2..7, FP32 and FP64
  // (native, or double-float in the block form):
  // one thread per column segment of zlen cells in registers (N = 2 from
  // 16384 cells on), N^2 threads per cell through shared memory (otherwise),
  // or, on request,
  // for FP32 N = 2..3 over all cells bricks staged in shared memory by TMA;
  // three-dimensional levels; dst += A src over the cells of z-planes
  // [zc0, zc1), grid.y = problem of a batch
  struct HeatTPArgs
  {
    double      kdt;
    bool        constrained;
    int         zc0, zc1, zlen;
    const void *src;
    void       *dst;
    int         batch   = 1;
    size_t      bstride = 0;
    // FP32 Q1-Q2 over all cells: the bricks staged by TMA instead of the
    // register kernel (measured slower; opt-in); err receives the bounded
    // waits' timeout flag (8)
    bool        tma = false;
    int        *err = nullptr;
    // FP64 vectors in double-float arithmetic (the block kernel)
    bool        df64 = false;
  };
  bool        heat_tp_supported(int N, int precision);
  // the assembled heat operator's diagonal on a box level from the 1D
  // element diagonals (out = diag for every node; constrained rows are the
  // caller's), FP32 or FP64 out
  cudaError_t launch_heat_diag_tp(const HostBasis &b, const LevelGeom &g, int precision, double kdt, void *out,
                                  cudaStream_t s);
  int         heat_tp_zlen(const LevelGeom &g, int zc0, int zc1, int N, int precision);
  cudaError_t launch_heat_tp(const HostBasis &b, const LevelGeom &g, int precision, const HeatTPArgs &a,
                             cudaStream_t s);
  // launches of fewer cells than this keep the point-parallel kernel for
  // the heat operator instead of the tensor-product one
  constexpr unsigned TP_MIN_CELLS = 512;

  // launches of fewer cells than this take the point-parallel kernel
  // (native FP64: up to 4096 cells; the native FP64 referential_qp tangent
  // at every size but Q2)
  constexpr unsigned POINT_CELLS = 1024;

  template <int N, typename T>
  cudaError_t launch_apply(const HostBasis &b, const LevelGeom &g,
                           const ApplyArgs &a, cudaStream_t s);

  // FP64 storage, double-float (float pair) arithmetic: heat and the
  // referential_qp tangent
  template <int N>
  cudaError_t launch_apply_df(const HostBasis &b, const LevelGeom &g,
                              const ApplyArgs &a, cudaStream_t s);
  template <int N>
  cudaError_t launch_nh_cache_df(const HostBasis &b, const LevelGeom &g,
                                 const NHMatD &m, const double *u, void *cache,
                                 int *err, cudaStream_t s);

  template <int N, typename T>
  cudaError_t launch_nh_cache(const HostBasis &b, const LevelGeom &g, int var,
                              const NHMatD &m, const void *u, void *cache,
                              void *ucell, int *err, cudaStream_t s);

  // kind 0 heat, 1 NH formulation 1, 2 NH formulation 0; diag += local diags
  template <int N, typename T>
  cudaError_t launch_diag(const HostBasis &b, const LevelGeom &g, int kind,
                          const NHMatD &m, double kdt, const void *u,
                          void *diag, cudaStream_t s);

  template <int N>
  cudaError_t launch_residual(const HostBasis &b, const LevelGeom &g, int form,
                              const NHMatD &m, double rho, const double *body,
                              const double *u, const double *acc, double *rhs,
                              cudaStream_t s);

  // heat right-hand side: rhs += int (u_old + dt f) v, f = constant +
  // sum of Gaussians
  struct SourceDesc
  {
    double constant;
    int    n_gauss;
    double center[8][3];
    double width[8];
    double amp[8];
  };

  // tab: device scratch of heat_rhs_table_size(g, N) doubles (the
  // per-direction factors of the Gaussians at the quadrature coordinates)
  template <int N>
  cudaError_t launch_heat_rhs(const HostBasis &b, const LevelGeom &g, double dt,
                              const SourceDesc &f, const double *u_old,
                              double *rhs, double *tab, cudaStream_t s);
  inline size_t
  heat_rhs_table_size(const LevelGeom &g, int N)
  {
    int j = 0;
    for (int d = 0; d < 3; ++d)
      j = g.C[d] * N > j ? g.C[d] * N : j;
    return size_t(8) * 3 * size_t(j);
  }

  // two-dimensional kernels (mf_kernels2d.cu); N = p+1, precision 32 / 64
  cudaError_t launch_apply2d(int N, int precision, const HostBasis &b, const LevelGeom &g,
                             const ApplyArgs &a, cudaStream_t s);
  cudaError_t launch_nh_cache2d(int N, int precision, const HostBasis &b, const LevelGeom &g, int form,
                                const NHMatD &m, const void *u, void *cache, int *err, cudaStream_t s);
  // kind: 0 heat (kdt), 1 neo-Hookean formulation 1, 2 formulation 0 (from the cache)
  cudaError_t launch_diag2d(int N, int precision, const HostBasis &b, const LevelGeom &g, int kind,
                            const NHMatD &m, double kdt, const void *cache, void *diag, cudaStream_t s);
  cudaError_t launch_residual2d(int N, const HostBasis &b, const LevelGeom &g, int form, const NHMatD &m,
                                double rho, const double *body, const double *u, const double *acc,
                                double *rhs, cudaStream_t s);
  cudaError_t launch_heat_rhs2d(int N, const HostBasis &b, const LevelGeom &g, double dt,
                                const SourceDesc &f, const double *u_old, double *rhs, cudaStream_t s);
} // namespace mfgpu
