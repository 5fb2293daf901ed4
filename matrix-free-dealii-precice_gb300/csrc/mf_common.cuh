// Shared definitions of the GB300 matrix-free library: level geometry,
// 1D shape matrices, error reporting.
//
// Data layout in HBM (one multigrid level):
//   * structured box of C[0] x C[1] x C[2] hexahedral cells with uniform cell
//     size h[d] (subdivided_hyper_rectangle + refine_global, the meshes of the
//     reference's cases, include/cases/elasticity/turek_hron.h:23-45);
//   * continuous Q_p nodes on Gauss-Lobatto points (FE_Q(p)), numbered
//     lexicographically on the global node grid Nn[d] = C[d]*p + 1 (x fastest);
//   * vector fields component-blocked: dof = comp * n_nodes + node;
//   * homogeneous Dirichlet constraints given per box face (x-,x+,y-,y+,z-,z+)
//     as a component bitmask, so no constraint index lists are stored.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "mf_df64.cuh"

namespace mfgpu
{
  constexpr int MAX_N = 7; // degree 6

  struct LevelGeom
  {
    int      dim; // 2: one node plane, C[2] = Nn[2] = 1, h[2] = 1
    int      C[3];
    int      Nn[3];
    int      p;
    size_t   n_nodes;
    size_t   n_cells;
    double   h[3];
    double   lo[3];
    unsigned face_mask[6];
  };

  // 1D matrices for a degree, in the compute precision T:
  //   S[q][i]  Gauss-Lobatto Lagrange basis at Gauss point q   (N x N)
  //   D[q][r]  collocation derivative on the Gauss points      (N x N)
  //   w[q]     Gauss weights on [0,1]
  template <int N, typename T>
  struct Shape
  {
    T S[N * N];
    T D[N * N];
    T w[N];
  };

  // Even-odd form of an N x N matrix M with M[N-1-r][N-1-k] = SIG M[r][k]
  // (SIG = +1: the interpolation S from the Gauss-Lobatto nodes to the
  // Gauss points, both symmetric about the cell centre; SIG = -1: the
  // collocation derivative D).  With H = N/2 and HR = (N+1)/2:
  //   e[r][k] = (M[r][k] + M[r][N-1-k]) / 2,  o[r][k] = (M[r][k] - M[r][N-1-k]) / 2
  // for r < HR, k < H, and e[r][H] = M[r][H] for odd N.  M and M^T then
  // apply with about half the products (see eo_apply in the cell kernels).
  template <int N, typename T, int SIG>
  struct EO
  {
    static constexpr int H = N / 2, HR = (N + 1) / 2;
    T                    e[HR * HR];
    T                    o[HR * H];
  };

  // shape data of the operator-application kernels: the collocation
  // derivative per direction already divided by the cell size h_d, so the
  // gradients come out in real coordinates; the same matrices in even-odd
  // form for the 1D sweeps
  template <int N, typename T>
  struct ShapeA
  {
    T S[N * N];
    T D[3][N * N];
    T Du[N * N]; // unscaled (reference-cell) derivative matrix
    T w[N];
    EO<N, T, 1>  Se;
    EO<N, T, -1> De[3];
    EO<N, T, -1> Due;
  };

  // unsigned division by a divisor fixed per level (the cells per row and
  // per layer), for dividends below 2^31: n / d = (umulhi(n, mul) + n) >>
  // shift with shift = ceil(log2 d), mul = floor(2^32 (2^shift - d) / d) + 1
  // (the round-up method of Granlund and Montgomery, "Division by invariant
  // integers using multiplication", 1994).  Replaces the integer division
  // sequence that a runtime divisor costs in every cell kernel thread.
  struct FastDiv
  {
    unsigned d, mul, shift;
    __host__ __device__ __forceinline__ unsigned
    div(unsigned n) const
    {
#ifdef __CUDA_ARCH__
      return (__umulhi(n, mul) + n) >> shift;
#else
      return unsigned(((unsigned long long)(n) * mul >> 32) + n) >> shift;
#endif
    }
    __host__ __device__ __forceinline__ unsigned
    mod(unsigned n) const
    {
      return n - div(n) * d;
    }
  };

  inline FastDiv
  make_fastdiv(unsigned d)
  {
    FastDiv f;
    f.d     = d;
    f.shift = 0;
    while ((1ull << f.shift) < d)
      ++f.shift;
    f.mul = unsigned(((1ull << 32) * ((1ull << f.shift) - d)) / d + 1);
    return f;
  }

  // geometry of a level as seen by a cell kernel, in precision T
  template <typename T>
  struct CellGeom
  {
    int      C[3];
    int      Nn[3];
    int      p;
    unsigned n_cells;
    unsigned cell_begin, cell_end; // cells [begin, end) of one application launch
    // parity colour of a coloured application launch (-1: all cells, atomic
    // scatter): cells (2i+px, 2j+py, 2k+pz), colour = px + 2 py + 4 pz, hc[d]
    // cells per direction, color_n = hc[0]*hc[1]*hc[2]
    int      color;
    unsigned color_n;
    int      hc[3];
    size_t   n_nodes;
    T        inv_h[3];
    T        vol; // h0*h1*h2
    unsigned face_mask[6];
    // a batch of problems on this level (same operator, different vectors):
    // problem blockIdx.y reads src and writes dst at offset blockIdx.y * bstride
    unsigned batch;
    size_t   bstride;
    // C[0] and C[1] as fast divisors: cell -> (x, y, z)
    FastDiv  dC0, dC1;
    // element-column launches: row stride of the dense matrix (0: NC n_nodes)
    size_t   unit_ld;
  };

  // host-side conversion of a double constant to a compute type
  template <typename T>
  inline T
  conv_host(double v)
  {
    return T(v);
  }
  template <>
  inline df64
  conv_host<df64>(double v)
  {
    return df_from_double_host(v);
  }

  template <typename T>
  inline CellGeom<T>
  make_cell_geom(const LevelGeom &g)
  {
    CellGeom<T> c;
    for (int d = 0; d < 3; ++d)
      {
        c.C[d]     = g.C[d];
        c.Nn[d]    = g.Nn[d];
        c.inv_h[d] = conv_host<T>(1.0 / g.h[d]);
      }
    c.p       = g.p;
    c.batch   = 1;
    c.bstride = 0;
    c.unit_ld = 0;
    c.n_cells    = unsigned(g.n_cells);
    c.cell_begin = 0;
    c.cell_end   = unsigned(g.n_cells);
    c.color      = -1;
    c.color_n    = 0;
    c.hc[0] = c.hc[1] = c.hc[2] = 0;
    c.n_nodes    = g.n_nodes;
    c.vol     = conv_host<T>(g.h[0] * g.h[1] * g.h[2]);
    c.dC0     = make_fastdiv(unsigned(g.C[0]));
    c.dC1     = make_fastdiv(unsigned(g.C[1]));
    for (int f = 0; f < 6; ++f)
      c.face_mask[f] = g.face_mask[f];
    return c;
  }

  // cells of parity colour `color` per direction (hc) and in total
  inline unsigned
  color_cells(const int *C, int color, int *hc)
  {
    unsigned n = 1;
    for (int d = 0; d < 3; ++d)
      {
        const int p = (color >> d) & 1;
        hc[d]       = (C[d] - p + 1) / 2;
        n *= unsigned(hc[d] > 0 ? hc[d] : 0);
      }
    return n;
  }

  // J - 1 = det(I + H) - 1 from the displacement gradient H = Grad u,
  // without forming det F: the principal invariants of H, tr H + (sum of
  // its principal 2x2 minors) + det H.  det F - 1 loses the relative
  // accuracy of a small strain to cancellation; this form keeps it, and
  // ln J = log1p(J - 1) follows.  The reference evaluates
  // std::log(determinant(F)) (mf_nh_operator.h:448,457).
  template <typename T>
  __host__ __device__ inline T
  jm1_from_grad3(const T (&H)[3][3])
  {
    const T i1 = H[0][0] + H[1][1] + H[2][2];
    const T i2 = (H[0][0] * H[1][1] - H[0][1] * H[1][0]) +
                 (H[0][0] * H[2][2] - H[0][2] * H[2][0]) +
                 (H[1][1] * H[2][2] - H[1][2] * H[2][1]);
    const T i3 = H[0][0] * (H[1][1] * H[2][2] - H[1][2] * H[2][1]) -
                 H[0][1] * (H[1][0] * H[2][2] - H[1][2] * H[2][0]) +
                 H[0][2] * (H[1][0] * H[2][1] - H[1][1] * H[2][0]);
    return i1 + (i2 + i3);
  }

  // the same in two dimensions: det(I + H) - 1 = tr H + det H
  template <typename T>
  __host__ __device__ inline T
  jm1_from_grad2(const T (&H)[2][2])
  {
    return (H[0][0] + H[1][1]) + (H[0][0] * H[1][1] - H[0][1] * H[1][0]);
  }

  // component mask of the Dirichlet constraints on node (ix,iy,iz)
  __host__ __device__ inline unsigned
  node_mask(const unsigned *fm, const int *Nn, int ix, int iy, int iz)
  {
    unsigned m = 0;
    m |= (ix == 0) ? fm[0] : 0u;
    m |= (ix == Nn[0] - 1) ? fm[1] : 0u;
    m |= (iy == 0) ? fm[2] : 0u;
    m |= (iy == Nn[1] - 1) ? fm[3] : 0u;
    m |= (iz == 0) ? fm[4] : 0u;
    m |= (iz == Nn[2] - 1) ? fm[5] : 0u;
    return m;
  }

  // status codes of the C-ABI
  enum Status
  {
    OK               = 0,
    ERR_ARG          = 1,
    ERR_CUDA         = 2,
    ERR_OOM          = 3,
    ERR_NONFINITE    = 4,
    ERR_NOT_CONVERGED = 5,
    ERR_STATE        = 6,
    ERR_DET_F        = 7,
    ERR_UNSUPPORTED  = 8,
    ERR_TIMEOUT      = 9
  };
  // neo-Hookean caching variants and the cached fields per quadrature point
  enum NHVariant
  {
    V_SCALAR_REF = 0,
    V_TENSOR2    = 1,
    V_TENSOR4    = 2,
    V_TENSOR4_NS = 3,
    V_QP10       = 4,
    V_FORM0      = 5
  };

  __host__ __device__ constexpr int
  nh_cache_fields(int v)
  {
    return v == V_SCALAR_REF ? 1 :
           v == V_TENSOR2    ? 18 :
           v == V_TENSOR4    ? 53 :
           v == V_TENSOR4_NS ? 81 :
           v == V_QP10       ? 10 :
                               20;
  }

} // namespace mfgpu
