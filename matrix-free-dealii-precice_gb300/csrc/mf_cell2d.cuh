// Two-dimensional (dim = 2) kernels: the reference's own test cases
// (tests/solid/*: 2D turek_hron flap; tests/heat/*: 2D partitioned heat).
//
// One thread block takes CPB2 cells with N threads per cell; thread l of a
// cell owns the x-line y = l and the y-line x = l of every sweep.  Cell
// arrays (N^2 values, element (a, b) at a + N b) live in shared memory.
// Evaluation follows the 3D kernels (collocation: S along x and y, then the
// collocation derivative D on the Gauss points); gradients are in real
// coordinates (D divided by h per direction).  The quadrature-point
// operators restate the reference's formulas for dim = 2
// (include/solid_mechanics/mf_nh_operator.h, material.h,
// include/heat_transfer/heat_transfer.h:236-250).
#pragma once

#include "mf_cell.cuh"

namespace mfgpu
{
  template <int N>
  __host__ __device__ constexpr int
  cpb2d()
  {
    return 128 / N;
  }

  // x-interpolation of the gathered x-row (registers) to G0 (scratch), then
  // y-interpolation (V) and y-derivative (G1) on y-lines, then the
  // x-derivative (G0) on x-lines.  Ends without a barrier.
  template <int N, typename T>
  __device__ __forceinline__ void
  eval2(const T *S, const T *Dx, const T *Dy, const T (&row)[N], T *V, T *G0, T *G1, int l,
        bool grad)
  {
    T x[N], y[N];
    mat_apply<N>(S, row, y);
#pragma unroll
    for (int a = 0; a < N; ++a)
      G0[a + N * l] = y[a];
    __syncthreads();
#pragma unroll
    for (int b = 0; b < N; ++b)
      x[b] = G0[l + N * b];
    mat_apply<N>(S, x, y);
#pragma unroll
    for (int b = 0; b < N; ++b)
      V[l + N * b] = y[b];
    if (grad)
      {
        mat_apply<N>(Dy, y, x);
#pragma unroll
        for (int b = 0; b < N; ++b)
          G1[l + N * b] = x[b];
      }
    __syncthreads();
    if (grad)
      {
#pragma unroll
        for (int a = 0; a < N; ++a)
          x[a] = V[a + N * l];
        mat_apply<N>(Dx, x, y);
#pragma unroll
        for (int a = 0; a < N; ++a)
          G0[a + N * l] = y[a];
      }
  }

  // nodal result S^T S^T (V + Dx^T G0 + Dy^T G1) as the y-line x = l in
  // registers; V and G0 are overwritten.  Starts with a barrier.
  template <int N, typename T>
  __device__ __forceinline__ void
  integ2(const T *S, const T *Dx, const T *Dy, T *V, T *G0, const T *G1, int l, bool grad,
         T (&col)[N])
  {
    T x[N], y[N];
    __syncthreads();
    if (grad)
      {
#pragma unroll
        for (int b = 0; b < N; ++b)
          {
            x[b] = G1[l + N * b];
            y[b] = V[l + N * b];
          }
        mat_apply_t_add<N>(Dy, x, y);
#pragma unroll
        for (int b = 0; b < N; ++b)
          V[l + N * b] = y[b];
        __syncthreads();
      }
#pragma unroll
    for (int a = 0; a < N; ++a)
      {
        y[a] = V[a + N * l];
        x[a] = grad ? G0[a + N * l] : zero<T>();
      }
    if (grad)
      mat_apply_t_add<N>(Dx, x, y);
    mat_apply_t<N>(S, y, x);
#pragma unroll
    for (int a = 0; a < N; ++a)
      G0[a + N * l] = x[a];
    __syncthreads();
#pragma unroll
    for (int b = 0; b < N; ++b)
      x[b] = G0[l + N * b];
    mat_apply_t<N>(S, x, col);
  }

  // ---------------------------------------------------------------------
  // operator application: dst += A src (constrained rows: dst += src)
  // QOp2: operator()(cell, q, T (&v)[NC], T (&H)[NC][2]) on real gradients
  // ---------------------------------------------------------------------
  template <int N, typename T, int NC, class QOp, bool CONSTRAINED>
  __global__ void __launch_bounds__(cpb2d<N>() * N)
  cell_apply2d_kernel(const __grid_constant__ ShapeA<N, T> sh, const __grid_constant__ CellGeom<T> g,
                      const QOp op, const T *__restrict__ src, T *__restrict__ dst)
  {
    constexpr int N2  = N * N;
    constexpr int CPB = cpb2d<N>();
    constexpr int SPC = NC * 3 * N2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T             *cb     = reinterpret_cast<T *>(smem_raw) + (threadIdx.x / N) * SPC;
    const int      l      = threadIdx.x % N;
    const unsigned cell   = g.cell_begin + blockIdx.x * CPB + threadIdx.x / N;
    const bool     active = cell < g.cell_end;
    const unsigned cc     = active ? cell : 0u;
    const int      cx = int(cc % unsigned(g.C[0])), cy = int(cc / unsigned(g.C[0]));
#pragma unroll 1
    for (int c = 0; c < NC; ++c)
      {
        T row[N];
#pragma unroll
        for (int a = 0; a < N; ++a)
          {
            T         v  = zero<T>();
            const int ix = cx * g.p + a, iy = cy * g.p + l;
            if (active && !(CONSTRAINED && ((node_mask_g(g, ix, iy, 0) >> c) & 1u)))
              v = __ldg(src + size_t(c) * g.n_nodes + size_t(ix) + size_t(g.Nn[0]) * size_t(iy));
            row[a] = v;
          }
        T *V = cb + c * 3 * N2;
        eval2<N>(sh.S, sh.D[0], sh.D[1], row, V, V + N2, V + 2 * N2, l, true);
      }
    __syncthreads();
    if (active)
      {
#pragma unroll 1
        for (int a = 0; a < N; ++a)
          {
            const int q = a + N * l;
            T         v[NC], H[NC][2];
#pragma unroll
            for (int c = 0; c < NC; ++c)
              {
                v[c]    = cb[c * 3 * N2 + q];
                H[c][0] = cb[c * 3 * N2 + N2 + q];
                H[c][1] = cb[c * 3 * N2 + 2 * N2 + q];
              }
            op(cell, q, v, H);
            const T jxw = sh.w[a] * sh.w[l] * g.vol;
#pragma unroll
            for (int c = 0; c < NC; ++c)
              {
                cb[c * 3 * N2 + q]          = v[c] * jxw;
                cb[c * 3 * N2 + N2 + q]     = H[c][0] * jxw;
                cb[c * 3 * N2 + 2 * N2 + q] = H[c][1] * jxw;
              }
          }
      }
#pragma unroll 1
    for (int c = 0; c < NC; ++c)
      {
        T *V = cb + c * 3 * N2;
        T  col[N];
        integ2<N>(sh.S, sh.D[0], sh.D[1], V, V + N2, V + 2 * N2, l, true, col);
        if (!active)
          continue;
#pragma unroll
        for (int b = 0; b < N; ++b)
          {
            const int    ix = cx * g.p + l, iy = cy * g.p + b;
            const size_t gi = size_t(c) * g.n_nodes + size_t(ix) + size_t(g.Nn[0]) * size_t(iy);
            if (CONSTRAINED && ((node_mask_g(g, ix, iy, 0) >> c) & 1u))
              {
                // constrained row: dst += src by the owner cell of the node
                if ((l < g.p || cx == g.C[0] - 1) && (b < g.p || cy == g.C[1] - 1))
                  dst[gi] += __ldg(src + gi);
                continue;
              }
            atomicAdd(dst + gi, col[b]);
          }
      }
  }

  // ---------------------------------------------------------------------
  // quadrature-point operators (dim = 2)
  // ---------------------------------------------------------------------
  // heat: mass + dt k Laplace
  template <typename T>
  struct Heat2QOp
  {
    T kdt;
    __device__ __forceinline__ void
    operator()(unsigned, int, T (&)[1], T (&H)[1][2]) const
    {
      H[0][0] *= kdt;
      H[0][1] *= kdt;
    }
  };

  // neo-Hookean, formulation 1, every caching variant (the same tangent):
  // cache [cell][5][N^2] = M = F^{-T} (row-major), c = mu - 2 lambda ln J;
  // P = mu H + c (M H^T) M + 2 lambda (M : H) M, value rho alpha_1 v
  template <typename T>
  struct NH2Form1QOp
  {
    const T *cache;
    NHMat<T> m;
    int      n2;
    __device__ __forceinline__ void
    operator()(unsigned cell, int q, T (&v)[2], T (&H)[2][2]) const
    {
      const T *cp = cache + size_t(cell) * 5 * n2 + q;
      T        M[2][2];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
          M[i][j] = __ldg(cp + (i * 2 + j) * n2);
      const T c = __ldg(cp + 4 * n2);
      const T t = M[0][0] * H[0][0] + M[0][1] * H[0][1] + M[1][0] * H[1][0] + M[1][1] * H[1][1];
      T       K[2][2];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int k = 0; k < 2; ++k)
          K[i][k] = M[i][0] * H[k][0] + M[i][1] * H[k][1];
      T P[2][2];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
          P[i][j] = m.mu * H[i][j] + c * (K[i][0] * M[0][j] + K[i][1] * M[1][j]) +
                    m.two_lambda * t * M[i][j];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
          H[i][j] = P[i][j];
      v[0] *= m.rho_alpha;
      v[1] *= m.rho_alpha;
    }
  };

  // neo-Hookean, formulation 0 (isochoric/volumetric split, tensor2 caching,
  // mf_nh_operator.h:701-840): cache [cell][10][N^2] = F^{-1} (4), J, F (4),
  // J^{-1/2}; current-frame flux Pc (the 3D form0_flux_dev with dim = 2),
  // P = J Pc F^{-T}
  template <typename T>
  struct NH2Form0QOp
  {
    const T *cache;
    NHMat<T> m;
    int      n2;
    __device__ __forceinline__ void
    operator()(unsigned cell, int q, T (&v)[2], T (&H)[2][2]) const
    {
      const T *cp = cache + size_t(cell) * 10 * n2 + q;
      T        Fi[2][2], F[2][2];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
          {
            Fi[i][j] = __ldg(cp + (i * 2 + j) * n2);
            F[i][j]  = __ldg(cp + (5 + i * 2 + j) * n2);
          }
      const T J  = __ldg(cp + 4 * n2);
      const T js = __ldg(cp + 9 * n2);
      T       gg[2][2], sg[2][2], bb[2][2], tau_bar[2][2];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
          gg[i][j] = H[i][0] * Fi[0][j] + H[i][1] * Fi[1][j];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
          {
            bb[i][j]      = (F[i][0] * F[j][0] + F[i][1] * F[j][1]) * js * js;
            sg[i][j]      = T(0.5) * (gg[i][j] + gg[j][i]);
            tau_bar[i][j] = bb[i][j] * (T(2.0) * m.c_1);
          }
      const T inv_dim = T(0.5), two_over_dim = T(1.0);
      const T tr_tb = tau_bar[0][0] + tau_bar[1][1], tr_tb_dim = tr_tb * inv_dim;
      const T dPsi   = (m.kappa / T(2.0)) * (J - T(1.0) / J);
      const T dPsi_J = dPsi * J;
      const T d2Psi  = (m.kappa / T(2.0)) * (T(1.0) + T(1.0) / (J * J));
      const T tr     = sg[0][0] + sg[1][1];
      T       tau_iso_src = T(0);
      T       jc[2][2], tau[2][2];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
          {
            const T dev     = sg[i][j] - (i == j ? tr * inv_dim : T(0));
            const T tau_iso = tau_bar[i][j] - (i == j ? tr_tb_dim : T(0));
            tau[i][j]       = tau_bar[i][j] + (i == j ? dPsi_J - tr_tb_dim : T(0));
            jc[i][j]        = sg[i][j] * (-dPsi_J * T(2.0)) + (i == j ? J * (dPsi + J * d2Psi) * tr : T(0)) +
                       (two_over_dim * tr_tb) * dev - (two_over_dim * tr) * tau_iso;
            tau_iso_src += tau_iso * sg[i][j];
          }
      T Pc[2][2];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
          Pc[i][j] = (jc[i][j] - (i == j ? two_over_dim * tau_iso_src : T(0)) + gg[i][0] * tau[0][j] +
                      gg[i][1] * tau[1][j]) /
                     J;
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
          H[i][j] = J * (Pc[i][0] * Fi[j][0] + Pc[i][1] * Fi[j][1]);
      v[0] *= m.rho_alpha;
      v[1] *= m.rho_alpha;
    }
  };

  // gradient of a 2-component nodal field at the Gauss points of a cell:
  // H[c][d] of quadrature point (a, l) for a = 0..N-1 (x-line y = l), from
  // the arrays W (values, G0, G1 per component)
  template <int N, typename T>
  __device__ __forceinline__ void
  gather_eval2_vec(const ShapeA<N, T> &sh, const CellGeom<T> &g, const T *u, int cx, int cy, int l,
                   bool active, T *W)
  {
    constexpr int N2 = N * N;
#pragma unroll 1
    for (int c = 0; c < 2; ++c)
      {
        T row[N];
#pragma unroll
        for (int a = 0; a < N; ++a)
          {
            const int ix = cx * g.p + a, iy = cy * g.p + l;
            row[a] = active ? u[size_t(c) * g.n_nodes + size_t(ix) + size_t(g.Nn[0]) * size_t(iy)] : zero<T>();
          }
        T *V = W + c * 3 * N2;
        eval2<N>(sh.S, sh.D[0], sh.D[1], row, V, V + N2, V + 2 * N2, l, true);
        __syncthreads();
      }
  }

  // per-qp cache of the neo-Hookean tangent from the linearisation u
  // (mf_nh_operator.h:394-523 restated for dim = 2); err[0] |= 1 if det F <= 0
  template <int N, typename T, int FORM>
  __global__ void __launch_bounds__(cpb2d<N>() * N)
  nh_cache2d_kernel(const __grid_constant__ ShapeA<N, T> sh, const __grid_constant__ CellGeom<T> g,
                    const NHMat<T> m, const T *__restrict__ u, T *__restrict__ cache, int *err)
  {
    constexpr int N2  = N * N;
    constexpr int CPB = cpb2d<N>();
    constexpr int NF  = FORM == 1 ? 5 : 10;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T             *W      = reinterpret_cast<T *>(smem_raw) + (threadIdx.x / N) * 6 * N2;
    const int      l      = threadIdx.x % N;
    const unsigned cell   = blockIdx.x * CPB + threadIdx.x / N;
    const bool     active = cell < g.n_cells;
    const unsigned cc     = active ? cell : 0u;
    const int      cx = int(cc % unsigned(g.C[0])), cy = int(cc / unsigned(g.C[0]));
    gather_eval2_vec<N>(sh, g, u, cx, cy, l, active, W);
    if (!active)
      return;
#pragma unroll 1
    for (int a = 0; a < N; ++a)
      {
        const int q = a + N * l;
        T         H[2][2], F[2][2];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < 2; ++j)
            {
              H[i][j] = W[i * 3 * N2 + (j + 1) * N2 + q];
              F[i][j] = H[i][j] + (i == j ? T(1) : T(0));
            }
        const T Jm1 = jm1_from_grad2(H);
        const T J   = T(1) + Jm1;
        if (!(J > T(0)))
          {
            atomicOr(err, 1);
            continue;
          }
        T Fi[2][2] = {{F[1][1] / J, -F[0][1] / J}, {-F[1][0] / J, F[0][0] / J}};
        T *cp = cache + size_t(cell) * NF * N2 + q;
        if constexpr (FORM == 1)
          {
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
              for (int j = 0; j < 2; ++j)
                cp[(i * 2 + j) * N2] = Fi[j][i];
            cp[4 * N2] = m.mu - m.two_lambda * log1p(Jm1);
          }
        else
          {
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
              for (int j = 0; j < 2; ++j)
                {
                  cp[(i * 2 + j) * N2]     = Fi[i][j];
                  cp[(5 + i * 2 + j) * N2] = F[i][j];
                }
            cp[4 * N2] = J;
            cp[9 * N2] = exp(log1p(Jm1) * T(-0.5));
          }
      }
  }

  // Exact diagonal of the cell operator (MatrixFreeTools::compute_diagonal
  // semantics): for every local DoF (c, a, b) the quadrature-point operator
  // is applied to its basis function; thread = local DoF.  Constrained rows
  // are left to finish_diagonal.
  template <int N, typename T, int NC, class QOp>
  __global__ void
  diag2d_kernel(const __grid_constant__ ShapeA<N, T> sh, const __grid_constant__ CellGeom<T> g, const QOp op,
                T *__restrict__ diag)
  {
    constexpr int N2   = N * N;
    const int     t    = threadIdx.x; // NC * N2 threads
    const unsigned cell = blockIdx.x;
    const int     c = t / N2, a = (t % N2) % N, b = (t % N2) / N;
    const int     cx = int(cell % unsigned(g.C[0])), cy = int(cell / unsigned(g.C[0]));
    // derivative of the Lagrange basis at the Gauss points: Gm = Du S
    T Sa[N], Sb[N], Ga[N], Gb[N];
#pragma unroll
    for (int q = 0; q < N; ++q)
      {
        Sa[q] = sh.S[q * N + a];
        Sb[q] = sh.S[q * N + b];
        T ga = zero<T>(), gb = zero<T>();
#pragma unroll
        for (int r = 0; r < N; ++r)
          {
            ga = fma_(sh.Du[q * N + r], sh.S[r * N + a], ga);
            gb = fma_(sh.Du[q * N + r], sh.S[r * N + b], gb);
          }
        Ga[q] = ga * g.inv_h[0];
        Gb[q] = gb * g.inv_h[1];
      }
    T acc = zero<T>();
    for (int qy = 0; qy < N; ++qy)
      for (int qx = 0; qx < N; ++qx)
        {
          T v[NC], H[NC][2];
#pragma unroll
          for (int k = 0; k < NC; ++k)
            v[k] = H[k][0] = H[k][1] = zero<T>();
          const T phi = Sa[qx] * Sb[qy], gx = Ga[qx] * Sb[qy], gy = Sa[qx] * Gb[qy];
          v[c]    = phi;
          H[c][0] = gx;
          H[c][1] = gy;
          op(cell, qx + N * qy, v, H);
          const T jxw = sh.w[qx] * sh.w[qy] * g.vol;
          acc         = acc + (v[c] * phi + H[c][0] * gx + H[c][1] * gy) * jxw;
        }
    const int ix = cx * g.p + a, iy = cy * g.p + b;
    atomicAdd(diag + size_t(c) * g.n_nodes + size_t(ix) + size_t(g.Nn[0]) * size_t(iy), acc);
  }

  // Newton residual (internal force + inertia + body force), dim = 2
  // (mf_elasticity.h:1649-1908): rhs += -int tau F^{-T} : grad v
  // + rho int (b - acc) . v
  template <int N, int FORM>
  __global__ void __launch_bounds__(cpb2d<N>() * N)
  residual2d_kernel(const __grid_constant__ ShapeA<N, double> sh, const __grid_constant__ CellGeom<double> g,
                    const NHMat<double> m, double rho, double b0, double b1, const double *__restrict__ u,
                    const double *__restrict__ acc, double *__restrict__ rhs)
  {
    using T           = double;
    constexpr int N2  = N * N;
    constexpr int CPB = cpb2d<N>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T             *W      = reinterpret_cast<T *>(smem_raw) + (threadIdx.x / N) * 8 * N2;
    T             *AV     = W + 6 * N2; // acceleration values [2][N2]
    const int      l      = threadIdx.x % N;
    const unsigned cell   = blockIdx.x * CPB + threadIdx.x / N;
    const bool     active = cell < g.n_cells;
    const unsigned cc     = active ? cell : 0u;
    const int      cx = int(cc % unsigned(g.C[0])), cy = int(cc / unsigned(g.C[0]));
    gather_eval2_vec<N>(sh, g, u, cx, cy, l, active, W);
#pragma unroll 1
    for (int c = 0; c < 2; ++c)
      {
        T row[N];
#pragma unroll
        for (int a = 0; a < N; ++a)
          {
            const int ix = cx * g.p + a, iy = cy * g.p + l;
            row[a] = active ? acc[size_t(c) * g.n_nodes + size_t(ix) + size_t(g.Nn[0]) * size_t(iy)] : 0.0;
          }
        // values only; the scratch G0 slot of the acceleration is AV + c*N2
        // shifted: use W's free y-gradient slot pattern via a local array pair
        eval2<N>(sh.S, sh.D[0], sh.D[1], row, AV + c * N2, AV + c * N2, AV + c * N2, l, false);
        __syncthreads();
      }
    if (active)
      {
        const T bf[2] = {b0, b1};
#pragma unroll 1
        for (int a = 0; a < N; ++a)
          {
            const int q   = a + N * l;
            const T   jxw = sh.w[a] * sh.w[l] * g.vol;
            T         H[2][2], F[2][2];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
              for (int j = 0; j < 2; ++j)
                {
                  H[i][j] = W[i * 3 * N2 + (j + 1) * N2 + q];
                  F[i][j] = H[i][j] + (i == j ? 1.0 : 0.0);
                }
            const T Jm1   = jm1_from_grad2(H);
            const T J     = 1.0 + Jm1;
            const T lnJ   = log1p(Jm1);
            T       Fi[2][2] = {{F[1][1] / J, -F[0][1] / J}, {-F[1][0] / J, F[0][0] / J}};
            T       tau[2][2];
            if constexpr (FORM == 1)
              {
                // mu b - (mu - 2 lambda ln J) I = mu (H + H^T + H H^T) + 2 lambda ln J I
#pragma unroll
                for (int i = 0; i < 2; ++i)
#pragma unroll
                  for (int j = 0; j < 2; ++j)
                    tau[i][j] = m.mu * (H[i][j] + H[j][i] + (H[i][0] * H[j][0] + H[i][1] * H[j][1])) +
                                (i == j ? 2.0 * m.lambda * lnJ : 0.0);
              }
            else
              {
                const T f = exp(-0.5 * lnJ);
#pragma unroll
                for (int i = 0; i < 2; ++i)
#pragma unroll
                  for (int j = 0; j < 2; ++j)
                    tau[i][j] = 2.0 * m.c_1 * f * f * (F[i][0] * F[j][0] + F[i][1] * F[j][1]);
                const T tr  = tau[0][0] + tau[1][1];
                const T tmp = (m.kappa / 2.0) * Jm1 * (2.0 + Jm1);
                tau[0][0] += tmp - tr / 2.0;
                tau[1][1] += tmp - tr / 2.0;
              }
#pragma unroll
            for (int i = 0; i < 2; ++i)
              {
#pragma unroll
                for (int j = 0; j < 2; ++j)
                  W[i * 3 * N2 + (j + 1) * N2 + q] = -(tau[i][0] * Fi[j][0] + tau[i][1] * Fi[j][1]) * jxw;
                W[i * 3 * N2 + q] = (-AV[i * N2 + q] + bf[i]) * rho * jxw;
              }
          }
      }
#pragma unroll 1
    for (int c = 0; c < 2; ++c)
      {
        T *V = W + c * 3 * N2;
        T  col[N];
        integ2<N>(sh.S, sh.D[0], sh.D[1], V, V + N2, V + 2 * N2, l, true, col);
        if (active)
#pragma unroll
          for (int b = 0; b < N; ++b)
            atomicAdd(rhs + size_t(c) * g.n_nodes + size_t(cx * g.p + l) + size_t(g.Nn[0]) * size_t(cy * g.p + b),
                      col[b]);
      }
  }

  // heat right-hand side M (u_old + dt f) in 2D (heat_transfer.h:579-655)
  template <int N>
  __global__ void __launch_bounds__(cpb2d<N>() * N)
  heat_rhs2d_kernel(const __grid_constant__ ShapeA<N, double> sh, const __grid_constant__ CellGeom<double> g,
                    const __grid_constant__ SourceDev f, double dt, const double *__restrict__ u_old,
                    double *__restrict__ rhs)
  {
    using T           = double;
    constexpr int N2  = N * N;
    constexpr int CPB = cpb2d<N>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T             *V      = reinterpret_cast<T *>(smem_raw) + (threadIdx.x / N) * 2 * N2;
    T             *G0     = V + N2;
    const int      l      = threadIdx.x % N;
    const unsigned cell   = blockIdx.x * CPB + threadIdx.x / N;
    const bool     active = cell < g.n_cells;
    const unsigned cc     = active ? cell : 0u;
    const int      cx = int(cc % unsigned(g.C[0])), cy = int(cc / unsigned(g.C[0]));
    T              row[N];
#pragma unroll
    for (int a = 0; a < N; ++a)
      row[a] = active ? u_old[size_t(cx * g.p + a) + size_t(g.Nn[0]) * size_t(cy * g.p + l)] : 0.0;
    eval2<N>(sh.S, sh.D[0], sh.D[1], row, V, G0, G0, l, false);
    __syncthreads();
    // x-line y = l: values + dt f, times JxW
    const double py = f.lo[1] + (cy + f.xq[l]) * f.h[1];
#pragma unroll
    for (int a = 0; a < N; ++a)
      {
        const double px = f.lo[0] + (cx + f.xq[a]) * f.h[0];
        double       fv = f.constant;
        for (int i = 0; i < f.n_gauss; ++i)
          {
            const double dx = px - f.center[i][0], dy = py - f.center[i][1];
            fv += f.amp[i] * exp(-(dx * dx + dy * dy) / (2 * f.width[i] * f.width[i]));
          }
        V[a + N * l] = (V[a + N * l] + dt * fv) * (sh.w[a] * sh.w[l] * g.vol);
      }
    T col[N];
    integ2<N>(sh.S, sh.D[0], sh.D[1], V, G0, G0, l, false, col);
    if (active)
#pragma unroll
      for (int b = 0; b < N; ++b)
        atomicAdd(rhs + size_t(cx * g.p + l) + size_t(g.Nn[0]) * size_t(cy * g.p + b), col[b]);
  }
} // namespace mfgpu
