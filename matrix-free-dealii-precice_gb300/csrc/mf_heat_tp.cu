// The heat operator (mass + dt k Laplace, LaplaceOperator::do_operation_on_
// cell, heat_transfer.h:236-250) on box levels in its tensor-product form,
// one thread per cell, registers only.
//
// Every cell of a box level is the same affine brick h0 x h1 x h2 and the
// coefficient is constant (heat_transfer.h:63-71).  The QGauss(p+1) cell
// integral the sum-factorization kernel evaluates is then exactly
//
//   A_e = vol [ Mz(x)My(x)Mx + kdt/h0^2 Mz(x)My(x)Kx
//                            + kdt/h1^2 Mz(x)Ky(x)Mx + kdt/h2^2 Kz(x)My(x)Mx ]
//
// with the 1D mass and stiffness matrices of the Gauss-Lobatto basis on
// [0,1], M_ij = sum_q w_q phi_i(x_q) phi_j(x_q) and K_ij = sum_q w_q
// phi_i'(x_q) phi_j'(x_q) (the (p+1)-point Gauss rule integrates both
// exactly, so this is the same operator, not an approximation of it).
// Grouped as
//   P = Mx x,  Q = (vol Mx + vol kdt/h0^2 Kx) x          (2 x-sweeps)
//   S1 = My Q + (vol kdt/h1^2 Ky) P,  S2 = My P         (3 y-sweeps)
//   y = Mz S1 + (kdt/h2^2 Kz) S2                        (2 z-sweeps)
// it costs 7 (p+1)^4 multiply-adds per cell, against 12 (p+1)^4 plus the
// quadrature-point work for evaluate / integrate through the Gauss points.
//
// Work split (heat_tp_kernel): thread = a column of `zlen` consecutive cells
// along z, threads of a warp consecutive along x.  The (p+1)^3 values of a
// cell live in registers; all sweeps are register FMAs with the 1D
// matrices in the kernel's constant bank.  Nodes shared between cells are
// loaded and written once where the layout allows:
//   * along z, the top node plane of a cell is the bottom plane of the next
//     cell of the column: its values are carried in registers, and its
//     results are added into the next cell's before they are written;
//   * along x, a thread takes the values of its last node column from the
//     next lane (warp shuffle) and hands the results of that column to it,
//     so each node column is written by one lane; a warp's last lane and a
//     row's last cell write their own last column.
// The remaining shared nodes (the y faces, the warp and column-segment
// ends) are added with atomics, as in the sum-factorization kernel.
// Constraints are those of the sum-factorization kernel: constrained
// source values read as zero, constrained rows get dst += src from the one
// cell that owns the node (local index < p in every direction, or the last
// cell along it).
#include <algorithm>
#include <cstring>

#include "mf_host.h"

namespace mfgpu
{
  namespace tp
  {
    constexpr int THREADS = 128;

    // the six 1D matrices, symmetric, scaled as above
    template <int N, typename T>
    struct HeatTP
    {
      T Mx[N][N], Ax[N][N];
      T My[N][N], Ky[N][N];
      T Mz[N][N], Kz[N][N];
    };

    template <int N, typename T>
    __device__ __forceinline__ T
    dot_row(const T (&M)[N][N], int i, const T (&v)[N])
    {
      T s = M[i][0] * v[0];
#pragma unroll
      for (int j = 1; j < N; ++j)
        s = fma(M[i][j], v[j], s);
      return s;
    }

    // y = A_e x for one cell, x and y indexed [k][b][a] (z, y, x)
    template <int N, typename T>
    __device__ __forceinline__ void
    cell_apply(const HeatTP<N, T> &m, const T (&x)[N][N][N], T (&y)[N][N][N])
    {
      T P[N][N][N], Q[N][N][N];
#pragma unroll
      for (int k = 0; k < N; ++k)
#pragma unroll
        for (int b = 0; b < N; ++b)
#pragma unroll
          for (int i = 0; i < N; ++i)
            {
              P[k][b][i] = dot_row<N, T>(m.Mx, i, x[k][b]);
              Q[k][b][i] = dot_row<N, T>(m.Ax, i, x[k][b]);
            }
      // y-sweeps in place: Q <- My Q + Ky P, P <- My P
#pragma unroll
      for (int k = 0; k < N; ++k)
#pragma unroll
        for (int a = 0; a < N; ++a)
          {
            T p[N], q[N];
#pragma unroll
            for (int j = 0; j < N; ++j)
              {
                p[j] = P[k][j][a];
                q[j] = Q[k][j][a];
              }
#pragma unroll
            for (int i = 0; i < N; ++i)
              {
                T s1 = dot_row<N, T>(m.My, i, q);
#pragma unroll
                for (int j = 0; j < N; ++j)
                  s1 = fma(m.Ky[i][j], p[j], s1);
                Q[k][i][a] = s1;
                P[k][i][a] = dot_row<N, T>(m.My, i, p);
              }
          }
      // z-sweeps: y = Mz S1 + Kz S2
#pragma unroll
      for (int b = 0; b < N; ++b)
#pragma unroll
        for (int a = 0; a < N; ++a)
          {
            T s1[N], s2[N];
#pragma unroll
            for (int j = 0; j < N; ++j)
              {
                s1[j] = Q[j][b][a];
                s2[j] = P[j][b][a];
              }
#pragma unroll
            for (int i = 0; i < N; ++i)
              {
                T s = dot_row<N, T>(m.Mz, i, s1);
#pragma unroll
                for (int j = 0; j < N; ++j)
                  s = fma(m.Kz[i][j], s2[j], s);
                y[i][b][a] = s;
              }
          }
    }

    // dst += A src over the cells of z-planes [zc0, zc1) of one level
    // (grid.y = problem of a batch: vectors at offset blockIdx.y * bstride)
    template <int N, typename T, bool CON>
    __global__ void __launch_bounds__(THREADS)
    heat_tp_kernel(const __grid_constant__ HeatTP<N, T> m, const __grid_constant__ CellGeom<T> g,
                   const int zlen, const int zc0, const int zc1, const T *__restrict__ src,
                   T *__restrict__ dst)
    {
      constexpr int      P        = N - 1;
      constexpr unsigned FULL     = 0xffffffffu;
      constexpr bool     PREFETCH = N * N * N * sizeof(T) <= 27 * 4;
      src += size_t(blockIdx.y) * g.bstride;
      dst += size_t(blockIdx.y) * g.bstride;
      const int      lane = int(threadIdx.x & 31u);
      const int      C0 = g.C[0], C1 = g.C[1], C2 = g.C[2];
      const unsigned ncol = unsigned(C0) * unsigned(C1);
      const unsigned nseg = unsigned(zc1 - zc0 + zlen - 1) / unsigned(zlen);
      const unsigned t    = blockIdx.x * THREADS + threadIdx.x;
      const bool     active = t < ncol * nseg;
      const unsigned tt     = active ? t : 0u;
      const int      cx     = int(tt % unsigned(C0));
      const int      r      = int(tt / unsigned(C0));
      const int      cy     = r % C1;
      const int      cz0    = zc0 + (r / C1) * zlen;
      const int      czn    = min(cz0 + zlen, zc1); // one past the column segment's last cell
      // lane+1 holds cell cx+1 of the same row, lane-1 cell cx-1
      const bool rmerge = active && lane < 31 && cx + 1 < C0;
      const bool lmerge = active && lane > 0 && cx > 0;
      // Dirichlet faces this cell column touches (component 0)
      const bool fx0 = CON && cx == 0 && (g.face_mask[0] & 1u);
      const bool fx1 = CON && cx == C0 - 1 && (g.face_mask[1] & 1u);
      const bool fy0 = CON && cy == 0 && (g.face_mask[2] & 1u);
      const bool fy1 = CON && cy == C1 - 1 && (g.face_mask[3] & 1u);
      const bool bz0 = CON && (g.face_mask[4] & 1u);
      const bool bz1 = CON && (g.face_mask[5] & 1u);
      const size_t Nx = size_t(g.Nn[0]), Nxy = size_t(g.Nn[0]) * size_t(g.Nn[1]);
      const size_t col = size_t(cx * P) + Nx * size_t(cy * P);

      auto constrained = [&](int a, int b, int k, int cz) {
        return (a == 0 && fx0) || (a == P && fx1) || (b == 0 && fy0) || (b == P && fy1) ||
               (k == 0 && bz0 && cz == 0) || (k == P && bz1 && cz == C2 - 1);
      };
      // node plane k of cell cz into v[b][a] (zero where constrained or
      // inactive); the last node column comes from lane+1 where it holds it
      auto gather_plane = [&](int k, int cz, bool act, T (&v)[N][N]) {
        const size_t base = col + Nxy * size_t(cz * P + k);
#pragma unroll
        for (int b = 0; b < N; ++b)
          {
#pragma unroll
            for (int a = 0; a < P; ++a)
              v[b][a] = (act && !(CON && constrained(a, b, k, cz))) ? __ldg(src + base + Nx * b + a) : T(0);
            const T right = __shfl_down_sync(FULL, v[b][0], 1);
            v[b][P]       = rmerge ? right :
                            (act && !(CON && constrained(P, b, k, cz))) ? __ldg(src + base + Nx * b + P) : T(0);
          }
      };
      // results of node plane k of cell cz: the last node column goes to
      // lane+1 where it holds it, the first column receives lane-1's
      auto scatter_plane = [&](int k, int cz, bool act, T (&v)[N][N]) {
        const size_t base = col + Nxy * size_t(cz * P + k);
#pragma unroll
        for (int b = 0; b < N; ++b)
          {
            const T left = __shfl_up_sync(FULL, v[b][P], 1);
            if (lmerge)
              v[b][0] += left;
            if (!act)
              continue;
#pragma unroll
            for (int a = 0; a < N; ++a)
              {
                if (a == P && rmerge)
                  continue;
                T *d = dst + base + Nx * b + a;
                if (CON && constrained(a, b, k, cz))
                  {
                    const bool owner = (a < P || cx == C0 - 1) && (b < P || cy == C1 - 1) && (k < P || cz == C2 - 1);
                    if (owner)
                      *d += __ldg(src + base + Nx * b + a);
                  }
                else
                  atomicAdd(d, v[b][a]);
              }
          }
      };

      T x[N][N][N];
#pragma unroll
      for (int k = 0; k < N; ++k)
        gather_plane(k, cz0, active && cz0 < czn, x[k]);
      T carry[N][N];
#pragma unroll
      for (int b = 0; b < N; ++b)
#pragma unroll
        for (int a = 0; a < N; ++a)
          carry[b][a] = T(0);
#pragma unroll 1
      for (int i = 0; i < zlen; ++i)
        {
          const int  cz  = cz0 + i;
          const bool act = active && cz < czn;
          // the next cell's node planes 1..p, loaded before this cell is
          // computed where the registers allow (FP32 Q1 and Q2, FP64 Q1)
          T xn[P][N][N];
          if (PREFETCH && i + 1 < zlen)
            {
#pragma unroll
              for (int k = 1; k < N; ++k)
                gather_plane(k, cz + 1, active && cz + 1 < czn, xn[k - 1]);
            }
          T y[N][N][N];
          cell_apply<N, T>(m, x, y);
          if (act)
            {
              // the previous cell's top plane results
#pragma unroll
              for (int b = 0; b < N; ++b)
#pragma unroll
                for (int a = 0; a < N; ++a)
                  y[0][b][a] += carry[b][a];
            }
#pragma unroll
          for (int k = 0; k < P; ++k)
            scatter_plane(k, cz, act, y[k]);
          if (act)
            {
#pragma unroll
              for (int b = 0; b < N; ++b)
#pragma unroll
                for (int a = 0; a < N; ++a)
                  carry[b][a] = y[P][b][a];
            }
          if (i + 1 < zlen)
            {
#pragma unroll
              for (int b = 0; b < N; ++b)
#pragma unroll
                for (int a = 0; a < N; ++a)
                  x[0][b][a] = x[P][b][a];
              if constexpr (PREFETCH)
                {
#pragma unroll
                  for (int k = 1; k < N; ++k)
#pragma unroll
                    for (int b = 0; b < N; ++b)
#pragma unroll
                      for (int a = 0; a < N; ++a)
                        x[k][b][a] = xn[k - 1][b][a];
                }
              else
                {
#pragma unroll
                  for (int k = 1; k < N; ++k)
                    gather_plane(k, cz + 1, active && cz + 1 < czn, x[k]);
                }
            }
        }
      // the top plane of the segment's last cell
      scatter_plane(P, czn - 1, active && czn > cz0, carry);
    }

    template <int N, typename T>
    HeatTP<N, T>
    make_matrices(const HostBasis &b, const LevelGeom &g, double kdt)
    {
      double M[N][N], K[N][N];
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
          {
            double m = 0, k = 0;
            for (int q = 0; q < N; ++q)
              {
                m += b.w[q] * b.S[q * N + i] * b.S[q * N + j];
                k += b.w[q] * b.G[q * N + i] * b.G[q * N + j];
              }
            M[i][j] = m;
            K[i][j] = k;
          }
      const double vol = g.h[0] * g.h[1] * g.h[2];
      HeatTP<N, T> h;
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
          {
            h.Mx[i][j] = T(M[i][j]);
            h.Ax[i][j] = T(vol * M[i][j] + vol * kdt / (g.h[0] * g.h[0]) * K[i][j]);
            h.My[i][j] = T(M[i][j]);
            h.Ky[i][j] = T(vol * kdt / (g.h[1] * g.h[1]) * K[i][j]);
            h.Mz[i][j] = T(M[i][j]);
            h.Kz[i][j] = T(vol * kdt / (g.h[2] * g.h[2]) * K[i][j]);
          }
      return h;
    }

    template <int N, typename T>
    cudaError_t
    launch(const HostBasis &b, const LevelGeom &g, const HeatTPArgs &a, cudaStream_t s)
    {
      const HeatTP<N, T> h  = make_matrices<N, T>(b, g, a.kdt);
      CellGeom<T>        cg = make_cell_geom<T>(g);
      cg.batch              = unsigned(a.batch > 1 ? a.batch : 1);
      cg.bstride            = a.batch > 1 ? a.bstride : 0;
      const int      nz     = a.zc1 - a.zc0;
      const int      zlen   = std::max(1, std::min(a.zlen, nz));
      const size_t   ncol   = size_t(g.C[0]) * size_t(g.C[1]);
      const size_t   thr    = ncol * size_t((nz + zlen - 1) / zlen);
      if (nz <= 0 || thr == 0)
        return cudaSuccess;
      const size_t grid = (thr + THREADS - 1) / THREADS;
      if (grid > 0x7fffffffu || cg.batch > 65535u)
        return cudaErrorInvalidValue;
      const dim3 gr(unsigned(grid), cg.batch);
      if (a.constrained)
        heat_tp_kernel<N, T, true><<<gr, THREADS, 0, s>>>(h, cg, zlen, a.zc0, a.zc1, static_cast<const T *>(a.src),
                                                          static_cast<T *>(a.dst));
      else
        heat_tp_kernel<N, T, false><<<gr, THREADS, 0, s>>>(h, cg, zlen, a.zc0, a.zc1, static_cast<const T *>(a.src),
                                                           static_cast<T *>(a.dst));
      return cudaGetLastError();
    }
  } // namespace tp

  bool
  heat_tp_supported(int N, int precision)
  {
    return precision == 32 ? (N >= 2 && N <= 4) : (N >= 2 && N <= 3);
  }

  int
  heat_tp_zlen(const LevelGeom &g, int zc0, int zc1)
  {
    // the longest column segment (at most 4 cells) that keeps 8 warps per
    // SM of the 152 busy
    const size_t ncol = size_t(g.C[0]) * size_t(g.C[1]);
    const int    nz   = zc1 - zc0;
    int          zlen = 4;
    while (zlen > 1 && ncol * size_t((nz + zlen - 1) / zlen) < size_t(152) * 256)
      zlen /= 2;
    return zlen;
  }

  cudaError_t
  launch_heat_tp(const HostBasis &b, const LevelGeom &g, int precision, const HeatTPArgs &a, cudaStream_t s)
  {
    if (g.dim == 2 || !heat_tp_supported(b.N, precision) || a.zc0 < 0 || a.zc1 > g.C[2] || a.zlen < 1)
      return cudaErrorInvalidValue;
    if (precision == 32)
      switch (b.N)
        {
          case 2: return tp::launch<2, float>(b, g, a, s);
          case 3: return tp::launch<3, float>(b, g, a, s);
          case 4: return tp::launch<4, float>(b, g, a, s);
        }
    else
      switch (b.N)
        {
          case 2: return tp::launch<2, double>(b, g, a, s);
          case 3: return tp::launch<3, double>(b, g, a, s);
        }
    return cudaErrorInvalidValue;
  }
} // namespace mfgpu
