// The heat operator (mass + dt k Laplace, LaplaceOperator::do_operation_on_
// cell, heat_transfer.h:236-250) on box levels in its tensor-product form:
// one thread per cell in registers at degree 1 on levels of 16384 cells or
// more, (p+1)^2 threads per cell through shared memory otherwise; the
// shared-memory form also in double-float arithmetic on FP64 vectors.
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
// Registers (heat_tp_kernel): thread = a column of `zlen` consecutive cells
// along z, threads of a warp consecutive along x.  The (p+1)^3 values of a
// cell live in registers; all sweeps are register FMAs with the 1D
// matrices in the kernel's constant bank.  Nodes shared between cells are
// loaded and written once where the layout allows:
//   * along z, the top node plane of a cell is the bottom plane of the next
//     cell of the column: its values are carried in registers, and its
//     results are added into the next cell's before they are written;
//   * along x, a thread hands the results of its last node column to the
//     next lane (warp shuffle), so each node column is written by one lane;
//     a warp's last lane and a row's last cell write their own last column.
// The remaining shared nodes (the y faces, the warp and column-segment
// ends) are added with atomics, as in the sum-factorization kernel.
// Constraints are those of the sum-factorization kernel: constrained
// source values read as zero, constrained rows get dst += src from the one
// cell that owns the node (local index < p in every direction, or the last
// cell along it).
#include <cuda.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <tuple>
#include <vector>

#include "mf_host.h"

namespace mfgpu
{
  namespace tp
  {
    constexpr int THREADS = 128;
#ifndef MF_TP_MIN_BLOCKS
#define MF_TP_MIN_BLOCKS 1
#endif

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

    // multiply-add and zero in the compute type (FP32, FP64 or double-float)
    __device__ __forceinline__ float
    tp_fma(float a, float b, float c)
    {
      return fmaf(a, b, c);
    }
    __device__ __forceinline__ double
    tp_fma(double a, double b, double c)
    {
      return fma(a, b, c);
    }
    __device__ __forceinline__ df64
    tp_fma(df64 a, df64 b, df64 c)
    {
      return fma_(a, b, c);
    }
    template <typename T>
    __host__ __device__ __forceinline__ T
    tp_zero()
    {
      return T(0);
    }
    template <>
    __host__ __device__ __forceinline__ df64
    tp_zero<df64>()
    {
      return df64{0.f, 0.f};
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
    __global__ void __launch_bounds__(THREADS, MF_TP_MIN_BLOCKS)
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
      const unsigned ru     = g.dC0.div(tt);
      const int      cx     = int(tt - ru * unsigned(C0));
      const int      seg    = int(g.dC1.div(ru));
      const int      cy     = int(ru) - seg * C1;
      const int      cz0    = zc0 + seg * zlen;
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
      // inactive).  Every lane loads its whole row: the last node column,
      // which lane+1 loads too, comes from the same L1 line; taking it by
      // a shuffle would make the prefetch of the next cell wait for its loads.
      auto gather_plane = [&](int k, int cz, bool act, T (&v)[N][N]) {
        const size_t base = col + Nxy * size_t(cz * P + k);
#pragma unroll
        for (int b = 0; b < N; ++b)
#pragma unroll
          for (int a = 0; a < N; ++a)
            v[b][a] = (act && !(CON && constrained(a, b, k, cz))) ? __ldg(src + base + Nx * b + a) : T(0);
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
    HeatTP<N, T> make_matrices(const HostBasis &b, const LevelGeom &g, double kdt);

    // -------------------------------------------------------------------
    // Higher degrees: the same seven sweeps with the cell in shared memory.
    //
    // A block takes CPB cells with N^2 threads per cell.  Thread (a, b)
    // gathers the z-column (a, b) of its cell into registers and applies the
    // z-matrices there (U = Mz x, V = Kz x), then the cell's lines are swept
    // through shared memory: thread (a, k) sweeps the y-lines (U <- My U,
    // V <- Ky U + My V, in place), thread (b, k) the x-lines
    // (y = Ax U + Mx V, in place), and thread (a, b) reads its z-column of y
    // back and scatters it (atomics; constrained rows as in the other cell
    // kernels).  Two arrays of N^3 per cell, three barriers; the line
    // products in even-odd form (below).
    // -------------------------------------------------------------------
    template <int N, typename T>
    __host__ __device__ constexpr int
    blk_cells()
    {
      return N == 2 ? 32 : N == 3 ? 14 : N == 4 ? 8 : N == 5 ? 5 : N == 6 ? 3 : 2;
    }

    // shared layout of a cell: node (a, b, k) at a + N b + SZ k of U, V at
    // U + N SZ, cells CS apart.  For 4-byte values the plane and cell
    // padding minimise the shared-memory wavefronts of the four access
    // patterns (z-column writes, y-lines, x-lines, z-column reads) over the
    // warps of a block, by exhaustive search over plane padding 0..8 and
    // cell padding 0..32 with a bank model (wavefronts per warp access,
    // whole kernel): N = 2 320 -> 104, 3 285 -> 204, 4 544 -> 224,
    // 5 385 -> 340, 6 534 -> 366, 7 462 -> 427.
    template <int N, typename T>
    struct BlkLay
    {
      static constexpr int PZ = sizeof(T) == 4 ? (N == 2 ? 2 : N == 3 ? 0 : N == 4 ? 3 : N == 5 ? 0 : 3) : 0;
      static constexpr int PC =
        sizeof(T) == 4 ? (N == 2 ? 4 : N == 3 ? 5 : N == 4 ? 24 : N == 5 ? 3 : N == 6 ? 16 : 25) : 0;
      static constexpr int SZ = N * N + PZ;
      static constexpr int CS = 2 * N * SZ + PC;
    };

    // Even-odd form of a symmetric matrix with M[N-1-i][N-1-j] = M[i][j]
    // (the 1D mass and stiffness matrices: Gauss-Lobatto nodes and Gauss
    // points are symmetric about the cell centre).  With H = N/2, sums
    // e_j = v_j + v_{N-1-j} and differences o_j = v_j - v_{N-1-j} (j < H):
    //   y_i = E e + O o (+ M[i][H] v_H),  y_{N-1-i} = E e - O o (+ ...),
    //   y_H = sum_j M[H][j] e_j + M[H][H] v_H                  (odd N)
    // with E_ij = (M_ij + M_i,N-1-j)/2, O_ij = (M_ij - M_i,N-1-j)/2: about
    // half the products of a plain matrix-vector product.
    template <int N, typename T>
    struct EOMat
    {
      static constexpr int H = N / 2;
      T E[H][H], O[H][H];
      T C[H + 1]; // odd N: M[i][H] for i < H, then M[H][H]
      T R[H];     // odd N: M[H][j] for j < H
    };

    template <int N, typename T>
    struct HeatTPEO
    {
      EOMat<N, T> Mx, Ax, My, Ky, Mz, Kz;
    };

    template <int N, typename T>
    struct EOSplit
    {
      T e[N / 2], o[N / 2], m;
    };

    template <int N, typename T>
    __device__ __forceinline__ EOSplit<N, T>
    eo_split(const T (&v)[N])
    {
      EOSplit<N, T> r;
#pragma unroll
      for (int j = 0; j < N / 2; ++j)
        {
          r.e[j] = v[j] + v[N - 1 - j];
          r.o[j] = v[j] - v[N - 1 - j];
        }
      r.m = (N & 1) ? v[N / 2] : tp_zero<T>();
      return r;
    }

    template <int N, typename T>
    struct EOAcc
    {
      T se[N / 2], so[N / 2], sm;
    };

    // acc (+)= M v, v given by its split; FIRST: start the sums
    template <int N, typename T, bool FIRST>
    __device__ __forceinline__ void
    eo_acc(EOAcc<N, T> &acc, const EOMat<N, T> &M, const EOSplit<N, T> &v)
    {
      constexpr int H = N / 2;
#pragma unroll
      for (int i = 0; i < H; ++i)
        {
          T se = FIRST ? M.E[i][0] * v.e[0] : tp_fma(M.E[i][0], v.e[0], acc.se[i]);
          T so = FIRST ? M.O[i][0] * v.o[0] : tp_fma(M.O[i][0], v.o[0], acc.so[i]);
#pragma unroll
          for (int j = 1; j < H; ++j)
            {
              se = tp_fma(M.E[i][j], v.e[j], se);
              so = tp_fma(M.O[i][j], v.o[j], so);
            }
          if (N & 1)
            se = tp_fma(M.C[i], v.m, se);
          acc.se[i] = se;
          acc.so[i] = so;
        }
      if (N & 1)
        {
          T sm = FIRST ? M.C[H] * v.m : tp_fma(M.C[H], v.m, acc.sm);
#pragma unroll
          for (int j = 0; j < H; ++j)
            sm = tp_fma(M.R[j], v.e[j], sm);
          acc.sm = sm;
        }
    }

    template <int N, typename T>
    __device__ __forceinline__ void
    eo_out(const EOAcc<N, T> &acc, T (&y)[N])
    {
#pragma unroll
      for (int i = 0; i < N / 2; ++i)
        {
          y[i]         = acc.se[i] + acc.so[i];
          y[N - 1 - i] = acc.se[i] - acc.so[i];
        }
      if (N & 1)
        y[N / 2] = acc.sm;
    }

    // TS: storage type of the vectors, T: compute type (TS = double, T =
    // df64: double-float arithmetic on FP64 vectors)
    template <int N, typename TS, typename T, bool CON>
    __global__ void __launch_bounds__(blk_cells<N, T>() * N * N)
    heat_tp_block_kernel(const __grid_constant__ HeatTPEO<N, T> m, const __grid_constant__ CellGeom<T> g,
                         const TS *__restrict__ src, TS *__restrict__ dst)
    {
      constexpr int N2 = N * N, P = N - 1;
      constexpr int CPB = blk_cells<N, T>();
      extern __shared__ __align__(16) unsigned char smraw[];
      src += size_t(blockIdx.y) * g.bstride;
      dst += size_t(blockIdx.y) * g.bstride;
      const int      lc   = int(threadIdx.x) / N2;
      const int      l    = int(threadIdx.x) - lc * N2;
      const int      i0   = l % N, i1 = l / N; // (a, b), (a, k) or (b, k) by phase
      const unsigned cell = g.cell_begin + blockIdx.x * CPB + unsigned(lc);
      const bool     act  = cell < g.cell_end;
      const unsigned cc   = act ? cell : g.cell_begin;
      const unsigned cyz  = g.dC0.div(cc);
      const int      cx   = int(cc - cyz * unsigned(g.C[0]));
      const int      cz   = int(g.dC1.div(cyz));
      const int      cy   = int(cyz) - cz * g.C[1];
      using L = BlkLay<N, T>;
      constexpr int SZ = L::SZ;
      T *U = reinterpret_cast<T *>(smraw) + size_t(lc) * L::CS; // (a, b, k) at a + N b + SZ k
      T *V = U + N * SZ;
      const size_t Nx = size_t(g.Nn[0]), Nxy = size_t(g.Nn[0]) * size_t(g.Nn[1]);
      const int    ix = cx * P + i0, iy = cy * P + i1;
      const size_t colb = size_t(ix) + Nx * size_t(iy) + Nxy * size_t(cz * P);
      // Dirichlet faces of the z-column (a, b) = (i0, i1), component 0
      const bool cxy = CON && (((ix == 0) && (g.face_mask[0] & 1u)) || ((ix == g.Nn[0] - 1) && (g.face_mask[1] & 1u)) ||
                               ((iy == 0) && (g.face_mask[2] & 1u)) || ((iy == g.Nn[1] - 1) && (g.face_mask[3] & 1u)));
      const bool cz0 = CON && cz == 0 && (g.face_mask[4] & 1u);
      const bool cz1 = CON && cz == g.C[2] - 1 && (g.face_mask[5] & 1u);
      auto       con = [&](int k) { return cxy || (k == 0 && cz0) || (k == P && cz1); };
      // gather the z-column (a, b) = (i0, i1) and apply the z-matrices
      {
        T x[N];
#pragma unroll
        for (int k = 0; k < N; ++k)
          x[k] = (act && !con(k)) ? to_compute<T, TS>(__ldg(src + colb + Nxy * k)) : tp_zero<T>();
        const EOSplit<N, T> xs = eo_split<N, T>(x);
        EOAcc<N, T>         au, av;
        eo_acc<N, T, true>(au, m.Mz, xs);
        eo_acc<N, T, true>(av, m.Kz, xs);
        T u[N], v[N];
        eo_out<N, T>(au, u);
        eo_out<N, T>(av, v);
#pragma unroll
        for (int i = 0; i < N; ++i)
          {
            U[i * SZ + i1 * N + i0] = u[i];
            V[i * SZ + i1 * N + i0] = v[i];
          }
      }
      __syncthreads();
      // y-lines (a, k) = (i0, i1): U <- My U, V <- Ky U + My V
      {
        T u[N], v[N];
#pragma unroll
        for (int j = 0; j < N; ++j)
          {
            u[j] = U[i1 * SZ + j * N + i0];
            v[j] = V[i1 * SZ + j * N + i0];
          }
        const EOSplit<N, T> us = eo_split<N, T>(u), vs = eo_split<N, T>(v);
        EOAcc<N, T>         au, av;
        eo_acc<N, T, true>(au, m.My, us);
        eo_acc<N, T, true>(av, m.Ky, us);
        eo_acc<N, T, false>(av, m.My, vs);
        eo_out<N, T>(au, u);
        eo_out<N, T>(av, v);
#pragma unroll
        for (int i = 0; i < N; ++i)
          {
            U[i1 * SZ + i * N + i0] = u[i];
            V[i1 * SZ + i * N + i0] = v[i];
          }
      }
      __syncthreads();
      // x-lines (b, k) = (i0, i1): y = Ax U + Mx V, into U
      {
        T u[N], v[N];
#pragma unroll
        for (int j = 0; j < N; ++j)
          {
            u[j] = U[i1 * SZ + i0 * N + j];
            v[j] = V[i1 * SZ + i0 * N + j];
          }
        const EOSplit<N, T> us = eo_split<N, T>(u), vs = eo_split<N, T>(v);
        EOAcc<N, T>         ay;
        eo_acc<N, T, true>(ay, m.Ax, us);
        eo_acc<N, T, false>(ay, m.Mx, vs);
        eo_out<N, T>(ay, u);
#pragma unroll
        for (int i = 0; i < N; ++i)
          U[i1 * SZ + i0 * N + i] = u[i];
      }
      __syncthreads();
      if (!act)
        return;
      // scatter the z-column (a, b) = (i0, i1)
#pragma unroll
      for (int k = 0; k < N; ++k)
        {
          TS *d = dst + colb + Nxy * k;
          if (con(k))
            {
              const bool owner = (i0 < P || cx == g.C[0] - 1) && (i1 < P || cy == g.C[1] - 1) &&
                                 (k < P || cz == g.C[2] - 1);
              if (owner)
                *d += __ldg(src + colb + Nxy * k);
            }
          else
            atomicAdd(d, to_storage<TS, T>(U[k * SZ + i1 * N + i0]));
        }
    }

    template <int N, typename TS, typename T = TS>
    EOMat<N, T>
    eo_mat(const TS (&M)[N][N])
    {
      constexpr int H = N / 2;
      EOMat<N, T>   r{};
      for (int i = 0; i < H; ++i)
        for (int j = 0; j < H; ++j)
          {
            r.E[i][j] = conv_host<T>((double(M[i][j]) + double(M[i][N - 1 - j])) / 2);
            r.O[i][j] = conv_host<T>((double(M[i][j]) - double(M[i][N - 1 - j])) / 2);
          }
      if (N & 1)
        {
          for (int i = 0; i < H; ++i)
            {
              r.C[i] = conv_host<T>(double(M[i][H]));
              r.R[i] = conv_host<T>(double(M[H][i]));
            }
          r.C[H] = conv_host<T>(double(M[H][H]));
        }
      return r;
    }

    template <int N, typename TS, typename T = TS>
    cudaError_t
    launch_block(const HostBasis &b, const LevelGeom &g, const HeatTPArgs &a, cudaStream_t s)
    {
      constexpr int      CPB  = blk_cells<N, T>();
      const size_t       smem = size_t(CPB) * BlkLay<N, T>::CS * sizeof(T);
      const HeatTP<N, TS> h0  = make_matrices<N, TS>(b, g, a.kdt);
      HeatTPEO<N, T>     h;
      h.Mx = eo_mat<N, TS, T>(h0.Mx);
      h.Ax = eo_mat<N, TS, T>(h0.Ax);
      h.My = eo_mat<N, TS, T>(h0.My);
      h.Ky = eo_mat<N, TS, T>(h0.Ky);
      h.Mz = eo_mat<N, TS, T>(h0.Mz);
      h.Kz = eo_mat<N, TS, T>(h0.Kz);
      CellGeom<T>        cg  = make_cell_geom<T>(g);
      cg.batch               = unsigned(a.batch > 1 ? a.batch : 1);
      cg.bstride             = a.batch > 1 ? a.bstride : 0;
      const size_t layer     = size_t(g.C[0]) * size_t(g.C[1]);
      cg.cell_begin          = unsigned(size_t(a.zc0) * layer);
      cg.cell_end            = unsigned(size_t(a.zc1) * layer);
      const size_t cells     = cg.cell_end - cg.cell_begin;
      if (cells == 0)
        return cudaSuccess;
      const size_t grid = (cells + CPB - 1) / CPB;
      if (grid > 0x7fffffffu || cg.batch > 65535u || smem > 48 * 1024)
        return cudaErrorInvalidValue;
      const dim3 gr(unsigned(grid), cg.batch);
      if (a.constrained)
        heat_tp_block_kernel<N, TS, T, true><<<gr, CPB * N * N, smem, s>>>(h, cg, static_cast<const TS *>(a.src),
                                                                           static_cast<TS *>(a.dst));
      else
        heat_tp_block_kernel<N, TS, T, false><<<gr, CPB * N * N, smem, s>>>(h, cg, static_cast<const TS *>(a.src),
                                                                            static_cast<TS *>(a.dst));
      return cudaGetLastError();
    }

    // -------------------------------------------------------------------
    // FP32 bricks staged by the tensor memory accelerator.
    //
    // A CTA takes bricks of 32 x BY x BZ cells (one cell per thread, x
    // fastest) in a persistent loop.  The brick's node box, (32p+1) x
    // (BY p+1) x (BZ p+1) nodes, is loaded row by row (x-rows of the node
    // grid) by 1D tiled TMA copies into shared memory, double-buffered: the
    // next brick's rows are in flight while the current brick is computed.
    // A row of the node grid starts at any float (the row length C0 p + 1 is
    // odd in general), and a TMA box must start on 16 bytes: each copy starts
    // at the row's first node rounded down to a multiple of 4 and is ROW
    // floats long; the cells index the row from its offset.  Each thread
    // computes its cell from the staged values (the same sweeps as above)
    // and adds its results into a shared-memory output box (shared atomics);
    // the box is then added to dst row by row by TMA bulk reductions
    // (cp.reduce.async.bulk.tensor .add), which the L2 performs atomically,
    // so no global atomics are issued.  The rounded copies load and add
    // slack floats of the neighbouring rows: loads are ignored, adds are of
    // zero.  The tensor maps are 1D over the whole vector (all problems of a
    // batch), so copies past its end are clipped by the hardware.
    // Constrained nodes: read as zero by the cells; the node's owning brick
    // (node index below the brick's upper face in every direction, or on
    // the domain's last one) writes src into its output box, the others 0.
    // Every mbarrier wait is bounded: past its limit the CTA sets the error
    // flag, waits for its copies in flight and returns.
    // Measured on 64^3 cells (CUDA events, L2 flushed), it is slower than the
    // register kernel for every brick shape tried (32 x 2 x 2, 32 x 4 x 2,
    // 32 x 4 x 4): Q1 14.0 against 9.9 us, Q2 40.6 against 26-30 us, Q3
    // 126 against 80 us; the brick's serial phases (wait, compute, shared
    // atomics, barrier, reduction) leave the SMs idle where the register
    // kernel's independent threads overlap.  So it is an opt-in (cell
    // kernel 5), not the default.
    // -------------------------------------------------------------------
    template <int N, int BY, int BZ>
    struct Brick
    {
      static constexpr int P       = N - 1;
      static constexpr int BX      = 32;
      static constexpr int THREADS = BX * BY * BZ;
      static constexpr int RX      = BX * P + 1;                // nodes of a row in the brick
      static constexpr int RY = BY * P + 1, RZ = BZ * P + 1;    // rows
      static constexpr int ROWS    = RY * RZ;
      static constexpr int ROW     = (RX + 3 + 3) / 4 * 4;      // floats per copy: up to 3 of slack before
      static constexpr int PITCH   = (ROW * 4 + 127) / 128 * 32; // floats per shared row (128-byte rows)
      static constexpr int BOX     = ROWS * PITCH;
      // in[2], out, 2 mbarriers, and 128 bytes to align the base
      static constexpr size_t SMEM = size_t(3 * BOX) * 4 + 64 + 128;
      static_assert(ROW <= 256, "TMA box too long");
    };

    __device__ __forceinline__ uint32_t
    saddr(const void *p)
    {
      return static_cast<uint32_t>(__cvta_generic_to_shared(p));
    }

    __device__ __forceinline__ bool
    mbar_try_wait(uint64_t *bar, unsigned parity)
    {
      uint32_t ok;
      asm volatile("{\n\t.reg .pred p;\n\t"
                   "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                   "selp.u32 %0, 1, 0, p;\n\t}"
                   : "=r"(ok)
                   : "r"(saddr(bar)), "r"(parity)
                   : "memory");
      return ok != 0;
    }

    // bounded wait: false after the limit
    __device__ __forceinline__ bool
    mbar_wait(uint64_t *bar, unsigned parity)
    {
      for (int i = 0; i < (1 << 22); ++i)
        if (mbar_try_wait(bar, parity))
          return true;
      return false;
    }

    template <int N, int BY, int BZ, bool CON>
    __global__ void __launch_bounds__(Brick<N, BY, BZ>::THREADS)
    heat_tp_tma_kernel(const __grid_constant__ CUtensorMap tsrc, const __grid_constant__ CUtensorMap tdst,
                       const __grid_constant__ HeatTP<N, float> m, const __grid_constant__ CellGeom<float> g,
                       const float *__restrict__ srcv, int *err)
    {
      using B                = Brick<N, BY, BZ>;
      constexpr int P        = N - 1;
      extern __shared__ __align__(128) unsigned char sm_raw[];
      // TMA rows start on 128 bytes
      float *sm = reinterpret_cast<float *>(sm_raw + ((128u - (saddr(sm_raw) & 127u)) & 127u));
      float    *in0  = sm;
      float    *out  = sm + 2 * B::BOX;
      uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + 3 * B::BOX);
      const int C0 = g.C[0], C1 = g.C[1], C2 = g.C[2];
      const int Nx = g.Nn[0], Ny = g.Nn[1], Nz = g.Nn[2];
      const int nbx = (C0 + B::BX - 1) / B::BX, nby = (C1 + BY - 1) / BY, nbz = (C2 + BZ - 1) / BZ;
      const unsigned nbrick = unsigned(nbx) * unsigned(nby) * unsigned(nbz) * g.batch;
      const int tid = int(threadIdx.x), lane = tid & 31, warp = tid >> 5;
      const int tx = tid % B::BX, ty = (tid / B::BX) % BY, tz = tid / (B::BX * BY);

      struct Pos
      {
        int      x0, y0, z0, ry, rz; // first node, rows in y and z
        unsigned prob;
        int      bx, by, bz;
      };
      auto pos = [&](unsigned br) {
        Pos q;
        q.bx      = int(br % unsigned(nbx));
        unsigned r = br / unsigned(nbx);
        q.by      = int(r % unsigned(nby));
        r /= unsigned(nby);
        q.bz      = int(r % unsigned(nbz));
        q.prob    = r / unsigned(nbz);
        q.x0      = q.bx * B::BX * P;
        q.y0      = q.by * BY * P;
        q.z0      = q.bz * BZ * P;
        q.ry      = min(B::RY, Ny - q.y0);
        q.rz      = min(B::RZ, Nz - q.z0);
        return q;
      };
      // flat index of the first node of row (j, l) of a brick
      auto row_flat = [&](const Pos &q, int j, int l) {
        return size_t(q.prob) * g.n_nodes + size_t(q.x0) +
               size_t(Nx) * (size_t(q.y0 + j) + size_t(Ny) * size_t(q.z0 + l));
      };
      // warp 0 issues the rows of brick q into buffer buf
      auto issue_loads = [&](const Pos &q, int buf) {
        if (warp != 0)
          return;
        uint64_t *bar = mbar + buf;
        if (lane == 0)
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)),
                       "r"(unsigned(q.ry * q.rz * B::ROW * 4))
                       : "memory");
        __syncwarp();
        float *dstb = in0 + buf * B::BOX;
        for (int r = lane; r < q.ry * q.rz; r += 32)
          {
            const int    j = r % q.ry, l = r / q.ry;
            const size_t f = row_flat(q, j, l);
            const int    c = int(f & ~size_t(3));
            asm volatile("cp.async.bulk.tensor.1d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                         " [%0], [%1, {%2}], [%3];" ::"r"(saddr(dstb + (l * B::RY + j) * B::PITCH)),
                         "l"(&tsrc), "r"(c), "r"(saddr(bar))
                         : "memory");
          }
      };

      if (tid == 0)
        {
          asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(mbar + 0)) : "memory");
          asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(mbar + 1)) : "memory");
          asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
      __syncthreads();
      // copies issued into each buffer and waited for (the k-th copy into a
      // buffer completes its mbarrier's phase k-1, parity (k-1) & 1)
      unsigned issued[2] = {0u, 0u}, landed[2] = {0u, 0u};
      unsigned br = blockIdx.x;
      if (br < nbrick)
        {
          issue_loads(pos(br), 0);
          ++issued[0];
        }
      bool failed = false;
      for (int it = 0; br < nbrick; ++it, br += gridDim.x)
        {
          const int  buf = it & 1;
          const Pos  q   = pos(br);
          // the previous brick's reductions have read the output box
          if (warp == 0)
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
          __syncthreads();
          {
            float4 *o4 = reinterpret_cast<float4 *>(out);
            for (int i = tid; i < B::BOX / 4; i += B::THREADS)
              o4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
          // the next brick's rows into the other buffer (its cells were
          // computed before the barrier above)
          const unsigned brn = br + gridDim.x;
          if (brn < nbrick)
            {
              issue_loads(pos(brn), buf ^ 1);
              ++issued[buf ^ 1];
            }
          if (mbar_wait(mbar + buf, (issued[buf] - 1) & 1u))
            ++landed[buf];
          else
            {
              failed = true;
              if (tid == 0)
                atomicOr(err, 8);
            }
          if (__syncthreads_or(failed))
            {
              failed = true;
              break;
            }
          const float *inb = in0 + buf * B::BOX;
          const int    cx = q.bx * B::BX + tx, cy = q.by * BY + ty, cz = q.bz * BZ + tz;
          const bool   act = cx < C0 && cy < C1 && cz < C2;
          if (act)
            {
              const bool fx0 = CON && cx == 0 && (g.face_mask[0] & 1u);
              const bool fx1 = CON && cx == C0 - 1 && (g.face_mask[1] & 1u);
              const bool fy0 = CON && cy == 0 && (g.face_mask[2] & 1u);
              const bool fy1 = CON && cy == C1 - 1 && (g.face_mask[3] & 1u);
              const bool fz0 = CON && cz == 0 && (g.face_mask[4] & 1u);
              const bool fz1 = CON && cz == C2 - 1 && (g.face_mask[5] & 1u);
              auto con = [&](int a, int b, int k) {
                return (a == 0 && fx0) || (a == P && fx1) || (b == 0 && fy0) || (b == P && fy1) ||
                       (k == 0 && fz0) || (k == P && fz1);
              };
              // shared index of local node (a, b, k): row (ty p + b, tz p + k),
              // from the row's offset
              int rowi[N][N];
#pragma unroll
              for (int k = 0; k < N; ++k)
#pragma unroll
                for (int b = 0; b < N; ++b)
                  {
                    const int j = ty * P + b, l = tz * P + k;
                    rowi[k][b] = (l * B::RY + j) * B::PITCH + int(row_flat(q, j, l) & 3) + tx * P;
                  }
              float x[N][N][N];
#pragma unroll
              for (int k = 0; k < N; ++k)
#pragma unroll
                for (int b = 0; b < N; ++b)
#pragma unroll
                  for (int a = 0; a < N; ++a)
                    x[k][b][a] = (CON && con(a, b, k)) ? 0.f : inb[rowi[k][b] + a];
              float y[N][N][N];
              cell_apply<N, float>(m, x, y);
#pragma unroll
              for (int k = 0; k < N; ++k)
#pragma unroll
                for (int b = 0; b < N; ++b)
#pragma unroll
                  for (int a = 0; a < N; ++a)
                    if (!(CON && con(a, b, k)))
                      atomicAdd(out + rowi[k][b] + a, y[k][b][a]);
            }
          __syncthreads();
          if (CON)
            {
              // constrained nodes this brick owns: dst += src
              const int  nx    = min(B::RX, Nx - q.x0);
              const bool touch = (q.bx == 0 && (g.face_mask[0] & 1u)) || (q.bx == nbx - 1 && (g.face_mask[1] & 1u)) ||
                                 (q.by == 0 && (g.face_mask[2] & 1u)) || (q.by == nby - 1 && (g.face_mask[3] & 1u)) ||
                                 (q.bz == 0 && (g.face_mask[4] & 1u)) || (q.bz == nbz - 1 && (g.face_mask[5] & 1u));
              if (touch)
                for (int i = tid; i < nx * q.ry * q.rz; i += B::THREADS)
                  {
                    const int a = i % nx, r = i / nx, j = r % q.ry, l = r / q.ry;
                    const int ix = q.x0 + a, iy = q.y0 + j, iz = q.z0 + l;
                    const bool c = (ix == 0 && (g.face_mask[0] & 1u)) || (ix == Nx - 1 && (g.face_mask[1] & 1u)) ||
                                   (iy == 0 && (g.face_mask[2] & 1u)) || (iy == Ny - 1 && (g.face_mask[3] & 1u)) ||
                                   (iz == 0 && (g.face_mask[4] & 1u)) || (iz == Nz - 1 && (g.face_mask[5] & 1u));
                    const bool own = (a < B::RX - 1 || ix == Nx - 1) && (j < B::RY - 1 || iy == Ny - 1) &&
                                     (l < B::RZ - 1 || iz == Nz - 1);
                    if (c && own)
                      {
                        const int si = (l * B::RY + j) * B::PITCH + int(row_flat(q, j, l) & 3) + a;
                        out[si]      = srcv[row_flat(q, j, l) + a];
                      }
                  }
            }
          // the output box to dst: generic-proxy writes made visible to the
          // bulk copies, then one reduction per row
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncthreads();
          if (warp == 0)
            {
              for (int r = lane; r < q.ry * q.rz; r += 32)
                {
                  const int    j = r % q.ry, l = r / q.ry;
                  const size_t f = row_flat(q, j, l);
                  const int    c = int(f & ~size_t(3));
                  asm volatile("cp.reduce.async.bulk.tensor.1d.global.shared::cta.add.tile.bulk_group"
                               " [%0, {%1}], [%2];" ::"l"(&tdst),
                               "r"(c), "r"(saddr(out + (l * B::RY + j) * B::PITCH))
                               : "memory");
                }
              asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            }
        }
      if (failed)
        {
          // copies still in flight into this CTA's buffers: wait for them
          // (bounded) before the CTA exits
          for (int b = 0; b < 2; ++b)
            if (issued[b] > landed[b])
              mbar_wait(mbar + b, (issued[b] - 1) & 1u);
        }
      if (warp == 0)
        asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
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
    // cuTensorMapEncodeTiled through the runtime's driver entry point (no
    // link against libcuda)
    using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

    EncodeFn
    encode_fn()
    {
      static std::once_flag once;
      static EncodeFn       fn = nullptr;
      std::call_once(once, [] {
        void                           *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
              cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
          fn = reinterpret_cast<EncodeFn>(p);
      });
      return fn;
    }

    // 1D map over n floats at ptr, boxes of `box` floats, zero fill
    bool
    encode_rows(CUtensorMap *map, const void *ptr, size_t n, int box)
    {
      EncodeFn fn = encode_fn();
      if (!fn || (reinterpret_cast<uintptr_t>(ptr) & 15u) || n == 0 || n >= (size_t(1) << 32))
        return false;
      const cuuint64_t dim[1]    = {cuuint64_t(n)};
      const cuuint64_t stride[1] = {cuuint64_t(n * 4)}; // unused for rank 1
      const cuuint32_t bx[1]     = {cuuint32_t(box)};
      const cuuint32_t es[1]     = {1};
      return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 1, const_cast<void *>(ptr), dim, stride, bx, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    }

    // resident CTAs per SM of a kernel and the SM count, per device
    template <typename K>
    int
    resident_ctas(K kernel, int threads, size_t smem, int &sms)
    {
      int dev = 0;
      if (cudaGetDevice(&dev) != cudaSuccess)
        return 0;
      static std::mutex                                        mu;
      static std::vector<std::tuple<const void *, int, int, int>> seen; // kernel, device, ctas, sms
      std::lock_guard<std::mutex>                              l(mu);
      for (auto &e : seen)
        if (std::get<0>(e) == reinterpret_cast<const void *>(kernel) && std::get<1>(e) == dev)
          {
            sms = std::get<3>(e);
            return std::get<2>(e);
          }
      int ctas = 0;
      if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas, kernel, threads, smem) != cudaSuccess ||
          cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
      seen.emplace_back(reinterpret_cast<const void *>(kernel), dev, ctas, sms);
      return ctas;
    }

    // the TMA brick kernel over all cells (false: not applicable, nothing
    // launched)
    template <int N, int BY, int BZ>
    bool
    launch_tma(const HostBasis &b, const LevelGeom &g, const HeatTPArgs &a, cudaStream_t s, cudaError_t &e)
    {
      using Bk            = Brick<N, BY, BZ>;
      const unsigned nb   = unsigned(a.batch > 1 ? a.batch : 1);
      const size_t   tot  = g.n_nodes * nb;
      CUtensorMap    ms, md;
      // row coordinates are 32-bit signed
      if (!a.err || tot >= (size_t(1) << 31) || !encode_rows(&ms, a.src, tot, Bk::ROW) ||
          !encode_rows(&md, a.dst, tot, Bk::ROW))
        return false;
      auto k   = a.constrained ? heat_tp_tma_kernel<N, BY, BZ, true> : heat_tp_tma_kernel<N, BY, BZ, false>;
      int  sms = 0;
      const int ctas = resident_ctas(k, Bk::THREADS, Bk::SMEM, sms);
      if (ctas <= 0)
        return false;
      const HeatTP<N, float> h  = make_matrices<N, float>(b, g, a.kdt);
      CellGeom<float>        cg = make_cell_geom<float>(g);
      cg.batch                  = nb;
      cg.bstride                = nb > 1 ? a.bstride : 0;
      const size_t bricks = size_t((g.C[0] + Bk::BX - 1) / Bk::BX) * size_t((g.C[1] + BY - 1) / BY) *
                            size_t((g.C[2] + BZ - 1) / BZ) * nb;
      const size_t grid = std::min(bricks, size_t(ctas) * size_t(sms));
      if (grid == 0)
        {
          e = cudaSuccess;
          return true;
        }
      k<<<unsigned(grid), Bk::THREADS, Bk::SMEM, s>>>(ms, md, h, cg, static_cast<const float *>(a.src), a.err);
      e = cudaGetLastError();
      return true;
    }
  } // namespace tp

  namespace tp
  {
    // The diagonal of the assembled heat operator on a box level.  The cells
    // form a Cartesian product, so the assembled operator is the same sum of
    // Kronecker products as the element operator, of the assembled 1D
    // matrices: diag = vol [dMz dMy dMx + c0 dMz dMy dKx + c1 dMz dKy dMx +
    // c2 dKz dMy dMx] with c_d = kdt / h_d^2, where the assembled 1D
    // diagonal at node i = c p + a is the element diagonal at a for an
    // interior node (0 < a < p) and the sum of the two elements' end entries
    // at a vertex.  Rows of constrained nodes are set by the caller.
    struct HeatDiag
    {
      int    N, p, C[3], Nn[3];
      size_t n_nodes;
      double m[MAX_N], k[MAX_N]; // element diagonals of M and K on [0,1]
      double vol, c[3];
    };

    __device__ __forceinline__ void
    diag1d(const HeatDiag &d, int i, int dir, double &m, double &k)
    {
      const int c = i / d.p, a = i - c * d.p;
      if (a != 0)
        {
          m = d.m[a];
          k = d.k[a];
          return;
        }
      m = (c > 0 ? d.m[d.p] : 0.0) + (c < d.C[dir] ? d.m[0] : 0.0);
      k = (c > 0 ? d.k[d.p] : 0.0) + (c < d.C[dir] ? d.k[0] : 0.0);
    }

    template <typename T>
    __global__ void
    heat_diag_kernel(const __grid_constant__ HeatDiag d, T *__restrict__ out)
    {
      for (size_t n = size_t(blockIdx.x) * blockDim.x + threadIdx.x; n < d.n_nodes;
           n += size_t(gridDim.x) * blockDim.x)
        {
          const int ix = int(n % size_t(d.Nn[0]));
          const int iy = int((n / size_t(d.Nn[0])) % size_t(d.Nn[1]));
          const int iz = int(n / (size_t(d.Nn[0]) * size_t(d.Nn[1])));
          double    mx, kx, my, ky, mz, kz;
          diag1d(d, ix, 0, mx, kx);
          diag1d(d, iy, 1, my, ky);
          diag1d(d, iz, 2, mz, kz);
          out[n] = T(d.vol * (mz * my * (mx + d.c[0] * kx) + d.c[1] * mz * ky * mx + d.c[2] * kz * my * mx));
        }
    }
  } // namespace tp

  cudaError_t
  launch_heat_diag_tp(const HostBasis &b, const LevelGeom &g, int precision, double kdt, void *out, cudaStream_t s)
  {
    if (g.dim == 2 || b.N < 2 || b.N > MAX_N || g.p != b.N - 1)
      return cudaErrorInvalidValue;
    tp::HeatDiag d{};
    d.N       = b.N;
    d.p       = b.N - 1;
    d.n_nodes = g.n_nodes;
    for (int dir = 0; dir < 3; ++dir)
      {
        d.C[dir]  = g.C[dir];
        d.Nn[dir] = g.Nn[dir];
        d.c[dir]  = kdt / (g.h[dir] * g.h[dir]);
      }
    d.vol = g.h[0] * g.h[1] * g.h[2];
    for (int i = 0; i < b.N; ++i)
      {
        double m = 0, k = 0;
        for (int q = 0; q < b.N; ++q)
          {
            m += b.w[q] * b.S[q * b.N + i] * b.S[q * b.N + i];
            k += b.w[q] * b.G[q * b.N + i] * b.G[q * b.N + i];
          }
        d.m[i] = m;
        d.k[i] = k;
      }
    const size_t blocks = std::min<size_t>((g.n_nodes + 255) / 256, size_t(152) * 32);
    if (blocks == 0)
      return cudaSuccess;
    if (precision == 32)
      tp::heat_diag_kernel<float><<<unsigned(blocks), 256, 0, s>>>(d, static_cast<float *>(out));
    else
      tp::heat_diag_kernel<double><<<unsigned(blocks), 256, 0, s>>>(d, static_cast<double *>(out));
    return cudaGetLastError();
  }

  bool
  heat_tp_supported(int N, int precision)
  {
    return (precision == 32 || precision == 64) && N >= 2 && N <= 7;
  }

  int
  heat_tp_zlen(const LevelGeom &g, int zc0, int zc1, int N, int precision)
  {
    // measured on 64^3 cells: two cells per thread where the next cell's
    // values are prefetched (FP32 Q1-Q2, FP64 Q1), one otherwise; one as
    // well where two would leave fewer than 256 threads per SM
    const size_t ncol = size_t(g.C[0]) * size_t(g.C[1]);
    const int    nz   = zc1 - zc0;
    int          zlen = size_t(N) * N * N * (precision / 8) <= 27 * 4 ? 2 : 1;
    while (zlen > 1 && ncol * size_t((nz + zlen - 1) / zlen) < size_t(152) * 256)
      zlen /= 2;
    return zlen;
  }

  cudaError_t
  launch_heat_tp(const HostBasis &b, const LevelGeom &g, int precision, const HeatTPArgs &a, cudaStream_t s)
  {
    if (g.dim == 2 || !heat_tp_supported(b.N, precision) || a.zc0 < 0 || a.zc1 > g.C[2] || a.zlen < 1)
      return cudaErrorInvalidValue;
    // FP32 Q1 and Q2 over all cells, 16-byte aligned vectors, on request:
    // the TMA brick kernel
    if (precision == 32 && a.tma && !a.df64 && a.zc0 == 0 && a.zc1 == g.C[2] && (a.batch <= 1 || a.bstride == g.n_nodes))
      {
        cudaError_t e  = cudaSuccess;
        bool        ok = false;
        if (b.N == 2)
          ok = tp::launch_tma<2, 2, 2>(b, g, a, s, e);
        else if (b.N == 3)
          ok = tp::launch_tma<3, 2, 2>(b, g, a, s, e);
        if (ok)
          return e;
      }
    // double-float arithmetic on FP64 vectors: the block kernel
    if (precision == 64 && a.df64)
      switch (b.N)
        {
          case 2: return tp::launch_block<2, double, df64>(b, g, a, s);
          case 3: return tp::launch_block<3, double, df64>(b, g, a, s);
          case 4: return tp::launch_block<4, double, df64>(b, g, a, s);
          case 5: return tp::launch_block<5, double, df64>(b, g, a, s);
          case 6: return tp::launch_block<6, double, df64>(b, g, a, s);
          case 7: return tp::launch_block<7, double, df64>(b, g, a, s);
        }
    // one thread per cell in registers at Q1 from 16384 cells on, the block
    // kernel above otherwise (measured with the padded block layout, CUDA
    // events, L2 flushed: 64^3 cells Q2 FP32 30.9 us in registers, 29.3 us
    // in blocks, FP64 314 against 246 us; Q1 FP64 70.3 against 70.0 us;
    // 16^3 cells FP64 Q2 32 us in registers, 12 us in blocks)
    const size_t cells = size_t(a.zc1 - a.zc0) * size_t(g.C[0]) * size_t(g.C[1]);
    const bool   regs  = cells >= 16384;
    if (precision == 32)
      switch (b.N)
        {
          case 2: return regs ? tp::launch<2, float>(b, g, a, s) : tp::launch_block<2, float>(b, g, a, s);
          case 3: return tp::launch_block<3, float>(b, g, a, s);
          case 4: return tp::launch_block<4, float>(b, g, a, s);
          case 5: return tp::launch_block<5, float>(b, g, a, s);
          case 6: return tp::launch_block<6, float>(b, g, a, s);
          case 7: return tp::launch_block<7, float>(b, g, a, s);
        }
    else
      switch (b.N)
        {
          case 2: return regs ? tp::launch<2, double>(b, g, a, s) : tp::launch_block<2, double>(b, g, a, s);
          case 3: return tp::launch_block<3, double>(b, g, a, s);
          case 4: return tp::launch_block<4, double>(b, g, a, s);
          case 5: return tp::launch_block<5, double>(b, g, a, s);
          case 6: return tp::launch_block<6, double>(b, g, a, s);
          case 7: return tp::launch_block<7, double>(b, g, a, s);
        }
    return cudaErrorInvalidValue;
  }
} // namespace mfgpu
