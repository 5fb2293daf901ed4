// Setup-phase cell kernels: the linearisation cache of the neo-Hookean
// tangent (NeoHookOperator::cache, mf_nh_operator.h:394-523), the operator
// diagonals (compute_diagonal, mf_nh_operator.h:1025-1060,
// heat_transfer.h:205-230) and the Newton residual
// (Solid::assemble_residual, mf_elasticity.h:1766-1845).
#pragma once

#include "mf_cell.cuh"

namespace mfgpu
{
  template <typename T>
  __device__ __forceinline__ T
  det3(const T (&F)[3][3])
  {
    return F[0][0] * (F[1][1] * F[2][2] - F[1][2] * F[2][1]) -
           F[0][1] * (F[1][0] * F[2][2] - F[1][2] * F[2][0]) +
           F[0][2] * (F[1][0] * F[2][1] - F[1][1] * F[2][0]);
  }

  template <typename T>
  __device__ __forceinline__ void
  inv3(const T (&F)[3][3], T det, T (&Fi)[3][3])
  {
    const T id = T(1) / det;
    Fi[0][0]   = (F[1][1] * F[2][2] - F[1][2] * F[2][1]) * id;
    Fi[0][1]   = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) * id;
    Fi[0][2]   = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) * id;
    Fi[1][0]   = (F[1][2] * F[2][0] - F[1][0] * F[2][2]) * id;
    Fi[1][1]   = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) * id;
    Fi[1][2]   = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) * id;
    Fi[2][0]   = (F[1][0] * F[2][1] - F[1][1] * F[2][0]) * id;
    Fi[2][1]   = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) * id;
    Fi[2][2]   = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) * id;
  }

  // gather the z-column (x=a, y=b) of component c of cell (cx,cy,cz), plain
  template <int N, typename T>
  __device__ __forceinline__ void
  gather_plain(const CellGeom<T> &g, const T *__restrict__ v, int c, int cx,
               int cy, int cz, int a, int b, bool active, T (&col)[N])
  {
#pragma unroll
    for (int k = 0; k < N; ++k)
      col[k] = active ? __ldg(v + size_t(c) * g.n_nodes + node_index(g, cx, cy, cz, a, b, k)) : T(0);
  }

  // ---------------------------------------------------------------------
  // NH cache: per quadrature point fields of the chosen variant
  // ---------------------------------------------------------------------
  template <int N, typename T, int VAR, typename TO = T>
  __global__ void __launch_bounds__(cells_per_block<N, 3, T>() * N * N)
  nh_cache_kernel(const __grid_constant__ Shape<N, T> sh,
                  const __grid_constant__ CellGeom<T> g, const NHMat<T> m,
                  const T *__restrict__ u, TO *__restrict__ cache,
                  TO *__restrict__ ucell, int *__restrict__ err)
  {
    constexpr int N2  = N * N;
    constexpr int N3  = N * N * N;
    constexpr int CPB = cells_per_block<N, 3, T>();
    constexpr int SPC = smem_per_cell<N, 3, false>();
    constexpr int NF  = nh_cache_fields(VAR);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T             *sm     = reinterpret_cast<T *>(smem_raw);
    const int      lc     = threadIdx.x / N2;
    const int      l      = threadIdx.x - lc * N2;
    const int      a      = l % N, b = l / N;
    const unsigned cell   = blockIdx.x * CPB + lc;
    const bool     active = cell < g.n_cells;
    const unsigned cc     = active ? cell : 0u;
    const int      cx = int(cc % unsigned(g.C[0])), cyz = int(cc / unsigned(g.C[0]));
    const int      cy = cyz % g.C[1], cz = cyz / g.C[1];
    T             *cb = sm + lc * SPC;
    T             *T0 = cb + 12 * N3;
    T             *T1 = T0 + N3;
#pragma unroll 1
    for (int c = 0; c < 3; ++c)
      {
        T col[N];
        gather_plain<N>(g, u, c, cx, cy, cz, a, b, active, col);
        if (VAR == V_SCALAR_REF && active)
#pragma unroll
          for (int k = 0; k < N; ++k)
            ucell[(size_t(cc) * 3 + c) * N3 + a + b * N + k * N2] = to_compute<TO, T>(col[k]);
        T *V = cb + c * 4 * N3;
        evaluate_field<N>(sh, col, V, V + N3, V + 2 * N3, V + 3 * N3, T0, T1, a, b, true);
      }
    __syncthreads();
    if (!active)
      return;
#pragma unroll 1
    for (int k = 0; k < N; ++k)
      {
        const int q = a + b * N + k * N2;
        T         H[3][3], F[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            {
              H[i][j] = cb[i * 4 * N3 + (j + 1) * N3 + q] * g.inv_h[j];
              F[i][j] = H[i][j] + (i == j ? T(1) : T(0));
            }
        const T Jm1 = jm1_from_grad3(H);
        const T J   = T(1) + Jm1;
        if (!(J > T(0)))
          {
            atomicOr(err, 1);
            continue;
          }
        T Fi[3][3];
        inv3(F, J, Fi);
        TO      *cp     = cache + size_t(cc) * NF * N3 + q;
        auto     st     = [&](int f, T v) { cp[size_t(f) * N3] = to_compute<TO, T>(v); };
        const T  lnJ    = log1p(Jm1);
        const T  scalar = m.mu - T(2.0) * m.lambda * lnJ;
        if constexpr (VAR == V_SCALAR_REF)
          {
            st(0, scalar);
          }
        else if constexpr (VAR == V_QP10)
          {
            // M~ = F^{-T} diag(1/h): the operator works with reference-cell
            // gradients (see NHQp10QOp)
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j < 3; ++j)
                st((i * 3 + j), Fi[j][i] * g.inv_h[j]);
            st(9, scalar);
          }
        else if constexpr (VAR == V_TENSOR4_NS)
          {
#pragma unroll 1
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j)
                for (int k2 = 0; k2 < 3; ++k2)
                  for (int l2 = 0; l2 < 3; ++l2)
                    st((((i * 3 + j) * 3 + k2) * 3 + l2), T(2.) * m.lambda * Fi[j][i] * Fi[l2][k2] +
                      scalar * Fi[l2][i] * Fi[j][k2] +
                      (i == k2 && j == l2 ? m.mu : T(0)));
          }
        else
          {
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j < 3; ++j)
                st((i * 3 + j), Fi[i][j]);
            st(9, J);
            if constexpr (VAR == V_FORM0)
              {
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                  for (int j = 0; j < 3; ++j)
                    st((10 + i * 3 + j), F[i][j]);
                st(19, exp(lnJ * T(-1.0 / 3.0)));
              }
            else
              {
                // tau = mu b - (mu - 2 lambda ln J) I
                //     = mu (H + H^T + H H^T) + 2 lambda ln J I
                T tau[3][3];
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                  for (int j = 0; j < 3; ++j)
                    tau[i][j] = m.mu * (H[i][j] + H[j][i] +
                                        (H[i][0] * H[j][0] + H[i][1] * H[j][1] + H[i][2] * H[j][2])) +
                                (i == j ? T(2.0) * m.lambda * lnJ : T(0));
                const T iJ = T(1.) / J;
                if constexpr (VAR == V_TENSOR2)
                  {
                    st(10, scalar * T(2.) / J);
                    st(11, iJ);
                    st(12, tau[0][0] / J);
                    st(13, tau[1][1] / J);
                    st(14, tau[2][2] / J);
                    st(15, tau[0][1] / J);
                    st(16, tau[0][2] / J);
                    st(17, tau[1][2] / J);
                  }
                else // V_TENSOR4
                  {
                    st(10, iJ);
                    st(11, tau[0][0] / J);
                    st(12, tau[1][1] / J);
                    st(13, tau[2][2] / J);
                    st(14, tau[0][1] / J);
                    st(15, tau[0][2] / J);
                    st(16, tau[1][2] / J);
                    const T aa = scalar * T(2.) / J;
                    const T bl = m.lambda * T(2.) / J;
                    // C4 : sym(g) in Voigt form with off-diagonal inputs g_kl + g_lk
                    const int vi[6] = {0, 1, 2, 0, 0, 1};
                    const int vj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll 1
                    for (int r = 0; r < 6; ++r)
                      for (int s = 0; s < 6; ++s)
                        {
                          const int i = vi[r], j = vj[r], k2 = vi[s], l2 = vj[s];
                          const T   C = aa * T(0.5) * (T(i == k2 && j == l2) + T(i == l2 && j == k2)) +
                                      bl * T(i == j && k2 == l2);
                          st((17 + r * 6 + s), C);
                        }
                  }
              }
          }
      }
  }

  // ---------------------------------------------------------------------
  // Diagonal: for every cell and component, the diagonal of the local
  // operator, by tensor-product contraction of the qp tangent blocks
  //   diag_c(i,j,k) = sum_q [ mass(q) S_i^2 S_j^2 S_k^2
  //                          + sum_de A_cde(q) dphi_d dphi_e ] JxW(q)
  // (the same numbers MatrixFreeTools::compute_diagonal obtains by applying
  // the cell operator to local unit vectors).
  // KIND: 0 heat (A = kdt I, mass 1), 1 NH formulation 1, 2 NH formulation 0.
  // ---------------------------------------------------------------------
  template <int N, typename T>
  struct DiagShape
  {
    T SS[N * N]; // S^2
    T SG[N * N]; // S*G
    T GG[N * N]; // G^2   (G = D S, derivative of the nodal basis)
    T w[N];
  };

  template <int N, typename T>
  __device__ __forceinline__ const T *
  diag_mat(const DiagShape<N, T> &ds, int kind)
  {
    return kind == 0 ? ds.SS : (kind == 1 ? ds.SG : ds.GG);
  }

  // matrix kind of direction dir for pair (d,e): 0 SS, 1 SG, 2 GG
  __device__ __forceinline__ int
  pair_kind(int dir, int d, int e)
  {
    return (dir == d) + (dir == e);
  }

  template <int N, typename T, int KIND>
  __global__ void __launch_bounds__(cells_per_block<N, 3, T>() * N * N)
  diag_kernel(const __grid_constant__ Shape<N, T> sh,
              const __grid_constant__ DiagShape<N, T> ds,
              const __grid_constant__ CellGeom<T> g, const NHMat<T> m, T kdt,
              const T *__restrict__ u, T *__restrict__ diag)
  {
    constexpr int N2  = N * N;
    constexpr int N3  = N * N * N;
    constexpr int NC  = KIND == 0 ? 1 : 3;
    constexpr int CPB = cells_per_block<N, 3, T>();
    // smem per cell: grad u (9 N3, NH only) + 7 pair buffers + T0/T1
    constexpr int SPC = (KIND == 0 ? 0 : 12 * N3) + 9 * N3;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T             *sm     = reinterpret_cast<T *>(smem_raw);
    const int      lc     = threadIdx.x / N2;
    const int      l      = threadIdx.x - lc * N2;
    const int      a      = l % N, b = l / N;
    const unsigned cell   = blockIdx.x * CPB + lc;
    const bool     active = cell < g.n_cells;
    const unsigned cc     = active ? cell : 0u;
    const int      cx = int(cc % unsigned(g.C[0])), cyz = int(cc / unsigned(g.C[0]));
    const int      cy = cyz % g.C[1], cz = cyz / g.C[1];
    T             *cb = sm + lc * SPC;
    T             *GU = cb;                                  // [c][4][N3] (V,G0,G1,G2)
    T             *PB = cb + (KIND == 0 ? 0 : 12 * N3);     // 7 pair buffers
    T             *T0 = PB;                                  // scratch during evaluate
    T             *T1 = PB + N3;
    if constexpr (KIND != 0)
      {
#pragma unroll 1
        for (int c = 0; c < 3; ++c)
          {
            T col[N];
            gather_plain<N>(g, u, c, cx, cy, cz, a, b, active, col);
            T *V = GU + c * 4 * N3;
            evaluate_field<N>(sh, col, V, V + N3, V + 2 * N3, V + 3 * N3, T0, T1, a, b, true);
          }
      }
    // pairs: 0..2 (d,d), 3 (0,1), 4 (0,2), 5 (1,2), 6 mass
    const int pd[7] = {0, 1, 2, 0, 0, 1, -1};
    const int pe[7] = {0, 1, 2, 1, 2, 2, -1};
#pragma unroll 1
    for (int c = 0; c < NC; ++c)
      {
        __syncthreads();
        // step 1: x-lines (qy=a, qz=b): weights W_p over qx, contracted in x
        {
          T W[7][N];
#pragma unroll
          for (int qx = 0; qx < N; ++qx)
            {
              const int q   = qx + a * N + b * N2;
              const T   jxw = sh.w[qx] * sh.w[a] * sh.w[b] * g.vol;
              T         A[3][3];
              T         mass;
              if constexpr (KIND == 0)
                {
#pragma unroll
                  for (int d = 0; d < 3; ++d)
#pragma unroll
                    for (int e = 0; e < 3; ++e)
                      A[d][e] = d == e ? kdt : T(0);
                  mass = T(1);
                }
              else
                {
                  T H[3][3], F[3][3];
#pragma unroll
                  for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j)
                      {
                        H[i][j] = GU[i * 4 * N3 + (j + 1) * N3 + q] * g.inv_h[j];
                        F[i][j] = H[i][j] + (i == j ? T(1) : T(0));
                      }
                  const T Jm1 = jm1_from_grad3(H);
                  const T J   = T(1) + Jm1;
                  T       Fi[3][3];
                  inv3(F, J, Fi);
                  mass = m.rho_alpha;
                  if constexpr (KIND == 1)
                    {
                      const T cl = m.mu - T(2.0) * m.lambda * log1p(Jm1) + T(2.0) * m.lambda;
#pragma unroll
                      for (int d = 0; d < 3; ++d)
#pragma unroll
                        for (int e = 0; e < 3; ++e)
                          A[d][e] = (d == e ? m.mu : T(0)) + cl * Fi[d][c] * Fi[e][c];
                    }
                  else
                    {
                      const T js = exp(log1p(Jm1) * T(-1.0 / 3.0));
#pragma unroll 1
                      for (int e = 0; e < 3; ++e)
                        {
                          // column e: H = E_ce
                          T gg[3][3], Pc[3][3];
#pragma unroll
                          for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int j = 0; j < 3; ++j)
                              gg[i][j] = (i == c) ? Fi[e][j] : T(0);
                          form0_flux_dev(m, F, js, gg, Pc);
#pragma unroll
                          for (int d = 0; d < 3; ++d)
                            A[d][e] = J * (Pc[c][0] * Fi[d][0] + Pc[c][1] * Fi[d][1] + Pc[c][2] * Fi[d][2]);
                        }
                    }
                }
#pragma unroll
              for (int p = 0; p < 7; ++p)
                {
                  T wv;
                  if (p < 3)
                    wv = A[p][p] * g.inv_h[p] * g.inv_h[p];
                  else if (p < 6)
                    wv = (A[pd[p]][pe[p]] + A[pe[p]][pd[p]]) * g.inv_h[pd[p]] * g.inv_h[pe[p]];
                  else
                    wv = mass;
                  W[p][qx] = wv * jxw;
                }
            }
          __syncthreads(); // T0/T1 aliases PB: evaluation scratch no longer needed
#pragma unroll
          for (int p = 0; p < 7; ++p)
            {
              if (KIND == 0 && p >= 3 && p < 6)
                continue;
              const T *M = diag_mat(ds, p == 6 ? 0 : pair_kind(0, pd[p], pe[p]));
              T        out[N];
              mat_apply_t<N>(M, W[p], out);
              store_line<N, T, 0>(PB + p * N3, a, b, out);
            }
        }
        __syncthreads();
        // step 2: y-lines (x=a, z=b)
#pragma unroll
        for (int p = 0; p < 7; ++p)
          {
            if (KIND == 0 && p >= 3 && p < 6)
              continue;
            const T *M = diag_mat(ds, p == 6 ? 0 : pair_kind(1, pd[p], pe[p]));
            T        x[N], y[N];
            load_line<N, T, 1>(PB + p * N3, a, b, x);
            mat_apply_t<N>(M, x, y);
            store_line<N, T, 1>(PB + p * N3, a, b, y);
          }
        __syncthreads();
        // step 3: z-lines (x=a, y=b) and accumulate
        T res[N];
#pragma unroll
        for (int k = 0; k < N; ++k)
          res[k] = T(0);
#pragma unroll
        for (int p = 0; p < 7; ++p)
          {
            if (KIND == 0 && p >= 3 && p < 6)
              continue;
            const T *M = diag_mat(ds, p == 6 ? 0 : pair_kind(2, pd[p], pe[p]));
            T        x[N];
            load_line<N, T, 2>(PB + p * N3, a, b, x);
            mat_apply_t_add<N>(M, x, res);
          }
        if (active)
#pragma unroll
          for (int k = 0; k < N; ++k)
            {
              const int ix = cx * g.p + a, iy = cy * g.p + b, iz = cz * g.p + k;
              if ((node_mask_g(g, ix, iy, iz) >> c) & 1u)
                continue;
              atomicAdd(diag + size_t(c) * g.n_nodes + node_index(g, cx, cy, cz, a, b, k), res[k]);
            }
      }
  }

  // ---------------------------------------------------------------------
  // Newton residual, cell part (fast FEEvaluation path of
  // assemble_residual): R = -int tau F^{-T} : Grad v + int rho (b - a) . v
  // FORM: formulation of the material (get_tau, material.h:116-161)
  // ---------------------------------------------------------------------
  template <int N, typename T, int FORM>
  __global__ void __launch_bounds__(cells_per_block<N, 3, T>() * N * N)
  residual_kernel(const __grid_constant__ Shape<N, T> sh,
                  const __grid_constant__ CellGeom<T> g, const NHMat<T> m,
                  T rho, T b0, T b1, T b2, const T *__restrict__ u,
                  const T *__restrict__ acc, T *__restrict__ rhs)
  {
    constexpr int N2  = N * N;
    constexpr int N3  = N * N * N;
    constexpr int CPB = cells_per_block<N, 3, T>();
    constexpr int SPC = smem_per_cell<N, 3, false>() + 3 * N3;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T             *sm     = reinterpret_cast<T *>(smem_raw);
    const int      lc     = threadIdx.x / N2;
    const int      l      = threadIdx.x - lc * N2;
    const int      a      = l % N, b = l / N;
    const unsigned cell   = blockIdx.x * CPB + lc;
    const bool     active = cell < g.n_cells;
    const unsigned cc     = active ? cell : 0u;
    const int      cx = int(cc % unsigned(g.C[0])), cyz = int(cc / unsigned(g.C[0]));
    const int      cy = cyz % g.C[1], cz = cyz / g.C[1];
    T             *cb = sm + lc * SPC;
    T             *T0 = cb + 12 * N3;
    T             *T1 = T0 + N3;
    T             *AV = T1 + N3; // acceleration values [3][N3]
#pragma unroll 1
    for (int c = 0; c < 3; ++c)
      {
        T col[N];
        gather_plain<N>(g, u, c, cx, cy, cz, a, b, active, col);
        T *V = cb + c * 4 * N3;
        evaluate_field<N>(sh, col, V, V + N3, V + 2 * N3, V + 3 * N3, T0, T1, a, b, true);
      }
#pragma unroll 1
    for (int c = 0; c < 3; ++c)
      {
        T col[N], x[N], y[N];
        gather_plain<N>(g, acc, c, cx, cy, cz, a, b, active, col);
        __syncthreads();
        mat_apply<N>(sh.S, col, y);
        store_line<N, T, 2>(T0, a, b, y);
        __syncthreads();
        load_line<N, T, 1>(T0, a, b, x);
        mat_apply<N>(sh.S, x, y);
        store_line<N, T, 1>(T1, a, b, y);
        __syncthreads();
        load_line<N, T, 0>(T1, a, b, x);
        mat_apply<N>(sh.S, x, y);
        store_line<N, T, 0>(AV + c * N3, a, b, y);
      }
    __syncthreads();
    if (active)
      {
        const T bf[3] = {b0, b1, b2};
#pragma unroll 1
        for (int k = 0; k < N; ++k)
          {
            const int q   = a + b * N + k * N2;
            const T   jxw = sh.w[a] * sh.w[b] * sh.w[k] * g.vol;
            T         H[3][3], F[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j < 3; ++j)
                {
                  H[i][j] = cb[i * 4 * N3 + (j + 1) * N3 + q] * g.inv_h[j];
                  F[i][j] = H[i][j] + (i == j ? T(1) : T(0));
                }
            const T Jm1 = jm1_from_grad3(H);
            const T J   = T(1) + Jm1;
            const T lnJ = log1p(Jm1);
            T       Fi[3][3];
            inv3(F, J, Fi);
            T tau[3][3];
            if constexpr (FORM == 1)
              {
                // tau = mu b - (mu - 2 lambda ln J) I (material.h:116-161),
                // evaluated as mu (H + H^T + H H^T) + 2 lambda ln J I so that
                // small strains keep their relative accuracy
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                  for (int j = 0; j < 3; ++j)
                    tau[i][j] = m.mu * (H[i][j] + H[j][i] +
                                        (H[i][0] * H[j][0] + H[i][1] * H[j][1] + H[i][2] * H[j][2])) +
                                (i == j ? T(2.0) * m.lambda * lnJ : T(0));
              }
            else
              {
                const T f = exp(lnJ * T(-1.0 / 3.0));
                T       tr = T(0);
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                  for (int j = 0; j < 3; ++j)
                    {
                      tau[i][j] = T(2.0) * m.c_1 * f * f *
                                  (F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2]);
                    }
                tr           = tau[0][0] + tau[1][1] + tau[2][2];
                // (kappa / 2) (J - 1/J) J = (kappa / 2) (J - 1)(J + 1)
                const T tmp  = (m.kappa / T(2.0)) * Jm1 * (T(2) + Jm1);
#pragma unroll
                for (int d = 0; d < 3; ++d)
                  tau[d][d] += tmp - tr / T(3);
              }
#pragma unroll
            for (int i = 0; i < 3; ++i)
              {
#pragma unroll
                for (int j = 0; j < 3; ++j)
                  cb[i * 4 * N3 + (j + 1) * N3 + q] =
                    -(tau[i][0] * Fi[j][0] + tau[i][1] * Fi[j][1] + tau[i][2] * Fi[j][2]) *
                    (jxw * g.inv_h[j]);
                cb[i * 4 * N3 + q] = (-AV[i * N3 + q] + bf[i]) * rho * jxw;
              }
          }
      }
#pragma unroll 1
    for (int c = 0; c < 3; ++c)
      {
        T *V = cb + c * 4 * N3;
        T  col[N];
        integrate_field<N>(sh, V, V + N3, V + 2 * N3, V + 3 * N3, T0, T1, a, b, true, true, col);
        if (active)
#pragma unroll
          for (int k = 0; k < N; ++k)
            atomicAdd(rhs + size_t(c) * g.n_nodes + node_index(g, cx, cy, cz, a, b, k), col[k]);
      }
  }
  // ---------------------------------------------------------------------
  // Heat right-hand side (LaplaceProblem::assemble_rhs cell part,
  // heat_transfer.h:603-614): rhs += int (u_old + dt f(x)) v, no constraints
  // ---------------------------------------------------------------------
  struct SourceDev
  {
    double constant;
    int    n_gauss;
    double center[8][3];
    double width[8];
    double amp[8];
    double lo[3];
    double h[3];
    double xq[MAX_N];
    int    C[3];
    int    N;
    int    J; // table row length: max_d C[d] N
  };

  // The Gaussians of the source are separable on the level's tensor grid of
  // quadrature points: exp(-|x - c|^2 / (2 w^2)) is the product of one
  // factor per direction, each a function of that direction's point
  // coordinate only.  tab[(3 i + d) J + j] = exp(-(x_j - c_id)^2 / (2 w_i^2))
  // for the j-th quadrature coordinate along d (cell j / N, point j % N), so
  // the right-hand side takes three table reads per Gaussian and point
  // instead of an exponential and a division (the same values to a few
  // units in the last place).
  static __global__ void
  heat_source_table_kernel(const __grid_constant__ SourceDev f, double *__restrict__ tab)
  {
    const int total = f.n_gauss * 3 * f.J;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
      {
        const int j = t % f.J, r = t / f.J, d = r % 3, i = r / 3;
        double    v = 0.0;
        if (j < f.C[d] * f.N)
          {
            const int    c = j / f.N, q = j - c * f.N;
            const double x = f.lo[d] + (c + f.xq[q]) * f.h[d] - f.center[i][d];
            v              = exp(-(x * x) / (2 * f.width[i] * f.width[i]));
          }
        tab[t] = v;
      }
  }

  template <int N>
  __global__ void __launch_bounds__(cells_per_block<N, 1, double>() * N * N)
  heat_rhs_kernel(const __grid_constant__ Shape<N, double> sh,
                  const __grid_constant__ CellGeom<double> g,
                  const __grid_constant__ SourceDev f, double dt,
                  const double *__restrict__ u_old, double *__restrict__ rhs,
                  const double *__restrict__ tab)
  {
    using T           = double;
    constexpr int N2  = N * N;
    constexpr int N3  = N * N * N;
    constexpr int CPB = cells_per_block<N, 1, double>();
    constexpr int SPC = smem_per_cell<N, 1, false>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T             *sm     = reinterpret_cast<T *>(smem_raw);
    const int      lc     = threadIdx.x / N2;
    const int      l      = threadIdx.x - lc * N2;
    const int      a      = l % N, b = l / N;
    const unsigned cell   = blockIdx.x * CPB + lc;
    const bool     active = cell < g.n_cells;
    const unsigned cc     = active ? cell : 0u;
    const int      cx = int(cc % unsigned(g.C[0])), cyz = int(cc / unsigned(g.C[0]));
    const int      cy = cyz % g.C[1], cz = cyz / g.C[1];
    T             *V  = sm + lc * SPC;
    T             *T0 = V + 4 * N3;
    T             *T1 = T0 + N3;
    T              col[N], x[N], y[N];
    gather_plain<N>(g, u_old, 0, cx, cy, cz, a, b, active, col);
    mat_apply<N>(sh.S, col, y);
    store_line<N, T, 2>(T0, a, b, y);
    __syncthreads();
    load_line<N, T, 1>(T0, a, b, x);
    mat_apply<N>(sh.S, x, y);
    store_line<N, T, 1>(T1, a, b, y);
    __syncthreads();
    load_line<N, T, 0>(T1, a, b, x);
    mat_apply<N>(sh.S, x, y);
    // x-line (qy=a, qz=b): add dt f at the quadrature points, times JxW;
    // the Gaussians as products of their per-direction factors
    double fyz[8];
    for (int i = 0; i < f.n_gauss; ++i)
      fyz[i] = f.amp[i] * tab[(3 * i + 1) * f.J + cy * N + a] * tab[(3 * i + 2) * f.J + cz * N + b];
#pragma unroll
    for (int qx = 0; qx < N; ++qx)
      {
        double fv = f.constant;
        for (int i = 0; i < f.n_gauss; ++i)
          fv += fyz[i] * tab[(3 * i) * f.J + cx * N + qx];
        y[qx] = (y[qx] + dt * fv) * (sh.w[qx] * sh.w[a] * sh.w[b] * g.vol);
      }
    store_line<N, T, 0>(V, a, b, y);
    integrate_field<N>(sh, V, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, T0, T1, a, b, true,
                       false, col);
    if (active)
#pragma unroll
      for (int k = 0; k < N; ++k)
        atomicAdd(rhs + node_index(g, cx, cy, cz, a, b, k), col[k]);
  }
} // namespace mfgpu
