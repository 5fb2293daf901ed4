// Sum-factorization cell kernels for sm_103a.
//
// One thread block takes CPB cells; every cell gets N*N threads (N = p+1).
// Thread (a,b) of a cell owns one line of N points in each 1D sweep: x-lines
// at (y=a,z=b), y-lines at (x=a,z=b), z-lines at (x=a,y=b).  A sweep loads its
// line from shared memory (or registers), applies an N x N matrix with the
// matrix entries read from the kernel's constant parameter bank (uniform
// across the warp), and stores the line.  The gather reads z-columns straight
// from global memory into registers (the first sweep runs in registers), and
// the scatter adds z-columns from registers with atomics.
//
// Evaluation uses deal.II's collocation scheme: interpolate the Gauss-Lobatto
// nodal values to the Gauss points with S (3 sweeps), then differentiate on
// the Gauss points with the collocation matrix D (3 sweeps); integration is
// the transpose.  This is what FEEvaluation::evaluate / integrate compute for
// n_q = p+1 (call sites include/solid_mechanics/mf_nh_operator.h:697,1018 and
// include/heat_transfer/heat_transfer.h:241,249).
#pragma once

#include <type_traits>

#include "mf_common.cuh"
#include "mf_df64.cuh"

namespace mfgpu
{
  // quadrature data of operators without a separate load step
  struct NoPre
  {
  };

  template <typename T>
  __device__ __forceinline__ T
  fma_(T a, T b, T c)
  {
    return fma(a, b, c);
  }

  // out[r] = sum_k M[r][k] in[k]
  template <int N, typename T>
  __device__ __forceinline__ void
  mat_apply(const T *__restrict__ M, const T (&in)[N], T (&out)[N])
  {
#pragma unroll
    for (int r = 0; r < N; ++r)
      {
        T s = M[r * N] * in[0];
#pragma unroll
        for (int k = 1; k < N; ++k)
          s = fma_(M[r * N + k], in[k], s);
        out[r] = s;
      }
  }

  // out[k] = sum_r M[r][k] in[r]
  template <int N, typename T>
  __device__ __forceinline__ void
  mat_apply_t(const T *__restrict__ M, const T (&in)[N], T (&out)[N])
  {
#pragma unroll
    for (int k = 0; k < N; ++k)
      {
        T s = M[k] * in[0];
#pragma unroll
        for (int r = 1; r < N; ++r)
          s = fma_(M[r * N + k], in[r], s);
        out[k] = s;
      }
  }

  // out[k] += sum_r M[r][k] in[r]
  template <int N, typename T>
  __device__ __forceinline__ void
  mat_apply_t_add(const T *__restrict__ M, const T (&in)[N], T (&out)[N])
  {
#pragma unroll
    for (int k = 0; k < N; ++k)
      {
        T s = out[k];
#pragma unroll
        for (int r = 0; r < N; ++r)
          s = fma_(M[r * N + k], in[r], s);
        out[k] = s;
      }
  }

  // df64 overloads of the 1D line operations: compensated dot products
  template <int N>
  __device__ __forceinline__ void
  mat_apply(const df64 *__restrict__ M, const df64 (&in)[N], df64 (&out)[N])
  {
#pragma unroll
    for (int r = 0; r < N; ++r)
      {
        DfAcc acc;
        acc.init(M[r * N], in[0]);
#pragma unroll
        for (int k = 1; k < N; ++k)
          acc.add(M[r * N + k], in[k]);
        out[r] = acc.result();
      }
  }

  template <int N>
  __device__ __forceinline__ void
  mat_apply_t(const df64 *__restrict__ M, const df64 (&in)[N], df64 (&out)[N])
  {
#pragma unroll
    for (int k = 0; k < N; ++k)
      {
        DfAcc acc;
        acc.init(M[k], in[0]);
#pragma unroll
        for (int r = 1; r < N; ++r)
          acc.add(M[r * N + k], in[r]);
        out[k] = acc.result();
      }
  }

  template <int N>
  __device__ __forceinline__ void
  mat_apply_t_add(const df64 *__restrict__ M, const df64 (&in)[N], df64 (&out)[N])
  {
#pragma unroll
    for (int k = 0; k < N; ++k)
      {
        DfAcc acc;
        acc.init_add(out[k]);
#pragma unroll
        for (int r = 0; r < N; ++r)
          acc.add(M[r * N + k], in[r]);
        out[k] = acc.result();
      }
  }

  // dot-product accumulator: FMA chain in float/double, compensated
  // (TwoSum-accumulated) in double-float
  template <typename T>
  struct Acc
  {
    T s;
    __device__ __forceinline__ void init(T a, T b) { s = a * b; }
    __device__ __forceinline__ void init_add(T c) { s = c; }
    __device__ __forceinline__ void add(T a, T b) { s = fma_(a, b, s); }
    __device__ __forceinline__ T result() const { return s; }
  };
  template <>
  struct Acc<df64> : DfAcc
  {
  };

  // ---------------------------------------------------------------------
  // Even-odd 1D line operations (the EO form of mf_common.cuh).  For
  // out = M in, with p_k = in[k] + in[N-1-k], m_k = in[k] - in[N-1-k]:
  //   E_r = sum_k e[r][k] p_k (+ e[r][H] in[H]),  O_r = sum_k o[r][k] m_k,
  //   out[r] = E_r + O_r,  out[N-1-r] = SIG (E_r - O_r)
  // (plus the middle row for odd N); for out = M^T in the sign moves into
  // the pre-sums: p_r = in[r] + SIG in[N-1-r], m_r = in[r] - SIG in[N-1-r],
  //   out[k] = E_k + O_k,  out[N-1-k] = E_k - O_k.
  // N = 5 takes 13 products instead of 25, N = 7 25 instead of 49 (deal.II's
  // FEEvaluation kernels use the same split for symmetric bases).
  // ---------------------------------------------------------------------
  template <typename T>
  __device__ __forceinline__ T
  eo_plus(T a, T b)
  {
    return a + b;
  }
  template <typename T>
  __device__ __forceinline__ T
  eo_minus(T a, T b)
  {
    return a - b;
  }
  // df64 pre-sums: one TwoSum of the high parts, the low parts added in
  // float (absolute error ~2^-48 (|a| + |b|), as the dot products that use
  // them)
  __device__ __forceinline__ df64
  eo_plus(df64 a, df64 b)
  {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    quick_two_sum(s, e, s, e);
    return {s, e};
  }
  __device__ __forceinline__ df64
  eo_minus(df64 a, df64 b)
  {
    return eo_plus(a, df64{-b.hi, -b.lo});
  }

  // sum = E + O, diff = E - O
  template <typename T>
  __device__ __forceinline__ void
  acc_pair(const Acc<T> &E, const Acc<T> &O, T &sum, T &diff)
  {
    sum  = E.s + O.s;
    diff = E.s - O.s;
  }
  // sum += E + O, diff += E - O
  template <typename T>
  __device__ __forceinline__ void
  acc_pair_add(const Acc<T> &E, const Acc<T> &O, T &sum, T &diff)
  {
    sum  = sum + (E.s + O.s);
    diff = diff + (E.s - O.s);
  }
  __device__ __forceinline__ void
  acc_pair(const Acc<df64> &E, const Acc<df64> &O, df64 &sum, df64 &diff)
  {
    float q, r;
    two_sum(E.s, O.s, q, r);
    quick_two_sum(q, __fadd_rn(__fadd_rn(E.t, O.t), r), sum.hi, sum.lo);
    two_sum(E.s, -O.s, q, r);
    quick_two_sum(q, __fadd_rn(__fsub_rn(E.t, O.t), r), diff.hi, diff.lo);
  }
  __device__ __forceinline__ void
  acc_pair_add(const Acc<df64> &E, const Acc<df64> &O, df64 &sum, df64 &diff)
  {
    float q, r, q2, r2;
    two_sum(E.s, O.s, q, r);
    two_sum(q, sum.hi, q2, r2);
    quick_two_sum(q2, __fadd_rn(__fadd_rn(__fadd_rn(E.t, O.t), __fadd_rn(r, r2)), sum.lo), sum.hi, sum.lo);
    two_sum(E.s, -O.s, q, r);
    two_sum(q, diff.hi, q2, r2);
    quick_two_sum(q2, __fadd_rn(__fadd_rn(__fsub_rn(E.t, O.t), __fadd_rn(r, r2)), diff.lo), diff.hi, diff.lo);
  }

  // out = M in
  template <int N, typename T, int SIG>
  __device__ __forceinline__ void
  mat_apply(const EO<N, T, SIG> &M, const T (&in)[N], T (&out)[N])
  {
    constexpr int  H = N / 2, HR = (N + 1) / 2;
    constexpr bool ODD = N % 2 == 1;
    T              p[H], m[H];
#pragma unroll
    for (int k = 0; k < H; ++k)
      {
        p[k] = eo_plus(in[k], in[N - 1 - k]);
        m[k] = eo_minus(in[k], in[N - 1 - k]);
      }
#pragma unroll
    for (int r = 0; r < H; ++r)
      {
        Acc<T> E, O;
        E.init(M.e[r * HR], p[0]);
#pragma unroll
        for (int k = 1; k < H; ++k)
          E.add(M.e[r * HR + k], p[k]);
        if constexpr (ODD)
          E.add(M.e[r * HR + H], in[H]);
        O.init(M.o[r * H], m[0]);
#pragma unroll
        for (int k = 1; k < H; ++k)
          O.add(M.o[r * H + k], m[k]);
        if constexpr (SIG > 0)
          acc_pair(E, O, out[r], out[N - 1 - r]);
        else
          acc_pair(O, E, out[r], out[N - 1 - r]);
      }
    if constexpr (ODD)
      {
        Acc<T> C;
        if constexpr (SIG > 0)
          {
            C.init(M.e[H * HR], p[0]);
#pragma unroll
            for (int k = 1; k < H; ++k)
              C.add(M.e[H * HR + k], p[k]);
            C.add(M.e[H * HR + H], in[H]);
          }
        else
          {
            C.init(M.o[H * H], m[0]);
#pragma unroll
            for (int k = 1; k < H; ++k)
              C.add(M.o[H * H + k], m[k]);
          }
        out[H] = C.result();
      }
  }

  // Whether the operator-application sweeps use the even-odd form for N
  // points per direction in arithmetic T.  The split trades products for
  // pre- and post-additions; on GB300 (heat operator, 64^3 cells) it wins
  // for N >= 3 in double-float, N = 3 and N >= 5 in FP64 and N >= 5 in FP32,
  // and loses at N = 2 (and N = 4 in FP64).
  template <int N, typename T>
  __host__ __device__ constexpr bool
  use_even_odd()
  {
    return std::is_same<T, df64>::value ? N >= 3 : (std::is_same<T, double>::value ? (N == 3 || N >= 5) : N >= 5);
  }

  // the interpolation and derivative matrices of the operator-application
  // sweeps, in the form use_even_odd selects
  template <int N, typename T>
  __device__ __forceinline__ const auto &
  sweep_S(const ShapeA<N, T> &sh)
  {
    if constexpr (use_even_odd<N, T>())
      return sh.Se;
    else
      return sh.S;
  }
  template <int N, typename T>
  __device__ __forceinline__ const auto &
  sweep_D(const ShapeA<N, T> &sh, int d)
  {
    if constexpr (use_even_odd<N, T>())
      return sh.De[d];
    else
      return sh.D[d];
  }
  template <int N, typename T>
  __device__ __forceinline__ const auto &
  sweep_Du(const ShapeA<N, T> &sh)
  {
    if constexpr (use_even_odd<N, T>())
      return sh.Due;
    else
      return sh.Du;
  }

  // out = M^T in (ADD: out += M^T in)
  template <bool ADD, int N, typename T, int SIG>
  __device__ __forceinline__ void
  eo_apply_t(const EO<N, T, SIG> &M, const T (&in)[N], T (&out)[N])
  {
    constexpr int  H = N / 2, HR = (N + 1) / 2;
    constexpr bool ODD = N % 2 == 1;
    T              p[H], m[H];
#pragma unroll
    for (int r = 0; r < H; ++r)
      {
        if constexpr (SIG > 0)
          {
            p[r] = eo_plus(in[r], in[N - 1 - r]);
            m[r] = eo_minus(in[r], in[N - 1 - r]);
          }
        else
          {
            p[r] = eo_minus(in[r], in[N - 1 - r]);
            m[r] = eo_plus(in[r], in[N - 1 - r]);
          }
      }
#pragma unroll
    for (int k = 0; k < H; ++k)
      {
        Acc<T> E, O;
        E.init(M.e[k], p[0]);
#pragma unroll
        for (int r = 1; r < H; ++r)
          E.add(M.e[r * HR + k], p[r]);
        O.init(M.o[k], m[0]);
#pragma unroll
        for (int r = 1; r < H; ++r)
          O.add(M.o[r * H + k], m[r]);
        if constexpr (ODD && SIG > 0)
          E.add(M.e[H * HR + k], in[H]);
        if constexpr (ODD && SIG < 0)
          O.add(M.o[H * H + k], in[H]);
        if constexpr (ADD)
          acc_pair_add(E, O, out[k], out[N - 1 - k]);
        else
          acc_pair(E, O, out[k], out[N - 1 - k]);
      }
    if constexpr (ODD)
      {
        Acc<T> C;
        if constexpr (ADD)
          {
            C.init_add(out[H]);
            C.add(M.e[H], p[0]);
          }
        else
          C.init(M.e[H], p[0]);
#pragma unroll
        for (int r = 1; r < H; ++r)
          C.add(M.e[r * HR + H], p[r]);
        if constexpr (SIG > 0)
          C.add(M.e[H * HR + H], in[H]);
        out[H] = C.result();
      }
  }

  template <int N, typename T, int SIG>
  __device__ __forceinline__ void
  mat_apply_t(const EO<N, T, SIG> &M, const T (&in)[N], T (&out)[N])
  {
    eo_apply_t<false>(M, in, out);
  }

  template <int N, typename T, int SIG>
  __device__ __forceinline__ void
  mat_apply_t_add(const EO<N, T, SIG> &M, const T (&in)[N], T (&out)[N])
  {
    eo_apply_t<true>(M, in, out);
  }

  template <typename T>
  __device__ __forceinline__ T
  zero()
  {
    return T(0);
  }
  template <>
  __device__ __forceinline__ df64
  zero<df64>()
  {
    return df64{0.f, 0.f};
  }

  template <typename T>
  __device__ __forceinline__ T
  one()
  {
    return T(1);
  }
  template <>
  __device__ __forceinline__ df64
  one<df64>()
  {
    return df64{1.f, 0.f};
  }

  template <typename T>
  __device__ __forceinline__ T
  ldg_(const T *p)
  {
    return __ldg(p);
  }
  template <>
  __device__ __forceinline__ df64
  ldg_<df64>(const df64 *p)
  {
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return df64{v.x, v.y};
  }

  template <int N>
  __device__ __forceinline__ int
  line_base(int dir, int a, int b)
  {
    return dir == 0 ? (a * N + b * N * N) : (dir == 1 ? (a + b * N * N) : (a + b * N));
  }

  template <int N>
  __host__ __device__ constexpr int
  line_stride(int dir)
  {
    return dir == 0 ? 1 : (dir == 1 ? N : N * N);
  }

  template <int N, typename T, int DIR>
  __device__ __forceinline__ void
  load_line(const T *buf, int a, int b, T (&x)[N])
  {
    const int base = line_base<N>(DIR, a, b);
#pragma unroll
    for (int i = 0; i < N; ++i)
      x[i] = buf[base + i * line_stride<N>(DIR)];
  }

  template <int N, typename T, int DIR>
  __device__ __forceinline__ void
  store_line(T *buf, int a, int b, const T (&x)[N])
  {
    const int base = line_base<N>(DIR, a, b);
#pragma unroll
    for (int i = 0; i < N; ++i)
      buf[base + i * line_stride<N>(DIR)] = x[i];
  }

  // Shared-memory layout of a cell's N^3 arrays: element (x,y,z) at
  // x + SY y + SZ z, arrays of A = SZ N elements.  The natural layout is
  // SY = N, SZ = N^2.
  template <int N, int SY_, int SZ_>
  struct Lay
  {
    static constexpr int SY = SY_, SZ = SZ_, A = SZ_ * N;
    __device__ static __forceinline__ int
    base(int dir, int a, int b)
    {
      return dir == 0 ? (a * SY + b * SZ) : (dir == 1 ? (a + b * SZ) : (a + b * SY));
    }
    __host__ __device__ static constexpr int
    stride(int dir)
    {
      return dir == 0 ? 1 : (dir == 1 ? SY : SZ);
    }
    // quadrature point / node (a, b, k) with a along x, b along y, k along z
    __device__ static __forceinline__ int
    at(int a, int b, int k)
    {
      return a + b * SY + k * SZ;
    }
  };

  // Padded layouts of the operator-application kernel, by N and element
  // size: SY, SZ and the cell padding PAD (for 12 arrays per cell) were
  // chosen by an exhaustive search that counts the shared-memory
  // wavefronts of every warp's line accesses in all three sweep directions
  // (thread (a,b) of cell c on line (a,b), the cells per block of
  // apply_cells_per_block), at most 25 % (4-byte) / 2 % (8-byte) more
  // shared memory.  Wavefronts per block and sweep step, natural -> padded:
  //   4-byte: N=2 192->40, 3 189->135, 4 160->64, 5 115->100, 6 306->234, 7 329->266
  //   8-byte: N=2 192->128, 3 360->324, 4 288 (natural), 5 200->180, 6 390->360, 7 357->343
  template <int N, int ES>
  struct ApplyPad
  {
    static constexpr int SY = N, SZ = N * N, PAD = 0;
  };
#define MF_PAD(n, es, sy, sz, pad)                                                                   \
  template <>                                                                                       \
  struct ApplyPad<n, es>                                                                            \
  {                                                                                                 \
    static constexpr int SY = sy, SZ = sz, PAD = pad;                                               \
  };
  MF_PAD(2, 4, 2, 4, 4)
  MF_PAD(3, 4, 3, 9, 23)
  MF_PAD(4, 4, 4, 19, 0)
  MF_PAD(5, 4, 5, 25, 1)
  MF_PAD(6, 4, 6, 39, 12)
  MF_PAD(7, 4, 7, 56, 17)
  MF_PAD(2, 8, 2, 4, 1)
  MF_PAD(3, 8, 3, 9, 1)
  MF_PAD(5, 8, 5, 25, 1)
  MF_PAD(6, 8, 6, 36, 7)
  MF_PAD(7, 8, 7, 49, 13)
#undef MF_PAD

  template <int N, typename T>
  using ApplyLay = Lay<N, ApplyPad<N, int(sizeof(T))>::SY, ApplyPad<N, int(sizeof(T))>::SZ>;

  // cell stride (elements) of NA arrays in the padded layout: the bank
  // offset between consecutive cells is that of the searched 12-array cell
  template <int N, typename T>
  __host__ __device__ constexpr int
  apply_cell_stride(int na)
  {
    constexpr int P   = sizeof(T) == 4 ? 32 : 16; // elements per bank period
    constexpr int A   = ApplyLay<N, T>::A;
    const int     off = 12 * A + ApplyPad<N, int(sizeof(T))>::PAD - na * A;
    return na * A + ((off % P) + P) % P;
  }

  template <int N, class L, typename T, int DIR>
  __device__ __forceinline__ void
  load_line_l(const T *buf, int a, int b, T (&x)[N])
  {
    const int base = L::base(DIR, a, b);
#pragma unroll
    for (int i = 0; i < N; ++i)
      x[i] = buf[base + i * L::stride(DIR)];
  }

  template <int N, class L, typename T, int DIR>
  __device__ __forceinline__ void
  store_line_l(T *buf, int a, int b, const T (&x)[N])
  {
    const int base = L::base(DIR, a, b);
#pragma unroll
    for (int i = 0; i < N; ++i)
      buf[base + i * L::stride(DIR)] = x[i];
  }

  // Cells per block for a degree / number of components / precision: aim
  // at 100-256 threads and <= ~100 KB of shared memory.
  template <int N, int NC, typename T>
  __host__ __device__ constexpr int
  cells_per_block()
  {
    return N == 2 ? 32 :
           N == 3 ? 16 :
           N == 4 ? 8 :
           N == 5 ? (NC == 1 ? 8 : (sizeof(T) == 8 ? 4 : 8)) :
           N == 6 ? (NC == 1 ? 4 : (sizeof(T) == 8 ? 2 : 4)) :
                    (NC == 1 ? 4 : 2);
  }

  // Cells per block of the operator-application kernels: blocks of
  // CPB*N^2 threads that fill whole warps (or nearly), within the shared
  // memory of one SM.
  template <int N, int NC, typename TS, bool EVAL_U>
  __host__ __device__ constexpr int
  apply_cells_per_block()
  {
    return N == 2 ? 32 :
           N == 3 ? 32 :
           N == 4 ? 8 :
           N == 5 ? 5 :
           N == 6 ? (NC == 1 ? 8 : (EVAL_U ? 4 : (sizeof(TS) == 8 ? 5 : 7))) :
                    (NC == 1 ? 5 : (sizeof(TS) == 8 ? 3 : 5));
  }

  // shared memory per cell of the operator-application kernel (elements of
  // T): NC*(value + 3 gradients); the 1D sweeps use the gradient slots of
  // the component being evaluated or integrated as their scratch.  With
  // EVAL_U, 3*NC gradients of the linearisation + one scratch array.
  template <int N, int NC, bool EVAL_U, typename T>
  __host__ __device__ constexpr int
  apply_smem_per_cell()
  {
    return apply_cell_stride<N, T>(NC * 4 + (EVAL_U ? 3 * NC + 1 : 0));
  }

  // shared memory per cell (in elements of T): NC*(value + 3 gradients)
  // + 2 scratch arrays + (optional) 3*NC gradients of the linearisation
  template <int N, int NC, bool EVAL_U>
  __host__ __device__ constexpr int
  smem_per_cell()
  {
    return (NC * 4 + 2 + (EVAL_U ? 3 * NC : 0)) * N * N * N;
  }

  // ---------------------------------------------------------------------
  // Evaluate values and reference gradients (at the Gauss points) of one
  // scalar field whose z-columns are in registers.  Writes V, G0, G1, G2.
  // Requires a __syncthreads() before V/G are read by other threads.
  // ---------------------------------------------------------------------
  template <int N, typename T, class L = Lay<N, N, N * N>, class MS, class MD>
  __device__ __forceinline__ void
  evaluate_field(const MS &S, const MD &D0, const MD &D1, const MD &D2,
                 const T (&col)[N], T *V, T *G0, T *G1, T *G2, T *T0, T *T1,
                 int a, int b, bool want_values)
  {
    T x[N], y[N];
    // z interpolation in registers, store z-line (x=a, y=b)
    mat_apply<N>(S, col, y);
    store_line_l<N, L, T, 2>(T0, a, b, y);
    __syncthreads();
    // y interpolation: line (x=a, z=b)
    load_line_l<N, L, T, 1>(T0, a, b, x);
    mat_apply<N>(S, x, y);
    store_line_l<N, L, T, 1>(T1, a, b, y);
    __syncthreads();
    // x interpolation: line (y=a, z=b) -> values; x-derivative from registers
    load_line_l<N, L, T, 0>(T1, a, b, x);
    mat_apply<N>(S, x, y);
    store_line_l<N, L, T, 0>(V, a, b, y); // values (also needed for the y/z derivatives)
    (void)want_values;
    mat_apply<N>(D0, y, x);
    store_line_l<N, L, T, 0>(G0, a, b, x);
    __syncthreads();
    // y and z derivatives of the values
    load_line_l<N, L, T, 1>(V, a, b, x);
    mat_apply<N>(D1, x, y);
    store_line_l<N, L, T, 1>(G1, a, b, y);
    load_line_l<N, L, T, 2>(V, a, b, x);
    mat_apply<N>(D2, x, y);
    store_line_l<N, L, T, 2>(G2, a, b, y);
  }

  template <int N, typename T>
  __device__ __forceinline__ void
  evaluate_field(const Shape<N, T> &sh, const T (&col)[N], T *V, T *G0, T *G1,
                 T *G2, T *T0, T *T1, int a, int b, bool want_values)
  {
    evaluate_field<N>(sh.S, sh.D, sh.D, sh.D, col, V, G0, G1, G2, T0, T1, a, b,
                      want_values);
  }

  // ---------------------------------------------------------------------
  // Integrate: nodal result = S^T (V + D^T G) in 3D, returned as the
  // z-column (x=a, y=b) in registers.  V is overwritten.  Starts with a
  // __syncthreads() so that the submitted values of all threads are visible.
  // ---------------------------------------------------------------------
  template <int N, typename T, class L = Lay<N, N, N * N>, class MS, class MD>
  __device__ __forceinline__ void
  integrate_field(const MS &S, const MD &D0, const MD &D1, const MD &D2, T *V,
                  const T *G0, const T *G1, const T *G2, T *T0, T *T1, int a,
                  int b, bool has_values, bool has_gradients, T (&col)[N])
  {
    T x[N], y[N];
    __syncthreads();
    if (has_gradients)
      {
        // z: V += D^T G2 on z-line (x=a,y=b)
        load_line_l<N, L, T, 2>(G2, a, b, x);
        if (has_values)
          load_line_l<N, L, T, 2>(V, a, b, y);
        else
#pragma unroll
          for (int i = 0; i < N; ++i)
            y[i] = zero<T>();
        mat_apply_t_add<N>(D2, x, y);
        store_line_l<N, L, T, 2>(V, a, b, y);
        __syncthreads();
        // y: V += D^T G1 on y-line (x=a,z=b)
        load_line_l<N, L, T, 1>(G1, a, b, x);
        load_line_l<N, L, T, 1>(V, a, b, y);
        mat_apply_t_add<N>(D1, x, y);
        store_line_l<N, L, T, 1>(V, a, b, y);
        __syncthreads();
        // x: t = V + D^T G0 on x-line (y=a,z=b); then S^T
        load_line_l<N, L, T, 0>(G0, a, b, x);
        load_line_l<N, L, T, 0>(V, a, b, y);
        mat_apply_t_add<N>(D0, x, y);
      }
    else
      load_line_l<N, L, T, 0>(V, a, b, y);
    mat_apply_t<N>(S, y, x);
    store_line_l<N, L, T, 0>(T0, a, b, x);
    __syncthreads();
    load_line_l<N, L, T, 1>(T0, a, b, x);
    mat_apply_t<N>(S, x, y);
    store_line_l<N, L, T, 1>(T1, a, b, y);
    __syncthreads();
    load_line_l<N, L, T, 2>(T1, a, b, x);
    mat_apply_t<N>(S, x, col);
  }

  template <int N, typename T>
  __device__ __forceinline__ void
  integrate_field(const Shape<N, T> &sh, T *V, const T *G0, const T *G1,
                  const T *G2, T *T0, T *T1, int a, int b, bool has_values,
                  bool has_gradients, T (&col)[N])
  {
    integrate_field<N>(sh.S, sh.D, sh.D, sh.D, V, G0, G1, G2, T0, T1, a, b,
                       has_values, has_gradients, col);
  }

  // runtime-direction line access (one copy of a sweep's code serves
  // several directions)
  template <int N, typename T>
  __device__ __forceinline__ void
  load_line_rt(const T *buf, int base, int stride, T (&x)[N])
  {
#pragma unroll
    for (int i = 0; i < N; ++i)
      x[i] = buf[base + i * stride];
  }

  template <int N, typename T>
  __device__ __forceinline__ void
  store_line_rt(T *buf, int base, int stride, const T (&x)[N])
  {
#pragma unroll
    for (int i = 0; i < N; ++i)
      buf[base + i * stride] = x[i];
  }

  // ---------------------------------------------------------------------
  // Compact-code evaluate / integrate with ONE derivative matrix D for all
  // three directions (reference-cell gradients): the sweeps that differ
  // only in their direction run as loops over the direction, so the
  // kernel carries 8 instead of 12 inlined copies of a line operation.
  // Scratch: evaluate uses G1, G2; integrate uses G0, G1 (as in
  // evaluate_field / integrate_field).
  // ---------------------------------------------------------------------
  template <int N, class L, typename T, class MS, class MD>
  __device__ __forceinline__ void
  evaluate_field_rg(const MS &S, const MD &D, const T (&col)[N], T *V, int a, int b)
  {
    constexpr int A = L::A;
    T             x[N], y[N];
    // the nodal z-column goes through G0 so that the three interpolation
    // sweeps share one copy of the code: z G0 -> G1, y G1 -> G2, x G2 -> V
    // (the z pass reads only the column this thread wrote)
    store_line_l<N, L, T, 2>(V + A, a, b, col);
#pragma unroll 1
    for (int pass = 0; pass < 3; ++pass)
      {
        const int dir = 2 - pass, base = L::base(dir, a, b), stride = L::stride(dir);
        load_line_rt<N>(V + (pass + 1) * A, base, stride, x);
        mat_apply<N>(S, x, y);
        store_line_rt<N>(pass == 2 ? V : V + (pass + 2) * A, base, stride, y);
        __syncthreads();
      }
    // derivatives G_d = D V along direction d
#pragma unroll 1
    for (int d = 0; d < 3; ++d)
      {
        const int base = L::base(d, a, b), stride = L::stride(d);
        load_line_rt<N>(V, base, stride, x);
        mat_apply<N>(D, x, y);
        store_line_rt<N>(V + (d + 1) * A, base, stride, y);
      }
  }

  template <int N, class L, typename T, class MS, class MD>
  __device__ __forceinline__ void
  integrate_field_rg(const MS &S, const MD &D, T *V, int a, int b, T (&col)[N])
  {
    constexpr int A = L::A;
    T             x[N], y[N];
    __syncthreads();
    // V += D^T G_d along z, y, x
#pragma unroll 1
    for (int d = 2; d >= 0; --d)
      {
        const int base = L::base(d, a, b), stride = L::stride(d);
        load_line_rt<N>(V + (d + 1) * A, base, stride, x);
        load_line_rt<N>(V, base, stride, y);
        mat_apply_t_add<N>(D, x, y);
        store_line_rt<N>(V, base, stride, y);
        __syncthreads();
      }
    // S^T along x (V -> G0) and y (G0 -> G1)
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass)
      {
        const int dir = pass, base = L::base(dir, a, b), stride = L::stride(dir);
        load_line_rt<N>(pass == 0 ? V : V + A, base, stride, x);
        mat_apply_t<N>(S, x, y);
        store_line_rt<N>(V + (pass + 1) * A, base, stride, y);
        __syncthreads();
      }
    // S^T along z into registers
    load_line_l<N, L, T, 2>(V + 2 * A, a, b, x);
    mat_apply_t<N>(S, x, col);
  }

  // node index of local node (a, b, k) of cell (cx,cy,cz)
  template <typename T>
  __device__ __forceinline__ size_t
  node_index(const CellGeom<T> &g, int cx, int cy, int cz, int a, int b, int k)
  {
    return size_t(cx * g.p + a) +
           size_t(g.Nn[0]) * (size_t(cy * g.p + b) + size_t(g.Nn[1]) * size_t(cz * g.p + k));
  }

  template <typename T>
  __device__ __forceinline__ unsigned
  node_mask_g(const CellGeom<T> &g, int ix, int iy, int iz)
  {
    return node_mask(g.face_mask, g.Nn, ix, iy, iz);
  }

  // ---------------------------------------------------------------------
  // Generic operator application kernel:
  //   dst += sum_cells  integrate( QOp( evaluate( gather(src) ) ) )
  // with homogeneous constraints applied on gather/scatter when CONSTRAINED.
  //
  // QOp interface:
  //   static constexpr bool eval_u;        // evaluate gradients of cached u
  //   const T* ucell;                       // cell-local u values if eval_u
  //   __device__ void operator()(unsigned cell, int q, T (&v)[NC],
  //                              T (&H)[NC][3], const T (*Hu)[3]) const;
  //   static constexpr bool ref_grad;      // H are reference-cell gradients
  //                                         // (the op applies the Jacobian)
  //   static constexpr bool prefetch;      // split into load() + apply():
  //   using Pre;                            // the quadrature data of a point
  //   __device__ Pre load(unsigned cell, int q) const;
  //   __device__ void apply(const Pre &, T (&v)[NC], T (&H)[NC][3], T jxw) const;
  //                                         // (returns value and flux times jxw)
  // v and H arrive as the values and REAL gradients at quadrature point q and
  // leave as the submitted value and flux (before JxW).
  // ---------------------------------------------------------------------
  //
  // UNIT: element columns instead of an application.  Block (c, j) applies
  // the operator of cell c to the unit vector of its local DoF j (component
  // j / N^3, node j % N^3) and adds the result to column j's global DoF of
  // the dense row-major matrix dst (NC n_nodes rows and columns); src is
  // not read, constrained rows and columns get nothing (the caller puts 1
  // on their diagonal).
  template <int N, typename TS, typename T, int NC, class QOp, bool CONSTRAINED, bool ONE_CELL = false,
            bool UNIT = false>
  __global__ void __launch_bounds__((ONE_CELL || UNIT ? 1 : apply_cells_per_block<N, NC, TS, QOp::eval_u>()) * N * N)
  cell_apply_kernel(const __grid_constant__ ShapeA<N, T> sh,
                    const __grid_constant__ CellGeom<T> g, const QOp op,
                    const TS *__restrict__ src, TS *__restrict__ dst)
  {
    constexpr int N2  = N * N;
    constexpr int N3  = N * N * N;
    // ONE_CELL: one cell per block, for grids smaller than the GPU (coarse
    // levels), so that their cells spread over as many SMs as possible
    constexpr int CPB = ONE_CELL || UNIT ? 1 : apply_cells_per_block<N, NC, TS, QOp::eval_u>();
    constexpr int SPC = apply_smem_per_cell<N, NC, QOp::eval_u, T>();
    using LA          = ApplyLay<N, T>; // padded shared-memory layout of the cell arrays
    constexpr int AS  = LA::A;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    // problem blockIdx.y of a batch
    src += size_t(blockIdx.y) * g.bstride;
    dst += size_t(blockIdx.y) * g.bstride;

    const int      lc     = threadIdx.x / N2;
    const int      l      = threadIdx.x - lc * N2;
    const int      a      = l % N;
    const int      b      = l / N;
    unsigned cell;
    bool     active;
    int      jc = 0, ja = 0, jb = 0, jk = 0; // UNIT: the local DoF of the unit vector
    if constexpr (UNIT)
      {
        const unsigned j = blockIdx.x % unsigned(NC * N3);
        cell             = g.cell_begin + blockIdx.x / unsigned(NC * N3);
        active           = cell < g.cell_end;
        jc               = int(j) / N3;
        ja               = int(j) % N;
        jb               = (int(j) / N) % N;
        jk               = (int(j) % N3) / N2;
      }
    else if (g.color < 0)
      {
        cell   = g.cell_begin + blockIdx.x * CPB + lc;
        active = cell < g.cell_end;
      }
    else
      {
        // cells (2i+px, 2j+py, 2k+pz) of one parity colour share no node
        const unsigned idx = blockIdx.x * CPB + lc;
        active             = idx < g.color_n;
        const unsigned i   = active ? idx : 0u;
        const unsigned ix  = i % unsigned(g.hc[0]), r = i / unsigned(g.hc[0]);
        const unsigned iy = r % unsigned(g.hc[1]), iz = r / unsigned(g.hc[1]);
        cell = (2 * ix + unsigned(g.color & 1)) +
               unsigned(g.C[0]) * ((2 * iy + unsigned((g.color >> 1) & 1)) +
                                   unsigned(g.C[1]) * (2 * iz + unsigned((g.color >> 2) & 1)));
      }
    T             *cb     = sm + lc * SPC;
    T             *GU     = cb + NC * 4 * AS; // 3*NC arrays if eval_u
    T             *XU     = GU + 3 * NC * AS; // 1 scratch array if eval_u

    const unsigned cc  = active ? cell : 0u;
    const unsigned cyz = g.dC0.div(cc);
    const int      cx  = int(cc - cyz * unsigned(g.C[0]));
    const int      cz  = int(g.dC1.div(cyz));
    const int      cy  = int(cyz) - cz * g.C[1];
    // Dirichlet component masks of the z-column (a, b): the x and y faces
    // once per thread, the z faces per node (node k of the column lies on
    // z- for k = 0 of the first cell layer, on z+ for k = p of the last)
    unsigned mxy = 0u, mz0 = 0u, mz1 = 0u;
    if (CONSTRAINED)
      {
        const int ix = cx * g.p + a, iy = cy * g.p + b;
        mxy = (ix == 0 ? g.face_mask[0] : 0u) | (ix == g.Nn[0] - 1 ? g.face_mask[1] : 0u) |
              (iy == 0 ? g.face_mask[2] : 0u) | (iy == g.Nn[1] - 1 ? g.face_mask[3] : 0u);
        mz0 = cz == 0 ? g.face_mask[4] : 0u;
        mz1 = cz == g.C[2] - 1 ? g.face_mask[5] : 0u;
      }
    auto col_mask = [&](int k) { return mxy | (k == 0 ? mz0 : 0u) | (k == N - 1 ? mz1 : 0u); };
    // node index of the column's node k: colb + k nxy
    const size_t nxy  = size_t(g.Nn[0]) * size_t(g.Nn[1]);
    const size_t colb = size_t(cx * g.p + a) + size_t(g.Nn[0]) * size_t(cy * g.p + b) + nxy * size_t(cz * g.p);

    // -------- gather + evaluate ------------------------------------------
    // z-column (x=a, y=b) of component c in the storage type; the column of
    // the next component is loaded before the current one is evaluated
    auto gather = [&](int c, TS (&raw)[N]) {
#pragma unroll
      for (int k = 0; k < N; ++k)
        {
          TS val = TS(0);
          if (active)
            {
              const size_t node = colb + size_t(k) * nxy;
              bool skip = false;
              if (CONSTRAINED)
                skip = (col_mask(k) >> c) & 1u;
              if constexpr (UNIT)
                val = (!skip && c == jc && a == ja && b == jb && k == jk) ? TS(1) : TS(0);
              else if (!skip)
                val = __ldg(src + size_t(c) * g.n_nodes + node);
            }
          raw[k] = val;
        }
    };
    TS next_col[N];
    gather(0, next_col);
#pragma unroll 1
    for (int c = 0; c < NC; ++c)
      {
        T col[N];
#pragma unroll
        for (int k = 0; k < N; ++k)
          col[k] = to_compute<T, TS>(next_col[k]);
        if (c + 1 < NC)
          gather(c + 1, next_col);
        // sweep scratch: the y and z gradient slots of this component
        T *V = cb + c * 4 * AS;
        // reference gradients: loops over the directions in double-float
        // (instruction-cache bound), unrolled compile-time strides otherwise
        if constexpr (QOp::ref_grad && std::is_same<T, df64>::value)
          evaluate_field_rg<N, LA>(sweep_S(sh), sweep_Du(sh), col, V, a, b);
        else if constexpr (QOp::ref_grad)
          evaluate_field<N, T, LA>(sweep_S(sh), sweep_Du(sh), sweep_Du(sh), sweep_Du(sh), col, V, V + AS,
                                   V + 2 * AS, V + 3 * AS, V + 2 * AS, V + 3 * AS, a, b, true);
        else
          evaluate_field<N, T, LA>(sweep_S(sh), sweep_D(sh, 0), sweep_D(sh, 1), sweep_D(sh, 2), col, V, V + AS,
                                   V + 2 * AS, V + 3 * AS, V + 2 * AS, V + 3 * AS, a, b, true);
      }
    if constexpr (QOp::eval_u)
      {
        // gradients of the cached linearisation values (cell-local layout)
#pragma unroll 1
        for (int c = 0; c < NC; ++c)
          {
            T col[N];
#pragma unroll
            for (int k = 0; k < N; ++k)
              col[k] = active ? op.ucell[(size_t(cc) * NC + c) * N3 + a + b * N + k * N2] : zero<T>();
            // the values go to XU (scratch); GU + c*3*AS holds the gradients
            // and serves as the sweep scratch
            T *Gc = GU + c * 3 * AS;
            __syncthreads();
            evaluate_field<N, T, LA>(sweep_S(sh), sweep_D(sh, 0), sweep_D(sh, 1), sweep_D(sh, 2), col, XU, Gc,
                                     Gc + AS, Gc + 2 * AS, Gc + AS, Gc + 2 * AS, a, b, false);
          }
      }
    __syncthreads();

    // -------- quadrature-point operation ---------------------------------
    if (active)
      {
        const T wab = sh.w[a] * sh.w[b] * g.vol;
        // quadrature data of the next point is loaded before the current
        // point is computed (operators with QOp::prefetch)
        typename QOp::Pre pre{};
        if constexpr (QOp::prefetch)
          pre = op.load(cell, a + b * N);
#pragma unroll 1
        for (int k = 0; k < N; ++k)
          {
            const int q  = a + b * N + k * N2; // global (cache) index
            const int qs = LA::at(a, b, k);     // shared-memory index
            T         v[NC];
            T         H[NC][3];
#pragma unroll
            for (int c = 0; c < NC; ++c)
              {
                const T *V = cb + c * 4 * AS;
                v[c]       = V[qs];
#pragma unroll
                for (int d = 0; d < 3; ++d)
                  H[c][d] = V[(d + 1) * AS + qs];
              }
            T Hu[NC][3];
            if constexpr (QOp::eval_u)
              {
#pragma unroll
                for (int c = 0; c < NC; ++c)
#pragma unroll
                  for (int d = 0; d < 3; ++d)
                    Hu[c][d] = GU[(c * 3 + d) * AS + qs];
              }
            const T jxw = wab * sh.w[k];
            if constexpr (QOp::prefetch)
              {
                const typename QOp::Pre cur = pre;
                if (k + 1 < N)
                  pre = op.load(cell, q + N2);
                op.apply(cur, v, H, jxw); // returns the JxW-scaled value and flux
#pragma unroll
                for (int c = 0; c < NC; ++c)
                  {
                    T *V  = cb + c * 4 * AS;
                    V[qs] = v[c];
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                      V[(d + 1) * AS + qs] = H[c][d];
                  }
              }
            else
              {
                op(cell, q, v, H, Hu);
#pragma unroll
                for (int c = 0; c < NC; ++c)
                  {
                    T *V  = cb + c * 4 * AS;
                    V[qs] = v[c] * jxw;
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                      V[(d + 1) * AS + qs] = H[c][d] * jxw;
                  }
              }
          }
      }

    // -------- integrate + scatter ----------------------------------------
#pragma unroll 1
    for (int c = 0; c < NC; ++c)
      {
        T *V = cb + c * 4 * AS;
        T  col[N];
        // sweep scratch: the x and y gradient slots (consumed by then)
        if constexpr (QOp::ref_grad && std::is_same<T, df64>::value)
          integrate_field_rg<N, LA>(sweep_S(sh), sweep_Du(sh), V, a, b, col);
        else if constexpr (QOp::ref_grad)
          integrate_field<N, T, LA>(sweep_S(sh), sweep_Du(sh), sweep_Du(sh), sweep_Du(sh), V, V + AS,
                                    V + 2 * AS, V + 3 * AS, V + AS, V + 2 * AS, a, b, true, true, col);
        else
          integrate_field<N, T, LA>(sweep_S(sh), sweep_D(sh, 0), sweep_D(sh, 1), sweep_D(sh, 2), V, V + AS,
                                    V + 2 * AS, V + 3 * AS, V + AS, V + 2 * AS, a, b, true, true, col);
        if (active)
          {
#pragma unroll
            for (int k = 0; k < N; ++k)
              {
                const size_t node = colb + size_t(k) * nxy;
                if constexpr (UNIT)
                  {
                    if (CONSTRAINED && ((col_mask(k) >> c) & 1u))
                      continue;
                    const size_t gcol = size_t(jc) * g.n_nodes + size_t(cx * g.p + ja) +
                                        size_t(g.Nn[0]) * (size_t(cy * g.p + jb) +
                                                           size_t(g.Nn[1]) * size_t(cz * g.p + jk));
                    const size_t ld = g.unit_ld ? g.unit_ld : size_t(NC) * g.n_nodes;
                    atomicAdd(dst + (size_t(c) * g.n_nodes + node) * ld + gcol, to_storage<TS, T>(col[k]));
                    continue;
                  }
                if (CONSTRAINED && ((col_mask(k) >> c) & 1u))
                  {
                    // constrained row: dst += src, written by the one cell
                    // that owns the node (local index < p in every
                    // direction, or the last cell along it); no other cell
                    // touches this row
                    const bool owner = (a < g.p || cx == g.C[0] - 1) && (b < g.p || cy == g.C[1] - 1) &&
                                       (k < g.p || cz == g.C[2] - 1);
                    if (owner)
                      dst[size_t(c) * g.n_nodes + node] += __ldg(src + size_t(c) * g.n_nodes + node);
                    continue;
                  }
                TS *d = dst + size_t(c) * g.n_nodes + node;
                if (g.color < 0)
                  atomicAdd(d, to_storage<TS, T>(col[k]));
                else
                  *d += to_storage<TS, T>(col[k]); // no other cell of this launch owns the node
              }
          }
      }
  }

  // ---------------------------------------------------------------------
  // Point-parallel application for launches with few cells (coarse
  // levels): one block per cell, one thread per point (N^3 threads).  In a
  // 1D sweep every thread computes one output, an N-term dot product along
  // the sweep direction; the three derivative contractions of evaluate
  // (and of integrate) are one pass.  The dependency chains are N times
  // shorter than cell_apply_kernel's (one line of N outputs per thread),
  // which is what a grid of a few hundred blocks is bound by.
  // ---------------------------------------------------------------------
  // out(t) = sum_i M[q][i] in(t with its DIR coordinate q replaced by i)
  // (TR: sum_i M[i][q] in(...)); M in shared memory
  template <int N, int DIR, bool TR, typename T>
  __device__ __forceinline__ T
  point_sweep(const T *M, const T *in, int t, int q)
  {
    constexpr int st   = DIR == 0 ? 1 : (DIR == 1 ? N : N * N);
    const int     base = t - q * st;
    Acc<T>        s;
    s.init(TR ? M[q] : M[q * N], in[base]);
#pragma unroll
    for (int i = 1; i < N; ++i)
      s.add(TR ? M[i * N + q] : M[q * N + i], in[base + i * st]);
    return s.result();
  }

  template <int N, int NC, bool EVAL_U>
  __host__ __device__ constexpr int
  point_smem_elems()
  {
    return 4 * N * N + (2 + 4 * NC + (EVAL_U ? 3 * NC + 1 : 0)) * N * N * N;
  }

  template <int N, typename TS, typename T, int NC, class QOp, bool CONSTRAINED>
  __global__ void __launch_bounds__(N *N *N)
  cell_apply_point_kernel(const __grid_constant__ ShapeA<N, T> sh, const __grid_constant__ CellGeom<T> g,
                          const QOp op, const TS *__restrict__ src, TS *__restrict__ dst)
  {
    constexpr int N2 = N * N, N3 = N * N * N;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *Sm = reinterpret_cast<T *>(smem_raw); // S, then the derivative matrix of x, y, z
    T *Dm = Sm + N2;
    T *U0 = Sm + 4 * N2, *U1 = U0 + N3;
    T *VG = U1 + N3; // [c][value, grad x, grad y, grad z][N3]
    T *GU = VG + 4 * NC * N3; // [c][3][N3] gradients of the linearisation (EVAL_U)
    T *XU = GU + 3 * NC * N3; // scratch values of the linearisation (EVAL_U)

    src += size_t(blockIdx.y) * g.bstride; // problem blockIdx.y of a batch
    dst += size_t(blockIdx.y) * g.bstride;
    const int      t    = threadIdx.x;
    const int      a    = t % N, b = (t / N) % N, k = t / N2;
    const unsigned cell = g.cell_begin + blockIdx.x;
    const unsigned cyz  = g.dC0.div(cell);
    const int      cx   = int(cell - cyz * unsigned(g.C[0]));
    const int      cz   = int(g.dC1.div(cyz));
    const int      cy   = int(cyz) - cz * g.C[1];
    const int      ix = cx * g.p + a, iy = cy * g.p + b, iz = cz * g.p + k;
    const size_t   node = size_t(ix) + size_t(g.Nn[0]) * (size_t(iy) + size_t(g.Nn[1]) * size_t(iz));
    const unsigned mask = CONSTRAINED ? node_mask_g(g, ix, iy, iz) : 0u;
    for (int i = t; i < N2; i += N3)
      {
        Sm[i] = sh.S[i];
#pragma unroll
        for (int d = 0; d < 3; ++d)
          Dm[d * N2 + i] = QOp::ref_grad ? sh.Du[i] : sh.D[d][i];
      }

    // values (V) and gradients (G + d N3) at the Gauss points of the nodal
    // field in U0; U0 is free again when it returns (its last reader, the
    // z sweep, is behind a barrier)
    auto evaluate = [&](T *V, T *G) {
      __syncthreads();
      U1[t] = point_sweep<N, 0, false>(Sm, U0, t, a);
      __syncthreads();
      U0[t] = point_sweep<N, 1, false>(Sm, U1, t, b);
      __syncthreads();
      V[t] = point_sweep<N, 2, false>(Sm, U0, t, k);
      __syncthreads();
      G[t]          = point_sweep<N, 0, false>(Dm, V, t, a);
      G[N3 + t]     = point_sweep<N, 1, false>(Dm + N2, V, t, b);
      G[2 * N3 + t] = point_sweep<N, 2, false>(Dm + 2 * N2, V, t, k);
    };
#pragma unroll 1
    for (int c = 0; c < NC; ++c)
      {
        TS raw = TS(0);
        if (!((mask >> c) & 1u))
          raw = __ldg(src + size_t(c) * g.n_nodes + node);
        U0[t] = to_compute<T, TS>(raw);
        evaluate(VG + c * 4 * N3, VG + c * 4 * N3 + N3);
      }
    if constexpr (QOp::eval_u)
      {
        // gradients of the cached linearisation values (cell-local layout);
        // the values go to the scratch XU
#pragma unroll 1
        for (int c = 0; c < NC; ++c)
          {
            U0[t] = op.ucell[(size_t(cell) * NC + c) * N3 + t];
            evaluate(XU, GU + c * 3 * N3);
          }
      }
    __syncthreads();

    // -------- quadrature-point operation (point t) ------------------------
    {
      T v[NC], H[NC][3];
#pragma unroll
      for (int c = 0; c < NC; ++c)
        {
          v[c] = VG[c * 4 * N3 + t];
#pragma unroll
          for (int d = 0; d < 3; ++d)
            H[c][d] = VG[(c * 4 + d + 1) * N3 + t];
        }
      const T jxw = (sh.w[a] * sh.w[b] * g.vol) * sh.w[k];
      if constexpr (QOp::prefetch)
        {
          const typename QOp::Pre pre = op.load(cell, t);
          op.apply(pre, v, H, jxw);
        }
      else
        {
          T Hu[NC][3];
          if constexpr (QOp::eval_u)
            {
#pragma unroll
              for (int c = 0; c < NC; ++c)
#pragma unroll
                for (int d = 0; d < 3; ++d)
                  Hu[c][d] = GU[(c * 3 + d) * N3 + t];
            }
          op(cell, t, v, H, Hu);
#pragma unroll
          for (int c = 0; c < NC; ++c)
            {
              v[c] = v[c] * jxw;
#pragma unroll
              for (int d = 0; d < 3; ++d)
                H[c][d] = H[c][d] * jxw;
            }
        }
#pragma unroll
      for (int c = 0; c < NC; ++c)
        {
          VG[c * 4 * N3 + t] = v[c];
#pragma unroll
          for (int d = 0; d < 3; ++d)
            VG[(c * 4 + d + 1) * N3 + t] = H[c][d];
        }
    }

    // -------- integrate + scatter ------------------------------------------
#pragma unroll 1
    for (int c = 0; c < NC; ++c)
      {
        const T *V = VG + c * 4 * N3;
        __syncthreads();
        // value + D^T (x, y, z gradients) in one pass
        {
          Acc<T> s;
          s.init_add(V[t]);
          const int b0 = t - a, b1 = t - b * N, b2 = t - k * N2;
#pragma unroll
          for (int i = 0; i < N; ++i)
            s.add(Dm[i * N + a], V[N3 + b0 + i]);
#pragma unroll
          for (int i = 0; i < N; ++i)
            s.add(Dm[N2 + i * N + b], V[2 * N3 + b1 + i * N]);
#pragma unroll
          for (int i = 0; i < N; ++i)
            s.add(Dm[2 * N2 + i * N + k], V[3 * N3 + b2 + i * N2]);
          U0[t] = s.result();
        }
        __syncthreads();
        U1[t] = point_sweep<N, 0, true>(Sm, U0, t, a);
        __syncthreads();
        U0[t] = point_sweep<N, 1, true>(Sm, U1, t, b);
        __syncthreads();
        const T out = point_sweep<N, 2, true>(Sm, U0, t, k);
        if ((mask >> c) & 1u)
          {
            // constrained row: dst += src by the cell that owns the node
            const bool owner = (a < g.p || cx == g.C[0] - 1) && (b < g.p || cy == g.C[1] - 1) &&
                               (k < g.p || cz == g.C[2] - 1);
            if (owner)
              dst[size_t(c) * g.n_nodes + node] += __ldg(src + size_t(c) * g.n_nodes + node);
          }
        else
          atomicAdd(dst + size_t(c) * g.n_nodes + node, to_storage<TS, T>(out));
      }
  }

  // ---------------------------------------------------------------------
  // quadrature-point operations
  // ---------------------------------------------------------------------

  // heat: mass + dt*k*Laplace (heat_transfer.h:242-248)
  template <typename T>
  struct HeatQOp
  {
    static constexpr bool eval_u   = false;
    static constexpr bool prefetch = false;
    static constexpr bool ref_grad = true; // H are reference-cell gradients
    using Pre                      = NoPre;
    const T              *ucell    = nullptr;
    T                     kd[3]; // k dt / h_d^2: the Jacobian of both gradients
    __device__ __forceinline__ void
    operator()(unsigned, int, T (&)[1], T (&H)[1][3], const T (*)[3]) const
    {
      H[0][0] *= kd[0];
      H[0][1] *= kd[1];
      H[0][2] *= kd[2];
    }
  };

  // neo-Hookean material constants (material.h:78-94)
  template <typename T>
  struct NHMat
  {
    T mu, lambda, rho_alpha, kappa, c_1, two_lambda;
  };

  // scalar_referential (mf_nh_operator.h:848-943): F from the gradient of the
  // cached cell-local displacement, c = mu - 2 lambda ln J cached per qp.
  template <typename T>
  struct NHScalarRefQOp
  {
    static constexpr bool eval_u   = true;
    static constexpr bool prefetch = false;
    static constexpr bool ref_grad = false;
    using Pre                      = NoPre;
    const T              *ucell;  // [cell][3][N^3]
    const T              *scalar; // [cell][N^3]
    NHMat<T>              m;
    int                   n3;
    __device__ __forceinline__ void
    operator()(unsigned cell, int q, T (&v)[3], T (&H)[3][3],
               const T (*Hu)[3]) const
    {
      T F[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          F[i][j] = Hu[i][j] + (i == j ? T(1) : T(0));
      const T c = scalar[size_t(cell) * n3 + q];
      // tau = mu F F^T - c I
      T tau[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          {
            T s = F[i][0] * F[j][0];
            s   = fma_(F[i][1], F[j][1], s);
            s   = fma_(F[i][2], F[j][2], s);
            tau[i][j] = m.mu * s - (i == j ? c : T(0));
          }
      // F^{-1}
      const T c00 = F[1][1] * F[2][2] - F[1][2] * F[2][1];
      const T c01 = F[1][2] * F[2][0] - F[1][0] * F[2][2];
      const T c02 = F[1][0] * F[2][1] - F[1][1] * F[2][0];
      const T det = F[0][0] * c00 + F[0][1] * c01 + F[0][2] * c02;
      const T id  = T(1) / det;
      T       Fi[3][3];
      Fi[0][0] = c00 * id;
      Fi[1][0] = c01 * id;
      Fi[2][0] = c02 * id;
      Fi[0][1] = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) * id;
      Fi[1][1] = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) * id;
      Fi[2][1] = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) * id;
      Fi[0][2] = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) * id;
      Fi[1][2] = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) * id;
      Fi[2][2] = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) * id;
      // g = H F^{-1}
      T gg[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          {
            T s = H[i][0] * Fi[0][j];
            s   = fma_(H[i][1], Fi[1][j], s);
            s   = fma_(H[i][2], Fi[2][j], s);
            gg[i][j] = s;
          }
      const T tr = gg[0][0] + gg[1][1] + gg[2][2];
      T       qd[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          {
            T s = gg[i][0] * tau[0][j];
            s   = fma_(gg[i][1], tau[1][j], s);
            s   = fma_(gg[i][2], tau[2][j], s);
            qd[i][j] = c * (gg[i][j] + gg[j][i]) + (i == j ? T(2) * m.lambda * tr : T(0)) + s;
          }
      // P = qd F^{-T}
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          {
            T s = qd[i][0] * Fi[j][0];
            s   = fma_(qd[i][1], Fi[j][1], s);
            s   = fma_(qd[i][2], Fi[j][2], s);
            H[i][j] = s;
          }
#pragma unroll
      for (int c2 = 0; c2 < 3; ++c2)
        v[c2] *= m.rho_alpha;
    }
  };

  // Referential tangent from 10 cached values per qp: M = F^{-T} (9) and
  // c = mu - 2 lambda ln J.  The scalar_referential flux
  //   [2c sym(g) + 2 lambda tr(g) I + g tau] F^{-T},  g = H F^{-1},
  //   tau = mu F F^T - c I
  // equals  mu H + c M H^T M + 2 lambda (M:H) M  identically, which needs no
  // gradient of the linearisation during the vmult.
  template <typename T>
  struct NHQp10QOp
  {
    static constexpr bool eval_u   = false;
    static constexpr bool prefetch = true;
    static constexpr bool ref_grad = true; // H are reference-cell gradients
    const T              *ucell    = nullptr;
    const T              *cache; // [cell][10][N^3]: M~ = F^{-T} diag(1/h), c
    NHMat<T>              m;
    T                     mu_d[3]; // mu / h_d^2
    int                   n3;
    struct Pre
    {
      T M[3][3];
      T c;
    };
    __device__ __forceinline__ Pre
    load(unsigned cell, int q) const
    {
      const T *cp = cache + size_t(cell) * 10 * n3 + q;
      Pre      p;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          p.M[i][j] = ldg_(cp + (i * 3 + j) * n3);
      p.c = ldg_(cp + 9 * n3);
      return p;
    }
    // With the reference gradient G (H = G J^{-1}, J^{-1} = diag(1/h)) and
    // M~ = M J^{-1}, the flux against reference test gradients is
    //   P J^{-T} = mu H J^{-T} + c (M H^T M) J^{-T} + 2 lambda (M:H) M J^{-T}
    //            = mu_d G + c (M~ G^T) M~ + 2 lambda (M~:G) M~,   mu_d = mu/h_d^2
    // (column d).  Times jxw, every entry one dot product; the value gets
    // rho alpha_1 jxw.
    __device__ __forceinline__ void
    apply(const Pre &p, T (&v)[3], T (&H)[3][3], T jxw) const
    {
      const auto &M = p.M;
      const T     cj = p.c * jxw;
      Acc<T>      at;
      at.init(M[0][0], H[0][0]);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          if (i + j > 0)
            at.add(M[i][j], H[i][j]);
      const T tlj = (m.two_lambda * jxw) * at.result();
      T       muj[3];
#pragma unroll
      for (int d = 0; d < 3; ++d)
        muj[d] = mu_d[d] * jxw;
      // cK = c jxw M H^T  (K_ik = sum_j M_ij H_kj)
      T cK[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k)
          {
            Acc<T> ak;
            ak.init(M[i][0], H[k][0]);
            ak.add(M[i][1], H[k][1]);
            ak.add(M[i][2], H[k][2]);
            cK[i][k] = cj * ak.result();
          }
      T P[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          {
            Acc<T> ap;
            ap.init(muj[j], H[i][j]);
            ap.add(cK[i][0], M[0][j]);
            ap.add(cK[i][1], M[1][j]);
            ap.add(cK[i][2], M[2][j]);
            ap.add(tlj, M[i][j]);
            P[i][j] = ap.result();
          }
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          H[i][j] = P[i][j];
      const T raj = m.rho_alpha * jxw;
#pragma unroll
      for (int c2 = 0; c2 < 3; ++c2)
        v[c2] = v[c2] * raj;
    }
    // unscaled form (value and flux before JxW)
    __device__ __forceinline__ void
    operator()(unsigned cell, int q, T (&v)[3], T (&H)[3][3],
               const T (*)[3]) const
    {
      apply(load(cell, q), v, H, one<T>());
    }
  };

  // Deformed-frame variants (mf_nh_operator.h:945-994, 701-840) and the
  // referential dP/dF variant (996-1010).  Eulerian geometry per qp: F^{-1}
  // (9) and det F (1) = the inverse Jacobian and JxW ratio of
  // MappingQEulerian; the current-frame flux Pc integrates as det F Pc F^{-T}.
  // cache layout [cell][field][N^3]:
  //   tensor2:    0-8 Finv, 9 J, 10 c2=2c/J, 11 s2=1/J, 12-17 tau/J (xx,yy,zz,xy,xz,yz)
  //   tensor4:    0-8 Finv, 9 J, 10 s2, 11-16 tau/J, 17-52 C4 (6x6, Voigt with
  //               sym(g) off-diagonals entered once: C4 : sym(g))
  //   tensor4_ns: 0-80 A_ijkl
  //   form0:      0-8 Finv, 9 J, 10-18 F, 19 J^{-1/3}
  __device__ __forceinline__ int
  voigt(int i, int j)
  {
    // xx,yy,zz,xy,xz,yz
    return i == j ? i : (i + j == 1 ? 3 : (i + j == 2 ? 4 : 5));
  }

  // Formulation-0 current-frame flux (mf_nh_operator.h:707-839)
  template <typename T>
  __device__ __forceinline__ void
  form0_flux_dev(const NHMat<T> &m, const T (&F)[3][3], T js, const T (&gg)[3][3],
                 T (&Pc)[3][3])
  {
    T Fb[3][3], bb[3][3], sg[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        Fb[i][j] = F[i][j] * js;
    const T J = F[0][0] * (F[1][1] * F[2][2] - F[1][2] * F[2][1]) -
                F[0][1] * (F[1][0] * F[2][2] - F[1][2] * F[2][0]) +
                F[0][2] * (F[1][0] * F[2][1] - F[1][1] * F[2][0]);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        {
          bb[i][j] = Fb[i][0] * Fb[j][0] + Fb[i][1] * Fb[j][1] + Fb[i][2] * Fb[j][2];
          sg[i][j] = T(0.5) * (gg[i][j] + gg[j][i]);
        }
    const T inv_dim = T(1.0 / 3.0), two_over_dim = T(2.0 / 3.0);
    T       tau_bar[3][3];
    T       tr_tb = T(0);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        tau_bar[i][j] = bb[i][j] * (T(2.0) * m.c_1);
    tr_tb               = tau_bar[0][0] + tau_bar[1][1] + tau_bar[2][2];
    const T tr_tb_dim   = tr_tb * inv_dim;
    const T dPsi        = (m.kappa / T(2.0)) * (J - T(1.0) / J);
    const T dPsi_J      = dPsi * J;
    const T d2Psi       = (m.kappa / T(2.0)) * (T(1.0) + T(1.0) / (J * J));
    const T tr          = sg[0][0] + sg[1][1] + sg[2][2];
    T       tau_iso_src = T(0);
    T       jc[3][3], tau[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        {
          const T dev     = sg[i][j] - (i == j ? tr * inv_dim : T(0));
          const T tau_iso = tau_bar[i][j] - (i == j ? tr_tb_dim : T(0));
          tau[i][j]       = tau_bar[i][j] + (i == j ? dPsi_J - tr_tb_dim : T(0));
          jc[i][j] = sg[i][j] * (-dPsi_J * T(2.0)) +
                     (i == j ? J * (dPsi + J * d2Psi) * tr : T(0)) +
                     (two_over_dim * tr_tb) * dev - (two_over_dim * tr) * tau_iso;
          tau_iso_src += tau_iso * sg[i][j];
        }
    const T inv_J = T(1.0) / J;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        {
          const T geo = gg[i][0] * tau[0][j] + gg[i][1] * tau[1][j] + gg[i][2] * tau[2][j];
          Pc[i][j] = (jc[i][j] - (i == j ? two_over_dim * tau_iso_src : T(0)) + geo) * inv_J;
        }
  }

  template <typename T, int VAR>
  struct NHCachedQOp
  {
    static constexpr bool eval_u   = false;
    static constexpr bool prefetch = false;
    static constexpr bool ref_grad = false;
    using Pre                      = NoPre;
    const T              *ucell    = nullptr;
    const T              *cache;
    NHMat<T>              m;
    int                   n3;
    __device__ __forceinline__ void
    operator()(unsigned cell, int q, T (&v)[3], T (&H)[3][3],
               const T (*)[3]) const
    {
      constexpr int NF = nh_cache_fields(VAR);
      const T      *cp = cache + size_t(cell) * NF * n3 + q;
      if constexpr (VAR == V_TENSOR4_NS)
        {
          T P[3][3];
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              {
                T s = T(0);
#pragma unroll
                for (int k = 0; k < 3; ++k)
#pragma unroll
                  for (int l = 0; l < 3; ++l)
                    s = fma_(__ldg(cp + (((i * 3 + j) * 3 + k) * 3 + l) * n3), H[k][l], s);
                P[i][j] = s;
              }
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              H[i][j] = P[i][j];
#pragma unroll
          for (int c = 0; c < 3; ++c)
            v[c] *= m.rho_alpha;
          return;
        }
      else
        {
          T Fi[3][3];
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              Fi[i][j] = __ldg(cp + (i * 3 + j) * n3);
          const T J = __ldg(cp + 9 * n3);
          T       gg[3][3];
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              gg[i][j] = H[i][0] * Fi[0][j] + H[i][1] * Fi[1][j] + H[i][2] * Fi[2][j];
          T Pc[3][3];
          T vscale;
          if constexpr (VAR == V_TENSOR2)
            {
              const T c2 = __ldg(cp + 10 * n3);
              const T s2 = __ldg(cp + 11 * n3);
              T       Tt[3][3];
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                  Tt[i][j] = __ldg(cp + (12 + voigt(i, j)) * n3);
              const T tmp = T(2) * m.lambda * s2 * (gg[0][0] + gg[1][1] + gg[2][2]);
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                  Pc[i][j] = c2 * T(0.5) * (gg[i][j] + gg[j][i]) + (i == j ? tmp : T(0)) +
                             gg[i][0] * Tt[0][j] + gg[i][1] * Tt[1][j] + gg[i][2] * Tt[2][j];
              vscale = m.rho_alpha * s2 * J;
            }
          else if constexpr (VAR == V_TENSOR4)
            {
              const T s2 = __ldg(cp + 10 * n3);
              T       Tt[3][3];
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                  Tt[i][j] = __ldg(cp + (11 + voigt(i, j)) * n3);
              T sgv[6];
              sgv[0] = gg[0][0];
              sgv[1] = gg[1][1];
              sgv[2] = gg[2][2];
              sgv[3] = gg[0][1] + gg[1][0];
              sgv[4] = gg[0][2] + gg[2][0];
              sgv[5] = gg[1][2] + gg[2][1];
              T cs[6];
#pragma unroll
              for (int r = 0; r < 6; ++r)
                {
                  T s = T(0);
#pragma unroll
                  for (int k = 0; k < 6; ++k)
                    s = fma_(__ldg(cp + (17 + r * 6 + k) * n3), sgv[k], s);
                  cs[r] = s;
                }
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                  Pc[i][j] = gg[i][0] * Tt[0][j] + gg[i][1] * Tt[1][j] + gg[i][2] * Tt[2][j] +
                             cs[voigt(i, j)];
              vscale = m.rho_alpha * s2 * J;
            }
          else // V_FORM0
            {
              T F[3][3];
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                  F[i][j] = __ldg(cp + (10 + i * 3 + j) * n3);
              const T js = __ldg(cp + 19 * n3);
              form0_flux_dev(m, F, js, gg, Pc);
              vscale = m.rho_alpha;
            }
          // P = J Pc F^{-T}
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              H[i][j] = J * (Pc[i][0] * Fi[j][0] + Pc[i][1] * Fi[j][1] + Pc[i][2] * Fi[j][2]);
#pragma unroll
          for (int c = 0; c < 3; ++c)
            v[c] *= vscale;
        }
    }
  };
} // namespace mfgpu
