// Vector kernels: BLAS-1 updates, deterministic reductions, constrained-row
// handling on the box faces, multigrid transfer passes and the boundary
// traction term.  All are memory-bound streaming kernels: grid-stride loops,
// grid size a multiple of the SM count.
#pragma once

#include "mf_common.cuh"

namespace mfgpu
{
  constexpr int RED_BLOCKS  = 1216; // 8 x 152 SMs: 2048 threads on every SM
  // vectors of at most RED_SHORT entries reduce in one block of
  // RED_SHORT_THREADS threads: no partials, ticket and fences, whose latency
  // chain dominated the reductions of coarse levels (a few thousand entries)
  constexpr int RED_SHORT         = 4096;
  constexpr int RED_SHORT_THREADS = 1024;
  constexpr int RED_THREADS = 256;

  template <typename T>
  __global__ void
  k_fill(size_t n, T v, T *__restrict__ x)
  {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      x[i] = v;
  }

  // y = a*x + b*y
  template <typename T>
  __global__ void
  k_axpby(size_t n, T a, const T *__restrict__ x, T b, T *__restrict__ y)
  {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      y[i] = a * x[i] + b * y[i];
  }

  // z = a*x + b*y
  template <typename T>
  __global__ void
  k_axpbyz(size_t n, T a, const T *__restrict__ x, T b, const T *__restrict__ y,
           T *__restrict__ z)
  {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      z[i] = a * x[i] + b * y[i];
  }

  template <typename T>
  __global__ void
  k_estimate_start(size_t n, size_t period, T mean, T *__restrict__ x)
  {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      x[i] = ((i % period) % 11 == 0 ? T(0) : T(1)) - mean;
  }

  template <typename TD, typename TS>
  __global__ void
  k_convert(size_t n, const TS *__restrict__ s, TD *__restrict__ d)
  {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      d[i] = TD(s[i]);
  }

  // y = d .* x
  template <typename T>
  __global__ void
  k_scale(size_t n, T omega, const T *__restrict__ d, const T *__restrict__ x,
          T *__restrict__ y)
  {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      y[i] = omega * d[i] * x[i];
  }

  template <typename T>
  __global__ void
  k_invert(size_t n, T *__restrict__ x, int *__restrict__ err)
  {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      {
        const T v = x[i];
        if (!(v > T(0)))
          atomicOr(err, 2);
        x[i] = T(1) / v;
      }
  }

  static __device__ __forceinline__ double
  block_sum(double v)
  {
    __shared__ double ws[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
      ws[wid] = v;
    __syncthreads();
    v = 0;
    if (wid == 0)
      {
        const int nw = (blockDim.x + 31) >> 5;
        v            = lane < nw ? ws[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
          v += __shfl_down_sync(0xffffffffu, v, o);
      }
    return v;
  }

  // block sum of values that only lane 0 of each warp holds
  __device__ __forceinline__ double
  block_sum_lane0(double v)
  {
    __shared__ double wl[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
      wl[wid] = v;
    __syncthreads();
    v = 0;
    if (wid == 0)
      {
        const int nw = (blockDim.x + 31) >> 5;
        v            = lane < nw ? wl[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
          v += __shfl_down_sync(0xffffffffu, v, o);
      }
    return v;
  }

  // num / den of two device scalars, divided by one thread per block and
  // shared: an FP64 division is a sequence of FP64 instructions, and on a
  // GPU whose FP64 rate is a small fraction of its FP32 rate, dividing in
  // every thread of a vector kernel took longer than the vector traffic
  // (same quotient in every thread; every thread of the block must call it)
  __device__ __forceinline__ double
  block_ratio(const double *__restrict__ num, const double *__restrict__ den)
  {
    __shared__ double q;
    if (threadIdx.x == 0)
      q = *num / *den;
    __syncthreads();
    return q;
  }

  // Single-launch reduction: every block stores its partial; the block that
  // finishes last (ticket) sums all partials in a fixed order (the same
  // order for the same partials, so the result is deterministic) into *out and
  // resets the ticket.
  __device__ __forceinline__ void
  finish_partials(double s, double *__restrict__ partial, unsigned *ticket,
                  double *__restrict__ out)
  {
    if (gridDim.x == 1)
      {
        // one block (short vectors): its sum is the result
        if (threadIdx.x == 0)
          *out = s;
        return;
      }
    __shared__ bool last;
    if (threadIdx.x == 0)
      {
        partial[blockIdx.x] = s;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
      }
    __syncthreads();
    if (!last)
      return;
    __threadfence();
    double r = 0;
    for (int i = threadIdx.x; i < int(gridDim.x); i += blockDim.x)
      r += __ldcg(partial + i);
    r = block_sum(r);
    if (threadIdx.x == 0)
      {
        *out    = r;
        *ticket = 0u;
      }
  }

  // two reductions of one launch: partial holds 2 gridDim.x values
  __device__ __forceinline__ void
  finish_partials2(double s0, double s1, double *__restrict__ partial, unsigned *ticket,
                   double *__restrict__ out0, double *__restrict__ out1)
  {
    if (gridDim.x == 1)
      {
        if (threadIdx.x == 0)
          {
            *out0 = s0;
            *out1 = s1;
          }
        return;
      }
    __shared__ bool last;
    if (threadIdx.x == 0)
      {
        partial[blockIdx.x]              = s0;
        partial[gridDim.x + blockIdx.x]  = s1;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
      }
    __syncthreads();
    if (!last)
      return;
    __threadfence();
    double r0 = 0, r1 = 0;
    for (int i = threadIdx.x; i < int(gridDim.x); i += blockDim.x)
      {
        r0 += __ldcg(partial + i);
        r1 += __ldcg(partial + gridDim.x + i);
      }
    r0 = block_sum(r0);
    __syncthreads(); // block_sum's shared scratch is reused
    r1 = block_sum(r1);
    if (threadIdx.x == 0)
      {
        *out0   = r0;
        *out1   = r1;
        *ticket = 0u;
      }
  }

  // per-thread sum of products x y: FP64 fused multiply-adds for double
  // vectors; for float vectors a compensated float pair on the FP32 pipe
  // (the product's rounding error from an FMA, the sum's from TwoSum), as
  // accurate as FP64 accumulation for the few terms one thread adds
  template <typename T>
  struct ProdAcc
  {
    double s = 0;
    __device__ __forceinline__ void add(T x, T y) { s = fma(double(x), double(y), s); }
    __device__ __forceinline__ double value() const { return s; }
  };
  template <>
  struct ProdAcc<float>
  {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void
    add(float x, float y)
    {
      const float p = __fmul_rn(x, y);
      const float e = __fmaf_rn(x, y, -p);
      float       s, t;
      two_sum(hi, p, s, t);
      hi = s;
      lo = __fadd_rn(lo, __fadd_rn(t, e));
    }
    __device__ __forceinline__ double value() const { return double(hi) + double(lo); }
  };

  // block sum of the per-thread accumulators.  For float vectors the warp
  // part adds the compensated pairs on the FP32 pipe (TwoSum of the high
  // parts, the low parts and the TwoSum errors added) and one value per
  // warp goes to FP64, instead of FP64 shuffles and adds in every thread.
  template <typename T>
  __device__ __forceinline__ double
  block_sum_acc(const ProdAcc<T> &a)
  {
    return block_sum(a.value());
  }
  template <>
  __device__ __forceinline__ double
  block_sum_acc<float>(const ProdAcc<float> &a)
  {
    float hi = a.hi, lo = a.lo;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      {
        const float h2 = __shfl_down_sync(0xffffffffu, hi, o);
        const float l2 = __shfl_down_sync(0xffffffffu, lo, o);
        float       s, t;
        two_sum(hi, h2, s, t);
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(l2, t));
      }
    return block_sum_lane0((threadIdx.x & 31u) == 0 ? double(hi) + double(lo) : 0.0);
  }

  template <typename T>
  __global__ void __launch_bounds__(RED_SHORT_THREADS)
  k_dot(size_t n, const T *__restrict__ x, const T *__restrict__ y,
        double *__restrict__ partial, unsigned *ticket, double *__restrict__ out)
  {
    ProdAcc<T> s;
#pragma unroll 4
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      s.add(x[i], y[i]);
    finish_partials(block_sum_acc(s), partial, ticket, out);
  }

  // CG update x += alpha p, r -= alpha q with alpha = num/den, and |r|^2
  template <typename T>
  __global__ void __launch_bounds__(RED_SHORT_THREADS)
  k_cg_update_rr(size_t n, const double *__restrict__ num, const double *__restrict__ den,
                 T *__restrict__ x, const T *__restrict__ p, T *__restrict__ r,
                 const T *__restrict__ q, double *__restrict__ partial, unsigned *ticket,
                 double *__restrict__ out)
  {
    const T    alpha = T(block_ratio(num, den));
    ProdAcc<T> s;
#pragma unroll 4
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      {
        x[i] += alpha * p[i];
        const T rr = r[i] - alpha * q[i];
        r[i]       = rr;
        s.add(rr, rr);
      }
    finish_partials(block_sum_acc(s), partial, ticket, out);
  }

  // Jacobi-preconditioned CG step: x += alpha p, r -= alpha q (alpha =
  // num/den), z = dinv r, and |r|^2 -> out_rr, r.z -> out_rz
  template <typename T>
  __global__ void __launch_bounds__(RED_SHORT_THREADS)
  k_cg_update_jacobi(size_t n, const double *__restrict__ num, const double *__restrict__ den,
                     T *__restrict__ x, const T *__restrict__ p, T *__restrict__ r,
                     const T *__restrict__ q, const T *__restrict__ dinv, T *__restrict__ z,
                     double *__restrict__ partial, unsigned *ticket, double *__restrict__ out_rr,
                     double *__restrict__ out_rz)
  {
    const T    alpha = T(block_ratio(num, den));
    ProdAcc<T> srr, srz;
#pragma unroll 4
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      {
        x[i] += alpha * p[i];
        const T rr = r[i] - alpha * q[i];
        const T zz = T(1) * dinv[i] * rr;
        r[i]       = rr;
        z[i]       = zz;
        srr.add(rr, rr);
        srz.add(rr, zz);
      }
    const double a = block_sum_acc(srr);
    __syncthreads(); // the block sum's shared scratch is reused
    const double b = block_sum_acc(srz);
    finish_partials2(a, b, partial, ticket, out_rr, out_rz);
  }

  // p = z + beta p (beta = s[rzn]/s[rz]); q = 0 for the next application
  // (q_zero, may be null); and the Lanczos record of this iteration
  // (k_lanczos_record) written by one thread
  template <typename T>
  __global__ void
  k_cg_direction_rec(size_t n, const double *__restrict__ s, int rz, int rzn, int pq, int rr,
                     const T *__restrict__ z, T *__restrict__ p, T *__restrict__ q_zero,
                     double *__restrict__ rec, int *__restrict__ counter)
  {
    const T beta = T(block_ratio(s + rzn, s + rz));
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      {
        p[i] = z[i] + beta * p[i];
        if (q_zero)
          q_zero[i] = T(0);
      }
    if (blockIdx.x == 0 && threadIdx.x == 0)
      {
        const int k    = (*counter)++;
        rec[3 * k]     = s[rz] / s[pq];
        rec[3 * k + 1] = s[rr];
        rec[3 * k + 2] = s[rzn] / s[rz];
      }
  }

  // p = z + beta p,  beta = num/den
  template <typename T>
  __global__ void
  k_cg_direction(size_t n, const double *__restrict__ num,
                 const double *__restrict__ den, const T *__restrict__ z,
                 T *__restrict__ p)
  {
    const T beta = T(block_ratio(num, den));
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      p[i] = z[i] + beta * p[i];
  }

  // Lanczos record of the next CG iteration (index from a device counter):
  // alpha = rz/pq, |r|^2, beta = rzn/rz
  static __global__ void
  k_lanczos_record(const double *__restrict__ s, int rz, int rzn, int pq, int rr,
                   double *__restrict__ rec, int *__restrict__ counter)
  {
    const int k    = (*counter)++;
    rec[3 * k]     = s[rz] / s[pq];
    rec[3 * k + 1] = s[rr];
    rec[3 * k + 2] = s[rzn] / s[rz];
  }

  // Chebyshev step (PreconditionChebyshev vector updates):
  //   t  = Dinv (b - Ax)
  //   xn = first ? (1+f1) x + f2 t : x + f1 (x - xold) + f2 t ; xold = x ; x = xn
  // (zero_ax: Ax is left zero, so the next application can add into it)
  template <typename T>
  __global__ void
  k_cheby_update(size_t n, T f1, T f2, int first, int zero_ax, const T *__restrict__ b,
                 T *__restrict__ Ax, const T *__restrict__ dinv,
                 T *__restrict__ x, T *__restrict__ xold)
  {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      {
        const T t  = dinv[i] * (b[i] - Ax[i]);
        if (zero_ax)
          Ax[i] = T(0);
        const T xi = x[i];
        const T xn = first ? (T(1) + f1) * xi + f2 * t : xi + f1 * (xi - xold[i]) + f2 * t;
        xold[i]    = xi;
        x[i]       = xn;
      }
  }

  // x = f * dinv .* b ; xold = 0   (first Chebyshev iterate from zero)
  template <typename T>
  __global__ void
  k_cheby_start(size_t n, T f, const T *__restrict__ b, const T *__restrict__ dinv,
                T *__restrict__ x, T *__restrict__ xold)
  {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
      {
        x[i]    = f * dinv[i] * b[i];
        xold[i] = T(0);
      }
  }

  // ---------------------------------------------------------------------
  // Constrained rows (homogeneous Dirichlet on box faces).  Each (node,
  // component) on a constrained face is visited exactly once: by the lowest
  // numbered face that constrains that component at that node.
  // op: 0 dst = src, 1 dst += src, 2 dst = 0, 3 dst = 1
  // ---------------------------------------------------------------------
  // ---------------------------------------------------------------------
  // Dense row-major n x n operators (small coarse levels, n <= 4096), rows
  // ld apart with ld a multiple of 4 (every row starts on a 16-byte
  // boundary; columns n..ld-1 hold zeros).  TPR threads per row (a power of
  // two from 32 to 256, chosen so that the grid covers the GPU) in blocks of
  // DENSE_THREADS.  Rows and x are read in 16-byte vectors (x in scalars
  // when it is not 16-byte aligned), several per thread in flight, where
  // one element per lane and step left the warps waiting on L2.  The
  // partial sums of a row are added in a fixed order, so results do not
  // vary from run to run.  (Staging x in shared memory first, or keeping
  // only each row's window of nonzero columns, measured slower: a step is
  // bound by latency, about 4 us per launch in a graph, not by the bytes.)
  // ---------------------------------------------------------------------
  constexpr int DENSE_THREADS = 512;

  template <typename T>
  struct Vec16;
  template <>
  struct Vec16<float>
  {
    using V                 = float4;
    static constexpr int W = 4;
  };
  template <>
  struct Vec16<double>
  {
    using V                 = double2;
    static constexpr int W = 2;
  };

  template <typename T, int W>
  __device__ __forceinline__ void
  dense_fma(const typename Vec16<T>::V &a, const T *x, T &s0, T &s1)
  {
    s0 = fma(a.x, x[0], s0);
    s1 = fma(a.y, x[1], s1);
    if constexpr (W == 4)
      {
        s0 = fma(a.z, x[2], s0);
        s1 = fma(a.w, x[3], s1);
      }
  }

  // row r . x, valid in the row's first thread (t == 0); every thread of
  // the block calls it (it synchronises the block when TPR > 32)
  template <typename T, int TPR>
  __device__ __forceinline__ T
  dense_row_dot(int n, int ld, int r, const T *__restrict__ A, const T *__restrict__ x, int t, T *red)
  {
    using V         = typename Vec16<T>::V;
    constexpr int W = Vec16<T>::W;
    T             s0 = T(0), s1 = T(0);
    if (r < n)
      {
        const T  *row  = A + size_t(r) * size_t(ld);
        const V  *rv   = reinterpret_cast<const V *>(row);
        const int full = n / W; // vectors whose W entries of x all exist
        if ((reinterpret_cast<uintptr_t>(x) & 15u) == 0u)
          {
            const V *xv = reinterpret_cast<const V *>(x);
#pragma unroll 4
            for (int g = t; g < full; g += TPR)
              {
                const V a  = __ldg(rv + g);
                const V xx = __ldg(xv + g);
                dense_fma<T, W>(a, reinterpret_cast<const T *>(&xx), s0, s1);
              }
          }
        else
          {
#pragma unroll 4
            for (int g = t; g < full; g += TPR)
              {
                const V a = __ldg(rv + g);
                T       xx[W];
#pragma unroll
                for (int k = 0; k < W; ++k)
                  xx[k] = __ldg(x + g * W + k);
                dense_fma<T, W>(a, xx, s0, s1);
              }
          }
        for (int j = full * W + t; j < n; j += TPR)
          s0 = fma(__ldg(row + j), __ldg(x + j), s0);
      }
    T s = s0 + s1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      s += __shfl_xor_sync(0xffffffffu, s, o);
    if constexpr (TPR > 32)
      {
        const int w = int(threadIdx.x) / 32;
        if ((threadIdx.x & 31u) == 0)
          red[w] = s;
        __syncthreads();
        if (t == 0)
#pragma unroll
          for (int k = 1; k < TPR / 32; ++k)
            s += red[w + k];
      }
    return s;
  }

  // y = A x (add: y += A x)
  template <typename T, int TPR>
  __global__ void __launch_bounds__(DENSE_THREADS)
  k_dense_mv(int n, int ld, const T *__restrict__ A, const T *__restrict__ x, T *__restrict__ y, int add)
  {
    __shared__ T red[DENSE_THREADS / 32];
    const int    r = int(blockIdx.x) * (DENSE_THREADS / TPR) + int(threadIdx.x) / TPR;
    const int    t = int(threadIdx.x) % TPR;
    const T      s = dense_row_dot<T, TPR>(n, ld, r, A, x, t, red);
    if (r < n && t == 0)
      y[r] = add ? y[r] + s : s;
  }

  // one Chebyshev step with the dense operator (k_cheby_update with
  // Ax = A x computed in place): xo <- the new iterate; x keeps the
  // current one (the caller swaps the two)
  template <typename T, int TPR>
  __global__ void __launch_bounds__(DENSE_THREADS)
  k_cheby_dense(int n, int ld, const T *__restrict__ A, T f1, T f2, int first, const T *__restrict__ b,
                const T *__restrict__ dinv, const T *__restrict__ x, T *__restrict__ xo)
  {
    __shared__ T red[DENSE_THREADS / 32];
    const int    r = int(blockIdx.x) * (DENSE_THREADS / TPR) + int(threadIdx.x) / TPR;
    const int    t = int(threadIdx.x) % TPR;
    const T      s = dense_row_dot<T, TPR>(n, ld, r, A, x, t, red);
    if (r < n && t == 0)
      {
        const T tt = dinv[r] * (b[r] - s);
        const T xi = x[r];
        xo[r]      = first ? (T(1) + f1) * xi + f2 * tt : xi + f1 * (xi - xo[r]) + f2 * tt;
      }
  }

  struct FaceInfo
  {
    int      Nn[3];
    size_t   n_nodes;
    unsigned face_mask[6];
    int      nc;
    size_t   ld; // op 4: row stride of the dense matrix
  };

  template <typename T>
  __global__ void
  k_constrained(const FaceInfo fi, int op, const T *__restrict__ src,
                T *__restrict__ dst)
  {
    const int f = blockIdx.y;
    if (!fi.face_mask[f])
      return;
    const int nd = f / 2, side = f % 2;
    const int d1 = nd == 0 ? 1 : 0, d2 = nd == 2 ? 1 : 2;
    const int n1 = fi.Nn[d1], n2 = fi.Nn[d2];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n1 * n2;
         t += gridDim.x * blockDim.x)
      {
        int ii[3];
        ii[nd] = side ? fi.Nn[nd] - 1 : 0;
        ii[d1] = t % n1;
        ii[d2] = t / n1;
        const size_t node = size_t(ii[0]) + size_t(fi.Nn[0]) * (size_t(ii[1]) + size_t(fi.Nn[1]) * ii[2]);
        for (int c = 0; c < fi.nc; ++c)
          {
            if (!((fi.face_mask[f] >> c) & 1u))
              continue;
            // owner: lowest face constraining component c at this node
            bool owner = true;
            for (int f2 = 0; f2 < f; ++f2)
              {
                const int nd2 = f2 / 2, s2 = f2 % 2;
                if (((fi.face_mask[f2] >> c) & 1u) && ii[nd2] == (s2 ? fi.Nn[nd2] - 1 : 0))
                  owner = false;
              }
            if (!owner)
              continue;
            const size_t i = size_t(c) * fi.n_nodes + node;
            if (op == 0)
              dst[i] = src[i];
            else if (op == 1)
              dst[i] += src[i];
            else if (op == 2)
              dst[i] = T(0);
            else if (op == 3)
              dst[i] = T(1);
            else // dense matrix: unit diagonal entry of row i
              dst[i * fi.ld + i] = T(1);
          }
      }
  }

  // ---------------------------------------------------------------------
  // One tensor-direction pass of a banded 1D operator (transfer):
  //   out[.., r, ..] = sum_t val[r][t] * in[.., col[r][t], ..]
  // along direction dir; the component index is the outermost dimension.
  // ---------------------------------------------------------------------
  struct PassDims
  {
    int ext_in[3];
    int ext_out[3];
    int nc;
    int dir;
    int width; // entries per row
    // constrained (homogeneous Dirichlet) entries: input entries on a face
    // whose mask face_in has the component's bit read as 0 (mask_in), and
    // such output entries get 0 (mask_out, face_out), as the zeroing of a
    // copy of the input and of the output did before; add: out += result
    // (constrained outputs untouched)
    int      mask_in, mask_out, add;
    unsigned face_in[6], face_out[6];
  };

  // constrained components at node (i0, i1, i2) of a box of ext nodes
  __device__ __forceinline__ unsigned
  pass_node_mask(const unsigned (&f)[6], const int (&ext)[3], int i0, int i1, int i2)
  {
    return (i0 == 0 ? f[0] : 0u) | (i0 == ext[0] - 1 ? f[1] : 0u) | (i1 == 0 ? f[2] : 0u) |
           (i1 == ext[1] - 1 ? f[3] : 0u) | (i2 == 0 ? f[4] : 0u) | (i2 == ext[2] - 1 ? f[5] : 0u);
  }

  template <typename T>
  __global__ void
  k_transfer_pass(const PassDims pd, const int *__restrict__ col,
                  const T *__restrict__ val, const T *__restrict__ in,
                  T *__restrict__ out)
  {
    const size_t per_c = size_t(pd.ext_out[0]) * pd.ext_out[1] * pd.ext_out[2];
    const size_t total = per_c * pd.nc;
    const size_t in_c  = size_t(pd.ext_in[0]) * pd.ext_in[1] * pd.ext_in[2];
    const int    dir   = pd.dir;
    const size_t stride_in = dir == 0 ? size_t(1) : (dir == 1 ? size_t(pd.ext_in[0]) :
                                                                size_t(pd.ext_in[0]) * pd.ext_in[1]);
    for (size_t o = blockIdx.x * size_t(blockDim.x) + threadIdx.x; o < total;
         o += size_t(gridDim.x) * blockDim.x)
      {
        const size_t c  = o / per_c;
        size_t       rm = o - c * per_c;
        const int    i0 = int(rm % pd.ext_out[0]);
        rm /= pd.ext_out[0];
        const int  i1  = int(rm % pd.ext_out[1]);
        const int  i2  = int(rm / pd.ext_out[1]);
        const int  r   = dir == 0 ? i0 : (dir == 1 ? i1 : i2);
        const bool con = pd.mask_out && ((pass_node_mask(pd.face_out, pd.ext_out, i0, i1, i2) >> c) & 1u);
        // input node (j0, j1, j2) = the output node with index cc along dir
        const int    b0   = dir == 0 ? 0 : i0, b1 = dir == 1 ? 0 : i1, b2 = dir == 2 ? 0 : i2;
        const size_t base = c * in_c + size_t(b0) + size_t(pd.ext_in[0]) * (size_t(b1) + size_t(pd.ext_in[1]) * b2);
        T            s    = T(0);
        for (int t = 0; t < pd.width; ++t)
          {
            const int cc = col[r * pd.width + t];
            if (cc >= 0)
              {
                T v = in[base + size_t(cc) * stride_in];
                if (pd.mask_in &&
                    ((pass_node_mask(pd.face_in, pd.ext_in, dir == 0 ? cc : i0, dir == 1 ? cc : i1,
                                     dir == 2 ? cc : i2) >>
                      c) &
                     1u))
                  v = T(0);
                s += val[r * pd.width + t] * v;
              }
          }
        if (pd.add)
          {
            if (!con)
              out[o] += s;
          }
        else
          out[o] = con ? T(0) : s;
      }
  }

  // ---------------------------------------------------------------------
  // Boundary traction (mf_elasticity.h:1849-1897): for each cell face on
  // the traction boundary, t0 = t |det F F^{-T} N| at the face Gauss points,
  // integrated against the face shape functions.  One block per boundary
  // cell face.
  // ---------------------------------------------------------------------
  struct TractionArgs
  {
    int      C[3], Nn[3], p, N;
    size_t   n_nodes;
    double   h[3];
    int      face; // box face 0..5
    double   t[3];
    double   S[MAX_N * MAX_N];   // [q][i]
    double   G[MAX_N * MAX_N];   // [q][i] derivative at Gauss points
    double   Ge[2][MAX_N];       // derivative at 0 and 1
    double   w[MAX_N];
  };

  // the same for a 2D box (faces 0..3 are edges; one block per boundary cell)
  static __global__ void
  k_traction2d(const __grid_constant__ TractionArgs A, const double *__restrict__ u,
               double *__restrict__ rhs)
  {
    __shared__ double tq[2][MAX_N];
    const int nd = A.face / 2, side = A.face % 2;
    const int d1 = 1 - nd;
    const int N  = A.N;
    int       cc[2];
    cc[nd]       = side ? A.C[nd] - 1 : 0;
    cc[d1]       = blockIdx.x;
    const int ln = side ? N - 1 : 0;
    for (int q1 = threadIdx.x; q1 < N; q1 += blockDim.x)
      {
        double F[2][2] = {{0, 0}, {0, 0}};
        for (int j = 0; j < N; ++j)
          for (int i = 0; i < N; ++i)
            {
              const int li[2] = {i, j};
              double    vv[2], dd[2];
              for (int d = 0; d < 2; ++d)
                {
                  if (d == nd)
                    {
                      vv[d] = li[d] == ln ? 1.0 : 0.0;
                      dd[d] = A.Ge[side][li[d]];
                    }
                  else
                    {
                      vv[d] = A.S[q1 * N + li[d]];
                      dd[d] = A.G[q1 * N + li[d]];
                    }
                }
              const double g0   = dd[0] * vv[1] / A.h[0];
              const double g1   = vv[0] * dd[1] / A.h[1];
              const size_t node = size_t(cc[0] * A.p + i) + size_t(A.Nn[0]) * size_t(cc[1] * A.p + j);
              for (int c = 0; c < 2; ++c)
                {
                  const double uv = u[size_t(c) * A.n_nodes + node];
                  F[c][0] += g0 * uv;
                  F[c][1] += g1 * uv;
                }
            }
        F[0][0] += 1.0;
        F[1][1] += 1.0;
        // n* = J F^{-T} N = cof(F) N, cof(F) = [[F11, -F10], [-F01, F00]]
        const double cof[2][2] = {{F[1][1], -F[1][0]}, {-F[0][1], F[0][0]}};
        const double sgn       = side ? 1.0 : -1.0;
        const double n0 = cof[0][nd] * sgn, n1 = cof[1][nd] * sgn;
        const double ns = sqrt(n0 * n0 + n1 * n1);
        const double jw = A.w[q1] * A.h[d1];
        for (int c = 0; c < 2; ++c)
          tq[c][q1] = A.t[c] * ns * jw;
      }
    __syncthreads();
    for (int i1 = threadIdx.x; i1 < N; i1 += blockDim.x)
      {
        int li[2];
        li[nd]      = ln;
        li[d1]      = i1;
        double r[2] = {0, 0};
        for (int q1 = 0; q1 < N; ++q1)
          {
            const double phi = A.S[q1 * N + i1];
            r[0] += phi * tq[0][q1];
            r[1] += phi * tq[1][q1];
          }
        const size_t node = size_t(cc[0] * A.p + li[0]) + size_t(A.Nn[0]) * size_t(cc[1] * A.p + li[1]);
        for (int c = 0; c < 2; ++c)
          atomicAdd(rhs + size_t(c) * A.n_nodes + node, r[c]);
      }
  }

  // 3D: one block per face cell.  The cell's values are staged in shared
  // memory; along the face normal only two quantities matter, the values on
  // the face nodes (for the tangential derivatives) and the normal
  // derivative at the face (Ge, one contraction over the normal index), so
  // the deformation gradient at a face Gauss point is a tensor-product
  // interpolation of those two face arrays.
  static __global__ void __launch_bounds__(128)
  k_traction(const __grid_constant__ TractionArgs A, const double *__restrict__ u,
             double *__restrict__ rhs)
  {
    __shared__ double uc[3][MAX_N * MAX_N * MAX_N]; // cell values [c][k][j][i]
    __shared__ double uf[3][MAX_N * MAX_N];          // face-node values [c][i2][i1]
    __shared__ double un[3][MAX_N * MAX_N];          // face-node normal derivatives
    __shared__ double Fs[9][MAX_N * MAX_N];          // grad u at the face points [c*3+d][q]
    __shared__ double tq[3][MAX_N * MAX_N];
    const int nd = A.face / 2, side = A.face % 2;
    const int d1 = nd == 0 ? 1 : 0, d2 = nd == 2 ? 1 : 2;
    const int N = A.N, N2 = N * N, N3 = N2 * N;
    // face cell (c1, c2) in the tangential directions
    const int c1 = blockIdx.x % A.C[d1], c2 = blockIdx.x / A.C[d1];
    int       cc[3];
    cc[nd] = side ? A.C[nd] - 1 : 0;
    cc[d1] = c1;
    cc[d2] = c2;
    const int    ln  = side ? N - 1 : 0; // local index of the face in nd
    const size_t Nx  = size_t(A.Nn[0]), Nxy = size_t(A.Nn[0]) * size_t(A.Nn[1]);
    const size_t org = size_t(cc[0] * A.p) + Nx * size_t(cc[1] * A.p) + Nxy * size_t(cc[2] * A.p);
    for (int t = threadIdx.x; t < 3 * N3; t += blockDim.x)
      {
        const int c = t / N3, l = t - c * N3;
        const int i = l % N, j = (l / N) % N, k = l / N2;
        uc[c][l] = u[size_t(c) * A.n_nodes + org + size_t(i) + Nx * size_t(j) + Nxy * size_t(k)];
      }
    __syncthreads();
    int str[3];
    str[0] = 1;
    str[1] = N;
    str[2] = N2;
    for (int t = threadIdx.x; t < 3 * N2; t += blockDim.x)
      {
        const int c = t / N2, l = t - c * N2;
        const int off = (l % N) * str[d1] + (l / N) * str[d2];
        double    s   = 0;
        for (int k = 0; k < N; ++k)
          s += A.Ge[side][k] * uc[c][off + k * str[nd]];
        un[c][l] = s;
        uf[c][l] = uc[c][off + ln * str[nd]];
      }
    __syncthreads();
    // grad u of component c at face point (q1, q2)
    for (int t = threadIdx.x; t < 3 * N2; t += blockDim.x)
      {
        const int c = t / N2, qq = t - c * N2, q1 = qq % N, q2 = qq / N;
        double    gn = 0, g1 = 0, g2 = 0;
        for (int i2 = 0; i2 < N; ++i2)
          {
            const double s2 = A.S[q2 * N + i2], e2 = A.G[q2 * N + i2];
            double       rn = 0, r1 = 0, r2 = 0;
            for (int i1 = 0; i1 < N; ++i1)
              {
                const double v = uf[c][i1 + N * i2];
                rn += A.S[q1 * N + i1] * un[c][i1 + N * i2];
                r1 += A.G[q1 * N + i1] * v;
                r2 += A.S[q1 * N + i1] * v;
              }
            gn += s2 * rn;
            g1 += s2 * r1;
            g2 += e2 * r2;
          }
        Fs[c * 3 + nd][qq] = gn / A.h[nd];
        Fs[c * 3 + d1][qq] = g1 / A.h[d1];
        Fs[c * 3 + d2][qq] = g2 / A.h[d2];
      }
    __syncthreads();
    for (int t = threadIdx.x; t < N2; t += blockDim.x)
      {
        const int q1 = t % N, q2 = t / N;
        double    F[3][3];
        for (int c = 0; c < 3; ++c)
          for (int d = 0; d < 3; ++d)
            F[c][d] = Fs[c * 3 + d][t] + (c == d ? 1.0 : 0.0);
        // n* = J F^{-T} N = cofactor(F) N: column nd of the cofactor matrix
        double cof[3];
        const int a1 = (nd + 1) % 3, a2 = (nd + 2) % 3;
        for (int i = 0; i < 3; ++i)
          {
            const int b1 = (i + 1) % 3, b2 = (i + 2) % 3;
            cof[i] = F[b1][a1] * F[b2][a2] - F[b1][a2] * F[b2][a1];
          }
        const double ns = sqrt(cof[0] * cof[0] + cof[1] * cof[1] + cof[2] * cof[2]);
        const double jw = A.w[q1] * A.h[d1] * A.w[q2] * A.h[d2];
        for (int c = 0; c < 3; ++c)
          tq[c][t] = A.t[c] * ns * jw;
      }
    __syncthreads();
    for (int t = threadIdx.x; t < N2; t += blockDim.x)
      {
        const int i1 = t % N, i2 = t / N;
        int       li[3];
        li[nd] = ln;
        li[d1] = i1;
        li[d2] = i2;
        double r[3] = {0, 0, 0};
        for (int q2 = 0; q2 < N; ++q2)
          for (int q1 = 0; q1 < N; ++q1)
            {
              const double phi = A.S[q1 * N + i1] * A.S[q2 * N + i2];
              for (int c = 0; c < 3; ++c)
                r[c] += phi * tq[c][q1 + q2 * N];
            }
        const size_t node = org + size_t(li[0]) + Nx * size_t(li[1]) + Nxy * size_t(li[2]);
        for (int c = 0; c < 3; ++c)
          atomicAdd(rhs + size_t(c) * A.n_nodes + node, r[c]);
      }
  }
} // namespace mfgpu
