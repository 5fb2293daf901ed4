// The heat operator (mass + dt k Laplace, LaplaceOperator::do_operation_on_
// cell, heat_transfer.h:236-250) in FP32 as a batched-cell contraction on
// the tensor cores.
//
// On a box level every cell has the same affine geometry and the heat
// coefficient is constant (heat_transfer.h:63-71), so every cell has the
// same element matrix A_e = M_e + dt k K_e (n_e = (p+1)^3 square), the
// QGauss(p+1) integral the sum-factorization kernel evaluates.  The cell
// loop is then one matrix product per batch of 128 cells:
//
//     Y[cell][i] = sum_j X[cell][j] A_e[i][j]     (M = 128 cells, N = n_e,
//                                                   K = n_e)
//
// computed by tcgen05.mma kind::tf32 from shared memory into a tensor-memory
// accumulator (one TMEM lane per cell), with the three-term split
// X A = Xh Ah + Xh Al + Xl Ah (Xh = tf32(X), Xl = tf32(X - Xh); likewise A)
// to keep FP32 accuracy.  Gather, constraint zeroing and the atomic
// scatter are those of the sum-factorization kernel (mf_cell.cuh).
//
// Per batch (one CTA, 128 threads, one cell per thread):
//   * tensor memory for the 128 x N_pad FP32 accumulator;
//   * K is walked in chunks of 32: the 128 x 32 tile of cell values (hi and
//     lo) is gathered by the threads into shared memory in the no-swizzle
//     K-major core-matrix layout, and the N_pad x 32 chunk of A_e (hi and
//     lo, prepared on the host in the same layout) arrives by one bulk copy
//     (cp.async.bulk) signalled on an mbarrier;
//   * thread 0 issues 4 K-steps x 3 split terms of MMA and commits them to
//     an mbarrier, which all threads wait on before the tile is rewritten;
//   * each warp reads its 32 TMEM lanes (tcgen05.ld) and scatters.
// Every wait is bounded: after its limit the kernel sets an error flag,
// skips the rest of the batch, and still frees its tensor memory.
#include <cstdint>
#include <cstring>
#include <vector>

#include "mf_host.h"

namespace mfgpu
{
  namespace em
  {
    constexpr int CELLS = 128; // MMA M: one cell per TMEM lane and per thread
    constexpr int KC    = 32;  // K per chunk: 4 MMA K-steps of 8 tf32

    template <int N>
    struct Dims
    {
      static constexpr int NE    = N * N * N;
      static constexpr int NP    = (NE + 15) / 16 * 16; // MMA N (M = 128: multiple of 16, <= 256)
      static constexpr int KCH   = (NE + KC - 1) / KC;  // K chunks
      static constexpr int TCOLS = NP <= 32 ? 32 : NP <= 64 ? 64 : NP <= 128 ? 128 : 256;
      static constexpr int A_BYTES = CELLS * KC * 4;     // one split term of the cell tile
      static constexpr int B_BYTES = NP * KC * 4;        // one split term of an A_e chunk
      static constexpr int SMEM    = 2 * A_BYTES + 2 * B_BYTES + 64;
      static_assert(NP <= 256, "element matrix too large for one MMA");
    };

    // byte offset of element (row, k) of a rows x 32 K-major tile in the
    // no-swizzle core-matrix layout: 8 x 16-byte core matrices, K-adjacent
    // core matrices 128 bytes apart (leading byte offset), 8-row groups
    // 1024 bytes apart (stride byte offset)
    __host__ __device__ constexpr unsigned
    tile_offset(int row, int k)
    {
      return unsigned(((row >> 3) * (KC / 4) + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4);
    }
    constexpr unsigned LBO = 128, SBO = 1024;

    __device__ __forceinline__ uint32_t
    smem_addr(const void *p)
    {
      return static_cast<uint32_t>(__cvta_generic_to_shared(p));
    }

    // tcgen05 shared-memory matrix descriptor: start address, leading and
    // stride byte offsets (all >> 4), descriptor version 1, no swizzle
    __device__ __forceinline__ uint64_t
    smem_desc(uint32_t saddr)
    {
      return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((LBO >> 4) & 0x3FFFu) << 16) |
             (uint64_t((SBO >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
    }

    // instruction descriptor of kind::tf32: D FP32, A and B TF32, both
    // K-major, N >> 3 and M >> 4
    __host__ __device__ constexpr uint32_t
    instr_desc(int n, int m)
    {
      return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
    }

    __device__ __forceinline__ float
    to_tf32(float x)
    {
      uint32_t r;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
      return __uint_as_float(r);
    }

    __device__ __forceinline__ void
    mbar_init(uint64_t *bar, unsigned count)
    {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    }

    __device__ __forceinline__ bool
    mbar_try_wait(uint64_t *bar, unsigned parity)
    {
      uint32_t ok;
      asm volatile("{\n\t.reg .pred p;\n\t"
                   "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                   "selp.u32 %0, 1, 0, p;\n\t}"
                   : "=r"(ok)
                   : "r"(smem_addr(bar)), "r"(parity)
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

    __device__ __forceinline__ void
    bulk_load(void *dst_smem, const void *src, unsigned bytes, uint64_t *bar)
    {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                   : "memory");
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst_smem)),
                   "l"(src), "r"(bytes), "r"(smem_addr(bar))
                   : "memory");
    }

    __device__ __forceinline__ void
    mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
    {
      asm volatile("{\n\t.reg .pred p;\n\t"
                   "setp.ne.b32 p, %4, 0;\n\t"
                   "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                   "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
                   : "memory");
    }

    __device__ __forceinline__ void
    mma_commit(uint64_t *bar)
    {
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(bar))
                   : "memory");
    }

    __device__ __forceinline__ void
    tmem_load8(uint32_t taddr, float (&v)[8])
    {
      uint32_t r[8];
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                   : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                     "=r"(r[7])
                   : "r"(taddr)
                   : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int i = 0; i < 8; ++i)
        v[i] = __uint_as_float(r[i]);
    }

    struct Args
    {
      int      C[3], Nn[3], p;
      size_t   n_nodes;
      unsigned face_mask[6];
      int      constrained;
      size_t   cell_begin, cell_end;
    };

    template <int N>
    __global__ void __launch_bounds__(CELLS)
    heat_em_kernel(const __grid_constant__ Args g, const unsigned char *__restrict__ bmat,
                   const float *__restrict__ src, float *__restrict__ dst, int *__restrict__ err)
    {
      using Dm = Dims<N>;
      constexpr int NE = Dm::NE, NP = Dm::NP, KCH = Dm::KCH;
      extern __shared__ __align__(1024) unsigned char smem[];
      unsigned char *sA_hi = smem;
      unsigned char *sA_lo = smem + Dm::A_BYTES;
      unsigned char *sB    = smem + 2 * Dm::A_BYTES; // hi then lo, one chunk
      uint64_t      *bar_b = reinterpret_cast<uint64_t *>(smem + 2 * Dm::A_BYTES + 2 * Dm::B_BYTES);
      uint64_t      *bar_m = bar_b + 1;
      uint32_t      *tslot = reinterpret_cast<uint32_t *>(bar_b + 2);
      int           *fail  = reinterpret_cast<int *>(bar_b + 3);

      const int    t    = threadIdx.x;
      const int    warp = t >> 5;
      const size_t cell = g.cell_begin + size_t(blockIdx.x) * CELLS + t;
      const bool   active = cell < g.cell_end;
      const size_t cc   = active ? cell : g.cell_begin;
      const int    cx = int(cc % unsigned(g.C[0])), cyz = int(cc / unsigned(g.C[0]));
      const int    cy = cyz % g.C[1], cz = cyz / g.C[1];
      const size_t base = size_t(cx * g.p) + size_t(g.Nn[0]) * (size_t(cy * g.p) + size_t(g.Nn[1]) * (cz * g.p));
      // constraint tests only on cells touching the box boundary
      const bool boundary = g.constrained && (cx == 0 || cy == 0 || cz == 0 || cx == g.C[0] - 1 ||
                                              cy == g.C[1] - 1 || cz == g.C[2] - 1);
      auto node_of = [&](int l, int &ix, int &iy, int &iz) {
        const int a = l % N, b = (l / N) % N, c = l / (N * N);
        ix = cx * g.p + a, iy = cy * g.p + b, iz = cz * g.p + c;
        return base + size_t(a) + size_t(g.Nn[0]) * (size_t(b) + size_t(g.Nn[1]) * size_t(c));
      };

      if (t == 0)
        {
          mbar_init(bar_b, 1);
          mbar_init(bar_m, 1);
          *fail = 0;
          asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
      if (warp == 0)
        {
          asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(tslot)),
                       "r"(Dm::TCOLS)
                       : "memory");
          asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tmem  = *tslot;
      constexpr uint32_t IDESC = instr_desc(NP, CELLS);
      int loads = 0, commits = 0; // thread 0: bulk loads and MMA commits issued

      for (int kc = 0; kc < KCH; ++kc)
        {
          if (kc > 0)
            {
              // the previous chunk's MMAs have read the tiles
              if (!mbar_wait(bar_m, unsigned(kc - 1) & 1u))
                atomicOr(fail, 1);
              __syncthreads();
              if (*fail)
                break;
            }
          if (t == 0)
            {
              bulk_load(sB, bmat + size_t(kc) * 2 * Dm::B_BYTES, 2 * Dm::B_BYTES, bar_b);
              ++loads;
            }
          // this thread's cell: values kc*32 .. kc*32+31, split into tf32 hi/lo
#pragma unroll
          for (int k4 = 0; k4 < KC; k4 += 4)
            {
              float hi[4], lo[4];
#pragma unroll
              for (int q = 0; q < 4; ++q)
                {
                  const int l = kc * KC + k4 + q;
                  float     v = 0.f;
                  if (active && l < NE)
                    {
                      int          ix, iy, iz;
                      const size_t node = node_of(l, ix, iy, iz);
                      bool         skip = false;
                      if (boundary)
                        skip = node_mask(g.face_mask, g.Nn, ix, iy, iz) & 1u;
                      if (!skip)
                        v = __ldg(src + node);
                    }
                  hi[q] = to_tf32(v);
                  lo[q] = to_tf32(v - hi[q]);
                }
              const unsigned off = tile_offset(t, k4);
              *reinterpret_cast<float4 *>(sA_hi + off) = make_float4(hi[0], hi[1], hi[2], hi[3]);
              *reinterpret_cast<float4 *>(sA_lo + off) = make_float4(lo[0], lo[1], lo[2], lo[3]);
            }
          // generic-proxy stores -> visible to the tensor core's async proxy
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncthreads();
          if (t == 0)
            {
              if (!mbar_wait(bar_b, unsigned(kc) & 1u))
                atomicOr(fail, 2);
              else
                {
                  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                  const uint32_t a_hi = smem_addr(sA_hi), a_lo = smem_addr(sA_lo);
                  const uint32_t b_hi = smem_addr(sB), b_lo = smem_addr(sB + Dm::B_BYTES);
#pragma unroll
                  for (int ks = 0; ks < KC / 8; ++ks)
                    {
                      // one K-step = 8 tf32 = two core matrices along K
                      const uint32_t o = uint32_t(ks) * 2u * LBO;
                      mma_tf32(tmem, smem_desc(a_hi + o), smem_desc(b_hi + o), IDESC, (kc > 0 || ks > 0) ? 1u : 0u);
                      mma_tf32(tmem, smem_desc(a_hi + o), smem_desc(b_lo + o), IDESC, 1u);
                      mma_tf32(tmem, smem_desc(a_lo + o), smem_desc(b_hi + o), IDESC, 1u);
                    }
                }
              mma_commit(bar_m);
              ++commits;
            }
        }
      // all MMAs done before the accumulator is read
      if (!*fail && !mbar_wait(bar_m, unsigned(KCH - 1) & 1u))
        atomicOr(fail, 4);
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (*fail)
        {
          if (t == 0)
            {
              atomicOr(err, 8 | *fail);
              // let the copies and MMAs in flight land before the shared and
              // tensor memory is released (bounded as well)
              if (loads > 0)
                mbar_wait(bar_b, unsigned(loads - 1) & 1u);
              if (commits > 0)
                mbar_wait(bar_m, unsigned(commits - 1) & 1u);
            }
        }
      else
        {
          const uint32_t lane_base = tmem + (uint32_t(warp * 32) << 16);
#pragma unroll 1
          for (int c0 = 0; c0 < NP; c0 += 8)
            {
              float y[8];
              tmem_load8(lane_base + uint32_t(c0), y);
              if (!active)
                continue;
#pragma unroll
              for (int q = 0; q < 8; ++q)
                {
                  const int l = c0 + q;
                  if (l >= NE)
                    break;
                  int          ix, iy, iz;
                  const size_t node = node_of(l, ix, iy, iz);
                  if (boundary && (node_mask(g.face_mask, g.Nn, ix, iy, iz) & 1u))
                    {
                      // constrained row: dst += src, by the node's owner cell
                      const int  a = l % N, b = (l / N) % N, c = l / (N * N);
                      const bool owner = (a < g.p || cx == g.C[0] - 1) && (b < g.p || cy == g.C[1] - 1) &&
                                         (c < g.p || cz == g.C[2] - 1);
                      if (owner)
                        dst[node] += __ldg(src + node);
                      continue;
                    }
                  atomicAdd(dst + node, y[q]);
                }
            }
        }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Dm::TCOLS)
                     : "memory");
    }

    // host: round to tf32 (nearest, ties away from zero), as cvt.rna.tf32
    float
    host_tf32(float x)
    {
      uint32_t u;
      std::memcpy(&u, &x, 4);
      if ((u & 0x7f800000u) != 0x7f800000u)
        u = (u + 0x1000u) & ~0x1fffu;
      float r;
      std::memcpy(&r, &u, 4);
      return r;
    }

    template <int N>
    void
    build_b(const HostBasis &b, const LevelGeom &g, double kdt, std::vector<unsigned char> &out)
    {
      using Dm = Dims<N>;
      // 1D mass and stiffness matrices on the unit interval (QGauss(N))
      double M1[N][N], K1[N][N];
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
          {
            double m = 0, k = 0;
            for (int q = 0; q < N; ++q)
              {
                m += b.w[q] * b.S[q * N + i] * b.S[q * N + j];
                k += b.w[q] * b.G[q * N + i] * b.G[q * N + j];
              }
            M1[i][j] = m;
            K1[i][j] = k;
          }
      const double vol = g.h[0] * g.h[1] * g.h[2];
      const double sx = kdt / (g.h[0] * g.h[0]), sy = kdt / (g.h[1] * g.h[1]), sz = kdt / (g.h[2] * g.h[2]);
      out.assign(size_t(Dm::KCH) * 2 * Dm::B_BYTES, 0);
      for (int i = 0; i < Dm::NE; ++i)
        for (int j = 0; j < Dm::NE; ++j)
          {
            const int    a = i % N, bb = (i / N) % N, c = i / (N * N);
            const int    a2 = j % N, b2 = (j / N) % N, c2 = j / (N * N);
            const double v  = vol * (M1[a][a2] * M1[bb][b2] * M1[c][c2] + sx * K1[a][a2] * M1[bb][b2] * M1[c][c2] +
                                    sy * M1[a][a2] * K1[bb][b2] * M1[c][c2] + sz * M1[a][a2] * M1[bb][b2] * K1[c][c2]);
            const float hi = host_tf32(float(v));
            const float lo = host_tf32(float(v - double(hi)));
            const int   kc = j / KC, k = j % KC;
            unsigned char *chunk = out.data() + size_t(kc) * 2 * Dm::B_BYTES;
            std::memcpy(chunk + tile_offset(i, k), &hi, 4);
            std::memcpy(chunk + Dm::B_BYTES + tile_offset(i, k), &lo, 4);
          }
    }

    template <int N>
    cudaError_t
    launch(const Args &a, const void *bmat, const float *src, float *dst, int *err, cudaStream_t s)
    {
      using Dm           = Dims<N>;
      static bool attr   = false;
      cudaError_t e      = cudaSuccess;
      if (!attr)
        {
          e = cudaFuncSetAttribute(heat_em_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, Dm::SMEM);
          if (e != cudaSuccess)
            return e;
          attr = true;
        }
      const size_t n = a.cell_end - a.cell_begin;
      if (n == 0)
        return cudaSuccess;
      const unsigned grid = unsigned((n + CELLS - 1) / CELLS);
      heat_em_kernel<N><<<grid, CELLS, Dm::SMEM, s>>>(a, static_cast<const unsigned char *>(bmat), src, dst, err);
      return cudaGetLastError();
    }
  } // namespace em

  bool
  heat_em_supported(int N)
  {
    return N >= 2 && N <= 6;
  }

  size_t
  heat_em_matrix(const HostBasis &b, const LevelGeom &g, double kdt, std::vector<unsigned char> &out)
  {
    switch (b.N)
      {
        case 2: em::build_b<2>(b, g, kdt, out); break;
        case 3: em::build_b<3>(b, g, kdt, out); break;
        case 4: em::build_b<4>(b, g, kdt, out); break;
        case 5: em::build_b<5>(b, g, kdt, out); break;
        case 6: em::build_b<6>(b, g, kdt, out); break;
        default: throw Error(ERR_UNSUPPORTED, "element-matrix heat kernel: degree 1..5 only");
      }
    return out.size();
  }

  cudaError_t
  launch_heat_em(const HostBasis &b, const LevelGeom &g, bool constrained, const void *bmat, const float *src,
                 float *dst, size_t c0, size_t c1, int *err, cudaStream_t s)
  {
    em::Args a;
    for (int d = 0; d < 3; ++d)
      {
        a.C[d]  = g.C[d];
        a.Nn[d] = g.Nn[d];
      }
    a.p       = g.p;
    a.n_nodes = g.n_nodes;
    for (int f = 0; f < 6; ++f)
      a.face_mask[f] = g.face_mask[f];
    a.constrained = constrained ? 1 : 0;
    a.cell_begin  = c1 > c0 ? c0 : 0;
    a.cell_end    = c1 > c0 ? c1 : g.n_cells;
    switch (b.N)
      {
        case 2: return em::launch<2>(a, bmat, src, dst, err, s);
        case 3: return em::launch<3>(a, bmat, src, dst, err, s);
        case 4: return em::launch<4>(a, bmat, src, dst, err, s);
        case 5: return em::launch<5>(a, bmat, src, dst, err, s);
        case 6: return em::launch<6>(a, bmat, src, dst, err, s);
      }
    return cudaErrorInvalidValue;
  }
} // namespace mfgpu
