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
#include <algorithm>
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
    };

    // a brick of 8 x 4 x 4 cells (x fastest), one cell per thread and per
    // TMEM lane; its (8p+1) x (4p+1) x (4p+1) nodes are staged in shared
    // memory, first as the source values, then as the accumulator of the
    // cells' results
    constexpr int BX = 8, BY = 4, BZ = 4;
    static_assert(BX * BY * BZ == CELLS, "one cell per thread");

    template <int N>
    struct Layout
    {
      using Dm                          = Dims<N>;
      static constexpr int P            = N - 1;
      static constexpr int NX           = BX * P + 1, NY = BY * P + 1, NZ = BZ * P + 1;
      static constexpr int NODES        = NX * NY * NZ;
      static constexpr int NODE_BYTES   = (NODES * 4 + 127) / 128 * 128;
      static constexpr int B_ALL        = Dm::KCH * 2 * Dm::B_BYTES;
      static constexpr bool RESIDENT_B  = B_ALL <= 140 * 1024; // the whole element matrix stays in smem
      static constexpr int B_REGION     = RESIDENT_B ? B_ALL : 2 * Dm::B_BYTES;
      static constexpr int OFF_B        = 2 * Dm::A_BYTES;
      static constexpr int OFF_NODES    = OFF_B + B_REGION;
      static constexpr int OFF_BAR      = OFF_NODES + NODE_BYTES;
      static constexpr int SMEM         = OFF_BAR + 64;
      static_assert(SMEM <= 227 * 1024, "shared memory");
    };

    // Persistent: each CTA walks bricks blockIdx.x, blockIdx.x + gridDim.x, ...
    // Per brick: stage the nodes (coalesced, constrained ones zeroed); per K
    // chunk build the tf32 hi/lo tile of the 128 cells from shared memory
    // and issue the MMAs; accumulate the results per node in shared memory
    // (red.shared); write the brick's nodes out, plain adds on nodes no other
    // brick touches and atomics on the shared faces.  Constrained rows get
    // dst += src from the cell that owns the node.
    template <int N>
    __global__ void __launch_bounds__(CELLS)
    heat_em_kernel(const __grid_constant__ Args g, const unsigned char *__restrict__ bmat,
                   const float *__restrict__ src, float *__restrict__ dst, int *__restrict__ err)
    {
      using Dm = Dims<N>;
      using Lo = Layout<N>;
      constexpr int NE = Dm::NE, NP = Dm::NP, KCH = Dm::KCH, P = N - 1;
      constexpr int NX = Lo::NX, NY = Lo::NY;
      extern __shared__ __align__(1024) unsigned char smem[];
      unsigned char *sA_hi = smem;
      unsigned char *sA_lo = smem + Dm::A_BYTES;
      unsigned char *sB    = smem + Lo::OFF_B;
      float         *sN    = reinterpret_cast<float *>(smem + Lo::OFF_NODES);
      uint64_t      *bar_b = reinterpret_cast<uint64_t *>(smem + Lo::OFF_BAR);
      uint64_t      *bar_m = bar_b + 1;
      uint32_t      *tslot = reinterpret_cast<uint32_t *>(bar_b + 2);
      int           *fail  = reinterpret_cast<int *>(bar_b + 3);

      const int t    = threadIdx.x;
      const int warp = t >> 5;
      const int tx = t % BX, ty = (t / BX) % BY, tz = t / (BX * BY);
      // the thread's cell's first node inside the brick
      const int cbase = tx * P + NX * (ty * P + NY * (tz * P));
      const int nbx = (g.C[0] + BX - 1) / BX, nby = (g.C[1] + BY - 1) / BY, nbz = (g.C[2] + BZ - 1) / BZ;
      const int n_bricks = nbx * nby * nbz;

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
      const uint32_t     tmem  = *tslot;
      constexpr uint32_t IDESC = instr_desc(NP, CELLS);
      // thread 0: bulk loads issued and waited for, MMA commits issued;
      // and MMA commits waited for (in order, so parity = count)
      int loads = 0, bwaits = 0, commits = 0, mwaits = 0;
      if (Lo::RESIDENT_B && t == 0)
        {
          bulk_load(sB, bmat, Lo::B_ALL, bar_b);
          ++loads;
        }

#pragma unroll 1
      for (int brick = blockIdx.x; brick < n_bricks; brick += gridDim.x)
        {
          const int bx = brick % nbx, by = (brick / nbx) % nby, bz = brick / (nbx * nby);
          const int x0 = bx * BX, y0 = by * BY, z0 = bz * BZ;          // first cell
          const int n0x = x0 * P, n0y = y0 * P, n0z = z0 * P;          // first node
          const int ex = min(NX, g.Nn[0] - n0x), ey = min(NY, g.Nn[1] - n0y), ez = min(Lo::NZ, g.Nn[2] - n0z);
          const bool touches = g.constrained && (x0 == 0 || y0 == 0 || z0 == 0 || x0 + BX >= g.C[0] ||
                                                 y0 + BY >= g.C[1] || z0 + BZ >= g.C[2]);
          // 1. the brick's nodes (zero outside the mesh and on constrained nodes)
#pragma unroll 4
          for (int i = t; i < Lo::NODES; i += CELLS)
            {
              const int ix = i % NX, iy = (i / NX) % NY, iz = i / (NX * NY);
              float     v  = 0.f;
              if (ix < ex && iy < ey && iz < ez)
                {
                  const int gx = n0x + ix, gy = n0y + iy, gz = n0z + iz;
                  if (!(touches && (node_mask(g.face_mask, g.Nn, gx, gy, gz) & 1u)))
                    v = __ldg(src + size_t(gx) + size_t(g.Nn[0]) * (size_t(gy) + size_t(g.Nn[1]) * gz));
                }
              sN[i] = v;
            }
          __syncthreads();
          const int  cx = x0 + tx, cy = y0 + ty, cz = z0 + tz;
          const bool active = cx < g.C[0] && cy < g.C[1] && cz < g.C[2];
          // 2. K chunks
#pragma unroll 1
          for (int kc = 0; kc < KCH; ++kc)
            {
              if (kc > 0)
                {
                  // the previous chunk's MMAs have read the tiles (one
                  // thread polls; the others wait at the barrier)
                  if (t == 0)
                    {
                      if (!mbar_wait(bar_m, unsigned(mwaits) & 1u))
                        atomicOr(fail, 1);
                      ++mwaits;
                    }
                  __syncthreads();
                }
              if (!Lo::RESIDENT_B && t == 0)
                {
                  bulk_load(sB, bmat + size_t(kc) * 2 * Dm::B_BYTES, 2 * Dm::B_BYTES, bar_b);
                  ++loads;
                }
#pragma unroll
              for (int k4 = 0; k4 < KC; k4 += 4)
                {
                  float hi[4], lo[4];
#pragma unroll
                  for (int q = 0; q < 4; ++q)
                    {
                      const int l = kc * KC + k4 + q;
                      float     v = 0.f;
                      if (l < NE && active)
                        v = sN[cbase + (l % N) + NX * ((l / N) % N + NY * (l / (N * N)))];
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
              if (*fail)
                break;
              if (t == 0)
                {
                  const bool need = !Lo::RESIDENT_B || bwaits == 0;
                  if (need && !mbar_wait(bar_b, unsigned(bwaits) & 1u))
                    atomicOr(fail, 2);
                  else
                    {
                      if (need)
                        ++bwaits;
                      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                      const uint32_t a_hi = smem_addr(sA_hi), a_lo = smem_addr(sA_lo);
                      const uint32_t bb   = smem_addr(sB) + (Lo::RESIDENT_B ? uint32_t(kc) * 2u * Dm::B_BYTES : 0u);
                      const uint32_t b_hi = bb, b_lo = bb + Dm::B_BYTES;
#pragma unroll
                      for (int ks = 0; ks < KC / 8; ++ks)
                        {
                          // one K-step = 8 tf32 = two core matrices along K
                          const uint32_t o = uint32_t(ks) * 2u * LBO;
                          mma_tf32(tmem, smem_desc(a_hi + o), smem_desc(b_hi + o), IDESC,
                                   (kc > 0 || ks > 0) ? 1u : 0u);
                          mma_tf32(tmem, smem_desc(a_hi + o), smem_desc(b_lo + o), IDESC, 1u);
                          mma_tf32(tmem, smem_desc(a_lo + o), smem_desc(b_hi + o), IDESC, 1u);
                        }
                    }
                  mma_commit(bar_m);
                  ++commits;
                }
            }
          // thread 0's MMA issue and any failure flag are visible to all
          __syncthreads();
          if (*fail)
            break;
          // 3. the staged values are consumed: the node array becomes the
          // accumulator (while the last MMAs run)
          for (int i = t; i < Lo::NODES; i += CELLS)
            sN[i] = 0.f;
          if (t == 0)
            {
              if (!mbar_wait(bar_m, unsigned(mwaits) & 1u))
                atomicOr(fail, 4);
              ++mwaits;
            }
          __syncthreads();
          if (*fail)
            break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          // 4. the cell's results into the node accumulator
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
                  const int a = l % N, b = (l / N) % N, c = l / (N * N);
                  if (touches)
                    {
                      const int gx = cx * P + a, gy = cy * P + b, gz = cz * P + c;
                      if (node_mask(g.face_mask, g.Nn, gx, gy, gz) & 1u)
                        {
                          // constrained row: dst += src, by the node's owner cell
                          const bool owner = (a < P || cx == g.C[0] - 1) && (b < P || cy == g.C[1] - 1) &&
                                             (c < P || cz == g.C[2] - 1);
                          if (owner)
                            {
                              const size_t gn = size_t(gx) + size_t(g.Nn[0]) * (size_t(gy) + size_t(g.Nn[1]) * gz);
                              dst[gn] += __ldg(src + gn);
                            }
                          continue;
                        }
                    }
                  atomicAdd(sN + cbase + a + NX * (b + NY * c), y[q]);
                }
            }
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncthreads();
          // 5. write the brick's nodes: plain adds on nodes only this brick
          // touches, atomics on faces shared with a neighbouring brick
#pragma unroll 4
          for (int i = t; i < Lo::NODES; i += CELLS)
            {
              const int ix = i % NX, iy = (i / NX) % NY, iz = i / (NX * NY);
              if (!(ix < ex && iy < ey && iz < ez))
                continue;
              const int gx = n0x + ix, gy = n0y + iy, gz = n0z + iz;
              if (touches && (node_mask(g.face_mask, g.Nn, gx, gy, gz) & 1u))
                continue;
              const size_t gn  = size_t(gx) + size_t(g.Nn[0]) * (size_t(gy) + size_t(g.Nn[1]) * gz);
              const bool   own = (ix > 0 || bx == 0) && (ix < NX - 1 || bx == nbx - 1) && (iy > 0 || by == 0) &&
                               (iy < NY - 1 || by == nby - 1) && (iz > 0 || bz == 0) &&
                               (iz < Lo::NZ - 1 || bz == nbz - 1);
              if (own)
                dst[gn] += sN[i];
              else
                atomicAdd(dst + gn, sN[i]);
            }
          __syncthreads();
        }
      __syncthreads();
      if (*fail)
        {
          if (t == 0)
            {
              atomicOr(err, 8 | *fail);
              // let the copies and MMAs in flight land before the shared and
              // tensor memory is released (bounded as well)
              if (loads > bwaits)
                mbar_wait(bar_b, unsigned(loads - 1) & 1u);
              if (commits > mwaits)
                mbar_wait(bar_m, unsigned(commits - 1) & 1u);
            }
        }
      else if (Lo::RESIDENT_B && t == 0 && loads > bwaits)
        mbar_wait(bar_b, 0u); // a CTA without bricks still lets its copy land
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
      using Lo         = Layout<N>;
      static bool attr = false;
      cudaError_t e    = cudaSuccess;
      if (!attr)
        {
          e = cudaFuncSetAttribute(heat_em_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, Lo::SMEM);
          if (e != cudaSuccess)
            return e;
          attr = true;
        }
      const long n_bricks = long((a.C[0] + BX - 1) / BX) * ((a.C[1] + BY - 1) / BY) * ((a.C[2] + BZ - 1) / BZ);
      // one CTA per brick: the resident CTAs of an SM hide each other's
      // load, MMA and scatter latencies
      const unsigned grid = unsigned(std::max(1L, n_bricks));
      heat_em_kernel<N><<<grid, CELLS, Lo::SMEM, s>>>(a, static_cast<const unsigned char *>(bmat), src, dst, err);
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
                 float *dst, int *err, cudaStream_t s)
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
