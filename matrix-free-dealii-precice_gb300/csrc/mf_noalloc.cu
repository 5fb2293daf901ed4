// Multigrid prolongation that allocates no device memory.
//
// Who needs this: callers that are not allowed to allocate device memory
// while they run.  A coupled multiphysics run, for example, often hands
// nearly all of the GPU's memory to the partner code's pool allocator at
// start-up, so a cudaMalloc issued later from inside a time step fails.
// Other callers have to keep per-step latency flat, and the implicit
// device synchronisation of cudaMalloc/cudaFree would stall their stream.
// Deployments can also forbid device allocations after initialisation
// altogether.  mfgpu_transfer_prolongate() builds a transfer object with
// device tables and two intermediate arrays on every call.  This variant
// runs the same three tensor-product passes, but:
//   * it tabulates the 1D prolongation weights on the host and passes them
//     to the kernel by value;
//   * it keeps the two intermediate arrays in the file-scope array below.
//
// Two-dimensional meshes (mesh.dim = 2) are supported: their single node
// plane in z is copied through by the third pass.
//
// Limit: each intermediate array holds at most SCRATCH_BYTES / 2 bytes
// (2 MiB, i.e. 262,144 doubles or 524,288 floats per intermediate,
// counting all components).  Every GPU that loads the library keeps this
// 4 MiB array until the process exits.  Larger levels are rejected with
// MFGPU_ERR_ARG.
//
// Sharing: all calls on a device use the same array, and it keeps whatever
// the last call left in it.  Every element the passes read was first written
// by the same call, so nothing has to be cleared between calls.  Two calls
// whose work overlaps on the GPU (different streams, or different host
// threads) race on the array and produce wrong results; serialise them.
//
// Set-up: the first call on a device, with that device current, looks up
// the device address of the array (cudaGetSymbolAddress) once and caches
// it.  Make that first call before any stream capture starts.
#include <mutex>
#include <string>

#include "../../include/mfgpu.h"
#include "mf_drivers.h"

namespace
{
  using namespace mfgpu;

  constexpr size_t SCRATCH_BYTES = size_t(4) << 20;
  constexpr size_t HALF_BYTES    = SCRATCH_BYTES / 2;
  constexpr int    MAX_DEVICES   = 64;

  static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

  std::mutex g_setup_mutex;
  void      *g_scratch_addr[MAX_DEVICES] = {};
  int        g_sm_count[MAX_DEVICES]     = {};

  struct NoAllocPass
  {
    int      ext_in[3];
    int      ext_out[3];
    int      nc;
    int      dir;
    int      p;
    // weight[h][lf][i]: Lagrange polynomial i of the coarse cell at the
    // fine node lf of its half h (0 lower, 1 upper), tabulated on the host
    double   weight[2][MAX_N][MAX_N];
    // pass 0 reads the coarse vector: zero its constrained entries
    int      mask_input;
    unsigned in_face_mask[6];
    // pass 2 writes the fine vector: zero its constrained entries
    int      mask_output;
    unsigned out_face_mask[6];
  };

  // One tensor-product pass of the prolongation along P.dir.  A direction
  // with a single node plane on both levels (z of a two-dimensional mesh)
  // is copied through unchanged.
  template <typename T>
  __global__ void
  k_prolongate_pass_noalloc(const __grid_constant__ NoAllocPass P,
                            const T *__restrict__ in, T *__restrict__ out)
  {
    const size_t per_c = size_t(P.ext_out[0]) * P.ext_out[1] * P.ext_out[2];
    const size_t total = per_c * P.nc;
    const size_t in_c  = size_t(P.ext_in[0]) * P.ext_in[1] * P.ext_in[2];
    size_t       stride_in = 1;
    for (int d = 0; d < P.dir; ++d)
      stride_in *= P.ext_in[d];
    const bool copy_through = P.ext_in[P.dir] == 1 && P.ext_out[P.dir] == 1;
    const int  n_fine_cells = (P.ext_out[P.dir] - 1) / P.p;
    for (size_t o = blockIdx.x * size_t(blockDim.x) + threadIdx.x; o < total;
         o += size_t(gridDim.x) * blockDim.x)
      {
        const int c  = int(o / per_c);
        size_t    rm = o - size_t(c) * per_c;
        int       idx[3];
        idx[0] = int(rm % P.ext_out[0]);
        rm /= P.ext_out[0];
        idx[1] = int(rm % P.ext_out[1]);
        idx[2] = int(rm / P.ext_out[1]);
        if (P.mask_output &&
            ((node_mask(P.out_face_mask, P.ext_out, idx[0], idx[1], idx[2]) >> c) & 1u))
          {
            out[o] = T(0);
            continue;
          }
        if (copy_through)
          {
            // same node grid on both sides in this direction
            const size_t io = size_t(c) * in_c + size_t(idx[0]) +
                              size_t(P.ext_in[0]) * (size_t(idx[1]) + size_t(P.ext_in[1]) * idx[2]);
            T v = in[io];
            if (P.mask_input &&
                ((node_mask(P.in_face_mask, P.ext_in, idx[0], idx[1], idx[2]) >> c) & 1u))
              v = T(0);
            out[o] = v;
            continue;
          }
        // fine node f along dir: fine cell, local node, coarse cell
        const int f  = idx[P.dir];
        const int fc = min(f / P.p, n_fine_cells - 1);
        const int lf = f - fc * P.p;
        const int cc = fc / 2;
        const int h  = fc % 2;
        idx[P.dir]   = 0;
        const size_t base = size_t(c) * in_c + size_t(idx[0]) +
                            size_t(P.ext_in[0]) * (size_t(idx[1]) + size_t(P.ext_in[1]) * idx[2]);
        T s = T(0);
        for (int i = 0; i <= P.p; ++i)
          {
            const int col = cc * P.p + i;
            T         v   = in[base + size_t(col) * stride_in];
            if (P.mask_input)
              {
                int ii[3] = {idx[0], idx[1], idx[2]};
                ii[P.dir] = col;
                if ((node_mask(P.in_face_mask, P.ext_in, ii[0], ii[1], ii[2]) >> c) & 1u)
                  v = T(0);
              }
            s += T(P.weight[h][lf][i]) * v;
          }
        out[o] = s;
      }
  }

  template <typename T>
  void
  run_passes(const LevelGeom &coarse, const LevelGeom &fine, int nc,
             const HostBasis &b, const T *coarse_v, T *fine_v, T *s0, T *s1,
             int n_sm, cudaStream_t stream)
  {
    int         ext[3] = {coarse.Nn[0], coarse.Nn[1], coarse.Nn[2]};
    const T    *cur    = coarse_v;
    T          *dsts[3] = {s0, s1, fine_v};
    for (int d = 0; d < 3; ++d)
      {
        NoAllocPass P;
        for (int e = 0; e < 3; ++e)
          {
            P.ext_in[e]  = ext[e];
            P.ext_out[e] = ext[e];
          }
        P.ext_out[d] = fine.Nn[d];
        P.nc         = nc;
        P.dir        = d;
        P.p          = coarse.p;
        for (int h = 0; h < 2; ++h)
          for (int lf = 0; lf < MAX_N; ++lf)
            for (int i = 0; i < MAX_N; ++i)
              P.weight[h][lf][i] = 0.0;
        for (int h = 0; h < 2; ++h)
          for (int lf = 0; lf <= coarse.p; ++lf)
            {
              const long double xi = 0.5L * h + 0.5L * (long double)b.nodes[lf];
              for (int i = 0; i <= coarse.p; ++i)
                {
                  long double w = 1.0L;
                  for (int j = 0; j <= coarse.p; ++j)
                    if (j != i)
                      w *= (xi - (long double)b.nodes[j]) /
                           ((long double)b.nodes[i] - (long double)b.nodes[j]);
                  P.weight[h][lf][i] = double(w);
                }
            }
        P.mask_input  = d == 0;
        P.mask_output = d == 2;
        for (int f = 0; f < 6; ++f)
          {
            P.in_face_mask[f]  = coarse.face_mask[f];
            P.out_face_mask[f] = fine.face_mask[f];
          }
        const size_t total = size_t(P.ext_out[0]) * P.ext_out[1] * P.ext_out[2] * nc;
        const unsigned grid = unsigned(
          std::min<size_t>(std::max<size_t>((total + 255) / 256, 1), size_t(n_sm) * 8));
        k_prolongate_pass_noalloc<T><<<grid, 256, 0, stream>>>(P, cur, dsts[d]);
        count_launch();
        MF_CK(cudaGetLastError());
        cur    = dsts[d];
        ext[d] = fine.Nn[d];
      }
  }

  // device address of the static scratch on the current device and the
  // device's SM count (set-up on the first call per device)
  void *
  scratch_address(int &n_sm)
  {
    int dev = 0;
    MF_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES)
      throw Error(ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev])
      {
        void             *ptr = nullptr;
        const cudaError_t rc  = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (rc != cudaSuccess || !ptr)
          throw Error(ERR_CUDA, std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                                  cudaGetErrorString(rc));
        int sms = 0;
        MF_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        g_sm_count[dev]     = sms > 0 ? sms : 1;
        g_scratch_addr[dev] = ptr;
      }
    n_sm = g_sm_count[dev];
    return g_scratch_addr[dev];
  }
} // namespace

extern "C" int
mfgpu_transfer_prolongate_noalloc(const mfgpu_mesh *mesh, int coarse_level,
                                  int n_components, int precision,
                                  const void *coarse, void *fine, void *stream)
{
  try
    {
      if (!mesh || !coarse || !fine)
        throw Error(ERR_ARG, "null argument");
      if (precision != 32 && precision != 64)
        throw Error(ERR_ARG, "precision must be 32 or 64");
      if (n_components < 1 || n_components > 3)
        throw Error(ERR_ARG, "n_components must be 1..3");
      const Mesh m = to_mesh(*mesh);
      if (coarse_level < 0 || coarse_level + 1 > m.n_ref)
        throw Error(ERR_ARG, "coarse_level must be in [0, n_refinements)");
      const LevelGeom cg = m.level(coarse_level), fg = m.level(coarse_level + 1);
      // intermediate sizes (elements, all components) of the x and y passes
      const size_t es = precision == 32 ? 4 : 8;
      const size_t i0 = size_t(fg.Nn[0]) * cg.Nn[1] * cg.Nn[2] * n_components;
      const size_t i1 = size_t(fg.Nn[0]) * fg.Nn[1] * cg.Nn[2] * n_components;
      const size_t cap = HALF_BYTES / es;
      if (i0 > cap || i1 > cap)
        throw Error(ERR_ARG, "level too large for the static scratch: the passes need " +
                               std::to_string(std::max(i0, i1)) + " elements per intermediate, the " +
                               "scratch holds " + std::to_string(cap));
      HostBasis b;
      make_host_basis(m.degree, b);
      int            n_sm = 1;
      unsigned char *base = static_cast<unsigned char *>(scratch_address(n_sm));
      cudaStream_t   s    = static_cast<cudaStream_t>(stream);
      if (precision == 32)
        run_passes<float>(cg, fg, n_components, b, static_cast<const float *>(coarse),
                          static_cast<float *>(fine), reinterpret_cast<float *>(base),
                          reinterpret_cast<float *>(base + HALF_BYTES), n_sm, s);
      else
        run_passes<double>(cg, fg, n_components, b, static_cast<const double *>(coarse),
                           static_cast<double *>(fine), reinterpret_cast<double *>(base),
                           reinterpret_cast<double *>(base + HALF_BYTES), n_sm, s);
      return MFGPU_OK;
    }
  catch (const Error &e)
    {
      set_last_error(e.what());
      return e.code;
    }
  catch (...)
    {
      set_last_error("unknown exception");
      return MFGPU_ERR_ARG;
    }
}
