// Internal host-side classes of the library (behind the C-ABI of mfgpu.h).
#pragma once

#include <cuda_runtime.h>

#include <chrono>

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "mf_launch.h"

namespace mfgpu
{
  // exception carrying a C-ABI status
  struct Error : std::runtime_error
  {
    int code;
    Error(int c, const std::string &m)
      : std::runtime_error(m)
      , code(c)
    {}
  };

  void check_cuda(cudaError_t e, const char *what);
#define MF_CK(x) ::mfgpu::check_cuda((x), #x)

  // message returned by mfgpu_last_error() on the calling thread
  void set_last_error(const char *msg);

  void count_launch(int n = 1);
  long long launch_count();

  // owning device buffer
  struct DevBuf
  {
    void  *ptr   = nullptr;
    size_t bytes = 0;
    DevBuf()     = default;
    explicit DevBuf(size_t b) { alloc(b); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept
      : ptr(o.ptr)
      , bytes(o.bytes)
    {
      o.ptr   = nullptr;
      o.bytes = 0;
    }
    DevBuf &
    operator=(DevBuf &&o) noexcept
    {
      release();
      ptr     = o.ptr;
      bytes   = o.bytes;
      o.ptr   = nullptr;
      o.bytes = 0;
      return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t b);
    // allocate b bytes unless the buffer already has exactly that size
    void ensure(size_t b)
    {
      if (bytes != b || (b != 0 && !ptr))
        alloc(b);
    }
    void release();
    template <typename T>
    T *
    as() const
    {
      return static_cast<T *>(ptr);
    }
  };

  struct Context
  {
    int          device = 0;
    int          n_sm   = 1; // multiprocessors of the device
    cudaStream_t stream = nullptr;
    DevBuf       err;      // int error flags
    DevBuf       ticket;   // unsigned: block counter of the single-launch reductions
    DevBuf       partial;  // reduction partials
    DevBuf       scalars;  // device scalars (double[32])
    double      *host_scalars = nullptr; // pinned
    explicit Context(int dev);
    ~Context();
    // error flags set by kernels since the last call (and reset)
    int  take_error_flags();
    void sync();
  };

  // pinned host array of doubles (move-only), grown on demand
  struct HostPinned
  {
    double *p = nullptr;
    size_t  n = 0;
    HostPinned() = default;
    HostPinned(const HostPinned &) = delete;
    HostPinned &operator=(const HostPinned &) = delete;
    HostPinned(HostPinned &&o) noexcept
      : p(o.p)
      , n(o.n)
    {
      o.p = nullptr;
      o.n = 0;
    }
    HostPinned &
    operator=(HostPinned &&o) noexcept
    {
      std::swap(p, o.p);
      std::swap(n, o.n);
      return *this;
    }
    ~HostPinned()
    {
      if (p)
        cudaFreeHost(p);
    }
    void
    ensure(size_t count)
    {
      if (count <= n)
        return;
      if (p)
        cudaFreeHost(p);
      p = nullptr;
      n = 0;
      if (cudaMallocHost(&p, count * sizeof(double)) != cudaSuccess)
        {
          p = nullptr;
          (void)cudaGetLastError();
          throw std::runtime_error("cudaMallocHost failed");
        }
      n = count;
    }
  };

  // Wall-clock sections of a driver, as the reference's TimerOutput with
  // wall_times (mf_elasticity.h:219,431-432; heat_transfer.h:381,405).
  // With timing enabled a section synchronises the context's stream when it
  // opens and when it closes, so that the device work a section issues is
  // charged to it; disabled, a section costs nothing.
  struct PhaseTimer
  {
    bool                                  enabled = false;
    std::vector<std::string>              names;
    std::vector<double>                   secs;
    std::vector<long>                     calls;
    std::chrono::steady_clock::time_point start = std::chrono::steady_clock::now();
    void                                  reset();
    int                                   index(const char *name);
    // the table of sections (calls, wall time, share of the time since
    // reset), in the order the sections first opened
    std::string summary() const;

    class Scope
    {
    public:
      Scope(PhaseTimer &t, Context *c, const char *name);
      ~Scope();
      Scope(const Scope &)            = delete;
      Scope &operator=(const Scope &) = delete;

    private:
      PhaseTimer                           *t_;
      Context                              *c_;
      int                                   i_ = -1;
      std::chrono::steady_clock::time_point t0_;
    };
  };

  // geometry of one level of the box hierarchy
  struct Mesh
  {
    int      dim = 3;
    int      degree, n_q, n_ref;
    int      rep[3];
    double   lo[3], hi[3];
    int      boundary_id[6];
    int      n_dirichlet;
    int      dirichlet_id[8];
    unsigned dirichlet_mask[8];
    LevelGeom level(int l) const; // l < 0: finest
    int       finest() const { return n_ref; }
  };

  // ---------------------------------------------------------------------
  // vector kernels (instantiated for float and double)
  // ---------------------------------------------------------------------
  template <typename T> void vec_fill(Context &c, size_t n, T v, T *x);
  // x[i] = (i % 11 == 0 ? 0 : 1) - mean of those values: the start vector of
  // the Chebyshev eigenvalue estimate (high-frequency content and the
  // constant mode)
  // the eigenvalue estimate's start vector; period > 0: the pattern repeats
  // every `period` entries (the blocks of a batch start alike)
  template <typename T> void vec_estimate_start(Context &c, size_t n, T *x, size_t period = 0);
  template <typename T> void vec_axpby(Context &c, size_t n, T a, const T *x, T b, T *y);
  template <typename T> void vec_axpbyz(Context &c, size_t n, T a, const T *x, T b, const T *y, T *z);
  template <typename T> void vec_copy(Context &c, size_t n, const T *x, T *y);
  template <typename TD, typename TS> void vec_convert(Context &c, size_t n, const TS *s, TD *d);
  template <typename T> void vec_scale(Context &c, size_t n, T omega, const T *d, const T *x, T *y);
  template <typename T> void vec_invert(Context &c, size_t n, T *x);
  // dot product into device scalar slot (deterministic)
  template <typename T> void vec_dot_dev(Context &c, size_t n, const T *x, const T *y, int slot);
  template <typename T> double vec_dot(Context &c, size_t n, const T *x, const T *y);
  template <typename T> void cg_update(Context &c, size_t n, int num_slot, int den_slot, T *x, const T *p, T *r, const T *q, int rr_slot);
  template <typename T> void cg_direction(Context &c, size_t n, int num_slot, int den_slot, const T *z, T *p);
  // Jacobi-preconditioned CG, fused: x += a p, r -= a q, z = dinv r, |r|^2
  // and r.z into two slots (one launch)
  template <typename T>
  void cg_update_jacobi(Context &c, size_t n, int num_slot, int den_slot, T *x, const T *p, T *r, const T *q,
                        const T *dinv, T *z, int rr_slot, int rz_slot);
  // p = z + (s[rzn]/s[rz]) p, q_zero = 0 (if given), and the Lanczos record
  // of lanczos_record (one launch)
  template <typename T>
  void cg_direction_rec(Context &c, size_t n, int rz, int rzn, int pq, int rr, const T *z, T *p, T *q_zero,
                        double *rec, int *counter);
  // rec[3k..3k+2] = (slots[rz]/slots[pq], slots[rr], slots[rzn]/slots[rz]),
  // k = (*counter)++ on the device
  void lanczos_record(Context &c, int rz, int rzn, int pq, int rr, double *rec, int *counter);
  template <typename T> void cheby_start(Context &c, size_t n, T f, const T *b, const T *dinv, T *x, T *xold);
  // (zero_ax: Ax is left zero)
  template <typename T>
  void cheby_update(Context &c, size_t n, T f1, T f2, bool first, bool zero_ax, const T *b, T *Ax, const T *dinv,
                    T *x, T *xold);
  // constrained rows: op 0 dst=src, 1 dst+=src, 2 dst=0, 3 dst=1, 4 (dst a
  // dense nc n_nodes square matrix of row stride ld, 0: nc n_nodes) unit
  // diagonal entry
  template <typename T>
  void constrained_op(Context &c, const LevelGeom &g, int nc, int op, const T *src, T *dst, size_t ld = 0);
  // dense row-major n x n operators in precision 32 (float) or 64 (double),
  // row stride ld = dense_row_stride(n), the entries past column n zero
  size_t dense_row_stride(size_t n);
  void   dense_mv(Context &c, int precision, size_t n, const void *A, const void *x, void *y, bool add);
  void   dense_constrained_identity(Context &c, int precision, const LevelGeom &g, int nc, void *A);
  // one Chebyshev step x_new = x + f1 (x - xo) + f2 dinv (b - A x) (first:
  // x_new = (1 + f1) x + f2 dinv (b - A x)) into xo
  template <typename T>
  void cheby_dense_step(Context &c, size_t n, const T *A, T f1, T f2, bool first, const T *b, const T *dinv,
                        const T *x, T *xo);
  double *scalar_slots(Context &c); // device pointer to the scalars
  void    read_scalars(Context &c, int n); // D2H of the first n slots (sync)

  // ---------------------------------------------------------------------
  // streams and events of the overlapped host-buffer vmult (created on
  // first use, on the operator's device)
  // ---------------------------------------------------------------------
  struct HostPipe
  {
    static constexpr int MAXC = 8;
    cudaStream_t         s_in = nullptr, s_out = nullptr, s_comp[MAXC] = {};
    cudaEvent_t          e_zero = nullptr, e_con = nullptr, e_done = nullptr;
    cudaEvent_t          e_in[MAXC] = {}, e_comp[MAXC] = {};
    int                  chunks = 0; // 0: chosen from the vector size
    // what a captured graph was built for: buffers, slab count, operator state
    struct Key
    {
      void       *dst_h = nullptr, *dst_d = nullptr;
      const void *src_h = nullptr, *src_d = nullptr;
      int         n     = 0;
      size_t      state = 0;
      bool
      operator==(const Key &o) const
      {
        return dst_h == o.dst_h && src_h == o.src_h && dst_d == o.dst_d && src_d == o.src_d &&
               n == o.n && state == o.state && n > 0;
      }
    };
    Key             last, g;
    cudaGraphExec_t gexec      = nullptr;
    long long       g_launches = 0;
    void            init();
    void            drop_graph();
    ~HostPipe();
  };

  // ---------------------------------------------------------------------
  // operators
  // ---------------------------------------------------------------------
  struct Operator
  {
    Context  *ctx = nullptr;
    Mesh      mesh;
    int       level = -1;
    LevelGeom geom;
    HostBasis basis;
    int       precision   = 64;
    int       nc          = 1;
    bool      constrained = true;
    int       arith       = 0; // 0 native, 1 double-float (FP64 operators only)
    int       scatter     = 0; // 0 atomic adds, 1 parity colours with plain adds (deterministic)
    int       cell_kernel = 0; // 0 by grid size, 1 line-parallel, 2 point-parallel (ApplyArgs::kernel),
                               // 3 element matrix on the tensor cores (FP32 heat, degree <= 5),
                               // 4 tensor-product form (heat; 0 takes it where supported), 5 the
                               // same with FP32 Q1-Q2 bricks staged by TMA
    DevBuf    inv_diag;
    DevBuf    diag;
    bool      diag_ready = false;
    // heat operators of a batch of problems (make_heat(..., batch)): nc is
    // the number of problems, each a scalar field of n_nodes entries
    bool      heat_batch = false;
    virtual ~Operator() = default;
    size_t
    m() const
    {
      return size_t(nc) * geom.n_nodes;
    }
    size_t
    elem_size() const
    {
      return precision == 32 ? 4 : 8;
    }
    // dst += A src; constrained rows (constrained operators): dst += src
    void apply_cells(void *dst, const void *src) { apply_cells_range(dst, src, 0, 0, ctx->stream); }
    // the same for the cells [c0, c1) (all cells if c1 <= c0) on stream s;
    // a constrained row is added by the launch that contains its owner cell
    // (kernel >= 0: this launch's cell kernel instead of cell_kernel)
    void apply_cells_range(void *dst, const void *src, size_t c0, size_t c1, cudaStream_t s, int kernel = -1);
    // the kernel arguments of the operator (no vectors, all cells); checks
    // that the operator is ready to apply
    virtual ApplyArgs cell_args() const = 0;
    virtual void      compute_diagonal() = 0;
    // Dense copy of a small operator (at most DENSE_MAX_BYTES): the entries
    // of A assembled from element columns (one launch), constrained rows
    // and columns as the identity, rows dense_row_stride(m()) apart.  vmult /
    // vmult_add multiply by it while value_state() is what it was at
    // assembly.
    static constexpr size_t DENSE_MAX_BYTES = size_t(64) << 20;
    DevBuf                  dense;
    size_t                  dense_key = 0;
    bool                    dense_on  = false;
    bool                    dense_fits() const;
    void                    assemble_dense();
    void                    drop_dense();
    bool                    use_dense() const { return dense_on && dense.ptr && dense_key == value_state(); }
    // vmult_state() plus the cached quadrature data's generation
    virtual size_t value_state() const { return vmult_state(); }
    virtual size_t memory_consumption() const { return 0; }
    virtual void clear() {}
    void vmult(void *dst, const void *src);
    void vmult_add(void *dst, const void *src);
    // dst_h = A src_h for host vectors, through the device buffers dst_d /
    // src_d: the source is copied in z-slabs, each slab of cells starts as
    // soon as its nodes have arrived, and each slab of the result is copied
    // back as soon as the cells touching it are done.  Synchronous.
    void vmult_host(void *dst_h, const void *src_h, void *dst_d, void *src_d, HostPipe &p);
    // everything a vmult's kernels take as parameters (a captured graph of
    // the host-buffer vmult is replayed only while this is unchanged)
    virtual size_t vmult_state() const;
  private:
    void enqueue_vmult_host(void *dst_h, const void *src_h, void *dst_d, void *src_d, HostPipe &p, int n);
  public:
    void finish_diagonal(); // constrained -> 1, invert
    // kernel launches of one application of the cells [c0, c1) (all if c1 <= c0)
    int cell_launches(size_t c0, size_t c1) const;
    // 2D meshes: FP32/FP64 arithmetic and the atomic scatter only
    void check_2d() const;
  };

  struct HeatOperator : Operator
  {
    double    delta_t     = 0;
    double    coefficient = 1;
    // the element matrix in the tensor-core kernel's layout (mf_heat_em.cu),
    // for the vmult_state() it was built for
    DevBuf    em_mat;
    size_t    em_key = 0;
    const void *element_matrix();
    ApplyArgs cell_args() const override;
    void      compute_diagonal() override;
    size_t    vmult_state() const override;
  };

  struct NHOperator : Operator
  {
    int        variant = 0; // NHVariant
    NHMatD     mat{};
    int        formulation = 1;
    bool       have_material = false;
    const void *u      = nullptr; // linearisation (not owned)
    DevBuf      cache;
    DevBuf      ucell;
    bool        cached    = false;
    size_t      cache_gen = 0; // incremented by every do_cache()
    ApplyArgs cell_args() const override;
    void      compute_diagonal() override;
    size_t    vmult_state() const override;
    size_t    value_state() const override;
    void   do_cache();
    size_t memory_consumption() const override { return cache.bytes + ucell.bytes; }
    void   clear() override;
  };

  int  parse_caching(const char *s);
  NHMatD make_material(double mu, double nu, double rho, double alpha_1);
  // batch > 1: one operator applied to `batch` problems on the same level
  // (vectors of batch blocks of n_nodes entries; one launch per application);
  // the Dirichlet bits of every face mask cover all blocks
  std::unique_ptr<HeatOperator> make_heat(Context *c, const Mesh &m, int level, int precision, bool constrained,
                                          int batch = 1);
  std::unique_ptr<NHOperator>   make_nh(Context *c, const Mesh &m, int level, int precision, int variant);

  // ---------------------------------------------------------------------
  // transfer between level l and l+1 (tensor product of 1D operators)
  // ---------------------------------------------------------------------
  struct Transfer
  {
    Context  *ctx = nullptr;
    LevelGeom coarse, fine;
    int       nc = 1, precision = 64;
    // per direction: prolongation (fine rows), restriction = P^T (coarse
    // rows), interpolation (coarse rows); banded gather lists
    struct Band
    {
      DevBuf col, val;
      int    rows = 0, width = 0;
    };
    Band   P[3], R[3], I[3];
    DevBuf tmp0, tmp1;
    Transfer(Context *c, const HostBasis &b, const LevelGeom &cg, const LevelGeom &fg, int nc, int precision);
    void prolongate(void *fine_v, const void *coarse_v);        // fine = P coarse
    void prolongate_add(void *fine_v, const void *coarse_v);    // fine += P coarse
    void restrict_add(void *coarse_v, const void *fine_v);      // coarse += P^T fine
    void interpolate(void *coarse_v, const void *fine_v);       // coarse = I fine
  private:
    void passes(const Band *B, const LevelGeom &from, const LevelGeom &to, const void *in, void *out,
                bool constrained = false, bool add = false);
  };
} // namespace mfgpu
