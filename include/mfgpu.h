/*
 * mfgpu.h — C-ABI of the GB300 matrix-free library (libmfgpu.so).
 *
 * A drop-in for the reference's CPU MatrixFree path
 * (davidscn/matrix-free-dealii-precice): the neo-Hookean tangent operator
 * (NeoHookOperator, include/solid_mechanics/mf_nh_operator.h:103-173), the
 * backward-Euler heat operator (LaplaceOperator,
 * include/heat_transfer/heat_transfer.h:81-127), the Chebyshev-smoothed
 * geometric multigrid V-cycle with its transfers, the CG solver and the
 * Newton-Newmark / backward-Euler drivers.
 *
 * Conventions
 *   - Every function returns an int status: MFGPU_OK (0) or an error code;
 *     mfgpu_last_error() returns a message for the calling thread.
 *   - Vectors are device pointers (double* for precision 64, float* for 32)
 *     of length m() = n_components * n_nodes, component-blocked:
 *     dof = component * n_nodes + node, nodes numbered lexicographically
 *     (x fastest) on the Q_p Gauss-Lobatto node grid of the level.
 *   - Meshes are boxes [lower, upper] with repetitions[d] coarse cells per
 *     direction, refined n_refinements times (subdivided_hyper_rectangle +
 *     refine_global, as the reference's cases build them); level L has
 *     repetitions[d] * 2^L cells per direction; level -1 means the finest.
 *   - Box faces are numbered x-, x+, y-, y+, z-, z+ (deal.II colorize
 *     numbering); boundary_id[f] gives each face's boundary id and the
 *     Dirichlet list maps boundary ids to component masks.
 *   - Objects are bound to the CUDA stream of their context; they are
 *     thread-compatible (one thread per object at a time).
 */
#ifndef MFGPU_H
#define MFGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MFGPU_OK 0
#define MFGPU_ERR_ARG 1
#define MFGPU_ERR_CUDA 2
#define MFGPU_ERR_OOM 3
#define MFGPU_ERR_NONFINITE 4
#define MFGPU_ERR_NOT_CONVERGED 5
#define MFGPU_ERR_STATE 6
#define MFGPU_ERR_DET_F 7
#define MFGPU_ERR_UNSUPPORTED 8
#define MFGPU_ERR_TIMEOUT 9

typedef struct mfgpu_context mfgpu_context;
typedef struct mfgpu_operator mfgpu_operator;
typedef struct mfgpu_mg mfgpu_mg;
typedef struct mfgpu_solid mfgpu_solid;
typedef struct mfgpu_heat mfgpu_heat;

typedef struct mfgpu_mesh
{
  int      degree;         /* FE_Q degree p, 1..6                    */
  int      n_q_1d;         /* Gauss points per direction (== p + 1)  */
  int      n_refinements;  /* global refinements of the coarse box   */
  int      repetitions[3]; /* coarse cells per direction             */
  double   lower[3];
  double   upper[3];
  int      boundary_id[6];    /* per box face x-,x+,y-,y+,z-,z+      */
  int      n_dirichlet;       /* entries used in the two lists below */
  int      dirichlet_id[8];   /* boundary ids with Dirichlet data     */
  unsigned dirichlet_mask[8]; /* component mask per boundary id       */
  int      dim;               /* 2 or 3 (0 means 3); in 2D the z
                                 entries and faces z-, z+ are unused  */
} mfgpu_mesh;

/* Material_Compressible_Neo_Hook_One_Field(mu, nu, rho, alpha_1,
 * formulation), include/solid_mechanics/material.h:78-94 */
typedef struct mfgpu_material
{
  double mu;
  double nu;
  double rho;
  double alpha_1; /* 1 / (beta dt^2) of the Newmark scheme */
  int    formulation;
} mfgpu_material;

/* ---------------------------------------------------------------- */
/* library / context                                                 */
/* ---------------------------------------------------------------- */
const char *mfgpu_last_error(void);
int         mfgpu_version(void);
/* number of kernel launches issued by this process so far */
long long mfgpu_launch_count(void);

/* context: one CUDA device + one stream + reduction scratch */
int mfgpu_context_create(int device, mfgpu_context **ctx);
/* fails with MFGPU_ERR_STATE while operators, solid or heat drivers created
 * on the context are alive: destroy those first */
int mfgpu_context_destroy(mfgpu_context *ctx);
int mfgpu_context_synchronize(mfgpu_context *ctx);
/* the cudaStream_t of the context, as void* */
int mfgpu_context_stream(mfgpu_context *ctx, void **stream);

/* copy bytes between any two host/device buffers on the context's stream
 * (unified addressing), then synchronize the stream */
int mfgpu_copy(mfgpu_context *ctx, void *dst, const void *src, size_t bytes);

/* number of nodes of a level (dofs = n_components * nodes) */
int mfgpu_mesh_n_nodes(const mfgpu_mesh *mesh, int level, size_t *n_nodes);

/* ---------------------------------------------------------------- */
/* operators                                                         */
/* ---------------------------------------------------------------- */

/* LaplaceOperator<3,number>: MatrixFreeOperators::Base API
 * (heat_transfer.h:81-127).  constrained = 0 builds the operator without
 * constraints (the reference's inhomogeneous_operator, heat_transfer.h:484-495). */
int mfgpu_heat_operator_create(mfgpu_context *ctx, const mfgpu_mesh *mesh,
                               int level, int precision, int constrained,
                               mfgpu_operator **op);
/* LaplaceOperator::set_delta_t (heat_transfer.h:101-105) */
int mfgpu_heat_operator_set_delta_t(mfgpu_operator *op, double delta_t);
/* LaplaceOperator::evaluate_coefficient (heat_transfer.h:150-166) with the
 * reference's constant Coefficient (heat_transfer.h:63-71) */
int mfgpu_heat_operator_evaluate_coefficient(mfgpu_operator *op,
                                             double coefficient);

/* NeoHookOperator<3,Number> (mf_nh_operator.h:103-173).  caching is one of
 * "scalar_referential", "tensor2", "tensor4", "tensor4_ns" (the reference's
 * MF caching options, parameter_handling.h:231-235) or "referential_qp",
 * a referential cache of F^{-T} and mu - 2 lambda ln J per quadrature point. */
int mfgpu_nh_operator_create(mfgpu_context *ctx, const mfgpu_mesh *mesh,
                             int level, int precision, const char *caching,
                             mfgpu_operator **op);
/* NeoHookOperator::set_material (mf_nh_operator.h:529-539): `material`
 * applies to cells of material id 0, `inclusion` (may be NULL; the
 * reference passes mu x 100, mf_elasticity.h:470-493) to the others
 * (mf_nh_operator.h:402-404,656-658).  Box meshes carry material id 0 on
 * every cell, as all of the reference's cases do, so the inclusion is
 * stored and checked (same formulation) but applies to no cell. */
int mfgpu_nh_operator_set_material(mfgpu_operator *op,
                                   const mfgpu_material *material,
                                   const mfgpu_material *inclusion);
/* Material ids of the level's cells (n_cells bytes, cells numbered
 * lexicographically, x fastest), as cell->material_id() gives them.  All
 * zero is accepted (the default); a cell with a nonzero id, i.e. the
 * inclusion material, returns MFGPU_ERR_UNSUPPORTED: the device cell
 * kernels apply one material to every cell. */
int mfgpu_nh_operator_set_cell_material_ids(mfgpu_operator *op,
                                            const unsigned char *ids,
                                            size_t n_cells);
/* NeoHookOperator::initialize (mf_nh_operator.h:333-388): registers the
 * linearisation displacement (device pointer of the operator's precision,
 * NOT owned; keep it alive while the operator is used) */
int mfgpu_nh_operator_initialize(mfgpu_operator *op, const void *displacement);
/* NeoHookOperator::cache (mf_nh_operator.h:394-523); MFGPU_ERR_DET_F if
 * det F <= 0 at a quadrature point */
int mfgpu_nh_operator_cache(mfgpu_operator *op);

/* Arithmetic of an FP64 operator: 0 native FP64 (default), 1 double-float
 * (each FP64 value carried as an unevaluated sum of two floats on the FP32
 * pipe, ~48 significant bits; the result agrees with native FP64 to ~1e-14
 * relative).  Supported for heat operators and the referential_qp tangent
 * (formulation 1); the neo-Hookean operator must be cache()d again after a
 * change.  No counterpart in the reference (its path is native FP64). */
int mfgpu_operator_set_fp64_emulation(mfgpu_operator *op, int enable);

/* vmult / vmult_add / Tvmult / Tvmult_add (mf_nh_operator.h:545-625 and
 * MatrixFreeOperators::Base::vmult): dst = A src with constrained rows
 * dst = src */
int mfgpu_operator_vmult(mfgpu_operator *op, void *dst, const void *src);
int mfgpu_operator_vmult_add(mfgpu_operator *op, void *dst, const void *src);
int mfgpu_operator_Tvmult(mfgpu_operator *op, void *dst, const void *src);
int mfgpu_operator_Tvmult_add(mfgpu_operator *op, void *dst, const void *src);
/* vmult with HOST buffers (pinned for overlap): the source is copied in
 * z-slabs, the cells of each slab start when their nodes have arrived and
 * each slab of the result is copied out when the cells touching it are
 * done; returns when dst_host holds the result */
int mfgpu_operator_vmult_host(mfgpu_operator *op, void *dst_host,
                              const void *src_host);
/* scatter of the cell contributions: 0 = atomic adds (default), 1 = cells
 * in 8 parity colours, one launch per colour with plain adds (results are
 * bitwise reproducible from run to run, as the reference's CPU loop is).
 * No counterpart in the reference (its CPU cell loop needs neither). */
int mfgpu_operator_set_scatter(mfgpu_operator *op, int mode);

/* number of z-slabs of the host-buffer vmult: 0 = from the vector size
 * (4 from 4 MB up), 1 = copy in, apply, copy out without overlap, <= 8.
 * No counterpart in the reference (its vectors live in host memory). */
int mfgpu_operator_set_host_chunks(mfgpu_operator *op, int n_chunks);
/* Dense copy of a small operator (three-dimensional, constrained, at most
 * 64 MiB): enable = 1 assembles A from the current state (cache(),
 * set_delta_t() first) and vmult / vmult_add multiply by it until the state
 * changes; 0 frees it.  The coarse-level counterpart of deal.II's assembled
 * coarse matrices; the solvers use it on level 0 (coarse_dense). */
int mfgpu_operator_set_dense(mfgpu_operator *op, int enable);
/* cell kernel of vmult: 0 by grid size (default: point-parallel, one
 * thread per quadrature point, below 1024 cells, up to 4096 in native
 * FP64, at every size for the native FP64 referential_qp tangent except
 * degree 2; line-parallel above; three-dimensional heat operators in FP32 and
 * native FP64, and in double-float up to degree 5, take kernel 4 from 512
 * cells on), 1 line-parallel,
 * 2 point-parallel, 3 tensor cores (three-dimensional FP32 heat
 * operators, degree 1..5: the cells' common element matrix applied to
 * batches of 128 cells by tcgen05.mma in TF32 with a three-term split,
 * FP32 accuracy), 4 tensor product (three-dimensional heat operators in
 * FP32, native FP64 or double-float, the default for double-float up to
 * degree 5: the element operator as sums of products of the 1D
 * mass and stiffness matrices, exact for the QGauss(p+1) integral on the
 * level's affine cells, 7 sweeps per cell; one thread per cell in
 * registers at degree 1 on levels of 16384 cells or more, (p+1)^2
 * threads per cell through shared memory otherwise), 5 the tensor product
 * with the cells' nodes staged in shared memory by TMA row copies and the
 * results added back by TMA bulk reductions (FP32, degree 1..2, 16-byte
 * aligned vectors; measured slower than 4, other cases take 4).  The
 * results agree to round-off. */
int mfgpu_operator_set_cell_kernel(mfgpu_operator *op, int mode);
/* compute_diagonal (mf_nh_operator.h:1025-1060, heat_transfer.h:205-230) */
int mfgpu_operator_compute_diagonal(mfgpu_operator *op);
/* get_matrix_diagonal_inverse: device pointer owned by the operator */
int mfgpu_operator_get_matrix_diagonal_inverse(mfgpu_operator *op,
                                               const void **inv_diag);
/* el(row, col): diagonal entries only (mf_nh_operator.h:1066-1073) */
int mfgpu_operator_el(mfgpu_operator *op, size_t row, size_t col,
                      double *value);
/* precondition_Jacobi (mf_nh_operator.h:283-291): dst = omega D^{-1} src */
int mfgpu_operator_precondition_jacobi(mfgpu_operator *op, void *dst,
                                       const void *src, double omega);
/* m(), n() */
int mfgpu_operator_m(mfgpu_operator *op, size_t *m);
/* memory_consumption (mf_nh_operator.h:243-260): cache bytes */
int mfgpu_operator_memory_consumption(mfgpu_operator *op, size_t *bytes);
/* clear (mf_nh_operator.h:315-327) */
int mfgpu_operator_clear(mfgpu_operator *op);
int mfgpu_operator_destroy(mfgpu_operator *op);

/* ---------------------------------------------------------------- */
/* multigrid transfer between level and level+1 (MGTransferMatrixFree) */
/* ---------------------------------------------------------------- */
/* fine = P coarse */
int mfgpu_transfer_prolongate(mfgpu_context *ctx, const mfgpu_mesh *mesh,
                              int coarse_level, int n_components,
                              int precision, const void *coarse, void *fine);
/* coarse += P^T fine */
int mfgpu_transfer_restrict_add(mfgpu_context *ctx, const mfgpu_mesh *mesh,
                                int coarse_level, int n_components,
                                int precision, void *coarse, const void *fine);
/* coarse = fine field evaluated at the coarse nodes (interpolate_to_mg) */
int mfgpu_transfer_interpolate(mfgpu_context *ctx, const mfgpu_mesh *mesh,
                               int coarse_level, int n_components,
                               int precision, void *coarse, const void *fine);

/* fine = P coarse without allocating any device memory: the same
 * prolongation as mfgpu_transfer_prolongate, for callers that may not
 * allocate device memory while they run.  Examples: a coupled solver whose
 * partner code's pool already holds the GPU memory, a time loop that must
 * not stall on cudaMalloc/cudaFree, a deployment that forbids allocation
 * after start-up.  No counterpart in the reference (deal.II's transfer
 * allocates its own vectors).  The two intermediate arrays live in a
 * static 4 MiB device array that every GPU loading the library keeps until
 * exit, so each intermediate (fine-x by coarse-y,z, then fine-x,y by
 * coarse-z, times n_components) may hold at most 262,144 doubles or 524,288
 * floats; larger levels return MFGPU_ERR_ARG.  Three- and two-dimensional
 * meshes (dim = 2: the single z node plane is copied through).  Needs no context: it runs
 * on `stream` (a cudaStream_t, NULL for the default stream) of the current
 * device and returns without synchronising.  The first call on a device
 * looks up the array's device address, so make it before any stream
 * capture.  Every call shares the array and nothing in it has to start at
 * zero; calls that overlap on the GPU race on it, so serialise them. */
int mfgpu_transfer_prolongate_noalloc(const mfgpu_mesh *mesh, int coarse_level,
                                      int n_components, int precision,
                                      const void *coarse, void *fine,
                                      void *stream);

/* ---------------------------------------------------------------- */
/* geometric multigrid preconditioner and CG                         */
/* ---------------------------------------------------------------- */
/* parameters of the linear solvers: CG, its preconditioner and the
 * multigrid smoothers (the reference's "Linear solver" section,
 * parameter_handling.h:177-253) */
typedef struct mfgpu_solver_params
{
  int    preconditioner;  /* 0 none, 1 jacobi, 2 gmg                        */
  double relaxation;      /* Jacobi relaxation                              */
  double tol;             /* relative CG tolerance                          */
  int    max_it_mult;     /* max CG iterations = n_dofs * multiplier        */
  int    cheb_degree;     /* Chebyshev degree on levels > 0                 */
  double cheb_range;      /* smoothing range on levels > 0                  */
  int    cheb_eig_its;    /* CG iterations for the eigenvalue estimate      */
  int    coarse_accurate; /* level 0: eigenvalue CG iterations = m()        */
  int    mg_precision;    /* 32: FP32 level operators, 64: all-FP64 V-cycle */
  int    coarse_fp64;     /* level-0 Chebyshev solve in FP64                */
  int    fp64_emulation;  /* FP64 operators in double-float arithmetic      */
  int    cuda_graphs;     /* replay the V-cycle as a CUDA graph              */
  int    coarse_dense;    /* level-0 operator (three-dimensional, <= 64 MiB)
                             assembled densely after each setup; the coarse
                             Chebyshev steps multiply by it, one launch
                             per step */
  int    estimate_condition; /* "Estimate condition number": before each
                                linear solve of the solid, unpreconditioned
                                CG (Lanczos) estimates the condition number
                                (mf_elasticity.h:1998-2013); no effect on
                                the solution                                 */
  int    cond_cg_iterations; /* "Condition number CG iterations" (20)        */
} mfgpu_solver_params;

/* PreconditionMG<dim, VectorType, MGTransferMatrixFree> over the level
 * hierarchy of a box mesh, as Solid::setup_gmg (mf_elasticity.h:
 * 1142-1279) and LaplaceProblem::setup_gmg / solve_gmg_preconditioner
 * (heat_transfer.h:515-573, 759-812) build it: level operators in FP32
 * (mg_precision 32, the reference's) or FP64, MGTransferMatrixFree,
 * mg::SmootherRelaxation with PreconditionChebyshev on levels > 0 and the
 * Chebyshev solver on level 0 (MGCoarseGridApplySmoother). */
typedef struct mfgpu_mg_params
{
  int            kind;     /* 0 heat (LaplaceOperator levels, M + dt K),
                              1 neo-Hookean (NeoHookOperator levels)       */
  double         delta_t;  /* heat: the time step of the level operators    */
  const char    *caching;  /* neo-Hookean: MF caching of the level operators */
  mfgpu_material material; /* neo-Hookean: alpha_1 as for the fine operator  */
  mfgpu_solver_params solver; /* mg_precision, coarse_fp64, coarse_dense,
                                 cuda_graphs, fp64_emulation and, for the
                                 neo-Hookean levels, cheb_degree, cheb_range,
                                 cheb_eig_its, coarse_accurate (the heat
                                 levels use degree 5, range 15 and 10
                                 iterations, as the reference)              */
} mfgpu_mg_params;

int mfgpu_mg_create(mfgpu_context *ctx, const mfgpu_mesh *mesh,
                    const mfgpu_mg_params *params, mfgpu_mg **mg);
/* Solid::update_matrix_free's level part (mf_elasticity.h:1291-1353):
 * neo-Hookean levels interpolate the finest-level FP64 linearisation
 * (device pointer, read during the call only) to every level
 * (interpolate_to_mg), cache() and compute_diagonal() there; heat levels
 * (linearisation NULL) compute their diagonals once.  Then the Chebyshev
 * eigenvalue estimates (PreconditionChebyshev::initialize).  A setup with
 * unchanged level operators keeps the previous smoothers. */
int mfgpu_mg_setup(mfgpu_mg *mg, const double *linearisation);
/* PreconditionMG::vmult: dst = one V-cycle applied to src (finest-level
 * FP64 device vectors, dst != src) */
int mfgpu_mg_vmult(mfgpu_mg *mg, double *dst, const double *src);
/* number of levels and degrees of freedom of the finest one */
int mfgpu_mg_info(mfgpu_mg *mg, int *n_levels, size_t *n_dofs);
int mfgpu_mg_destroy(mfgpu_mg *mg);

/* SolverCG<Vector<double>>::solve(A, x, b, preconditioner) under
 * SolverControl(max_iterations, tol) (mf_elasticity.h:2015-2051,
 * heat_transfer.h:729-737, 811): x holds the initial guess and receives
 * the solution; stops when |r|_2 <= tol (absolute, as SolverControl).
 * The preconditioner is mg when non-NULL, else PreconditionJacobi with
 * relaxation jacobi_omega (> 0; compute_diagonal() of A first), else the
 * identity.  A is an FP64 operator on the same context as mg.  Returns
 * MFGPU_ERR_NOT_CONVERGED after max_iterations; iterations and residual
 * (may be NULL) receive solver_control.last_step() / last_value(). */
int mfgpu_pcg_solve(mfgpu_operator *A, mfgpu_mg *mg, double jacobi_omega,
                    double *x, const double *b, double tol,
                    int max_iterations, int *iterations, double *residual);
/* SolverCG::connect_condition_number_slot under IterationNumberControl
 * (mf_elasticity.h:1998-2013): n_iterations unpreconditioned CG iterations
 * on A y = b from y = 0 (fewer when |r| <= tol), then the ratio of the
 * extreme eigenvalues of the Lanczos tridiagonal matrix.  b is not
 * changed. */
int mfgpu_estimate_condition_number(mfgpu_operator *A, const double *b,
                                    int n_iterations, double tol,
                                    double *condition_number);

/* ---------------------------------------------------------------- */
/* DoF numbering: a caller's numbering <-> the library's              */
/* ---------------------------------------------------------------- */
/* deal.II numbers the DoFs of the reference's solid by DoFRenumbering::
 * Cuthill_McKee (mf_elasticity.h:669), the heat problem's in the
 * DoFHandler's default order; the library
 * numbers them component-blocked on the lexicographic node grid.  Given the
 * support point (x, y, z; z ignored in 2D) and the vector component of each
 * of the caller's n_dofs DoFs (DoFTools::map_dofs_to_support_points and
 * FiniteElement::system_to_component_index; components NULL means all 0),
 * library_dof[i] receives the library's index of the caller's DoF i.
 * Points must lie within tol (relative to the cell size) of a node of the
 * level; every library DoF must be hit exactly once (MFGPU_ERR_ARG
 * otherwise).  Host only. */
int mfgpu_dof_permutation(const mfgpu_mesh *mesh, int level, size_t n_dofs,
                          const double *support_points,
                          const unsigned *components, double tol,
                          size_t *library_dof);
/* the same map kept on the device, to move vectors between the numberings
 * on the context's stream: to_library dst[library_dof[i]] = src[i],
 * from_library dst[i] = src[library_dof[i]] (precision 32 or 64) */
typedef struct mfgpu_permutation mfgpu_permutation;
int mfgpu_permutation_create(mfgpu_context *ctx, const mfgpu_mesh *mesh,
                             int level, size_t n_dofs,
                             const double *support_points,
                             const unsigned *components, double tol,
                             mfgpu_permutation **perm);
int mfgpu_permutation_to_library(mfgpu_permutation *perm, int precision,
                                 const void *src, void *dst);
int mfgpu_permutation_from_library(mfgpu_permutation *perm, int precision,
                                   const void *src, void *dst);
int mfgpu_permutation_destroy(mfgpu_permutation *perm);

/* ---------------------------------------------------------------- */
/* drivers                                                           */
/* ---------------------------------------------------------------- */

typedef struct mfgpu_solid_params
{
  mfgpu_mesh          mesh;
  mfgpu_material      material; /* alpha_1 is set from dt */
  const char         *caching;
  mfgpu_solver_params solver;
  int                 max_newton;
  double              tol_f, tol_f_abs, tol_u, tol_u_abs;
  double              dt;
  int                 n_steps;
  double              body_force[3];
  int                 traction_id;
  double              traction[3];
  double              watch[3];
} mfgpu_solid_params;

typedef struct mfgpu_solid_result
{
  int    newton_its[64];
  double watch_disp[64][3];
  long   total_cg;
  int    n_solves;
  int    n_steps;
  double seconds;
} mfgpu_solid_result;

/* Solid<3,double>::run with the coupling replaced by a constant traction */
int mfgpu_solid_create(mfgpu_context *ctx, const mfgpu_solid_params *p,
                       mfgpu_solid **s);
int mfgpu_solid_run(mfgpu_solid *s, mfgpu_solid_result *r);
/* one time step of Solid::run from the current state (solve_nonlinear_
 * timestep, update_velocity and the watchpoint, mf_elasticity.h:576-613):
 * its Newton iterations, CG iterations and linear solves, and the
 * watchpoint displacement (any output pointer may be null) */
int mfgpu_solid_step(mfgpu_solid *s, int *newton_iterations, long *cg_iterations,
                     int *linear_solves, double *watch_displacement);
/* Newton residual (Solid::assemble_residual, mf_elasticity.h:1649-1908):
 * rhs = -int tau F^{-T} : Grad v + int rho (b - a) . v + traction term,
 * constrained rows zero; u, acceleration, rhs are device vectors */
int mfgpu_solid_residual(mfgpu_solid *s, const double *u,
                         const double *acceleration, double *rhs,
                         double *l2_norm);
/* final displacement (device pointer owned by the solver) */
int mfgpu_solid_displacement(mfgpu_solid *s, const double **u);
/* one linear system of the Newton loop: linearise at u (device), solve
 * K du = rhs (device) to tol * |rhs|; returns the CG iteration count */
int mfgpu_solid_linear_solve(mfgpu_solid *s, const double *u,
                             const double *rhs, double *du, int *iterations,
                             double *seconds);
/* Wall-clock sections of the driver, as the reference's TimerOutput
 * (mf_elasticity.h:219,431-432: "Assemble residual", "Linear solver",
 * "Setup MF: ..."). enable = 1 turns timing on and clears the table; each
 * section then synchronises the device at its start and end. */
int mfgpu_solid_set_timing(mfgpu_solid *s, int enable);
/* the section table as text: calls, wall time and share per section;
 * NUL-terminated, truncated to len bytes */
int mfgpu_solid_timing_summary(mfgpu_solid *s, char *buf, size_t len);
/* The convergence table of the last time step, as Solid::
 * solve_nonlinear_timestep prints it (mf_elasticity.h:1402-1491,1502-1515):
 * per Newton iteration LIN_IT, LIN_RES, COND_NUM (1 unless
 * estimate_condition), RES_NORM, RES_U, NU_NORM, NU_U; NUL-terminated,
 * truncated to len bytes */
int mfgpu_solid_convergence_table(mfgpu_solid *s, char *buf, size_t len);
int mfgpu_solid_destroy(mfgpu_solid *s);

typedef struct mfgpu_heat_params
{
  mfgpu_mesh          mesh;
  double              dt;
  int                 n_steps;
  mfgpu_solver_params solver;
  int                 analytic; /* 1: u = 1 + x^2 + alpha y^2 + beta t */
  double              alpha, beta;
  int                 n_gauss; /* source = sum of Gaussians */
  double              g_center[8][3];
  double              g_width[8];
  double              g_amp[8];
} mfgpu_heat_params;

typedef struct mfgpu_heat_result
{
  int    cg_its[64];
  int    n_steps;
  double seconds;
} mfgpu_heat_result;

/* LaplaceProblem<3>::run with the coupling replaced by Dirichlet data */
int mfgpu_heat_create(mfgpu_context *ctx, const mfgpu_heat_params *p,
                      mfgpu_heat **h);
int mfgpu_heat_run(mfgpu_heat *h, mfgpu_heat_result *r);
/* one backward-Euler step (the first call sets up the initial state);
 * returns the CG iterations of the step */
int mfgpu_heat_step(mfgpu_heat *h, int *cg_iterations);
int mfgpu_heat_solution(mfgpu_heat *h, const double **u);
/* sections of LaplaceProblem's TimerOutput (heat_transfer.h:381,581,717:
 * "assemble rhs", "solve system"; here also "GMG setup") */
int mfgpu_heat_set_timing(mfgpu_heat *h, int enable);
int mfgpu_heat_timing_summary(mfgpu_heat *h, char *buf, size_t len);
int mfgpu_heat_destroy(mfgpu_heat *h);

/* ---------------------------------------------------------------- */
/* request server: independent solves served concurrently            */
/* ---------------------------------------------------------------- */
/* No counterpart in the reference (one problem per MPI job there).
 * Requests queue FIFO; a request starts when a worker is free and its
 * estimated device memory fits in the budget (half of memory_fraction of
 * the free HBM at creation).  Every problem runs on its own CUDA stream,
 * so admitted solves overlap on the device; a solve keeps its hierarchy
 * resident until
 * it finishes, and afterwards in the server's pool of resident problems
 * (the other half of the budget, shared by the workers): a later request
 * of the same shape
 * (everything but its loads) reuses operators, multigrid setup and
 * buffers.  A free worker prefers, among the first 16 queued requests, one
 * whose shape is resident.  Results do not depend on what else runs
 * (deterministic reductions; scatter round-off only). */
typedef struct mfgpu_server mfgpu_server;

typedef struct mfgpu_request
{
  int                kind; /* 0 heat (uses `heat`), 1 solid (uses `solid`) */
  mfgpu_heat_params  heat;
  mfgpu_solid_params solid;
} mfgpu_request;

typedef struct mfgpu_request_result
{
  int    status; /* MFGPU_OK or the error of the solve */
  char   message[128];
  int    cg_iterations;
  int    newton_iterations;
  double watch[3];
  double solution_norm;
  double n_dofs;
  double queue_seconds;
  double run_seconds;
  double latency_seconds;
} mfgpu_request_result;

int mfgpu_server_create(int device, int max_concurrent, double memory_fraction,
                        mfgpu_server **server);
/* queue a request (copied); returns its id */
int mfgpu_server_submit(mfgpu_server *server, const mfgpu_request *request,
                        long long *id);
/* block until request `id` finished; its record is released */
int mfgpu_server_wait(mfgpu_server *server, long long id,
                      mfgpu_request_result *result);
/* highest number of solves that ran at the same time; memory budget */
int mfgpu_server_stats(mfgpu_server *server, int *max_running,
                       size_t *budget_bytes);
/* requests that reused a resident problem of their shape, and requests
 * that built a new one */
int mfgpu_server_pool_stats(mfgpu_server *server, long long *reused,
                            long long *built);
/* Continuous batching: a worker that takes a heat request also takes the
 * queued heat requests of the same shape and step count (among the first
 * 16, up to max_batch in all, default 4; 1 turns batching off) and solves
 * them together: one operator, one multigrid hierarchy and one CG for all,
 * so every cell kernel, transfer and smoother step is one launch over all
 * of them, replayed as one CUDA graph per V-cycle; each problem keeps its
 * own CG scalars and stopping test, so its iterates are the ones it gets
 * alone. */
int mfgpu_server_set_max_batch(mfgpu_server *server, int max_batch);
/* requests that ran in a batch of two or more, and the largest batch */
int mfgpu_server_batch_stats(mfgpu_server *server, long long *batched_requests,
                             int *largest_batch);
/* finishes queued requests, then stops the workers */
int mfgpu_server_destroy(mfgpu_server *server);

#ifdef __cplusplus
}
#endif

#endif /* MFGPU_H */
