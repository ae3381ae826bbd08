/*
 * autopdex_gb300 -- C ABI of the GB300 solve backend for AutoPDEx.
 *
 * The library replaces, for the built-in Q1 models, the device work and the host hop of
 * AutoPDEx's Newton solve path:
 *   element residual/tangent assembly   autopdex/assembler.py:587-777, :1064-1389
 *   COO -> CSR summation + Dirichlet row/column deletion
 *                                       autopdex/solver.py:1180-1222 (scipy_assembling)
 *   the linear solve of each Newton step
 *                                       autopdex/solver.py:544-659 (solve_linear),
 *                                       :1493-1539 (linear_solve_scipy), :951-1178 (linear_solve_jax)
 *   the damped Newton loop              autopdex/solver.py:740-948
 * The Python layer (autopdex_gb300.solver) mirrors solver.solver(dofs, settings,
 * static_settings) and calls these functions through ctypes.
 *
 * Conventions
 *   - Every function returns an int status: AGX_OK (0); > 0 numerical outcome
 *     (AGX_NOT_CONVERGED, AGX_DIVERGED); < 0 usage or CUDA error.  No C++ exception
 *     crosses the ABI.  agx_last_error() gives the message of the last failure.
 *   - Set-up functions (agx_set_nodes, agx_add_element_set, agx_set_dirichlet,
 *     agx_set_model, agx_set_element_field) take HOST pointers and copy.  Compute
 *     functions take DEVICE pointers owned by the caller; the library owns the pattern,
 *     the matrix values and all scratch vectors.
 *   - DOFs are one flat float64 vector, node-major: dof = node * ndof + component, the
 *     numbering AutoPDEx uses for a single-field dict or an (n_nodes, ndof) array
 *     (assembler.py:47-141, :331-436).
 *   - One context per CUDA stream; a context is not thread-safe.
 */
#ifndef AUTOPDEX_GB300_H
#define AUTOPDEX_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define AGX_OK 0
#define AGX_NOT_CONVERGED 1   /* iteration limit reached (solver.py:926-930) */
#define AGX_DIVERGED 2        /* NaN/Inf or growth > 10x (solver.py:914-925), Krylov breakdown */
#define AGX_ERR_ARG (-1)
#define AGX_ERR_CUDA (-2)
#define AGX_ERR_UNSUPPORTED (-3)
#define AGX_ERR_STATE (-5)

/* element types: Q1 quad (spaces.py:1913-1922), Q1 hex (spaces.py:12057-12081),
   2-node line for surface tractions (spaces.py:356-358) */
#define AGX_QUAD4 0
#define AGX_HEX8 1
#define AGX_LINE2 2
#define AGX_QUAD9 3 /* 9-node quadratic quad: corners, mid-sides (bottom, right, top, left), centre */
#define AGX_LINE3 4 /* 3-node quadratic line: end nodes, then the middle node */
/* simplices of fem_iso_line_tri_tet (spaces.py:12193, node orders of its n_dim 2 / 3 cases):
   reference triangle (0,0) (1,0) (0,1) and tetrahedron (0,0,0) (1,0,0) (0,1,0) (0,0,1) */
#define AGX_TRI3 5  /* linear triangle: N = 1 - xi - eta, xi, eta */
#define AGX_TRI6 6  /* quadratic triangle: corners, then mid-sides (0-1), (1-2), (2-0) */
#define AGX_TET4 7  /* linear tetrahedron: N = 1 - xi - eta - zeta, xi, eta, zeta */
#define AGX_TET10 8 /* quadratic tetrahedron: corners, then edges 0-1, 1-2, 0-2, 0-3, 1-3, 2-3 */
/* 27-node quadratic brick of fem_iso_line_quad_brick (spaces.py:12083-12154): corners as the
   8-node brick, mid-edges of the bottom face (x, y, x, y edges from node 0), of the top face,
   the vertical edges, the face centres x-, x+, y-, y+, z-, z+, the centre; scalar models */
#define AGX_HEX27 9
#define AGX_MAX_QPOINTS 16

/* built-in models (descriptors of the closures AutoPDEx builds in models.py) */
#define AGX_MODEL_POISSON_SINCOS 0 /* 'user potential' 1/2|grad u|^2 - b(x) u,
                                      b = a (sin(w x.x) - cos(w |x-c|^2)); params a, w, c[dim]
                                      (tests/test_dicts_as_dofs_user_potential.py:25-35) */
#define AGX_MODEL_HEAT_POTENTIAL 1 /* 'user potential' 1/2 k_e |grad u|^2 - f u; params f;
                                      element field k_e (models.py:1188-1269) */
#define AGX_MODEL_NEO_HOOKE 2      /* 'user element' hyperelastic Galerkin, Ciarlet neo-Hooke,
                                      plane strain (quad) or 3d (hex); params E, nu
                                      (models.py:917-1000, :1122-1146, :1616-1718) */
#define AGX_MODEL_NEUMANN 3        /* 'user element' surface traction, zero tangent; params t[dim]
                                      (models.py:744-780, :1723-1851) */
#define AGX_MODEL_HEAT_BE 4        /* 'user residual' backward Euler, k(T) = k0 + k2 T^2;
                                      params k0, k2, rho_c, dt; node field T_n
                                      (models.py:1272-1357) */

/* matrix value types */
#define AGX_F64 0
#define AGX_F32 1

/* Krylov methods for agx_solve / the linear step of agx_newton */
#define AGX_PCG 0        /* Jacobi-PCG, float64 matrix and vectors */
#define AGX_PCG_MIXED 1  /* Jacobi-PCG in float32 (matrix, vectors), float64 dots */
#define AGX_BICGSTAB 2   /* Jacobi-BiCGStab in float64, for non-symmetric tangents */
#define AGX_FCG_MIXED 3  /* flexible CG in float32 with the registered preconditioner
                            (agx_set_preconditioner), Jacobi when none is registered */
#define AGX_FCG_F64 5    /* flexible CG in float64 (vectors, products with the float64 tangent)
                            with the registered preconditioner applied in float32 on the
                            residual scaled by 1 / ||b|| (its two-level smoothing on a float32
                            copy of the tangent, the callback's network in bf16); Jacobi when
                            none is registered.  For tangents whose conditioning float32 Krylov
                            vectors cannot resolve (nearly incompressible solids). */
#define AGX_CHOL_BAND 4  /* direct: banded Cholesky of the float64 tangent with float64
                            refinement to rtol (the 'lapack' / 'umfpack' spsolve of
                            linear_solve_scipy, solver.py:1493-1539) for symmetric definite
                            tangents whose band fits in memory (structured 2-D meshes);
                            AGX_ERR_UNSUPPORTED otherwise, AGX_DIVERGED when a pivot is not
                            positive */

typedef struct agx_context agx_context;

/* Preconditioner callback for AGX_FCG_MIXED: z = M(r) on the free DOFs, float32 device
   vectors of length n_dofs, launched on `stream`.  Returns 0 on success. */
typedef int (*agx_precond_fn)(void* user, const float* r, float* z, int64_t n, void* stream);

typedef struct {
  int method;          /* AGX_PCG, AGX_PCG_MIXED, AGX_BICGSTAB, AGX_FCG_MIXED, AGX_CHOL_BAND,
                          AGX_FCG_F64 */
  double rtol;         /* stop when ||r|| <= rtol ||b|| (jax.scipy cg semantics, solver.py:1116) */
  double atol;         /* ... or ||r|| <= atol */
  int maxiter;
  int check_every;     /* iterations between host convergence checks (>= 1) */
} agx_solve_opts;

typedef struct {
  int iterations;
  double rel_residual; /* ||r|| / ||b|| of the recurrence residual */
  int status;          /* AGX_OK, AGX_NOT_CONVERGED, AGX_DIVERGED */
} agx_solve_info;

typedef struct {
  double newton_tol;   /* absolute tolerance on ||R_free||_2 (solver.py:899-903) */
  double newton_rtol;  /* stop also when ||R_free|| <= newton_rtol * ||R_free(first iterate)||;
                          0 disables (the reference has the absolute test only) */
  int maxiter;         /* solver.py:740-768 default 30 */
  double damping;      /* 1.0 for 'newton' (solver.py:767) */
  int tangent_dtype;   /* AGX_F64 or AGX_F32 */
  agx_solve_opts krylov;
  int reuse_tangent;   /* 1: assemble the tangent once (models whose tangent does not
                          depend on the DOFs: iterative refinement) */
  int verbose;
} agx_newton_opts;

typedef struct {
  int iterations;                 /* Newton iterations performed */
  double res_norm;                /* ||R_free||_2 after the last iteration */
  double res0;                    /* ||R_free||_2 at the first iterate (prescribed values set) */
  int diverged;                   /* solver.py:914-930 semantics */
  int krylov_iterations;          /* total inner iterations */
  int n_history;
  double res_history[64];
  int krylov_history[64];
} agx_newton_info;

/* ---- context ---------------------------------------------------------------------- */
/* Replaces the jit set-up of solver.solver (solver.py:41, utility.py:32-80). */
int agx_create(agx_context** ctx, void* cuda_stream);
int agx_destroy(agx_context* ctx);
const char* agx_last_error(const agx_context* ctx);

/* ---- problem definition (host pointers) -------------------------------------------- */
/* settings['node coordinates'] and the DOF layout (assembler.py:143-183). */
int agx_set_nodes(agx_context* ctx, int64_t n_nodes, int dim, const double* coords, int ndof);
/* One entry of settings['connectivity'] / static_settings['assembling mode']
   (assembler.py:587-777); returns the set index in *set_id. */
int agx_add_element_set(agx_context* ctx, int elem_type, int64_t n_elem, int nen,
                        const int64_t* conn, int* set_id);
/* settings['dirichlet dofs'] flattened (solver.py:586-604); 1 = prescribed. */
int agx_set_dirichlet(agx_context* ctx, const uint8_t* mask);
/* Builds the node-block CSR pattern and the element -> pattern scatter map, the work
   that scipy_assembling redoes on the host every Newton step (solver.py:1180-1222). */
int agx_finalize(agx_context* ctx);
/* static_settings['model'][set] (models.py builders); params as listed per model. */
int agx_set_model(agx_context* ctx, int set_id, int model, const double* params, int n_params);
/* per-element coefficient (host pointer, n_elem values), e.g. conductivity k_e */
/* Gauss-Legendre points per reference direction of a set (2, the default, or 3): the rule
   seeder.gauss_legendre_nd(dim, order) gives for order 2-3 and 4-5 (seeder.py:303-386,
   :1046-1062), which the model closures integrate with (models.py:1188-1269, :1616-1718). */
int agx_set_quadrature(agx_context* ctx, int set_id, int points_per_direction);
/* The integration points of a simplex set (AGX_TRI3/TRI6/TET4): n_points <= AGX_MAX_QPOINTS
   reference coordinates (n_points x 2 or x 3, row-major) and weights, as the model builders
   receive them from seeder.int_pts_ref_tri / int_pts_ref_tet (seeder.py:1813-2290). */
int agx_set_quadrature_points(agx_context* ctx, int set_id, int n_points, const double* points,
                              const double* weights);
int agx_set_element_field(agx_context* ctx, int set_id, const double* field);
/* per-DOF auxiliary field (DEVICE pointer, kept by reference), e.g. settings['dofs n'] */
int agx_set_node_field(agx_context* ctx, int set_id, const double* field_dev);

/* ---- compute (device pointers) ----------------------------------------------------- */
/* assemble_residual (assembler.py:587-637) into `residual` (n_dofs, may be NULL) and,
   when tangent_dtype >= 0, assemble_tangent (assembler.py:682-777) into the library's
   BSR values with Dirichlet rows/columns eliminated (identity rows). */
int agx_assemble(agx_context* ctx, const double* dofs, double* residual, int tangent_dtype);
/* Pattern and values of the last assembled tangent (device pointers owned by the
   library): rowptr (n_nodes+1), col (nnzb), vals (nnzb*ndof*ndof of the dtype) stored
   entry-major: entry (i, j) of block k at vals[(i*ndof + j)*nnzb + k]. */
int agx_get_matrix(agx_context* ctx, int dtype, const int32_t** rowptr, const int32_t** col,
                   const void** vals, int64_t* nnzb);
/* Copies the pattern and the values of the last assembled tangent of `dtype` into
   caller-owned DEVICE buffers (rowptr n_nodes+1, col nnzb, vals nnzb*ndof*ndof as
   row-major ndof x ndof blocks, block k at vals + k*ndof*ndof). */
int agx_copy_matrix(agx_context* ctx, int dtype, int32_t* rowptr, int32_t* col, void* vals);
/* y = K x with the last assembled tangent of `dtype` (x, y of that dtype). */
int agx_spmv(agx_context* ctx, int dtype, const void* x, void* y);
/* y = K x with the library's pattern and caller-provided values in the library's layout
   (entry-major planes, as agx_copy_values writes them): products with stored tangents. */
int agx_spmv_values(agx_context* ctx, int dtype, const void* values, const void* x, void* y);
/* Diagonal of the last assembled tangent of `dtype` as float64 (n_dofs, DEVICE pointer):
   assemble_tangent_diagonal (assembler.py:639-680, :1090-1113); identity entries on
   eliminated Dirichlet DOFs. */
int agx_get_diagonal(agx_context* ctx, int dtype, double* diag);
/* Raw copy of the last assembled tangent values in the library's layout (nnzb*ndof*ndof). */
int agx_copy_values(agx_context* ctx, int dtype, void* values);
/* z = D^-1 r with the diagonal of the last assembled tangent of `dtype` (Jacobi,
   solver.py:1093-1099). */
int agx_jacobi(agx_context* ctx, int dtype, const void* r, void* z);
/* Linear solve K x = rhs on the free DOFs, zeros on prescribed DOFs: the callback
   contract of linear_solve_scipy (solver.py:1493-1539) with an iterative method. */
int agx_solve(agx_context* ctx, const double* rhs, double* x, const agx_solve_opts* opts,
              agx_solve_info* info);
/* The Newton loop of solve_damped_newton/damped_newton (solver.py:770-948): `dofs` is
   updated in place; `dirichlet_values` (n_dofs) holds settings['dirichlet conditions']. */
int agx_newton(agx_context* ctx, double* dofs, const double* dirichlet_values,
               const agx_newton_opts* opts, agx_newton_info* info);
/* Registers the preconditioner used by AGX_FCG_MIXED (NULL restores Jacobi). */
int agx_set_preconditioner(agx_context* ctx, agx_precond_fn fn, void* user);
/* How FCG applies the registered preconditioner M (no counterpart in the reference).
   mode 0: z = M(r).
   mode 1, two-level: `sweeps` damped Jacobi sweeps z += w D^-1 (r - K z) from z = 0, then
   y = M(r - K z) and z += c y with the energy-optimal c = (r - K z, y) / (y, K y) -- never a
   worse step than the sweeps alone.
   mode 2 (default), symmetric two-level: mode 1 followed by `sweeps` post-smoothing sweeps.
   mode 3, symmetric two-level with Chebyshev smoothing: the sweeps of mode 2 replaced by the
   Chebyshev polynomial of degree `sweeps` for D^-1 K on [w lmax, lmax] (same cost per
   degree: one product), lmax the Gershgorin bound of the float32 tangent, computed once
   per assembled tangent.
   w: the Jacobi damping in (0, 1] (modes 1, 2; default 2/3) or the interval fraction in
   (0, 1) (mode 3); sweeps (default 1) in 1 .. 16.
   flags: AGX_PRECOND_CAPTURABLE declares that the callback only enqueues device work on the
   stream it is given (no synchronisation, allocation or host reads), so that FCG captures
   its iterations, callback included, into CUDA graphs and replays them; the callback's
   buffers must then stay valid until the preconditioner is replaced.
   AGX_PRECOND_BF16_SMOOTHING (modes 1-3): the smoothing, residual and step products of the
   two-level application read a bf16 copy of the float32 tangent's values (made once per
   assembled tangent; float32 vectors and accumulation), which halves their value traffic; the
   Krylov product itself keeps the float32 values. */
#define AGX_PRECOND_CAPTURABLE 1
#define AGX_PRECOND_BF16_SMOOTHING 2
int agx_set_preconditioner_mode(agx_context* ctx, int mode, double omega, int sweeps, int flags);
/* Kernel timing.  While enabled, the library brackets its kernel launches with CUDA events
   on its stream and accumulates the elapsed time per category; agx_profile_read
   synchronizes the stream, returns totals (ms) and launch counts, and resets them. */
#define AGX_PROF_TANGENT 0   /* element passes that assemble a tangent (with the residual
                                when fused) */
#define AGX_PROF_RESIDUAL 1  /* float64 residual-only element passes */
#define AGX_PROF_SPMV 2      /* sparse products of the Krylov iterations */
#define AGX_PROF_VECTOR 3    /* Krylov vector updates with their reductions */
#define AGX_PROF_PRECOND 4   /* the registered preconditioner callback (the network) */
#define AGX_PROF_FACTOR 5    /* direct factorizations */
#define AGX_PROF_SMOOTH 6    /* products of the two-level preconditioner's smoothing and step */
#define AGX_PROF_CATEGORIES 8
int agx_profile(agx_context* ctx, int enable);
int agx_profile_read(agx_context* ctx, double* ms, int64_t* launches);
/* ---- allocation-free solve ----------------------------------------------------------
   No counterpart in the reference.  Jacobi-PCG on a caller-provided float64 node-block
   CSR matrix (rowptr n_nodes+1, col nnzb, vals nnzb*ndof*ndof; device pointers, e.g. from
   agx_copy_matrix) for callers that cannot allocate device memory during a solve: solves
   K x = rhs from x = 0 until ||r|| <= rtol ||rhs||, without any context.  Its work vectors
   live in a fixed file-scope device array of AGX_NOALLOC_MAX_DOFS DOFs (10 MiB, reserved on
   every device that loads the library until the process exits); larger systems are
   rejected with AGX_ERR_ARG and a message in errbuf (nullable).  The first call on a device
   looks the array's address up (call it once before any stream capture).  The stream must
   belong to the current device (another device's stream is rejected with AGX_ERR_ARG).  All
   calls share the array: calls that overlap on the GPU race.  Returns AGX_OK,
   AGX_NOT_CONVERGED, AGX_DIVERGED or a negative error. */
#define AGX_NOALLOC_MAX_DOFS 262144
int agx_pcg_noalloc(const int32_t* rowptr, const int32_t* col, const double* vals, int64_t n_nodes, int ndof,
                    const double* rhs, double* x, double rtol, int maxiter, void* cuda_stream,
                    agx_solve_info* info, char* errbuf, int errbuf_len);
/* Autotuner: times every variant of the Krylov product -- lanes per block row 1, 2, 4, 8, 16
   with two blocks per lane and trip, 2, 4, 8 lanes with four blocks (code lanes + 256), and,
   when the pattern is the 3 x 3 stencil of a structured QUAD4 grid with 1 or 2 DOFs per node,
   the grid product that computes each row's block offsets and columns instead of reading them
   (code 512; 1024 with two rows per lane), and when it is the 27-node stencil of a structured
   HEX8 grid with 1 to 3 DOFs per node the brick product of the same kind (code 2048) -- on
   the last assembled tangent (CUDA events),
   keeps the fastest for that tangent's precision and reports its code. */
int agx_autotune(agx_context* ctx, int* spmv_tpr, float* spmv_ms);
/* Applies a tuning decision for the float64 (AGX_F64) or float32 (AGX_F32) product, e.g. from
   the autotuner's cache; 0 restores the default. */
int agx_set_tuning(agx_context* ctx, int dtype, int spmv_tpr);
/* Programmatic dependent launch of the Krylov iterations' kernels and of the learned
   preconditioner's (process-wide, on by default): each of them waits at its start for the grid
   before it and then lets the next one launch, so the next kernel's blocks are scheduled while
   the current one runs.  0 launches them plainly (same results). */
int agx_set_pdl(int enable);
/* Device address of the current Krylov solve's status (an int: 0 while iterating, 1
   converged, 2 broken down), written by the library's kernels between iterations; a
   registered preconditioner's kernels may read it to skip work the solve no longer needs. */
int agx_solve_flag(agx_context* ctx, const int** flag);
/* ny of the structured QUAD4 grid whose 3 x 3 stencil the pattern is (the grid products,
   codes 512 and 1024, apply), else 0; for keys of a tuning cache. */
int agx_grid_pattern(const agx_context* ctx, int* ny);
/* (ny << 16) | nz of the structured HEX8 grid whose 27-node stencil the pattern is (the brick
   product, code 2048, applies), else 0; for keys of a tuning cache. */
int agx_brick_pattern(const agx_context* ctx, int* code);
/* Number of kernels this context has launched since it was created. */
int agx_launch_count(const agx_context* ctx, int64_t* launches);
/* Sizes for the host layer: n_dofs, nnzb, ndof. */
int agx_get_sizes(const agx_context* ctx, int64_t* n_dofs, int64_t* nnzb, int* ndof);

#ifdef __cplusplus
}
#endif
#endif /* AUTOPDEX_GB300_H */
