// Shared declarations of the GB300 solve backend: context layout, error handling and
// small device helpers.  Everything here is internal; the public C ABI lives in
// include/autopdex_gb300.h.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/autopdex_gb300.h"

#define AGX_MAX_PARAMS 16
#define AGX_MAX_HISTORY 64

// Threads per block for every streaming kernel; grids are multiples of the SM count.
#define AGX_BLOCK 256

struct agx_element_set {
  int elem_type = -1;        // AGX_QUAD4 / AGX_HEX8 / AGX_LINE2 / AGX_QUAD9 / AGX_LINE3
  int nen = 0;               // nodes per element
  int ngauss = 2;            // Gauss-Legendre points per reference direction (2 or 3)
  int nqp = 0;               // simplex sets: integration points and weights on the reference simplex
  double qp[AGX_MAX_QPOINTS][3] = {};
  double qw[AGX_MAX_QPOINTS] = {};
  int64_t n_elem = 0;
  int32_t* d_conn = nullptr; // n_elem * nen
  int32_t* d_epos = nullptr; // n_elem * nen * nen node-block positions in the BSR pattern
  std::vector<int32_t> h_conn;
  int model = -1;
  int n_params = 0;
  double params[AGX_MAX_PARAMS] = {0};
  double* d_elem_field = nullptr;        // one value per element (owned)
  float* d_elem_field32 = nullptr;       // the same rounded to float32 once (float32 tangent passes)
  const double* d_node_field = nullptr;  // one value per DOF (caller-owned device pointer)
  double* d_geo = nullptr;  // float64 geometry cache: per element, Gauss point and node, (g_a, w det J)
  // structured quad grid of the mesher's numbering (element i ny + j has nodes (i, j), (i, j+1),
  // (i+1, j+1), (i+1, j), node (i, j) = i (ny + 1) + j) whose pattern rows are exactly the
  // in-range 3 x 3 node stencils; 0 when the set is not such a grid
  int grid_nx = 0, grid_ny = 0;
  bool grid_affine = false;  // every element of the grid is a parallelogram (float64 coordinates)
  // every element is the same parallelogram (edge vectors equal to 1e-14 of the element size):
  // grid_m = (M00, M01, M11, det J) of the constant Jacobian J, M = adj(J) adj(J)^T / det J
  bool grid_uniform = false;
  double grid_m[4] = {0.0, 0.0, 0.0, 0.0};
  // structured HEX8 brick grid of the mesher's numbering (brick_n = nx, ny, nz; 0 when the set
  // is not one) whose pattern rows are exactly the in-range 27-node stencils; brick_uniform:
  // every node on one lattice x0 + i e1 + j e2 + k e3, so J = [e1 | e2 | e3] / 2 everywhere,
  // brick_m = (J^T J)^-1 as M00 M01 M02 M11 M12 M22, brick_det = det J
  int brick_n[3] = {0, 0, 0};
  bool brick_uniform = false;
  double brick_m[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double brick_det = 0.0;
};

// Scalars of one Krylov solve, kept in device memory so that iterations need no host
// round trip.  Written only by one thread: of the last block of a reduction kernel, or of a
// one-block kernel that sums block partials.
struct agx_krylov_scalars {
  double rz;         // (r, z) of the current iterate
  double rr;         // (r, r)
  double pq;         // (p, A p)
  double alpha, beta;
  double rr_stop;    // stop when rr <= rr_stop
  double omega, rho, rhat_v, ts, tt;  // BiCGStab scalars
  double rz_old;     // flexible CG: (r_old, z_old)
  double extra[4];
  int converged;     // 1: tolerance met, 2: breakdown (zero or non-finite denominator)
  int iters;         // iterations completed
  int pad[2];
};

// Krylov product variant codes: lanes per block row (1, 2, 4, 8, 16), plus SPMV_UNROLL4 for
// four blocks per lane and trip (2, 4, 8 lanes); SPMV_GRID the structured grid's index-free
// product (one lane per row, 1 or 2 DOFs per node), SPMV_GRID2 the same with two rows per lane
constexpr int SPMV_UNROLL4 = 256;
constexpr int SPMV_GRID = 512;
constexpr int SPMV_GRID2 = 1024;  // the grid product with two rows per lane
constexpr int SPMV_BRICK = 2048;  // the structured brick grid's index-free 27-node product
inline int spmv_lanes(int code) {
  return (code == SPMV_GRID || code == SPMV_GRID2 || code == SPMV_BRICK) ? 1 : (code & (SPMV_UNROLL4 - 1));
}
inline bool spmv_is_grid(int code) { return code == SPMV_GRID || code == SPMV_GRID2; }

struct agx_context {
  cudaStream_t stream = nullptr;
  std::string err;
  int device = 0;
  int sm_count = 152;
  int debug = 0;  // AGX_DEBUG=1 in the environment: print Krylov scalars at every host check
  size_t geo_cache_limit = (size_t)16 << 30;  // largest float64 geometry cache per set (bytes)

  // nodes and DOFs
  int64_t n_nodes = 0;
  int dim = 0;
  int ndof = 0;            // DOFs per node (BSR block size)
  int64_t n_dofs = 0;
  double* d_coords = nullptr;   // n_nodes * dim
  std::vector<double> h_coords; // the same on the host (set-up checks)
  float* d_coords32 = nullptr;  // the same rounded to float32 once: float32 tangent passes read
                                // half the bytes and convert nothing on the 1/59-rate FP64 pipe
  std::vector<agx_element_set> sets;

  // Dirichlet DOFs
  std::vector<uint8_t> h_dmask;          // n_dofs
  uint8_t* d_dmask_node = nullptr;       // n_nodes, bit c set if component c is prescribed
  uint8_t* d_dmask_dof = nullptr;        // n_dofs, 1 if prescribed
  int32_t* d_dir_dofs = nullptr;         // list of prescribed DOFs
  int64_t n_dir = 0;

  // BSR pattern (node blocks of ndof x ndof)
  bool pattern_ready = false;
  int64_t nnzb = 0;
  int32_t* d_rowptr = nullptr;  // n_nodes + 1
  int32_t* d_col = nullptr;     // nnzb
  int32_t* d_diagpos = nullptr; // n_nodes
  double* d_vals64 = nullptr;   // nnzb * ndof^2
  float* d_vals32 = nullptr;
  double* d_dinv64 = nullptr;   // inverse diagonal (Jacobi)
  float* d_dinv32 = nullptr;
  int tangent_valid = -1;       // dtype of the last assembled tangent, -1 none

  // Newton / Krylov work vectors (double)
  double *d_R = nullptr, *d_b = nullptr, *d_dx = nullptr;
  double *d_r = nullptr, *d_z = nullptr, *d_p = nullptr, *d_q = nullptr;
  double *d_s = nullptr, *d_t = nullptr, *d_rhat = nullptr, *d_v = nullptr;
  // single-precision Krylov vectors (mixed precision inner solve)
  float *f_x = nullptr, *f_r = nullptr, *f_z = nullptr, *f_p = nullptr, *f_q = nullptr, *f_rold = nullptr;
  float *f_w1 = nullptr, *f_w2 = nullptr, *f_w3 = nullptr, *f_w4 = nullptr;  // two-level preconditioner work
  float* f_dofs32 = nullptr;  // float32 copy of the DOFs (the brick grid's float32 tangent reads it)

  // > 0: the pattern is the in-range 3 x 3 stencil of a structured nx x ny QUAD4 grid with
  // ny = pattern_grid_ny (the index-free product SPMV_GRID applies)
  int pattern_grid_ny = 0;
  // pattern of a structured nx x ny x nz brick grid (27-node stencils, 1 to 3 DOFs per node):
  // (ny << 16) | nz, 0 otherwise (the index-free product SPMV_BRICK applies)
  int pattern_brick = 0;
  // the grid argument of the product kernels: pattern_grid_ny or pattern_brick
  int pattern_stencil = 0;

  // reductions
  int red_blocks = 0;   // largest grid of a reducing kernel (8 per SM)
  int vec_blocks = 0;   // grid of the reducing vector kernels (2 per SM: short reduction tails)
  double* d_partials = nullptr;          // red_blocks * 4
  unsigned int* d_counter = nullptr;
  agx_krylov_scalars* d_scal = nullptr;
  agx_krylov_scalars* h_scal = nullptr;  // pinned
  double* d_norm = nullptr;              // 4 doubles
  double* h_norm = nullptr;              // pinned

  // kernels launched by this context (for the benchmark's launch count)
  int64_t n_launches = 0;

  // kernel timing (agx_profile): event pairs per category, reused across reads
  bool prof_on = false;
  std::vector<cudaEvent_t> prof_ev[AGX_PROF_CATEGORIES];
  size_t prof_used[AGX_PROF_CATEGORIES] = {0};
  double prof_extra_ms[AGX_PROF_CATEGORIES] = {0};   // from replayed CUDA graphs
  int64_t prof_extra_n[AGX_PROF_CATEGORIES] = {0};

  // CUDA graphs of Krylov iteration chunks (one per method slot)
  struct graph_rec {
    cudaGraphExec_t exec = nullptr;
    const void* key_x = nullptr;  // output vector captured in the graph
    int64_t pc_key = -1;          // preconditioner generation captured (flexible CG), else -1
    int every = 0;
    bool prof = false;             // captured with timing events
    int tpr = 0;                   // lanes per row of the captured products
    int64_t kernels = 0;           // kernel nodes of the graph (the callback's included)
    bool pdl = false;              // captured with programmatic dependent launch
    std::vector<cudaEvent_t> ev[AGX_PROF_CATEGORIES];  // event pairs recorded by each replay
  };
  graph_rec graphs[3];  // Jacobi-PCG float64, float32 methods, flexible CG float64
  graph_rec* capturing = nullptr;  // set while a chunk is being captured
  bool use_graphs = true;
  // the legacy default stream cannot be captured: graphs then run on this private stream,
  // ordered against the context stream by events
  cudaStream_t graph_stream = nullptr;
  cudaEvent_t graph_ev[2] = {nullptr, nullptr};

  // learned preconditioner hook (set by the host layer; null = Jacobi)
  agx_precond_fn precond = nullptr;
  void* precond_user = nullptr;
  int precond_mode = 2;
  double precond_omega = 2.0 / 3.0;
  int precond_sweeps = 1;
  double cheb_lmax = 2.0;      // Gershgorin bound of D^-1 K for the Chebyshev smoother
  int64_t cheb_gen = -1;       // tangent generation the bound belongs to
  int64_t tangent_gen = 0;     // bumped by every tangent assembly
  int precond_capturable = 0;  // the callback only enqueues work on the stream it is given
  int precond_bf16 = 0;        // two-level products on a bf16 copy of the float32 values
  __nv_bfloat16* d_vals16 = nullptr;
  int64_t bf16_copy_gen = -1;  // tangent generation whose bf16 copy is current
  int64_t precond_gen = 0;     // bumped whenever the callback or its mode changes
  int spmv_tpr[2] = {0, 0};  // lanes per block row of the Krylov product, float64 / float32 (0: default)
  int64_t f32_copy_gen = -1;  // tangent generation whose float32 copy (values, inverse diagonal) is current

  // banded Cholesky factor of the float64 tangent (AGX_CHOL_BAND): lower band stored by
  // columns, entry (j + k, j) at d_band[j (band_w + 1) + k], k = 0 .. band_w
  int64_t band_w = -1;          // half bandwidth in DOFs of the pattern (-1: not computed yet)
  double* d_band = nullptr;     // n_dofs * (band_w + 1)
  int* d_band_err = nullptr;    // first column whose pivot was not positive (+1), 0 if none
  double* d_band_l11 = nullptr; // factored diagonal block of the current panel (scratch)
  double* d_band_rdiag = nullptr;  // reciprocals of the factor's diagonal (n_dofs)
  int64_t band_gen = -1;        // tangent generation the factor belongs to
  double band_sign = 1.0;       // the factor is of band_sign * K (-1 for negative definite tangents)
  size_t band_max_bytes = (size_t)24 << 30;  // largest factor this context allocates
};

// ------------------------------------------------------------------------------------
// error handling: every entry point returns an int status and records a message
// ------------------------------------------------------------------------------------
int agx_fail(agx_context* ctx, int code, const char* fmt, ...);

// Programmatic dependent launch.  The kernels of the Krylov iterations and of the learned
// preconditioner begin with agx_pdl_entry(): griddepcontrol.wait returns once the grid before
// them in the stream has completed and its writes are visible, then launch_dependents lets the
// next grid launch.  agx_launch_pdl launches with programmatic stream serialization, so the next
// kernel's blocks are scheduled while this one runs instead of after it (the launch latency of a
// chain of short dependent kernels is hidden).  Only kernels that begin with the entry may be
// launched this way; without the attribute the entry costs nothing.  agx_set_pdl(0) turns the
// attribute off process-wide.
extern bool g_agx_pdl;
__device__ __forceinline__ void agx_pdl_entry() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t agx_launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                  Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = g_agx_pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

#define AGX_CUDA(ctx, call)                                                          \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return agx_fail((ctx), AGX_ERR_CUDA, "%s failed: %s (%s:%d)", #call,           \
                      cudaGetErrorString(e_), __FILE__, __LINE__);                   \
  } while (0)

#define AGX_CHECK_LAUNCH(ctx) AGX_CUDA((ctx), cudaGetLastError())

// internal entry points shared across translation units
int agx_build_pattern(agx_context* ctx);
int agx_assemble_impl(agx_context* ctx, const double* dofs, double* residual, int tangent_dtype);
// uniform structured brick grids with the backward-Euler heat model (agx_brick.cu)
bool agx_brick_heat_be(const agx_context* ctx, const agx_element_set& s);
void agx_launch_brick_residual(agx_context* ctx, const agx_element_set& s, const double* dofs, double* R);
void agx_launch_brick_tangent(agx_context* ctx, const agx_element_set& s, const double* dofs, float* vals,
                              float* dinv);
int agx_krylov_impl(agx_context* ctx, const double* rhs, double* x, const agx_solve_opts* opts,
                    agx_solve_info* info);
int agx_residual_norm(agx_context* ctx, const double* R, double* norm2, double* nonfinite);
void agx_launch_masked_scale(agx_context* ctx, const double* src, double* dst, double s);
void agx_launch_set_dirichlet(agx_context* ctx, double* dofs, const double* values);
void agx_launch_newton_update(agx_context* ctx, double* dofs, const double* dx, const double* values,
                              double damping);
void agx_launch_negate_free(agx_context* ctx, const double* R, double* b);
int agx_spmv_impl(agx_context* ctx, int dtype, const void* x, void* y);
int agx_spmv_values_impl(agx_context* ctx, int dtype, const void* values, const void* x, void* y);
void agx_launch_jacobi(agx_context* ctx, int dtype, const void* r, void* z);
void agx_launch_diagonal(agx_context* ctx, int dtype, double* diag);
int agx_autotune_spmv(agx_context* ctx, int* chosen, float* best_ms);
int agx_band_solve_impl(agx_context* ctx, const double* b, double* x, const agx_solve_opts* opts,
                        agx_solve_info* info);
void agx_launch_planes_to_blocks(agx_context* ctx, const double* planes, double* blocks);
void agx_launch_planes_to_blocks(agx_context* ctx, const float* planes, float* blocks);

// Brackets the launches issued during its lifetime with events of category `cat`.
struct agx_prof_scope {
  agx_context* ctx;
  int cat;
  cudaEvent_t stop = nullptr;
  agx_prof_scope(agx_context* c, int k) : ctx(c), cat(k) {
    if (!ctx->prof_on) return;
    if (ctx->capturing) {  // the graph owns the events; each replay records them again
      auto& gev = ctx->capturing->ev[cat];
      cudaEvent_t a, b;
      if (cudaEventCreate(&a) != cudaSuccess) return;
      if (cudaEventCreate(&b) != cudaSuccess) return;
      gev.push_back(a);
      gev.push_back(b);
      cudaEventRecord(a, ctx->stream);
      stop = b;
      return;
    }
    auto& ev = ctx->prof_ev[cat];
    size_t u = ctx->prof_used[cat];
    while (ev.size() < 2 * (u + 1)) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return;
      ev.push_back(e);
    }
    cudaEventRecord(ev[2 * u], ctx->stream);
    stop = ev[2 * u + 1];
    ctx->prof_used[cat] = u + 1;
  }
  ~agx_prof_scope() {
    if (stop) cudaEventRecord(stop, ctx->stream);
  }
};

static inline int agx_grid(const agx_context* ctx, int64_t n, int per_sm = 8) {
  int64_t want = (n + AGX_BLOCK - 1) / AGX_BLOCK;
  int64_t cap = (int64_t)ctx->sm_count * per_sm;
  if (want < 1) want = 1;
  return (int)(want < cap ? want : cap);
}
