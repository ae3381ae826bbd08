// extern "C" entry points of libautopdex_gb300 (declared in include/autopdex_gb300.h) and
// the native Newton driver.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <new>

#include "agx_common.cuh"

int agx_fail(agx_context* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

namespace {

// float32 copy of a set-up array, rounded to nearest as every float32 pass would round it
__global__ void round_to_float(int64_t n, const double* __restrict__ in, float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

template <typename T>
int alloc(agx_context* ctx, T** p, int64_t n) {
  AGX_CUDA(ctx, cudaMalloc((void**)p, sizeof(T) * (size_t)(n > 0 ? n : 1)));
  return AGX_OK;
}

template <typename T>
void release(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

void free_device(agx_context* ctx) {
  release(ctx->d_coords);
  release(ctx->d_coords32);
  for (auto& s : ctx->sets) {
    release(s.d_conn);
    release(s.d_epos);
    release(s.d_elem_field);
    release(s.d_elem_field32);
    release(s.d_geo);
  }
  release(ctx->d_dmask_node);
  release(ctx->d_dmask_dof);
  release(ctx->d_dir_dofs);
  release(ctx->d_rowptr);
  release(ctx->d_col);
  release(ctx->d_diagpos);
  release(ctx->d_vals64);
  release(ctx->d_vals32);
  release(ctx->d_vals16);
  release(ctx->d_dinv64);
  release(ctx->d_dinv32);
  release(ctx->d_band);
  release(ctx->d_band_err);
  release(ctx->d_band_l11);
  release(ctx->d_band_rdiag);
  for (double** p : {&ctx->d_R, &ctx->d_b, &ctx->d_dx, &ctx->d_r, &ctx->d_z, &ctx->d_p, &ctx->d_q, &ctx->d_s,
                     &ctx->d_t, &ctx->d_rhat, &ctx->d_v})
    release(*p);
  for (float** p : {&ctx->f_x, &ctx->f_r, &ctx->f_z, &ctx->f_p, &ctx->f_q, &ctx->f_rold, &ctx->f_w1, &ctx->f_w2,
                    &ctx->f_w3, &ctx->f_w4, &ctx->f_dofs32})
    release(*p);
  release(ctx->d_partials);
  release(ctx->d_counter);
  release(ctx->d_scal);
  release(ctx->d_norm);
  for (int c = 0; c < AGX_PROF_CATEGORIES; ++c) {
    for (auto e : ctx->prof_ev[c]) cudaEventDestroy(e);
    ctx->prof_ev[c].clear();
  }
  if (ctx->graph_stream) cudaStreamDestroy(ctx->graph_stream);
  for (auto& e : ctx->graph_ev)
    if (e) cudaEventDestroy(e);
  ctx->graph_stream = nullptr;
  for (auto& gr : ctx->graphs) {
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
    gr.exec = nullptr;
    for (auto& v : gr.ev) {
      for (auto e : v) cudaEventDestroy(e);
      v.clear();
    }
  }
  if (ctx->h_scal) cudaFreeHost(ctx->h_scal);
  if (ctx->h_norm) cudaFreeHost(ctx->h_norm);
  ctx->h_scal = nullptr;
  ctx->h_norm = nullptr;
}

bool model_ok(int elem_type, int model, int dim, int ndof, int n_params, std::string& why) {
  const int sdim = dim;
  const bool domain = elem_type == AGX_QUAD4 || elem_type == AGX_HEX8 || elem_type == AGX_QUAD9 ||
                      elem_type == AGX_TRI3 || elem_type == AGX_TRI6 || elem_type == AGX_TET4 ||
                      elem_type == AGX_TET10 || elem_type == AGX_HEX27;
  switch (model) {
    case AGX_MODEL_POISSON_SINCOS:
      if (ndof != 1) return why = "POISSON_SINCOS needs 1 DOF per node", false;
      if (n_params < 2 + sdim) return why = "POISSON_SINCOS needs params a, w, c[dim]", false;
      return domain ? true : (why = "domain element required", false);
    case AGX_MODEL_HEAT_POTENTIAL:
      if (ndof != 1) return why = "HEAT_POTENTIAL needs 1 DOF per node", false;
      if (n_params < 1) return why = "HEAT_POTENTIAL needs param f", false;
      return domain ? true : (why = "domain element required", false);
    case AGX_MODEL_NEO_HOOKE:
      if (ndof != sdim) return why = "NEO_HOOKE needs dim DOFs per node", false;
      if (n_params < 2) return why = "NEO_HOOKE needs params E, nu", false;
      if (domain) return true;
      return why = "NEO_HOOKE needs a domain element (quad4/quad9/tri3/tri6 in 2-D, hex8/tet4/tet10 in 3-D)", false;
    case AGX_MODEL_NEUMANN:
      if ((elem_type != AGX_LINE2 && elem_type != AGX_LINE3) || dim != 2)
        return why = "NEUMANN supports 2- and 3-node lines in 2-D", false;
      if (ndof != 2 || n_params < 2) return why = "NEUMANN needs 2 DOFs per node and params t0, t1", false;
      return true;
    case AGX_MODEL_HEAT_BE:
      if (ndof != 1) return why = "HEAT_BE needs 1 DOF per node", false;
      if (n_params < 4) return why = "HEAT_BE needs params k0, k2, rho_c, dt", false;
      return elem_type == AGX_QUAD4 || elem_type == AGX_HEX8 ? true : (why = "domain element required", false);
    default:
      return why = "unknown model", false;
  }
}

}  // namespace

bool g_agx_pdl = true;  // agx_set_pdl

extern "C" {

int agx_create(agx_context** out, void* stream) {
  if (!out) return AGX_ERR_ARG;
  agx_context* ctx = new (std::nothrow) agx_context();
  if (!ctx) return AGX_ERR_ARG;
  ctx->stream = (cudaStream_t)stream;
  const char* dbg = getenv("AGX_DEBUG");
  ctx->debug = (dbg && dbg[0] == '1') ? 1 : 0;
  cudaError_t e = cudaGetDevice(&ctx->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
  if (e != cudaSuccess) {
    delete ctx;
    *out = nullptr;
    return AGX_ERR_CUDA;
  }
  *out = ctx;
  return AGX_OK;
}

int agx_destroy(agx_context* ctx) {
  if (!ctx) return AGX_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_device(ctx);
  delete ctx;
  return AGX_OK;
}

const char* agx_last_error(const agx_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int agx_set_nodes(agx_context* ctx, int64_t n_nodes, int dim, const double* coords, int ndof) {
  if (!ctx || !coords || n_nodes <= 0 || n_nodes >= INT32_MAX) return agx_fail(ctx, AGX_ERR_ARG, "bad node arguments");
  if (dim < 2 || dim > 3 || ndof < 1 || ndof > 3) return agx_fail(ctx, AGX_ERR_UNSUPPORTED, "dim 2-3 and 1-3 DOFs per node");
  if (ctx->d_coords) return agx_fail(ctx, AGX_ERR_STATE, "nodes already set");
  ctx->n_nodes = n_nodes;
  ctx->dim = dim;
  ctx->ndof = ndof;
  ctx->n_dofs = n_nodes * ndof;
  if (int rc = alloc(ctx, &ctx->d_coords, n_nodes * dim)) return rc;
  AGX_CUDA(ctx, cudaMemcpy(ctx->d_coords, coords, sizeof(double) * n_nodes * dim, cudaMemcpyHostToDevice));
  ctx->h_coords.assign(coords, coords + n_nodes * dim);
  if (int rc = alloc(ctx, &ctx->d_coords32, n_nodes * dim)) return rc;
  round_to_float<<<agx_grid(ctx, n_nodes * dim), AGX_BLOCK, 0, ctx->stream>>>(n_nodes * dim, ctx->d_coords,
                                                                               ctx->d_coords32);
  AGX_CHECK_LAUNCH(ctx);
  ctx->h_dmask.assign(ctx->n_dofs, 0);
  return AGX_OK;
}

int agx_add_element_set(agx_context* ctx, int elem_type, int64_t n_elem, int nen, const int64_t* conn, int* set_id) {
  if (!ctx || !conn || n_elem <= 0) return agx_fail(ctx, AGX_ERR_ARG, "bad element set arguments");
  if (ctx->n_nodes == 0) return agx_fail(ctx, AGX_ERR_STATE, "agx_set_nodes first");
  if (ctx->pattern_ready) return agx_fail(ctx, AGX_ERR_STATE, "pattern already finalized");
  const int want = elem_type == AGX_QUAD4   ? 4
                   : elem_type == AGX_HEX8  ? 8
                   : elem_type == AGX_LINE2 ? 2
                   : elem_type == AGX_QUAD9 ? 9
                   : elem_type == AGX_LINE3 ? 3
                   : elem_type == AGX_TRI3  ? 3
                   : elem_type == AGX_TRI6  ? 6
                   : elem_type == AGX_TET4  ? 4
                   : elem_type == AGX_TET10 ? 10
                   : elem_type == AGX_HEX27 ? 27
                                            : -1;
  if (want < 0 || nen != want) return agx_fail(ctx, AGX_ERR_UNSUPPORTED, "element type %d with %d nodes", elem_type, nen);
  if ((elem_type == AGX_HEX8 || elem_type == AGX_HEX27 || elem_type == AGX_TET4 || elem_type == AGX_TET10) !=
      (ctx->dim == 3))
    return agx_fail(ctx, AGX_ERR_UNSUPPORTED, "bricks and tetrahedra need 3-D nodes, quads, triangles and lines 2-D nodes");
  agx_element_set s;
  s.elem_type = elem_type;
  s.nen = nen;
  s.n_elem = n_elem;
  s.h_conn.resize((size_t)n_elem * nen);
  for (int64_t i = 0; i < n_elem * nen; ++i) {
    if (conn[i] < 0 || conn[i] >= ctx->n_nodes)
      return agx_fail(ctx, AGX_ERR_ARG, "connectivity entry %lld out of range", (long long)conn[i]);
    s.h_conn[i] = (int32_t)conn[i];
  }
  if (int rc = alloc(ctx, &s.d_conn, n_elem * nen)) return rc;
  AGX_CUDA(ctx, cudaMemcpy(s.d_conn, s.h_conn.data(), sizeof(int32_t) * n_elem * nen, cudaMemcpyHostToDevice));
  ctx->sets.push_back(std::move(s));
  if (set_id) *set_id = (int)ctx->sets.size() - 1;
  return AGX_OK;
}

int agx_set_dirichlet(agx_context* ctx, const uint8_t* mask) {
  if (!ctx || !mask) return agx_fail(ctx, AGX_ERR_ARG, "null mask");
  if (ctx->n_nodes == 0) return agx_fail(ctx, AGX_ERR_STATE, "agx_set_nodes first");
  for (int64_t i = 0; i < ctx->n_dofs; ++i) ctx->h_dmask[i] = mask[i] ? 1 : 0;
  std::vector<uint8_t> node(ctx->n_nodes, 0);
  std::vector<int32_t> dir;
  for (int64_t i = 0; i < ctx->n_dofs; ++i)
    if (ctx->h_dmask[i]) {
      node[i / ctx->ndof] |= (uint8_t)(1u << (i % ctx->ndof));
      dir.push_back((int32_t)i);
    }
  release(ctx->d_dmask_node);
  release(ctx->d_dmask_dof);
  release(ctx->d_dir_dofs);
  if (int rc = alloc(ctx, &ctx->d_dmask_node, ctx->n_nodes)) return rc;
  if (int rc = alloc(ctx, &ctx->d_dmask_dof, ctx->n_dofs)) return rc;
  if (int rc = alloc(ctx, &ctx->d_dir_dofs, (int64_t)dir.size())) return rc;
  AGX_CUDA(ctx, cudaMemcpy(ctx->d_dmask_node, node.data(), ctx->n_nodes, cudaMemcpyHostToDevice));
  AGX_CUDA(ctx, cudaMemcpy(ctx->d_dmask_dof, ctx->h_dmask.data(), ctx->n_dofs, cudaMemcpyHostToDevice));
  if (!dir.empty())
    AGX_CUDA(ctx, cudaMemcpy(ctx->d_dir_dofs, dir.data(), sizeof(int32_t) * dir.size(), cudaMemcpyHostToDevice));
  ctx->n_dir = (int64_t)dir.size();
  ctx->tangent_valid = -1;
  return AGX_OK;
}

int agx_finalize(agx_context* ctx) {
  if (!ctx) return AGX_ERR_ARG;
  if (ctx->sets.empty()) return agx_fail(ctx, AGX_ERR_STATE, "no element sets");
  if (ctx->pattern_ready) return agx_fail(ctx, AGX_ERR_STATE, "already finalized");
  if (!ctx->d_dmask_node) {
    std::vector<uint8_t> none(ctx->n_dofs, 0);
    if (int rc = agx_set_dirichlet(ctx, none.data())) return rc;
  }
  if (int rc = agx_build_pattern(ctx)) return rc;
  const int64_t n = ctx->n_dofs;
  for (double** p : {&ctx->d_R, &ctx->d_b, &ctx->d_dx, &ctx->d_r, &ctx->d_z, &ctx->d_p, &ctx->d_q, &ctx->d_s,
                     &ctx->d_t, &ctx->d_rhat, &ctx->d_v, &ctx->d_dinv64})
    if (int rc = alloc(ctx, p, n)) return rc;
  for (float** p : {&ctx->f_x, &ctx->f_r, &ctx->f_z, &ctx->f_p, &ctx->f_q, &ctx->f_rold, &ctx->d_dinv32, &ctx->f_w1,
                    &ctx->f_w2, &ctx->f_w3, &ctx->f_w4, &ctx->f_dofs32})
    if (int rc = alloc(ctx, p, n)) return rc;
  ctx->red_blocks = ctx->sm_count * 8;  // one resident wave of 256-thread blocks
  ctx->vec_blocks = ctx->sm_count * 4;  // reducing vector kernels (16-byte accesses)
  if (int rc = alloc(ctx, &ctx->d_partials, (int64_t)ctx->red_blocks * 4)) return rc;  // up to 4 values per block
  if (int rc = alloc(ctx, &ctx->d_counter, 1)) return rc;
  if (int rc = alloc(ctx, &ctx->d_scal, 1)) return rc;
  if (int rc = alloc(ctx, &ctx->d_norm, 4)) return rc;
  AGX_CUDA(ctx, cudaMemset(ctx->d_counter, 0, sizeof(unsigned)));
  AGX_CUDA(ctx, cudaMemset(ctx->d_scal, 0, sizeof(agx_krylov_scalars)));
  AGX_CUDA(ctx, cudaMemset(ctx->d_q, 0, sizeof(double) * n));
  AGX_CUDA(ctx, cudaMemset(ctx->f_q, 0, sizeof(float) * n));
  AGX_CUDA(ctx, cudaMallocHost((void**)&ctx->h_scal, sizeof(agx_krylov_scalars)));
  AGX_CUDA(ctx, cudaMallocHost((void**)&ctx->h_norm, 4 * sizeof(double)));
  AGX_CUDA(ctx, cudaDeviceSynchronize());
  return AGX_OK;
}

int agx_set_model(agx_context* ctx, int set_id, int model, const double* params, int n_params) {
  if (!ctx || set_id < 0 || set_id >= (int)ctx->sets.size()) return agx_fail(ctx, AGX_ERR_ARG, "bad set id");
  if (n_params < 0 || n_params > AGX_MAX_PARAMS || (n_params > 0 && !params))
    return agx_fail(ctx, AGX_ERR_ARG, "bad parameter list");
  auto& s = ctx->sets[set_id];
  std::string why;
  if (!model_ok(s.elem_type, model, ctx->dim, ctx->ndof, n_params, why))
    return agx_fail(ctx, AGX_ERR_UNSUPPORTED, "set %d: %s", set_id, why.c_str());
  s.model = model;
  s.n_params = n_params;
  for (int i = 0; i < AGX_MAX_PARAMS; ++i) s.params[i] = i < n_params ? params[i] : 0.0;
  ctx->tangent_valid = -1;
  return AGX_OK;
}

int agx_set_quadrature(agx_context* ctx, int set_id, int points_per_direction) {
  if (!ctx || set_id < 0 || set_id >= (int)ctx->sets.size()) return agx_fail(ctx, AGX_ERR_ARG, "bad set id");
  if (points_per_direction != 2 && points_per_direction != 3)
    return agx_fail(ctx, AGX_ERR_UNSUPPORTED, "2 or 3 Gauss points per direction are implemented");
  auto& s = ctx->sets[set_id];
  if (s.ngauss != points_per_direction) {
    s.ngauss = points_per_direction;
    if (s.d_geo) {  // the float64 geometry cache holds the old points
      cudaFree(s.d_geo);
      s.d_geo = nullptr;
    }
    ctx->tangent_valid = -1;
  }
  return AGX_OK;
}

int agx_set_quadrature_points(agx_context* ctx, int set_id, int n_points, const double* points,
                              const double* weights) {
  if (!ctx || set_id < 0 || set_id >= (int)ctx->sets.size()) return agx_fail(ctx, AGX_ERR_ARG, "bad set id");
  auto& s = ctx->sets[set_id];
  const int rdim = (s.elem_type == AGX_TET4 || s.elem_type == AGX_TET10) ? 3 : 2;
  if (s.elem_type != AGX_TRI3 && s.elem_type != AGX_TRI6 && s.elem_type != AGX_TET4 && s.elem_type != AGX_TET10)
    return agx_fail(ctx, AGX_ERR_UNSUPPORTED, "integration point tables are for simplex sets");
  if (!points || !weights || n_points < 1 || n_points > AGX_MAX_QPOINTS)
    return agx_fail(ctx, AGX_ERR_ARG, "1 to %d integration points", AGX_MAX_QPOINTS);
  s.nqp = n_points;
  for (int q = 0; q < AGX_MAX_QPOINTS; ++q) {
    for (int d = 0; d < 3; ++d) s.qp[q][d] = (q < n_points && d < rdim) ? points[q * rdim + d] : 0.0;
    s.qw[q] = q < n_points ? weights[q] : 0.0;
  }
  ctx->tangent_valid = -1;
  return AGX_OK;
}

int agx_set_element_field(agx_context* ctx, int set_id, const double* field) {
  if (!ctx || set_id < 0 || set_id >= (int)ctx->sets.size()) return agx_fail(ctx, AGX_ERR_ARG, "bad set id");
  auto& s = ctx->sets[set_id];
  if (!field) {
    release(s.d_elem_field);
    release(s.d_elem_field32);
    return AGX_OK;
  }
  if (!s.d_elem_field)
    if (int rc = alloc(ctx, &s.d_elem_field, s.n_elem)) return rc;
  if (!s.d_elem_field32)
    if (int rc = alloc(ctx, &s.d_elem_field32, s.n_elem)) return rc;
  AGX_CUDA(ctx, cudaMemcpy(s.d_elem_field, field, sizeof(double) * s.n_elem, cudaMemcpyHostToDevice));
  round_to_float<<<agx_grid(ctx, s.n_elem), AGX_BLOCK, 0, ctx->stream>>>(s.n_elem, s.d_elem_field, s.d_elem_field32);
  AGX_CHECK_LAUNCH(ctx);
  ctx->tangent_valid = -1;
  return AGX_OK;
}

int agx_set_node_field(agx_context* ctx, int set_id, const double* field_dev) {
  if (!ctx || set_id < 0 || set_id >= (int)ctx->sets.size()) return agx_fail(ctx, AGX_ERR_ARG, "bad set id");
  ctx->sets[set_id].d_node_field = field_dev;
  ctx->tangent_valid = -1;
  return AGX_OK;
}

static int check_ready(agx_context* ctx) {
  if (!ctx) return AGX_ERR_ARG;
  if (!ctx->pattern_ready) return agx_fail(ctx, AGX_ERR_STATE, "agx_finalize first");
  for (size_t i = 0; i < ctx->sets.size(); ++i) {
    const auto& s = ctx->sets[i];
    if (s.model < 0) return agx_fail(ctx, AGX_ERR_STATE, "set %zu has no model", i);
    if (s.model == AGX_MODEL_HEAT_BE && !s.d_node_field)
      return agx_fail(ctx, AGX_ERR_STATE, "set %zu: HEAT_BE needs the node field T_n", i);
  }
  return AGX_OK;
}

int agx_assemble(agx_context* ctx, const double* dofs, double* residual, int tangent_dtype) {
  if (int rc = check_ready(ctx)) return rc;
  if (!dofs) return agx_fail(ctx, AGX_ERR_ARG, "null dofs");
  if (tangent_dtype != -1 && tangent_dtype != AGX_F64 && tangent_dtype != AGX_F32)
    return agx_fail(ctx, AGX_ERR_ARG, "tangent dtype must be -1, AGX_F64 or AGX_F32");
  return agx_assemble_impl(ctx, dofs, residual, tangent_dtype);
}

int agx_get_matrix(agx_context* ctx, int dtype, const int32_t** rowptr, const int32_t** col, const void** vals,
                   int64_t* nnzb) {
  if (!ctx || !ctx->pattern_ready) return agx_fail(ctx, AGX_ERR_STATE, "agx_finalize first");
  if (rowptr) *rowptr = ctx->d_rowptr;
  if (col) *col = ctx->d_col;
  if (vals) *vals = dtype == AGX_F64 ? (const void*)ctx->d_vals64 : (const void*)ctx->d_vals32;
  if (nnzb) *nnzb = ctx->nnzb;
  return AGX_OK;
}

int agx_copy_matrix(agx_context* ctx, int dtype, int32_t* rowptr, int32_t* col, void* vals) {
  if (!ctx || !ctx->pattern_ready) return agx_fail(ctx, AGX_ERR_STATE, "agx_finalize first");
  if (dtype != AGX_F64 && dtype != AGX_F32) return agx_fail(ctx, AGX_ERR_ARG, "dtype must be AGX_F64 or AGX_F32");
  if (rowptr)
    AGX_CUDA(ctx, cudaMemcpyAsync(rowptr, ctx->d_rowptr, sizeof(int32_t) * (ctx->n_nodes + 1),
                                  cudaMemcpyDeviceToDevice, ctx->stream));
  if (col)
    AGX_CUDA(ctx, cudaMemcpyAsync(col, ctx->d_col, sizeof(int32_t) * ctx->nnzb, cudaMemcpyDeviceToDevice, ctx->stream));
  if (vals) {
    // library layout: entry-major planes; caller layout: row-major ndof x ndof blocks
    if (dtype == AGX_F64)
      agx_launch_planes_to_blocks(ctx, ctx->d_vals64, (double*)vals);
    else
      agx_launch_planes_to_blocks(ctx, ctx->d_vals32, (float*)vals);
    AGX_CHECK_LAUNCH(ctx);
  }
  AGX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return AGX_OK;
}

int agx_profile(agx_context* ctx, int enable) {
  if (!ctx) return AGX_ERR_ARG;
  ctx->prof_on = enable != 0;
  for (int c = 0; c < AGX_PROF_CATEGORIES; ++c) {
    ctx->prof_used[c] = 0;
    ctx->prof_extra_ms[c] = 0;
    ctx->prof_extra_n[c] = 0;
  }
  return AGX_OK;
}

int agx_profile_read(agx_context* ctx, double* ms, int64_t* launches) {
  if (!ctx) return AGX_ERR_ARG;
  AGX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int c = 0; c < AGX_PROF_CATEGORIES; ++c) {
    double tot = 0;
    for (size_t i = 0; i < ctx->prof_used[c]; ++i) {
      float t = 0;
      AGX_CUDA(ctx, cudaEventElapsedTime(&t, ctx->prof_ev[c][2 * i], ctx->prof_ev[c][2 * i + 1]));
      tot += t;
    }
    if (ms) ms[c] = tot + ctx->prof_extra_ms[c];
    if (launches) launches[c] = (int64_t)ctx->prof_used[c] + ctx->prof_extra_n[c];
    ctx->prof_used[c] = 0;
    ctx->prof_extra_ms[c] = 0;
    ctx->prof_extra_n[c] = 0;
  }
  return AGX_OK;
}

int agx_launch_count(const agx_context* ctx, int64_t* launches) {
  if (!ctx || !launches) return AGX_ERR_ARG;
  *launches = ctx->n_launches;
  return AGX_OK;
}

int agx_get_sizes(const agx_context* ctx, int64_t* n_dofs, int64_t* nnzb, int* ndof) {
  if (!ctx) return AGX_ERR_ARG;
  if (n_dofs) *n_dofs = ctx->n_dofs;
  if (nnzb) *nnzb = ctx->nnzb;
  if (ndof) *ndof = ctx->ndof;
  return AGX_OK;
}

int agx_spmv(agx_context* ctx, int dtype, const void* x, void* y) {
  if (!ctx || !ctx->pattern_ready) return agx_fail(ctx, AGX_ERR_STATE, "agx_finalize first");
  if (!x || !y) return agx_fail(ctx, AGX_ERR_ARG, "null vector");
  if (ctx->tangent_valid != dtype) return agx_fail(ctx, AGX_ERR_STATE, "no assembled tangent of dtype %d", dtype);
  return agx_spmv_impl(ctx, dtype, x, y);
}

int agx_spmv_values(agx_context* ctx, int dtype, const void* values, const void* x, void* y) {
  if (!ctx || !ctx->pattern_ready) return agx_fail(ctx, AGX_ERR_STATE, "agx_finalize first");
  if (!values || !x || !y) return agx_fail(ctx, AGX_ERR_ARG, "null pointer");
  if (dtype != AGX_F64 && dtype != AGX_F32) return agx_fail(ctx, AGX_ERR_ARG, "dtype must be AGX_F64 or AGX_F32");
  return agx_spmv_values_impl(ctx, dtype, values, x, y);
}

int agx_jacobi(agx_context* ctx, int dtype, const void* r, void* z) {
  if (!ctx || !ctx->pattern_ready) return agx_fail(ctx, AGX_ERR_STATE, "agx_finalize first");
  if (ctx->tangent_valid != dtype) return agx_fail(ctx, AGX_ERR_STATE, "no assembled tangent of dtype %d", dtype);
  if (!r || !z) return agx_fail(ctx, AGX_ERR_ARG, "null pointer");
  agx_launch_jacobi(ctx, dtype, r, z);
  AGX_CHECK_LAUNCH(ctx);
  return AGX_OK;
}

int agx_get_diagonal(agx_context* ctx, int dtype, double* diag) {
  if (!ctx || !ctx->pattern_ready) return agx_fail(ctx, AGX_ERR_STATE, "agx_finalize first");
  if (ctx->tangent_valid != dtype) return agx_fail(ctx, AGX_ERR_STATE, "no assembled tangent of dtype %d", dtype);
  if (!diag) return agx_fail(ctx, AGX_ERR_ARG, "null pointer");
  agx_launch_diagonal(ctx, dtype, diag);
  AGX_CHECK_LAUNCH(ctx);
  return AGX_OK;
}

int agx_copy_values(agx_context* ctx, int dtype, void* values) {
  if (!ctx || !ctx->pattern_ready || !values) return agx_fail(ctx, AGX_ERR_ARG, "bad arguments");
  const size_t bs = (size_t)ctx->ndof * ctx->ndof * ctx->nnzb;
  if (dtype == AGX_F64)
    AGX_CUDA(ctx, cudaMemcpyAsync(values, ctx->d_vals64, sizeof(double) * bs, cudaMemcpyDeviceToDevice, ctx->stream));
  else
    AGX_CUDA(ctx, cudaMemcpyAsync(values, ctx->d_vals32, sizeof(float) * bs, cudaMemcpyDeviceToDevice, ctx->stream));
  return AGX_OK;
}

int agx_set_preconditioner(agx_context* ctx, agx_precond_fn fn, void* user) {
  if (!ctx) return AGX_ERR_ARG;
  ctx->precond = fn;
  ctx->precond_user = user;
  ctx->precond_gen += 1;
  return AGX_OK;
}

int agx_autotune(agx_context* ctx, int* spmv_tpr, float* spmv_ms) {
  if (int rc = check_ready(ctx)) return rc;
  return agx_autotune_spmv(ctx, spmv_tpr, spmv_ms);
}

int agx_set_tuning(agx_context* ctx, int dtype, int spmv_tpr) {
  if (!ctx) return AGX_ERR_ARG;
  if (dtype != AGX_F64 && dtype != AGX_F32) return agx_fail(ctx, AGX_ERR_ARG, "dtype must be AGX_F64 or AGX_F32");
  if (spmv_tpr == SPMV_BRICK) {
    if (ctx->pattern_brick <= 0)
      return agx_fail(ctx, AGX_ERR_ARG, "the brick product (2048) needs the pattern of a structured HEX8 grid "
                                        "with 1 to 3 DOFs per node");
    ctx->spmv_tpr[dtype == AGX_F32 ? 1 : 0] = spmv_tpr;
    return AGX_OK;
  }
  if (spmv_is_grid(spmv_tpr)) {
    if (ctx->pattern_grid_ny <= 0)
      return agx_fail(ctx, AGX_ERR_ARG, "the grid products (512, 1024) need the pattern of a structured QUAD4 grid "
                                        "with 1 or 2 DOFs per node");
    ctx->spmv_tpr[dtype == AGX_F32 ? 1 : 0] = spmv_tpr;
    return AGX_OK;
  }
  const int lanes = spmv_tpr & (SPMV_UNROLL4 - 1), unroll4 = spmv_tpr / SPMV_UNROLL4;
  const bool plain_ok = unroll4 == 0 && (lanes == 0 || lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8 ||
                                          lanes == 16);
  const bool unroll_ok = unroll4 == 1 && (lanes == 2 || lanes == 4 || lanes == 8);
  if (!plain_ok && !unroll_ok)
    return agx_fail(ctx, AGX_ERR_ARG, "lanes per row must be 0, 1, 2, 4, 8 or 16 (2, 4 or 8 with 256 added for four "
                                      "blocks per lane and trip; 512 / 1024 the structured grid's product with one / two rows per lane)");
  if (ctx->ndof == 3 && spmv_tpr != 0 && lanes < 4)
    return agx_fail(ctx, AGX_ERR_ARG, "3 DOFs per node need 4 or more lanes per row");
  ctx->spmv_tpr[dtype == AGX_F32 ? 1 : 0] = spmv_tpr;
  return AGX_OK;
}

int agx_set_pdl(int enable) {
  g_agx_pdl = enable != 0;
  return AGX_OK;
}

int agx_solve_flag(agx_context* ctx, const int** flag) {
  if (!ctx || !flag) return AGX_ERR_ARG;
  if (!ctx->d_scal) return agx_fail(ctx, AGX_ERR_STATE, "no solve state before agx_finalize");
  *flag = &ctx->d_scal->converged;
  return AGX_OK;
}

int agx_grid_pattern(const agx_context* ctx, int* ny) {
  if (!ctx || !ny) return AGX_ERR_ARG;
  *ny = ctx->pattern_grid_ny;
  return AGX_OK;
}

int agx_brick_pattern(const agx_context* ctx, int* code) {
  if (!ctx || !code) return AGX_ERR_ARG;
  *code = ctx->pattern_brick;
  return AGX_OK;
}

int agx_set_preconditioner_mode(agx_context* ctx, int mode, double omega, int sweeps, int flags) {
  if (!ctx || mode < 0 || mode > 3) return agx_fail(ctx, AGX_ERR_ARG, "preconditioner mode must be 0 .. 3");
  if (!(omega > 0.0 && omega < (mode == 3 ? 1.0 : 1.0000001)))
    return agx_fail(ctx, AGX_ERR_ARG, mode == 3 ? "the Chebyshev interval fraction must lie in (0, 1)"
                                               : "Jacobi damping must lie in (0, 1]");
  if (sweeps < 1 || sweeps > 16) return agx_fail(ctx, AGX_ERR_ARG, "smoothing sweeps must lie in 1 .. 16");
  if (flags & ~(AGX_PRECOND_CAPTURABLE | AGX_PRECOND_BF16_SMOOTHING))
    return agx_fail(ctx, AGX_ERR_ARG, "unknown preconditioner flags");
  ctx->precond_mode = mode;
  ctx->precond_omega = omega;
  ctx->precond_sweeps = sweeps;
  ctx->precond_capturable = (flags & AGX_PRECOND_CAPTURABLE) != 0;
  ctx->precond_bf16 = (flags & AGX_PRECOND_BF16_SMOOTHING) != 0;
  ctx->precond_gen += 1;
  return AGX_OK;
}

int agx_solve(agx_context* ctx, const double* rhs, double* x, const agx_solve_opts* opts, agx_solve_info* info) {
  if (int rc = check_ready(ctx)) return rc;
  if (!rhs || !x || !opts) return agx_fail(ctx, AGX_ERR_ARG, "null argument");
  // the solve acts on the free DOFs: prescribed rows of rhs are ignored (solver.py:1514-1517)
  agx_launch_masked_scale(ctx, rhs, ctx->d_b, 1.0);
  agx_solve_info local{};
  int rc = agx_krylov_impl(ctx, ctx->d_b, x, opts, &local);
  if (rc) return rc;
  AGX_CHECK_LAUNCH(ctx);
  AGX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (info) *info = local;
  return local.status;
}

int agx_newton(agx_context* ctx, double* dofs, const double* dvals, const agx_newton_opts* opts, agx_newton_info* info) {
  if (int rc = check_ready(ctx)) return rc;
  if (!dofs || !dvals || !opts) return agx_fail(ctx, AGX_ERR_ARG, "null argument");
  const int tdt = opts->tangent_dtype;
  const int kry = opts->krylov.method;
  if ((kry == AGX_PCG || kry == AGX_BICGSTAB || kry == AGX_CHOL_BAND || kry == AGX_FCG_F64) && tdt != AGX_F64)
    return agx_fail(ctx, AGX_ERR_ARG, "PCG, BiCGStab, float64 FCG and the banded Cholesky solve need a float64 tangent");
  if ((kry == AGX_PCG_MIXED || kry == AGX_FCG_MIXED) && tdt != AGX_F32)
    return agx_fail(ctx, AGX_ERR_ARG, "mixed methods need a float32 tangent");
  agx_newton_info out{};
  int itt = 0;
  double res_old = 0.0, res = 0.0;
  bool not_stop = true, div = false, have_R = false, have_K = false;
  double tol = opts->newton_tol;
  while (not_stop) {
    // solve_linear: impose the prescribed values, rhs = -R, tangent, solve (solver.py:586-659)
    agx_launch_set_dirichlet(ctx, dofs, dvals);
    AGX_CHECK_LAUNCH(ctx);
    const bool need_K = !(opts->reuse_tangent && have_K && ctx->tangent_valid == tdt);
    int rc = AGX_OK;
    if (need_K) rc = agx_assemble_impl(ctx, dofs, have_R ? nullptr : ctx->d_R, tdt);
    else if (!have_R) rc = agx_assemble_impl(ctx, dofs, ctx->d_R, -1);
    if (rc) return rc;
    have_K = true;
    if (itt == 0) {
      double n0 = 0, nf0 = 0;
      rc = agx_residual_norm(ctx, ctx->d_R, &n0, &nf0);
      if (rc) return rc;
      out.res0 = std::sqrt(n0);
      if (opts->newton_rtol > 0.0) tol = std::max(tol, opts->newton_rtol * out.res0);
    }
    agx_launch_negate_free(ctx, ctx->d_R, ctx->d_b);
    agx_solve_info si{};
    rc = agx_krylov_impl(ctx, ctx->d_b, ctx->d_dx, &opts->krylov, &si);
    if (rc) return rc;
    out.krylov_iterations += si.iterations;
    if (kry == AGX_CHOL_BAND && si.status == AGX_DIVERGED) {
      // the tangent is not definite: no Newton step exists from this factorization; stop with
      // the diverged flag (the reference's LU would take an indefinite step)
      out.iterations = itt + 1;
      out.res_norm = res;
      out.diverged = 1;
      if (info) *info = out;
      return AGX_OK;
    }
    // damped update of the free DOFs, prescribed DOFs set (solver.py:879-892)
    agx_launch_newton_update(ctx, dofs, ctx->d_dx, dvals, opts->damping);
    // residual for the convergence test (solver.py:898-903); reused as next iteration's rhs
    rc = agx_assemble_impl(ctx, dofs, ctx->d_R, -1);
    if (rc) return rc;
    have_R = true;
    double n2 = 0, nonfinite = 0;
    rc = agx_residual_norm(ctx, ctx->d_R, &n2, &nonfinite);
    if (rc) return rc;
    res = std::sqrt(n2);
    const bool keep = res > tol;
    bool next_step;
    if (itt < opts->maxiter) {
      if (opts->verbose > 0) printf("Residual after Newton iteration %d: %.17g\n", itt + 1, res);
      div = (itt > 1) && (res_old > 0.0 ? res / res_old > 10.0 : res > 0.0);
      if (nonfinite > 0 || !std::isfinite(res)) div = true;
      next_step = !div;
    } else {
      // the reference prints this warning (solver.py:926-927); a library writes it to stderr so
      // that it cannot interleave with a caller's output on stdout
      fprintf(stderr, "Warning: Newton scheme could not converge!\n");
      next_step = false;
      div = true;
    }
    if (out.n_history < AGX_MAX_HISTORY) {
      out.res_history[out.n_history] = res;
      out.krylov_history[out.n_history] = si.iterations;
      out.n_history++;
    }
    itt += 1;
    res_old = res;
    not_stop = keep && next_step;
  }
  out.iterations = itt;
  out.res_norm = res;
  out.diverged = div ? 1 : 0;
  if (info) *info = out;
  return AGX_OK;
}

}  // extern "C"
