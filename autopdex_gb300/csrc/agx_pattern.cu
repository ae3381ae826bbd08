// Node-block CSR (BSR) pattern of the tangent and the element -> pattern scatter map.
//
// AutoPDEx keeps the tangent as a BCOO with one entry per element-matrix entry
// (assembler.py:1142-1148, indices from _get_indices, assembler.py:47-141) and sums the
// duplicates on the host in every Newton step (scipy_assembling, solver.py:1180-1222).
// Here the pattern is built once per mesh: row p holds every node that shares an element
// with node p (sorted), each row/column entry is an ndof x ndof block, and for every
// element and local node pair (a, b) the position of block (conn[a], conn[b]) is stored,
// so that assembly adds element blocks straight into their final slots.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>

#include "agx_common.cuh"

namespace {

template <class F>
void parallel_for(int64_t n, F&& f) {
  unsigned hw = std::thread::hardware_concurrency();
  int nt = (int)std::min<int64_t>(std::max(1u, hw), std::max<int64_t>(1, n / 4096));
  if (nt <= 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  int64_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    int64_t b = t * chunk, e = std::min<int64_t>(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([&f, b, e] { f(b, e); });
  }
  for (auto& t : th) t.join();
}

// A QUAD4 set that is the mesher's structured nx x ny grid over all nodes, with every pattern
// row the in-range 3 x 3 stencil of its node: then a node row's entries, in column order, are
// its stencil neighbours in (di, dj) order, and the tangent can be assembled row by row.
void detect_structured_grid(agx_context* ctx, agx_element_set& s, const std::vector<int32_t>& rowptr) {
  s.grid_nx = s.grid_ny = 0;
  if (s.elem_type != AGX_QUAD4 || ctx->dim != 2 || s.n_elem < 1) return;
  const int32_t* c = s.h_conn.data();
  const int64_t ny = (int64_t)c[3] - 1;
  if (ny < 1 || s.n_elem % ny) return;
  const int64_t nx = s.n_elem / ny;
  if ((nx + 1) * (ny + 1) != ctx->n_nodes) return;
  for (int64_t i = 0; i < nx; ++i)
    for (int64_t j = 0; j < ny; ++j) {
      const int32_t* e = c + (i * ny + j) * 4;
      const int64_t n00 = i * (ny + 1) + j;
      if (e[0] != n00 || e[1] != n00 + 1 || e[2] != n00 + ny + 2 || e[3] != n00 + ny + 1) return;
    }
  for (int64_t i = 0; i <= nx; ++i)
    for (int64_t j = 0; j <= ny; ++j) {
      const int64_t ri = (i > 0) + 1 + (i < nx), rj = (j > 0) + 1 + (j < ny);
      const int64_t p = i * (ny + 1) + j;
      if (rowptr[p + 1] - rowptr[p] != ri * rj) return;
    }
  s.grid_nx = (int)nx;
  s.grid_ny = (int)ny;
  // parallelograms (x0 + x2 = x1 + x3 to float64 rounding, the row kernel's own test): the
  // row kernel then takes the one-Jacobian integral for every element without testing
  s.grid_affine = true;
  const double* X = ctx->h_coords.data();
  for (int64_t e = 0; e < s.n_elem && s.grid_affine; ++e) {
    const int32_t* n = c + e * 4;
    const double* x0 = X + 2 * (int64_t)n[0];
    const double* x1 = X + 2 * (int64_t)n[1];
    const double* x2 = X + 2 * (int64_t)n[2];
    const double* x3 = X + 2 * (int64_t)n[3];
    const double ex = x0[0] + x2[0] - x1[0] - x3[0], ey = x0[1] + x2[1] - x1[1] - x3[1];
    const double scale =
        std::fabs(x2[0] - x0[0]) + std::fabs(x2[1] - x0[1]) + std::fabs(x1[0] - x3[0]) + std::fabs(x1[1] - x3[1]);
    s.grid_affine = std::fabs(ex) + std::fabs(ey) <= scale * 1e-13;
  }
  // one parallelogram for the whole grid: the element matrices differ only by their coefficient
  s.grid_uniform = false;
  if (s.grid_affine) {
    auto edges = [&](int64_t e, double* v) {
      const int32_t* n = c + e * 4;
      const double* x0 = X + 2 * (int64_t)n[0];
      const double* x1 = X + 2 * (int64_t)n[1];
      const double* x3 = X + 2 * (int64_t)n[3];
      v[0] = x1[0] - x0[0], v[1] = x1[1] - x0[1], v[2] = x3[0] - x0[0], v[3] = x3[1] - x0[1];
    };
    double r[4];
    edges(0, r);
    const double size = std::fabs(r[0]) + std::fabs(r[1]) + std::fabs(r[2]) + std::fabs(r[3]);
    bool uni = size > 0.0;
    for (int64_t e = 1; e < s.n_elem && uni; ++e) {
      double v[4];
      edges(e, v);
      uni = std::fabs(v[0] - r[0]) + std::fabs(v[1] - r[1]) + std::fabs(v[2] - r[2]) + std::fabs(v[3] - r[3]) <=
            size * 1e-14;
    }
    if (uni) {
      // J = (1/2) [x1 - x0 | x3 - x0] (mesher's node order), as the element kernels form it
      const double J00 = 0.5 * r[0], J01 = 0.5 * r[2], J10 = 0.5 * r[1], J11 = 0.5 * r[3];
      const double det = J00 * J11 - J01 * J10;
      s.grid_uniform = det != 0.0;
      s.grid_m[0] = (J11 * J11 + J01 * J01) / det;
      s.grid_m[1] = -(J11 * J10 + J01 * J00) / det;
      s.grid_m[2] = (J10 * J10 + J00 * J00) / det;
      s.grid_m[3] = det;
    }
  }
}

// A HEX8 set that is the mesher's structured nx x ny x nz brick grid over all nodes (element
// (i ny + j) nz + k with local nodes (i,j,k), (i+1,j,k), (i+1,j+1,k), (i,j+1,k), then the same
// at k + 1; node (i, j, k) = (i (ny + 1) + j)(nz + 1) + k), every pattern row the in-range
// 27-node stencil; uniform when every node is x0 + i e1 + j e2 + k e3 (to 1e-13 of the grid's
// extent): then J = [e1 | e2 | e3] / 2 for every element.
void detect_structured_brick(agx_context* ctx, agx_element_set& s, const std::vector<int32_t>& rowptr) {
  s.brick_n[0] = s.brick_n[1] = s.brick_n[2] = 0;
  s.brick_uniform = false;
  if (s.elem_type != AGX_HEX8 || ctx->dim != 3 || s.n_elem < 1) return;
  const int32_t* c = s.h_conn.data();
  if (c[0] != 0 || c[4] != 1) return;
  const int64_t nz = (int64_t)c[3] - 1;
  if (nz < 1 || c[1] % (nz + 1)) return;
  const int64_t ny = (int64_t)c[1] / (nz + 1) - 1;
  if (ny < 1 || s.n_elem % (ny * nz)) return;
  const int64_t nx = s.n_elem / (ny * nz);
  const int64_t sa = (ny + 1) * (nz + 1), sb = nz + 1;
  if ((nx + 1) * sa != ctx->n_nodes) return;
  std::atomic<bool> conn_ok{true};  // written by the host threads of parallel_for
  parallel_for(nx, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e && conn_ok.load(std::memory_order_relaxed); ++i)
      for (int64_t j = 0; j < ny; ++j)
        for (int64_t k = 0; k < nz; ++k) {
          const int32_t* el = c + ((i * ny + j) * nz + k) * 8;
          const int64_t n0 = i * sa + j * sb + k;
          if (el[0] != n0 || el[1] != n0 + sa || el[2] != n0 + sa + sb || el[3] != n0 + sb || el[4] != n0 + 1 ||
              el[5] != n0 + sa + 1 || el[6] != n0 + sa + sb + 1 || el[7] != n0 + sb + 1) {
            conn_ok.store(false, std::memory_order_relaxed);
            return;
          }
        }
  });
  if (!conn_ok.load()) return;
  bool ok = true;
  for (int64_t i = 0; i <= nx && ok; ++i)
    for (int64_t j = 0; j <= ny && ok; ++j)
      for (int64_t k = 0; k <= nz; ++k) {
        const int64_t len = ((i > 0) + 1 + (i < nx)) * ((j > 0) + 1 + (j < ny)) * ((k > 0) + 1 + (k < nz));
        const int64_t p = i * sa + j * sb + k;
        if (rowptr[p + 1] - rowptr[p] != len) {
          ok = false;
          break;
        }
      }
  if (!ok) return;
  s.brick_n[0] = (int)nx, s.brick_n[1] = (int)ny, s.brick_n[2] = (int)nz;
  const double* X = ctx->h_coords.data();
  double e[3][3], ext = 0.0;
  for (int d = 0; d < 3; ++d) {
    e[0][d] = X[3 * sa + d] - X[d];
    e[1][d] = X[3 * sb + d] - X[d];
    e[2][d] = X[3 * 1 + d] - X[d];
    ext += std::fabs(e[0][d]) * nx + std::fabs(e[1][d]) * ny + std::fabs(e[2][d]) * nz;
  }
  bool uni = ext > 0.0;
  for (int64_t i = 0; i <= nx && uni; ++i)
    for (int64_t j = 0; j <= ny && uni; ++j)
      for (int64_t k = 0; k <= nz; ++k) {
        const double* x = X + 3 * (i * sa + j * sb + k);
        double dev = 0.0;
        for (int d = 0; d < 3; ++d) dev += std::fabs(x[d] - (X[d] + i * e[0][d] + j * e[1][d] + k * e[2][d]));
        if (dev > 1e-13 * ext) {
          uni = false;
          break;
        }
      }
  if (!uni) return;
  // J[d][m] = e_m[d] / 2; (J^T J)^-1 by the adjugate of the Gram matrix
  double G[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) G[a][b] = 0.25 * (e[a][0] * e[b][0] + e[a][1] * e[b][1] + e[a][2] * e[b][2]);
  const double det = 0.125 * (e[0][0] * (e[1][1] * e[2][2] - e[2][1] * e[1][2]) -
                              e[1][0] * (e[0][1] * e[2][2] - e[2][1] * e[0][2]) +
                              e[2][0] * (e[0][1] * e[1][2] - e[1][1] * e[0][2]));
  const double g = det * det;  // det(J^T J)
  if (!(g > 0.0)) return;
  s.brick_m[0] = (G[1][1] * G[2][2] - G[1][2] * G[2][1]) / g;
  s.brick_m[1] = (G[0][2] * G[2][1] - G[0][1] * G[2][2]) / g;
  s.brick_m[2] = (G[0][1] * G[1][2] - G[0][2] * G[1][1]) / g;
  s.brick_m[3] = (G[0][0] * G[2][2] - G[0][2] * G[2][0]) / g;
  s.brick_m[4] = (G[0][2] * G[1][0] - G[0][0] * G[1][2]) / g;
  s.brick_m[5] = (G[0][0] * G[1][1] - G[0][1] * G[1][0]) / g;
  s.brick_det = det;
  s.brick_uniform = true;
}

}  // namespace

int agx_build_pattern(agx_context* ctx) {
  const int64_t nn = ctx->n_nodes;
  // node -> (set, element) incidence, counting sort
  std::vector<int64_t> inc_ptr(nn + 1, 0);
  for (auto& s : ctx->sets)
    for (int64_t i = 0; i < s.n_elem * s.nen; ++i) inc_ptr[s.h_conn[i] + 1]++;
  for (int64_t p = 0; p < nn; ++p) inc_ptr[p + 1] += inc_ptr[p];
  std::vector<int64_t> inc(inc_ptr[nn]);   // encoded (set << 40) | element
  {
    std::vector<int64_t> fill(inc_ptr.begin(), inc_ptr.end() - 1);
    for (size_t si = 0; si < ctx->sets.size(); ++si) {
      auto& s = ctx->sets[si];
      for (int64_t e = 0; e < s.n_elem; ++e)
        for (int a = 0; a < s.nen; ++a) {
          int32_t p = s.h_conn[e * s.nen + a];
          inc[fill[p]++] = ((int64_t)si << 40) | e;
        }
    }
  }
  // neighbours of every node: sorted unique union of the nodes of its elements
  std::vector<int32_t> row_len(nn);
  auto neighbours = [&](int64_t p, std::vector<int32_t>& buf) {
    buf.clear();
    for (int64_t k = inc_ptr[p]; k < inc_ptr[p + 1]; ++k) {
      auto& s = ctx->sets[inc[k] >> 40];
      int64_t e = inc[k] & ((1LL << 40) - 1);
      for (int b = 0; b < s.nen; ++b) buf.push_back(s.h_conn[e * s.nen + b]);
    }
    buf.push_back((int32_t)p);  // keep the diagonal even for nodes outside every element
    std::sort(buf.begin(), buf.end());
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
  };
  parallel_for(nn, [&](int64_t b, int64_t e) {
    std::vector<int32_t> buf;
    for (int64_t p = b; p < e; ++p) {
      neighbours(p, buf);
      row_len[p] = (int32_t)buf.size();
    }
  });
  std::vector<int32_t> rowptr(nn + 1, 0);
  int64_t acc = 0;
  for (int64_t p = 0; p < nn; ++p) {
    rowptr[p] = (int32_t)acc;
    acc += row_len[p];
    if (acc > INT32_MAX) return agx_fail(ctx, AGX_ERR_UNSUPPORTED, "pattern exceeds 2^31 blocks");
  }
  rowptr[nn] = (int32_t)acc;
  ctx->nnzb = acc;
  std::vector<int32_t> col(acc), diagpos(nn);
  parallel_for(nn, [&](int64_t b, int64_t e) {
    std::vector<int32_t> buf;
    for (int64_t p = b; p < e; ++p) {
      neighbours(p, buf);
      std::copy(buf.begin(), buf.end(), col.begin() + rowptr[p]);
      diagpos[p] = rowptr[p] + (int32_t)(std::lower_bound(buf.begin(), buf.end(), (int32_t)p) - buf.begin());
    }
  });
  // element scatter maps
  std::vector<std::vector<int32_t>> epos(ctx->sets.size());
  for (size_t si = 0; si < ctx->sets.size(); ++si) {
    auto& s = ctx->sets[si];
    auto& ep = epos[si];
    ep.resize((size_t)s.n_elem * s.nen * s.nen);
    parallel_for(s.n_elem, [&](int64_t b, int64_t e) {
      for (int64_t el = b; el < e; ++el)
        for (int a = 0; a < s.nen; ++a) {
          int32_t p = s.h_conn[el * s.nen + a];
          const int32_t* rb = col.data() + rowptr[p];
          const int32_t* re = col.data() + rowptr[p + 1];
          for (int c = 0; c < s.nen; ++c) {
            int32_t q = s.h_conn[el * s.nen + c];
            ep[(el * s.nen + a) * s.nen + c] = rowptr[p] + (int32_t)(std::lower_bound(rb, re, q) - rb);
          }
        }
    });
  }
  ctx->pattern_grid_ny = 0;
  ctx->pattern_brick = 0;
  for (auto& s : ctx->sets) {
    detect_structured_grid(ctx, s, rowptr);
    detect_structured_brick(ctx, s, rowptr);
    // the row lengths matched the grid's stencil: every other set's entries lie inside it
    if (s.grid_nx > 0 && ctx->ndof <= 2) ctx->pattern_grid_ny = s.grid_ny;
    if (s.brick_n[0] > 0 && ctx->ndof <= 3 && s.brick_n[1] < 32768 && s.brick_n[2] < 65536)
      ctx->pattern_brick = (s.brick_n[1] << 16) | s.brick_n[2];
  }
  ctx->pattern_stencil = ctx->pattern_grid_ny > 0 ? ctx->pattern_grid_ny : ctx->pattern_brick;
  // upload
  const int bs = ctx->ndof * ctx->ndof;
  AGX_CUDA(ctx, cudaMalloc(&ctx->d_rowptr, sizeof(int32_t) * (nn + 1)));
  AGX_CUDA(ctx, cudaMalloc(&ctx->d_col, sizeof(int32_t) * std::max<int64_t>(1, acc)));
  AGX_CUDA(ctx, cudaMalloc(&ctx->d_diagpos, sizeof(int32_t) * nn));
  AGX_CUDA(ctx, cudaMalloc(&ctx->d_vals64, sizeof(double) * std::max<int64_t>(1, acc * bs)));
  AGX_CUDA(ctx, cudaMalloc(&ctx->d_vals32, sizeof(float) * std::max<int64_t>(1, acc * bs)));
  AGX_CUDA(ctx, cudaMemcpy(ctx->d_rowptr, rowptr.data(), sizeof(int32_t) * (nn + 1), cudaMemcpyHostToDevice));
  AGX_CUDA(ctx, cudaMemcpy(ctx->d_col, col.data(), sizeof(int32_t) * acc, cudaMemcpyHostToDevice));
  AGX_CUDA(ctx, cudaMemcpy(ctx->d_diagpos, diagpos.data(), sizeof(int32_t) * nn, cudaMemcpyHostToDevice));
  for (size_t si = 0; si < ctx->sets.size(); ++si) {
    auto& s = ctx->sets[si];
    size_t n = epos[si].size();
    AGX_CUDA(ctx, cudaMalloc(&s.d_epos, sizeof(int32_t) * std::max<size_t>(1, n)));
    AGX_CUDA(ctx, cudaMemcpy(s.d_epos, epos[si].data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
  }
  ctx->pattern_ready = true;
  return AGX_OK;
}
