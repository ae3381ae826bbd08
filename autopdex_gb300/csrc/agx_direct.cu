// Banded Cholesky direct solve of the float64 tangent (AGX_CHOL_BAND).
//
// Replaces the sparse direct solve of the 'scipy' backend -- scipy.sparse.linalg.spsolve of the
// reduced CSR matrix (solver.py:1493-1539 with 'lapack'; 'umfpack' at :1522) -- on meshes whose
// node numbering keeps the matrix in a narrow band, as the mesher's structured grids do (node
// (i, j) = i (ny + 1) + j, mesher.py:88-94): the 200^2 Poisson mesh has a half bandwidth of 202
// DOFs, the 512^2 Cook membrane (2 DOFs per node) 1029.  Tangents of potentials and of
// hyperelastic elements are symmetric and definite; on the clockwise quads of the mesher they
// are negative definite, and the factor is then the one of -K.
//
// Layout: the lower band by columns, entry (j + k, j) at band[j (w + 1) + k], k = 0 .. w.  The
// entries of a column are contiguous, so every kernel below loads consecutive rows of one
// column with consecutive lanes.
//
// Factorization: right-looking in panels of NB = 32 columns.  For each panel, panel_factor
// factors the NB x NB diagonal block in shared memory (every CTA, redundantly; CTA 0 leaves the
// result in a scratch block) and solves one row of the w x NB block below per thread
// (L21 = A21 L11^-T); syrk_update then subtracts L21 L21^T from the w x w lower triangle that
// follows, in 16 x 16 to 64 x 64 tiles (whichever leaves the busiest SM the least float64 work),
// and copies the diagonal block from the scratch into the band.
// Work: about n w^2 float64 flops (0.56 TFLOP for the 512^2 membrane).
// Solves: one CTA walks blocks of NB rows -- forward substitution with column updates of the
// rows below, backward substitution with per-column dot products of the rows below -- and the
// result is refined with the float64 product until ||b - K x|| <= rtol ||b|| (at most three
// steps, fewer once a step no longer halves the residual).
#include <algorithm>
#include <cmath>
#include <vector>

#include "agx_common.cuh"

namespace {

constexpr int NB = 32;   // panel width
constexpr int PF_THREADS = 64;  // rows of the block below the diagonal block per CTA
constexpr int SOLVE_THREADS = 1024;

__host__ __device__ __forceinline__ int64_t imin(int64_t a, int64_t b) { return a < b ? a : b; }

// 1 / sqrt(d) for a positive float64 pivot: a float32 estimate refined by two steps of the
// Newton-Raphson iteration y <- y (3 - d y^2) / 2 for the reciprocal square root (each step
// roughly squares the relative error: ~1e-7 -> ~1e-14 -> rounding level).  GB300 runs float64 at
// 1/64 of its float32 rate, and the pivots of a band factorization form a sequential chain, so
// this replaces a float64 square root and a float64 division per column.  Outside the float32
// range the float64 square root is used instead.
__device__ __forceinline__ double pivot_rsqrt(double d) {
  if (!(d > 1e-30 && d < 1e30)) return 1.0 / sqrt(d);
  double y = (double)rsqrtf((float)d);
  y = y * (1.5 - 0.5 * d * y * y);
  y = y * (1.5 - 0.5 * d * y * y);
  return y;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// band from the node-block CSR tangent (Dirichlet rows and columns already eliminated):
// sign * K, with the identity diagonal of prescribed DOFs kept at +1
template <int ND>
__global__ void band_build(int64_t n_nodes, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const double* __restrict__ vals, int64_t nnzb, const uint8_t* __restrict__ dmask,
                           int64_t w, double sign, double* __restrict__ band) {
  const int64_t ld = w + 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes; i += (int64_t)gridDim.x * blockDim.x) {
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int64_t j = col[k];
      if (j > i) continue;
#pragma unroll
      for (int a = 0; a < ND; ++a)
#pragma unroll
        for (int b = 0; b < ND; ++b) {
          const int64_t r = i * ND + a, c = j * ND + b;
          if (r < c || r - c > w) continue;
          const double v = vals[(int64_t)(a * ND + b) * nnzb + k];
          band[c * ld + (r - c)] = (r == c && dmask[r]) ? 1.0 : sign * v;
        }
    }
  }
}

// counts of positive and negative diagonal entries of the free DOFs
__global__ void diag_signs(int64_t n_dofs, int ndof, int64_t nnzb, const int32_t* __restrict__ diagpos,
                           const double* __restrict__ vals, const uint8_t* __restrict__ dmask,
                           unsigned long long* __restrict__ counts) {
  unsigned long long pos = 0, neg = 0;
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n_dofs; d += (int64_t)gridDim.x * blockDim.x) {
    if (dmask[d]) continue;
    const int64_t p = d / ndof;
    const int c = (int)(d - p * ndof);
    const double v = vals[(int64_t)(c * ndof + c) * nnzb + diagpos[p]];
    pos += v > 0.0;
    neg += v < 0.0;
  }
  if (pos) atomicAdd(counts, pos);
  if (neg) atomicAdd(counts + 1, neg);
}

// Factor of the diagonal block of panel j0 (nbp columns) and the rows below it.
__global__ void __launch_bounds__(PF_THREADS)
panel_factor(double* __restrict__ band, int64_t n, int64_t w, int64_t j0, int nbp, double* __restrict__ l11,
             double* __restrict__ rdiag, int* __restrict__ err) {
  __shared__ double L[NB][NB + 1];
  __shared__ double rinv[NB];  // reciprocals of the pivots L_qq (0 past a partial last panel)
  const int64_t ld = w + 1;
  if (threadIdx.x < NB) rinv[threadIdx.x] = 0.0;
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int i = idx / NB, q = idx % NB;
    L[i][q] = (q <= i && i < nbp && (int64_t)(i - q) <= w) ? band[(j0 + q) * ld + (i - q)] : 0.0;
  }
  __syncthreads();
  for (int q = 0; q < nbp; ++q) {
    if (threadIdx.x == 0) {
      double d = L[q][q];
      if (!(d > 0.0) || !isfinite(d)) {  // not positive definite: record the column, continue with 1
        if (blockIdx.x == 0) atomicCAS(err, 0, (int)(j0 + q + 1));
        d = 1.0;
      }
      const double y = pivot_rsqrt(d);
      L[q][q] = d * y;
      rinv[q] = y;
    }
    __syncthreads();
    const double ri = rinv[q];
    for (int i = q + 1 + threadIdx.x; i < nbp; i += blockDim.x) L[i][q] *= ri;
    __syncthreads();
    const int m = nbp - q - 1;
    for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
      const int i = q + 1 + t / m, c = q + 1 + t % m;
      if (c <= i) L[i][c] -= L[i][q] * L[c][q];
    }
    __syncthreads();
  }
  if (blockIdx.x == 0) {
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) l11[idx] = L[idx / NB][idx % NB];
    if (threadIdx.x < nbp) rdiag[j0 + threadIdx.x] = rinv[threadIdx.x];
  }
  // one row of L21 per thread: x L11^T = a  (rows r = j0 + nbp + R, R < w)
  const int64_t R = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t r = j0 + nbp + R;
  if (R >= w || r >= n) return;
  double x[NB];
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int64_t off = nbp + R - q;
    x[q] = (q < nbp && off <= w) ? band[(j0 + q) * ld + off] : 0.0;
  }
  // right-looking: once x_q is final it updates every later x_p; each x_p subtracts the same
  // terms in the same order (q = 0 .. p-1) as a row-by-row solve would, but consecutive FMAs
  // go to different accumulators, so the float64 latency overlaps instead of forming one
  // chain of NB (NB - 1) / 2 dependent FMAs.  Columns past a partial last panel are zero in
  // x and L and have rinv = 0, so the loop needs no bound.
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    x[q] *= rinv[q];
#pragma unroll
    for (int p = q + 1; p < NB; ++p) x[p] -= x[q] * L[p][q];
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int64_t off = nbp + R - q;
    if (q < nbp && off <= w) band[(j0 + q) * ld + off] = x[q];
  }
}

// A22 -= L21 L21^T on the w x w lower triangle after panel j0, in TM x TM tiles (TM = 16, 32 or
// 64: the largest that still gives every SM a tile, since the update is bound by each SM's float64
// rate); CTA 0 also stores the factored diagonal block (kept in l11 by panel_factor so that no CTA
// of that kernel read it half-written)
template <int TM>
__global__ void __launch_bounds__(256)
syrk_update(double* __restrict__ band, int64_t n, int64_t w, int64_t j0, int nbp, const double* __restrict__ l11) {
  constexpr int R = TM / 16;  // a thread's R x R accumulators
  const int64_t ld = w + 1;
  if (blockIdx.x == 0)
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
      const int i = idx / NB, q = idx % NB;
      if (q <= i && i < nbp && (int64_t)(i - q) <= w) band[(j0 + q) * ld + (i - q)] = l11[idx];
    }
  // tile (ti, tj), ti >= tj, of the lower triangle
  const int64_t b = blockIdx.x;
  int64_t ti = (int64_t)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while (ti * (ti + 1) / 2 > b) --ti;
  while ((ti + 1) * (ti + 2) / 2 <= b) ++ti;
  const int64_t tj = b - ti * (ti + 1) / 2;
  __shared__ double Xa[NB][TM + 1], Xb[NB][TM + 1];
  for (int idx = threadIdx.x; idx < NB * TM; idx += blockDim.x) {
    const int q = idx / TM, rr = idx % TM;
    const int64_t Ra = ti * TM + rr, Rb = tj * TM + rr;
    const int64_t oa = nbp + Ra - q, ob = nbp + Rb - q;
    Xa[q][rr] = (q < nbp && Ra < w && j0 + nbp + Ra < n && oa <= w) ? band[(j0 + q) * ld + oa] : 0.0;
    Xb[q][rr] = (q < nbp && Rb < w && j0 + nbp + Rb < n && ob <= w) ? band[(j0 + q) * ld + ob] : 0.0;
  }
  __syncthreads();
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[R][R] = {};
#pragma unroll 8
  for (int q = 0; q < NB; ++q) {
    double a[R], bb[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
      a[u] = Xa[q][tx + 16 * u];
      bb[u] = Xb[q][ty + 16 * u];
    }
#pragma unroll
    for (int u = 0; u < R; ++u)
#pragma unroll
      for (int v = 0; v < R; ++v) acc[u][v] += a[u] * bb[v];
  }
#pragma unroll
  for (int u = 0; u < R; ++u)
#pragma unroll
    for (int v = 0; v < R; ++v) {
      const int64_t Rr = ti * TM + tx + 16 * u, Cc = tj * TM + ty + 16 * v;
      if (Rr < w && Cc <= Rr && j0 + nbp + Rr < n) band[(j0 + nbp + Cc) * ld + (Rr - Cc)] -= acc[u][v];
    }
}

// v <- L^-1 v (one CTA)
__global__ void __launch_bounds__(SOLVE_THREADS) band_forward(const double* __restrict__ band,
                                                              const double* __restrict__ rdiag, int64_t n, int64_t w,
                                                              double* __restrict__ v) {
  __shared__ double L[NB][NB + 1];
  __shared__ double y[NB];
  const int64_t ld = w + 1;
  const int lane = threadIdx.x & 31;
  for (int64_t j0 = 0; j0 < n; j0 += NB) {
    const int nbp = (int)imin(NB, n - j0);
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
      const int i = idx / NB, q = idx % NB;
      L[i][q] = (q <= i && i < nbp && (int64_t)(i - q) <= w) ? band[(j0 + q) * ld + (i - q)] : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      // the block's pivot reciprocals in registers before the sequential chain (a global load
      // inside it would put one memory latency on every step)
      const double rd = lane < nbp ? rdiag[j0 + lane] : 1.0;
      double yi = lane < nbp ? v[j0 + lane] : 0.0;
      for (int q = 0; q < nbp; ++q) {
        if (lane == q) yi *= rd;
        const double yq = __shfl_sync(0xffffffffu, yi, q);
        if (lane > q && lane < nbp) yi -= L[lane][q] * yq;
      }
      if (lane < nbp) {
        y[lane] = yi;
        v[j0 + lane] = yi;
      }
    }
    __syncthreads();
    for (int64_t R = threadIdx.x; R < w; R += blockDim.x) {
      const int64_t r = j0 + nbp + R;
      if (r >= n) break;
      double s4[4] = {0.0, 0.0, 0.0, 0.0};  // four partial sums: short float64 dependency chains
#pragma unroll
      for (int q = 0; q < NB; ++q) {
        const int64_t off = nbp + R - q;
        if (q < nbp && off <= w) s4[q & 3] += band[(j0 + q) * ld + off] * y[q];
      }
      v[r] -= (s4[0] + s4[1]) + (s4[2] + s4[3]);
    }
    __syncthreads();
  }
}

// v <- L^-T v (one CTA)
__global__ void __launch_bounds__(SOLVE_THREADS) band_backward(const double* __restrict__ band,
                                                               const double* __restrict__ rdiag, int64_t n, int64_t w,
                                                               double* __restrict__ v) {
  __shared__ double L[NB][NB + 1];
  __shared__ double s[NB];
  const int64_t ld = w + 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nblk = (n + NB - 1) / NB;
  for (int64_t bk = nblk - 1; bk >= 0; --bk) {
    const int64_t j0 = bk * NB;
    const int nbp = (int)imin(NB, n - j0);
    if (warp < nbp) {  // column c = j0 + warp: dot of its entries below the block with v
      const int64_t c = j0 + warp;
      const int64_t rend = imin(n, c + w + 1);
      double acc = 0.0;
      for (int64_t r = j0 + nbp + lane; r < rend; r += 32) acc += band[c * ld + (r - c)] * v[r];
      acc = warp_sum_d(acc);
      if (lane == 0) s[warp] = acc;
    }
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
      const int i = idx / NB, q = idx % NB;
      L[i][q] = (q <= i && i < nbp && (int64_t)(i - q) <= w) ? band[(j0 + q) * ld + (i - q)] : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      const double rd = lane < nbp ? rdiag[j0 + lane] : 1.0;
      double xi = lane < nbp ? v[j0 + lane] - s[lane] : 0.0;
      for (int q = nbp - 1; q >= 0; --q) {
        if (lane == q) xi *= rd;
        const double xq = __shfl_sync(0xffffffffu, xi, q);
        if (lane < q) xi -= L[q][lane] * xq;
      }
      if (lane < nbp) v[j0 + lane] = xi;
    }
    __syncthreads();
  }
}

// dst = sign * src
__global__ void scale_copy(int64_t n, const double* src, double* dst, double sign) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = sign * src[i];
}

// r = b - y
__global__ void residual_of(int64_t n, const double* __restrict__ b, const double* __restrict__ y,
                            double* __restrict__ r) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    r[i] = b[i] - y[i];
}

// x += sign * d
__global__ void add_scaled(int64_t n, double* __restrict__ x, const double* __restrict__ d, double sign) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += sign * d[i];
}

// half bandwidth in DOFs of the node-block pattern (host copy of the pattern, once per context)
int band_width(agx_context* ctx) {
  if (ctx->band_w >= 0) return AGX_OK;
  std::vector<int32_t> rp(ctx->n_nodes + 1), cl(ctx->nnzb);
  AGX_CUDA(ctx, cudaMemcpyAsync(rp.data(), ctx->d_rowptr, sizeof(int32_t) * rp.size(), cudaMemcpyDeviceToHost,
                                ctx->stream));
  AGX_CUDA(ctx, cudaMemcpyAsync(cl.data(), ctx->d_col, sizeof(int32_t) * cl.size(), cudaMemcpyDeviceToHost,
                                ctx->stream));
  AGX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  int64_t wn = 0;
  for (int64_t i = 0; i < ctx->n_nodes; ++i)
    for (int k = rp[i]; k < rp[i + 1]; ++k) wn = std::max<int64_t>(wn, i > cl[k] ? i - cl[k] : cl[k] - i);
  ctx->band_w = wn * ctx->ndof + ctx->ndof - 1;
  return AGX_OK;
}

void forward_backward(agx_context* ctx, double* v) {
  band_forward<<<1, SOLVE_THREADS, 0, ctx->stream>>>(ctx->d_band, ctx->d_band_rdiag, ctx->n_dofs, ctx->band_w, v);
  band_backward<<<1, SOLVE_THREADS, 0, ctx->stream>>>(ctx->d_band, ctx->d_band_rdiag, ctx->n_dofs, ctx->band_w, v);
  ctx->n_launches += 2;
}

int band_factor(agx_context* ctx) {
  const int64_t n = ctx->n_dofs, w = ctx->band_w, ld = w + 1;
  const int gv = agx_grid(ctx, n);
  // the sign of the definite tangent from its free diagonal
  unsigned long long* counts = reinterpret_cast<unsigned long long*>(ctx->d_partials);
  AGX_CUDA(ctx, cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned long long), ctx->stream));
  diag_signs<<<gv, AGX_BLOCK, 0, ctx->stream>>>(n, ctx->ndof, ctx->nnzb, ctx->d_diagpos, ctx->d_vals64,
                                                ctx->d_dmask_dof, counts);
  AGX_CHECK_LAUNCH(ctx);
  unsigned long long hc[2] = {0, 0};
  AGX_CUDA(ctx, cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, ctx->stream));
  AGX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (hc[0] && hc[1])
    return agx_fail(ctx, AGX_ERR_UNSUPPORTED,
                    "banded Cholesky needs a definite tangent: %llu positive and %llu negative free diagonal "
                    "entries", hc[0], hc[1]);
  ctx->band_sign = hc[1] ? -1.0 : 1.0;
  AGX_CUDA(ctx, cudaMemsetAsync(ctx->d_band, 0, sizeof(double) * (size_t)n * (size_t)ld, ctx->stream));
  AGX_CUDA(ctx, cudaMemsetAsync(ctx->d_band_err, 0, sizeof(int), ctx->stream));
  const int gb = agx_grid(ctx, ctx->n_nodes);
  switch (ctx->ndof) {
    case 1:
      band_build<1><<<gb, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_nodes, ctx->d_rowptr, ctx->d_col, ctx->d_vals64,
                                                       ctx->nnzb, ctx->d_dmask_dof, w, ctx->band_sign, ctx->d_band);
      break;
    case 2:
      band_build<2><<<gb, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_nodes, ctx->d_rowptr, ctx->d_col, ctx->d_vals64,
                                                       ctx->nnzb, ctx->d_dmask_dof, w, ctx->band_sign, ctx->d_band);
      break;
    default:
      band_build<3><<<gb, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_nodes, ctx->d_rowptr, ctx->d_col, ctx->d_vals64,
                                                       ctx->nnzb, ctx->d_dmask_dof, w, ctx->band_sign, ctx->d_band);
  }
  AGX_CHECK_LAUNCH(ctx);
  const int pf_grid = (int)std::max<int64_t>(1, (w + PF_THREADS - 1) / PF_THREADS);
  auto tiles = [&](int tm) {
    const int64_t nt = (w + tm - 1) / tm;
    return (int)std::max<int64_t>(1, nt * (nt + 1) / 2);
  };
  // the tile size with the least float64 work on the busiest SM: ceil(tiles / SMs) tiles of tm^3
  int tm = 64;
  double best = 1e300;
  for (int t : {64, 32, 16}) {
    const double cost = std::ceil((double)tiles(t) / ctx->sm_count) * (double)t * t * t;
    if (cost < best * 0.999) {
      best = cost;
      tm = t;
    }
  }
  const int sy_grid = tiles(tm);
  for (int64_t j0 = 0; j0 < n; j0 += NB) {
    const int nbp = (int)imin(NB, n - j0);
    panel_factor<<<pf_grid, PF_THREADS, 0, ctx->stream>>>(ctx->d_band, n, w, j0, nbp, ctx->d_band_l11,
                                                          ctx->d_band_rdiag, ctx->d_band_err);
    if (tm == 64) syrk_update<64><<<sy_grid, 256, 0, ctx->stream>>>(ctx->d_band, n, w, j0, nbp, ctx->d_band_l11);
    else if (tm == 32) syrk_update<32><<<sy_grid, 256, 0, ctx->stream>>>(ctx->d_band, n, w, j0, nbp, ctx->d_band_l11);
    else syrk_update<16><<<sy_grid, 256, 0, ctx->stream>>>(ctx->d_band, n, w, j0, nbp, ctx->d_band_l11);
    ctx->n_launches += 2;
  }
  AGX_CHECK_LAUNCH(ctx);
  int herr = 0;
  AGX_CUDA(ctx, cudaMemcpyAsync(&herr, ctx->d_band_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  AGX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->n_launches += 2;
  if (herr) return herr;  // > 0: column (1-based) whose pivot was not positive
  ctx->band_gen = ctx->tangent_gen;
  return AGX_OK;
}

}  // namespace

int agx_band_solve_impl(agx_context* ctx, const double* b, double* x, const agx_solve_opts* opts,
                        agx_solve_info* info) {
  if (ctx->tangent_valid != AGX_F64)
    return agx_fail(ctx, AGX_ERR_STATE, "the banded Cholesky solve needs a float64 tangent (assemble first)");
  if (int rc = band_width(ctx)) return rc;
  const int64_t n = ctx->n_dofs;
  const double bytes = 8.0 * (double)n * (double)(ctx->band_w + 1);
  if (bytes > (double)ctx->band_max_bytes)
    return agx_fail(ctx, AGX_ERR_UNSUPPORTED,
                    "banded Cholesky: half bandwidth %lld DOFs needs %.1f GB for the factor (limit %.1f GB); use an "
                    "iterative method",
                    (long long)ctx->band_w, bytes / 1e9, (double)ctx->band_max_bytes / 1e9);
  if (!ctx->d_band) {
    AGX_CUDA(ctx, cudaMalloc(&ctx->d_band, (size_t)bytes));
    AGX_CUDA(ctx, cudaMalloc(&ctx->d_band_err, sizeof(int)));
    AGX_CUDA(ctx, cudaMalloc(&ctx->d_band_l11, sizeof(double) * NB * NB));
    AGX_CUDA(ctx, cudaMalloc(&ctx->d_band_rdiag, sizeof(double) * n));
  }
  if (ctx->band_gen != ctx->tangent_gen) {
    agx_prof_scope ps(ctx, AGX_PROF_FACTOR);
    const int rc = band_factor(ctx);
    if (rc < 0) return rc;
    if (rc > 0) {  // not positive definite: reported like a Krylov breakdown, with x = 0
      AGX_CUDA(ctx, cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream));
      if (info) {
        info->iterations = 0;
        info->rel_residual = NAN;
        info->status = AGX_DIVERGED;
      }
      return AGX_OK;
    }
  }
  const int gv = agx_grid(ctx, n);
  const double sg = ctx->band_sign;
  // x = K^-1 b, then refinement steps d = K^-1 (b - K x), x += d
  scale_copy<<<gv, AGX_BLOCK, 0, ctx->stream>>>(n, b, x, sg);
  forward_backward(ctx, x);
  double bb = 0.0, nf = 0.0;
  if (int rc = agx_residual_norm(ctx, b, &bb, &nf)) return rc;
  const double rtol = opts ? opts->rtol : 1e-13;
  double rel = 0.0;
  int steps = 0;
  for (int it = 0; it < 4; ++it) {
    if (int rc = agx_spmv_impl(ctx, AGX_F64, x, ctx->d_t)) return rc;
    residual_of<<<gv, AGX_BLOCK, 0, ctx->stream>>>(n, b, ctx->d_t, ctx->d_v);
    ctx->n_launches += 2;
    double rr = 0.0;
    if (int rc = agx_residual_norm(ctx, ctx->d_v, &rr, &nf)) return rc;
    const double prev = rel;
    rel = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
    // done, or refinement no longer gains (the float64 residual of an ill-conditioned system
    // stagnates near eps ||K|| ||x|| / ||b||)
    if (!(rel > rtol) || it == 3 || nf > 0 || (it > 0 && rel > 0.5 * prev)) break;
    scale_copy<<<gv, AGX_BLOCK, 0, ctx->stream>>>(n, ctx->d_v, ctx->d_v, sg);
    forward_backward(ctx, ctx->d_v);
    add_scaled<<<gv, AGX_BLOCK, 0, ctx->stream>>>(n, x, ctx->d_v, 1.0);
    ctx->n_launches += 2;
    steps += 1;
  }
  AGX_CHECK_LAUNCH(ctx);
  if (info) {
    info->iterations = steps;
    info->rel_residual = rel;
    info->status = (nf > 0 || !std::isfinite(rel)) ? AGX_DIVERGED : (rel <= rtol ? AGX_OK : AGX_NOT_CONVERGED);
  }
  return AGX_OK;
}
