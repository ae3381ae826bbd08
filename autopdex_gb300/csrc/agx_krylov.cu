// Sparse products and Krylov solvers on the node-block CSR tangent.
//
// Replaces the host solve behind jax.pure_callback (solver.py:642-659 -> scipy_assembling +
// spsolve, solver.py:1180-1222, :1493-1539) and the matrix-free CG of the 'jax' backend
// (jax.scipy.sparse.linalg.cg with a Jacobi preconditioner, solver.py:1084-1116).
//
// Every iteration is a handful of fused kernels: the sparse product carries the dot product
// that the step length needs, the vector update carries the dots of the next step.  Each
// reduction writes one partial per block; the last block to finish (atomic ticket, no
// waiting) sums the partials in block order -- deterministic -- and updates the scalars
// in device memory.  Once a solve has converged every kernel returns at entry, so the host
// launches iterations in chunks and reads the scalars only between chunks.
#include <algorithm>

#include <type_traits>

#include "agx_common.cuh"

namespace {

constexpr int NWARP = AGX_BLOCK / 32;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-reduces NV values, publishes the block's partials and lets the last block combine
// them.  Returns true in the last block (all threads), with totals in `tot` (thread 0).
template <int NV>
__device__ bool reduce_last_block(double (&v)[NV], double* __restrict__ partials, unsigned* __restrict__ counter,
                                  double (&tot)[NV]) {
  __shared__ double sh[NV][NWARP];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = warp_sum(v[k]);
    if (lane == 0) sh[k][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0;
      for (int w = 0; w < NWARP; ++w) s += sh[k][w];
      partials[(size_t)k * gridDim.x + blockIdx.x] = s;
    }
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    // all partial loads of a thread issued before any add (grids are at most 8 x 256 blocks)
    double part[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const unsigned i = threadIdx.x + u * blockDim.x;
      part[u] = i < gridDim.x ? __ldcg(partials + (size_t)k * gridDim.x + i) : 0.0;
    }
    double s = ((part[0] + part[1]) + (part[2] + part[3])) + ((part[4] + part[5]) + (part[6] + part[7]));
    s = warp_sum(s);
    __syncthreads();
    if (lane == 0) sh[k][warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int w = 0; w < NWARP; ++w) t += sh[k][w];
      tot[k] = t;
    }
  }
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// Reductions of the Jacobi-PCG iteration: the product and the update kernels only write one
// partial per block and value (no fence, no counter: the kernel boundary orders them), and a
// one-block kernel after each sums them in block order and sets the step scalars.  The last-
// block pattern above costs these two kernels 7-12 us per launch at 600-900 blocks on this
// GPU (measured against the same kernels without a reduction); a separate one-block launch
// costs a few microseconds.
template <int NV>
__device__ __forceinline__ void write_block_partials(const double (&v)[NV], double* __restrict__ partials) {
  __shared__ double sh[NV][NWARP];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double s = warp_sum(v[k]);
    if (lane == 0) sh[k][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0;
    for (int w = 0; w < NWARP; ++w) s += sh[threadIdx.x][w];
    partials[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = s;
  }
}

// totals of NV partial arrays of `np` blocks each (np <= 8 * AGX_BLOCK), valid in thread 0
template <int NV>
__device__ __forceinline__ void sum_block_partials(const double* __restrict__ partials, int np, double (&tot)[NV]) {
  __shared__ double sh[NV][NWARP];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double part[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int i = threadIdx.x + u * AGX_BLOCK;
      part[u] = i < np ? __ldcg(partials + (size_t)k * np + i) : 0.0;
    }
    const double s = warp_sum(((part[0] + part[1]) + (part[2] + part[3])) + ((part[4] + part[5]) + (part[6] + part[7])));
    if (lane == 0) sh[k][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = 0;
      for (int w = 0; w < NWARP; ++w) t += sh[k][w];
      tot[k] = t;
    }
  }
}

__device__ __forceinline__ bool bad(double x) { return !isfinite(x) || x == 0.0; }

// ---- sparse product ------------------------------------------------------------------
// Values are stored entry-major: entry (i, j) of block k at vals[(i ndof + j) nnzb + k], so
// the TPR lanes of a row (consecutive k) read each entry plane with contiguous loads.
// y = A x for the node-block CSR with TPR lanes per block row; with `dir` the operand is
// formed on the fly as x = z + beta p_old (the CG direction update folded into the product).
// U (2 or 4) blocks per lane and trip: all U blocks' columns and value planes are requested
// before any gather or FMA, so each lane keeps U blocks of loads in flight (the product is bound
// by bytes in flight per SM, not by traffic); matrix data is streamed (evict-first) so that the
// gathered vectors stay in L2.
// a stored value (float, double or the bf16 smoothing copy) in the product's precision, streamed
template <typename T, typename VT>
__device__ __forceinline__ T load_val(const VT* p) {
  if constexpr (std::is_same<VT, __nv_bfloat16>::value) return (T)__bfloat162float(__ldcs(p));
  else return (T)__ldcs(p);
}

template <typename T, int NDOF, int TPR, bool DIR, int U = 2, typename VT = T>
__device__ __forceinline__ void bsr_row(int64_t row, int sub, const int32_t* __restrict__ rowptr,
                                        const int32_t* __restrict__ col, const VT* __restrict__ vals, int64_t nnzb,
                                        const T* __restrict__ x, const T* __restrict__ pold, T beta, T (&y)[NDOF]) {
#pragma unroll
  for (int i = 0; i < NDOF; ++i) y[i] = 0;
  const int beg = rowptr[row], end = rowptr[row + 1];
  for (int k = beg + sub; k < end; k += U * TPR) {
    int64_t c[U];
    bool ok[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int kk = k + u * TPR;
      ok[u] = kk < end;
      c[u] = ok[u] ? __ldcs(col + kk) : 0;
    }
    T v[U][NDOF * NDOF];
#pragma unroll
    for (int e = 0; e < NDOF * NDOF; ++e)
#pragma unroll
      for (int u = 0; u < U; ++u) v[u][e] = ok[u] ? load_val<T>(vals + (int64_t)e * nnzb + k + u * TPR) : T(0);
    T xs[U][NDOF];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int j = 0; j < NDOF; ++j) {
        xs[u][j] = ok[u] ? x[c[u] * NDOF + j] : T(0);
        if constexpr (DIR) {
          if (ok[u]) xs[u][j] += beta * pold[c[u] * NDOF + j];
        }
      }
#pragma unroll
    for (int i = 0; i < NDOF; ++i)
#pragma unroll
      for (int j = 0; j < NDOF; ++j) {
        T t = 0;
#pragma unroll
        for (int u = 0; u < U; ++u) t += v[u][i * NDOF + j] * xs[u][j];
        y[i] += t;
      }
  }
#pragma unroll
  for (int o = TPR / 2; o >= 1; o >>= 1)
#pragma unroll
    for (int i = 0; i < NDOF; ++i) y[i] += __shfl_xor_sync(0xffffffffu, y[i], o);
}

// The same product for the tangent of a structured nx x ny QUAD4 grid (node p = i (ny + 1) + j,
// every pattern row the in-range 3 x 3 stencil of its node, checked when the pattern is built):
// row p's blocks are its stencil neighbours in (di, dj) order starting at
//   rowptr(p) = S(i) (3 ny + 1) + r_i S(j),  S(m) = 3 m - [m > 0],  r_i = [i > 0] + 1 + [i < nx]
// (S(m) blocks in the rows or columns before m, 3 ny + 1 in a full row of nodes), so one lane per
// row reads only its values and the gathered vector: no row pointer, no column index.
template <typename T, int NDOF, bool DIR, typename VT = T>
__device__ __forceinline__ void grid_row(int64_t row, int ny, int64_t n_rows, const VT* __restrict__ vals,
                                         int64_t nnzb, const T* __restrict__ x, const T* __restrict__ pold, T beta,
                                         T (&y)[NDOF]) {
  // node counts below 2^31 (the pattern's int32 offsets): 32-bit division
  const uint32_t ny1 = (uint32_t)ny + 1u, nx = (uint32_t)n_rows / ny1 - 1u;
  const uint32_t i = (uint32_t)row / ny1;
  const int j = (int)((uint32_t)row - i * ny1);
  const int ri = (i > 0) + 1 + (i < nx);
  const int64_t k0 = (int64_t)(3 * i - (i > 0)) * (3 * (int64_t)ny + 1) + (int64_t)ri * (3 * j - (j > 0));
  bool ok[9];
  int m[9];
  int cnt = 0;
#pragma unroll
  for (int t = 0; t < 9; ++t) {
    const int di = t / 3 - 1, dj = t % 3 - 1;
    ok[t] = (di >= 0 || i > 0) && (di <= 0 || i < nx) && (dj >= 0 || j > 0) && (dj <= 0 || j < ny);
    m[t] = cnt;
    cnt += ok[t] ? 1 : 0;
  }
  T v[9][NDOF * NDOF];
#pragma unroll
  for (int e = 0; e < NDOF * NDOF; ++e)
#pragma unroll
    for (int t = 0; t < 9; ++t) v[t][e] = ok[t] ? load_val<T>(vals + (int64_t)e * nnzb + k0 + m[t]) : T(0);
#pragma unroll
  for (int q = 0; q < NDOF; ++q) y[q] = 0;
#pragma unroll
  for (int t = 0; t < 9; ++t) {
    const int64_t c = row + (int64_t)(t / 3 - 1) * (int64_t)ny1 + (t % 3 - 1);
#pragma unroll
    for (int jj = 0; jj < NDOF; ++jj) {
      T xv = ok[t] ? x[c * NDOF + jj] : T(0);
      if constexpr (DIR) {
        if (ok[t]) xv += beta * pold[c * NDOF + jj];
      }
#pragma unroll
      for (int q = 0; q < NDOF; ++q) y[q] += v[t][q * NDOF + jj] * xv;
    }
  }
}

// The same for the tangent of a structured nx x ny x nz brick grid (node p = (i (ny + 1) + j)
// (nz + 1) + k, every pattern row the in-range 27-node stencil): the blocks before row p are
//   S(i) (3 ny + 1)(3 nz + 1) + r_i S(j) (3 nz + 1) + r_i r_j S(k)
// with S and r as above per direction, and row p's blocks are its in-range neighbours in
// (di, dj, dk) order.  code = (ny << 16) | nz.  Scalar fields load all 27 values at once; block
// fields one plane of 9 neighbours at a time (register pressure).
template <typename T, int NDOF, bool DIR, typename VT = T>
__device__ __forceinline__ void brick_row(int64_t row, int code, int64_t n_rows, const VT* __restrict__ vals,
                                          int64_t nnzb, const T* __restrict__ x, const T* __restrict__ pold, T beta,
                                          T (&y)[NDOF]) {
  const uint32_t ny = (uint32_t)code >> 16, nz = (uint32_t)code & 0xFFFFu;
  const uint32_t NZ = nz + 1u, plane = (ny + 1u) * NZ;
  const uint32_t nx = (uint32_t)n_rows / plane - 1u;
  const uint32_t i = (uint32_t)row / plane, rem = (uint32_t)row - i * plane;
  const uint32_t j = rem / NZ, k = rem - j * NZ;
  const int ri = (i > 0) + 1 + (i < nx), rj = (j > 0) + 1 + (j < ny);
  const int64_t k0 = (int64_t)(3 * i - (i > 0)) * (3 * (int64_t)ny + 1) * (3 * (int64_t)nz + 1) +
                     (int64_t)ri * (3 * j - (j > 0)) * (3 * (int64_t)nz + 1) + (int64_t)(ri * rj) * (3 * k - (k > 0));
  bool ok[27];
  int m[27];
  int cnt = 0;
#pragma unroll
  for (int t = 0; t < 27; ++t) {
    const int di = t / 9 - 1, dj = (t / 3) % 3 - 1, dk = t % 3 - 1;
    ok[t] = (di >= 0 || i > 0) && (di <= 0 || i < nx) && (dj >= 0 || j > 0) && (dj <= 0 || j < ny) &&
            (dk >= 0 || k > 0) && (dk <= 0 || k < nz);
    m[t] = cnt;
    cnt += ok[t] ? 1 : 0;
  }
#pragma unroll
  for (int q = 0; q < NDOF; ++q) y[q] = 0;
  if constexpr (NDOF == 1 && sizeof(VT) <= 4) {
    // The warp's 32 consecutive rows (every kernel's lanes hold consecutive rows, the tail
    // clamped to the last row) own one contiguous range of at most 32 x 27 values: copied
    // asynchronously in 16-byte chunks (cp.async, the last chunk zero-filled past the range) into
    // the warp's slice of shared memory while each lane gathers its 27 vector entries (the fused
    // product: through registers, below); then each lane reads its row from the slice (a stride
    // of 27 words: no bank conflicts).
    constexpr int EPC = 16 / (int)sizeof(VT);  // values per chunk
    __shared__ __align__(16) VT stage[AGX_BLOCK / 32][32 * 27 + 16];
    VT* sw = stage[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int64_t base = __shfl_sync(0xffffffffu, k0, 0);
    const int64_t endk = __shfl_sync(0xffffffffu, k0 + cnt, 31);
    const int64_t abase = base & ~(int64_t)(EPC - 1);  // 16-byte aligned start
    const int nchunks = (int)((endk - abase + EPC - 1) / EPC);
    if constexpr (DIR) {
      // the fused product (direction update): its gather also reads the old direction, and the
      // asynchronous form would spill; the values go through registers, 27 loads in flight
      VT r[27];
#pragma unroll
      for (int u = 0; u < 27; ++u) {
        const int sidx = lane + 32 * u;
        r[u] = sidx < (int)(endk - base) ? __ldcs(vals + base + sidx) : VT(0);
      }
      __syncwarp();  // the previous row's reads of the slice are done
#pragma unroll
      for (int u = 0; u < 27; ++u) {
        const int sidx = lane + 32 * u;
        if (sidx < (int)(endk - base)) sw[sidx] = r[u];
      }
      __syncwarp();
      const VT* my = sw + (k0 - base);
#pragma unroll
      for (int t = 0; t < 27; ++t) {
        if (!ok[t]) continue;
        const int64_t c = row + (int64_t)(t / 9 - 1) * plane + (int64_t)((t / 3) % 3 - 1) * NZ + (t % 3 - 1);
        const T xv = x[c] + beta * pold[c];
        T v;
        if constexpr (std::is_same<VT, __nv_bfloat16>::value) v = (T)__bfloat162float(my[m[t]]);
        else v = (T)my[m[t]];
        y[0] += v * xv;
      }
      return;
    }
    __syncwarp();  // the previous row's reads of the slice are done
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sw);
    for (int c = lane; c < nchunks; c += 32) {
      const int64_t e0 = abase + (int64_t)c * EPC;
      const int64_t rem = endk - e0;
      const uint32_t bytes = rem >= EPC ? 16u : (uint32_t)rem * (uint32_t)sizeof(VT);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(sbase + (uint32_t)(c * 16)),
                   "l"(vals + e0), "r"(bytes)
                   : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    T xv[27];
#pragma unroll
    for (int t = 0; t < 27; ++t) {
      const int64_t c = row + (int64_t)(t / 9 - 1) * plane + (int64_t)((t / 3) % 3 - 1) * NZ + (t % 3 - 1);
      xv[t] = ok[t] ? x[c] : T(0);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncwarp();
    const VT* my = sw + (k0 - abase);
#pragma unroll
    for (int t = 0; t < 27; ++t) {
      if (!ok[t]) continue;
      T v;
      if constexpr (std::is_same<VT, __nv_bfloat16>::value) v = (T)__bfloat162float(my[m[t]]);
      else v = (T)my[m[t]];
      y[0] += v * xv[t];
    }
    return;
  }
  constexpr int CH = NDOF == 1 ? 27 : 9;  // neighbours whose values are in flight together
#pragma unroll
  for (int t0 = 0; t0 < 27; t0 += CH) {
    T v[CH][NDOF * NDOF];
#pragma unroll
    for (int e = 0; e < NDOF * NDOF; ++e)
#pragma unroll
      for (int u = 0; u < CH; ++u)
        v[u][e] = ok[t0 + u] ? load_val<T>(vals + (int64_t)e * nnzb + k0 + m[t0 + u]) : T(0);
#pragma unroll
    for (int u = 0; u < CH; ++u) {
      const int t = t0 + u;
      const int64_t c = row + (int64_t)(t / 9 - 1) * plane + (int64_t)((t / 3) % 3 - 1) * NZ + (t % 3 - 1);
#pragma unroll
      for (int jj = 0; jj < NDOF; ++jj) {
        T xv = ok[t] ? x[c * NDOF + jj] : T(0);
        if constexpr (DIR) {
          if (ok[t]) xv += beta * pold[c * NDOF + jj];
        }
#pragma unroll
        for (int q = 0; q < NDOF; ++q) y[q] += v[u][q * NDOF + jj] * xv;
      }
    }
  }
}

// A product row in the tangent's storage: U > 0 the node-block CSR with TPR lanes per row,
// U <= 0 the structured grid's stencil (one lane per row, gny = ny; U == -2: the kernels give
// each lane two consecutive rows, whose loads are then in flight together; U == -3: the brick
// grid's stencil, gny = its packed code)
template <typename T, int NDOF, int TPR, bool DIR, int U, typename VT = T>
__device__ __forceinline__ void tangent_row(int64_t row, int sub, const int32_t* __restrict__ rowptr,
                                            const int32_t* __restrict__ col, const VT* __restrict__ vals,
                                            int64_t nnzb, int64_t n_rows, int gny, const T* __restrict__ x,
                                            const T* __restrict__ pold, T beta, T (&y)[NDOF]) {
  if constexpr (U == -3) {
    static_assert(TPR == 1, "the brick product has one lane per row");
    brick_row<T, NDOF, DIR, VT>(row, gny, n_rows, vals, nnzb, x, pold, beta, y);
  } else if constexpr (U <= 0) {  // 0: one row per lane, -2: two rows per lane (the kernels' loops)
    static_assert(TPR == 1, "the grid product has one lane per row");
    grid_row<T, NDOF, DIR, VT>(row, gny, n_rows, vals, nnzb, x, pold, beta, y);
  } else {
    bsr_row<T, NDOF, TPR, DIR, U, VT>(row, sub, rowptr, col, vals, nnzb, x, pold, beta, y);
  }
}

// the brick product's staged scalar rows: three blocks per SM (registers capped), since the
// product is bound by the latency of its two dependent load rounds
template <int U, int NDOF, int VBYTES>
constexpr int brick_min_blocks() { return (U == -3 && NDOF == 1 && VBYTES <= 4) ? 3 : 0; }  // 0: no bound

template <typename T, int NDOF, int TPR, int U = 2>
__global__ void __launch_bounds__(AGX_BLOCK, brick_min_blocks<U, NDOF, sizeof(T)>()) spmv_kernel(int64_t n_rows, const int32_t* __restrict__ rowptr,
                                                         const int32_t* __restrict__ col, const T* __restrict__ vals,
                                                         int64_t nnzb, int gny, const T* __restrict__ x,
                                                         T* __restrict__ y) {
  constexpr int RPT = U == -2 ? 2 : 1;  // rows per lane
  const int sub = threadIdx.x % TPR;
  const int64_t total = (((n_rows + RPT - 1) / RPT * TPR + 31) / 32) * 32;
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = (L / TPR) * RPT;
    T yr[RPT][NDOF];
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int64_t row = r0 + rr;
      tangent_row<T, NDOF, TPR, false, U>(row < n_rows ? row : n_rows - 1, sub, rowptr, col, vals, nnzb, n_rows,
                                          gny, x, nullptr, T(0), yr[rr]);
    }
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int64_t row = r0 + rr;
      if (row < n_rows && sub == 0) {
#pragma unroll
        for (int i = 0; i < NDOF; ++i) y[row * NDOF + i] = yr[rr][i];
      }
    }
  }
}

// p_new = z + beta p_old (own rows), q = A p_new, block partials of (p_new, q) for the step
// alpha = rz / (p_new, q).  beta = 0 on the first iteration (p_old = 0), which makes p_new = z.
template <typename T, int NDOF, int TPR, int U = 2>
__global__ void __launch_bounds__(AGX_BLOCK, brick_min_blocks<U, NDOF, sizeof(T)>())
spmv_dot_kernel(int64_t n_rows, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                const T* __restrict__ vals, int64_t nnzb, int gny, const T* __restrict__ z,
                const T* __restrict__ pold, T* __restrict__ pnew, T* __restrict__ q, agx_krylov_scalars* sc,
                double* __restrict__ partials, const T* __restrict__ rflex) {
  agx_pdl_entry();
  if (sc->converged) return;
  const T beta = (T)sc->beta;
  constexpr int RPT = U == -2 ? 2 : 1;  // rows per lane
  const int sub = threadIdx.x % TPR;
  const int64_t total = (((n_rows + RPT - 1) / RPT * TPR + 31) / 32) * 32;
  T acc_t = 0, accr_t = 0;  // per-thread partials in T (a few rows), block and grid sums in float64
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = (L / TPR) * RPT;
    T yr[RPT][NDOF];
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int64_t row = r0 + rr;
      tangent_row<T, NDOF, TPR, true, U>(row < n_rows ? row : n_rows - 1, sub, rowptr, col, vals, nnzb, n_rows, gny,
                                         z, pold, beta, yr[rr]);
    }
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int64_t row = r0 + rr;
      if (row < n_rows && sub == 0) {
#pragma unroll
        for (int i = 0; i < NDOF; ++i) {
          const int64_t d = row * NDOF + i;
          const T pn = z[d] + beta * pold[d];
          pnew[d] = pn;
          q[d] = yr[rr][i];
          acc_t += yr[rr][i] * pn;
          if (rflex) accr_t += rflex[d] * pn;
        }
      }
    }
  }
  // block partials of (p, A p) -- and of (p, r) for the flexible method -- for pcg_finish_pq
  // (Jacobi-PCG) or fcg_finish_pq (flexible CG)
  double acc[2] = {(double)acc_t, (double)accr_t};
  if (rflex) {
    write_block_partials<2>(acc, partials);
  } else {
    const double acc1[1] = {acc[0]};
    write_block_partials<1>(acc1, partials);
  }
}

// ---- PCG (Jacobi or external preconditioner) ------------------------------------------
// norm of b and the scale used by the single-precision inner solve
__global__ void __launch_bounds__(AGX_BLOCK) norm_init_kernel(int64_t n, const double* __restrict__ b,
                                                              agx_krylov_scalars* sc, double* partials,
                                                              unsigned* counter, double rtol, double atol) {
  double acc[1] = {0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc[0] += b[i] * b[i];
  double tot[1];
  if (reduce_last_block<1>(acc, partials, counter, tot) && threadIdx.x == 0) {
    const double bb = tot[0];
    sc->extra[0] = bb > 0.0 ? 1.0 / sqrt(bb) : 1.0;  // inner scale
    sc->extra[1] = bb > 0.0 ? sqrt(bb) : 1.0;
    sc->rr = bb;
    sc->rr_stop = fmax(rtol * rtol * bb, atol * atol);
    sc->iters = 0;
    sc->converged = (bb <= sc->rr_stop || bb == 0.0) ? 1 : (isfinite(bb) ? 0 : 2);
    sc->alpha = sc->beta = sc->pq = 0.0;
    sc->omega = sc->rho = 1.0;
  }
}

// x = 0; r = s b; z = Dinv r (when jacobi); rz, rr.  For the mixed method s = 1/||b||.
template <typename T>
__global__ void __launch_bounds__(AGX_BLOCK)
pcg_init_kernel(int64_t n, const double* __restrict__ b, const T* __restrict__ dinv, T* __restrict__ x,
                T* __restrict__ r, T* __restrict__ z, T* __restrict__ p, agx_krylov_scalars* sc, double* partials,
                unsigned* counter, int scaled, int jacobi) {
  const double s = scaled ? sc->extra[0] : 1.0;
  double acc[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T ri = (T)(b[i] * s);
    x[i] = 0;
    r[i] = ri;
    p[i] = 0;  // p_old of the first fused product (beta = 0)
    if (jacobi) {
      const T zi = dinv[i] * ri;
      z[i] = zi;
      acc[0] += (double)ri * (double)zi;
    }
    acc[1] += (double)ri * (double)ri;
  }
  double tot[2];
  if (reduce_last_block<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
    if (jacobi) sc->rz = tot[0];
    sc->rr = tot[1];
    if (scaled) sc->rr_stop *= sc->extra[0] * sc->extra[0];
  }
}

// x += a p; r -= a q; z = Dinv r; block partials of (r, z) and (r, r) for pcg_finish_rz.
// 16-byte vector loads and stores (4 floats or 2 doubles per access) when every vector is
// 16-byte aligned (the library's own are; a caller's x may not be), a scalar loop for the rest.
template <typename T>
struct alignas(16) vec16 {
  T v[16 / sizeof(T)];
};

template <typename T>
__global__ void __launch_bounds__(AGX_BLOCK)
pcg_update_kernel(int64_t n, T* __restrict__ x, T* __restrict__ r, T* __restrict__ z, const T* __restrict__ p,
                  const T* __restrict__ q, const T* __restrict__ dinv, agx_krylov_scalars* sc,
                  double* __restrict__ partials) {
  agx_pdl_entry();
  if (sc->converged) return;
  constexpr int V = 16 / sizeof(T);
  using W = vec16<T>;
  const T a = (T)sc->alpha;
  T rz_t = 0, rr_t = 0;  // per-thread partials in T, block and grid sums in float64
  const bool aligned = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(r) |
                         reinterpret_cast<uintptr_t>(z) | reinterpret_cast<uintptr_t>(p) |
                         reinterpret_cast<uintptr_t>(q) | reinterpret_cast<uintptr_t>(dinv)) & 15u) == 0;
  const int64_t nv = aligned ? n / V : 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nv; k += stride) {
    W xv = reinterpret_cast<const W*>(x)[k], rv = reinterpret_cast<const W*>(r)[k];
    const W pv = reinterpret_cast<const W*>(p)[k], qv = reinterpret_cast<const W*>(q)[k];
    const W dv = reinterpret_cast<const W*>(dinv)[k];
    W zv;
#pragma unroll
    for (int u = 0; u < V; ++u) {
      xv.v[u] += a * pv.v[u];
      const T ri = rv.v[u] - a * qv.v[u];
      rv.v[u] = ri;
      const T zi = dv.v[u] * ri;
      zv.v[u] = zi;
      rz_t += ri * zi;
      rr_t += ri * ri;
    }
    reinterpret_cast<W*>(x)[k] = xv;
    reinterpret_cast<W*>(r)[k] = rv;
    reinterpret_cast<W*>(z)[k] = zv;
  }
  for (int64_t i = nv * V + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] += a * p[i];
    const T ri = r[i] - a * q[i];
    r[i] = ri;
    const T zi = dinv[i] * ri;
    z[i] = zi;
    rz_t += ri * zi;
    rr_t += ri * ri;
  }
  const double acc[2] = {(double)rz_t, (double)rr_t};
  write_block_partials<2>(acc, partials);  // pcg_finish_rz sums them
}

// one block: alpha = (r, z) / (p, A p) from the product's block partials
__global__ void __launch_bounds__(AGX_BLOCK)
pcg_finish_pq(agx_krylov_scalars* sc, const double* __restrict__ parts, int np) {
  agx_pdl_entry();
  if (sc->converged) return;
  double t[1];
  sum_block_partials<1>(parts, np, t);
  if (threadIdx.x == 0) {
    sc->pq = t[0];
    // Only a zero or non-finite (p, Ap) is a breakdown: the tangents of clockwise-numbered
    // quads (mesher.py:88-94 numbers quads clockwise, so det J < 0) are negative definite,
    // and CG with a Jacobi preconditioner of the same sign runs as on (-K, -D).
    if (bad(t[0])) sc->converged = 2;
    else sc->alpha = sc->rz / t[0];
  }
}

// one block: the update's (r, z) and (r, r): iteration count, convergence test, beta
__global__ void __launch_bounds__(AGX_BLOCK)
pcg_finish_rz(agx_krylov_scalars* sc, const double* __restrict__ parts, int np) {
  agx_pdl_entry();
  if (sc->converged) return;
  double t[2];
  sum_block_partials<2>(parts, np, t);
  if (threadIdx.x == 0) {
    sc->iters += 1;
    sc->rr = t[1];
    if (!isfinite(t[0]) || !isfinite(t[1])) {
      sc->converged = 2;
    } else if (t[1] <= sc->rr_stop) {
      sc->converged = 1;
    } else if (sc->rz == 0.0) {
      sc->converged = 2;
    } else {
      sc->beta = t[0] / sc->rz;
      sc->rz = t[0];
    }
  }
}

// ---- flexible CG (Notay FCG(1)): beta = -(z_new, q) / (p, q) ----------------------------
// The update and direction kernels write block partials (16-byte accesses when every vector is
// aligned, a scalar loop otherwise); one-block kernels after them finish the sums and set the
// step scalars, as in the Jacobi-PCG iteration.

// x += a p; r -= a q; block partials of (r, r) for fcg_finish_update
template <typename T>
__global__ void __launch_bounds__(AGX_BLOCK)
fcg_update_kernel(int64_t n, T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p, const T* __restrict__ q,
                  agx_krylov_scalars* sc, double* __restrict__ partials) {
  agx_pdl_entry();
  if (sc->converged) return;
  constexpr int V = 16 / sizeof(T);
  using W = vec16<T>;
  const T a = (T)sc->alpha;
  T rr_t = 0;
  const bool aligned = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(r) |
                         reinterpret_cast<uintptr_t>(p) | reinterpret_cast<uintptr_t>(q)) & 15u) == 0;
  const int64_t nv = aligned ? n / V : 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nv; k += stride) {
    W xv = reinterpret_cast<const W*>(x)[k], rv = reinterpret_cast<const W*>(r)[k];
    const W pv = reinterpret_cast<const W*>(p)[k], qv = reinterpret_cast<const W*>(q)[k];
#pragma unroll
    for (int u = 0; u < V; ++u) {
      xv.v[u] += a * pv.v[u];
      const T ri = rv.v[u] - a * qv.v[u];
      rv.v[u] = ri;
      rr_t += ri * ri;
    }
    reinterpret_cast<W*>(x)[k] = xv;
    reinterpret_cast<W*>(r)[k] = rv;
  }
  for (int64_t i = nv * V + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    x[i] += a * p[i];
    const T ri = r[i] - a * q[i];
    r[i] = ri;
    rr_t += ri * ri;
  }
  const double acc[1] = {(double)rr_t};
  write_block_partials<1>(acc, partials);
}

// one block: iteration count, (r, r) and the convergence test
__global__ void __launch_bounds__(AGX_BLOCK)
fcg_finish_update(agx_krylov_scalars* sc, const double* __restrict__ parts, int np) {
  agx_pdl_entry();
  if (sc->converged) return;
  double t[1];
  sum_block_partials<1>(parts, np, t);
  if (threadIdx.x == 0) {
    sc->iters += 1;
    sc->rr = t[0];
    if (!isfinite(t[0])) sc->converged = 2;
    else if (t[0] <= sc->rr_stop) sc->converged = 1;
  }
}

// after z = M r: block partials of (r, z) and (z, q) for fcg_finish_direction
template <typename T>
__global__ void __launch_bounds__(AGX_BLOCK)
fcg_direction_dots(int64_t n, const T* __restrict__ r, const T* __restrict__ z, const T* __restrict__ q,
                   agx_krylov_scalars* sc, double* __restrict__ partials) {
  agx_pdl_entry();
  if (sc->converged) return;
  constexpr int V = 16 / sizeof(T);
  using W = vec16<T>;
  T rz_t = 0, zq_t = 0;
  const bool aligned = ((reinterpret_cast<uintptr_t>(r) | reinterpret_cast<uintptr_t>(z) |
                         reinterpret_cast<uintptr_t>(q)) & 15u) == 0;
  const int64_t nv = aligned ? n / V : 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nv; k += stride) {
    const W rv = reinterpret_cast<const W*>(r)[k], zv = reinterpret_cast<const W*>(z)[k];
    const W qv = reinterpret_cast<const W*>(q)[k];
#pragma unroll
    for (int u = 0; u < V; ++u) {
      rz_t += rv.v[u] * zv.v[u];
      zq_t += zv.v[u] * qv.v[u];
    }
  }
  for (int64_t i = nv * V + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    rz_t += r[i] * z[i];
    zq_t += z[i] * q[i];
  }
  const double acc[2] = {(double)rz_t, (double)zq_t};
  write_block_partials<2>(acc, partials);
}

// one block: rz = (r, z), beta = -(z, q) / (p, q) (0 on the first direction)
__global__ void __launch_bounds__(AGX_BLOCK)
fcg_finish_direction(agx_krylov_scalars* sc, const double* __restrict__ parts, int np) {
  agx_pdl_entry();
  if (sc->converged) return;
  double t[2];
  sum_block_partials<2>(parts, np, t);
  if (threadIdx.x == 0) {
    sc->rz = t[0];
    sc->beta = sc->iters == 0 ? 0.0 : -t[1] / sc->pq;
    if (bad(t[0])) sc->converged = 2;
  }
}

// one block: (p, A p) and the flexible step's (p, r) from spmv_dot_kernel's partials: the
// step is the exact line minimiser (p, r) / (p, A p), which differs from (r, z) / (p, A p)
// once the preconditioner varies from one iteration to the next
__global__ void __launch_bounds__(AGX_BLOCK)
fcg_finish_pq(agx_krylov_scalars* sc, const double* __restrict__ parts, int np) {
  agx_pdl_entry();
  if (sc->converged) return;
  double t[2];
  sum_block_partials<2>(parts, np, t);
  if (threadIdx.x == 0) {
    sc->pq = t[0];
    sc->rz = t[1];
    if (bad(t[0])) sc->converged = 2;
    else sc->alpha = t[1] / t[0];
  }
}

template <typename T>
__global__ void jacobi_dinv(int64_t n, const T* __restrict__ dinv, const T* __restrict__ r, T* __restrict__ z) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = dinv[i] * r[i];
}

template <typename T>
__global__ void __launch_bounds__(AGX_BLOCK)
jacobi_apply(int64_t n, const T* __restrict__ dinv, const T* __restrict__ r, T* __restrict__ z,
             const agx_krylov_scalars* sc) {
  agx_pdl_entry();
  if (sc->converged) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = dinv[i] * r[i];
}

// ---- two-level application of a registered preconditioner -----------------------------
// One smoothing step on the running residual: rc = rin - t (t = K d of the previous step, or
// none), d = a d + b D^-1 rc, z = d (first step) or z + d.  Damped Jacobi: a = 0, b = w;
// Chebyshev: the coefficients of the three-term recurrence.
__global__ void __launch_bounds__(AGX_BLOCK)
tl_sweep(int64_t n, const float* __restrict__ dinv, float b, float a, const float* rin, float* rc,
         const float* __restrict__ t, float* __restrict__ z, float* __restrict__ dz, int first,
         const agx_krylov_scalars* sc) {
  agx_pdl_entry();
  if (sc->converged) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = t ? rin[i] - t[i] : rin[i];
    rc[i] = v;
    const float d = (a != 0.0f ? a * dz[i] : 0.0f) + b * dinv[i] * v;
    dz[i] = d;
    z[i] = first ? d : z[i] + d;
  }
}

// Gershgorin bound of the spectrum of D^-1 K: max over rows of sum_j |K_ij| / |K_ii|
// (float32 tangent; one value per block, the host takes the maximum)
template <int NDOF>
__global__ void __launch_bounds__(AGX_BLOCK)
gershgorin_kernel(int64_t n_rows, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ diagpos,
                  const float* __restrict__ vals, int64_t nnzb, float* __restrict__ block_max) {
  float m = 0.0f;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_rows * NDOF;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t node = r / NDOF;
    const int i = (int)(r - node * NDOF);
    float s = 0.0f;
    for (int k = rowptr[node]; k < rowptr[node + 1]; ++k)
#pragma unroll
      for (int j = 0; j < NDOF; ++j) s += fabsf(vals[(int64_t)(i * NDOF + j) * nnzb + k]);
    const float d = fabsf(vals[(int64_t)(i * NDOF + i) * nnzb + diagpos[node]]);
    if (d > 0.0f) m = fmaxf(m, s / d);
  }
  for (int o = 16; o >= 1; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ float sh[AGX_BLOCK / 32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < AGX_BLOCK / 32; ++w) t = fmaxf(t, sh[w]);
    block_max[blockIdx.x] = t;
  }
}

// z += c y; rc -= c t (t = K y): rc stays r - K z
__global__ void __launch_bounds__(AGX_BLOCK)
tl_combine(int64_t n, float* __restrict__ z, const float* __restrict__ y, float* __restrict__ rc,
           const float* __restrict__ t, const agx_krylov_scalars* sc) {
  agx_pdl_entry();
  if (sc->converged) return;
  const float c = (float)sc->extra[2];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    z[i] += c * y[i];
    rc[i] -= c * t[i];
  }
}

// ---- the two-level application's products with their element-wise work fused in ---------
// One kernel per smoothing step: the product t = K x for the lane group's rows, then, for the
// same rows, the step's element-wise update -- no separate sweep kernel and no t vector.
//   TL_SWEEP  rc -= t; d = a x + b D^-1 rc (into dnew: x, the previous increment, is still
//             being gathered by other rows); z += d
//   TL_RESID  rc -= t                     (the residual after the last pre-smoothing step)
//   TL_STEP   t written; block partials of (rc, y) and (y, t) for tl_finish_step
enum { TL_SWEEP = 0, TL_RESID = 1, TL_STEP = 2 };

template <int NDOF, int TPR, int U, int EPI, typename VT = float>
__global__ void __launch_bounds__(AGX_BLOCK, brick_min_blocks<U, NDOF, sizeof(VT)>())
tl_spmv(int64_t n_rows, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
        const VT* __restrict__ vals, int64_t nnzb, int gny, const float* __restrict__ x, float* __restrict__ rc,
        const float* __restrict__ dinv, float a, float b, float* __restrict__ dnew, float* __restrict__ z,
        float* __restrict__ tout, agx_krylov_scalars* sc, double* __restrict__ partials) {
  agx_pdl_entry();
  if (sc->converged) return;
  constexpr int RPT = U == -2 ? 2 : 1;  // rows per lane
  const int sub = threadIdx.x % TPR;
  const int64_t total = (((n_rows + RPT - 1) / RPT * TPR + 31) / 32) * 32;
  float acc_a = 0.0f, acc_b = 0.0f;
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = (L / TPR) * RPT;
    float yr[RPT][NDOF];
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int64_t row = r0 + rr;
      tangent_row<float, NDOF, TPR, false, U, VT>(row < n_rows ? row : n_rows - 1, sub, rowptr, col, vals, nnzb,
                                                  n_rows, gny, x, nullptr, 0.0f, yr[rr]);
    }
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int64_t row = r0 + rr;
      if (row < n_rows && sub == 0) {
#pragma unroll
        for (int i = 0; i < NDOF; ++i) {
          const int64_t d = row * NDOF + i;
          const float t = yr[rr][i];
          if constexpr (EPI == TL_SWEEP) {
            const float r = rc[d] - t;
            rc[d] = r;
            const float dn = (a != 0.0f ? a * x[d] : 0.0f) + b * dinv[d] * r;
            dnew[d] = dn;
            z[d] += dn;
          } else if constexpr (EPI == TL_RESID) {
            rc[d] -= t;
          } else {
            tout[d] = t;
            acc_a += rc[d] * x[d];
            acc_b += x[d] * t;
          }
        }
      }
    }
  }
  if constexpr (EPI == TL_STEP) {
    const double acc[2] = {(double)acc_a, (double)acc_b};
    write_block_partials<2>(acc, partials);  // tl_finish_step sums them
  }
}

// one block: the energy-optimal step c = (rc, y) / (y, K y) from TL_STEP's partials
__global__ void __launch_bounds__(AGX_BLOCK)
tl_finish_step(agx_krylov_scalars* sc, const double* __restrict__ parts, int np) {
  agx_pdl_entry();
  if (sc->converged) return;
  double t[2];
  sum_block_partials<2>(parts, np, t);
  if (threadIdx.x == 0) sc->extra[2] = (isfinite(t[0]) && isfinite(t[1]) && t[1] != 0.0) ? t[0] / t[1] : 0.0;
}

// z += c y; rc -= c t; then the first post-smoothing step: d = b D^-1 rc into dz, z += d
__global__ void __launch_bounds__(AGX_BLOCK)
tl_combine_sweep(int64_t n, float* __restrict__ z, const float* __restrict__ y, float* __restrict__ rc,
                 const float* __restrict__ t, const float* __restrict__ dinv, float b, float* __restrict__ dz,
                 const agx_krylov_scalars* sc) {
  agx_pdl_entry();
  if (sc->converged) return;
  const float c = (float)sc->extra[2];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float r = rc[i] - c * t[i];
    rc[i] = r;
    const float d = b * dinv[i] * r;
    dz[i] = d;
    z[i] = (z[i] + c * y[i]) + d;
  }
}

// ---- BiCGStab (right Jacobi preconditioning), float64 --------------------------------
// p = r + beta (p - omega v); y = Dinv p
__global__ void __launch_bounds__(AGX_BLOCK)
bicg_p_kernel(int64_t n, double* __restrict__ p, const double* __restrict__ r, const double* __restrict__ v,
              double* __restrict__ y, const double* __restrict__ dinv, const agx_krylov_scalars* sc) {
  if (sc->converged) return;
  const double bta = sc->beta, om = sc->omega;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double pi = r[i] + bta * (p[i] - om * v[i]);
    p[i] = pi;
    y[i] = dinv[i] * pi;
  }
}

// v = A y; alpha = rho / (rhat, v)
template <int NDOF, int TPR>
__global__ void __launch_bounds__(AGX_BLOCK)
bicg_spmv_rhat(int64_t n_rows, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
               const double* __restrict__ vals, int64_t nnzb, const double* __restrict__ y, double* __restrict__ v,
               const double* __restrict__ rhat, agx_krylov_scalars* sc, double* partials, unsigned* counter) {
  if (sc->converged) return;
  const int sub = threadIdx.x % TPR;
  const int64_t total = ((n_rows * TPR + 31) / 32) * 32;
  double acc[1] = {0.0};
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = L / TPR;
    double yr[NDOF];
    bsr_row<double, NDOF, TPR, false>(row < n_rows ? row : n_rows - 1, sub, rowptr, col, vals, nnzb, y, nullptr, 0.0,
                                      yr);
    if (row < n_rows && sub == 0) {
#pragma unroll
      for (int i = 0; i < NDOF; ++i) {
        v[row * NDOF + i] = yr[i];
        acc[0] += rhat[row * NDOF + i] * yr[i];
      }
    }
  }
  double tot[1];
  if (reduce_last_block<1>(acc, partials, counter, tot) && threadIdx.x == 0) {
    if (bad(tot[0])) sc->converged = 2;
    else sc->alpha = sc->rho / tot[0];
  }
}

// s = r - alpha v; z = Dinv s
__global__ void __launch_bounds__(AGX_BLOCK)
bicg_s_kernel(int64_t n, const double* __restrict__ r, const double* __restrict__ v, double* __restrict__ s,
              double* __restrict__ z, const double* __restrict__ dinv, const agx_krylov_scalars* sc) {
  if (sc->converged) return;
  const double a = sc->alpha;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double si = r[i] - a * v[i];
    s[i] = si;
    z[i] = dinv[i] * si;
  }
}

// t = A z; omega = (t, s)/(t, t)
template <int NDOF, int TPR>
__global__ void __launch_bounds__(AGX_BLOCK)
bicg_spmv_ts(int64_t n_rows, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
             const double* __restrict__ vals, int64_t nnzb, const double* __restrict__ z, double* __restrict__ t,
             const double* __restrict__ s, agx_krylov_scalars* sc, double* partials, unsigned* counter) {
  if (sc->converged) return;
  const int sub = threadIdx.x % TPR;
  const int64_t total = ((n_rows * TPR + 31) / 32) * 32;
  double acc[2] = {0.0, 0.0};
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = L / TPR;
    double yr[NDOF];
    bsr_row<double, NDOF, TPR, false>(row < n_rows ? row : n_rows - 1, sub, rowptr, col, vals, nnzb, z, nullptr, 0.0,
                                      yr);
    if (row < n_rows && sub == 0) {
#pragma unroll
      for (int i = 0; i < NDOF; ++i) {
        t[row * NDOF + i] = yr[i];
        acc[0] += yr[i] * s[row * NDOF + i];
        acc[1] += yr[i] * yr[i];
      }
    }
  }
  double tot[2];
  if (reduce_last_block<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
    if (!isfinite(tot[0]) || bad(tot[1])) sc->converged = 2;
    else sc->omega = tot[0] / tot[1];
  }
}

// x += alpha y + omega z; r = s - omega t; rho_new = (rhat, r); rr
__global__ void __launch_bounds__(AGX_BLOCK)
bicg_update(int64_t n, double* __restrict__ x, double* __restrict__ r, const double* __restrict__ y,
            const double* __restrict__ z, const double* __restrict__ s, const double* __restrict__ t,
            const double* __restrict__ rhat, agx_krylov_scalars* sc, double* partials, unsigned* counter) {
  if (sc->converged) return;
  const double a = sc->alpha, om = sc->omega;
  double acc[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += a * y[i] + om * z[i];
    const double ri = s[i] - om * t[i];
    r[i] = ri;
    acc[0] += rhat[i] * ri;
    acc[1] += ri * ri;
  }
  double tot[2];
  if (reduce_last_block<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
    sc->iters += 1;
    sc->rr = tot[1];
    if (!isfinite(tot[1])) sc->converged = 2;
    else if (tot[1] <= sc->rr_stop) sc->converged = 1;
    else if (bad(tot[0]) || sc->omega == 0.0) sc->converged = 2;
    else {
      sc->beta = (tot[0] / sc->rho) * (a / om);
      sc->rho = tot[0];
    }
  }
}

__global__ void __launch_bounds__(AGX_BLOCK)
bicg_init(int64_t n, const double* __restrict__ b, double* __restrict__ x, double* __restrict__ r,
          double* __restrict__ rhat, double* __restrict__ p, double* __restrict__ v, agx_krylov_scalars* sc) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = 0.0;
    r[i] = b[i];
    rhat[i] = b[i];
    p[i] = 0.0;
    v[i] = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->rho = sc->rr;  // (rhat, r0) = (b, b)
    sc->beta = 0.0;
    sc->omega = 1.0;
    sc->alpha = 1.0;
  }
}

// ---- float64 flexible CG with a float32 preconditioner ---------------------------------
// f_r = r / ||b|| (float32), and back: z = f_z ||b||
__global__ void __launch_bounds__(AGX_BLOCK) to_f32_scaled(int64_t n, const double* __restrict__ r,
                                                           float* __restrict__ f, const agx_krylov_scalars* sc) {
  agx_pdl_entry();
  if (sc->converged) return;
  const double s = sc->extra[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    f[i] = (float)(r[i] * s);
}

__global__ void __launch_bounds__(AGX_BLOCK) from_f32_scaled(int64_t n, const float* __restrict__ f,
                                                             double* __restrict__ z, const agx_krylov_scalars* sc) {
  agx_pdl_entry();
  if (sc->converged) return;
  const double s = sc->extra[1];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = (double)f[i] * s;
}

// float32 copy of a float64 array (tangent values, inverse diagonal)
__global__ void copy_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// ---- conversions and helpers ---------------------------------------------------------
template <typename T>
__global__ void to_double_scaled(int64_t n, const T* __restrict__ x, double* __restrict__ out,
                                 const agx_krylov_scalars* sc, int scaled) {
  const double s = scaled ? sc->extra[1] : 1.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)x[i] * s;
}

__global__ void __launch_bounds__(AGX_BLOCK) masked_norm_kernel(int64_t n, const double* __restrict__ v,
                                                                const uint8_t* __restrict__ dmask, double* out,
                                                                double* partials, unsigned* counter) {
  double acc[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = dmask[i] ? 0.0 : v[i];
    acc[0] += x * x;
    if (!isfinite(x)) acc[1] += 1.0;
  }
  double tot[2];
  if (reduce_last_block<2>(acc, partials, counter, tot) && threadIdx.x == 0) {
    out[0] = tot[0];
    out[1] = tot[1];
  }
}

__global__ void set_dirichlet_kernel(int64_t n_dir, const int32_t* __restrict__ dir, double* __restrict__ dofs,
                                     const double* __restrict__ values) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n_dir; k += (int64_t)gridDim.x * blockDim.x)
    dofs[dir[k]] = values[dir[k]];
}

// dofs[free] += damping dx; dofs[prescribed] = values (solver.py:879-892)
__global__ void newton_update_kernel(int64_t n, double* __restrict__ dofs, const double* __restrict__ dx,
                                     const double* __restrict__ values, const uint8_t* __restrict__ dmask,
                                     double damping) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dofs[i] = dmask[i] ? values[i] : dofs[i] + damping * dx[i];
}

// dst = s * src on free DOFs, 0 on prescribed DOFs; s = -1 gives rhs = -R
// (solver.py:610-611 with the row deletion of solver.py:1514-1517)
__global__ void masked_scale_kernel(int64_t n, const double* __restrict__ src, double* __restrict__ dst,
                                    const uint8_t* __restrict__ dmask, double s) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = dmask[i] ? 0.0 : s * src[i];
}

template <typename T>
__global__ void zero_prescribed(int64_t n_dir, const int32_t* __restrict__ dir, T* __restrict__ v) {
  agx_pdl_entry();
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n_dir; k += (int64_t)gridDim.x * blockDim.x)
    v[dir[k]] = T(0);
}

template <int NDOF>
constexpr int tpr_for(int dim) {
  return NDOF == 1 ? (dim == 3 ? 8 : 4) : (NDOF == 2 ? 4 : 8);
}

// launch helpers dispatching on the block size
// One resident wave: blocks per SM from the occupancy calculator (cached per kernel), capped by
// the partials buffer (red_blocks).
template <class K>
int resident_grid(agx_context* ctx, K kernel) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, AGX_BLOCK, 0) != cudaSuccess || nb < 1) nb = 4;
  const int g = nb * ctx->sm_count;
  return g < ctx->red_blocks ? g : ctx->red_blocks;
}

// returns the grid (the number of block partials written)
template <typename T, int ND, int TP, int U = 2>
int spmv_dot_variant(agx_context* ctx, const T* vals, const T* z, const T* pold, T* pnew, T* q, const T* rflex) {
  static int g_cache = 0;
  if (!g_cache) g_cache = resident_grid(ctx, spmv_dot_kernel<T, ND, TP, U>);
  agx_launch_pdl(spmv_dot_kernel<T, ND, TP, U>, g_cache, AGX_BLOCK, 0, ctx->stream, ctx->n_nodes, ctx->d_rowptr, ctx->d_col,
                                                                        vals, ctx->nnzb, ctx->pattern_stencil, z, pold,
                                                                        pnew, q, ctx->d_scal, ctx->d_partials, rflex);
  return g_cache;
}


// default lanes per block row when the autotuner has not chosen one
int default_tpr(const agx_context* ctx) { return ctx->ndof == 1 ? (ctx->dim == 3 ? 8 : 4) : (ctx->ndof == 2 ? 4 : 8); }

template <typename T, int ND>
int spmv_dot_nd(agx_context* ctx, int tpr, const T* vals, const T* z, const T* pold, T* pnew, T* q,
                const T* rflex) {
  switch (tpr) {
    case 1: return spmv_dot_variant<T, ND, 1>(ctx, vals, z, pold, pnew, q, rflex);
    case 2: return spmv_dot_variant<T, ND, 2>(ctx, vals, z, pold, pnew, q, rflex);
    case 4: return spmv_dot_variant<T, ND, 4>(ctx, vals, z, pold, pnew, q, rflex);
    case 16: return spmv_dot_variant<T, ND, 16>(ctx, vals, z, pold, pnew, q, rflex);
    case 2 | SPMV_UNROLL4: return spmv_dot_variant<T, ND, 2, 4>(ctx, vals, z, pold, pnew, q, rflex);
    case 4 | SPMV_UNROLL4: return spmv_dot_variant<T, ND, 4, 4>(ctx, vals, z, pold, pnew, q, rflex);
    case 8 | SPMV_UNROLL4: return spmv_dot_variant<T, ND, 8, 4>(ctx, vals, z, pold, pnew, q, rflex);
    case SPMV_GRID:
      if constexpr (ND <= 2) return spmv_dot_variant<T, ND, 1, 0>(ctx, vals, z, pold, pnew, q, rflex);
      [[fallthrough]];
    case SPMV_GRID2:
      if constexpr (ND <= 2) return spmv_dot_variant<T, ND, 1, -2>(ctx, vals, z, pold, pnew, q, rflex);
      [[fallthrough]];
    case SPMV_BRICK:
      if (tpr == SPMV_BRICK) return spmv_dot_variant<T, ND, 1, -3>(ctx, vals, z, pold, pnew, q, rflex);
      [[fallthrough]];
    default: return spmv_dot_variant<T, ND, 8>(ctx, vals, z, pold, pnew, q, rflex);
  }
}

// rflex (flexible CG only): the residual whose dot with the new direction gives the step
template <typename T>
int launch_spmv_dot(agx_context* ctx, const T* vals, const T* z, const T* pold, T* pnew, T* q,
                    const T* rflex = nullptr) {
  agx_prof_scope ps(ctx, AGX_PROF_SPMV);
  const int tuned = ctx->spmv_tpr[std::is_same<T, float>::value ? 1 : 0];
  const int tpr = tuned > 0 ? tuned : default_tpr(ctx);
  if (ctx->ndof == 1) return spmv_dot_nd<T, 1>(ctx, tpr, vals, z, pold, pnew, q, rflex);
  if (ctx->ndof == 2) return spmv_dot_nd<T, 2>(ctx, tpr, vals, z, pold, pnew, q, rflex);
  return spmv_dot_nd<T, 3>(ctx, tpr, vals, z, pold, pnew, q, rflex);
}

template <int NDOF, int TPR>
void launch_bicg_spmvs(agx_context* ctx, int which, double* a, double* b, double* c) {
  const int g = ctx->red_blocks;
  if (which == 0)
    bicg_spmv_rhat<NDOF, TPR><<<g, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_nodes, ctx->d_rowptr, ctx->d_col,
                                                                ctx->d_vals64, ctx->nnzb, a, b, c, ctx->d_scal,
                                                                ctx->d_partials, ctx->d_counter);
  else
    bicg_spmv_ts<NDOF, TPR><<<g, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_nodes, ctx->d_rowptr, ctx->d_col, ctx->d_vals64,
                                                              ctx->nnzb, a, b, c, ctx->d_scal, ctx->d_partials,
                                                              ctx->d_counter);
}

void launch_bicg_spmv(agx_context* ctx, int which, double* a, double* b, double* c) {
  agx_prof_scope ps(ctx, AGX_PROF_SPMV);
  if (ctx->ndof == 1) {
    if (ctx->dim == 3) launch_bicg_spmvs<1, 8>(ctx, which, a, b, c);
    else launch_bicg_spmvs<1, 4>(ctx, which, a, b, c);
  } else if (ctx->ndof == 2) {
    launch_bicg_spmvs<2, 4>(ctx, which, a, b, c);
  } else {
    launch_bicg_spmvs<3, 8>(ctx, which, a, b, c);
  }
}

// Issues kn iterations through `chunk`: full chunks of an even length replay a CUDA graph
// captured at the first use (keyed by the output vector; re-captured when it changes), the
// remainder is launched directly.  `counted`: the launches the caller has already added to
// the context's count for this chunk; a replay replaces them by the graph's kernel nodes,
// which include a registered preconditioner's own kernels.
template <class F>
int run_chunk(agx_context* ctx, int slot, const void* x, int every, int kn, F&& chunk, int64_t counted,
              int64_t pc_key = -1) {
  auto& gr = ctx->graphs[slot];
  // events recorded by graph nodes cannot be timed: profiling runs launch directly
  if (!ctx->use_graphs || ctx->prof_on || kn != every || every % 2 != 0) {
    chunk(kn);
    AGX_CHECK_LAUNCH(ctx);
    return AGX_OK;
  }
  const cudaStream_t work = ctx->stream;
  const bool legacy = work == nullptr || work == cudaStreamLegacy;
  if (legacy && !ctx->graph_stream) {
    AGX_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->graph_stream, cudaStreamNonBlocking));
    AGX_CUDA(ctx, cudaEventCreateWithFlags(&ctx->graph_ev[0], cudaEventDisableTiming));
    AGX_CUDA(ctx, cudaEventCreateWithFlags(&ctx->graph_ev[1], cudaEventDisableTiming));
  }
  const cudaStream_t gs = legacy ? ctx->graph_stream : work;
  if (!gr.exec || gr.key_x != x || gr.every != every || gr.prof != ctx->prof_on ||
      gr.tpr != ctx->spmv_tpr[0] * 4096 + ctx->spmv_tpr[1] || gr.pc_key != pc_key || gr.pdl != g_agx_pdl) {
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
    gr.exec = nullptr;
    for (auto& v : gr.ev) {
      for (auto e : v) cudaEventDestroy(e);
      v.clear();
    }
    cudaGraph_t graph = nullptr;
    const int64_t launches_before = ctx->n_launches;
    AGX_CUDA(ctx, cudaStreamBeginCapture(gs, cudaStreamCaptureModeThreadLocal));
    ctx->capturing = &gr;
    ctx->stream = gs;  // the chunk's launches go to the capturing stream
    chunk(every);
    ctx->stream = work;
    ctx->capturing = nullptr;
    ctx->n_launches = launches_before;  // captured, not launched: the replay below counts them
    cudaError_t e = cudaStreamEndCapture(gs, &graph);
    if (e != cudaSuccess) return agx_fail(ctx, AGX_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    size_t nn = 0;
    gr.kernels = 0;
    if (cudaGraphGetNodes(graph, nullptr, &nn) == cudaSuccess && nn > 0) {
      std::vector<cudaGraphNode_t> nodes(nn);
      if (cudaGraphGetNodes(graph, nodes.data(), &nn) == cudaSuccess)
        for (size_t i = 0; i < nn; ++i) {
          cudaGraphNodeType t;
          if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++gr.kernels;
        }
    }
    e = cudaGraphInstantiate(&gr.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return agx_fail(ctx, AGX_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
    gr.key_x = x;
    gr.every = every;
    gr.prof = ctx->prof_on;
    gr.tpr = ctx->spmv_tpr[0] * 4096 + ctx->spmv_tpr[1];
    gr.pc_key = pc_key;
    gr.pdl = g_agx_pdl;
  }
  if (legacy) {
    AGX_CUDA(ctx, cudaEventRecord(ctx->graph_ev[0], work));
    AGX_CUDA(ctx, cudaStreamWaitEvent(gs, ctx->graph_ev[0], 0));
    AGX_CUDA(ctx, cudaGraphLaunch(gr.exec, gs));
    AGX_CUDA(ctx, cudaEventRecord(ctx->graph_ev[1], gs));
    AGX_CUDA(ctx, cudaStreamWaitEvent(work, ctx->graph_ev[1], 0));
  } else {
    AGX_CUDA(ctx, cudaGraphLaunch(gr.exec, work));
  }
  ctx->n_launches += gr.kernels - counted;
  if (gr.prof) {
    // the replay re-recorded the graph's events: add their times once the chunk is done
    AGX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < AGX_PROF_CATEGORIES; ++c)
      for (size_t i = 0; i + 1 < gr.ev[c].size(); i += 2) {
        float t = 0;
        AGX_CUDA(ctx, cudaEventElapsedTime(&t, gr.ev[c][i], gr.ev[c][i + 1]));
        ctx->prof_extra_ms[c] += t;
        ctx->prof_extra_n[c] += 1;
      }
  }
  return AGX_OK;
}

int read_scalars(agx_context* ctx) {
  AGX_CUDA(ctx, cudaMemcpyAsync(ctx->h_scal, ctx->d_scal, sizeof(agx_krylov_scalars), cudaMemcpyDeviceToHost,
                                ctx->stream));
  AGX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->debug) {
    const agx_krylov_scalars& s = *ctx->h_scal;
    fprintf(stderr, "[agx] it=%d conv=%d rz=%.6e rr=%.6e pq=%.6e alpha=%.6e beta=%.6e rr_stop=%.6e\n", s.iters,
            s.converged, s.rz, s.rr, s.pq, s.alpha, s.beta, s.rr_stop);
  }
  return AGX_OK;
}

}  // namespace

template <typename T>
__global__ void planes_to_blocks_kernel(int64_t nnzb, int bs, const T* __restrict__ planes, T* __restrict__ blocks) {
  const int64_t total = nnzb * bs;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = t / bs;
    const int e = (int)(t - k * bs);
    blocks[t] = planes[(int64_t)e * nnzb + k];
  }
}

void agx_launch_planes_to_blocks(agx_context* ctx, const double* planes, double* blocks) {
  const int bs = ctx->ndof * ctx->ndof;
  planes_to_blocks_kernel<double><<<agx_grid(ctx, ctx->nnzb * bs), AGX_BLOCK, 0, ctx->stream>>>(ctx->nnzb, bs, planes,
                                                                                               blocks);
  ctx->n_launches += 1;
}

void agx_launch_planes_to_blocks(agx_context* ctx, const float* planes, float* blocks) {
  const int bs = ctx->ndof * ctx->ndof;
  planes_to_blocks_kernel<float><<<agx_grid(ctx, ctx->nnzb * bs), AGX_BLOCK, 0, ctx->stream>>>(ctx->nnzb, bs, planes,
                                                                                             blocks);
  ctx->n_launches += 1;
}

template <typename T>
__global__ void fill_kernel(int64_t n, T* __restrict__ v, T value) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = value;
}

// Times the fused product for every lanes-per-row candidate on the last assembled tangent (its
// precision) and keeps the fastest (the Krylov scalars are reset afterwards by the next solve).
// The operand is all ones and the solve scalars are cleared before every timed launch: a
// product whose (p, A p) came out zero would flag a breakdown and turn the following launches
// into no-ops.
int agx_autotune_spmv(agx_context* ctx, int* chosen, float* best_ms) {
  if (ctx->tangent_valid != AGX_F32 && ctx->tangent_valid != AGX_F64)
    return agx_fail(ctx, AGX_ERR_STATE, "autotune needs an assembled tangent");
  const bool f32 = ctx->tangent_valid == AGX_F32;
  std::vector<int> cands = {1, 2, 4, 8, 16, 2 | SPMV_UNROLL4, 4 | SPMV_UNROLL4, 8 | SPMV_UNROLL4};
  if (ctx->pattern_grid_ny > 0) {
    cands.push_back(SPMV_GRID);
    cands.push_back(SPMV_GRID2);
  }
  // the brick product stages scalar rows only; for node blocks its unstaged form (a thread's 9
  // blocks of 3 x 3 in registers) lost to the BSR variants inside the 64^3 neo-Hooke solve
  if (ctx->pattern_brick > 0 && ctx->ndof == 1) cands.push_back(SPMV_BRICK);
  cudaEvent_t e0, e1;
  AGX_CUDA(ctx, cudaEventCreate(&e0));
  AGX_CUDA(ctx, cudaEventCreate(&e1));
  AGX_CUDA(ctx, cudaMemsetAsync(ctx->d_scal, 0, sizeof(agx_krylov_scalars), ctx->stream));
  const int gv = agx_grid(ctx, ctx->n_dofs);
  fill_kernel<float><<<gv, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dofs, ctx->f_z, 1.0f);
  fill_kernel<double><<<gv, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dofs, ctx->d_z, 1.0);
  AGX_CUDA(ctx, cudaMemsetAsync(ctx->f_p, 0, sizeof(float) * ctx->n_dofs, ctx->stream));
  AGX_CUDA(ctx, cudaMemsetAsync(ctx->d_p, 0, sizeof(double) * ctx->n_dofs, ctx->stream));
  float best = 1e30f;
  int pick = default_tpr(ctx);
  for (int c : cands) {
    if (ctx->ndof == 3 && spmv_lanes(c) < 4 && c != SPMV_BRICK) continue;
    auto run = [&]() {
      cudaMemsetAsync(ctx->d_scal, 0, sizeof(agx_krylov_scalars), ctx->stream);
      if (f32) {
        if (ctx->ndof == 1)
          spmv_dot_nd<float, 1>(ctx, c, ctx->d_vals32, ctx->f_z, ctx->f_p, ctx->f_rold, ctx->f_q, nullptr);
        else if (ctx->ndof == 2)
          spmv_dot_nd<float, 2>(ctx, c, ctx->d_vals32, ctx->f_z, ctx->f_p, ctx->f_rold, ctx->f_q, nullptr);
        else
          spmv_dot_nd<float, 3>(ctx, c, ctx->d_vals32, ctx->f_z, ctx->f_p, ctx->f_rold, ctx->f_q, nullptr);
      } else {
        if (ctx->ndof == 1)
          spmv_dot_nd<double, 1>(ctx, c, ctx->d_vals64, ctx->d_z, ctx->d_p, ctx->d_s, ctx->d_q, nullptr);
        else if (ctx->ndof == 2)
          spmv_dot_nd<double, 2>(ctx, c, ctx->d_vals64, ctx->d_z, ctx->d_p, ctx->d_s, ctx->d_q, nullptr);
        else
          spmv_dot_nd<double, 3>(ctx, c, ctx->d_vals64, ctx->d_z, ctx->d_p, ctx->d_s, ctx->d_q, nullptr);
      }
    };
    for (int w = 0; w < 3; ++w) run();
    AGX_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
    for (int r = 0; r < 10; ++r) run();
    AGX_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
    AGX_CUDA(ctx, cudaEventSynchronize(e1));
    float ms = 0;
    AGX_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
    ms /= 10.0f;
    if (ms < best) {
      best = ms;
      pick = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  AGX_CHECK_LAUNCH(ctx);
  ctx->spmv_tpr[f32 ? 1 : 0] = pick;
  if (chosen) *chosen = pick;
  if (best_ms) *best_ms = best;
  return AGX_OK;
}

int agx_spmv_impl(agx_context* ctx, int dtype, const void* x, void* y) {
  return agx_spmv_values_impl(ctx, dtype, dtype == AGX_F64 ? (const void*)ctx->d_vals64 : (const void*)ctx->d_vals32,
                              x, y);
}

void agx_launch_jacobi(agx_context* ctx, int dtype, const void* r, void* z) {
  const int gv = agx_grid(ctx, ctx->n_dofs);
  if (dtype == AGX_F64)
    jacobi_dinv<double><<<gv, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dofs, ctx->d_dinv64, (const double*)r, (double*)z);
  else
    jacobi_dinv<float><<<gv, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dofs, ctx->d_dinv32, (const float*)r, (float*)z);
  ctx->n_launches += 1;
}

template <typename T, int ND>
void spmv_nd(agx_context* ctx, int tpr, int g, const T* v, const T* x, T* y) {
  const int64_t nr = ctx->n_nodes;
  const int gny = ctx->pattern_stencil;
  switch (tpr) {
    case 1: spmv_kernel<T, ND, 1><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y); break;
    case 2: spmv_kernel<T, ND, 2><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y); break;
    case 4: spmv_kernel<T, ND, 4><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y); break;
    case 16: spmv_kernel<T, ND, 16><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y); break;
    case 2 | SPMV_UNROLL4: spmv_kernel<T, ND, 2, 4><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y); break;
    case 4 | SPMV_UNROLL4: spmv_kernel<T, ND, 4, 4><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y); break;
    case 8 | SPMV_UNROLL4: spmv_kernel<T, ND, 8, 4><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y); break;
    case SPMV_GRID:
      if constexpr (ND <= 2) {
        spmv_kernel<T, ND, 1, 0><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y);
        break;
      }
      [[fallthrough]];
    case SPMV_GRID2:
      if constexpr (ND <= 2) {
        spmv_kernel<T, ND, 1, -2><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y);
        break;
      }
      [[fallthrough]];
    case SPMV_BRICK:
      if (tpr == SPMV_BRICK) {
        spmv_kernel<T, ND, 1, -3><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y);
        break;
      }
      [[fallthrough]];
    default: spmv_kernel<T, ND, 8><<<g, AGX_BLOCK, 0, ctx->stream>>>(nr, ctx->d_rowptr, ctx->d_col, v, ctx->nnzb, gny, x, y); break;
  }
}

// y = K x with the lanes per row the autotuner chose for the precision (the fused product's)
int agx_spmv_values_impl(agx_context* ctx, int dtype, const void* values, const void* x, void* y) {
  const int64_t nr = ctx->n_nodes;
  const int tuned = ctx->spmv_tpr[dtype == AGX_F32 ? 1 : 0];
  const int tpr = tuned > 0 ? tuned : default_tpr(ctx);
  const int g = agx_grid(ctx, nr * spmv_lanes(tpr), 8);
  auto go = [&](auto tag) {
    using T = decltype(tag);
    const T* v = (const T*)values;
    if (ctx->ndof == 1) spmv_nd<T, 1>(ctx, tpr, g, v, (const T*)x, (T*)y);
    else if (ctx->ndof == 2) spmv_nd<T, 2>(ctx, tpr, g, v, (const T*)x, (T*)y);
    else spmv_nd<T, 3>(ctx, tpr, g, v, (const T*)x, (T*)y);
  };
  if (dtype == AGX_F64) go(double{});
  else go(float{});
  AGX_CHECK_LAUNCH(ctx);
  return AGX_OK;
}

void agx_launch_set_dirichlet(agx_context* ctx, double* dofs, const double* values) {
  ctx->n_launches += ctx->n_dir > 0 ? 1 : 0;
  if (ctx->n_dir > 0)
    set_dirichlet_kernel<<<agx_grid(ctx, ctx->n_dir), AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dir, ctx->d_dir_dofs, dofs,
                                                                                  values);
}

void agx_launch_newton_update(agx_context* ctx, double* dofs, const double* dx, const double* values, double damping) {
  ctx->n_launches += 1;
  newton_update_kernel<<<agx_grid(ctx, ctx->n_dofs), AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dofs, dofs, dx, values,
                                                                                  ctx->d_dmask_dof, damping);
}

void agx_launch_negate_free(agx_context* ctx, const double* R, double* b) {
  agx_launch_masked_scale(ctx, R, b, -1.0);
}

void agx_launch_masked_scale(agx_context* ctx, const double* src, double* dst, double s) {
  ctx->n_launches += 1;
  masked_scale_kernel<<<agx_grid(ctx, ctx->n_dofs), AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dofs, src, dst,
                                                                                ctx->d_dmask_dof, s);
}

int agx_residual_norm(agx_context* ctx, const double* R, double* norm2, double* nonfinite) {
  ctx->n_launches += 1;
  masked_norm_kernel<<<ctx->vec_blocks, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dofs, R, ctx->d_dmask_dof, ctx->d_norm,
                                                                   ctx->d_partials, ctx->d_counter);
  AGX_CHECK_LAUNCH(ctx);
  AGX_CUDA(ctx, cudaMemcpyAsync(ctx->h_norm, ctx->d_norm, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  AGX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *norm2 = ctx->h_norm[0];
  *nonfinite = ctx->h_norm[1];
  return AGX_OK;
}

// z = M(r) on the float32 Krylov vectors (f_r -> f_z) for the flexible method; VT the stored
// values the products read (float, or the bf16 smoothing copy)
template <int ND, int EPI, typename VT>
void tl_spmv_nd(agx_context* ctx, int code, int g, const VT* vals, const float* x, float* rc, float a, float b,
                float* dnew, float* tout) {
  auto* sc = ctx->d_scal;
  const int64_t nr = ctx->n_nodes;
#define AGX_TL(TP_, U_)                                                                                         \
  agx_launch_pdl(tl_spmv<ND, TP_, U_, EPI, VT>, g, AGX_BLOCK, 0, ctx->stream, nr, ctx->d_rowptr, ctx->d_col, \
                 vals, ctx->nnzb, ctx->pattern_stencil, x, rc, ctx->d_dinv32, a, b, dnew, ctx->f_z, tout, sc,   \
                 ctx->d_partials)
  switch (code) {
    case 1: AGX_TL(1, 2); break;
    case 2: AGX_TL(2, 2); break;
    case 4: AGX_TL(4, 2); break;
    case 16: AGX_TL(16, 2); break;
    case 2 | SPMV_UNROLL4: AGX_TL(2, 4); break;
    case 4 | SPMV_UNROLL4: AGX_TL(4, 4); break;
    case 8 | SPMV_UNROLL4: AGX_TL(8, 4); break;
    case SPMV_GRID:
      if constexpr (ND <= 2) {
        AGX_TL(1, 0);
        break;
      }
      [[fallthrough]];
    case SPMV_GRID2:
      if constexpr (ND <= 2) {
        AGX_TL(1, -2);
        break;
      }
      [[fallthrough]];
    case SPMV_BRICK:
      if (code == SPMV_BRICK) {
        AGX_TL(1, -3);
        break;
      }
      [[fallthrough]];
    default: AGX_TL(8, 2); break;
  }
#undef AGX_TL
}

// t = K x with the step's element-wise work (TL_SWEEP / TL_RESID / TL_STEP), the float32 tangent,
// the autotuner's product variant for float32
template <int EPI>
void launch_tl_spmv(agx_context* ctx, const float* x, float* rc, float a, float b, float* dnew, float* tout) {
  agx_prof_scope ps(ctx, AGX_PROF_SMOOTH);
  const int tuned = ctx->spmv_tpr[1];
  const int code = tuned > 0 ? tuned : default_tpr(ctx);
  // a reducing kernel writes one partial per block: its grid stays within the partials buffer
  const int g = EPI == TL_STEP ? ctx->red_blocks : agx_grid(ctx, ctx->n_nodes * spmv_lanes(code), 8);
  auto go = [&](auto* vals) {
    using VT = std::remove_const_t<std::remove_pointer_t<decltype(vals)>>;
    if (ctx->ndof == 1) tl_spmv_nd<1, EPI, VT>(ctx, code, g, vals, x, rc, a, b, dnew, tout);
    else if (ctx->ndof == 2) tl_spmv_nd<2, EPI, VT>(ctx, code, g, vals, x, rc, a, b, dnew, tout);
    else tl_spmv_nd<3, EPI, VT>(ctx, code, g, vals, x, rc, a, b, dnew, tout);
  };
  if (ctx->precond_bf16) go(ctx->d_vals16);
  else go(ctx->d_vals32);
  ctx->n_launches += 1;
}

int apply_registered_preconditioner(agx_context* ctx) {
  const int64_t n = ctx->n_dofs;
  const int gv = agx_grid(ctx, n);
  auto* sc = ctx->d_scal;
  if (ctx->precond_mode == 0) {
    agx_prof_scope pn(ctx, AGX_PROF_PRECOND);
    if (ctx->precond(ctx->precond_user, ctx->f_r, ctx->f_z, n, ctx->stream) != 0) return -1;
    agx_launch_pdl(zero_prescribed<float>, agx_grid(ctx, ctx->n_dir), AGX_BLOCK, 0, ctx->stream, ctx->n_dir, ctx->d_dir_dofs,
                                                                                   ctx->f_z);
    ctx->n_launches += 1;
    return 0;
  }
  // nu smoothing steps from z = 0 (the running residual rc = r - K z in f_w2, the last
  // increment in f_w4, products in f_w1), then y = M(rc) in f_w3 with the energy-optimal step
  // c = (rc, y) / (y, K y), z += c y, and in modes 2 and 3 nu post-smoothing steps.  Modes 1
  // and 2 smooth with damped Jacobi (weight w); mode 3 with the Chebyshev polynomial of
  // degree nu for D^-1 K on [w lmax, lmax], lmax the Gershgorin bound of the tangent.
  const int nu = ctx->precond_sweeps;
  float ca[16], cb[16];
  if (ctx->precond_mode == 3) {
    const double lmax = ctx->cheb_lmax, lmin = ctx->precond_omega * lmax;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
    double rho = 1.0 / sigma;
    ca[0] = 0.0f;
    cb[0] = (float)(1.0 / theta);
    for (int k = 1; k < nu; ++k) {
      const double rn = 1.0 / (2.0 * sigma - rho);
      ca[k] = (float)(rn * rho);
      cb[k] = (float)(2.0 * rn / delta);
      rho = rn;
    }
  } else {
    for (int k = 0; k < nu; ++k) {
      ca[k] = 0.0f;
      cb[k] = (float)ctx->precond_omega;
    }
  }
  // rc the running residual r - K z, y the network's output, dA / dB the increments of
  // consecutive smoothing steps (a step reads the previous one while writing its own), t = K y.
  // Profiling categories: the products (with their fused element-wise work) under
  // AGX_PROF_SMOOTH, the element-wise kernels under AGX_PROF_VECTOR, the registered callback
  // (the network) under AGX_PROF_PRECOND.
  float *rc = ctx->f_w2, *y = ctx->f_w3, *dA = ctx->f_w4, *dB = ctx->f_w1, *t = ctx->f_w1;
  {
    agx_prof_scope pv(ctx, AGX_PROF_VECTOR);  // first step from z = 0: rc = r, d = b0 D^-1 r, z = d
    agx_launch_pdl(tl_sweep, gv, AGX_BLOCK, 0, ctx->stream, n, ctx->d_dinv32, cb[0], ca[0], ctx->f_r, rc, nullptr, ctx->f_z, dA,
                                                1, sc);
    ctx->n_launches += 1;
  }
  for (int s = 1; s < nu; ++s) {
    launch_tl_spmv<TL_SWEEP>(ctx, dA, rc, ca[s], cb[s], dB, nullptr);
    std::swap(dA, dB);
  }
  launch_tl_spmv<TL_RESID>(ctx, dA, rc, 0.0f, 0.0f, nullptr, nullptr);
  {
    agx_prof_scope pn(ctx, AGX_PROF_PRECOND);
    if (ctx->precond(ctx->precond_user, rc, y, n, ctx->stream) != 0) return -1;
    agx_launch_pdl(zero_prescribed<float>, agx_grid(ctx, ctx->n_dir), AGX_BLOCK, 0, ctx->stream, ctx->n_dir, ctx->d_dir_dofs, y);
    ctx->n_launches += 1;
  }
  launch_tl_spmv<TL_STEP>(ctx, y, rc, 0.0f, 0.0f, nullptr, t);
  agx_launch_pdl(tl_finish_step, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, ctx->red_blocks);
  ctx->n_launches += 1;
  if (ctx->precond_mode < 2) {
    agx_prof_scope pv(ctx, AGX_PROF_VECTOR);
    agx_launch_pdl(tl_combine, gv, AGX_BLOCK, 0, ctx->stream, n, ctx->f_z, y, rc, t, sc);
    ctx->n_launches += 1;
    return 0;
  }
  // z += c y, rc -= c t and the first post-smoothing step in one kernel; then the others
  float *pA = ctx->f_w4, *pB = ctx->f_w1;  // t (in f_w1) is consumed by the combined kernel
  {
    agx_prof_scope pv(ctx, AGX_PROF_VECTOR);
    agx_launch_pdl(tl_combine_sweep, gv, AGX_BLOCK, 0, ctx->stream, n, ctx->f_z, y, rc, t, ctx->d_dinv32, cb[0], pA, sc);
    ctx->n_launches += 1;
  }
  for (int s = 1; s < nu; ++s) {
    launch_tl_spmv<TL_SWEEP>(ctx, pA, rc, ca[s], cb[s], pB, nullptr);
    std::swap(pA, pB);
  }
  return 0;
}

// bf16 copy of the float32 tangent's values for the two-level products
// (AGX_PRECOND_BF16_SMOOTHING), made once per assembled tangent (before any capture)
__global__ void copy_to_bf16(int64_t n, const float* __restrict__ src, __nv_bfloat16* __restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = __float2bfloat16(src[i]);
}

int ensure_bf16_copy(agx_context* ctx) {
  if (!ctx->precond_bf16 || ctx->precond_mode == 0 || ctx->bf16_copy_gen == ctx->tangent_gen) return AGX_OK;
  const int64_t nv = ctx->nnzb * ctx->ndof * ctx->ndof;
  if (!ctx->d_vals16) AGX_CUDA(ctx, cudaMalloc(&ctx->d_vals16, sizeof(__nv_bfloat16) * std::max<int64_t>(1, nv)));
  copy_to_bf16<<<agx_grid(ctx, nv), AGX_BLOCK, 0, ctx->stream>>>(nv, ctx->d_vals32, ctx->d_vals16);
  AGX_CHECK_LAUNCH(ctx);
  ctx->n_launches += 1;
  ctx->bf16_copy_gen = ctx->tangent_gen;
  return AGX_OK;
}

// float32 copy of the float64 tangent (values and inverse diagonal) for the float32
// preconditioner of the float64 flexible CG, made once per assembled tangent
int ensure_f32_copy(agx_context* ctx) {
  if (ctx->tangent_valid != AGX_F64)
    return agx_fail(ctx, AGX_ERR_STATE, "float64 flexible CG needs a float64 tangent (assemble first)");
  if (ctx->f32_copy_gen == ctx->tangent_gen) return AGX_OK;
  const int64_t nv = ctx->nnzb * ctx->ndof * ctx->ndof;
  copy_to_f32<<<agx_grid(ctx, nv), AGX_BLOCK, 0, ctx->stream>>>(nv, ctx->d_vals64, ctx->d_vals32);
  copy_to_f32<<<agx_grid(ctx, ctx->n_dofs), AGX_BLOCK, 0, ctx->stream>>>(ctx->n_dofs, ctx->d_dinv64, ctx->d_dinv32);
  AGX_CHECK_LAUNCH(ctx);
  ctx->n_launches += 2;
  ctx->f32_copy_gen = ctx->tangent_gen;
  return AGX_OK;
}

// Gershgorin bound for the Chebyshev smoother, recomputed once per float32 tangent (host
// synchronisation; called before any capture)
int update_chebyshev_bound(agx_context* ctx) {
  if (ctx->precond_mode != 3 || ctx->cheb_gen == ctx->tangent_gen) return AGX_OK;
  const int g = ctx->red_blocks;
  float* bm = reinterpret_cast<float*>(ctx->d_partials);  // red_blocks * 4 doubles: room to spare
  if (ctx->ndof == 1)
    gershgorin_kernel<1><<<g, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_nodes, ctx->d_rowptr, ctx->d_diagpos,
                                                           ctx->d_vals32, ctx->nnzb, bm);
  else if (ctx->ndof == 2)
    gershgorin_kernel<2><<<g, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_nodes, ctx->d_rowptr, ctx->d_diagpos,
                                                           ctx->d_vals32, ctx->nnzb, bm);
  else
    gershgorin_kernel<3><<<g, AGX_BLOCK, 0, ctx->stream>>>(ctx->n_nodes, ctx->d_rowptr, ctx->d_diagpos,
                                                           ctx->d_vals32, ctx->nnzb, bm);
  std::vector<float> h(g);
  AGX_CUDA(ctx, cudaMemcpyAsync(h.data(), bm, sizeof(float) * g, cudaMemcpyDeviceToHost, ctx->stream));
  AGX_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  float m = 0.0f;
  for (float v : h) m = v > m ? v : m;
  ctx->cheb_lmax = m > 0.0f ? m : 2.0;
  ctx->cheb_gen = ctx->tangent_gen;
  ctx->precond_gen += 1;  // the coefficients are baked into captured graphs
  ctx->n_launches += 1;
  return AGX_OK;
}

int agx_krylov_impl(agx_context* ctx, const double* rhs, double* x, const agx_solve_opts* opts, agx_solve_info* info) {
  if (opts->method == AGX_CHOL_BAND) return agx_band_solve_impl(ctx, rhs, x, opts, info);
  const int64_t n = ctx->n_dofs;
  const int g = ctx->vec_blocks;  // reducing vector kernels
  const int gv = agx_grid(ctx, n);
  const int method = opts->method;
  const int every = opts->check_every > 0 ? opts->check_every : 16;
  const int maxiter = opts->maxiter > 0 ? opts->maxiter : 10000;
  auto* sc = ctx->d_scal;
  if ((method == AGX_PCG || method == AGX_BICGSTAB) && ctx->tangent_valid != AGX_F64)
    return agx_fail(ctx, AGX_ERR_STATE, "float64 Krylov method needs a float64 tangent (assemble first)");
  if ((method == AGX_PCG_MIXED || method == AGX_FCG_MIXED) && ctx->tangent_valid != AGX_F32)
    return agx_fail(ctx, AGX_ERR_STATE, "mixed Krylov method needs a float32 tangent (assemble first)");

  norm_init_kernel<<<g, AGX_BLOCK, 0, ctx->stream>>>(n, rhs, sc, ctx->d_partials, ctx->d_counter, opts->rtol,
                                                    opts->atol);
  AGX_CHECK_LAUNCH(ctx);
  ctx->n_launches += 2;  // norm + method initialisation
  int it_done = 0;
  if (method == AGX_PCG) {
    // two direction buffers used alternately: the product of iteration k forms p_k from
    // z_k and p_(k-1) (d_p and d_s; BiCGStab's s is free here)
    double* pbuf[2] = {ctx->d_p, ctx->d_s};
    int cur = 0;
    pcg_init_kernel<double><<<g, AGX_BLOCK, 0, ctx->stream>>>(n, rhs, ctx->d_dinv64, x, ctx->d_r, ctx->d_z, pbuf[0],
                                                             sc, ctx->d_partials, ctx->d_counter, 0, 1);
    auto chunk = [&](int kn) {
      for (int k = 0; k < kn; ++k) {
        double* pnew = pbuf[cur ^ 1];
        const int ns = launch_spmv_dot<double>(ctx, ctx->d_vals64, ctx->d_z, pbuf[cur], pnew, ctx->d_q);
        agx_launch_pdl(pcg_finish_pq, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, ns);
        agx_prof_scope ps(ctx, AGX_PROF_VECTOR);
        agx_launch_pdl(pcg_update_kernel<double>, g, AGX_BLOCK, 0, ctx->stream, n, x, ctx->d_r, ctx->d_z, pnew, ctx->d_q,
                                                                   ctx->d_dinv64, sc, ctx->d_partials);
        agx_launch_pdl(pcg_finish_rz, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, g);
        cur ^= 1;
      }
    };
    while (true) {
      const int kn = std::min(every, maxiter - it_done);
      ctx->n_launches += 4 * kn;
      if (int rc = run_chunk(ctx, 0, x, every, kn, chunk, 4 * kn)) return rc;
      int rc = read_scalars(ctx);
      if (rc) return rc;
      it_done = ctx->h_scal->iters;
      if (ctx->h_scal->converged || it_done >= maxiter) break;
    }
  } else if (method == AGX_PCG_MIXED || method == AGX_FCG_MIXED) {
    const bool flexible = method == AGX_FCG_MIXED && ctx->precond != nullptr;
    bool precond_failed = false;
    float* pbuf[2] = {ctx->f_p, ctx->f_rold};
    int cur = 0;
    pcg_init_kernel<float><<<g, AGX_BLOCK, 0, ctx->stream>>>(n, rhs, ctx->d_dinv32, ctx->f_x, ctx->f_r, ctx->f_z,
                                                            pbuf[0], sc, ctx->d_partials, ctx->d_counter, 1,
                                                            flexible ? 0 : 1);
    if (flexible) {
      if (int rc = update_chebyshev_bound(ctx)) return rc;
      if (int rc = ensure_bf16_copy(ctx)) return rc;
      if (apply_registered_preconditioner(ctx) != 0)
        return agx_fail(ctx, AGX_ERR_ARG, "preconditioner callback failed");
      agx_launch_pdl(fcg_direction_dots<float>, g, AGX_BLOCK, 0, ctx->stream, n, ctx->f_r, ctx->f_z, ctx->f_q, sc, ctx->d_partials);
      agx_launch_pdl(fcg_finish_direction, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, g);
      ctx->n_launches += 3;
    }
    auto chunk = [&](int kn) {
      for (int k = 0; k < kn; ++k) {
        float* pnew = pbuf[cur ^ 1];
        const int ns = launch_spmv_dot<float>(ctx, ctx->d_vals32, ctx->f_z, pbuf[cur], pnew, ctx->f_q,
                                              flexible ? (const float*)ctx->f_r : nullptr);
        if (!flexible) {
          agx_launch_pdl(pcg_finish_pq, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, ns);
          agx_prof_scope ps(ctx, AGX_PROF_VECTOR);
          agx_launch_pdl(pcg_update_kernel<float>, g, AGX_BLOCK, 0, ctx->stream, n, ctx->f_x, ctx->f_r, ctx->f_z, pnew,
                                                                    ctx->f_q, ctx->d_dinv32, sc, ctx->d_partials);
          agx_launch_pdl(pcg_finish_rz, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, g);
        } else {
          agx_launch_pdl(fcg_finish_pq, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, ns);
          {
            agx_prof_scope ps(ctx, AGX_PROF_VECTOR);
            agx_launch_pdl(fcg_update_kernel<float>, g, AGX_BLOCK, 0, ctx->stream, n, ctx->f_x, ctx->f_r, pnew, ctx->f_q, sc,
                                                                      ctx->d_partials);
            agx_launch_pdl(fcg_finish_update, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, g);
          }
          if (apply_registered_preconditioner(ctx) != 0) precond_failed = true;
          agx_launch_pdl(fcg_direction_dots<float>, g, AGX_BLOCK, 0, ctx->stream, n, ctx->f_r, ctx->f_z, ctx->f_q, sc,
                                                                     ctx->d_partials);
          agx_launch_pdl(fcg_finish_direction, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, g);
          ctx->n_launches += 2;  // the flexible iteration's two extra finishers
        }
        cur ^= 1;
      }
    };
    while (true) {
      const int kn = std::min(every, maxiter - it_done);
      ctx->n_launches += 4 * kn;
      if (flexible && !ctx->precond_capturable) {
        chunk(kn);  // a preconditioner that may synchronise or allocate: no graph
        AGX_CHECK_LAUNCH(ctx);
      } else if (int rc = run_chunk(ctx, 1, ctx->f_x, every, kn, chunk, 4 * kn, flexible ? ctx->precond_gen : -1)) {
        return rc;
      }
      if (precond_failed) return agx_fail(ctx, AGX_ERR_ARG, "preconditioner callback failed");
      int rc = read_scalars(ctx);
      if (rc) return rc;
      it_done = ctx->h_scal->iters;
      if (ctx->h_scal->converged || it_done >= maxiter) break;
    }
    to_double_scaled<float><<<gv, AGX_BLOCK, 0, ctx->stream>>>(n, ctx->f_x, x, sc, 1);
    ctx->n_launches += 1;
  } else if (method == AGX_FCG_F64) {
    if (int rc = ensure_f32_copy(ctx)) return rc;
    const bool flexible = ctx->precond != nullptr;
    bool precond_failed = false;
    double* pbuf[2] = {ctx->d_p, ctx->d_s};
    int cur = 0;
    pcg_init_kernel<double><<<g, AGX_BLOCK, 0, ctx->stream>>>(n, rhs, ctx->d_dinv64, x, ctx->d_r, ctx->d_z, pbuf[0],
                                                             sc, ctx->d_partials, ctx->d_counter, 0, flexible ? 0 : 1);
    // z = M r: the float32 preconditioner on r / ||b|| (Jacobi in float64 without a callback)
    auto precond = [&]() {
      if (!flexible) {
        agx_prof_scope pv(ctx, AGX_PROF_VECTOR);
        agx_launch_pdl(jacobi_apply<double>, gv, AGX_BLOCK, 0, ctx->stream, n, ctx->d_dinv64, ctx->d_r, ctx->d_z, sc);
        ctx->n_launches += 1;
        return;
      }
      {
        agx_prof_scope pv(ctx, AGX_PROF_VECTOR);
        agx_launch_pdl(to_f32_scaled, gv, AGX_BLOCK, 0, ctx->stream, n, ctx->d_r, ctx->f_r, sc);
      }
      if (apply_registered_preconditioner(ctx) != 0) precond_failed = true;
      {
        agx_prof_scope pv(ctx, AGX_PROF_VECTOR);
        agx_launch_pdl(from_f32_scaled, gv, AGX_BLOCK, 0, ctx->stream, n, ctx->f_z, ctx->d_z, sc);
      }
      ctx->n_launches += 2;
    };
    if (flexible) {
      if (int rc = update_chebyshev_bound(ctx)) return rc;
      if (int rc = ensure_bf16_copy(ctx)) return rc;
      precond();
      if (precond_failed) return agx_fail(ctx, AGX_ERR_ARG, "preconditioner callback failed");
    }
    agx_launch_pdl(fcg_direction_dots<double>, g, AGX_BLOCK, 0, ctx->stream, n, ctx->d_r, ctx->d_z, ctx->d_q, sc, ctx->d_partials);
    agx_launch_pdl(fcg_finish_direction, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, g);
    ctx->n_launches += 2;
    auto chunk = [&](int kn) {
      for (int k = 0; k < kn; ++k) {
        double* pnew = pbuf[cur ^ 1];
        const int ns =
            launch_spmv_dot<double>(ctx, ctx->d_vals64, ctx->d_z, pbuf[cur], pnew, ctx->d_q, (const double*)ctx->d_r);
        agx_launch_pdl(fcg_finish_pq, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, ns);
        {
          agx_prof_scope ps(ctx, AGX_PROF_VECTOR);
          agx_launch_pdl(fcg_update_kernel<double>, g, AGX_BLOCK, 0, ctx->stream, n, x, ctx->d_r, pnew, ctx->d_q, sc,
                                                                     ctx->d_partials);
          agx_launch_pdl(fcg_finish_update, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, g);
        }
        precond();
        {
          agx_prof_scope ps(ctx, AGX_PROF_VECTOR);
          agx_launch_pdl(fcg_direction_dots<double>, g, AGX_BLOCK, 0, ctx->stream, n, ctx->d_r, ctx->d_z, ctx->d_q, sc,
                                                                      ctx->d_partials);
          agx_launch_pdl(fcg_finish_direction, 1, AGX_BLOCK, 0, ctx->stream, sc, ctx->d_partials, g);
        }
        ctx->n_launches += 3;  // the three finishers
        cur ^= 1;
      }
    };
    while (true) {
      const int kn = std::min(every, maxiter - it_done);
      ctx->n_launches += 3 * kn;
      if (flexible && !ctx->precond_capturable) {
        chunk(kn);
        AGX_CHECK_LAUNCH(ctx);
      } else if (int rc = run_chunk(ctx, 2, x, every, kn, chunk, 3 * kn, flexible ? ctx->precond_gen : -1)) {
        return rc;
      }
      if (precond_failed) return agx_fail(ctx, AGX_ERR_ARG, "preconditioner callback failed");
      int rc = read_scalars(ctx);
      if (rc) return rc;
      it_done = ctx->h_scal->iters;
      if (ctx->h_scal->converged || it_done >= maxiter) break;
    }
  } else if (method == AGX_BICGSTAB) {
    bicg_init<<<gv, AGX_BLOCK, 0, ctx->stream>>>(n, rhs, x, ctx->d_r, ctx->d_rhat, ctx->d_p, ctx->d_v, sc);
    while (true) {
      const int kn = std::min(every, maxiter - it_done);
      ctx->n_launches += 5 * kn;
      for (int k = 0; k < kn; ++k) {
        agx_prof_scope pv(ctx, AGX_PROF_VECTOR);
        bicg_p_kernel<<<gv, AGX_BLOCK, 0, ctx->stream>>>(n, ctx->d_p, ctx->d_r, ctx->d_v, ctx->d_q, ctx->d_dinv64, sc);
        launch_bicg_spmv(ctx, 0, ctx->d_q, ctx->d_v, ctx->d_rhat);  // v = A y, y in d_q
        bicg_s_kernel<<<gv, AGX_BLOCK, 0, ctx->stream>>>(n, ctx->d_r, ctx->d_v, ctx->d_s, ctx->d_z, ctx->d_dinv64, sc);
        launch_bicg_spmv(ctx, 1, ctx->d_z, ctx->d_t, ctx->d_s);  // t = A z
        bicg_update<<<g, AGX_BLOCK, 0, ctx->stream>>>(n, x, ctx->d_r, ctx->d_q, ctx->d_z, ctx->d_s, ctx->d_t,
                                                     ctx->d_rhat, sc, ctx->d_partials, ctx->d_counter);
      }
      AGX_CHECK_LAUNCH(ctx);
      int rc = read_scalars(ctx);
      if (rc) return rc;
      it_done = ctx->h_scal->iters;
      if (ctx->h_scal->converged || it_done >= maxiter) break;
    }
  } else {
    return agx_fail(ctx, AGX_ERR_ARG, "unknown Krylov method %d", method);
  }
  AGX_CHECK_LAUNCH(ctx);
  int rc = read_scalars(ctx);
  if (rc) return rc;
  const agx_krylov_scalars& s = *ctx->h_scal;
  const double bb_scale = (method == AGX_PCG_MIXED || method == AGX_FCG_MIXED) ? 1.0 : s.extra[0] * s.extra[0];
  if (info) {
    info->iterations = s.iters;
    info->rel_residual = sqrt(s.rr * bb_scale);
    info->status = s.converged == 1 ? AGX_OK : (s.converged == 2 ? AGX_DIVERGED : AGX_NOT_CONVERGED);
  }
  return AGX_OK;
}
