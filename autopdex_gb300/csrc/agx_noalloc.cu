// Allocation-free Jacobi-PCG: agx_pcg_noalloc.
//
// Some callers cannot allocate device memory while they solve: code running inside a
// memory pool with a fixed budget that must not grow, a host that forbids cudaMalloc after
// start-up (real-time or certified runs that allocate everything up front), or a caller
// that would otherwise need a context (agx_create/agx_finalize allocate the pattern and
// work vectors).  This entry point takes the matrix, the right-hand side and the solution
// buffer from the caller and keeps its own work vectors (r, z, p, q, the inverse diagonal,
// reduction partials and scalars) in one file-scope device array of fixed size, so it calls
// no cudaMalloc, cudaFree or allocating library routine.
//
// The array exists once per device that loads this library and stays reserved until the
// process exits.  Every call shares it and it keeps the last call's contents, so each call
// first clears what must start at zero (the reduction ticket and the solver scalars) and
// rebuilds every vector it reads.  Calls that overlap on the GPU -- two streams, or two host
// threads -- race on the array and corrupt each other's solves.
//
// Host code cannot hand the array's name to a kernel: on the host the name is a stand-in,
// not a device address.  The first call on a device, with that device current, looks the
// address up with cudaGetSymbolAddress and caches it; that first call should therefore come
// before any stream capture.  The address is the current device's, so the stream passed in
// must belong to the current device (checked; a stream of another device is rejected).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "agx_common.cuh"

namespace {

constexpr int64_t kMaxDofs = AGX_NOALLOC_MAX_DOFS;
constexpr int kMaxGrid = 1024;
constexpr int kNwarp = AGX_BLOCK / 32;

struct NaScalars {
  double rz, rr, pq, alpha, beta, rr_stop, bb;
  int converged, iters;
  unsigned counter;
  unsigned pad;
};

constexpr size_t kVecBytes = sizeof(double) * kMaxDofs;
constexpr size_t kPartialBytes = sizeof(double) * 2 * kMaxGrid;
constexpr size_t kScratchBytes = 5 * kVecBytes + kPartialBytes + 256;

}  // namespace

// Work space of agx_pcg_noalloc: r, z, p, q, inverse diagonal, partials, scalars.
static __device__ __align__(256) unsigned char agx_noalloc_scratch[kScratchBytes];

namespace {

struct NaWork {
  double *r, *z, *p, *q, *dinv, *partials;
  NaScalars* sc;
};

NaWork carve(unsigned char* base) {
  NaWork w;
  w.r = (double*)(base);
  w.z = (double*)(base + kVecBytes);
  w.p = (double*)(base + 2 * kVecBytes);
  w.q = (double*)(base + 3 * kVecBytes);
  w.dinv = (double*)(base + 4 * kVecBytes);
  w.partials = (double*)(base + 5 * kVecBytes);
  w.sc = (NaScalars*)(base + 5 * kVecBytes + kPartialBytes);
  return w;
}

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block partials in block order, combined by the last block to finish (no waiting)
template <int NV>
__device__ bool na_reduce(double (&v)[NV], double* partials, unsigned* counter, double (&tot)[NV]) {
  __shared__ double sh[NV][kNwarp];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double s = na_warp_sum(v[k]);
    if (lane == 0) sh[k][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0;
      for (int w = 0; w < kNwarp; ++w) s += sh[k][w];
      partials[k * gridDim.x + blockIdx.x] = s;
    }
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = 0;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) s += __ldcg(partials + k * gridDim.x + i);
    s = na_warp_sum(s);
    __syncthreads();
    if (lane == 0) sh[k][warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int w = 0; w < kNwarp; ++w) t += sh[k][w];
      tot[k] = t;
    }
  }
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

template <int NDOF, int TPR>
__device__ __forceinline__ void na_row(int64_t row, int sub, const int32_t* __restrict__ rowptr,
                                       const int32_t* __restrict__ col, const double* __restrict__ vals,
                                       const double* __restrict__ x, double (&y)[NDOF]) {
#pragma unroll
  for (int i = 0; i < NDOF; ++i) y[i] = 0;
  for (int k = rowptr[row] + sub; k < rowptr[row + 1]; k += TPR) {
    const int64_t c = col[k];
    const double* v = vals + (int64_t)k * NDOF * NDOF;
#pragma unroll
    for (int i = 0; i < NDOF; ++i)
#pragma unroll
      for (int j = 0; j < NDOF; ++j) y[i] += v[i * NDOF + j] * x[c * NDOF + j];
  }
#pragma unroll
  for (int o = TPR / 2; o >= 1; o >>= 1)
#pragma unroll
    for (int i = 0; i < NDOF; ++i) y[i] += __shfl_xor_sync(0xffffffffu, y[i], o);
}

// zero the ticket and the scalars; inverse diagonal from the matrix; x = 0, r = b, z = p = D^-1 r
template <int NDOF>
__global__ void __launch_bounds__(AGX_BLOCK)
na_init(int64_t n_nodes, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
        const double* __restrict__ vals, const double* __restrict__ b, double* __restrict__ x, NaWork w,
        double rtol) {
  const int64_t n = n_nodes * NDOF;
  double acc[2] = {0.0, 0.0};
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n; d += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = d / NDOF;
    const int c = (int)(d - p * NDOF);
    double diag = 0.0;
    for (int k = rowptr[p]; k < rowptr[p + 1]; ++k)
      if (col[k] == p) diag = vals[(int64_t)k * NDOF * NDOF + c * NDOF + c];
    const double di = diag != 0.0 ? 1.0 / diag : 0.0;
    w.dinv[d] = di;
    x[d] = 0.0;
    const double bi = b[d];
    w.r[d] = bi;
    w.z[d] = di * bi;
    w.p[d] = di * bi;
    acc[0] += bi * di * bi;
    acc[1] += bi * bi;
  }
  double tot[2];
  if (na_reduce<2>(acc, w.partials, &w.sc->counter, tot) && threadIdx.x == 0) {
    w.sc->rz = tot[0];
    w.sc->rr = tot[1];
    w.sc->rr_stop = rtol * rtol * tot[1];
    w.sc->bb = tot[1];
    w.sc->iters = 0;
    w.sc->converged = (tot[1] == 0.0 || tot[1] <= w.sc->rr_stop) ? 1 : (isfinite(tot[1]) ? 0 : 2);
  }
}

__global__ void na_clear(NaScalars* sc) {
  sc->counter = 0u;
  sc->converged = 0;
  sc->iters = 0;
  sc->rz = sc->rr = sc->pq = sc->alpha = sc->beta = sc->rr_stop = sc->bb = 0.0;
}

template <int NDOF, int TPR>
__global__ void __launch_bounds__(AGX_BLOCK)
na_spmv_dot(int64_t n_rows, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
            const double* __restrict__ vals, NaWork w) {
  if (w.sc->converged) return;
  const int sub = threadIdx.x % TPR;
  const int64_t total = ((n_rows * TPR + 31) / 32) * 32;
  double acc[1] = {0.0};
  for (int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; L < total; L += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = L / TPR;
    double y[NDOF];
    na_row<NDOF, TPR>(row < n_rows ? row : n_rows - 1, sub, rowptr, col, vals, w.p, y);
    if (row < n_rows && sub == 0) {
#pragma unroll
      for (int i = 0; i < NDOF; ++i) {
        w.q[row * NDOF + i] = y[i];
        acc[0] += y[i] * w.p[row * NDOF + i];
      }
    }
  }
  double tot[1];
  if (na_reduce<1>(acc, w.partials, &w.sc->counter, tot) && threadIdx.x == 0) {
    w.sc->pq = tot[0];
    if (!isfinite(tot[0]) || tot[0] == 0.0) w.sc->converged = 2;
    else w.sc->alpha = w.sc->rz / tot[0];
  }
}

__global__ void __launch_bounds__(AGX_BLOCK) na_update(int64_t n, double* __restrict__ x, NaWork w) {
  if (w.sc->converged) return;
  const double a = w.sc->alpha;
  double acc[2] = {0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += a * w.p[i];
    const double ri = w.r[i] - a * w.q[i];
    w.r[i] = ri;
    const double zi = w.dinv[i] * ri;
    w.z[i] = zi;
    acc[0] += ri * zi;
    acc[1] += ri * ri;
  }
  double tot[2];
  if (na_reduce<2>(acc, w.partials, &w.sc->counter, tot) && threadIdx.x == 0) {
    NaScalars* sc = w.sc;
    sc->iters += 1;
    sc->rr = tot[1];
    if (!isfinite(tot[0]) || !isfinite(tot[1])) sc->converged = 2;
    else if (tot[1] <= sc->rr_stop) sc->converged = 1;
    else if (sc->rz == 0.0) sc->converged = 2;
    else {
      sc->beta = tot[0] / sc->rz;
      sc->rz = tot[0];
    }
  }
}

__global__ void __launch_bounds__(AGX_BLOCK) na_direction(int64_t n, NaWork w) {
  if (w.sc->converged) return;
  const double bta = w.sc->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w.p[i] = w.z[i] + bta * w.p[i];
}

std::mutex g_mu;
void* g_scratch[256] = {nullptr};

int fail(char* errbuf, int len, int code, const char* msg) {
  if (errbuf && len > 0) snprintf(errbuf, (size_t)len, "%s", msg);
  return code;
}

template <int NDOF, int TPR>
int run(const int32_t* rowptr, const int32_t* col, const double* vals, int64_t n_nodes, const double* rhs,
        double* x, double rtol, int maxiter, cudaStream_t s, NaWork w, int grid, agx_solve_info* info, char* errbuf,
        int errlen) {
  const int64_t n = n_nodes * NDOF;
  na_clear<<<1, 1, 0, s>>>(w.sc);
  na_init<NDOF><<<grid, AGX_BLOCK, 0, s>>>(n_nodes, rowptr, col, vals, rhs, x, w, rtol);
  NaScalars h{};
  int done = 0;
  while (true) {
    const int kn = std::min(32, maxiter - done);
    for (int k = 0; k < kn; ++k) {
      na_spmv_dot<NDOF, TPR><<<grid, AGX_BLOCK, 0, s>>>(n_nodes, rowptr, col, vals, w);
      na_update<<<grid, AGX_BLOCK, 0, s>>>(n, x, w);
      na_direction<<<grid, AGX_BLOCK, 0, s>>>(n, w);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, w.sc, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(errbuf, errlen, AGX_ERR_CUDA, cudaGetErrorString(e));
    done = h.iters;
    if (h.converged || done >= maxiter || kn <= 0) break;
  }
  if (info) {
    info->iterations = h.iters;
    info->rel_residual = h.bb > 0.0 ? std::sqrt(h.rr / h.bb) : 0.0;
    info->status = h.converged == 1 ? AGX_OK : (h.converged == 2 ? AGX_DIVERGED : AGX_NOT_CONVERGED);
  }
  return h.converged == 1 ? AGX_OK : (h.converged == 2 ? AGX_DIVERGED : AGX_NOT_CONVERGED);
}

}  // namespace

extern "C" int agx_pcg_noalloc(const int32_t* rowptr, const int32_t* col, const double* vals, int64_t n_nodes,
                               int ndof, const double* rhs, double* x, double rtol, int maxiter, void* stream,
                               agx_solve_info* info, char* errbuf, int errbuf_len) {
  if (!rowptr || !col || !vals || !rhs || !x || n_nodes <= 0 || maxiter <= 0 || !(rtol >= 0.0))
    return fail(errbuf, errbuf_len, AGX_ERR_ARG, "agx_pcg_noalloc: null pointer or invalid size/tolerance");
  if (ndof < 1 || ndof > 3)
    return fail(errbuf, errbuf_len, AGX_ERR_ARG, "agx_pcg_noalloc: ndof must be 1, 2 or 3");
  if (n_nodes * ndof > kMaxDofs) {
    char msg[160];
    snprintf(msg, sizeof(msg), "agx_pcg_noalloc: %lld DOFs exceed the fixed work space of %lld DOFs",
             (long long)(n_nodes * ndof), (long long)kMaxDofs);
    return fail(errbuf, errbuf_len, AGX_ERR_ARG, msg);
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail(errbuf, errbuf_len, AGX_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= 256) return fail(errbuf, errbuf_len, AGX_ERR_ARG, "agx_pcg_noalloc: device index too large");
  // the work array is looked up for the current device, so the stream must belong to it
  int sdev = dev;
  e = cudaStreamGetDevice((cudaStream_t)stream, &sdev);
  if (e != cudaSuccess) return fail(errbuf, errbuf_len, AGX_ERR_CUDA, cudaGetErrorString(e));
  if (sdev != dev)
    return fail(errbuf, errbuf_len, AGX_ERR_ARG, "agx_pcg_noalloc: the stream belongs to another device than the current one");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch[dev]) {
      // once per device, with that device current: the array's device address
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, agx_noalloc_scratch);
      if (e != cudaSuccess) return fail(errbuf, errbuf_len, AGX_ERR_CUDA, cudaGetErrorString(e));
      g_scratch[dev] = p;
    }
    base = g_scratch[dev];
  }
  NaWork w = carve((unsigned char*)base);
  const int grid = std::min(kMaxGrid, std::max(1, sms * 2));
  cudaStream_t s = (cudaStream_t)stream;
  switch (ndof) {
    case 1:
      return run<1, 4>(rowptr, col, vals, n_nodes, rhs, x, rtol, maxiter, s, w, grid, info, errbuf, errbuf_len);
    case 2:
      return run<2, 4>(rowptr, col, vals, n_nodes, rhs, x, rtol, maxiter, s, w, grid, info, errbuf, errbuf_len);
    default:
      return run<3, 8>(rowptr, col, vals, n_nodes, rhs, x, rtol, maxiter, s, w, grid, info, errbuf, errbuf_len);
  }
}
