// GPU throughput probe: FP64 / FP32 FMA rates, FP32/FP64 atomic scatter rates and copy bandwidth.
// Built and run by `python -m autopdex_gb300.diag`; every access is in bounds (indices taken mod the
// buffer sizes), no waits.
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("ERR %s line %d: %s\n",#x,__LINE__,cudaGetErrorString(e)); return 1;}}while(0)

template<typename T>
__global__ void fma_kernel(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template<typename T>
__global__ void atomic_kernel(T* dst, const int* idx, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(dst + idx[i], (T)1);
}
__global__ void copy_kernel(const float4* a, float4* b, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) b[i] = a[i];
}

int main() {
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  int dev = 0; cudaDeviceProp p; CK(cudaGetDeviceProperties(&p, dev));
  printf("dev %s SMs %d cc %d.%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
  double* dout; float* fout; CK(cudaMalloc(&dout, 1 << 26)); CK(cudaMalloc(&fout, 1 << 26));
  int blocks = p.multiProcessorCount * 8, threads = 256;
  // FP64
  for (int rep = 0; rep < 2; ++rep) {
    int iters = 4096;
    cudaEventRecord(e0);
    fma_kernel<double><<<blocks, threads>>>(dout, iters, 0.999999, 1e-7);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    double flops = 2.0 * 8 * iters * (double)blocks * threads;
    printf("fp64 fma: %.3f ms  %.2f TFLOP/s\n", ms, flops / ms / 1e9);
  }
  for (int rep = 0; rep < 2; ++rep) {
    int iters = 65536;
    cudaEventRecord(e0);
    fma_kernel<float><<<blocks, threads>>>(fout, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    double flops = 2.0 * 8 * iters * (double)blocks * threads;
    printf("fp32 fma: %.3f ms  %.2f TFLOP/s\n", ms, flops / ms / 1e9);
  }
  // atomics: n = 16M adds into m = 9M slots, index pattern: element-local scatter (i/16*9/16 + i%16 ...)
  int n = 16 << 20, m = 9 << 20;
  int* hidx = (int*)malloc(sizeof(int) * n);
  // mimic a 2D Q1 scatter: element e with 16 entries; entries clustered
  for (int i = 0; i < n; ++i) { long e = i / 16; int l = i % 16; hidx[i] = (int)(((e * 9) / 16 * 16 + l * 9 / 16 + (l % 4)) % m); }
  int* didx; CK(cudaMalloc(&didx, sizeof(int) * n)); CK(cudaMemcpy(didx, hidx, sizeof(int) * n, cudaMemcpyHostToDevice));
  float* fa; double* da; CK(cudaMalloc(&fa, sizeof(float) * m)); CK(cudaMalloc(&da, sizeof(double) * m));
  for (int rep = 0; rep < 3; ++rep) {
    cudaMemset(fa, 0, sizeof(float) * m);
    cudaEventRecord(e0);
    atomic_kernel<float><<<(n + 255) / 256, 256>>>(fa, didx, n);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    printf("atomic f32 clustered: %.3f ms  %.1f Gatom/s\n", ms, n / ms / 1e6);
    cudaMemset(da, 0, sizeof(double) * m);
    cudaEventRecord(e0);
    atomic_kernel<double><<<(n + 255) / 256, 256>>>(da, didx, n);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("atomic f64 clustered: %.3f ms  %.1f Gatom/s\n", ms, n / ms / 1e6);
  }
  // random pattern
  unsigned s = 12345;
  for (int i = 0; i < n; ++i) { s = s * 1664525u + 1013904223u; hidx[i] = (int)(s % (unsigned)m); }
  CK(cudaMemcpy(didx, hidx, sizeof(int) * n, cudaMemcpyHostToDevice));
  for (int rep = 0; rep < 2; ++rep) {
    cudaEventRecord(e0);
    atomic_kernel<float><<<(n + 255) / 256, 256>>>(fa, didx, n);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    printf("atomic f32 random: %.3f ms  %.1f Gatom/s\n", ms, n / ms / 1e6);
    cudaEventRecord(e0);
    atomic_kernel<double><<<(n + 255) / 256, 256>>>(da, didx, n);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("atomic f64 random: %.3f ms  %.1f Gatom/s\n", ms, n / ms / 1e6);
  }
  // copy 2 GB
  size_t nb = (size_t)1 << 31; float4 *ca, *cb; CK(cudaMalloc(&ca, nb)); CK(cudaMalloc(&cb, nb));
  cudaMemset(ca, 0, nb);
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    copy_kernel<<<p.multiProcessorCount * 16, 512>>>(ca, cb, nb / 16);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    printf("copy: %.3f ms %.1f GB/s\n", ms, 2.0 * nb / ms / 1e6);
  }
  CK(cudaGetLastError());
  printf("done\n");
  return 0;
}
