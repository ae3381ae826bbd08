// Shared pieces of the BF16 tensor-core kernels (agx_nn.cu: the 2-D U-Net, agx_nn3d.cu: the
// 3-D one): tcgen05 shared-memory and instruction descriptors, the MMA, bounded mbarrier waits,
// TMEM allocation and loads, bulk copies, and the host lookups of the SM count and of the
// tensor-map encoder.  Everything sits in an anonymous namespace, so each translation unit
// has its own copy.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <cstdint>

// the solve's converged flag while a learned preconditioner runs inside a captured solve
// (agx_nn_set_skip_flag; defined in agx_nn.cu)
extern const int* g_nn_skip;

namespace {

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

__device__ __forceinline__ bool nn_skip(const int* skip) { return skip && __ldcg(skip) != 0; }

constexpr int kTile = 128;        // output pixels per CTA (MMA M)
constexpr int kWaitLimit = 1 << 22;

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  // tcgen05 shared-memory matrix descriptor, no swizzle: start >> 4 (bits 0-13), leading
  // byte offset >> 4 (16-29: distance of core matrices along K), stride byte offset >> 4
  // (32-45: distance of 8-row groups along M/N), descriptor version 1 (bits 46-47)
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
  // kind::f16 instruction descriptor: f32 accumulator (bits 4-5 = 1), A and B bf16 (bits 7-9,
  // 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ int mbar_wait(uint32_t addr, uint32_t phase) {
  for (int it = 0; it < kWaitLimit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(ok)
        : "r"(addr), "r"(phase)
        : "memory");
    if (ok) return 1;
  }
  return 0;
}

// 32 lanes x 16 consecutive f32 columns of TMEM per call (thread = lane = row)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

template <int NCOLS>
__device__ __forceinline__ void tmem_alloc(uint32_t* slot) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(slot);
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s), "n"(NCOLS) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

template <int NCOLS>
__device__ __forceinline__ void tmem_free(uint32_t tmem) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(NCOLS) : "memory");
}

__host__ __device__ constexpr int tmem_cols(int n) { return n <= 32 ? 32 : (n <= 64 ? 64 : 128); }

// byte offset of element (row, k) in a K-major no-swizzle operand with `rgroups` 8-row groups
__device__ __forceinline__ uint32_t core_off(int row, int k, int rgroups) {
  return (uint32_t)((((k >> 3) * rgroups + (row >> 3)) * 8 + (row & 7)) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void mbar_expect(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// one thread: a contiguous global -> shared copy of `bytes` (both ends 16-byte aligned, bytes
// a multiple of 16), completing on `bar`
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

}  // namespace
