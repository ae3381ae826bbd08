// BF16 tensor-core kernels of the learned preconditioner (a small convolutional U-Net on
// the structured node grid, applied inside flexible CG).  Nothing in AutoPDEx corresponds to
// this part; it is the learned-preconditioner addition of this backend.
//
// Tensors are NHWC bf16 with 16, 32 or 64 channels.  A 3x3 convolution (stride 1, zero
// padding 1) is an implicit GEMM D[pixel, cout] = sum_k A[pixel, k] B[cout, k] with
// k = tap * CIN + cin: each persistent CTA holds the packed weight image and double-buffered
// input halos of 128-pixel row tiles in shared memory in the no-swizzle K-major core-matrix
// layout (8 rows x 16 bytes per core matrix), one thread issues tcgen05.mma (kind::f16, bf16 in,
// f32 accumulate, M = 128, N = COUT, K = 16 per instruction) into a TMEM accumulator, the
// MMA completion is committed to an mbarrier, and the four warps read their 32 TMEM lanes
// back with tcgen05.ld for the epilogue (bias, ReLU, bf16 store).  The input gradient is the
// same kernel with the weights flipped and transposed at packing time.  The weight gradient
// is a second tcgen05 GEMM with the reduction running over pixels.
//
// Every wait is bounded: a CTA whose MMA does not complete in time records an error flag
// and still releases its TMEM.
#include <algorithm>
#include <cooperative_groups.h>
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "agx_common.cuh"
#include "agx_tc.cuh"
#include "../../include/autopdex_gb300_nn.h"

// agx_nn_set_skip_flag: a device int that the inference kernels read after their
// programmatic-launch wait; nonzero makes them return at once (passed to every launch, so a
// captured graph keeps it)
const int* g_nn_skip = nullptr;

namespace {

namespace cg = cooperative_groups;

struct ConvArgs {
  const __nv_bfloat16* in1;  // NHWC, C1 channels
  const __nv_bfloat16* in2;  // NHWC, C2 channels (concatenated after in1), or null when C2 == 0
  const __nv_bfloat16* wpk;  // packed B image (COUT rows x 9 CIN), core-matrix order
  const float* bias;         // COUT values or null
  __nv_bfloat16* out1;       // channels [0, S) (NHWC with S channels)
  __nv_bfloat16* out2;       // channels [S, COUT) or null when S == COUT
  int split;                 // S
  int B, H, W;
  int* err;
  int const_weights;         // weights and bias not written by the kernel just before this one
  const int* skip;           // nonzero there: return at once (the solve using the network has converged)
};

// out = epi(conv3x3(concat(in1, in2)) + bias); EPI 0: identity, 1: ReLU.
//
// Persistent over row tiles of 128 output pixels (b, y, x0 .. x0 + 127).  A tile's input is a
// halo of 3 rows x 130 pixels, stored as CIN / 8 channel planes of 16-byte pixel chunks
// (plane c holds channels 8c .. 8c + 7 of every halo pixel, 16 bytes apart): each plane is one
// TMA box {8 channels, 130 pixels, 3 rows} of the NHWC tensor, with the zero fill of the
// tensor copy supplying the padding.  In that layout the A operand of tap (dy, dx) -- 128
// pixels x 16 channels -- is a no-swizzle K-major view starting at halo pixel
// ((dy + 1) * 130 + dx + 1) of plane 2 kc: 8-pixel core matrices 128 bytes apart (SBO) and
// channel chunks one plane apart (LBO), so the nine taps are nine descriptors over one copy of
// the input instead of a nine-fold gather.  The packed weights arrive in one bulk copy issued
// with the first halos and stay in shared memory for the CTA's lifetime; the bias sits in
// shared memory too.  Halos cycle through kStages buffers filled kStages - 1 tiles ahead (one
// mbarrier each, completed by the copies' transaction bytes), and the accumulator alternates
// between two TMEM column ranges, so the MMAs of tile k run while the four warps drain tile
// k - 1 through tcgen05.ld, and the copies of tiles k + 1 .. k + kStages - 1 are in flight.
constexpr int kHaloW = kTile + 2;                 // halo pixels per row
constexpr int kHaloPx = 3 * kHaloW;               // halo pixels per tile
constexpr int kPlaneData = kHaloPx * 16;          // bytes one TMA box writes
constexpr int kPlaneBytes = (kPlaneData + 127) / 128 * 128;  // plane stride (128-byte aligned)
constexpr int kStages = 3;                        // halo buffers in the ring

struct ConvMaps {
  CUtensorMap in1;  // {C1, W, H, B} bf16, box {8, 130, 3, 1}
  CUtensorMap in2;  // {C2, W, H, B}, unused when C2 == 0
};

__device__ __forceinline__ void tma_load4(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                          uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}

// one thread: the CIN / 8 plane copies of a tile's halo, completing on `bar`
template <int C1, int C2>
__device__ __forceinline__ void issue_halo(const ConvMaps& m, const ConvArgs& a, int64_t tile, int tiles_x,
                                           uint32_t halo, uint32_t bar) {
  constexpr int NCH = (C1 + C2) / 8;
  const int64_t row = tile / tiles_x;  // b * H + y
  const int x0 = (int)(tile - row * tiles_x) * kTile;
  const int b = (int)(row / a.H), y = (int)(row - (int64_t)b * a.H);
  mbar_expect(bar, (uint32_t)(NCH * kPlaneData));
#pragma unroll
  for (int c = 0; c < C1 / 8; ++c) tma_load4(halo + (uint32_t)(c * kPlaneBytes), &m.in1, 8 * c, x0 - 1, y - 1, b, bar);
  if constexpr (C2 > 0) {
#pragma unroll
    for (int c = 0; c < C2 / 8; ++c)
      tma_load4(halo + (uint32_t)((C1 / 8 + c) * kPlaneBytes), &m.in2, 8 * c, x0 - 1, y - 1, b, bar);
  }
}

template <int COUT, int EPI>
__device__ __forceinline__ void conv_epilogue(const ConvArgs& a, const float* sbias, uint32_t tacc, int64_t tile,
                                              int tiles_x, int tid, int warp) {
  float acc[COUT];
#pragma unroll
  for (int c = 0; c < COUT; c += 16) tmem_ld16(tacc + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, acc + c);
  const int64_t row = tile / tiles_x;
  const int x = (int)(tile - row * tiles_x) * kTile + tid;
  if (x >= a.W) return;
  const int64_t p = row * a.W + x;
#pragma unroll
  for (int c = 0; c < COUT; ++c) {
    float v = acc[c] + sbias[c];
    if (EPI == 1) v = fmaxf(v, 0.0f);
    acc[c] = v;
  }
  const int S = a.split;
#pragma unroll
  for (int c0 = 0; c0 < COUT; c0 += 8) {
    __align__(16) __nv_bfloat16 h[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) h[u] = __float2bfloat16(acc[c0 + u]);
    if (c0 < S)
      *reinterpret_cast<uint4*>(a.out1 + p * S + c0) = *reinterpret_cast<uint4*>(h);
    else
      *reinterpret_cast<uint4*>(a.out2 + p * (COUT - S) + (c0 - S)) = *reinterpret_cast<uint4*>(h);
  }
}

// Halo loaders.  kLoadTma (the default): one tensor copy per 8-channel plane by thread 0,
// completing on the buffer's mbarrier.  kLoadAsync: the CTA's 128 threads copy the halo's 16-byte
// pixel chunks with cp.async (consecutive lanes take consecutive chunks of the NHWC rows, so a
// warp reads whole 64-byte pixels, 512 contiguous bytes; padding and pixels past the image edge
// are zero-filled), one commit group per tile, made visible to the tensor cores by a proxy fence
// and the iteration's barrier.  Measured on the U-Net's 320^2 levels the tensor copies are
// 15-30 % faster; both fill shared memory identically.
constexpr int kLoadAsync = 0, kLoadTma = 1, kLoadTmaWs = 2;

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// all threads: the halo of `tile` into the plane layout at `halo` (one commit group follows)
template <int C1, int C2>
__device__ __forceinline__ void copy_halo_async(const ConvArgs& a, int64_t tile, int tiles_x, uint32_t halo, int tid) {
  constexpr int NCH = (C1 + C2) / 8, NCH1 = C1 / 8;
  const int64_t row = tile / tiles_x;  // b * H + y
  const int x0 = (int)(tile - row * tiles_x) * kTile;
  const int b = (int)(row / a.H), y = (int)(row - (int64_t)b * a.H);
  for (int u = tid; u < NCH * kHaloPx; u += kTile) {
    const int c = u % NCH, hp = u / NCH;
    const int r = hp / kHaloW, px = hp - r * kHaloW;
    const int yy = y - 1 + r, xx = x0 - 1 + px;
    const bool in = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
    const int64_t pix = in ? ((int64_t)b * a.H + yy) * a.W + xx : 0;
    const __nv_bfloat16* src = c < NCH1 ? a.in1 + pix * C1 + 8 * c : a.in2 + pix * C2 + 8 * (c - NCH1);
    cp_async16(halo + (uint32_t)(c * kPlaneBytes + hp * 16), src, in ? 16u : 0u);
  }
}

template <int C1, int C2, int COUT, int EPI, int LD>
__global__ void __launch_bounds__(kTile) conv3x3_tc(const __grid_constant__ ConvMaps maps, ConvArgs a) {
  constexpr int CIN = C1 + C2, K = 9 * CIN, NG = COUT / 8, NCH = CIN / 8;
  constexpr int B_BYTES = K * COUT * 2;
  constexpr int HALO_BYTES = NCH * kPlaneBytes;
  constexpr int NCOLS = tmem_cols(2 * COUT);  // two accumulators
  static_assert(CIN % 16 == 0 && COUT % 16 == 0, "channel counts must be multiples of 16");
  static_assert(B_BYTES % 1024 == 0 && HALO_BYTES % 128 == 0, "shared-memory carve-up");
  static_assert(kStages >= 2, "the cp.async ring waits for all but kStages - 2 groups");
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sB = smem;
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t full_bar[kStages];
  __shared__ __align__(8) uint64_t mma_bar[2];
  __shared__ __align__(8) uint64_t w_bar;
  __shared__ float sbias[COUT];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int tiles_x = (a.W + kTile - 1) / kTile;
  const int64_t ntiles = (int64_t)a.B * a.H * tiles_x;
  const int64_t first = blockIdx.x, stride = gridDim.x;
  const int64_t my_tiles = first < ntiles ? (ntiles - first + stride - 1) / stride : 0;
  const uint32_t b0 = (uint32_t)__cvta_generic_to_shared(sB);
  const uint32_t halo_base = b0 + B_BYTES;
  const uint32_t fbar0 = (uint32_t)__cvta_generic_to_shared(&full_bar[0]);
  const uint32_t mbar0 = (uint32_t)__cvta_generic_to_shared(&mma_bar[0]);
  const uint32_t wbar = (uint32_t)__cvta_generic_to_shared(&w_bar);
  if (tid == 0) {
    if constexpr (LD == kLoadTma) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&maps.in1)) : "memory");
      if constexpr (C2 > 0)
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&maps.in2)) : "memory");
#pragma unroll
      for (int s = 0; s < kStages; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fbar0 + 8u * s));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0 + 8u));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(wbar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // constant weights: their bulk copy overlaps the tail of the kernel before this one
    if (a.const_weights && my_tiles > 0) {
      mbar_expect(wbar, (uint32_t)B_BYTES);
      bulk_load(b0, a.wpk, (uint32_t)B_BYTES, wbar);
    }
  }
  if (a.const_weights && tid < COUT) sbias[tid] = a.bias ? a.bias[tid] : 0.0f;
  if (warp == 0) tmem_alloc<NCOLS>(&tmem_slot);
  // the previous kernel's outputs are visible from here on (programmatic dependent launch)
  agx_pdl_entry();
  if (nn_skip(a.skip)) {  // release what the prologue took: the weight copy in flight, TMEM
    if (tid == 0 && a.const_weights && my_tiles > 0) mbar_wait(wbar, 0u);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) tmem_free<NCOLS>(tmem_slot);
    return;
  }
  if (tid == 0) {
    // the packed weights (already in core-matrix order) in one bulk copy, in flight together
    // with the first kStages halos
    if (!a.const_weights && my_tiles > 0) {
      mbar_expect(wbar, (uint32_t)B_BYTES);
      bulk_load(b0, a.wpk, (uint32_t)B_BYTES, wbar);
    }
    if constexpr (LD == kLoadTma)
      for (int j = 0; j < kStages && j < my_tiles; ++j)
        issue_halo<C1, C2>(maps, a, first + j * stride, tiles_x, halo_base + (uint32_t)(j * HALO_BYTES),
                           fbar0 + 8u * j);
  }
  if constexpr (LD == kLoadAsync) {
    // the first kStages halos, one commit group per buffer (empty groups past the last tile)
    for (int j = 0; j < kStages; ++j) {
      if (j < my_tiles)
        copy_halo_async<C1, C2>(a, first + j * stride, tiles_x, halo_base + (uint32_t)(j * HALO_BYTES), tid);
      cp_async_commit();
    }
  }
  if (!a.const_weights && tid < COUT) sbias[tid] = a.bias ? a.bias[tid] : 0.0f;
  if constexpr (LD == kLoadAsync) {
    // tile 0 complete and visible to the tensor cores (generic-proxy writes, then the
    // proxy fence, then the barrier before the MMAs are issued)
    cp_async_wait<kStages - 1>();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t id = idesc_bf16(kTile, COUT);
  int ok = 1;
  int64_t issued = kStages < my_tiles ? kStages : my_tiles;  // TMA halos issued so far (thread 0's count)
  int64_t consumed = 0;                                       // TMA halos waited for by thread 0
  bool weights = my_tiles == 0;                               // weight copy waited for (thread 0)
  for (int64_t k = 0; k <= my_tiles && ok; ++k) {
    // (1) MMAs of tile k into accumulator k % 2 (its previous use, tile k - 2, was drained
    //     before the barrier that closed the last iteration)
    if (k < my_tiles && tid == 0) {
      const int st = (int)(k % kStages);
      if (!weights && mbar_wait(wbar, 0u)) weights = true;
      bool have = weights;
      if constexpr (LD == kLoadTma) have = have && mbar_wait(fbar0 + 8u * st, (uint32_t)((k / kStages) & 1));
      if (!have) {
        atomicExch(a.err, 1);
        ok = 0;
      } else {
        consumed = k + 1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t halo = halo_base + (uint32_t)(st * HALO_BYTES);
        const uint32_t tacc = tmem + (uint32_t)((k & 1) * COUT);
        // descriptors of tap 0 / k-step 0; every other step adds a compile-time offset (>> 4)
        const uint64_t da0 = smem_desc(halo, kPlaneBytes, 128);
        const uint64_t db0 = smem_desc(b0, NG * 128, 128);
#pragma unroll
        for (int t = 0; t < 9; ++t) {
#pragma unroll
          for (int kc = 0; kc < CIN / 16; ++kc) {
            const int s = t * (CIN / 16) + kc;
            const uint32_t aoff = (uint32_t)(2 * kc * kPlaneBytes + ((t / 3) * kHaloW + t % 3) * 16) >> 4;
            const uint32_t boff = (uint32_t)(2 * s * NG * 128) >> 4;
            mma_bf16(tacc, da0 + aoff, db0 + boff, id, s > 0 ? 1u : 0u);
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         mbar0 + 8u * (uint32_t)(k & 1))
                     : "memory");
      }
    }
    // (2) drain tile k - 1: its MMAs done also frees its halo buffer, refilled with tile
    //     k - 1 + kStages (the prologue filled every buffer)
    if (k >= 1) {
      const int64_t j = k - 1;
      const int done = mbar_wait(mbar0 + 8u * (uint32_t)(j & 1), (uint32_t)((j >> 1) & 1));
      if (!done) {
        if (tid == 0) atomicExch(a.err, 1);
        ok = 0;
      } else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if constexpr (LD == kLoadTma) {
          if (tid == 0 && issued < my_tiles) {
            const int st = (int)(issued % kStages);
            issue_halo<C1, C2>(maps, a, first + issued * stride, tiles_x, halo_base + (uint32_t)(st * HALO_BYTES),
                               fbar0 + 8u * st);
            ++issued;
          }
        } else {
          const int64_t nt = j + kStages;
          if (nt < my_tiles)
            copy_halo_async<C1, C2>(a, first + nt * stride, tiles_x,
                                    halo_base + (uint32_t)((nt % kStages) * HALO_BYTES), tid);
          cp_async_commit();
        }
        conv_epilogue<COUT, EPI>(a, sbias, tmem + (uint32_t)((j & 1) * COUT), first + j * stride, tiles_x, tid,
                                 warp);
      }
    }
    if constexpr (LD == kLoadAsync) {
      // tile k + 1 complete (all groups but the kStages - 2 newest) and visible to the MMAs
      cp_async_wait<kStages - 2>();
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  // copies issued but never waited for (only after an error): wait for them (bounded for the
  // tensor copies; each is the latest use of its buffer, so its phase parity identifies it)
  if constexpr (LD == kLoadAsync) asm volatile("cp.async.wait_all;" ::: "memory");
  if (tid == 0) {
    if constexpr (LD == kLoadTma)
      for (int64_t j = consumed; j < issued; ++j)
        mbar_wait(fbar0 + 8u * (uint32_t)(j % kStages), (uint32_t)((j / kStages) & 1));
    if (!weights) mbar_wait(wbar, 0u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) tmem_free<NCOLS>(tmem);
}

// Warp-specialised variant (kLoadTmaWs): six warps and mbarrier rings instead of one loop with
// a CTA barrier per tile.  Warp 5 (one lane) streams the halos with tensor copies into kStages
// buffers (full[s] completes with the bytes; empty[s] is released by the MMAs that read the
// buffer), warp 4 (one lane) issues each tile's MMAs into one of two TMEM accumulators
// (acc_full[a] is committed when they are done; acc_empty[a] is released by the epilogue), and
// warps 0-3 drain the accumulators (warp w reads TMEM lanes 32 w .. 32 w + 31).  So the copies of
// later tiles, the MMAs of tile k and the epilogue of tile k - 1 all proceed at once.  Every wait
// is bounded; a role that gives up sets `abort`, the others leave their loops at their next wait,
// and before the CTA exits the copies and MMAs still in flight are waited for (bounded) and TMEM
// is released.
constexpr int kWsThreads = 192;

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// bounded wait that also gives up once another role has aborted
__device__ __forceinline__ int mbar_wait_or_abort(uint32_t addr, uint32_t phase, volatile int* abort) {
  for (int it = 0; it < kWaitLimit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(ok)
        : "r"(addr), "r"(phase)
        : "memory");
    if (ok) return 1;
    if ((it & 63) == 63 && *abort) return 0;
  }
  return 0;
}

template <int C1, int C2, int COUT, int EPI>
__global__ void __launch_bounds__(kWsThreads) conv3x3_ws(const __grid_constant__ ConvMaps maps, ConvArgs a) {
  constexpr int CIN = C1 + C2, K = 9 * CIN, NG = COUT / 8, NCH = CIN / 8;
  constexpr int B_BYTES = K * COUT * 2;
  constexpr int HALO_BYTES = NCH * kPlaneBytes;
  constexpr int NCOLS = tmem_cols(2 * COUT);
  static_assert(CIN % 16 == 0 && COUT % 16 == 0, "channel counts must be multiples of 16");
  static_assert(B_BYTES % 1024 == 0 && HALO_BYTES % 128 == 0, "shared-memory carve-up");
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], accf_bar[2], acce_bar[2], w_bar;
  __shared__ float sbias[COUT];
  __shared__ int abort_flag;
  __shared__ int64_t copies_issued, tiles_consumed, mmas_issued, tiles_drained;
  volatile int* abort = &abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_x = (a.W + kTile - 1) / kTile;
  const int64_t ntiles = (int64_t)a.B * a.H * tiles_x;
  const int64_t first = blockIdx.x, stride = gridDim.x;
  const int64_t my_tiles = first < ntiles ? (ntiles - first + stride - 1) / stride : 0;
  const uint32_t b0 = (uint32_t)__cvta_generic_to_shared(smem);
  const uint32_t halo_base = b0 + B_BYTES;
  const uint32_t fb = (uint32_t)__cvta_generic_to_shared(&full_bar[0]);
  const uint32_t eb = (uint32_t)__cvta_generic_to_shared(&empty_bar[0]);
  const uint32_t afb = (uint32_t)__cvta_generic_to_shared(&accf_bar[0]);
  const uint32_t aeb = (uint32_t)__cvta_generic_to_shared(&acce_bar[0]);
  const uint32_t wbar = (uint32_t)__cvta_generic_to_shared(&w_bar);
  if (tid == 0) {
    for (int st = 0; st < kStages; ++st) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fb + 8u * st));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(eb + 8u * st));
    }
    for (int q = 0; q < 2; ++q) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(afb + 8u * q));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(aeb + 8u * q));  // one arrival per epilogue warp
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(wbar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
    copies_issued = tiles_consumed = mmas_issued = tiles_drained = 0;
    // constant weights: their bulk copy overlaps the tail of the kernel before this one
    if (a.const_weights && my_tiles > 0) {
      mbar_expect(wbar, (uint32_t)B_BYTES);
      bulk_load(b0, a.wpk, (uint32_t)B_BYTES, wbar);
    }
  }
  if (a.const_weights && tid < COUT) sbias[tid] = a.bias ? a.bias[tid] : 0.0f;
  if (warp == 0) tmem_alloc<NCOLS>(&tmem_slot);
  // the previous kernel's outputs are visible from here on (programmatic dependent launch)
  agx_pdl_entry();
  if (nn_skip(a.skip)) {  // release what the prologue took: the weight copy in flight, TMEM
    if (tid == 0 && a.const_weights && my_tiles > 0) mbar_wait(wbar, 0u);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) tmem_free<NCOLS>(tmem_slot);
    return;
  }
  if (!a.const_weights && tid < COUT) sbias[tid] = a.bias ? a.bias[tid] : 0.0f;
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  if (warp == 5 && lane == 0) {
    // ---- producer: the weights once, then the halos through the ring
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&maps.in1)) : "memory");
    if constexpr (C2 > 0) asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&maps.in2)) : "memory");
    if (!a.const_weights && my_tiles > 0) {
      mbar_expect(wbar, (uint32_t)B_BYTES);
      bulk_load(b0, a.wpk, (uint32_t)B_BYTES, wbar);
    }
    int64_t j = 0;
    for (; j < my_tiles; ++j) {
      const int st = (int)(j % kStages);
      if (j >= kStages && !mbar_wait_or_abort(eb + 8u * st, (uint32_t)((j / kStages - 1) & 1), abort)) break;
      issue_halo<C1, C2>(maps, a, first + j * stride, tiles_x, halo_base + (uint32_t)(st * HALO_BYTES), fb + 8u * st);
    }
    copies_issued = j;
    if (j < my_tiles) {
      *abort = 1;
      atomicExch(a.err, 1);
    }
  } else if (warp == 4 && lane == 0) {
    // ---- MMA issuer
    const uint32_t id = idesc_bf16(kTile, COUT);
    int64_t k = 0;
    if (my_tiles > 0 && mbar_wait_or_abort(wbar, 0u, abort)) {
      for (; k < my_tiles; ++k) {
        const int st = (int)(k % kStages);
        const uint32_t acc = (uint32_t)(k & 1);
        if (!mbar_wait_or_abort(fb + 8u * st, (uint32_t)((k / kStages) & 1), abort)) break;
        tiles_consumed = k + 1;
        if (k >= 2 && !mbar_wait_or_abort(aeb + 8u * acc, (uint32_t)((k / 2 - 1) & 1), abort)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t halo = halo_base + (uint32_t)(st * HALO_BYTES);
        const uint32_t tacc = tmem + acc * (uint32_t)COUT;
        const uint64_t da0 = smem_desc(halo, kPlaneBytes, 128);
        const uint64_t db0 = smem_desc(b0, NG * 128, 128);
#pragma unroll
        for (int t = 0; t < 9; ++t) {
#pragma unroll
          for (int kc = 0; kc < CIN / 16; ++kc) {
            const int s = t * (CIN / 16) + kc;
            const uint32_t aoff = (uint32_t)(2 * kc * kPlaneBytes + ((t / 3) * kHaloW + t % 3) * 16) >> 4;
            const uint32_t boff = (uint32_t)(2 * s * NG * 128) >> 4;
            mma_bf16(tacc, da0 + aoff, db0 + boff, id, s > 0 ? 1u : 0u);
          }
        }
        // the accumulator for the epilogue, the halo buffer back to the producer
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(afb + 8u * acc)
                     : "memory");
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(eb + 8u * st)
                     : "memory");
        mmas_issued = k + 1;
      }
    }
    if (k < my_tiles) {
      *abort = 1;
      atomicExch(a.err, 1);
    }
  } else if (warp < 4) {
    // ---- epilogue: accumulators to bf16 outputs
    int64_t k = 0;
    for (; k < my_tiles; ++k) {
      const uint32_t acc = (uint32_t)(k & 1);
      if (!mbar_wait_or_abort(afb + 8u * acc, (uint32_t)((k / 2) & 1), abort)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      float v[COUT];
#pragma unroll
      for (int c = 0; c < COUT; c += 16) tmem_ld16(tmem + acc * (uint32_t)COUT + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v + c);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(aeb + 8u * acc);
      const int64_t tile = first + k * stride;
      const int64_t row = tile / tiles_x;
      const int x = (int)(tile - row * tiles_x) * kTile + tid;
      if (x < a.W) {
        const int64_t p = row * a.W + x;
        const int S = a.split;
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 8) {
          __align__(16) __nv_bfloat16 h[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            float t = v[c0 + u] + sbias[c0 + u];
            if (EPI == 1) t = fmaxf(t, 0.0f);
            h[u] = __float2bfloat16(t);
          }
          if (c0 < S)
            *reinterpret_cast<uint4*>(a.out1 + p * S + c0) = *reinterpret_cast<uint4*>(h);
          else
            *reinterpret_cast<uint4*>(a.out2 + p * (COUT - S) + (c0 - S)) = *reinterpret_cast<uint4*>(h);
        }
      }
    }
    if (k < my_tiles) {
      *abort = 1;
      if (lane == 0) atomicExch(a.err, 1);
    }
    if (tid == 0) tiles_drained = k;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // after an abort: copies issued but not consumed (at most one per buffer, each the latest
  // phase of its barrier), and the last MMAs if their accumulator was not drained, are waited
  // for (bounded) before shared memory and TMEM are released; the weight copy likewise
  if (tid == 0 && abort_flag) {
    for (int64_t j = tiles_consumed; j < copies_issued; ++j)
      mbar_wait(fb + 8u * (uint32_t)(j % kStages), (uint32_t)((j / kStages) & 1));
    if (tiles_drained < mmas_issued) {
      const int64_t k = mmas_issued - 1;
      mbar_wait(afb + 8u * (uint32_t)(k & 1), (uint32_t)((k / 2) & 1));
    }
  }
  if (tid == 5 * 32 && my_tiles > 0) mbar_wait(wbar, 0u);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) tmem_free<NCOLS>(tmem);
}

struct WgradArgs {
  const __nv_bfloat16* in1;  // forward inputs, NHWC (NDHWC for 27 taps), C1 (+ C2) channels
  const __nv_bfloat16* in2;
  const __nv_bfloat16* dout; // gradient of the pre-activation output, NHWC, COUT channels
  float* dw;                 // (TAPS CIN) x COUT, f32, accumulated with atomics
  int B, D, H, W;            // D = 1 for the 2-D convolution
  int64_t pix_per_cta;       // pixels reduced by one CTA (multiple of 16)
  int* err;
};

// dW[k, co] += sum_p A[k, p] dOut[p, co], A[t CIN + ci, p] = in[p + tap_t, ci]; one CTA per
// (128-row slice of k, pixel chunk); the pixel chunk is consumed in sub-chunks of PCH pixels.
// TAPS = 9: 3x3 taps t = 3 dy + dx of a 2-D image; TAPS = 27: 3x3x3 taps t = 9 dz + 3 dy + dx
// of a 3-D one (offsets dz - 1, dy - 1, dx - 1).
template <int C1, int C2, int COUT, int PCH, int TAPS>
__global__ void __launch_bounds__(kTile) wgrad_tc(WgradArgs a) {
  constexpr int CIN = C1 + C2, KW = TAPS * CIN;
  constexpr int A_BYTES = kTile * PCH * 2;   // 128 rows x PCH pixels
  constexpr int NCOLS = tmem_cols(COUT);
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sA = smem;
  unsigned char* sB = smem + A_BYTES;        // COUT rows x PCH pixels
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t mbar;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row0 = blockIdx.y * kTile;       // first k row of this CTA
  const int64_t HW = (int64_t)a.H * a.W, P = HW * a.D * a.B;
  const int64_t pbeg = (int64_t)blockIdx.x * a.pix_per_cta;
  const int64_t pend = pbeg + a.pix_per_cta < P ? pbeg + a.pix_per_cta : P;
  const uint32_t mbar_addr = (uint32_t)__cvta_generic_to_shared(&mbar);
  if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_addr) : "memory");
  if (warp == 0) tmem_alloc<NCOLS>(&tmem_slot);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t a0 = (uint32_t)__cvta_generic_to_shared(sA), b0 = (uint32_t)__cvta_generic_to_shared(sB);
  uint32_t phase = 0;
  int ok_all = 1;
  int first = 1;
  for (int64_t c0 = pbeg; c0 < pend; c0 += PCH) {
    // A tile: thread handles (8 consecutive k rows = 8 channels of one tap, 8 pixels) blocks
    for (int blk = tid; blk < (kTile / 8) * (PCH / 8); blk += kTile) {
      const int rg = blk / (PCH / 8), pg = blk % (PCH / 8);
      const int krow = row0 + rg * 8;  // first of 8 k rows (same tap: CIN % 8 == 0)
      __align__(16) __nv_bfloat16 tile[8][8];  // [pixel][channel]
      const int t = krow / CIN, ci = krow % CIN;
      const bool rowok = krow < KW;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int64_t pp = c0 + pg * 8 + u;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (rowok && pp < pend) {
          const int64_t bz = pp / HW;  // b D + z
          const int64_t rem = pp - bz * HW;
          const int y = (int)(rem / a.W), x = (int)(rem - (int64_t)y * a.W);
          const int dz = TAPS == 27 ? t / 9 - 1 : 0;
          const int z = (int)(bz % a.D), zz = z + dz;
          const int yy = y + (t / 3) % 3 - 1, xx = x + t % 3 - 1;
          if (zz >= 0 && zz < a.D && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W) {
            const int64_t q = ((bz + dz) * a.H + yy) * a.W + xx;
            if (ci < C1)
              v = *reinterpret_cast<const uint4*>(a.in1 + q * C1 + ci);
            else
              v = *reinterpret_cast<const uint4*>(a.in2 + q * C2 + (ci - C1));
          }
        }
        *reinterpret_cast<uint4*>(tile[u]) = v;
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        __align__(16) __nv_bfloat16 col[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) col[u] = tile[u][r];
        *reinterpret_cast<uint4*>(sA + core_off(rg * 8 + r, pg * 8, kTile / 8)) = *reinterpret_cast<uint4*>(col);
      }
    }
    // B tile: dOut^T, rows co, k = pixel
    for (int blk = tid; blk < (COUT / 8) * (PCH / 8); blk += kTile) {
      const int ng = blk / (PCH / 8), pg = blk % (PCH / 8);
      __align__(16) __nv_bfloat16 tile[8][8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int64_t pp = c0 + pg * 8 + u;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (pp < pend) v = *reinterpret_cast<const uint4*>(a.dout + pp * COUT + ng * 8);
        *reinterpret_cast<uint4*>(tile[u]) = v;
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        __align__(16) __nv_bfloat16 col[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) col[u] = tile[u][r];
        *reinterpret_cast<uint4*>(sB + core_off(ng * 8 + r, pg * 8, COUT / 8)) = *reinterpret_cast<uint4*>(col);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t id = idesc_bf16(kTile, COUT);
#pragma unroll 1
      for (int s = 0; s < PCH / 16; ++s) {
        const uint64_t da = smem_desc(a0 + (uint32_t)(2 * s * (kTile / 8)) * 128u, (kTile / 8) * 128, 128);
        const uint64_t db = smem_desc(b0 + (uint32_t)(2 * s * (COUT / 8)) * 128u, (COUT / 8) * 128, 128);
        mma_bf16(tmem, da, db, id, first ? 0u : 1u);
        first = 0;
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_addr)
                   : "memory");
    }
    first = 0;
    // the shared tiles are reused by the next sub-chunk only after the MMAs have read them
    const int done = mbar_wait(mbar_addr, phase);
    phase ^= 1u;
    if (!done) {
      ok_all = 0;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
  }
  if (!ok_all && tid == 0) atomicExch(a.err, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok_all && pbeg < pend) {
    float acc[COUT];
#pragma unroll
    for (int c = 0; c < COUT; c += 16) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, acc + c);
    const int k = row0 + tid;
    if (k < KW) {
#pragma unroll
      for (int c = 0; c < COUT; ++c) atomicAdd(a.dw + (int64_t)k * COUT + c, acc[c]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) tmem_free<NCOLS>(tmem);
}

// ---- small kernels ----------------------------------------------------------------------
// Packs f32 weights W[co][ci][taps] (taps = 9: [3][3]; 27: [3][3][3]) into the B image of the
// forward conv (rows co, k = tap CIN + ci) or of the input-gradient conv (rows ci,
// k = tap' COUT + co with the taps flipped, tap' = taps - 1 - tap: the offsets are symmetric).
__global__ void pack_weights_kernel(const float* __restrict__ w, int cout, int cin, int taps, int mode,
                                    __nv_bfloat16* __restrict__ img) {
  const int total = cout * cin * taps;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int co = i / (cin * taps), rem = i % (cin * taps), ci = rem / taps, t = rem % taps;
    int row, k, rows;
    if (mode == 0) {
      row = co;
      k = t * cin + ci;
      rows = cout;
    } else {
      row = ci;
      k = (taps - 1 - t) * cout + co;
      rows = cin;
    }
    const int off = (((k >> 3) * (rows / 8) + (row >> 3)) * 8 + (row & 7)) * 8 + (k & 7);
    img[off] = __float2bfloat16(w[i]);
  }
}

// dW rows (tap CIN + ci) x cout -> torch layout [co][ci][taps]
__global__ void unpack_wgrad_kernel(const float* __restrict__ dwk, int cout, int cin, int taps,
                                    float* __restrict__ dw) {
  const int total = cout * cin * taps;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int co = i / (cin * taps), rem = i % (cin * taps), ci = rem / taps, t = rem % taps;
    dw[i] = dwk[(t * cin + ci) * cout + co];
  }
}

// 2x2 average pooling (H, W even) and its adjoint
__global__ void avgpool2_kernel(const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out, int B, int H,
                                int W, int C, int backward) {
  const int Ho = H / 2, Wo = W / 2;
  const int64_t total = (int64_t)B * Ho * Wo * C;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t pix = i / C;
    const int xo = (int)(pix % Wo), yo = (int)((pix / Wo) % Ho), b = (int)(pix / ((int64_t)Wo * Ho));
    const int64_t base = (((int64_t)b * H + 2 * yo) * W + 2 * xo) * C + c;
    if (!backward) {
      const float s = __bfloat162float(in[base]) + __bfloat162float(in[base + C]) +
                      __bfloat162float(in[base + (int64_t)W * C]) + __bfloat162float(in[base + (int64_t)W * C + C]);
      out[i] = __float2bfloat16(0.25f * s);
    } else {  // in: gradient at the pooled size; out: gradient at full size
      const __nv_bfloat16 g = __float2bfloat16(0.25f * __bfloat162float(in[i]));
      out[base] = g;
      out[base + C] = g;
      out[base + (int64_t)W * C] = g;
      out[base + (int64_t)W * C + C] = g;
    }
  }
}

// f x f block transfers between a fine NHWC image (H x W) and a coarse one (H / f x W / f),
// eight channels (16 bytes) per thread, float sums rounded to bf16 once:
//   block_sum:   coarse = scale * (sum over the f x f block of fine)   (pooling, adjoint of upsampling)
//   block_bcast: fine   = scale * coarse of its block                  (upsampling, adjoint of pooling)
__device__ __forceinline__ void bf16x8_acc(const uint4& v, float* a) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const float2 f = __bfloat1622float2(h[u]);
    a[2 * u] += f.x;
    a[2 * u + 1] += f.y;
  }
}

__device__ __forceinline__ uint4 bf16x8_pack(const float* a, float scale) {
  uint4 v;
  __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&v);
#pragma unroll
  for (int u = 0; u < 4; ++u) h[u] = __floats2bfloat162_rn(scale * a[2 * u], scale * a[2 * u + 1]);
  return v;
}

// F: the block size as a template constant (the f x f loads unrolled and in flight together),
// 0 for a runtime f; C8 = 4 (32 channels) is the U-Net's hidden width
template <int F>
__global__ void block_sum_kernel(const uint4* __restrict__ fine, uint4* __restrict__ coarse, int B, int H, int W,
                                 int C8, int f_rt, float scale, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  const int f = F > 0 ? F : f_rt;
  const int Ho = H / f, Wo = W / f;
  const int64_t total = (int64_t)B * Ho * Wo * C8;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C8);
    const int64_t pix = i / C8;
    const int xo = (int)(pix % Wo), yo = (int)((pix / Wo) % Ho), b = (int)(pix / ((int64_t)Wo * Ho));
    float a[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if constexpr (F > 0) {
      uint4 v[F * F];
#pragma unroll
      for (int dy = 0; dy < F; ++dy) {
        const uint4* row = fine + (((int64_t)b * H + (int64_t)F * yo + dy) * W + (int64_t)F * xo) * C8 + c;
#pragma unroll
        for (int dx = 0; dx < F; ++dx) v[dy * F + dx] = __ldg(row + (int64_t)dx * C8);
      }
#pragma unroll
      for (int u = 0; u < F * F; ++u) bf16x8_acc(v[u], a);
    } else {
      for (int dy = 0; dy < f; ++dy) {
        const uint4* row = fine + (((int64_t)b * H + (int64_t)f * yo + dy) * W + (int64_t)f * xo) * C8 + c;
        for (int dx = 0; dx < f; ++dx) bf16x8_acc(__ldg(row + (int64_t)dx * C8), a);
      }
    }
    coarse[i] = bf16x8_pack(a, scale);
  }
}

template <int F>
__global__ void block_bcast_kernel(const uint4* __restrict__ coarse, uint4* __restrict__ fine, int B, int H, int W,
                                   int C8, int f_rt, float scale, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  const int f = F > 0 ? F : f_rt;
  const int Ho = H / f, Wo = W / f;
  const int64_t total = (int64_t)B * H * W * C8;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C8);
    const int64_t pix = i / C8;
    const int x = (int)(pix % W), y = (int)((pix / W) % H), b = (int)(pix / ((int64_t)W * H));
    const uint4 v = __ldg(coarse + (((int64_t)b * Ho + y / f) * Wo + x / f) * C8 + c);
    if (scale == 1.0f) {
      fine[i] = v;
    } else {
      float a[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      bf16x8_acc(v, a);
      fine[i] = bf16x8_pack(a, scale);
    }
  }
}

// nearest 2x upsampling and its adjoint (sum over the 2x2 block)
__global__ void upsample2_kernel(const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out, int B, int H,
                                 int W, int C, int backward) {
  // H, W: the coarse size
  const int64_t total = (int64_t)B * H * W * C;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t pix = i / C;
    const int x = (int)(pix % W), y = (int)((pix / W) % H), b = (int)(pix / ((int64_t)W * H));
    const int64_t base = (((int64_t)b * 2 * H + 2 * y) * 2 * W + 2 * x) * C + c;
    const int64_t W2C = (int64_t)2 * W * C;
    if (!backward) {
      const __nv_bfloat16 v = in[i];
      out[base] = v;
      out[base + C] = v;
      out[base + W2C] = v;
      out[base + W2C + C] = v;
    } else {
      const float s = __bfloat162float(in[base]) + __bfloat162float(in[base + C]) + __bfloat162float(in[base + W2C]) +
                      __bfloat162float(in[base + W2C + C]);
      out[i] = __float2bfloat16(s);
    }
  }
}

// g *= (y > 0): gradient through a ReLU whose output is y
__global__ void relu_backward_kernel(__nv_bfloat16* __restrict__ g, const __nv_bfloat16* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!(__bfloat162float(y[i]) > 0.0f)) g[i] = __float2bfloat16(0.0f);
}

// a += b (bf16, for gradients that meet at a skip connection)
__global__ void add_inplace_kernel(__nv_bfloat16* __restrict__ a, const __nv_bfloat16* __restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = __float2bfloat16(__bfloat162float(a[i]) + __bfloat162float(b[i]));
}

// dbias[c] += sum over pixels of g[p, c]
__global__ void bias_grad_kernel(const __nv_bfloat16* __restrict__ g, int64_t P, int C, float* __restrict__ db) {
  extern __shared__ float sh[];
  for (int c = threadIdx.x; c < C; c += blockDim.x) sh[c] = 0.0f;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P * C; i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&sh[i % C], __bfloat162float(g[i]));
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) atomicAdd(&db[c], sh[c]);
}

// node vector (float, n_nodes = Hn x Wn, node i*Wn + j) -> NHWC C = 16 image (Hp x Wp) with
// channel 0 = s * r, channel 1 = aux (per-node feature), other channels 0; s = 1/rms(r) read
// from scale[0] (null: 1).  One image per call (B = 1).
// node field (Hn x Wn nodes, nd interleaved components: r[node nd + c]) -> NHWC 16-channel
// image Hp x Wp: channels 0 .. nd-1 the field (times scale[0] when given), channels
// nd .. nd+naux-1 the per-node features aux[node naux + a], zeros elsewhere
__global__ void grid_from_field_kernel(const float* __restrict__ r, int nd, const float* __restrict__ aux, int naux,
                                       const float* __restrict__ scale, int Hn, int Wn, int Hp, int Wp,
                                       __nv_bfloat16* __restrict__ img, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  const int64_t total = (int64_t)Hp * Wp;
  const float s = scale ? scale[0] : 1.0f;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p / Wp), j = (int)(p % Wp);
    __align__(16) __nv_bfloat16 h[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) h[c] = __float2bfloat16(0.0f);
    if (i < Hn && j < Wn) {
      const int64_t node = (int64_t)i * Wn + j;
      for (int c = 0; c < nd; ++c) h[c] = __float2bfloat16(s * r[node * nd + c]);
      if (aux)
        for (int a = 0; a < naux; ++a) h[nd + a] = __float2bfloat16(aux[node * naux + a]);
    }
    uint4* dst = reinterpret_cast<uint4*>(img + p * 16);
    dst[0] = reinterpret_cast<uint4*>(h)[0];
    dst[1] = reinterpret_cast<uint4*>(h)[1];
  }
}

// channels 0 .. nd-1 of an NHWC image with C channels -> node field z[node nd + c]
__global__ void field_from_grid_kernel(const __nv_bfloat16* __restrict__ img, int C, int nd, int Hn, int Wn, int Wp,
                                       float* __restrict__ z, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  const int64_t total = (int64_t)Hn * Wn * nd;
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < total; d += (int64_t)gridDim.x * blockDim.x) {
    const int64_t node = d / nd;
    const int c = (int)(d - node * nd);
    const int i = (int)(node / Wn), j = (int)(node % Wn);
    z[d] = __bfloat162float(img[((int64_t)i * Wp + j) * C + c]);
  }
}

// 1 / rms of a float vector (single block)
// 1 / rms of r over a cluster of kRmsCluster CTAs: float4 loads (when r is 16-byte aligned),
// float partial sums per thread, float64 within and across the CTAs, the CTA totals read by
// rank 0 through distributed shared memory (no global workspace, no atomics)
constexpr int kRmsCluster = 8;
__global__ void __cluster_dims__(kRmsCluster, 1, 1) __launch_bounds__(1024)
    inv_rms_kernel(const float* __restrict__ r, int64_t n, float* __restrict__ out) {
  cg::cluster_group cluster = cg::this_cluster();
  __shared__ double sh[32];
  __shared__ double total;
  const int rank = (int)cluster.block_rank();
  const int64_t t0 = (int64_t)rank * blockDim.x + threadIdx.x, nt = (int64_t)kRmsCluster * blockDim.x;
  float s0 = 0.f, s1 = 0.f;
  int64_t tail = 0;
  if ((reinterpret_cast<uintptr_t>(r) & 15u) == 0) {
    const float4* r4 = reinterpret_cast<const float4*>(r);
    const int64_t n4 = n >> 2;
    int64_t i = t0;
    for (; i + 3 * nt < n4; i += 4 * nt) {  // four independent 16-byte loads in flight per thread
      const float4 a = __ldg(r4 + i), b = __ldg(r4 + i + nt), c = __ldg(r4 + i + 2 * nt), d = __ldg(r4 + i + 3 * nt);
      s0 += (a.x * a.x + a.y * a.y) + (a.z * a.z + a.w * a.w) + (b.x * b.x + b.y * b.y) + (b.z * b.z + b.w * b.w);
      s1 += (c.x * c.x + c.y * c.y) + (c.z * c.z + c.w * c.w) + (d.x * d.x + d.y * d.y) + (d.z * d.z + d.w * d.w);
    }
    for (; i < n4; i += nt) {
      const float4 a = __ldg(r4 + i);
      s0 += (a.x * a.x + a.y * a.y) + (a.z * a.z + a.w * a.w);
    }
    tail = n4 << 2;
  }
  for (int64_t i = tail + t0; i < n; i += nt) s1 += r[i] * r[i];
  double d = (double)s0 + (double)s1;
  for (int o = 16; o >= 1; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = d;
  __syncthreads();
  if (threadIdx.x < 32) {
    d = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o >= 1; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if (threadIdx.x == 0) total = d;
  }
  cluster.sync();
  if (rank == 0 && threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < kRmsCluster; ++q) t += *cluster.map_shared_rank(&total, q);
    out[0] = t > 0.0 ? (float)(1.0 / sqrt(t / (double)n)) : 1.0f;
  }
  cluster.sync();  // the other CTAs' shared memory stays valid until rank 0 has read it
}

// Bilinear transfer between a structured coarse node grid Hc x Wc and the fine grid
// Hf x Wf = ((Hc - 1) f + 1) x ((Wc - 1) f + 1) whose node (f I, f J) is coarse node (I, J).
// Prolongation: fine(i, j) = sum over the (up to 4) surrounding coarse nodes of
// w(i - f I) w(j - f J) coarse(I, J), w(d) = 1 - |d| / f.  Restriction is its transpose,
// evaluated as a gather over the (2f - 1)^2 fine nodes around each coarse node.
__global__ void prolong_kernel(const float* __restrict__ c, int nd, int Hc, int Wc, int f, float* __restrict__ out) {
  const int Wf = (Wc - 1) * f + 1;
  const int64_t total = (int64_t)((Hc - 1) * f + 1) * Wf * nd;
  const float inv = 1.0f / (float)f;
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < total; d += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = d / nd;
    const int k = (int)(d - p * nd);
    const int i = (int)(p / Wf), j = (int)(p - (int64_t)(p / Wf) * Wf);
    const int I = i / f, J = j / f;
    const float ti = (float)(i - I * f) * inv, tj = (float)(j - J * f) * inv;
    const int I1 = I + 1 < Hc ? I + 1 : I, J1 = J + 1 < Wc ? J + 1 : J;
    const float v00 = c[((int64_t)I * Wc + J) * nd + k], v01 = c[((int64_t)I * Wc + J1) * nd + k];
    const float v10 = c[((int64_t)I1 * Wc + J) * nd + k], v11 = c[((int64_t)I1 * Wc + J1) * nd + k];
    out[d] = (1.0f - ti) * ((1.0f - tj) * v00 + tj * v01) + ti * ((1.0f - tj) * v10 + tj * v11);
  }
}

// coarse = P^T fine per component; `fixed` (optional) flags fine DOFs (node nd + component):
// a coarse component whose fine DOF at the same node is fixed is zero
__global__ void restrict_kernel(const float* __restrict__ fine, const unsigned char* __restrict__ fixed, int nd, int Hc,
                                int Wc, int f, float* __restrict__ out) {
  const int Hf = (Hc - 1) * f + 1, Wf = (Wc - 1) * f + 1;
  const int64_t total = (int64_t)Hc * Wc * nd;
  const float inv = 1.0f / (float)f;
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < total; d += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = d / nd;
    const int k = (int)(d - q * nd);
    const int I = (int)(q / Wc), J = (int)(q - (int64_t)(q / Wc) * Wc);
    const int ci = I * f, cj = J * f;
    float acc = 0.0f;
    if (!(fixed && fixed[((int64_t)ci * Wf + cj) * nd + k])) {
      for (int di = -(f - 1); di <= f - 1; ++di) {
        const int i = ci + di;
        if (i < 0 || i >= Hf) continue;
        const float wi = 1.0f - (float)abs(di) * inv;
        float row = 0.0f;
        for (int dj = -(f - 1); dj <= f - 1; ++dj) {
          const int j = cj + dj;
          if (j < 0 || j >= Wf) continue;
          row += (1.0f - (float)abs(dj) * inv) * fine[((int64_t)i * Wf + j) * nd + k];
        }
        acc += wi * row;
      }
    }
    out[d] = acc;
  }
}

// ---- the coarse-grid network's transfers, fused ------------------------------------------
// restrict_sq_kernel: coarse = P^T fine as restrict_kernel, with the block size F of the
// transfer a template constant (the (2F - 1)^2 taps unrolled, so a thread's loads are all in
// flight together; F = 0: runtime f), 32-bit index arithmetic, and one float64 partial sum of
// squares of the block's outputs in partials[blockIdx.x].  image_from_coarse_kernel: every
// block first adds the np partials itself (fixed order), so 1 / rms needs no launch of its own,
// then writes (coarse / rms, aux) into the image as grid_from_field_kernel does.
// prolong_image_kernel: fine = P applied to channels 0 .. nd-1 of the network's output image
// (the coarse field is never written out), zero at fixed DOFs.
constexpr int kRestrictBlocks = 1024;  // largest grid of restrict_sq_kernel (partials it writes)

template <int F>
__global__ void __launch_bounds__(256)
restrict_sq_kernel(const float* __restrict__ fine, const unsigned char* __restrict__ fixed, int nd, int Hc, int Wc,
                   int f_rt, float* __restrict__ out, double* __restrict__ partials, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  const int f = F > 0 ? F : f_rt;
  const int Hf = (Hc - 1) * f + 1, Wf = (Wc - 1) * f + 1;
  const int total = Hc * Wc * nd;
  const float inv = 1.0f / (float)f;
  float sq = 0.0f;
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < total; d += gridDim.x * blockDim.x) {
    const int q = d / nd, k = d - q * nd;
    const int I = q / Wc, J = q - I * Wc;
    const int ci = I * f, cj = J * f;
    float acc = 0.0f;
    if (!(fixed && fixed[((int64_t)ci * Wf + cj) * nd + k])) {
      if constexpr (F > 0) {
#pragma unroll
        for (int di = -(F - 1); di <= F - 1; ++di) {
          const int i = ci + di;
          const float wi = (i >= 0 && i < Hf) ? 1.0f - (float)(di < 0 ? -di : di) * inv : 0.0f;
          const int ii = i < 0 ? 0 : (i >= Hf ? Hf - 1 : i);
          float row = 0.0f;
#pragma unroll
          for (int dj = -(F - 1); dj <= F - 1; ++dj) {
            const int j = cj + dj;
            const float wj = (j >= 0 && j < Wf) ? 1.0f - (float)(dj < 0 ? -dj : dj) * inv : 0.0f;
            const int jj = j < 0 ? 0 : (j >= Wf ? Wf - 1 : j);
            row += wj * __ldg(fine + ((int64_t)ii * Wf + jj) * nd + k);
          }
          acc += wi * row;
        }
      } else {
        for (int di = -(f - 1); di <= f - 1; ++di) {
          const int i = ci + di;
          if (i < 0 || i >= Hf) continue;
          const float wi = 1.0f - (float)abs(di) * inv;
          float row = 0.0f;
          for (int dj = -(f - 1); dj <= f - 1; ++dj) {
            const int j = cj + dj;
            if (j < 0 || j >= Wf) continue;
            row += (1.0f - (float)abs(dj) * inv) * fine[((int64_t)i * Wf + j) * nd + k];
          }
          acc += wi * row;
        }
      }
    }
    out[d] = acc;
    sq += acc * acc;
  }
  __shared__ double sh[8];
  double v = (double)sq;
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    partials[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(256)
image_from_coarse_kernel(const float* __restrict__ r, int nd, const float* __restrict__ aux, int naux,
                         const double* __restrict__ partials, int np, int64_t n, float* __restrict__ scale, int Hn,
                         int Wn, int Hp, int Wp, __nv_bfloat16* __restrict__ img, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  __shared__ double sh[8];
  __shared__ float s_sh;
  double v = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) v += partials[i];
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    const float sc = t > 0.0 ? (float)(1.0 / sqrt(t / (double)n)) : 1.0f;
    s_sh = sc;
    if (blockIdx.x == 0) scale[0] = sc;
  }
  __syncthreads();
  const float s = s_sh;
  const int total = Hp * Wp;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
    const int i = p / Wp, j = p - i * Wp;
    __align__(16) __nv_bfloat16 h[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) h[c] = __float2bfloat16(0.0f);
    if (i < Hn && j < Wn) {
      const int64_t node = (int64_t)i * Wn + j;
      for (int c = 0; c < nd; ++c) h[c] = __float2bfloat16(s * r[node * nd + c]);
      if (aux)
        for (int a = 0; a < naux; ++a) h[nd + a] = __float2bfloat16(aux[node * naux + a]);
    }
    uint4* dst = reinterpret_cast<uint4*>(img + (int64_t)p * 16);
    dst[0] = reinterpret_cast<uint4*>(h)[0];
    dst[1] = reinterpret_cast<uint4*>(h)[1];
  }
}

// one fine row per blockIdx.y; F as in restrict_sq_kernel
template <int F>
__global__ void __launch_bounds__(256)
prolong_image_kernel(const __nv_bfloat16* __restrict__ img, int C, int nd, int Hc, int Wc, int Wp, int f_rt,
                     const unsigned char* __restrict__ fixed, float* __restrict__ out, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  const int f = F > 0 ? F : f_rt;
  const int Wf = (Wc - 1) * f + 1;
  const int i = blockIdx.y;
  const int I = i / f;
  const float inv = 1.0f / (float)f;
  const float ti = (float)(i - I * f) * inv;
  const int I1 = I + 1 < Hc ? I + 1 : I;
  const int row_len = Wf * nd;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < row_len; t += gridDim.x * blockDim.x) {
    const int j = t / nd, k = t - j * nd;
    const int64_t d = (int64_t)i * row_len + t;
    float v = 0.0f;
    if (!(fixed && fixed[d])) {
      const int J = j / f;
      const float tj = (float)(j - J * f) * inv;
      const int J1 = J + 1 < Wc ? J + 1 : J;
      const float v00 = __bfloat162float(img[((int64_t)I * Wp + J) * C + k]);
      const float v01 = __bfloat162float(img[((int64_t)I * Wp + J1) * C + k]);
      const float v10 = __bfloat162float(img[((int64_t)I1 * Wp + J) * C + k]);
      const float v11 = __bfloat162float(img[((int64_t)I1 * Wp + J1) * C + k]);
      v = (1.0f - ti) * ((1.0f - tj) * v00 + tj * v01) + ti * ((1.0f - tj) * v10 + tj * v11);
    }
    out[d] = v;
  }
}

// NHWC bf16 tensor {C, W, H, B} with the halo box {8, 130, 3, 1}
int make_halo_map(CUtensorMap* m, const void* base, int C, int B, int H, int W) {
  auto fn = encode_fn();
  if (!fn) return AGX_ERR_CUDA;
  const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
  const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
  const cuuint32_t box[4] = {8, (cuuint32_t)kHaloW, 3, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? AGX_OK : AGX_ERR_ARG;
}

constexpr int kLoadAuto = 3;  // the warp-specialised kernel for concatenating layers of >= 128^2 pixels
int g_halo_loader = kLoadAuto;  // agx_nn_set_halo_loader

template <int C1, int C2, int COUT, int EPI, int LD>
int launch_conv_as(const ConvArgs& a, cudaStream_t s) {
  constexpr int CIN = C1 + C2;
  constexpr int smem = 9 * CIN * COUT * 2 + kStages * (CIN / 8) * kPlaneBytes;
  void (*kernel)(ConvMaps, ConvArgs);
  if constexpr (LD == kLoadTmaWs) kernel = conv3x3_ws<C1, C2, COUT, EPI>;
  else kernel = conv3x3_tc<C1, C2, COUT, EPI, LD>;
  const int threads = LD == kLoadTmaWs ? kWsThreads : kTile;
  static int per_sm = 0;
  if (!per_sm) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
        cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared) != cudaSuccess)
      return AGX_ERR_CUDA;
    // resident CTAs per SM from the shared-memory budget (at most 8: TMEM holds 512 columns)
    int dev = 0, per_sm_smem = 0, reserved = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    per_sm = per_sm_smem / (smem + reserved + 256);
    const int tmem_cap = 512 / tmem_cols(2 * COUT);
    per_sm = per_sm < 1 ? 1 : (per_sm > tmem_cap ? tmem_cap : per_sm);
  }
  ConvMaps maps{};
  if constexpr (LD != kLoadAsync) {
    if (int rc = make_halo_map(&maps.in1, a.in1, C1, a.B, a.H, a.W)) return rc;
    if (C2 > 0) {
      if (int rc = make_halo_map(&maps.in2, a.in2, C2, a.B, a.H, a.W)) return rc;
    } else {
      maps.in2 = maps.in1;
    }
  } else if ((reinterpret_cast<uintptr_t>(a.in1) | reinterpret_cast<uintptr_t>(a.in2)) & 15u) {
    return AGX_ERR_ARG;  // 16-byte pixel chunks
  }
  const int64_t tiles = (int64_t)a.B * a.H * ((a.W + kTile - 1) / kTile);
  const int64_t cap = (int64_t)per_sm * sm_count();
  const int grid = (int)(tiles < cap ? tiles : cap);
  agx_launch_pdl(kernel, grid, threads, smem, s, maps, a);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

template <int C1, int C2, int COUT, int EPI>
int launch_conv(const ConvArgs& a, cudaStream_t s, int loader) {
  // measured (320^2 U-Net levels): the warp-specialised kernel 18 % faster on the two-input
  // layers, within a few percent either way on the others
  const bool ws = loader == kLoadTmaWs || (loader == kLoadAuto && C2 > 0 && (int64_t)a.H * a.W >= 128 * 128);
  if (ws) return launch_conv_as<C1, C2, COUT, EPI, kLoadTmaWs>(a, s);
  return loader == kLoadAsync ? launch_conv_as<C1, C2, COUT, EPI, kLoadAsync>(a, s)
                              : launch_conv_as<C1, C2, COUT, EPI, kLoadTma>(a, s);
}

template <int C1, int C2, int COUT, int TAPS = 9>
int launch_wgrad(const WgradArgs& a0, cudaStream_t s) {
  constexpr int CIN = C1 + C2, PCH = 256;
  const int smem = kTile * PCH * 2 + COUT * PCH * 2;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(wgrad_tc<C1, C2, COUT, PCH, TAPS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess)
      return AGX_ERR_CUDA;
    attr = true;
  }
  WgradArgs a = a0;
  const int64_t P = (int64_t)a.B * a.D * a.H * a.W;
  a.pix_per_cta = 2048;
  const dim3 grid((unsigned)((P + a.pix_per_cta - 1) / a.pix_per_cta), (unsigned)((TAPS * CIN + kTile - 1) / kTile));
  wgrad_tc<C1, C2, COUT, PCH, TAPS><<<grid, kTile, smem, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int grid1(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g < 152 * 8 ? (g < 1 ? 1 : g) : 152 * 8);
}

// fine (H x W) -> coarse block sums times `scale`, and coarse -> fine broadcasts times `scale`
void launch_block_sum(const void* fine, void* coarse, int B, int H, int W, int C, int f, float scale, cudaStream_t s) {
  const int g = grid1((int64_t)B * (H / f) * (W / f) * (C / 8));
  const uint4* in = (const uint4*)fine;
  uint4* out = (uint4*)coarse;
  if (f == 2) agx_launch_pdl(block_sum_kernel<2>, g, 256, 0, s, in, out, B, H, W, C / 8, f, scale, g_nn_skip);
  else if (f == 4) agx_launch_pdl(block_sum_kernel<4>, g, 256, 0, s, in, out, B, H, W, C / 8, f, scale, g_nn_skip);
  else agx_launch_pdl(block_sum_kernel<0>, g, 256, 0, s, in, out, B, H, W, C / 8, f, scale, g_nn_skip);
}

void launch_block_bcast(const void* coarse, void* fine, int B, int H, int W, int C, int f, float scale,
                        cudaStream_t s) {
  const int g = grid1((int64_t)B * H * W * (C / 8));
  const uint4* in = (const uint4*)coarse;
  uint4* out = (uint4*)fine;
  if (f == 2) agx_launch_pdl(block_bcast_kernel<2>, g, 256, 0, s, in, out, B, H, W, C / 8, f, scale, g_nn_skip);
  else if (f == 4) agx_launch_pdl(block_bcast_kernel<4>, g, 256, 0, s, in, out, B, H, W, C / 8, f, scale, g_nn_skip);
  else agx_launch_pdl(block_bcast_kernel<0>, g, 256, 0, s, in, out, B, H, W, C / 8, f, scale, g_nn_skip);
}

}  // namespace

extern "C" {

int agx_nn_conv3x3(const void* in1, const void* in2, int c1, int c2, const void* wpk, const float* bias, void* out1,
                   void* out2, int split, int cout, int relu, int B, int H, int W, int* err, void* stream) {
  if (relu & ~(1 | AGX_NN_CONST_WEIGHTS | (3 << 4))) return AGX_ERR_ARG;
  const int const_weights = (relu & AGX_NN_CONST_WEIGHTS) ? 1 : 0;
  const int pick = (relu >> 4) & 3;  // AGX_NN_LOADER(l) = (l + 1) << 4; 0: the process-wide choice
  const int loader = pick ? pick - 1 : g_halo_loader;
  relu &= 1;
  ConvArgs a{(const __nv_bfloat16*)in1, (const __nv_bfloat16*)in2, (const __nv_bfloat16*)wpk, bias,
             (__nv_bfloat16*)out1, (__nv_bfloat16*)out2, split, B, H, W, err, const_weights, g_nn_skip};
  cudaStream_t s = (cudaStream_t)stream;
  if (!in1 || !wpk || !out1 || !err || B <= 0 || H <= 0 || W <= 0) return AGX_ERR_ARG;
  if (split <= 0 || split > cout || split % 8 || (split < cout && !out2)) return AGX_ERR_ARG;
  if (reinterpret_cast<uintptr_t>(wpk) & 15u) return AGX_ERR_ARG;  // one bulk copy into shared memory
#define AGX_CONV(C1_, C2_, CO_, R_)                                                         \
  if (c1 == C1_ && c2 == C2_ && cout == CO_ && relu == R_) return launch_conv<C1_, C2_, CO_, R_>(a, s, loader);
  AGX_CONV(16, 0, 32, 1)
  AGX_CONV(32, 0, 32, 1)
  AGX_CONV(32, 32, 32, 1)
  AGX_CONV(32, 0, 16, 0)
  // input-gradient convolutions (no epilogue): dOut channels in, layer-input channels out
  AGX_CONV(32, 0, 16, 0)
  AGX_CONV(32, 0, 32, 0)
  AGX_CONV(32, 0, 64, 0)
  AGX_CONV(16, 0, 32, 0)
#undef AGX_CONV
  return AGX_ERR_UNSUPPORTED;
}

int agx_nn_set_skip_flag(const int* flag) {
  g_nn_skip = flag;
  return AGX_OK;
}

int agx_nn_set_halo_loader(int loader) {
  if (loader < kLoadAsync || loader > kLoadAuto) return AGX_ERR_ARG;
  g_halo_loader = loader;
  return AGX_OK;
}

int agx_nn_wgrad3x3(const void* in1, const void* in2, int c1, int c2, const void* dout, int cout, float* dw_rows,
                    int B, int H, int W, int* err, void* stream) {
  if (!in1 || !dout || !dw_rows || !err || B <= 0 || H <= 0 || W <= 0) return AGX_ERR_ARG;
  WgradArgs a{(const __nv_bfloat16*)in1, (const __nv_bfloat16*)in2, (const __nv_bfloat16*)dout, dw_rows, B, 1, H, W,
              0, err};
  cudaStream_t s = (cudaStream_t)stream;
#define AGX_WG(C1_, C2_, CO_) \
  if (c1 == C1_ && c2 == C2_ && cout == CO_) return launch_wgrad<C1_, C2_, CO_>(a, s);
  AGX_WG(16, 0, 32)
  AGX_WG(32, 0, 32)
  AGX_WG(32, 32, 32)
  AGX_WG(32, 0, 16)
#undef AGX_WG
  return AGX_ERR_UNSUPPORTED;
}

int agx_nn_wgrad3x3x3(const void* in1, const void* in2, int c1, int c2, const void* dout, int cout, float* dw_rows,
                      int B, int D, int H, int W, int* err, void* stream) {
  if (!in1 || !dout || !dw_rows || !err || B <= 0 || D <= 0 || H <= 0 || W <= 0 || (c2 > 0 && !in2))
    return AGX_ERR_ARG;
  WgradArgs a{(const __nv_bfloat16*)in1, (const __nv_bfloat16*)in2, (const __nv_bfloat16*)dout, dw_rows, B, D, H, W,
              0, err};
  cudaStream_t s = (cudaStream_t)stream;
  if (c1 == 16 && c2 == 0 && cout == 16) return launch_wgrad<16, 0, 16, 27>(a, s);
  if (c1 == 16 && c2 == 16 && cout == 16) return launch_wgrad<16, 16, 16, 27>(a, s);
  return AGX_ERR_UNSUPPORTED;
}

int agx_nn_pack_weights(const float* w, int cout, int cin, int mode, void* img, void* stream) {
  if (!w || !img || cout % 8 || cin % 8) return AGX_ERR_ARG;
  pack_weights_kernel<<<grid1((int64_t)cout * cin * 9), 256, 0, (cudaStream_t)stream>>>(w, cout, cin, 9, mode,
                                                                                       (__nv_bfloat16*)img);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_unpack_wgrad(const float* dw_rows, int cout, int cin, float* dw, void* stream) {
  unpack_wgrad_kernel<<<grid1((int64_t)cout * cin * 9), 256, 0, (cudaStream_t)stream>>>(dw_rows, cout, cin, 9, dw);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_pack_weights3d(const float* w, int cout, int cin, int mode, void* img, void* stream) {
  if (!w || !img || cout % 8 || cin % 8) return AGX_ERR_ARG;
  pack_weights_kernel<<<grid1((int64_t)cout * cin * 27), 256, 0, (cudaStream_t)stream>>>(w, cout, cin, 27, mode,
                                                                                        (__nv_bfloat16*)img);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_unpack_wgrad3d(const float* dw_rows, int cout, int cin, float* dw, void* stream) {
  if (!dw_rows || !dw) return AGX_ERR_ARG;
  unpack_wgrad_kernel<<<grid1((int64_t)cout * cin * 27), 256, 0, (cudaStream_t)stream>>>(dw_rows, cout, cin, 27, dw);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_pool2(const void* in, void* out, int B, int H, int W, int C, int backward, void* stream) {
  if (H % 2 || W % 2) return AGX_ERR_ARG;
  avgpool2_kernel<<<grid1((int64_t)B * H * W * C / 4), 256, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)in, (__nv_bfloat16*)out, B, H, W, C, backward);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_pool(const void* in, void* out, int B, int H, int W, int C, int f, int backward, void* stream) {
  if (!in || !out || B <= 0 || f < 1 || f > 64 || H % f || W % f || C % 8 ||
      ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u))
    return AGX_ERR_ARG;
  const float inv = 1.0f / (float)(f * f);
  if (!backward)
    launch_block_sum(in, out, B, H, W, C, f, inv, (cudaStream_t)stream);
  else
    launch_block_bcast(in, out, B, H, W, C, f, inv, (cudaStream_t)stream);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_upsample(const void* in, void* out, int B, int H, int W, int C, int f, int backward, void* stream) {
  if (!in || !out || B <= 0 || f < 1 || f > 64 || C % 8 ||
      ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u))
    return AGX_ERR_ARG;
  if (!backward)
    launch_block_bcast(in, out, B, H * f, W * f, C, f, 1.0f, (cudaStream_t)stream);
  else
    launch_block_sum(in, out, B, H * f, W * f, C, f, 1.0f, (cudaStream_t)stream);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_upsample2(const void* in, void* out, int B, int H, int W, int C, int backward, void* stream) {
  upsample2_kernel<<<grid1((int64_t)B * H * W * C), 256, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)in, (__nv_bfloat16*)out, B, H, W, C, backward);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_relu_backward(void* g, const void* y, int64_t n, void* stream) {
  relu_backward_kernel<<<grid1(n), 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16*)g, (const __nv_bfloat16*)y, n);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_add(void* a, const void* b, int64_t n, void* stream) {
  add_inplace_kernel<<<grid1(n), 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16*)a, (const __nv_bfloat16*)b, n);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_bias_grad(const void* g, int64_t P, int C, float* db, void* stream) {
  bias_grad_kernel<<<grid1(P * C), 256, C * sizeof(float), (cudaStream_t)stream>>>((const __nv_bfloat16*)g, P, C, db);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_grid_from_vector(const float* r, const float* aux, int Hn, int Wn, int Hp, int Wp, int normalize,
                            float* scale, void* img, void* stream) {
  return agx_nn_grid_from_field(r, 1, aux, aux ? 1 : 0, Hn, Wn, Hp, Wp, normalize, scale, img, stream);
}

int agx_nn_grid_from_field(const float* r, int nd, const float* aux, int naux, int Hn, int Wn, int Hp, int Wp,
                           int normalize, float* scale, void* img, void* stream) {
  if (!r || !img || nd < 1 || nd > 3 || naux < 0 || nd + naux > 16 || (naux > 0 && !aux) || Hn > Hp || Wn > Wp ||
      (normalize && !scale))
    return AGX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (normalize) inv_rms_kernel<<<kRmsCluster, 1024, 0, s>>>(r, (int64_t)Hn * Wn * nd, scale);
  agx_launch_pdl(grid_from_field_kernel, grid1((int64_t)Hp * Wp), 256, 0, s, r, nd, naux > 0 ? aux : nullptr, naux,
                 normalize ? scale : nullptr, Hn, Wn, Hp, Wp, (__nv_bfloat16*)img, g_nn_skip);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_restrict_image_work(void) { return kRestrictBlocks; }

int agx_nn_restrict_image(const float* fine, const unsigned char* fixed, int nd, const float* aux, int naux, int Hc,
                          int Wc, int f, int Hp, int Wp, float* coarse, double* work, float* scale, void* img,
                          void* stream) {
  if (!fine || !coarse || !work || !scale || !img || nd < 1 || nd > 3 || naux < 0 || nd + naux > 16 ||
      (naux > 0 && !aux) || Hc < 2 || Wc < 2 || f < 1 || f > 64 || Hc > Hp || Wc > Wp ||
      (int64_t)Hc * Wc * nd >= (1LL << 31) || (int64_t)Hp * Wp >= (1LL << 31))
    return AGX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t total = (int64_t)Hc * Wc * nd;
  const int nb = (int)std::min<int64_t>(kRestrictBlocks, (total + 255) / 256);
  switch (f) {
    case 2: agx_launch_pdl(restrict_sq_kernel<2>, nb, 256, 0, s, fine, fixed, nd, Hc, Wc, f, coarse, work, g_nn_skip); break;
    case 4: agx_launch_pdl(restrict_sq_kernel<4>, nb, 256, 0, s, fine, fixed, nd, Hc, Wc, f, coarse, work, g_nn_skip); break;
    case 8: agx_launch_pdl(restrict_sq_kernel<8>, nb, 256, 0, s, fine, fixed, nd, Hc, Wc, f, coarse, work, g_nn_skip); break;
    default: agx_launch_pdl(restrict_sq_kernel<0>, nb, 256, 0, s, fine, fixed, nd, Hc, Wc, f, coarse, work, g_nn_skip); break;
  }
  agx_launch_pdl(image_from_coarse_kernel, grid1((int64_t)Hp * Wp), 256, 0, s, coarse, nd, naux > 0 ? aux : nullptr,
                 naux, work, nb, total, scale, Hc, Wc, Hp, Wp, (__nv_bfloat16*)img, g_nn_skip);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_prolong_image(const void* img, int C, int nd, int Hc, int Wc, int Wp, int f, const unsigned char* fixed,
                         float* fine, void* stream) {
  if (!img || !fine || nd < 1 || nd > C || Hc < 2 || Wc < 2 || Wc > Wp || f < 1 || f > 64) return AGX_ERR_ARG;
  const int64_t Hf = (int64_t)(Hc - 1) * f + 1, row = ((int64_t)(Wc - 1) * f + 1) * nd;
  if (Hf > 65535 || Hf * row >= (1LL << 31)) return AGX_ERR_ARG;
  const dim3 grid((unsigned)((row + 255) / 256), (unsigned)Hf);
  cudaStream_t s = (cudaStream_t)stream;
  const __nv_bfloat16* im = (const __nv_bfloat16*)img;
  switch (f) {
    case 2: agx_launch_pdl(prolong_image_kernel<2>, grid, 256, 0, s, im, C, nd, Hc, Wc, Wp, f, fixed, fine, g_nn_skip); break;
    case 4: agx_launch_pdl(prolong_image_kernel<4>, grid, 256, 0, s, im, C, nd, Hc, Wc, Wp, f, fixed, fine, g_nn_skip); break;
    case 8: agx_launch_pdl(prolong_image_kernel<8>, grid, 256, 0, s, im, C, nd, Hc, Wc, Wp, f, fixed, fine, g_nn_skip); break;
    default: agx_launch_pdl(prolong_image_kernel<0>, grid, 256, 0, s, im, C, nd, Hc, Wc, Wp, f, fixed, fine, g_nn_skip); break;
  }
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_restrict(const float* fine, const unsigned char* fixed, int Hc, int Wc, int f, float* coarse,
                    void* stream) {
  return agx_nn_restrict_field(fine, fixed, 1, Hc, Wc, f, coarse, stream);
}

int agx_nn_restrict_field(const float* fine, const unsigned char* fixed, int nd, int Hc, int Wc, int f, float* coarse,
                          void* stream) {
  if (!fine || !coarse || nd < 1 || nd > 3 || Hc < 2 || Wc < 2 || f < 1 || f > 64) return AGX_ERR_ARG;
  restrict_kernel<<<grid1((int64_t)Hc * Wc * nd), 256, 0, (cudaStream_t)stream>>>(fine, fixed, nd, Hc, Wc, f, coarse);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_prolong(const float* coarse, int Hc, int Wc, int f, float* fine, void* stream) {
  return agx_nn_prolong_field(coarse, 1, Hc, Wc, f, fine, stream);
}

int agx_nn_prolong_field(const float* coarse, int nd, int Hc, int Wc, int f, float* fine, void* stream) {
  if (!fine || !coarse || nd < 1 || nd > 3 || Hc < 2 || Wc < 2 || f < 1 || f > 64) return AGX_ERR_ARG;
  prolong_kernel<<<grid1((int64_t)((Hc - 1) * f + 1) * ((Wc - 1) * f + 1) * nd), 256, 0, (cudaStream_t)stream>>>(
      coarse, nd, Hc, Wc, f, fine);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_vector_from_grid(const void* img, int C, int Hn, int Wn, int Wp, float* z, void* stream) {
  return agx_nn_field_from_grid(img, C, 1, Hn, Wn, Wp, z, stream);
}

int agx_nn_field_from_grid(const void* img, int C, int nd, int Hn, int Wn, int Wp, float* z, void* stream) {
  if (!img || !z || nd < 1 || nd > C || Wn > Wp) return AGX_ERR_ARG;
  agx_launch_pdl(field_from_grid_kernel, grid1((int64_t)Hn * Wn * nd), 256, 0, (cudaStream_t)stream,
                 (const __nv_bfloat16*)img, C, nd, Hn, Wn, Wp, z, g_nn_skip);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

}  // extern "C"
