// BF16 tensor-core kernels of the 3-D learned preconditioner: 3x3x3 convolutions, 2x2x2
// pooling and upsampling, and the transfers between the node field of a structured brick
// mesh and the network's coarse image.  Nothing in AutoPDEx corresponds to this part.
//
// Tensors are NDHWC bf16 (batch, z, y, x, channel) with 16 or 32 channels.  A 3x3x3
// convolution (stride 1, zero padding 1) is the implicit GEMM D[voxel, cout] =
// sum_k A[voxel, k] B[cout, k], k = tap * CIN + cin, tap = 9 dz + 3 dy + dx.  A tile is 8 (x)
// by 16 (y) output voxels of one z plane, so that a volume of a few dozen voxels a side fills
// its 128-row MMAs.  Its input halo -- 3 planes x 18 rows x 10 voxels -- is one 5-D TMA box
// per 8-channel slice, written to shared memory as [z][y][x] 16-byte voxel chunks (the zero
// fill of the tensor copy is the padding).  In that layout the A operand of every tap is a
// no-swizzle K-major view of the one halo copy: the 8 voxels of a core matrix are one halo
// row's consecutive x (16 bytes apart), consecutive 8-row groups are consecutive y rows (the
// stride byte offset is the halo row, 160 bytes), and the two 8-channel halves of a K = 16
// step are consecutive slices (the leading byte offset); the 27 taps are 27 start addresses.
// The packed weights stay in shared memory for the CTA's lifetime; halos cycle through a ring
// of kStages3 buffers filled ahead by one thread, and the accumulator alternates between two
// TMEM column ranges so the MMAs of tile k overlap the epilogue of tile k - 1.  The input
// gradient is the same kernel with the packed weights flipped and transposed.
//
// Every wait is bounded: a CTA whose copies or MMAs do not complete in time records an error
// flag, waits (bounded) for what it issued and still releases its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "agx_common.cuh"
#include "agx_tc.cuh"
#include "../../include/autopdex_gb300_nn.h"

namespace {

constexpr int kTx = 8, kTy = 16;                            // output tile: 8 x 16 voxels (= kTile)
constexpr int kHx = kTx + 2, kHy = kTy + 2, kHz = 3;        // halo box
constexpr int kSlice3Data = kHx * kHy * kHz * 16;           // bytes one box writes (8640)
constexpr int kSlice3Bytes = (kSlice3Data + 127) / 128 * 128;  // slice stride in shared memory
constexpr int kStages3 = 3;
static_assert(kTx * kTy == kTile, "one MMA row per tile voxel");

struct Conv3Args {
  const __nv_bfloat16* in1;  // NDHWC, C1 channels
  const __nv_bfloat16* in2;  // NDHWC, C2 channels (concatenated after in1), or null when C2 == 0
  const __nv_bfloat16* wpk;  // packed B image (COUT rows x 27 CIN), core-matrix order
  const float* bias;         // COUT values or null
  __nv_bfloat16* out1;       // channels [0, S) (NDHWC with S channels)
  __nv_bfloat16* out2;       // channels [S, COUT) or null when S == COUT
  int split;                 // S
  int B, D, H, W;
  int* err;
  int const_weights;         // weights and bias not written by the kernel just before this one
  const int* skip;           // nonzero there: return at once (the solve using the network has converged)
};

struct Conv3Maps {
  CUtensorMap in1;  // {C1, W, H, D, B} bf16, box {8, 10, 18, 3, 1}
  CUtensorMap in2;  // {C2, W, H, D, B}, unused when C2 == 0
};

__device__ __forceinline__ void tma_load5(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                          uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
      "[%7];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}

struct Tile3 {
  int b, z, y0, x0;
};

// tile index -> (b, z, y0, x0); x tiles fastest, then y tiles, then z, then b
__device__ __forceinline__ Tile3 tile3(const Conv3Args& a, int64_t tile, int tiles_x, int tiles_y) {
  Tile3 t;
  const int64_t r = tile / tiles_x;
  t.x0 = (int)(tile - r * tiles_x) * kTx;
  const int64_t bz = r / tiles_y;
  t.y0 = (int)(r - bz * tiles_y) * kTy;
  t.b = (int)(bz / a.D);
  t.z = (int)(bz - (int64_t)t.b * a.D);
  return t;
}

// one thread: the CIN / 8 slice copies of a tile's halo, completing on `bar`
template <int C1, int C2>
__device__ __forceinline__ void issue_halo3(const Conv3Maps& m, const Conv3Args& a, int64_t tile, int tiles_x,
                                            int tiles_y, uint32_t halo, uint32_t bar) {
  constexpr int NCH = (C1 + C2) / 8;
  const Tile3 t = tile3(a, tile, tiles_x, tiles_y);
  mbar_expect(bar, (uint32_t)(NCH * kSlice3Data));
#pragma unroll
  for (int c = 0; c < C1 / 8; ++c)
    tma_load5(halo + (uint32_t)(c * kSlice3Bytes), &m.in1, 8 * c, t.x0 - 1, t.y0 - 1, t.z - 1, t.b, bar);
  if constexpr (C2 > 0) {
#pragma unroll
    for (int c = 0; c < C2 / 8; ++c)
      tma_load5(halo + (uint32_t)((C1 / 8 + c) * kSlice3Bytes), &m.in2, 8 * c, t.x0 - 1, t.y0 - 1, t.z - 1, t.b, bar);
  }
}

template <int COUT, int EPI>
__device__ __forceinline__ void conv3_epilogue(const Conv3Args& a, const float* sbias, uint32_t tacc, int64_t tile,
                                               int tiles_x, int tiles_y, int tid, int warp) {
  float acc[COUT];
#pragma unroll
  for (int c = 0; c < COUT; c += 16) tmem_ld16(tacc + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, acc + c);
  const Tile3 t = tile3(a, tile, tiles_x, tiles_y);
  const int x = t.x0 + (tid & (kTx - 1)), y = t.y0 + tid / kTx;
  if (x >= a.W || y >= a.H) return;
  const int64_t p = (((int64_t)t.b * a.D + t.z) * a.H + y) * a.W + x;
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

__host__ __device__ constexpr int round1k(int b) { return (b + 1023) / 1024 * 1024; }

// out = epi(conv3x3x3(concat(in1, in2)) + bias); EPI 0: identity, 1: ReLU.  Persistent over
// tiles; the loop is that of the 2-D tensor-copy kernel: (1) thread 0 waits for the halo of
// tile k and issues its 27 CIN / 16 MMAs into accumulator k % 2; (2) all threads wait for the
// MMAs of tile k - 1, thread 0 refills its halo buffer with tile k - 1 + kStages3, and the four
// warps drain the accumulator; a CTA barrier closes the iteration.
template <int C1, int C2, int COUT, int EPI>
__global__ void __launch_bounds__(kTile) conv3x3x3_tc(const __grid_constant__ Conv3Maps maps, Conv3Args a) {
  constexpr int CIN = C1 + C2, K = 27 * CIN, NG = COUT / 8, NCH = CIN / 8;
  constexpr int B_BYTES = K * COUT * 2, B_REGION = round1k(B_BYTES);
  constexpr int HALO_BYTES = NCH * kSlice3Bytes;
  constexpr int NCOLS = tmem_cols(2 * COUT);  // two accumulators
  static_assert(CIN % 16 == 0 && COUT % 16 == 0, "channel counts must be multiples of 16");
  static_assert(B_BYTES % 16 == 0 && HALO_BYTES % 128 == 0, "shared-memory carve-up");
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t full_bar[kStages3];
  __shared__ __align__(8) uint64_t mma_bar[2];
  __shared__ __align__(8) uint64_t w_bar;
  __shared__ float sbias[COUT];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int tiles_x = (a.W + kTx - 1) / kTx, tiles_y = (a.H + kTy - 1) / kTy;
  const int64_t ntiles = (int64_t)a.B * a.D * tiles_y * tiles_x;
  const int64_t first = blockIdx.x, stride = gridDim.x;
  const int64_t my_tiles = first < ntiles ? (ntiles - first + stride - 1) / stride : 0;
  const uint32_t b0 = (uint32_t)__cvta_generic_to_shared(smem);
  const uint32_t halo_base = b0 + B_REGION;
  const uint32_t fbar0 = (uint32_t)__cvta_generic_to_shared(&full_bar[0]);
  const uint32_t mbar0 = (uint32_t)__cvta_generic_to_shared(&mma_bar[0]);
  const uint32_t wbar = (uint32_t)__cvta_generic_to_shared(&w_bar);
  if (tid == 0) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&maps.in1)) : "memory");
    if constexpr (C2 > 0)
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&maps.in2)) : "memory");
#pragma unroll
    for (int s = 0; s < kStages3; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fbar0 + 8u * s));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0 + 8u));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(wbar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (a.const_weights && my_tiles > 0) {
      mbar_expect(wbar, (uint32_t)B_BYTES);
      bulk_load(b0, a.wpk, (uint32_t)B_BYTES, wbar);
    }
  }
  if (a.const_weights && tid < COUT) sbias[tid] = a.bias ? a.bias[tid] : 0.0f;
  if (warp == 0) tmem_alloc<NCOLS>(&tmem_slot);
  agx_pdl_entry();
  if (nn_skip(a.skip)) {
    if (tid == 0 && a.const_weights && my_tiles > 0) mbar_wait(wbar, 0u);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) tmem_free<NCOLS>(tmem_slot);
    return;
  }
  if (tid == 0) {
    if (!a.const_weights && my_tiles > 0) {
      mbar_expect(wbar, (uint32_t)B_BYTES);
      bulk_load(b0, a.wpk, (uint32_t)B_BYTES, wbar);
    }
    for (int j = 0; j < kStages3 && j < my_tiles; ++j)
      issue_halo3<C1, C2>(maps, a, first + j * stride, tiles_x, tiles_y, halo_base + (uint32_t)(j * HALO_BYTES),
                          fbar0 + 8u * j);
  }
  if (!a.const_weights && tid < COUT) sbias[tid] = a.bias ? a.bias[tid] : 0.0f;
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t id = idesc_bf16(kTile, COUT);
  int ok = 1;
  int64_t issued = kStages3 < my_tiles ? kStages3 : my_tiles;  // halos issued (thread 0's count)
  int64_t consumed = 0;                                         // halos waited for (thread 0)
  bool weights = my_tiles == 0;
  for (int64_t k = 0; k <= my_tiles && ok; ++k) {
    if (k < my_tiles && tid == 0) {
      const int st = (int)(k % kStages3);
      if (!weights && mbar_wait(wbar, 0u)) weights = true;
      const bool have = weights && mbar_wait(fbar0 + 8u * st, (uint32_t)((k / kStages3) & 1));
      if (!have) {
        atomicExch(a.err, 1);
        ok = 0;
      } else {
        consumed = k + 1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t halo = halo_base + (uint32_t)(st * HALO_BYTES);
        const uint32_t tacc = tmem + (uint32_t)((k & 1) * COUT);
        // A: leading byte offset = one 8-channel slice, stride byte offset = one halo row
        const uint64_t da0 = smem_desc(halo, kSlice3Bytes, kHx * 16);
        const uint64_t db0 = smem_desc(b0, NG * 128, 128);
#pragma unroll
        for (int t = 0; t < 27; ++t) {
#pragma unroll
          for (int kc = 0; kc < CIN / 16; ++kc) {
            const int s = t * (CIN / 16) + kc;
            const int tap = ((t / 9) * kHy + (t / 3) % 3) * kHx + t % 3;  // halo voxel of output voxel 0
            const uint32_t aoff = (uint32_t)(2 * kc * kSlice3Bytes + tap * 16) >> 4;
            const uint32_t boff = (uint32_t)(2 * s * NG * 128) >> 4;
            mma_bf16(tacc, da0 + aoff, db0 + boff, id, s > 0 ? 1u : 0u);
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         mbar0 + 8u * (uint32_t)(k & 1))
                     : "memory");
      }
    }
    if (k >= 1) {
      const int64_t j = k - 1;
      const int done = mbar_wait(mbar0 + 8u * (uint32_t)(j & 1), (uint32_t)((j >> 1) & 1));
      if (!done) {
        if (tid == 0) atomicExch(a.err, 1);
        ok = 0;
      } else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0 && issued < my_tiles) {
          const int st = (int)(issued % kStages3);
          issue_halo3<C1, C2>(maps, a, first + issued * stride, tiles_x, tiles_y,
                              halo_base + (uint32_t)(st * HALO_BYTES), fbar0 + 8u * st);
          ++issued;
        }
        conv3_epilogue<COUT, EPI>(a, sbias, tmem + (uint32_t)((j & 1) * COUT), first + j * stride, tiles_x, tiles_y,
                                  tid, warp);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  // copies issued but never waited for (only after an error), bounded
  if (tid == 0) {
    for (int64_t j = consumed; j < issued; ++j)
      mbar_wait(fbar0 + 8u * (uint32_t)(j % kStages3), (uint32_t)((j / kStages3) & 1));
    if (!weights) mbar_wait(wbar, 0u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) tmem_free<NCOLS>(tmem);
}

// NDHWC bf16 tensor {C, W, H, D, B} with the halo box {8, 10, 18, 3, 1}
int make_halo_map3(CUtensorMap* m, const void* base, int C, int B, int D, int H, int W) {
  auto fn = encode_fn();
  if (!fn) return AGX_ERR_CUDA;
  if (reinterpret_cast<uintptr_t>(base) & 15u) return AGX_ERR_ARG;
  const cuuint64_t dims[5] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D, (cuuint64_t)B};
  const cuuint64_t strides[4] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2,
                                 (cuuint64_t)D * H * W * C * 2};
  const cuuint32_t box[5] = {8, (cuuint32_t)kHx, (cuuint32_t)kHy, (cuuint32_t)kHz, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? AGX_OK : AGX_ERR_ARG;
}

template <int C1, int C2, int COUT, int EPI>
int launch_conv3(const Conv3Args& a, cudaStream_t s) {
  constexpr int CIN = C1 + C2;
  constexpr int smem = round1k(27 * CIN * COUT * 2) + kStages3 * (CIN / 8) * kSlice3Bytes;
  auto kernel = conv3x3x3_tc<C1, C2, COUT, EPI>;
  static int per_sm = 0;
  if (!per_sm) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
        cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared) != cudaSuccess)
      return AGX_ERR_CUDA;
    int dev = 0, per_sm_smem = 0, reserved = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    per_sm = per_sm_smem / (smem + reserved + 256);
    const int tmem_cap = 512 / tmem_cols(2 * COUT);
    per_sm = per_sm < 1 ? 1 : (per_sm > tmem_cap ? tmem_cap : per_sm);
  }
  Conv3Maps maps{};
  if (int rc = make_halo_map3(&maps.in1, a.in1, C1, a.B, a.D, a.H, a.W)) return rc;
  if (C2 > 0) {
    if (int rc = make_halo_map3(&maps.in2, a.in2, C2, a.B, a.D, a.H, a.W)) return rc;
  } else {
    maps.in2 = maps.in1;
  }
  const int64_t tiles = (int64_t)a.B * a.D * ((a.H + kTy - 1) / kTy) * ((a.W + kTx - 1) / kTx);
  const int64_t cap = (int64_t)per_sm * sm_count();
  const int grid = (int)(tiles < cap ? tiles : cap);
  agx_launch_pdl(kernel, grid, kTile, smem, s, maps, a);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int grid256(int64_t n) {
  int64_t g = (n + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 8;
  return (int)(g < cap ? (g < 1 ? 1 : g) : cap);
}

// ---- f x f x f block transfers (pooling, upsampling and their adjoints) --------------------
// eight channels (16 bytes) per thread, float sums rounded to bf16 once:
//   block_sum3:   coarse = scale * (sum over the f^3 block of fine)   (pooling, adjoint of upsampling)
//   block_bcast3: fine   = scale * coarse of its block                (upsampling, adjoint of pooling)
__device__ __forceinline__ void acc8(const uint4& v, float* a) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const float2 f = __bfloat1622float2(h[u]);
    a[2 * u] += f.x;
    a[2 * u + 1] += f.y;
  }
}

__device__ __forceinline__ uint4 pack8(const float* a, float scale) {
  uint4 v;
  __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&v);
#pragma unroll
  for (int u = 0; u < 4; ++u) h[u] = __floats2bfloat162_rn(scale * a[2 * u], scale * a[2 * u + 1]);
  return v;
}

__global__ void __launch_bounds__(256)
block_sum3_kernel(const uint4* __restrict__ fine, uint4* __restrict__ coarse, int B, int D, int H, int W, int C8,
                  int f, float scale, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  const int Dc = D / f, Hc = H / f, Wc = W / f;
  const int64_t total = (int64_t)B * Dc * Hc * Wc * C8;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C8);
    int64_t q = i / C8;
    const int xc = (int)(q % Wc);
    q /= Wc;
    const int yc = (int)(q % Hc);
    q /= Hc;
    const int zc = (int)(q % Dc);
    const int64_t b = q / Dc;
    float a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int dz = 0; dz < f; ++dz)
      for (int dy = 0; dy < f; ++dy) {
        const int64_t row = ((b * D + (int64_t)zc * f + dz) * H + (int64_t)yc * f + dy) * W + (int64_t)xc * f;
        for (int dx = 0; dx < f; ++dx) acc8(__ldg(fine + (row + dx) * C8 + c), a);
      }
    coarse[i] = pack8(a, scale);
  }
}

__global__ void __launch_bounds__(256)
block_bcast3_kernel(const uint4* __restrict__ coarse, uint4* __restrict__ fine, int B, int D, int H, int W, int C8,
                    int f, float scale, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  const int Dc = D / f, Hc = H / f, Wc = W / f;
  const int64_t total = (int64_t)B * D * H * W * C8;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C8);
    int64_t q = i / C8;
    const int x = (int)(q % W);
    q /= W;
    const int y = (int)(q % H);
    q /= H;
    const int z = (int)(q % D);
    const int64_t b = q / D;
    float a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    acc8(__ldg(coarse + (((b * Dc + z / f) * Hc + y / f) * Wc + x / f) * C8 + c), a);
    fine[i] = pack8(a, scale);
  }
}

// ---- transfers between a brick mesh's node field and the network's coarse grid -----------
// The fine node grid has ((Dc - 1) f + 1) x ((Hc - 1) f + 1) x ((Wc - 1) f + 1) nodes, node
// (i, j, k) at index (i Hf + j) Wf + k; coarse node (I, J, K) sits on fine node (f I, f J, f K).
// P is trilinear interpolation, P^T its transpose (full weighting).  A coarse value whose
// fine node is fixed (Dirichlet) is zero on restriction; a fixed fine node is zero on
// prolongation.
constexpr int kRestrict3Blocks = 1024;  // largest grid of restrict3_kernel (partials it writes)

__global__ void __launch_bounds__(256)
restrict3_kernel(const float* __restrict__ fine, const unsigned char* __restrict__ fixed, int Dc, int Hc, int Wc,
                 int f, float* __restrict__ out, double* __restrict__ partials, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  const int Hf = (Hc - 1) * f + 1, Wf = (Wc - 1) * f + 1, Df = (Dc - 1) * f + 1;
  const int total = Dc * Hc * Wc;
  const float inv = 1.0f / (float)f;
  float sq = 0.0f;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int K = q % Wc, IJ = q / Wc, J = IJ % Hc, I = IJ / Hc;
    const int ci = I * f, cj = J * f, ck = K * f;
    float acc = 0.0f;
    if (!(fixed && fixed[((int64_t)ci * Hf + cj) * Wf + ck])) {
      for (int di = -(f - 1); di <= f - 1; ++di) {
        const int i = ci + di;
        if (i < 0 || i >= Df) continue;
        const float wi = 1.0f - (float)abs(di) * inv;
        float plane = 0.0f;
        for (int dj = -(f - 1); dj <= f - 1; ++dj) {
          const int j = cj + dj;
          if (j < 0 || j >= Hf) continue;
          const float wj = 1.0f - (float)abs(dj) * inv;
          const float* rowp = fine + ((int64_t)i * Hf + j) * Wf;
          float row = 0.0f;
          for (int dk = -(f - 1); dk <= f - 1; ++dk) {
            const int k = ck + dk;
            if (k < 0 || k >= Wf) continue;
            row += (1.0f - (float)abs(dk) * inv) * __ldg(rowp + k);
          }
          plane += wj * row;
        }
        acc += wi * plane;
      }
    }
    out[q] = acc;
    sq += acc * acc;
  }
  if (!partials) return;
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

// every block adds the np partials (fixed order) for 1 / rms, then writes the padded image:
// channel 0 = coarse / rms, channel 1 = 1 inside the coarse grid (the domain indicator), 0 else
__global__ void __launch_bounds__(256)
image3_kernel(const float* __restrict__ rc, const double* __restrict__ partials, int np, int Dc, int Hc, int Wc, int Dp,
              int Hp, int Wp, float* __restrict__ scale, __nv_bfloat16* __restrict__ img, const int* skip) {
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
    const double n = (double)Dc * Hc * Wc;
    const float sc = t > 0.0 ? (float)(1.0 / sqrt(t / n)) : 1.0f;
    s_sh = sc;
    if (blockIdx.x == 0) scale[0] = sc;
  }
  __syncthreads();
  const float s = s_sh;
  const int total = Dp * Hp * Wp;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
    const int k = p % Wp, ij = p / Wp, j = ij % Hp, i = ij / Hp;
    __align__(16) __nv_bfloat16 h[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) h[c] = __float2bfloat16(0.0f);
    if (i < Dc && j < Hc && k < Wc) {
      h[0] = __float2bfloat16(s * rc[((int64_t)i * Hc + j) * Wc + k]);
      h[1] = __float2bfloat16(1.0f);
    }
    uint4* dst = reinterpret_cast<uint4*>(img + (int64_t)p * 16);
    dst[0] = reinterpret_cast<uint4*>(h)[0];
    dst[1] = reinterpret_cast<uint4*>(h)[1];
  }
}

// fine = P (channel 0 of the image, C channels per voxel), zero at fixed nodes
__global__ void __launch_bounds__(256)
prolong3_kernel(const __nv_bfloat16* __restrict__ img, int C, int Dc, int Hc, int Wc, int Hp, int Wp, int f,
                const unsigned char* __restrict__ fixed, float* __restrict__ out, const int* skip) {
  agx_pdl_entry();
  if (nn_skip(skip)) return;
  const int Hf = (Hc - 1) * f + 1, Wf = (Wc - 1) * f + 1, Df = (Dc - 1) * f + 1;
  const int64_t total = (int64_t)Df * Hf * Wf;
  const float inv = 1.0f / (float)f;
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < total; d += (int64_t)gridDim.x * blockDim.x) {
    float v = 0.0f;
    if (!(fixed && fixed[d])) {
      const int k = (int)(d % Wf);
      const int64_t ij = d / Wf;
      const int j = (int)(ij % Hf), i = (int)(ij / Hf);
      const int I = i / f, J = j / f, K = k / f;
      const float ti = (float)(i - I * f) * inv, tj = (float)(j - J * f) * inv, tk = (float)(k - K * f) * inv;
      const int I1 = I + 1 < Dc ? I + 1 : I, J1 = J + 1 < Hc ? J + 1 : J, K1 = K + 1 < Wc ? K + 1 : K;
      auto at = [&](int a, int b, int c) {
        return __bfloat162float(img[(((int64_t)a * Hp + b) * Wp + c) * C]);
      };
      const float c00 = (1.0f - tk) * at(I, J, K) + tk * at(I, J, K1);
      const float c01 = (1.0f - tk) * at(I, J1, K) + tk * at(I, J1, K1);
      const float c10 = (1.0f - tk) * at(I1, J, K) + tk * at(I1, J, K1);
      const float c11 = (1.0f - tk) * at(I1, J1, K) + tk * at(I1, J1, K1);
      v = (1.0f - ti) * ((1.0f - tj) * c00 + tj * c01) + ti * ((1.0f - tj) * c10 + tj * c11);
    }
    out[d] = v;
  }
}

}  // namespace

extern "C" {

int agx_nn_conv3x3x3(const void* in1, const void* in2, int c1, int c2, const void* wpk, const float* bias, void* out1,
                     void* out2, int split, int cout, int relu, int B, int D, int H, int W, int* err, void* stream) {
  if (relu & ~(1 | AGX_NN_CONST_WEIGHTS)) return AGX_ERR_ARG;
  const int const_weights = (relu & AGX_NN_CONST_WEIGHTS) ? 1 : 0;
  relu &= 1;
  if (!in1 || !wpk || !out1 || !err || B <= 0 || D <= 0 || H <= 0 || W <= 0 || (c2 > 0 && !in2)) return AGX_ERR_ARG;
  if (split <= 0 || split > cout || split % 8 || (split < cout && !out2)) return AGX_ERR_ARG;
  if (reinterpret_cast<uintptr_t>(wpk) & 15u) return AGX_ERR_ARG;  // one bulk copy into shared memory
  if ((reinterpret_cast<uintptr_t>(out1) | reinterpret_cast<uintptr_t>(out2)) & 15u) return AGX_ERR_ARG;
  Conv3Args a{(const __nv_bfloat16*)in1, (const __nv_bfloat16*)in2, (const __nv_bfloat16*)wpk, bias,
              (__nv_bfloat16*)out1, (__nv_bfloat16*)out2, split, B, D, H, W, err, const_weights, g_nn_skip};
  cudaStream_t s = (cudaStream_t)stream;
  // forward layers of the 16-channel network; input gradients (relu 0) take the 16 output
  // gradient channels to the layer's 16 or 16 + 16 input channels
  if (c1 == 16 && c2 == 0 && cout == 16) return relu ? launch_conv3<16, 0, 16, 1>(a, s) : launch_conv3<16, 0, 16, 0>(a, s);
  if (c1 == 16 && c2 == 16 && cout == 16 && relu) return launch_conv3<16, 16, 16, 1>(a, s);
  if (c1 == 16 && c2 == 0 && cout == 32 && !relu) return launch_conv3<16, 0, 32, 0>(a, s);
  return AGX_ERR_UNSUPPORTED;
}

int agx_nn_pool3d(const void* in, void* out, int B, int D, int H, int W, int C, int f, int backward, void* stream) {
  if (!in || !out || B <= 0 || f < 1 || f > 16 || D % f || H % f || W % f || C % 8 ||
      ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u))
    return AGX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const float inv = 1.0f / (float)(f * f * f);
  if (!backward) {
    const int g = grid256((int64_t)B * (D / f) * (H / f) * (W / f) * (C / 8));
    agx_launch_pdl(block_sum3_kernel, g, 256, 0, s, (const uint4*)in, (uint4*)out, B, D, H, W, C / 8, f, inv,
                   g_nn_skip);
  } else {  // in: gradient at the pooled size, out: at full size
    const int g = grid256((int64_t)B * D * H * W * (C / 8));
    agx_launch_pdl(block_bcast3_kernel, g, 256, 0, s, (const uint4*)in, (uint4*)out, B, D, H, W, C / 8, f, inv,
                   g_nn_skip);
  }
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_upsample3d(const void* in, void* out, int B, int D, int H, int W, int C, int f, int backward,
                      void* stream) {
  // forward: in (D, H, W) -> out (f D, f H, f W); backward: in (f D, f H, f W) -> out (D, H, W)
  if (!in || !out || B <= 0 || f < 1 || f > 16 || C % 8 ||
      ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u))
    return AGX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int Df = f * D, Hf = f * H, Wf = f * W;
  if (!backward) {
    const int g = grid256((int64_t)B * Df * Hf * Wf * (C / 8));
    agx_launch_pdl(block_bcast3_kernel, g, 256, 0, s, (const uint4*)in, (uint4*)out, B, Df, Hf, Wf, C / 8, f, 1.0f,
                   g_nn_skip);
  } else {
    const int g = grid256((int64_t)B * D * H * W * (C / 8));
    agx_launch_pdl(block_sum3_kernel, g, 256, 0, s, (const uint4*)in, (uint4*)out, B, Df, Hf, Wf, C / 8, f, 1.0f,
                   g_nn_skip);
  }
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_restrict_image3d_work(void) { return kRestrict3Blocks; }

int agx_nn_restrict_image3d(const float* fine, const unsigned char* fixed, int Dc, int Hc, int Wc, int f, int Dp,
                            int Hp, int Wp, float* rc, double* work, float* scale, void* img, void* stream) {
  if (!fine || !rc || !work || !scale || !img || f < 1 || Dc < 2 || Hc < 2 || Wc < 2 || Dp < Dc || Hp < Hc ||
      Wp < Wc || (reinterpret_cast<uintptr_t>(img) & 15u))
    return AGX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nc = (int64_t)Dc * Hc * Wc;
  int g = (int)((nc + 255) / 256);
  g = g < kRestrict3Blocks ? g : kRestrict3Blocks;
  agx_launch_pdl(restrict3_kernel, g, 256, 0, s, fine, fixed, Dc, Hc, Wc, f, rc, work, g_nn_skip);
  agx_launch_pdl(image3_kernel, grid256((int64_t)Dp * Hp * Wp), 256, 0, s, (const float*)rc, (const double*)work, g,
                 Dc, Hc, Wc, Dp, Hp, Wp, scale, (__nv_bfloat16*)img, g_nn_skip);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_restrict3d(const float* fine, const unsigned char* fixed, int Dc, int Hc, int Wc, int f, float* coarse,
                      void* stream) {
  if (!fine || !coarse || f < 1 || Dc < 2 || Hc < 2 || Wc < 2) return AGX_ERR_ARG;
  const int64_t nc = (int64_t)Dc * Hc * Wc;
  int g = (int)((nc + 255) / 256);
  g = g < kRestrict3Blocks ? g : kRestrict3Blocks;
  agx_launch_pdl(restrict3_kernel, g, 256, 0, (cudaStream_t)stream, fine, fixed, Dc, Hc, Wc, f, coarse,
                 (double*)nullptr, g_nn_skip);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

int agx_nn_prolong_image3d(const void* img, int C, int Dc, int Hc, int Wc, int Hp, int Wp, int f,
                           const unsigned char* fixed, float* fine, void* stream) {
  if (!img || !fine || C < 1 || f < 1 || Dc < 2 || Hc < 2 || Wc < 2 || Hp < Hc || Wp < Wc) return AGX_ERR_ARG;
  const int64_t nf = (int64_t)((Dc - 1) * f + 1) * ((Hc - 1) * f + 1) * ((Wc - 1) * f + 1);
  agx_launch_pdl(prolong3_kernel, grid256(nf), 256, 0, (cudaStream_t)stream, (const __nv_bfloat16*)img, C, Dc, Hc, Wc,
                 Hp, Wp, f, fixed, fine, g_nn_skip);
  return cudaGetLastError() == cudaSuccess ? AGX_OK : AGX_ERR_CUDA;
}

}  // extern "C"
