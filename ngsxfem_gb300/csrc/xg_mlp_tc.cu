// Inference of the learned-quadrature MLP (10 -> 256 -> 256 -> 24, SiLU) on
// the fifth-generation tensor cores of sm_103a, all three layers fused per
// tile of 128 rows so that the activations never leave the SM.
//
// No counterpart in the reference (the learned rule replaces its
// isoparametric workflow; see xg_learn.cu).
//
// Per CTA (persistent, one per SM, 256 threads):
//   shared memory   the three weight matrices, transposed to N x K (K
//                   contiguous) and stored as the no-swizzle K-major
//                   canonical layout of 8 x 16-byte core matrices (packed
//                   once per parameter update by k_tc_pack), the input tile
//                   (128 x 16, features 10..15 zero) and one activation tile
//                   (128 x 256) reused by both hidden layers: 220 KiB;
//   tensor memory   512 columns: layer 1 and 2 accumulators (128 x 256 FP32)
//                   in columns 0..255, layer 3 (128 x 32) in 256..287;
//   per tile        one thread issues the MMAs of a layer (tcgen05.mma
//                   kind::f16, BF16 x BF16 -> FP32, M = 128, K = 16 per
//                   instruction) and commits them to an mbarrier; the eight
//                   warps read the accumulators back (tcgen05.ld 32x32b, warp
//                   w reads lanes 32 (w mod 4) .. + 31, warps 0-3 the first
//                   half of the columns, 4-7 the second), add the bias,
//                   apply SiLU, round to BF16 and write the next layer's A
//                   operand; layer 3's output (+ bias) goes to global memory.
// Every wait on an mbarrier gives up after a bounded number of polls: the
// kernel then records XG_ERR_TIMEOUT, stops issuing work, frees its tensor
// memory and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>

#include "xg_internal.h"

namespace xg {

constexpr int kTcIn = 10, kTcHid = 256, kTcOut = 24;
constexpr int kTcM = 128;  // rows per tile
// byte sizes of the shared operand images
constexpr int kTcX = kTcM * 16 * 2;       // input tile 128 x 16
constexpr int kTcW1 = kTcHid * 16 * 2;    // W1^T 256 x 16
constexpr int kTcW2 = kTcHid * kTcHid * 2;  // W2^T 256 x 256
constexpr int kTcW3 = 32 * kTcHid * 2;    // W3^T 32 x 256 (rows 24..31 zero)
constexpr int kTcH = kTcM * kTcHid * 2;   // activation tile 128 x 256
constexpr int kTcPacked = kTcW1 + kTcW2 + kTcW3;  // bytes of the packed weights
constexpr int kTcSmem = kTcX + kTcPacked + kTcH;
extern const int kTcPackedBytes = kTcPacked;

namespace {

// element (r, k) of an R x K operand in the no-swizzle K-major layout:
// core matrix (r / 8, k / 8) of 8 rows x 16 bytes at ((r / 8) * K / 8 + k / 8)
// * 128 bytes, row r % 8 at 16 bytes each, element k % 8 at 2 bytes each.
// Core matrices adjacent in K are 128 bytes apart (leading byte offset),
// adjacent 8-row groups K / 8 * 128 bytes (stride byte offset).
__host__ __device__ constexpr int tc_off(int r, int k, int K) {
  return ((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// weights (FP32 masters, [K][N] row-major like the SIMT path) -> BF16 images
__global__ void k_tc_pack(const float* __restrict__ p, int64_t off_w1, int64_t off_w2, int64_t off_w3,
                          unsigned char* __restrict__ out) {
  const int n1 = kTcHid * 16, n2 = kTcHid * kTcHid, n3 = 32 * kTcHid;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n1 + n2 + n3; t += gridDim.x * blockDim.x) {
    float v = 0.f;
    int byte;
    if (t < n1) {  // W1^T: row n (output), column k (input)
      const int n = t / 16, k = t % 16;
      if (k < kTcIn) v = p[off_w1 + (int64_t)k * kTcHid + n];
      byte = tc_off(n, k, 16);
    } else if (t < n1 + n2) {
      const int u = t - n1, n = u / kTcHid, k = u % kTcHid;
      v = p[off_w2 + (int64_t)k * kTcHid + n];
      byte = kTcW1 + tc_off(n, k, kTcHid);
    } else {
      const int u = t - n1 - n2, n = u / kTcHid, k = u % kTcHid;
      if (n < kTcOut) v = p[off_w3 + (int64_t)k * kTcOut + n];
      byte = kTcW1 + kTcW2 + tc_off(n, k, kTcHid);
    }
    *reinterpret_cast<__nv_bfloat16*>(out + byte) = __float2bfloat16_rn(v);
  }
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading (K) and stride
// (8-row group) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

// bounded wait for the phase of an mbarrier; false on time-out
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t phase) {
  const uint32_t a = smem_u32(mbar);
  for (int it = 0; it < (1 << 22); it++) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 32 consecutive accumulator columns of this thread's row into r (no wait)
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  tmem_ld32_nowait(taddr, r);
  tmem_wait_ld();
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// SiLU with the fast reciprocal division (the result is rounded to BF16)
__device__ __forceinline__ float silu_tc(float z) { return __fdividef(z, 1.f + __expf(-z)); }

// 64 accumulator columns of one row (two loads, one wait) -> bias, SiLU,
// BF16 -> the activation tile
__device__ __forceinline__ void epilogue_hidden(uint32_t taddr, const float* bias, int c0, int row,
                                                unsigned char* H) {
  uint32_t r[64];
  tmem_ld32_nowait(taddr, r);
  tmem_ld32_nowait(taddr + 32u, r + 32);
  tmem_wait_ld();
#pragma unroll
  for (int g = 0; g < 8; g++) {
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int c = g * 8 + 2 * q;
      const __nv_bfloat162 h = __floats2bfloat162_rn(silu_tc(__uint_as_float(r[c]) + bias[c0 + c]),
                                                     silu_tc(__uint_as_float(r[c + 1]) + bias[c0 + c + 1]));
      w[q] = *reinterpret_cast<const uint32_t*>(&h);
    }
    *reinterpret_cast<uint4*>(H + tc_off(row, c0 + g * 8, kTcHid)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__global__ void __launch_bounds__(256, 1) k_mlp_tc(const float* __restrict__ x, int64_t B,
                                                    const uint4* __restrict__ packed, const float* __restrict__ b1,
                                                    const float* __restrict__ b2, const float* __restrict__ b3,
                                                    float* __restrict__ y, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm_tc[];
  unsigned char* X = sm_tc;
  unsigned char* W1 = X + kTcX;
  unsigned char* W2 = W1 + kTcW1;
  unsigned char* W3 = W2 + kTcW2;
  unsigned char* H = W3 + kTcW3;
  __shared__ float s_b1[kTcHid], s_b2[kTcHid], s_b3[32];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // weights and biases, once per CTA
  for (int i = tid; i < kTcPacked / 16; i += 256) reinterpret_cast<uint4*>(W1)[i] = packed[i];
  for (int i = tid; i < kTcHid; i += 256) {
    s_b1[i] = b1[i];
    s_b2[i] = b2[i];
  }
  if (tid < 32) s_b3[tid] = tid < kTcOut ? b3[tid] : 0.f;
  if (tid == 0) {
    abort_s = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tm = tmem_base;
  const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;  // TMEM lanes of this warp
  const int row_l = 32 * (warp & 3) + lane;                       // tile row of this thread
  const int half = warp >> 2;                                     // column half of this warp
  const uint32_t idesc_h = idesc_bf16(kTcM, kTcHid), idesc_o = idesc_bf16(kTcM, 32);
  const uint32_t aX = smem_u32(X), aW1 = smem_u32(W1), aW2 = smem_u32(W2), aW3 = smem_u32(W3), aH = smem_u32(H);
  uint32_t phase = 0;
  const int64_t ntiles = (B + kTcM - 1) / kTcM;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t r0 = tile * kTcM;
    // input tile: BF16 features, columns 10..15 zero
    if (tid < kTcM) {
      const int64_t r = r0 + tid;
      float f[16];
#pragma unroll
      for (int k = 0; k < 16; k++) f[k] = (k < kTcIn && r < B) ? x[r * kTcIn + k] : 0.f;
#pragma unroll
      for (int g = 0; g < 2; g++) {
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const __nv_bfloat162 h = __floats2bfloat162_rn(f[g * 8 + 2 * q], f[g * 8 + 2 * q + 1]);
          w[q] = *reinterpret_cast<const uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(X + tc_off(tid, g * 8, 16)) = make_uint4(w[0], w[1], w[2], w[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // layer 1: D[0..255] = X W1 (one K step)
    if (tid == 0) {
      mma_bf16(tm, sdesc(aX, 128, 256), sdesc(aW1, 128, 256), idesc_h, 0);
      mma_commit(&mbar);
    }
    if (!mbar_wait(&mbar, phase)) abort_s = 1;
    phase ^= 1;
    __syncthreads();  // every thread sees the same abort flag
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (abort_s) break;
    for (int cc = 0; cc < 2; cc++) {
      const int c0 = half * 128 + cc * 64;
      epilogue_hidden(tm + lane_base + (uint32_t)c0, s_b1, c0, row_l, H);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // layer 2: D[0..255] = H1 W2 (16 K steps of 16)
    if (tid == 0) {
      for (int k = 0; k < kTcHid / 16; k++)
        mma_bf16(tm, sdesc(aH + k * 256, 128, 4096), sdesc(aW2 + k * 256, 128, 4096), idesc_h, k > 0);
      mma_commit(&mbar);
    }
    if (!mbar_wait(&mbar, phase)) abort_s = 1;
    phase ^= 1;
    __syncthreads();  // every thread sees the same abort flag
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (abort_s) break;
    for (int cc = 0; cc < 2; cc++) {
      const int c0 = half * 128 + cc * 64;
      epilogue_hidden(tm + lane_base + (uint32_t)c0, s_b2, c0, row_l, H);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // layer 3: D[256..287] = H2 W3
    if (tid == 0) {
      for (int k = 0; k < kTcHid / 16; k++)
        mma_bf16(tm + 256, sdesc(aH + k * 256, 128, 4096), sdesc(aW3 + k * 256, 128, 4096), idesc_o, k > 0);
      mma_commit(&mbar);
    }
    if (!mbar_wait(&mbar, phase)) abort_s = 1;
    phase ^= 1;
    __syncthreads();  // every thread sees the same abort flag
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (abort_s) break;
    if (half == 0) {
      float v[32];
      tmem_ld32(tm + lane_base + 256u, v);
      const int64_t r = r0 + row_l;
      if (r < B) {
#pragma unroll
        for (int j = 0; j < kTcOut; j++) y[r * kTcOut + j] = v[j] + s_b3[j];
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  if (abort_s && tid == 0) {
    set_err(err, XG_ERR_TIMEOUT);
    // the tensor-core work already issued: one more bounded wait before the
    // tensor memory is released
    mma_commit(&mbar);
    mbar_wait(&mbar, phase);
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tm));
}

}  // namespace

int mlp_tc_pack(const float* d_params, int64_t off_w1, int64_t off_w2, int64_t off_w3, void* d_packed,
                cudaStream_t s) {
  k_tc_pack<<<152, 256, 0, s>>>(d_params, off_w1, off_w2, off_w3, (unsigned char*)d_packed);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_tc_pack");
}

int mlp_tc_forward(const float* d_x, int64_t B, const void* d_packed, const float* d_b1, const float* d_b2,
                   const float* d_b3, float* d_y, int* d_err, cudaStream_t s) {
  if (B <= 0) return XG_OK;
  static int grid = 0;
  if (!grid) {
    XG_CUDA(cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    int dev = 0;
    XG_CUDA(cudaGetDevice(&dev));
    XG_CUDA(cudaDeviceGetAttribute(&grid, cudaDevAttrMultiProcessorCount, dev));
  }
  const int64_t ntiles = (B + kTcM - 1) / kTcM;
  const int g = (int)std::min<int64_t>(ntiles, grid);
  k_mlp_tc<<<g, 256, kTcSmem, s>>>(d_x, B, (const uint4*)d_packed, d_b1, d_b2, d_b3, d_y, d_err);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? XG_OK : cuda_fail(e, "k_mlp_tc");
}

}  // namespace xg
