// gemm_tc.cu -- BF16 x BF16 -> FP32 GEMM on the 5th-generation tensor cores.
//
// One CTA of 4 warps computes a 128 x 128 output tile:
//   * warp 0 / lane 0 streams 128 x 64 tiles of A and B into shared memory
//     with TMA (cp.async.bulk.tensor, 128-byte swizzle) through a 4-stage
//     ring guarded by mbarriers;
//   * warp 1 / lane 0 issues tcgen05.mma (M=128, N=128, K=16, BF16 inputs,
//     FP32 accumulation) into a 128-column TMEM accumulator and releases
//     each ring slot with tcgen05.commit;
//   * all four warps then read their 32 accumulator rows with tcgen05.ld and
//     apply the fused epilogue.
// Every mbarrier wait is bounded: when one runs out the kernel records an
// error code in *err, stops issuing work, lets the copies already in flight
// land, frees its TMEM and returns, so a fault in the pipeline cannot hang
// the GPU.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "gemm_tc.h"

namespace rte {

namespace {

constexpr int BM = 128, BN = 128, BK = 64, STAGES = 4;
constexpr int A_BYTES = BM * BK * 2;
constexpr int B_BYTES = BN * BK * 2;
constexpr int SMEM_BYTES = STAGES * (A_BYTES + B_BYTES) + 1024 /*align*/ + 256 /*barriers*/;
constexpr long long kWaitLimit = 1ll << 24;  // try_wait rounds before giving up (~seconds)

// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), leading byte offset unused (1),
// descriptor version 1 (bits 46-47), layout type 2 = SWIZZLE_128B (61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; returns false (and records `code`) when the limit runs out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, int code) {
  for (long long i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  if (err) atomicCAS(err, 0, code);
  return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(128, 1)
    gemm_bf16_tn_kernel(const __grid_constant__ CUtensorMap tmA,
                        const __grid_constant__ CUtensorMap tmB, GemmArgs g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * A_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + STAGES * B_BYTES);
  const uint32_t full0 = smem_u32(bars);             // full[s]  = bars[s]
  const uint32_t empty0 = smem_u32(bars + STAGES);   // empty[s] = bars[STAGES + s]
  const uint32_t done = smem_u32(bars + 2 * STAGES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int nk = (g.K + BK - 1) / BK;

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer: TMA ring
    int issued = 0;
    for (int kt = 0; kt < nk; ++kt) {
      const int s = kt % STAGES, r = kt / STAGES;
      if (kt >= STAGES && !mbar_wait(empty0 + 8 * s, (r - 1) & 1, g.err, 1)) break;
      if (*(volatile int*)&s_abort) break;
      mbar_expect_tx(full0 + 8 * s, A_BYTES + B_BYTES);
      tma_load_2d(smem_u32(sA + s * A_BYTES), &tmA, kt * BK, m0, full0 + 8 * s);
      tma_load_2d(smem_u32(sB + s * B_BYTES), &tmB, kt * BK, n0, full0 + 8 * s);
      issued = kt + 1;
    }
    // let every copy in flight land before the CTA can exit
    for (int kt = (issued > STAGES ? issued - STAGES : 0); kt < issued; ++kt)
      mbar_wait(full0 + 8 * (kt % STAGES), (kt / STAGES) & 1, g.err, 2);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    bool ok = true;
    for (int kt = 0; kt < nk && ok; ++kt) {
      const int s = kt % STAGES, r = kt / STAGES;
      if (!mbar_wait(full0 + 8 * s, r & 1, g.err, 3)) {
        ok = false;
        *(volatile int*)&s_abort = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t ad = sw128_desc(smem_u32(sA + s * A_BYTES));
      const uint64_t bd = sw128_desc(smem_u32(sB + s * B_BYTES));
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk)  // +32 bytes per K=16 step inside the swizzle atom
        mma_bf16(tmem, ad + (uint64_t)(2 * kk), bd + (uint64_t)(2 * kk), (kt | kk) != 0);
      mma_commit(empty0 + 8 * s);
    }
    mma_commit(done);
  }
  __syncwarp();

  // epilogue: warp w owns accumulator rows 32w .. 32w+31 (TMEM lanes)
  // tcgen05.ld is warp-collective: the whole warp decides together
  const bool ok = __all_sync(0xffffffffu, mbar_wait(done, 0, g.err, 4) && !*(volatile int*)&s_abort);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int row = m0 + warp * 32 + lane;
  float best = -3.402823466e38f;
  int best_col = 0;
  if (ok) {
    for (int c0 = 0; c0 < BN; c0 += 8) {
      float v[8];
      tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (row >= g.M) continue;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int col = n0 + c0 + i;
        if (col >= g.N) continue;
        float x = v[i];
        switch (g.epilogue) {
          case kEpiStoreF32:
            reinterpret_cast<float*>(g.C)[(size_t)row * g.ldc + col] = x;
            break;
          case kEpiAccumF32:
            reinterpret_cast<float*>(g.C)[(size_t)row * g.ldc + col] += x;
            break;
          case kEpiBiasF32:
            reinterpret_cast<float*>(g.C)[(size_t)row * g.ldc + col] = x + g.bias[col];
            break;
          case kEpiBiasReluBF16:
            x += g.bias[col];
            reinterpret_cast<__nv_bfloat16*>(g.C)[(size_t)row * g.ldc + col] =
                __float2bfloat16_rn(x > 0.f ? x : 0.f);
            break;
          case kEpiBiasArgmax:
            x += g.bias[col];
            if (x > best) {
              best = x;
              best_col = col;
            }
            break;
        }
      }
    }
    if (g.epilogue == kEpiBiasArgmax && row < g.M && best_col < g.N)
      atomicMax(g.out_argmax + row, argmax_key(best, best_col));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
  }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point, so the
// library needs no link-time dependency on libcuda.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encoder() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

bool make_map(CUtensorMap* m, const void* base, int rows, int K, int box_rows) {
  EncodeTiledFn enc = encoder();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

cudaError_t gemm_bf16_tn(const GemmArgs& g, cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0 || g.K <= 0 || (g.K & 7) || !g.A || !g.B) return cudaErrorInvalidValue;
  if (((uintptr_t)g.A & 15) || ((uintptr_t)g.B & 15)) return cudaErrorInvalidValue;
  if (g.epilogue != kEpiBiasArgmax && !g.C) return cudaErrorInvalidValue;
  if ((g.epilogue == kEpiBiasArgmax && !g.out_argmax) ||
      ((g.epilogue == kEpiBiasArgmax || g.epilogue == kEpiBiasF32 ||
        g.epilogue == kEpiBiasReluBF16) && !g.bias))
    return cudaErrorInvalidValue;
  CUtensorMap ma, mb;
  if (!make_map(&ma, g.A, g.M, g.K, BM) || !make_map(&mb, g.B, g.N, g.K, BN))
    return cudaErrorNotSupported;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(gemm_bf16_tn_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM);
  gemm_bf16_tn_kernel<<<grid, 128, SMEM_BYTES, st>>>(ma, mb, g);
  return cudaGetLastError();
}

}  // namespace rte
