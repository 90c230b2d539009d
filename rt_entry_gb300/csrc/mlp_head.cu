// mlp_head.cu -- the learned head's three layers fused into one persistent
// tcgen05 kernel.
//
// The last layer dominates (N = classes >> H): its 128 x BN3 output tiles
// are split into contiguous ranges, row-block major, one range per CTA (one
// CTA per SM).  For every 128-row block its range touches, a CTA first runs
// the two hidden layers on that block, keeping h1 and then h2 in a 64 KB
// shared-memory A region in the 128-byte-swizzled K-major layout that the
// MMA reads, then sweeps its last-layer tiles over the resident h2:
//   * warp 16 / lane 0 (producer) loads the block's X rows into the A region
//     with TMA once the previous block's MMAs are done with it (`afree`), and
//     streams 64-wide K chunks of W1, W2 and W3 through a 5-stage ring;
//   * warp 17 / lane 0 issues tcgen05.mma (M = 128, K = 16, BF16 inputs, FP32
//     accumulation) into one of two 256-column TMEM accumulators, so that an
//     epilogue overlaps the next job's MMAs;
//   * warps 0-15 drain the accumulators: for a hidden layer they add the bias,
//     apply relu, round to BF16 and write the result into the A region (the
//     next layer's A operand), then signal `hready`; for the last layer they
//     keep a running argmax per row and combine it across CTAs with atomicMax
//     on the packed key.
// Each job's K order and instruction shape along K are those of the
// layer-by-layer GEMMs (gemm_tc.cu), and the hidden activations are rounded
// the same way, so the keys equal theirs.  Every wait is bounded, as in
// gemm_tc.cu: on a timeout the kernel records an error code, raises an abort
// flag the other roles poll, lets its copies land, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>

#include "gemm_tc.h"
#include "mlp_head.h"
#include "tc_common.cuh"

namespace rte {

namespace {

using namespace tc;

constexpr int kBM = 128, kBK = 64;
constexpr int kChunkBytes = kBM * kBK * 2;         // one 128 x 64 chunk of an A operand
constexpr int kAChunks = 4;                        // the A region holds K <= 256
constexpr int kABytes = kAChunks * kChunkBytes;    // 64 KB
constexpr int kStageBytes = 256 * kBK * 2;         // one (<= 256) x 64 chunk of a weight matrix
constexpr int kStages = 5;
constexpr int kAccCols = 256;                      // columns per TMEM accumulator
constexpr int kEpiWarps = 16;
constexpr int kEpiParts = kEpiWarps / 4;           // epilogue warps per TMEM lane quarter
constexpr int kProducerWarp = kEpiWarps, kMmaWarp = kEpiWarps + 1;
constexpr int kThreads = 32 * (kEpiWarps + 2);
constexpr int kSmemBytes = kABytes + kStages * kStageBytes + 1024 /*align*/ + 256 /*barriers*/;

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major,
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__device__ __forceinline__ uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}

template <int BN3>
__global__ void __launch_bounds__(kThreads, 1)
    mlp_head_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmW1,
                    const __grid_constant__ CUtensorMap tmW2, const __grid_constant__ CUtensorMap tmW3,
                    MlpHeadArgs g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* abuf = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* ring = abuf + kABytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(ring + kStages * kStageBytes);
  const uint32_t full0 = smem_u32(bars);                     // full[s]
  const uint32_t empty0 = smem_u32(bars + kStages);          // empty[s]
  const uint32_t tfull0 = smem_u32(bars + 2 * kStages);      // accumulator a ready
  const uint32_t tempty0 = smem_u32(bars + 2 * kStages + 2); // accumulator a drained
  const uint32_t afull = smem_u32(bars + 2 * kStages + 4);   // X rows landed in the A region
  const uint32_t afree = smem_u32(bars + 2 * kStages + 5);   // MMAs done with the A region
  const uint32_t hready = smem_u32(bars + 2 * kStages + 6);  // h1 / h2 written to the A region
  const uint32_t drain = smem_u32(bars + 2 * kStages + 7);   // every MMA issued has completed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 8);
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int H = g.H;
  const int M = g.M_dev ? min(g.M, max(*g.M_dev, 0)) : g.M;  // rows of this launch
  const int nk1 = (g.dp + kBK - 1) / kBK, nkh = H / kBK;
  const int n3 = (g.N + BN3 - 1) / BN3;
  const int m_tiles = (M + kBM - 1) / kBM;
  const long long total = (long long)m_tiles * n3;
  const long long t_begin = total * blockIdx.x / gridDim.x;
  const long long t_end = total * (blockIdx.x + 1) / gridDim.x;
  if (t_begin >= t_end) return;  // uniform over the CTA: nothing initialised yet
  const int rb_first = (int)(t_begin / n3), rb_last = (int)((t_end - 1) / n3);
  // last-layer tiles [lo, hi) of row block rb inside this CTA's range
  auto tile_lo = [&](int rb) { return rb == rb_first ? (int)(t_begin - (long long)rb * n3) : 0; };
  auto tile_hi = [&](int rb) { return rb == rb_last ? (int)(t_end - (long long)rb * n3) : n3; };

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int i = 0; i < kStages; ++i) {
      mbar_init(full0 + 8 * i, 1);
      mbar_init(empty0 + 8 * i, 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(tfull0 + 8 * a, 1);
      mbar_init(tempty0 + 8 * a, kEpiWarps * 32);
    }
    mbar_init(afull, 1);
    mbar_init(afree, 1);
    mbar_init(hready, kEpiWarps * 32);
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(2 * kAccCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  int* abort = &s_abort;

  if (warp == kProducerWarp) {
    if (lane == 0) {
      int issued = 0;
      bool ok = true;
      // one weight chunk into the next ring stage
      auto push = [&](const CUtensorMap* map, int x, int y, uint32_t bytes) -> bool {
        const int s = issued % kStages, r = issued / kStages;
        if (issued >= kStages && !mbar_wait(empty0 + 8 * s, (r - 1) & 1, g.err, 11, abort, g.wait_limit)) return false;
        if (*(volatile int*)abort) return false;
        mbar_expect_tx(full0 + 8 * s, bytes);
        tma_load_2d(smem_u32(ring + s * kStageBytes), map, x, y, full0 + 8 * s);
        ++issued;
        return true;
      };
      const uint32_t hbytes = (uint32_t)H * kBK * 2, w3bytes = (uint32_t)BN3 * kBK * 2;
      for (int rb = rb_first; rb <= rb_last && ok; ++rb) {
        const int rbi = rb - rb_first;
        if (rbi > 0 && !mbar_wait(afree, (rbi - 1) & 1, g.err, 12, abort, g.wait_limit)) {
          ok = false;
          break;
        }
        mbar_expect_tx(afull, (uint32_t)(nk1 * kChunkBytes));
        for (int kc = 0; kc < nk1; ++kc)
          tma_load_2d(smem_u32(abuf + kc * kChunkBytes), &tmX, kc * kBK, rb * kBM, afull);
        for (int kc = 0; kc < nk1 && ok; ++kc) ok = push(&tmW1, kc * kBK, 0, hbytes);
        for (int kc = 0; kc < nkh && ok; ++kc) ok = push(&tmW2, kc * kBK, 0, hbytes);
        for (int nt = tile_lo(rb); nt < tile_hi(rb) && ok; ++nt)
          for (int kc = 0; kc < nkh && ok; ++kc) ok = push(&tmW3, kc * kBK, nt * BN3, w3bytes);
        // the A region's copies land before it can be reused or the CTA exits
        if (!mbar_wait(afull, rbi & 1, g.err, 13, ok ? nullptr : abort)) ok = false;
      }
      if (!ok) *(volatile int*)abort = 1;
      // let every weight copy in flight land before the CTA can exit
      for (int i = (issued > kStages ? issued - kStages : 0); i < issued; ++i)
        mbar_wait(full0 + 8 * (i % kStages), (i / kStages) & 1, g.err, 14);
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0) {
      bool ok = true;
      int used = 0, t = 0, hw = 0;
      // one job: nk chunks of K into accumulator t & 1
      auto job = [&](int nk, uint32_t idesc) -> bool {
        const int a = t & 1;
        if (t >= 2 && !mbar_wait(tempty0 + 8 * a, ((t >> 1) - 1) & 1, g.err, 15, abort, g.wait_limit)) return false;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + (uint32_t)(a * kAccCols);
        for (int kc = 0; kc < nk; ++kc, ++used) {
          const int s = used % kStages, r = used / kStages;
          if (!mbar_wait(full0 + 8 * s, r & 1, g.err, 16, abort, g.wait_limit)) return false;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint64_t ad = sw128_desc(smem_u32(abuf + kc * kChunkBytes));
          const uint64_t bd = sw128_desc(smem_u32(ring + s * kStageBytes));
#pragma unroll
          for (int kk = 0; kk < kBK / 16; ++kk)  // +32 bytes per K = 16 step inside the swizzle atom
            mma_bf16(d, ad + (uint64_t)(2 * kk), bd + (uint64_t)(2 * kk), idesc, (kc | kk) != 0);
          mma_commit(empty0 + 8 * s);
        }
        mma_commit(tfull0 + 8 * a);
        ++t;
        return true;
      };
      auto wait_h = [&]() -> bool {
        if (!mbar_wait(hready, hw & 1, g.err, 17, abort, g.wait_limit)) return false;
        ++hw;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        return true;
      };
      for (int rb = rb_first; rb <= rb_last && ok; ++rb) {
        const int rbi = rb - rb_first;
        ok = mbar_wait(afull, rbi & 1, g.err, 18, abort, g.wait_limit);
        if (ok) ok = job(nk1, idesc_bf16(H));               // layer 1 on X
        if (ok) ok = wait_h();                               // h1 in the A region
        if (ok) ok = job(nkh, idesc_bf16(H));               // layer 2 on h1
        if (ok) ok = wait_h();                               // h2 in the A region
        for (int nt = tile_lo(rb); nt < tile_hi(rb) && ok; ++nt) ok = job(nkh, idesc_bf16(BN3));
        if (ok) mma_commit(afree);  // arrives once the MMAs reading the A region are done
      }
      if (!ok) *(volatile int*)abort = 1;
      // no MMA may still run when TMEM is freed, whatever path led here
      mma_commit(drain);
      mbar_wait(drain, 0, g.err, 20);
    }
  } else {
    // epilogue: warp w owns TMEM lanes (rows) 32q .. 32q+31, q = w % 4, and
    // the 32-column chunks part, part + kEpiParts, ... of the job's columns,
    // part = w / 4 (increasing column order within a thread)
    const int quarter = warp & 3, part = warp >> 2;
    const int row_l = quarter * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
    int t = 0;
    bool ok = true;
    auto wait_full = [&]() -> bool {
      const int a = t & 1;
      const bool w = __all_sync(0xffffffffu, mbar_wait(tfull0 + 8 * a, (t >> 1) & 1, g.err, 19, abort, g.wait_limit));
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      return w;
    };
    auto load_bias = [&](const float* bias, int col, int n, float (&bv)[32]) {
      if (((uintptr_t)bias & 15) == 0 && col + 31 < n) {
#pragma unroll
        for (int i = 0; i < 32; i += 4) {
          const float4 b4 = __ldg(reinterpret_cast<const float4*>(bias + col + i));
          bv[i] = b4.x;
          bv[i + 1] = b4.y;
          bv[i + 2] = b4.z;
          bv[i + 3] = b4.w;
        }
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) bv[i] = col + i < n ? __ldg(bias + col + i) : 0.f;
      }
    };
    // a hidden layer's accumulator -> relu(acc + bias) in BF16, into the A
    // region: column c of row r goes to chunk c / 64, 16-byte unit
    // ((c % 64) / 8) ^ (r % 8) of the row's 128 bytes (the TMA swizzle)
    auto hidden = [&](const float* bias) -> bool {
      if (!wait_full()) return false;
      const int a = t & 1;
      const int nch = H / 32;
      if (part >= nch) {  // no chunk for this warp: the accumulator is not its to read
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        mbar_arrive(tempty0 + 8 * a);
      }
      for (int ch = part; ch < nch; ch += kEpiParts) {
        const int c = ch * 32;
        uint32_t r[32];
        tmem_ld32(lane_base + (uint32_t)(a * kAccCols + c), r);
        float bv[32];
        load_bias(bias, c, H, bv);
        tmem_wait_ld();
        if (ch + kEpiParts >= nch) {  // accumulator drained: hand it back to the MMA issuer
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          mbar_arrive(tempty0 + 8 * a);
        }
        uint32_t pk[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          float x0 = __uint_as_float(r[2 * i]) + bv[2 * i];
          float x1 = __uint_as_float(r[2 * i + 1]) + bv[2 * i + 1];
          x0 = x0 > 0.f ? x0 : 0.f;
          x1 = x1 > 0.f ? x1 : 0.f;
          __nv_bfloat162 p = __floats2bfloat162_rn(x0, x1);
          pk[i] = *reinterpret_cast<uint32_t*>(&p);
        }
        uint8_t* rowp = abuf + (c / kBK) * kChunkBytes + row_l * 128;
        const int u0 = (c % kBK) / 8;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int phys = (u0 + u) ^ (row_l & 7);
          *reinterpret_cast<uint4*>(rowp + phys * 16) = make_uint4(pk[4 * u], pk[4 * u + 1], pk[4 * u + 2], pk[4 * u + 3]);
        }
      }
      // generic-proxy writes become visible to the tensor core's reads
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(hready);
      ++t;
      return true;
    };
    // four running maxima (columns i % 4); each keeps its first maximum and
    // the merge prefers the smaller column on equal values
    float best[4];
    int best_col[4];
    auto reset_best = [&]() {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        best[j] = -3.402823466e38f;
        best_col[j] = -1;
      }
    };
    auto flush_best = [&](int row) {
      float bb = best[0];
      int bc = best_col[0];
#pragma unroll
      for (int j = 1; j < 4; ++j)
        if (best_col[j] >= 0 && (bc < 0 || best[j] > bb || (best[j] == bb && best_col[j] < bc))) {
          bb = best[j];
          bc = best_col[j];
        }
      if (row < M && bc >= 0) atomicMax(g.keys + row, argmax_key(bb, bc));
    };
    auto last = [&](int nt) -> bool {
      if (!wait_full()) return false;
      const int a = t & 1;
      constexpr int nch = BN3 / 32;
      static_assert(nch % kEpiParts == 0, "every epilogue warp reads the same number of chunks");
      const bool full_cols = nt * BN3 + BN3 <= g.N;
#pragma unroll 1
      for (int ch = part; ch < nch; ch += kEpiParts) {
        const int n0 = nt * BN3 + ch * 32;
        uint32_t r[32];
        tmem_ld32(lane_base + (uint32_t)(a * kAccCols + ch * 32), r);
        float bv[32];
        load_bias(g.b3, n0, g.N, bv);
        tmem_wait_ld();
        if (ch + kEpiParts >= nch) {
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          mbar_arrive(tempty0 + 8 * a);
        }
        if (full_cols) {
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const float x = __uint_as_float(r[i]) + bv[i];
            if (x > best[i & 3]) {
              best[i & 3] = x;
              best_col[i & 3] = n0 + i;
            }
          }
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int col = n0 + i;
            const float x = col < g.N ? __uint_as_float(r[i]) + bv[i] : -3.402823466e38f;
            if (x > best[i & 3]) {
              best[i & 3] = x;
              best_col[i & 3] = col;
            }
          }
        }
      }
      ++t;
      return true;
    };
    for (int rb = rb_first; rb <= rb_last && ok; ++rb) {
      ok = hidden(g.b1);
      if (ok) ok = hidden(g.b2);
      reset_best();
      for (int nt = tile_lo(rb); nt < tile_hi(rb) && ok; ++nt) ok = last(nt);
      if (ok) flush_best(rb * kBM + row_l);
    }
    if (!ok) *(volatile int*)abort = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kAccCols));
  }
}

}  // namespace

bool mlp_head_supported(const MlpHeadArgs& a) {
  return a.M > 0 && a.N > 0 && a.H > 0 && a.H % kBK == 0 && a.H <= kAChunks * kBK && a.dp > 0 &&
         a.dp % 8 == 0 && a.dp <= kAChunks * kBK && a.X && a.W1 && a.W2 && a.W3 && a.b1 && a.b2 &&
         a.b3 && a.keys && ((uintptr_t)a.X & 15) == 0 && ((uintptr_t)a.W1 & 15) == 0 &&
         ((uintptr_t)a.W2 & 15) == 0 && ((uintptr_t)a.W3 & 15) == 0;
}

namespace {
// per-device caches, set once; concurrent host threads may race to set them,
// which is harmless (the same values), hence atomics
std::atomic<int> g_num_sms[64];
std::atomic<bool> g_attr[2][64];
}  // namespace

cudaError_t mlp_head_prepare(int N) {
  const bool wide = N >= 256;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!g_attr[wide][dev].load(std::memory_order_acquire)) {
    cudaError_t e = wide ? cudaFuncSetAttribute(mlp_head_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                kSmemBytes)
                         : cudaFuncSetAttribute(mlp_head_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                kSmemBytes);
    if (e != cudaSuccess) return e;
    g_attr[wide][dev].store(true, std::memory_order_release);
  }
  if (g_num_sms[dev].load(std::memory_order_relaxed) == 0) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
    g_num_sms[dev].store(sms, std::memory_order_relaxed);
  }
  return cudaSuccess;
}

cudaError_t mlp_head_argmax(const MlpHeadArgs& a, cudaStream_t st) {
  if (!mlp_head_supported(a)) return cudaErrorNotSupported;
  const bool wide = a.N >= 256;
  const int bn3 = wide ? 256 : 128;
  CUtensorMap mx, m1, m2, m3;
  if (!make_map_bf16(&mx, a.X, a.M, a.dp, kBK, kBM) || !make_map_bf16(&m1, a.W1, a.H, a.dp, kBK, a.H) ||
      !make_map_bf16(&m2, a.W2, a.H, a.H, kBK, a.H) || !make_map_bf16(&m3, a.W3, a.N, a.H, kBK, bn3))
    return cudaErrorNotSupported;
  cudaError_t pe = mlp_head_prepare(a.N);
  if (pe != cudaSuccess) return pe;
  int dev = 0;
  cudaGetDevice(&dev);
  const int sms = g_num_sms[dev].load(std::memory_order_relaxed);
  const long long tiles = (long long)((a.M + kBM - 1) / kBM) * ((a.N + bn3 - 1) / bn3);
  const dim3 grid((unsigned)(tiles < sms ? tiles : sms));
  MlpHeadArgs ha = a;
  ha.wait_limit = wait_limit();
  if (wide)
    mlp_head_kernel<256><<<grid, kThreads, kSmemBytes, st>>>(mx, m1, m2, m3, ha);
  else
    mlp_head_kernel<128><<<grid, kThreads, kSmemBytes, st>>>(mx, m1, m2, m3, ha);
  return cudaGetLastError();
}

}  // namespace rte
