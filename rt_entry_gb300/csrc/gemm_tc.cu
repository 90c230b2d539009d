// gemm_tc.cu -- BF16 x BF16 -> FP32 GEMM on the 5th-generation tensor cores.
//
// A persistent grid (one CTA of 10 warps per SM) splits the 128 x 128 output
// tiles into contiguous ranges, row-block major:
//   * warp 8 / lane 0 streams 128 x 64 tiles into shared memory with TMA
//     (cp.async.bulk.tensor, 128-byte swizzle) through an mbarrier ring.
//     When K <= 256 the A block is loaded once per row block and stays
//     resident while 7 stages of B tiles stream; otherwise 5 stages carry
//     both;
//   * warp 9 / lane 0 issues tcgen05.mma (M=128, N=128, K=16, BF16 inputs,
//     FP32 accumulation) into one of two 128-column TMEM accumulators, so the
//     next tile's MMAs overlap the epilogue of the previous one;
//   * warps 0-7 (two per TMEM lane quarter, each on half of the columns)
//     read the accumulator with wide tcgen05.ld, hand it back, and apply the
//     fused epilogue: a running argmax kept in registers across tiles, or
//     stores staged through shared memory so each warp writes 128-byte row
//     segments (coalesced).
// Every mbarrier wait is bounded: when one runs out the kernel records an
// error code in *err, raises an abort flag the other roles poll, lets the
// copies already in flight land, frees its TMEM and returns, so a fault in
// the pipeline cannot hang the GPU.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "gemm_tc.h"
#include "tc_common.cuh"

namespace rte {

namespace {

using namespace tc;

constexpr int BM = 128, BK = 64;
constexpr int A_BYTES = BM * BK * 2;  // one 128 x 64 chunk of A
constexpr int RING_BYTES = 11 * A_BYTES;
constexpr int kResidentChunks = 4;
constexpr int kResidentK = kResidentChunks * BK;
constexpr int kMaxStages = 7;
constexpr int kChunk = 32;                // accumulator columns per TMEM load
constexpr int kStageLd = kChunk + 4;      // staging row pitch (floats): conflict-free v4 access
constexpr int kEpiWarps = 8;             // two per TMEM lane quarter, one per column half

// Output tiles are 128 x BN, BN = 128 or 256 (one MMA instruction covers the
// whole tile width).  Resident A (K <= 256): 4 A chunks + 7 (BN = 128) or 3
// (BN = 256) B stages; streamed: 5 or 3 stages of A + B.  Two accumulators
// of BN columns each: 256 or all 512 TMEM columns.
template <int BN_>
struct Tile {
  static constexpr int BN = BN_;
  static constexpr int B_BYTES = BN * BK * 2;  // one BN x 64 chunk of B
  static constexpr int kStagesResident = (RING_BYTES - kResidentChunks * A_BYTES) / B_BYTES;
  static constexpr int kStagesStreamed = RING_BYTES / (A_BYTES + B_BYTES);
  static constexpr int kHalf = BN / 2;           // columns per epilogue warp
  // Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
  // (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
  // 17-22, M >> 4 at bits 24-28.
  static constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                                     ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
  static_assert(kStagesResident <= kMaxStages && kStagesStreamed <= kMaxStages, "barrier slots");
};

constexpr int STAGE_BYTES = kEpiWarps * 32 * kStageLd * 4;
constexpr int SMEM_BYTES = RING_BYTES + STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr int kProducerWarp = kEpiWarps, kMmaWarp = kEpiWarps + 1;
constexpr int kThreads = 32 * (kEpiWarps + 2);

template <int BN_>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_bf16_tn_kernel(const __grid_constant__ CUtensorMap tmA,
                        const __grid_constant__ CUtensorMap tmB, GemmArgs g) {
  using T = Tile<BN_>;
  constexpr int BN = T::BN, B_BYTES = T::B_BYTES, kHalf = T::kHalf;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* ring = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float* stage = reinterpret_cast<float*>(ring + RING_BYTES);
  uint64_t* bars = reinterpret_cast<uint64_t*>(stage + kEpiWarps * 32 * kStageLd);
  const uint32_t full0 = smem_u32(bars);                       // full[s]
  const uint32_t empty0 = smem_u32(bars + kMaxStages);         // empty[s]
  const uint32_t tfull0 = smem_u32(bars + 2 * kMaxStages);     // accumulator a ready
  const uint32_t tempty0 = smem_u32(bars + 2 * kMaxStages + 2);  // accumulator a drained
  const uint32_t afull = smem_u32(bars + 2 * kMaxStages + 4);  // resident A block landed
  const uint32_t afree = smem_u32(bars + 2 * kMaxStages + 5);  // MMAs done with the A block
  const uint32_t drain = smem_u32(bars + 2 * kMaxStages + 6);  // every MMA issued has completed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kMaxStages + 7);
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = (g.K + BK - 1) / BK;
  const int n_tiles = (g.N + BN - 1) / BN;
  const int m_tiles = (g.M + BM - 1) / BM;
  const bool resident = g.K <= kResidentK;
  const int nst = resident ? T::kStagesResident : T::kStagesStreamed;
  // this CTA's contiguous range of output tiles, row-block major
  const long long total = (long long)m_tiles * n_tiles;
  const long long t_begin = total * blockIdx.x / gridDim.x;
  const long long t_end = total * (blockIdx.x + 1) / gridDim.x;
  // ring addresses: resident A chunks first, then B stages; or A+B per stage
  auto a_addr = [&](int s, int kt) -> uint8_t* { return resident ? ring + kt * A_BYTES : ring + s * (A_BYTES + B_BYTES); };
  auto b_addr = [&](int s) -> uint8_t* {
    return resident ? ring + kResidentChunks * A_BYTES + s * B_BYTES : ring + s * (A_BYTES + B_BYTES) + A_BYTES;
  };

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int i = 0; i < kMaxStages; ++i) {
      mbar_init(full0 + 8 * i, 1);
      mbar_init(empty0 + 8 * i, 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(tfull0 + 8 * a, 1);
      mbar_init(tempty0 + 8 * a, kEpiWarps * 32);
    }
    mbar_init(afull, 1);
    mbar_init(afree, 1);
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(2 * BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  int* abort = &s_abort;

  if (warp == kProducerWarp) {
    if (lane == 0) {  // producer: TMA ring
      int issued = 0, a_loads = 0, cur_mt = -1;
      bool ok = true;
      for (long long ti = t_begin; ti < t_end && ok; ++ti) {
        const int mt = (int)(ti / n_tiles), nt = (int)(ti % n_tiles);
        if (resident && mt != cur_mt) {
          // a new row block: wait until the MMAs are done with the old one
          if (a_loads > 0 && !mbar_wait(afree, (a_loads - 1) & 1, g.err, 6, abort, g.wait_limit)) {
            ok = false;
            break;
          }
          mbar_expect_tx(afull, (uint32_t)(nk * A_BYTES));
          for (int kt = 0; kt < nk; ++kt) tma_load_2d(smem_u32(a_addr(0, kt)), &tmA, kt * BK, mt * BM, afull);
          ++a_loads;
          cur_mt = mt;
        }
        for (int kt = 0; kt < nk; ++kt) {
          const int s = issued % nst, r = issued / nst;
          if (issued >= nst && !mbar_wait(empty0 + 8 * s, (r - 1) & 1, g.err, 1, abort, g.wait_limit)) {
            ok = false;
            break;
          }
          if (*(volatile int*)abort) {
            ok = false;
            break;
          }
          mbar_expect_tx(full0 + 8 * s, resident ? B_BYTES : A_BYTES + B_BYTES);
          if (!resident) tma_load_2d(smem_u32(a_addr(s, kt)), &tmA, kt * BK, mt * BM, full0 + 8 * s);
          tma_load_2d(smem_u32(b_addr(s)), &tmB, kt * BK, nt * BN, full0 + 8 * s);
          ++issued;
        }
      }
      if (!ok) *(volatile int*)abort = 1;
      // let every copy in flight land before the CTA can exit
      for (int i = (issued > nst ? issued - nst : 0); i < issued; ++i)
        mbar_wait(full0 + 8 * (i % nst), (i / nst) & 1, g.err, 2);
      if (a_loads > 0) mbar_wait(afull, (a_loads - 1) & 1, g.err, 2);
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0) {  // MMA issuer
      bool ok = true;
      int used = 0, t = 0, a_uses = 0, cur_mt = -1;
      for (long long ti = t_begin; ti < t_end && ok; ++ti, ++t) {
        const int mt = (int)(ti / n_tiles);
        if (resident && mt != cur_mt) {
          if (cur_mt >= 0) mma_commit(afree);  // arrives once the MMAs on the old block finish
          if (!mbar_wait(afull, a_uses & 1, g.err, 3, abort, g.wait_limit)) {
            ok = false;
            break;
          }
          ++a_uses;
          cur_mt = mt;
        }
        const int a = t & 1;
        if (t >= 2 && !mbar_wait(tempty0 + 8 * a, ((t >> 1) - 1) & 1, g.err, 5, abort, g.wait_limit)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + (uint32_t)(a * BN);
        for (int kt = 0; kt < nk; ++kt, ++used) {
          const int s = used % nst, r = used / nst;
          if (!mbar_wait(full0 + 8 * s, r & 1, g.err, 3, abort, g.wait_limit)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint64_t ad = sw128_desc(smem_u32(a_addr(s, kt)));
          const uint64_t bd = sw128_desc(smem_u32(b_addr(s)));
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk)  // +32 bytes per K=16 step inside the swizzle atom
            mma_bf16(d, ad + (uint64_t)(2 * kk), bd + (uint64_t)(2 * kk), T::kIdesc, (kt | kk) != 0);
          mma_commit(empty0 + 8 * s);
        }
        if (!ok) break;
        mma_commit(tfull0 + 8 * a);
      }
      if (!ok) *(volatile int*)abort = 1;
      // no MMA may still run when TMEM is freed, whatever path led here
      mma_commit(drain);
      mbar_wait(drain, 0, g.err, 7);
    }
  } else {
    // epilogue: warp w owns accumulator rows 32q .. 32q+31 (TMEM lanes,
    // q = w % 4) and columns 64h .. 64h+63 (h = w / 4); tcgen05.ld is
    // warp-collective, so the whole warp decides together
    const int quarter = warp & 3, half = warp >> 2;
    const int row_l = quarter * 32 + lane;
    float* wstage = stage + (size_t)warp * 32 * kStageLd;
    float* srow = wstage + (size_t)lane * kStageLd;
    // four running maxima (columns i % 4) for instruction-level parallelism;
    // each keeps its first maximum, and the merge prefers the smaller column
    // on equal values, so the result is the first maximum of the row
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
      if (row < g.M && bc >= 0) atomicMax(g.out_argmax + row, argmax_key(bb, bc));
    };
    reset_best();
    const bool has_bias = g.epilogue == kEpiBiasArgmax || g.epilogue == kEpiBiasF32 ||
                          g.epilogue == kEpiBiasReluBF16;
    const bool bias_vec = has_bias && ((uintptr_t)g.bias & 15) == 0;
    const bool vec_ok = g.epilogue != kEpiBiasArgmax && (g.ldc & 3) == 0 &&
                        ((uintptr_t)g.C & 15) == 0;
    int t = 0, cur_mt = -1;
    for (long long ti = t_begin; ti < t_end; ++ti, ++t) {
      const int mt = (int)(ti / n_tiles), nt = (int)(ti % n_tiles);
      if (g.epilogue == kEpiBiasArgmax && mt != cur_mt) {
        if (cur_mt >= 0) flush_best(cur_mt * BM + row_l);
        reset_best();
      }
      cur_mt = mt;
      const int a = t & 1;
      const bool ok = __all_sync(0xffffffffu, mbar_wait(tfull0 + 8 * a, (t >> 1) & 1, g.err, 4, abort, g.wait_limit));
      if (!ok) {
        *(volatile int*)abort = 1;
        cur_mt = -1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int m0 = mt * BM, n0 = nt * BN + half * kHalf;
      const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(a * BN + half * kHalf);
      const bool full_cols = n0 + kHalf <= g.N;
#pragma unroll 1
      for (int c0 = 0; c0 < kHalf; c0 += kChunk) {
        uint32_t r[32];
        tmem_ld32(taddr + (uint32_t)c0, r);
        // the chunk's bias (same for every row) while the TMEM load is in flight
        float bv[32];
        if (has_bias) {
#pragma unroll
          for (int i = 0; i < 32; i += 4) {
            const int col = n0 + c0 + i;
            if (bias_vec && col + 3 < g.N) {
              const float4 b4 = __ldg(reinterpret_cast<const float4*>(g.bias + col));
              bv[i] = b4.x;
              bv[i + 1] = b4.y;
              bv[i + 2] = b4.z;
              bv[i + 3] = b4.w;
            } else {
#pragma unroll
              for (int e = 0; e < 4; ++e) bv[i + e] = col + e < g.N ? __ldg(g.bias + col + e) : 0.f;
            }
          }
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i) bv[i] = 0.f;
        }
        tmem_wait_ld();
        if (c0 + kChunk == kHalf) {  // accumulator drained: hand it back to the MMA issuer
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          mbar_arrive(tempty0 + 8 * a);
        }
        if (g.epilogue == kEpiBiasArgmax) {
          if (full_cols) {
#pragma unroll
            for (int i = 0; i < 32; ++i) {
              const float x = __uint_as_float(r[i]) + bv[i];
              if (x > best[i & 3]) {
                best[i & 3] = x;
                best_col[i & 3] = n0 + c0 + i;
              }
            }
          } else {
#pragma unroll
            for (int i = 0; i < 32; ++i) {
              const int col = n0 + c0 + i;
              const float x = col < g.N ? __uint_as_float(r[i]) + bv[i] : -3.402823466e38f;
              if (x > best[i & 3]) {
                best[i & 3] = x;
                best_col[i & 3] = col;
              }
            }
          }
          continue;
        }
#pragma unroll
        for (int i = 0; i < 32; i += 4) {
          float4 v;
          v.x = __uint_as_float(r[i]) + bv[i];
          v.y = __uint_as_float(r[i + 1]) + bv[i + 1];
          v.z = __uint_as_float(r[i + 2]) + bv[i + 2];
          v.w = __uint_as_float(r[i + 3]) + bv[i + 3];
          if (g.epilogue == kEpiBiasReluBF16) {
            v.x = v.x > 0.f ? v.x : 0.f;
            v.y = v.y > 0.f ? v.y : 0.f;
            v.z = v.z > 0.f ? v.z : 0.f;
            v.w = v.w > 0.f ? v.w : 0.f;
          }
          *reinterpret_cast<float4*>(srow + i) = v;
        }
        __syncwarp();
        // the warp's 32 staged rows x 32 columns: 8 lanes per row, 4 rows per pass
        const int cc = 4 * (lane & 7);
        const int col = n0 + c0 + cc;
#pragma unroll
        for (int pass = 0; pass < 8; ++pass) {
          const int rr = pass * 4 + (lane >> 3);
          const int orow = m0 + quarter * 32 + rr;
          if (orow < g.M) {
            const float4 v = *reinterpret_cast<const float4*>(wstage + (size_t)rr * kStageLd + cc);
            if (g.epilogue == kEpiBiasReluBF16) {
              __nv_bfloat16* c = reinterpret_cast<__nv_bfloat16*>(g.C) + (size_t)orow * g.ldc + col;
              if (vec_ok && col + 3 < g.N) {
                __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
                uint2 u;
                u.x = *reinterpret_cast<uint32_t*>(&lo);
                u.y = *reinterpret_cast<uint32_t*>(&hi);
                *reinterpret_cast<uint2*>(c) = u;
              } else {
                const float vv[4] = {v.x, v.y, v.z, v.w};
                for (int e = 0; e < 4; ++e)
                  if (col + e < g.N) c[e] = __float2bfloat16_rn(vv[e]);
              }
            } else {
              float* c = reinterpret_cast<float*>(g.C) + (size_t)orow * g.ldc + col;
              if (vec_ok && col + 3 < g.N) {
                float4 o = v;
                if (g.epilogue == kEpiAccumF32) {
                  const float4 q = *reinterpret_cast<const float4*>(c);
                  o.x += q.x;
                  o.y += q.y;
                  o.z += q.z;
                  o.w += q.w;
                }
                *reinterpret_cast<float4*>(c) = o;
              } else {
                const float vv[4] = {v.x, v.y, v.z, v.w};
                for (int e = 0; e < 4; ++e)
                  if (col + e < g.N) c[e] = g.epilogue == kEpiAccumF32 ? c[e] + vv[e] : vv[e];
              }
            }
          }
        }
        __syncwarp();
      }
    }
    if (g.epilogue == kEpiBiasArgmax && cur_mt >= 0) flush_best(cur_mt * BM + row_l);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN));
  }
}

}  // namespace

namespace tc {

// cuTensorMapEncodeTiled through the runtime's driver entry point, so the
// library needs no link-time dependency on libcuda.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encoder() {
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

namespace {
std::atomic<long long> g_wait_limit{kWaitLimit};
}  // namespace

long long wait_limit() { return g_wait_limit.load(std::memory_order_relaxed); }
void set_wait_limit(long long rounds) {
  g_wait_limit.store(rounds > 0 ? rounds : kWaitLimit, std::memory_order_relaxed);
}

bool make_map_f32(CUtensorMap* m, const void* base, int64_t rows, int cols, int64_t pitch, int box_k,
                  int box_rows) {
  EncodeTiledFn enc = encoder();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)pitch * 4};
  cuuint32_t box[2] = {(cuuint32_t)box_k, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_map_bf16(CUtensorMap* m, const void* base, int rows, int K, int box_k, int box_rows) {
  EncodeTiledFn enc = encoder();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  cuuint32_t box[2] = {(cuuint32_t)box_k, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tc

cudaError_t gemm_bf16_tn(const GemmArgs& g, cudaStream_t st) {
  using namespace tc;
  if (g.M <= 0 || g.N <= 0 || g.K <= 0 || (g.K & 7) || !g.A || !g.B) return cudaErrorInvalidValue;
  if (((uintptr_t)g.A & 15) || ((uintptr_t)g.B & 15)) return cudaErrorInvalidValue;
  if (g.epilogue != kEpiBiasArgmax && !g.C) return cudaErrorInvalidValue;
  if ((g.epilogue == kEpiBiasArgmax && !g.out_argmax) ||
      ((g.epilogue == kEpiBiasArgmax || g.epilogue == kEpiBiasF32 ||
        g.epilogue == kEpiBiasReluBF16) && !g.bias))
    return cudaErrorInvalidValue;
  // 128 x 256 tiles (half the MMA instructions per FLOP) for the wide
  // argmax layer, 128 x 128 elsewhere (twice the CTAs for narrow outputs)
  const bool wide = g.epilogue == kEpiBiasArgmax && g.N >= 1024;
  const int bn = wide ? 256 : 128;
  CUtensorMap ma, mb;
  if (!make_map_bf16(&ma, g.A, g.M, g.K, BK, BM) || !make_map_bf16(&mb, g.B, g.N, g.K, BK, bn))
    return cudaErrorNotSupported;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  // per-device caches, set once; concurrent host threads may race to set
  // them, which is harmless (the same values), hence atomics
  static std::atomic<int> num_sms[64];
  static std::atomic<bool> attr[2][64];
  if (dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[wide][dev].load(std::memory_order_acquire)) {
    cudaError_t e = wide ? cudaFuncSetAttribute(gemm_bf16_tn_kernel<256>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES)
                         : cudaFuncSetAttribute(gemm_bf16_tn_kernel<128>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr[wide][dev].store(true, std::memory_order_release);
  }
  // one CTA per SM, each taking a contiguous range of the output tiles
  int sms = num_sms[dev].load(std::memory_order_relaxed);
  if (sms == 0) {
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
    num_sms[dev].store(sms, std::memory_order_relaxed);
  }
  const long long tiles = (long long)((g.M + BM - 1) / BM) * ((g.N + bn - 1) / bn);
  dim3 grid((unsigned)(tiles < sms ? tiles : sms));
  GemmArgs ga = g;
  ga.wait_limit = wait_limit();
  if (wide)
    gemm_bf16_tn_kernel<256><<<grid, kThreads, SMEM_BYTES, st>>>(ma, mb, ga);
  else
    gemm_bf16_tn_kernel<128><<<grid, kThreads, SMEM_BYTES, st>>>(ma, mb, ga);
  return cudaGetLastError();
}

}  // namespace rte
