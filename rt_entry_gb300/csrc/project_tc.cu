// project_tc.cu -- the PCA projection on the 5th-generation tensor cores.
//
//   out[r][j] = sum_k (x[r][k] - mean[k]) * V[k][j]
//
// for the query projection (the reference's cuBLAS TENSOR_OP GEMM with the
// mean folded in through beta = -1, matrix.cu:39-69 and graph.cu:258-273)
// and the base projection at build time ((B - mean) V, pca.cpp:122-126).
// FP32 operands run on the TF32 tensor cores with a three-term split: with
// v = x - mean, v_hi = tf32(v) and v_lo = tf32(v - v_hi) (V likewise, split
// once when the PCA is installed),
//     v . V  ~=  v_hi . V_hi + v_hi . V_lo + v_lo . V_hi
// accumulated in FP32.  v_hi + v_lo carries v to 2^-22 relative, every TF32
// product is exact in FP32, and the dropped v_lo . V_lo term is below
// 2^-22 |v| |V|, so the result is as accurate as an FP32 FMA chain.
//
// One CTA of 10 warps per SM, persistent over (128-row block, column block)
// work items, row-block major:
//   * warp 8 / lane 0 streams, per 32-wide K chunk, the 128 x 32 FP32 tile
//     of x and the column block's V_hi and V_lo tiles into an mbarrier ring
//     with TMA (128-byte swizzle: each tile lands in the K-major layout the
//     MMA reads);
//   * warps 4-7 split the x tile in place: subtract the mean, round to TF32
//     into the hi tile (the same bytes) and write the remainder's TF32 into
//     the lo tile, then hand the stage to the MMA issuer.  The swizzle only
//     permutes 16-byte units within a row, so each unit's K offset is its
//     position XOR the row's low three bits;
//   * warp 9 / lane 0 issues tcgen05.mma.kind::tf32 (M = 128, N = the column
//     block, K = 8 per instruction), three products per K step, into one of
//     two TMEM accumulators, so a block's MMAs overlap the previous block's
//     epilogue;
//   * warps 0-3 (one per TMEM lane quarter) read the accumulator with
//     tcgen05.ld and write the FP32 rows, and on the learned path the
//     model's BF16 input rows (out16 = bf16(out * s16), zero-padded).
// Every pipeline wait is bounded (rte_set_wait_limit); the waits that let
// copies and MMAs in flight finish before the CTA exits or frees TMEM use
// the long default.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "index_kernels.h"
#include "tc_common.cuh"

namespace rte {

namespace {

using namespace tc;

constexpr int kPM = 128;                 // rows per tile (MMA M)
constexpr int kPK = 32;                  // K per chunk: one 128-byte row of FP32
constexpr int kXBytes = kPM * kPK * 4;   // 16 KB
constexpr int kMaxStages = 4;
constexpr int kMaxD = 1024;              // input dims the mean buffer holds
constexpr int kProdWarp = 8, kMmaWarp = 9, kThreads = 320;
constexpr int kConvThreads = 128;        // warps 4-7
constexpr int kEpiThreads = 128;         // warps 0-3
constexpr int kSmemBytes = 226 * 1024;    // dynamic; 1 KB stays for static shared memory
constexpr int kRingBytes = kSmemBytes - 1024 /*align*/ - kMaxD * 4 - 256 /*barriers*/;

struct ProjTcArgs {
  int64_t n;            // rows (the capacity when n_dev is set)
  const int* n_dev;     // live row count read at run time (graph replay) or null
  int d, k;             // input and output dims
  int bnc;              // output columns per MMA (multiple of 32, <= 256)
  int stages;
  const float* mean;    // [d] or null
  float* out;
  int64_t ostride;
  __nv_bfloat16* out16; // [n][ld16] or null
  float s16;
  int ld16;
  uint32_t* zero;       // words set to 0 on the way, or null
  int64_t zero_words;
  int* err;             // set to a non-zero code when a bounded wait runs out (or null)
  long long wait_limit;
};

__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r & 0xFFFFE000u);
}

template <bool kOut16>
__global__ void __launch_bounds__(kThreads, 1)
    project_tf32_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmVh,
                        const __grid_constant__ CUtensorMap tmVl, ProjTcArgs p) {
  extern __shared__ uint8_t smem_raw[];
  if (p.zero) {  // a query call's counters and keys, zeroed on the way
    const int64_t nt = (int64_t)gridDim.x * blockDim.x;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < p.zero_words; w += nt) p.zero[w] = 0u;
  }
  const int64_t n = p.n_dev ? min(p.n, (int64_t)max(*p.n_dev, 0)) : p.n;
  const int n_nt = (p.k + p.bnc - 1) / p.bnc;
  const long long items = (long long)((n + kPM - 1) / kPM) * n_nt;
  if ((long long)blockIdx.x >= items) return;  // the whole CTA: nothing to do
  const int nk = (p.d + kPK - 1) / kPK;
  const int S = p.stages;
  const uint32_t bbytes = (uint32_t)p.bnc * 128;  // one bnc x 32 tile of V_hi or V_lo
  const uint32_t stage_bytes = 2 * kXBytes + 2 * bbytes;
  uint8_t* ring = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float* mean_s = reinterpret_cast<float*>(ring + kRingBytes);
  uint64_t* bars = reinterpret_cast<uint64_t*>(mean_s + kMaxD);
  const uint32_t full0 = smem_u32(bars);                        // stage landed (TMA)
  const uint32_t aready0 = smem_u32(bars + kMaxStages);         // x tile split into hi / lo
  const uint32_t empty0 = smem_u32(bars + 2 * kMaxStages);      // MMAs done with the stage
  const uint32_t tfull0 = smem_u32(bars + 3 * kMaxStages);      // accumulator a complete
  const uint32_t tempty0 = smem_u32(bars + 3 * kMaxStages + 2); // accumulator a read out
  const uint32_t drain = smem_u32(bars + 3 * kMaxStages + 4);   // every MMA issued has completed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3 * kMaxStages + 5);
  __shared__ int s_abort;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int tmem_cols = 32;
  while (tmem_cols < 2 * p.bnc) tmem_cols <<= 1;

  // the mean, zero past d (a K chunk reads 32 values)
  for (int i = threadIdx.x; i < nk * kPK; i += blockDim.x) mean_s[i] = p.mean && i < p.d ? p.mean[i] : 0.0f;
  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int i = 0; i < kMaxStages; ++i) {
      mbar_init(full0 + 8 * i, 1);
      mbar_init(aready0 + 8 * i, kConvThreads);
      mbar_init(empty0 + 8 * i, 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(tfull0 + 8 * a, 1);
      mbar_init(tempty0 + 8 * a, kEpiThreads);
    }
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  int* abort = &s_abort;
  auto xs = [&](int s) { return ring + (size_t)s * stage_bytes; };
  auto los = [&](int s) { return ring + (size_t)s * stage_bytes + kXBytes; };
  auto bhs = [&](int s) { return ring + (size_t)s * stage_bytes + 2 * kXBytes; };
  auto bls = [&](int s) { return ring + (size_t)s * stage_bytes + 2 * kXBytes + bbytes; };

  if (warp == kProdWarp) {
    if (lane == 0) {
      int issued = 0;
      bool ok = true;
      for (long long it = blockIdx.x; it < items && ok; it += gridDim.x) {
        const int mt = (int)(it / n_nt), nt = (int)(it % n_nt);
        for (int kt = 0; kt < nk; ++kt) {
          const int s = issued % S, r = issued / S;
          if (issued >= S && !mbar_wait(empty0 + 8 * s, (r - 1) & 1, p.err, 31, abort, p.wait_limit)) {
            ok = false;
            break;
          }
          if (*(volatile int*)abort) {
            ok = false;
            break;
          }
          mbar_expect_tx(full0 + 8 * s, (uint32_t)kXBytes + 2 * bbytes);
          tma_load_2d(smem_u32(xs(s)), &tmX, kt * kPK, mt * kPM, full0 + 8 * s);
          tma_load_2d(smem_u32(bhs(s)), &tmVh, kt * kPK, nt * p.bnc, full0 + 8 * s);
          tma_load_2d(smem_u32(bls(s)), &tmVl, kt * kPK, nt * p.bnc, full0 + 8 * s);
          ++issued;
        }
      }
      if (!ok) *(volatile int*)abort = 1;
      // let every copy in flight land before the CTA can exit
      for (int i = (issued > S ? issued - S : 0); i < issued; ++i)
        mbar_wait(full0 + 8 * (i % S), (i / S) & 1, p.err, 32);
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0) {
      // kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32 (bits 7-9, 10-12 =
      // 2), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
      const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(p.bnc >> 3) << 17) |
                             ((uint32_t)(kPM >> 4) << 24);
      bool ok = true;
      int used = 0, t = 0;
      for (long long it = blockIdx.x; it < items && ok; it += gridDim.x, ++t) {
        const int a = t & 1;
        if (t >= 2 && !mbar_wait(tempty0 + 8 * a, ((t >> 1) - 1) & 1, p.err, 33, abort, p.wait_limit)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + (uint32_t)(a * p.bnc);
        for (int kt = 0; kt < nk; ++kt, ++used) {
          const int s = used % S, r = used / S;
          if (!mbar_wait(full0 + 8 * s, r & 1, p.err, 34, abort, p.wait_limit) ||
              !mbar_wait(aready0 + 8 * s, r & 1, p.err, 35, abort, p.wait_limit)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint64_t ah = sw128_desc(smem_u32(xs(s))), al = sw128_desc(smem_u32(los(s)));
          const uint64_t bh = sw128_desc(smem_u32(bhs(s))), bl = sw128_desc(smem_u32(bls(s)));
#pragma unroll
          for (int kk = 0; kk < kPK / 8; ++kk) {  // +32 bytes per K = 8 step inside the swizzle row
            const uint64_t o = (uint64_t)(2 * kk);
            mma_tf32(d, ah + o, bh + o, idesc, (kt | kk) != 0);
            mma_tf32(d, ah + o, bl + o, idesc, 1);
            mma_tf32(d, al + o, bh + o, idesc, 1);
          }
          mma_commit(empty0 + 8 * s);
        }
        if (!ok) break;
        mma_commit(tfull0 + 8 * a);
      }
      if (!ok) *(volatile int*)abort = 1;
      // no MMA may still run when TMEM is freed, whatever path led here
      mma_commit(drain);
      mbar_wait(drain, 0, p.err, 36);
    }
  } else if (warp >= 4) {
    // converters: 16-byte unit u of a stage's x tile is row u / 8 and, under
    // the 128-byte swizzle, K chunk-quarter (u % 8) ^ (row % 8)
    const int c = threadIdx.x - 4 * 32;
    int used = 0;
    bool ok = true;
    for (long long it = blockIdx.x; it < items && ok; it += gridDim.x) {
      for (int kt = 0; kt < nk; ++kt, ++used) {
        const int s = used % S, r = used / S;
        if (!mbar_wait(full0 + 8 * s, r & 1, p.err, 37, abort, p.wait_limit)) {
          ok = false;
          break;
        }
        float4* xt = reinterpret_cast<float4*>(xs(s));
        float4* lt = reinterpret_cast<float4*>(los(s));
#pragma unroll
        for (int u = c; u < kXBytes / 16; u += kConvThreads) {
          const int row = u >> 3;
          const int kq = (u & 7) ^ (row & 7);
          const float4 xv = xt[u];
          const float4 m = *reinterpret_cast<const float4*>(mean_s + kt * kPK + 4 * kq);
          float4 v, hi, lo;
          v.x = __fsub_rn(xv.x, m.x);
          v.y = __fsub_rn(xv.y, m.y);
          v.z = __fsub_rn(xv.z, m.z);
          v.w = __fsub_rn(xv.w, m.w);
          hi.x = to_tf32(v.x);
          hi.y = to_tf32(v.y);
          hi.z = to_tf32(v.z);
          hi.w = to_tf32(v.w);
          lo.x = to_tf32(__fsub_rn(v.x, hi.x));
          lo.y = to_tf32(__fsub_rn(v.y, hi.y));
          lo.z = to_tf32(__fsub_rn(v.z, hi.z));
          lo.w = to_tf32(__fsub_rn(v.w, hi.w));
          xt[u] = hi;
          lt[u] = lo;
        }
        // make the generic-proxy writes visible to the tensor core's reads
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(aready0 + 8 * s);
      }
    }
    if (!ok) *(volatile int*)abort = 1;
  } else {
    // epilogue: warp w reads TMEM lanes (rows) 32w .. 32w+31
    int t = 0;
    for (long long it = blockIdx.x; it < items; it += gridDim.x, ++t) {
      const int mt = (int)(it / n_nt), nt = (int)(it % n_nt);
      const int a = t & 1;
      const bool ok = __all_sync(0xffffffffu, mbar_wait(tfull0 + 8 * a, (t >> 1) & 1, p.err, 38, abort, p.wait_limit));
      if (!ok) {
        *(volatile int*)abort = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int64_t row = (int64_t)mt * kPM + warp * 32 + lane;
      const int col0 = nt * p.bnc;
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(a * p.bnc);
      for (int c0 = 0; c0 < p.bnc && col0 + c0 < p.k; c0 += 32) {
        uint32_t rv[32];
        tmem_ld32(taddr + (uint32_t)c0, rv);
        tmem_wait_ld();
        if (row >= n) continue;
        const int cb = col0 + c0;
        float* o = p.out + row * p.ostride + cb;
        if (cb + 32 <= p.k && (p.ostride & 3) == 0 && ((uintptr_t)p.out & 15) == 0) {
#pragma unroll
          for (int i = 0; i < 32; i += 4)
            *reinterpret_cast<float4*>(o + i) = make_float4(__uint_as_float(rv[i]), __uint_as_float(rv[i + 1]),
                                                            __uint_as_float(rv[i + 2]), __uint_as_float(rv[i + 3]));
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i)
            if (cb + i < p.k) o[i] = __uint_as_float(rv[i]);
        }
        if (kOut16) {
          __nv_bfloat16* h = p.out16 + row * p.ld16 + cb;
          if (cb + 32 <= p.k && (p.ld16 & 7) == 0 && ((uintptr_t)p.out16 & 15) == 0) {
#pragma unroll
            for (int i = 0; i < 32; i += 8) {
              uint4 u;
              uint32_t w[4];
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const __nv_bfloat16 lo = __float2bfloat16_rn(__fmul_rn(__uint_as_float(rv[i + 2 * e]), p.s16));
                const __nv_bfloat16 hi = __float2bfloat16_rn(__fmul_rn(__uint_as_float(rv[i + 2 * e + 1]), p.s16));
                w[e] = (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
              }
              u.x = w[0];
              u.y = w[1];
              u.z = w[2];
              u.w = w[3];
              *reinterpret_cast<uint4*>(h + i) = u;
            }
          } else {
#pragma unroll
            for (int i = 0; i < 32; ++i)
              if (cb + i < p.k) h[i] = __float2bfloat16_rn(__fmul_rn(__uint_as_float(rv[i]), p.s16));
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(tempty0 + 8 * a);
      if (kOut16 && nt == n_nt - 1 && row < n)  // the model input's padding columns
        for (int cpad = p.k; cpad < p.ld16; ++cpad) p.out16[row * p.ld16 + cpad] = __float2bfloat16_rn(0.0f);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols));
  }
}

// V [d][k] (row pitch vstride) -> the transposed split [2][k][dpad]:
// hi = tf32(V), lo = tf32(V - hi), K-major rows for the MMA's B operand.
__global__ void split_rotation_t(const float* __restrict__ V, int d, int k, int vstride, int dpad,
                                 float* __restrict__ out) {
  const int64_t total = (int64_t)k * dpad;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(i / dpad), c = (int)(i % dpad);
    const float v = c < d ? V[(int64_t)c * vstride + j] : 0.0f;
    const float hi = to_tf32(v);
    out[i] = hi;
    out[total + i] = to_tf32(__fsub_rn(v, hi));
  }
}

// Tensor maps of a split rotation, encoded once per (array, shape, block).
struct VMaps {
  const float* vt = nullptr;
  int d = 0, k = 0, bnc = 0;
  CUtensorMap hi, lo;
};

bool rotation_maps(const float* vt, int d, int k, int bnc, CUtensorMap* hi, CUtensorMap* lo) {
  static std::mutex mu;
  static VMaps cache[8];
  static int next = 0;
  std::lock_guard<std::mutex> lk(mu);
  for (const VMaps& c : cache)
    if (c.vt == vt && c.d == d && c.k == k && c.bnc == bnc) {
      *hi = c.hi;
      *lo = c.lo;
      return true;
    }
  const int dpad = (d + 3) & ~3;
  VMaps m;
  m.vt = vt;
  m.d = d;
  m.k = k;
  m.bnc = bnc;
  if (!make_map_f32(&m.hi, vt, k, d, dpad, kPK, bnc) ||
      !make_map_f32(&m.lo, vt + (size_t)k * dpad, k, d, dpad, kPK, bnc))
    return false;
  cache[next] = m;
  next = (next + 1) % 8;
  *hi = m.hi;
  *lo = m.lo;
  return true;
}

}  // namespace

size_t rotation_split_floats(int d, int k) { return 2 * (size_t)k * (size_t)((d + 3) & ~3); }

cudaError_t launch_split_rotation(const float* V, int d, int k, int vstride, float* out, cudaStream_t st) {
  const int dpad = (d + 3) & ~3;
  const int64_t total = (int64_t)k * dpad;
  const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  split_rotation_t<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(V, d, k, vstride, dpad, out);
  return cudaGetLastError();
}

cudaError_t launch_project_tc(const float* x, int64_t n, const int* n_dev, int d, int xstride,
                              const float* mean, const float* vt_split, int k, float* out, int ostride,
                              void* out16, float s16, int ld16, uint32_t* zero, int64_t zero_words,
                              int* err, cudaStream_t st) {
  if (!x || !vt_split || !out || n <= 0 || d <= 0 || d > kMaxD || k <= 0 || k > 1024) return cudaErrorNotSupported;
  if ((xstride & 3) || ((uintptr_t)x & 15) || n > (int64_t)INT32_MAX) return cudaErrorNotSupported;
  if (out16 && ld16 < k) return cudaErrorInvalidValue;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return cudaErrorInvalidDevice;
  static std::atomic<int> arch[64];  // 0 unknown, 1 tensor-core path, -1 not
  static std::atomic<int> num_sms[64];
  static std::atomic<bool> attr[2][64];
  int ar = arch[dev].load(std::memory_order_relaxed);
  if (ar == 0) {
    int major = 0, sms = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    num_sms[dev].store(sms > 0 ? sms : 1, std::memory_order_relaxed);
    ar = major >= 10 ? 1 : -1;
    arch[dev].store(ar, std::memory_order_relaxed);
  }
  if (ar < 0) return cudaErrorNotSupported;
  const bool o16 = out16 != nullptr;
  if (!attr[o16][dev].load(std::memory_order_acquire)) {
    cudaError_t e = o16 ? cudaFuncSetAttribute(project_tf32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes)
                        : cudaFuncSetAttribute(project_tf32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    attr[o16][dev].store(true, std::memory_order_release);
  }
  ProjTcArgs p{};
  p.n = n;
  p.n_dev = n_dev;
  p.d = d;
  p.k = k;
  p.bnc = k >= 256 ? 256 : (k + 31) & ~31;
  const int stage_bytes = 2 * kXBytes + 2 * p.bnc * 128;
  p.stages = kRingBytes / stage_bytes < kMaxStages ? kRingBytes / stage_bytes : kMaxStages;
  p.mean = mean;
  p.out = out;
  p.ostride = ostride;
  p.out16 = static_cast<__nv_bfloat16*>(out16);
  p.s16 = s16;
  p.ld16 = ld16;
  p.zero = zero;
  p.zero_words = zero_words;
  p.err = err;
  p.wait_limit = wait_limit();
  CUtensorMap mx, mh, ml;
  if (!make_map_f32(&mx, x, n, d, xstride, kPK, kPM) || !rotation_maps(vt_split, d, k, p.bnc, &mh, &ml))
    return cudaErrorNotSupported;
  const long long items = (long long)((n + kPM - 1) / kPM) * ((k + p.bnc - 1) / p.bnc);
  const int sms = num_sms[dev].load(std::memory_order_relaxed);
  const dim3 grid((unsigned)(items < sms ? items : sms));
  if (o16)
    project_tf32_kernel<true><<<grid, kThreads, kSmemBytes, st>>>(mx, mh, ml, p);
  else
    project_tf32_kernel<false><<<grid, kThreads, kSmemBytes, st>>>(mx, mh, ml, p);
  return cudaGetLastError();
}

}  // namespace rte
