// index_kernels.cu -- build-side and entry-stage kernels for sm_103a.
//
//   mean/covariance  FP64, deterministic (fixed row chunks, fixed reduction
//                    order).  The reference forms C = X^T X / (n-1) of the
//                    centred base in FP64 with Eigen on one host thread
//                    (pca.cpp:4-10,44-48).
//   projection       out = (X - mean) V[:, :k], FP32 accumulation.  Used for
//                    the base (pca.cpp:122-126, which does it in FP64 on the
//                    host) and for the queries (graph.cu:258-273, a cuBLAS
//                    FP32 GEMM with the mean term folded in via beta = -1).
//   interleave       row-major FP32 -> lane-interleaved FP32 / BF16 / FP8-E4M3
//                    (layout.cuh), plus the first three coordinates for the
//                    kd-tree.
//   locate           smallest-index expanded leaf box containing a point,
//                    0 on a miss; replaces the OptiX ray cast
//                    (devicePrograms.cu:29-96, raytracing.cpp:283-334).
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <stdint.h>

#include "index_kernels.h"
#include "layout.cuh"

namespace rte {

// ---------------------------------------------------------------- mean ----
// Block b sums rows [b*rows_per_block, ...) of every column in FP64 into
// partial[b][col]; a second kernel adds the partials in block order.
__global__ void col_sum_partial(const float* __restrict__ x, int64_t n, int d,
                                int64_t rows_per_block, double* __restrict__ partial) {
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
  const int64_t r1 = min(n, r0 + rows_per_block);
  for (int c = threadIdx.x; c < d; c += blockDim.x) {
    double s = 0.0;
    for (int64_t r = r0; r < r1; ++r) s += (double)x[r * d + c];
    partial[(int64_t)blockIdx.x * d + c] = s;
  }
}

__global__ void col_sum_finish(const double* __restrict__ partial, int nblocks, int d, int64_t n,
                               double* __restrict__ mean) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partial[(int64_t)b * d + c];
  mean[c] = s / (double)n;
}

// ---------------------------------------------------------- covariance ----
// Tile of 32x32 outputs per block (16x16 threads, 2x2 each) over a chunk of
// rows; rows are centred in FP64 as they are staged in shared memory.
constexpr int kCovTile = 32;
constexpr int kCovK = 32;

__global__ void cov_partial(const float* __restrict__ x, int64_t n, int d,
                            const double* __restrict__ mean, int64_t rows_per_chunk,
                            double* __restrict__ partial) {
  __shared__ double sa[kCovK][kCovTile + 1];
  __shared__ double sb[kCovK][kCovTile + 1];
  const int i0 = blockIdx.y * kCovTile, j0 = blockIdx.x * kCovTile;
  const int64_t r0 = (int64_t)blockIdx.z * rows_per_chunk;
  const int64_t r1 = min(n, r0 + rows_per_chunk);
  const int tx = threadIdx.x, ty = threadIdx.y;
  double acc[2][2] = {{0, 0}, {0, 0}};
  for (int64_t rb = r0; rb < r1; rb += kCovK) {
    for (int t = ty * 16 + tx; t < kCovK * kCovTile; t += 256) {
      const int rr = t / kCovTile, cc = t % kCovTile;
      const int64_t r = rb + rr;
      double va = 0.0, vb = 0.0;
      if (r < r1) {
        if (i0 + cc < d) va = (double)x[r * d + i0 + cc] - mean[i0 + cc];
        if (j0 + cc < d) vb = (double)x[r * d + j0 + cc] - mean[j0 + cc];
      }
      sa[rr][cc] = va;
      sb[rr][cc] = vb;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kCovK; ++k) {
      const double a0 = sa[k][ty], a1 = sa[k][ty + 16];
      const double b0 = sb[k][tx], b1 = sb[k][tx + 16];
      acc[0][0] = fma(a0, b0, acc[0][0]);
      acc[0][1] = fma(a0, b1, acc[0][1]);
      acc[1][0] = fma(a1, b0, acc[1][0]);
      acc[1][1] = fma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
  double* out = partial + (int64_t)blockIdx.z * d * d;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const int i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
      if (i < d && j < d) out[(int64_t)i * d + j] = acc[a][b];
    }
}

__global__ void cov_finish(const double* __restrict__ partial, int nchunks, int d, int64_t n,
                           double* __restrict__ cov) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t dd = (int64_t)d * d;
  if (e >= dd) return;
  double s = 0.0;
  for (int c = 0; c < nchunks; ++c) s += partial[c * dd + e];
  cov[e] = s / (double)(n - 1);
}

// ---------------------------------------------------------- projection ----
// out[r][j] = sum_c (x[r][c] - mean[c]) * V[c][j], one fmaf per c in
// ascending order.  A block of 256 threads computes a 32 x 128 tile; warp w
// owns rows 4w .. 4w+3 and lane l columns 4l .. 4l+3.  Shared memory keeps
// each warp's four rows interleaved (sx[w][c][0..3]), so one broadcast
// 16-byte load gives a thread its four x values and one 16-byte load its
// four V values: two loads (five shared-memory wavefronts) per 16 FMAs.
// The 32-wide slices of c are double-buffered in shared memory (40 KB): the
// next slice's global loads are in flight while the current one is
// multiplied.  At most 85 registers a thread keep three blocks on an SM, so
// a batch of up to 152 x 3 x 32 rows runs in a single wave.  With kOut16 the
// block also writes the learned head's BF16 input row: bf16(out * s16),
// zero-padded to ld16 columns.
constexpr int kPrRows = 32;
constexpr int kPrCols = 128;
constexpr int kPrK = 32;
constexpr int kPrThreads = 256;
constexpr int kPrXFloats = kPrRows * kPrK;   // one buffer of sx
constexpr int kPrVFloats = kPrK * kPrCols;   // one buffer of sv

template <bool kOut16>
__global__ void __launch_bounds__(kPrThreads, 3) project_rows(const float* __restrict__ x, int64_t n, int d,
                                                           int xstride, const float* __restrict__ mean,
                                                           const float* __restrict__ V, int vstride, int k,
                                                           float* __restrict__ out, int ostride,
                                                           const int* __restrict__ n_dev,
                                                           __nv_bfloat16* __restrict__ out16, float s16,
                                                           int ld16, uint32_t* __restrict__ zero,
                                                           int64_t zero_words) {
  if (zero) {  // the query call's counters and argmax keys, zeroed on the way
    const int64_t nt = (int64_t)gridDim.x * gridDim.y * blockDim.x;
    for (int64_t w = ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x; w < zero_words; w += nt)
      zero[w] = 0u;
  }
  if (n_dev) n = min(n, (int64_t)*n_dev);  // graph replay: rows beyond the batch are idle
  if ((int64_t)blockIdx.x * kPrRows >= n) return;
  __shared__ __align__(16) float pr_smem[2 * (kPrXFloats + kPrVFloats)];
  float* sx = pr_smem;                    // [2][kPrRows/4][kPrK][4]
  float* sv = pr_smem + 2 * kPrXFloats;   // [2][kPrK][kPrCols]
  const int64_t row0 = (int64_t)blockIdx.x * kPrRows;
  const int col0 = blockIdx.y * kPrCols;
  const int tx = threadIdx.x & 31;  // columns 4tx .. 4tx+3
  const int ty = threadIdx.x >> 5;  // rows 4ty .. 4ty+3
  constexpr int kXPer = kPrXFloats / kPrThreads, kVPer = kPrVFloats / kPrThreads;
  float rx[kXPer], rv[kVPer];
  auto gload = [&](int c0) {
#pragma unroll
    for (int u = 0; u < kXPer; ++u) {
      const int t = threadIdx.x + kPrThreads * u;
      const int rr = t / kPrK, cc = t % kPrK;
      const int64_t r = row0 + rr;
      float v = 0.0f;
      if (r < n && c0 + cc < d) v = __fsub_rn(x[r * xstride + c0 + cc], mean ? mean[c0 + cc] : 0.0f);
      rx[u] = v;
    }
#pragma unroll
    for (int u = 0; u < kVPer; ++u) {
      const int t = threadIdx.x + kPrThreads * u;
      const int cc = t / kPrCols, jj = t % kPrCols;
      float v = 0.0f;
      if (c0 + cc < d && col0 + jj < k) v = V[(int64_t)(c0 + cc) * vstride + col0 + jj];
      rv[u] = v;
    }
  };
  auto sstore = [&](int b) {
#pragma unroll
    for (int u = 0; u < kXPer; ++u) {
      const int t = threadIdx.x + kPrThreads * u;
      const int rr = t / kPrK, cc = t % kPrK;
      sx[b * kPrXFloats + ((rr >> 2) * kPrK + cc) * 4 + (rr & 3)] = rx[u];
    }
#pragma unroll
    for (int u = 0; u < kVPer; ++u) sv[b * kPrVFloats + threadIdx.x + kPrThreads * u] = rv[u];
  };
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
  gload(0);
  sstore(0);
  __syncthreads();
  int b = 0;
  for (int c0 = 0; c0 < d; c0 += kPrK) {
    const bool more = c0 + kPrK < d;
    if (more) gload(c0 + kPrK);
    const float4* xs = reinterpret_cast<const float4*>(sx + b * kPrXFloats) + ty * kPrK;
    const float4* vs = reinterpret_cast<const float4*>(sv + b * kPrVFloats) + tx;
#pragma unroll 8
    for (int cc = 0; cc < kPrK; ++cc) {
      const float4 xv = xs[cc];
      const float4 v = vs[cc * (kPrCols / 4)];
      const float xr[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        acc[i][0] = __fmaf_rn(xr[i], v.x, acc[i][0]);
        acc[i][1] = __fmaf_rn(xr[i], v.y, acc[i][1]);
        acc[i][2] = __fmaf_rn(xr[i], v.z, acc[i][2]);
        acc[i][3] = __fmaf_rn(xr[i], v.w, acc[i][3]);
      }
    }
    if (more) sstore(b ^ 1);
    __syncthreads();
    b ^= 1;
  }
  const int c4 = col0 + 4 * tx;
  const bool vec32 = (ostride & 3) == 0 && ((uintptr_t)out & 15) == 0 && c4 + 3 < k;
  const bool vec16 = kOut16 && (ld16 & 3) == 0 && ((uintptr_t)out16 & 7) == 0 && c4 + 3 < ld16;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t r = row0 + 4 * ty + i;
    if (r >= n) break;
    if (vec32) {
      *reinterpret_cast<float4*>(out + r * ostride + c4) = make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (c4 + j < k) out[r * ostride + c4 + j] = acc[i][j];
    }
    if (kOut16) {
      // acc is 0 in the padding columns k .. ld16-1
      __nv_bfloat16 h[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) h[j] = __float2bfloat16_rn(__fmul_rn(acc[i][j], s16));
      if (vec16) {
        uint2 u;
        u.x = (uint32_t)__bfloat16_as_ushort(h[0]) | ((uint32_t)__bfloat16_as_ushort(h[1]) << 16);
        u.y = (uint32_t)__bfloat16_as_ushort(h[2]) | ((uint32_t)__bfloat16_as_ushort(h[3]) << 16);
        *reinterpret_cast<uint2*>(out16 + r * ld16 + c4) = u;
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (c4 + j < ld16) out16[r * ld16 + c4 + j] = h[j];
      }
    }
  }
}

// ---------------------------------------------------------- interleave ----
__global__ void interleave_rows(const float* __restrict__ src, int64_t n, int d, int C,
                                float* __restrict__ il32, __nv_bfloat16* __restrict__ il16,
                                uint8_t* __restrict__ il8, float* __restrict__ scale8,
                                float* __restrict__ xyz) {
  // one warp per row
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n; r += nwarps) {
    const float* s = src + r * d;
    float amax = 0.0f;
    for (int c = 0; c < C; ++c) {
      const int dim = lane + 32 * c;
      const float v = dim < d ? s[dim] : 0.0f;
      amax = fmaxf(amax, fabsf(v));
      const int64_t o = r * (32 * C) + interleaved_offset(c, lane, C);
      if (il32) il32[o] = v;
      if (il16) il16[o] = __float2bfloat16_rn(v);
    }
    if (il8) {
      for (int off = 16; off >= 1; off >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, off));
      const float sc = amax > 0.0f ? amax / 448.0f : 1.0f;
      if (lane == 0) scale8[r] = sc;
      for (int c = 0; c < C; ++c) {
        const int dim = lane + 32 * c;
        const float v = dim < d ? s[dim] : 0.0f;
        const int64_t o = r * (32 * C) + interleaved_offset(c, lane, C);
        il8[o] = (uint8_t)__nv_cvt_float_to_fp8(__fdiv_rn(v, sc), __NV_SATFINITE, __NV_E4M3);
      }
    }
    if (xyz && lane < 3) xyz[r * 3 + lane] = lane < d ? s[lane] : 0.0f;
  }
}

// The BF16 and FP8 copies from the interleaved FP32 copy, one warp per row:
// the same offsets, roundings and per-row scale (max |x| / 448 over the
// row's dims) as interleave_rows writes from row-major input.
__global__ void lowp_from_il32(const float* __restrict__ il32, int64_t n, int C,
                               __nv_bfloat16* __restrict__ il16, uint8_t* __restrict__ il8,
                               float* __restrict__ scale8) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n; r += nwarps) {
    const float* s = il32 + r * (32 * C);
    float amax = 0.0f;
    for (int c = 0; c < C; ++c) {
      const int64_t o = interleaved_offset(c, lane, C);
      const float v = s[o];
      amax = fmaxf(amax, fabsf(v));
      if (il16) il16[r * (32 * C) + o] = __float2bfloat16_rn(v);
    }
    if (il8) {
      for (int off = 16; off >= 1; off >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, off));
      const float sc = amax > 0.0f ? amax / 448.0f : 1.0f;
      if (lane == 0) scale8[r] = sc;
      for (int c = 0; c < C; ++c) {
        const int64_t o = interleaved_offset(c, lane, C);
        il8[r * (32 * C) + o] = (uint8_t)__nv_cvt_float_to_fp8(__fdiv_rn(s[o], sc), __NV_SATFINITE, __NV_E4M3);
      }
    }
  }
}

__global__ void deinterleave_rows(const float* __restrict__ il32, int64_t n, int d, int C,
                                  float* __restrict__ dst) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n; r += nwarps)
    for (int c = 0; c < C; ++c) {
      const int dim = lane + 32 * c;
      if (dim < d) dst[r * d + dim] = il32[r * (32 * C) + interleaved_offset(c, lane, C)];
    }
}

// The values the BF16 / FP8 search paths compute with, de-interleaved:
// exactly the widening done by load_interleaved_bf16 / _fp8 (and the FP8
// scale multiply of the search kernel's row loader).
__global__ void dequant_rows(const void* __restrict__ il, const float* __restrict__ scale8,
                             int precision, int64_t n, int d, int C, float* __restrict__ dst) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n; r += nwarps)
    for (int c = 0; c < C; ++c) {
      const int dim = lane + 32 * c;
      if (dim >= d) continue;
      const int64_t o = r * (32 * C) + interleaved_offset(c, lane, C);
      float v;
      if (precision == 1) {
        v = __uint_as_float((uint32_t)reinterpret_cast<const uint16_t*>(il)[o] << 16);
      } else {
        const uint8_t b = reinterpret_cast<const uint8_t*>(il)[o];
        v = fp8x2_to_float2((uint16_t)b).x * scale8[r];
      }
      dst[r * d + dim] = v;
    }
}

// -------------------------------------------------------------- locate ----
// Pre-order, left-first traversal of the kd-tree with each node bounded by
// the union of its leaves' expanded boxes.  Leaves are numbered in the same
// order, so the first leaf whose box contains the point is the smallest such
// index (canonical rule for the ray cast's arbitrary hit).
// Point location on the 8-wide tree: a depth-first search whose stack holds
// references to containing children, pushed last-first so that children pop
// in pre-order; the first leaf popped is the smallest containing leaf (every
// ancestor of a containing leaf contains the point, because node bounds are
// unions).  The first kTopWide wide nodes (breadth-first: the top three wide
// levels, nine binary levels) are copied into shared memory by every block.
constexpr int kTopWide = 73;
constexpr int kLocStack = 64;
constexpr int64_t kTreePrefetchLines = (32ll << 20) / 128;  // at most the first 32 MB

// One wide-tree step shared by the locate kernels: the containing children of
// wide node w pushed last-first onto the stack.
__device__ __forceinline__ void push_containing(const WideNode* w, bool shared_copy, float x, float y,
                                                float z, int* stack, int& sp) {
  float4 b[12];  // lo x, lo y, lo z, hi x, hi y, hi z: two float4 each
  int4 ch[2];
  if (shared_copy) {
#pragma unroll
    for (int u = 0; u < 12; ++u) b[u] = reinterpret_cast<const float4*>(w)[u];
    ch[0] = reinterpret_cast<const int4*>(w->child)[0];
    ch[1] = reinterpret_cast<const int4*>(w->child)[1];
  } else {
#pragma unroll
    for (int u = 0; u < 12; ++u) b[u] = __ldg(reinterpret_cast<const float4*>(w) + u);
    ch[0] = __ldg(reinterpret_cast<const int4*>(w->child));
    ch[1] = __ldg(reinterpret_cast<const int4*>(w->child) + 1);
  }
  const float* lo = reinterpret_cast<const float*>(b);
  const float* hi = lo + 24;
  const int* child = reinterpret_cast<const int*>(ch);
#pragma unroll
  for (int c = kWide - 1; c >= 0; --c) {
    const bool in = lo[c] <= x && x <= hi[c] && lo[8 + c] <= y && y <= hi[8 + c] && lo[16 + c] <= z &&
                    z <= hi[16 + c];
    if (in && sp < kLocStack) stack[sp++] = child[c];
  }
}


// The first three coordinates of point i (rows of `stride` floats; a search
// space of fewer than three dimensions has zeros beyond them, as the kd-tree
// build pads them).
__device__ __forceinline__ void load_xyz(const float* __restrict__ pts, int64_t i, int stride, float& x,
                                         float& y, float& z) {
  const float* p = pts + i * stride;
  x = p[0];
  y = stride > 1 ? p[1] : 0.0f;
  z = stride > 2 ? p[2] : 0.0f;
}

// Requests the first `lines` 128-byte lines of the wide tree into L2, spread
// over the grid's threads, so that the searches' deeper levels find their
// nodes in L2 rather than in DRAM.
__device__ __forceinline__ void prefetch_tree(const WideNode* wide, int n_wide) {
  const int64_t lines = min((int64_t)n_wide * (int64_t)sizeof(WideNode) / 128, (int64_t)kTreePrefetchLines);
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nt = (int64_t)gridDim.x * blockDim.x;
  for (int64_t l = t; l < lines; l += nt)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<const char*>(wide) + l * 128));
}

// kTop: the first kTopWide nodes are copied into shared memory by every
// block.  Without it the kernel uses no shared memory, so its blocks can sit
// beside a kernel that takes most of an SM's shared memory (the learned
// head's GEMMs, which it runs beside).
template <bool kTop>
__global__ void locate_points(const WideNode* __restrict__ wide, int n_wide,
                              const float* __restrict__ pts, int64_t n, int stride,
                              int32_t* __restrict__ out, const int* __restrict__ n_dev) {
  __shared__ WideNode top[kTop ? kTopWide : 1];
  if (n_dev) n = min(n, (int64_t)*n_dev);
  if ((int64_t)blockIdx.x * blockDim.x >= n) return;
  prefetch_tree(wide, n_wide);
  const int ntop = kTop ? min(kTopWide, n_wide) : 0;
  if (kTop) {
    const float4* src = reinterpret_cast<const float4*>(wide);
    float4* dst = reinterpret_cast<float4*>(top);
    for (int i = threadIdx.x; i < 16 * ntop; i += blockDim.x) dst[i] = __ldg(src + i);
    __syncthreads();
  }
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x, y, z;
  load_xyz(pts, i, stride, x, y, z);
  int stack[kLocStack];
  int sp = 0;
  stack[sp++] = 0;
  int32_t hit = 0;
  while (sp > 0) {
    const int ref = stack[--sp];
    if (ref < 0) {  // a containing leaf: the first in pre-order
      hit = -ref - 1;
      break;
    }
    push_containing(ref < ntop ? top + ref : wide + ref, ref < ntop, x, y, z, stack, sp);
  }
  out[i] = hit;
}

// locate_points, continued past the first leaf.
__global__ void locate_points_multi(const WideNode* __restrict__ wide, int n_wide,
                                    const float* __restrict__ pts, int64_t n, int stride, int H,
                                    int32_t* __restrict__ out) {
  __shared__ WideNode top[kTopWide];
  if ((int64_t)blockIdx.x * blockDim.x >= n) return;
  const int ntop = min(kTopWide, n_wide);
  {
    const float4* src = reinterpret_cast<const float4*>(wide);
    float4* dst = reinterpret_cast<float4*>(top);
    for (int i = threadIdx.x; i < 16 * ntop; i += blockDim.x) dst[i] = __ldg(src + i);
    __syncthreads();
  }
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x, y, z;
  load_xyz(pts, i, stride, x, y, z);
  int stack[kLocStack];
  int sp = 0;
  stack[sp++] = 0;
  int found = 0;
  while (sp > 0 && found < H) {
    const int ref = stack[--sp];
    if (ref < 0) {
      out[i * H + found++] = -ref - 1;
      continue;
    }
    push_containing(ref < ntop ? top + ref : wide + ref, ref < ntop, x, y, z, stack, sp);
  }
  if (found == 0) out[i * H + found++] = 0;
  for (; found < H; ++found) out[i * H + found] = -1;
}

// Point location inside the predicted subtree, on the 8-wide tree: the same
// pre-order search from the subtree's wide node; the subtree's first leaf
// when none of its leaves contains the point.
__global__ void locate_in_subtree_wide(const WideNode* __restrict__ wide,
                                       const float* __restrict__ pts, int64_t n, int stride,
                                       const unsigned long long* __restrict__ keys,
                                       const int32_t* __restrict__ start_ref,
                                       const int32_t* __restrict__ fallback_leaf, int n_classes,
                                       const int* __restrict__ n_dev, int32_t* __restrict__ out) {
  if (n_dev) n = min(n, (int64_t)*n_dev);  // graph replay: points beyond the batch are idle
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = 0x7fffffff - (int)(keys[i] & 0xffffffffu);
  if (c < 0 || c >= n_classes) {  // no key (the head wrote none): leaf 0, as on a miss
    out[i] = 0;
    return;
  }
  float x, y, z;
  load_xyz(pts, i, stride, x, y, z);
  int stack[kLocStack];
  int sp = 0;
  stack[sp++] = start_ref[c];
  int32_t hit = fallback_leaf[c];
  while (sp > 0) {
    const int ref = stack[--sp];
    if (ref < 0) {
      hit = -ref - 1;
      break;
    }
    push_containing(wide + ref, false, x, y, z, stack, sp);
  }
  out[i] = hit;
}

// Point location inside one subtree per point: the traversal starts at
// start_node[cls[i]] instead of the root; when no leaf box of that subtree
// contains the point, the subtree's first leaf (fallback_leaf[cls[i]]).
// Used by the learned entry, whose model predicts the subtree.
__global__ void locate_in_subtree(const BvhNode* __restrict__ nodes, const float* __restrict__ pts,
                                  int64_t n, int stride, const int32_t* __restrict__ cls,
                                  const unsigned long long* __restrict__ keys,
                                  const int32_t* __restrict__ start_node,
                                  const int32_t* __restrict__ fallback_leaf, int n_classes,
                                  int32_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // the class is given, or decoded from the packed argmax key (gemm_tc.h)
  const int c = keys ? 0x7fffffff - (int)(keys[i] & 0xffffffffu) : cls[i];
  if (c < 0 || c >= n_classes) {  // no key (the head wrote none): leaf 0, as on a miss
    out[i] = 0;
    return;
  }
  float x, y, z;
  load_xyz(pts, i, stride, x, y, z);
  int stack[kBvhMaxDepth];
  int sp = 0;
  stack[sp++] = start_node[c];
  int32_t hit = fallback_leaf[c];
  while (sp > 0) {
    const BvhNode nd = nodes[stack[--sp]];
    if (!(nd.lo[0] <= x && x <= nd.hi[0] && nd.lo[1] <= y && y <= nd.hi[1] && nd.lo[2] <= z &&
          z <= nd.hi[2]))
      continue;
    if (nd.left < 0) {
      hit = -nd.left - 1;
      break;
    }
    if (sp + 2 > kBvhMaxDepth) break;
    stack[sp++] = nd.right;
    stack[sp++] = nd.left;
  }
  out[i] = hit;
}

// One warp per row: the squared norm of the BF16 row, summed in FP64 in a
// fixed order (lane partials, then a butterfly), rounded to FP32.
__global__ void bf16_norms(const uint16_t* __restrict__ il16, int64_t n, int C,
                           float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n; r += nwarps) {
    const uint16_t* row = il16 + r * 32 * C;
    double s = 0.0;
    for (int e = lane; e < 32 * C; e += 32) {
      const double v = (double)__uint_as_float((uint32_t)row[e] << 16);
      s += v * v;
    }
    for (int off = 16; off >= 1; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) out[r] = (float)s;
  }
}

// -------------------------------------------------------------- launches ----
cudaError_t launch_locate_in_subtree(const BvhNode* nodes, const float* pts, int64_t n, int stride,
                                     const int32_t* cls, const unsigned long long* keys,
                                     const int32_t* start_node, const int32_t* fallback_leaf,
                                     int n_classes, int32_t* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (!cls == !keys) return cudaErrorInvalidValue;
  locate_in_subtree<<<(unsigned)((n + 63) / 64), 64, 0, st>>>(nodes, pts, n, stride, cls, keys,
                                                                start_node, fallback_leaf, n_classes, out);
  return cudaGetLastError();
}

cudaError_t launch_mean(const float* x, int64_t n, int d, double* partial, int nblocks,
                        double* mean, cudaStream_t st) {
  const int64_t rpb = (n + nblocks - 1) / nblocks;
  col_sum_partial<<<nblocks, 128, 0, st>>>(x, n, d, rpb, partial);
  col_sum_finish<<<(d + 127) / 128, 128, 0, st>>>(partial, nblocks, d, n, mean);
  return cudaGetLastError();
}

cudaError_t launch_cov(const float* x, int64_t n, int d, const double* mean, double* partial,
                       int nchunks, double* cov, cudaStream_t st) {
  const int64_t rpc = (n + nchunks - 1) / nchunks;
  dim3 grid((d + kCovTile - 1) / kCovTile, (d + kCovTile - 1) / kCovTile, nchunks);
  cov_partial<<<grid, dim3(16, 16), 0, st>>>(x, n, d, mean, rpc, partial);
  const int64_t dd = (int64_t)d * d;
  cov_finish<<<(unsigned)((dd + 255) / 256), 256, 0, st>>>(partial, nchunks, d, n, cov);
  return cudaGetLastError();
}

cudaError_t launch_project(const float* x, int64_t n, int d, int xstride, const float* mean,
                           const float* V, int vstride, int k, float* out, int ostride,
                           cudaStream_t st, uint32_t* zero, int64_t zero_words, const float* vt_split) {
  if (n == 0) return cudaSuccess;
  if (vt_split) {
    const cudaError_t e = launch_project_tc(x, n, nullptr, d, xstride, mean, vt_split, k, out, ostride, nullptr,
                                            0.0f, 0, zero, zero_words, nullptr, st);
    if (e != cudaErrorNotSupported) return e;
  }
  dim3 grid((unsigned)((n + kPrRows - 1) / kPrRows), (k + kPrCols - 1) / kPrCols);
  project_rows<false><<<grid, kPrThreads, 0, st>>>(x, n, d, xstride, mean, V, vstride, k, out, ostride,
                                            nullptr, nullptr, 0.0f, 0, zero, zero_words);
  return cudaGetLastError();
}

cudaError_t launch_project_bf16(const float* x, int64_t n, int d, int xstride, const float* mean,
                                const float* V, int vstride, int k, float* out, int ostride,
                                void* out16, float s16, int ld16, cudaStream_t st, uint32_t* zero,
                                int64_t zero_words, const float* vt_split) {
  if (n == 0) return cudaSuccess;
  if (ld16 < k || ld16 > ((k + kPrCols - 1) / kPrCols) * kPrCols) return cudaErrorInvalidValue;
  if (vt_split) {
    const cudaError_t e = launch_project_tc(x, n, nullptr, d, xstride, mean, vt_split, k, out, ostride, out16,
                                            s16, ld16, zero, zero_words, nullptr, st);
    if (e != cudaErrorNotSupported) return e;
  }
  dim3 grid((unsigned)((n + kPrRows - 1) / kPrRows), (k + kPrCols - 1) / kPrCols);
  project_rows<true><<<grid, kPrThreads, 0, st>>>(x, n, d, xstride, mean, V, vstride, k, out, ostride, nullptr,
                                           reinterpret_cast<__nv_bfloat16*>(out16), s16, ld16, zero,
                                           zero_words);
  return cudaGetLastError();
}

cudaError_t launch_project_dyn(const float* x, int64_t cap, const int* n_dev, int d, int xstride,
                               const float* mean, const float* V, int vstride, int k, float* out,
                               int ostride, cudaStream_t st, const float* vt_split) {
  if (vt_split) {
    const cudaError_t e = launch_project_tc(x, cap, n_dev, d, xstride, mean, vt_split, k, out, ostride, nullptr,
                                            0.0f, 0, nullptr, 0, nullptr, st);
    if (e != cudaErrorNotSupported) return e;
  }
  dim3 grid((unsigned)((cap + kPrRows - 1) / kPrRows), (k + kPrCols - 1) / kPrCols);
  project_rows<false><<<grid, kPrThreads, 0, st>>>(x, cap, d, xstride, mean, V, vstride, k, out, ostride,
                                            n_dev, nullptr, 0.0f, 0, nullptr, 0);
  return cudaGetLastError();
}

cudaError_t launch_project_bf16_dyn(const float* x, int64_t cap, const int* n_dev, int d, int xstride,
                                    const float* mean, const float* V, int vstride, int k, float* out,
                                    int ostride, void* out16, float s16, int ld16, uint32_t* zero,
                                    int64_t zero_words, cudaStream_t st, const float* vt_split) {
  if (ld16 < k || ld16 > ((k + kPrCols - 1) / kPrCols) * kPrCols) return cudaErrorInvalidValue;
  if (vt_split) {
    const cudaError_t e = launch_project_tc(x, cap, n_dev, d, xstride, mean, vt_split, k, out, ostride, out16,
                                            s16, ld16, zero, zero_words, nullptr, st);
    if (e != cudaErrorNotSupported) return e;
  }
  dim3 grid((unsigned)((cap + kPrRows - 1) / kPrRows), (k + kPrCols - 1) / kPrCols);
  project_rows<true><<<grid, kPrThreads, 0, st>>>(x, cap, d, xstride, mean, V, vstride, k, out, ostride, n_dev,
                                                  reinterpret_cast<__nv_bfloat16*>(out16), s16, ld16, zero,
                                                  zero_words);
  return cudaGetLastError();
}

cudaError_t launch_lowp_copies(const float* il32, int64_t n, int C, void* il16, uint8_t* il8,
                               float* scale8, cudaStream_t st) {
  const int64_t blocks = std::min<int64_t>((n + 7) / 8, 65535 * 8);
  lowp_from_il32<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, st>>>(
      il32, n, C, reinterpret_cast<__nv_bfloat16*>(il16), il8, scale8);
  return cudaGetLastError();
}

cudaError_t launch_interleave(const float* src, int64_t n, int d, int C, float* il32,
                              void* il16, uint8_t* il8, float* scale8, float* xyz,
                              cudaStream_t st) {
  const int64_t blocks = std::min<int64_t>((n + 7) / 8, 65535 * 8);
  interleave_rows<<<(unsigned)blocks, 256, 0, st>>>(src, n, d, C, il32,
                                                    reinterpret_cast<__nv_bfloat16*>(il16), il8,
                                                    scale8, xyz);
  return cudaGetLastError();
}

cudaError_t launch_deinterleave(const float* il32, int64_t n, int d, int C, float* dst,
                                cudaStream_t st) {
  const int64_t blocks = std::min<int64_t>((n + 7) / 8, 65535 * 8);
  deinterleave_rows<<<(unsigned)blocks, 256, 0, st>>>(il32, n, d, C, dst);
  return cudaGetLastError();
}

cudaError_t launch_bf16_norms(const uint16_t* il16, int64_t n, int C, float* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((n + 7) / 8, 4096);
  bf16_norms<<<(unsigned)blocks, 256, 0, st>>>(il16, n, C, out);
  return cudaGetLastError();
}

cudaError_t launch_dequant(const void* il, const float* scale8, int precision, int64_t n, int d,
                           int C, float* dst, cudaStream_t st) {
  const int64_t blocks = std::min<int64_t>((n + 7) / 8, 65535 * 8);
  dequant_rows<<<(unsigned)blocks, 256, 0, st>>>(il, scale8, precision, n, d, C, dst);
  return cudaGetLastError();
}

// 64 points per block: enough blocks to spread a batch of a few thousand
// points over every SM (each block copies the top of the tree once).
cudaError_t launch_locate_in_subtree_wide(const WideNode* wide, const float* pts, int64_t n,
                                          int stride, const unsigned long long* keys,
                                          const int32_t* start_ref, const int32_t* fallback_leaf,
                                          int n_classes, int32_t* out, cudaStream_t st,
                                          const int* n_dev) {
  if (n == 0) return cudaSuccess;
  locate_in_subtree_wide<<<(unsigned)((n + 63) / 64), 64, 0, st>>>(wide, pts, n, stride, keys,
                                                                     start_ref, fallback_leaf, n_classes,
                                                                     n_dev, out);
  return cudaGetLastError();
}

cudaError_t launch_locate_multi(const WideNode* wide, int n_wide, const float* pts, int64_t n,
                                int stride, int H, int32_t* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  locate_points_multi<<<(unsigned)((n + 63) / 64), 64, 0, st>>>(wide, n_wide, pts, n, stride, H, out);
  return cudaGetLastError();
}

cudaError_t launch_locate(const WideNode* wide, int n_wide, const float* pts, int64_t n, int stride,
                          int32_t* out, cudaStream_t st, bool top_cache) {
  if (n == 0) return cudaSuccess;
  if (top_cache)
    locate_points<true><<<(unsigned)((n + 63) / 64), 64, 0, st>>>(wide, n_wide, pts, n, stride, out, nullptr);
  else
    locate_points<false><<<(unsigned)((n + 63) / 64), 64, 0, st>>>(wide, n_wide, pts, n, stride, out, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_locate_dyn(const WideNode* wide, int n_wide, const float* pts, int64_t cap,
                              const int* n_dev, int stride, int32_t* out, cudaStream_t st, bool top_cache) {
  if (top_cache)
    locate_points<true><<<(unsigned)((cap + 63) / 64), 64, 0, st>>>(wide, n_wide, pts, cap, stride, out, n_dev);
  else
    locate_points<false><<<(unsigned)((cap + 63) / 64), 64, 0, st>>>(wide, n_wide, pts, cap, stride, out, n_dev);
  return cudaGetLastError();
}

// Counting sort of the queries by leaf range: count per range, exclusive
// scan of the counts, then scatter.  Shared-memory atomics: 4096 counters
// leave few collisions for batches of up to a few hundred thousand queries.
constexpr int kOrderBins = 4096;
constexpr int kOrderThreads = 1024;
constexpr int kOrderKeys = 8;

// A range of 2^shift consecutive leaves per counter (shift: the smallest
// that maps the last leaf below kOrderBins).
__device__ __forceinline__ int order_bin(int32_t leaf, int n_leaves, int shift) {
  if (leaf < 0 || leaf >= n_leaves) leaf = 0;
  return leaf >> shift;
}

__global__ void __launch_bounds__(kOrderThreads) order_by_leaf_kernel(const int32_t* __restrict__ leaf,
                                                                      int stride, int64_t n, int n_leaves,
                                                                      int shift, int32_t* __restrict__ order,
                                                                      const int* n_dev, int64_t min_n) {
  __shared__ int cnt[kOrderBins];
  __shared__ int wsum[kOrderThreads / 32];
  if (n_dev) {  // the live count, at most the capacity n
    const int64_t live = *n_dev;
    n = live < 0 ? 0 : live < n ? live : n;
  }
  if (n <= min_n) return;  // the whole block returns: n is uniform
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < kOrderBins; i += kOrderThreads) cnt[i] = 0;
  __syncthreads();
  // each thread issues kOrderKeys independent loads per loop trip, so that
  // a batch of up to kOrderKeys * 1024 queries costs one memory latency per
  // pass rather than a chain of them
  for (int64_t r0 = 0; r0 < n; r0 += (int64_t)kOrderKeys * kOrderThreads) {
    int b[kOrderKeys];
#pragma unroll
    for (int j = 0; j < kOrderKeys; ++j) {
      const int64_t q = r0 + (int64_t)j * kOrderThreads + tid;
      b[j] = q < n ? order_bin(leaf[q * stride], n_leaves, shift) : -1;
    }
#pragma unroll
    for (int j = 0; j < kOrderKeys; ++j)
      if (b[j] >= 0) atomicAdd(&cnt[b[j]], 1);
  }
  __syncthreads();
  // exclusive scan: thread t owns the ranges [per * t, per * t + per)
  constexpr int per = kOrderBins / kOrderThreads;
  int v[per];
  int own = 0;
#pragma unroll
  for (int j = 0; j < per; ++j) {
    v[j] = cnt[tid * per + j];
    own += v[j];
  }
  int inc = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const int w = wsum[lane];
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    wsum[lane] = wi - w;
  }
  __syncthreads();
  int at = wsum[warp] + inc - own;
#pragma unroll
  for (int j = 0; j < per; ++j) {
    cnt[tid * per + j] = at;
    at += v[j];
  }
  __syncthreads();
  for (int64_t r0 = 0; r0 < n; r0 += (int64_t)kOrderKeys * kOrderThreads) {
    int b[kOrderKeys];
#pragma unroll
    for (int j = 0; j < kOrderKeys; ++j) {
      const int64_t q = r0 + (int64_t)j * kOrderThreads + tid;
      b[j] = q < n ? order_bin(leaf[q * stride], n_leaves, shift) : -1;
    }
#pragma unroll
    for (int j = 0; j < kOrderKeys; ++j)
      if (b[j] >= 0) order[atomicAdd(&cnt[b[j]], 1)] = (int32_t)(r0 + (int64_t)j * kOrderThreads + tid);
  }
}

cudaError_t launch_order_by_leaf(const int32_t* leaf, int stride, int64_t n, int n_leaves,
                                 int32_t* order, cudaStream_t st, const int* n_dev, int64_t min_n) {
  if (n <= 0) return cudaSuccess;
  if (n > INT32_MAX || n_leaves < 1 || stride < 1) return cudaErrorInvalidValue;
  int shift = 0;
  while (((n_leaves - 1) >> shift) >= kOrderBins) ++shift;
  order_by_leaf_kernel<<<1, kOrderThreads, 0, st>>>(leaf, stride, n, n_leaves, shift, order, n_dev, min_n);
  return cudaGetLastError();
}

}  // namespace rte
