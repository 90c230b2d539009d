// layout.cuh -- lane-interleaved row layout of the search-space base.
//
// A row of d values is stored as C = ceil(d/32) "chunks" of 32 values; chunk
// c holds dims 32c .. 32c+31 and lane l of a warp owns dim l + 32c of every
// chunk, which is the assignment the reference's distance code uses
// (graph_search.cuh:500-878: lane l loads d_data[p*DIM + lane + 32c]).
// Within a row the chunks are packed so that each lane's values are
// contiguous and one warp-wide vector load moves them:
//   chunks 4s..4s+3 -> slab s: 32 lanes x 4 values   (one 128-bit load for FP32)
//   next two chunks -> 32 lanes x 2 values           (when C % 4 >= 2)
//   last odd chunk  -> 32 lanes x 1 value            (when C is odd)
// Element offset of (chunk c, lane l) is interleaved_offset(c, l, C); a row
// takes 32*C elements (dims >= d are stored as 0, which adds nothing to a
// squared distance).  The same offsets are used for the FP32, BF16 and
// FP8-E4M3 copies, so each copy is one coalesced gather per row.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <stdint.h>

namespace rte {

__host__ __device__ inline int interleaved_offset(int c, int lane, int C) {
  const int n4 = C >> 2, rem = C & 3;
  if (c < 4 * n4) return 128 * (c >> 2) + 4 * lane + (c & 3);
  if (rem >= 2 && c < 4 * n4 + 2) return 128 * n4 + 2 * lane + (c - 4 * n4);
  return 128 * n4 + (rem >= 2 ? 64 : 0) + lane;
}

template <int C>
__device__ __forceinline__ void load_interleaved(const float* __restrict__ row, int lane,
                                                 float (&v)[C]) {
  constexpr int n4 = C / 4, rem = C % 4;
#pragma unroll
  for (int s = 0; s < n4; ++s) {
    const float4 x = __ldg(reinterpret_cast<const float4*>(row + 128 * s) + lane);
    v[4 * s + 0] = x.x;
    v[4 * s + 1] = x.y;
    v[4 * s + 2] = x.z;
    v[4 * s + 3] = x.w;
  }
  int off = 128 * n4;
  if (rem >= 2) {
    const float2 y = __ldg(reinterpret_cast<const float2*>(row + off) + lane);
    v[4 * n4 + 0] = y.x;
    v[4 * n4 + 1] = y.y;
    off += 64;
  }
  if (rem & 1) v[C - 1] = __ldg(row + off + lane);
}

__device__ __forceinline__ float bf16lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

template <int C>
__device__ __forceinline__ void load_interleaved_bf16(const __nv_bfloat16* __restrict__ row,
                                                      int lane, float (&v)[C]) {
  constexpr int n4 = C / 4, rem = C % 4;
  const uint16_t* r = reinterpret_cast<const uint16_t*>(row);
#pragma unroll
  for (int s = 0; s < n4; ++s) {
    const uint2 x = __ldg(reinterpret_cast<const uint2*>(r + 128 * s) + lane);
    v[4 * s + 0] = bf16lo(x.x);
    v[4 * s + 1] = bf16hi(x.x);
    v[4 * s + 2] = bf16lo(x.y);
    v[4 * s + 3] = bf16hi(x.y);
  }
  int off = 128 * n4;
  if (rem >= 2) {
    const uint32_t y = __ldg(reinterpret_cast<const unsigned int*>(r + off) + lane);
    v[4 * n4 + 0] = bf16lo(y);
    v[4 * n4 + 1] = bf16hi(y);
    off += 64;
  }
  if (rem & 1) v[C - 1] = __uint_as_float((uint32_t)__ldg(r + off + lane) << 16);
}

__device__ __forceinline__ float2 fp8x2_to_float2(uint16_t w) {
  const __half2_raw h = __nv_cvt_fp8x2_to_halfraw2((__nv_fp8x2_storage_t)w, __NV_E4M3);
  const __half2 hh = *reinterpret_cast<const __half2*>(&h);
  return __half22float2(hh);
}

template <int C>
__device__ __forceinline__ void load_interleaved_fp8(const uint8_t* __restrict__ row, int lane,
                                                     float (&v)[C]) {
  constexpr int n4 = C / 4, rem = C % 4;
#pragma unroll
  for (int s = 0; s < n4; ++s) {
    const uint32_t x = __ldg(reinterpret_cast<const unsigned int*>(row + 128 * s) + lane);
    const float2 a = fp8x2_to_float2((uint16_t)(x & 0xffffu));
    const float2 b = fp8x2_to_float2((uint16_t)(x >> 16));
    v[4 * s + 0] = a.x;
    v[4 * s + 1] = a.y;
    v[4 * s + 2] = b.x;
    v[4 * s + 3] = b.y;
  }
  int off = 128 * n4;
  if (rem >= 2) {
    const uint16_t y = __ldg(reinterpret_cast<const unsigned short*>(row + off) + lane);
    const float2 a = fp8x2_to_float2(y);
    v[4 * n4 + 0] = a.x;
    v[4 * n4 + 1] = a.y;
    off += 64;
  }
  if (rem & 1) {
    const uint8_t b = __ldg(row + off + lane);
    v[C - 1] = fp8x2_to_float2((uint16_t)b).x;
  }
}

}  // namespace rte
