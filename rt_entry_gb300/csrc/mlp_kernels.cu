// mlp_kernels.cu -- element-wise and reduction kernels of the learned-entry
// MLP (BF16 storage, FP32 arithmetic).  The GEMMs are gemm_tc.cu.
#include <algorithm>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp_kernels.h"

namespace rte {

// out[r][c] = bf16(x[r][c] * scale) for c < d, 0 for d <= c < dp.
__global__ void cast_rows_bf16_k(const float* __restrict__ x, int64_t rows, int d, int ld,
                                 float scale, int dp, __nv_bfloat16* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * dp) return;
  const int64_t r = i / dp;
  const int c = (int)(i % dp);
  out[i] = __float2bfloat16_rn(c < d ? x[r * ld + c] * scale : 0.0f);
}

// out[c][r] = in[r][c] through 32x32 shared-memory tiles.
__global__ void transpose_bf16_k(const __nv_bfloat16* __restrict__ in, int R, int C,
                                 __nv_bfloat16* __restrict__ out) {
  __shared__ __nv_bfloat16 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = r0 + j, c = c0 + threadIdx.x;
    if (r < R && c < C) t[j][threadIdx.x] = in[(int64_t)r * C + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int c = c0 + j, r = r0 + threadIdx.x;
    if (r < R && c < C) out[(int64_t)c * R + r] = t[threadIdx.x][j];
  }
}

// Row-wise softmax cross-entropy: loss[m] = logsumexp(z_m) - z_m[y_m];
// dz[m][c] = (softmax(z_m)[c] - [c == y_m]) * inv_m, stored as BF16.
__global__ void softmax_ce_k(const float* __restrict__ z, int M, int C, const int32_t* __restrict__ y,
                             float inv_m, __nv_bfloat16* __restrict__ dz, float* __restrict__ loss) {
  const int m = blockIdx.x;
  const float* row = z + (int64_t)m * C;
  __shared__ float red[32];
  float mx = -3.402823466e38f;
  for (int c = threadIdx.x; c < C; c += blockDim.x) mx = fmaxf(mx, row[c]);
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : -3.402823466e38f;
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  mx = red[0];
  __syncthreads();
  float s = 0.f;
  for (int c = threadIdx.x; c < C; c += blockDim.x) s += __expf(row[c] - mx);
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.f;
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  const float sum = red[0];
  const float inv = 1.0f / sum;
  const int label = y[m];
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    float p = __expf(row[c] - mx) * inv;
    if (c == label) p -= 1.0f;
    dz[(int64_t)m * C + c] = __float2bfloat16_rn(p * inv_m);
  }
  if (threadIdx.x == 0 && loss) loss[m] = logf(sum) + mx - row[label];
}

// out = bf16(g * (h > 0)).
__global__ void relu_grad_k(const float* __restrict__ g, const __nv_bfloat16* __restrict__ h,
                            int64_t n, __nv_bfloat16* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = __float2bfloat16_rn(__bfloat162float(h[i]) > 0.f ? g[i] : 0.f);
}

// Column sums out[n] = sum over m of x[m][n] (BF16 input, FP32 sums) in two
// passes with a fixed order, so results are reproducible: block (bx, by)
// takes columns 32 bx .. 32 bx + 31 and row slice by (rows by*rs ..
// by*rs + rs - 1); its thread (c, r) sums rows r, r + 8, ... of the slice
// for column c, the eight row lanes are added in lane order, and
// part[by][n] receives the slice's sum.  The second pass adds the slices in
// order.
constexpr int kColSumRowLanes = 8;
__global__ void col_sum_part_k(const __nv_bfloat16* __restrict__ x, int M, int N, int rs,
                               float* __restrict__ part) {
  __shared__ float sh[kColSumRowLanes][32];
  const int c = threadIdx.x, r = threadIdx.y;
  const int n = blockIdx.x * 32 + c;
  const int m0 = blockIdx.y * rs, m1 = min(M, m0 + rs);
  float s = 0.f;
  if (n < N) {
#pragma unroll 4
    for (int m = m0 + r; m < m1; m += kColSumRowLanes) s += __bfloat162float(x[(int64_t)m * N + n]);
  }
  sh[r][c] = s;
  __syncthreads();
  if (r == 0 && n < N) {
    float t = sh[0][c];
#pragma unroll
    for (int i = 1; i < kColSumRowLanes; ++i) t += sh[i][c];
    part[(int64_t)blockIdx.y * N + n] = t;
  }
}

__global__ void col_sum_finish_k(const float* __restrict__ part, int slices, int N, float* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int i = 0; i < slices; ++i) s += part[(int64_t)i * N + n];
  out[n] = s;
}

// Adam on FP32 master weights; refreshes the BF16 copy.
__global__ void adam_k(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, int64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2, __nv_bfloat16* __restrict__ w16) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  const float upd = lr * (a * c1) / (sqrtf(b * c2) + eps);
  const float nw = w[i] - upd;
  w[i] = nw;
  if (w16) w16[i] = __float2bfloat16_rn(nw);
}

__global__ void f32_to_bf16_k(const float* __restrict__ x, int64_t n, __nv_bfloat16* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2bfloat16_rn(x[i]);
}

__global__ void gather_rows_k(const __nv_bfloat16* __restrict__ src, int dp,
                              const int64_t* __restrict__ idx, int rows,
                              const int32_t* __restrict__ labels_src, __nv_bfloat16* __restrict__ dst,
                              int32_t* __restrict__ labels_dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)rows * dp) return;
  const int r = (int)(i / dp), c = (int)(i % dp);
  const int64_t s = idx[r];
  dst[i] = src[s * dp + c];
  if (c == 0) labels_dst[r] = labels_src[s];
}

// argmax key -> class column; class -> leaf through class_leaf (null: identity).
// A zero key (no column was a maximum: every logit NaN) gives -1.
__global__ void argmax_to_leaf_k(const unsigned long long* __restrict__ keys, int n,
                                 const int32_t* __restrict__ class_leaf, int32_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (keys[i] == 0ull) {
    out[i] = -1;
    return;
  }
  const int col = 0x7fffffff - (int)(keys[i] & 0xffffffffu);
  out[i] = class_leaf ? class_leaf[col] : col;
}

static unsigned blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

cudaError_t launch_cast_rows_bf16(const float* x, int64_t rows, int d, int ld, float scale, int dp,
                                  void* out, cudaStream_t st) {
  if (rows == 0) return cudaSuccess;
  cast_rows_bf16_k<<<blocks(rows * dp, 256), 256, 0, st>>>(x, rows, d, ld, scale, dp,
                                                          (__nv_bfloat16*)out);
  return cudaGetLastError();
}
cudaError_t launch_transpose_bf16(const void* in, int R, int C, void* out, cudaStream_t st) {
  dim3 grid((C + 31) / 32, (R + 31) / 32);
  transpose_bf16_k<<<grid, dim3(32, 8), 0, st>>>((const __nv_bfloat16*)in, R, C, (__nv_bfloat16*)out);
  return cudaGetLastError();
}
cudaError_t launch_softmax_ce(const float* z, int M, int C, const int32_t* y, float inv_m, void* dz,
                              float* loss, cudaStream_t st) {
  softmax_ce_k<<<M, 512, 0, st>>>(z, M, C, y, inv_m, (__nv_bfloat16*)dz, loss);
  return cudaGetLastError();
}
cudaError_t launch_relu_grad(const float* g, const void* h, int64_t n, void* out, cudaStream_t st) {
  relu_grad_k<<<blocks(n, 256), 256, 0, st>>>(g, (const __nv_bfloat16*)h, n, (__nv_bfloat16*)out);
  return cudaGetLastError();
}
int col_sum_slices(int M) { return std::max(1, std::min(kColSumMaxSlices, M / 256)); }
cudaError_t launch_col_sum_bf16(const void* x, int M, int N, float* out, float* part, cudaStream_t st) {
  const int slices = col_sum_slices(M);
  const int rs = (M + slices - 1) / slices;
  col_sum_part_k<<<dim3((N + 31) / 32, slices), dim3(32, kColSumRowLanes), 0, st>>>(
      (const __nv_bfloat16*)x, M, N, rs, part);
  col_sum_finish_k<<<blocks(N, 256), 256, 0, st>>>(part, slices, N, out);
  return cudaGetLastError();
}
cudaError_t launch_adam(float* w, const float* g, float* m1, float* m2, int64_t n, float lr,
                        float b1, float b2, float eps, float c1, float c2, void* w16,
                        cudaStream_t st) {
  adam_k<<<blocks(n, 256), 256, 0, st>>>(w, g, m1, m2, n, lr, b1, b2, eps, c1, c2,
                                          (__nv_bfloat16*)w16);
  return cudaGetLastError();
}
cudaError_t launch_f32_to_bf16(const float* x, int64_t n, void* out, cudaStream_t st) {
  f32_to_bf16_k<<<blocks(n, 256), 256, 0, st>>>(x, n, (__nv_bfloat16*)out);
  return cudaGetLastError();
}
cudaError_t launch_gather_rows(const void* src, int dp, const int64_t* idx, int rows,
                               const int32_t* labels_src, void* dst, int32_t* labels_dst,
                               cudaStream_t st) {
  gather_rows_k<<<blocks((int64_t)rows * dp, 256), 256, 0, st>>>(
      (const __nv_bfloat16*)src, dp, idx, rows, labels_src, (__nv_bfloat16*)dst, labels_dst);
  return cudaGetLastError();
}
cudaError_t launch_argmax_to_leaf(const unsigned long long* keys, int n, const int32_t* class_leaf,
                                  int32_t* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  argmax_to_leaf_k<<<blocks(n, 256), 256, 0, st>>>(keys, n, class_leaf, out);
  return cudaGetLastError();
}

}  // namespace rte
