// mlp_kernels.h -- launches of the learned-entry MLP's small kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rte {

cudaError_t launch_cast_rows_bf16(const float* x, int64_t rows, int d, int ld, float scale, int dp,
                                  void* out, cudaStream_t st);
cudaError_t launch_transpose_bf16(const void* in, int R, int C, void* out, cudaStream_t st);
cudaError_t launch_softmax_ce(const float* z, int M, int C, const int32_t* y, float inv_m, void* dz,
                              float* loss, cudaStream_t st);
cudaError_t launch_relu_grad(const float* g, const void* h, int64_t n, void* out, cudaStream_t st);
// Column sums of a BF16 [M x N] matrix into out [N] (FP32, fixed order);
// part: scratch of col_sum_slices(M) * N floats.
constexpr int kColSumMaxSlices = 64;
int col_sum_slices(int M);
cudaError_t launch_col_sum_bf16(const void* x, int M, int N, float* out, float* part, cudaStream_t st);
cudaError_t launch_adam(float* w, const float* g, float* m1, float* m2, int64_t n, float lr,
                        float b1, float b2, float eps, float c1, float c2, void* w16,
                        cudaStream_t st);
cudaError_t launch_f32_to_bf16(const float* x, int64_t n, void* out, cudaStream_t st);
cudaError_t launch_gather_rows(const void* src, int dp, const int64_t* idx, int rows,
                               const int32_t* labels_src, void* dst, int32_t* labels_dst,
                               cudaStream_t st);
cudaError_t launch_argmax_to_leaf(const unsigned long long* keys, int n, const int32_t* class_leaf,
                                  int32_t* out, cudaStream_t st);

}  // namespace rte
