// gemm_tc.h -- BF16 tensor-core GEMM for sm_103a (tcgen05 + TMA + TMEM).
//
//   C[M x N] = A[M x K] * B[N x K]^T      (A, B row-major BF16, K contiguous)
//
// with a fused epilogue.  Used by the learned-entry MLP (training and
// inference).  K must be a multiple of 8 (16-byte TMA row strides).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace rte {

enum GemmEpilogue : int {
  kEpiStoreF32 = 0,      // C (FP32) = acc
  kEpiBiasReluBF16 = 1,  // C (BF16) = relu(acc + bias[n])
  kEpiBiasF32 = 2,       // C (FP32) = acc + bias[n]
  kEpiBiasArgmax = 3,    // out_argmax[m] = max over n of (acc + bias[n]), packed (value, n)
  kEpiAccumF32 = 4,      // C (FP32) += acc   (gradient accumulation)
};

struct GemmArgs {
  const void* A;        // BF16 [M][K]
  const void* B;        // BF16 [N][K]
  int M, N, K;
  int epilogue;
  void* C;              // FP32 or BF16 [M][ldc]
  int ldc;
  const float* bias;    // [N] or null
  unsigned long long* out_argmax;  // [M], packed key (see gemm_tc.cu), pre-set to 0
  int* err;             // device flag: set to a non-zero code when a bounded wait runs out
  long long wait_limit; // try_wait rounds of the pipeline waits (set by gemm_bf16_tn)
};

// Returns cudaErrorInvalidValue for unsupported shapes, cudaErrorNotSupported
// when the driver's tensor-map encoder is unavailable.
cudaError_t gemm_bf16_tn(const GemmArgs& g, cudaStream_t st);

// Packed argmax key <-> (value, column).
__host__ __device__ inline unsigned long long argmax_key(float v, int col) {
#ifdef __CUDA_ARCH__
  unsigned int u = __float_as_uint(v);
#else
  unsigned int u;
  memcpy(&u, &v, 4);
#endif
  u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);  // order-preserving
  return ((unsigned long long)u << 32) | (unsigned int)(0x7fffffff - col);  // ties: smaller col
}
__host__ __device__ inline int argmax_col(unsigned long long key) {
  return 0x7fffffff - (int)(key & 0xffffffffu);
}

}  // namespace rte
