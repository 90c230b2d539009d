// mlp_head.h -- the learned head's forward pass in one tcgen05 kernel.
//
//   h1 = relu(X W1^T + b1), h2 = relu(h1 W2^T + b2),
//   keys[m] = max over n of argmax_key(h2 W3^T + b3)   (gemm_tc.h)
//
// X [M][dp], W1 [H][dp], W2 [H][H], W3 [N][H] are row-major BF16; h1 and h2
// are rounded to BF16 exactly as the layer-by-layer GEMMs round them, and
// never leave shared memory.  keys must be zero on entry (atomicMax).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rte {

struct MlpHeadArgs {
  const void* X;
  const void* W1;
  const void* W2;
  const void* W3;
  const float* b1;
  const float* b2;
  const float* b3;
  int M, dp, H, N;
  unsigned long long* keys;  // [M], zero on entry
  int* err;                  // device flag: a bounded wait ran out (non-zero code)
  long long wait_limit;      // try_wait rounds of the pipeline waits (set by the launcher)
  // graph replay: the live row count, read at run time (<= M; the grid and
  // tensor maps are sized for M rows); null for a plain launch
  const int* M_dev = nullptr;
};

// True when the fused kernel takes this shape: H a multiple of 64 up to 256,
// dp a multiple of 8 up to 256, 16-byte aligned operands.
bool mlp_head_supported(const MlpHeadArgs& a);

// The launch attributes (shared-memory size) and the SM count for the
// current device, set once; call it before capturing mlp_head_argmax into a
// CUDA graph.
cudaError_t mlp_head_prepare(int N);

// cudaErrorNotSupported for shapes mlp_head_supported rejects (or when the
// driver's tensor-map encoder is unavailable); the caller then runs the
// three GEMMs.
cudaError_t mlp_head_argmax(const MlpHeadArgs& a, cudaStream_t st);

}  // namespace rte
