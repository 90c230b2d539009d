// rerank_full.h -- exact rerank of final pools against the original rows
// (rerank_full.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rte {

// pool [nq x L] ids (visited marks and padding >= np allowed) -> the first k
// of the ascending exact FP32 distances over base [np x dim] and
// queries [nq x qstride].  L is 16, 32, 64, 128 or 256.
cudaError_t launch_rerank_full(const float* base, int64_t np, int dim, const float* queries,
                               int qstride, const int32_t* pool, int nq, int L, int k,
                               int32_t* out_ids, float* out_dists, int num_sms, cudaStream_t st);

}  // namespace rte
