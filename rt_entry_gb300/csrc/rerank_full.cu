// rerank_full.cu -- exact rerank of final pools against the original rows.
//
// The GPU form of the reference's REORDER step (parallel_reorder,
// graph_helper.cu:146-213): for each query, the FP32 squared L2 distance of
// every pool id over the original (pre-PCA) rows, an ascending sort, the
// first k kept.  It lets the beam search run in a truncated PCA space (fewer
// bytes per row) and still return distances in the original space.
//
// One warp per query.  Distances use the search kernel's FP32 arithmetic
// (per lane s = t0*t0, then fmaf over the dims lane + 32c, then the
// shuffle-down tree 16, 8, 4, 2, 1); the sort is the ascending bitonic
// network of the search kernel's rerank over the L pool slots held in
// registers, so ties are ordered by that network.
#include <cuda_runtime.h>

#include <algorithm>

#include "rerank_full.h"
#include "search_kernel.cuh"

namespace rte {

template <int NL>
__global__ void __launch_bounds__(256) rerank_full_kernel(const float* __restrict__ base, int64_t np,
                                                          int dim, const float* __restrict__ queries,
                                                          int qstride,
                                                          const int32_t* __restrict__ pool, int nq,
                                                          int k, int32_t* __restrict__ out_ids,
                                                          float* __restrict__ out_dists) {
  constexpr int L = pool_slots(NL), PR = pool_regs(NL);
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int nch = (dim + 31) / 32;
  for (int64_t q = warp; q < nq; q += nwarps) {
    const float* qr = queries + q * qstride;
    float pd[PR];
    int pi[PR];
#pragma unroll
    for (int j = 0; j < PR; ++j) {
      pd[j] = kMaxDist;
      pi[j] = (int)np;
    }
    for (int i = 0; i < L; ++i) {
      int id = __ldg(pool + q * L + i);
      id = id < 0 ? -id : id;  // visited marks
      float s = kMaxDist;
      if (id < np) {  // the same id in every lane
        const float* pr = base + (int64_t)id * dim;
        float part = 0.0f;
        for (int c = 0; c < nch; ++c) {
          const int dd = lane + 32 * c;
          const float t = dd < dim ? __fsub_rn(__ldg(pr + dd), __ldg(qr + dd)) : 0.0f;
          part = c == 0 ? __fmul_rn(t, t) : __fmaf_rn(t, t, part);
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) part = __fadd_rn(part, __shfl_down_sync(kFull, part, off));
        s = __shfl_sync(kFull, part, 0);
      }
      if (lane == (i & 31)) {
#pragma unroll
        for (int j = 0; j < PR; ++j)
          if (j == (i >> 5)) {
            pd[j] = s;
            pi[j] = id;
          }
      }
    }
    sort_batch_desc<PR, false, L>(pd, pi, lane);
#pragma unroll
    for (int j = 0; j < PR; ++j) {
      const int i = (j << 5) + lane;
      if (i < k && i < L) {
        out_ids[q * k + i] = pi[j];
        if (out_dists) out_dists[q * k + i] = pd[j];
      }
    }
  }
}

cudaError_t launch_rerank_full(const float* base, int64_t np, int dim, const float* queries,
                               int qstride, const int32_t* pool, int nq, int L, int k,
                               int32_t* out_ids, float* out_dists, int num_sms, cudaStream_t st) {
  if (nq == 0) return cudaSuccess;
  if (k <= 0 || k > L) return cudaErrorInvalidValue;
  const int64_t blocks = std::min<int64_t>((nq + 7) / 8, (int64_t)num_sms * 8);
  const dim3 grid((unsigned)blocks), block(256);
  switch (L) {
    case 16:
      rerank_full_kernel<0><<<grid, block, 0, st>>>(base, np, dim, queries, qstride, pool, nq, k, out_ids, out_dists);
      break;
    case 32:
      rerank_full_kernel<1><<<grid, block, 0, st>>>(base, np, dim, queries, qstride, pool, nq, k, out_ids, out_dists);
      break;
    case 64:
      rerank_full_kernel<2><<<grid, block, 0, st>>>(base, np, dim, queries, qstride, pool, nq, k, out_ids, out_dists);
      break;
    case 128:
      rerank_full_kernel<4><<<grid, block, 0, st>>>(base, np, dim, queries, qstride, pool, nq, k, out_ids, out_dists);
      break;
    case 256:
      rerank_full_kernel<8><<<grid, block, 0, st>>>(base, np, dim, queries, qstride, pool, nq, k, out_ids, out_dists);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace rte
