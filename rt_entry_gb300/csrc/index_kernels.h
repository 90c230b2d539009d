// index_kernels.h -- launches of the build-side and entry-stage kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

namespace rte {

// kd-tree node for point location: bound = union of the expanded boxes of
// the leaves below it.  left < 0 marks a leaf with index -left-1.
struct BvhNode {
  float lo[3];
  float hi[3];
  int32_t left;
  int32_t right;
};
static_assert(sizeof(BvhNode) == 32, "BvhNode is 32 bytes");

constexpr int kBvhMaxDepth = 64;

// The kd-tree again, 8 wide: a wide node holds the boxes of the binary
// descendants three levels below one binary node (or of the leaves met
// before that), in pre-order.  Point location then needs a third of the
// dependent node loads.  child[c] >= 0 is a wide node, < 0 the leaf
// -(child+1); unused slots have empty boxes (lo > hi).  Wide nodes are
// numbered breadth-first.
constexpr int kWide = 8;
struct WideNode {
  float lo[3][kWide];  // lo[axis][child]
  float hi[3][kWide];
  int32_t child[kWide];
  int32_t pad[kWide];
};
static_assert(sizeof(WideNode) == 256, "WideNode is 256 bytes");

cudaError_t launch_mean(const float* x, int64_t n, int d, double* partial, int nblocks,
                        double* mean, cudaStream_t st);
cudaError_t launch_cov(const float* x, int64_t n, int d, const double* mean, double* partial,
                       int nchunks, double* cov, cudaStream_t st);
// The projection out[r][c] = sum_k (x[r][k] - mean[k]) V[k][c], c < k.
// vt_split: the rotation split for the tensor cores (launch_split_rotation);
// when it is given and x meets the tensor map's alignment (16-byte base,
// row pitch a multiple of 4 floats) the product runs on tcgen05
// (project_tc.cu), otherwise on the FP32 FMA kernel.
// zero / zero_words: a word range the kernel also sets to 0 (a query call's
// work counter, error flag and argmax keys), so that the call needs no
// separate memsets.
cudaError_t launch_project(const float* x, int64_t n, int d, int xstride, const float* mean,
                           const float* V, int vstride, int k, float* out, int ostride,
                           cudaStream_t st, uint32_t* zero = nullptr, int64_t zero_words = 0,
                           const float* vt_split = nullptr);
// launch_project plus a BF16 copy of the output: out16[r][c] =
// bf16(out[r][c] * s16) for c < k, 0 for k <= c < ld16 (the learned head's
// input rows, ld16 >= k).
cudaError_t launch_project_bf16(const float* x, int64_t n, int d, int xstride, const float* mean,
                                const float* V, int vstride, int k, float* out, int ostride,
                                void* out16, float s16, int ld16, cudaStream_t st,
                                uint32_t* zero = nullptr, int64_t zero_words = 0,
                                const float* vt_split = nullptr);
// Variants for graph replay: grids sized for `cap` rows, the live row count
// read from device memory at run time.
cudaError_t launch_project_dyn(const float* x, int64_t cap, const int* n_dev, int d, int xstride,
                               const float* mean, const float* V, int vstride, int k, float* out,
                               int ostride, cudaStream_t st, const float* vt_split = nullptr);
// launch_project_bf16 for graph replay, plus the zeroed word range.
cudaError_t launch_project_bf16_dyn(const float* x, int64_t cap, const int* n_dev, int d, int xstride,
                                    const float* mean, const float* V, int vstride, int k, float* out,
                                    int ostride, void* out16, float s16, int ld16, uint32_t* zero,
                                    int64_t zero_words, cudaStream_t st, const float* vt_split = nullptr);
// The rotation V [d][k] (row pitch vstride) split for the tensor cores:
// [2][k][round_up(d, 4)] floats, V^T rounded to TF32 then the TF32 of the
// remainder (project_tc.cu).
size_t rotation_split_floats(int d, int k);
cudaError_t launch_split_rotation(const float* V, int d, int k, int vstride, float* out, cudaStream_t st);
// The tensor-core projection (project_tc.cu); cudaErrorNotSupported when the
// shapes or alignments do not fit it.  err: set to a non-zero code when a
// bounded pipeline wait runs out (may be null).
cudaError_t launch_project_tc(const float* x, int64_t n, const int* n_dev, int d, int xstride,
                              const float* mean, const float* vt_split, int k, float* out, int ostride,
                              void* out16, float s16, int ld16, uint32_t* zero, int64_t zero_words,
                              int* err, cudaStream_t st);
cudaError_t launch_locate_dyn(const WideNode* wide, int n_wide, const float* pts, int64_t cap,
                              const int* n_dev, int stride, int32_t* out, cudaStream_t st, bool top_cache = true);
cudaError_t launch_interleave(const float* src, int64_t n, int d, int C, float* il32, void* il16,
                              uint8_t* il8, float* scale8, float* xyz, cudaStream_t st);
cudaError_t launch_deinterleave(const float* il32, int64_t n, int d, int C, float* dst,
                                cudaStream_t st);
// The BF16 copy (il16, may be null) and the FP8 copy with per-row scales
// (il8 and scale8, may be null) made from the interleaved FP32 copy, equal
// to what launch_interleave writes from row-major input.
cudaError_t launch_lowp_copies(const float* il32, int64_t n, int C, void* il16, uint8_t* il8,
                               float* scale8, cudaStream_t st);
// Squared norm of every BF16 row (FP64 sum of the BF16 values squared,
// rounded to FP32).
cudaError_t launch_bf16_norms(const uint16_t* il16, int64_t n, int C, float* out, cudaStream_t st);
cudaError_t launch_dequant(const void* il, const float* scale8, int precision, int64_t n, int d,
                           int C, float* dst, cudaStream_t st);
// The class of point i is cls[i], or decoded from the packed argmax key
// keys[i] (exactly one of the two is given).  A class outside [0, n_classes)
// (a key the head never wrote) gives leaf 0, the miss rule's leaf.
cudaError_t launch_locate_in_subtree(const BvhNode* nodes, const float* pts, int64_t n, int stride,
                                     const int32_t* cls, const unsigned long long* keys,
                                     const int32_t* start_node, const int32_t* fallback_leaf,
                                     int n_classes, int32_t* out, cudaStream_t st);
// launch_locate_in_subtree on the 8-wide tree: the class of point i, decoded
// from keys[i], starts at start_ref[class] (a wide node, or a leaf).  n_dev:
// the live point count for graph replay (grid sized for n).
cudaError_t launch_locate_in_subtree_wide(const WideNode* wide, const float* pts, int64_t n,
                                          int stride, const unsigned long long* keys,
                                          const int32_t* start_ref, const int32_t* fallback_leaf,
                                          int n_classes, int32_t* out, cudaStream_t st,
                                          const int* n_dev = nullptr);
// The first H containing leaves per point ([n][H], -1 padded, leaf 0 first on
// a miss).
cudaError_t launch_locate_multi(const WideNode* wide, int n_wide, const float* pts, int64_t n,
                                int stride, int H, int32_t* out, cudaStream_t st);
// top_cache: copy the top of the tree into each block's shared memory; off
// when the launch runs beside a kernel that needs most of an SM's shared
// memory.
cudaError_t launch_locate(const WideNode* wide, int n_wide, const float* pts, int64_t n, int stride,
                          int32_t* out, cudaStream_t st, bool top_cache = true);
// The order in which a search takes its queries: a permutation of [0, n)
// grouping queries by entry leaf (leaf[i * stride]; a leaf outside
// [0, n_leaves) counts as leaf 0, the search's own fallback).  Leaves are
// numbered in the kd-tree build's depth-first order, so queries close in
// the order start in nearby parts of the base, and the queries a persistent
// search runs at the same time then share more graph rows and vectors in
// L2.  Within one of the (at most 4096) ranges of 2^s consecutive leaves
// the order is that of the atomic counters; each query's result does not
// depend on it.  One block.
// For graph replay, n_dev gives the live count (n is then the capacity),
// and a live count of min_n or fewer writes nothing: the search reads the
// order only for more than min_n queries (SearchArgs::order_min).
cudaError_t launch_order_by_leaf(const int32_t* leaf, int stride, int64_t n, int n_leaves,
                                 int32_t* order, cudaStream_t st, const int* n_dev = nullptr,
                                 int64_t min_n = 0);

}  // namespace rte
