/*
 * oracle.h -- CPU restatement of rt_entry's query path (test infrastructure).
 *
 * THIS IS THE ORACLE, NOT THE PRODUCT.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load liboracle.so.  The product path
 * (librtentry.so) never links, loads or calls anything here.
 *
 * Every function restates one piece of the reference (thmyl/rt_entry) and
 * cites the file:line it follows.  Points where the reference is racy or
 * unspecified are fixed by the canonical rules H1..H5 written next to the
 * code that implements them (search_ref.cpp, kdtree_ref.cpp).
 *
 * Parity pins: kdtree_ref is checked against the reference's own kdtree.cpp
 * compiled from source (oracle/ref/Makefile); search_ref is checked against
 * the reference's GraphSearchKernel compiled for sm_103a and run on a GB300
 * (fixtures in tests/golden/, made by tests/golden/make_search_golden.py).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Sentinel distance of an empty pool slot: the int 0x1fffffff stored into a
 * float (graph_search.cuh:474 with MAX from structure_on_device.cuh:6). */
#define ORC_MAX_DIST 536870912.0f

/* Per-query work counters used for the roofline byte count. */
typedef struct {
  int64_t entries_valid;   /* E_q: entry slots with id < np                 */
  int64_t expanded;        /* X_q: selected nodes whose row was read        */
  int64_t dist_evals;      /* D_q: main-loop distance evaluations           */
  int64_t iterations;      /* main-loop iterations executed                 */
  int64_t merges;          /* batches merged into the pool (entry + main)   */
  int64_t merges_idle;     /* of those, batches with no distance below the
                              pool's largest: the merge leaves the pool as
                              it was                                        */
  int64_t merges_few;      /* main-loop batches with 1..8 pairwise distinct
                              distances below the pool's largest (no NaN):
                              the ones a merge by rank can serve            */
} orc_counters;

/* Beam search over a fixed-degree graph, GraphSearchKernel semantics
 * (graph_search.cuh:56-1964).
 *   base      [np x d] row-major FP32 (the space the search runs in)
 *   queries   [nq x d] row-major FP32
 *   graph     [np x degree] int32, padding value np, degree a power of two
 *   leaf_pids [n_leaves x leaf_cap] int32 padded with np (computeAabbPid)
 *   hits      [nq] leaf index per query (entry_mode 1)
 *   L         pool size (n_candidates, power of two), k <= L
 *   entry_mode 0 = random LCG entries (ALGO 0/2), 1 = kd-tree leaf entries
 *   out_ids   [nq x k], out_dists [nq x k] (may be NULL), counters [nq] (may be NULL)
 * Returns 0 on success, -1 on invalid arguments. */
int orc_search(const float* base, int64_t np, int d, const float* queries, int64_t nq,
               const int32_t* graph, int degree, const int32_t* leaf_pids, int leaf_cap,
               const int32_t* hits, int L, int k, int search_width, int max_iter,
               int bloom_words, int bloom_hashes, int entry_mode,
               int32_t* out_ids, float* out_dists, orc_counters* counters, int n_threads);

/* orc_search, then (rerank_base != NULL) the exact FP32 rerank of the final
 * pool: |ids|, distances on rerank_base, ascending bitonic sort.  `base` is
 * then the reduced-precision copy the search ran on (dequantized to FP32). */
int orc_search_rerank(const float* base, const float* rerank_base, int64_t np, int d,
                      const float* queries, int64_t nq, const int32_t* graph, int degree,
                      const int32_t* leaf_pids, int leaf_cap, const int32_t* hits,
                      const int32_t* hits2, int L, int k, int search_width, int max_iter, int bloom_words, int bloom_hashes,
                      int entry_mode, int32_t* out_ids, float* out_dists, orc_counters* counters,
                      int n_threads);

/* One distance with the reference's arithmetic (graph_search.cuh:500-886):
 * per-lane FMA chain over chunks, then the shfl_down tree 16,8,4,2,1. */
float orc_l2_ref(const float* p, const float* q, int d);

/* Entry mode 1 with max_hits leaves per query, hits_multi [nq x max_hits]
 * (-1 padded): every point of each leaf, max(L, max_hits*leaf_cap) entry
 * slots.  The reference's disabled multi-hit entry (entry_helper.cu:5-241). */
int orc_search_multi(const float* base, int64_t np, int d, const float* queries, int64_t nq,
                     const int32_t* graph, int degree, const int32_t* leaf_pids, int leaf_cap,
                     const int32_t* hits_multi, int max_hits, int L, int k, int search_width,
                     int max_iter, int bloom_words, int bloom_hashes, int32_t* out_ids,
                     float* out_dists, orc_counters* counters, int n_threads);
/* The first H containing leaves in index order, -1 padded. */
void orc_locate_multi(const float* boxes, int64_t n_leaves, const float* qp, int64_t nq, int stride,
                      int H, int32_t* out_leaves, int n_threads);

/* Exact FP32 rerank of pools [nq x L] (ids, visited marks allowed) against
 * the original rows base [np x dim] and queries [nq x dim]: the first k of
 * the ascending bitonic sort.  graph_helper.cu:146-213. */
int orc_rerank_full(const float* base, int64_t np, int dim, const float* queries, int64_t nq,
                    const int32_t* pool, int L, int k, int32_t* out_ids, float* out_dists,
                    int n_threads);

/* kd-tree build over 3-d points (kdtree.cpp:4-196).  Outputs leaves in the
 * reference's DFS order: tight boxes [n_leaves x 6] (minX,minY,minZ,maxX,maxY,maxZ)
 * and leaf pids [n_leaves x leaf_cap] padded with np.  The caller passes
 * capacity max_leaves; *n_leaves receives the count.  Returns 0, -1 on bad
 * arguments, -2 when a split fails (the reference exits there), -3 when
 * max_leaves is too small. */
int orc_kdtree_build(const float* pts3, int64_t np, int leaf_cap, int64_t max_leaves,
                     float* out_boxes, int32_t* out_pids, int64_t* n_leaves);

/* expandAabb (aabb.cu:27-38), in place on [n x 6] boxes. */
void orc_expand_boxes(float* boxes, int64_t n, float expand_ratio);

/* Point location, canonical rule H1: the smallest leaf index whose expanded
 * box contains (x,y,z) inclusively; 0 when none does.  qp has row stride
 * `stride` floats and the first three columns are used. */
void orc_locate(const float* boxes, int64_t n_leaves, const float* qp, int64_t nq,
                int stride, int32_t* out_leaf, int n_threads);

/* FP64 brute-force k nearest neighbours (ties by smaller id). */
void orc_knn_fp64(const float* base, int64_t np, int d, const float* queries, int64_t nq,
                  int k, int32_t* out_ids, double* out_d2, int n_threads);

#ifdef __cplusplus
}
#endif
