/*
 * rtentry.h -- C ABI of rt_entry_gb300, a GB300 (sm_103a) implementation of
 * rt_entry's query path: PCA projection, kd-tree leaf point location (the
 * entry points) and proximity-graph beam search.
 *
 * The reference has no library API; its boundary is the `Graph` class
 * (graph.h:10-82) driven from main.cpp:82-92.  Each entry point below names
 * the reference method it replaces.  Conventions:
 *   - No function exits the process; every failure returns a status and sets
 *     a thread-local message readable with rte_last_error().
 *   - Pointers to vectors/ids may be host or device memory (detected per
 *     call); results are written to the same kind of memory they point to.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  A call that
 *     reads or writes host memory returns after its results are in place.
 *   - An index is single-writer: build/load/free must not overlap other calls
 *     on the same index.  Searches on distinct streams may run concurrently.
 *   - Data contract (graph.h, file_read.cu): FP32 row-major vectors, int32
 *     graph [np x degree] with a power-of-two degree and padding value np,
 *     ids in [0, np], np < 2^31.
 */
#ifndef RTENTRY_H_
#define RTENTRY_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTE_ABI_VERSION 1

typedef struct rte_index rte_index;

typedef enum {
  RTE_OK = 0,
  RTE_EINVAL = 1,   /* bad argument (reference: undefined behaviour or exit) */
  RTE_ENOMEM = 2,   /* host or device allocation failed                      */
  RTE_EIO = 3,      /* file missing, truncated or malformed (file_read.cu exit(1)) */
  RTE_ECUDA = 4,    /* a CUDA call failed (helper.h CUDA_CHECK exit(2))       */
  RTE_ETIMEOUT = 5, /* a bounded device wait ran out                          */
  RTE_ESTATE = 6    /* a required build step has not run yet                  */
} rte_status;

typedef enum { RTE_PREC_FP32 = 0, RTE_PREC_BF16 = 1, RTE_PREC_FP8 = 2 } rte_precision;

typedef enum {
  RTE_ENTRY_RANDOM = 0, /* LCG entries per query, ALGO 0/2 (graph_search.cuh:50-54,485) */
  RTE_ENTRY_KDTREE = 1, /* kd-tree leaf of the projected query, ALGO 1 (entry.cu:100-149) */
  RTE_ENTRY_LEARNED = 2 /* MLP-proposed leaf (no reference counterpart)                 */
} rte_entry_mode;

/* Search parameters (flags.cpp:3-101 + graph_search.cuh:4-5 macros). */
typedef struct {
  int k;             /* topk returned per query; 0 -> beam (graph.cu:54)              */
  int beam;          /* n_candidates L; rounded up to a power of two (graph.cu:53)    */
  int search_width;  /* W: nodes expanded per iteration (FLAGS_search_width)          */
  int max_iter;      /* FLAGS_max_iter, default 100                                   */
  int bloom_words;   /* visited-set filter size in 32-bit words (SIZE, default 512)   */
  int bloom_hashes;  /* hash functions (num_hash, default 3)                          */
  int precision;     /* rte_precision of candidate distances                          */
  int rerank;        /* 1: exact FP32 rerank of the final beam in the searched space;
                        2: exact FP32 rerank of the final beam against the original
                           (pre-PCA) rows, rte_search only (graph_helper.cu:146-213) */
  int entry_mode;    /* rte_entry_mode                                                */
  int warps_per_block; /* 0 = automatic                                                */
  int max_hits;      /* kd-tree entries from the first max_hits containing leaves (1..8;
                        the reference's max_hits, flags.cpp:100, multi-hit entry
                        entry_helper.cu:5-241); caller hits are then [nq x max_hits]  */
  int team_warps;    /* warps that share one query's distance evaluations: 1, 2, 4 or 8
                        (a multiple of warps_per_block), or 0 = automatic: the most, up
                        to 8, that the batch leaves room for in the resident warps, so a
                        small batch still fills the GPU.  Results do not depend on it.  */
} rte_search_params;

typedef struct {
  int64_t np;          /* base vectors                                   */
  int dim;             /* input dimension                                */
  int search_dim;      /* dimension searched (PCA keep_dims or dim)      */
  int degree;          /* graph degree                                   */
  int has_pca;
  int has_kdtree;
  int64_t n_leaves;
  int leaf_size;       /* max points per leaf (max_node)                 */
  float expand_ratio;
  int has_bf16;
  int has_fp8;
  int device;
  int64_t device_bytes; /* device memory held by the index               */
} rte_index_info;

/* Default parameters: k=10, beam=64, W=1, max_iter=100, 512 words, 3 hashes,
 * FP32, no rerank, kd-tree entries. */
void rte_default_params(rte_search_params* p);

/* Build an index from host or device arrays (Graph::Input + Graph::RB_Graph,
 * graph.cu:73-139).  base [np x dim] FP32, graph [np x degree] int32.  The
 * graph is validated (ids in [0, np], power-of-two degree). */
rte_status rte_index_from_host(const float* base, int64_t np, int dim, const int32_t* graph,
                               int degree, int device, rte_index** out);

/* Load base vectors (.fvecs / .fbin / .bvecs, file_read.cu:16-80) and a raw
 * int32 graph whose degree is file size / (4 np) (file_read.cu:237-255). */
rte_status rte_index_load(const char* base_path, const char* graph_path, int device,
                          rte_index** out);

/* PCA of the base (Graph::Projection, graph.cu:141-252; pca.cpp:4-58,122-126):
 * FP64 mean and covariance, FP64 eigendecomposition, eigenvectors sorted by
 * descending eigenvalue; the base is projected onto the first keep_dims
 * components ((B - mean) V) and searched in that space.  keep_dims in
 * [3, dim]; 0 -> dim. */
rte_status rte_build_pca(rte_index* idx, int keep_dims);

/* Install a PCA computed elsewhere (mean [dim], rotation [dim x dim], row =
 * input dim, column = component -- the layout of O.fbin, pca.cpp:78-87) and
 * project the base with it. */
rte_status rte_set_pca(rte_index* idx, const float* mean, const float* rotation, int keep_dims);

/* kd-tree over the first three search-space coordinates with at most
 * leaf_size points per leaf, then boxes enlarged by expand_ratio * width per
 * side (RT_Entry::BlockUp, entry.cu:8-77; kdtree.cpp:140-196; aabb.cu:27-38).
 * The reference's point_ratio maps to leaf_size = (int)(np * point_ratio). */
rte_status rte_build_kdtree(rte_index* idx, int leaf_size, float expand_ratio);

/* Query projection (Graph::Search step 1, graph.cu:258-273): out[nq x
 * search_dim] = (Q - mean) V[:, :search_dim]. */
rte_status rte_project(rte_index* idx, const float* queries, int64_t nq, float* out,
                       void* stream);

/* Entry stage alone (RT_Entry::Search, entry.cu:100-149; devicePrograms.cu:
 * 29-96): out_leaf[q] = smallest leaf whose expanded box contains the first
 * three coordinates of projected[q] (row stride search_dim), 0 if none. */
rte_status rte_locate(rte_index* idx, const float* projected, int64_t nq, int32_t* out_leaf,
                      void* stream);

/* The whole query path (Graph::Search, graph.cu:254-293): projection, entry
 * selection, beam search (GraphSearchKernel, graph_search.cuh:56-1964).
 * out_ids [nq x k] (|pool id|, np for an empty slot), out_dists [nq x k]
 * squared L2 in the search space (536870912.0f for an empty slot) or NULL.
 * With host buffers the call returns when the results are in them, and
 * RTE_ETIMEOUT if a bounded device wait in the path ran out (the learned
 * head's pipeline, or a search warp waiting on the block's tail helpers);
 * with device buffers the call is asynchronous and such a wait only sets
 * a device word.  Page-locked host outputs are written by the kernels
 * directly; pageable ones are filled by copies after the search.  The same
 * holds for rte_search_projected. */
rte_status rte_search(rte_index* idx, const float* queries, int64_t nq,
                      const rte_search_params* params, int32_t* out_ids, float* out_dists,
                      void* stream);

/* Beam search from already projected queries [nq x search_dim].  hits [nq]
 * gives each query's leaf (NULL: run rte_locate first).  Used to feed
 * identical inputs to the search and to the oracle. */
rte_status rte_search_projected(rte_index* idx, const float* projected, const int32_t* hits,
                                int64_t nq, const rte_search_params* params, int32_t* out_ids,
                                float* out_dists, void* stream);

/* rte_search_projected without any memory allocation.  No counterpart in the
 * reference.  Meant for callers that cannot let a library allocate device
 * memory once they are running: a server that reserves all of its GPU
 * memory at start-up and treats a later cudaMalloc as a failure (it can
 * stall on a device-wide synchronisation or fail under memory pressure), or
 * a framework whose allocator owns the device.  Differences from
 * rte_search_projected:
 *   - every pointer must be device memory; entry_mode random or kd-tree;
 *   - a BF16 or FP8 search needs that copy to exist already
 *     (rte_index_prepare, or an earlier search): RTE_ESTATE otherwise;
 *   - at most RTE_NOALLOC_MAX_QUERIES queries per call (RTE_EINVAL beyond);
 *   - its scratch (each query's leaf, the order in which a large batch's
 *     queries are taken, and the search's work counter: about 512 KB) is
 *     one fixed array inside the library that every GPU holds
 *     until the process exits.  Creating an index on a device
 *     (rte_index_from_host, rte_index_load, rte_index_load_dir) looks up the
 *     array's device address there, which is when the GPU reserves it (CUDA
 *     loads modules lazily), so the searches themselves reserve nothing.
 *     Should that lookup fail at index creation, the first call retries it:
 *     make that call before any stream capture.  All calls share the one
 *     array: calls that overlap on the GPU (other streams, other threads)
 *     race on it, so the caller must not let them overlap. */
#define RTE_NOALLOC_MAX_QUERIES 65536
rte_status rte_search_projected_noalloc(rte_index* idx, const float* projected,
                                        const int32_t* hits, int64_t nq,
                                        const rte_search_params* params, int32_t* out_ids,
                                        float* out_dists, void* stream);

/* ---- uneven query streams (no reference counterpart:
 * the reference launches each stage separately and synchronises the device
 * after each, graph.cu:254-337) ----
 * A batcher captures the whole query path (projection, kd-tree location,
 * persistent search) once into a CUDA graph sized for max_nq queries; the
 * kernels read the batch size from device memory, so every batch of up to
 * max_nq queries replays the same graph.  Random, kd-tree or learned
 * entries; learned entries need a PCA index whose trained head the fused
 * head kernel takes (RTE_EINVAL otherwise) and give the same results as
 * rte_search's learned path. */
typedef struct rte_batcher rte_batcher;
rte_status rte_batcher_create(rte_index* idx, int64_t max_nq, const rte_search_params* params,
                              rte_batcher** out);
/* queries [nq x dim] (host or device) -> out_ids / out_dists [nq x k]. */
rte_status rte_batcher_search(rte_batcher* b, const float* queries, int64_t nq, int32_t* out_ids,
                              float* out_dists, void* stream);
int rte_batcher_k(const rte_batcher* b);
void rte_batcher_free(rte_batcher* b);

typedef struct {
  int met_target;  /* 1 if some candidate reached the recall target          */
  float recall;    /* k@k recall of the chosen parameters on the sample       */
  float ms;        /* device time of one search of the sample                 */
  float qps;
  int evaluated;   /* candidates measured                                     */
} rte_autotune_report;

/* Picks beam, search width, bloom filter size and warps per block: every
 * candidate runs on the sample queries [nq x dim]; recall@k is measured
 * against gt [nq x gt_k] (true neighbour ids, gt_k >= k); the fastest
 * candidate reaching target_recall wins (else the one with the best
 * recall), where 4 warps per block must beat 8 by more than 3 % (8 leave
 * room for larger teams on a batcher's small batches).  Other fields of
 * *params (precision, entry mode, max_iter, hashes) are kept. */
rte_status rte_autotune(rte_index* idx, const float* queries, int64_t nq, const int32_t* gt,
                        int gt_k, int k, float target_recall, rte_search_params* params,
                        rte_autotune_report* report);

/* Per-query work counters of the last rte_search_projected-equivalent run:
 * [nq x 4] int64 = valid entries, expanded nodes, distance evaluations,
 * iterations.  Runs the search once more with counting enabled. */
rte_status rte_search_counters(rte_index* idx, const float* projected, const int32_t* hits,
                               int64_t nq, const rte_search_params* params, int64_t* counters,
                               void* stream);

rte_status rte_index_get_info(const rte_index* idx, rte_index_info* info);

/* Copies of built artifacts (host pointers): mean [dim], rotation
 * [dim x dim], eigenvalues [dim] (descending, FP64). */
rte_status rte_get_pca(const rte_index* idx, float* mean, float* rotation, double* eigvals);
/* Search-space base vectors, row-major [np x search_dim]. */
rte_status rte_get_search_base(const rte_index* idx, float* out);
/* The search-space base as a reduced-precision search sees it, widened to
 * FP32, row-major [np x search_dim]: precision 1 = BF16 values, 2 = FP8-E4M3
 * values times their per-vector scale (scale = max|x| / 448). */
rte_status rte_get_search_base_lowp(const rte_index* idx, int precision, float* out);
/* Leaves in DFS order: tight [n_leaves x 6], expanded [n_leaves x 6]
 * (minX,minY,minZ,maxX,maxY,maxZ), pids [n_leaves x leaf_size] padded np.
 * Any pointer may be NULL. */
rte_status rte_get_kdtree(const rte_index* idx, float* tight, float* expanded, int32_t* pids);

/* Open an index from a data directory as the reference leaves it (Graph's
 * data_name, graph.cu:42-45; RT_Entry::BlockUp, entry.cu:8-77):
 *   base_path   base vectors: .fvecs, .bvecs, .fbin, .hvecs, .hh or .txt
 *               (file_read.cu:16-117);
 *   graph_path  raw int32 [np x degree] (file_read.cu:237-255);
 *   dir/O.fbin + dir/mean.fbin (pca.cpp:60-90), when present: the PCA is
 *               installed with keep_dims components (0 = all);
 *   dir/pca_base.fbin (pca.cpp:128-139), when present: its first keep_dims
 *               columns become the search space as stored (the reference
 *               searches exactly these values); otherwise the base is
 *               projected here;
 *   dir/<leaf_size>_0.aabbs (entry.cu:171-190), when present and
 *               leaf_size > 0: the kd-tree is rebuilt over the search space
 *               and must reproduce the file's leaves and point ids exactly
 *               (RTE_EIO if not: the file belongs to another base); the
 *               leaves are then expanded by expand_ratio.
 * leaf_size <= 0 builds no kd-tree.  Missing PCA files leave the raw base
 * as the search space (keep_dims must then be 0). */
rte_status rte_index_load_reference(const char* dir, const char* base_path, const char* graph_path,
                                    int keep_dims, int leaf_size, float expand_ratio, int device,
                                    rte_index** out);

/* Reads a vector file by its extension (.fvecs, .bvecs, .fbin, .hvecs, .hh,
 * .txt; file_read.cu:16-117) on the host, no device needed: *n and *d
 * receive its shape; with out != NULL the n*d values are copied there
 * (RTE_EINVAL if capacity < n*d).  Call once with out = NULL to size the
 * buffer. */
rte_status rte_read_vectors(const char* path, float* out, int64_t capacity, int64_t* n, int* d);

/* Save / load every built artifact to / from a directory (base.fbin,
 * graph.ibin, mean.fbin, O.fbin, pca_base.fbin and the leaf cache
 * <leaf_size>_0.aabbs in the reference's layouts, entry.cu:171-190). */
rte_status rte_index_save(const rte_index* idx, const char* dir);
rte_status rte_index_load_dir(const char* dir, int device, rte_index** out);

/* Device copies an index can hold besides its FP32 search space.  An index
 * starts with the FP32 search space and the raw base (the vectors as given:
 * PCA builds, rerank 2 and rte_index_save read them).  The BF16 and FP8
 * copies (precision 1 and 2) are made from the FP32 copy on the first
 * search that needs them, or now by rte_index_prepare -- before a stream
 * capture or rte_search_projected_noalloc, which cannot make them.
 * rte_index_release frees copies once no search on the index is in flight;
 * the BF16 and FP8 copies come back on their next use, the raw base does
 * not (the calls that need it then return RTE_ESTATE).  No counterpart in
 * the reference, which keeps one FP32 copy. */
#define RTE_COPY_BF16 1u
#define RTE_COPY_FP8 2u
#define RTE_COPY_RAW 4u
rte_status rte_index_prepare(rte_index* idx, unsigned copies);
rte_status rte_index_release(rte_index* idx, unsigned copies);

void rte_index_free(rte_index* idx);

/* Host build steps on their own (no device, no index): the kd-tree leaves
 * of rte_build_kdtree (kdtree.cpp:140-196 + aabb.cu:27-38) over xyz [n x 3],
 * written to caller arrays of capacity max_leaves (tight / expanded
 * [max_leaves x 6], pids [max_leaves x leaf_size]); *n_leaves receives the
 * count (RTE_EINVAL with the count set when max_leaves is too small). */
rte_status rte_kdtree_build_host(const float* xyz, int64_t n, int leaf_size, float expand_ratio,
                                 int64_t max_leaves, float* tight, float* expanded, int32_t* pids,
                                 int64_t* n_leaves);

/* FP64 symmetric eigendecomposition used by rte_build_pca (pca.cpp:11-29):
 * a [n x n] row-major; w [n] descending; v [n x n] with eigenvector j in
 * column j, largest-magnitude component positive. */
rte_status rte_sym_eig_host(const double* a, int n, double* w, double* v);

/* ---- learned entry (no reference counterpart) ----
 * A 3-layer MLP (search-space query -> hidden -> hidden -> kd-tree subtree)
 * proposes the region of each query's entry; point location inside that
 * subtree picks the entry leaf.  With RTE_ENTRY_LEARNED the entry list
 * is the proposed leaf's points followed by the kd-tree leaf's points (the
 * kd-tree stays the fallback), truncated to the beam. */
typedef struct {
  int hidden;      /* hidden width, multiple of 8 (256)                       */
  int epochs;      /* passes over the training queries (4)                    */
  int batch;       /* rows per step, multiple of 128 (4096)                   */
  float lr;        /* Adam learning rate, cosine-decayed to lr/10 (2e-3)      */
  int label_beam;  /* beam of the plain search that labels the queries (64)   */
  int seed;        /* initialisation and shuffling seed (3003)                */
  int max_classes; /* model output width: the kd-tree nodes at the deepest
                      level with at most this many nodes (4096); the model
                      picks that subtree, point location inside it picks the
                      leaf                                                   */
} rte_train_params;

typedef struct {
  float first_loss, last_loss; /* mean cross-entropy of the first / last batch */
  float train_acc;             /* top-1 leaf accuracy on one training batch    */
  int64_t n_train;
  int classes;                 /* output width = kd-tree subtrees at one depth */
  int64_t steps;
  float train_ms;              /* device time of the optimisation loop         */
} rte_train_report;

void rte_default_train_params(rte_train_params* p);
/* Labels every training query with the subtree holding the best result of
 * the plain kd-tree search (beam label_beam), then trains the MLP on the
 * GPU with BF16 tensor-core GEMMs (FP32 accumulation), softmax
 * cross-entropy and Adam.  Requires the kd-tree. */
rte_status rte_learned_train(rte_index* idx, const float* train_queries, int64_t n,
                             const rte_train_params* params, rte_train_report* report);
/* The learned entry leaf for each projected query [nq x search_dim]. */
rte_status rte_learned_predict(rte_index* idx, const float* projected, int64_t nq,
                               int32_t* out_leaf, void* stream);

/* One forward + backward pass of the learned-entry MLP on given FP32
 * inputs and weights (rounded to BF16 as training does), for checking the
 * GPU gradients against a CPU restatement.  X [M x d], labels [M], W1
 * [hidden x d], W2 [hidden x hidden], W3 [classes x hidden]; gradients of
 * the mean cross-entropy in the same shapes, per-row loss [M] (may be NULL). */
rte_status rte_mlp_grad_check(const float* X, const int32_t* labels, int M, int d, int hidden,
                              int classes, const float* W1, const float* b1, const float* W2,
                              const float* b2, const float* W3, const float* b3, float* gW1,
                              float* gb1, float* gW2, float* gb2, float* gW3, float* gb3,
                              float* loss);

/* BF16 tensor-core GEMM of the learned-entry MLP (tcgen05 + TMA + TMEM):
 * C [M x N] FP32 = A [M x K] * B [N x K]^T, A and B BF16 bit patterns,
 * row-major, K a multiple of 8.  Host or device pointers.  RTE_ETIMEOUT if
 * a bounded pipeline wait ran out.  (No reference counterpart.) */
rte_status rte_gemm_bf16(const uint16_t* A, const uint16_t* B, int M, int N, int K, float* C,
                         void* stream);

/* The learned head's last layer alone: for each row m, the column n of the
 * largest A[m]·B[n] + bias[n] (the first one on ties), through the same
 * tensor-core kernel and fused argmax epilogue as rte_learned_predict.
 * Host or device pointers; cols [M] int32, -1 for a row whose logits are
 * all NaN.  (No reference counterpart.) */
rte_status rte_gemm_bf16_bias_argmax(const uint16_t* A, const uint16_t* B, const float* bias, int M,
                                     int N, int K, int32_t* cols, void* stream);

/* The learned head's whole forward pass: for each row m of X [M x dp], the
 * column n of the largest (relu(relu(X W1^T + b1) W2^T + b2) W3^T + b3)[m][n]
 * (the first on ties), the hidden activations rounded to BF16.  W1 [H x dp],
 * W2 [H x H], W3 [N x H], X: BF16 bit patterns, row-major; biases FP32.
 * path 0: the fused single-kernel form rte_search uses (H a multiple of 64
 * up to 256, dp up to 256; RTE_EINVAL otherwise); path 1: the three
 * layer-by-layer GEMMs.  Both give the same columns.  Device pointers;
 * cols [M] int32, -1 for a row whose logits are all NaN.  RTE_ETIMEOUT if a bounded pipeline wait ran out.  (No
 * reference counterpart.) */
rte_status rte_mlp_head_argmax(const uint16_t* X, int M, int dp, const uint16_t* W1, const float* b1,
                               const uint16_t* W2, const float* b2, const uint16_t* W3, const float* b3,
                               int H, int N, int path, int32_t* cols, void* stream);

/* The first max_hits (1..8) leaves whose expanded boxes contain each
 * projected query, smallest index first, -1 padded; a query in no box gets
 * leaf 0 first.  out [nq x max_hits].  Host or device pointers.  The entry
 * stage of kd-tree search with max_hits > 1 (raytracing.cpp:283-334 with
 * max_hits, entry_helper.cu:5-241). */
rte_status rte_locate_multi(rte_index* idx, const float* projected, int64_t nq, int max_hits,
                            int32_t* out_leaves, void* stream);

/* The exact degree-R kNN graph of base [n x d] (FP32, host or device): row i
 * lists the R rows j != i nearest to row i by squared L2 distance in FP64,
 * in (distance, id) order, into graph [n x R] (host or device).  Candidates
 * come from tensor-core BF16 hi/lo GEMMs; every row is then certified exact
 * against an error bound, and rows that cannot be certified are redone with
 * more candidates (RTE_EIO if one still cannot).  The reference loads its
 * graph from a file (graph.cu:120); no counterpart. */
rte_status rte_knn_graph(const float* base, int64_t n, int d, int degree, int device, int32_t* graph,
                         void* stream);

/* Limit of the bounded waits in the tensor-core kernels (the learned head,
 * its GEMMs and the tensor-core projection), in mbarrier try_wait rounds:
 * a pipeline wait that runs out records an error, raises a flag the
 * kernel's other roles poll, lets the copies and MMAs in flight finish,
 * frees its tensor memory and returns, and synchronous calls report
 * RTE_ETIMEOUT.  rounds <= 0 restores the default (2^24 rounds, a second or
 * more).  Process-wide, read at each launch; meant for tests of the timeout
 * path.  (No reference counterpart.) */
void rte_set_wait_limit(long long rounds);

/* The library's scratch memory pool on `device` (the stream-ordered pool
 * the query calls take their per-call buffers from; it keeps up to 1 GiB
 * mapped between calls): bytes in use now and the high-water mark (either
 * pointer may be NULL), then, if reset_high, the mark restarts from the
 * current use.  For monitoring, and for tests that a call allocates
 * nothing.  (No reference counterpart.) */
rte_status rte_scratch_pool_usage(int device, uint64_t* used_now, uint64_t* used_high, int reset_high);

/* Message of the last failure on this thread ("" if none). */
const char* rte_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* RTENTRY_H_ */
