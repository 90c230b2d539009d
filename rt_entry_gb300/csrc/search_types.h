// search_types.h -- arguments of the search kernel (host and device).
#pragma once
#include <stdint.h>

namespace rte {

enum : int { kPrecF32 = 0, kPrecBF16 = 1, kPrecFP8 = 2 };

#ifdef __CUDACC__
#define RTE_HD __host__ __device__
#else
#define RTE_HD
#endif

// Shared memory of one warp of the search kernel, in 32-bit words: the bloom
// filter, 2*max(batch, beam) compaction slots, a slot for the query, and
// (search_kernel_team) two control words.  The query slot holds
// the query's BF16 row (tensor-core distances, up to 128 dims) in the kernels built
// for one chunk count, or its FP32 row of `chunks` chunks in the kernels
// built for any chunk count (kernel template C == 0).
constexpr int kQuerySlotWords = 64;
RTE_HD constexpr int query_slot_words_for(int C, int chunks) {
  return C == 0 ? (32 * chunks > kQuerySlotWords ? 32 * chunks : kQuerySlotWords) : kQuerySlotWords;
}
// Control words of a team (the query, the phase; two spare) at the end of
// each warp's region in search_kernel_team; every launch reserves them.
// Four words keep every region, and so every query slot, on a 16-byte
// boundary: the query slot is read with 16-byte vector loads.  The filter
// (a power of two >= 32 words), the compaction words (2 x 16..256) and the
// query slot (64 or 32 x chunks words) are all multiples of 4 words.
constexpr int kTeamCtlWords = 4;
// Automatic teams keep their floor of warps per query (more than one: FP32
// rows with pools of up to 64 slots) only while a batch is at most this
// many times the resident warps; above it one warp per query is faster.
constexpr int kTeamFloorLoad = 3;
// Shared memory a search block keeps after its warps' regions: the tail
// helping state (a count of idle warps and one phase descriptor per warp,
// search_kernel.cuh's BlockShare).  Every launch reserves it.
constexpr int kBlockShareBytes = 16 + 8 * 32;
// Codes the search kernels write to SearchArgs::err when a bounded wait runs out.
constexpr int kErrHelpWait = 3;
constexpr int kMaxHits = 8;  // leaves per query for kd-tree entries
constexpr int kMaxChunks = 32;  // rows of up to 1024 dims

struct SearchArgs {
  const float* base;        // lane-interleaved FP32 rows, stride 32*C floats
  const uint16_t* base_bf16;  // lane-interleaved BF16 rows (precision 1)
  const uint8_t* base_fp8;  // lane-interleaved E4M3 rows (precision 2)
  const float* fp8_scale;   // per-row scale (precision 2)
  const float* norm16;      // per-row squared norm of the BF16 row (precision 1, d <= 128)
  const float* queries;     // row-major [nq][qstride]
  const int32_t* graph;     // [np][R], padding np
  const int32_t* leaf_pids; // [n_leaves][leaf_cap], padding np
  const int32_t* hits;      // [nq] leaf per query
  const int32_t* hits2;     // [nq] second leaf (entry mode 2: the kd-tree leaf)
  int32_t* out_ids;         // [nq][k]
  float* out_dists;         // [nq][k] or null
  long long* counters;      // [nq][4] or null
  unsigned int* work;       // query counter, zero at launch
  int np, d, qstride, nq, R, W, k, max_iter, bloom_words, bloom_hashes, leaf_cap, entry_mode;
  int rerank;
  int n_leaves;             // hits outside [0, n_leaves) fall back to leaf 0
  int max_hits;             // entry mode 1: hits holds [nq][max_hits] leaves (-1 padded)
  const int* nq_dev;        // if set, the query count is read here (graph replay)
  int C;                    // chunks of 32 dims per row (set by launch_search)
  int team;                 // warps per query: 0 or 1 alone, 2/4/8 a team, < 0 chosen
                            // by the kernel from the live query count, at least -team
  int* err;                 // device word set to a non-zero code when a bounded wait runs out, or null
  const int32_t* order;     // [nq] the order in which queries are taken (a permutation), or null
  int order_min;            // the order is read only for more than this many queries
};

}  // namespace rte
