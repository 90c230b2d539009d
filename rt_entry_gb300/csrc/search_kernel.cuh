// search_kernel.cuh -- persistent warp-per-query beam search for sm_103a.
//
// Computes exactly what the reference's GraphSearchKernel computes
// (graph_search.cuh:56-1964, one 64-thread block per query), reorganised for
// one warp per query:
//   * the pool (L = 32*NL slots, or 16 slots for NL = 0) and the batch
//     (B = 32*NB slots) live in registers: slot p sits in lane p%32,
//     register p/32.  The reference's
//     comparator network (bitonic batch sort, pool/batch merge, half-cleaner,
//     graph_search.cuh:888-957 and :1424-1493) runs on those registers,
//     across lanes through shuffles and inside a lane for distances >= 32;
//   * base rows are stored lane-interleaved (see layout.cuh): one 128-bit
//     load gives lane l the dims l, l+32, l+64, l+96 -- exactly the dims the
//     reference's reduction tree assigns to lane l -- so a neighbour row is a
//     single fully coalesced 512-byte gather at d = 128;
//   * distances of up to 16 neighbours are reduced together by a butterfly
//     whose every addition pairs the same partial sums as the reference's
//     shuffle-down tree (16,8,4,2,1), so the results are bit-identical while
//     using one shuffle per neighbour instead of five;
//   * the visited-set bloom filter lives in shared memory per warp, sized at
//     run time (the reference fixes 512 words, graph_search.cuh:4-5);
//   * warps pull queries from an atomic counter until none are left; a
//     batch larger than the resident warps is pulled through a permutation
//     that groups its queries by entry leaf (SearchArgs::order), so that
//     the queries running at the same time share rows in L2.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <stdint.h>

#include "layout.cuh"
#include "search_types.h"

namespace rte {

constexpr float kMaxDist = 536870912.0f;  // (float)0x1fffffff, structure_on_device.cuh:6
constexpr unsigned kFull = 0xffffffffu;

// Bloom-filter hash multipliers (graph_search.cuh:89-97).
__constant__ uint32_t c_hash_mul[20] = {
    0x924ed183U, 0xd854fc0aU, 0xecf5e3b7U, 0x1bead407U, 0x28a30449U,
    0xbfc4d99fU, 0x715030e2U, 0xffcfb45bU, 0x6e4ce166U, 0xeb53c362U,
    0xa93c4f40U, 0xcecde0a4U, 0x0288592dU, 0x362c37bcU, 0x9d4824f0U,
    0xfdbdd68bU, 0x63258c85U, 0x6726905cU, 0x609500f9U, 0x4de48422U};


__device__ __forceinline__ uint32_t bloom_hash(int h, uint32_t x, uint32_t mask_bits) {
  // hash_ (graph_search.cuh:13-22); x % (SIZE<<5) with SIZE a power of two.
  x ^= x >> 16;
  x *= c_hash_mul[h << 1];
  x ^= x >> 13;
  x *= c_hash_mul[(h << 1) + 1];
  x ^= x >> 16;
  return x & mask_bits;
}

struct Bloom {
  uint32_t* w;
  uint32_t words_mask;  // words - 1
  uint32_t bits_mask;   // 32*words - 1
  int lw;               // log2(words)
  int nh;
  // set_bit / test_bit: word x % SIZE, bit x / SIZE (graph_search.cuh:7-28).
  // The first kUnrolled hashes are unrolled, so their multipliers are
  // constant-bank operands; further hashes (up to 10) run in a loop, which
  // keeps the kernel's code small.
  static constexpr int kUnrolled = 3;
  __device__ __forceinline__ void add(uint32_t x) const {
#pragma unroll
    for (int h = 0; h < kUnrolled; ++h) {
      if (h >= nh) break;
      uint32_t b = bloom_hash(h, x, bits_mask);
      atomicOr(&w[b & words_mask], 1u << (b >> lw));
    }
#pragma unroll 1
    for (int h = kUnrolled; h < nh; ++h) {
      uint32_t b = bloom_hash(h, x, bits_mask);
      atomicOr(&w[b & words_mask], 1u << (b >> lw));
    }
  }
  __device__ __forceinline__ bool test(uint32_t x) const {
    bool ok = true;
#pragma unroll
    for (int h = 0; h < kUnrolled; ++h) {
      if (h >= nh) break;
      uint32_t b = bloom_hash(h, x, bits_mask);
      ok &= ((w[b & words_mask] >> (b >> lw)) & 1u) != 0;
    }
#pragma unroll 1
    for (int h = kUnrolled; h < nh; ++h) {
      uint32_t b = bloom_hash(h, x, bits_mask);
      ok &= ((w[b & words_mask] >> (b >> lw)) & 1u) != 0;
    }
    return ok;
  }
  __device__ __forceinline__ void clear(int lane) const {
    for (uint32_t i = lane; i <= words_mask; i += 32) w[i] = 0u;
  }
};

template <int N>
__device__ __forceinline__ int pick(const int (&a)[N], int c) {
  int v = a[0];
#pragma unroll
  for (int j = 1; j < N; ++j)
    if (c == j) v = a[j];
  return v;
}

// Compare-exchange of slot p with slot p^sub held by another lane (sub < 32).
// `desc` is the direction of the pair; both lanes evaluate the same
// predicate on (lower, upper), so ties never swap (strict comparisons).
__device__ __forceinline__ void cx_lanes(float& d, int& id, int sub, bool desc, int lane) {
  float od = __shfl_xor_sync(kFull, d, sub);
  int oi = __shfl_xor_sync(kFull, id, sub);
  bool lower = (lane & sub) == 0;
  float da = lower ? d : od;
  float db = lower ? od : d;
  bool sw = desc ? (da < db) : (da > db);
  if (sw) {
    d = od;
    id = oi;
  }
}

__device__ __forceinline__ void cx_regs(float& da, int& ia, float& db, int& ib, bool desc) {
  bool sw = desc ? (da < db) : (da > db);
  if (sw) {
    float t = da;
    da = db;
    db = t;
    int u = ia;
    ia = ib;
    ib = u;
  }
}

// Pool geometry: NL registers of 32 slots each, or NL == 0 for a 16-slot pool
// (beam 16) held in lanes 0..15 of one register; lanes 16..31 of that
// register keep (MAX, np) padding that no step ever reads back.
__host__ __device__ constexpr int pool_slots(int NL) { return NL == 0 ? 16 : 32 * NL; }
__host__ __device__ constexpr int pool_regs(int NL) { return NL == 0 ? 1 : NL; }
// Batch geometry: NB registers of 32 slots, or NB == 0 for a 16-slot batch
// (search width 1 over a degree-16 graph) in lanes 0..15 of one register;
// lanes 16..31 then hold (MAX, np) padding.
__host__ __device__ constexpr int batch_slots(int NB) { return NB == 0 ? 16 : 32 * NB; }
__host__ __device__ constexpr int batch_regs(int NB) { return NB == 0 ? 1 : NB; }
// Query registers per lane: C, or one unused register for the kernels built
// for any chunk count (C == 0), which keep the query in shared memory.
__host__ __device__ constexpr int qregs(int C) { return C == 0 ? 1 : C; }

// Bitonic sort of N slots (graph_search.cuh:888-919), N = 32*NB by default or
// 16 for the one-register beam-16 pool.  With DESC_FINAL the pair (a, a+sub)
// is descending when a's 2*step block index is even, so the result is
// descending, as the reference sorts its batch; otherwise the directions are
// mirrored and the result is ascending.  Registers below KEEP_FROM are not
// read after the sort (the merge reads only the last ones): the final step's
// in-register stages skip them, which leaves every register that is read
// unchanged.
template <int NB, bool DESC_FINAL = true, int N = 32 * NB, int KEEP_FROM = 0>
__device__ __forceinline__ void sort_batch_desc(float (&d)[NB], int (&id)[NB], int lane) {
  constexpr int B = N;
#pragma unroll
  for (int step = 1; step <= B / 2; step <<= 1) {
#pragma unroll
    for (int sub = step; sub >= 1; sub >>= 1) {
      if (sub >= 32) {
        const int rs = sub >> 5;
#pragma unroll
        for (int j = 0; j < NB; ++j) {
          if (j & rs) continue;
          const bool desc = (((j << 5) & (2 * step)) == 0) == DESC_FINAL;
          cx_regs(d[j], id[j], d[j + rs], id[j + rs], desc);
        }
      } else {
#pragma unroll
        for (int j = 0; j < NB; ++j) {
          if (step == B / 2 && j < KEEP_FROM) continue;  // dead after the sort
          const bool desc = ((((j << 5) + lane) & (2 * step)) == 0) == DESC_FINAL;
          cx_lanes(d[j], id[j], sub, desc, lane);
        }
      }
    }
  }
}

// The pool's ascending half-cleaner (graph_search.cuh:933-957): compare-
// exchanges at distances L/2 .. 1, in registers for distances >= 32.
template <int NL>
__device__ __forceinline__ void half_clean(float (&pd)[pool_regs(NL)], int (&pi)[pool_regs(NL)], int lane) {
  constexpr int L = pool_slots(NL), PR = pool_regs(NL);
#pragma unroll
  for (int sub = L / 2; sub >= 1; sub >>= 1) {
    if (sub >= 32) {
      const int rs = sub >> 5;
#pragma unroll
      for (int j = 0; j < PR; ++j) {
        if (j & rs) continue;
        cx_regs(pd[j], pi[j], pd[j + rs], pi[j + rs], false);
      }
    } else {
#pragma unroll
      for (int j = 0; j < PR; ++j) cx_lanes(pd[j], pi[j], sub, false, lane);
    }
  }
}

// Pool/batch merge then the ascending half-cleaner (graph_search.cuh:921-957,
// :1454-1493).  Pool slot L-n+i meets batch slot B-n+i (n = min(L,B)); both
// are in the same lane.  The main loop skips a batch slot holding MAX.
template <int NL, int NB>
__device__ __forceinline__ void merge_pool(float (&pd)[pool_regs(NL)], int (&pi)[pool_regs(NL)],
                                           const float (&bd)[batch_regs(NB)],
                                           const int (&bi)[batch_regs(NB)], bool skip_max, int lane) {
  if constexpr (NB == 0) {
    // 16-slot batch: n = 16, batch slot i (lane i) meets pool slot L-16+i,
    // which is lane i of a 16-slot pool or lane 16+i of the last register
    float od = bd[0];
    int oi = bi[0];
    if constexpr (NL != 0) {
      od = __shfl_up_sync(kFull, od, 16);
      oi = __shfl_up_sync(kFull, oi, 16);
    }
    constexpr int PR = pool_regs(NL);
    const bool mine = NL == 0 ? lane < 16 : lane >= 16;
    bool take = mine && pd[PR - 1] > od;
    if (skip_max && od == kMaxDist) take = false;
    if (take) {
      pd[PR - 1] = od;
      pi[PR - 1] = oi;
    }
    half_clean<NL>(pd, pi, lane);
  } else if constexpr (NL == 0) {
    // 16-slot pool: pool slot i (lane i) meets batch slot B-16+i, which is
    // lane 16+i of the last batch register.
    const float od = __shfl_down_sync(kFull, bd[NB - 1], 16);
    const int oi = __shfl_down_sync(kFull, bi[NB - 1], 16);
    bool take = lane < 16 && pd[0] > od;
    if (skip_max && od == kMaxDist) take = false;
    if (take) {
      pd[0] = od;
      pi[0] = oi;
    }
    half_clean<0>(pd, pi, lane);
  } else {
    constexpr int NC = NL < NB ? NL : NB;
#pragma unroll
    for (int m = 0; m < NC; ++m) {
      const int pr = NL - NC + m, br = NB - NC + m;
      bool take = pd[pr] > bd[br];
      if (skip_max && bd[br] == kMaxDist) take = false;
      if (take) {
        pd[pr] = bd[br];
        pi[pr] = bi[br];
      }
    }
    half_clean<NL>(pd, pi, lane);
  }
}

// True when some batch distance lies strictly below the pool's largest
// distance (slot L-1: lane 31 of the last register, or lane 15 of the
// 16-slot pool).  When none does, the merge takes nothing -- it swaps only
// where pool > batch, and every pool slot is <= the largest -- and the
// half-cleaner then meets a pool that is still sorted ascending (the pool
// leaves every merge sorted, and visiting a slot only negates its id), where
// its strict comparisons swap nothing.  Sorting and merging such a batch
// therefore leaves the pool unchanged, ids and order included, and
// search_query skips both.
template <int NL, int NB>
__device__ __forceinline__ bool batch_can_enter(const float (&pd)[pool_regs(NL)],
                                                const float (&bd)[batch_regs(NB)]) {
  const float pmax = __shfl_sync(kFull, pd[pool_regs(NL) - 1], NL == 0 ? 15 : 31);
  bool below = false;
#pragma unroll
  for (int j = 0; j < batch_regs(NB); ++j) below |= bd[j] < pmax;
  return __any_sync(kFull, below);
}

// Candidates a batch may hold for merge_few.
constexpr int kFewMax = 8;

// Main-loop merge of a batch in which only a few slots (the candidates) hold
// distances below the pool's largest, pmax.
// The descending batch sort puts those candidates, if their distances are
// pairwise distinct, in the batch's last slots in descending order whatever
// the network does with the other slots: the candidate of ascending rank r
// lands in batch slot B-1-r, which the merge pairs with pool slot L-1-r.
// Every other batch slot holds a distance >= the pool's largest, so its
// comparison (pool > batch, strict) takes nothing.  Placing each candidate
// against pool slot L-1-r by its rank and running the half-cleaner therefore
// gives exactly the network's pool.  Returns false, changing nothing, when
// two candidates tie (the network's order of equal distances then decides
// which id lands where, so the caller runs it).
template <int NL, int NB>
__device__ __forceinline__ bool merge_few(float (&pd)[pool_regs(NL)], int (&pi)[pool_regs(NL)],
                                          const float (&bd)[batch_regs(NB)], const int (&bi)[batch_regs(NB)],
                                          float pmax, int lane) {
  constexpr int BR = batch_regs(NB), PR = pool_regs(NL), L = pool_slots(NL);
  unsigned cm[BR];
#pragma unroll
  for (int j = 0; j < BR; ++j) cm[j] = __ballot_sync(kFull, bd[j] < pmax);
  // ascending rank of this lane's candidate in batch register t, 4 bits
  // at bit 4t (ranks stay below kFewMax = 8; BR <= 8)
  unsigned rank = 0;
  bool tie = false;
#pragma unroll
  for (int j = 0; j < BR; ++j) {
    unsigned mask = cm[j];
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1;
      const float v = __shfl_sync(kFull, bd[j], src);
#pragma unroll
      for (int t = 0; t < BR; ++t) {
        if ((cm[t] >> lane) & 1u) {
          rank += bd[t] > v ? 1u << (4 * t) : 0u;
          tie |= bd[t] == v && !(t == j && lane == src);
        }
      }
    }
  }
  if (__any_sync(kFull, tie)) return false;
#pragma unroll
  for (int j = 0; j < BR; ++j) {
    unsigned mask = cm[j];
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1;
      const float v = __shfl_sync(kFull, bd[j], src);
      const int id = __shfl_sync(kFull, bi[j], src);
      const int slot = L - 1 - (int)((__shfl_sync(kFull, rank, src) >> (4 * j)) & 15u);
      if (lane == (slot & 31) && v != kMaxDist) {  // the main loop never takes a MAX slot
#pragma unroll
        for (int p = 0; p < PR; ++p) {
          if (p == (slot >> 5) && pd[p] > v) {
            pd[p] = v;
            pi[p] = id;
          }
        }
      }
    }
  }
  half_clean<NL>(pd, pi, lane);
  return true;
}

// Partial sum of one lane for one row: s = t0*t0, then fmaf(tc, tc, s) over
// chunks c (t = p - q on dims lane + 32c).  PREC selects the stored format;
// BF16 and FP8 rows are widened to FP32 before the subtraction.
template <int C, int PREC>
struct RowLoader;

template <int C>
struct RowLoader<C, kPrecF32> {
  float v[C];
  __device__ __forceinline__ void load(const SearchArgs& a, int id, int lane) {
    load_interleaved<C>(a.base + (size_t)id * (32 * C), lane, v);
  }
  __device__ __forceinline__ float value(int c) const { return v[c]; }
};

template <int C>
struct RowLoader<C, kPrecBF16> {
  float v[C];
  __device__ __forceinline__ void load(const SearchArgs& a, int id, int lane) {
    load_interleaved_bf16<C>(reinterpret_cast<const __nv_bfloat16*>(a.base_bf16) + (size_t)id * (32 * C), lane, v);
  }
  __device__ __forceinline__ float value(int c) const { return v[c]; }
};

template <int C>
struct RowLoader<C, kPrecFP8> {
  float v[C];
  __device__ __forceinline__ void load(const SearchArgs& a, int id, int lane) {
    float s = __ldg(a.fp8_scale + id);
    load_interleaved_fp8<C>(a.base_fp8 + (size_t)id * (32 * C), lane, v);
#pragma unroll
    for (int c = 0; c < C; ++c) v[c] *= s;
  }
  __device__ __forceinline__ float value(int c) const { return v[c]; }
};

template <int C>
__device__ __forceinline__ float lane_partial(const float (&p)[C], const float (&q)[C]) {
  float t = __fsub_rn(p[0], q[0]);
  float s = __fmul_rn(t, t);
#pragma unroll
  for (int c = 1; c < C; ++c) {
    t = __fsub_rn(p[c], q[c]);
    s = __fmaf_rn(t, t, s);
  }
  return s;
}

// ---- BF16 distances on the tensor cores (rows of 32*C <= 128 dims) ----
// A team: K warps of one block that serve one query (search_kernel_team).
// The leader (w == 0)
// runs the search; at each distance phase it publishes the row count in
// ctl[1] and the K warps each compute an interleaved share of the row groups
// into the leader's compaction buffers, between two crossings of the team's
// named barrier.  ctl[0] carries the team's query, ctl[1] = -1 ends it.
// Named barriers are hardware waits that every member reaches on every path,
// so a team needs no spin-wait.
struct Team {
  int K = 1;                     // warps per query
  int w = 0;                     // this warp's index in the team
  int bar = 0;                   // named barrier id (1 + team index in the block)
  volatile int* ctl = nullptr;   // [0] query, [1] phase: row count (+ 1<<16 for the rerank), -1 = done
};

__device__ __forceinline__ void team_sync(const Team& t) {
  asm volatile("bar.sync %0, %1;" ::"r"(t.bar), "r"(32 * t.K) : "memory");
}

// dist = |p|^2 + |q|^2 - 2 p.q, p the BF16 row, q the query rounded to BF16,
// p.q from mma.sync m16n8k16 (BF16 inputs, exact products, FP32
// accumulation).  A BF16 row (32*C values, 64*C bytes) is read as C pieces
// of 64 bytes; thread t of each 4-thread group reads bytes [16t + 64i, +16)
// of piece i -- storage elements 32i + 8t + j, j < 8 -- and uses them as the
// MMA k-slots {2t, 2t+1, 2t+8, 2t+9} of k-tiles 2i (j < 4) and 2i+1 (j >= 4).
// The query fragment comes from the query's own BF16 row at the same storage
// positions, so each k pairs the base and query values of one dimension.
// With integer-valued data of magnitude < 2^8 every term is exact and the
// distances equal the FP32 path's bit for bit.
template <int C, int PREC, bool MMA = (PREC == kPrecBF16 && C >= 1 && C <= 4)>
struct QueryExtra {};
// Kernels for any chunk count (C == 0): the FP32 query row in the warp's
// shared memory, in the base rows' interleaved layout.
template <int PREC>
struct QueryExtra<0, PREC, false> {
  const float* qs;
};
template <int C, int PREC>
struct QueryExtra<C, PREC, true> {
  const uint32_t* qs;  // the query's BF16 row in the warp's shared memory (16*C words)
  float qn;            // squared norm of the BF16 query
};

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                               uint32_t a3, uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
      "{%8, %9}, {%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// The query in the base's BF16 layout, kept in `slot` (16*C words of the
// warp's shared memory) for the whole query, and its squared norm.
template <int C>
__device__ __forceinline__ void make_query_extra(QueryExtra<C, kPrecBF16, true>& qx,
                                                 const float (&qv)[C], uint32_t* slot, int lane) {
  uint16_t* qs = reinterpret_cast<uint16_t*>(slot);
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const __nv_bfloat16 b = __float2bfloat16_rn(qv[c]);
    const float f = __bfloat162float(b);
    s = __fmaf_rn(f, f, s);
    qs[interleaved_offset(c, lane, C)] = __bfloat16_as_ushort(b);
  }
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) s = __fadd_rn(s, __shfl_xor_sync(kFull, s, off));
  qx.qn = s;
  qx.qs = slot;
  __syncwarp();
}

// L2 prefetch of the rows a warp is about to gather.  A batch of up to
// kPrefetchWhole bytes is prefetched at once.  A larger one goes through a
// window of about kPrefetchBytes per warp: the first `ahead` rows of the
// warp's share before its first group, then at each group the rows `ahead`
// further on.  Without the window a batch of 256 rows of 3.8 KB would put
// ~1 MB per warp in flight, several GB over the grid against a 129 MB L2,
// and the lines would be evicted before use (on one GB300: 1.7x the
// algorithmic bytes read from DRAM).  Batches of up to 128 KB (256 FP32
// rows of 128 dims) measured faster prefetched whole.
constexpr int kPrefetchBytes = 16384;
constexpr int kPrefetchWhole = 196608;

__host__ __device__ constexpr int prefetch_ahead(int row_bytes, int G) {
  return kPrefetchBytes / row_bytes >= G ? kPrefetchBytes / row_bytes / G * G : G;
}
// Rows to prefetch before the first group: all n, or the window.
__device__ __forceinline__ int prefetch_first(int n, int row_bytes, int ahead) {
  return n * row_bytes <= kPrefetchWhole ? n : ahead;
}

// Prefetches rows [lr0, lr1) of member w's share of a K-warp team (groups
// of G rows, group g belonging to member g % K; a single warp is w = 0,
// K = 1), `lines` 128-byte lines per row.
template <int G>
__device__ __forceinline__ void prefetch_local(const char* rows, size_t row_bytes, int lines,
                                               const int* s_ids, int n, int lane, int w, int K, int lr0,
                                               int lr1) {
  for (int i = lane + lr0 * lines; i < lr1 * lines; i += 32) {
    const int lr = i / lines, line = i - lr * lines;
    const int j = lr / G;
    const int row = G * (w + j * K) + (lr - j * G);
    if (row >= n) break;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(rows + (size_t)s_ids[row] * row_bytes + line * 128));
  }
}

// Distances of the n ids in s_ids[0..n) by the tensor cores, 8 rows per MMA
// group: thread (g, t) supplies row g of the group as column g of the MMA's
// B operand; the query is every row of A, so D[.][col] is the dot product of
// row col, and lanes 0..3 hold the group's eight results.
// One group of 8 rows from r0 (rows >= n are skipped).
template <int C>
__device__ __forceinline__ void mma_group(const SearchArgs& a, const QueryExtra<C, kPrecBF16, true>& qx,
                                          const int* s_ids, float* s_dist, int n, int lane, int r0) {
  constexpr int kRowBytes = 64 * C;
  const char* rows = reinterpret_cast<const char*>(a.base_bf16);
  const int g = lane >> 2, t = lane & 3;
  const int ra = r0 + g;
  const int id = s_ids[ra < n ? ra : r0];
  const char* p = rows + (size_t)id * kRowBytes + 16 * t;
  uint4 v[C];
#pragma unroll
  for (int i = 0; i < C; ++i) v[i] = __ldg(reinterpret_cast<const uint4*>(p + 64 * i));
  // the norms of this lane's two output rows, loaded while the MMAs run
  float pn[2] = {0.0f, 0.0f};
  if (g == 0) {
#pragma unroll
    for (int e = 0; e < 2; ++e)
      if (r0 + 2 * t + e < n) pn[e] = __ldg(a.norm16 + s_ids[r0 + 2 * t + e]);
  }
  float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int i = 0; i < C; ++i) {
    const uint4 q = *reinterpret_cast<const uint4*>(qx.qs + 4 * t + 16 * i);
    mma_bf16_16816(d, q.x, q.x, q.y, q.y, v[i].x, v[i].y);
    mma_bf16_16816(d, q.z, q.z, q.w, q.w, v[i].z, v[i].w);
  }
  if (g == 0) {
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int row = r0 + 2 * t + e;
      if (row < n) s_dist[row] = __fmaf_rn(-2.0f, d[e], __fadd_rn(pn[e], qx.qn));
    }
  }
}

template <int C, bool TEAM>
__device__ __forceinline__ void distances_mma(const SearchArgs& a, const QueryExtra<C, kPrecBF16, true>& qx,
                                              const int* s_ids, float* s_dist, int n, int lane, int w, int K) {
  constexpr int kRowBytes = 64 * C, kLines = (kRowBytes + 127) / 128;
  constexpr int kAhead = prefetch_ahead(kRowBytes, 8);
  const char* rows = reinterpret_cast<const char*>(a.base_bf16);
  const int ws = TEAM ? w : 0, ks = TEAM ? K : 1;
  const int first_rows = prefetch_first(n, kRowBytes, kAhead);
  prefetch_local<8>(rows, kRowBytes, kLines, s_ids, n, lane, ws, ks, 0, first_rows);
  const bool windowed = first_rows < n;
  const int first = 8 * ws, step = 8 * ks;
  int j = 0;
  for (int r0 = first; r0 < n; r0 += step, ++j) {
    if (windowed) prefetch_local<8>(rows, kRowBytes, kLines, s_ids, n, lane, ws, ks, kAhead + 8 * j, kAhead + 8 * j + 8);
    mma_group<C>(a, qx, s_ids, s_dist, n, lane, r0);
  }
}

// ---- rows of a run-time chunk count (kernels built for any dimension) ----
// A row of C chunks is streamed slab by slab in the interleaved layout
// (layout.cuh): chunks 4s..4s+3 as one 4-value load per lane, then a pair,
// then a single chunk.  Each value is widened to FP32 (BF16 exactly; FP8
// times the row's scale) before the subtraction, as RowLoader does.
template <int PREC>
struct SlabLoader;

template <>
struct SlabLoader<kPrecF32> {
  static constexpr int kBytes = 4;
  const float* row;
  __device__ __forceinline__ void init(const SearchArgs& a, int id, size_t stride) { row = a.base + (size_t)id * stride; }
  __device__ __forceinline__ float4 quad(int off, int lane) const {
    return __ldg(reinterpret_cast<const float4*>(row + off) + lane);
  }
  __device__ __forceinline__ float2 pair(int off, int lane) const {
    return __ldg(reinterpret_cast<const float2*>(row + off) + lane);
  }
  __device__ __forceinline__ float one(int off, int lane) const { return __ldg(row + off + lane); }
};

template <>
struct SlabLoader<kPrecBF16> {
  static constexpr int kBytes = 2;
  const uint16_t* row;
  __device__ __forceinline__ void init(const SearchArgs& a, int id, size_t stride) {
    row = a.base_bf16 + (size_t)id * stride;
  }
  __device__ __forceinline__ float4 quad(int off, int lane) const {
    const uint2 x = __ldg(reinterpret_cast<const uint2*>(row + off) + lane);
    return make_float4(bf16lo(x.x), bf16hi(x.x), bf16lo(x.y), bf16hi(x.y));
  }
  __device__ __forceinline__ float2 pair(int off, int lane) const {
    const uint32_t y = __ldg(reinterpret_cast<const unsigned int*>(row + off) + lane);
    return make_float2(bf16lo(y), bf16hi(y));
  }
  __device__ __forceinline__ float one(int off, int lane) const {
    return __uint_as_float((uint32_t)__ldg(row + off + lane) << 16);
  }
};

template <>
struct SlabLoader<kPrecFP8> {
  static constexpr int kBytes = 1;
  const uint8_t* row;
  float sc;
  __device__ __forceinline__ void init(const SearchArgs& a, int id, size_t stride) {
    row = a.base_fp8 + (size_t)id * stride;
    sc = __ldg(a.fp8_scale + id);
  }
  __device__ __forceinline__ float4 quad(int off, int lane) const {
    const uint32_t x = __ldg(reinterpret_cast<const unsigned int*>(row + off) + lane);
    const float2 u = fp8x2_to_float2((uint16_t)(x & 0xffffu));
    const float2 v = fp8x2_to_float2((uint16_t)(x >> 16));
    return make_float4(__fmul_rn(u.x, sc), __fmul_rn(u.y, sc), __fmul_rn(v.x, sc), __fmul_rn(v.y, sc));
  }
  __device__ __forceinline__ float2 pair(int off, int lane) const {
    const float2 u = fp8x2_to_float2(__ldg(reinterpret_cast<const unsigned short*>(row + off) + lane));
    return make_float2(__fmul_rn(u.x, sc), __fmul_rn(u.y, sc));
  }
  __device__ __forceinline__ float one(int off, int lane) const {
    return __fmul_rn(fp8x2_to_float2((uint16_t)__ldg(row + off + lane)).x, sc);
  }
};

// One chunk of a lane's partial: fmaf(t, t, s) with t = p - q.  The first
// chunk starts from s = +0, and fmaf(t, t, +0) rounds exactly as t * t, so
// the sum equals lane_partial's.
__device__ __forceinline__ float chunk_acc(float p, float q, float s) {
  const float t = __fsub_rn(p, q);
  return __fmaf_rn(t, t, s);
}

// The butterfly reduction of G rows' lane partials (see `distances`): row
// g0 + lane / (32/G) is complete in the first lane of each 32/G-lane span.
template <int G>
__device__ __forceinline__ void reduce_rows(float (&part)[G], float* s_dist, int g0, int n, int lane) {
  constexpr int SPAN = 32 / G;
#pragma unroll
  for (int off = 16, half = G / 2; half >= 1; off >>= 1, half >>= 1) {
    const bool up = (lane & off) != 0;
#pragma unroll
    for (int t = 0; t < half; ++t) {
      float send = up ? part[t] : part[t + half];
      float keep = up ? part[t + half] : part[t];
      part[t] = __fadd_rn(keep, __shfl_xor_sync(kFull, send, off));
    }
  }
  float total = part[0];
#pragma unroll
  for (int off = SPAN / 2; off >= 1; off >>= 1) total = __fadd_rn(total, __shfl_xor_sync(kFull, total, off));
  const int row = g0 + lane / SPAN;
  if ((lane % SPAN) == 0 && row < n) s_dist[row] = total;
}

// Distances of n rows of a.C chunks against the query row in shared memory
// qs (interleaved layout), G rows in flight.
// One group of 4 rows from g0 of a run-time chunk count (rows >= n give 0).
template <int PREC>
__device__ __forceinline__ void rt_group(const SearchArgs& a, const float* qs, const int* s_ids,
                                         float* s_dist, int n, int lane, int g0) {
  constexpr int G = 4;
  const int C = a.C, n4 = C >> 2, rem = C & 3;
  const size_t stride = 32 * (size_t)C;  // elements per row
  SlabLoader<PREC> r[G];
#pragma unroll
  for (int t = 0; t < G; ++t) r[t].init(a, s_ids[g0 + t < n ? g0 + t : g0], stride);
  float part[G];
#pragma unroll
  for (int t = 0; t < G; ++t) part[t] = 0.0f;
#pragma unroll 2
  for (int sl = 0; sl < n4; ++sl) {
    const float4 q = *reinterpret_cast<const float4*>(qs + 128 * sl + 4 * lane);
    float4 v[G];
#pragma unroll
    for (int t = 0; t < G; ++t) v[t] = r[t].quad(128 * sl, lane);
#pragma unroll
    for (int t = 0; t < G; ++t) {
      part[t] = chunk_acc(v[t].x, q.x, part[t]);
      part[t] = chunk_acc(v[t].y, q.y, part[t]);
      part[t] = chunk_acc(v[t].z, q.z, part[t]);
      part[t] = chunk_acc(v[t].w, q.w, part[t]);
    }
  }
  int off = 128 * n4;
  if (rem >= 2) {
    const float2 q = *reinterpret_cast<const float2*>(qs + off + 2 * lane);
#pragma unroll
    for (int t = 0; t < G; ++t) {
      const float2 v = r[t].pair(off, lane);
      part[t] = chunk_acc(v.x, q.x, part[t]);
      part[t] = chunk_acc(v.y, q.y, part[t]);
    }
    off += 64;
  }
  if (rem & 1) {
    const float q = qs[off + lane];
#pragma unroll
    for (int t = 0; t < G; ++t) part[t] = chunk_acc(r[t].one(off, lane), q, part[t]);
  }
#pragma unroll
  for (int t = 0; t < G; ++t)
    if (g0 + t >= n) part[t] = 0.0f;
  reduce_rows<G>(part, s_dist, g0, n, lane);
}

template <int PREC>
__host__ __device__ constexpr int slab_bytes() {
  return PREC == kPrecF32 ? 4 : PREC == kPrecBF16 ? 2 : 1;
}

template <int PREC>
__device__ __forceinline__ const char* search_rows(const SearchArgs& a) {
  return PREC == kPrecF32    ? reinterpret_cast<const char*>(a.base)
         : PREC == kPrecBF16 ? reinterpret_cast<const char*>(a.base_bf16)
                             : reinterpret_cast<const char*>(a.base_fp8);
}

template <int PREC, bool TEAM>
__device__ __forceinline__ void distances_rt(const SearchArgs& a, const float* qs, const int* s_ids,
                                             float* s_dist, int n, int lane, int w, int K) {
  constexpr int G = 4;
  const size_t rb = 32 * (size_t)a.C * slab_bytes<PREC>();
  const int lines = (int)((rb + 127) / 128);
  const char* rows = search_rows<PREC>(a);
  const int ws = TEAM ? w : 0, ks = TEAM ? K : 1;
  const int ahead = prefetch_ahead((int)rb, G);
  const int first_rows = prefetch_first(n, (int)rb, ahead);
  prefetch_local<G>(rows, rb, lines, s_ids, n, lane, ws, ks, 0, first_rows);
  const bool windowed = first_rows < n;
  const int first = G * ws, step = G * ks;
  int j = 0;
  for (int g0 = first; g0 < n; g0 += step, ++j) {
    if (windowed) prefetch_local<G>(rows, rb, lines, s_ids, n, lane, ws, ks, ahead + G * j, ahead + G * j + G);
    rt_group<PREC>(a, qs, s_ids, s_dist, n, lane, g0);
  }
}

// Distances of the n (<= B) ids in s_ids[0..n) written to s_dist[0..n).
// Groups of G rows (16, or 8 for long rows): each lane forms its partial for
// the G rows; a butterfly over offsets 16, 8, ... exchanges half of the rows
// at each level until every lane holds one row, then plain xor-shuffles
// finish the sum, which lands in the 32/G lanes lane = t*(32/G) + ...
// Every addition pairs the same two partial sums as the reference's
// shuffle-down tree (addition is commutative, so the results are equal).
// With TEAM, the groups of rows of member w of a K-warp team only.
// Rows per distance group of each path.
template <int C, int PREC>
__host__ __device__ constexpr int distance_group_size() {
  return C == 0 ? 4 : (PREC == kPrecBF16 && C <= 4) ? 8 : C <= 4 ? 8 : 2;
}

// One group of rows with the query in registers (C > 0, scalar path): all
// G loads first, unconditionally (a short group re-reads its first row), so
// they are issued back to back before any use.
template <int C, int PREC>
__device__ __forceinline__ void regs_group(const SearchArgs& a, const float (&qv)[qregs(C)], const int* s_ids,
                                           float* s_dist, int n, int lane, int g0) {
  constexpr int G = distance_group_size<C, PREC>();
  RowLoader<C, PREC> r[G];
#pragma unroll
  for (int t = 0; t < G; ++t) r[t].load(a, s_ids[g0 + t < n ? g0 + t : g0], lane);
  float part[G];
#pragma unroll
  for (int t = 0; t < G; ++t) part[t] = g0 + t < n ? lane_partial<C>(r[t].v, qv) : 0.0f;
  reduce_rows<G>(part, s_dist, g0, n, lane);
}

// Group `grp` (rows grp*G ..) of a batch, on whichever path the kernel uses.
template <int C, int PREC>
__device__ __forceinline__ void distance_group(const SearchArgs& a, const float (&qv)[qregs(C)],
                                               const QueryExtra<C, PREC>& qx, const int* s_ids,
                                               float* s_dist, int n, int lane, int grp) {
  constexpr int G = distance_group_size<C, PREC>();
  if constexpr (C == 0)
    rt_group<PREC>(a, qx.qs, s_ids, s_dist, n, lane, G * grp);
  else if constexpr (PREC == kPrecBF16 && C <= 4)
    mma_group<C>(a, qx, s_ids, s_dist, n, lane, G * grp);
  else
    regs_group<C, PREC>(a, qv, s_ids, s_dist, n, lane, G * grp);
}

// The L2 prefetch a batch's distances start with (the whole batch, or the
// first window of a large one), for a warp that computes any of its groups.
template <int C, int PREC>
__device__ __forceinline__ void prefetch_batch(const SearchArgs& a, const int* s_ids, int n, int lane) {
  constexpr int G = distance_group_size<C, PREC>();
  const int rb = 32 * (C == 0 ? a.C : C) * slab_bytes<PREC>();
  const int lines = (rb + 127) / 128;
  prefetch_local<G>(search_rows<PREC>(a), rb, lines, s_ids, n, lane, 0, 1, 0,
                    prefetch_first(n, rb, prefetch_ahead(rb, G)));
}

// ---- helping in the tail ----
// When the query counter runs out, the warps left without a query help the
// warps of their block still searching: a leader with idle warps in its
// block publishes each batch's distance phase, and leader and helpers take
// its groups of rows from one ticket.  Every row's arithmetic is the
// leader's own, so results are unchanged.  While no warp of the block is
// idle (all but the last queries) a leader only reads the idle count.
struct PhaseDesc {
  unsigned long long ticket;  // (generation << 32) | next group to take
  unsigned long long gen_n;   // (generation << 32) | rows of the phase, one word
  int q;                      // the phase's query
  float qn;                   // its BF16 squared norm (tensor-core distances)
  int done;                   // groups finished by helpers
  int pad;
};
struct BlockShare {
  unsigned int idle;          // warps of the block with no query left
  unsigned int pad[3];
  PhaseDesc desc[8];
};
static_assert(sizeof(BlockShare) == kBlockShareBytes, "block share layout");

// The kernels that help in the tail: the tensor-core BF16 rows and the rows
// of any chunk count, with batches of up to 64 slots.  The scalar register
// path (FP32 and FP8 rows of up to 4 chunks, and 30 chunks) holds a group of
// rows in registers, and a second copy of it for the helped phase made those
// kernels spill at 64 registers.  Batches of 128 and 256 slots measured
// slower helped (one ticket per group of 8 rows over 16-32 groups).
template <int C, int PREC, int NB>
__host__ __device__ constexpr bool tail_helping() {
  return (C == 0 || (PREC == kPrecBF16 && C >= 1 && C <= 4)) && NB <= 2;
}

constexpr long long kHelpWaitLimit = 1ll << 24;   // leader's polls for helpers' groups
constexpr long long kHelperIdleLimit = 1ll << 21; // empty scans (~0.4 s) before a helper leaves

// The block's share, after its warps' regions (per_warp words each; a
// multiple of 4, so 16-byte aligned).
__device__ __forceinline__ BlockShare* block_share(uint32_t* smem, int per_warp) {
  return reinterpret_cast<BlockShare*>(smem + (size_t)(blockDim.x >> 5) * per_warp);
}

// The leader's side of a helped distance phase.  Publishes (q, qn, n) and
// the generation, takes groups from the ticket, then waits for the groups
// helpers took (bounded; on timeout the error word is set).
template <int C, int PREC>
__device__ __forceinline__ void helped_distances(const SearchArgs& a, const float (&qv)[qregs(C)],
                                                 const QueryExtra<C, PREC>& qx, const int* s_ids,
                                                 float* s_dist, int n, int lane, int q, float qn,
                                                 BlockShare* bs) {
  constexpr int G = distance_group_size<C, PREC>();
  PhaseDesc& d = bs->desc[threadIdx.x >> 5];
  const int ng = (n + G - 1) / G;
  if (lane == 0) {
    const unsigned gen = (unsigned)(*reinterpret_cast<volatile unsigned long long*>(&d.gen_n) >> 32) + 1u;
    d.q = q;
    d.qn = qn;
    d.done = 0;
    *reinterpret_cast<volatile unsigned long long*>(&d.gen_n) = ((unsigned long long)gen << 32) | (unsigned)n;
    __threadfence_block();
    atomicExch(&d.ticket, (unsigned long long)gen << 32);
  }
  __syncwarp();
  prefetch_batch<C, PREC>(a, s_ids, n, lane);
  int mine = 0;
  for (;;) {
    unsigned long long old = 0;
    if (lane == 0) old = atomicAdd(&d.ticket, 1ull);
    const int grp = (int)__shfl_sync(kFull, (unsigned)old, 0);
    if (grp >= ng) break;
    distance_group<C, PREC>(a, qv, qx, s_ids, s_dist, n, lane, grp);
    ++mine;
  }
  if (lane == 0) {
    const int expect = ng - mine;  // every group below ng was taken by someone
    long long it = 0;
    while (*reinterpret_cast<volatile int*>(&d.done) < expect) {
      if (++it > kHelpWaitLimit) {
        if (a.err) atomicExch(a.err, kErrHelpWait);
        break;
      }
    }
    __threadfence_block();
  }
  __syncwarp();
}

template <int C, int PREC, bool TEAM = false>
__device__ __forceinline__ void distances(const SearchArgs& a, const float (&qv)[qregs(C)],
                                          const QueryExtra<C, PREC>& qx, const int* s_ids,
                                          float* s_dist, int n, int lane, int w = 0, int K = 1) {
  if constexpr (C == 0) {
    distances_rt<PREC, TEAM>(a, qx.qs, s_ids, s_dist, n, lane, w, K);
  } else if constexpr (PREC == kPrecBF16 && C <= 4) {
    distances_mma<C, TEAM>(a, qx, s_ids, s_dist, n, lane, w, K);
  } else {
    constexpr int G = C <= 4 ? 8 : 2;
    constexpr int kRowBytes = 32 * C * (PREC == kPrecF32 ? 4 : PREC == kPrecBF16 ? 2 : 1);
    constexpr int kLines = (kRowBytes + 127) / 128, kAhead = prefetch_ahead(kRowBytes, G);
    const char* rows = PREC == kPrecF32    ? reinterpret_cast<const char*>(a.base)
                       : PREC == kPrecBF16 ? reinterpret_cast<const char*>(a.base_bf16)
                                           : reinterpret_cast<const char*>(a.base_fp8);
    const int ws = TEAM ? w : 0, ks = TEAM ? K : 1;
    const int first_rows = prefetch_first(n, kRowBytes, kAhead);
    prefetch_local<G>(rows, kRowBytes, kLines, s_ids, n, lane, ws, ks, 0, first_rows);
    const int first = G * ws, step = G * ks;
    auto group = [&](int g0) { regs_group<C, PREC>(a, qv, s_ids, s_dist, n, lane, g0); };
    // the window's loop is a copy of its own: the whole-batch loop keeps no
    // window state in the registers these rows fill
    if (first_rows >= n) {
      for (int g0 = first; g0 < n; g0 += step) group(g0);
    } else {
      int j = 0;
      for (int g0 = first; g0 < n; g0 += step, ++j) {
        prefetch_local<G>(rows, kRowBytes, kLines, s_ids, n, lane, ws, ks, kAhead + G * j, kAhead + G * j + G);
        group(g0);
      }
    }
  }
}

// Compact the valid batch ids (0 <= id < np) into s_ids in slot order,
// compute their distances, and scatter them back (invalid slots -> MAX).
// With TEAM, the team's warps share the distances (team leader only).
// Alone (not TEAM), with bs, idle warps of the block may help (tail).
template <int C, int NB, int PREC, bool TEAM = false>
__device__ __forceinline__ int batch_distances(const SearchArgs& a, const float (&qv)[qregs(C)],
                                               const QueryExtra<C, PREC>& qx,
                                               float (&bd)[batch_regs(NB)],
                                               const int (&bi)[batch_regs(NB)], int* s_ids,
                                               float* s_dist, int lane, const Team& t = Team(),
                                               int q = 0, BlockShare* bs = nullptr) {
  constexpr int BR = batch_regs(NB);
  const unsigned lt = (1u << lane) - 1u;
  int kidx[BR];
  int n = 0;
#pragma unroll
  for (int j = 0; j < BR; ++j) {
    const bool v = bi[j] >= 0 && bi[j] < a.np;
    const unsigned m = __ballot_sync(kFull, v);
    kidx[j] = v ? n + __popc(m & lt) : -1;
    if (v) s_ids[kidx[j]] = bi[j];
    n += __popc(m);
  }
  if constexpr (TEAM) {
    if (lane == 0) t.ctl[1] = n;
    team_sync(t);
    distances<C, PREC, true>(a, qv, qx, s_ids, s_dist, n, lane, 0, t.K);
    team_sync(t);
  } else {
    __syncwarp();
    constexpr int G = distance_group_size<C, PREC>();
    if (tail_helping<C, PREC, NB>() && bs && n > G && *reinterpret_cast<volatile unsigned*>(&bs->idle) != 0u) {
      float qn = 0.0f;
      if constexpr (PREC == kPrecBF16 && C >= 1 && C <= 4) qn = qx.qn;
      if constexpr (tail_helping<C, PREC, NB>()) helped_distances<C, PREC>(a, qv, qx, s_ids, s_dist, n, lane, q, qn, bs);
    } else {
      distances<C, PREC>(a, qv, qx, s_ids, s_dist, n, lane);
    }
    __syncwarp();
  }
#pragma unroll
  for (int j = 0; j < BR; ++j) bd[j] = kidx[j] >= 0 ? s_dist[kidx[j]] : kMaxDist;
  __syncwarp();
  return n;
}


// Exact FP32 rerank of the final pool for the reduced-precision paths: the
// pool ids (visited marks dropped) get FP32 distances computed exactly as
// the FP32 path computes them, then the pool is bitonic-sorted ascending.
// The reference's precedent is the host-side parallel_reorder
// (graph_helper.cu:146-213), which recomputes FP32 L2 and std::sorts.
template <int C, int NL, bool TEAM = false>
__device__ __forceinline__ void rerank_pool(const SearchArgs& a, const float (&qv)[qregs(C)],
                                            const float* qsm, float (&pd)[pool_regs(NL)],
                                            int (&pi)[pool_regs(NL)], int* s_ids, float* s_dist,
                                            int lane, const Team& t = Team()) {
  constexpr int PR = pool_regs(NL);
  const unsigned lt = (1u << lane) - 1u;
  int kidx[PR];
  int n = 0;
#pragma unroll
  for (int j = 0; j < PR; ++j) {
    pi[j] = pi[j] < 0 ? -pi[j] : pi[j];
    const bool v = pi[j] < a.np;
    const unsigned m = __ballot_sync(kFull, v);
    kidx[j] = v ? n + __popc(m & lt) : -1;
    if (v) s_ids[kidx[j]] = pi[j];
    n += __popc(m);
  }
  QueryExtra<C, kPrecF32> q32{};
  if constexpr (C == 0) q32.qs = qsm;
  if constexpr (TEAM) {
    if (lane == 0) t.ctl[1] = n | (1 << 16);
    team_sync(t);
    distances<C, kPrecF32, true>(a, qv, q32, s_ids, s_dist, n, lane, 0, t.K);
    team_sync(t);
  } else {
    __syncwarp();
    distances<C, kPrecF32>(a, qv, q32, s_ids, s_dist, n, lane);
    __syncwarp();
  }
#pragma unroll
  for (int j = 0; j < PR; ++j) pd[j] = kidx[j] >= 0 ? s_dist[kidx[j]] : kMaxDist;
  __syncwarp();
  sort_batch_desc<PR, false, pool_slots(NL)>(pd, pi, lane);
}

// One query.  Batch slot p (lane p % 32 of register p / 32) belongs to the
// (p / R)-th node selected in the iteration and holds entry p % R of its
// neighbour list.  For R >= 32 a node's list fills R / 32 whole registers
// (register j holds node j / (R / 32)); R16 kernels serve degree-16 graphs,
// whose lists fill half a register (slot p holds node p / 16).
// The query's registers and shared-memory slot: FP32 chunks in registers
// (C > 0; plus its BF16 row in q_slot for the tensor-core distances), or the
// FP32 row in q_slot in the base's interleaved layout (C == 0).
template <int C, int PREC>
__device__ __forceinline__ void load_query(const SearchArgs& a, int q, int lane, float (&qv)[qregs(C)],
                                           QueryExtra<C, PREC>& qx, uint32_t* q_slot) {
  if constexpr (C == 0) {
    float* qs = reinterpret_cast<float*>(q_slot);
    for (int c = 0; c < a.C; ++c) {
      const int dim = lane + 32 * c;
      qs[interleaved_offset(c, lane, a.C)] = dim < a.d ? __ldg(a.queries + (size_t)q * a.qstride + dim) : 0.0f;
    }
    qv[0] = 0.0f;
    qx.qs = qs;
    __syncwarp();
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int dim = lane + 32 * c;
      qv[c] = dim < a.d ? __ldg(a.queries + (size_t)q * a.qstride + dim) : 0.0f;
    }
    if constexpr (PREC == kPrecBF16 && C <= 4) make_query_extra<C>(qx, qv, q_slot, lane);
  }
}

template <int C, int NL, int NB, int PREC, bool R16, bool TEAM = false>
__device__ __forceinline__ void search_query(const SearchArgs& a, int q, int lane, const Bloom& bloom,
                                             int* s_ids, float* s_dist, uint32_t* q_slot,
                                             const Team& t = Team(), BlockShare* bs = nullptr) {
  constexpr int L = pool_slots(NL);
  constexpr int PR = pool_regs(NL);  // pool registers
  constexpr int BR = batch_regs(NB);  // batch registers
  // the merge reads batch registers BR - min(PR, BR) .. BR-1 only
  constexpr int kMergeFrom = BR - (PR < BR ? PR : BR);
  constexpr int B = batch_slots(NB);
  static_assert(R16 || NB > 0, "a 16-slot batch comes from a degree-16 graph");
  const int np = a.np;
  const int R = R16 ? 16 : a.R;
  const int NR = R >> 5;               // batch registers per node (R >= 32)
  const int nr_shift = __ffs(NR) - 1;  // j / NR == j >> nr_shift
  int c_entries = 0, c_expanded = 0, c_dists = 0;  // per query: far below 2^31

  float qv[qregs(C)];
  QueryExtra<C, PREC> qx;
  load_query<C, PREC>(a, q, lane, qv, qx, q_slot);

  float pd[PR];
  int pi[PR];
#pragma unroll
  for (int j = 0; j < PR; ++j) {
    pd[j] = kMaxDist;
    pi[j] = np;
  }
  float bd[BR];
  int bi[BR];

  bloom.clear(lane);
  __syncwarp();

  // ---- entry phase (graph_search.cuh:479-959) ----
  // kd-tree entries from several leaves (mode 1, max_hits H > 1, the
  // reference's multi-hit entry, entry_helper.cu:5-241): every point of each
  // leaf, leaf h in slots [h*cap, (h+1)*cap), -1 leaves as padding,
  // max(L, H*cap) entry slots; the pool keeps the best L.
  const int H = a.entry_mode == 1 ? a.max_hits : 1;
  int hit = a.entry_mode != 0 ? __ldg(a.hits + (size_t)q * H) : 0;
  if (hit < 0 || hit >= a.n_leaves) hit = 0;
  const int32_t* lp = a.leaf_pids + (size_t)hit * a.leaf_cap;
  // learned entries (mode 2): every point of the proposed leaf, then every
  // point of the kd-tree leaf, max(L, both leaves) entry slots in all; the
  // pool keeps the best L of them.  Modes 0 and 1 have L entry slots (:479).
  int hit2 = a.entry_mode == 2 ? __ldg(a.hits2 + q) : -1;
  if (hit2 >= a.n_leaves || hit2 == hit) hit2 = -1;
  const int32_t* lp2 = a.leaf_pids + (size_t)(hit2 < 0 ? 0 : hit2) * a.leaf_cap;
  const int n_first = a.leaf_cap;
  const int n_second = hit2 >= 0 ? a.leaf_cap : 0;
  const int n_entries = a.entry_mode == 2 ? max(L, n_first + n_second)
                        : H > 1            ? max(L, H * a.leaf_cap)
                                           : L;
  uint32_t seed0 = (uint32_t)q * 64u + (uint32_t)lane;  // reference thread `lane`
  uint32_t seed1 = seed0 + 32u;                           // reference thread `lane + 32`
  const int n_ebatch = (n_entries + B - 1) / B;
#pragma unroll 1
  for (int it = 0; it < n_ebatch; ++it) {
#pragma unroll
    for (int j = 0; j < BR; ++j) {
      const int slot = (j << 5) + lane;
      const int pos = it * B + slot;
      int id = np;
      if (slot < B && pos < n_entries) {
        if (a.entry_mode == 0) {
          uint32_t& s = (j & 1) ? seed1 : seed0;
          s = s * 1103515245u + 12345u;
          id = (int)(s % (uint32_t)np);
        } else if (H > 1) {
          const int h = pos / a.leaf_cap, s = pos - h * a.leaf_cap;
          const int lf = h < H ? __ldg(a.hits + (size_t)q * H + h) : -1;
          if (lf >= 0 && lf < a.n_leaves) id = __ldg(a.leaf_pids + (size_t)lf * a.leaf_cap + s);
        } else if (pos < n_first) {
          id = __ldg(lp + pos);
        } else if (hit2 >= 0 && pos < n_first + n_second) {
          id = __ldg(lp2 + pos - n_first);
        }
        bloom.add((uint32_t)id);  // every entry, padding included (:490)
      }
      bi[j] = id;
    }
    __syncwarp();
    c_entries += batch_distances<C, NB, PREC, TEAM>(a, qv, qx, bd, bi, s_ids, s_dist, lane, t, q, bs);
    if (batch_can_enter<NL, NB>(pd, bd)) {
      sort_batch_desc<BR, true, B, kMergeFrom>(bd, bi, lane);
      merge_pool<NL, NB>(pd, pi, bd, bi, false, lane);
    }
  }

  // ---- main loop (graph_search.cuh:961-1532) ----
  uint32_t tmp_flag = L >= 32 ? 0xFFFFFFFFu : ((1u << L) - 1u);  // (1 << min(L,32)) - 1 (:969)
  int iteration = 0;
  bool cz = false;  // this lane's check_zero (:967)
  int hash_iteration = 0;
  int iter = 0;

  auto scan = [&](int chunk) -> uint32_t {  // :1019-1028, :1495-1510
    bool pred = false;
    if (chunk < PR && (L >= 32 || lane < L)) {
      const int id = pick<PR>(pi, chunk);
      if (id > 0 && id < np) {
        pred = true;
      } else if (id == 0 && !cz) {
        cz = true;
        pred = true;
      }
    }
    return __ballot_sync(kFull, pred);
  };

#pragma unroll 1
  while (iter < a.max_iter) {
    iter++;
    // select up to W unvisited pool slots in pool order; mark them visited by
    // negating the id (:986-1031).  nodes[s]: the s-th selected node (R >=
    // 32); slot_node[j]: the node whose list fills this lane's slot of batch
    // register j (R16).
    int nodes[R16 ? 1 : BR];
    int slot_node[R16 ? BR : 1];
    int nsel = 0;
#pragma unroll 1
    while (nsel < a.W && tmp_flag != 0) {
      const int pos = __ffs(tmp_flag) - 1;
      const int chunk = iteration;
      const int v = __shfl_sync(kFull, pick<PR>(pi, chunk), pos);
      if (lane == pos) {
#pragma unroll
        for (int j = 0; j < PR; ++j)
          if (j == chunk) pi[j] = -pi[j];
      }
      tmp_flag &= ~(1u << pos);
      const int node = v < 0 ? -v : v;
      if constexpr (R16) {
#pragma unroll
        for (int j = 0; j < BR; ++j)
          if ((((j << 5) + lane) >> 4) == nsel) slot_node[j] = node;
        if (lane == 0) c_expanded += node < np ? 1 : 0;
      } else {
#pragma unroll
        for (int s = 0; s < BR; ++s)
          if (s == nsel) nodes[s] = node;
      }
      nsel++;
      if (nsel == a.W) break;
      while (tmp_flag == 0 && iteration < PR) {
        iteration++;
        tmp_flag = scan(iteration);
      }
    }
    if (nsel == 0) break;
    // the next unvisited pool node, often the next iteration's choice: its
    // adjacency row into L2 while this iteration's rows are gathered (the
    // reduced-precision paths, which latency bounds; the FP32 path is
    // bandwidth-bound and loses more to the prefetches that miss)
    if (PREC != kPrecF32 && tmp_flag != 0) {
      const int u = __shfl_sync(kFull, pick<PR>(pi, iteration), __ffs(tmp_flag) - 1);
      if (u >= 0 && u < np && lane < ((R + 31) >> 5))
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a.graph + (size_t)u * R + 32 * lane));
    }

    // neighbour rows of the selected nodes (:995-1010); a node id >= np
    // expands nothing (the reference would read past the graph)
#pragma unroll
    for (int j = 0; j < BR; ++j) {
      int id = np;
      if constexpr (R16) {
        const int slot = (j << 5) + lane;
        if (slot < B && (slot >> 4) < nsel) {
          const int node = slot_node[j];
          if (node < np) id = __ldg(a.graph + (size_t)node * 16 + (slot & 15));
        }
      } else {
        const int s = j >> nr_shift;
        if (s < nsel) {
          const int node = pick<BR>(nodes, s);
          if (node < np) id = __ldg(a.graph + (size_t)node * R + ((j - s * NR) << 5) + lane);
        }
      }
      bi[j] = id;
    }
    // canonical rule: every test of one list sees the filter before any add
    // of that list; lists in selection order
    if constexpr (R16) {
#pragma unroll 1
      for (int s = 0; s < nsel; ++s) {
        bool pass[BR];
#pragma unroll
        for (int j = 0; j < BR; ++j) {
          pass[j] = false;
          if ((((j << 5) + lane) >> 4) == s) pass[j] = bi[j] != np && !bloom.test((uint32_t)bi[j]);
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < BR; ++j) {
          if ((((j << 5) + lane) >> 4) == s) {
            if (pass[j])
              bloom.add((uint32_t)bi[j]);
            else
              bi[j] = np;
          }
        }
        __syncwarp();
      }
    } else {
#pragma unroll
      for (int s = 0; s < BR; ++s) {
        if (s >= nsel) break;
        if (lane == 0) c_expanded += pick<BR>(nodes, s) < np ? 1 : 0;
        bool pass[BR];
#pragma unroll
        for (int j = 0; j < BR; ++j) {
          pass[j] = false;
          if ((j >> nr_shift) == s) pass[j] = bi[j] != np && !bloom.test((uint32_t)bi[j]);
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < BR; ++j) {
          if ((j >> nr_shift) == s) {
            if (pass[j])
              bloom.add((uint32_t)bi[j]);
            else
              bi[j] = np;
          }
        }
        __syncwarp();
      }
    }

    c_dists += batch_distances<C, NB, PREC, TEAM>(a, qv, qx, bd, bi, s_ids, s_dist, lane, t, q, bs);
    {
      // batch slots below the pool's largest distance: none -> the merge
      // changes nothing (batch_can_enter); a few distinct ones -> placed
      // by rank (merge_few); otherwise the reference's network
      const float pmax = __shfl_sync(kFull, pd[PR - 1], NL == 0 ? 15 : 31);
      int m = 0;
      bool nan = false;
#pragma unroll
      for (int j = 0; j < BR; ++j) {
        m += __popc(__ballot_sync(kFull, bd[j] < pmax));
        nan |= bd[j] != bd[j];
      }
      if (m > 0 && (m > kFewMax || __any_sync(kFull, nan) || !merge_few<NL, NB>(pd, pi, bd, bi, pmax, lane))) {
        sort_batch_desc<BR, true, B, kMergeFrom>(bd, bi, lane);
        merge_pool<NL, NB>(pd, pi, bd, bi, true, lane);
      }
    }

    bool any = false;
#pragma unroll 1
    for (iteration = 0; iteration < PR; iteration++) {
      tmp_flag = scan(iteration);
      if (tmp_flag != 0) {
        any = true;
        break;
      }
    }
    if (hash_iteration == 4) {  // rebuild from the pool (:1518-1529)
      __syncwarp();
      bloom.clear(lane);
      __syncwarp();
#pragma unroll
      for (int j = 0; j < PR; ++j) {
        const int id = pi[j] < 0 ? -pi[j] : pi[j];
        if (id < np) bloom.add((uint32_t)id);
      }
      __syncwarp();
      hash_iteration = 0;
    }
    hash_iteration++;
    if (!any) break;
  }

  // ---- exact FP32 rerank of the final pool (precision paths) ----
  if (PREC != kPrecF32 && a.rerank)
    rerank_pool<C, NL, TEAM>(a, qv, reinterpret_cast<const float*>(q_slot), pd, pi, s_ids, s_dist, lane, t);
  if constexpr (TEAM) {  // releases the helpers
    if (lane == 0) t.ctl[1] = -1;
    team_sync(t);
  }

  // ---- output (:1959-1963) ----
#pragma unroll
  for (int j = 0; j < PR; ++j) {
    const int i = (j << 5) + lane;
    if (i < a.k) {
      a.out_ids[(size_t)q * a.k + i] = pi[j] < 0 ? -pi[j] : pi[j];
      if (a.out_dists) a.out_dists[(size_t)q * a.k + i] = pd[j];
    }
  }
  if (a.counters && lane == 0) {
    long long* c = a.counters + (size_t)q * 4;
    c[0] = c_entries;
    c[1] = c_expanded;
    c[2] = c_dists;
    c[3] = iter;
  }
}

// A team member other than the leader, for one query: the query in its own
// registers and slot, then its share of every distance phase the leader
// opens, until the leader ends the query.
template <int C, int PREC>
__device__ __forceinline__ void help_query(const SearchArgs& a, int q, int lane, const int* s_ids,
                                           float* s_dist, uint32_t* q_slot, const Team& t) {
  float qv[qregs(C)];
  QueryExtra<C, PREC> qx;
  load_query<C, PREC>(a, q, lane, qv, qx, q_slot);
  for (;;) {
    team_sync(t);
    const int code = t.ctl[1];
    if (code < 0) break;
    const int n = code & 0xffff;
    if (code >> 16) {  // the exact FP32 rerank of the final pool
      QueryExtra<C, kPrecF32> q32{};
      if constexpr (C == 0) q32.qs = reinterpret_cast<const float*>(q_slot);
      distances<C, kPrecF32, true>(a, qv, q32, s_ids, s_dist, n, lane, t.w, t.K);
    } else {
      distances<C, PREC, true>(a, qv, qx, s_ids, s_dist, n, lane, t.w, t.K);
    }
    team_sync(t);
  }
}

// A warp with no query left: helps the block's searching warps with their
// distance phases until every warp of the block is idle (or, as a safety
// bound, after kHelperIdleLimit scans that found nothing).  A group is taken
// only through the leader's ticket, and only when the ticket's generation
// matches the published (generation, rows) word read after taking it, so a
// stale take of an ended phase is dropped; the leader cannot end a phase
// while a group it counts on is being computed.
template <int C, int NL, int NB, int PREC>
__device__ __noinline__ void help_block(const SearchArgs a, uint32_t* smem, int per_warp, int lane,
                                        BlockShare* bs) {
  constexpr int G = distance_group_size<C, PREC>();
  constexpr int S = batch_slots(NB) > pool_slots(NL) ? batch_slots(NB) : pool_slots(NL);
  const int wpb = blockDim.x >> 5, me = threadIdx.x >> 5;
  if (lane == 0) atomicAdd(&bs->idle, 1u);
  __syncwarp();
  float qv[qregs(C)];
#pragma unroll
  for (int c = 0; c < qregs(C); ++c) qv[c] = 0.0f;
  QueryExtra<C, PREC> qx{};
  long long empty = 0;
  for (;;) {
    if (*reinterpret_cast<volatile unsigned*>(&bs->idle) >= (unsigned)wpb) break;
    bool worked = false;
    for (int w = 0; w < wpb; ++w) {
      if (w == me) continue;
      PhaseDesc& d = bs->desc[w];
      const unsigned long long t0 = *reinterpret_cast<volatile unsigned long long*>(&d.ticket);
      const unsigned long long gn0 = *reinterpret_cast<volatile unsigned long long*>(&d.gen_n);
      if ((t0 >> 32) == 0 || (t0 >> 32) != (gn0 >> 32)) continue;
      if ((int)(unsigned)t0 >= ((int)(unsigned)gn0 + G - 1) / G) continue;
      unsigned long long old = 0;
      if (lane == 0) old = atomicAdd(&d.ticket, 1ull);
      old = __shfl_sync(kFull, old, 0);
      __threadfence_block();
      const unsigned long long gn = *reinterpret_cast<volatile unsigned long long*>(&d.gen_n);
      const unsigned gs = (unsigned)(old >> 32);
      const int grp = (int)(unsigned)old;
      const int n = (int)(unsigned)gn;
      if (gs == 0u || gs != (unsigned)(gn >> 32) || grp >= (n + G - 1) / G) continue;
      const int q = *reinterpret_cast<volatile int*>(&d.q);
      uint32_t* lb = smem + (size_t)w * per_warp;  // the leader's region
      const int* ls_ids = reinterpret_cast<const int*>(lb + a.bloom_words);
      float* ls_dist = reinterpret_cast<float*>(lb + a.bloom_words + S);
      const uint32_t* lslot = lb + a.bloom_words + 2 * S;
      // the leader's query: its shared-memory row, or the FP32 chunks again
      if constexpr (C == 0) {
        qx.qs = reinterpret_cast<const float*>(lslot);
      } else {
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const int dim = lane + 32 * c;
          qv[c] = dim < a.d ? __ldg(a.queries + (size_t)q * a.qstride + dim) : 0.0f;
        }
        if constexpr (PREC == kPrecBF16 && C <= 4) {
          qx.qs = lslot;
          qx.qn = *reinterpret_cast<volatile float*>(&d.qn);
        }
      }
      distance_group<C, PREC>(a, qv, qx, ls_ids, ls_dist, n, lane, grp);
      __syncwarp();
      if (lane == 0) {
        __threadfence_block();
        atomicAdd(&d.done, 1);
      }
      worked = true;
    }
    if (!worked) {
      __nanosleep(256);
      if (++empty > kHelperIdleLimit) break;
    }
  }
}

// Blocks of 8 warps per SM the register budget is set for: 4 (64 registers
// a thread), or 2 (128) for rows of more than 4 chunks in registers and for
// the kernels built for any chunk count with a pool or batch of 8
// registers.  Those spilled over 1 KB at 64 registers; at 128 the 960-d
// search with 256-slot pools and batches ran 1.5x faster on one GB300,
// while the specialised 96- and 128-d kernels of the same pool ran slower.
__host__ __device__ constexpr int search_min_blocks(int C, int NL, int NB) {
  return C > 4 || (C == 0 && (NL >= 8 || NB >= 8)) ? 2 : 4;
}

// The next query of the persistent loop (one lane): the work counter's
// next slot, through the order permutation when there is one (written for
// batches of more than a.order_min queries); nq or more once every query
// is taken.
__device__ __forceinline__ int next_query(const SearchArgs& a, int nq) {
  const int t = (int)atomicAdd(a.work, 1u);
  return a.order && nq > a.order_min && t < nq ? __ldg(a.order + t) : t;
}

template <int C, int NL, int NB, int PREC, bool R16 = false>
__global__ void __launch_bounds__(256, search_min_blocks(C, NL, NB)) search_kernel(SearchArgs a) {
  extern __shared__ uint32_t smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  constexpr int B = batch_slots(NB);
  constexpr int S = B > pool_slots(NL) ? B : pool_slots(NL);  // compaction slots per warp
  int qwords = kQuerySlotWords;
  if constexpr (C == 0) qwords = query_slot_words_for(0, a.C);
  const int per_warp = a.bloom_words + 2 * S + qwords;
  uint32_t* wbase = smem + (size_t)wib * per_warp;
  Bloom bloom;
  bloom.w = wbase;
  bloom.words_mask = (uint32_t)a.bloom_words - 1u;
  bloom.bits_mask = ((uint32_t)a.bloom_words << 5) - 1u;
  bloom.lw = __ffs(a.bloom_words) - 1;
  bloom.nh = a.bloom_hashes;
  int* s_ids = reinterpret_cast<int*>(wbase + a.bloom_words);
  float* s_dist = reinterpret_cast<float*>(s_ids + S);
  const int nq = a.nq_dev ? *a.nq_dev : a.nq;
  constexpr bool kHelps = tail_helping<C, PREC, NB>();
  BlockShare* bs = nullptr;
  if constexpr (kHelps) {
    bs = block_share(smem, per_warp);
    for (int i = threadIdx.x; i < kBlockShareBytes / 4; i += blockDim.x) reinterpret_cast<uint32_t*>(bs)[i] = 0u;
    __syncthreads();
  }
  for (;;) {
    int q = 0;
    if (lane == 0) q = next_query(a, nq);
    q = __shfl_sync(kFull, q, 0);
    if (q >= nq) break;
    search_query<C, NL, NB, PREC, R16>(a, q, lane, bloom, s_ids, s_dist,
                                       reinterpret_cast<uint32_t*>(s_dist + S), Team(), bs);
  }
  if constexpr (kHelps) help_block<C, NL, NB, PREC>(a, smem, per_warp, lane, bs);
}

// search_kernel with teams of K warps per query (Team): K = a.team, or,
// for a.team < 0, at least -a.team (one above kTeamFloorLoad times the
// grid's warps) and otherwise the most (up to 8) that the live query count
// leaves room for in the grid.  K = 1 runs as a team of one.  A kernel of its own, so
// that the single-warp kernel's code and register allocation stay as they
// are; a team never spans blocks (the launch keeps warps per block a
// multiple of K, and K falls back to 1 otherwise).
template <int C, int NL, int NB, int PREC, bool R16 = false>
__global__ void __launch_bounds__(256, search_min_blocks(C, NL, NB)) search_kernel_team(SearchArgs a) {
  extern __shared__ uint32_t smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  constexpr int B = batch_slots(NB);
  constexpr int S = B > pool_slots(NL) ? B : pool_slots(NL);
  int qwords = kQuerySlotWords;
  if constexpr (C == 0) qwords = query_slot_words_for(0, a.C);
  // per warp: filter, compaction words, query slot, then the team's control
  // words (used in the leader's region)
  const int per_warp = a.bloom_words + 2 * S + qwords + kTeamCtlWords;
  uint32_t* wbase = smem + (size_t)wib * per_warp;
  Bloom bloom;
  bloom.w = wbase;
  bloom.words_mask = (uint32_t)a.bloom_words - 1u;
  bloom.bits_mask = ((uint32_t)a.bloom_words << 5) - 1u;
  bloom.lw = __ffs(a.bloom_words) - 1;
  bloom.nh = a.bloom_hashes;
  const int nq = a.nq_dev ? *a.nq_dev : a.nq;
  const int wpb = blockDim.x >> 5;
  int K = a.team;
  if (K < 0) {  // at least -a.team warps, then as many as the live batch leaves room for
    const long long total = (long long)gridDim.x * wpb;
    K = -a.team;
    if ((long long)nq > kTeamFloorLoad * total) K = 1;  // the floor holds for moderate batches only
    while (K < 8 && wpb % (2 * K) == 0 && (long long)nq * 2 * K <= total) K *= 2;
  }
  if (K < 1 || K > 8 || wpb % K != 0) K = 1;
  Team t;
  t.K = K;
  t.w = wib & (K - 1);
  t.bar = 1 + wib / K;
  uint32_t* lbase = smem + (size_t)(wib - t.w) * per_warp;  // the leader's region
  t.ctl = reinterpret_cast<volatile int*>(lbase + per_warp - kTeamCtlWords);
  int* ts_ids = reinterpret_cast<int*>(lbase + a.bloom_words);
  float* ts_dist = reinterpret_cast<float*>(ts_ids + S);
  // this warp's own query slot, after its filter and compaction words
  uint32_t* own_slot = wbase + a.bloom_words + 2 * S;
  if (t.w == 0) {
    for (;;) {
      int q = 0;
      if (lane == 0) q = next_query(a, nq);
      q = __shfl_sync(kFull, q, 0);
      if (lane == 0) t.ctl[0] = q;
      team_sync(t);
      if (q >= nq) break;
      search_query<C, NL, NB, PREC, R16, true>(a, q, lane, bloom, ts_ids, ts_dist, own_slot, t);
    }
  } else {
    for (;;) {
      team_sync(t);
      const int q = t.ctl[0];
      if (q >= nq) break;
      help_query<C, PREC>(a, q, lane, ts_ids, ts_dist, own_slot, t);
    }
  }
}

}  // namespace rte
