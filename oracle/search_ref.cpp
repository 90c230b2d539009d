// search_ref.cpp -- ORACLE (test infrastructure, never the product).
//
// A sequential restatement of the reference's GraphSearchKernel
// (graph_search.cuh:56-1964, launched <<<nq, 64>>> at graph.cu:320).  The
// reference keeps, per query, one shared array `neighbors_array` of
// n_candidates + search_width*degree (dist, id) pairs: the sorted pool first,
// then the batch of freshly computed neighbours.  This file simulates that
// array and the exact comparator network applied to it.
//
// Canonical rules where the reference is racy or unspecified:
//   H2  ties: the comparator network with strict '<' / '>' is executed as if
//       every substep were separated by a barrier (the reference omits the
//       barrier between substeps of the batch sort, graph_search.cuh:888-919;
//       for batches of <= 64 slots only warp 0 sorts, so it is in lockstep).
//   H3  bloom race: all test() calls for one node's neighbour list see the
//       filter as it was before any add() of that list (graph_search.cuh:
//       998-1007 runs test and add concurrently across threads); lists are
//       processed in selection order.
//   H4  distance arithmetic: per virtual lane l, s = t0*t0 then
//       s = fmaf(tc, tc, s) over chunks c (t = p - q, dims l + 32c), then the
//       shuffle-down tree 16,8,4,2,1 (the reference is built with fmad on).
//   H5  check_zero is per lane (graph_search.cuh:967,1022-1026,1504-1509).
//   H7  the visited filter starts empty for every query.  The reference never
//       clears its `__shared__ uint data[SIZE]` (graph_search.cuh:88), so a
//       block starts with the bits the previous block on that SM left behind;
//       run one query per launch on zeroed shared memory, the reference
//       returns exactly what this restatement returns.
//   H6  a selected pool slot whose |id| >= np (only possible in the first
//       iteration when search_width exceeds the valid entries, because the
//       first selection mask is all ones, graph_search.cuh:969) expands no
//       neighbours; the reference reads past the graph there.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Pair {
  float d;
  int id;
};

// Hash multipliers of the visited-set bloom filter (graph_search.cuh:89-97).
const uint32_t kHashMul[20] = {
    0x924ed183U, 0xd854fc0aU, 0xecf5e3b7U, 0x1bead407U, 0x28a30449U,
    0xbfc4d99fU, 0x715030e2U, 0xffcfb45bU, 0x6e4ce166U, 0xeb53c362U,
    0xa93c4f40U, 0xcecde0a4U, 0x0288592dU, 0x362c37bcU, 0x9d4824f0U,
    0xfdbdd68bU, 0x63258c85U, 0x6726905cU, 0x609500f9U, 0x4de48422U};

// hash_ (graph_search.cuh:13-22) generalised from SIZE=512 words to `words`.
inline uint32_t bloom_hash(int h, uint32_t x, uint32_t words) {
  x ^= x >> 16;
  x *= kHashMul[h << 1];
  x ^= x >> 13;
  x *= kHashMul[(h << 1) + 1];
  x ^= x >> 16;
  return x % (words << 5);
}

struct Bloom {
  std::vector<uint32_t> data;
  uint32_t words;
  int hashes;
  Bloom(int w, int h) : data(w, 0u), words(w), hashes(h) {}
  // set_bit: word x % SIZE, bit x / SIZE (graph_search.cuh:7-11).
  void set(uint32_t bit) { data[bit % words] |= 1u << (bit / words); }
  bool get(uint32_t bit) const { return (data[bit % words] >> (bit / words)) & 1u; }
  void add(uint32_t x) {  // graph_search.cuh:30-33
    for (int i = 0; i < hashes; ++i) set(bloom_hash(i, x, words));
  }
  bool test(uint32_t x) const {  // graph_search.cuh:36-42
    bool ok = true;
    for (int i = 0; i < hashes; ++i) ok &= get(bloom_hash(i, x, words));
    return ok;
  }
  void clear() { std::fill(data.begin(), data.end(), 0u); }
};

inline void cswap(Pair& a, Pair& b) {
  Pair t = a;
  a = b;
  b = t;
}

// Bitonic sort of n slots, final order descending (graph_search.cuh:888-919).
// Pair index i, distance sub, stage step: a = (i/sub)*2*sub + i%sub; the
// direction is descending when (i/step) is even.
void batch_sort_desc(Pair* v, int n) {
  for (int step = 1; step <= n / 2; step *= 2)
    for (int sub = step; sub >= 1; sub /= 2)
      for (int i = 0; i < n / 2; ++i) {
        int a = (i / sub) * 2 * sub + (i & (sub - 1));
        int b = a + sub;
        if (((i / step) & 1) == 0) {
          if (v[a].d < v[b].d) cswap(v[a], v[b]);
        } else {
          if (v[a].d > v[b].d) cswap(v[a], v[b]);
        }
      }
}

// Merge of the descending batch into the ascending pool (graph_search.cuh:
// 921-931 for entries, 1454-1464 in the main loop where a MAX batch slot is
// skipped), then the ascending half-cleaner over the pool (:933-957).
void merge_pool(Pair* na, int L, int B, bool skip_max) {
  int ncmp = std::min(L, B);
  for (int i = 0; i < ncmp; ++i) {
    int a = L - ncmp + i;
    int b = a + B;
    if (skip_max && na[b].d == ORC_MAX_DIST) continue;
    if (na[a].d > na[b].d) cswap(na[a], na[b]);
  }
  for (int sub = L / 2; sub >= 1; sub /= 2)
    for (int i = 0; i < L / 2; ++i) {
      int a = (i / sub) * 2 * sub + (i & (sub - 1));
      int b = a + sub;
      if (na[a].d > na[b].d) cswap(na[a], na[b]);
    }
}

inline uint32_t lcg_next(uint32_t& seed, uint32_t np) {  // random_entry, :50-54
  seed = seed * 1103515245u + 12345u;
  return seed % np;
}

}  // namespace

extern "C" float orc_l2_ref(const float* p, const float* q, int d) {
  const int chunks = (d + 31) / 32;
  float part[32];
  for (int l = 0; l < 32; ++l) {
    float s = 0.0f;
    for (int c = 0; c < chunks; ++c) {
      int dim = l + 32 * c;
      float pv = dim < d ? p[dim] : 0.0f;
      float qv = dim < d ? q[dim] : 0.0f;
      float t = pv - qv;
      s = (c == 0) ? t * t : std::fmaf(t, t, s);
    }
    part[l] = s;
  }
  for (int off = 16; off >= 1; off >>= 1)
    for (int l = 0; l < off; ++l) part[l] = part[l] + part[l + off];
  return part[0];
}

namespace {

struct SearchArgs {
  const float* base;
  const float* rerank_base;  // FP32 base for the final rerank, or null
  int64_t np;
  int d;
  const int32_t* graph;
  int degree;
  const int32_t* leaf_pids;
  int leaf_cap;
  int L, k, W, max_iter, bloom_words, bloom_hashes, entry_mode;
  int max_hits = 1;                   // entry mode 1: leaves per query
  const int32_t* hits_multi = nullptr;  // [nq][max_hits] when max_hits > 1, -1 padded
};

// One query, one "block" of the reference.
void search_one(const SearchArgs& A, const float* q, int64_t qid, int32_t hit, int32_t hit2, int32_t* out_ids,
                float* out_dists, orc_counters* cnt) {
  const int L = A.L, R = A.degree, W = A.W;
  const int B = W * R;
  const int np = (int)A.np;
  const int nchunks = (L + 31) / 32;
  std::vector<Pair> na(L + B, Pair{ORC_MAX_DIST, np});  // :473-477
  Pair* batch = na.data() + L;
  Bloom bloom(A.bloom_words, A.bloom_hashes);
  orc_counters c = {0, 0, 0, 0, 0, 0, 0};

  auto dist_of = [&](int id) { return orc_l2_ref(A.base + (int64_t)id * A.d, q, A.d); };
  // counts a merge, and whether any batch distance is below the pool's
  // largest the merge cannot change the pool)
  // (otherwise the merge cannot change the pool); for a main-loop batch,
  // also whether 1..8 pairwise distinct distances (no NaN) lie below it
  auto count_merge = [&](bool main_loop) {
    c.merges++;
    const float pmax = na[L - 1].d;
    float below[9];
    int m = 0;
    bool nan = false;
    for (int i = 0; i < B; ++i) {
      nan |= batch[i].d != batch[i].d;
      if (batch[i].d < pmax) {
        if (m < 9) below[m] = batch[i].d;
        ++m;
      }
    }
    if (m == 0) {
      c.merges_idle++;
      return;
    }
    if (!main_loop || nan || m > 8) return;
    for (int i = 0; i < m; ++i)
      for (int j = i + 1; j < m; ++j)
        if (below[i] == below[j]) return;
    c.merges_few++;
  };

  // ---- entry phase (:479-959) ----
  uint32_t seed[64];
  for (int t = 0; t < 64; ++t) seed[t] = (uint32_t)(qid * 64 + t);  // :64
  // Entry mode 2 (no reference counterpart): every point of the first leaf,
  // then every point of the second leaf (hit2), max(L, both) entry slots.
  const bool two = A.entry_mode == 2 && hit2 >= 0 && hit2 != hit;
  const int n_first = A.leaf_cap;
  const int n_second = two ? A.leaf_cap : 0;
  // Entry mode 1 with max_hits H > 1 (the reference's disabled multi-hit
  // entry, entry_helper.cu:5-241): every point of each of the H leaves
  // (slots h*leaf_cap + j, -1 leaves padded with np), max(L, H*leaf_cap)
  // entry slots; the pool keeps the best L.
  const int H = A.entry_mode == 1 ? A.max_hits : 1;
  const int32_t* hm = H > 1 ? A.hits_multi + qid * H : nullptr;
  const int n_entries = A.entry_mode == 2 ? std::max(L, n_first + n_second)
                        : H > 1            ? std::max(L, H * A.leaf_cap)
                                           : L;  // :479
  const int n_ebatch = (n_entries + B - 1) / B;
  for (int it = 0; it < n_ebatch; ++it) {
    for (int i = 0; i < B; ++i) {
      int j = it * B + i;
      if (j < n_entries) {
        int id;
        if (A.entry_mode == 0) {
          id = (int)lcg_next(seed[i % 64], (uint32_t)np);
        } else {
          // entry.cu:60-69 (mode 1: the leaf's points, then padding)
          if (H > 1) {
            const int h = j / A.leaf_cap, s = j - h * A.leaf_cap;
            const int lf = h < H ? hm[h] : -1;
            id = lf >= 0 ? A.leaf_pids[(int64_t)lf * A.leaf_cap + s] : np;
          } else if (j < n_first)
            id = A.leaf_pids[(int64_t)hit * A.leaf_cap + j];
          else if (j < n_first + n_second)
            id = A.leaf_pids[(int64_t)hit2 * A.leaf_cap + (j - n_first)];
          else
            id = np;
        }
        batch[i].id = id;
        bloom.add((uint32_t)id);  // :490 adds every entry, padding included
      } else {
        batch[i].id = np;
      }
      if (batch[i].id >= np) batch[i].d = ORC_MAX_DIST;
    }
    for (int i = 0; i < B; ++i)
      if (batch[i].id < np) {
        batch[i].d = dist_of(batch[i].id);
        c.entries_valid++;
      }
    count_merge(false);
    batch_sort_desc(batch, B);
    merge_pool(na.data(), L, B, false);
  }

  // ---- main loop (:961-1532) ----
  const int n_flag = std::min(std::min(L, 32), n_entries);
  uint32_t tmp_flag = n_flag >= 32 ? 0xFFFFFFFFu : ((1u << n_flag) - 1u);  // :969
  uint32_t check_zero = 0;  // bit l = lane l's check_zero (H5)
  int iteration = 0;
  bool flag_all = true;
  int iter = 0;
  int hash_iteration = 0;

  auto scan_chunk = [&](int chunk) -> uint32_t {  // :1019-1028 and :1495-1510
    uint32_t m = 0;
    for (int lane = 0; lane < 32; ++lane) {
      int pos = lane + 32 * chunk;
      if (pos >= L) continue;
      int id = na[pos].id;
      if (id > 0 && id < np) {
        m |= 1u << lane;
      } else if (id == 0) {
        if (!(check_zero & (1u << lane))) {
          check_zero |= 1u << lane;
          m |= 1u << lane;
        }
      }
    }
    return m;
  };

  std::vector<int> nbr(R);
  std::vector<char> pass(R);
  while (flag_all && iter < A.max_iter) {
    iter++;
    for (int i = 0; i < B; ++i) batch[i] = Pair{ORC_MAX_DIST, np};  // :979-983
    int search_cnt = 0;
    while (search_cnt < W && tmp_flag != 0) {
      int pos = __builtin_ctz(tmp_flag);
      int loc = iteration * 32 + pos;
      int node = std::abs(na[loc].id);
      na[loc].id = -na[loc].id;
      tmp_flag &= ~(1u << pos);
      Pair* slot = batch + search_cnt * R;
      if (node < np) {  // H6
        c.expanded++;
        const int32_t* row = A.graph + (int64_t)node * R;
        for (int i = 0; i < R; ++i) {  // H3: snapshot test, then adds
          nbr[i] = row[i];
          pass[i] = !(nbr[i] == np || bloom.test((uint32_t)nbr[i]));
        }
        for (int i = 0; i < R; ++i) {
          if (pass[i]) {
            slot[i].id = nbr[i];
            bloom.add((uint32_t)nbr[i]);
          } else {
            slot[i].id = np;
          }
        }
      } else {
        for (int i = 0; i < R; ++i) slot[i].id = np;
      }
      search_cnt++;
      if (search_cnt == W) break;
      while (tmp_flag == 0 && iteration < nchunks) {
        iteration++;
        tmp_flag = scan_chunk(iteration);
      }
    }
    if (search_cnt == 0) break;
    for (int i = 0; i < search_cnt * R; ++i) {  // :1036-1422
      if (batch[i].id >= np) {
        batch[i].d = ORC_MAX_DIST;
        continue;
      }
      batch[i].d = dist_of(batch[i].id);
      c.dist_evals++;
    }
    count_merge(true);
    batch_sort_desc(batch, B);
    merge_pool(na.data(), L, B, true);
    for (iteration = 0; iteration < nchunks; iteration++) {  // :1495-1516
      tmp_flag = scan_chunk(iteration);
      if (tmp_flag != 0) break;
      if (iteration == nchunks - 1) flag_all = false;
    }
    if (hash_iteration == 4) {  // :1518-1529
      bloom.clear();
      for (int i = 0; i < L; ++i) {
        int id = std::abs(na[i].id);
        if (id < np) bloom.add((uint32_t)id);
      }
      hash_iteration = 0;
    }
    hash_iteration++;
  }
  c.iterations = iter;

  if (A.rerank_base) {
    // exact FP32 rerank of the final pool (reduced-precision search paths):
    // ids without visited marks, FP32 distances on the full-precision base,
    // then a bitonic sort into ascending order (mirror of batch_sort_desc)
    for (int i = 0; i < L; ++i) {
      na[i].id = std::abs(na[i].id);
      na[i].d = na[i].id < np ? orc_l2_ref(A.rerank_base + (int64_t)na[i].id * A.d, q, A.d)
                              : ORC_MAX_DIST;
    }
    for (int step = 1; step <= L / 2; step *= 2)
      for (int sub = step; sub >= 1; sub /= 2)
        for (int i = 0; i < L / 2; ++i) {
          int a = (i / sub) * 2 * sub + (i & (sub - 1));
          int b = a + sub;
          if (((i / step) & 1) == 0) {
            if (na[a].d > na[b].d) cswap(na[a], na[b]);
          } else {
            if (na[a].d < na[b].d) cswap(na[a], na[b]);
          }
        }
  }

  for (int i = 0; i < A.k; ++i) {  // :1959-1963
    out_ids[i] = std::abs(na[i].id);
    if (out_dists) out_dists[i] = na[i].d;
  }
  if (cnt) *cnt = c;
}

}  // namespace

extern "C" int orc_search(const float* base, int64_t np, int d, const float* queries, int64_t nq,
                          const int32_t* graph, int degree, const int32_t* leaf_pids, int leaf_cap,
                          const int32_t* hits, int L, int k, int search_width, int max_iter,
                          int bloom_words, int bloom_hashes, int entry_mode, int32_t* out_ids,
                          float* out_dists, orc_counters* counters, int n_threads) {
  return orc_search_rerank(base, nullptr, np, d, queries, nq, graph, degree, leaf_pids, leaf_cap,
                           hits, nullptr, L, k, search_width, max_iter, bloom_words, bloom_hashes,
                           entry_mode, out_ids, out_dists, counters, n_threads);
}

extern "C" int orc_search_rerank(const float* base, const float* rerank_base, int64_t np, int d,
                                 const float* queries, int64_t nq, const int32_t* graph,
                                 int degree, const int32_t* leaf_pids, int leaf_cap,
                                 const int32_t* hits, const int32_t* hits2, int L, int k,
                                 int search_width, int max_iter,
                                 int bloom_words, int bloom_hashes, int entry_mode,
                                 int32_t* out_ids, float* out_dists, orc_counters* counters,
                                 int n_threads) {
  if (!base || !queries || !graph || !out_ids || np <= 0 || np >= (int64_t)INT32_MAX || d <= 0 ||
      nq < 0 || degree <= 0 || (degree & (degree - 1)) || L <= 0 || (L & (L - 1)) || k <= 0 ||
      k > L || search_width <= 0 || max_iter < 0 || bloom_words <= 0 ||
      (bloom_words & (bloom_words - 1)) || bloom_hashes <= 0 || bloom_hashes > 10)
    return -1;
  if (entry_mode != 0 && (!leaf_pids || !hits || leaf_cap <= 0)) return -1;
  if (entry_mode == 2 && !hits2) return -1;
  if (entry_mode < 0 || entry_mode > 2) return -1;
  SearchArgs A{base, rerank_base, np, d, graph, degree, leaf_pids, leaf_cap, L, k, search_width,
               max_iter, bloom_words, bloom_hashes, entry_mode};
#ifdef _OPENMP
  if (n_threads <= 0) n_threads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic, 4) num_threads(n_threads)
#endif
  for (int64_t qi = 0; qi < nq; ++qi) {
    search_one(A, queries + qi * d, qi, entry_mode != 0 ? hits[qi] : 0,
               entry_mode == 2 ? hits2[qi] : -1, out_ids + qi * k,
               out_dists ? out_dists + qi * k : nullptr, counters ? counters + qi : nullptr);
  }
  (void)n_threads;
  return 0;
}

// Entry mode 1 with several leaves per query: hits_multi [nq][max_hits]
// (-1 padded), the H smallest containing leaf indices (orc_locate_multi).
extern "C" int orc_search_multi(const float* base, int64_t np, int d, const float* queries,
                                int64_t nq, const int32_t* graph, int degree,
                                const int32_t* leaf_pids, int leaf_cap, const int32_t* hits_multi,
                                int max_hits, int L, int k, int search_width, int max_iter,
                                int bloom_words, int bloom_hashes, int32_t* out_ids,
                                float* out_dists, orc_counters* counters, int n_threads) {
  if (!base || !queries || !graph || !out_ids || !leaf_pids || !hits_multi || leaf_cap <= 0 ||
      max_hits < 1 || np <= 0 || np >= (int64_t)INT32_MAX || d <= 0 || nq < 0 || degree <= 0 ||
      (degree & (degree - 1)) || L <= 0 || (L & (L - 1)) || k <= 0 || k > L || search_width <= 0 ||
      max_iter < 0 || bloom_words <= 0 || (bloom_words & (bloom_words - 1)) || bloom_hashes <= 0 ||
      bloom_hashes > 10)
    return -1;
  SearchArgs A{base, nullptr, np, d, graph, degree, leaf_pids, leaf_cap, L, k, search_width,
               max_iter, bloom_words, bloom_hashes, 1};
  A.max_hits = max_hits;
  A.hits_multi = hits_multi;
#ifdef _OPENMP
  if (n_threads <= 0) n_threads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic, 4) num_threads(n_threads)
#endif
  for (int64_t qi = 0; qi < nq; ++qi) {
    const int32_t h0 = hits_multi[qi * max_hits];
    search_one(A, queries + qi * d, qi, h0 >= 0 ? h0 : 0, -1, out_ids + qi * k,
               out_dists ? out_dists + qi * k : nullptr, counters ? counters + qi : nullptr);
  }
  (void)n_threads;
  return 0;
}

// Exact rerank of final pools against the original vectors: the GPU form of
// the reference's host-side REORDER (parallel_reorder, graph_helper.cu:146-213:
// FP32 L2 over the original rows of the L pool ids, sorted by distance, the
// first topk kept).  Distances follow rule H4 (orc_l2_ref); ids >= np get
// the MAX sentinel.  The sort is the ascending bitonic network over L slots
// (the reference's std::sort leaves ties unordered; this fixes them: rule H8).
extern "C" int orc_rerank_full(const float* base, int64_t np, int dim, const float* queries,
                               int64_t nq, const int32_t* pool, int L, int k, int32_t* out_ids,
                               float* out_dists, int n_threads) {
  if (!base || !queries || !pool || !out_ids || L <= 0 || (L & (L - 1)) || k <= 0 || k > L)
    return -1;
#ifdef _OPENMP
  if (n_threads <= 0) n_threads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads)
#endif
  for (int64_t qi = 0; qi < nq; ++qi) {
    std::vector<Pair> na(L);
    for (int i = 0; i < L; ++i) {
      int id = pool[qi * L + i];
      id = id < 0 ? -id : id;
      na[i].id = id;
      na[i].d = id < np ? orc_l2_ref(base + (int64_t)id * dim, queries + qi * dim, dim) : ORC_MAX_DIST;
    }
    for (int step = 1; step <= L / 2; step *= 2)
      for (int sub = step; sub >= 1; sub /= 2)
        for (int i = 0; i < L / 2; ++i) {
          int a = (i / sub) * 2 * sub + (i & (sub - 1));
          int b = a + sub;
          if (((i / step) & 1) == 0) {
            if (na[a].d > na[b].d) cswap(na[a], na[b]);
          } else {
            if (na[a].d < na[b].d) cswap(na[a], na[b]);
          }
        }
    for (int i = 0; i < k; ++i) {
      out_ids[qi * k + i] = na[i].id;
      if (out_dists) out_dists[qi * k + i] = na[i].d;
    }
  }
  (void)n_threads;
  return 0;
}
