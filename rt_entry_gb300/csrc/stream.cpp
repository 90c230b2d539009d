// stream.cpp -- uneven query batches through one CUDA graph, and the
// autotuner of the search parameters (the reference
// launches one kernel per stage with a device-wide synchronisation after
// each, graph.cu:254-337, and its bloom autotune, auto_tune_bloom.h:71-89,
// is computed but never used).
//
// rte_batcher: the query path (projection -> kd-tree location -> persistent
// search) captured once into a CUDA graph for batches of up to max_nq
// queries.  The kernels read the batch size from device memory, so one
// instantiated graph serves every batch size without re-capture; a batch
// costs one graph launch plus the copies of its queries and results.  With
// learned entries the graph holds the same five kernels as rte_search's
// learned path: the projection (with the head's BF16 input and the zeroed
// keys / counters), the fused head and the subtree location on the main
// branch, the kd-tree location on a parallel branch, then the search.
//
// rte_autotune: measures every candidate (beam, search width, bloom filter
// size, warps per block) on a sample of queries with known neighbours and
// keeps the fastest one that reaches the recall target.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "index_impl.h"
#include "index_kernels.h"
#include "mlp_head.h"
#include "rtentry.h"
#include "search_dispatch.h"

using namespace rte;

struct rte_batcher {
  rte_index* idx = nullptr;
  rte_search_params prm{};
  int64_t cap = 0;
  int k = 0;
  cudaStream_t cap_stream = nullptr, side_stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  DevBuf<float> dq, dproj, ddist;
  DevBuf<int32_t> dhits, dhits2, dids, dn, dorder;
  DevBuf<unsigned int> dwork;
  // learned entries: the head's BF16 input, and [keys (2 words a row) | error
  // flag | work counter], zeroed by the projection
  DevBuf<uint16_t> dxb;
  DevBuf<uint32_t> dzero;
  int* hn = nullptr;  // pinned batch-size slot
  ~rte_batcher() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (cap_stream) cudaStreamDestroy(cap_stream);
    if (side_stream) cudaStreamDestroy(side_stream);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (hn) cudaFreeHost(hn);
  }
};

namespace {

rte_status capture(rte_batcher* b) {
  rte_index* x = b->idx;
  int L, k, NL, NB, wpb, grid, team;
  size_t smem;
  rte_status s = search_plan(x, &b->prm, b->cap, &L, &k, &NL, &NB, &wpb, &grid, &smem, &team, nullptr);
  if (s != RTE_OK) return s;
  b->k = k;
  // A live batch of more queries than the grid's warps hold at their
  // fewest per query is taken in entry-leaf order, as rte_search takes
  // one; smaller batches skip the order (the sort kernel returns at once).
  const int per_query = b->prm.team_warps == 0 ? team_floor(b->prm.precision, L, wpb) : std::max(team, 1);
  const int64_t order_min = (int64_t)grid * wpb / per_query;
  const int32_t* order = b->dorder.p;
  RTE_CUDA(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
  cudaStream_t st = b->cap_stream;
  const bool learned = b->prm.entry_mode == RTE_ENTRY_LEARNED;
  if (learned) {
    RTE_CUDA(mlp_head_prepare(x->mlp.classes));  // no attribute calls inside the capture
    RTE_CUDA(cudaStreamCreateWithFlags(&b->side_stream, cudaStreamNonBlocking));
    RTE_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    RTE_CUDA(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming));
  }
  RTE_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  const float* qp = b->dq.p;
  unsigned int* work = b->dwork.p;
  unsigned long long* keys = nullptr;
  if (learned) {
    // projection + head input + zeroed keys, error flag and work counter
    const int64_t zwords = b->cap * 2 + 2;
    keys = reinterpret_cast<unsigned long long*>(b->dzero.p);
    work = b->dzero.p + b->cap * 2 + 1;
    e = launch_project_bf16_dyn(b->dq.p, b->cap, b->dn.p, x->dim, x->dim, x->d_mean.p, x->d_rot.p,
                                x->search_dim, x->search_dim, b->dproj.p, x->search_dim, b->dxb.p,
                                x->mlp.in_scale, x->mlp.dp, b->dzero.p, zwords, st, x->d_rot_split.p);
    qp = b->dproj.p;
    // the kd-tree leaf on a parallel branch
    if (e == cudaSuccess) e = cudaEventRecord(b->fork, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->side_stream, b->fork, 0);
    if (e == cudaSuccess)
      e = launch_locate_dyn(x->d_wide.p, (int)x->d_wide.n, qp, b->cap, b->dn.p, x->search_dim, b->dhits2.p,
                            b->side_stream, /*top_cache=*/false);
    // ordered by the kd-tree leaf, on the branch beside the model
    if (e == cudaSuccess)
      e = launch_order_by_leaf(b->dhits2.p, 1, b->cap, (int)x->kd.n_leaves, b->dorder.p, b->side_stream,
                               b->dn.p, order_min);
    if (e == cudaSuccess) e = cudaEventRecord(b->join, b->side_stream);
    if (e == cudaSuccess) {
      const Mlp& m = x->mlp;
      MlpHeadArgs h{};
      h.X = b->dxb.p;
      h.W1 = m.W16[0].p;
      h.W2 = m.W16[1].p;
      h.W3 = m.W16[2].p;
      h.b1 = m.b[0].p;
      h.b2 = m.b[1].p;
      h.b3 = m.b[2].p;
      h.M = (int)b->cap;
      h.dp = m.dp;
      h.H = m.hidden;
      h.N = m.classes;
      h.keys = keys;
      h.err = reinterpret_cast<int*>(b->dzero.p + b->cap * 2);
      h.M_dev = b->dn.p;
      e = mlp_head_argmax(h, st);
    }
    if (e == cudaSuccess)
      e = launch_locate_in_subtree_wide(x->d_wide.p, qp, b->cap, x->search_dim, keys, x->mlp.class_wide.p,
                                        x->mlp.class_leaf0.p, x->mlp.real_classes, b->dhits.p, st, b->dn.p);
    // the join also ends the side branch inside the capture
    cudaError_t ej = cudaStreamWaitEvent(st, b->join, 0);
    if (e == cudaSuccess) e = ej;
  } else {
    e = cudaMemsetAsync(b->dwork.p, 0, 2 * sizeof(unsigned int), st);
    if (e == cudaSuccess && x->has_pca) {
      e = launch_project_dyn(b->dq.p, b->cap, b->dn.p, x->dim, x->dim, x->d_mean.p, x->d_rot.p,
                             x->search_dim, x->search_dim, b->dproj.p, x->search_dim, st,
                             x->d_rot_split.p);
      qp = b->dproj.p;
    }
    if (e == cudaSuccess && b->prm.entry_mode == RTE_ENTRY_KDTREE)
      e = launch_locate_dyn(x->d_wide.p, (int)x->d_wide.n, qp, b->cap, b->dn.p, x->search_dim, b->dhits.p, st);
    if (e == cudaSuccess && b->prm.entry_mode == RTE_ENTRY_KDTREE)
      e = launch_order_by_leaf(b->dhits.p, 1, b->cap, (int)x->kd.n_leaves, b->dorder.p, st, b->dn.p,
                               order_min);
  }
  if (e == cudaSuccess) {
    SearchArgs a{};
    a.base = x->il32.p;
    a.base_bf16 = x->il16.p;
    a.base_fp8 = x->il8.p;
    a.fp8_scale = x->scale8.p;
    a.norm16 = x->norm16.p;
    a.queries = qp;
    a.graph = x->graph.p;
    a.leaf_pids = x->has_kdtree ? x->d_pids.p : nullptr;
    a.hits = b->dhits.p;
    a.hits2 = learned ? b->dhits2.p : nullptr;
    a.out_ids = b->dids.p;
    a.out_dists = b->ddist.p;
    a.work = work;
    a.np = (int)x->np;
    a.d = x->search_dim;
    a.qstride = x->search_dim;
    a.nq = (int)b->cap;
    a.nq_dev = b->dn.p;
    a.R = x->degree;
    a.W = b->prm.search_width;
    a.k = k;
    a.max_iter = b->prm.max_iter;
    a.bloom_words = b->prm.bloom_words;
    a.bloom_hashes = b->prm.bloom_hashes;
    a.leaf_cap = x->has_kdtree ? x->kd.cap : 1;
    a.entry_mode = b->prm.entry_mode;
    a.rerank = b->prm.rerank;
    a.n_leaves = x->has_kdtree ? (int)x->kd.n_leaves : 1;
    a.max_hits = 1;
    // automatic teams follow the live batch size, which the graph reads on
    // the device; the grid, planned for the capacity, leaves them room
    a.team = b->prm.team_warps == 0 ? -team_floor(b->prm.precision, L, wpb) : team;
    // bounded waits report into the head's error word (learned entries) or
    // the word after the work counter
    a.err = learned ? reinterpret_cast<int*>(b->dzero.p + b->cap * 2) : reinterpret_cast<int*>(b->dwork.p + 1);
    a.order = b->prm.entry_mode == RTE_ENTRY_RANDOM ? nullptr : order;
    a.order_min = (int)std::min<int64_t>(order_min, INT32_MAX);
    e = launch_search(a, x->C, NL, NB, b->prm.precision, wpb, grid, smem, st);
  }
  cudaError_t e2 = cudaStreamEndCapture(st, &b->graph);
  RTE_CUDA(e);
  RTE_CUDA(e2);
  RTE_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
  return RTE_OK;
}

}  // namespace

extern "C" rte_status rte_batcher_create(rte_index* x, int64_t max_nq,
                                         const rte_search_params* params, rte_batcher** out) {
  clear_error();
  if (!x || !params || !out) return fail(RTE_EINVAL, "NULL argument");
  *out = nullptr;
  if (max_nq <= 0 || max_nq >= INT32_MAX) return fail(RTE_EINVAL, "max_nq must be in [1, 2^31)");
  if (params->entry_mode == RTE_ENTRY_LEARNED) {
    const Mlp& m = x->mlp;
    if (!m.trained) return fail(RTE_ESTATE, "learned entries requested before rte_learned_train");
    MlpHeadArgs h{};
    h.X = h.W1 = h.W2 = h.W3 = m.W16[0].p;  // alignment of the model's own buffers
    h.b1 = h.b2 = h.b3 = m.b[0].p;
    h.keys = reinterpret_cast<unsigned long long*>(1);
    h.M = 1;
    h.dp = m.dp;
    h.H = m.hidden;
    h.N = m.classes;
    if (!x->has_pca || !x->has_kdtree || m.d_in != x->search_dim || !m.class_wide.p ||
        !mlp_head_supported(h))
      return fail(RTE_EINVAL, "the batcher's learned path needs a PCA index, the 8-wide kd-tree classes "
                              "and a head the fused kernel takes");
  }
  if (params->rerank == 2) return fail(RTE_EINVAL, "the batcher does not rerank against the original rows");
  if (params->max_hits > 1) return fail(RTE_EINVAL, "the batcher locates one leaf per query");
  DeviceGuard guard(x->device);
  // the copy the search reads must exist before the graph is captured
  rte_status ps = ensure_precision(x, params->precision);
  if (ps != RTE_OK) return ps;
  auto* b = new rte_batcher();
  b->idx = x;
  b->prm = *params;
  b->cap = max_nq;
  auto bail = [&](rte_status s) {
    delete b;
    return s;
  };
  const int kmax = 256;  // outputs sized for k <= beam <= 256
  if (b->dq.alloc((size_t)max_nq * x->dim) != cudaSuccess ||
      b->dproj.alloc((size_t)max_nq * x->search_dim) != cudaSuccess ||
      b->dhits.alloc(max_nq) != cudaSuccess || b->dids.alloc((size_t)max_nq * kmax) != cudaSuccess ||
      b->ddist.alloc((size_t)max_nq * kmax) != cudaSuccess || b->dn.alloc(1) != cudaSuccess ||
      b->dwork.alloc(2) != cudaSuccess || cudaMallocHost(&b->hn, sizeof(int)) != cudaSuccess)
    return bail(fail(RTE_ENOMEM, "batcher buffers"));
  if (params->entry_mode != RTE_ENTRY_RANDOM && b->dorder.alloc(max_nq) != cudaSuccess)
    return bail(fail(RTE_ENOMEM, "batcher buffers"));
  if (params->entry_mode == RTE_ENTRY_LEARNED &&
      (b->dhits2.alloc(max_nq) != cudaSuccess || b->dxb.alloc((size_t)max_nq * x->mlp.dp) != cudaSuccess ||
       b->dzero.alloc((size_t)max_nq * 2 + 2) != cudaSuccess))
    return bail(fail(RTE_ENOMEM, "batcher buffers"));
  rte_status s = capture(b);
  if (s != RTE_OK) return bail(s);
  *out = b;
  return RTE_OK;
}

extern "C" rte_status rte_batcher_search(rte_batcher* b, const float* queries, int64_t nq,
                                         int32_t* out_ids, float* out_dists, void* stream) {
  clear_error();
  if (!b || (nq && (!queries || !out_ids))) return fail(RTE_EINVAL, "NULL argument");
  if (nq < 0 || nq > b->cap) return fail(RTE_EINVAL, "batch larger than the batcher's max_nq");
  if (nq == 0) return RTE_OK;
  DeviceGuard guard(b->idx->device);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t qb = (size_t)nq * b->idx->dim * 4, ob = (size_t)nq * b->k * 4;
  // the pinned slot is reused by the next call only after this one synced
  RTE_CUDA(cudaStreamSynchronize(st));
  *b->hn = (int)nq;
  RTE_CUDA(cudaMemcpyAsync(b->dn.p, b->hn, sizeof(int), cudaMemcpyHostToDevice, st));
  RTE_CUDA(cudaMemcpyAsync(b->dq.p, queries, qb, cudaMemcpyDefault, st));
  RTE_CUDA(cudaGraphLaunch(b->exec, st));
  RTE_CUDA(cudaMemcpyAsync(out_ids, b->dids.p, ob, cudaMemcpyDefault, st));
  if (out_dists) RTE_CUDA(cudaMemcpyAsync(out_dists, b->ddist.p, ob, cudaMemcpyDefault, st));
  RTE_CUDA(cudaStreamSynchronize(st));
  return RTE_OK;
}

extern "C" int rte_batcher_k(const rte_batcher* b) { return b ? b->k : 0; }

extern "C" void rte_batcher_free(rte_batcher* b) {
  if (!b) return;
  DeviceGuard guard(b->idx->device);
  delete b;
}

// ---------------------------------------------------------------- autotune --
extern "C" rte_status rte_autotune(rte_index* x, const float* queries, int64_t nq,
                                   const int32_t* gt, int gt_k, int k, float target_recall,
                                   rte_search_params* inout, rte_autotune_report* rep) {
  clear_error();
  if (!x || !queries || !gt || !inout || nq <= 0 || k <= 0 || gt_k < k)
    return fail(RTE_EINVAL, "bad autotune arguments (gt_k >= k > 0)");
  DeviceGuard guard(x->device);
  cudaStream_t st = nullptr;
  // queries on the device once
  DevBuf<float> dq;
  RTE_CUDA(dq.alloc((size_t)nq * x->dim));
  RTE_CUDA(cudaMemcpy(dq.p, queries, dq.bytes(), cudaMemcpyDefault));
  std::vector<int32_t> hgt((size_t)nq * gt_k);
  RTE_CUDA(cudaMemcpy(hgt.data(), gt, hgt.size() * 4, cudaMemcpyDefault));
  DevBuf<int32_t> dids;
  RTE_CUDA(dids.alloc((size_t)nq * k));
  std::vector<int32_t> hids((size_t)nq * k);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int beams[] = {16, 32, 64, 128, 256};
  const int widths[] = {1, 2, 4};
  const int blooms[] = {512, 2048, 8192};
  const int wpbs[] = {4, 8};
  rte_search_params best = *inout;
  float best_ms = 1e30f, best_score = 1e30f, best_rec = -1.f, fallback_rec = -1.f;
  rte_search_params fallback = *inout;
  int evaluated = 0;
  for (int L : beams) {
    if (L < k) continue;
    for (int W : widths) {
      if (W * x->degree > 256) continue;
      for (int bw : blooms)
        for (int wpb : wpbs) {
          rte_search_params p = *inout;
          p.beam = L;
          p.k = k;
          p.search_width = W;
          p.bloom_words = bw;
          p.warps_per_block = wpb;
          float ms = 0;
          bool ok = true;
          for (int rep_i = 0; rep_i < 3 && ok; ++rep_i) {  // first run warms up
            cudaEventRecord(e0, st);
            if (rte_search(x, dq.p, nq, &p, dids.p, nullptr, st) != RTE_OK) ok = false;
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            if (rep_i > 0) ms += t / 2;
          }
          if (!ok) {
            clear_error();
            continue;
          }
          ++evaluated;
          RTE_CUDA(cudaMemcpy(hids.data(), dids.p, hids.size() * 4, cudaMemcpyDeviceToHost));
          int64_t hit = 0;
          for (int64_t q = 0; q < nq; ++q)
            for (int i = 0; i < k; ++i) {
              const int32_t g = hgt[q * gt_k + i];
              for (int j = 0; j < k; ++j)
                if (hids[q * k + j] == g) {
                  ++hit;
                  break;
                }
            }
          const float rec = (float)hit / (float)(nq * k);
          // Four warps per block must beat eight by more than 3 %: eight
          // leave a batcher's graph room for teams of eight warps per query
          // on its small batches, which the sample's one batch size does
          // not measure, and the two often time within noise of each other.
          const float score = wpb < 8 ? ms * 1.03f : ms;
          if (rec >= target_recall && score < best_score) {
            best_score = score;
            best_ms = ms;
            best = p;
            best_rec = rec;
          }
          if (rec > fallback_rec) {
            fallback_rec = rec;
            fallback = p;
          }
        }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const bool met = best_rec >= 0;
  *inout = met ? best : fallback;
  if (rep) {
    rep->met_target = met;
    rep->recall = met ? best_rec : fallback_rec;
    rep->ms = met ? best_ms : 0.f;
    rep->qps = met && best_ms > 0 ? (float)(nq / (best_ms / 1000.0)) : 0.f;
    rep->evaluated = evaluated;
  }
  if (evaluated == 0) return fail(RTE_EINVAL, "no candidate configuration could run");
  return RTE_OK;
}
