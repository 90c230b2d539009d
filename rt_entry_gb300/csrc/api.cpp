// api.cpp -- C ABI of rt_entry_gb300 (include/rtentry.h).
//
// The index object owns every device buffer of one index on one GPU.  Query
// calls allocate their per-call buffers from the library's stream-ordered
// memory pool on that device (scratch_pool, on the caller's stream), so
// calls on distinct streams do not share scratch and the pool keeps memory
// mapped across calls and synchronisations.
#include "rtentry.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "host_build.h"
#include "index_impl.h"
#include "index_kernels.h"
#include "io.h"
#include "rerank_full.h"
#include "search_dispatch.h"

using namespace rte;

namespace {
thread_local std::string g_err;
int chunks_of(int d) { return (d + 31) / 32; }
}  // namespace

namespace rte {
rte_status fail(rte_status s, const std::string& msg) {
  g_err = msg;
  return s;
}
void clear_error() { g_err.clear(); }

rte_status ensure_precision(rte_index* x, int precision) {
  if (precision != RTE_PREC_BF16 && precision != RTE_PREC_FP8) return RTE_OK;
  std::lock_guard<std::mutex> lk(x->copy_mu);
  if (precision == RTE_PREC_BF16 ? x->il16.p != nullptr : x->il8.p != nullptr) return RTE_OK;
  DeviceGuard g(x->device);
  const size_t n = 32 * (size_t)x->C * x->np;
  if (precision == RTE_PREC_BF16) {
    DevBuf<uint16_t> il16;
    DevBuf<float> norm16;
    RTE_CUDA(il16.alloc(n));
    RTE_CUDA(norm16.alloc(x->np));
    RTE_CUDA(launch_lowp_copies(x->il32.p, x->np, x->C, il16.p, nullptr, nullptr, 0));
    RTE_CUDA(launch_bf16_norms(il16.p, x->np, x->C, norm16.p, 0));
    RTE_CUDA(cudaStreamSynchronize(0));
    x->il16 = std::move(il16);
    x->norm16 = std::move(norm16);
  } else {
    DevBuf<uint8_t> il8;
    DevBuf<float> scale8;
    RTE_CUDA(il8.alloc(n));
    RTE_CUDA(scale8.alloc(x->np));
    RTE_CUDA(launch_lowp_copies(x->il32.p, x->np, x->C, nullptr, il8.p, scale8.p, 0));
    RTE_CUDA(cudaStreamSynchronize(0));
    x->il8 = std::move(il8);
    x->scale8 = std::move(scale8);
  }
  return RTE_OK;
}
// Host or device memory?  Unregistered host memory reports
// cudaMemoryTypeUnregistered; pinned host memory cudaMemoryTypeHost.
bool is_device_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}
cudaMemPool_t scratch_pool() {
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static cudaMemPool_t pools[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    unsigned long long keep = kScratchKeepBytes;
    if (cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
      cudaGetLastError();
      cudaMemPoolDestroy(p);
      return nullptr;
    }
    pools[dev] = p;
  }
  return pools[dev];
}

// The device address of page-locked host memory that the device can reach
// (every page-locked allocation under unified addressing), else null.
void* mapped_host_ptr(void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}
rte_status noalloc_prepare(int dev);
namespace tc {
void set_wait_limit(long long rounds);  // tc_common.cuh
}  // namespace tc
rte_status learned_leaves(const rte_index* x, const float* d_proj, int64_t nq, int32_t* d_leaf,
                          cudaStream_t st, const uint16_t* xb_in = nullptr,
                          unsigned long long* zkeys = nullptr, int* zerr = nullptr);
}  // namespace rte

namespace {

size_t index_bytes(const rte_index* x) {
  return x->raw.bytes() + x->graph.bytes() + x->d_mean.bytes() + x->d_rot.bytes() + x->d_rot_split.bytes() +
         x->il32.bytes() + x->il16.bytes() + x->il8.bytes() + x->scale8.bytes() + x->norm16.bytes() +
         x->d_nodes.bytes() + x->d_wide.bytes() + x->d_pids.bytes();
}

// (Re)build the lane-interleaved FP32 copy of the search space from a
// row-major device array [np][search_dim]; the BF16 and FP8 copies of the
// previous search space are dropped (they are made again on first use).
rte_status make_search_space(rte_index* x, const float* rm) {
  x->C = chunks_of(x->search_dim);
  const size_t row = 32 * (size_t)x->C;
  {
    std::lock_guard<std::mutex> lk(x->copy_mu);
    x->il16.reset();
    x->norm16.reset();
    x->il8.reset();
    x->scale8.reset();
  }
  RTE_CUDA(x->il32.alloc(row * x->np));
  DevBuf<float> xyz;
  RTE_CUDA(xyz.alloc(3 * x->np));
  if (x->search_dim < 3) RTE_CUDA(cudaMemset(xyz.p, 0, xyz.bytes()));
  RTE_CUDA(launch_interleave(rm, x->np, x->search_dim, x->C, x->il32.p, nullptr, nullptr, nullptr, xyz.p,
                             0));
  x->xyz.resize(3 * x->np);
  RTE_CUDA(cudaMemcpy(x->xyz.data(), xyz.p, xyz.bytes(), cudaMemcpyDeviceToHost));
  RTE_CUDA(cudaDeviceSynchronize());
  // a new search space invalidates the kd-tree built on the old one
  x->has_kdtree = false;
  x->d_nodes.reset();
  x->d_wide.reset();
  x->d_pids.reset();
  return RTE_OK;
}

rte_status validate_graph(const int32_t* g, int64_t np, int degree) {
  const int64_t n = np * degree;
  for (int64_t i = 0; i < n; ++i)
    if (g[i] < 0 || g[i] > np)
      return fail(RTE_EINVAL, "graph id out of range [0, np] at row " + std::to_string(i / degree));
  return RTE_OK;
}

rte_status create_index(const float* base, int64_t np, int dim, const int32_t* graph, int degree,
                        int device, rte_index** out) {
  if (!out) return fail(RTE_EINVAL, "out is NULL");
  *out = nullptr;
  if (!base || !graph) return fail(RTE_EINVAL, "base or graph is NULL");
  if (np <= 0 || np >= INT32_MAX) return fail(RTE_EINVAL, "np must be in [1, 2^31-1)");
  if (dim <= 0 || dim > 32 * 32) return fail(RTE_EINVAL, "dim must be in [1, 1024]");
  if (degree <= 0 || (degree & (degree - 1)))
    return fail(RTE_EINVAL, "graph degree must be a power of two (graph.cu:134)");
  // host-side checks first, so a bad graph is reported without a device
  const bool gdev = is_device_ptr(graph);
  if (!gdev) {
    rte_status s0 = validate_graph(graph, np, degree);
    if (s0 != RTE_OK) return s0;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(RTE_ECUDA, "no CUDA device available");
  }
  if (device < 0 || device >= ndev) return fail(RTE_EINVAL, "device index out of range");
  DeviceGuard g(device);
  // reserve the allocation-free search's scratch on this device now, while
  // the caller is still setting up (see noalloc.cu); a failure here only
  // resurfaces in rte_search_projected_noalloc, which retries the lookup
  if (noalloc_prepare(device) != RTE_OK) {
    cudaGetLastError();
    g_err.clear();
  }
  std::unique_ptr<rte_index> x(new rte_index());
  x->device = device;
  cudaDeviceGetAttribute(&x->num_sms, cudaDevAttrMultiProcessorCount, device);
  x->np = np;
  x->dim = dim;
  x->degree = degree;
  // the library's scratch pool on this device, made here rather than in the
  // first search (a new pool holds no memory); the device's default pool is
  // the host program's and keeps its settings
  scratch_pool();
  std::vector<int32_t> hg;
  const int32_t* gh = graph;
  if (gdev) {
    hg.resize((size_t)np * degree);
    RTE_CUDA(cudaMemcpy(hg.data(), graph, hg.size() * 4, cudaMemcpyDeviceToHost));
    gh = hg.data();
    rte_status s1 = validate_graph(gh, np, degree);
    if (s1 != RTE_OK) return s1;
  }
  rte_status s = RTE_OK;
  RTE_CUDA(x->raw.alloc((size_t)np * dim));
  RTE_CUDA(cudaMemcpy(x->raw.p, base, x->raw.bytes(), cudaMemcpyDefault));
  RTE_CUDA(x->graph.alloc((size_t)np * degree));
  RTE_CUDA(cudaMemcpy(x->graph.p, gh, x->graph.bytes(), cudaMemcpyHostToDevice));
  x->search_dim = dim;
  s = make_search_space(x.get(), x->raw.p);
  if (s != RTE_OK) return s;
  *out = x.release();
  return RTE_OK;
}

int next_pow2(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

struct Plan {
  int L, k, NL, NB, wpb, grid, prec, team;
  size_t smem;
  bool ordered;  // more queries than resident warps: take them in entry-leaf order
};

}  // namespace

namespace rte {
// The fewest warps per query that automatic teams use.  FP32 rows with pools
// of up to 64 slots: their gathers bound the search, and two warps per query
// keep twice the rows in flight, which is faster even when the batch fills
// the GPU a few times over (measured on one GB300 with queries in leaf
// order: 6-11 % at 10k queries, beams 16 to 64).  Above kTeamFloorLoad
// times the resident warps one warp per query wins (9-20 % at 40k queries),
// as it always does at beams 128 and 256 and for BF16 or FP8 rows.
int team_floor(int prec, int L, int wpb) {
  return prec == kPrecF32 && L <= 64 && wpb % 2 == 0 ? 2 : 1;
}
}  // namespace rte

namespace {

rte_status plan_search(const rte_index* x, const rte_search_params* prm, int64_t nq, Plan& pl) {
  if (!prm) return fail(RTE_EINVAL, "params is NULL");
  if (prm->beam <= 0) return fail(RTE_EINVAL, "beam must be > 0");
  pl.L = next_pow2(prm->beam);  // graph.cu:53
  pl.k = prm->k == 0 ? pl.L : prm->k;  // graph.cu:54
  if (pl.k < 0 || pl.k > pl.L) return fail(RTE_EINVAL, "k must be in [1, beam] (topk <= n_candidates)");
  if (pl.L < 16 || pl.L > 256) return fail(RTE_EINVAL, "beam must round to 16..256");
  if (x->degree < 16) return fail(RTE_EINVAL, "graph degree must be >= 16 for the warp kernel");
  if (prm->search_width <= 0) return fail(RTE_EINVAL, "search_width must be >= 1");
  const int B = prm->search_width * x->degree;
  if (B > 256 || (B & (B - 1)))
    return fail(RTE_EINVAL, "search_width * degree must be a power of two <= 256");
  if (prm->max_iter < 0) return fail(RTE_EINVAL, "max_iter must be >= 0");
  if (prm->bloom_words < 32 || prm->bloom_words > 16384 || (prm->bloom_words & (prm->bloom_words - 1)))
    return fail(RTE_EINVAL, "bloom_words must be a power of two in [32, 16384]");
  if (prm->bloom_hashes < 1 || prm->bloom_hashes > 10) return fail(RTE_EINVAL, "bloom_hashes must be in [1, 10]");
  if (prm->precision < 0 || prm->precision > 2) return fail(RTE_EINVAL, "precision must be 0, 1 or 2");
  if (prm->rerank < 0 || prm->rerank > 2) return fail(RTE_EINVAL, "rerank must be 0, 1 or 2");
  if (prm->max_hits < 1 || prm->max_hits > kMaxHits) return fail(RTE_EINVAL, "max_hits must be in [1, 8]");
  if (prm->max_hits > 1 && prm->entry_mode != RTE_ENTRY_KDTREE)
    return fail(RTE_EINVAL, "max_hits > 1 needs kd-tree entries");
  if (prm->team_warps != 0 && prm->team_warps != 1 && prm->team_warps != 2 && prm->team_warps != 4 &&
      prm->team_warps != 8)
    return fail(RTE_EINVAL, "team_warps must be 0, 1, 2, 4 or 8");
  if (prm->entry_mode < RTE_ENTRY_RANDOM || prm->entry_mode > RTE_ENTRY_LEARNED)
    return fail(RTE_EINVAL, "entry_mode must be RTE_ENTRY_RANDOM, _KDTREE or _LEARNED");
  if (prm->entry_mode == RTE_ENTRY_LEARNED && !x->mlp.trained)
    return fail(RTE_ESTATE, "learned entries requested before rte_learned_train");
  if (prm->entry_mode != RTE_ENTRY_RANDOM && !x->has_kdtree)
    return fail(RTE_ESTATE, "kd-tree entries requested before rte_build_kdtree");
  if (!search_chunks_supported(x->C))
    return fail(RTE_EINVAL, "search dimension " + std::to_string(x->search_dim) + " has no kernel instantiation");
  pl.NL = pl.L / 32;  // 0 selects the 16-slot pool
  pl.NB = B / 32;     // 0 selects the 16-slot batch (width 1, degree 16)
  pl.prec = prm->precision;
  // per warp: the bloom filter, the compaction buffers (ids, distances) and
  // the query slot, whose size depends on the kernel that serves this shape
  const int S = std::max(B, pl.L);
  const bool r16 = x->degree == 16;
  const int kc = search_kernel_chunks(x->C, pl.NL, pl.NB, pl.prec, r16);
  const size_t per_warp =
      (size_t)(prm->bloom_words + 2 * S + query_slot_words_for(kc, x->C) + kTeamCtlWords) * 4;
  const size_t smem_cap = 227 * 1024;
  const int team = prm->team_warps;
  if (prm->warps_per_block > 0) {
    pl.wpb = prm->warps_per_block;
    if (pl.wpb > 8) return fail(RTE_EINVAL, "warps_per_block must be <= 8");
    if (team > 1 && pl.wpb % team != 0)
      return fail(RTE_EINVAL, "warps_per_block must be a multiple of team_warps");
  } else {
    pl.wpb = (int)std::min<size_t>(8, (smem_cap - kBlockShareBytes) / per_warp);
    if (team > 1) pl.wpb -= pl.wpb % team;  // whole teams per block
    if (team > 1 && pl.wpb < team)
      return fail(RTE_EINVAL, "the bloom filter leaves room for fewer warps per block than team_warps");
  }
  pl.smem = (size_t)pl.wpb * per_warp + kBlockShareBytes;
  if (pl.wpb < 1 || pl.smem > smem_cap)
    return fail(RTE_EINVAL, "bloom filter too large for the block's shared memory");
  const int occ = occupancy_search(x->C, pl.NL, pl.NB, pl.prec, r16, pl.wpb, pl.smem);
  if (occ <= 0)
    return fail(RTE_EINVAL, "no kernel instantiation for beam " + std::to_string(pl.L) + ", batch " +
                                std::to_string(B) + ", precision " + std::to_string(pl.prec));
  const int64_t resident = (int64_t)x->num_sms * occ * pl.wpb;  // warps
  pl.team = team;
  if (team == 0) {  // automatic: spread a small batch's queries over the idle warps
    pl.team = team_floor(pl.prec, pl.L, pl.wpb);
    if (nq > kTeamFloorLoad * resident) pl.team = 1;
    while (pl.team < 8 && pl.wpb % (2 * pl.team) == 0 && nq * 2 * pl.team <= resident) pl.team *= 2;
  }
  const int64_t need = (nq * pl.team + pl.wpb - 1) / pl.wpb;
  pl.grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)x->num_sms * occ));
  // When the batch does not fit the resident warps at once, the queries
  // running together are the ones close in the work order: taking them by
  // entry leaf makes them neighbours in the base, which share graph rows
  // and vectors in L2 (measured on one GB300 at 10k config-2 queries: plain
  // FP32 beam 32 -13 %, learned BF16 beam 16 -8 %).
  pl.ordered = need > (int64_t)x->num_sms * occ && prm->entry_mode != RTE_ENTRY_RANDOM;
  return RTE_OK;
}

// A second stream per host thread and device, with a fork and a join event,
// created on first use and kept for the life of the thread.
struct SideStream {
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};

cudaError_t side_stream(int dev, SideStream** out) {
  thread_local SideStream sides[64];
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  SideStream& sd = sides[dev];
  if (!sd.s) {
    cudaError_t e = cudaStreamCreateWithFlags(&sd.s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sd.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sd.join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      cudaGetLastError();
      sd = SideStream{};
      return e;
    }
  }
  *out = &sd;
  return cudaSuccess;
}

// Projection + locate + search on device buffers.
// host_err (pinned), when given, receives in stream order the call's error
// word: a bounded device wait ran out when it is non-zero.
rte_status run_query_path(rte_index* x, const float* d_queries, bool already_projected,
                          const int32_t* d_hits_in, int64_t nq, const rte_search_params* prm,
                          int32_t* d_ids, float* d_dists, long long* d_counters, cudaStream_t st,
                          int* host_err = nullptr) {
  Plan pl;
  rte_status s = plan_search(x, prm, nq, pl);
  if (s != RTE_OK) return s;
  if (nq == 0) return RTE_OK;
  // rerank 2: the search returns its whole pool, which is reranked against
  // the original rows and queries (graph_helper.cu:146-213)
  const bool full_rerank = prm->rerank == 2;
  if (full_rerank && already_projected)
    return fail(RTE_EINVAL, "rerank 2 needs the original queries: use rte_search");
  if (full_rerank && !x->raw.p) return fail(RTE_ESTATE, "rerank 2 needs the raw base, which was released");
  s = ensure_precision(x, prm->precision);
  if (s != RTE_OK) return s;
  const float* qp = d_queries;
  AsyncBuf proj, hitsb, work, xb, zs;
  // learned entries without caller hits: the projection also writes the
  // model's BF16 input rows
  const bool head_input = prm->entry_mode == RTE_ENTRY_LEARNED && !d_hits_in && x->mlp.trained &&
                          x->mlp.d_in == x->search_dim;
  const bool projecting = !already_projected && x->has_pca;
  // Scratch the projection zeroes on its way: the argmax keys (learned head),
  // the head's error flag and the search's work counter, in that order.
  const int64_t n_keys = projecting && head_input ? nq : 0;
  unsigned long long* zkeys = nullptr;
  int* zerr = nullptr;
  unsigned int* zwork = nullptr;
  if (projecting) {
    RTE_CUDA(zs.alloc((size_t)n_keys * 8 + 8, st));
    zkeys = n_keys ? zs.as<unsigned long long>() : nullptr;
    zerr = reinterpret_cast<int*>(zs.as<char>() + n_keys * 8);
    zwork = reinterpret_cast<unsigned int*>(zs.as<char>() + n_keys * 8 + 4);
  }
  const int32_t* hits2 = nullptr;
  AsyncBuf hits2b, ordb;
  if (pl.ordered) RTE_CUDA(ordb.alloc((size_t)nq * 4, st));
  const int32_t* order = nullptr;
  SideStream* sd = nullptr;
  // Any return after a fork waits for the side stream first, so that the
  // buffers it writes are not freed (in stream order on st) under it.  The
  // guard is declared after those buffers and so runs before their frees.
  struct JoinGuard {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    ~JoinGuard() {
      if (ev) cudaStreamWaitEvent(st, ev, 0);
    }
  } join_guard;
  join_guard.st = st;
  if (projecting) {
    RTE_CUDA(proj.alloc((size_t)nq * x->search_dim * 4, st));
    const int64_t zwords = n_keys * 2 + 2;
    if (head_input) {
      RTE_CUDA(xb.alloc((size_t)nq * x->mlp.dp * 2, st));
      RTE_CUDA(launch_project_bf16(d_queries, nq, x->dim, x->dim, x->d_mean.p, x->d_rot.p,
                                   x->search_dim, x->search_dim, proj.as<float>(), x->search_dim,
                                   xb.p, x->mlp.in_scale, x->mlp.dp, st, zs.as<uint32_t>(), zwords,
                                   x->d_rot_split.p));
    } else {
      RTE_CUDA(launch_project(d_queries, nq, x->dim, x->dim, x->d_mean.p, x->d_rot.p,
                              x->search_dim, x->search_dim, proj.as<float>(), x->search_dim, st,
                              zs.as<uint32_t>(), zwords, x->d_rot_split.p));
    }
    qp = proj.as<float>();
  }
  const int32_t* hits = d_hits_in;
  if (prm->entry_mode == RTE_ENTRY_KDTREE && !hits) {
    RTE_CUDA(hitsb.alloc((size_t)nq * prm->max_hits * 4, st));
    if (prm->max_hits > 1)
      RTE_CUDA(launch_locate_multi(x->d_wide.p, (int)x->d_wide.n, qp, nq, x->search_dim, prm->max_hits,
                                   hitsb.as<int32_t>(), st));
    else
      RTE_CUDA(launch_locate(x->d_wide.p, (int)x->d_wide.n, qp, nq, x->search_dim, hitsb.as<int32_t>(), st));
    hits = hitsb.as<int32_t>();
  }
  if (pl.ordered && prm->entry_mode == RTE_ENTRY_KDTREE) {  // by the first leaf of each query
    RTE_CUDA(launch_order_by_leaf(hits, prm->max_hits, nq, (int)x->kd.n_leaves, ordb.as<int32_t>(), st));
    order = ordb.as<int32_t>();
  }
  if (prm->entry_mode == RTE_ENTRY_LEARNED) {
    // proposed leaf (MLP) first, kd-tree leaf second; when the model runs
    // here, the kd-tree location runs beside it on this thread's side
    // stream, without shared memory so that its blocks fit beside the GEMMs
    RTE_CUDA(hits2b.alloc((size_t)nq * 4, st));
    hits2 = hits2b.as<int32_t>();
    const bool fork = !hits && side_stream(x->device, &sd) == cudaSuccess;
    if (fork) {
      RTE_CUDA(cudaEventRecord(sd->fork, st));
      RTE_CUDA(cudaStreamWaitEvent(sd->s, sd->fork, 0));
    }
    cudaError_t le = launch_locate(x->d_wide.p, (int)x->d_wide.n, qp, nq, x->search_dim,
                                   hits2b.as<int32_t>(), fork ? sd->s : st, /*top_cache=*/!fork);
    // ordered by the kd-tree leaf, which is ready before the model's: off
    // the model's path when the side stream runs it
    if (le == cudaSuccess && pl.ordered) {
      le = launch_order_by_leaf(hits2, 1, nq, (int)x->kd.n_leaves, ordb.as<int32_t>(), fork ? sd->s : st);
      order = ordb.as<int32_t>();
    }
    if (fork) {
      RTE_CUDA(cudaEventRecord(sd->join, sd->s));
      join_guard.ev = sd->join;
    }
    RTE_CUDA(le);
    rte_status ls = RTE_OK;
    if (!hits) {
      RTE_CUDA(hitsb.alloc((size_t)nq * 4, st));
      ls = learned_leaves(x, qp, nq, hitsb.as<int32_t>(), st, xb.p ? xb.as<uint16_t>() : nullptr,
                          zkeys, zkeys ? zerr : nullptr);
      hits = hitsb.as<int32_t>();
    }
    // join before anything returns: the buffers are freed in stream order on st
    if (fork) {
      join_guard.ev = nullptr;
      RTE_CUDA(cudaStreamWaitEvent(st, sd->join, 0));
    }
    if (ls != RTE_OK) return ls;
  }
  if (!zwork) {  // the work counter and an error word
    RTE_CUDA(work.alloc(8, st));
    RTE_CUDA(cudaMemsetAsync(work.p, 0, 8, st));
  }
  int* err_word = zwork ? zerr : work.as<int>() + 1;
  AsyncBuf poolb;
  if (full_rerank) RTE_CUDA(poolb.alloc((size_t)nq * pl.L * 4, st));
  SearchArgs a{};
  a.base = x->il32.p;
  a.base_bf16 = x->il16.p;
  a.base_fp8 = x->il8.p;
  a.fp8_scale = x->scale8.p;
  a.norm16 = x->norm16.p;
  a.queries = qp;
  a.graph = x->graph.p;
  a.leaf_pids = x->has_kdtree ? x->d_pids.p : nullptr;
  a.hits = hits;
  a.hits2 = hits2;
  a.out_ids = full_rerank ? poolb.as<int32_t>() : d_ids;
  a.out_dists = full_rerank ? nullptr : d_dists;
  a.counters = d_counters;
  a.work = zwork ? zwork : work.as<unsigned int>();
  a.np = (int)x->np;
  a.d = x->search_dim;
  a.qstride = x->search_dim;
  a.nq = (int)nq;
  a.R = x->degree;
  a.W = prm->search_width;
  a.k = full_rerank ? pl.L : pl.k;
  a.max_iter = prm->max_iter;
  a.bloom_words = prm->bloom_words;
  a.bloom_hashes = prm->bloom_hashes;
  a.leaf_cap = x->has_kdtree ? x->kd.cap : 1;
  a.entry_mode = prm->entry_mode;
  a.rerank = full_rerank ? 0 : prm->rerank;
  a.n_leaves = x->has_kdtree ? (int)x->kd.n_leaves : 1;
  a.max_hits = prm->max_hits;
  a.team = pl.team;
  a.err = err_word;
  a.order = order;
  RTE_CUDA(launch_search(a, x->C, pl.NL, pl.NB, pl.prec, pl.wpb, pl.grid, pl.smem, st));
  if (host_err) RTE_CUDA(cudaMemcpyAsync(host_err, err_word, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (full_rerank)
    RTE_CUDA(launch_rerank_full(x->raw.p, x->np, x->dim, d_queries, x->dim, poolb.as<int32_t>(),
                                (int)nq, pl.L, pl.k, d_ids, d_dists, x->num_sms, st));
  return RTE_OK;
}

}  // namespace

namespace rte {
// Launch plan of a search, for entry points defined in other files.
rte_status search_plan(const rte_index* x, const rte_search_params* prm, int64_t nq, int* L, int* k,
                       int* NL, int* NB, int* wpb, int* grid, size_t* smem, int* team, bool* ordered) {
  Plan pl;
  rte_status s = plan_search(x, prm, nq, pl);
  if (s != RTE_OK) return s;
  *team = pl.team;
  if (ordered) *ordered = pl.ordered;
  *L = pl.L;
  *k = pl.k;
  *NL = pl.NL;
  *NB = pl.NB;
  *wpb = pl.wpb;
  *grid = pl.grid;
  *smem = pl.smem;
  return RTE_OK;
}

rte_status plain_top1(rte_index* x, const float* d_proj, int64_t n, int beam, int32_t* d_ids,
                      cudaStream_t st) {
  rte_search_params p;
  rte_default_params(&p);
  p.beam = beam;
  p.k = 1;
  p.entry_mode = RTE_ENTRY_KDTREE;
  return run_query_path(x, d_proj, true, nullptr, n, &p, d_ids, nullptr, nullptr, st);
}
}  // namespace rte

extern "C" {

void rte_default_params(rte_search_params* p) {
  if (!p) return;
  p->k = 10;
  p->beam = 64;
  p->search_width = 1;
  p->max_iter = 100;
  p->bloom_words = 512;
  p->bloom_hashes = 3;
  p->precision = RTE_PREC_FP32;
  p->rerank = 0;
  p->entry_mode = RTE_ENTRY_KDTREE;
  p->warps_per_block = 0;
  p->max_hits = 1;
  p->team_warps = 0;
}

const char* rte_last_error(void) { return g_err.c_str(); }

void rte_set_wait_limit(long long rounds) { rte::tc::set_wait_limit(rounds); }

rte_status rte_scratch_pool_usage(int device, uint64_t* used_now, uint64_t* used_high, int reset_high) {
  g_err.clear();
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return fail(RTE_ECUDA, "cudaGetDeviceCount failed");
  }
  if (device < 0 || device >= n) return fail(RTE_EINVAL, "device index out of range");
  DeviceGuard g(device);
  cudaMemPool_t pool = scratch_pool();
  if (!pool) return fail(RTE_ECUDA, "the scratch memory pool could not be created");
  unsigned long long v = 0;
  if (used_now) {
    RTE_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &v));
    *used_now = v;
  }
  if (used_high) {
    RTE_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &v));
    *used_high = v;
  }
  if (reset_high) {
    unsigned long long zero = 0;
    RTE_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero));
  }
  return RTE_OK;
}

rte_status rte_index_from_host(const float* base, int64_t np, int dim, const int32_t* graph,
                               int degree, int device, rte_index** out) {
  g_err.clear();
  return create_index(base, np, dim, graph, degree, device, out);
}

rte_status rte_index_load(const char* base_path, const char* graph_path, int device,
                          rte_index** out) {
  g_err.clear();
  if (!base_path || !graph_path || !out) return fail(RTE_EINVAL, "NULL argument");
  std::vector<float> base;
  int64_t np = 0;
  int dim = 0;
  std::string err;
  if (!io::read_vectors(base_path, base, np, dim, err)) return fail(RTE_EIO, err);
  std::vector<int32_t> graph;
  int degree = 0;
  if (!io::read_graph(graph_path, np, graph, degree, err)) return fail(RTE_EIO, err);
  return create_index(base.data(), np, dim, graph.data(), degree, device, out);
}

rte_status rte_index_prepare(rte_index* x, unsigned copies) {
  g_err.clear();
  if (!x) return fail(RTE_EINVAL, "index is NULL");
  if (copies & ~(unsigned)(RTE_COPY_BF16 | RTE_COPY_FP8 | RTE_COPY_RAW))
    return fail(RTE_EINVAL, "unknown copy flags");
  if ((copies & RTE_COPY_RAW) && !x->raw.p)
    return fail(RTE_ESTATE, "the raw base was released and cannot be made again");
  rte_status s = RTE_OK;
  if (copies & RTE_COPY_BF16) s = ensure_precision(x, RTE_PREC_BF16);
  if (s == RTE_OK && (copies & RTE_COPY_FP8)) s = ensure_precision(x, RTE_PREC_FP8);
  return s;
}

rte_status rte_index_release(rte_index* x, unsigned copies) {
  g_err.clear();
  if (!x) return fail(RTE_EINVAL, "index is NULL");
  if (copies & ~(unsigned)(RTE_COPY_BF16 | RTE_COPY_FP8 | RTE_COPY_RAW))
    return fail(RTE_EINVAL, "unknown copy flags");
  DeviceGuard g(x->device);
  RTE_CUDA(cudaDeviceSynchronize());  // no search may still read what is freed
  std::lock_guard<std::mutex> lk(x->copy_mu);
  if (copies & RTE_COPY_BF16) {
    x->il16.reset();
    x->norm16.reset();
  }
  if (copies & RTE_COPY_FP8) {
    x->il8.reset();
    x->scale8.reset();
  }
  if (copies & RTE_COPY_RAW) x->raw.reset();
  return RTE_OK;
}

void rte_index_free(rte_index* idx) {
  if (!idx) return;
  DeviceGuard g(idx->device);
  delete idx;
}

}  // extern "C"

namespace {
// Installs a PCA (mean [dim], rotation [dim x dim]) and makes the first
// keep_dims components the search space: projected here, or taken from
// `projected` (host, [np][ld], ld >= keep_dims) when the caller has it.
rte_status install_pca(rte_index* x, const float* mean, const float* rotation, int keep_dims,
                       const float* projected, int ld) {
  if (keep_dims == 0) keep_dims = x->dim;
  if (keep_dims < 3 || keep_dims > x->dim) return fail(RTE_EINVAL, "keep_dims must be in [3, dim]");
  if (!projected && !x->raw.p) return fail(RTE_ESTATE, "the raw base was released (rte_index_release)");
  DeviceGuard g(x->device);
  const int d = x->dim;
  x->mean32.assign(mean, mean + d);
  x->rot32.assign(rotation, rotation + (size_t)d * d);
  if (x->mean64.size() != (size_t)d) {
    x->mean64.assign(mean, mean + d);
    x->vec64.assign(rotation, rotation + (size_t)d * d);
    x->eig64.assign(d, 0.0);
  }
  x->search_dim = keep_dims;
  std::vector<float> rk((size_t)d * keep_dims);
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < keep_dims; ++j) rk[(size_t)i * keep_dims + j] = x->rot32[(size_t)i * d + j];
  RTE_CUDA(x->d_mean.alloc(d));
  RTE_CUDA(cudaMemcpy(x->d_mean.p, x->mean32.data(), d * 4, cudaMemcpyHostToDevice));
  RTE_CUDA(x->d_rot.alloc(rk.size()));
  RTE_CUDA(cudaMemcpy(x->d_rot.p, rk.data(), rk.size() * 4, cudaMemcpyHostToDevice));
  RTE_CUDA(x->d_rot_split.alloc(rotation_split_floats(d, keep_dims)));
  RTE_CUDA(launch_split_rotation(x->d_rot.p, d, keep_dims, keep_dims, x->d_rot_split.p, 0));
  DevBuf<float> proj;
  RTE_CUDA(proj.alloc((size_t)x->np * keep_dims));
  if (projected) {
    RTE_CUDA(cudaMemcpy2D(proj.p, (size_t)keep_dims * 4, projected, (size_t)ld * 4, (size_t)keep_dims * 4,
                          (size_t)x->np, cudaMemcpyHostToDevice));
  } else {
    RTE_CUDA(launch_project(x->raw.p, x->np, d, d, x->d_mean.p, x->d_rot.p, keep_dims, keep_dims,
                            proj.p, keep_dims, 0, nullptr, 0, x->d_rot_split.p));
  }
  x->has_pca = true;
  return make_search_space(x, proj.p);
}
}  // namespace

extern "C" {

rte_status rte_set_pca(rte_index* x, const float* mean, const float* rotation, int keep_dims) {
  g_err.clear();
  if (!x || !mean || !rotation) return fail(RTE_EINVAL, "NULL argument");
  return install_pca(x, mean, rotation, keep_dims, nullptr, 0);
}

rte_status rte_index_load_reference(const char* dir, const char* base_path, const char* graph_path,
                                    int keep_dims, int leaf_size, float expand_ratio, int device,
                                    rte_index** out) {
  g_err.clear();
  if (!dir || !base_path || !graph_path || !out) return fail(RTE_EINVAL, "NULL argument");
  *out = nullptr;
  std::string err;
  std::vector<float> base;
  int64_t np = 0;
  int dim = 0;
  if (!io::read_vectors(base_path, base, np, dim, err)) return fail(RTE_EIO, err);
  std::vector<int32_t> graph;
  int degree = 0;
  if (!io::read_graph(graph_path, np, graph, degree, err)) return fail(RTE_EIO, err);
  rte_index* raw = nullptr;
  rte_status s = create_index(base.data(), np, dim, graph.data(), degree, device, &raw);
  if (s != RTE_OK) return s;
  std::unique_ptr<rte_index, void (*)(rte_index*)> x(raw, rte_index_free);
  base.clear();
  base.shrink_to_fit();
  const std::string D(dir);
  const bool has_o = io::file_exists(D + "/O.fbin"), has_m = io::file_exists(D + "/mean.fbin");
  if (has_o != has_m) return fail(RTE_EIO, D + ": O.fbin and mean.fbin must both be present or both absent");
  if (has_o) {
    std::vector<float> mean, rot;
    int64_t n1 = 0;
    int d1 = 0;
    if (!io::read_matrix_fbin(D + "/mean.fbin", mean, n1, d1, err)) return fail(RTE_EIO, err);
    if (n1 != 1 || d1 != dim) return fail(RTE_EIO, D + "/mean.fbin is not [1 x " + std::to_string(dim) + "]");
    if (!io::read_matrix_fbin(D + "/O.fbin", rot, n1, d1, err)) return fail(RTE_EIO, err);
    if (n1 != dim || d1 != dim)
      return fail(RTE_EIO, D + "/O.fbin is not [" + std::to_string(dim) + " x " + std::to_string(dim) + "]");
    const int keep = keep_dims == 0 ? dim : keep_dims;
    if (keep < 3 || keep > dim) return fail(RTE_EINVAL, "keep_dims must be in [3, dim]");
    std::vector<float> pb;
    int pd = 0;
    if (io::file_exists(D + "/pca_base.fbin")) {
      int64_t pn = 0;
      if (!io::read_matrix_fbin(D + "/pca_base.fbin", pb, pn, pd, err)) return fail(RTE_EIO, err);
      if (pn != np || pd < keep)
        return fail(RTE_EIO, D + "/pca_base.fbin is [" + std::to_string(pn) + " x " + std::to_string(pd) +
                                 "], the base needs [" + std::to_string(np) + " x >= " + std::to_string(keep) + "]");
    }
    s = install_pca(x.get(), mean.data(), rot.data(), keep, pb.empty() ? nullptr : pb.data(), pd);
    if (s != RTE_OK) return s;
  } else if (keep_dims != 0) {
    return fail(RTE_EIO, D + ": keep_dims given but no O.fbin / mean.fbin");
  }
  if (leaf_size > 0) {
    s = rte_build_kdtree(x.get(), leaf_size, expand_ratio);
    if (s != RTE_OK) return s;
    const std::string af = D + "/" + std::to_string(leaf_size) + "_0.aabbs";
    if (io::file_exists(af)) {
      int64_t nl = 0;
      int ls = 0;
      std::vector<float> boxes;
      std::vector<int32_t> pids;
      if (!io::read_aabbs(af, nl, ls, boxes, pids, err)) return fail(RTE_EIO, err);
      if (nl != x->kd.n_leaves || ls != x->kd.cap || boxes != x->kd.tight || pids != x->kd.pids)
        return fail(RTE_EIO, af + " does not hold the kd-tree of this search space (" + std::to_string(nl) +
                                 " leaves in the file, " + std::to_string(x->kd.n_leaves) + " built)");
    }
  }
  *out = x.release();
  return RTE_OK;
}

rte_status rte_read_vectors(const char* path, float* out, int64_t capacity, int64_t* n, int* d) {
  g_err.clear();
  if (!path || !n || !d) return fail(RTE_EINVAL, "NULL argument");
  std::vector<float> data;
  int64_t n0 = 0;
  int d0 = 0;
  std::string err;
  if (!io::read_vectors(path, data, n0, d0, err)) return fail(RTE_EIO, err);
  *n = n0;
  *d = d0;
  if (!out) return RTE_OK;
  if (capacity < (int64_t)data.size())
    return fail(RTE_EINVAL, "capacity " + std::to_string(capacity) + " < n*d = " + std::to_string(data.size()));
  std::copy(data.begin(), data.end(), out);
  return RTE_OK;
}

rte_status rte_build_pca(rte_index* x, int keep_dims) {
  g_err.clear();
  if (!x) return fail(RTE_EINVAL, "index is NULL");
  if (!x->raw.p) return fail(RTE_ESTATE, "the raw base was released (rte_index_release)");
  if (x->np < 2) return fail(RTE_EINVAL, "PCA needs at least two vectors");
  DeviceGuard g(x->device);
  const int d = x->dim;
  const int nblocks = (int)std::min<int64_t>(1024, x->np);
  const int nchunks = (int)std::max<int64_t>(1, std::min<int64_t>(64, x->np / 4096));
  DevBuf<double> part, mean, cov;
  RTE_CUDA(part.alloc(std::max<size_t>((size_t)nblocks * d, (size_t)nchunks * d * d)));
  RTE_CUDA(mean.alloc(d));
  RTE_CUDA(cov.alloc((size_t)d * d));
  RTE_CUDA(launch_mean(x->raw.p, x->np, d, part.p, nblocks, mean.p, 0));
  RTE_CUDA(launch_cov(x->raw.p, x->np, d, mean.p, part.p, nchunks, cov.p, 0));
  std::vector<double> hmean(d), hcov((size_t)d * d);
  RTE_CUDA(cudaMemcpy(hmean.data(), mean.p, d * 8, cudaMemcpyDeviceToHost));
  RTE_CUDA(cudaMemcpy(hcov.data(), cov.p, hcov.size() * 8, cudaMemcpyDeviceToHost));
  std::vector<double> w(d), v((size_t)d * d);
  std::string err;
  if (!sym_eig(hcov.data(), d, w.data(), v.data(), err)) return fail(RTE_EINVAL, err);
  x->mean64 = hmean;
  x->eig64 = w;
  x->vec64 = v;
  std::vector<float> m32(d), r32((size_t)d * d);
  for (int i = 0; i < d; ++i) m32[i] = (float)hmean[i];
  for (size_t i = 0; i < r32.size(); ++i) r32[i] = (float)v[i];
  return rte_set_pca(x, m32.data(), r32.data(), keep_dims);
}

rte_status rte_build_kdtree(rte_index* x, int leaf_size, float expand_ratio) {
  g_err.clear();
  if (!x) return fail(RTE_EINVAL, "index is NULL");
  if (leaf_size <= 0) return fail(RTE_EINVAL, "leaf_size must be > 0");
  if (!(expand_ratio >= 0.f) || !std::isfinite(expand_ratio))
    return fail(RTE_EINVAL, "expand_ratio must be finite and >= 0");
  DeviceGuard g(x->device);
  KdTree t;
  std::string err;
  if (!kd_build(x->xyz.data(), x->np, leaf_size, t, err)) return fail(RTE_EINVAL, err);
  if (t.depth + 2 > kBvhMaxDepth) return fail(RTE_EINVAL, "kd-tree deeper than the locate stack");
  kd_expand(t, expand_ratio);
  RTE_CUDA(x->d_nodes.alloc(t.nodes.size()));
  RTE_CUDA(cudaMemcpy(x->d_nodes.p, t.nodes.data(), x->d_nodes.bytes(), cudaMemcpyHostToDevice));
  std::vector<WideNode> wide;
  kd_wide(t, wide, &x->wide_of);
  RTE_CUDA(x->d_wide.alloc(wide.size()));
  RTE_CUDA(cudaMemcpy(x->d_wide.p, wide.data(), x->d_wide.bytes(), cudaMemcpyHostToDevice));
  RTE_CUDA(x->d_pids.alloc(t.pids.size()));
  RTE_CUDA(cudaMemcpy(x->d_pids.p, t.pids.data(), x->d_pids.bytes(), cudaMemcpyHostToDevice));
  x->kd = std::move(t);
  x->expand_ratio = expand_ratio;
  x->has_kdtree = true;
  return RTE_OK;
}

rte_status rte_project(rte_index* x, const float* queries, int64_t nq, float* out, void* stream) {
  g_err.clear();
  if (!x || (!queries && nq) || (!out && nq)) return fail(RTE_EINVAL, "NULL argument");
  if (nq < 0) return fail(RTE_EINVAL, "nq < 0");
  if (nq == 0) return RTE_OK;
  DeviceGuard g(x->device);
  cudaStream_t st = (cudaStream_t)stream;
  const bool qd = is_device_ptr(queries), od = is_device_ptr(out);
  AsyncBuf qb, ob;
  const float* dq = queries;
  if (!qd) {
    RTE_CUDA(qb.alloc((size_t)nq * x->dim * 4, st));
    RTE_CUDA(cudaMemcpyAsync(qb.p, queries, (size_t)nq * x->dim * 4, cudaMemcpyHostToDevice, st));
    dq = qb.as<float>();
  }
  float* dout = out;
  if (!od) {
    RTE_CUDA(ob.alloc((size_t)nq * x->search_dim * 4, st));
    dout = ob.as<float>();
  }
  if (x->has_pca) {
    RTE_CUDA(launch_project(dq, nq, x->dim, x->dim, x->d_mean.p, x->d_rot.p, x->search_dim,
                            x->search_dim, dout, x->search_dim, st, nullptr, 0, x->d_rot_split.p));
  } else {
    RTE_CUDA(cudaMemcpyAsync(dout, dq, (size_t)nq * x->dim * 4, cudaMemcpyDeviceToDevice, st));
  }
  if (!od) {
    RTE_CUDA(cudaMemcpyAsync(out, dout, (size_t)nq * x->search_dim * 4, cudaMemcpyDeviceToHost, st));
    RTE_CUDA(cudaStreamSynchronize(st));
  }
  return RTE_OK;
}

rte_status rte_locate(rte_index* x, const float* projected, int64_t nq, int32_t* out_leaf,
                      void* stream) {
  g_err.clear();
  if (!x || (!projected && nq) || (!out_leaf && nq)) return fail(RTE_EINVAL, "NULL argument");
  if (nq < 0) return fail(RTE_EINVAL, "nq < 0");
  if (!x->has_kdtree) return fail(RTE_ESTATE, "rte_locate before rte_build_kdtree");
  if (nq == 0) return RTE_OK;
  DeviceGuard g(x->device);
  cudaStream_t st = (cudaStream_t)stream;
  const bool pd = is_device_ptr(projected), od = is_device_ptr(out_leaf);
  AsyncBuf pb, ob;
  const float* dp = projected;
  if (!pd) {
    RTE_CUDA(pb.alloc((size_t)nq * x->search_dim * 4, st));
    RTE_CUDA(cudaMemcpyAsync(pb.p, projected, (size_t)nq * x->search_dim * 4, cudaMemcpyHostToDevice, st));
    dp = pb.as<float>();
  }
  int32_t* dout = out_leaf;
  if (!od) {
    RTE_CUDA(ob.alloc((size_t)nq * 4, st));
    dout = ob.as<int32_t>();
  }
  RTE_CUDA(launch_locate(x->d_wide.p, (int)x->d_wide.n, dp, nq, x->search_dim, dout, st));
  if (!od) {
    RTE_CUDA(cudaMemcpyAsync(out_leaf, dout, (size_t)nq * 4, cudaMemcpyDeviceToHost, st));
    RTE_CUDA(cudaStreamSynchronize(st));
  }
  return RTE_OK;
}

rte_status rte_locate_multi(rte_index* x, const float* projected, int64_t nq, int max_hits,
                            int32_t* out_leaves, void* stream) {
  g_err.clear();
  if (!x || (!projected && nq) || (!out_leaves && nq)) return fail(RTE_EINVAL, "NULL argument");
  if (nq < 0) return fail(RTE_EINVAL, "nq < 0");
  if (max_hits < 1 || max_hits > kMaxHits) return fail(RTE_EINVAL, "max_hits must be in [1, 8]");
  if (!x->has_kdtree) return fail(RTE_ESTATE, "rte_locate_multi before rte_build_kdtree");
  if (nq == 0) return RTE_OK;
  DeviceGuard g(x->device);
  cudaStream_t st = (cudaStream_t)stream;
  const bool pd = is_device_ptr(projected), od = is_device_ptr(out_leaves);
  AsyncBuf pb, ob;
  const float* dp = projected;
  if (!pd) {
    RTE_CUDA(pb.alloc((size_t)nq * x->search_dim * 4, st));
    RTE_CUDA(cudaMemcpyAsync(pb.p, projected, (size_t)nq * x->search_dim * 4, cudaMemcpyHostToDevice, st));
    dp = pb.as<float>();
  }
  int32_t* dout = out_leaves;
  if (!od) {
    RTE_CUDA(ob.alloc((size_t)nq * max_hits * 4, st));
    dout = ob.as<int32_t>();
  }
  RTE_CUDA(launch_locate_multi(x->d_wide.p, (int)x->d_wide.n, dp, nq, x->search_dim, max_hits, dout, st));
  if (!od) {
    RTE_CUDA(cudaMemcpyAsync(out_leaves, dout, (size_t)nq * max_hits * 4, cudaMemcpyDeviceToHost, st));
    RTE_CUDA(cudaStreamSynchronize(st));
  }
  return RTE_OK;
}

static rte_status search_common(rte_index* x, const float* q, bool projected, const int32_t* hits,
                                int64_t nq, const rte_search_params* prm, int32_t* out_ids,
                                float* out_dists, int64_t* counters, void* stream) {
  if (!x || !prm) return fail(RTE_EINVAL, "NULL argument");
  if (nq < 0) return fail(RTE_EINVAL, "nq < 0");
  if (nq > 0 && (!q || (!out_ids && !counters))) return fail(RTE_EINVAL, "NULL argument");
  if (nq >= INT32_MAX) return fail(RTE_EINVAL, "nq must be < 2^31");
  DeviceGuard g(x->device);
  cudaStream_t st = (cudaStream_t)stream;
  Plan pl;
  rte_status s = plan_search(x, prm, nq, pl);
  if (s != RTE_OK) return s;
  if (nq == 0) return RTE_OK;
  const int qdim = projected ? x->search_dim : x->dim;
  const size_t qbytes = (size_t)nq * qdim * 4;
  const size_t obytes = (size_t)nq * pl.k * 4;
  bool host_io = false;
  AsyncBuf qb, hb, ib, db, cb;
  const float* dq = q;
  if (!is_device_ptr(q)) {
    host_io = true;
    RTE_CUDA(qb.alloc(qbytes, st));
    RTE_CUDA(cudaMemcpyAsync(qb.p, q, qbytes, cudaMemcpyHostToDevice, st));
    dq = qb.as<float>();
  }
  const int32_t* dh = hits;
  if (hits && !is_device_ptr(hits)) {
    host_io = true;
    // [nq x max_hits] for kd-tree entries from several leaves, else [nq]
    const size_t hbytes = (size_t)nq * 4 *
                          (prm->entry_mode == RTE_ENTRY_KDTREE && prm->max_hits > 1 ? prm->max_hits : 1);
    RTE_CUDA(hb.alloc(hbytes, st));
    RTE_CUDA(cudaMemcpyAsync(hb.p, hits, hbytes, cudaMemcpyHostToDevice, st));
    dh = hb.as<int32_t>();
  }
  // Page-locked host outputs are written by the kernels themselves, through
  // their device address: each query's results cross the host link as the
  // query finishes, overlapped with the rest of the search, instead of in
  // copies after it.  Pageable host outputs go through device buffers.
  int32_t* di = out_ids;
  const bool ids_host = out_ids && !is_device_ptr(out_ids);
  int32_t* ids_mapped = ids_host ? static_cast<int32_t*>(mapped_host_ptr(out_ids)) : nullptr;
  if (ids_mapped) {
    di = ids_mapped;
  } else if (!out_ids || ids_host) {
    RTE_CUDA(ib.alloc(obytes, st));
    di = ib.as<int32_t>();
  }
  float* dd = out_dists;
  const bool dists_host = out_dists && !is_device_ptr(out_dists);
  float* dists_mapped = dists_host ? static_cast<float*>(mapped_host_ptr(out_dists)) : nullptr;
  if (dists_mapped) {
    dd = dists_mapped;
  } else if (dists_host) {
    RTE_CUDA(db.alloc(obytes, st));
    dd = db.as<float>();
  }
  long long* dc = nullptr;
  const bool cnt_host = counters && !is_device_ptr(counters);
  if (counters) {
    if (cnt_host) {
      RTE_CUDA(cb.alloc((size_t)nq * 32, st));
      dc = cb.as<long long>();
    } else {
      dc = reinterpret_cast<long long*>(counters);
    }
  }
  const bool syncs = host_io || ids_host || dists_host || cnt_host;
  // the error word comes back to pinned memory, so its copy stays in stream order
  thread_local int* herr = nullptr;
  if (syncs && !herr) RTE_CUDA(cudaMallocHost(&herr, sizeof(int)));
  if (syncs) *herr = 0;
  s = run_query_path(x, dq, projected, dh, nq, prm, di, dd, dc, st, syncs ? herr : nullptr);
  if (s != RTE_OK) return s;
  if (ids_host && !ids_mapped) RTE_CUDA(cudaMemcpyAsync(out_ids, di, obytes, cudaMemcpyDeviceToHost, st));
  if (dists_host && !dists_mapped)
    RTE_CUDA(cudaMemcpyAsync(out_dists, dd, obytes, cudaMemcpyDeviceToHost, st));
  if (cnt_host) RTE_CUDA(cudaMemcpyAsync(counters, dc, (size_t)nq * 32, cudaMemcpyDeviceToHost, st));
  if (syncs) {
    RTE_CUDA(cudaStreamSynchronize(st));
    if (*herr) return fail(RTE_ETIMEOUT, "a bounded wait in the query path ran out (code " + std::to_string(*herr) + ")");
  }
  return RTE_OK;
}

rte_status rte_search(rte_index* x, const float* queries, int64_t nq,
                      const rte_search_params* params, int32_t* out_ids, float* out_dists,
                      void* stream) {
  g_err.clear();
  return search_common(x, queries, false, nullptr, nq, params, out_ids, out_dists, nullptr, stream);
}

rte_status rte_search_projected(rte_index* x, const float* projected, const int32_t* hits,
                                int64_t nq, const rte_search_params* params, int32_t* out_ids,
                                float* out_dists, void* stream) {
  g_err.clear();
  return search_common(x, projected, true, hits, nq, params, out_ids, out_dists, nullptr, stream);
}

rte_status rte_search_counters(rte_index* x, const float* projected, const int32_t* hits,
                               int64_t nq, const rte_search_params* params, int64_t* counters,
                               void* stream) {
  g_err.clear();
  if (!counters && nq) return fail(RTE_EINVAL, "counters is NULL");
  return search_common(x, projected, true, hits, nq, params, nullptr, nullptr, counters, stream);
}

rte_status rte_kdtree_build_host(const float* xyz, int64_t n, int leaf_size, float expand_ratio,
                                 int64_t max_leaves, float* tight, float* expanded, int32_t* pids,
                                 int64_t* n_leaves) {
  g_err.clear();
  if (!xyz || !n_leaves) return fail(RTE_EINVAL, "NULL argument");
  if (n <= 0 || n >= INT32_MAX || leaf_size <= 0) return fail(RTE_EINVAL, "bad sizes");
  KdTree t;
  std::string err;
  if (!kd_build(xyz, n, leaf_size, t, err)) return fail(RTE_EINVAL, err);
  kd_expand(t, expand_ratio);
  *n_leaves = t.n_leaves;
  if (t.n_leaves > max_leaves) return fail(RTE_EINVAL, "max_leaves too small");
  if (tight) std::copy(t.tight.begin(), t.tight.end(), tight);
  if (expanded) std::copy(t.expanded.begin(), t.expanded.end(), expanded);
  if (pids) std::copy(t.pids.begin(), t.pids.end(), pids);
  return RTE_OK;
}

rte_status rte_sym_eig_host(const double* a, int n, double* w, double* v) {
  g_err.clear();
  if (!a || !w || !v || n <= 0) return fail(RTE_EINVAL, "bad argument");
  std::string err;
  if (!sym_eig(a, n, w, v, err)) return fail(RTE_EINVAL, err);
  return RTE_OK;
}

rte_status rte_index_get_info(const rte_index* x, rte_index_info* info) {
  g_err.clear();
  if (!x || !info) return fail(RTE_EINVAL, "NULL argument");
  info->np = x->np;
  info->dim = x->dim;
  info->search_dim = x->search_dim;
  info->degree = x->degree;
  info->has_pca = x->has_pca;
  info->has_kdtree = x->has_kdtree;
  info->n_leaves = x->has_kdtree ? x->kd.n_leaves : 0;
  info->leaf_size = x->has_kdtree ? x->kd.cap : 0;
  info->expand_ratio = x->expand_ratio;
  info->has_bf16 = x->il16.p != nullptr;
  info->has_fp8 = x->il8.p != nullptr;
  info->device = x->device;
  info->device_bytes = (int64_t)index_bytes(x);
  return RTE_OK;
}

rte_status rte_get_pca(const rte_index* x, float* mean, float* rotation, double* eigvals) {
  g_err.clear();
  if (!x) return fail(RTE_EINVAL, "index is NULL");
  if (!x->has_pca) return fail(RTE_ESTATE, "no PCA built");
  if (mean) std::copy(x->mean32.begin(), x->mean32.end(), mean);
  if (rotation) std::copy(x->rot32.begin(), x->rot32.end(), rotation);
  if (eigvals) std::copy(x->eig64.begin(), x->eig64.end(), eigvals);
  return RTE_OK;
}

rte_status rte_get_search_base(const rte_index* x, float* out) {
  g_err.clear();
  if (!x || !out) return fail(RTE_EINVAL, "NULL argument");
  DeviceGuard g(x->device);
  DevBuf<float> tmp;
  RTE_CUDA(tmp.alloc((size_t)x->np * x->search_dim));
  RTE_CUDA(launch_deinterleave(x->il32.p, x->np, x->search_dim, x->C, tmp.p, 0));
  RTE_CUDA(cudaMemcpy(out, tmp.p, tmp.bytes(), cudaMemcpyDefault));
  return RTE_OK;
}

rte_status rte_get_search_base_lowp(const rte_index* x, int precision, float* out) {
  g_err.clear();
  if (!x || !out) return fail(RTE_EINVAL, "NULL argument");
  if (precision != RTE_PREC_BF16 && precision != RTE_PREC_FP8)
    return fail(RTE_EINVAL, "precision must be RTE_PREC_BF16 or RTE_PREC_FP8");
  rte_status s = ensure_precision(const_cast<rte_index*>(x), precision);
  if (s != RTE_OK) return s;
  DeviceGuard g(x->device);
  DevBuf<float> tmp;
  RTE_CUDA(tmp.alloc((size_t)x->np * x->search_dim));
  const void* src = precision == RTE_PREC_BF16 ? (const void*)x->il16.p : (const void*)x->il8.p;
  RTE_CUDA(launch_dequant(src, x->scale8.p, precision, x->np, x->search_dim, x->C, tmp.p, 0));
  RTE_CUDA(cudaMemcpy(out, tmp.p, tmp.bytes(), cudaMemcpyDefault));
  return RTE_OK;
}

rte_status rte_get_kdtree(const rte_index* x, float* tight, float* expanded, int32_t* pids) {
  g_err.clear();
  if (!x) return fail(RTE_EINVAL, "index is NULL");
  if (!x->has_kdtree) return fail(RTE_ESTATE, "no kd-tree built");
  if (tight) std::copy(x->kd.tight.begin(), x->kd.tight.end(), tight);
  if (expanded) std::copy(x->kd.expanded.begin(), x->kd.expanded.end(), expanded);
  if (pids) std::copy(x->kd.pids.begin(), x->kd.pids.end(), pids);
  return RTE_OK;
}

rte_status rte_index_save(const rte_index* x, const char* dir) {
  g_err.clear();
  if (!x || !dir) return fail(RTE_EINVAL, "NULL argument");
  if (!x->raw.p) return fail(RTE_ESTATE, "the raw base was released (rte_index_release)");
  DeviceGuard g(x->device);
  std::string err;
  std::vector<float> raw((size_t)x->np * x->dim);
  RTE_CUDA(cudaMemcpy(raw.data(), x->raw.p, raw.size() * 4, cudaMemcpyDeviceToHost));
  std::vector<int32_t> graph((size_t)x->np * x->degree);
  RTE_CUDA(cudaMemcpy(graph.data(), x->graph.p, graph.size() * 4, cudaMemcpyDeviceToHost));
  io::IndexFiles f;
  f.np = x->np;
  f.dim = x->dim;
  f.degree = x->degree;
  f.base = &raw;
  f.graph = &graph;
  std::vector<float> pca_base;
  if (x->has_pca) {
    f.has_pca = true;
    f.search_dim = x->search_dim;
    f.mean = &x->mean32;
    f.rot = &x->rot32;
    pca_base.resize((size_t)x->np * x->search_dim);
    DevBuf<float> tmp;
    RTE_CUDA(tmp.alloc(pca_base.size()));
    RTE_CUDA(launch_deinterleave(x->il32.p, x->np, x->search_dim, x->C, tmp.p, 0));
    RTE_CUDA(cudaMemcpy(pca_base.data(), tmp.p, tmp.bytes(), cudaMemcpyDeviceToHost));
    f.pca_base = &pca_base;
  }
  if (x->has_kdtree) {
    f.has_kdtree = true;
    f.leaf_size = x->kd.cap;
    f.expand_ratio = x->expand_ratio;
    f.n_leaves = x->kd.n_leaves;
    f.tight = &x->kd.tight;
    f.pids = &x->kd.pids;
  }
  if (!io::save_index(dir, f, err)) return fail(RTE_EIO, err);
  return RTE_OK;
}

rte_status rte_index_load_dir(const char* dir, int device, rte_index** out) {
  g_err.clear();
  if (!dir || !out) return fail(RTE_EINVAL, "NULL argument");
  io::LoadedIndex L;
  std::string err;
  if (!io::load_index(dir, L, err)) return fail(RTE_EIO, err);
  rte_status s = create_index(L.base.data(), L.np, L.dim, L.graph.data(), L.degree, device, out);
  if (s != RTE_OK) return s;
  if (L.has_pca) {
    s = rte_set_pca(*out, L.mean.data(), L.rot.data(), L.search_dim);
    if (s != RTE_OK) {
      rte_index_free(*out);
      *out = nullptr;
      return s;
    }
  }
  if (L.has_kdtree) {
    s = rte_build_kdtree(*out, L.leaf_size, L.expand_ratio);
    if (s != RTE_OK) {
      rte_index_free(*out);
      *out = nullptr;
      return s;
    }
  }
  return RTE_OK;
}

}  // extern "C"
