// noalloc.cu -- a search entry point that allocates no memory.
//
// Some callers cannot let a library allocate device memory once they are
// running: a serving process that reserves all of its GPU memory at start-up
// and treats any later cudaMalloc as a failure (an allocation can stall on
// a device-wide synchronisation or fail under memory pressure in the middle
// of a request), or a host framework whose own allocator owns the device and
// forbids third-party libraries to allocate behind its back.  For them
// rte_search_projected_noalloc runs the entry-point location and the beam
// search with every buffer supplied: the caller passes the inputs and the
// outputs, and the only scratch the kernels need -- the leaf of each query,
// the order in which the persistent search takes them and its work-queue
// counter -- lives in the file-scope array below.  The array is reserved on a device when an index
// is first created there (noalloc_prepare; with lazy module loading the
// address lookup is what loads it) and kept until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "index_impl.h"
#include "index_kernels.h"
#include "search_dispatch.h"

using namespace rte;

namespace {

// Largest batch one call accepts (RTE_NOALLOC_MAX_QUERIES in rtentry.h).
constexpr int kMaxQueries = 65536;

// [0, 256): the search's work counter (first 4 bytes) and its error word
// (next 4: a bounded wait ran out); then the leaf and the place in the
// search order of each query.
struct NoallocScratch {
  unsigned int counter[64];
  int32_t hits[kMaxQueries];
  int32_t order[kMaxQueries];
};

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Host code cannot use the symbol as a device address: it is a host-side
// stand-in.  The device address comes from cudaGetSymbolAddress, looked up
// once per device with that device current, and cached.
constexpr int kMaxDevices = 64;
std::mutex g_lock;
NoallocScratch* g_addr[kMaxDevices] = {};

rte_status scratch_for_device(int dev, NoallocScratch** out) {
  if (dev < 0 || dev >= kMaxDevices) return fail(RTE_EINVAL, "device index out of range");
  std::lock_guard<std::mutex> lk(g_lock);
  if (!g_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(RTE_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_addr[dev] = static_cast<NoallocScratch*>(p);
  }
  *out = g_addr[dev];
  return RTE_OK;
}

}  // namespace

namespace rte {
// Looks up the scratch array's device address for `dev` (the current
// device).  Index creation calls this, so that the array is allocated -- the
// lookup loads the module holding it -- when the index is built, not in the
// middle of the first allocation-free search.
rte_status noalloc_prepare(int dev) {
  NoallocScratch* scr = nullptr;
  return scratch_for_device(dev, &scr);
}
}  // namespace rte

extern "C" rte_status rte_search_projected_noalloc(rte_index* x, const float* projected,
                                                   const int32_t* hits, int64_t nq,
                                                   const rte_search_params* params,
                                                   int32_t* out_ids, float* out_dists,
                                                   void* stream) {
  clear_error();
  if (!x || !params) return fail(RTE_EINVAL, "NULL argument");
  if (nq < 0) return fail(RTE_EINVAL, "nq < 0");
  if (nq > kMaxQueries)
    return fail(RTE_EINVAL, "rte_search_projected_noalloc takes at most " +
                                std::to_string(kMaxQueries) + " queries per call");
  if (params->entry_mode != RTE_ENTRY_RANDOM && params->entry_mode != RTE_ENTRY_KDTREE)
    return fail(RTE_EINVAL, "rte_search_projected_noalloc supports random and kd-tree entries only");
  DeviceGuard guard(x->device);
  // parameters are validated before an empty batch returns, as
  // rte_search_projected does
  int L, k, NL, NB, wpb, grid, team;
  size_t smem;
  bool ordered = false;
  rte_status s = search_plan(x, params, nq, &L, &k, &NL, &NB, &wpb, &grid, &smem, &team, &ordered);
  if (s != RTE_OK) return s;
  if (params->rerank == 2)
    return fail(RTE_EINVAL, "rerank 2 needs the original queries: use rte_search");
  if (params->max_hits > 1) return fail(RTE_EINVAL, "max_hits > 1 needs rte_search");
  // making a reduced-precision copy would allocate
  if ((params->precision == RTE_PREC_BF16 && !x->il16.p) || (params->precision == RTE_PREC_FP8 && !x->il8.p))
    return fail(RTE_ESTATE, "the index has no copy in this precision: call rte_index_prepare first");
  if (nq == 0) return RTE_OK;
  if (!projected || !out_ids) return fail(RTE_EINVAL, "NULL argument");
  // inputs and outputs must already be device memory: copying host data
  // would need staging buffers
  if (!is_device_ptr(projected) || !is_device_ptr(out_ids) ||
      (out_dists && !is_device_ptr(out_dists)) || (hits && !is_device_ptr(hits)))
    return fail(RTE_EINVAL, "rte_search_projected_noalloc takes device pointers only");
  cudaStream_t st = (cudaStream_t)stream;
  NoallocScratch* scr = nullptr;
  s = scratch_for_device(x->device, &scr);
  if (s != RTE_OK) return s;
  const int32_t* h = hits;
  if (params->entry_mode == RTE_ENTRY_KDTREE && !h) {
    RTE_CUDA(launch_locate(x->d_wide.p, (int)x->d_wide.n, projected, nq, x->search_dim, scr->hits, st));
    h = scr->hits;
  }
  const int32_t* order = nullptr;
  if (ordered && params->entry_mode == RTE_ENTRY_KDTREE) {
    RTE_CUDA(launch_order_by_leaf(h, 1, nq, (int)x->kd.n_leaves, scr->order, st));
    order = scr->order;
  }
  // the array keeps the previous call's contents: the counter and the error
  // word must restart at 0
  RTE_CUDA(cudaMemsetAsync(scr->counter, 0, 2 * sizeof(unsigned int), st));
  SearchArgs a{};
  a.base = x->il32.p;
  a.base_bf16 = x->il16.p;
  a.base_fp8 = x->il8.p;
  a.fp8_scale = x->scale8.p;
  a.norm16 = x->norm16.p;
  a.queries = projected;
  a.graph = x->graph.p;
  a.leaf_pids = x->has_kdtree ? x->d_pids.p : nullptr;
  a.hits = h;
  a.hits2 = nullptr;
  a.out_ids = out_ids;
  a.out_dists = out_dists;
  a.counters = nullptr;
  a.work = scr->counter;
  a.err = reinterpret_cast<int*>(scr->counter + 1);
  a.np = (int)x->np;
  a.d = x->search_dim;
  a.qstride = x->search_dim;
  a.nq = (int)nq;
  a.R = x->degree;
  a.W = params->search_width;
  a.k = k;
  a.max_iter = params->max_iter;
  a.bloom_words = params->bloom_words;
  a.bloom_hashes = params->bloom_hashes;
  a.leaf_cap = x->has_kdtree ? x->kd.cap : 1;
  a.entry_mode = params->entry_mode;
  a.rerank = params->rerank;
  a.n_leaves = x->has_kdtree ? (int)x->kd.n_leaves : 1;
  a.max_hits = 1;
  a.team = team;
  a.order = order;
  RTE_CUDA(launch_search(a, x->C, NL, NB, params->precision, wpb, grid, smem, st));
  return RTE_OK;
}
