// ref_launch.cpp -- ORACLE side: runs the reference's own GraphSearchKernel
// (compiled from graph_search.cuh by oracle/ref/Makefile into
// oracle/_ref/graph_search_d<D>.cubin) on a GPU through the CUDA driver API,
// exactly as Graph::GraphSearch launches it (graph.cu:318-324):
//   <<<nq, 64, ((search_width << offset_shift) + n_candidates) * 8>>>
// with the kd-tree entry table aabb_entries [n_leaves x n_candidates]
// (entry.cu:60-69) and hits [nq].  Used to make and check fixtures and to
// time the reference kernel beside this library's search on the same
// inputs; never part of the product.
//
// A session (ref_open) uploads the base rows and the graph once; each
// ref_search uploads that call's queries, entry table and hits.
//
// Safe-launch conditions (checked below): search_width == 1 (the reference's
// first selection mask is all ones, so a wider first expansion can reach an
// empty slot whose id np indexes one row past the graph); degree <= 64;
// n_candidates a power of two in [16, 256]; every hit and entry in range.
//
// scrub != 0: one launch per query (grid 1, pointers offset to that query),
// each preceded by scrub_smem (oracle/ref/scrub.cu) on every SM, so that the
// reference's never-cleared shared bloom filter (graph_search.cuh:88) starts
// empty.  Only meaningful for kd-tree entries: random entries seed from
// blockIdx.x (graph_search.cuh:64), which a per-query launch changes.
//
// reps > 0 (batched launches only): after one untimed launch, reps launches
// are timed with driver events, each preceded by a 256 MB memset that
// evicts the inputs from L2; ms[r] receives launch r's device time.
#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace {

std::string g_msg;

#define DRV(call)                                               \
  do {                                                          \
    CUresult r_ = (call);                                       \
    if (r_ != CUDA_SUCCESS) {                                   \
      const char* s_ = nullptr;                                 \
      cuGetErrorString(r_, &s_);                                \
      g_msg = std::string(#call) + ": " + (s_ ? s_ : "?");      \
      return -2;                                                \
    }                                                           \
  } while (0)

struct Mem {
  CUdeviceptr p = 0;
  ~Mem() {
    if (p) cuMemFree(p);
  }
};

constexpr size_t kFlushBytes = 256u << 20;

struct Session {
  CUdevice dev = 0;
  CUcontext ctx = nullptr;
  CUmodule mod = nullptr, smod = nullptr;
  CUfunction fn = nullptr, sf = nullptr;
  Mem data, graph, flush;
  int np = 0, dim = 0, degree = 0, offset_shift = 0;
  int max_smem = 0, nsm = 0;
  std::string dir;
};

// Pushes the session's context for the lifetime of the object.
struct CtxScope {
  CUcontext c;
  explicit CtxScope(CUcontext ctx) : c(ctx) { cuCtxPushCurrent(c); }
  ~CtxScope() {
    CUcontext o;
    cuCtxPopCurrent(&o);
  }
};

int load(Session* s, const char* cubin_path) {
  if (cuModuleLoad(&s->mod, cubin_path) != CUDA_SUCCESS) {
    g_msg = std::string("cannot load ") + cubin_path;
    s->mod = nullptr;
    return -2;
  }
  unsigned int nf = 0;
  DRV(cuModuleGetFunctionCount(&nf, s->mod));
  std::vector<CUfunction> fs(nf);
  DRV(cuModuleEnumerateFunctions(fs.data(), nf, s->mod));
  for (CUfunction f : fs) {
    const char* name = nullptr;
    if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name &&
        std::string(name).find("GraphSearchKernel") != std::string::npos)
      s->fn = f;
  }
  if (!s->fn) {
    g_msg = "GraphSearchKernel not found in cubin";
    return -2;
  }
  std::string dir(cubin_path);
  s->dir = dir.substr(0, dir.find_last_of('/') + 1);
  return 0;
}

int load_scrub(Session* s) {
  if (s->sf) return 0;
  if (cuModuleLoad(&s->smod, (s->dir + "scrub.cubin").c_str()) != CUDA_SUCCESS) {
    g_msg = "cannot load scrub.cubin";
    s->smod = nullptr;
    return -2;
  }
  DRV(cuModuleGetFunction(&s->sf, s->smod, "scrub_smem"));
  DRV(cuDeviceGetAttribute(&s->max_smem, CU_DEVICE_ATTRIBUTE_MAX_SHARED_MEMORY_PER_BLOCK_OPTIN, s->dev));
  DRV(cuDeviceGetAttribute(&s->nsm, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, s->dev));
  DRV(cuFuncSetAttribute(s->sf, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, s->max_smem));
  DRV(cuFuncSetAttribute(s->sf, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, 100));
  DRV(cuFuncSetAttribute(s->fn, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, 100));
  return 0;
}

void destroy(Session* s) {
  if (!s) return;
  if (s->ctx) {
    CtxScope scope(s->ctx);
    if (s->data.p) cuMemFree(s->data.p);
    if (s->graph.p) cuMemFree(s->graph.p);
    if (s->flush.p) cuMemFree(s->flush.p);
    s->data.p = s->graph.p = s->flush.p = 0;
    if (s->smod) cuModuleUnload(s->smod);
    if (s->mod) cuModuleUnload(s->mod);
  }
  if (s->ctx) cuDevicePrimaryCtxRelease(s->dev);
  delete s;
}

int open_impl(Session* s, const char* cubin_path, const float* data, int np, int dim,
              const int* graph, int degree) {
  DRV(cuInit(0));
  DRV(cuDeviceGet(&s->dev, 0));
  DRV(cuDevicePrimaryCtxRetain(&s->ctx, s->dev));
  CtxScope scope(s->ctx);
  int rc = load(s, cubin_path);
  if (rc) return rc;
  s->np = np;
  s->dim = dim;
  s->degree = degree;
  while ((1 << s->offset_shift) < degree) ++s->offset_shift;
  DRV(cuMemAlloc(&s->data.p, (size_t)np * dim * 4));
  DRV(cuMemAlloc(&s->graph.p, (size_t)np * degree * 4));
  DRV(cuMemcpyHtoD(s->data.p, data, (size_t)np * dim * 4));
  DRV(cuMemcpyHtoD(s->graph.p, graph, (size_t)np * degree * 4));
  return 0;
}

int search_impl(Session* s, const float* queries, int nq, const int* entries, int n_leaves,
                int n_candidates, const int* hits, int topk, int search_width, int max_iter,
                int algo, int scrub, int reps, float* ms, int* out) {
  CtxScope scope(s->ctx);
  Mem d_q, d_res, d_entries, d_hits;
  DRV(cuMemAlloc(&d_q.p, (size_t)nq * s->dim * 4));
  DRV(cuMemAlloc(&d_res.p, (size_t)nq * topk * 4));
  DRV(cuMemAlloc(&d_entries.p, (size_t)n_leaves * n_candidates * 4));
  DRV(cuMemAlloc(&d_hits.p, (size_t)nq * 4));
  DRV(cuMemcpyHtoD(d_q.p, queries, (size_t)nq * s->dim * 4));
  DRV(cuMemcpyHtoD(d_entries.p, entries, (size_t)n_leaves * n_candidates * 4));
  DRV(cuMemcpyHtoD(d_hits.p, hits, (size_t)nq * 4));
  CUdeviceptr d_cand = 0;
  int np = s->np, offset_shift = s->offset_shift;
  const unsigned smem = (unsigned)(((search_width << offset_shift) + n_candidates) * 8);
  if (!scrub) {
    void* args[] = {&s->data.p, &d_q.p,     &d_res.p,      &s->graph.p,   &d_cand,
                    &np,        &offset_shift, &n_candidates, &topk,         &search_width,
                    &d_entries.p, &d_hits.p, &max_iter,    &algo};
    DRV(cuLaunchKernel(s->fn, nq, 1, 1, 64, 1, 1, smem, nullptr, args, nullptr));
    DRV(cuCtxSynchronize());
    if (reps > 0) {
      if (!s->flush.p) DRV(cuMemAlloc(&s->flush.p, kFlushBytes));
      std::vector<CUevent> ev(2 * (size_t)reps, nullptr);
      for (auto& e : ev) DRV(cuEventCreate(&e, CU_EVENT_DEFAULT));
      int erc = 0;
      for (int r = 0; r < reps && !erc; ++r) {
        if (cuMemsetD8Async(s->flush.p, (unsigned char)r, kFlushBytes, nullptr) != CUDA_SUCCESS ||
            cuEventRecord(ev[2 * r], nullptr) != CUDA_SUCCESS ||
            cuLaunchKernel(s->fn, nq, 1, 1, 64, 1, 1, smem, nullptr, args, nullptr) != CUDA_SUCCESS ||
            cuEventRecord(ev[2 * r + 1], nullptr) != CUDA_SUCCESS)
          erc = -2;
      }
      if (!erc && cuCtxSynchronize() != CUDA_SUCCESS) erc = -2;
      for (int r = 0; r < reps && !erc; ++r)
        if (cuEventElapsedTime(&ms[r], ev[2 * r], ev[2 * r + 1]) != CUDA_SUCCESS) erc = -2;
      for (auto& e : ev)
        if (e) cuEventDestroy(e);
      if (erc) {
        g_msg = "timed launches failed";
        return erc;
      }
    }
  } else {
    int rc = load_scrub(s);
    if (rc) return rc;
    unsigned nwords = (unsigned)(s->max_smem / 4);
    void* sargs[] = {&nwords};
    for (int q = 0; q < nq; ++q) {
      DRV(cuLaunchKernel(s->sf, s->nsm, 1, 1, 1024, 1, 1, (unsigned)s->max_smem, nullptr, sargs, nullptr));
      CUdeviceptr dq = d_q.p + (CUdeviceptr)q * s->dim * 4, dr = d_res.p + (CUdeviceptr)q * topk * 4,
                  dh = d_hits.p + (CUdeviceptr)q * 4;
      void* qargs[] = {&s->data.p, &dq,          &dr,           &s->graph.p, &d_cand,
                       &np,        &offset_shift, &n_candidates, &topk,       &search_width,
                       &d_entries.p, &dh,        &max_iter,     &algo};
      DRV(cuLaunchKernel(s->fn, 1, 1, 1, 64, 1, 1, smem, nullptr, qargs, nullptr));
    }
    DRV(cuCtxSynchronize());
  }
  DRV(cuMemcpyDtoH(out, d_res.p, (size_t)nq * topk * 4));
  return 0;
}

}  // namespace

extern "C" const char* ref_last_error() { return g_msg.c_str(); }

// Returns 0 and *out = a session, -1 on rejected arguments, -2 on a driver error.
extern "C" int ref_open(const char* cubin_path, const float* data, int np, int dim, const int* graph,
                        int degree, void** out) {
  if (!out || !cubin_path || !data || !graph || np <= 0 || dim <= 0 || degree > 64 || degree <= 0 ||
      (degree & (degree - 1))) {
    g_msg = "rejected arguments (degree must be a power of two <= 64)";
    return -1;
  }
  for (int64_t i = 0; i < (int64_t)np * degree; ++i)
    if (graph[i] < 0 || graph[i] > np) {
      g_msg = "graph id out of range";
      return -1;
    }
  Session* s = new Session();
  const int rc = open_impl(s, cubin_path, data, np, dim, graph, degree);
  if (rc) {
    destroy(s);
    return rc;
  }
  *out = s;
  return 0;
}

extern "C" void ref_close(void* s) { destroy(static_cast<Session*>(s)); }

// One search of nq queries; out [nq x topk] = the reference's d_results.
extern "C" int ref_search(void* sess, const float* queries, int nq, const int* entries, int n_leaves,
                          int n_candidates, const int* hits, int topk, int search_width, int max_iter,
                          int algo, int scrub, int reps, float* ms, int* out) {
  Session* s = static_cast<Session*>(sess);
  if (!s || !queries || !entries || !hits || !out || search_width != 1 || topk <= 0 ||
      topk > n_candidates || n_candidates < 16 || n_candidates > 256 ||
      (n_candidates & (n_candidates - 1)) || nq <= 0 || n_leaves <= 0 || reps < 0 ||
      (reps > 0 && (!ms || scrub))) {
    g_msg = "rejected arguments (search_width must be 1, n_candidates a power of two in [16, 256])";
    return -1;
  }
  for (int q = 0; q < nq; ++q)
    if (hits[q] < 0 || hits[q] >= n_leaves) {
      g_msg = "hit out of range";
      return -1;
    }
  for (int64_t i = 0; i < (int64_t)n_leaves * n_candidates; ++i)
    if (entries[i] < 0 || entries[i] > s->np) {
      g_msg = "entry id out of range";
      return -1;
    }
  return search_impl(s, queries, nq, entries, n_leaves, n_candidates, hits, topk, search_width,
                     max_iter, algo, scrub, reps, ms, out);
}

// One-shot form: open, search, close (used by the fixture recipe).
extern "C" int ref_graph_search(const char* cubin_path, const float* data, int np, int dim,
                                const float* queries, int nq, const int* graph, int degree,
                                const int* entries, int n_leaves, int n_candidates,
                                const int* hits, int topk, int search_width, int max_iter, int algo,
                                int scrub, int* out) {
  void* s = nullptr;
  int rc = ref_open(cubin_path, data, np, dim, graph, degree, &s);
  if (rc) return rc;
  rc = ref_search(s, queries, nq, entries, n_leaves, n_candidates, hits, topk, search_width, max_iter,
                  algo, scrub, 0, nullptr, out);
  ref_close(s);
  return rc;
}
