// ref_launch.cpp -- ORACLE side: runs the reference's own GraphSearchKernel
// (compiled from graph_search.cuh by oracle/ref/Makefile into
// oracle/_ref/graph_search_d<D>.cubin) on a GPU through the CUDA driver API,
// exactly as Graph::GraphSearch launches it (graph.cu:318-324):
//   <<<nq, 64, ((search_width << offset_shift) + n_candidates) * 8>>>
// with the kd-tree entry table aabb_entries [n_leaves x n_candidates]
// (entry.cu:60-69) and hits [nq].  Only used to make and check fixtures.
//
// Safe-launch conditions (checked below): search_width == 1 (the reference's
// first selection mask is all ones, so a wider first expansion can reach an
// empty slot whose id np indexes one row past the graph); degree <= 64.
//
// scrub != 0: one launch per query (grid 1, pointers offset to that query),
// each preceded by scrub_smem (oracle/ref/scrub.cu) on every SM, so that the
// reference's never-cleared shared bloom filter (graph_search.cuh:88) starts
// empty.  Only meaningful for kd-tree entries: random entries seed from
// blockIdx.x (graph_search.cuh:64), which a per-query launch changes.
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

}  // namespace

extern "C" const char* ref_last_error() { return g_msg.c_str(); }

// Returns 0 on success, -1 on rejected arguments, -2 on a driver error.
extern "C" int ref_graph_search(const char* cubin_path, const float* data, int np, int dim,
                                const float* queries, int nq, const int* graph, int degree,
                                const int* entries, int n_leaves, int n_candidates,
                                const int* hits, int topk, int search_width, int max_iter, int algo,
                                int scrub, int* out) {
  if (search_width != 1 || degree > 64 || degree <= 0 || (degree & (degree - 1)) || topk <= 0 ||
      topk > n_candidates || nq <= 0 || np <= 0 || n_leaves <= 0) {
    g_msg = "rejected arguments (search_width must be 1, degree a power of two <= 64)";
    return -1;
  }
  for (int q = 0; q < nq; ++q)
    if (hits[q] < 0 || hits[q] >= n_leaves) {
      g_msg = "hit out of range";
      return -1;
    }
  DRV(cuInit(0));
  CUdevice dev;
  DRV(cuDeviceGet(&dev, 0));
  CUcontext ctx;
  DRV(cuDevicePrimaryCtxRetain(&ctx, dev));
  DRV(cuCtxPushCurrent(ctx));
  int rc = 0;
  {
    CUmodule mod;
    if (cuModuleLoad(&mod, cubin_path) != CUDA_SUCCESS) {
      g_msg = std::string("cannot load ") + cubin_path;
      cuCtxPopCurrent(&ctx);
      return -2;
    }
    unsigned int nf = 0;
    DRV(cuModuleGetFunctionCount(&nf, mod));
    std::vector<CUfunction> fs(nf);
    DRV(cuModuleEnumerateFunctions(fs.data(), nf, mod));
    CUfunction fn = nullptr;
    for (CUfunction f : fs) {
      const char* name = nullptr;
      if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name &&
          std::string(name).find("GraphSearchKernel") != std::string::npos)
        fn = f;
    }
    if (!fn) {
      g_msg = "GraphSearchKernel not found in cubin";
      cuModuleUnload(mod);
      cuCtxPopCurrent(&ctx);
      return -2;
    }
    int offset_shift = 0;
    while ((1 << offset_shift) < degree) ++offset_shift;
    Mem d_data, d_q, d_res, d_graph, d_entries, d_hits;
    DRV(cuMemAlloc(&d_data.p, (size_t)np * dim * 4));
    DRV(cuMemAlloc(&d_q.p, (size_t)nq * dim * 4));
    DRV(cuMemAlloc(&d_res.p, (size_t)nq * topk * 4));
    DRV(cuMemAlloc(&d_graph.p, (size_t)np * degree * 4));
    DRV(cuMemAlloc(&d_entries.p, (size_t)n_leaves * n_candidates * 4));
    DRV(cuMemAlloc(&d_hits.p, (size_t)nq * 4));
    DRV(cuMemcpyHtoD(d_data.p, data, (size_t)np * dim * 4));
    DRV(cuMemcpyHtoD(d_q.p, queries, (size_t)nq * dim * 4));
    DRV(cuMemcpyHtoD(d_graph.p, graph, (size_t)np * degree * 4));
    DRV(cuMemcpyHtoD(d_entries.p, entries, (size_t)n_leaves * n_candidates * 4));
    DRV(cuMemcpyHtoD(d_hits.p, hits, (size_t)nq * 4));
    CUdeviceptr d_cand = 0;
    void* args[] = {&d_data.p, &d_q.p,     &d_res.p,      &d_graph.p,    &d_cand,
                    &np,       &offset_shift, &n_candidates, &topk,         &search_width,
                    &d_entries.p, &d_hits.p, &max_iter,    &algo};
    const unsigned smem = (unsigned)(((search_width << offset_shift) + n_candidates) * 8);
    if (!scrub) {
      DRV(cuLaunchKernel(fn, nq, 1, 1, 64, 1, 1, smem, nullptr, args, nullptr));
      DRV(cuCtxSynchronize());
    } else {
      std::string dir(cubin_path);
      dir = dir.substr(0, dir.find_last_of('/') + 1);
      CUmodule smod;
      if (cuModuleLoad(&smod, (dir + "scrub.cubin").c_str()) != CUDA_SUCCESS) {
        g_msg = "cannot load scrub.cubin";
        cuModuleUnload(mod);
        cuCtxPopCurrent(&ctx);
        return -2;
      }
      CUfunction sf;
      DRV(cuModuleGetFunction(&sf, smod, "scrub_smem"));
      int max_smem = 0, nsm = 0;
      DRV(cuDeviceGetAttribute(&max_smem, CU_DEVICE_ATTRIBUTE_MAX_SHARED_MEMORY_PER_BLOCK_OPTIN, dev));
      DRV(cuDeviceGetAttribute(&nsm, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev));
      DRV(cuFuncSetAttribute(sf, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, max_smem));
      DRV(cuFuncSetAttribute(sf, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, 100));
      DRV(cuFuncSetAttribute(fn, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, 100));
      unsigned nwords = (unsigned)(max_smem / 4);
      void* sargs[] = {&nwords};
      for (int q = 0; q < nq; ++q) {
        DRV(cuLaunchKernel(sf, nsm, 1, 1, 1024, 1, 1, (unsigned)max_smem, nullptr, sargs, nullptr));
        CUdeviceptr dq = d_q.p + (CUdeviceptr)q * dim * 4, dr = d_res.p + (CUdeviceptr)q * topk * 4,
                    dh = d_hits.p + (CUdeviceptr)q * 4;
        void* qargs[] = {&d_data.p, &dq,         &dr,           &d_graph.p, &d_cand,
                         &np,       &offset_shift, &n_candidates, &topk,      &search_width,
                         &d_entries.p, &dh,      &max_iter,     &algo};
        DRV(cuLaunchKernel(fn, 1, 1, 1, 64, 1, 1, smem, nullptr, qargs, nullptr));
      }
      DRV(cuCtxSynchronize());
      cuModuleUnload(smod);
    }
    DRV(cuMemcpyDtoH(out, d_res.p, (size_t)nq * topk * 4));
    cuModuleUnload(mod);
  }
  cuCtxPopCurrent(&ctx);
  return rc;
}
