// index_impl.h -- the index object and small RAII helpers shared by the
// C-ABI implementation files (api.cpp, learned.cpp).
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "host_build.h"
#include "index_kernels.h"
#include "rtentry.h"

namespace rte {

rte_status fail(rte_status s, const std::string& msg);
// The BF16 (precision 1) or FP8 (2) copy of the search space, made now if
// the index has none; precision 0 needs nothing.  Synchronous.
rte_status ensure_precision(rte_index* x, int precision);
void clear_error();
bool is_device_ptr(const void* p);
void* mapped_host_ptr(void* p);
// Launch plan of a search of nq queries (api.cpp): pool and batch shape,
// warps per block, grid, shared memory and warps per query; *ordered is
// set when the batch outnumbers the resident warps and has entry leaves, so
// that taking its queries in leaf order (launch_order_by_leaf) pays.
rte_status search_plan(const rte_index* x, const rte_search_params* prm, int64_t nq, int* L, int* k,
                       int* NL, int* NB, int* wpb, int* grid, size_t* smem, int* team, bool* ordered);
// The fewest warps per query that automatic teams use (api.cpp).
int team_floor(int prec, int L, int wpb);

#define RTE_CUDA(call)                                                                     \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return ::rte::fail(e_ == cudaErrorMemoryAllocation ? RTE_ENOMEM : RTE_ECUDA,         \
                         std::string(#call) + ": " + cudaGetErrorString(e_));              \
  } while (0)

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      reset();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    reset();
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// Device scratch from the stream-ordered pool, released on scope exit
// (stream-ordered, so the memory is reused only after prior work finishes).
// The library's stream-ordered memory pool on the current device (created
// on first use, kept until the process exits), or null if it cannot be
// made.  It keeps up to kScratchKeepBytes mapped across synchronisations,
// so that a call after a synchronising call does not map its scratch again;
// the device's default pool, which releases everything at each
// synchronisation unless its owner says otherwise, is left to the host
// program.
constexpr unsigned long long kScratchKeepBytes = 1ull << 30;
cudaMemPool_t scratch_pool();

struct AsyncBuf {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  AsyncBuf() = default;
  AsyncBuf(const AsyncBuf&) = delete;
  ~AsyncBuf() {
    if (p) cudaFreeAsync(p, st);
  }
  cudaError_t alloc(size_t bytes, cudaStream_t s) {
    st = s;
    if (bytes == 0) bytes = 16;
    cudaMemPool_t pool = scratch_pool();
    if (!pool) return cudaErrorMemoryAllocation;
    return cudaMallocFromPoolAsync(&p, bytes, pool, s);
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// Learned entry model: input (search-space query * in_scale, padded to dp)
// -> hidden -> hidden -> classes (kd-tree leaves), ReLU between layers.
struct Mlp {
  bool trained = false;
  int d_in = 0, dp = 0, hidden = 0, classes = 0;
  float in_scale = 1.f;
  DevBuf<float> W[3], b[3];   // FP32 master weights: W1 [hidden x dp], W2 [hidden x hidden], W3 [classes x hidden]
  DevBuf<uint16_t> W16[3];    // BF16 copies used by the GEMMs
  // classes are kd-tree nodes at one depth (leaves above it are their own
  // class): class c covers the subtree of node class_node[c], whose first
  // leaf in pre-order is class_leaf0[c]
  int real_classes = 0;
  int depth = 0;
  DevBuf<int32_t> class_node, class_leaf0;
  // when every class starts a wide node (or is a leaf): its reference in the
  // 8-wide tree (>= 0 wide node, < 0 the leaf -(ref+1)); empty otherwise
  DevBuf<int32_t> class_wide;
};

}  // namespace rte

struct rte_index {
  int device = 0;
  int num_sms = 0;
  int64_t np = 0;
  int dim = 0;
  int degree = 0;
  rte::DevBuf<float> raw;      // [np][dim] row-major input vectors
  rte::DevBuf<int32_t> graph;  // [np][degree]
  // PCA
  bool has_pca = false;
  int search_dim = 0;
  std::vector<double> mean64, eig64, vec64;  // vec64[dim][dim], column = component
  std::vector<float> mean32, rot32;          // rot32[dim][dim]
  rte::DevBuf<float> d_mean, d_rot;          // d_rot[dim][search_dim]
  rte::DevBuf<float> d_rot_split;            // d_rot split for the tensor cores (launch_split_rotation)
  // search space
  int C = 0;
  rte::DevBuf<float> il32;
  // reduced-precision copies, made from il32 on first use or by
  // rte_index_prepare (under copy_mu), freed by rte_index_release
  rte::DevBuf<uint16_t> il16;
  rte::DevBuf<uint8_t> il8;
  rte::DevBuf<float> scale8;
  rte::DevBuf<float> norm16;  // squared norms of the BF16 rows
  std::mutex copy_mu;
  std::vector<float> xyz;  // first three search-space coordinates [np][3]
  // kd-tree
  bool has_kdtree = false;
  rte::KdTree kd;
  float expand_ratio = 0.f;
  rte::DevBuf<rte::BvhNode> d_nodes;
  rte::DevBuf<rte::WideNode> d_wide;  // 8-wide copy for point location
  std::vector<int32_t> wide_of;       // binary node -> wide node that it starts, or -1
  rte::DevBuf<int32_t> d_pids;
  // learned entry
  rte::Mlp mlp;
};
