// learned.cpp -- learned entry (MLP) training and inference on the GPU, and
// the BF16 tensor-core GEMM export.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <string>
#include <vector>

#include "gemm_tc.h"
#include "index_impl.h"
#include "mlp_head.h"
#include "mlp_kernels.h"
#include "rtentry.h"

using namespace rte;

extern "C" rte_status rte_gemm_bf16(const uint16_t* A, const uint16_t* B, int M, int N, int K,
                                    float* C, void* stream) {
  clear_error();
  if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0) return fail(RTE_EINVAL, "bad GEMM arguments");
  if (K % 8) return fail(RTE_EINVAL, "K must be a multiple of 8");
  cudaStream_t st = (cudaStream_t)stream;
  const bool ad = is_device_ptr(A), bd = is_device_ptr(B), cd = is_device_ptr(C);
  AsyncBuf a, b, c, e;
  const void* pa = A;
  const void* pb = B;
  float* pc = C;
  if (!ad) {
    RTE_CUDA(a.alloc((size_t)M * K * 2, st));
    RTE_CUDA(cudaMemcpyAsync(a.p, A, (size_t)M * K * 2, cudaMemcpyHostToDevice, st));
    pa = a.p;
  }
  if (!bd) {
    RTE_CUDA(b.alloc((size_t)N * K * 2, st));
    RTE_CUDA(cudaMemcpyAsync(b.p, B, (size_t)N * K * 2, cudaMemcpyHostToDevice, st));
    pb = b.p;
  }
  if (!cd) {
    RTE_CUDA(c.alloc((size_t)M * N * 4, st));
    pc = c.as<float>();
  }
  RTE_CUDA(e.alloc(4, st));
  RTE_CUDA(cudaMemsetAsync(e.p, 0, 4, st));
  GemmArgs g{};
  g.A = pa;
  g.B = pb;
  g.M = M;
  g.N = N;
  g.K = K;
  g.epilogue = kEpiStoreF32;
  g.C = pc;
  g.ldc = N;
  g.err = e.as<int>();
  RTE_CUDA(gemm_bf16_tn(g, st));
  int herr = 0;
  RTE_CUDA(cudaMemcpyAsync(&herr, e.p, 4, cudaMemcpyDeviceToHost, st));
  if (!cd) RTE_CUDA(cudaMemcpyAsync(C, pc, (size_t)M * N * 4, cudaMemcpyDeviceToHost, st));
  RTE_CUDA(cudaStreamSynchronize(st));
  if (herr) return fail(RTE_ETIMEOUT, "GEMM pipeline wait ran out (code " + std::to_string(herr) + ")");
  return RTE_OK;
}

extern "C" rte_status rte_gemm_bf16_bias_argmax(const uint16_t* A, const uint16_t* B,
                                                const float* bias, int M, int N, int K,
                                                int32_t* cols, void* stream) {
  clear_error();
  if (!A || !B || !bias || !cols || M <= 0 || N <= 0 || K <= 0)
    return fail(RTE_EINVAL, "bad GEMM arguments");
  if (K % 8) return fail(RTE_EINVAL, "K must be a multiple of 8");
  cudaStream_t st = (cudaStream_t)stream;
  AsyncBuf a, b, bb, keys, out, e;
  const void* pa = A;
  const void* pb = B;
  const float* pbias = bias;
  if (!is_device_ptr(A)) {
    RTE_CUDA(a.alloc((size_t)M * K * 2, st));
    RTE_CUDA(cudaMemcpyAsync(a.p, A, (size_t)M * K * 2, cudaMemcpyHostToDevice, st));
    pa = a.p;
  }
  if (!is_device_ptr(B)) {
    RTE_CUDA(b.alloc((size_t)N * K * 2, st));
    RTE_CUDA(cudaMemcpyAsync(b.p, B, (size_t)N * K * 2, cudaMemcpyHostToDevice, st));
    pb = b.p;
  }
  if (!is_device_ptr(bias)) {
    RTE_CUDA(bb.alloc((size_t)N * 4, st));
    RTE_CUDA(cudaMemcpyAsync(bb.p, bias, (size_t)N * 4, cudaMemcpyHostToDevice, st));
    pbias = bb.as<float>();
  }
  const bool cd = is_device_ptr(cols);
  RTE_CUDA(keys.alloc((size_t)M * 8, st));
  RTE_CUDA(cudaMemsetAsync(keys.p, 0, (size_t)M * 8, st));
  RTE_CUDA(e.alloc(4, st));
  RTE_CUDA(cudaMemsetAsync(e.p, 0, 4, st));
  int32_t* pc = cols;
  if (!cd) {
    RTE_CUDA(out.alloc((size_t)M * 4, st));
    pc = out.as<int32_t>();
  }
  GemmArgs g{};
  g.A = pa;
  g.B = pb;
  g.M = M;
  g.N = N;
  g.K = K;
  g.epilogue = kEpiBiasArgmax;
  g.bias = pbias;
  g.out_argmax = keys.as<unsigned long long>();
  g.err = e.as<int>();
  RTE_CUDA(gemm_bf16_tn(g, st));
  RTE_CUDA(launch_argmax_to_leaf(keys.as<unsigned long long>(), M, nullptr, pc, st));
  int herr = 0;
  RTE_CUDA(cudaMemcpyAsync(&herr, e.p, 4, cudaMemcpyDeviceToHost, st));
  if (!cd) RTE_CUDA(cudaMemcpyAsync(cols, pc, (size_t)M * 4, cudaMemcpyDeviceToHost, st));
  RTE_CUDA(cudaStreamSynchronize(st));
  if (herr) return fail(RTE_ETIMEOUT, "GEMM pipeline wait ran out (code " + std::to_string(herr) + ")");
  return RTE_OK;
}

// ---------------------------------------------------------------------------
// Learned entry.  A 3-layer MLP (search-space query -> hidden -> hidden ->
// kd-tree leaf) proposes the entry leaf.  It is trained on (query, leaf of
// the best result of the plain kd-tree search) pairs produced by this
// library's own search kernel; every GEMM runs on the tensor cores
// (gemm_tc.cu) in BF16 with FP32 accumulation, the softmax cross-entropy,
// ReLU backward, bias gradients and Adam in mlp_kernels.cu.
// ---------------------------------------------------------------------------

namespace {

struct Bf16Mat {
  AsyncBuf buf;
  uint16_t* p = nullptr;
};

cudaError_t gemm(const void* A, const void* B, int M, int N, int K, int epi, void* C, int ldc,
                 const float* bias, unsigned long long* am, int* err, cudaStream_t st) {
  GemmArgs g{};
  g.A = A;
  g.B = B;
  g.M = M;
  g.N = N;
  g.K = K;
  g.epilogue = epi;
  g.C = C;
  g.ldc = ldc;
  g.bias = bias;
  g.out_argmax = am;
  g.err = err;
  return gemm_bf16_tn(g, st);
}

int round8(int v) { return (v + 7) & ~7; }

// The head's forward pass on zeroed keys: the fused kernel (path 0,
// mlp_head.cu) or the three layer-by-layer GEMMs (path 1).  Both round the
// hidden activations to BF16 the same way and give the same keys.
rte_status head_keys(const MlpHeadArgs& h, int path, cudaStream_t st) {
  if (path == 0) {
    if (!mlp_head_supported(h)) return fail(RTE_EINVAL, "shape not supported by the fused head kernel");
    RTE_CUDA(mlp_head_argmax(h, st));
    return RTE_OK;
  }
  AsyncBuf h1, h2;
  RTE_CUDA(h1.alloc((size_t)h.M * h.H * 2, st));
  RTE_CUDA(h2.alloc((size_t)h.M * h.H * 2, st));
  RTE_CUDA(gemm(h.X, h.W1, h.M, h.H, h.dp, kEpiBiasReluBF16, h1.p, h.H, h.b1, nullptr, h.err, st));
  RTE_CUDA(gemm(h1.p, h.W2, h.M, h.H, h.H, kEpiBiasReluBF16, h2.p, h.H, h.b2, nullptr, h.err, st));
  RTE_CUDA(gemm(h2.p, h.W3, h.M, h.N, h.H, kEpiBiasArgmax, nullptr, 0, h.b3, h.keys, h.err, st));
  return RTE_OK;
}

// MLP forward for nq rows of X (BF16 [nq x dp]) -> packed argmax key per row
// (keys [nq], zeroed here unless keys_zeroed).  The fused kernel where it
// takes the shape, the layer-by-layer GEMMs otherwise.
rte_status mlp_keys_bf16(const rte_index* x, const uint16_t* X, int64_t nq, unsigned long long* keys,
                         int* d_err, cudaStream_t st, bool keys_zeroed) {
  const Mlp& m = x->mlp;
  if (!keys_zeroed) RTE_CUDA(cudaMemsetAsync(keys, 0, (size_t)nq * 8, st));
  MlpHeadArgs h{};
  h.X = X;
  h.W1 = m.W16[0].p;
  h.W2 = m.W16[1].p;
  h.W3 = m.W16[2].p;
  h.b1 = m.b[0].p;
  h.b2 = m.b[1].p;
  h.b3 = m.b[2].p;
  h.M = (int)nq;
  h.dp = m.dp;
  h.H = m.hidden;
  h.N = m.classes;
  h.keys = keys;
  h.err = d_err;
  if (mlp_head_supported(h)) {
    const cudaError_t e = mlp_head_argmax(h, st);
    if (e == cudaSuccess) return RTE_OK;
    if (e != cudaErrorNotSupported) RTE_CUDA(e);  // NotSupported: nothing was launched
  }
  return head_keys(h, 1, st);
}

// MLP forward for nq rows of X (BF16 [nq x dp]) -> class (subtree) per row.
rte_status mlp_predict_bf16(const rte_index* x, const uint16_t* X, int64_t nq, int32_t* d_cls,
                            int* d_err, cudaStream_t st) {
  AsyncBuf keys;
  RTE_CUDA(keys.alloc((size_t)nq * 8, st));
  rte_status s = mlp_keys_bf16(x, X, nq, keys.as<unsigned long long>(), d_err, st, false);
  if (s != RTE_OK) return s;
  RTE_CUDA(launch_argmax_to_leaf(keys.as<unsigned long long>(), (int)nq, nullptr, d_cls, st));
  return RTE_OK;
}

// Classes of the learned head: the kd-tree nodes at `depth` (or leaves above
// it), numbered in pre-order, left first.
void subtree_classes(const KdTree& t, int depth, std::vector<int32_t>& leaf_class,
                     std::vector<int32_t>& class_node, std::vector<int32_t>& class_leaf0) {
  leaf_class.assign(t.n_leaves, 0);
  class_node.clear();
  class_leaf0.clear();
  std::vector<std::pair<int, int>> st{{0, 0}};  // (node, depth)
  while (!st.empty()) {
    auto [nd, dep] = st.back();
    st.pop_back();
    const BvhNode& N = t.nodes[nd];
    if (dep == depth || N.left < 0) {
      const int32_t c = (int32_t)class_node.size();
      class_node.push_back(nd);
      class_leaf0.push_back(-1);
      std::vector<int> sub{nd};
      while (!sub.empty()) {  // pre-order, left first: the first leaf met is the smallest
        const int m = sub.back();
        sub.pop_back();
        const BvhNode& Q = t.nodes[m];
        if (Q.left < 0) {
          const int32_t leaf = -Q.left - 1;
          leaf_class[leaf] = c;
          if (class_leaf0[c] < 0) class_leaf0[c] = leaf;
        } else {
          sub.push_back(Q.right);
          sub.push_back(Q.left);
        }
      }
      continue;
    }
    st.push_back({N.right, dep + 1});
    st.push_back({N.left, dep + 1});
  }
}

// Buffers of one optimisation step on a batch of M rows.
struct StepBufs {
  DevBuf<uint16_t> H1, H2, dZ, dZT, H2T, W3T, dH2, dH2T, H1T, W2T, dH1, dH1T, XT;
  DevBuf<float> Z, dH2f, dH1f, loss, colpart;
  rte_status alloc(int M, int H, int C, int dp) {
    RTE_CUDA(colpart.alloc((size_t)col_sum_slices(M) * std::max(H, C)));
    RTE_CUDA(H1.alloc((size_t)M * H));
    RTE_CUDA(H2.alloc((size_t)M * H));
    RTE_CUDA(Z.alloc((size_t)M * C));
    RTE_CUDA(dZ.alloc((size_t)M * C));
    RTE_CUDA(dZT.alloc((size_t)M * C));
    RTE_CUDA(H2T.alloc((size_t)M * H));
    RTE_CUDA(W3T.alloc((size_t)H * C));
    RTE_CUDA(dH2f.alloc((size_t)M * H));
    RTE_CUDA(dH2.alloc((size_t)M * H));
    RTE_CUDA(dH2T.alloc((size_t)M * H));
    RTE_CUDA(H1T.alloc((size_t)M * H));
    RTE_CUDA(W2T.alloc((size_t)H * H));
    RTE_CUDA(dH1f.alloc((size_t)M * H));
    RTE_CUDA(dH1.alloc((size_t)M * H));
    RTE_CUDA(dH1T.alloc((size_t)M * H));
    RTE_CUDA(XT.alloc((size_t)M * dp));
    RTE_CUDA(loss.alloc(M));
    return RTE_OK;
  }
};

// Forward and backward of the MLP on one batch: Xb [M x dp] BF16, labels
// yb [M]; writes the FP32 gradients gw[l] (same shapes as the weights) and
// gb[l] and the per-row loss.  Mean cross-entropy over the batch.
rte_status fwd_bwd(const Mlp& m, const uint16_t* Xb, const int32_t* yb, int M, StepBufs& b,
                   float* const gw[3], float* const gb[3], int* err, cudaStream_t st) {
  const int H = m.hidden, C = m.classes, dp = m.dp;
  RTE_CUDA(gemm(Xb, m.W16[0].p, M, H, dp, kEpiBiasReluBF16, b.H1.p, H, m.b[0].p, nullptr, err, st));
  RTE_CUDA(gemm(b.H1.p, m.W16[1].p, M, H, H, kEpiBiasReluBF16, b.H2.p, H, m.b[1].p, nullptr, err, st));
  RTE_CUDA(gemm(b.H2.p, m.W16[2].p, M, C, H, kEpiBiasF32, b.Z.p, C, m.b[2].p, nullptr, err, st));
  RTE_CUDA(launch_softmax_ce(b.Z.p, M, C, yb, 1.0f / M, b.dZ.p, b.loss.p, st));
  // layer 3: dW3 = dZ^T H2, db3 = colsum(dZ), dH2 = relu'(H2) * (dZ W3)
  RTE_CUDA(launch_transpose_bf16(b.dZ.p, M, C, b.dZT.p, st));
  RTE_CUDA(launch_transpose_bf16(b.H2.p, M, H, b.H2T.p, st));
  RTE_CUDA(gemm(b.dZT.p, b.H2T.p, C, H, M, kEpiStoreF32, gw[2], H, nullptr, nullptr, err, st));
  RTE_CUDA(launch_col_sum_bf16(b.dZ.p, M, C, gb[2], b.colpart.p, st));
  RTE_CUDA(launch_transpose_bf16(m.W16[2].p, C, H, b.W3T.p, st));
  RTE_CUDA(gemm(b.dZ.p, b.W3T.p, M, H, C, kEpiStoreF32, b.dH2f.p, H, nullptr, nullptr, err, st));
  RTE_CUDA(launch_relu_grad(b.dH2f.p, b.H2.p, (int64_t)M * H, b.dH2.p, st));
  // layer 2
  RTE_CUDA(launch_transpose_bf16(b.dH2.p, M, H, b.dH2T.p, st));
  RTE_CUDA(launch_transpose_bf16(b.H1.p, M, H, b.H1T.p, st));
  RTE_CUDA(gemm(b.dH2T.p, b.H1T.p, H, H, M, kEpiStoreF32, gw[1], H, nullptr, nullptr, err, st));
  RTE_CUDA(launch_col_sum_bf16(b.dH2.p, M, H, gb[1], b.colpart.p, st));
  RTE_CUDA(launch_transpose_bf16(m.W16[1].p, H, H, b.W2T.p, st));
  RTE_CUDA(gemm(b.dH2.p, b.W2T.p, M, H, H, kEpiStoreF32, b.dH1f.p, H, nullptr, nullptr, err, st));
  RTE_CUDA(launch_relu_grad(b.dH1f.p, b.H1.p, (int64_t)M * H, b.dH1.p, st));
  // layer 1
  RTE_CUDA(launch_transpose_bf16(b.dH1.p, M, H, b.dH1T.p, st));
  RTE_CUDA(launch_transpose_bf16(Xb, M, dp, b.XT.p, st));
  RTE_CUDA(gemm(b.dH1T.p, b.XT.p, H, dp, M, kEpiStoreF32, gw[0], dp, nullptr, nullptr, err, st));
  RTE_CUDA(launch_col_sum_bf16(b.dH1.p, M, H, gb[0], b.colpart.p, st));
  return RTE_OK;
}

}  // namespace

extern "C" rte_status rte_mlp_head_argmax(const uint16_t* X, int M, int dp, const uint16_t* W1,
                                          const float* b1, const uint16_t* W2, const float* b2,
                                          const uint16_t* W3, const float* b3, int H, int N, int path,
                                          int32_t* cols, void* stream) {
  clear_error();
  if (!X || !W1 || !b1 || !W2 || !b2 || !W3 || !b3 || !cols || M <= 0 || dp <= 0 || H <= 0 || N <= 0)
    return fail(RTE_EINVAL, "bad head arguments");
  if (path != 0 && path != 1) return fail(RTE_EINVAL, "path must be 0 (fused) or 1 (layer by layer)");
  if (dp % 8 || H % 8) return fail(RTE_EINVAL, "dp and H must be multiples of 8");
  const void* ptrs[] = {X, W1, b1, W2, b2, W3, b3, cols};
  for (const void* q : ptrs)
    if (!is_device_ptr(q)) return fail(RTE_EINVAL, "rte_mlp_head_argmax takes device pointers");
  cudaStream_t st = (cudaStream_t)stream;
  AsyncBuf keys, e;
  RTE_CUDA(keys.alloc((size_t)M * 8, st));
  RTE_CUDA(cudaMemsetAsync(keys.p, 0, (size_t)M * 8, st));
  RTE_CUDA(e.alloc(4, st));
  RTE_CUDA(cudaMemsetAsync(e.p, 0, 4, st));
  MlpHeadArgs h{};
  h.X = X;
  h.W1 = W1;
  h.W2 = W2;
  h.W3 = W3;
  h.b1 = b1;
  h.b2 = b2;
  h.b3 = b3;
  h.M = M;
  h.dp = dp;
  h.H = H;
  h.N = N;
  h.keys = keys.as<unsigned long long>();
  h.err = e.as<int>();
  rte_status s = head_keys(h, path, st);
  if (s != RTE_OK) return s;
  RTE_CUDA(launch_argmax_to_leaf(keys.as<unsigned long long>(), M, nullptr, cols, st));
  int herr = 0;
  RTE_CUDA(cudaMemcpyAsync(&herr, e.p, 4, cudaMemcpyDeviceToHost, st));
  RTE_CUDA(cudaStreamSynchronize(st));
  if (herr) return fail(RTE_ETIMEOUT, "head pipeline wait ran out (code " + std::to_string(herr) + ")");
  return RTE_OK;
}

namespace rte {

// Leaf prediction for projected queries already on the device.
// xb: the head's BF16 input rows ([nq x dp], from launch_project_bf16), or
// null to form them here from d_proj.
rte_status learned_leaves(const rte_index* x, const float* d_proj, int64_t nq, int32_t* d_leaf,
                          cudaStream_t st, const uint16_t* xb_in, unsigned long long* zkeys, int* zerr) {
  if (!x->mlp.trained) return fail(RTE_ESTATE, "learned entries requested before rte_learned_train");
  if (nq == 0) return RTE_OK;
  const Mlp& m = x->mlp;
  AsyncBuf xb, errb, keysb;
  // zkeys / zerr: scratch the caller has already zeroed
  const bool zeroed = zkeys && zerr;
  int* err = zerr;
  unsigned long long* keys = zkeys;
  if (!zeroed) {
    RTE_CUDA(errb.alloc(4, st));
    RTE_CUDA(cudaMemsetAsync(errb.p, 0, 4, st));
    RTE_CUDA(keysb.alloc((size_t)nq * 8, st));
    err = errb.as<int>();
    keys = keysb.as<unsigned long long>();
  }
  const uint16_t* X = xb_in;
  if (!X) {
    RTE_CUDA(xb.alloc((size_t)nq * m.dp * 2, st));
    RTE_CUDA(launch_cast_rows_bf16(d_proj, nq, m.d_in, x->search_dim, m.in_scale, m.dp, xb.p, st));
    X = xb.as<uint16_t>();
  }
  rte_status s = mlp_keys_bf16(x, X, nq, keys, err, st, zeroed);
  if (s != RTE_OK) return s;
  // the model picks the subtree (decoded from its argmax key), the kd-tree
  // picks the leaf inside it
  if (m.class_wide.p) {
    RTE_CUDA(launch_locate_in_subtree_wide(x->d_wide.p, d_proj, nq, x->search_dim,
                                           keys, m.class_wide.p,
                                           m.class_leaf0.p, m.real_classes, d_leaf, st));
  } else {
    RTE_CUDA(launch_locate_in_subtree(x->d_nodes.p, d_proj, nq, x->search_dim, nullptr,
                                      keys, m.class_node.p,
                                      m.class_leaf0.p, m.real_classes, d_leaf, st));
  }
  return RTE_OK;
}

// Plain-search top-1 for each projected query (device arrays) -> ids.
rte_status plain_top1(rte_index* x, const float* d_proj, int64_t n, int beam, int32_t* d_ids,
                      cudaStream_t st);

}  // namespace rte

extern "C" void rte_default_train_params(rte_train_params* p) {
  if (!p) return;
  p->hidden = 256;
  p->epochs = 4;
  p->batch = 4096;
  p->lr = 2e-3f;
  p->label_beam = 64;
  p->seed = 3003;
  p->max_classes = 4096;
}

extern "C" rte_status rte_learned_train(rte_index* x, const float* train_queries, int64_t n,
                                        const rte_train_params* tp, rte_train_report* rep) {
  clear_error();
  if (!x || !train_queries || !tp) return fail(RTE_EINVAL, "NULL argument");
  if (!x->has_kdtree) return fail(RTE_ESTATE, "rte_learned_train needs the kd-tree");
  if (tp->hidden <= 0 || tp->hidden % 8 || tp->epochs <= 0 || tp->batch <= 0 || tp->batch % 128 ||
      !(tp->lr > 0.f) || tp->label_beam <= 0)
    return fail(RTE_EINVAL, "bad training parameters (hidden % 8 == 0, batch % 128 == 0)");
  if (n < tp->batch) return fail(RTE_EINVAL, "fewer training queries than one batch");
  if (tp->max_classes < 2 || tp->max_classes > 65536)
    return fail(RTE_EINVAL, "max_classes must be in [2, 65536]");
  // classes: kd-tree nodes at the deepest level with at most max_classes nodes
  int depth = 0;
  while ((2 << depth) <= tp->max_classes) ++depth;
  std::vector<int32_t> leaf_class, class_node, class_leaf0;
  subtree_classes(x->kd, depth, leaf_class, class_node, class_leaf0);
  const int64_t C = (int64_t)class_node.size();
  DeviceGuard guard(x->device);
  cudaStream_t st = nullptr;
  const int H = tp->hidden, d = x->search_dim, dp = round8(d), M = tp->batch;
  // 1. project the training queries
  DevBuf<float> q32, proj;
  RTE_CUDA(q32.alloc((size_t)n * x->dim));
  RTE_CUDA(cudaMemcpy(q32.p, train_queries, q32.bytes(), cudaMemcpyDefault));
  RTE_CUDA(proj.alloc((size_t)n * d));
  if (x->has_pca) {
    RTE_CUDA(launch_project(q32.p, n, x->dim, x->dim, x->d_mean.p, x->d_rot.p, d, d, proj.p, d, st,
                            nullptr, 0, x->d_rot_split.p));
  } else {
    RTE_CUDA(cudaMemcpy(proj.p, q32.p, proj.bytes(), cudaMemcpyDeviceToDevice));
  }
  q32.reset();
  // 2. labels: leaf of the plain search's best result
  DevBuf<int32_t> top;
  RTE_CUDA(top.alloc(n));
  rte_status s = plain_top1(x, proj.p, n, tp->label_beam, top.p, st);
  if (s != RTE_OK) return s;
  std::vector<int32_t> ids(n), leaf_of(x->np, 0), labels(n);
  RTE_CUDA(cudaMemcpy(ids.data(), top.p, n * 4, cudaMemcpyDeviceToHost));
  for (int64_t l = 0; l < x->kd.n_leaves; ++l)
    for (int j = 0; j < x->kd.cap; ++j) {
      const int32_t p = x->kd.pids[l * x->kd.cap + j];
      if (p < x->np) leaf_of[p] = (int32_t)l;
    }
  for (int64_t i = 0; i < n; ++i)
    labels[i] = leaf_class[(ids[i] >= 0 && ids[i] < x->np) ? leaf_of[ids[i]] : 0];
  DevBuf<int32_t> d_labels;
  RTE_CUDA(d_labels.alloc(n));
  RTE_CUDA(cudaMemcpy(d_labels.p, labels.data(), n * 4, cudaMemcpyHostToDevice));
  // 3. inputs: BF16 of the projected query scaled to unit RMS
  std::vector<float> sample((size_t)std::min<int64_t>(n, 4096) * d);
  RTE_CUDA(cudaMemcpy(sample.data(), proj.p, sample.size() * 4, cudaMemcpyDeviceToHost));
  double ss = 0;
  for (float v : sample) ss += (double)v * v;
  const float in_scale = (float)(1.0 / std::sqrt(std::max(ss / sample.size(), 1e-30)));
  DevBuf<uint16_t> X;
  RTE_CUDA(X.alloc((size_t)n * dp));
  RTE_CUDA(launch_cast_rows_bf16(proj.p, n, d, d, in_scale, dp, X.p, st));
  proj.reset();
  // 4. parameters (He-uniform, fixed seed), Adam moments
  Mlp m;
  m.d_in = d;
  m.dp = dp;
  m.hidden = H;
  // class dimension padded to a multiple of 8 (16-byte TMA row pitch of the
  // logits / dlogits); padded classes have bias -1e30: zero probability,
  // zero gradient, never the argmax
  const int64_t Cp = round8((int)C);
  m.classes = (int)Cp;
  m.in_scale = in_scale;
  const int64_t wn[3] = {(int64_t)H * dp, (int64_t)H * H, Cp * H};
  const int64_t bn[3] = {H, H, Cp};
  const int fan[3] = {d, H, H};
  DevBuf<float> mw[3], vw[3], mb[3], vb[3], gw[3], gb[3];
  std::mt19937 rng((uint32_t)tp->seed);
  for (int l = 0; l < 3; ++l) {
    std::vector<float> w(wn[l]);
    const float lim = std::sqrt(6.0f / fan[l]);
    std::uniform_real_distribution<float> U(-lim, lim);
    for (int64_t i = 0; i < wn[l]; ++i) w[i] = U(rng);
    if (l == 0)  // padded input columns stay zero
      for (int r = 0; r < H; ++r)
        for (int c = d; c < dp; ++c) w[(int64_t)r * dp + c] = 0.f;
    if (l == 2)  // padded classes: zero weights
      for (int64_t i = C * H; i < Cp * H; ++i) w[i] = 0.f;
    std::vector<float> bias(bn[l], 0.f);
    if (l == 2)
      for (int64_t i = C; i < Cp; ++i) bias[i] = -1e30f;
    RTE_CUDA(m.W[l].alloc(wn[l]));
    RTE_CUDA(m.W16[l].alloc(wn[l]));
    RTE_CUDA(m.b[l].alloc(bn[l]));
    RTE_CUDA(cudaMemcpy(m.W[l].p, w.data(), wn[l] * 4, cudaMemcpyHostToDevice));
    RTE_CUDA(cudaMemcpy(m.b[l].p, bias.data(), bn[l] * 4, cudaMemcpyHostToDevice));
    RTE_CUDA(launch_f32_to_bf16(m.W[l].p, wn[l], m.W16[l].p, st));
    for (DevBuf<float>* b : {&mw[l], &vw[l], &gw[l]}) {
      RTE_CUDA(b->alloc(wn[l]));
      RTE_CUDA(cudaMemset(b->p, 0, b->bytes()));
    }
    for (DevBuf<float>* b : {&mb[l], &vb[l], &gb[l]}) {
      RTE_CUDA(b->alloc(bn[l]));
      RTE_CUDA(cudaMemset(b->p, 0, b->bytes()));
    }
  }
  // 5. per-batch buffers
  StepBufs sb;
  s = sb.alloc(M, H, (int)Cp, dp);
  if (s != RTE_OK) return s;
  DevBuf<uint16_t> Xb;
  DevBuf<int32_t> yb;
  DevBuf<int64_t> perm;
  DevBuf<int> err;
  RTE_CUDA(Xb.alloc((size_t)M * dp));
  RTE_CUDA(yb.alloc(M));
  RTE_CUDA(perm.alloc(n));
  RTE_CUDA(err.alloc(1));
  RTE_CUDA(cudaMemset(err.p, 0, 4));
  float* const gwp[3] = {gw[0].p, gw[1].p, gw[2].p};
  float* const gbp[3] = {gb[0].p, gb[1].p, gb[2].p};
  std::vector<int64_t> order(n);
  for (int64_t i = 0; i < n; ++i) order[i] = i;
  const int64_t steps_per_epoch = n / M;
  const int64_t total = steps_per_epoch * tp->epochs;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  int64_t t = 0;
  float first_loss = -1.f, last_loss = 0.f;
  std::vector<float> hl(M);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, st);
  for (int ep = 0; ep < tp->epochs; ++ep) {
    std::shuffle(order.begin(), order.end(), rng);
    RTE_CUDA(cudaMemcpy(perm.p, order.data(), n * 8, cudaMemcpyHostToDevice));
    for (int64_t sidx = 0; sidx < steps_per_epoch; ++sidx, ++t) {
      RTE_CUDA(launch_gather_rows(X.p, dp, perm.p + sidx * M, M, d_labels.p, Xb.p, yb.p, st));
      s = fwd_bwd(m, Xb.p, yb.p, M, sb, gwp, gbp, err.p, st);
      if (s != RTE_OK) return s;
      // Adam with a cosine decay to a tenth of the rate
      const float frac = total > 1 ? (float)t / (float)(total - 1) : 0.f;
      const float lr = tp->lr * (0.1f + 0.9f * 0.5f * (1.f + std::cos(3.14159265f * frac)));
      const float c1 = 1.f / (1.f - std::pow(b1, (float)(t + 1)));
      const float c2 = 1.f / (1.f - std::pow(b2, (float)(t + 1)));
      for (int l = 0; l < 3; ++l) {
        RTE_CUDA(launch_adam(m.W[l].p, gw[l].p, mw[l].p, vw[l].p, wn[l], lr, b1, b2, eps, c1, c2,
                             m.W16[l].p, st));
        RTE_CUDA(launch_adam(m.b[l].p, gb[l].p, mb[l].p, vb[l].p, bn[l], lr, b1, b2, eps, c1, c2,
                             nullptr, st));
      }
      if (t == 0 || t == total - 1) {
        RTE_CUDA(cudaMemcpy(hl.data(), sb.loss.p, M * 4, cudaMemcpyDeviceToHost));
        double sl = 0;
        for (float v : hl) sl += v;
        (t == 0 ? first_loss : last_loss) = (float)(sl / M);
      }
    }
  }
  cudaEventRecord(e1, st);
  RTE_CUDA(cudaStreamSynchronize(st));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int herr = 0;
  RTE_CUDA(cudaMemcpy(&herr, err.p, 4, cudaMemcpyDeviceToHost));
  if (herr) return fail(RTE_ETIMEOUT, "a GEMM pipeline wait ran out during training");
  m.trained = true;
  m.real_classes = (int)C;
  m.depth = depth;
  RTE_CUDA(m.class_node.alloc(C));
  RTE_CUDA(m.class_leaf0.alloc(C));
  RTE_CUDA(cudaMemcpy(m.class_node.p, class_node.data(), C * 4, cudaMemcpyHostToDevice));
  RTE_CUDA(cudaMemcpy(m.class_leaf0.p, class_leaf0.data(), C * 4, cudaMemcpyHostToDevice));
  {
    // classes three binary levels apart start wide nodes: locate on the 8-wide tree
    std::vector<int32_t> ref(C);
    bool all = x->wide_of.size() == x->kd.nodes.size();
    for (int64_t c = 0; c < C && all; ++c) {
      const BvhNode& nd = x->kd.nodes[class_node[c]];
      ref[c] = nd.left < 0 ? nd.left : x->wide_of[class_node[c]];
      if (nd.left >= 0 && ref[c] < 0) all = false;
    }
    if (all) {
      RTE_CUDA(m.class_wide.alloc(C));
      RTE_CUDA(cudaMemcpy(m.class_wide.p, ref.data(), C * 4, cudaMemcpyHostToDevice));
    }
  }
  // training accuracy (of the class) on the first batch of the last permutation
  {
    DevBuf<int32_t> pred;
    RTE_CUDA(pred.alloc(M));
    RTE_CUDA(launch_gather_rows(X.p, dp, perm.p, M, d_labels.p, Xb.p, yb.p, st));
    std::swap(x->mlp, m);
    rte_status s2 = mlp_predict_bf16(x, Xb.p, M, pred.p, err.p, st);
    if (s2 != RTE_OK) return s2;
    std::vector<int32_t> hp(M), hy(M);
    RTE_CUDA(cudaMemcpy(hp.data(), pred.p, M * 4, cudaMemcpyDeviceToHost));
    RTE_CUDA(cudaMemcpy(hy.data(), yb.p, M * 4, cudaMemcpyDeviceToHost));
    int hit = 0;
    for (int i = 0; i < M; ++i) hit += hp[i] == hy[i];
    if (rep) {
      rep->first_loss = first_loss;
      rep->last_loss = last_loss;
      rep->train_acc = (float)hit / M;
      rep->n_train = n;
      rep->classes = (int)C;
      rep->steps = total;
      rep->train_ms = ms;
    }
  }
  return RTE_OK;
}

extern "C" rte_status rte_learned_predict(rte_index* x, const float* projected, int64_t nq,
                                          int32_t* out_leaf, void* stream) {
  clear_error();
  if (!x || (!projected && nq) || (!out_leaf && nq)) return fail(RTE_EINVAL, "NULL argument");
  if (!x->mlp.trained) return fail(RTE_ESTATE, "no learned model");
  if (nq <= 0) return nq == 0 ? RTE_OK : fail(RTE_EINVAL, "nq < 0");
  DeviceGuard guard(x->device);
  cudaStream_t st = (cudaStream_t)stream;
  AsyncBuf pb, ob;
  const float* dp = projected;
  if (!is_device_ptr(projected)) {
    RTE_CUDA(pb.alloc((size_t)nq * x->search_dim * 4, st));
    RTE_CUDA(cudaMemcpyAsync(pb.p, projected, (size_t)nq * x->search_dim * 4, cudaMemcpyHostToDevice, st));
    dp = pb.as<float>();
  }
  int32_t* dout = out_leaf;
  const bool host_out = !is_device_ptr(out_leaf);
  if (host_out) {
    RTE_CUDA(ob.alloc((size_t)nq * 4, st));
    dout = ob.as<int32_t>();
  }
  rte_status s = learned_leaves(x, dp, nq, dout, st, nullptr, nullptr, nullptr);
  if (s != RTE_OK) return s;
  if (host_out) {
    RTE_CUDA(cudaMemcpyAsync(out_leaf, dout, (size_t)nq * 4, cudaMemcpyDeviceToHost, st));
    RTE_CUDA(cudaStreamSynchronize(st));
  }
  return RTE_OK;
}

extern "C" rte_status rte_mlp_grad_check(const float* X, const int32_t* labels, int M, int d,
                                         int hidden, int classes, const float* W1, const float* b1,
                                         const float* W2, const float* b2, const float* W3,
                                         const float* b3, float* gW1, float* gb1, float* gW2,
                                         float* gb2, float* gW3, float* gb3, float* loss) {
  clear_error();
  if (!X || !labels || !W1 || !b1 || !W2 || !b2 || !W3 || !b3 || M <= 0 || d <= 0 ||
      hidden <= 0 || hidden % 8 || classes <= 0)
    return fail(RTE_EINVAL, "bad arguments");
  cudaStream_t st = nullptr;
  Mlp m;
  m.d_in = d;
  m.dp = round8(d);
  m.hidden = hidden;
  const int Cp = round8(classes);  // padded as in training
  m.classes = Cp;
  const int H = hidden, dp = m.dp;
  const int64_t wn[3] = {(int64_t)H * dp, (int64_t)H * H, (int64_t)Cp * H};
  const int64_t bn[3] = {H, H, Cp};
  std::vector<float> w1p(wn[0], 0.f), w3p(wn[2], 0.f), b3p(Cp, -1e30f);
  for (int r = 0; r < H; ++r)
    for (int c = 0; c < d; ++c) w1p[(int64_t)r * dp + c] = W1[(int64_t)r * d + c];
  std::copy(W3, W3 + (int64_t)classes * H, w3p.begin());
  std::copy(b3, b3 + classes, b3p.begin());
  const float* wsrc[3] = {w1p.data(), W2, w3p.data()};
  const float* bsrc[3] = {b1, b2, b3p.data()};
  DevBuf<float> gw[3], gb[3];
  for (int l = 0; l < 3; ++l) {
    RTE_CUDA(m.W[l].alloc(wn[l]));
    RTE_CUDA(m.W16[l].alloc(wn[l]));
    RTE_CUDA(m.b[l].alloc(bn[l]));
    RTE_CUDA(cudaMemcpy(m.W[l].p, wsrc[l], wn[l] * 4, cudaMemcpyHostToDevice));
    RTE_CUDA(cudaMemcpy(m.b[l].p, bsrc[l], bn[l] * 4, cudaMemcpyHostToDevice));
    RTE_CUDA(launch_f32_to_bf16(m.W[l].p, wn[l], m.W16[l].p, st));
    RTE_CUDA(gw[l].alloc(wn[l]));
    RTE_CUDA(gb[l].alloc(bn[l]));
  }
  DevBuf<float> x32;
  DevBuf<uint16_t> xb;
  DevBuf<int32_t> y;
  DevBuf<int> err;
  RTE_CUDA(x32.alloc((size_t)M * d));
  RTE_CUDA(xb.alloc((size_t)M * dp));
  RTE_CUDA(y.alloc(M));
  RTE_CUDA(err.alloc(1));
  RTE_CUDA(cudaMemset(err.p, 0, 4));
  RTE_CUDA(cudaMemcpy(x32.p, X, x32.bytes(), cudaMemcpyHostToDevice));
  RTE_CUDA(cudaMemcpy(y.p, labels, (size_t)M * 4, cudaMemcpyHostToDevice));
  RTE_CUDA(launch_cast_rows_bf16(x32.p, M, d, d, 1.0f, dp, xb.p, st));
  StepBufs sb;
  rte_status s = sb.alloc(M, H, Cp, dp);
  if (s != RTE_OK) return s;
  float* const gwp[3] = {gw[0].p, gw[1].p, gw[2].p};
  float* const gbp[3] = {gb[0].p, gb[1].p, gb[2].p};
  s = fwd_bwd(m, xb.p, y.p, M, sb, gwp, gbp, err.p, st);
  if (s != RTE_OK) return s;
  RTE_CUDA(cudaDeviceSynchronize());
  int herr = 0;
  RTE_CUDA(cudaMemcpy(&herr, err.p, 4, cudaMemcpyDeviceToHost));
  if (herr) return fail(RTE_ETIMEOUT, "a GEMM pipeline wait ran out");
  std::vector<float> g1(wn[0]);
  RTE_CUDA(cudaMemcpy(g1.data(), gw[0].p, wn[0] * 4, cudaMemcpyDeviceToHost));
  for (int r = 0; r < H; ++r)
    for (int c = 0; c < d; ++c) gW1[(int64_t)r * d + c] = g1[(int64_t)r * dp + c];
  RTE_CUDA(cudaMemcpy(gW2, gw[1].p, wn[1] * 4, cudaMemcpyDeviceToHost));
  RTE_CUDA(cudaMemcpy(gW3, gw[2].p, (size_t)classes * H * 4, cudaMemcpyDeviceToHost));
  RTE_CUDA(cudaMemcpy(gb1, gb[0].p, bn[0] * 4, cudaMemcpyDeviceToHost));
  RTE_CUDA(cudaMemcpy(gb2, gb[1].p, bn[1] * 4, cudaMemcpyDeviceToHost));
  RTE_CUDA(cudaMemcpy(gb3, gb[2].p, (size_t)classes * 4, cudaMemcpyDeviceToHost));
  if (loss) RTE_CUDA(cudaMemcpy(loss, sb.loss.p, (size_t)M * 4, cudaMemcpyDeviceToHost));
  return RTE_OK;
}
