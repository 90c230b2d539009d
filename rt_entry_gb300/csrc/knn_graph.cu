// knn_graph.cu -- exact k-nearest-neighbour graph of a base, on the GPU.
//
// The reference loads its proximity graph from a file and has no builder
// (graph.cu:120).  This builds the degree-R exact kNN graph that its search
// runs on: row i lists the R nearest rows j != i by exact squared L2
// distance (FP64), in (distance, id) order.
//
//   0. The rows are centred on their column mean mu (FP64 sums in a fixed
//      order, rounded to FP32): c = fl(x - mu).  Distances do not change
//      under a shift, and the error bound of step 3 scales with the norms of
//      what the GEMM multiplies, so centring tightens it by |x| / |c| (about
//      5x for values in [0, 1] around 0.5).
//   1. Each centred row c is split into BF16 c_hi = bf16(c) and
//      c_lo = bf16(c - c_hi);
//      A = [hi | hi | lo] and B = [hi | lo | hi] along K, so one tensor-core
//      GEMM (gemm_tc.cu, K = 3*dp) gives hi.hi + hi.lo + lo.hi, the dot
//      product to about 2^-16 relative.
//   2. Block of rows by block of rows: approximate distances
//      |x|^2 + |y|^2 - 2 x.y for all n columns, the K = 2R + 32 smallest per
//      row (select_rows), and a lower bound on every column left out.
//   3. Exact FP64 distances of the K candidates, sorted by (distance, id),
//      self excluded (rerank_rows).  The row is certified exact when its R-th
//      distance is below the left-out bound minus the approximation's error
//      bound; rows that fail are redone with 1024 candidates selected from
//      the same block of dot products (still in memory), and a row that
//      fails again is an error.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <vector>

#include "gemm_tc.h"
#include "index_impl.h"
#include "rtentry.h"

namespace rte {
namespace {

constexpr int kSelThreads = 256;
constexpr int kSelT = 16;                         // candidates kept per thread
constexpr int kSelPool = kSelThreads * kSelT;     // 4096 merged per row
constexpr int kMaxCand = 1024;                    // the retry's candidate count

constexpr int kMeanSlices = 256;  // row slices of the column mean's first pass

// Column sums of row slice blockIdx.y in FP64 (rows in order), one thread
// per column: part[slice][c].
__global__ void col_sum_slices(const float* __restrict__ x, int64_t n, int d, double* __restrict__ part) {
  const int s = blockIdx.y;
  const int64_t r0 = n * s / kMeanSlices, r1 = n * (s + 1) / kMeanSlices;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < d; c += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int64_t r = r0; r < r1; ++r) acc += (double)__ldg(x + r * d + c);
    part[(int64_t)s * d + c] = acc;
  }
}

// mu[c] = (sum of the slices' sums in slice order) / n, rounded to FP32.
__global__ void col_mean_finish(const double* __restrict__ part, int64_t n, int d, float* __restrict__ mu) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d) return;
  double acc = 0.0;
  for (int s = 0; s < kMeanSlices; ++s) acc += part[(int64_t)s * d + c];
  mu[c] = (float)(acc / (double)n);
}

// Centring, split and norms of the centred rows: one warp per row.
__global__ void split_rows(const float* __restrict__ x, const float* __restrict__ mu, int64_t n, int d,
                           int dp, __nv_bfloat16* __restrict__ a, __nv_bfloat16* __restrict__ b,
                           float* __restrict__ nrm32, double* __restrict__ nrm64) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t ld = 3 * (int64_t)dp;
  for (int64_t r = warp; r < n; r += nwarps) {
    double s = 0.0;
    for (int c = lane; c < dp; c += 32) {
      const float v = c < d ? __fsub_rn(x[r * d + c], mu[c]) : 0.0f;
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      const __nv_bfloat16 lo = __float2bfloat16_rn(__fsub_rn(v, __bfloat162float(hi)));
      a[r * ld + c] = hi;           // A = [hi | hi | lo]
      a[r * ld + dp + c] = hi;
      a[r * ld + 2 * dp + c] = lo;
      b[r * ld + c] = hi;           // B = [hi | lo | hi]
      b[r * ld + dp + c] = lo;
      b[r * ld + 2 * dp + c] = hi;
      s += (double)v * (double)v;
    }
    for (int off = 16; off >= 1; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) {
      nrm64[r] = s;
      nrm32[r] = (float)s;
    }
  }
}

__device__ __forceinline__ bool key_less(float da, int ia, float db, int ib) {
  return da < db || (da == db && ia < ib);
}

// In-place ascending bitonic sort of kSelPool (distance, id) pairs in shared
// memory by all threads of the block.
__device__ void block_sort(float* sd, int* si) {
  for (int step = 2; step <= kSelPool; step <<= 1)
    for (int sub = step >> 1; sub >= 1; sub >>= 1) {
      for (int i = threadIdx.x; i < kSelPool; i += blockDim.x) {
        const int j = i ^ sub;
        if (j > i) {
          const bool up = (i & step) == 0;
          const bool sw = up ? key_less(sd[j], si[j], sd[i], si[i]) : key_less(sd[i], si[i], sd[j], si[j]);
          if (sw) {
            const float t = sd[i];
            sd[i] = sd[j];
            sd[j] = t;
            const int u = si[i];
            si[i] = si[j];
            si[j] = u;
          }
        }
      }
      __syncthreads();
    }
}

// One block per row: approximate distances from the dot products in
// D[row][0..n), the K smallest by (distance, id), and the smallest
// approximate distance any left-out column can have.
// With `local`, block i serves row local[i] of the block of dot products.
__global__ void __launch_bounds__(kSelThreads) select_rows(const float* __restrict__ D, int64_t ld,
                                                           int64_t r0, int64_t n,
                                                           const float* __restrict__ nrm32, int K,
                                                           const int32_t* __restrict__ local,
                                                           int32_t* __restrict__ cand,
                                                           float* __restrict__ excl) {
  __shared__ float sd[kSelPool];
  __shared__ int si[kSelPool];
  __shared__ float sdrop[kSelThreads];
  const int r = local ? local[blockIdx.x] : (int)blockIdx.x;
  const float qn = nrm32[r0 + r];
  float kd[kSelT];
  int ki[kSelT];
#pragma unroll
  for (int s = 0; s < kSelT; ++s) {
    kd[s] = INFINITY;
    ki[s] = INT32_MAX;
  }
  const float* row = D + (int64_t)r * ld;
  for (int64_t j = threadIdx.x; j < n; j += kSelThreads) {
    const float a = __fmaf_rn(-2.0f, __ldg(row + j), __fadd_rn(qn, __ldg(nrm32 + j)));
    if (a < kd[kSelT - 1]) {  // insert, keeping the list sorted (ties keep scan order)
      float cd = a;
      int ci = (int)j;
#pragma unroll
      for (int s = 0; s < kSelT; ++s)
        if (cd < kd[s]) {
          const float t = kd[s];
          kd[s] = cd;
          cd = t;
          const int u = ki[s];
          ki[s] = ci;
          ci = u;
        }
    }
  }
  // what this thread dropped is no smaller than its last kept value (when full)
  sdrop[threadIdx.x] = ki[kSelT - 1] != INT32_MAX ? kd[kSelT - 1] : INFINITY;
#pragma unroll
  for (int s = 0; s < kSelT; ++s) {
    sd[threadIdx.x * kSelT + s] = kd[s];
    si[threadIdx.x * kSelT + s] = ki[s];
  }
  __syncthreads();
  block_sort(sd, si);
  const int64_t o = blockIdx.x;
  for (int k = threadIdx.x; k < K; k += kSelThreads) cand[o * K + k] = si[k] < n ? si[k] : -1;
  if (threadIdx.x == 0) {
    float m = K < kSelPool ? sd[K] : INFINITY;
    for (int t = 0; t < kSelThreads; ++t) m = fminf(m, sdrop[t]);
    excl[o] = m;
  }
}

__device__ __forceinline__ bool key_less64(double da, int ia, double db, int ib) {
  return da < db || (da == db && ia < ib);
}

// One block per row: exact FP64 distances of the candidates, sorted by
// (distance, id) with the row itself excluded; certified when the R-th
// distance is below the left-out bound minus the error bound.
__global__ void __launch_bounds__(256) rerank_rows(const float* __restrict__ x, int d, const int64_t* __restrict__ rows,
                                                   const int32_t* __restrict__ cand, int K, int Kp,
                                                   const float* __restrict__ excl,
                                                   const double* __restrict__ nrm64, double max_norm,
                                                   int R, int32_t* __restrict__ out,
                                                   int* __restrict__ failed) {
  extern __shared__ unsigned char sm_raw[];
  double* sd = reinterpret_cast<double*>(sm_raw);
  int* si = reinterpret_cast<int*>(sd + Kp);
  const int r = blockIdx.x;
  const int64_t gi = rows[r];
  const float* q = x + gi * d;
  for (int k = threadIdx.x; k < Kp; k += blockDim.x) {
    const int id = k < K ? cand[(int64_t)r * K + k] : -1;
    double s = INFINITY;
    if (id >= 0 && id != gi) {
      const float* p = x + (int64_t)id * d;
      s = 0.0;
      for (int c = 0; c < d; ++c) {
        const double t = (double)__ldg(p + c) - (double)__ldg(q + c);
        s = fma(t, t, s);
      }
    }
    sd[k] = s;
    si[k] = id >= 0 && id != gi ? id : INT32_MAX;
  }
  __syncthreads();
  for (int step = 2; step <= Kp; step <<= 1)
    for (int sub = step >> 1; sub >= 1; sub >>= 1) {
      for (int i = threadIdx.x; i < Kp; i += blockDim.x) {
        const int j = i ^ sub;
        if (j > i) {
          const bool up = (i & step) == 0;
          const bool sw = up ? key_less64(sd[j], si[j], sd[i], si[i]) : key_less64(sd[i], si[i], sd[j], si[j]);
          if (sw) {
            const double t = sd[i];
            sd[i] = sd[j];
            sd[j] = t;
            const int u = si[i];
            si[i] = si[j];
            si[j] = u;
          }
        }
      }
      __syncthreads();
    }
  // |approximate - exact| <= err for every column: the hi/lo split and the
  // FP32 sums over the centred rows (norms qnorm, at most max_norm), plus
  // the centring's rounding -- each fl(x - mu) is off by at most 2^-24 of
  // |x - mu|, which moves a squared distance by at most about
  // 2^-23 (qnorm + max_norm)^2; the last term doubles that for room
  const double qnorm = sqrt(nrm64[gi]);
  const double err = (ldexp(1.0, -14) + d * ldexp(1.0, -21)) * qnorm * max_norm +
                     ldexp(1.0, -20) * (nrm64[gi] + max_norm * max_norm) +
                     ldexp(1.0, -22) * (qnorm + max_norm) * (qnorm + max_norm);
  if (threadIdx.x == 0) {
    const bool ok = si[R - 1] != INT32_MAX && sd[R - 1] < (double)excl[r] - err;
    if (!ok) atomicAdd(failed, 1);
    out[gi * R] = ok ? si[0] : -1;  // -1 marks the row for the retry
  }
  __syncthreads();
  if (out[gi * R] >= 0)
    for (int k = threadIdx.x + 1; k < R; k += blockDim.x) out[gi * R + k] = si[k];
}

struct Buf {
  void* p = nullptr;
  ~Buf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes); }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

}  // namespace
}  // namespace rte

using namespace rte;

extern "C" rte_status rte_knn_graph(const float* base, int64_t n, int d, int degree, int device,
                                    int32_t* graph, void* stream) {
  clear_error();
  if (!base || !graph || n <= 0 || d <= 0) return fail(RTE_EINVAL, "bad kNN graph arguments");
  if (degree <= 0 || degree > 256 || n <= degree) return fail(RTE_EINVAL, "degree must be in [1, min(256, n - 1)]");
  if (n >= INT32_MAX) return fail(RTE_EINVAL, "n must be below 2^31");
  DeviceGuard guard(device);
  cudaStream_t st = (cudaStream_t)stream;
  const int dp = (d + 7) & ~7;
  const int K = std::min<int64_t>(std::min(2 * degree + 32, kSelPool), n);
  // rows per block: the FP32 dot-product block stays under 8 GB
  int64_t mb = std::max<int64_t>(128, std::min<int64_t>(8192, (int64_t)(8ll << 30) / (n * 4)));
  mb = std::min<int64_t>(mb, n);
  Buf xd, A, B, n32, n64, D, cand, excl, rows, fl, outd, part, mu, loc;
  const bool base_dev = is_device_ptr(base), graph_dev = is_device_ptr(graph);
  const float* x = base;
  if (!base_dev) {
    RTE_CUDA(xd.alloc((size_t)n * d * 4));
    RTE_CUDA(cudaMemcpyAsync(xd.p, base, (size_t)n * d * 4, cudaMemcpyHostToDevice, st));
    x = xd.as<float>();
  }
  RTE_CUDA(A.alloc((size_t)n * 3 * dp * 2));
  RTE_CUDA(B.alloc((size_t)n * 3 * dp * 2));
  RTE_CUDA(n32.alloc((size_t)n * 4));
  RTE_CUDA(n64.alloc((size_t)n * 8));
  RTE_CUDA(D.alloc((size_t)mb * n * 4));
  RTE_CUDA(cand.alloc((size_t)mb * kMaxCand * 4));
  RTE_CUDA(excl.alloc((size_t)mb * 4));
  RTE_CUDA(rows.alloc((size_t)mb * 8));
  RTE_CUDA(fl.alloc(4));
  int32_t* g = graph;
  if (!graph_dev) {
    RTE_CUDA(outd.alloc((size_t)n * degree * 4));
    g = outd.as<int32_t>();
  }
  RTE_CUDA(part.alloc((size_t)kMeanSlices * d * 8));
  RTE_CUDA(mu.alloc((size_t)d * 4));
  RTE_CUDA(loc.alloc((size_t)mb * 4));
  col_sum_slices<<<dim3((unsigned)((d + 127) / 128), kMeanSlices), 128, 0, st>>>(x, n, d, part.as<double>());
  col_mean_finish<<<(unsigned)((d + 127) / 128), 128, 0, st>>>(part.as<double>(), n, d, mu.as<float>());
  split_rows<<<(unsigned)std::min<int64_t>((n + 7) / 8, 65535), 256, 0, st>>>(
      x, mu.as<float>(), n, d, dp, A.as<__nv_bfloat16>(), B.as<__nv_bfloat16>(), n32.as<float>(),
      n64.as<double>());
  RTE_CUDA(cudaGetLastError());
  std::vector<double> hn(n);
  RTE_CUDA(cudaMemcpyAsync(hn.data(), n64.p, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
  RTE_CUDA(cudaStreamSynchronize(st));
  double max_norm = 0.0;
  for (double v : hn) max_norm = std::max(max_norm, std::sqrt(v));
  Buf errb;
  RTE_CUDA(errb.alloc(4));
  int* err = errb.as<int>();
  RTE_CUDA(cudaMemsetAsync(err, 0, 4, st));
  std::vector<int64_t> hrows(mb), rrows;
  std::vector<int32_t> hfirst(mb), rlocal;
  const int Kp = 1 << (int)std::ceil(std::log2((double)std::max(K, 2)));
  const int K2 = (int)std::min<int64_t>(kMaxCand, n);
  int64_t n_retried = 0;
  for (int64_t r0 = 0; r0 < n; r0 += mb) {
    const int64_t m = std::min(mb, n - r0);
    GemmArgs ga{};
    ga.A = A.as<__nv_bfloat16>() + r0 * 3 * dp;
    ga.B = B.p;
    ga.M = (int)m;
    ga.N = (int)n;
    ga.K = 3 * dp;
    ga.epilogue = kEpiStoreF32;
    ga.C = D.p;
    ga.ldc = (int)n;
    ga.err = err;
    RTE_CUDA(gemm_bf16_tn(ga, st));
    select_rows<<<(unsigned)m, kSelThreads, 0, st>>>(D.as<float>(), n, r0, n, n32.as<float>(), K, nullptr,
                                                       cand.as<int32_t>(), excl.as<float>());
    RTE_CUDA(cudaGetLastError());
    for (int64_t i = 0; i < m; ++i) hrows[i] = r0 + i;
    RTE_CUDA(cudaMemcpyAsync(rows.p, hrows.data(), m * 8, cudaMemcpyHostToDevice, st));
    RTE_CUDA(cudaMemsetAsync(fl.p, 0, 4, st));
    const size_t smem = (size_t)Kp * 12;
    rerank_rows<<<(unsigned)m, 256, smem, st>>>(x, d, rows.as<int64_t>(), cand.as<int32_t>(), K, Kp,
                                                 excl.as<float>(), n64.as<double>(), max_norm, degree,
                                                 g, fl.as<int>());
    RTE_CUDA(cudaGetLastError());
    int nfail = 0;
    RTE_CUDA(cudaMemcpyAsync(&nfail, fl.p, 4, cudaMemcpyDeviceToHost, st));
    RTE_CUDA(cudaStreamSynchronize(st));
    if (!nfail) continue;
    // rows not certified (first entry -1): K2 candidates from the same
    // block of dot products, which the next block's GEMM has not yet
    // overwritten (same stream)
    RTE_CUDA(cudaMemcpy2DAsync(hfirst.data(), 4, g + r0 * degree, (size_t)degree * 4, 4, (size_t)m,
                               cudaMemcpyDeviceToHost, st));
    RTE_CUDA(cudaStreamSynchronize(st));
    rrows.clear();
    rlocal.clear();
    for (int64_t i = 0; i < m; ++i)
      if (hfirst[i] < 0) {
        rrows.push_back(r0 + i);
        rlocal.push_back((int32_t)i);
      }
    const int64_t mr = (int64_t)rrows.size();
    n_retried += mr;
    RTE_CUDA(cudaMemcpyAsync(loc.p, rlocal.data(), mr * 4, cudaMemcpyHostToDevice, st));
    RTE_CUDA(cudaMemcpyAsync(rows.p, rrows.data(), mr * 8, cudaMemcpyHostToDevice, st));
    select_rows<<<(unsigned)mr, kSelThreads, 0, st>>>(D.as<float>(), n, r0, n, n32.as<float>(), K2,
                                                        loc.as<int32_t>(), cand.as<int32_t>(),
                                                        excl.as<float>());
    RTE_CUDA(cudaGetLastError());
    RTE_CUDA(cudaMemsetAsync(fl.p, 0, 4, st));
    rerank_rows<<<(unsigned)mr, 256, (size_t)kMaxCand * 12, st>>>(
        x, d, rows.as<int64_t>(), cand.as<int32_t>(), K2, kMaxCand, excl.as<float>(), n64.as<double>(),
        max_norm, degree, g, fl.as<int>());
    RTE_CUDA(cudaGetLastError());
    RTE_CUDA(cudaMemcpyAsync(&nfail, fl.p, 4, cudaMemcpyDeviceToHost, st));
    RTE_CUDA(cudaStreamSynchronize(st));
    if (nfail) return fail(RTE_EIO, "kNN graph: " + std::to_string(nfail) + " rows could not be certified exact");
  }
  if (getenv("RTE_KNN_VERBOSE"))
    fprintf(stderr, "rte_knn_graph: n %lld d %d degree %d: %lld rows retried with %d candidates\n",
            (long long)n, d, degree, (long long)n_retried, K2);
  int herr = 0;
  RTE_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
  if (!graph_dev) RTE_CUDA(cudaMemcpyAsync(graph, g, (size_t)n * degree * 4, cudaMemcpyDeviceToHost, st));
  RTE_CUDA(cudaStreamSynchronize(st));
  if (herr) return fail(RTE_ETIMEOUT, "GEMM pipeline wait ran out (code " + std::to_string(herr) + ")");
  return RTE_OK;
}
