// kdtree_ref.cpp -- ORACLE (test infrastructure, never the product).
//
// Restates the reference's entry-selection build and point location:
//   kd-tree build      kdtree.cpp:4-196 (Kdtree::Kdtree, buildWithStack,
//                      findWidest, findxM, split, tight_box, add_aabb)
//   leaf -> point ids  kdtree.cpp:91-101 (computeAabbPid)
//   box expansion      aabb.cu:27-38 (expandAabb)
//   point location     devicePrograms.cu:29-96 (zero-length ray over the
//                      leaf boxes).  OptiX reports an arbitrary containing
//                      box; canonical rule H1 fixes it to the smallest leaf
//                      index whose expanded box contains the point, faces
//                      inclusive, and leaf 0 on a miss (hits are zero-filled,
//                      entry.cu:88-89).
// Built with -ffp-contract=off: the reference's host code runs on x86-64
// without FMA contraction.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Builder {
  std::vector<float> x;  // [n][3], permuted in place by split()
  std::vector<int> id;
  std::vector<int> belong;
  std::vector<float> boxes;  // [leaf][6]
  int max_node;
  bool failed = false;

  void tight_box(int l, int r, float* mn, float* mx) {  // kdtree.cpp:127-138
    for (int i = 0; i < 3; i++) mn[i] = mx[i] = x[3 * l + i];
    for (int i = l + 1; i < r; i++)
      for (int j = 0; j < 3; j++) {
        mn[j] = std::min(mn[j], x[3 * i + j]);
        mx[j] = std::max(mx[j], x[3 * i + j]);
      }
  }

  static int widest(const float* mn, const float* mx) {  // kdtree.cpp:30-42
    float max_width = 0;
    int axis = 0;
    for (int dim = 0; dim < 3; dim++)
      if (mx[dim] - mn[dim] > max_width) {
        max_width = mx[dim] - mn[dim];
        axis = dim;
      }
    return axis;
  }

  // Bisection towards the median (kdtree.cpp:103-125).  (l+r)/2.0 is a float
  // sum halved exactly, rounded back to float.
  float find_xm(float l, float r, int dl, int dr, int axis) {
    float xm = (float)((double)(l + r) / 2.0);
    float mid;
    int n = dr - dl;
    float eps = std::max((r - l) / 1000, 0.00001f);
    while (r - l > eps) {
      mid = (float)((double)(r + l) / 2.0);
      int cnt = 0;
      for (int i = dl; i < dr; i++)
        if (x[3 * i + axis] <= mid) cnt++;
      if (cnt <= n / 2) {
        l = mid;
        xm = mid;
        if (cnt == n / 2) break;
      } else {
        r = mid;
      }
    }
    return xm;
  }

  int split(int l, int r, int axis, float xm) {  // kdtree.cpp:44-62
    r = r - 1;
    while (l < r) {
      if (x[3 * l + axis] >= xm) {
        while (x[3 * r + axis] >= xm && l < r) r--;
        if (l < r) {
          for (int i = 0; i < 3; i++) std::swap(x[3 * l + i], x[3 * r + i]);
          std::swap(id[l], id[r]);
          r--;
        } else {
          break;
        }
      }
      l++;
    }
    if (x[3 * l + axis] < xm) l++;
    return l;
  }

  // buildWithStack (kdtree.cpp:140-196): the left child is pushed last, so the
  // traversal is pre-order, left first; leaves are numbered in that order.
  void build(int l, int r) {
    if (failed || l >= r) return;
    float mn[3], mx[3];
    tight_box(l, r, mn, mx);
    if (r - l <= max_node) {  // add_aabb, kdtree.cpp:64-70
      int leaf = (int)(boxes.size() / 6);
      for (int i = l; i < r; i++) belong[id[i]] = leaf;
      for (int j = 0; j < 3; j++) boxes.push_back(mn[j]);
      for (int j = 0; j < 3; j++) boxes.push_back(mx[j]);
      return;
    }
    int axis = widest(mn, mx);
    float xm = find_xm(mn[axis], mx[axis], l, r, axis);
    int median = split(l, r, axis, xm);
    if (median == l || median == r) {  // kdtree.cpp:182-185 exits the process
      failed = true;
      return;
    }
    build(l, median);
    build(median, r);
  }
};

}  // namespace

extern "C" int orc_kdtree_build(const float* pts3, int64_t np, int leaf_cap, int64_t max_leaves,
                                float* out_boxes, int32_t* out_pids, int64_t* n_leaves) {
  if (!pts3 || np <= 0 || np >= (int64_t)INT32_MAX || leaf_cap <= 0 || !n_leaves) return -1;
  Builder b;
  b.x.assign(pts3, pts3 + 3 * np);
  b.id.resize(np);
  for (int64_t i = 0; i < np; i++) b.id[i] = (int)i;
  b.belong.assign(np, -1);
  b.max_node = leaf_cap;
  b.build(0, (int)np);
  if (b.failed) return -2;
  int64_t nl = (int64_t)(b.boxes.size() / 6);
  *n_leaves = nl;
  if (nl > max_leaves) return -3;
  if (out_boxes) std::copy(b.boxes.begin(), b.boxes.end(), out_boxes);
  if (out_pids) {  // computeAabbPid: ascending point id inside each leaf
    std::fill(out_pids, out_pids + nl * leaf_cap, (int32_t)np);
    std::vector<int> count(nl, 0);
    for (int64_t i = 0; i < np; i++) {
      int leaf = b.belong[i];
      out_pids[(int64_t)leaf * leaf_cap + count[leaf]] = (int32_t)i;
      count[leaf]++;
    }
  }
  return 0;
}

extern "C" void orc_expand_boxes(float* boxes, int64_t n, float expand_ratio) {
  for (int64_t i = 0; i < n; i++) {
    float* mn = boxes + 6 * i;
    float* mx = mn + 3;
    for (int j = 0; j < 3; j++) {
      float width = mx[j] - mn[j];
      mn[j] -= width * expand_ratio;
      mx[j] += width * expand_ratio;
    }
  }
}

extern "C" void orc_locate(const float* boxes, int64_t n_leaves, const float* qp, int64_t nq,
                           int stride, int32_t* out_leaf, int n_threads) {
#ifdef _OPENMP
  if (n_threads <= 0) n_threads = omp_get_num_procs();
#pragma omp parallel for schedule(static) num_threads(n_threads)
#endif
  for (int64_t q = 0; q < nq; q++) {
    const float* p = qp + q * stride;
    int32_t hit = 0;
    for (int64_t i = 0; i < n_leaves; i++) {
      const float* b = boxes + 6 * i;
      if (b[0] <= p[0] && p[0] <= b[3] && b[1] <= p[1] && p[1] <= b[4] && b[2] <= p[2] &&
          p[2] <= b[5]) {
        hit = (int32_t)i;
        break;
      }
    }
    out_leaf[q] = hit;
  }
  (void)n_threads;
}

// The first H containing leaves in index order (rule H1 extended to the
// reference's max_hits > 1); -1 where fewer contain the point; a point in no
// leaf gets leaf 0 first, as with one leaf.
extern "C" void orc_locate_multi(const float* boxes, int64_t n_leaves, const float* qp, int64_t nq,
                                 int stride, int H, int32_t* out_leaves, int n_threads) {
#ifdef _OPENMP
  if (n_threads <= 0) n_threads = omp_get_num_procs();
#pragma omp parallel for schedule(static) num_threads(n_threads)
#endif
  for (int64_t q = 0; q < nq; q++) {
    const float* p = qp + q * stride;
    int found = 0;
    for (int64_t i = 0; i < n_leaves && found < H; i++) {
      const float* b = boxes + 6 * i;
      if (b[0] <= p[0] && p[0] <= b[3] && b[1] <= p[1] && p[1] <= b[4] && b[2] <= p[2] &&
          p[2] <= b[5])
        out_leaves[q * H + found++] = (int32_t)i;
    }
    if (found == 0) out_leaves[q * H + found++] = 0;  // a miss enters at leaf 0 (H1)
    for (; found < H; ++found) out_leaves[q * H + found] = -1;
  }
  (void)n_threads;
}

extern "C" void orc_knn_fp64(const float* base, int64_t np, int d, const float* queries,
                             int64_t nq, int k, int32_t* out_ids, double* out_d2, int n_threads) {
#ifdef _OPENMP
  if (n_threads <= 0) n_threads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads)
#endif
  for (int64_t q = 0; q < nq; q++) {
    std::vector<std::pair<double, int>> all(np);
    const float* qv = queries + q * d;
    for (int64_t i = 0; i < np; i++) {
      const float* p = base + i * d;
      double s = 0;
      for (int j = 0; j < d; j++) {
        double t = (double)p[j] - (double)qv[j];
        s += t * t;
      }
      all[i] = {s, (int)i};
    }
    int kk = (int)std::min<int64_t>(k, np);
    std::partial_sort(all.begin(), all.begin() + kk, all.end());
    for (int j = 0; j < kk; j++) {
      out_ids[q * k + j] = all[j].second;
      if (out_d2) out_d2[q * k + j] = all[j].first;
    }
  }
  (void)n_threads;
}
