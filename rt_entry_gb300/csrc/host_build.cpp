// host_build.cpp -- kd-tree build, leaf expansion and the FP64 eigensolver.
//
// Compiled with -ffp-contract=off so that every float operation rounds as in
// the reference's x86-64 host build (no FMA contraction there), which makes
// split values, tight boxes and expanded boxes bit-identical.
#include "host_build.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace rte {

namespace {

struct Pts {
  std::vector<float> c[3];  // coordinates, permuted by the partition
  std::vector<int32_t> id;
};

// count of coordinate <= v on axis over [l, r); parallel for large ranges
// (integer counts, so the result does not depend on the split of work)
int64_t count_le(const Pts& p, int axis, int64_t l, int64_t r, float v) {
  const float* x = p.c[axis].data();
  int64_t cnt = 0;
  if (r - l >= (1 << 20)) {
#pragma omp parallel for reduction(+ : cnt) schedule(static)
    for (int64_t i = l; i < r; ++i) cnt += x[i] <= v;
  } else {
    for (int64_t i = l; i < r; ++i) cnt += x[i] <= v;
  }
  return cnt;
}

void tight_box(const Pts& p, int64_t l, int64_t r, float* mn, float* mx) {
  for (int a = 0; a < 3; ++a) {
    const float* x = p.c[a].data();
    float lo = x[l], hi = x[l];
    for (int64_t i = l + 1; i < r; ++i) {
      lo = std::min(lo, x[i]);
      hi = std::max(hi, x[i]);
    }
    mn[a] = lo;
    mx[a] = hi;
  }
}

// Split value: bisection of [lo, hi] until the count of coordinates <= mid
// is exactly half (integer division) or the interval is below
// max((hi-lo)/1000, 1e-5); the last mid whose count did not exceed half.
float split_value(const Pts& p, int axis, int64_t l, int64_t r, float lo, float hi) {
  float xm = (float)((double)(lo + hi) / 2.0);
  const int64_t half = (r - l) / 2;
  const float eps = std::max((hi - lo) / 1000, 0.00001f);
  while (hi - lo > eps) {
    const float mid = (float)((double)(hi + lo) / 2.0);
    const int64_t cnt = count_le(p, axis, l, r, mid);
    if (cnt <= half) {
      lo = mid;
      xm = mid;
      if (cnt == half) break;
    } else {
      hi = mid;
    }
  }
  return xm;
}

void swap_pts(Pts& p, int64_t a, int64_t b) {
  for (int k = 0; k < 3; ++k) std::swap(p.c[k][a], p.c[k][b]);
  std::swap(p.id[a], p.id[b]);
}

// Two-pointer partition: values >= xm move to the back.  Returns the first
// index of the right part.
int64_t partition(Pts& p, int axis, int64_t l, int64_t r, float xm) {
  const float* x = p.c[axis].data();
  int64_t i = l, j = r - 1;
  while (i < j) {
    if (x[i] >= xm) {
      while (x[j] >= xm && i < j) --j;
      if (i < j) {
        swap_pts(p, i, j);
        --j;
      } else {
        break;
      }
    }
    ++i;
  }
  if (x[i] < xm) ++i;
  return i;
}

struct Frame {
  int64_t l, r;
  int node;
  int depth;
};

}  // namespace

bool kd_build(const float* xyz, int64_t n, int cap, KdTree& out, std::string& err) {
  if (n <= 0 || cap <= 0) {
    err = "kd-tree needs n > 0 and leaf size > 0";
    return false;
  }
  Pts p;
  for (int a = 0; a < 3; ++a) p.c[a].resize(n);
  p.id.resize(n);
  for (int64_t i = 0; i < n; ++i) {
    for (int a = 0; a < 3; ++a) p.c[a][i] = xyz[3 * i + a];
    p.id[i] = (int32_t)i;
  }
  std::vector<int32_t> leaf_of(n, -1);
  out = KdTree();
  out.cap = cap;
  out.nodes.clear();
  out.nodes.push_back(BvhNode{});
  // explicit stack, right pushed before left: pre-order, left first
  std::vector<Frame> stack;
  stack.push_back({0, n, 0, 0});
  while (!stack.empty()) {
    Frame f = stack.back();
    stack.pop_back();
    out.depth = std::max(out.depth, f.depth);
    float mn[3], mx[3];
    tight_box(p, f.l, f.r, mn, mx);
    if (f.r - f.l <= cap) {
      const int32_t leaf = (int32_t)out.n_leaves++;
      for (int64_t i = f.l; i < f.r; ++i) leaf_of[p.id[i]] = leaf;
      for (int a = 0; a < 3; ++a) out.tight.push_back(mn[a]);
      for (int a = 0; a < 3; ++a) out.tight.push_back(mx[a]);
      out.nodes[f.node].left = -leaf - 1;
      out.nodes[f.node].right = -1;
      continue;
    }
    int axis = 0;
    float width = 0;
    for (int a = 0; a < 3; ++a)
      if (mx[a] - mn[a] > width) {
        width = mx[a] - mn[a];
        axis = a;
      }
    const float xm = split_value(p, axis, f.l, f.r, mn[axis], mx[axis]);
    const int64_t mid = partition(p, axis, f.l, f.r, xm);
    if (mid == f.l || mid == f.r) {
      err = "kd-tree split failed: a node's points cannot be separated (duplicate points?)";
      return false;
    }
    const int left = (int)out.nodes.size();
    out.nodes.push_back(BvhNode{});
    const int right = (int)out.nodes.size();
    out.nodes.push_back(BvhNode{});
    out.nodes[f.node].left = left;
    out.nodes[f.node].right = right;
    stack.push_back({mid, f.r, right, f.depth + 1});
    stack.push_back({f.l, mid, left, f.depth + 1});
  }
  // renumber the nodes breadth-first (structure and leaf ids unchanged), so
  // that the top levels of the tree are the first nodes of the array
  {
    std::vector<int> order;
    order.reserve(out.nodes.size());
    order.push_back(0);
    for (size_t h = 0; h < order.size(); ++h) {
      const BvhNode& nd = out.nodes[order[h]];
      if (nd.left >= 0) {
        order.push_back(nd.left);
        order.push_back(nd.right);
      }
    }
    std::vector<int> renum(out.nodes.size());
    for (size_t i = 0; i < order.size(); ++i) renum[order[i]] = (int)i;
    std::vector<BvhNode> bfs(order.size());
    for (size_t i = 0; i < order.size(); ++i) {
      bfs[i] = out.nodes[order[i]];
      if (bfs[i].left >= 0) {
        bfs[i].left = renum[bfs[i].left];
        bfs[i].right = renum[bfs[i].right];
      }
    }
    out.nodes.swap(bfs);
  }
  const int64_t nl = out.n_leaves;
  out.pids.assign(nl * cap, (int32_t)n);
  std::vector<int32_t> fill(nl, 0);
  for (int64_t i = 0; i < n; ++i) {
    const int32_t leaf = leaf_of[i];
    out.pids[(int64_t)leaf * cap + fill[leaf]++] = (int32_t)i;
  }
  return true;
}

void kd_wide(const KdTree& t, std::vector<WideNode>& out, std::vector<int32_t>* wide_of) {
  out.clear();
  std::vector<int> start{0};  // binary node that each wide node expands, breadth-first
  std::vector<int> kids;
  for (size_t h = 0; h < start.size(); ++h) {
    const int b = start[h];
    kids.clear();
    if (t.nodes[b].left < 0) {
      kids.push_back(b);  // a tree that is one leaf
    } else {
      // pre-order, left first: descendants 3 levels down, or leaves met before
      std::vector<std::pair<int, int>> st{{t.nodes[b].right, 1}, {t.nodes[b].left, 1}};
      while (!st.empty()) {
        auto [k, rel] = st.back();
        st.pop_back();
        const BvhNode& nd = t.nodes[k];
        if (nd.left < 0 || rel == 3) {
          kids.push_back(k);
        } else {
          st.push_back({nd.right, rel + 1});
          st.push_back({nd.left, rel + 1});
        }
      }
    }
    WideNode w;
    for (int c = 0; c < kWide; ++c) {
      for (int a = 0; a < 3; ++a) {
        w.lo[a][c] = 3.402823466e38f;
        w.hi[a][c] = -3.402823466e38f;
      }
      w.child[c] = 0;
      w.pad[c] = 0;
    }
    for (size_t c = 0; c < kids.size(); ++c) {
      const BvhNode& nd = t.nodes[kids[c]];
      for (int a = 0; a < 3; ++a) {
        w.lo[a][c] = nd.lo[a];
        w.hi[a][c] = nd.hi[a];
      }
      if (nd.left < 0) {
        w.child[c] = nd.left;  // -(leaf + 1)
      } else {
        w.child[c] = (int32_t)start.size();
        start.push_back(kids[c]);
      }
    }
    out.push_back(w);
  }
  if (wide_of) {
    wide_of->assign(t.nodes.size(), -1);
    for (size_t i = 0; i < start.size(); ++i) (*wide_of)[start[i]] = (int32_t)i;
  }
}

void kd_expand(KdTree& t, float ratio) {
  t.expanded = t.tight;
  for (int64_t i = 0; i < t.n_leaves; ++i) {
    float* mn = &t.expanded[6 * i];
    float* mx = mn + 3;
    for (int a = 0; a < 3; ++a) {
      const float width = mx[a] - mn[a];
      mn[a] -= width * ratio;
      mx[a] += width * ratio;
    }
  }
  // bounds bottom-up: children always have larger node indices than parents
  // (breadth-first numbering)
  for (int64_t k = (int64_t)t.nodes.size() - 1; k >= 0; --k) {
    BvhNode& nd = t.nodes[k];
    if (nd.left < 0) {
      const float* b = &t.expanded[6 * (int64_t)(-nd.left - 1)];
      for (int a = 0; a < 3; ++a) {
        nd.lo[a] = b[a];
        nd.hi[a] = b[3 + a];
      }
    } else {
      const BvhNode& L = t.nodes[nd.left];
      const BvhNode& R = t.nodes[nd.right];
      for (int a = 0; a < 3; ++a) {
        nd.lo[a] = std::min(L.lo[a], R.lo[a]);
        nd.hi[a] = std::max(L.hi[a], R.hi[a]);
      }
    }
  }
}

// ------------------------------------------------------------ eigensolver --
// Householder reduction of the symmetric matrix to tridiagonal form
// T = Q^T A Q (Q accumulated explicitly), then implicit QL iterations with
// Wilkinson-style shifts on T, applying every plane rotation to Q.
bool sym_eig(const double* a_in, int n, double* w, double* v, std::string& err) {
  if (n <= 0) {
    err = "eigendecomposition of an empty matrix";
    return false;
  }
  std::vector<double> A(a_in, a_in + (size_t)n * n);
  auto Aat = [&](int i, int j) -> double& { return A[(size_t)i * n + j]; };
  std::vector<double> Q((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
  std::vector<double> vh(n), p(n), wv(n);
  // tridiagonalisation: for column k, reflect A[k+1.., k] onto e_{k+1}
  for (int k = 0; k + 2 < n; ++k) {
    double scale = 0.0;
    for (int i = k + 1; i < n; ++i) scale = std::max(scale, std::fabs(Aat(i, k)));
    if (scale == 0.0) continue;
    double norm2 = 0.0;
    for (int i = k + 1; i < n; ++i) {
      vh[i] = Aat(i, k) / scale;
      norm2 += vh[i] * vh[i];
    }
    const double alpha = (vh[k + 1] >= 0 ? -1.0 : 1.0) * std::sqrt(norm2);
    vh[k + 1] -= alpha;
    double vtv = 0.0;
    for (int i = k + 1; i < n; ++i) vtv += vh[i] * vh[i];
    if (vtv == 0.0) continue;
    const double beta = 2.0 / vtv;
    // p = beta * A' v over the trailing block
#pragma omp parallel for schedule(static) if (n > 256)
    for (int i = k; i < n; ++i) {
      double s = 0.0;
      for (int j = k + 1; j < n; ++j) s += Aat(i, j) * vh[j];
      p[i] = beta * s;
    }
    double vp = 0.0;
    for (int i = k + 1; i < n; ++i) vp += vh[i] * p[i];
    const double K = 0.5 * beta * vp;
    for (int i = k + 1; i < n; ++i) wv[i] = p[i] - K * vh[i];
    // A' <- A' - v w^T - w v^T on rows/cols k+1..n-1; column k becomes alpha*scale e_{k+1}
#pragma omp parallel for schedule(static) if (n > 256)
    for (int i = k + 1; i < n; ++i)
      for (int j = k + 1; j < n; ++j) Aat(i, j) -= vh[i] * wv[j] + wv[i] * vh[j];
    for (int i = k + 2; i < n; ++i) Aat(i, k) = Aat(k, i) = 0.0;
    Aat(k + 1, k) = Aat(k, k + 1) = alpha * scale;
    // Q <- Q H, H = I - beta v v^T
#pragma omp parallel for schedule(static) if (n > 256)
    for (int r = 0; r < n; ++r) {
      double s = 0.0;
      for (int j = k + 1; j < n; ++j) s += Q[(size_t)r * n + j] * vh[j];
      s *= beta;
      for (int j = k + 1; j < n; ++j) Q[(size_t)r * n + j] -= s * vh[j];
    }
  }
  std::vector<double> d(n), e(n, 0.0);
  for (int i = 0; i < n; ++i) d[i] = Aat(i, i);
  for (int i = 0; i + 1 < n; ++i) e[i] = Aat(i + 1, i);  // e[i] couples i and i+1

  // implicit QL
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    for (;;) {
      int m = l;
      for (; m + 1 < n; ++m) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= std::numeric_limits<double>::epsilon() * dd) break;
      }
      if (m == l) break;
      if (++iter > 60) {
        err = "eigensolver did not converge";
        return false;
      }
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
      double s = 1.0, c = 1.0, pp = 0.0;
      int i = m - 1;
      bool early = false;
      for (; i >= l; --i) {
        double f = s * e[i];
        const double b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {
          d[i + 1] -= pp;
          e[m] = 0.0;
          early = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - pp;
        r = (d[i] - g) * s + 2.0 * c * b;
        pp = s * r;
        d[i + 1] = g + pp;
        g = c * r - b;
        for (int k = 0; k < n; ++k) {
          double* row = &Q[(size_t)k * n];
          f = row[i + 1];
          row[i + 1] = s * row[i] + c * f;
          row[i] = c * row[i] - s * f;
        }
      }
      if (early) continue;
      d[l] -= pp;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  // sort descending, canonical sign
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return d[x] > d[y]; });
  for (int j = 0; j < n; ++j) {
    const int src = ord[j];
    w[j] = d[src];
    int big = 0;
    for (int i = 1; i < n; ++i)
      if (std::fabs(Q[(size_t)i * n + src]) > std::fabs(Q[(size_t)big * n + src])) big = i;
    const double sg = Q[(size_t)big * n + src] < 0 ? -1.0 : 1.0;
    for (int i = 0; i < n; ++i) v[(size_t)i * n + j] = sg * Q[(size_t)i * n + src];
  }
  return true;
}

}  // namespace rte
