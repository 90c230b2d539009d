// host_build.h -- host-side index build steps (C++, FP64 where it matters).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "index_kernels.h"

namespace rte {

// kd-tree over 3-d points with the reference's splitting rule
// (kdtree.cpp:103-196): widest axis of the node's tight box, split value by
// bisection towards the median count, Hoare-style partition, leaves of at
// most `cap` points numbered in pre-order, left first.
struct KdTree {
  int cap = 0;
  int64_t n_leaves = 0;
  std::vector<float> tight;     // [n_leaves][6] minX,minY,minZ,maxX,maxY,maxZ
  std::vector<float> expanded;  // [n_leaves][6]
  std::vector<int32_t> pids;    // [n_leaves][cap], ascending ids, padded np
  std::vector<BvhNode> nodes;   // node 0 = root; bounds from expanded boxes
  int depth = 0;
};

// The 8-wide copy of the tree for point location (index_kernels.h), built
// from the expanded node bounds (call after kd_expand).
// wide_of (optional): for every binary node that starts a wide node, that
// wide node's index; -1 elsewhere.
void kd_wide(const KdTree& t, std::vector<WideNode>& out, std::vector<int32_t>* wide_of = nullptr);

// Returns false (with err) when a split leaves one side empty (the
// reference exits the process there, kdtree.cpp:182-185).
bool kd_build(const float* xyz, int64_t n, int cap, KdTree& out, std::string& err);

// expandAabb (aabb.cu:27-38) on every leaf, then node bounds bottom-up.
void kd_expand(KdTree& t, float ratio);

// Symmetric eigendecomposition in FP64: a[n*n] row-major (read only);
// eigenvalues descending in w[n]; eigenvectors as columns of v[n*n]
// (row-major, v[i*n + j] = component i of vector j), each with its
// largest-magnitude component positive.  Householder tridiagonalisation
// followed by implicit-shift QL.
bool sym_eig(const double* a, int n, double* w, double* v, std::string& err);

}  // namespace rte
