// Driver for the reference's own kd-tree (kdtree.cpp), built by
// oracle/ref/Makefile.  Reads n float3 points, runs Kdtree's constructor
// (buildWithStack) and computeAabbPid exactly as RT_Entry::BlockUp does
// (entry.cu:34-40), and writes: int64 n_leaves, float[n_leaves*6] boxes,
// int32[n_leaves*leaf_cap] pids.
// usage: kdtree_ref_main <in.bin> <leaf_cap> <out.bin>; in.bin = int64 n, float[n*3]
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "kdtree.h"

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 3;
  long long n = 0;
  if (fread(&n, 8, 1, f) != 1) return 4;
  std::vector<float3> pts(n);
  if (fread(pts.data(), sizeof(float3), n, f) != (size_t)n) return 5;
  fclose(f);
  int cap = atoi(argv[2]);
  OptixAabb world{0, 0, 0, 0, 0, 0};
  thrust::host_vector<OptixAabb> aabbs;
  thrust::host_vector<int> pids;
  {
    Kdtree kd(pts.data(), (int)n, cap, world, aabbs);
    kd.computeAabbPid(pids, (int)aabbs.size());
  }
  FILE* o = fopen(argv[3], "wb");
  long long nl = aabbs.size();
  fwrite(&nl, 8, 1, o);
  fwrite(&aabbs[0], sizeof(OptixAabb), nl, o);
  fwrite(&pids[0], sizeof(int), pids.size(), o);
  fclose(o);
  return 0;
}
