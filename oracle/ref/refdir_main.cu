// Driver that writes a data directory the way the reference's Graph does,
// with the reference's own code, built by oracle/ref/Makefile:
//   mean.fbin, O.fbin   PCA::calc_eigenvalues + PCA::save_mean_rotation
//                       (graph.cu:145-150, pca.cpp:60-90)
//   pca_base.fbin       PCA::calc_result + PCA::save_result (graph.cu:157-158,
//                       pca.cpp:122-139)
//   <cap>_0.aabbs       Kdtree over the first three columns of the projected
//                       base + computeAabbPid (entry.cu:34-43), in the layout
//                       RT_Entry::write_aabbs writes (entry.cu:171-178: int
//                       n, int cap, n OptixAabb, n*cap int pids).  write_aabbs
//                       itself sits in entry.cu beside the OptiX code and
//                       does not build here; this file repeats its four
//                       writes.
// usage: refdir_main <in.bin> <cap> <outdir>; in.bin = int64 n, int64 d, float[n*d]
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "kdtree.h"
#include "pca.h"

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 3;
  long long n = 0, d = 0;
  if (fread(&n, 8, 1, f) != 1 || fread(&d, 8, 1, f) != 1) return 4;
  std::vector<float> x(n * d);
  if (fread(x.data(), 4, n * d, f) != (size_t)(n * d)) return 5;
  fclose(f);
  const int cap = atoi(argv[2]);
  const std::string dir(argv[3]);
  PCA pca(x.data(), (uint)n, (uint)d);
  pca.calc_eigenvalues();
  pca.save_mean_rotation((dir + "/mean.fbin").c_str(), (dir + "/O.fbin").c_str());
  pca.calc_result((uint)d);
  pca.save_result((uint)d, (dir + "/pca_base.fbin").c_str());
  // the kd-tree runs on float3 points taken from the stored (float) projected
  // base, as RT_Entry::set_pca_points does (entry.cu:150-168)
  std::vector<float3> pts(n);
  for (long long i = 0; i < n; ++i)
    pts[i] = float3{(float)pca.B_res(i, 0), (float)pca.B_res(i, 1), (float)pca.B_res(i, 2)};
  OptixAabb world{0, 0, 0, 0, 0, 0};
  thrust::host_vector<OptixAabb> aabbs;
  thrust::host_vector<int> pids;
  {
    Kdtree kd(pts.data(), (int)n, cap, world, aabbs);
    kd.computeAabbPid(pids, (int)aabbs.size());
  }
  FILE* o = fopen((dir + "/" + std::to_string(cap) + "_0.aabbs").c_str(), "wb");
  if (!o) return 6;
  int na = (int)aabbs.size();
  fwrite(&na, sizeof(int), 1, o);
  fwrite(&cap, sizeof(int), 1, o);
  fwrite(&aabbs[0], sizeof(OptixAabb), na, o);
  fwrite(&pids[0], sizeof(int), (size_t)na * cap, o);
  fclose(o);
  return 0;
}
