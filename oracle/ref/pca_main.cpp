// Driver for the reference's own PCA (pca.cpp + vendored Eigen 3.4.0), built
// by oracle/ref/Makefile.  Runs PCA(data).calc_eigenvalues() and
// calc_result(dim) as Graph::Projection does (graph.cu:143-157) and writes
// doubles: mean[d], eigenvalues[d] (descending), vec[d*d] (row = input dim,
// column = component), then float projected base [n*d] (as save_result).
// usage: pca_ref_main <in.bin> <out.bin>; in.bin = int64 n, int64 d, float[n*d]
#include <cstdio>
#include <vector>
#include "pca.h"

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 3;
  long long n = 0, d = 0;
  if (fread(&n, 8, 1, f) != 1 || fread(&d, 8, 1, f) != 1) return 4;
  std::vector<float> x(n * d);
  if (fread(x.data(), 4, n * d, f) != (size_t)(n * d)) return 5;
  fclose(f);
  PCA pca(x.data(), (uint)n, (uint)d);
  pca.calc_eigenvalues();
  pca.calc_result((uint)d);
  FILE* o = fopen(argv[2], "wb");
  for (int i = 0; i < d; i++) { double v = pca.meanvecRow(i); fwrite(&v, 8, 1, o); }
  for (int i = 0; i < d; i++) { double v = pca.val(i, 0); fwrite(&v, 8, 1, o); }
  for (int i = 0; i < d; i++)
    for (int j = 0; j < d; j++) { double v = pca.vec(i, j); fwrite(&v, 8, 1, o); }
  for (long long i = 0; i < n; i++)
    for (int j = 0; j < d; j++) { float v = (float)pca.B_res(i, j); fwrite(&v, 4, 1, o); }
  fclose(o);
  return 0;
}
