// io.h -- readers and writers for the reference's on-disk formats.
//   .fvecs / .bvecs / .ivecs   per vector: int32 d, then d values
//                              (file_read.cu:132-154, :196-229, :231-253)
//   .fbin                      int32 n, int32 d, then n*d float
//                              (file_read.cu:156-171; also mean.fbin, O.fbin
//                              and pca_base.fbin, pca.cpp:60-90,128-139)
//   graph                      raw int32 [np x degree], no header; degree =
//                              file size / (4 np) (file_read.cu:237-255)
//   <leaf_size>_0.aabbs        int32 n_leaves, int32 leaf_size, 6 floats per
//                              tight leaf box, int32 pids [n_leaves x
//                              leaf_size] (entry.cu:171-190)
//   .hvecs / .hh               int32 d, then n*d float, n from the file size
//                              (file_read.cu:83-101, :171-193)
//   .txt                       "n d", then rows of comma-separated values
//                              (file_read.cu:103-117)
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace rte {
namespace io {

bool file_exists(const std::string& path);
// Vectors by extension: .fvecs .bvecs .fbin .hvecs .hh .txt (file_read.cu:16-80).
bool read_vectors(const std::string& path, std::vector<float>& data, int64_t& n, int& d,
                  std::string& err);
// An .fbin matrix whatever its name (mean.fbin, O.fbin, pca_base.fbin).
bool read_matrix_fbin(const std::string& path, std::vector<float>& data, int64_t& n, int& d,
                      std::string& err);
bool read_ivecs(const std::string& path, std::vector<int32_t>& data, int64_t& n, int& d,
                std::string& err);
bool read_graph(const std::string& path, int64_t np, std::vector<int32_t>& data, int& degree,
                std::string& err);
bool write_fbin(const std::string& path, const float* data, int64_t n, int d, std::string& err);
bool read_aabbs(const std::string& path, int64_t& n_leaves, int& leaf_size,
                std::vector<float>& boxes, std::vector<int32_t>& pids, std::string& err);
bool write_aabbs(const std::string& path, int64_t n_leaves, int leaf_size, const float* boxes,
                 const int32_t* pids, std::string& err);

struct IndexFiles {
  int64_t np = 0;
  int dim = 0, degree = 0;
  const std::vector<float>* base = nullptr;
  const std::vector<int32_t>* graph = nullptr;
  bool has_pca = false;
  int search_dim = 0;
  const std::vector<float>* mean = nullptr;
  const std::vector<float>* rot = nullptr;
  const std::vector<float>* pca_base = nullptr;
  bool has_kdtree = false;
  int leaf_size = 0;
  float expand_ratio = 0;
  int64_t n_leaves = 0;
  const std::vector<float>* tight = nullptr;
  const std::vector<int32_t>* pids = nullptr;
};

struct LoadedIndex {
  int64_t np = 0;
  int dim = 0, degree = 0;
  std::vector<float> base;
  std::vector<int32_t> graph;
  bool has_pca = false;
  int search_dim = 0;
  std::vector<float> mean, rot;
  bool has_kdtree = false;
  int leaf_size = 0;
  float expand_ratio = 0;
};

bool save_index(const std::string& dir, const IndexFiles& f, std::string& err);
bool load_index(const std::string& dir, LoadedIndex& out, std::string& err);

}  // namespace io
}  // namespace rte
