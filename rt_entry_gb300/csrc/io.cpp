// io.cpp -- the reference's on-disk formats (see io.h).  Unlike the
// reference readers, which exit(1) on a missing file, every failure here is
// reported to the caller; truncated or inconsistent files are rejected.
#include "io.h"

#include <sys/stat.h>

#include <cstdio>
#include <cstring>
#include <memory>

namespace rte {
namespace io {

namespace {

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

bool file_size(const std::string& path, int64_t& sz, std::string& err) {
  struct stat st;
  if (stat(path.c_str(), &st) != 0) {
    err = "cannot open " + path;
    return false;
  }
  sz = (int64_t)st.st_size;
  return true;
}

bool ends_with(const std::string& s, const char* suf) {
  const size_t n = strlen(suf);
  return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

// Per-vector framed formats: int32 d, then d elements of `esize` bytes.
template <typename T, typename Out>
bool read_framed(const std::string& path, std::vector<Out>& data, int64_t& n, int& d,
                 std::string& err) {
  int64_t sz;
  if (!file_size(path, sz, err)) return false;
  File fh;
  fh.f = fopen(path.c_str(), "rb");
  if (!fh.f) {
    err = "cannot open " + path;
    return false;
  }
  int32_t d0 = 0;
  if (sz < 4 || fread(&d0, 4, 1, fh.f) != 1 || d0 <= 0) {
    err = path + ": bad header";
    return false;
  }
  const int64_t rec = 4 + (int64_t)d0 * sizeof(T);
  if (sz % rec != 0) {
    err = path + ": size is not a multiple of the record size (truncated?)";
    return false;
  }
  n = sz / rec;
  d = d0;
  data.resize((size_t)n * d);
  fseek(fh.f, 0, SEEK_SET);
  std::vector<T> row(d);
  for (int64_t i = 0; i < n; ++i) {
    int32_t di = 0;
    if (fread(&di, 4, 1, fh.f) != 1 || di != d0 || fread(row.data(), sizeof(T), d, fh.f) != (size_t)d) {
      err = path + ": inconsistent record " + std::to_string(i);
      return false;
    }
    for (int j = 0; j < d; ++j) data[(size_t)i * d + j] = (Out)row[j];
  }
  return true;
}

bool read_fbin(const std::string& path, std::vector<float>& data, int64_t& n, int& d,
               std::string& err) {
  int64_t sz;
  if (!file_size(path, sz, err)) return false;
  File fh;
  fh.f = fopen(path.c_str(), "rb");
  if (!fh.f) {
    err = "cannot open " + path;
    return false;
  }
  int32_t hdr[2];
  if (fread(hdr, 4, 2, fh.f) != 2 || hdr[0] < 0 || hdr[1] <= 0) {
    err = path + ": bad header";
    return false;
  }
  n = hdr[0];
  d = hdr[1];
  if (sz != 8 + n * (int64_t)d * 4) {
    err = path + ": size does not match its header (truncated?)";
    return false;
  }
  data.resize((size_t)n * d);
  if (fread(data.data(), 4, data.size(), fh.f) != data.size()) {
    err = path + ": short read";
    return false;
  }
  return true;
}

bool write_all(const std::string& path, const void* a, size_t na, const void* b, size_t nb,
               const void* c, size_t nc, const void* e, size_t ne, std::string& err) {
  File fh;
  fh.f = fopen(path.c_str(), "wb");
  if (!fh.f) {
    err = "cannot create " + path;
    return false;
  }
  if ((na && fwrite(a, 1, na, fh.f) != na) || (nb && fwrite(b, 1, nb, fh.f) != nb) ||
      (nc && fwrite(c, 1, nc, fh.f) != nc) || (ne && fwrite(e, 1, ne, fh.f) != ne)) {
    err = "write failed: " + path;
    return false;
  }
  return true;
}

// int32 d, then n*d floats with n = (size - 4) / (4d): the .hvecs and .hh
// layouts (file_read.cu:83-101 and :171-193, whose readers infer n the
// same way).
bool read_dhead(const std::string& path, std::vector<float>& data, int64_t& n, int& d,
                std::string& err) {
  int64_t sz;
  if (!file_size(path, sz, err)) return false;
  File fh;
  fh.f = fopen(path.c_str(), "rb");
  if (!fh.f) {
    err = "cannot open " + path;
    return false;
  }
  int32_t d0 = 0;
  if (sz < 4 || fread(&d0, 4, 1, fh.f) != 1 || d0 <= 0) {
    err = path + ": bad header";
    return false;
  }
  if ((sz - 4) % ((int64_t)d0 * 4) != 0) {
    err = path + ": size is not 4 + a multiple of 4d (truncated?)";
    return false;
  }
  n = (sz - 4) / ((int64_t)d0 * 4);
  d = d0;
  data.resize((size_t)n * d);
  if (fread(data.data(), 4, data.size(), fh.f) != data.size()) {
    err = path + ": short read";
    return false;
  }
  return true;
}

// Text: "n d", then n rows of d values separated by commas (the last value
// of a row without one), file_read.cu:103-117.  Whitespace between values
// is accepted too.
bool read_txt(const std::string& path, std::vector<float>& data, int64_t& n, int& d, std::string& err) {
  File fh;
  fh.f = fopen(path.c_str(), "r");
  if (!fh.f) {
    err = "cannot open " + path;
    return false;
  }
  long long n0 = 0;
  int d0 = 0;
  if (fscanf(fh.f, "%lld %d", &n0, &d0) != 2 || n0 < 0 || d0 <= 0) {
    err = path + ": bad header (expected \"n d\")";
    return false;
  }
  n = n0;
  d = d0;
  data.resize((size_t)n * d);
  for (size_t i = 0; i < data.size(); ++i) {
    if (fscanf(fh.f, " %f", &data[i]) != 1) {
      err = path + ": expected " + std::to_string(data.size()) + " values, read " + std::to_string(i);
      return false;
    }
    int c = fgetc(fh.f);
    while (c == ' ' || c == '\t' || c == '\r' || c == '\n') c = fgetc(fh.f);
    if (c != ',' && c != EOF) ungetc(c, fh.f);
  }
  return true;
}

}  // namespace

bool file_exists(const std::string& path) {
  struct stat st;
  return stat(path.c_str(), &st) == 0;
}

bool read_vectors(const std::string& path, std::vector<float>& data, int64_t& n, int& d,
                  std::string& err) {
  if (ends_with(path, ".fvecs")) return read_framed<float>(path, data, n, d, err);
  if (ends_with(path, ".bvecs")) return read_framed<uint8_t>(path, data, n, d, err);
  if (ends_with(path, ".fbin")) return read_fbin(path, data, n, d, err);
  if (ends_with(path, ".hvecs") || ends_with(path, ".hh")) return read_dhead(path, data, n, d, err);
  if (ends_with(path, ".txt")) return read_txt(path, data, n, d, err);
  err = path + ": unknown vector format (expected .fvecs, .bvecs, .fbin, .hvecs, .hh or .txt)";
  return false;
}

bool read_matrix_fbin(const std::string& path, std::vector<float>& data, int64_t& n, int& d,
                      std::string& err) {
  return read_fbin(path, data, n, d, err);
}

bool read_ivecs(const std::string& path, std::vector<int32_t>& data, int64_t& n, int& d,
                std::string& err) {
  return read_framed<int32_t>(path, data, n, d, err);
}

bool read_graph(const std::string& path, int64_t np, std::vector<int32_t>& data, int& degree,
                std::string& err) {
  int64_t sz;
  if (!file_size(path, sz, err)) return false;
  if (np <= 0 || sz % (4 * np) != 0 || sz == 0) {
    err = path + ": size is not a multiple of 4*np";
    return false;
  }
  degree = (int)(sz / (4 * np));
  File fh;
  fh.f = fopen(path.c_str(), "rb");
  if (!fh.f) {
    err = "cannot open " + path;
    return false;
  }
  data.resize((size_t)np * degree);
  if (fread(data.data(), 4, data.size(), fh.f) != data.size()) {
    err = path + ": short read";
    return false;
  }
  return true;
}

bool write_fbin(const std::string& path, const float* data, int64_t n, int d, std::string& err) {
  const int32_t hdr[2] = {(int32_t)n, d};
  return write_all(path, hdr, 8, data, (size_t)n * d * 4, nullptr, 0, nullptr, 0, err);
}

bool read_aabbs(const std::string& path, int64_t& n_leaves, int& leaf_size,
                std::vector<float>& boxes, std::vector<int32_t>& pids, std::string& err) {
  int64_t sz;
  if (!file_size(path, sz, err)) return false;
  File fh;
  fh.f = fopen(path.c_str(), "rb");
  if (!fh.f) {
    err = "cannot open " + path;
    return false;
  }
  int32_t hdr[2];
  if (fread(hdr, 4, 2, fh.f) != 2 || hdr[0] <= 0 || hdr[1] <= 0) {
    err = path + ": bad header";
    return false;
  }
  n_leaves = hdr[0];
  leaf_size = hdr[1];
  if (sz != 8 + n_leaves * 24 + n_leaves * (int64_t)leaf_size * 4) {
    err = path + ": size does not match its header";
    return false;
  }
  boxes.resize((size_t)n_leaves * 6);
  pids.resize((size_t)n_leaves * leaf_size);
  if (fread(boxes.data(), 4, boxes.size(), fh.f) != boxes.size() ||
      fread(pids.data(), 4, pids.size(), fh.f) != pids.size()) {
    err = path + ": short read";
    return false;
  }
  return true;
}

bool write_aabbs(const std::string& path, int64_t n_leaves, int leaf_size, const float* boxes,
                 const int32_t* pids, std::string& err) {
  const int32_t hdr[2] = {(int32_t)n_leaves, leaf_size};
  return write_all(path, hdr, 8, boxes, (size_t)n_leaves * 24, pids,
                   (size_t)n_leaves * leaf_size * 4, nullptr, 0, err);
}

bool save_index(const std::string& dir, const IndexFiles& f, std::string& err) {
  mkdir(dir.c_str(), 0755);
  if (!write_fbin(dir + "/base.fbin", f.base->data(), f.np, f.dim, err)) return false;
  if (!write_all(dir + "/graph.ibin", f.graph->data(), f.graph->size() * 4, nullptr, 0, nullptr, 0,
                 nullptr, 0, err))
    return false;
  std::string meta = "rt_entry_gb300 index v1\nsearch_dim " + std::to_string(f.search_dim) +
                     "\nhas_pca " + std::to_string(f.has_pca ? 1 : 0) + "\nhas_kdtree " +
                     std::to_string(f.has_kdtree ? 1 : 0) + "\nleaf_size " +
                     std::to_string(f.leaf_size) + "\n";
  char ratio[64];
  snprintf(ratio, sizeof ratio, "expand_ratio %.9g\n", (double)f.expand_ratio);
  meta += ratio;
  if (f.has_pca) {
    if (!write_fbin(dir + "/mean.fbin", f.mean->data(), 1, f.dim, err)) return false;
    if (!write_fbin(dir + "/O.fbin", f.rot->data(), f.dim, f.dim, err)) return false;
    if (!write_fbin(dir + "/pca_base.fbin", f.pca_base->data(), f.np, f.search_dim, err))
      return false;
  }
  if (f.has_kdtree) {
    if (!write_aabbs(dir + "/" + std::to_string(f.leaf_size) + "_0.aabbs", f.n_leaves, f.leaf_size,
                     f.tight->data(), f.pids->data(), err))
      return false;
  }
  return write_all(dir + "/meta.txt", meta.data(), meta.size(), nullptr, 0, nullptr, 0, nullptr, 0,
                   err);
}

bool load_index(const std::string& dir, LoadedIndex& out, std::string& err) {
  int64_t n;
  int d;
  if (!read_fbin(dir + "/base.fbin", out.base, n, d, err)) return false;
  out.np = n;
  out.dim = d;
  int degree = 0;
  if (!read_graph(dir + "/graph.ibin", n, out.graph, degree, err)) return false;
  out.degree = degree;
  FILE* m = fopen((dir + "/meta.txt").c_str(), "r");
  if (!m) {
    err = "cannot open " + dir + "/meta.txt";
    return false;
  }
  char line[256];
  int has_pca = 0, has_kd = 0;
  while (fgets(line, sizeof line, m)) {
    sscanf(line, "search_dim %d", &out.search_dim);
    sscanf(line, "has_pca %d", &has_pca);
    sscanf(line, "has_kdtree %d", &has_kd);
    sscanf(line, "leaf_size %d", &out.leaf_size);
    sscanf(line, "expand_ratio %f", &out.expand_ratio);
  }
  fclose(m);
  out.has_pca = has_pca != 0;
  out.has_kdtree = has_kd != 0;
  if (out.has_pca) {
    int64_t n1;
    int d1;
    if (!read_fbin(dir + "/mean.fbin", out.mean, n1, d1, err)) return false;
    if (n1 != 1 || d1 != d) {
      err = "mean.fbin does not match base.fbin";
      return false;
    }
    if (!read_fbin(dir + "/O.fbin", out.rot, n1, d1, err)) return false;
    if (n1 != d || d1 != d) {
      err = "O.fbin does not match base.fbin";
      return false;
    }
  }
  return true;
}

}  // namespace io
}  // namespace rte
