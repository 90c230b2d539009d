// search_dispatch.cu -- maps (chunks, precision) to the instantiation files.
#include "search_dispatch.h"

#include <map>
#include <mutex>
#include <tuple>

namespace rte {

void* search_lookup_c1_f32(int, int, bool, bool);
void* search_lookup_c1_f32_r16(int, int, bool, bool);
void* search_lookup_c2_f32(int, int, bool, bool);
void* search_lookup_c2_f32_r16(int, int, bool, bool);
void* search_lookup_c30_bf16(int, int, bool, bool);
void* search_lookup_c30_f32(int, int, bool, bool);
void* search_lookup_c30_fp8(int, int, bool, bool);
void* search_lookup_c3_bf16(int, int, bool, bool);
void* search_lookup_c3_bf16_r16(int, int, bool, bool);
void* search_lookup_c3_bf16_wide(int, int, bool, bool);
void* search_lookup_c3_f32(int, int, bool, bool);
void* search_lookup_c3_f32_r16(int, int, bool, bool);
void* search_lookup_c3_fp8(int, int, bool, bool);
void* search_lookup_c3_fp8_r16(int, int, bool, bool);
void* search_lookup_c3_fp8_wide(int, int, bool, bool);
void* search_lookup_c4_bf16(int, int, bool, bool);
void* search_lookup_c4_bf16_r16(int, int, bool, bool);
void* search_lookup_c4_f32(int, int, bool, bool);
void* search_lookup_c4_f32_r16(int, int, bool, bool);
void* search_lookup_c4_fp8(int, int, bool, bool);
void* search_lookup_c4_fp8_r16(int, int, bool, bool);
void* search_lookup_c4_fp8_wide(int, int, bool, bool);
void* search_lookup_cg_bf16(int, int, bool, bool);
void* search_lookup_cg_bf16_wide(int, int, bool, bool);
void* search_lookup_cg_bf16_r16(int, int, bool, bool);
void* search_lookup_cg_f32(int, int, bool, bool);
void* search_lookup_cg_f32_wide(int, int, bool, bool);
void* search_lookup_cg_f32_r16(int, int, bool, bool);
void* search_lookup_cg_fp8(int, int, bool, bool);
void* search_lookup_cg_fp8_wide(int, int, bool, bool);
void* search_lookup_cg_fp8_r16(int, int, bool, bool);

namespace {
// The instantiations of one (chunk count, precision) are spread over a few
// translation units, so they compile in parallel: the lookup tries each.
template <KernelLookup... F>
void* chain(int NL, int NB, bool r16, bool team) {
  void* k = nullptr;
  ((k = k ? k : F(NL, NB, r16, team)), ...);
  return k;
}

struct Entry {
  int C;
  KernelLookup f32, bf16, fp8;
};
const Entry kTable[] = {
    {1, chain<search_lookup_c1_f32, search_lookup_c1_f32_r16>, nullptr, nullptr},
    {2, chain<search_lookup_c2_f32, search_lookup_c2_f32_r16>, nullptr, nullptr},
    {3, chain<search_lookup_c3_f32, search_lookup_c3_f32_r16>,
     chain<search_lookup_c3_bf16, search_lookup_c3_bf16_wide, search_lookup_c3_bf16_r16>,
     chain<search_lookup_c3_fp8, search_lookup_c3_fp8_wide, search_lookup_c3_fp8_r16>},
    {4, chain<search_lookup_c4_f32, search_lookup_c4_f32_r16>,
     chain<search_lookup_c4_bf16, search_lookup_c4_bf16_r16>,
     chain<search_lookup_c4_fp8, search_lookup_c4_fp8_wide, search_lookup_c4_fp8_r16>},
    {30, search_lookup_c30_f32, search_lookup_c30_bf16, search_lookup_c30_fp8},
};
// Kernels for any chunk count (template C == 0): every other dimension up
// to 1024, and the precisions a specialised chunk count lacks.
const Entry kGeneric = {0,
                        chain<search_lookup_cg_f32, search_lookup_cg_f32_wide, search_lookup_cg_f32_r16>,
                        chain<search_lookup_cg_bf16, search_lookup_cg_bf16_wide, search_lookup_cg_bf16_r16>,
                        chain<search_lookup_cg_fp8, search_lookup_cg_fp8_wide, search_lookup_cg_fp8_r16>};

KernelLookup pick_prec(const Entry& e, int prec) {
  return prec == kPrecF32 ? e.f32 : prec == kPrecBF16 ? e.bf16 : prec == kPrecFP8 ? e.fp8 : nullptr;
}
}  // namespace

bool search_chunks_supported(int C) { return C >= 1 && C <= kMaxChunks; }

int search_kernel_chunks(int C, int NL, int NB, int prec, bool r16) {
  for (const Entry& e : kTable) {
    if (e.C != C) continue;
    KernelLookup f = pick_prec(e, prec);
    if (f && f(NL, NB, r16, false)) return C;
  }
  return 0;
}

void* search_kernel_ptr(int C, int NL, int NB, int prec, bool r16, bool team) {
  if (!search_chunks_supported(C)) return nullptr;
  const int kc = search_kernel_chunks(C, NL, NB, prec, r16);
  const Entry* e = &kGeneric;
  for (const Entry& t : kTable)
    if (kc != 0 && t.C == kc) e = &t;
  KernelLookup f = pick_prec(*e, prec);
  return f ? f(NL, NB, r16, team) : nullptr;
}

cudaError_t launch_search(const SearchArgs& a, int C, int NL, int NB, int prec, int wpb, int grid,
                          size_t smem, cudaStream_t st) {
  void* k = search_kernel_ptr(C, NL, NB, prec, a.R == 16, a.team != 0 && a.team != 1);
  if (!k) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  SearchArgs args = a;
  args.C = C;
  void* params[] = {&args};
  return cudaLaunchKernel(k, dim3(grid), dim3(32 * wpb), params, smem, st);
}

int occupancy_search(int C, int NL, int NB, int prec, bool r16, int wpb, size_t smem) {
  void* k = search_kernel_ptr(C, NL, NB, prec, r16);
  if (!k) return 0;
  // the answer depends only on (kernel, device, block, shared memory): cache it
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  static std::mutex mu;
  static std::map<std::tuple<void*, int, int, size_t>, int> cache;
  const auto key = std::make_tuple(k, dev, wpb, smem);
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, 32 * wpb, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = n;
  return n;
}

}  // namespace rte
