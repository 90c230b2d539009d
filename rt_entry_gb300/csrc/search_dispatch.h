// search_dispatch.h -- host-side selection and launch of the templated
// search kernel search_kernel<C, NL, NB, PREC>.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "search_types.h"

namespace rte {

// Each search_c<C>_<prec>.cu defines one of these; it returns the kernel for
// (NL, NB) or nullptr when that combination is not instantiated.
using KernelLookup = void* (*)(int NL, int NB);

bool search_chunks_supported(int C);
void* search_kernel_ptr(int C, int NL, int NB, int prec);
cudaError_t launch_search(const SearchArgs& a, int C, int NL, int NB, int prec, int wpb, int grid,
                          size_t smem, cudaStream_t st);
int occupancy_search(int C, int NL, int NB, int prec, int wpb, size_t smem);

}  // namespace rte
