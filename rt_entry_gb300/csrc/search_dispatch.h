// search_dispatch.h -- host-side selection and launch of the templated
// search kernel search_kernel<C, NL, NB, PREC>.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "search_types.h"

namespace rte {

// Each search_c<C>_<prec>*.cu defines one of these; it returns the kernel for
// (NL, NB) over a degree-16 graph (r16) or a graph of degree >= 32 -- the
// single-warp search_kernel, or search_kernel_team with `team` -- or nullptr
// when that combination is not instantiated.
using KernelLookup = void* (*)(int NL, int NB, bool r16, bool team);

bool search_chunks_supported(int C);
// The kernel template's C for rows of C chunks, pool registers NL, batch
// registers NB, a precision and the graph degree (r16: degree 16): C itself where a kernel was built for that
// combination, else 0 (the kernels built for any chunk count, which keep
// the query in shared memory).
int search_kernel_chunks(int C, int NL, int NB, int prec, bool r16);
void* search_kernel_ptr(int C, int NL, int NB, int prec, bool r16, bool team = false);
// The degree comes from a.R (16 selects the degree-16 kernels); a.team other
// than 0 and 1 selects search_kernel_team.
cudaError_t launch_search(const SearchArgs& a, int C, int NL, int NB, int prec, int wpb, int grid,
                          size_t smem, cudaStream_t st);
int occupancy_search(int C, int NL, int NB, int prec, bool r16, int wpb, size_t smem);

}  // namespace rte
