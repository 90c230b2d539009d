/* Stand-in for the reference's head.h when compiling graph_search.cuh alone:
 * only the macros the search kernel reads.  REF_DIM comes from the command
 * line (the reference fixes DIM = GRAPH_DIM at compile time, head.h:27-29). */
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <sys/types.h>
#define DIM REF_DIM
#define GRAPH_DIM REF_DIM
#define USE_L2_DIST_
