// Instantiations of search_kernel for d <= 96, FP8-E4M3.
// Degree-16 graphs (R16 kernels).
#define SEARCH_C 3
#define SEARCH_PREC kPrecFP8
#define SEARCH_FN search_lookup_c3_fp8_r16
#define SEARCH_CASES RTE_CASE16(0, 0) RTE_CASE16(0, 1) RTE_CASE16(1, 0) RTE_CASE16(1, 1) RTE_CASE16(2, 0) RTE_CASE16(2, 1) RTE_CASE16(4, 0) RTE_CASE16(4, 1)
#include "search_inst.inc"
