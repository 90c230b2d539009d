// Instantiations of search_kernel for rows of any chunk count (the
// dimensions and (beam, batch) pairs without a specialised kernel), FP8.
// Degree-16 graphs (R16 kernels).
#define SEARCH_C 0
#define SEARCH_PREC kPrecFP8
#define SEARCH_FN search_lookup_cg_fp8_r16
#define SEARCH_CASES RTE_CASE16(0, 0) RTE_CASE16(0, 1) RTE_CASE16(0, 2) RTE_CASE16(1, 0) RTE_CASE16(1, 1) RTE_CASE16(1, 2) RTE_CASE16(2, 0) RTE_CASE16(2, 1) RTE_CASE16(2, 2) RTE_CASE16(4, 0) RTE_CASE16(4, 1) RTE_CASE16(4, 2) RTE_CASE16(8, 0) RTE_CASE16(8, 1) RTE_CASE16(8, 2)
#include "search_inst.inc"
