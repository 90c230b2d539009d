// Instantiations of search_kernel for rows of any chunk count (the
// dimensions and (beam, batch) pairs without a specialised kernel), FP8.
// Graphs of degree >= 32, pools of 16 to 64 slots.
#define SEARCH_C 0
#define SEARCH_PREC kPrecFP8
#define SEARCH_FN search_lookup_cg_fp8
#define SEARCH_CASES RTE_CASE(0, 1) RTE_CASE(0, 2) RTE_CASE(0, 4) RTE_CASE(0, 8) RTE_CASE(1, 1) RTE_CASE(1, 2) RTE_CASE(1, 4) RTE_CASE(1, 8) RTE_CASE(2, 1) RTE_CASE(2, 2) RTE_CASE(2, 4) RTE_CASE(2, 8)
#include "search_inst.inc"
