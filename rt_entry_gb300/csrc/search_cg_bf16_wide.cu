// Instantiations of search_kernel for rows of any chunk count (the
// dimensions and (beam, batch) pairs without a specialised kernel), BF16.
// Graphs of degree >= 32, pools of 128 and 256 slots.
#define SEARCH_C 0
#define SEARCH_PREC kPrecBF16
#define SEARCH_FN search_lookup_cg_bf16_wide
#define SEARCH_CASES RTE_CASE(4, 1) RTE_CASE(4, 2) RTE_CASE(4, 4) RTE_CASE(4, 8) RTE_CASE(8, 1) RTE_CASE(8, 2) RTE_CASE(8, 4) RTE_CASE(8, 8)
#include "search_inst.inc"
