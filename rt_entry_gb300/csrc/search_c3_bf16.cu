// Instantiations of search_kernel for d <= 96, BF16.
// Graphs of degree >= 32.
#define SEARCH_C 3
#define SEARCH_PREC kPrecBF16
#define SEARCH_FN search_lookup_c3_bf16
#define SEARCH_CASES RTE_CASE(0, 1) RTE_CASE(0, 2) RTE_CASE(1, 1) RTE_CASE(1, 2) RTE_CASE(2, 1) RTE_CASE(2, 2) RTE_CASE(4, 1) RTE_CASE(4, 2) RTE_CASE(8, 1) RTE_CASE(8, 2)
#include "search_inst.inc"
