// Instantiations of search_kernel for d <= 96, BF16.
// Graphs of degree >= 32, batches of 4 and 8 registers (width 4 over degree
// 32, widths 2 and 4 over degree 64).
#define SEARCH_C 3
#define SEARCH_PREC kPrecBF16
#define SEARCH_FN search_lookup_c3_bf16_wide
#define SEARCH_CASES RTE_CASE(2, 4) RTE_CASE(4, 4) RTE_CASE(8, 4) RTE_CASE(4, 8) RTE_CASE(8, 8)
#include "search_inst.inc"
