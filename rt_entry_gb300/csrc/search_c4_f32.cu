// Instantiations of search_kernel for d <= 128, FP32.
// Graphs of degree >= 32.
#define SEARCH_C 4
#define SEARCH_PREC kPrecF32
#define SEARCH_FN search_lookup_c4_f32
#define SEARCH_CASES RTE_CASE(0, 1) RTE_CASE(0, 2) RTE_CASE(1, 1) RTE_CASE(1, 2) RTE_CASE(1, 4) RTE_CASE(2, 1) RTE_CASE(2, 2) RTE_CASE(2, 4) RTE_CASE(4, 1) RTE_CASE(4, 2) RTE_CASE(4, 4) RTE_CASE(8, 1) RTE_CASE(8, 2) RTE_CASE(8, 4) RTE_CASE(4, 8) RTE_CASE(8, 8)
#include "search_inst.inc"
