// Instantiations of search_kernel for d <= 960, FP32.
#define SEARCH_C 30
#define SEARCH_PREC kPrecF32
#define SEARCH_FN search_lookup_c30_f32
#define SEARCH_CASES RTE_CASE(0, 2) RTE_CASE(1, 2) RTE_CASE(2, 2) RTE_CASE(4, 2) RTE_CASE(8, 2)
#include "search_inst.inc"
