// Instantiations of search_kernel for d <= 32, FP32.
// Degree-16 graphs (R16 kernels).
#define SEARCH_C 1
#define SEARCH_PREC kPrecF32
#define SEARCH_FN search_lookup_c1_f32_r16
#define SEARCH_CASES RTE_CASE16(0, 0) RTE_CASE16(0, 1) RTE_CASE16(1, 0) RTE_CASE16(1, 1) RTE_CASE16(2, 0) RTE_CASE16(2, 1) RTE_CASE16(4, 0) RTE_CASE16(4, 1)
#include "search_inst.inc"
