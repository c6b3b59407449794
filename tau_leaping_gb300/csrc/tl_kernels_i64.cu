// Kernels and launchers for 64-bit populations.
#include "tl_kernels.cuh"
#define TL_POP long long
#include "tl_kernels_pop.inc"
#undef TL_POP
