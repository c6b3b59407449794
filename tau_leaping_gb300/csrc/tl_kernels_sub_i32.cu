// Sub-warp fused kernels for 32-bit populations.
#include "tl_kernels.cuh"
#define TL_POP int
#include "tl_kernels_sub.inc"
#undef TL_POP
