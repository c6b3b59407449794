// Sub-warp fused kernels for 64-bit populations.
#include "tl_kernels.cuh"
#define TL_POP long long
#include "tl_kernels_sub.inc"
#undef TL_POP
