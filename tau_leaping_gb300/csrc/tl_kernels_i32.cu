// Kernels and launchers for 32-bit populations.
#define TL_COMMON_KERNELS
#include "tl_kernels.cuh"
#define TL_POP int
#include "tl_kernels_pop.inc"
#undef TL_POP

namespace tl {

cudaError_t launch_plain_tally(const SimParams& p, cudaStream_t st) {
    k_plain_tally<<<152, 256, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_philox(const void* ctr, const void* key, int n, void* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_philox<<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<const uint4*>(ctr), reinterpret_cast<const uint2*>(key),
                                              n, reinterpret_cast<uint4*>(out));
    return cudaGetLastError();
}

cudaError_t launch_poisson(const float* mean, int n, unsigned k0, unsigned k1, unsigned step, int compat, int* out,
                           cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_poisson<<<(n + 255) / 256, 256, 0, st>>>(mean, n, k0, k1, step, compat, out);
    return cudaGetLastError();
}

}  // namespace tl
