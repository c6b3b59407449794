// tl_launch.h - host launchers of the kernels, one set per population type
// (Pop = int for 32-bit, long long for 64-bit populations).
#pragma once

#include <cuda_runtime.h>

namespace tl {

struct SimParams;

// kind: 1 = thread, 32 = warp, 0 = CTA, 2/4/8/16 = lanes per realization,
// kKindCtaGlobal = CTA with its slot in global memory.
constexpr int kKindCtaGlobal = 64;
// mode: the kernel build a run needs.  Fast: no likelihood-ratio scores and
// no reference-compatibility switches; Scores: with scores; General: both.
// The sub-warp and global-slot kinds come in Fast and General only.
constexpr int kModeFast = 0, kModeScores = 1, kModeGeneral = 2;
template <class Pop>
cudaError_t launch_fused(const SimParams& p, int kind, int mode, int block, int grid, size_t smem,
                         cudaStream_t st);
template <class Pop>
cudaError_t fused_occupancy(int kind, int mode, int block, size_t smem, int* blocks_per_sm);
// sub-warp kinds (2, 4, 8, 16 lanes per realization), compiled in their own units
template <class Pop>
cudaError_t launch_fused_sub(const SimParams& p, int kind, int mode, int block, int grid, size_t smem,
                             cudaStream_t st);
template <class Pop>
cudaError_t fused_occupancy_sub(int kind, int mode, int block, size_t smem, int* blocks_per_sm);
struct BatchParams;
template <class Pop>
cudaError_t launch_batch(const BatchParams& bp, int mode, int block, int grid, size_t smem, cudaStream_t st);
template <class Pop>
cudaError_t batch_occupancy(int mode, int block, size_t smem, int* blocks_per_sm);
template <class Pop>
cudaError_t launch_plain_init(const SimParams& p, cudaStream_t st);
template <class Pop>
cudaError_t launch_plain_step(const SimParams& p, float* a_all, cudaStream_t st);
cudaError_t launch_plain_tally(const SimParams& p, cudaStream_t st);
template <class Pop>
cudaError_t launch_stats(const void* samp, long long R, int P, int K, int S, double* mean, double* sd,
                         cudaStream_t st);
template <class Pop>
cudaError_t launch_grad(const void* samp, const float* scores, long long R, int P, int K, int M, int S,
                        double* grad, double* se, double* meanf, cudaStream_t st);
template <class Pop>
cudaError_t launch_eval(const SimParams& p, const long long* x, int n, float* a, unsigned char* crit, float* mu,
                        float* s2, float* tau, double* a0, size_t smem, cudaStream_t st);
template <class Pop>
cudaError_t launch_replay(const SimParams& p, const long long* x0, const int* k, int n_leaps, long long* x_out,
                          int* status, size_t smem, cudaStream_t st);
cudaError_t launch_philox(const void* ctr, const void* key, int n, void* out, cudaStream_t st);
cudaError_t launch_poisson(const float* mean, int n, unsigned k0, unsigned k1, unsigned step, int compat,
                           int* out, cudaStream_t st);

}  // namespace tl
