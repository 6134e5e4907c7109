// Launch entry points of the CUDA translation units (host side).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "hexo_types.h"
#include "hexo_plan.h"

namespace hexo {

// Dynamic shared memory of the path kernel: the RNG rings plus the payoff
// reduction scratch.
inline size_t paths_smem_bytes(uint32_t block, uint32_t ppt) {
    return (size_t)ppt * kRingSlots * kRngWords * block * sizeof(uint64_t) + 64u * kLimbs * sizeof(unsigned long long);
}

// nullptr when (ppt, unroll) is not instantiated.
const void *paths_kernel_ptr_f64(uint32_t ppt, uint32_t unroll);
const void *paths_kernel_ptr_f32(uint32_t ppt, uint32_t unroll);
inline const void *paths_kernel_ptr(bool f32, uint32_t ppt, uint32_t unroll) {
    return f32 ? paths_kernel_ptr_f32(ppt, unroll) : paths_kernel_ptr_f64(ppt, unroll);
}
cudaError_t launch_paths(bool f32, const LaunchShape &sh, uint32_t grid, size_t smem, cudaStream_t st,
                         const KernelArgs &a);

// Finaliser: price and standard error per output slot from the limb sums.
cudaError_t launch_finalize(const unsigned long long *acc, const uint64_t *n_paths, const double *disc, uint32_t n,
                            double *price, double *se, cudaStream_t st);

// Debug kernels.
cudaError_t launch_dbg_words(uint32_t seed, uint32_t n_streams, uint32_t n_words, uint64_t *out, cudaStream_t st);
cudaError_t launch_dbg_draws(uint32_t seed, uint32_t n_streams, const uint8_t *kinds, uint32_t n, double *out,
                             cudaStream_t st);
cudaError_t launch_dbg_normals(const uint64_t *words, uint64_t n, double *out, cudaStream_t st);
cudaError_t measure_pipe_peaks(int sm_count, cudaStream_t st, double *out4);

} // namespace hexo
