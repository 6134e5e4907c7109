// Launch entry points of the CUDA translation units (host side).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>
#include "hexo_types.h"
#include "hexo_plan.h"

namespace hexo {

// Dynamic shared memory of the path kernel: per path two raw slots (16 x u64)
// and two normal slots (16 x f32); per warp the conversion queue
// (kWarpScratchBytes) and a 64-option window of 32-bit payoff sums (16-byte
// aligned); the 128-entry double-single log table (2 KB).
inline size_t paths_smem_bytes(uint32_t block, uint32_t ppt) {
    const size_t rings = (size_t)ppt * 2 * kRngWords * block * (sizeof(uint64_t) + sizeof(float)) +
                         (size_t)(block / 32) * kWarpScratchBytes;
    return (rings + 15) / 16 * 16 + (size_t)(block / 32) * 64u * kLimbs * sizeof(uint32_t) + 128u * 16u;
}

// nullptr when (ppt, unroll) is not instantiated; the control-variate
// kernels (cv) exist for one path per thread and no unrolling.
const void *paths_kernel_ptr_f64(uint32_t ppt, uint32_t unroll, bool cv);
const void *paths_kernel_ptr_f32(uint32_t ppt, uint32_t unroll, bool cv);
inline const void *paths_kernel_ptr(bool f32, uint32_t ppt, uint32_t unroll, bool cv = false) {
    return f32 ? paths_kernel_ptr_f32(ppt, unroll, cv) : paths_kernel_ptr_f64(ppt, unroll, cv);
}
cudaError_t launch_paths(bool f32, const LaunchShape &sh, uint32_t grid, size_t smem, cudaStream_t st,
                         const KernelArgs &a);
// Sets the path kernel fn's dynamic shared-memory limit to the most it can
// have on device dev (the opt-in maximum less its static shared memory).
// Every entry point sets this same value before it launches fn, so one
// caller's launch shape never lowers the limit under another's launch.
cudaError_t paths_smem_limit(const void *fn, int dev);

// Finaliser: sums the n_slots private copies of the limbs and writes price
// and standard error per output slot.
struct FinalizeArgs {
    const unsigned long long *acc = nullptr;   // [slot * slot_stride + out * kLimbs + limb]
    uint32_t n_slots = 1;
    uint64_t slot_stride = 0;
    const uint64_t *n_paths = nullptr;         // per output: paths that price it
    const double *disc = nullptr;              // per output: exp(-r T)
    const int32_t *pay_exp = nullptr;          // per output: E, payoffs summed in units of 2^E
    uint32_t n = 0;                            // outputs
    double *price = nullptr, *se = nullptr;
    unsigned long long *acc_sum = nullptr;     // optional: the totals of this launch
    const double *cv_eg = nullptr;             // optional control variate: E[(G - K)^+] per output
    const uint32_t *cv_partner = nullptr;      //   and the slot of its geometric sums (~0 elsewhere)
    unsigned long long *carry = nullptr;       // optional: running sums of requests split across launches
    const uint64_t *carry_row = nullptr;       //   per output: (row << 1) | last block, ~0 = not carried
};
cudaError_t launch_finalize(const FinalizeArgs &f, cudaStream_t st);
// The geometric control variate's analytic part for a planned batch:
// The control variate's analytic part, in two halves so that its device
// memory is a region of the batch's arena (no allocation, so no device-wide
// synchronisation, per batch).  cv_plan builds, on the host, what the
// kernels need and the region's size; cv_run uploads it into `region` (256-byte
// aligned, cv_plan's bytes long) on stream st and enqueues the kernels that
// write E[(G - K)^+] per control-variate option into *eg and its geometric-sum
// slot into *partner (arrays of n_out entries inside the region).  The plan's
// host vectors must outlive the stream's copies.
struct CvPlan {
    std::vector<double> eg;          // n_out: NaN, filled on the device
    std::vector<uint32_t> partner;   // n_out: ~0 except the control-variate options
    std::vector<unsigned char> mats, opts;   // packed device records
    std::vector<double2> steps, nodes;
    uint32_t n_mats = 0, n_warp_mats = 0, n_opts = 0;
    size_t bytes = 0;                // the device region
};
void cv_plan(const BatchPlan &bp, CvPlan &cp);
cudaError_t cv_run(const CvPlan &cp, void *region, cudaStream_t st, double **eg, uint32_t **partner);

// Debug kernels.
cudaError_t launch_dbg_words(uint32_t seed, uint32_t stream, uint32_t n_streams, uint32_t n_words, uint64_t *out,
                             cudaStream_t st);
cudaError_t launch_dbg_draws(uint32_t seed, uint32_t stream, uint32_t n_streams, const uint8_t *kinds, uint32_t n,
                             double *out, cudaStream_t st);
cudaError_t launch_dbg_normals(const uint64_t *words, uint64_t n, double *out, cudaStream_t st);
cudaError_t launch_dbg_as241_check(uint32_t branch, uint64_t lo, uint64_t hi, unsigned long long *out,
                                   cudaStream_t st);
cudaError_t launch_dbg_limbs(const double *pay, uint64_t n, bool f32, int E, uint32_t *out, cudaStream_t st);
cudaError_t measure_pipe_peaks(int sm_count, cudaStream_t st, double *out5);

} // namespace hexo
