// Finaliser, launch dispatch and debug kernels.
#include <algorithm>
#include "hexo_device.cuh"
#include "hexo_final.h"
#include "hexo_launch.h"

namespace hexo {

cudaError_t launch_paths(bool f32, const LaunchShape &sh, uint32_t grid, size_t smem, cudaStream_t st,
                         const KernelArgs &a) {
    const void *fn = paths_kernel_ptr(f32, sh.ppt, sh.unroll, sh.cv);
    if (fn == nullptr) return cudaErrorInvalidValue;
    KernelArgs args = a;
    void *params[] = {&args};
    return cudaLaunchKernel(fn, dim3(grid), dim3(sh.block), params, smem, st);
}

cudaError_t paths_smem_limit(const void *fn, int dev) {
    if (fn == nullptr) return cudaErrorInvalidValue;
    int optin = 0;
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, fn)) != cudaSuccess) return e;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}

// Sums the CTA-private copies of the limbs (exact integer additions) and
// finalises each option.  With carried sums (the serving loop's requests
// that run as several path blocks across launches), a slot's totals are
// first added into its request's running sums in device memory, and only
// the launch that carries the request's last block finalises, from those.
__global__ void finalize_kernel(const FinalizeArgs f) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    auto total = [&](uint32_t o, uint64_t (&l)[kLimbs]) {
#pragma unroll
        for (int x = 0; x < kLimbs; ++x) l[x] = 0;
        for (uint32_t s = 0; s < f.n_slots; ++s)
#pragma unroll
            for (int x = 0; x < kLimbs; ++x) l[x] += f.acc[(size_t)s * f.slot_stride + (size_t)o * kLimbs + x];
    };
    uint64_t l[kLimbs];
    total(i, l);
    if (f.acc_sum != nullptr)
#pragma unroll
        for (int x = 0; x < kLimbs; ++x) f.acc_sum[(size_t)i * kLimbs + x] = l[x];
    const uint64_t cr = f.carry_row != nullptr ? f.carry_row[i] : ~0ull;
    if (cr != ~0ull) {   // one launch at a time touches a request's running sums
        unsigned long long *row = f.carry + (size_t)(cr >> 1) * kLimbs;
#pragma unroll
        for (int x = 0; x < kLimbs; ++x) {
            row[x] += l[x];
            l[x] = row[x];
        }
        if ((cr & 1ull) == 0ull) {   // more blocks to come
            f.price[i] = __longlong_as_double(0x7ff8000000000000ll);
            f.se[i] = __longlong_as_double(0x7ff8000000000000ll);
            return;
        }
    }
    double p, s;
    const uint32_t g = f.cv_partner != nullptr ? f.cv_partner[i] : ~0u;
    if (g != ~0u) {   // an Asian option with the control variate: its geometric and difference sums
        uint64_t lg[kLimbs], ld[kLimbs];
        total(g, lg);
        total(g + 1u, ld);
        finalize_cv(l, lg, ld, f.n_paths[i], f.disc[i], f.pay_exp[i], f.cv_eg[i], &p, &s);
    } else {
        finalize_limbs6(l, f.n_paths[i], f.disc[i], f.pay_exp[i], &p, &s);
    }
    f.price[i] = p;
    f.se[i] = s;
}

cudaError_t launch_finalize(const FinalizeArgs &f, cudaStream_t st) {
    if (f.n == 0) return cudaSuccess;
    finalize_kernel<<<(f.n + 255) / 256, 256, 0, st>>>(f);
    return cudaGetLastError();
}

// Raw stream words: block 0 is the state after initialisation with its
// lanes reversed, then one block per round.
__global__ void dbg_words_kernel(uint32_t seed, uint32_t stream, uint32_t n_streams, uint32_t n_words,
                                 uint64_t *out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_streams) return;
    dev::Shishua g;
    dev::sh_init(g, (uint64_t)(uint32_t)(seed + k), (uint64_t)stream);
    uint64_t o[16];
#pragma unroll
    for (int L = 0; L < 4; ++L)
#pragma unroll
        for (int q = 0; q < 4; ++q) o[4 * L + q] = g.s[4 * (3 - L) + q];
    for (uint32_t w = 0; w < n_words; w += 16) {
        if (w > 0) dev::sh_round(g, o);
#pragma unroll
        for (int q = 0; q < 16; ++q)
            if (w + q < n_words) out[(size_t)k * n_words + w + q] = o[q];
    }
}

// The two-buffer RNG through the same ring code as the path kernel.
__global__ void dbg_draws_kernel(uint32_t seed, uint32_t stream, uint32_t n_streams, const uint8_t *kinds, uint32_t n,
                                 double *out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t bd = blockDim.x, tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    uint64_t *raw = reinterpret_cast<uint64_t *>(smem_raw);
    float *nrm = reinterpret_cast<float *>(raw + 2 * kRngWords * bd);
    uint16_t *tq_i = reinterpret_cast<uint16_t *>(nrm + 2 * kRngWords * bd);
    const uint32_t k = blockIdx.x * bd + tid;
    dev::Ring r{raw + tid, nrm + tid, bd};
    dev::WarpScratch ws{raw + tid - lane, nrm + tid - lane, tq_i + warp * kConvQueue, lane};
    dev::Shishua g;
    dev::RngLane c;
    dev::rng_start<true>(g, c, r, ws, seed + k, stream);
    for (uint32_t i = 0; i < n; i += 2) {
        if (i + 1 < n && kinds[i + 1] == 0) {
            // a QE-shaped pair (normal, normal) or (uniform, normal): the path kernel's draw code
            const bool quad = kinds[i] == 0;
            dev::DrawPlan dp = dev::draw_prefetch(c, r);
            if (dev::draw_prepare<true>(g, c, r, ws, quad)) dp = dev::draw_prefetch(c, r);
            float z1 = 0.0f, z2;
            uint64_t uw = 0;
            dev::draw_commit(g, c, r, dp, quad, z1, uw, z2);
            if (k < n_streams) {
                out[(size_t)k * n + i] = kinds[i] ? dev::uniform_f64(uw) : (double)z1;
                out[(size_t)k * n + i + 1] = (double)z2;
            }
            continue;
        }
        for (uint32_t h = i; h < i + 2 && h < n; ++h) {
            double v;
            if (kinds[h]) v = dev::uniform_f64(dev::rng_next_u(g, c, r));
            else v = (double)dev::rng_next_g<true>(g, c, r);
            if (k < n_streams) out[(size_t)k * n + h] = v;
        }
    }
}

__global__ void dbg_normals_kernel(const uint64_t *words, uint64_t n, double *out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {   // both input stages; a disagreement shows as NaN
        const float a = dev::as241_word<false>(words[i]), b = dev::as241_word<true>(words[i]);
        out[i] = __float_as_uint(a) == __float_as_uint(b) ? (double)a : __longlong_as_double(0x7ff8000000000badll);
    }
}

// Branches 0 and 1: every float bit pattern b in [lo, hi) through AS241's
// central branch (Q = b) or its tail (R = b), once with the kernels' division
// and root and once with the IEEE intrinsics.  Branch 2: every high word
// b in [lo, hi) of a raw word, with low words at both ends of the range the
// 32-bit input stage accepts (0x800 and 2^32 - 0x801), at 2^31 and at a hash
// of b: where that stage certifies Q, it must equal the exact stage's Q on
// the central branch.  Counts the disagreements and keeps the smallest b.
__global__ void dbg_as241_check_kernel(uint32_t branch, uint64_t lo, uint64_t hi, unsigned long long *out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long bad = 0;
    uint32_t first = 0xffffffffu;
    for (uint64_t b = lo + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < hi; b += stride) {
        bool differ = false;
        if (branch == 2u) {
            const uint32_t lows[4] = {0x800u, 0xfffff7ffu, 0x80000000u, (uint32_t)b * 2654435761u ^ 0x5bd1e995u};
            for (int k = 0; k < 4; ++k) {
                const uint64_t w = (b << 32) | lows[k];
                float q;
                if (dev::as241_fast_q(w, q)) {
                    const dev::As241In ex = dev::as241_prep(w);
                    differ |= !ex.central || __float_as_uint(q) != __float_as_uint(ex.q);
                }
            }
        } else {
            const float x = __uint_as_float((uint32_t)b);
            const float f = branch == 0u ? dev::as241_central<false>(x) : dev::as241_tail<false>(x, false);
            const float r = branch == 0u ? dev::as241_central<true>(x) : dev::as241_tail<true>(x, false);
            differ = __float_as_uint(f) != __float_as_uint(r);
        }
        if (differ) {
            ++bad;
            first = min(first, (uint32_t)b);
        }
    }
    if (bad != 0) {
        atomicAdd(&out[0], bad);
        atomicMin(&out[1], (unsigned long long)first);
    }
}

__global__ void dbg_limbs_kernel(const double *pay, uint64_t n, bool f32, int E, uint32_t *out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        uint32_t l[kLimbs] = {0, 0, 0, 0, 0, 0};
        const bool ok = f32 ? dev::limbs_add_f32((float)pay[i], E + 103, l) : dev::limbs_add_f64(pay[i], E, l);
        for (int x = 0; x < kLimbs; ++x) out[i * kLimbs + x] = ok ? l[x] : 0xFFFFFFFFu;
    }
}

cudaError_t launch_dbg_words(uint32_t seed, uint32_t stream, uint32_t n_streams, uint32_t n_words, uint64_t *out,
                             cudaStream_t st) {
    dbg_words_kernel<<<(n_streams + 127) / 128, 128, 0, st>>>(seed, stream, n_streams, n_words, out);
    return cudaGetLastError();
}

cudaError_t launch_dbg_draws(uint32_t seed, uint32_t stream, uint32_t n_streams, const uint8_t *kinds, uint32_t n,
                             double *out,
                             cudaStream_t st) {
    const uint32_t bd = 64;
    const size_t smem = (size_t)2 * kRngWords * bd * (sizeof(uint64_t) + sizeof(float)) + (bd / 32) * kWarpScratchBytes;
    dbg_draws_kernel<<<(n_streams + bd - 1) / bd, bd, smem, st>>>(seed, stream, n_streams, kinds, n, out);
    return cudaGetLastError();
}

cudaError_t launch_dbg_limbs(const double *pay, uint64_t n, bool f32, int E, uint32_t *out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    dbg_limbs_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pay, n, f32, E, out);
    return cudaGetLastError();
}

cudaError_t launch_dbg_as241_check(uint32_t branch, uint64_t lo, uint64_t hi, unsigned long long *out,
                                   cudaStream_t st) {
    if (hi <= lo) return cudaSuccess;
    const uint64_t blocks = std::min<uint64_t>((hi - lo + 255) / 256, 152ull * 64);
    dbg_as241_check_kernel<<<(unsigned)blocks, 256, 0, st>>>(branch, lo, hi, out);
    return cudaGetLastError();
}

cudaError_t launch_dbg_normals(const uint64_t *words, uint64_t n, double *out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    dbg_normals_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(words, n, out);
    return cudaGetLastError();
}

} // namespace hexo

namespace hexo {

// ------------------------------------------------------ pipe peak probes
// Eight independent dependency chains per thread keep each pipe busy; the
// result is written only if it is impossible, so the work is not removed.

__global__ void peak_ffma_kernel(int iters, float *sink) {
    float a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = 1.0f + 1e-3f * (threadIdx.x + j);
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = fmaf(a[j], 0.9999f, 1e-4f);
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += a[j];
    if (s == -1.0f) sink[0] = s;
}

__global__ void peak_dfma_kernel(int iters, double *sink) {
    double a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = 1.0 + 1e-3 * (threadIdx.x + j);
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = fma(a[j], 0.9999, 1e-4);
    double s = 0.;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += a[j];
    if (s == -1.0) sink[0] = s;
}

__global__ void peak_mufu_kernel(int iters, float *sink) {
    float a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = 0.5f + 1e-3f * (threadIdx.x + j);
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(a[j]));
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += a[j];
    if (s == -1.0f) sink[0] = s;
}

// The multiplier is a launch argument: with a compile-time constant the
// compiler composes unrolled links of the affine chain into one.
__global__ void peak_int_kernel(int iters, unsigned mul, unsigned *sink) {
    unsigned a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = threadIdx.x * 2654435761u + j;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = a[j] * mul + 1013904223u;
    unsigned s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s ^= a[j];
    if (s == 0xFFFFFFFFu) sink[0] = s;
}

// Two ALU-pipe operations per link: a funnel-shift rotate and an xor.
__global__ void peak_alu_kernel(int iters, unsigned *sink) {
    unsigned a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = threadIdx.x * 2654435761u + j;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = __funnelshift_l(a[j], a[j], 7) ^ 0x9e3779b9u;
    unsigned s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s ^= a[j];
    if (s == 0xFFFFFFFFu) sink[0] = s;
}

// Lane operations per second for {FP32 FMA, FP64 FMA, MUFU ex2, INT32 IMAD,
// INT32 ALU (shift, logic)}.
cudaError_t measure_pipe_peaks(int sm_count, cudaStream_t st, double *out5) {
    void *sink = nullptr;
    cudaError_t e = cudaMalloc(&sink, 64);
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int threads = 256, blocks = sm_count * 8;
    const int iters[5] = {4096, 256, 1024, 4096, 4096};
    const double ops[5] = {1.0, 1.0, 1.0, 1.0, 2.0};   // lane operations per link
    for (int k = 0; k < 5 && e == cudaSuccess; ++k) {
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep) {   // first launch warms up
            cudaEventRecord(a, st);
            switch (k) {
            case 0: peak_ffma_kernel<<<blocks, threads, 0, st>>>(iters[k], (float *)sink); break;
            case 1: peak_dfma_kernel<<<blocks, threads, 0, st>>>(iters[k], (double *)sink); break;
            case 2: peak_mufu_kernel<<<blocks, threads, 0, st>>>(iters[k], (float *)sink); break;
            case 3: peak_int_kernel<<<blocks, threads, 0, st>>>(iters[k], 1664525u, (unsigned *)sink); break;
            case 4: peak_alu_kernel<<<blocks, threads, 0, st>>>(iters[k], (unsigned *)sink); break;
            }
            cudaEventRecord(b, st);
            e = cudaEventSynchronize(b);
            if (e != cudaSuccess) break;
            cudaEventElapsedTime(&ms, a, b);
        }
        out5[k] = (double)blocks * threads * iters[k] * 8.0 * ops[k] / (ms * 1e-3);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    return e;
}

} // namespace hexo
