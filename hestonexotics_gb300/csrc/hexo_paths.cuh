// Persistent Monte Carlo path kernel.
//
// Each CTA repeatedly takes the next tile (set, block of consecutive paths)
// from a global queue and simulates its paths, PPT paths per thread, through
// the set's step schedule up to the last maturity that block needs.  One
// path follows the reference's per-path loop (HSimulation.tpp:30-46):
//   QE step (tpp:52-86)  ->  at a pricing step, the Asian and European final
//   values (AsianContract.h:29-34, VanillaContract.h:28-31) and the call
//   payoffs of every option of that maturity  ->  trapezoid accumulation
//   (AsianContract.h:25-28) with the width in force after the pricing check.
// Payoffs are folded into exact fixed-point limb sums: per option a warp
// reduction (redux.sync), a shared-memory accumulation across the CTA's
// warps, and one global atomic add per limb per CTA.
//
// kF32 = false: the plain FP64 form.  kF32 = true: paths evolve in float
// (log-spot kept relative to log S0); AS241 is float32 in both forms, so
// both forms consume bit-identical normals.
#pragma once
#include <stdint.h>
#include "hexo_types.h"
#include "hexo_device.cuh"

namespace hexo {

constexpr int kPayChunk = 64;   // options reduced per CTA barrier round

// Square root of max(x, 0) from the MUFU reciprocal square root.
__device__ __forceinline__ float fsqrt_fast(float x) {
    const float y = fmaxf(x, 0.0f);
    return __fmul_rn(y, rsqrtf(fmaxf(y, 1e-30f)));
}

template <bool kF32> struct Real;
template <> struct Real<false> { typedef double T; };
template <> struct Real<true> { typedef float T; };

template <bool kF32>
struct PathVars {
    typename Real<kF32>::T lx, v, X, Xp, acc;  // lx: log X (FP64); log X - log S0 - (rho/sigma) v (FP32)
};

// The path arithmetic below names every rounding (__fma_rn, __dmul_rn, ...)
// so that the compiler cannot contract or reassociate differently in
// different template instantiations: every launch shape computes the same
// bits for the same path.

// One QE step of one path (HSimulation.tpp:52-86), FP64.
__device__ __forceinline__ void qe_step(PathVars<false> &pv, const SegDesc &sg, double theta, dev::Shishua &g,
                                        dev::RngCursor &c, uint64_t *base, uint32_t stride) {
    const double v = pv.v;
    const double m = __fma_rn(__dsub_rn(v, theta), sg.disc, theta);         // tpp:59
    const double sp2 = fabs(__fma_rn(v, sg.cA, sg.cB));                      // tpp:60
    const double mm = __dmul_rn(m, m);
    const bool quad = sp2 < __dmul_rn(1.5, mm);                              // Psi < PSI_C, tpp:61,63
    const uint64_t w1 = quad ? dev::rng_next_g(g, c, base, stride) : dev::rng_next_u(g, c, base, stride);
    const uint64_t w2 = dev::rng_next_g(g, c, base, stride);
    const double z1 = (double)dev::as241_word(w1);
    const double z2 = (double)dev::as241_word(w2);
    double vn;
    if (quad) {                                                              // tpp:64-68
        const double inv = __ddiv_rn(__dmul_rn(2.0, mm), sp2);               // 2/Psi
        const double im1 = __dsub_rn(inv, 1.0);
        const double bp2 = __dadd_rn(im1, __dsqrt_rn(__dmul_rn(inv, im1)));
        const double b = __dsqrt_rn(bp2);
        const double a = __ddiv_rn(m, __dadd_rn(1.0, bp2));
        const double zb = __dadd_rn(b, z1);
        vn = __dmul_rn(__dmul_rn(a, zb), zb);
    } else {                                                                 // tpp:70-73
        const double Psi = __ddiv_rn(sp2, mm);
        const double p = __ddiv_rn(__dsub_rn(Psi, 1.0), __dadd_rn(Psi, 1.0));
        const double beta = __ddiv_rn(2.0, __dmul_rn(m, __dadd_rn(Psi, 1.0)));
        const double U = dev::uniform_f64(w1);
        vn = p < U ? __ddiv_rn(log(__ddiv_rn(__dsub_rn(1.0, p), __dsub_rn(1.0, U))), beta) : 0.0;
    }
    pv.v = vn;
    double t = __dadd_rn(pv.lx, sg.K0);                                     // tpp:80
    t = __fma_rn(sg.K1, v, t);
    t = __fma_rn(sg.K2, vn, t);
    const double sd = __dsqrt_rn(__fma_rn(sg.K3, v, __dmul_rn(sg.K4, vn)));
    pv.lx = __fma_rn(sd, z2, t);
    pv.Xp = pv.X;
    pv.X = exp(pv.lx);                                                       // tpp:82
}

// One QE step, FP32 form: the same scheme and draws with float state.
__device__ __forceinline__ void qe_step(PathVars<true> &pv, const SegDesc &sg, float theta, dev::Shishua &g,
                                        dev::RngCursor &c, uint64_t *base, uint32_t stride, float S0, float r) {
    const float v = pv.v;
    const float m = __fmaf_rn(__fsub_rn(v, theta), sg.f_disc, theta);
    const float sp2 = fabsf(__fmaf_rn(v, sg.f_cA, sg.f_cB));
    const float mm = __fmul_rn(m, m);
    const bool quad = sp2 < __fmul_rn(1.5f, mm);
    const uint64_t w1 = quad ? dev::rng_next_g(g, c, base, stride) : dev::rng_next_u(g, c, base, stride);
    const uint64_t w2 = dev::rng_next_g(g, c, base, stride);
    const float z1 = dev::as241_word(w1);
    const float z2 = dev::as241_word(w2);
    float vn;
    if (quad) {
        const float inv = __fdividef(__fmul_rn(2.0f, mm), sp2);
        const float im1 = __fsub_rn(inv, 1.0f);
        const float bp2 = __fadd_rn(im1, fsqrt_fast(__fmul_rn(inv, im1)));
        const float b = fsqrt_fast(bp2);
        const float a = __fdividef(m, __fadd_rn(1.0f, bp2));
        const float zb = __fadd_rn(b, z1);
        vn = __fmul_rn(__fmul_rn(a, zb), zb);
    } else {
        const float Psi = __fdividef(sp2, mm);
        const float pp1 = __fadd_rn(Psi, 1.0f);
        const float p = __fdividef(__fsub_rn(Psi, 1.0f), pp1);
        bool ovf;
        const uint64_t W = dev::rn53(w1, &ovf);                    // U = W 2^-64, 1 - U = (2^64 - W) 2^-64
        const float U = ovf ? 1.0f : __fmul_rn(__ull2float_rn(W), 0x1p-64f);
        const float omU = ovf ? 0.0f : (W == 0 ? 1.0f : __fmul_rn(__ull2float_rn(0ull - W), 0x1p-64f));
        // v = log((1-p)/(1-U)) / beta with 1-p = 2/(Psi+1), 1/beta = m (Psi+1) / 2; never below 0
        const float lr = __logf(__fdividef(__fdividef(2.0f, pp1), omU));
        vn = p < U ? fmaxf(0.0f, __fmul_rn(__fmul_rn(__fmul_rn(0.5f, m), pp1), lr)) : 0.0f;
    }
    pv.v = vn;
    // K1 v + K2 vn = c (v + vn) + (rho/sigma)(vn - v): the second part
    // telescopes over the steps, so it is not accumulated in float (its
    // rounding would add up step after step); lx = log X - log S0 - r v.
    float inc = __fmaf_rn(sg.f_c, __fadd_rn(v, vn), sg.f_K0);
    inc = __fmaf_rn(fsqrt_fast(__fmaf_rn(sg.f_K3, v, __fmul_rn(sg.f_K4, vn))), z2, inc);
    pv.lx = __fadd_rn(pv.lx, inc);
    pv.Xp = pv.X;
    pv.X = __fmul_rn(S0, __expf(__fmaf_rn(r, vn, pv.lx)));
}

__device__ __forceinline__ float add_r(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_r(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float fma_r(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_r(double a, double b, double c) { return __fma_rn(a, b, c); }

template <bool kF32, int PPT, int UNROLL>
__global__ void __launch_bounds__(512) paths_kernel(const KernelArgs a) {
    typedef typename Real<kF32>::T R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t bd = blockDim.x, tid = threadIdx.x, lane = tid & 31u;
    uint64_t *ring = reinterpret_cast<uint64_t *>(smem_raw);
    unsigned long long *scratch =
        reinterpret_cast<unsigned long long *>(ring + (size_t)PPT * kRingSlots * kRngWords * bd);
    __shared__ uint32_t s_tile;

    for (uint32_t i = tid; i < (uint32_t)(kPayChunk * kLimbs); i += bd) scratch[i] = 0ull;

    for (;;) {
        if (tid == 0) s_tile = atomicAdd(a.queue, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        __syncthreads();
        if (tile >= a.n_tiles) break;
        const TileDesc td = a.tiles[tile];
        const SetDesc &S = a.sets[td.set];
        const R theta = kF32 ? (R)S.f_theta : (R)S.theta;
        const float S0f = S.f_S0, rf = S.f_r;

        dev::Shishua g[PPT];
        dev::RngCursor c[PPT];
        PathVars<kF32> pv[PPT];
        uint64_t kpath[PPT];
        bool active[PPT];
#pragma unroll
        for (int p = 0; p < PPT; ++p) {
            kpath[p] = td.path_begin + (uint64_t)p * bd + tid;
            active[p] = kpath[p] < S.n_paths;
            uint64_t *base = ring + (size_t)p * kRingSlots * kRngWords * bd + tid;
            dev::rng_start(g[p], c[p], base, bd, S.seed + (uint32_t)kpath[p]);
            pv[p].lx = kF32 ? (R)(-(float)S.f_r * S.f_v0) : (R)S.logS0;   // FP32: log X - log S0 - (rho/sigma) v
            pv[p].v = kF32 ? (R)S.f_v0 : (R)S.v0;
            pv[p].X = kF32 ? (R)S.f_S0 : (R)S.S0;
            pv[p].Xp = pv[p].X;
            pv[p].acc = (R)0;
        }

        for (uint32_t si = 0; si < td.seg_count; ++si) {
            const SegDesc sg = a.segs[S.seg_begin + si];
            const R hdt = kF32 ? (R)sg.f_hdt : (R)sg.hdt;
            // all steps but the last: step, then trapezoid with this width
#pragma unroll UNROLL
            for (uint32_t st = 1; st < sg.n_steps; ++st) {
#pragma unroll
                for (int p = 0; p < PPT; ++p) {
                    uint64_t *base = ring + (size_t)p * kRingSlots * kRngWords * bd + tid;
                    dev::rng_topup(g[p], c[p], base, bd);
                    if constexpr (kF32) qe_step(pv[p], sg, theta, g[p], c[p], base, bd, S0f, rf);
                    else qe_step(pv[p], sg, theta, g[p], c[p], base, bd);
                    pv[p].acc = fma_r(hdt, add_r(pv[p].X, pv[p].Xp), pv[p].acc);
                }
            }
            // the pricing step
#pragma unroll
            for (int p = 0; p < PPT; ++p) {
                uint64_t *base = ring + (size_t)p * kRingSlots * kRngWords * bd + tid;
                dev::rng_topup(g[p], c[p], base, bd);
                if constexpr (kF32) qe_step(pv[p], sg, theta, g[p], c[p], base, bd, S0f, rf);
                else qe_step(pv[p], sg, theta, g[p], c[p], base, bd);
            }
            for (uint32_t mj = sg.mat_begin; mj < sg.mat_end; ++mj) {
                const MatDesc M = a.mats[S.mat_begin + mj];
                R asian[PPT], euro[PPT];
#pragma unroll
                for (int p = 0; p < PPT; ++p) {
                    R interp;
                    if constexpr (kF32) {
                        interp = __fmul_rn(__fsub_rn(pv[p].X, pv[p].Xp), M.f_w);
                        asian[p] = __fmul_rn(__fadd_rn(pv[p].acc, interp), M.f_invT);
                    } else {                                               // AsianContract.h:30-32
                        interp = __ddiv_rn(__dmul_rn(__dsub_rn(pv[p].X, pv[p].Xp), M.tmtp), M.dt);
                        asian[p] = __ddiv_rn(__dadd_rn(pv[p].acc, interp), M.T);
                    }
                    euro[p] = add_r(pv[p].Xp, interp);                     // VanillaContract.h:28-29
                    if (a.dbg_asian != nullptr && active[p]) {
                        const size_t at = (size_t)(kpath[p] - a.dbg_lo) * a.dbg_mats + mj;
                        a.dbg_asian[at] = (double)asian[p];
                        a.dbg_euro[at] = (double)euro[p];
                    }
                }
                for (uint32_t ob = M.opt_begin; ob < M.opt_end; ob += kPayChunk) {
                    const uint32_t n = min((uint32_t)kPayChunk, M.opt_end - ob);
                    for (uint32_t i = 0; i < n; ++i) {
                        const OptDesc O = a.opts[S.opt_begin + ob + i];
                        uint32_t l[kLimbs] = {0, 0, 0, 0, 0, 0};
                        bool ok = true;
#pragma unroll
                        for (int p = 0; p < PPT; ++p) {
                            if (active[p] && kpath[p] < O.n_paths) {
                                if constexpr (kF32) {
                                    const float f = O.kind == 0 ? asian[p] : euro[p];
                                    ok &= dev::limbs_add_f32(fmaxf(0.0f, __fsub_rn(f, O.f_strike)), l);
                                } else {
                                    const double f = O.kind == 0 ? asian[p] : euro[p];
                                    ok &= dev::limbs_add_f64(fmax(0.0, __dsub_rn(f, O.strike)), l);   // AsianContract.h:43-47
                                }
                            }
                        }
                        if (!ok) atomicOr(a.error, 1);
#pragma unroll
                        for (int x = 0; x < kLimbs; ++x) {
                            const uint32_t sum = __reduce_add_sync(0xffffffffu, l[x]);
                            if (lane == 0 && sum != 0u) atomicAdd(&scratch[i * kLimbs + x], (unsigned long long)sum);
                        }
                    }
                    __syncthreads();
                    for (uint32_t idx = tid; idx < n * kLimbs; idx += bd) {
                        const unsigned long long v = scratch[idx];
                        if (v != 0ull) {
                            const OptDesc &O = a.opts[S.opt_begin + ob + idx / kLimbs];
                            atomicAdd(&a.acc[(size_t)O.out_index * kLimbs + idx % kLimbs], v);
                            scratch[idx] = 0ull;
                        }
                    }
                    __syncthreads();
                }
            }
            const R hda = kF32 ? (R)sg.f_hdt_after : (R)sg.hdt_after;
#pragma unroll
            for (int p = 0; p < PPT; ++p) pv[p].acc = fma_r(hda, add_r(pv[p].X, pv[p].Xp), pv[p].acc);
        }
    }
}

} // namespace hexo
