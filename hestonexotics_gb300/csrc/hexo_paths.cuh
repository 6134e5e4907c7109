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
// reduction (redux.sync) and one global atomic add per limb per warp.
//
// kF32 = false: the plain FP64 form.  kF32 = true: paths evolve in float,
// except the variance, which is kept in double-single so that the scheme's
// branch decisions match FP64 (hexo_ds.cuh); AS241 is float32 in both
// forms, so both consume bit-identical normals.
#pragma once
#include <stdint.h>
#include "hexo_types.h"
#include "hexo_device.cuh"
#include "hexo_ds.cuh"

namespace hexo {


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
    ds::F2 vd;                                  // FP32 form: the variance in double-single (v == vd.h)
};

// The path arithmetic below names every rounding (__fma_rn, __dmul_rn, ...)
// so that the compiler cannot contract or reassociate differently in
// different template instantiations: every launch shape computes the same
// bits for the same path.

// One QE step of one path (HSimulation.tpp:52-86), FP64; returns whether it
// took the quadratic branch.
__device__ __forceinline__ bool qe_step(PathVars<false> &pv, const SegDesc &sg, double theta, dev::Shishua &g,
                                        dev::RngLane &c, const dev::Ring &r, const dev::WarpScratch &ws) {
    dev::DrawPlan dp = dev::draw_prefetch(c, r);
    const double v = pv.v;
    const double m = __fma_rn(__dsub_rn(v, theta), sg.disc, theta);         // tpp:59
    const double sp2 = fabs(__fma_rn(v, sg.cA, sg.cB));                      // tpp:60
    const double mm = __dmul_rn(m, m);
    const bool quad = sp2 < __dmul_rn(1.5, mm);                              // Psi < PSI_C, tpp:61,63
    if (dev::draw_prepare<false>(g, c, r, ws, quad)) dp = dev::draw_prefetch(c, r);
    float z1f = 0.0f, z2f;                                                   // draw order, tpp:67,72,80
    uint64_t uw = 0;
    dev::draw_commit(g, c, r, dp, quad, z1f, uw, z2f);
    const double z1 = (double)z1f;
    const double z2 = (double)z2f;
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
        const double U = dev::uniform_f64(uw);
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
    return quad;
}

// One QE step, FP32 form: the same scheme and draws; the variance in
// double-single (m = v disc + m0 and s^2 = v cA + cB, algebraically the
// reference's tpp:59-60), everything else in float; returns whether it took
// the quadratic branch.
__device__ __forceinline__ bool qe_step(PathVars<true> &pv, const SegDesc &sg, dev::Shishua &g, dev::RngLane &c,
                                        const dev::Ring &r, const dev::WarpScratch &ws, float S0, float rr,
                                        const ds::LogTab *ltab) {
    dev::DrawPlan dp = dev::draw_prefetch(c, r);
    const ds::F2 v = pv.vd;
    const ds::F2 m = ds::fma(v, ds::F2{sg.ds_disc[0], sg.ds_disc[1]}, ds::F2{sg.ds_m0[0], sg.ds_m0[1]});
    const ds::F2 sp2 = ds::fma(v, ds::F2{sg.ds_cA[0], sg.ds_cA[1]}, ds::F2{sg.ds_cB[0], sg.ds_cB[1]});
    const ds::F2 mm = ds::sqr(m);
    // Psi < PSI_C; the float comparison decides unless it is within 2^-20 of the threshold
    const float t15 = __fmul_rn(1.5f, mm.h);
    const bool quad = fabsf(__fsub_rn(sp2.h, t15)) > __fmul_rn(0x1p-20f, sp2.h) ? sp2.h < t15
                                                                                 : ds::less(sp2, ds::mul_f(mm, 1.5f));
    if (dev::draw_prepare<true>(g, c, r, ws, quad)) dp = dev::draw_prefetch(c, r);
    float z1 = 0.0f, z2;
    uint64_t uw = 0;
    dev::draw_commit(g, c, r, dp, quad, z1, uw, z2);
    ds::F2 vn;
    if (quad) {
        const ds::F2 inv = ds::div(ds::F2{__fmul_rn(2.0f, mm.h), __fmul_rn(2.0f, mm.l)}, sp2);   // 2/Psi
        // inv > 4/3, sqrt(inv (inv - 1)) > inv - 1 and bp2 >= 1 order the additions
        const ds::F2 im1 = ds::add_f_ordered(inv, -1.0f);
        const ds::F2 bp2 = ds::add_ordered(ds::sqrt(ds::mul(inv, im1)), im1);
        const ds::F2 b = ds::sqrt(bp2);
        const ds::F2 a = ds::div(m, ds::add_f_ordered(bp2, 1.0f));
        const ds::F2 zb = ds::add_f(b, z1);
        vn = ds::mul(ds::mul(a, zb), zb);
    } else {
        const float Psi = __fdividef(sp2.h, mm.h);
        const float pp1 = __fadd_rn(Psi, 1.0f);
        const float p = __fdividef(__fsub_rn(Psi, 1.0f), pp1);
        // U = w 2^-64 to float accuracy from the two 32-bit halves
        const uint32_t whi = (uint32_t)(uw >> 32), wlo = (uint32_t)uw;
        const float U = __fmaf_rn(__uint2float_rn(wlo), 0x1p-64f, __fmul_rn(__uint2float_rn(whi), 0x1p-32f));
        // p < U sends the variance to 0 or not: decided in float when the two
        // are further apart than float error (2^-19 relative), else exactly as
        // the FP64 form decides it (rare: a few 1e-5 of these steps), so that
        // the path does not take the other branch than in FP64
        bool take = p < U;
        if (fabsf(__fsub_rn(p, U)) <= __fmul_rn(0x1p-17f, __fadd_rn(p, U))) {
            const double Pd = __ddiv_rn(__dadd_rn((double)sp2.h, (double)sp2.l), __dadd_rn((double)mm.h, (double)mm.l));
            take = __ddiv_rn(__dsub_rn(Pd, 1.0), __dadd_rn(Pd, 1.0)) < dev::uniform_f64(uw);
        }
        // v = log((1-p)/(1-U)) / beta, in double-single like the quadratic
        // branch (a float-size error here would move later branch decisions).
        // With Y = (s^2 + m^2) / (2 m^2) = 1/(1-p) = 1/(beta m):
        // v = -m Y log(Y (1 - U)), 1 - U = (2^64 - w) 2^-64 from the whole word
        vn = ds::F2{0.0f, 0.0f};
        if (take) {
            const ds::F2 Y = ds::div(ds::add(sp2, mm), ds::F2{__fmul_rn(2.0f, mm.h), __fmul_rn(2.0f, mm.l)});
            const ds::F2 v1 = ds::mul(ds::mul(m, Y), ds::neg(ds::log(ds::mul(Y, ds::from_u64_2m64(0ull - uw)), ltab)));
            if (v1.h > 0.0f) vn = v1;
        }
    }
    pv.vd = vn;
    pv.v = vn.h;
    // K1 v + K2 vn = c (v + vn) + (rho/sigma)(vn - v): the second part
    // telescopes over the steps, so it is not accumulated in float (its
    // rounding would add up step after step); lx = log X - log S0 - r v.
    float inc = __fmaf_rn(sg.f_c, __fadd_rn(v.h, vn.h), sg.f_K0);
    inc = __fmaf_rn(fsqrt_fast(__fmaf_rn(sg.f_K3, v.h, __fmul_rn(sg.f_K4, vn.h))), z2, inc);
    pv.lx = __fadd_rn(pv.lx, inc);
    pv.Xp = pv.X;
    pv.X = __fmul_rn(S0, __expf(__fmaf_rn(rr, vn.h, pv.lx)));
    return quad;
}

__device__ __forceinline__ float add_r(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_r(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float fma_r(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_r(double a, double b, double c) { return __fma_rn(a, b, c); }

// A CTA takes one tile (blockDim * PPT consecutive paths) at a time, so its
// warps read the same set's descriptors (shared through L1); thread t holds
// paths begin + p * blockDim + t.  A tile prices its set's options in
// increasing (maturity-sorted) index order.  Each warp's sums (redux.sync)
// are stored, without atomics, in the warp's own window of kWindow
// consecutive options (one 32-bit value per option and limb, written once per
// tile); the windows are summed and flushed to this CTA's private copy of the
// global sums only when an option falls past the window and at the end of the
// tile, so the warps meet at a barrier a few times per tile rather than at
// every maturity (measured on the uneven batch: 12 % faster than a flush per
// maturity; the per-warp windows another 4 %, 17 % on a 100-strike chain).
constexpr uint32_t kWindow = 64;

// Folds the call payoffs (AsianContract.h:43-47, VanillaContract.h:37-39) of
// option oi of this warp's paths into the warp's window entry wslot: exact
// limbs per path, one warp sum per limb (redux.sync), stored by lane 0.  A
// warp whose payoffs are all 0 leaves its (cleared) window entry as it is.
// With the control variate (kCV), kind 2 folds the geometric-average call
// (G - K)^+ and kind 3 the signed difference (A - K)^+ - (G - K)^+, whose
// biased limbs are written for every counted path.
template <bool kF32, int PPT, bool kCV>
__device__ __forceinline__ void fold_option(const KernelArgs &a, const SetDesc &S, uint32_t oi, uint32_t *wslot,
                                            uint32_t lane, const bool (&active)[PPT], const uint64_t (&kpath)[PPT],
                                            const typename Real<kF32>::T (&asian)[PPT],
                                            const typename Real<kF32>::T (&euro)[PPT],
                                            const typename Real<kF32>::T (&geo)[PPT]) {
    const OptDesc &O = a.opts[S.opt_begin + oi];
    uint32_t l[kLimbs] = {0, 0, 0, 0, 0, 0};
    bool ok = true, any = false;
    const uint32_t kind = O.kind;
    const int E = S.pay_exp, eoff = S.pay_exp + 103;   // payoffs in units of 2^E
#pragma unroll
    for (int p = 0; p < PPT; ++p) {
        if (active[p] && kpath[p] < O.n_paths) {
            if constexpr (kF32) {
                const float K = O.f_strike;
                if (kCV && kind == 3u) {
                    const float d = __fsub_rn(fmaxf(0.0f, __fsub_rn(asian[p], K)), fmaxf(0.0f, __fsub_rn(geo[p], K)));
                    any = true;   // every counted path adds its 2^63 bias, zero or not
                    ok &= dev::limbs_add_signed_f32(d, eoff, l);
                } else {
                    const float f = kind == 0u ? asian[p] : (kCV && kind == 2u) ? geo[p] : euro[p];
                    const float pay = fmaxf(0.0f, __fsub_rn(f, K));
                    any |= pay != 0.0f;
                    ok &= dev::limbs_add_f32(pay, eoff, l);
                }
            } else {
                const double K = O.strike;
                if (kCV && kind == 3u) {
                    const double d = __dsub_rn(fmax(0.0, __dsub_rn(asian[p], K)), fmax(0.0, __dsub_rn(geo[p], K)));
                    any = true;   // every counted path adds its 2^63 bias, zero or not
                    ok &= dev::limbs_add_signed_f64(d, E, l);
                } else {
                    const double f = kind == 0u ? asian[p] : (kCV && kind == 2u) ? geo[p] : euro[p];
                    const double pay = fmax(0.0, __dsub_rn(f, K));
                    any |= pay != 0.0;
                    ok &= dev::limbs_add_f64(pay, E, l);
                }
            }
        }
    }
    if (!ok) atomicOr(a.error, 1);
    if (__any_sync(0xffffffffu, any)) {
        uint32_t sum[kLimbs];
#pragma unroll
        for (int x = 0; x < kLimbs; ++x) sum[x] = __reduce_add_sync(0xffffffffu, l[x]);
        if (lane == 0u) {   // once per option and tile; 8-byte aligned (24 B per option)
            uint2 *w = reinterpret_cast<uint2 *>(wslot);
            w[0] = make_uint2(sum[0], sum[1]);
            w[1] = make_uint2(sum[2], sum[3]);
            w[2] = make_uint2(sum[4], sum[5]);
        }
    }
}

template <bool kF32, int PPT, int UNROLL, bool kCV = false>
__global__ void __launch_bounds__(512) paths_kernel(const KernelArgs a) {
    typedef typename Real<kF32>::T R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t bd = blockDim.x, tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    // shared memory: raw words, normals, per-warp conversion scratch
    uint64_t *raw_all = reinterpret_cast<uint64_t *>(smem_raw);
    float *nrm_all = reinterpret_cast<float *>(raw_all + (size_t)PPT * 2 * kRngWords * bd);
    uint16_t *tq_i_all = reinterpret_cast<uint16_t *>(nrm_all + (size_t)PPT * 2 * kRngWords * bd);
    uint32_t *win = reinterpret_cast<uint32_t *>(
        smem_raw + ((size_t)PPT * 2 * kRngWords * bd * 12 + (size_t)(bd >> 5) * kWarpScratchBytes + 15) / 16 * 16);
    // double-single log table of the FP32 form's exponential branch, after the windows
    ds::LogTab *ltab = reinterpret_cast<ds::LogTab *>(win + (size_t)(bd >> 5) * kWindow * kLimbs);
    if constexpr (kF32) ds::log_table_init(ltab, tid, bd);   // visible after the first tile's barrier

    dev::Ring ring[PPT];
    dev::WarpScratch ws[PPT];
#pragma unroll
    for (int p = 0; p < PPT; ++p) {
        ring[p].raw = raw_all + (size_t)p * 2 * kRngWords * bd + tid;
        ring[p].nrm = nrm_all + (size_t)p * 2 * kRngWords * bd + tid;
        ring[p].stride = bd;
        ws[p].raw0 = ring[p].raw - lane;
        ws[p].nrm0 = ring[p].nrm - lane;
        ws[p].tq_i = tq_i_all + warp * kConvQueue;
        ws[p].lane = lane;
#ifdef HEXO_CHECKS
        ws[p].error = a.error;
        ws[p].check = a.check;
#endif
    }
    __shared__ uint32_t s_tile;
    // this CTA's private copy of the sums: CTAs never contend for one address
    unsigned long long *const acc = a.acc + (size_t)(blockIdx.x % a.n_slots) * a.acc_slot_stride;
    const uint32_t n_warps = bd >> 5;
    for (uint32_t i = tid; i < n_warps * kWindow * kLimbs; i += bd) win[i] = 0u;
    uint32_t *const wwin = win + warp * kWindow * kLimbs;   // this warp's window: one u32 per option and limb
    // adds the warps' window sums for set options [base, base + kWindow) to the global copy and clears them
    auto flush = [&](const SetDesc &S, uint32_t base) {
        __syncthreads();
        for (uint32_t i = tid; i < kWindow * kLimbs; i += bd) {
            unsigned long long v = 0ull;
            for (uint32_t w = 0; w < n_warps; ++w) {
                v += win[w * kWindow * kLimbs + i];
                win[w * kWindow * kLimbs + i] = 0u;
            }
            if (v != 0ull) {
                const uint32_t oi = S.opt_begin + base + i / kLimbs;
                if (HEXO_CHECK(oi < a.n_opts, a.error, a.check, kCheckOpt, oi)) {
                    const OptDesc &O = a.opts[oi];
                    if (HEXO_CHECK(O.out_index < a.n_out, a.error, a.check, kCheckOut, O.out_index))
                        atomicAdd(&acc[(size_t)O.out_index * kLimbs + i % kLimbs], v);
                }
            }
        }
        __syncthreads();
    };

    for (;;) {
        if (tid == 0) s_tile = atomicAdd(a.queue, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        __syncthreads();
        if (tile >= a.n_tiles) break;
        const TileDesc td = a.tiles[tile];
        if (!HEXO_CHECK(td.set < a.n_sets, a.error, a.check, kCheckSet, tile)) continue;   // CTA-uniform skips
        const SetDesc &S = a.sets[td.set];
        if (!HEXO_CHECK((uint64_t)S.seg_begin + td.seg_count <= a.n_segs && td.seg_count <= S.seg_count, a.error,
                        a.check, kCheckSegs, td.set))
            continue;
        const double theta = S.theta;
        const float S0f = S.f_S0, rf = S.f_r;
        uint32_t win_base = 0;   // first set option of the staging window

        dev::Shishua g[PPT];
        dev::RngLane c[PPT];
        PathVars<kF32> pv[PPT];
        // control variate: y = log(X / S0) now and one step back, and the
        // Asian contract's trapezoid sum on y (the geometric average's log)
        R yc[PPT], yp[PPT], accg[PPT];
        uint64_t kpath[PPT];
        bool active[PPT];
#pragma unroll
        for (int p = 0; p < PPT; ++p) {
            kpath[p] = td.path_begin + (uint64_t)p * bd + tid;
            active[p] = kpath[p] < S.n_paths;
            dev::rng_start<kF32>(g[p], c[p], ring[p], ws[p], S.seed + (uint32_t)kpath[p], S.stream);
            pv[p].vd = ds::F2{S.ds_v0[0], S.ds_v0[1]};
            pv[p].lx = kF32 ? (R)(-(float)S.f_r * S.f_v0) : (R)S.logS0;   // FP32: log X - log S0 - (rho/sigma) v
            pv[p].v = kF32 ? (R)S.f_v0 : (R)S.v0;
            pv[p].X = kF32 ? (R)S.f_S0 : (R)S.S0;
            pv[p].Xp = pv[p].X;
            pv[p].acc = (R)0;
            yc[p] = yp[p] = accg[p] = (R)0;
        }

        for (uint32_t si = 0; si < td.seg_count; ++si) {
            const SegDesc sg = a.segs[S.seg_begin + si];
            const R hdt = kF32 ? (R)sg.f_hdt : (R)sg.hdt;
            // every step, then the trapezoid with this width except after the
            // last (pricing) step; one copy of the step code
#pragma unroll UNROLL
            for (uint32_t st = 1; st <= sg.n_steps; ++st) {
#pragma unroll
                for (int p = 0; p < PPT; ++p) {
                    if constexpr (kF32) qe_step(pv[p], sg, g[p], c[p], ring[p], ws[p], S0f, rf, ltab);
                    else qe_step(pv[p], sg, theta, g[p], c[p], ring[p], ws[p]);
                    if constexpr (kCV) {
                        yp[p] = yc[p];   // FP32: the exponent of X / S0 that qe_step used
                        if constexpr (kF32) yc[p] = __fmaf_rn(rf, pv[p].v, pv[p].lx);
                        else yc[p] = __dsub_rn(pv[p].lx, S.logS0);
                    }
                    if (st < sg.n_steps) {
                        pv[p].acc = fma_r(hdt, add_r(pv[p].X, pv[p].Xp), pv[p].acc);
                        if constexpr (kCV) accg[p] = fma_r(hdt, add_r(yc[p], yp[p]), accg[p]);
                    }
                }
            }
            for (uint32_t mj = sg.mat_begin; mj < sg.mat_end; ++mj) {
                if (!HEXO_CHECK(S.mat_begin + mj < a.n_mats && mj < S.mat_count, a.error, a.check, kCheckMat, mj))
                    continue;
                const MatDesc M = a.mats[S.mat_begin + mj];
                if (!HEXO_CHECK(M.opt_end <= S.opt_count && (uint64_t)S.opt_begin + M.opt_end <= a.n_opts, a.error,
                                a.check, kCheckOpt, M.opt_end))
                    continue;
                R asian[PPT], euro[PPT], geo[PPT];
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
                    geo[p] = (R)0;
                    if constexpr (kCV) {   // G = S0 exp(L), L the Asian weights on y
                        if constexpr (kF32) {
                            const float L = __fmul_rn(__fadd_rn(accg[p], __fmul_rn(__fsub_rn(yc[p], yp[p]), M.f_w)),
                                                      M.f_invT);
                            geo[p] = __fmul_rn(S0f, expf(L));
                        } else {
                            const double L = __ddiv_rn(
                                __dadd_rn(accg[p], __ddiv_rn(__dmul_rn(__dsub_rn(yc[p], yp[p]), M.tmtp), M.dt)), M.T);
                            geo[p] = __dmul_rn(S.S0, exp(L));
                        }
                    }
                    if (a.dbg_asian != nullptr && active[p]) {
                        const size_t at = (size_t)(kpath[p] - a.dbg_lo) * a.dbg_mats + mj;
                        a.dbg_asian[at] = (double)asian[p];
                        a.dbg_euro[at] = (double)euro[p];
                    }
                }
                // payoffs of the maturity's options, staged in the warp's window
                for (uint32_t oi = M.opt_begin; oi < M.opt_end; ++oi) {
                    if (oi >= win_base + kWindow) {           // CTA-uniform: all warps price the same options
                        flush(S, win_base);
                        win_base = oi - oi % kWindow;
                    }
                    if (!HEXO_CHECK(oi - win_base < kWindow, a.error, a.check, kCheckWindow, oi - win_base)) continue;
                    fold_option<kF32, PPT, kCV>(a, S, oi, wwin + (oi - win_base) * kLimbs, lane, active, kpath, asian,
                                                euro, geo);
                }
            }
            const R hda = kF32 ? (R)sg.f_hdt_after : (R)sg.hdt_after;
#pragma unroll
            for (int p = 0; p < PPT; ++p) {
                pv[p].acc = fma_r(hda, add_r(pv[p].X, pv[p].Xp), pv[p].acc);
                if constexpr (kCV) accg[p] = fma_r(hda, add_r(yc[p], yp[p]), accg[p]);
            }
        }
        flush(S, win_base);
        if (a.exp_steps != nullptr) {   // branch mix: each exponential-branch step drew one uniform
            uint32_t n_exp = 0;
#pragma unroll
            for (int p = 0; p < PPT; ++p)
                if (active[p]) n_exp += c[p].n_u;
            const uint32_t we = __reduce_add_sync(0xffffffffu, n_exp);
            if (lane == 0u && we != 0u) atomicAdd(a.exp_steps, (unsigned long long)we);
        }
    }
}

} // namespace hexo
