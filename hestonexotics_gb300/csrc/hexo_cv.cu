// Geometric-average control variate (the future idea named in
// HSimulation.h:51), its analytic half: E[(G - K)^+] under the Heston model
// for every Asian option a batch prices with the control variate.
//
// Per path the kernels form L = (sum_k h_k (y_k + y_{k-1}) + (y_n - y_{n-1}) w) / T
// on y = log(X / S0): the Asian contract's own weights (AsianContract.h:25-34,
// its spot-difference term included) on the log-spot, and G = S0 exp(L).
// L = sum_k c_k y_k is linear in the log-spot at the grid times, so its
// characteristic function is a backward recursion of the Heston affine
// solution over the grid steps: with Theta_k = z sum_{j >= k} c_j,
//   E_{t_{k-1}}[exp(Theta_k (y_k - y_{k-1}) + b_k v_k)] = exp(A_k + b_{k-1} v_{k-1}),
// and E[exp(z L)] = exp(sum_k A_k + b_0 v0).  The call follows from Lewis's
// single integral (F = E[G], k = log(F / K)):
//   E[(G - K)^+] = F - sqrt(F K) / pi  int_0^inf Re[e^{iuk} E[e^{(iu + 1/2)(L - log(F/S0))}]] / (u^2 + 1/4) du,
// evaluated with Gauss-Legendre on [0, U] (256 nodes) and, through u = U / s,
// on [U, inf) (128 nodes), U = 40 standard deviations of L.
//
// One thread per (maturity, node) runs the recursion in FP64 complex
// arithmetic; one thread per option then sums the nodes.  Done once when a
// batch is uploaded; the finaliser combines it with the path sums.
#include <cuda_runtime.h>
#include <math.h>
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>
#include "hexo_plan.h"
#include "hexo_launch.h"

namespace hexo {

namespace {

constexpr int kCvNodesNear = 256, kCvNodesTail = 128;
constexpr int kCvNodes = kCvNodesNear + kCvNodesTail;
constexpr double kCvRange = 40.0;
// A parameter set with at most this many control-variate maturities runs
// their recursions one warp per (maturity, node) (cv_cf_warp_kernel): alone,
// its few thousand pairs could not fill the GPU one thread each.  The choice
// depends on the set only, never on the batch around it, so a request's
// prices stay the same bits in any batch.
constexpr uint32_t kCvWarpMats = 32;

struct CvMat {                     // one (set, maturity) with control-variate options
    uint32_t step_begin, n_steps;  // its grid steps: (dt, c) in the step array
    double U;                      // integration scale
    double v0, kappa, theta, sigma, rho, mu, S0;
};
struct CvOpt {
    uint32_t mat, out;             // CvMat index; output slot of the Asian option
    double K;
};

struct cd { double x, y; };
__device__ __forceinline__ cd cadd(cd a, cd b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cd csub(cd a, cd b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cd cmul(cd a, cd b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cd cscale(cd a, double s) { return {a.x * s, a.y * s}; }
__device__ __forceinline__ cd cdiv(cd a, cd b) {   // one FP64 division (slow on this GPU) per quotient
    const double d = 1.0 / (b.x * b.x + b.y * b.y);
    return {(a.x * b.x + a.y * b.y) * d, (a.y * b.x - a.x * b.y) * d};
}
__device__ __forceinline__ cd cexp(cd a) {
    double s, c;
    sincos(a.y, &s, &c);
    const double e = exp(a.x);
    return {e * c, e * s};
}
__device__ __forceinline__ cd clog(cd a) { return {log(hypot(a.x, a.y)), atan2(a.y, a.x)}; }
__device__ __forceinline__ cd csqrt(cd a) {   // principal branch
    const double r = hypot(a.x, a.y);
    if (r == 0.0) return {0.0, 0.0};
    const double t = sqrt(0.5 * (r + fabs(a.x)));
    return a.x >= 0.0 ? cd{t, a.y / (2.0 * t)} : cd{fabs(a.y) / (2.0 * t), copysign(t, a.y)};
}

// The Heston affine solution over tau with terminal exponent b:
// E_t[exp(a (y_T - y_t) + b v_T)] = exp(A + B v_t) ("little trap" form).
__device__ __forceinline__ void heston_affine(cd a, cd b, double tau, const CvMat &m, cd &A, cd &B) {
    const double s2 = m.sigma * m.sigma;
    const cd beta = {m.kappa - m.rho * m.sigma * a.x, -m.rho * m.sigma * a.y};
    const cd am1 = {a.x - 1.0, a.y};
    cd D = csqrt(csub(cmul(beta, beta), cscale(cmul(a, am1), s2)));
    if (D.x < 0.0) D = {-D.x, -D.y};
    const cd s2b = cscale(b, s2);
    const cd g = cdiv(csub(csub(beta, D), s2b), csub(cadd(beta, D), s2b));
    const cd e = cexp(cscale(D, -tau));
    const cd ge = cmul(g, e);
    const cd one_ge = {1.0 - ge.x, -ge.y};
    B = cdiv(csub(csub(beta, D), cmul(cadd(beta, D), ge)), cscale(one_ge, s2));
    const cd lg = clog(cdiv(one_ge, cd{1.0 - g.x, -g.y}));
    const cd inner = csub(cscale(csub(beta, D), tau), cscale(lg, 2.0));
    A = cadd(cscale(a, m.mu * tau), cscale(inner, m.kappa * m.theta / s2));
}

// phi[m * (kCvNodes + 1) + i] = E[exp(z L)], z = 1/2 + i U x_i for the nodes
// and z = 1 (E[G] / S0) at i = kCvNodes.
__global__ void cv_cf_kernel(const CvMat *__restrict__ mats, uint32_t mat0, uint32_t n_mats,
                             const double2 *__restrict__ steps, const double2 *__restrict__ nodes,
                             double2 *__restrict__ phi) {
    const uint32_t t = mat0 * (kCvNodes + 1) + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (mat0 + n_mats) * (uint32_t)(kCvNodes + 1)) return;
    const uint32_t mi = t / (kCvNodes + 1), i = t % (kCvNodes + 1);
    const CvMat m = mats[mi];
    const cd z = i == (uint32_t)kCvNodes ? cd{1.0, 0.0} : cd{0.5, m.U * nodes[i].x};
    cd Asum = {0.0, 0.0}, b = {0.0, 0.0}, Th = {0.0, 0.0};
    for (uint32_t k = m.n_steps; k-- > 0;) {
        const double2 s = steps[m.step_begin + k];   // (dt, c)
        Th = cadd(Th, cscale(z, s.y));
        cd A, B;
        heston_affine(Th, b, s.x, m, A, B);
        Asum = cadd(Asum, A);
        b = B;
    }
    const cd r = cexp(cadd(Asum, cscale(b, m.v0)));
    phi[t] = make_double2(r.x, r.y);
}

// The same recursion for one (maturity, node) per warp, for requests too
// small to fill the GPU with one thread per pair (each SM's FP64 pipe then
// serves a single warp that walks every grid step in turn).  Over a fixed
// step, heston_affine's B is a Moebius map of the terminal exponent b:
//   B(b) = (M00 b + M01) / (M10 b + M11),  e = exp(-D tau),
//   M = [[(beta + D) e - (beta - D), a (a - 1) (1 - e)], [s2 (e - 1), (beta + D) - (beta - D) e]]
// ((beta - D)(beta + D) = s2 a (a - 1) by the definition of D).  Lane l
// takes a block of consecutive steps; one warp scan gives every block the
// sum of the c_j after it and the product of the later blocks' maps, whose
// value at b = 0 is the b entering the block's last step; the lane then runs
// heston_affine backward over its own steps, exactly as the one-thread
// kernel does, and the warp sums the A terms.
__device__ __forceinline__ void mobius(cd a, double tau, const CvMat &m, cd (&M)[4]) {
    const double s2 = m.sigma * m.sigma;
    const cd beta = {m.kappa - m.rho * m.sigma * a.x, -m.rho * m.sigma * a.y};
    const cd aam1 = cmul(a, cd{a.x - 1.0, a.y});
    cd D = csqrt(csub(cmul(beta, beta), cscale(aam1, s2)));
    if (D.x < 0.0) D = {-D.x, -D.y};
    const cd e = cexp(cscale(D, -tau));
    const cd bpd = cadd(beta, D), bmd = csub(beta, D);
    M[0] = csub(cmul(bpd, e), bmd);
    M[1] = cmul(aam1, cd{1.0 - e.x, -e.y});
    M[2] = cscale(cd{e.x - 1.0, e.y}, s2);
    M[3] = csub(bpd, cmul(bmd, e));
}
// X <- X Y, rescaled by a power of two (a Moebius map does not change when
// its matrix is scaled, and the products of many steps would otherwise
// drift out of range).
__device__ __forceinline__ void mobius_mul(cd (&X)[4], const cd (&Y)[4]) {
    cd R[4];
    R[0] = cadd(cmul(X[0], Y[0]), cmul(X[1], Y[2]));
    R[1] = cadd(cmul(X[0], Y[1]), cmul(X[1], Y[3]));
    R[2] = cadd(cmul(X[2], Y[0]), cmul(X[3], Y[2]));
    R[3] = cadd(cmul(X[2], Y[1]), cmul(X[3], Y[3]));
    double mx = 0.0;
    for (int i = 0; i < 4; ++i) mx = fmax(mx, fmax(fabs(R[i].x), fabs(R[i].y)));
    const int ex = mx > 0.0 ? ilogb(mx) : 0;
    for (int i = 0; i < 4; ++i) X[i] = {scalbn(R[i].x, -ex), scalbn(R[i].y, -ex)};
}
__device__ __forceinline__ cd shfl_down_cd(cd v, unsigned d) {
    return {__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d)};
}

__global__ void cv_cf_warp_kernel(const CvMat *__restrict__ mats, uint32_t n_mats, const double2 *__restrict__ steps,
                                  const double2 *__restrict__ nodes, double2 *__restrict__ phi) {
    const uint32_t t = (uint32_t)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31u;
    if (t >= n_mats * (uint32_t)(kCvNodes + 1)) return;   // warp-uniform
    const uint32_t mi = t / (kCvNodes + 1), i = t % (kCvNodes + 1);
    const CvMat m = mats[mi];
    const cd z = i == (uint32_t)kCvNodes ? cd{1.0, 0.0} : cd{0.5, m.U * nodes[i].x};
    const uint32_t per = (m.n_steps + 31u) / 32u, k0 = min(lane * per, m.n_steps), k1 = min(k0 + per, m.n_steps);
    const double2 *st = steps + m.step_begin;
    // the block's own sum of c and product of maps (steps k0 .. k1 - 1, applied last to first)
    double csum = 0.0;
    for (uint32_t k = k0; k < k1; ++k) csum += st[k].y;
    // c after the block: an exclusive suffix sum over the lanes
    double cs = csum;
    for (unsigned d = 1; d < 32u; d <<= 1) {
        const double x = __shfl_down_sync(0xffffffffu, cs, d);
        if (lane + d < 32u) cs += x;
    }
    double c_after = __shfl_down_sync(0xffffffffu, cs, 1);
    if (lane == 31u) c_after = 0.0;
    cd P[4] = {{1.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}, {1.0, 0.0}};
    {
        double C = c_after;
        cd Mk[4];
        for (uint32_t k = k1; k-- > k0;) {   // P = M_k0 ... M_(k1-1)
            C += st[k].y;
            mobius(cscale(z, C), st[k].x, m, Mk);
            cd T[4] = {Mk[0], Mk[1], Mk[2], Mk[3]};
            mobius_mul(T, P);
            for (int q = 0; q < 4; ++q) P[q] = T[q];
        }
    }
    // the later blocks' maps: an inclusive suffix product, then shifted by one lane
    cd S[4] = {P[0], P[1], P[2], P[3]};
    for (unsigned d = 1; d < 32u; d <<= 1) {
        cd X[4];
        for (int q = 0; q < 4; ++q) X[q] = shfl_down_cd(S[q], d);
        if (lane + d < 32u) mobius_mul(S, X);
    }
    cd N[4];
    for (int q = 0; q < 4; ++q) N[q] = shfl_down_cd(S[q], 1);
    cd b = lane == 31u ? cd{0.0, 0.0} : cdiv(N[1], N[3]);   // the later blocks' map at b = 0
    // this block's steps, backward, as the one-thread recursion runs them
    cd Asum = {0.0, 0.0};
    double C = c_after;
    for (uint32_t k = k1; k-- > k0;) {
        C += st[k].y;
        cd A, B;
        heston_affine(cscale(z, C), b, st[k].x, m, A, B);
        Asum = cadd(Asum, A);
        b = B;
    }
    for (unsigned d = 16; d > 0u; d >>= 1) Asum = cadd(Asum, shfl_down_cd(Asum, d));
    if (lane == 0u) {   // lane 0's block is the first: its b is b_0
        const cd r = cexp(cadd(Asum, cscale(b, m.v0)));
        phi[t] = make_double2(r.x, r.y);
    }
}

// eg[out] = E[(G - K)^+] (undiscounted) for each control-variate option:
// one warp per option, its lanes over the quadrature nodes.
__global__ void cv_price_kernel(const CvMat *__restrict__ mats, const CvOpt *__restrict__ opts, uint32_t n_opts,
                                const double2 *__restrict__ nodes, const double2 *__restrict__ phi,
                                double *__restrict__ eg) {
    const uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (q >= n_opts) return;   // warp-uniform
    const CvOpt o = opts[q];
    const CvMat m = mats[o.mat];
    const double2 *ph = phi + (size_t)o.mat * (kCvNodes + 1);
    const double F = m.S0 * ph[kCvNodes].x;
    const double lf = log(F / m.S0), k = log(F / o.K);
    double sum = 0.0;
    for (int i = (int)lane; i < kCvNodes; i += 32) {
        const double u = m.U * nodes[i].x, w = m.U * nodes[i].y;
        const cd z = {0.5, u};
        const cd psi = cmul(cd{ph[i].x, ph[i].y}, cexp(cscale(z, -lf)));
        const cd ek = cexp(cd{0.0, u * k});
        sum += w * cmul(ek, psi).x / (u * u + 0.25);
    }
    for (unsigned d = 16; d > 0u; d >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, d);
    if (lane == 0u) eg[o.out] = F - sqrt(F * o.K) / M_PI * sum;
}

// Gauss-Legendre nodes and weights on [-1, 1] (Newton on P_N).
void gauss_legendre(int N, std::vector<double> &x, std::vector<double> &w) {
    x.assign(N, 0.0);
    w.assign(N, 0.0);
    for (int i = 0; i < (N + 1) / 2; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (N + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1.0, p2 = 0.0;
            for (int k = 1; k <= N; ++k) {
                const double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * k - 1.0) * z * p2 - (k - 1.0) * p3) / k;
            }
            pp = N * (z * p1 - p2) / (z * z - 1.0);
            const double dz = p1 / pp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        x[i] = -z;
        x[N - 1 - i] = z;
        w[i] = w[N - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

// Unit-scale nodes: u = U x, weight U w, on [0, 1] and on [1, inf) via 1 / s.
std::vector<double2> unit_nodes() {
    std::vector<double> x1, w1, x2, w2;
    gauss_legendre(kCvNodesNear, x1, w1);
    gauss_legendre(kCvNodesTail, x2, w2);
    std::vector<double2> n;
    for (int i = 0; i < kCvNodesNear; ++i) n.push_back(make_double2(0.5 * (x1[i] + 1.0), 0.5 * w1[i]));
    for (int i = 0; i < kCvNodesTail; ++i) {
        const double s = 0.5 * (x2[i] + 1.0);
        n.push_back(make_double2(1.0 / s, 0.5 * w2[i] / (s * s)));
    }
    return n;
}

// Grid steps (dt, c) of set s up to set-local maturity j: every step of the
// segments up to the one that prices j; h_k is the segment's half width
// after a non-pricing step and the next segment's after a pricing step.
void cv_schedule(const BatchPlan &bp, uint32_t s, uint32_t j, std::vector<double2> &out, double &U) {
    const SetDesc &sd = bp.sets[s];
    std::vector<double> dts, h;
    for (uint32_t q = 0; q < sd.seg_count; ++q) {
        const SegDesc &g = bp.segs[sd.seg_begin + q];
        const bool last = j >= g.mat_begin && j < g.mat_end;
        for (uint32_t st = 1; st <= g.n_steps; ++st) {
            dts.push_back(g.dt);
            if (st < g.n_steps) h.push_back(g.hdt);
            else if (!last) h.push_back(g.hdt_after);
        }
        if (last) break;
    }
    const MatDesc &md = bp.mats[sd.mat_begin + j];
    const double T = md.T, w = md.tmtp / md.dt;
    const size_t n = dts.size();
    std::vector<double> c(n, 0.0);
    for (size_t k = 1; k < n; ++k) {
        c[k - 1] += h[k - 1];
        if (k >= 2) c[k - 2] += h[k - 1];
    }
    if (n >= 2) c[n - 2] -= w;
    c[n - 1] += w;
    for (double &x : c) x /= T;
    // the scale of L: its variance along the variance's mean path
    const hexo_params &p = bp.set_params[s];
    std::vector<double> Cws(n);
    double Cw = 0.0, var = 0.0, t = 0.0;
    for (size_t k = n; k-- > 0;) { Cw += c[k]; Cws[k] = Cw; }
    for (size_t k = 0; k < n; ++k) {
        const double Ev = p.theta + (p.v0 - p.theta) * std::exp(-p.kappa * t);
        var += Cws[k] * Cws[k] * Ev * dts[k];
        t += dts[k];
    }
    U = kCvRange / std::sqrt(std::max(var, 1e-12));
    for (size_t k = 0; k < n; ++k) out.push_back(make_double2(dts[k], c[k]));
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

} // namespace

void cv_plan(const BatchPlan &bp, CvPlan &cp) {
    cp = CvPlan{};
    cp.eg.assign(bp.n_out, std::nan(""));
    cp.partner.assign(bp.n_out, ~0u);
    std::vector<CvMat> mats;
    std::vector<CvOpt> opts;
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> mat_of;
    // sets with few control-variate maturities first: their recursions run one warp per pair
    std::map<uint32_t, uint32_t> n_mats_of_set;
    {
        std::map<std::pair<uint32_t, uint32_t>, bool> seen;
        for (const BatchPlan::CvLeader &l : bp.cv)
            if (seen.emplace(std::make_pair(l.set, l.mat), true).second) ++n_mats_of_set[l.set];
    }
    std::vector<const BatchPlan::CvLeader *> order;
    for (int pass = 0; pass < 2; ++pass)
        for (const BatchPlan::CvLeader &l : bp.cv)
            if ((n_mats_of_set[l.set] <= kCvWarpMats) == (pass == 0)) order.push_back(&l);
    for (const BatchPlan::CvLeader *lp : order) {
        const BatchPlan::CvLeader &l = *lp;
        cp.partner[l.leader] = l.gslot;
        const auto key = std::make_pair(l.set, l.mat);
        auto it = mat_of.find(key);
        if (it == mat_of.end()) {
            CvMat m{};
            m.step_begin = (uint32_t)cp.steps.size();
            cv_schedule(bp, l.set, l.mat, cp.steps, m.U);
            m.n_steps = (uint32_t)cp.steps.size() - m.step_begin;
            const hexo_params &p = bp.set_params[l.set];
            m.v0 = p.v0; m.kappa = p.kappa; m.theta = p.theta; m.sigma = p.sigma; m.rho = p.rho;
            m.mu = p.r - p.q;
            m.S0 = bp.sets[l.set].S0;
            it = mat_of.emplace(key, (uint32_t)mats.size()).first;
            mats.push_back(m);
            if (n_mats_of_set[l.set] <= kCvWarpMats) ++cp.n_warp_mats;
        }
        opts.push_back(CvOpt{it->second, l.leader, l.strike});
    }
    static const std::vector<double2> kNodes = unit_nodes();   // the same nodes for every batch
    cp.nodes = kNodes;
    cp.n_mats = (uint32_t)mats.size();
    cp.n_opts = (uint32_t)opts.size();
    cp.mats.resize(mats.size() * sizeof(CvMat));
    if (!mats.empty()) std::memcpy(cp.mats.data(), mats.data(), cp.mats.size());
    cp.opts.resize(opts.size() * sizeof(CvOpt));
    if (!opts.empty()) std::memcpy(cp.opts.data(), opts.data(), cp.opts.size());
    cp.bytes = align256(cp.eg.size() * sizeof(double)) + align256(cp.partner.size() * sizeof(uint32_t)) +
               align256(cp.mats.size()) + align256(cp.opts.size()) + align256(cp.steps.size() * sizeof(double2)) +
               align256(cp.nodes.size() * sizeof(double2)) +
               align256((size_t)cp.n_mats * (kCvNodes + 1) * sizeof(double2));
}

cudaError_t cv_run(const CvPlan &cp, void *region, cudaStream_t st, double **eg, uint32_t **partner) {
    char *d = static_cast<char *>(region);
    size_t off = 0;
    auto take = [&](size_t bytes) { char *p = d + off; off += align256(bytes); return p; };
    double *d_eg = reinterpret_cast<double *>(take(cp.eg.size() * sizeof(double)));
    uint32_t *d_partner = reinterpret_cast<uint32_t *>(take(cp.partner.size() * sizeof(uint32_t)));
    CvMat *d_mats = reinterpret_cast<CvMat *>(take(cp.mats.size()));
    CvOpt *d_opts = reinterpret_cast<CvOpt *>(take(cp.opts.size()));
    double2 *d_steps = reinterpret_cast<double2 *>(take(cp.steps.size() * sizeof(double2)));
    double2 *d_nodes = reinterpret_cast<double2 *>(take(cp.nodes.size() * sizeof(double2)));
    double2 *d_phi = reinterpret_cast<double2 *>(take((size_t)cp.n_mats * (kCvNodes + 1) * sizeof(double2)));
    *eg = d_eg;
    *partner = d_partner;
    auto up = [&](void *dst, const void *src, size_t bytes) -> cudaError_t {
        return bytes == 0 ? cudaSuccess : cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    cudaError_t e = up(d_eg, cp.eg.data(), cp.eg.size() * sizeof(double));
    if (e == cudaSuccess) e = up(d_partner, cp.partner.data(), cp.partner.size() * sizeof(uint32_t));
    if (e == cudaSuccess) e = up(d_mats, cp.mats.data(), cp.mats.size());
    if (e == cudaSuccess) e = up(d_opts, cp.opts.data(), cp.opts.size());
    if (e == cudaSuccess) e = up(d_steps, cp.steps.data(), cp.steps.size() * sizeof(double2));
    if (e == cudaSuccess) e = up(d_nodes, cp.nodes.data(), cp.nodes.size() * sizeof(double2));
    if (e != cudaSuccess || cp.n_mats == 0) return e;
    // the recursion is bound by each SM's FP64 pipe: sets with few maturities one warp per
    // (maturity, node) over the steps (about 1.5 times the arithmetic, over 32 lanes), the
    // rest one thread per pair, one warp per block so that the pairs spread over the SMs
    if (cp.n_warp_mats > 0) {
        const uint64_t n_thr = (uint64_t)cp.n_warp_mats * (kCvNodes + 1) * 32u;
        cv_cf_warp_kernel<<<(unsigned)((n_thr + 63) / 64), 64, 0, st>>>(d_mats, cp.n_warp_mats, d_steps, d_nodes,
                                                                       d_phi);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const uint32_t n_thread_mats = cp.n_mats - cp.n_warp_mats;
    if (n_thread_mats > 0) {
        const uint32_t n_pairs = n_thread_mats * (kCvNodes + 1);
        cv_cf_kernel<<<(n_pairs + 31) / 32, 32, 0, st>>>(d_mats, cp.n_warp_mats, n_thread_mats, d_steps, d_nodes,
                                                         d_phi);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const uint64_t n_thr = (uint64_t)cp.n_opts * 32u;
    cv_price_kernel<<<(unsigned)((n_thr + 127) / 128), 128, 0, st>>>(d_mats, d_opts, cp.n_opts, d_nodes, d_phi, d_eg);
    return cudaGetLastError();
}

} // namespace hexo
