// swb_step_impl.cuh -- the fused D2Q9 thin-film step, one CTA per tile.
//
// One launch performs one iteration of the reference's time loop
// (src/simulate.jl:15-22) on a lattice:
//
//   pull-stream  f(t-1)_q(x) = fpost(t-1)_q(x - c_q)        BGKandStream! streaming
//   moments      h, u of f(t-1)                              moments!
//   pressure     p = Π(h) - γ ∇²h on the tile + 1 halo        filmpressure!
//   force        F = -h∇p - slip (+ inclination)              h∇p!, slippage!, inclination!
//   collision    fpost(t)_q = (1-1/τ) f_q + feq_q/τ + S_q     equilibrium!, BGKandStream!
//
// Storage is the reference's own layout: nine SoA population planes,
// column-major (x fastest).  The kernel keeps post-collision populations and
// pulls them at the start of the next step, so a step reads 9 and writes 9
// values per cell; the pressure's radius-2 dependence on h is served from a
// (TX+4)x(TY+4) shared-memory tile of heights computed from the pulled
// populations (halo reads come from L2).
//
// Two arithmetic variants:
//   Literal (Float64): the reference's operations in its association order,
//     compiled with --fmad=false; bit-identical to the CPU oracle.
//   Fast (FP32): the same physics with fewer operations; f0 is stored as
//     h - Σ_{q>0} f_q (using the values as stored) so that storage rounding
//     does not leak mass, plus an optional FP64-measured mass correction.
#pragma once
#include <cuda_fp16.h>

#include <type_traits>

#include "swb_internal.h"

namespace swb {

// ------------------------------------------------------------ storage
// Load policies.  LdNC reads through the non-coherent path (__ldg), valid
// while the populations are read-only for the whole launch: kernels that do
// one time step.  LdCG reads at L2 (__ldcg), which other CTAs' writes reach
// before a grid barrier releases: kernels that do several time steps.
struct LdNC {
    template <class T>
    __device__ __forceinline__ static T ld(const T *p) { return __ldg(p); }
};
struct LdCG {
    template <class T>
    __device__ __forceinline__ static T ld(const T *p) { return __ldcg(p); }
};

template <class L>
struct StoreF64T {
    using real = double;
    static constexpr bool kLiteral = true;
    static constexpr bool kHalf = false;
    __device__ __forceinline__ static double ld(const void *b, int pitch, int q, int i) {
        return L::ld(reinterpret_cast<const double *>(b) + q * pitch + i);
    }
    __device__ __forceinline__ static void st(void *b, int pitch, int q, int i, double v) {
        reinterpret_cast<double *>(b)[q * pitch + i] = v;
    }
};

template <class L>
struct StoreF32T {
    using real = float;
    static constexpr bool kLiteral = false;
    static constexpr bool kHalf = false;
    __device__ __forceinline__ static float ld(const void *b, int pitch, int q, int i) {
        return L::ld(reinterpret_cast<const float *>(b) + q * pitch + i);
    }
    __device__ __forceinline__ static void st(void *b, int pitch, int q, int i, float v) {
        reinterpret_cast<float *>(b)[q * pitch + i] = v;
    }
};

// f0 as an FP32 plane, f1..f8 as FP16 planes holding 2^10 f_q (the scale
// keeps populations of order 1e-5..1e-2 in the normal FP16 range).
template <class L>
struct StoreF16T {
    using real = float;
    static constexpr bool kLiteral = false;
    static constexpr bool kHalf = true;
    static constexpr float kScale = 1024.0f;
    static constexpr float kInv = 1.0f / 1024.0f;
    __device__ __forceinline__ static const __half *hp(const void *b, int pitch) {
        return reinterpret_cast<const __half *>(reinterpret_cast<const float *>(b) + pitch);
    }
    __device__ __forceinline__ static float ld(const void *b, int pitch, int q, int i) {
        if (q == 0) return L::ld(reinterpret_cast<const float *>(b) + i);
        return __half2float(L::ld(hp(b, pitch) + (q - 1) * pitch + i)) * kInv;
    }
    __device__ __forceinline__ static void st(void *b, int pitch, int q, int i, float v) {
        if (q == 0) {
            reinterpret_cast<float *>(b)[i] = v;
        } else {
            __half *h = const_cast<__half *>(hp(b, pitch));
            h[(q - 1) * pitch + i] = __float2half_rn(v * kScale);
        }
    }
};

using StoreF64 = StoreF64T<LdNC>;
using StoreF32 = StoreF32T<LdNC>;
using StoreF16 = StoreF16T<LdNC>;

// ------------------------------------------------------------ launch overlap
// Programmatic dependent launch.  The kernels of a step sequence (step,
// advance; single lattice and batch) are launched with the programmatic
// stream-serialization attribute, so that the next launch is scheduled
// during the tail of the current one instead of after it.  Every such kernel
// begins with grid_dep_wait(): griddepcontrol.wait returns once the previous
// grid has completed and its writes are visible, so nothing is read early.
// A CTA calls grid_dep_launch() when its main work is done (griddepcontrol.
// launch_dependents; an exiting CTA counts as well): the next grid is
// scheduled once every CTA of this one got there, so its CTAs do not hold
// registers and shared memory (and so L1) while this grid's strips run.
// Launched without the attribute, both are no-ops.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch of a kernel that begins with grid_dep_wait(), with the
// programmatic-serialization attribute when launch overlap is on.
template <class... P, class... A>
cudaError_t launch_step(void (*kern)(P...), int grid, int block, cudaStream_t st, A &&...args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = launch_overlap() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<A &&>(args)...);
}

// ------------------------------------------------------------ helpers
__device__ __forceinline__ int wrapc(int x, int L) {
    while (x < 0) x += L;
    while (x >= L) x -= L;
    return x;
}

template <class R>
__device__ __forceinline__ R pow_loop(R x, int n) {  // power_broad (src/pressure.jl:363-369)
    R t = R(1);
    for (int i = 0; i < n; ++i) t *= x;
    return t;
}

__device__ __forceinline__ double cospi_r(double x) { return cospi(x); }
__device__ __forceinline__ float cospi_r(float x) { return cospif(x); }
__device__ __forceinline__ double sinpi_r(double x) { return sinpi(x); }
__device__ __forceinline__ float sinpi_r(float x) { return sinpif(x); }
__device__ __forceinline__ double tanh_r(double x) { return tanh(x); }
__device__ __forceinline__ float tanh_r(float x) { return tanhf(x); }

// kappa prefactor ((1 - cospi θ)(n-1)(m-1))/((n-m) hmin), left to right as
// in src/pressure.jl:141-147.
template <class R>
__device__ __forceinline__ R kappa_of(R theta, int n, int m, R hmin) {
    R a = R(1) - cospi_r(theta);
    a = a * R(n - 1);
    a = a * R(m - 1);
    return a / (R(n - m) * hmin);
}

// κ and cospi(θ) of column x at iteration t of the moving-wettability wave
// θ(x, t) = θ0 + Δθ sinpi(2 (x - v t) / Lx).  Not inlined: the kernels
// evaluate it once per column, and its sinpi / cospi code stays out of their
// register budget.  Every kernel and the measure reduction use this one
// function, so they all see the same values.
template <class R>
struct KapCos {
    R kap, cs;
};
template <class R>
__device__ __noinline__ KapCos<R> wave_kap_cos(R theta0, R dtheta, R v, int x, long long t, int Lx,
                                               int n, int m, R hmin) {
    const R th = theta0 + dtheta * sinpi_r(R(2) * (R(x) - v * R(t)) / R(Lx));
    KapCos<R> r;
    r.kap = kappa_of(th, n, m, hmin);
    r.cs = cospi_r(th);
    return r;
}
template <class R>
__device__ __forceinline__ KapCos<R> wave_at(const StepArgs &a, int x, long long t) {
    return wave_kap_cos<R>(R(a.theta0), R(a.dtheta), R(a.wave_v), x, t, a.Lx, a.n, a.m, R(a.hmin));
}

// Pull the nine populations of cell (gx, gy) from the post-collision buffer:
// f_q(x) = fpost_q(x - c_q), c_q as in src/collide.jl:92-100.
template <class S>
__device__ __forceinline__ void pull9(const void *src, int pitch, int Lx, int gx, int gy,
                                      int gxm, int gxp, int gym, int gyp,
                                      typename S::real ft[9]) {
    const int rc = gy * Lx, rm = gym * Lx, rp = gyp * Lx;
    ft[0] = S::ld(src, pitch, 0, rc + gx);
    ft[1] = S::ld(src, pitch, 1, rc + gxm);
    ft[2] = S::ld(src, pitch, 2, rm + gx);
    ft[3] = S::ld(src, pitch, 3, rc + gxp);
    ft[4] = S::ld(src, pitch, 4, rp + gx);
    ft[5] = S::ld(src, pitch, 5, rm + gxm);
    ft[6] = S::ld(src, pitch, 6, rm + gxp);
    ft[7] = S::ld(src, pitch, 7, rp + gxp);
    ft[8] = S::ld(src, pitch, 8, rp + gxm);
}

// pull9 for a cell whose neighbours need no periodic wrap: one base pointer
// at (gx, gy) and offsets that are the same for every thread of the launch
// (q pitch, ±1 column, ±Lx row), so that each load needs no index arithmetic
// of its own.
template <class S>
__device__ __forceinline__ void pull9_interior(const void *src, int pitch, int Lx, int cell,
                                               typename S::real ft[9]) {
    ft[0] = S::ld(src, pitch, 0, cell);
    ft[1] = S::ld(src, pitch, 1, cell - 1);
    ft[2] = S::ld(src, pitch, 2, cell - Lx);
    ft[3] = S::ld(src, pitch, 3, cell + 1);
    ft[4] = S::ld(src, pitch, 4, cell + Lx);
    ft[5] = S::ld(src, pitch, 5, cell - Lx - 1);
    ft[6] = S::ld(src, pitch, 6, cell - Lx + 1);
    ft[7] = S::ld(src, pitch, 7, cell + Lx + 1);
    ft[8] = S::ld(src, pitch, 8, cell + Lx - 1);
}

// Sum of the eight moving populations (pairwise).
// Packed FP32 pairs: Blackwell's FADD2 / FMUL2 / FFMA2 issue two FP32
// operations as one instruction, each lane rounded like the scalar
// operation, so pairing changes no result bit.  A - B is written
// fma(-1, B, A) (exact).
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    return __ffma2_rn(make_float2(-1.0f, -1.0f), b, a);
}

template <class R>
__device__ __forceinline__ R small8(const R f[9]) {
    return ((f[1] + f[3]) + (f[2] + f[4])) + ((f[5] + f[7]) + (f[6] + f[8]));
}
// FP32: ((f1+f3) + (f5+f7)) + ((f2+f4) + (f6+f8)), two lanes at a time
__device__ __forceinline__ float small8(const float f[9]) {
    const float2 s1 = add2(f2(f[1], f[2]), f2(f[3], f[4]));  // f1+f3, f2+f4
    const float2 s2 = add2(f2(f[5], f[6]), f2(f[7], f[8]));  // f5+f7, f6+f8
    const float2 ss = add2(s1, s2);
    return ss.x + ss.y;
}

// moments! (src/moments.jl:43-51): h and the momentum numerators.
template <bool LIT, class R>
__device__ __forceinline__ void moments9(const R f[9], R &h, R &jx, R &jy) {
    if constexpr (LIT) {
        R s = R(0);
#pragma unroll
        for (int q = 0; q < 9; ++q) s = s + f[q];
        h = s;
        jx = f[1] - f[3] + f[5] - f[6] - f[7] + f[8];
        jy = f[2] - f[4] + f[5] + f[6] - f[7] - f[8];
    } else {
        // differences of opposite pairs, two lanes at a time:
        // jx = ((f1-f3) + (f5-f7)) + (f8-f6), jy = ((f2-f4) + (f5-f7)) + (f6-f8)
        h = f[0] + small8(f);
        const float2 d1 = sub2(f2(f[1], f[2]), f2(f[3], f[4]));
        const float2 d2 = sub2(f2(f[5], f[6]), f2(f[7], f[8]));
        const float2 jj = add2(d1, f2(d2.x, d2.x));
        jx = jj.x - d2.y;
        jy = jj.y + d2.y;
    }
}

// Rounding error of h = f0 + small8(f) (Fast2Sum: exact when |f0| >= |small|,
// which holds for thin-film populations where f0 ~ h dominates).
template <class R>
__device__ __forceinline__ R moments_lo(const R f[9], R h) {
    return small8(f) - (h - f[0]);
}

// a / b: IEEE in Float64 (the reference's rounding); in FP32 arithmetic the
// fast reciprocal-based quotient (<= 2 ulp), whose error is far inside the
// tolerance the FP32 modes are checked against.
__device__ __forceinline__ double qdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float qdiv(float a, float b) { return __fdividef(a, b); }

template <bool LIT, class R>
__device__ __forceinline__ void velocity(R h, R jx, R jy, R &ux, R &uy) {
    if constexpr (LIT) {
        ux = jx / h;
        uy = jy / h;
    } else {
        R inv = qdiv(R(1), h);
        ux = jx * inv;
        uy = jy * inv;
    }
}

// filmpressure! for one cell (src/pressure.jl:141-153).  Neighbour names
// follow the reference: ip = h[i-1,j], im = h[i+1,j], jp = h[i,j-1], ...
template <bool LIT, class R>
__device__ __forceinline__ R pressure_cell(R h, R ip, R jp, R im, R jm, R ipjp, R imjp, R imjm,
                                           R ipjm, R kap, R gamma, R hmin, R hcrit, int n,
                                           int m) {
    R x;
    if constexpr (LIT)
        x = hmin / (h + hcrit);
    else
        x = qdiv(hmin, h + hcrit);
    R pn, pm;
    if (!LIT && n == 9 && m == 3) {
        R x3 = x * x * x;
        pn = x3 * x3 * x3;
        pm = x3;
    } else {
        pn = pow_loop(x, n);
        pm = pow_loop(x, m);
    }
    if constexpr (LIT) {
        R p = -gamma * (kap * (pn - pm));
        R lap = R(2.0 / 3.0) * (((jp + ip) + im) + jm) +
                R(1.0 / 6.0) * (((ipjp + imjp) + imjm) + ipjm) - R(10.0 / 3.0) * h;
        return p - gamma * lap;
    } else {  // -γ (κ (x^n - x^m) + ∇²h), with fused multiply-adds
        const R lap = __fmaf_rn(R(2.0 / 3.0), ((jp + ip) + im) + jm,
                                __fmaf_rn(R(1.0 / 6.0), ((ipjp + imjp) + imjm) + ipjm,
                                          R(-10.0 / 3.0) * h));
        return -gamma * __fmaf_rn(kap, pn - pm, lap);
    }
}

// Gradient stencil of h∇p! / ∇f_simple! (src/forcing.jl:181-184).
template <class R>
__device__ __forceinline__ void grad9(R ip, R jp, R im, R jm, R ipjp, R imjp, R imjm, R ipjm,
                                      R &gx, R &gy) {
    if constexpr (std::is_same<R, float>::value) {
        gx = __fmaf_rn(-1.0f / 3.0f, ip - im, (-1.0f / 12.0f) * (((ipjp - imjp) - imjm) + ipjm));
        gy = __fmaf_rn(-1.0f / 3.0f, jp - jm, (-1.0f / 12.0f) * (((ipjp + imjp) - imjm) - ipjm));
    } else {
        gx = R(-1.0 / 3.0) * (ip - im) - R(1.0 / 12.0) * (((ipjp - imjp) - imjm) + ipjm);
        gy = R(-1.0 / 3.0) * (jp - jm) - R(1.0 / 12.0) * (((ipjp + imjp) - imjm) - ipjm);
    }
}

// equilibrium! for one cell, literal (src/equilibrium.jl:67-114).
template <class R>
__device__ __forceinline__ void feq_literal(R h, R ux, R uy, R g, R fe[9]) {
    const R g0 = R(1.5) * g, w1 = R(1.0 / 9.0), w5 = R(1.0 / 36.0);
    R vsq = ux * ux + uy * uy;
    fe[0] = h * ((R(1) - R(5.0 / 6.0) * g * h) - R(2.0 / 3.0) * vsq);
    fe[1] = w1 * h * (g0 * h + R(3) * ux + R(4.5) * (ux * ux) - R(1.5) * vsq);
    fe[2] = w1 * h * (g0 * h + R(3) * uy + R(4.5) * (uy * uy) - R(1.5) * vsq);
    fe[3] = w1 * h * (g0 * h - R(3) * ux + R(4.5) * (ux * ux) - R(1.5) * vsq);
    fe[4] = w1 * h * (g0 * h - R(3) * uy + R(4.5) * (uy * uy) - R(1.5) * vsq);
    fe[5] = w5 * h * (g0 * h + R(3) * (ux + uy) + R(4.5) * ((ux + uy) * (ux + uy)) - R(1.5) * vsq);
    fe[6] = w5 * h * (g0 * h + R(3) * (uy - ux) + R(4.5) * ((uy - ux) * (uy - ux)) - R(1.5) * vsq);
    fe[7] = w5 * h * (g0 * h - R(3) * (ux + uy) + R(4.5) * ((ux + uy) * (ux + uy)) - R(1.5) * vsq);
    fe[8] = w5 * h * (g0 * h + R(3) * (ux - uy) + R(4.5) * ((ux - uy) * (ux - uy)) - R(1.5) * vsq);
}

// Force source of BGKandStream! (src/collide.jl:80-89).
template <class R>
__device__ __forceinline__ R source(int q, R Fx, R Fy) {
    switch (q) {
        case 1: return R(1.0 / 3.0) * Fx;
        case 2: return R(1.0 / 3.0) * Fy;
        case 3: return -(R(1.0 / 3.0) * Fx);
        case 4: return -(R(1.0 / 3.0) * Fy);
        case 5: return R(1.0 / 24.0) * (Fx + Fy);
        case 6: return R(1.0 / 24.0) * (Fy - Fx);
        case 7: return -(R(1.0 / 24.0) * (Fx + Fy));
        case 8: return R(1.0 / 24.0) * (Fx - Fy);
        default: return R(0);
    }
}

__device__ __forceinline__ unsigned int mix32(unsigned int a, unsigned int b) {
    unsigned int x = a * 0x9E3779B9u ^ (b * 0x85EBCA6Bu + 0x27d4eb2fu);
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}

// v + c with stochastic rounding to the ulp of v: c (a few ulp at most: the
// rounding residues of the cell and its share of the mass correction) is
// rounded down or up to a multiple of ulp(v) with probabilities that make the
// result exact in expectation.  ulp(v) and 1/ulp(v) are powers of two built
// from v's exponent field, so c / ulp is exact.
__device__ __forceinline__ float add_stochastic(float v, float c, unsigned int rnd) {
    const int eu = max(((__float_as_int(v) >> 23) & 0xff) - 23, 1);  // exponent field of ulp(v)
    const float ulp = __int_as_float(eu << 23);
    const float r = c * __int_as_float((254 - eu) << 23);
    const float fl = floorf(r);
    const float u = (float)(rnd >> 8) * (1.0f / 16777216.0f);
    const float k = fl + ((u < r - fl) ? 1.0f : 0.0f);
    return __fmaf_rn(k, ulp, v);
}

// ------------------------------------------------------------ reductions
// Per-block partial measures in the compute type R.  Float64 states sum the
// mass as a two-term (hi + lo) compensated sum.  FP32-arithmetic states sum it
// in fixed point instead: each cell's h and rounding residue are converted to
// integers in units of 2^-32 and added as 64-bit integers, so the sum is exact
// and does not depend on the order of the additions.  The strip geometry, the
// 2D tiles, a batch's layout and the reduction trees then all give the same
// bits for the mass, and so for the mass correction that is driven by it:
// FP32 results do not depend on how the lattice is cut into CTAs.  Only the
// per-block result leaves the compute type, which keeps FP64 instructions
// (1/64 of the FP32 rate on GB300) out of the per-cell path.
template <class R>
struct PartT {
    R mhi, mlo;
    int wet;
    R hmax, hmin, area, cossum;
};

// FP32 cells: the mass, area and cos-sum in units of kMassUnit.  A block
// holds at most 252 x 512 cells, so its 64-bit sums are exact for mean
// heights below 1.6e4.
constexpr float kMassScale = 0x1p32f;
constexpr double kMassUnit = 0x1p-32;
struct PartQ {
    long long mq, area, cossum;
    int wet;
    float hmax, hmin;
};

// The per-cell partials of the step kernels of compute type R.
template <class R>
struct StepPartSel { using type = PartT<R>; };
template <>
struct StepPartSel<float> { using type = PartQ; };
template <class R>
using StepPart = typename StepPartSel<R>::type;

template <class R>
__device__ __forceinline__ void part_init(PartT<R> &p) {
    p.mhi = R(0);
    p.mlo = R(0);
    p.wet = 0;
    p.hmax = R(-INFINITY);
    p.hmin = R(INFINITY);
    p.area = R(0);
    p.cossum = R(0);
}

__device__ __forceinline__ void part_init(PartQ &p) {
    p.mq = 0;
    p.area = 0;
    p.cossum = 0;
    p.wet = 0;
    p.hmax = -INFINITY;
    p.hmin = INFINITY;
}

// (s, e) = a + b exactly (Knuth's TwoSum).
template <class R>
__device__ __forceinline__ void two_sum(R a, R b, R &s, R &e) {
    s = a + b;
    R bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

template <class R>
__device__ __forceinline__ void mass_add(PartT<R> &p, R v) {
    R s, e;
    two_sum(p.mhi, v, s, e);
    p.mhi = s;
    p.mlo = p.mlo + e;
}

// h of a cell: v * 2^32 is exact (a power-of-two scaling) and an integer for
// v >= 2^-9; the conversion rounds smaller heights to the unit.
__device__ __forceinline__ void mass_add(PartQ &p, float v) {
    p.mq += __float2ll_rn(v * kMassScale);
}

// The rounding residue of a cell's pulled height (a few ulp of h).
template <class R>
__device__ __forceinline__ void mass_add_lo(PartT<R> &p, R lo) { p.mlo = p.mlo + lo; }
__device__ __forceinline__ void mass_add_lo(PartQ &p, float lo) {
    p.mq += __float2ll_rn(lo * kMassScale);
}

// A wetted cell's surface element and cos θ (surfacearea!, src/measures.jl).
template <class R>
__device__ __forceinline__ void area_add(PartT<R> &p, R v) { p.area += v; }
__device__ __forceinline__ void area_add(PartQ &p, float v) {
    p.area += __float2ll_rn(v * kMassScale);
}
template <class R>
__device__ __forceinline__ void cos_add(PartT<R> &p, R v) { p.cossum += v; }
__device__ __forceinline__ void cos_add(PartQ &p, float v) {
    p.cossum += __float2ll_rn(v * kMassScale);
}

template <class R>
__device__ __forceinline__ void part_merge(PartT<R> &a, const PartT<R> &b) {
    R s, e;
    two_sum(a.mhi, b.mhi, s, e);
    a.mhi = s;
    a.mlo = a.mlo + b.mlo + e;
    a.wet += b.wet;
    a.hmax = fmax(a.hmax, b.hmax);
    a.hmin = fmin(a.hmin, b.hmin);
    a.area += b.area;
    a.cossum += b.cossum;
}

__device__ __forceinline__ void part_merge(PartQ &a, const PartQ &b) {
    a.mq += b.mq;
    a.area += b.area;
    a.cossum += b.cossum;
    a.wet += b.wet;
    a.hmax = fmaxf(a.hmax, b.hmax);
    a.hmin = fminf(a.hmin, b.hmin);
}

template <class R>
__device__ __forceinline__ PartT<R> part_shfl(const PartT<R> &p, int off) {
    PartT<R> o;
    o.mhi = __shfl_down_sync(0xffffffffu, p.mhi, off);
    o.mlo = __shfl_down_sync(0xffffffffu, p.mlo, off);
    o.wet = __shfl_down_sync(0xffffffffu, p.wet, off);
    o.hmax = __shfl_down_sync(0xffffffffu, p.hmax, off);
    o.hmin = __shfl_down_sync(0xffffffffu, p.hmin, off);
    o.area = __shfl_down_sync(0xffffffffu, p.area, off);
    o.cossum = __shfl_down_sync(0xffffffffu, p.cossum, off);
    return o;
}

__device__ __forceinline__ PartQ part_shfl(const PartQ &p, int off) {
    PartQ o;
    o.mq = __shfl_down_sync(0xffffffffu, p.mq, off);
    o.area = __shfl_down_sync(0xffffffffu, p.area, off);
    o.cossum = __shfl_down_sync(0xffffffffu, p.cossum, off);
    o.wet = __shfl_down_sync(0xffffffffu, p.wet, off);
    o.hmax = __shfl_down_sync(0xffffffffu, p.hmax, off);
    o.hmin = __shfl_down_sync(0xffffffffu, p.hmin, off);
    return o;
}

// Lattice-wide accumulation of the Float64 reducer.
struct RedPart {
    double m;
    int wet;
    double hmax, hmin, area, cossum;
};

__device__ __forceinline__ void part_init(RedPart &p) {
    p.m = 0.0;
    p.wet = 0;
    p.hmax = -INFINITY;
    p.hmin = INFINITY;
    p.area = 0.0;
    p.cossum = 0.0;
}

__device__ __forceinline__ void part_merge(RedPart &a, const RedPart &b) {
    a.m += b.m;
    a.wet += b.wet;
    a.hmax = fmax(a.hmax, b.hmax);
    a.hmin = fmin(a.hmin, b.hmin);
    a.area += b.area;
    a.cossum += b.cossum;
}

__device__ __forceinline__ RedPart part_shfl(const RedPart &p, int off) {
    RedPart o;
    o.m = __shfl_down_sync(0xffffffffu, p.m, off);
    o.wet = __shfl_down_sync(0xffffffffu, p.wet, off);
    o.hmax = __shfl_down_sync(0xffffffffu, p.hmax, off);
    o.hmin = __shfl_down_sync(0xffffffffu, p.hmin, off);
    o.area = __shfl_down_sync(0xffffffffu, p.area, off);
    o.cossum = __shfl_down_sync(0xffffffffu, p.cossum, off);
    return o;
}

// Order-preserving keys of a float for unsigned atomicMax, 0 meaning "no
// cell": key_max grows with v, key_min shrinks with v.
__device__ __forceinline__ unsigned int float_order(float v) {
    const unsigned int u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float float_unorder(unsigned int o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}
__device__ __forceinline__ unsigned long long key_max(float v) {
    return (unsigned long long)float_order(v) + 1ull;
}
__device__ __forceinline__ unsigned long long key_min(float v) {
    return (unsigned long long)(0xffffffffu - float_order(v)) + 1ull;
}

// hi * 2^64 + lo += v (a two-word signed 128-bit integer)
__device__ __forceinline__ void fix_add(long long &hi, unsigned long long &lo, long long v) {
    const unsigned long long n = lo + (unsigned long long)v;
    hi += (v < 0 ? -1 : 0) + (n < lo ? 1 : 0);
    lo = n;
}

// Warp-wide exact sum of one signed 64-bit value per lane, as a double in
// units of kMassUnit.
__device__ __forceinline__ double warp_fix_sum(long long v) {
    long long hi = 0;
    unsigned long long lo = 0;
    fix_add(hi, lo, v);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const long long ohi = __shfl_down_sync(0xffffffffu, hi, off);
        const unsigned long long olo = __shfl_down_sync(0xffffffffu, lo, off);
        const unsigned long long n = lo + olo;
        hi += ohi + (n < lo ? 1 : 0);
        lo = n;
    }
    return ((double)hi * 0x1p64 + (double)lo) * kMassUnit;
}

// Block-wide reduction; the result is valid in thread 0.  red: NT/32 slots.
template <int NT, class P>
__device__ __forceinline__ P block_reduce(P p, P *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) part_merge(p, part_shfl(p, off));
    if (lane == 0) red[warp] = p;
    __syncthreads();
    if (warp == 0) {
        P q;
        part_init(q);
        if (lane < NT / 32) q = red[lane];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) part_merge(q, part_shfl(q, off));
        p = q;
    }
    __syncthreads();
    return p;
}

// ------------------------------------------------------------ the marching step
// A CTA of NT threads owns a strip of W = NT - 4 columns and H rows of one
// lattice; thread t owns column x0 - 2 + t for the whole strip.  It sweeps the
// rows in order, keeping in shared memory the heights of rows y-2..y+2 (ring
// of 5), the film pressure of rows y-1..y+1 and the momenta of the rows whose
// output is pending (rings of 4).  Per output row y it
//   1. turns the pulled populations of row y+2 (prefetched into registers one
//      row earlier) into h, j = Σ c_q f_q and the rounding residue of h;
//   2. issues the pull of row y+3 (in flight during 3-4);
//   3. computes p on row y+1 (columns 1..NT-2);
//   4. computes forces, equilibrium and collision of row y and stores it.
// Only the x halo (4 of NT columns) and the 4 extra rows of each strip are
// recomputed; the column index math is done once per thread.
template <class S, int NT>
struct MarchSmem {
    using R = typename S::real;
    R h[8][NT];  // ring of 5 live rows; 8 slots so that the index is a mask
    R p[4][NT];
    R jx[4][NT];
    R jy[4][NT];
    R lo[4][NT];  // FP32 paths: rounding error of the pulled height
    StepPart<R> red[NT / 32];
    RedPart redd[NT / 32];
};

// Block partial measures of iteration t.  Float64 states: into the block's
// parity slot of the partials array.
template <int NT, class R>
__device__ __forceinline__ void write_partials(const StepArgs &a, const PartT<R> &part,
                                               long long t, int blin, PartT<R> *red) {
    const PartT<R> tot = block_reduce<NT>(part, red);
    if (threadIdx.x == 0) {
        double *pp = a.partials + ((size_t)(t & 1) * (size_t)a.part_stride + (size_t)blin) * kNPart;
        pp[0] = (double)tot.mhi + (double)tot.mlo;
        pp[1] = (double)tot.wet;
        pp[2] = (double)tot.hmax;
        pp[3] = (double)tot.hmin;
        pp[4] = (double)tot.area;
        pp[5] = (double)tot.cossum;
    }
}

// FP32-arithmetic states: added by integer atomics into lane blin % 32 of the
// iteration's accumulators (exact and order-free; fire-and-forget reductions
// in L2, so no CTA waits).
__device__ __forceinline__ void add_partials(const StepArgs &a, const PartQ &tot, long long t,
                                             int blin) {  // one thread
    unsigned long long(*acc)[kAccLanes] = a.ctl->acc[t & 1];
    const int l = blin & (kAccLanes - 1);
    atomicAdd(&acc[kAccMass][l], (unsigned long long)tot.mq);
    atomicAdd(&acc[kAccWet][l], (unsigned long long)tot.wet);
    atomicMax(&acc[kAccHmax][l], key_max(tot.hmax));
    atomicMax(&acc[kAccHmin][l], key_min(tot.hmin));
    if (a.meas_mask & SWB_MEAS_AREA) {
        atomicAdd(&acc[kAccArea][l], (unsigned long long)tot.area);
        atomicAdd(&acc[kAccCos][l], (unsigned long long)tot.cossum);
    }
}
template <int NT>
__device__ __forceinline__ void write_partials(const StepArgs &a, const PartQ &part, long long t,
                                               int blin, PartQ *red) {
    const PartQ tot = block_reduce<NT>(part, red);
    if (threadIdx.x == 0) add_partials(a, tot, t, blin);
}

// The record of iteration s and, with the mass correction on, the
// correction of iteration s + 2.  M(s) is the mass of the populations
// iteration s pulled; the corrections c(s) and c(s+1) were applied after that
// and are not in it, so
//   c(s+2) = (M_target - M(s) - N (c(s) + c(s+1))) / N
// makes M(s+3) = M_target up to three steps of rounding noise.  One thread.
__device__ __forceinline__ void finish_step(const StepArgs &a, long long s, double mass,
                                            double wet, double hmax, double hmin, double area,
                                            double cossum) {
    Control *c = a.ctl;
    if (a.meas_mask) {
        Record &r = a.records[(s - 1) % a.rec_cap];
        r.t = s;
        r.mass = mass;
        r.wetted = wet;
        r.hmax = hmax;
        r.hmin = hmin;
        r.area = area;
        r.cos_sum = a.theta_mode == THETA_SCALAR ? wet * a.cos_theta : cossum;
        c->rec_head = __ldcg(&c->rec_head) + 1;
    }
    if (a.mass_corr) {
        if (s == __ldcg(&c->fresh_step)) c->mass_target = mass;
        const double N = (double)a.Lx * (double)a.Ly;
        const double in_flight = __ldcg(&c->corr[s & 1]) + __ldcg(&c->corr[(s + 1) & 1]);
        c->corr[s & 1] = (__ldcg(&c->mass_target) - mass - N * in_flight) / N;
    }
}

// Lattice-wide measures of iteration s (complete: an earlier launch, or the
// previous phase of a multi-step launch, produced them).
//  * FP32-arithmetic states: one warp reads the kAccLanes lanes of the
//    integer accumulators, clears them for iteration s + 2 and sums them
//    exactly (128-bit), so the result does not depend on the CTAs at all.
//  * Float64 states: plain Float64 sums over the block partials (each already
//    a compensated sum, ~1e-15 relative for a few thousand blocks) in a fixed
//    order, so deterministic.  Unrolled so that many partials are in flight
//    at once: this CTA runs beside the strips and must not become the
//    launch's straggler.
// No __syncthreads in the FP32 path: the other warps return at once.
template <int NT>
__device__ void reduce_step(const StepArgs &a, long long s, RedPart *redd) {
    if (a.mass_fixed) {
        if (threadIdx.x >= 32) return;
        const int l = threadIdx.x;
        unsigned long long(*acc)[kAccLanes] = a.ctl->acc[s & 1];
        const unsigned long long m = __ldcg(&acc[kAccMass][l]), w = __ldcg(&acc[kAccWet][l]);
        unsigned long long kx = __ldcg(&acc[kAccHmax][l]), kn = __ldcg(&acc[kAccHmin][l]);
        const unsigned long long ar = __ldcg(&acc[kAccArea][l]), cs = __ldcg(&acc[kAccCos][l]);
#pragma unroll
        for (int f = 0; f < kAccFields; ++f) acc[f][l] = 0ull;
        const double mass = warp_fix_sum((long long)m);
        const double area = warp_fix_sum((long long)ar);
        const double cossum = warp_fix_sum((long long)cs);
        unsigned long long wt = w;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            wt += __shfl_down_sync(0xffffffffu, wt, off);
            kx = max(kx, __shfl_down_sync(0xffffffffu, kx, off));
            kn = max(kn, __shfl_down_sync(0xffffffffu, kn, off));
        }
        if (l == 0) {
            const double hmax = kx ? (double)float_unorder((unsigned int)(kx - 1ull)) : -INFINITY;
            const double hmin =
                kn ? (double)float_unorder(0xffffffffu - (unsigned int)(kn - 1ull)) : INFINITY;
            finish_step(a, s, mass, (double)wt, hmax, hmin, area, cossum);
        }
        return;
    }
    const int nblocks = a.tiles_x * a.tiles_y;
    const double *base = a.partials + (size_t)(s & 1) * (size_t)a.part_stride * kNPart;
    // a partial is 48 bytes, 16-byte aligned: three 16-byte loads each
    static_assert(kNPart == 6, "partials of six doubles");
    double m = 0.0, wt = 0.0, ar = 0.0, cs = 0.0, mx = -INFINITY, mn = INFINITY;
#pragma unroll 8
    for (int b = threadIdx.x; b < nblocks; b += NT) {
        const double2 *pp = reinterpret_cast<const double2 *>(base + (size_t)b * kNPart);
        const double2 v0 = __ldcg(pp), v1 = __ldcg(pp + 1), v2 = __ldcg(pp + 2);
        m += v0.x;
        wt += v0.y;
        mx = fmax(mx, v1.x);
        mn = fmin(mn, v1.y);
        ar += v2.x;
        cs += v2.y;
    }
    RedPart acc;
    acc.m = m;
    acc.wet = (int)wt;
    acc.hmax = mx;
    acc.hmin = mn;
    acc.area = ar;
    acc.cossum = cs;
    acc = block_reduce<NT>(acc, redd);
    if (threadIdx.x == 0)
        finish_step(a, s, acc.m, (double)acc.wet, acc.hmax, acc.hmin, acc.area, acc.cossum);
}

// ------------------------------------------------------------ thermal noise
// thermal! (src/forcing.jl:297-320) draws two standard normals per cell and
// iteration.  They come from Philox-4x32-10 (Salmon et al., SC'11; the same
// generator as the oracle) with key = seed and counter = (cell, t), and the
// Box-Muller transform: Float64 in the literal mode, FP32 otherwise.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k.x += 0x9E3779B9u;
            k.y += 0xBB67AE85u;
        }
        const unsigned int hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const unsigned int hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

__device__ __forceinline__ uint4 thermal_bits(unsigned long long seed, long long cell,
                                              long long t) {
    const unsigned long long k = (unsigned long long)cell, tu = (unsigned long long)t;
    return philox4x32_10(make_uint4((unsigned)k, (unsigned)tu, (unsigned)(tu >> 32),
                                    (unsigned)(k >> 32)),
                         make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
}

__device__ __forceinline__ void thermal_normals(unsigned long long seed, long long cell,
                                                long long t, double &zx, double &zy) {
    const uint4 w = thermal_bits(seed, cell, t);
    const double u1 =
        (double)(((((unsigned long long)w.x) << 32) | w.y) >> 11) * 0x1p-53 + 0x1p-54;
    const double u2 = (double)(((((unsigned long long)w.z) << 32) | w.w) >> 11) * 0x1p-53;
    const double r = sqrt(-2.0 * log(u1));
    zx = r * cos(6.283185307179586 * u2);
    zy = r * sin(6.283185307179586 * u2);
}

__device__ __forceinline__ void thermal_normals(unsigned long long seed, long long cell,
                                                long long t, float &zx, float &zy) {
    const uint4 w = thermal_bits(seed, cell, t);
    const float u1 = (float)(w.x >> 8) * 0x1p-24f + 0x1p-25f;
    const float u2 = (float)(w.z >> 8) * 0x1p-24f;
    const float r = sqrtf(-2.0f * logf(u1));
    float sn, cs;
    sincospif(2.0f * u2, &sn, &cs);
    zx = r * cs;
    zy = r * sn;
}

// thermal!'s force on a cell: (zx, zy) * sigma(h).  Not inlined: the noise
// (Philox, log, sin/cos) stays out of the register budget of steps without
// fluctuations.
template <bool LIT, class R>
__device__ __noinline__ void thermal_force(unsigned long long seed, long long cell, long long t,
                                           R k6, R h, R delta, R *fx, R *fy);

// Standard deviation of the thermal force at height h:
// sqrt(2 kbt mu 6 h / (2h^2 + 6 h delta + 3 delta^2)), in the reference's order.
template <bool LIT, class R>
__device__ __forceinline__ R thermal_sigma(R k6, R h, R delta) {
    if constexpr (LIT)
        return sqrt(k6 * h / (((R(2) * h) * h + (R(6) * h) * delta) + (R(3) * delta) * delta));
    else
        return sqrtf(qdiv(k6 * h, __fmaf_rn(__fmaf_rn(R(2), h, R(6) * delta), h,
                                             (R(3) * delta) * delta)));
}

template <bool LIT, class R>
__device__ __noinline__ void thermal_force(unsigned long long seed, long long cell, long long t,
                                           R k6, R h, R delta, R *fx, R *fy) {
    R zx, zy;
    thermal_normals(seed, cell, t, zx, zy);
    const R sg = thermal_sigma<LIT, R>(k6, h, delta);
    *fx = zx * sg;
    *fy = zy * sg;
}

// Per-tile constants of the force and collision stage.
template <class R>
struct CellConst {
    R delta6, delta3sq, mu6, omeg, invtau, g, incl_fac;
    R corr;  // mass correction per cell of this iteration, converted once per CTA
};

template <class R>
__device__ __forceinline__ CellConst<R> cell_consts(const StepArgs &a, long long tt, double corr) {
    CellConst<R> c;
    c.incl_fac = R(0);
    if (a.incl) {
        c.incl_fac = a.incl_loop_time
                         ? R(0.5) + R(0.5) * tanh_r(R(tt - a.incl_tstart) / R(a.incl_tsmooth))
                         : R(a.incl_fixed);
    }
    c.delta6 = R(6.0 * a.delta);
    c.delta3sq = R(3.0 * (a.delta * a.delta));
    c.mu6 = R(6.0 * a.mu);
    c.omeg = R(a.omeg);
    c.invtau = R(a.invtau);
    c.g = R(a.g);
    c.corr = R(corr);
    return c;
}

// slippage! (src/forcing.jl:43-44) and the force sum (src/simulate.jl:18-19)
// in FP32 arithmetic: (Fx, Fy) = -h ∇p - c u with c = 6 μ h / (2h² + 6δh +
// 3δ²), both components in one packed pair.
__device__ __forceinline__ float2 force_fast(const CellConst<float> &cc, float h, float ux,
                                             float uy, float gpx, float gpy) {
    const float c = qdiv(cc.mu6 * h, __fmaf_rn(__fmaf_rn(2.0f, h, cc.delta6), h, cc.delta3sq));
    return fma2(f2(-h, -h), f2(gpx, gpy), mul2(f2(-c, -c), f2(ux, uy)));
}

// The FP32-arithmetic collision of one cell: its nine post-collision
// populations fo (for FP16 storage also the stored half bits hb of the pairs
// (1, 2), (3, 4), (5, 6), (7, 8); fo then holds the values they represent).
// (Fx, Fy): the force; hft, fq: the pulled mass and populations (τ != 1
// only); *hlo_p: the rounding residue of the pulled height (not read for a
// fresh step).  Shared by every FP32-arithmetic kernel, so that they all
// round identically.
// HB_ONLY (FP16 storage): the caller stores planes 1..8 from hb and reads
// only fo[0], so fo[1..8] may hold the stored values x kScale, and at τ = 1
// the populations are computed x kScale from the start (the weights and
// sources scaled by the power of two kScale: the same bits, fewer
// multiplications).
template <class S, bool FRESH, bool TAU1, bool HB_ONLY = false>
__device__ __forceinline__ void collide_fast(const CellConst<float> &cc, float h, float ux,
                                             float uy, float Fx, float Fy, float hft,
                                             const float *fq, int cell, long long tt,
                                             const float *hlo_p, float fo[9],
                                             __half2 hb[4]) {
    using R = float;
    // FP32 arithmetic.  f0 closes the mass balance with the values as
    // stored: f0 = M - Σ_{q>0} f_q, where M (the pulled mass, hi + lo)
    // is what the cell must hold.  The residue c (e, the exact rounding
    // error of f0 (Fast2Sum), the lo part of M and the cell's share of
    // the mass correction) is added to f0 by stochastic rounding, so it
    // stays in the cell, at rest, in expectation: no bias, whatever the
    // state.  FP32 populations also keep what that rounding left out:
    // c - k ulp(f0) is zero-mean and resolved by ulp(f5), so folding it
    // into f5 and f7 keeps the mass (~1e-12 relative over 100,000
    // iterations) without a systematic transport.  Folding all of c into
    // a moving pair instead moves the residue to the neighbours every
    // iteration, which biases slow dynamics: 2-3e-4 relative L2 in h
    // against Float64 after 100,000 iterations of a 2048² film h = 1 ± 0.1
    // (which levels over that time), against 6e-7 this way (measured
    // on GB300).  FP16
    // populations cannot hold the left-out part; their mass is kept by
    // the FP64-measured correction.
    // Opposite populations (q+, q-) share their equilibrium's even part
    // A and odd part B (feq = A ± B, src/equilibrium.jl:67-114) and their
    // force source ±S (src/collide.jl:80-89).
    // populations computed x ks (FP16 planes stored from them directly)
    constexpr bool kScaled = S::kHalf && TAU1 && HB_ONLY;
    constexpr float ks = kScaled ? StoreF16::kScale : 1.0f;
    const R vsq = __fmaf_rn(ux, ux, uy * uy);
    const R base = __fmaf_rn(R(1.5) * cc.g, h, R(-1.5) * vsq);
    const R w1h = h * (R(1.0 / 9.0) * ks), w5h = h * (R(1.0 / 36.0) * ks);
    // the k = (1, 2) and (5, 6) directions as packed pairs: velocities
    // cu = (ux, uy) and (ux + uy, uy - ux), weights w1 h and w5 h, sources
    // (Fx, Fy) / 3 and (Fx + Fy, Fy - Fx) / 24
    const float2 U = f2(ux, uy), F2 = f2(Fx, Fy);
    const float2 CU[2] = {U, add2(U, f2(uy, -ux))};
    const float2 SQ[2] = {mul2(f2(1.0f / 3.0f * ks, 1.0f / 3.0f * ks), F2),
                          mul2(f2(1.0f / 24.0f * ks, 1.0f / 24.0f * ks), add2(F2, f2(Fy, -Fx)))};
    const R wq[2] = {w1h, w5h};
    const float2 BASE = f2(base, base);
    constexpr int qp[2] = {1, 5}, qm[2] = {3, 7};  // and qp + 1, qm + 1
    // FP16 planes: the stored bits of (f1, f2), (f3, f4), (f5, f6), (f7, f8),
    // rounded once per pair; fo holds the values they represent
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const float2 WQ = f2(wq[j], wq[j]);
        const float2 A = mul2(WQ, fma2(mul2(f2(4.5f, 4.5f), CU[j]), CU[j], BASE));
        float2 P, M;
        if constexpr (TAU1) {
            const float2 BS = fma2(mul2(f2(3.0f, 3.0f), WQ), CU[j], SQ[j]);
            P = add2(A, BS);
            M = sub2(A, BS);
        } else {
            const float2 B = mul2(mul2(f2(3.0f, 3.0f), WQ), CU[j]);
            const float2 OM = f2(cc.omeg, cc.omeg), IT = f2(cc.invtau, cc.invtau);
            P = add2(fma2(OM, f2(fq[qp[j]], fq[qp[j] + 1]), mul2(IT, add2(A, B))), SQ[j]);
            M = sub2(fma2(OM, f2(fq[qm[j]], fq[qm[j] + 1]), mul2(IT, sub2(A, B))), SQ[j]);
        }
        if constexpr (S::kHalf) {
            const float2 sc = f2(S::kScale, S::kScale), inv = f2(S::kInv, S::kInv);
            if constexpr (kScaled) {
                hb[2 * j] = __float22half2_rn(P);
                hb[2 * j + 1] = __float22half2_rn(M);
            } else {
                hb[2 * j] = __float22half2_rn(mul2(P, sc));
                hb[2 * j + 1] = __float22half2_rn(mul2(M, sc));
            }
            // the values the planes hold (x kScale with HB_ONLY)
            float2 rp = __half22float2(hb[2 * j]), rm = __half22float2(hb[2 * j + 1]);
            if constexpr (!HB_ONLY) {
                rp = mul2(rp, inv);
                rm = mul2(rm, inv);
            }
            fo[qp[j]] = rp.x;
            fo[qp[j] + 1] = rp.y;
            fo[qm[j]] = rm.x;
            fo[qm[j] + 1] = rm.y;
        } else {
            fo[qp[j]] = P.x;
            fo[qp[j] + 1] = P.y;
            fo[qm[j]] = M.x;
            fo[qm[j] + 1] = M.y;
        }
    }
    R hlo = R(0);
    if constexpr (!FRESH) hlo = *hlo_p;
    // Σ_q fpost_q = (1-1/τ) Σ ft + Σ feq/τ = h once h is the pulled mass
    const R mc = (TAU1 || !FRESH) ? h : cc.omeg * hft + cc.invtau * h;
    // Σ_{q>0} f_q as stored (with HB_ONLY, FP16 values x kScale: the sum of
    // the scaled values times 1/kScale is the same bits)
    const R ssum = (S::kHalf && HB_ONLY) ? small8(fo) * R(StoreF16::kInv) : small8(fo);
    const R f0 = mc - ssum;
    const R e = (mc - f0) - ssum;
    const R c = e + hlo + cc.corr;
    fo[0] = add_stochastic((float)f0, (float)c, mix32((unsigned)cell, (unsigned)tt));
    if constexpr (!S::kHalf) {
        // What the rounding left out, c - k ulp(f0): zero-mean whatever
        // the state, at most ~ulp(f0), and on a grid that ulp(f5) = ulp(f0)/16
        // resolves, so folding it into the diagonal pair keeps the mass
        // (momentum unchanged) without a systematic transport.
        const R d = R(0.5) * (c - (fo[0] - f0));
        fo[5] = fo[5] + d;
        fo[7] = fo[7] + d;
    }
}

// Forces, equilibrium and collision of one cell and the store of its nine
// post-collision populations: slippage! (src/forcing.jl:43-44), the force sum
// (src/simulate.jl:18-19), inclination! (src/forcing.jl:364-365),
// equilibrium! and BGKandStream! (src/collide.jl:76-89).  (gpx, gpy) is
// ∇p at the cell (h∇p!, src/forcing.jl:181-184); *hlo_p the rounding
// residue of the pulled height (FP32 arithmetic; not read for a fresh step).
// GEN = false compiles out the rare forces (thermal, inclination) for the
// common step; the caller guarantees they are off.
template <class S, bool FRESH, bool TAU1, bool GEN>
__device__ __forceinline__ void collide_cell(const StepArgs &a,
                                             const CellConst<typename S::real> &cc,
                                             const void *src, void *dst, int gx, int gy, int gxm,
                                             int gxp, int cell, long long tt,
                                             typename S::real h, typename S::real ux,
                                             typename S::real uy, typename S::real gpx,
                                             typename S::real gpy,
                                             const typename S::real *hlo_p) {
    using R = typename S::real;
    constexpr bool LIT = S::kLiteral;
    const int pitch = (int)a.pitch;  // 9 * pitch < 2^31 (checked at creation)
    const int Lx = a.Lx, Ly = a.Ly;
    // slippage! (src/forcing.jl:43-44) and the force sum (src/simulate.jl:18-19)
    R Fx, Fy;
    if constexpr (LIT) {
        const R hgx = h * gpx, hgy = h * gpy;
        const R den = R(2) * (h * h) + cc.delta6 * h + cc.delta3sq;
        const R sx = (cc.mu6 * h * ux) / den;
        const R sy = (cc.mu6 * h * uy) / den;
        Fx = -hgx - sx;
        Fy = -hgy - sy;
        if (GEN && a.thermal) {  // Fx .= -h∇px .- slipx .- kbtx (scripts/Rivulet_stability.jl:123)
            R kx, ky;
            thermal_force<true, R>(a.seed, (long long)cell, tt, R(a.k6), h, R(a.delta), &kx, &ky);
            Fx = Fx - kx;
            Fy = Fy - ky;
        }
        if (GEN && a.incl) {  // inclination! (src/forcing.jl:364-365)
            Fx = Fx + (h * R(a.ax)) * cc.incl_fac;
            Fy = Fy + (h * R(a.ay)) * cc.incl_fac;
        }
    } else {
        const float2 F = force_fast(cc, h, ux, uy, gpx, gpy);
        Fx = F.x;
        Fy = F.y;
        if (GEN && a.thermal) {
            R kx, ky;
            thermal_force<false, R>(a.seed, (long long)cell, tt, R(a.k6), h, R(a.delta), &kx, &ky);
            Fx = Fx - kx;
            Fy = Fy - ky;
        }
        if (GEN && a.incl) {
            Fx = __fmaf_rn(h * R(a.ax), cc.incl_fac, Fx);
            Fy = __fmaf_rn(h * R(a.ay), cc.incl_fac, Fy);
        }
    }
    // collision (src/collide.jl:76-89); ftemp only matters for τ != 1
    R fq[9];
    R hft = h;
    if constexpr (!TAU1) {
        const int gym = gy == 0 ? Ly - 1 : gy - 1, gyp = gy == Ly - 1 ? 0 : gy + 1;
        pull9<S>(src, pitch, Lx, gx, gy, gxm, gxp, gym, gyp, fq);
        if constexpr (!LIT) hft = fq[0] + small8(fq);
    }
    if constexpr (LIT) {
        R fe[9];
        feq_literal<R>(h, ux, uy, cc.g, fe);
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            R v;
            if constexpr (TAU1)
                v = fe[q];
            else
                v = cc.omeg * fq[q] + cc.invtau * fe[q];
            if (q > 0) v = v + source<R>(q, Fx, Fy);
            S::st(dst, pitch, q, cell, v);
        }
    } else {
        float fo[9];
        [[maybe_unused]] __half2 hb[4];
        collide_fast<S, FRESH, TAU1, true>(cc, h, ux, uy, Fx, Fy, hft, fq, cell, tt, hlo_p, fo, hb);
        if constexpr (S::kHalf) {
            reinterpret_cast<float *>(dst)[cell] = fo[0];
            __half *hpl = const_cast<__half *>(S::hp(dst, pitch)) + cell;
            // planes 1..8 in the order of hb: (1, 2), (3, 4), (5, 6), (7, 8)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                hpl[(2 * k) * pitch] = __low2half(hb[k]);
                hpl[(2 * k + 1) * pitch] = __high2half(hb[k]);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 9; ++q) S::st(dst, pitch, q, cell, fo[q]);
        }
    }
}

// One time_loop iteration on strip (bx, by) of the lattice described by `a`,
// compiled for the iteration's rare cases: FRESH (the first iteration after
// the fields were set: h, u come from the fields) and TAU1 (τ = 1: the
// previous populations drop out of the collision).
template <class S, int NT, bool FRESH, bool TAU1, bool GEN, bool WAVE = false>
__device__ __forceinline__ void march_run(const StepArgs &a, int bx, int by, long long done,
                                          MarchSmem<S, NT> &sm) {
    using R = typename S::real;
    constexpr bool LIT = S::kLiteral;
    constexpr int W = NT - 4;
    const int t = threadIdx.x;
    const int Lx = a.Lx, Ly = a.Ly;
    const int H = a.march_h;
    const int pitch = (int)a.pitch;  // 9 * pitch < 2^31 (checked at creation)
    const long long tt = done + 1;  // this time_loop iteration (1-based)
    const void *src = (done & 1) ? a.fb : a.fa;
    void *dst = (done & 1) ? a.fa : a.fb;
    const int x0 = bx * W, y0 = by * H;
    const int rows = min(H, Ly - y0);
    const R gamma = R(a.gamma), hmin = R(a.hmin), hcrit = R(a.hcrit);
    // periodic row index; rows run from y0-2 to y0+rows+1, one wrap suffices
    // unless the lattice is thinner than 3 rows
    const bool tiny_y = Ly < 3;
    auto wrow = [&](int yy) {
        return tiny_y ? wrapc(yy, Ly) : (yy < 0 ? yy + Ly : (yy >= Ly ? yy - Ly : yy));
    };

    // this thread's column
    const int gx = wrapc(x0 - 2 + t, Lx);
    const int gxm = gx == 0 ? Lx - 1 : gx - 1, gxp = gx == Lx - 1 ? 0 : gx + 1;
    const bool interior = t >= 2 && t < NT - 2 && x0 + t - 2 < Lx;
    const bool pcol = t >= 1 && t < NT - 1;

    // FP16: per-cell share of the mass correction of this iteration
    const double corr = (!LIT && !FRESH && a.mass_corr) ? __ldcg(&a.ctl->corr[tt & 1]) : 0.0;
    // kappa and cospi(θ) of this column: constant (scalar θ) or θ(x, t) of
    // the moving-wettability mode, which depends on x only
    // GEN = false: scalar θ, or with WAVE also the θ wave (a per-column κ)
    const int mode = GEN ? a.theta_mode
                         : ((WAVE && a.theta_mode == THETA_WAVE) ? THETA_WAVE : THETA_SCALAR);
    // θ field: column of this thread and row offset in the (possibly moving) field
    int fsx = 0, fsy = 0;
    if (mode == THETA_FIELD) substrate_shift(a, tt, &fsx, &fsy);
    const int gxf = fsx ? (gx - fsx < 0 ? gx - fsx + Lx : gx - fsx) : gx;
    auto frow = [&](int gyy) { return fsy ? (gyy - fsy < 0 ? gyy - fsy + Ly : gyy - fsy) : gyy; };
    R kap_col = R(a.kap), cos_col = R(a.cos_theta);
    if (mode == THETA_WAVE) {
        const KapCos<R> w = wave_at<R>(a, gx, tt);
        kap_col = w.kap;
        cos_col = w.cs;
    }

    // pulled populations of the next leading row (prefetch; two in flight in the prologue)
    R fa_[9], fb_[9];
    // strips whose pulls never cross the periodic boundary (rows y0-3 ..
    // y0+rows+2, columns x0-3 .. x0+NT-2): the interior pull (FP32
    // populations; for FP16 planes it costs more registers than it saves)
    const bool no_wrap = !FRESH && !LIT && !S::kHalf && y0 >= 3 && y0 + rows + 2 < Ly &&
                         x0 >= 3 && x0 + NT - 2 < Lx;
    auto issue = [&](R(&ft)[9], int yy) {
        if constexpr (FRESH) {
            ft[0] = reinterpret_cast<const R *>(a.hF)[wrow(yy) * Lx + gx];
        } else {
            if (no_wrap) {
                pull9_interior<S>(src, pitch, Lx, yy * Lx + gx, ft);
            } else {
                const int gy = wrow(yy);
                const int gym = gy == 0 ? Ly - 1 : gy - 1, gyp = gy == Ly - 1 ? 0 : gy + 1;
                pull9<S>(src, pitch, Lx, gx, gy, gxm, gxp, gym, gyp, ft);
            }
        }
    };
    auto consume = [&](const R(&ft)[9], int yy) {
        const int r = yy - y0 + 2;  // >= 0
        if constexpr (FRESH) {
            sm.h[r & 7][t] = ft[0];
        } else {
            R h, jx, jy;
            moments9<LIT>(ft, h, jx, jy);
            sm.h[r & 7][t] = h;
            sm.jx[r & 3][t] = jx;
            sm.jy[r & 3][t] = jy;
            if constexpr (!LIT) sm.lo[r & 3][t] = moments_lo(ft, h);
        }
    };
    auto pressure_row = [&](int yy) {
        if (!pcol) return;
        const int r = yy - y0 + 2;  // >= 1
        const R *hm = sm.h[(r + 7) & 7], *hc = sm.h[r & 7], *hp = sm.h[(r + 1) & 7];
        const R kap = mode == THETA_FIELD
                          ? reinterpret_cast<const R *>(a.kapF)[frow(wrow(yy)) * Lx + gxf]
                          : kap_col;
        // ip = h[i-1,j], jp = h[i,j-1], im = h[i+1,j], jm = h[i,j+1], ...
        sm.p[r & 3][t] = pressure_cell<LIT, R>(hc[t], hc[t - 1], hm[t], hc[t + 1], hp[t],
                                               hm[t - 1], hm[t + 1], hp[t + 1], hp[t - 1], kap,
                                               gamma, hmin, hcrit, a.n, a.m);
    };

    // prologue: heights of rows y0-2..y0+1 (two pulls in flight), then the
    // pull of row y0+2 stays in flight into the loop
    issue(fa_, y0 - 2);
    issue(fb_, y0 - 1);
    consume(fa_, y0 - 2);
    issue(fa_, y0);
    consume(fb_, y0 - 1);
    issue(fb_, y0 + 1);
    consume(fa_, y0);
    issue(fa_, y0 + 2);
    consume(fb_, y0 + 1);
    __syncthreads();
    pressure_row(y0 - 1);
    pressure_row(y0);

    const CellConst<R> cc = cell_consts<R>(a, tt, corr);
    const R thr = R(a.hthresh);
    const bool measure = a.meas_mask || a.mass_corr;
    StepPart<R> part;
    part_init(part);
    int any_nan = 0;

#pragma unroll 1
    for (int j = 0; j < rows; ++j) {
        const int y = y0 + j;
        consume(fa_, y + 2);
        if (j + 1 < rows) issue(fa_, y + 3);  // one row ahead
        __syncthreads();
        pressure_row(y + 1);
        __syncthreads();
        if (!interior) continue;
        // ---- output row y, column gx ----
        const int r = y - y0 + 2;
        const int gy = wrow(y);
        const int cell = gy * Lx + gx;
        const R *hrow = sm.h[r & 7];
        const R h = hrow[t];
        R ux, uy;
        if constexpr (FRESH) {
            ux = reinterpret_cast<const R *>(a.uxF)[cell];
            uy = reinterpret_cast<const R *>(a.uyF)[cell];
        } else {
            velocity<LIT>(h, sm.jx[r & 3][t], sm.jy[r & 3][t], ux, uy);
        }
        // h∇p! (src/forcing.jl:181-184)
        const R *pm = sm.p[(r + 3) & 3], *pc = sm.p[r & 3], *pp = sm.p[(r + 1) & 3];
        R gpx, gpy;
        grad9<R>(pc[t - 1], pm[t], pc[t + 1], pp[t], pm[t - 1], pm[t + 1], pp[t + 1], pp[t - 1],
                 gpx, gpy);
        collide_cell<S, FRESH, TAU1, GEN>(a, cc, src, dst, gx, gy, gxm, gxp, cell, tt, h, ux, uy,
                                          gpx, gpy, &sm.lo[r & 3][t]);
        // measures of the height at the start of this iteration
        if (!isfinite(h)) any_nan = 1;
        if (measure) {
            mass_add(part, h);
            if constexpr (!LIT && !FRESH) mass_add_lo(part, sm.lo[r & 3][t]);
            const bool wet = h > thr;
            part.wet += wet ? 1 : 0;
            part.hmax = fmax(part.hmax, h);
            part.hmin = fmin(part.hmin, h);
            if ((a.meas_mask & SWB_MEAS_AREA) && wet) {
                const R *hm = sm.h[(r + 7) & 7], *hp = sm.h[(r + 1) & 7];
                R gx2, gy2;
                grad9<R>(hrow[t - 1], hm[t], hrow[t + 1], hp[t], hm[t - 1], hm[t + 1], hp[t + 1],
                         hp[t - 1], gx2, gy2);
                area_add(part, R(sqrt(gx2 * gx2 + gy2 * gy2 + R(1))));
                if (mode == THETA_FIELD)
                    cos_add(part, reinterpret_cast<const R *>(a.cosF)[frow(gy) * Lx + gxf]);
                else if (mode == THETA_WAVE)
                    cos_add(part, cos_col);
            }
        }
        }
    grid_dep_launch();
    any_nan = __syncthreads_or(any_nan);
    if (any_nan && t == 0) a.ctl->nan_flag = 1;
    if (measure) write_partials<NT>(a, part, tt, by * a.tiles_x + bx, sm.red);
}

// Iteration done + 1 of strip (bx, by), dispatched on its rare cases: the
// first iteration after the fields were set (FRESH) and τ = 1 (TAU1).  GEN
// is chosen per launch by the host (step_general): the common kernel
// (scalar θ, no thermal noise, no inclination) leaves that code out and so
// needs fewer registers, which keeps more CTAs per SM.
template <class S, int NT, bool GEN>
__device__ __forceinline__ void march_tile(const StepArgs &a, int bx, int by, long long done,
                                           MarchSmem<S, NT> &sm) {
    const bool fresh = done + 1 == __ldcg(&a.ctl->fresh_step);
    if (fresh) {
        if (a.tau_is_one)
            march_run<S, NT, true, true, GEN>(a, bx, by, done, sm);
        else
            march_run<S, NT, true, false, GEN>(a, bx, by, done, sm);
    } else {
        if (a.tau_is_one)
            march_run<S, NT, false, true, GEN>(a, bx, by, done, sm);
        else
            march_run<S, NT, false, false, GEN>(a, bx, by, done, sm);
    }
}

// ------------------------------------------------------------ pair strips
// The steady step (FP32 arithmetic, τ = 1, no rare forces; scalar θ, or with
// WAVE the moving-wettability θ wave) with two adjacent columns per thread.  A CTA of NT threads owns a strip of
// W = 2 NT - 4 columns and H rows; thread t owns columns c = x0 - 2 + 2t and
// c + 1 for the whole strip.  Lx is even, so c is even: the pair never
// straddles the periodic boundary, and every plane's pair is one aligned
// access, 8 bytes for FP32 populations (and f0 of FP16 storage), 4 bytes for
// FP16 planes.  A row of pulls is nine such loads per thread: the planes
// pulled across x (f1, f5, f8 from x - 1; f3, f6, f7 from x + 1) take the
// neighbouring lane's half of its pair by a warp shuffle, and lanes 0 and 31
// load the one value from outside their warp directly.  The stores are nine
// pair stores.  Shared-memory rings hold pairs, so a pressure or gradient
// stencil of two cells is three pair reads and six scalar reads, and the
// row's index and address arithmetic is paid once per two cells.  The
// per-cell arithmetic is march_run's (moments9, pressure_cell, grad9,
// force_fast, collide_fast): results are bit-identical to the one-column
// strips.
template <int NT>
struct PairSmem {
    float2 h[8][NT];  // heights of the pairs, ring of 5 live rows
    float2 p[4][NT];  // film pressure
    float2 jx[4][NT];
    float2 jy[4][NT];
    float2 lo[4][NT];  // rounding residue of the pulled height
    PartQ red[NT / 32];
    RedPart redd[NT / 32];
};

// One row of pulls of a pair, as loaded: f0 and the planes 1..8 at the
// pair's own two columns (FP32 pairs or FP16 pairs), and in lanes 0 / 31 the
// three values from outside the warp (planes 1, 5, 8 at c - 1 / planes 3, 6,
// 7 at c + 2).
template <class S>
struct PairPull {
    using W = typename std::conditional<S::kHalf, __half2, float2>::type;
    using E = typename std::conditional<S::kHalf, __half, float>::type;
    float2 f0;
    W q[8];
    E e[3];
};

template <class S>
__device__ __forceinline__ float2 pair_f0(const void *b, int i) {
    return __ldg(reinterpret_cast<const float2 *>(reinterpret_cast<const float *>(b) + i));
}

// plane q (1..8) at element i (even): the pair as stored
template <class S>
__device__ __forceinline__ typename PairPull<S>::W pair_ld(const void *b, int pitch, int q, int i) {
    if constexpr (S::kHalf)
        return __ldg(reinterpret_cast<const __half2 *>(S::hp(b, pitch) + (q - 1) * pitch + i));
    else
        return __ldg(reinterpret_cast<const float2 *>(reinterpret_cast<const float *>(b) + q * pitch + i));
}

template <class S>
__device__ __forceinline__ typename PairPull<S>::E one_ld(const void *b, int pitch, int q, int i) {
    if constexpr (S::kHalf)
        return __ldg(S::hp(b, pitch) + (q - 1) * pitch + i);
    else
        return __ldg(reinterpret_cast<const float *>(b) + q * pitch + i);
}

// The pulled values of a plane at the pair, (f_q(c), f_q(c + 1)), from the
// pair as stored (planes not pulled across x), or from the value at c - 1
// and the stored pair (planes pulled from x - 1), or from the stored pair
// and the value at c + 2 (planes pulled from x + 1).  FP16 values are
// widened and unscaled exactly as StoreF16T::ld does, one value at a time.
__device__ __forceinline__ float2 pair_val(float2 w) { return w; }
__device__ __forceinline__ float2 pair_val(__half2 w) {
    return mul2(__half22float2(w), f2(StoreF16::kInv, StoreF16::kInv));
}
__device__ __forceinline__ float2 left_pull(float left, float2 own) { return f2(left, own.x); }
__device__ __forceinline__ float2 right_pull(float2 own, float right) { return f2(own.y, right); }
__device__ __forceinline__ float2 left_pull(__half left, __half2 own) {
    return pair_val(__halves2half2(left, __low2half(own)));
}
__device__ __forceinline__ float2 right_pull(__half2 own, __half right) {
    return pair_val(__halves2half2(__high2half(own), right));
}
// the upper value of the lane below's pair / the lower value of the lane above's
__device__ __forceinline__ float shfl_hi_up(float2 w) { return __shfl_up_sync(0xffffffffu, w.y, 1); }
__device__ __forceinline__ float shfl_lo_down(float2 w) { return __shfl_down_sync(0xffffffffu, w.x, 1); }
__device__ __forceinline__ __half shfl_hi_up(__half2 w) {
    return __high2half(__shfl_up_sync(0xffffffffu, w, 1));
}
__device__ __forceinline__ __half shfl_lo_down(__half2 w) {
    return __low2half(__shfl_down_sync(0xffffffffu, w, 1));
}

// One iteration on pair strip (bx, by): thread t owns columns c = x0 - 2 + 2t
// and c + 1 and marches the strip's rows with shared-memory rings of pairs,
// as march_run does with one column.  Strips of odd index march up, the
// others down (below).  Measured on GB300 (A/B on one box): the 512-member
// ensemble 74.8k -> 78.0k MLUPS; a single 2048² lattice (one wave of strips)
// FP32 53.3 us either way, FP16 storage 55.7 -> 54.7 us.  Results are the
// same bits (the per-cell arithmetic and each cell's neighbours do not
// change).
template <class S, int NT, bool WAVE>
__device__ __forceinline__ void march2_run(const StepArgs &a, int bx, int by, long long done,
                                           PairSmem<NT> &sm) {
    static_assert(!S::kLiteral && NT % 32 == 0, "pair strips: FP32 arithmetic, whole warps");
    using R = float;
    using PP = PairPull<S>;
    constexpr int W = 2 * NT - 4;
    const int t = threadIdx.x, lane = t & 31;
    const int Lx = a.Lx, Ly = a.Ly;
    const int H = a.march_h;
    const int pitch = (int)a.pitch;  // 9 * pitch < 2^31 (checked at creation)
    const long long tt = done + 1;
    const void *src = (done & 1) ? a.fb : a.fa;
    void *dst = (done & 1) ? a.fa : a.fb;
    const int x0 = bx * W, y0 = by * H;
    const int rows = min(H, Ly - y0);
    const R gamma = R(a.gamma), hmin = R(a.hmin), hcrit = R(a.hcrit);
    const bool tiny_y = Ly < 3;
    auto wrow = [&](int yy) {
        return tiny_y ? wrapc(yy, Ly) : (yy < 0 ? yy + Ly : (yy >= Ly ? yy - Ly : yy));
    };
    // Strips of odd index march up, the others down, so that two strips
    // adjacent in y pull the rows they share (each strip's 2 halo rows on
    // either side) at about the same time, while L2 still holds them,
    // instead of one at the start and the other at the end of its march.
    // Y(m): the row at march position m (output rows m = 0 .. rows - 1, halo
    // rows -2, -1, rows, rows + 1); ring(yy): its ring slot, m + 2 either
    // way.  In the rings the previous march row is the row above (y - 1)
    // when marching down and the row below (y + 1) when marching up.
    const bool up = (by & 1) != 0;
    auto Y = [&](int m) { return up ? y0 + rows - 1 - m : y0 + m; };
    auto ring = [&](int yy) { return up ? y0 + rows + 1 - yy : yy - y0 + 2; };
    // this thread's pair (c, c + 1); x0 and Lx are even
    const int cx = wrapc(x0 - 2 + 2 * t, Lx);
    // κ and cospi(θ) of the two columns: the scalar θ, or θ(x, t) of the
    // moving-wettability wave (depends on x only), as march_run computes them
    constexpr bool wave = WAVE;
    R kapA = R(a.kap), kapB = R(a.kap), cosA = R(a.cos_theta), cosB = R(a.cos_theta);
    if constexpr (WAVE) {
        const KapCos<R> wA = wave_at<R>(a, cx, tt), wB = wave_at<R>(a, cx + 1, tt);
        kapA = wA.kap;
        kapB = wB.kap;
        cosA = wA.cs;
        cosB = wB.cs;
    }
    const bool interior = t >= 1 && t < NT - 1 && x0 - 2 + 2 * t < Lx;
    // lanes 0 / 31: the column and planes of the values from outside the warp
    const bool edge = lane == 0 || lane == 31;
    const int ecol = lane == 0 ? (cx == 0 ? Lx - 1 : cx - 1) : (cx + 2 >= Lx ? cx + 2 - Lx : cx + 2);
    const int eq0 = lane == 0 ? 1 : 3, eq1 = lane == 0 ? 5 : 6, eq2 = lane == 0 ? 8 : 7;
    // neighbours of the pair in a ring row of pairs, read as floats (clamped
    // at the CTA's ends, whose values are not used)
    const int tl = t > 0 ? 2 * t - 1 : 0, tr = t < NT - 1 ? 2 * t + 2 : 2 * NT - 1;

    PP fa_, fb_;
    auto issue = [&](PP &P, int yy) {
        const int gy = wrow(yy);
        const int gym = gy == 0 ? Ly - 1 : gy - 1, gyp = gy == Ly - 1 ? 0 : gy + 1;
        const int rc = gy * Lx, rm = gym * Lx, rp = gyp * Lx;
        P.f0 = pair_f0<S>(src, rc + cx);
        P.q[0] = pair_ld<S>(src, pitch, 1, rc + cx);  // f1 from x - 1
        P.q[1] = pair_ld<S>(src, pitch, 2, rm + cx);  // f2 from y - 1
        P.q[2] = pair_ld<S>(src, pitch, 3, rc + cx);  // f3 from x + 1
        P.q[3] = pair_ld<S>(src, pitch, 4, rp + cx);  // f4 from y + 1
        P.q[4] = pair_ld<S>(src, pitch, 5, rm + cx);  // f5 from (x - 1, y - 1)
        P.q[5] = pair_ld<S>(src, pitch, 6, rm + cx);  // f6 from (x + 1, y - 1)
        P.q[6] = pair_ld<S>(src, pitch, 7, rp + cx);  // f7 from (x + 1, y + 1)
        P.q[7] = pair_ld<S>(src, pitch, 8, rp + cx);  // f8 from (x - 1, y + 1)
        if (edge) {
            P.e[0] = one_ld<S>(src, pitch, eq0, rc + ecol);
            P.e[1] = one_ld<S>(src, pitch, eq1, rm + ecol);
            P.e[2] = one_ld<S>(src, pitch, eq2, rp + ecol);
        }
    };
    auto consume = [&](const PP &P, int yy) {
        const int r = ring(yy);  // >= 0
        // the halves of the x-pulled planes that come from the neighbouring pairs
        auto l1 = shfl_hi_up(P.q[0]), l5 = shfl_hi_up(P.q[4]), l8 = shfl_hi_up(P.q[7]);
        auto r3 = shfl_lo_down(P.q[2]), r6 = shfl_lo_down(P.q[5]), r7 = shfl_lo_down(P.q[6]);
        if (lane == 0) {
            l1 = P.e[0];
            l5 = P.e[1];
            l8 = P.e[2];
        }
        if (lane == 31) {
            r3 = P.e[0];
            r6 = P.e[1];
            r7 = P.e[2];
        }
        float2 F[9];
        F[0] = P.f0;
        F[1] = left_pull(l1, P.q[0]);
        F[2] = pair_val(P.q[1]);
        F[3] = right_pull(P.q[2], r3);
        F[4] = pair_val(P.q[3]);
        F[5] = left_pull(l5, P.q[4]);
        F[6] = right_pull(P.q[5], r6);
        F[7] = right_pull(P.q[6], r7);
        F[8] = left_pull(l8, P.q[7]);
        R fA[9], fB[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            fA[q] = F[q].x;
            fB[q] = F[q].y;
        }
        R hA, jxA, jyA, hB, jxB, jyB;
        moments9<false>(fA, hA, jxA, jyA);
        moments9<false>(fB, hB, jxB, jyB);
        sm.h[r & 7][t] = f2(hA, hB);
        sm.jx[r & 3][t] = f2(jxA, jxB);
        sm.jy[r & 3][t] = f2(jyA, jyB);
        sm.lo[r & 3][t] = f2(moments_lo(fA, hA), moments_lo(fB, hB));
    };
    auto pressure_row = [&](int yy) {
        const int r = ring(yy);  // >= 1
        const float2 *hm = sm.h[(r + 7) & 7], *hc = sm.h[r & 7], *hp = sm.h[(r + 1) & 7];
        if (up) {  // rows y - 1 and y + 1
            const float2 *sw = hm;
            hm = hp;
            hp = sw;
        }
        const float2 m = hm[t], c = hc[t], pl = hp[t];
        const float *m1 = reinterpret_cast<const float *>(hm), *c1 = reinterpret_cast<const float *>(hc),
                    *p1 = reinterpret_cast<const float *>(hp);
        // ip = h[i-1,j], jp = h[i,j-1], im = h[i+1,j], jm = h[i,j+1], ...
        const R pA = pressure_cell<false, R>(c.x, c1[tl], m.x, c.y, pl.x, m1[tl], m.y, pl.y, p1[tl],
                                             kapA, gamma, hmin, hcrit, a.n, a.m);
        const R pB = pressure_cell<false, R>(c.y, c.x, m.y, c1[tr], pl.y, m.x, m1[tr], p1[tr], pl.x,
                                             kapB, gamma, hmin, hcrit, a.n, a.m);
        sm.p[r & 3][t] = f2(pA, pB);
    };

    issue(fa_, Y(-2));
    issue(fb_, Y(-1));
    consume(fa_, Y(-2));
    issue(fa_, Y(0));
    consume(fb_, Y(-1));
    issue(fb_, Y(1));
    consume(fa_, Y(0));
    issue(fa_, Y(2));
    consume(fb_, Y(1));
    __syncthreads();
    pressure_row(Y(-1));
    pressure_row(Y(0));

    const CellConst<R> cc = cell_consts<R>(a, tt, a.mass_corr ? __ldcg(&a.ctl->corr[tt & 1]) : 0.0);
    const R thr = R(a.hthresh);
    const bool measure = a.meas_mask || a.mass_corr;
    PartQ part;
    part_init(part);
    int any_nan = 0;

#pragma unroll 1
    for (int j = 0; j < rows; ++j) {
        const int y = Y(j);
        consume(fa_, Y(j + 2));
        if (j + 1 < rows) issue(fa_, Y(j + 3));  // one row ahead
        __syncthreads();
        pressure_row(Y(j + 1));
        __syncthreads();
        if (!interior) continue;
        // ---- output row y, columns cx, cx + 1 ----
        const int r = ring(y);
        const int cellA = wrow(y) * Lx + cx;
        const float2 h2 = sm.h[r & 7][t], jx2 = sm.jx[r & 3][t], jy2 = sm.jy[r & 3][t];
        const float2 lo2 = sm.lo[r & 3][t];
        const float2 *pm = sm.p[(r + 3) & 3], *pc = sm.p[r & 3], *pp = sm.p[(r + 1) & 3];
        if (up) {  // rows y - 1 and y + 1
            const float2 *sw = pm;
            pm = pp;
            pp = sw;
        }
        const float2 m = pm[t], c = pc[t], pl = pp[t];
        const float *m1 = reinterpret_cast<const float *>(pm), *c1 = reinterpret_cast<const float *>(pc),
                    *p1 = reinterpret_cast<const float *>(pp);
        float foA[9], foB[9];
        [[maybe_unused]] __half2 hbA[4], hbB[4];
        {
            R ux, uy, gpx, gpy;
            velocity<false>(h2.x, jx2.x, jy2.x, ux, uy);
            grad9<R>(c1[tl], m.x, c.y, pl.x, m1[tl], m.y, pl.y, p1[tl], gpx, gpy);  // h∇p!
            const float2 F = force_fast(cc, h2.x, ux, uy, gpx, gpy);
            collide_fast<S, false, true, true>(cc, h2.x, ux, uy, F.x, F.y, h2.x, nullptr, cellA, tt,
                                         &lo2.x, foA, hbA);
        }
        {
            R ux, uy, gpx, gpy;
            velocity<false>(h2.y, jx2.y, jy2.y, ux, uy);
            grad9<R>(c.x, m.y, c1[tr], pl.y, m.x, m1[tr], p1[tr], pl.x, gpx, gpy);
            const float2 F = force_fast(cc, h2.y, ux, uy, gpx, gpy);
            collide_fast<S, false, true, true>(cc, h2.y, ux, uy, F.x, F.y, h2.y, nullptr, cellA + 1, tt,
                                         &lo2.y, foB, hbB);
        }
        reinterpret_cast<float2 *>(reinterpret_cast<float *>(dst) + cellA)[0] = f2(foA[0], foB[0]);
        if constexpr (S::kHalf) {
            __half2 *hpl = reinterpret_cast<__half2 *>(const_cast<__half *>(S::hp(dst, pitch)) + cellA);
            const int pitch2 = pitch >> 1;  // pitch in pairs (pitch is a multiple of 64)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                hpl[(2 * k) * pitch2] = __lows2half2(hbA[k], hbB[k]);
                hpl[(2 * k + 1) * pitch2] = __highs2half2(hbA[k], hbB[k]);
            }
        } else {
            float2 *d2 = reinterpret_cast<float2 *>(reinterpret_cast<float *>(dst) + cellA);
            const int pitch2 = pitch >> 1;
#pragma unroll
            for (int q = 1; q < 9; ++q) d2[q * pitch2] = f2(foA[q], foB[q]);
        }
        // measures of the heights at the start of this iteration
        if (!isfinite(h2.x) || !isfinite(h2.y)) any_nan = 1;
        if (measure) {
            mass_add(part, h2.x);
            mass_add(part, h2.y);
            mass_add_lo(part, lo2.x);
            mass_add_lo(part, lo2.y);
            const bool wA = h2.x > thr, wB = h2.y > thr;
            part.wet += (wA ? 1 : 0) + (wB ? 1 : 0);
            part.hmax = fmaxf(part.hmax, fmaxf(h2.x, h2.y));
            part.hmin = fminf(part.hmin, fminf(h2.x, h2.y));
            if ((a.meas_mask & SWB_MEAS_AREA) && (wA || wB)) {
                const float2 *hm = sm.h[(r + 7) & 7], *hc = sm.h[r & 7], *hp = sm.h[(r + 1) & 7];
                if (up) {  // rows y - 1 and y + 1
                    const float2 *sw = hm;
                    hm = hp;
                    hp = sw;
                }
                const float2 hm2 = hm[t], hp2 = hp[t];
                const float *hm1 = reinterpret_cast<const float *>(hm),
                            *hc1 = reinterpret_cast<const float *>(hc),
                            *hp1 = reinterpret_cast<const float *>(hp);
                R gx2, gy2;
                if (wA) {
                    grad9<R>(hc1[tl], hm2.x, h2.y, hp2.x, hm1[tl], hm2.y, hp2.y, hp1[tl], gx2, gy2);
                    area_add(part, R(sqrt(gx2 * gx2 + gy2 * gy2 + R(1))));
                    if constexpr (wave) cos_add(part, cosA);
                }
                if (wB) {
                    grad9<R>(h2.x, hm2.y, hc1[tr], hp2.y, hm2.x, hm1[tr], hp1[tr], hp2.x, gx2, gy2);
                    area_add(part, R(sqrt(gx2 * gx2 + gy2 * gy2 + R(1))));
                    if constexpr (wave) cos_add(part, cosB);
                }
            }
        }
    }
    grid_dep_launch();
    any_nan = __syncthreads_or(any_nan);
    if (any_nan && t == 0) a.ctl->nan_flag = 1;
    if (measure) write_partials<NT>(a, part, tt, by * a.tiles_x + bx, sm.red);
}

// One iteration of the common steady step on pair strips, plus (when
// measures are kept and k > 0) the reducer CTA, block 0.
template <class S, int NT, bool WAVE>
__global__ void __launch_bounds__(NT) pair_step_kernel(const StepArgs a, int k) {
    __shared__ __align__(16) PairSmem<NT> sm;
    grid_dep_wait();
    int b = blockIdx.x;
    if (needs_partials(a) && k > 0) {
        if (b == 0) {
            grid_dep_launch();
            reduce_step<NT>(a, a.ctl->step_base + k, sm.redd);
            return;
        }
        b -= 1;
    }
    march2_run<S, NT, WAVE>(a, b % a.tiles_x, b / a.tiles_x, a.ctl->step_base + k, sm);
}

// ------------------------------------------------------------ 2D tiles
// For lattices whose populations stay in L2, the strip march above is bound
// by one L2 round trip per row.  A 2D tile instead pulls all its cells at
// once: a CTA of kT2NT threads owns kT2X x kT2Y output cells and
//   A. pulls the (kT2X+4) x (kT2Y+4) cells around them (three per thread,
//      27 loads in flight) and keeps h, and j and the rounding residue of
//      the output cells, in shared memory;
//   B. computes p on the (kT2X+2) x (kT2Y+2) cells around the outputs;
//   C. computes forces and collision of the outputs (collide_cell, the same
//      code as the strips: FP32 results are identical).
// Halo pulls are 1.4x the outputs; they are served by L2.
constexpr int kT2X = 32, kT2Y = 16, kT2NT = 256;
constexpr int kT2HX = kT2X + 4, kT2HY = kT2Y + 4;  // heights
constexpr int kT2PX = kT2X + 2, kT2PY = kT2Y + 2;  // pressures
constexpr int kT2Out = kT2X * kT2Y;
static_assert(kT2HX * kT2HY <= 3 * kT2NT, "three pulls per thread");
static_assert(kT2PX * kT2PY <= 3 * kT2NT, "three pressures per thread");
static_assert(kT2Out == 2 * kT2NT, "two outputs per thread");

template <class S>
struct TileSmem {
    using R = typename S::real;
    R h[kT2HY * kT2HX];
    R p[kT2PY * kT2PX];
    R jx[kT2Out];
    R jy[kT2Out];
    R lo[kT2Out];
    StepPart<R> red[kT2NT / 32];
    RedPart redd[kT2NT / 32];
};

template <class S, bool FRESH, bool TAU1>
__device__ __forceinline__ void tile2d_run(const StepArgs &a, int bx, int by, long long done,
                                           TileSmem<S> &sm) {
    using R = typename S::real;
    static_assert(!S::kLiteral, "2D tiles: FP32 arithmetic only");
    const int t = threadIdx.x;
    const int Lx = a.Lx, Ly = a.Ly;
    const int pitch = (int)a.pitch;  // 9 * pitch < 2^31 (checked at creation)
    const long long tt = done + 1;
    const void *src = (done & 1) ? a.fb : a.fa;
    void *dst = (done & 1) ? a.fa : a.fb;
    const int x0 = bx * kT2X, y0 = by * kT2Y;
    const R gamma = R(a.gamma), hmin = R(a.hmin), hcrit = R(a.hcrit);
    const int mode = a.theta_mode;
    const double corr = (!FRESH && a.mass_corr) ? __ldcg(&a.ctl->corr[tt & 1]) : 0.0;
    int fsx = 0, fsy = 0;  // offset of a moving θ field
    if (mode == THETA_FIELD) substrate_shift(a, tt, &fsx, &fsy);

    // A. pulls and moments
    R ft[3][9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int i = t + k * kT2NT;
        if (i < kT2HX * kT2HY) {
            const int gx = wrapc(x0 - 2 + i % kT2HX, Lx), gy = wrapc(y0 - 2 + i / kT2HX, Ly);
            if constexpr (FRESH) {
                ft[k][0] = reinterpret_cast<const R *>(a.hF)[gy * Lx + gx];
            } else {
                const int gxm = gx == 0 ? Lx - 1 : gx - 1, gxp = gx == Lx - 1 ? 0 : gx + 1;
                const int gym = gy == 0 ? Ly - 1 : gy - 1, gyp = gy == Ly - 1 ? 0 : gy + 1;
                pull9<S>(src, pitch, Lx, gx, gy, gxm, gxp, gym, gyp, ft[k]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int i = t + k * kT2NT;
        if (i < kT2HX * kT2HY) {
            const int lx = i % kT2HX, ly = i / kT2HX;
            if constexpr (FRESH) {
                sm.h[i] = ft[k][0];
            } else {
                R h, jx, jy;
                moments9<false>(ft[k], h, jx, jy);
                sm.h[i] = h;
                if (lx >= 2 && lx < kT2X + 2 && ly >= 2 && ly < kT2Y + 2) {
                    const int o = (ly - 2) * kT2X + (lx - 2);
                    sm.jx[o] = jx;
                    sm.jy[o] = jy;
                    sm.lo[o] = moments_lo(ft[k], h);
                }
            }
        }
    }
    __syncthreads();

    // B. film pressure around the outputs
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int i = t + k * kT2NT;
        if (i < kT2PX * kT2PY) {
            const int px = i % kT2PX, py = i / kT2PX;
            const R *hm = sm.h + py * kT2HX + px + 1;  // row above, column of the cell
            const R *hc = hm + kT2HX, *hp = hc + kT2HX;
            R kap = R(a.kap);
            if (mode != THETA_SCALAR) {
                const int gx = wrapc(x0 - 1 + px, Lx);
                if (mode == THETA_FIELD) {
                    const int gy = wrapc(y0 - 1 + py - fsy, Ly);
                    kap = reinterpret_cast<const R *>(a.kapF)[gy * Lx + wrapc(gx - fsx, Lx)];
                } else {
                    kap = wave_at<R>(a, gx, tt).kap;
                }
            }
            // ip = h[i-1,j], jp = h[i,j-1], im = h[i+1,j], jm = h[i,j+1], ...
            sm.p[i] = pressure_cell<false, R>(hc[0], hc[-1], hm[0], hc[1], hp[0], hm[-1], hm[1],
                                              hp[1], hp[-1], kap, gamma, hmin, hcrit, a.n, a.m);
        }
    }
    __syncthreads();

    // C. forces, collision, stores and measures of the outputs
    const CellConst<R> cc = cell_consts<R>(a, tt, corr);
    const R thr = R(a.hthresh);
    const bool measure = a.meas_mask || a.mass_corr;
    StepPart<R> part;
    part_init(part);
    int any_nan = 0;
#pragma unroll 1
    for (int k = 0; k < 2; ++k) {
        const int o = t + k * kT2NT;
        const int ox = o % kT2X, oy = o / kT2X;
        const int gx = x0 + ox, gy = y0 + oy;
        if (gx >= Lx || gy >= Ly) continue;
        const int cell = gy * Lx + gx;
        const int gxm = gx == 0 ? Lx - 1 : gx - 1, gxp = gx == Lx - 1 ? 0 : gx + 1;
        const R *hc = sm.h + (oy + 2) * kT2HX + ox + 2;
        const R h = hc[0];
        R ux, uy;
        if constexpr (FRESH) {
            ux = reinterpret_cast<const R *>(a.uxF)[cell];
            uy = reinterpret_cast<const R *>(a.uyF)[cell];
        } else {
            velocity<false>(h, sm.jx[o], sm.jy[o], ux, uy);
        }
        const R *pc = sm.p + (oy + 1) * kT2PX + ox + 1, *pm = pc - kT2PX, *pp = pc + kT2PX;
        R gpx, gpy;
        grad9<R>(pc[-1], pm[0], pc[1], pp[0], pm[-1], pm[1], pp[1], pp[-1], gpx, gpy);
        collide_cell<S, FRESH, TAU1, true>(a, cc, src, dst, gx, gy, gxm, gxp, cell, tt, h, ux, uy,
                                           gpx, gpy, &sm.lo[o]);
        if (!isfinite(h)) any_nan = 1;
        if (measure) {
            mass_add(part, h);
            if constexpr (!FRESH) mass_add_lo(part, sm.lo[o]);
            const bool wet = h > thr;
            part.wet += wet ? 1 : 0;
            part.hmax = fmax(part.hmax, h);
            part.hmin = fmin(part.hmin, h);
            if ((a.meas_mask & SWB_MEAS_AREA) && wet) {
                const R *hm = hc - kT2HX, *hp = hc + kT2HX;
                R gx2, gy2;
                grad9<R>(hc[-1], hm[0], hc[1], hp[0], hm[-1], hm[1], hp[1], hp[-1], gx2, gy2);
                area_add(part, R(sqrt(gx2 * gx2 + gy2 * gy2 + R(1))));
                if (mode == THETA_FIELD) {
                    cos_add(part, reinterpret_cast<const R *>(
                                      a.cosF)[wrapc(gy - fsy, Ly) * Lx + wrapc(gx - fsx, Lx)]);
                } else if (mode == THETA_WAVE) {
                    cos_add(part, wave_at<R>(a, gx, tt).cs);
                }
            }
        }
    }
    grid_dep_launch();
    any_nan = __syncthreads_or(any_nan);
    if (any_nan && t == 0) a.ctl->nan_flag = 1;
    if (measure) write_partials<kT2NT>(a, part, tt, by * a.tiles_x + bx, sm.red);
}

template <class S>
__device__ __forceinline__ void tile2d_tile(const StepArgs &a, int bx, int by, long long done,
                                            TileSmem<S> &sm) {
    const bool fresh = done + 1 == __ldcg(&a.ctl->fresh_step);
    if (fresh) {
        if (a.tau_is_one)
            tile2d_run<S, true, true>(a, bx, by, done, sm);
        else
            tile2d_run<S, true, false>(a, bx, by, done, sm);
    } else {
        if (a.tau_is_one)
            tile2d_run<S, false, true>(a, bx, by, done, sm);
        else
            tile2d_run<S, false, false>(a, bx, by, done, sm);
    }
}

// One iteration, one CTA per 2D tile plus the reducer (block 0).
template <class S>
__global__ void __launch_bounds__(kT2NT, 4) fused_tile_kernel(const StepArgs a, int k) {
    __shared__ TileSmem<S> sm;
    grid_dep_wait();
    int b = blockIdx.x;
    if (needs_partials(a) && k > 0) {
        if (b == 0) {
            grid_dep_launch();
            reduce_step<kT2NT>(a, a.ctl->step_base + k, sm.redd);
            return;
        }
        b -= 1;
    }
    tile2d_tile<S>(a, b % a.tiles_x, b / a.tiles_x, a.ctl->step_base + k, sm);
}

// ------------------------------------------------------------ multi-step
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Barrier across all CTAs of a cooperative launch (all co-resident), in two
// levels so that no counter takes more than ~G/kBarGroups arrivals: CTA b
// arrives on the counter of group b % kBarGroups; the last of a group
// re-arms that counter and arrives on the top counter; the last group
// re-arms the top counter and bumps every group's generation word, which the
// group's CTAs poll (each word on its own 128-byte line).  Arrivals are
// released by a device-scope fence.  Every wait is bounded by
// kBarrierTimeoutNs and a spin cap; on expiry the CTA raises *err, and all
// CTAs waiting now or later give up.  Returns false when the launch must stop.
__device__ __forceinline__ bool grid_barrier(unsigned int *bar, int *err, unsigned int G) {
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0) {
        const unsigned int grp = blockIdx.x % kBarGroups;
        const unsigned int ngroups = G < kBarGroups ? G : kBarGroups;
        const unsigned int gsize = (G - 1 - grp) / kBarGroups + 1;
        unsigned int *sub = bar + kBarStride * (1 + grp);
        volatile unsigned int *gen = bar + kBarStride * (1 + kBarGroups + grp);
        volatile int *verr = err;
        const unsigned int g0 = *gen;
        __threadfence();
        bool released = false;
        if (atomicAdd(sub, 1u) == gsize - 1) {
            atomicExch(sub, 0u);
            __threadfence();
            if (atomicAdd(bar, 1u) == ngroups - 1) {
                atomicExch(bar, 0u);
                __threadfence();
                for (unsigned int k = 0; k < ngroups; ++k)
                    atomicAdd(bar + kBarStride * (1 + kBarGroups + k), 1u);
                released = true;
            }
        }
        if (!released) {
            const unsigned long long t0 = globaltimer_ns();
            unsigned int spins = 0;
            while (*gen == g0) {
                if (*verr) {
                    ok = 0;
                    break;
                }
                if ((++spins & 255u) == 0u &&
                    (globaltimer_ns() - t0 > kBarrierTimeoutNs || spins > (1u << 28))) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    return __syncthreads_and(ok) != 0;
}

// n time_loop iterations of one lattice in one cooperative launch.  CTA b
// walks tiles b, b + G, ... of each iteration (strips of NT threads, or 2D
// tiles when T2D); CTA G - 1 also reduces the previous iteration's measures
// (with G = tiles + 1 it does nothing else), and after the last barrier the
// last iteration's, and advances step_base.  S uses L2 loads (LdCG):
// populations written by other CTAs one iteration earlier are read after a
// grid barrier.
template <class S, int NT, bool T2D>
__global__ void __launch_bounds__(NT, T2D ? 2 : 1) fused_run_kernel(const StepArgs a, int n) {
    using Smem = typename std::conditional<T2D, TileSmem<S>, MarchSmem<S, NT>>::type;
    __shared__ Smem sm;
    const int G = gridDim.x, b = blockIdx.x;
    const int ntiles = a.tiles_x * a.tiles_y;
    const bool red = needs_partials(a);
    const long long base = __ldcg(&a.ctl->step_base);
    for (int k = 0; k < n; ++k) {
        if (red && k > 0 && b == G - 1) {
            reduce_step<NT>(a, base + k, sm.redd);
            __syncthreads();
        }
        for (int e = b; e < ntiles; e += G) {
            if constexpr (T2D)
                tile2d_tile<S>(a, e % a.tiles_x, e / a.tiles_x, base + k, sm);
            else
                march_tile<S, NT, true>(a, e % a.tiles_x, e / a.tiles_x, base + k, sm);
            __syncthreads();
        }
        if (!grid_barrier(a.bar, &a.ctl->bar_err, (unsigned int)G)) return;
    }
    if (b == G - 1) {
        if (red && n > 0) reduce_step<NT>(a, base + n, sm.redd);
        __syncthreads();
        if (threadIdx.x == 0) a.ctl->step_base = base + n;
    }
}

// Iterations a single-lattice step kernel is compiled for.  kFormAny
// decides at run time (the first iteration after the fields were set, τ = 1
// or not); the steady forms leave the first-iteration code out, and the τ
// code they do not need, so that the common step (steady, τ = 1, no rare
// forces) is allocated the registers of its own path (64 instead of 80 for
// FP32 strips of 64 threads: 16 CTAs per SM instead of 12).  The host runs
// the first iteration after the fields were set as a one-step sequence of
// kFormAny.
enum StepForm { kFormAny = 0, kFormSteadyTau1 = 1, kFormSteady = 2 };

// Single lattice: one CTA per strip, plus (when measures are kept and k > 0)
// a reducer CTA, block 0, for the previous iteration's measures.
template <class S, int NT, bool GEN, int FORM = kFormAny, bool WAVE = false>
__global__ void __launch_bounds__(NT) fused_step_kernel(const StepArgs a, int k) {
    __shared__ MarchSmem<S, NT> sm;
    grid_dep_wait();
    int b = blockIdx.x;
    if (needs_partials(a) && k > 0) {
        if (b == 0) {
            grid_dep_launch();
            reduce_step<NT>(a, a.ctl->step_base + k, sm.redd);
            return;
        }
        b -= 1;
    }
    const long long done = a.ctl->step_base + k;
    if constexpr (FORM == kFormSteadyTau1)
        march_run<S, NT, false, true, GEN, WAVE>(a, b % a.tiles_x, b / a.tiles_x, done, sm);
    else if constexpr (FORM == kFormSteady)
        march_run<S, NT, false, false, GEN, WAVE>(a, b % a.tiles_x, b / a.tiles_x, done, sm);
    else
        march_tile<S, NT, GEN>(a, b % a.tiles_x, b / a.tiles_x, done, sm);
}

// Closes a sequence of n step launches: the last iteration's measures, then
// the step counter.  One CTA.
template <int NT>
__global__ void __launch_bounds__(NT) advance_kernel(const StepArgs a, int n) {
    __shared__ RedPart redd[NT / 32];
    grid_dep_wait();
    grid_dep_launch();
    const long long s = a.ctl->step_base + n;
    if (needs_partials(a) && n > 0) reduce_step<NT>(a, s, redd);
    __syncthreads();
    if (threadIdx.x == 0) a.ctl->step_base = s;
}

// Batch: persistent CTAs walk a packed table of strips of many lattices;
// entries with tx = -1 reduce their lattice's previous iteration.
// FORM = kFormSteadyTau1 when no lattice is at its first iteration after
// its fields were set and every lattice has τ = 1 (the host knows both).
template <class S, int NT, bool GEN, int FORM = kFormAny, bool WAVE = false>
__global__ void __launch_bounds__(NT) batch_step_kernel(const StepArgs *__restrict__ args,
                                                        const TileRef *__restrict__ tiles,
                                                        int ntiles, int k) {
    __shared__ MarchSmem<S, NT> sm;
    __shared__ StepArgs sa;
    grid_dep_wait();
    for (int e = blockIdx.x; e < ntiles; e += gridDim.x) {
        if (e + (int)gridDim.x >= ntiles) grid_dep_launch();  // this CTA's last entry
        const TileRef tr = tiles[e];
        if (threadIdx.x == 0) {
            sa = args[tr.lattice];
            // a lattice that has stopped: strips of no output rows, which
            // write nothing (a branch around the march would cost registers)
            if (sa.ctl->step_base + k >= sa.stop_at) sa.march_h = 0;
        }
        __syncthreads();
        const long long done = sa.ctl->step_base + k;
        if (tr.tx >= 0) {
            if constexpr (FORM == kFormSteadyTau1)
                march_run<S, NT, false, true, GEN, WAVE>(sa, tr.tx, tr.ty, done, sm);
            else
                march_tile<S, NT, GEN>(sa, tr.tx, tr.ty, done, sm);
        } else if (k > 0 && done <= sa.stop_at)
            reduce_step<NT>(sa, done, sm.redd);
        __syncthreads();
    }
}

// Batch on pair strips: the table's strips are pair strips of NT threads;
// every lattice is at a steady τ = 1 iteration without rare forces or θ
// field (WAVE: some lattice has the θ wave) and has even Lx (the host knows).
// Register budget: left alone the compiler gives the WAVE form 148 registers
// (6 CTAs of 64 threads per SM) and the plain form 128; capped at 128 and 96
// (8 and 10 CTAs) they spill nothing and 24 bytes.  Measured on GB300: the
// θ-wave serving mix 53 -> 74 GLUPS at 128, the plain ensemble 70 -> 74
// GLUPS at 96 (the WAVE form at 96 spills 80 bytes and is slower).
template <int NT, bool WAVE>
constexpr int batch_pair_min_blocks() {
    return 65536 / ((WAVE || NT < 64 ? 128 : 96) * NT);
}
template <class S, int NT, bool WAVE>
__global__ void __launch_bounds__(NT, (batch_pair_min_blocks<NT, WAVE>())) batch_pair_kernel(const StepArgs *__restrict__ args,
                                                                 const TileRef *__restrict__ tiles,
                                                                 int ntiles, int k) {
    __shared__ __align__(16) PairSmem<NT> sm;
    __shared__ StepArgs sa;
    grid_dep_wait();
    for (int e = blockIdx.x; e < ntiles; e += gridDim.x) {
        if (e + (int)gridDim.x >= ntiles) grid_dep_launch();  // this CTA's last entry
        const TileRef tr = tiles[e];
        if (threadIdx.x == 0) {
            sa = args[tr.lattice];
            if (sa.ctl->step_base + k >= sa.stop_at) sa.march_h = 0;  // stopped: no output rows
        }
        __syncthreads();
        const long long done = sa.ctl->step_base + k;
        if (tr.tx >= 0) {
            if (WAVE && sa.theta_mode == THETA_WAVE) {
                march2_run<S, NT, WAVE>(sa, tr.tx, tr.ty, done, sm);
            } else {
                march2_run<S, NT, false>(sa, tr.tx, tr.ty, done, sm);
            }
        } else if (k > 0 && done <= sa.stop_at) {
            reduce_step<NT>(sa, done, sm.redd);
        }
        __syncthreads();
    }
}

// One CTA per lattice closes a batch sequence of n launches.
template <int NT>
__global__ void __launch_bounds__(NT) batch_advance_kernel(const StepArgs *__restrict__ args,
                                                           int n) {
    __shared__ RedPart redd[NT / 32];
    __shared__ StepArgs sa;
    grid_dep_wait();
    grid_dep_launch();
    if (threadIdx.x == 0) sa = args[blockIdx.x];
    __syncthreads();
    // a lattice that stopped during the sequence had its last iteration
    // reduced by the launch after it
    const long long s = sa.ctl->step_base + n;
    if (needs_partials(sa) && n > 0 && s <= sa.stop_at) reduce_step<NT>(sa, s, redd);
    __syncthreads();
    if (threadIdx.x == 0) sa.ctl->step_base = s < sa.stop_at ? s : sa.stop_at;
}

// thermal!(fx, fy, h, kbt, mu, delta) of the current height field for
// iteration t: the fluctuating forces the fused step adds (swb_thermal_field).
template <class S>
__global__ void thermal_field_kernel(const StepArgs a, long long t, double *fx, double *fy) {
    using R = typename S::real;
    const long long N = (long long)a.Lx * a.Ly;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x) {
        const R h = reinterpret_cast<const R *>(a.hF)[c];
        R zx, zy;
        thermal_normals(a.seed, c, t, zx, zy);
        const R sg = thermal_sigma<S::kLiteral, R>(R(a.k6), h, R(a.delta));
        fx[c] = (double)(zx * sg);
        fy[c] = (double)(zy * sg);
    }
}

// moments! into the fields (used when the host reads h/u).
template <class S>
__global__ void moments_kernel(const StepArgs a) {
    using R = typename S::real;
    const int Lx = a.Lx, Ly = a.Ly;
    const long long step = a.ctl->step_base;
    const void *src = (step & 1) ? a.fb : a.fa;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < (long long)Lx * Ly;
         c += (long long)gridDim.x * blockDim.x) {
        const int gx = (int)(c % Lx), gy = (int)(c / Lx);
        const int gxm = gx == 0 ? Lx - 1 : gx - 1, gxp = gx == Lx - 1 ? 0 : gx + 1;
        const int gym = gy == 0 ? Ly - 1 : gy - 1, gyp = gy == Ly - 1 ? 0 : gy + 1;
        R ft[9], h, jx, jy, ux, uy;
        pull9<S>(src, (int)a.pitch, Lx, gx, gy, gxm, gxp, gym, gyp, ft);
        moments9<S::kLiteral>(ft, h, jx, jy);
        velocity<S::kLiteral>(h, jx, jy, ux, uy);
        reinterpret_cast<R *>(a.hF)[c] = h;
        reinterpret_cast<R *>(a.uxF)[c] = ux;
        reinterpret_cast<R *>(a.uyF)[c] = uy;
    }
}

// Streamed populations (the reference's fout) into a Float64 array.
template <class S>
__global__ void fout_kernel(const StepArgs a, double *out) {
    using R = typename S::real;
    const int Lx = a.Lx, Ly = a.Ly;
    const long long N = (long long)Lx * Ly;
    const long long step = a.ctl->step_base;
    const void *src = (step & 1) ? a.fb : a.fa;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x) {
        const int gx = (int)(c % Lx), gy = (int)(c / Lx);
        const int gxm = gx == 0 ? Lx - 1 : gx - 1, gxp = gx == Lx - 1 ? 0 : gx + 1;
        const int gym = gy == 0 ? Ly - 1 : gy - 1, gyp = gy == Ly - 1 ? 0 : gy + 1;
        R ft[9];
        pull9<S>(src, (int)a.pitch, Lx, gx, gy, gxm, gxp, gym, gyp, ft);
        for (int q = 0; q < 9; ++q) out[q * N + c] = (double)ft[q];
    }
}

// Film pressure of the current height field (filmpressure! applied now).
template <class S>
__global__ void pressure_now_kernel(const StepArgs a, double *out) {
    using R = typename S::real;
    const int Lx = a.Lx, Ly = a.Ly;
    const R *h = reinterpret_cast<const R *>(a.hF);
    const long long t = a.ctl->step_base + 1;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < (long long)Lx * Ly;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % Lx), j = (int)(c / Lx);
        const int im1 = i == 0 ? Lx - 1 : i - 1, ip1 = i == Lx - 1 ? 0 : i + 1;
        const int jm1 = j == 0 ? Ly - 1 : j - 1, jp1 = j == Ly - 1 ? 0 : j + 1;
        R kap;
        if (a.theta_mode == THETA_SCALAR)
            kap = R(a.kap);
        else if (a.theta_mode == THETA_FIELD) {
            int sx, sy;
            substrate_shift(a, t, &sx, &sy);
            kap = reinterpret_cast<const R *>(a.kapF)[wrapc(j - sy, Ly) * Lx + wrapc(i - sx, Lx)];
        } else
            kap = wave_at<R>(a, i, t).kap;
        out[c] = (double)pressure_cell<S::kLiteral, R>(
            h[c], h[j * Lx + im1], h[jm1 * Lx + i], h[j * Lx + ip1], h[jp1 * Lx + i],
            h[jm1 * Lx + im1], h[jm1 * Lx + ip1], h[jp1 * Lx + ip1], h[jp1 * Lx + im1], kap,
            R(a.gamma), R(a.hmin), R(a.hcrit), a.n, a.m);
    }
}

}  // namespace swb
