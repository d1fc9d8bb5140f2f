// swb_resident.cu -- resident tiles: many time_loop iterations of one
// FP32-arithmetic lattice (FP32 or FP16 storage) in one cooperative launch,
// every CTA keeping the populations of its tile in shared memory.
//
// For lattices whose state fits in the GPU's shared memory (512² FP32: 9.4
// MB of populations against 152 x 227 KB), the strip march is bound by one
// L2 round trip per row and by the launch per iteration.  Here each CTA owns
// a tile of kResTW x h cells for the whole launch.  Per iteration it
//   0. loads from L2 only the 3-cell ring around its tile (populations the
//      neighbouring tiles wrote in the previous iteration; the first
//      iteration loads the whole region);
//   A. pulls and takes the moments of the tile and 2 rings (h on the tile
//      and 2 rings; j and the height's rounding residue on the tile);
//   B. computes the film pressure on the tile and 1 ring;
//   C. forces, equilibrium and collision of the tile: the new populations go
//      to shared memory (in place: every read of phase A is done) and to the
//      global buffer of the iteration, for the neighbours and the host;
// then all CTAs meet at the bounded grid barrier of the multi-step kernel.
// The per-cell arithmetic is the strip march's (moments9, pressure_cell,
// grad9, force_fast, collide_fast), so results are bit-identical to it; the
// measures go through the same integer accumulators and reducer.  The common
// steady τ = 1 step only (scalar θ, no rare forces): the host runs every
// other iteration on strips.
#include <type_traits>

#include "swb_step_impl.cuh"

namespace swb {

namespace {

constexpr int kEW = kResTW + 6;  // population rows: tile + 3-cell ring each side
constexpr int kHW = kResTW + 4;  // heights: tile + 2 rings
constexpr int kPW = kResTW + 2;  // pressure: tile + 1 ring

// Shared memory of a tile of h rows (floats, then the reduction slots).
__host__ __device__ constexpr size_t res_floats(int h) {
    return (size_t)9 * (h + 6) * kEW + (size_t)(h + 4) * kHW + (size_t)(h + 2) * kPW +
           (size_t)3 * h * kResTW;
}

// Barrier of the resident-tile launch (all CTAs co-resident, at most a few
// hundred).  Arrival k of every CTA adds 1 to one counter (fire-and-forget,
// after a fence that releases the CTA's writes); a CTA waits until the
// counter reaches (k + 1) G, polling it without sleeping, so the last
// arrival releases everybody with no further round trip.  The counter grows
// through the launch and the launch's last CTA sets it back to 0 (no CTA
// waits on it any more by then).  Every wait is bounded like the multi-step
// kernel's (kBarrierTimeoutNs by %globaltimer and a spin cap): on expiry the
// CTA raises *err and all CTAs stop at their next wait; the host re-arms the
// words.  The counter is the multi-step barrier's top counter, which that
// barrier also leaves at 0.
__device__ __forceinline__ bool res_wait(unsigned int *ctr, int *err, unsigned int target) {
    int ok = 1;
    if (threadIdx.x == 0) {
        volatile unsigned int *vc = ctr;
        volatile int *verr = err;
        const unsigned long long t0 = globaltimer_ns();
        unsigned int spins = 0;
        while (*vc < target) {
            if (*verr) {
                ok = 0;
                break;
            }
            if ((++spins & 1023u) == 0u &&
                (globaltimer_ns() - t0 > kBarrierTimeoutNs || spins > (1u << 30))) {
                atomicExch(err, 1);
                ok = 0;
                break;
            }
        }
        __threadfence();
    }
    return __syncthreads_and(ok) != 0;
}

template <class S, int NT>
__global__ void __launch_bounds__(NT, kResThreads / NT) resident_run_kernel(const StepArgs a, int n) {
    using R = float;
    extern __shared__ __align__(16) float dsm[];
    const int TH = a.march_h;
    const int PL = (TH + 6) * kEW;  // one population plane of the region
    float *F = dsm;                 // [9][TH + 6][kEW]
    float *Hs = F + 9 * PL;         // [TH + 4][kHW]
    float *Ps = Hs + (TH + 4) * kHW;
    float *JX = Ps + (TH + 2) * kPW;  // [TH][kResTW]
    float *JY = JX + TH * kResTW;
    float *LO = JY + TH * kResTW;
    PartQ *red = reinterpret_cast<PartQ *>(LO + TH * kResTW);  // 8-byte aligned: every size above is even
    RedPart *redd = reinterpret_cast<RedPart *>(red + NT / 32);

    const int t = threadIdx.x;
    const int G = gridDim.x, b = blockIdx.x;
    const int Lx = a.Lx, Ly = a.Ly;
    const int pitch = (int)a.pitch;  // 9 * pitch < 2^31 (checked at creation)
    const int X0 = (b % a.tiles_x) * kResTW, Y0 = (b / a.tiles_x) * TH;
    const int tw = min(kResTW, Lx - X0), th = min(TH, Ly - Y0);  // this tile
    const int ew = tw + 6, eh = th + 6;
    const long long base = __ldcg(&a.ctl->step_base);
    const bool red_on = needs_partials(a);
    const bool measure = a.meas_mask || a.mass_corr;
    const R gamma = R(a.gamma), hmin = R(a.hmin), hcrit = R(a.hcrit), kap = R(a.kap);
    const R thr = R(a.hthresh);

    // Populations of the region from the buffer iteration done + 1 pulls
    // from (L2 loads: other CTAs wrote them in this launch); ring_only:
    // the 3-cell ring around the tile.  Index maps use the compile-time row
    // widths (kEW), so they cost a multiply-shift, not a division.
    auto load_cell = [&](const void *src, int lx, int ly) {
        const int c = wrapc(Y0 - 3 + ly, Ly) * Lx + wrapc(X0 - 3 + lx, Lx);
        float *fp = F + ly * kEW + lx;
#pragma unroll
        for (int q = 0; q < 9; ++q) fp[q * PL] = S::ld(src, pitch, q, c);
    };
    auto load = [&](long long done, bool ring_only) {
        const void *src = (done & 1) ? a.fb : a.fa;
        if (!ring_only) {
            for (int i = t; i < kEW * eh; i += NT) {
                const int lx = i % kEW, ly = i / kEW;
                if (lx < ew) load_cell(src, lx, ly);
            }
            return;
        }
        // 3 rows above and below the tile (all columns), then 3 columns
        // left and right of it (the tile's rows)
        constexpr int kLd = NT - 32;  // threads 32.. (warp 0 may be reducing)
        for (int i = t - 32; i < 6 * kEW; i += kLd) {
            const int lx = i % kEW, r = i / kEW;
            if (lx < ew) load_cell(src, lx, r < 3 ? r : th + r);
        }
        for (int i = t - 32; i < 6 * th; i += kLd) {
            const int k6 = i % 6, ly = 3 + i / 6;
            load_cell(src, k6 < 3 ? k6 : tw + k6, ly);
        }
    };

    load(base, false);
    for (int k = 0; k < n; ++k) {
        const long long done = base + k, tt = done + 1;
        if (k > 0) {
            // the previous iteration's measures (warp 0 of the last CTA),
            // while warps 1.. load the ring
            if (t < 32) {
                if (red_on && b == G - 1) reduce_step<NT>(a, done, redd);
            } else {
                load(done, true);
            }
        }
        __syncthreads();
        // A. pull and moments on the tile and 2 rings
        {
            const int w2 = tw + 4;
            for (int i = t; i < kHW * (th + 4); i += NT) {
                const int hx = i % kHW, hy = i / kHW;
                if (hx >= w2) continue;
                const float *c = F + (hy + 1) * kEW + (hx + 1);
                R f[9];  // f_q(x) = fpost_q(x - c_q)
                f[0] = c[0];
                f[1] = c[PL - 1];
                f[2] = c[2 * PL - kEW];
                f[3] = c[3 * PL + 1];
                f[4] = c[4 * PL + kEW];
                f[5] = c[5 * PL - kEW - 1];
                f[6] = c[6 * PL - kEW + 1];
                f[7] = c[7 * PL + kEW + 1];
                f[8] = c[8 * PL + kEW - 1];
                R h, jx, jy;
                moments9<false>(f, h, jx, jy);
                Hs[hy * kHW + hx] = h;
                const int ox = hx - 2, oy = hy - 2;
                if (ox >= 0 && ox < tw && oy >= 0 && oy < th) {
                    const int o = oy * kResTW + ox;
                    JX[o] = jx;
                    JY[o] = jy;
                    LO[o] = moments_lo(f, h);
                }
            }
        }
        __syncthreads();
        // B. film pressure on the tile and 1 ring
        {
            const int w1 = tw + 2;
            for (int i = t; i < kPW * (th + 2); i += NT) {
                const int px = i % kPW, py = i / kPW;
                if (px >= w1) continue;
                const float *hc = Hs + (py + 1) * kHW + (px + 1), *hm = hc - kHW, *hp = hc + kHW;
                // ip = h[i-1,j], jp = h[i,j-1], im = h[i+1,j], jm = h[i,j+1], ...
                Ps[py * kPW + px] = pressure_cell<false, R>(hc[0], hc[-1], hm[0], hc[1], hp[0],
                                                            hm[-1], hm[1], hp[1], hp[-1], kap,
                                                            gamma, hmin, hcrit, a.n, a.m);
            }
        }
        __syncthreads();
        // C. forces, collision, stores and measures of the tile
        const CellConst<R> cc =
            cell_consts<R>(a, tt, a.mass_corr ? __ldcg(&a.ctl->corr[tt & 1]) : 0.0);
        void *dst = (done & 1) ? a.fa : a.fb;
        PartQ part;
        part_init(part);
        int any_nan = 0;
        for (int i = t; i < kResTW * th; i += NT) {
            const int ox = i % kResTW, oy = i / kResTW;
            if (ox >= tw) continue;
            const int cell = (Y0 + oy) * Lx + X0 + ox;
            const int o = oy * kResTW + ox;
            const float *hc = Hs + (oy + 2) * kHW + ox + 2;
            const R h = hc[0];
            R ux, uy, gpx, gpy;
            velocity<false>(h, JX[o], JY[o], ux, uy);
            const float *pc = Ps + (oy + 1) * kPW + ox + 1, *pm = pc - kPW, *pp = pc + kPW;
            grad9<R>(pc[-1], pm[0], pc[1], pp[0], pm[-1], pm[1], pp[1], pp[-1], gpx, gpy);  // h∇p!
            const float2 Fv = force_fast(cc, h, ux, uy, gpx, gpy);
            float fo[9];
            [[maybe_unused]] __half2 hb[4];
            collide_fast<S, false, true>(cc, h, ux, uy, Fv.x, Fv.y, h, nullptr, cell, tt, &LO[o], fo,
                                         hb);
            float *fc = F + (oy + 3) * kEW + ox + 3;
#pragma unroll
            for (int q = 0; q < 9; ++q) fc[q * PL] = fo[q];
            if constexpr (S::kHalf) {
                reinterpret_cast<float *>(dst)[cell] = fo[0];
                __half *hpl = const_cast<__half *>(S::hp(dst, pitch)) + cell;
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    hpl[(2 * kk) * pitch] = __low2half(hb[kk]);
                    hpl[(2 * kk + 1) * pitch] = __high2half(hb[kk]);
                }
            } else {
#pragma unroll
                for (int q = 0; q < 9; ++q) S::st(dst, pitch, q, cell, fo[q]);
            }
            if (!isfinite(h)) any_nan = 1;
            if (measure) {
                mass_add(part, h);
                mass_add_lo(part, LO[o]);
                const bool wet = h > thr;
                part.wet += wet ? 1 : 0;
                part.hmax = fmaxf(part.hmax, h);
                part.hmin = fminf(part.hmin, h);
                if ((a.meas_mask & SWB_MEAS_AREA) && wet) {
                    const float *hm = hc - kHW, *hp = hc + kHW;
                    R gx2, gy2;
                    grad9<R>(hc[-1], hm[0], hc[1], hp[0], hm[-1], hm[1], hp[1], hp[-1], gx2, gy2);
                    area_add(part, R(sqrt(gx2 * gx2 + gy2 * gy2 + R(1))));
                }
            }
        }
        // The CTA's measures and its arrival with one CTA barrier: each warp
        // reduces its partials into red[warp]; the barrier (which also ORs
        // the NaN flags) orders every thread's stores of this iteration
        // before thread 0's fence; warp 0 reduces red, thread 0 adds the
        // result to the accumulators, fences and arrives.  red is written
        // again only after the next iteration's phase barriers.
        if (measure) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) part_merge(part, part_shfl(part, off));
            if ((t & 31) == 0) red[t >> 5] = part;
        }
        any_nan = __syncthreads_or(any_nan);
        if (t < 32) {
            if (measure) {
                PartQ q;
                part_init(q);
                if (t < NT / 32) q = red[t];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) part_merge(q, part_shfl(q, off));
                if (t == 0) add_partials(a, q, tt, b);
            }
            if (t == 0) {
                if (any_nan) a.ctl->nan_flag = 1;
                __threadfence();
                atomicAdd(a.bar, 1u);
            }
        }
        // after the last iteration only the last CTA waits (to reduce it)
        if ((k + 1 < n || b == G - 1) &&
            !res_wait(a.bar, &a.ctl->bar_err, (unsigned int)(k + 1) * (unsigned int)G))
            return;
    }
    if (b == G - 1) {
        if (red_on && n > 0) reduce_step<NT>(a, base + n, redd);
        __syncthreads();
        if (t == 0) {
            a.ctl->step_base = base + n;
            atomicExch(a.bar, 0u);  // every CTA has arrived for the last time
        }
    }
}

// Allow the kernel the dynamic shared memory of a tile (a host-side
// attribute of the current device's context; set before every query or
// launch, which is cheap and keeps it right on every device).
template <class S, int NT>
cudaError_t prepare(size_t bytes) {
    return cudaFuncSetAttribute(resident_run_kernel<S, NT>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Runs f(store tag, threads) for a precision and resident geometry.
template <class F>
cudaError_t res_dispatch(int precision, int nt, F &&f) {
    const bool half = precision == SWB_F16;
    if (nt == kResGeom2)
        return half ? f(StoreF16T<LdCG>{}, std::integral_constant<int, kResThreads / 2>{})
                    : f(StoreF32T<LdCG>{}, std::integral_constant<int, kResThreads / 2>{});
    return half ? f(StoreF16T<LdCG>{}, std::integral_constant<int, kResThreads>{})
                : f(StoreF32T<LdCG>{}, std::integral_constant<int, kResThreads>{});
}

}  // namespace

size_t resident_smem_bytes(int h, int nt) {
    const size_t threads = nt == kResGeom2 ? kResThreads / 2 : kResThreads;
    return res_floats(h) * sizeof(float) + (threads / 32) * (sizeof(PartQ) + sizeof(RedPart));
}

int resident_blocks_per_sm(int precision, int h, int nt) {
    if ((precision != SWB_F32 && precision != SWB_F16) || h < 1 || h > kResMaxTH) return 0;
    const size_t bytes = resident_smem_bytes(h, nt);
    int n = 0;
    cudaError_t e = res_dispatch(precision, nt, [&](auto store, auto threads) {
        using S = decltype(store);
        constexpr int NT = decltype(threads)::value;
        cudaError_t r = prepare<S, NT>(bytes);
        if (r == cudaSuccess)
            r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, resident_run_kernel<S, NT>, NT, bytes);
        return r;
    });
    return e == cudaSuccess ? n : 0;
}

cudaError_t launch_resident_run(int precision, const StepArgs &a, int n, cudaStream_t st) {
    if ((precision != SWB_F32 && precision != SWB_F16) || !resident_geometry(a.march_nt) || !a.bar ||
        a.march_h < 1 || a.march_h > kResMaxTH)
        return cudaErrorInvalidValue;
    const size_t bytes = resident_smem_bytes(a.march_h, a.march_nt);
    StepArgs args = a;
    int steps = n;
    void *params[] = {&args, &steps};
    const dim3 grid((unsigned)(a.tiles_x * a.tiles_y));
    return res_dispatch(precision, a.march_nt, [&](auto store, auto threads) {
        using S = decltype(store);
        constexpr int NT = decltype(threads)::value;
        cudaError_t r = prepare<S, NT>(bytes);
        if (r == cudaSuccess)
            r = cudaLaunchCooperativeKernel((const void *)resident_run_kernel<S, NT>, grid, dim3(NT),
                                            params, bytes, st);
        return r;
    });
}

}  // namespace swb
