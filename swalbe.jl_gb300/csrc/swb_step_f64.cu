// swb_step_f64.cu -- Float64 kernels.  Compiled with --fmad=false so that no
// a*b+c is contracted into an FMA: the reference (Julia broadcasts) rounds
// every operation, and this translation unit reproduces it bit for bit.
//
// Contents: the fused step in Float64 (literal arithmetic), the plain
// one-kernel-per-reference-op path, and the standalone measure reduction.
#include "swb_step_impl.cuh"

namespace swb {

// ------------------------------------------------------------ fused, Float64
#define DISPATCH_NT(nt, ...)                       \
    do {                                           \
        if ((nt) == 64) {                          \
            constexpr int NT = 64;                 \
            __VA_ARGS__;                           \
        } else if ((nt) == 256) {                  \
            constexpr int NT = 256;                \
            __VA_ARGS__;                           \
        } else {                                   \
            constexpr int NT = 128;                \
            __VA_ARGS__;                           \
        }                                          \
    } while (0)

cudaError_t launch_fused_step_f64(const StepArgs &a, int k, cudaStream_t st) {
    const int grid = step_grid(a, k);
    cudaError_t e = cudaSuccess;
    if (step_general(a))
        DISPATCH_NT(a.march_nt, e = launch_step(fused_step_kernel<StoreF64, NT, true>, grid, NT, st, a, k));
    else
        DISPATCH_NT(a.march_nt, e = launch_step(fused_step_kernel<StoreF64, NT, false>, grid, NT, st, a, k));
    return e;
}

cudaError_t launch_advance(const StepArgs &a, int n, cudaStream_t st) {
    count_launches(1);
    return launch_step(advance_kernel<128>, 1, 128, st, a, n);
}

cudaError_t launch_batch_advance(const StepArgs *d_args, int count, int n, cudaStream_t st) {
    count_launches(1);
    return launch_step(batch_advance_kernel<128>, count, 128, st, d_args, n);
}

static int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b > 152LL * 32) b = 152LL * 32;
    return (int)(b < 1 ? 1 : b);
}

cudaError_t launch_moments_f64(const StepArgs &a, cudaStream_t st) {
    moments_kernel<StoreF64><<<grid_for((long long)a.Lx * a.Ly, 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_fout_f64(const StepArgs &a, double *out, cudaStream_t st) {
    fout_kernel<StoreF64><<<grid_for((long long)a.Lx * a.Ly, 256), 256, 0, st>>>(a, out);
    return cudaGetLastError();
}

cudaError_t launch_thermal_field_f64(const StepArgs &a, long long t, double *fx, double *fy,
                                     cudaStream_t st) {
    thermal_field_kernel<StoreF64><<<grid_for((long long)a.Lx * a.Ly, 256), 256, 0, st>>>(a, t, fx, fy);
    return cudaGetLastError();
}

cudaError_t launch_pressure_now_f64(const StepArgs &a, double *out, cudaStream_t st) {
    pressure_now_kernel<StoreF64><<<grid_for((long long)a.Lx * a.Ly, 256), 256, 0, st>>>(a, out);
    return cudaGetLastError();
}

cudaError_t launch_batch_step_f64(int nt, bool gen, const StepArgs *d_args, const TileRef *d_tiles,
                                  int ntiles, int grid, int k, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    if (gen)
        DISPATCH_NT(nt, e = launch_step(batch_step_kernel<StoreF64, NT, true>, grid, NT, st, d_args, d_tiles, ntiles, k));
    else
        DISPATCH_NT(nt, e = launch_step(batch_step_kernel<StoreF64, NT, false>, grid, NT, st, d_args, d_tiles, ntiles, k));
    return e;
}

int batch_blocks_per_sm_f64(int nt) {
    int n = 0;
    DISPATCH_NT(nt, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_step_kernel<StoreF64, NT, false>, NT, 0));
    return n < 1 ? 1 : n;
}

// ------------------------------------------------------------ plain path
// One kernel per reference function, Float64, same per-element operations.
// Neighbour (i±1, j±1) indexing replaces the reference's circshift! copies.
#define PLAIN_LOOP(s)                                                              \
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < (s).N; \
         c += (long long)gridDim.x * blockDim.x)

struct Nb {
    long long c, ip, im, jp, jm, ipjp, imjp, imjm, ipjm;  // reference names
};
__device__ __forceinline__ Nb neighbours(long long c, int Lx, int Ly) {
    const int i = (int)(c % Lx), j = (int)(c / Lx);
    const int im1 = i == 0 ? Lx - 1 : i - 1, ip1 = i == Lx - 1 ? 0 : i + 1;
    const int jm1 = j == 0 ? Ly - 1 : j - 1, jp1 = j == Ly - 1 ? 0 : j + 1;
    Nb n;
    n.c = c;
    n.ip = (long long)j * Lx + im1;      // h[i-1, j]
    n.im = (long long)j * Lx + ip1;      // h[i+1, j]
    n.jp = (long long)jm1 * Lx + i;      // h[i, j-1]
    n.jm = (long long)jp1 * Lx + i;      // h[i, j+1]
    n.ipjp = (long long)jm1 * Lx + im1;  // h[i-1, j-1]
    n.imjp = (long long)jm1 * Lx + ip1;  // h[i+1, j-1]
    n.imjm = (long long)jp1 * Lx + ip1;  // h[i+1, j+1]
    n.ipjm = (long long)jp1 * Lx + im1;  // h[i-1, j+1]
    return n;
}

// (sx, sy): offset of a moving θ field (0 for a fixed one)
__global__ void k_filmpressure(PlainState s, const double *kapF, double kap, double gamma, int n,
                               int m, double hmin, double hcrit, int sx, int sy) {
    PLAIN_LOOP(s) {
        const Nb b = neighbours(c, s.Lx, s.Ly);
        const double *h = s.h;
        double k = kap;
        if (kapF) {
            int i = (int)(c % s.Lx) - sx, j = (int)(c / s.Lx) - sy;
            if (i < 0) i += s.Lx;
            if (j < 0) j += s.Ly;
            k = kapF[(long long)j * s.Lx + i];
        }
        s.p[c] = pressure_cell<true, double>(h[c], h[b.ip], h[b.jp], h[b.im], h[b.jm], h[b.ipjp],
                                             h[b.imjp], h[b.imjm], h[b.ipjm], k, gamma, hmin,
                                             hcrit, n, m);
    }
}

__global__ void k_hgradp(PlainState s) {
    PLAIN_LOOP(s) {
        const Nb b = neighbours(c, s.Lx, s.Ly);
        const double *p = s.p;
        double gx, gy;
        grad9<double>(p[b.ip], p[b.jp], p[b.im], p[b.jm], p[b.ipjp], p[b.imjp], p[b.imjm],
                      p[b.ipjm], gx, gy);
        s.hgx[c] = s.h[c] * gx;
        s.hgy[c] = s.h[c] * gy;
    }
}

__global__ void k_slippage(PlainState s, double delta6, double delta3sq, double mu6) {
    PLAIN_LOOP(s) {
        const double h = s.h[c];
        s.sx[c] = (mu6 * h * s.ux[c]) / (2.0 * (h * h) + delta6 * h + delta3sq);
        s.sy[c] = (mu6 * h * s.uy[c]) / (2.0 * (h * h) + delta6 * h + delta3sq);
    }
}

__global__ void k_force_sum(PlainState s) {
    PLAIN_LOOP(s) {
        s.Fx[c] = -s.hgx[c] - s.sx[c];
        s.Fy[c] = -s.hgy[c] - s.sy[c];
    }
}

// Fx .-= kbtx, Fy .-= kbty with thermal!'s forces of iteration t
// (src/forcing.jl:297-311; the force sum of scripts/Rivulet_stability.jl:123).
__global__ void k_thermal(PlainState s, double k6, double delta, unsigned long long seed,
                          long long t) {
    PLAIN_LOOP(s) {
        double kx, ky;
        thermal_force<true, double>(seed, c, t, k6, s.h[c], delta, &kx, &ky);
        s.Fx[c] = s.Fx[c] - kx;
        s.Fy[c] = s.Fy[c] - ky;
    }
}

__global__ void k_inclination(PlainState s, double ax, double ay, double fac) {
    PLAIN_LOOP(s) {
        s.Fx[c] = s.Fx[c] + (s.h[c] * ax) * fac;
        s.Fy[c] = s.Fy[c] + (s.h[c] * ay) * fac;
    }
}

__global__ void k_equilibrium(PlainState s, double g) {
    PLAIN_LOOP(s) {
        double fe[9];
        const double ux = s.ux[c], uy = s.uy[c];
        feq_literal<double>(s.h[c], ux, uy, g, fe);
        s.vsq[c] = ux * ux + uy * uy;
        for (int q = 0; q < 9; ++q) s.feq[q * s.N + c] = fe[q];
    }
}

__global__ void k_collide(PlainState s, double omeg, double invtau) {
    PLAIN_LOOP(s) {
        const double Fx = s.Fx[c], Fy = s.Fy[c];
        for (int q = 0; q < 9; ++q) {
            double v = omeg * s.ftemp[q * s.N + c] + invtau * s.feq[q * s.N + c];
            if (q > 0) v = v + source<double>(q, Fx, Fy);
            s.fout[q * s.N + c] = v;
        }
    }
}

__global__ void k_stream(PlainState s) {  // circshift!(ft_q, fo_q, c_q)
    const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
    const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    PLAIN_LOOP(s) {
        const int i = (int)(c % s.Lx), j = (int)(c / s.Lx);
        for (int q = 0; q < 9; ++q) {
            const int si = wrapc(i - CX[q], s.Lx), sj = wrapc(j - CY[q], s.Ly);
            s.ftemp[q * s.N + c] = s.fout[q * s.N + (long long)sj * s.Lx + si];
        }
    }
}

__global__ void k_moments(PlainState s) {
    PLAIN_LOOP(s) {
        double f[9], h, jx, jy, ux, uy;
        for (int q = 0; q < 9; ++q) f[q] = s.fout[q * s.N + c];
        moments9<true>(f, h, jx, jy);
        velocity<true>(h, jx, jy, ux, uy);
        s.h[c] = h;
        s.ux[c] = ux;
        s.uy[c] = uy;
    }
}

#define PLAIN_LAUNCH(kernel, s, st, ...)                                  \
    do {                                                                  \
        count_launches(1);                                                \
        kernel<<<grid_for((s).N, 256), 256, 0, st>>>(s, ##__VA_ARGS__);   \
        return cudaGetLastError();                                        \
    } while (0)

cudaError_t plain_filmpressure(const PlainState &s, const double *kapF, double kap, double gamma,
                               int n, int m, double hmin, double hcrit, int sx, int sy,
                               cudaStream_t st) {
    PLAIN_LAUNCH(k_filmpressure, s, st, kapF, kap, gamma, n, m, hmin, hcrit, sx, sy);
}
cudaError_t plain_hgradp(const PlainState &s, cudaStream_t st) { PLAIN_LAUNCH(k_hgradp, s, st); }
cudaError_t plain_slippage(const PlainState &s, double delta, double mu, cudaStream_t st) {
    PLAIN_LAUNCH(k_slippage, s, st, 6.0 * delta, 3.0 * (delta * delta), 6.0 * mu);
}
cudaError_t plain_force_sum(const PlainState &s, cudaStream_t st) {
    PLAIN_LAUNCH(k_force_sum, s, st);
}
cudaError_t plain_thermal(const PlainState &s, double k6, double delta, unsigned long long seed,
                          long long t, cudaStream_t st) {
    PLAIN_LAUNCH(k_thermal, s, st, k6, delta, seed, t);
}
cudaError_t plain_inclination(const PlainState &s, double ax, double ay, double fac,
                              cudaStream_t st) {
    PLAIN_LAUNCH(k_inclination, s, st, ax, ay, fac);
}
cudaError_t plain_equilibrium(const PlainState &s, double g, cudaStream_t st) {
    PLAIN_LAUNCH(k_equilibrium, s, st, g);
}
cudaError_t plain_collide(const PlainState &s, double omeg, double invtau, cudaStream_t st) {
    PLAIN_LAUNCH(k_collide, s, st, omeg, invtau);
}
cudaError_t plain_stream(const PlainState &s, cudaStream_t st) {
    count_launches(1);
    k_stream<<<grid_for(s.N, 256), 256, 0, st>>>(s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // fout .= ftemp (src/collide.jl:103)
    return cudaMemcpyAsync(s.fout, s.ftemp, 9 * s.N * sizeof(double), cudaMemcpyDeviceToDevice,
                           st);
}
cudaError_t plain_moments(const PlainState &s, cudaStream_t st) { PLAIN_LAUNCH(k_moments, s, st); }

// ------------------------------------------------------------ measures
// Grid-stride partials per block, then the last block (ticket) reduces the
// partials in a fixed order and writes one Record.  Per-cell values are
// computed in the height's type R (as the fused step computes them); the
// block sums are Float64 for every R.  cos θ of a wetted cell comes from the
// θ source `cs`: a scalar, a (possibly moving) field, or the θ wave, with the
// fused step's formulas for its iteration cs.t.
template <class R>
__device__ __forceinline__ R cos_of_cell(const CosSrc &cs, long long c, int Lx, int Ly) {
    const int i = (int)(c % Lx), j = (int)(c / Lx);
    if (cs.mode == THETA_FIELD) {
        const int fi = cs.sx ? (i - cs.sx < 0 ? i - cs.sx + Lx : i - cs.sx) : i;
        const int fj = cs.sy ? (j - cs.sy < 0 ? j - cs.sy + Ly : j - cs.sy) : j;
        return reinterpret_cast<const R *>(cs.cosF)[(long long)fj * Lx + fi];
    }
    return wave_kap_cos<R>(R(cs.theta0), R(cs.dtheta), R(cs.wave_v), i, cs.t, Lx, 2, 1, R(1)).cs;
}

template <class R>
__global__ void __launch_bounds__(256) measure_kernel(const R *h, int Lx, int Ly, R thr,
                                                      const CosSrc cs, double *scratch,
                                                      unsigned int *ticket, Record *rec,
                                                      long long t) {
    __shared__ PartT<double> red[8];
    __shared__ int last;
    const long long N = (long long)Lx * Ly;
    const bool percell = cs.mode != THETA_SCALAR;
    PartT<double> p;
    part_init(p);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x) {
        const R v = h[c];
        mass_add(p, (double)v);
        const bool wet = v > thr;
        p.wet += wet ? 1 : 0;
        p.hmax = fmax(p.hmax, (double)v);
        p.hmin = fmin(p.hmin, (double)v);
        if (wet) {
            const Nb b = neighbours(c, Lx, Ly);
            R gx, gy;
            grad9<R>(h[b.ip], h[b.jp], h[b.im], h[b.jm], h[b.ipjp], h[b.imjp], h[b.imjm],
                     h[b.ipjm], gx, gy);
            p.area += (double)R(sqrt(gx * gx + gy * gy + R(1)));
            if (percell) p.cossum += (double)cos_of_cell<R>(cs, c, Lx, Ly);
        }
    }
    PartT<double> tot = block_reduce<256>(p, red);
    if (threadIdx.x == 0) {
        double *pp = scratch + (size_t)blockIdx.x * kNPart;
        pp[0] = tot.mhi + tot.mlo;
        pp[1] = (double)tot.wet;
        pp[2] = tot.hmax;
        pp[3] = tot.hmin;
        pp[4] = tot.area;
        pp[5] = tot.cossum;
        __threadfence();
        last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    PartT<double> acc;
    part_init(acc);
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        const double *pp = scratch + (size_t)b * kNPart;
        PartT<double> q;
        q.mhi = __ldcg(pp + 0);
        q.mlo = 0.0;
        q.wet = (int)__ldcg(pp + 1);
        q.hmax = __ldcg(pp + 2);
        q.hmin = __ldcg(pp + 3);
        q.area = __ldcg(pp + 4);
        q.cossum = __ldcg(pp + 5);
        part_merge(acc, q);
    }
    acc = block_reduce<256>(acc, red);
    if (threadIdx.x == 0) {
        rec->t = t;
        rec->mass = acc.mhi + acc.mlo;
        rec->wetted = (double)acc.wet;
        rec->hmax = acc.hmax;
        rec->hmin = acc.hmin;
        rec->area = acc.area;
        rec->cos_sum = percell ? acc.cossum : (double)acc.wet * cs.cos_theta;
        *ticket = 0u;
    }
}

int measure_blocks(long long N) {
    long long b = (N + 255) / 256;
    if (b > 1024) b = 1024;
    return (int)(b < 1 ? 1 : b);
}

cudaError_t launch_measure(const void *h, int is_double, int Lx, int Ly, double hthresh,
                           const CosSrc &cs, double *scratch, unsigned int *ticket, Record *rec,
                           long long t, cudaStream_t st) {
    const int blocks = measure_blocks((long long)Lx * Ly);
    count_launches(1);
    if (is_double)
        measure_kernel<double><<<blocks, 256, 0, st>>>((const double *)h, Lx, Ly, hthresh, cs,
                                                       scratch, ticket, rec, t);
    else
        measure_kernel<float><<<blocks, 256, 0, st>>>((const float *)h, Lx, Ly, (float)hthresh,
                                                      cs, scratch, ticket, rec, t);
    return cudaGetLastError();
}

cudaError_t launch_measure(const void *h, int is_double, int Lx, int Ly, double hthresh,
                           const void *cosF, double cos_theta, double *scratch, unsigned int *ticket,
                           Record *rec, long long t, cudaStream_t st) {
    CosSrc cs{};
    cs.mode = cosF ? THETA_FIELD : THETA_SCALAR;
    cs.cosF = cosF;
    cs.cos_theta = cos_theta;
    return launch_measure(h, is_double, Lx, Ly, hthresh, cs, scratch, ticket, rec, t, st);
}

}  // namespace swb
