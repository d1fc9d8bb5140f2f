// swb_d1q3.cu -- the one-dimensional thin-film solver (D1Q3), GPU side.
//
// One iteration is the reference's 1D time loop body (src/simulate.jl:98-179):
//   filmpressure!  p = -γ κ (x^n - x^m) - γ (h[i-1] - 2h + h[i+1])   (src/pressure.jl:231-256)
//   h∇p!           h (-1/2) (p[i-1] - p[i+1])                       (src/forcing.jl:189-198)
//   slippage!      6μ h u / (2h^2 + 6δh + 3δ^2)                      (src/forcing.jl:68-71)
//   force          F = -h∇p - slip (- ∇γ with a γ field, src/simulate.jl:548)
//   equilibrium!   D1Q3 feq                                          (src/equilibrium.jl:169-181)
//   BGKandStream!  collision + streaming f1 -> i+1, f2 -> i-1          (src/collide.jl:179-201)
//   moments!       h = f0 + f1 + f2, u = (f1 - f2) / h                (src/moments.jl:54-62)
// in the reference's operation order (this unit is compiled with
// --fmad=false), so Float64 results equal the oracle's bit for bit.
//
// 1D lattices are small, so a CTA owns a whole lattice and runs all the
// iterations of a call in one launch: three phases per iteration (pressure,
// collision with push streaming, moments) separated by __syncthreads; the
// fields and populations stay in L2.  A batch of lattices is one CTA each.
// No CTA waits for another.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "swb_lattice.h"

namespace swb {

struct D1Args {
    int L;
    int n, m;
    double gamma, hmin, hcrit, delta, mu, g, kap, omeg, invtau;
    void *fa, *fb;          // streamed populations (the reference's fout), 3 planes of L
    void *h, *u, *p;        // fields (compute type)
    const void *kapF;       // θ field: κ per cell (or null)
    const void *gamF;       // γ field (or null)
    const void *dgF;        // ∇γ of the γ field (or null)
    Record *rec;            // per-iteration measures (ring of rec_cap, or null)
    int rec_cap;
    long long *step;        // iterations done (device)
    int *nan_flag;
};

namespace {

template <class R>
__device__ __forceinline__ R pow_n(R x, int n) {  // power_broad (src/pressure.jl:363-369)
    R t = R(1);
    for (int i = 0; i < n; ++i) t *= x;
    return t;
}

template <class R>
__device__ __forceinline__ void block_stats(R &mx, R &mn, double &sum, int &wet, R *sh,
                                            double *shd, int *shi) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        wet += __shfl_xor_sync(0xffffffffu, wet, o);
    }
    if (lane == 0) {
        sh[w] = mx;
        sh[32 + w] = mn;
        shd[w] = sum;
        shi[w] = wet;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < nw; ++k) {
            mx = fmax(mx, sh[k]);
            mn = fmin(mn, sh[32 + k]);
            sum += shd[k];
            wet += shi[k];
        }
    }
}

// n iterations of lattice blockIdx.x.  rec_on: record the measures of the
// height at the start of every iteration.
template <class R>
__global__ void __launch_bounds__(256) d1q3_run_kernel(const D1Args *__restrict__ args, int n) {
    __shared__ R sh[64];
    __shared__ double shd[32];
    __shared__ int shi[32];
    __shared__ D1Args a;
    if (threadIdx.x == 0) a = args[blockIdx.x];
    __syncthreads();
    const int L = a.L, NT = blockDim.x;
    R *h = reinterpret_cast<R *>(a.h), *u = reinterpret_cast<R *>(a.u), *p = reinterpret_cast<R *>(a.p);
    const R *kapF = reinterpret_cast<const R *>(a.kapF);
    const R *gamF = reinterpret_cast<const R *>(a.gamF);
    const R *dgF = reinterpret_cast<const R *>(a.dgF);
    const R gamma = R(a.gamma), hmin = R(a.hmin), hcrit = R(a.hcrit), g = R(a.g);
    const R mu6 = R(6) * R(a.mu), delta6 = R(6) * R(a.delta), delta3sq = R(3) * (R(a.delta) * R(a.delta));
    const R omeg = R(a.omeg), invtau = R(a.invtau), kap_s = R(a.kap);
    const long long t0 = *a.step;
    int bad = 0;
    for (int k = 0; k < n; ++k) {
        const long long t = t0 + k + 1;
        const R *fo = reinterpret_cast<const R *>(((t0 + k) & 1) ? a.fb : a.fa);
        R *fn = reinterpret_cast<R *>(((t0 + k) & 1) ? a.fa : a.fb);
        // A. film pressure (and the measures of the current height)
        R mx = R(-INFINITY), mn = R(INFINITY);
        double sum = 0.0;
        int wet = 0;
        for (int i = threadIdx.x; i < L; i += NT) {
            const R hc = h[i], hip = h[i == 0 ? L - 1 : i - 1], him = h[i == L - 1 ? 0 : i + 1];
            const R gi = gamF ? gamF[i] : gamma;
            const R kap = kapF ? kapF[i] : kap_s;
            const R x = hmin / (hc + hcrit);
            R pi = -gi * (kap * (pow_n(x, a.n) - pow_n(x, a.m)));
            pi = pi - gi * ((hip - R(2) * hc) + him);
            p[i] = pi;
            if (a.rec) {
                mx = fmax(mx, hc);
                mn = fmin(mn, hc);
                sum += (double)hc;
                wet += hc > R(0.055) ? 1 : 0;
            }
        }
        if (a.rec) {
            block_stats(mx, mn, sum, wet, sh, shd, shi);
            if (threadIdx.x == 0) {
                Record &r = a.rec[(t - 1) % a.rec_cap];
                r.t = t;
                r.mass = sum;
                r.wetted = (double)wet;
                r.hmax = (double)mx;
                r.hmin = (double)mn;
                r.area = 0.0;
                r.cos_sum = 0.0;
            }
        }
        __syncthreads();
        // B. forces, equilibrium, collision; push streaming into fn
        for (int i = threadIdx.x; i < L; i += NT) {
            const int im = i == 0 ? L - 1 : i - 1, ip = i == L - 1 ? 0 : i + 1;
            const R hc = h[i], uc = u[i];
            const R hgp = (hc * R(-0.5)) * (p[im] - p[ip]);
            const R slip = (mu6 * hc * uc) / ((R(2) * (hc * hc) + delta6 * hc) + delta3sq);
            R F = -hgp - slip;
            if (dgF) F = F - dgF[i];
            const R uu = uc * uc;
            const R fe0 = hc * ((R(1) - (R(0.5) * g) * hc) - uu);
            const R fe1 = hc * (((R(0.25) * g) * hc + R(0.5) * uc) + R(0.5) * uu);
            const R fe2 = hc * (((R(0.25) * g) * hc - R(0.5) * uc) + R(0.5) * uu);
            const R o0 = omeg * fo[i] + invtau * fe0;
            const R o1 = omeg * fo[L + i] + invtau * fe1 + R(0.5) * F;
            const R o2 = omeg * fo[2 * L + i] + invtau * fe2 - R(0.5) * F;
            fn[i] = o0;
            fn[L + ip] = o1;
            fn[2 * L + im] = o2;
        }
        __syncthreads();
        // C. moments
        for (int i = threadIdx.x; i < L; i += NT) {
            const R f0 = fn[i], f1 = fn[L + i], f2 = fn[2 * L + i];
            const R hh = (f0 + f1) + f2;
            h[i] = hh;
            u[i] = (f1 - f2) / hh;
            if (!isfinite(hh)) bad = 1;
        }
        __syncthreads();
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        *a.step = t0 + n;
        if (bad) *a.nan_flag = 1;
    }
}

// ∇γ = -3/2 (γ[i-1] - γ[i+1]) / 2 (src/forcing.jl:423-432), once per γ field.
template <class R>
__global__ void d1q3_gradgamma_kernel(const R *gam, R *dg, int L) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x)
        dg[i] = R(-3.0 / 2.0) * ((gam[i == 0 ? L - 1 : i - 1] - gam[i == L - 1 ? 0 : i + 1]) / R(2.0));
}

}  // namespace
}  // namespace swb

using swb::D1Args;
using swb::Record;

namespace {
thread_local std::string d1_err;
int d1fail(std::string *slot, int code, const std::string &m) {
    if (slot) *slot = m;
    d1_err = m;
    swb::set_global_error(m.c_str());
    return code;
}
}  // namespace

struct swb1d {
    int count = 0, precision = SWB_F64, rb = 8;
    std::vector<swb_params> params;
    std::vector<D1Args> args;
    std::vector<char *> mem;  // one block per lattice
    D1Args *d_args = nullptr;
    long long *d_steps = nullptr;
    int *d_flags = nullptr;
    int rec_cap = 0;
    bool args_dirty = true;
    cudaStream_t stream = nullptr;
    std::string err;
    ~swb1d() {
        if (stream) cudaStreamSynchronize(stream);
        for (char *q : mem) cudaFree(q);
        cudaFree(d_args);
        cudaFree(d_steps);
        cudaFree(d_flags);
        if (stream) cudaStreamDestroy(stream);
    }
};

#define D1_TRY(b, expr)                                                                        \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return d1fail(&(b)->err, e_ == cudaErrorMemoryAllocation ? SWB_ERR_OOM : SWB_ERR_CUDA, \
                          std::string(#expr) + ": " + cudaGetErrorString(e_));                 \
    } while (0)

namespace {
// Bytes of one lattice's block: fa, fb (3L), h, u, p, κ, γ, ∇γ (L each) and
// the measure ring.
size_t d1_bytes(int L, int rb, int rec_cap) {
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    return 2 * al((size_t)3 * L * rb) + 6 * al((size_t)L * rb) + al((size_t)rec_cap * sizeof(Record));
}

int layout(swb1d *b, int i, char *base) {
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const int L = b->params[i].Lx, rb = b->rb;
    D1Args &a = b->args[i];
    size_t o = 0;
    a.fa = base + o; o += al((size_t)3 * L * rb);
    a.fb = base + o; o += al((size_t)3 * L * rb);
    a.h = base + o; o += al((size_t)L * rb);
    a.u = base + o; o += al((size_t)L * rb);
    a.p = base + o; o += al((size_t)L * rb);
    o += 3 * al((size_t)L * rb);  // κ, γ, ∇γ: addressed through field_ptr
    a.rec = b->rec_cap ? reinterpret_cast<Record *>(base + o) : nullptr;
    a.rec_cap = b->rec_cap;
    return SWB_OK;
}

char *field_ptr(swb1d *b, int i, int which) {  // 0 κ, 1 γ, 2 ∇γ (allocated slots)
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const int L = b->params[i].Lx, rb = b->rb;
    return b->mem[i] + 2 * al((size_t)3 * L * rb) + (3 + which) * al((size_t)L * rb);
}

int upload(swb1d *b, void *dst, const double *host, int L) {
    if (b->rb == 8) {
        D1_TRY(b, cudaMemcpyAsync(dst, host, (size_t)L * 8, cudaMemcpyHostToDevice, b->stream));
    } else {
        std::vector<float> tmp(host, host + L);
        D1_TRY(b, cudaMemcpyAsync(dst, tmp.data(), (size_t)L * 4, cudaMemcpyHostToDevice, b->stream));
        D1_TRY(b, cudaStreamSynchronize(b->stream));
    }
    return SWB_OK;
}

int download(swb1d *b, const void *src, double *host, size_t n) {
    if (b->rb == 8) {
        D1_TRY(b, cudaMemcpyAsync(host, src, n * 8, cudaMemcpyDeviceToHost, b->stream));
        D1_TRY(b, cudaStreamSynchronize(b->stream));
    } else {
        std::vector<float> tmp(n);
        D1_TRY(b, cudaMemcpyAsync(tmp.data(), src, n * 4, cudaMemcpyDeviceToHost, b->stream));
        D1_TRY(b, cudaStreamSynchronize(b->stream));
        for (size_t k = 0; k < n; ++k) host[k] = tmp[k];
    }
    return SWB_OK;
}

__global__ void fill1(void *p, int L, int rb, double v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
        if (rb == 8)
            reinterpret_cast<double *>(p)[i] = v;
        else
            reinterpret_cast<float *>(p)[i] = (float)v;
    }
}
}  // namespace

extern "C" {

int swb1d_create(const swb_params *params, int count, int precision, int rec_cap, swb1d **out) {
    if (!out || !params || count < 1 || rec_cap < 0)
        return d1fail(nullptr, SWB_ERR_ARG, "bad arguments");
    *out = nullptr;
    if (precision != SWB_F64 && precision != SWB_F32)
        return d1fail(nullptr, SWB_ERR_ARG, "1D precision must be SWB_F64 or SWB_F32");
    for (int i = 0; i < count; ++i) {
        const swb_params &p = params[i];
        if (p.Lx < 3 || p.Ly != 1 || 3LL * p.Lx >= (1LL << 31) || !(p.tau > 0) || p.n <= p.m ||
            p.m < 1 || !(p.hmin > 0))
            return d1fail(nullptr, SWB_ERR_ARG, "invalid 1D params for lattice " + std::to_string(i) +
                                                    " (L = Lx >= 3, Ly = 1)");
        if (p.kbt != 0.0)
            return d1fail(nullptr, SWB_ERR_UNSUPPORTED, "1D thermal fluctuations are not supported");
    }
    swb1d *b = new swb1d();
    b->count = count;
    b->precision = precision;
    b->rb = precision == SWB_F64 ? 8 : 4;
    b->rec_cap = rec_cap;
    b->params.assign(params, params + count);
    b->args.resize(count);
    auto bad = [&](int code) {
        std::string m = b->err;
        delete b;
        d1_err = m;
        swb::set_global_error(m.c_str());
        return code;
    };
#define C1_TRY(expr)                                                                       \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            b->err = std::string(#expr) + ": " + cudaGetErrorString(e_);                   \
            return bad(e_ == cudaErrorMemoryAllocation ? SWB_ERR_OOM : SWB_ERR_CUDA);      \
        }                                                                                  \
    } while (0)
    C1_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    C1_TRY(cudaMalloc((void **)&b->d_steps, sizeof(long long) * count));
    C1_TRY(cudaMalloc((void **)&b->d_flags, sizeof(int) * count));
    C1_TRY(cudaMemsetAsync(b->d_steps, 0, sizeof(long long) * count, b->stream));
    C1_TRY(cudaMemsetAsync(b->d_flags, 0, sizeof(int) * count, b->stream));
    C1_TRY(cudaMalloc((void **)&b->d_args, sizeof(D1Args) * count));
    for (int i = 0; i < count; ++i) {
        const swb_params &p = params[i];
        char *m = nullptr;
        const size_t bytes = d1_bytes(p.Lx, b->rb, rec_cap);
        C1_TRY(cudaMalloc((void **)&m, bytes));
        b->mem.push_back(m);
        C1_TRY(cudaMemsetAsync(m, 0, bytes, b->stream));  // populations 0 (Sys(), src/initialize.jl:587-599)
        D1Args &a = b->args[i];
        a = D1Args{};
        a.L = p.Lx;
        a.n = p.n;
        a.m = p.m;
        a.gamma = p.gamma;
        a.hmin = p.hmin;
        a.hcrit = p.hcrit;
        a.delta = p.delta;
        a.mu = p.mu;
        a.g = p.g;
        a.kap = swb::host_kappa_shared(p.theta, p.n, p.m, p.hmin);
        a.omeg = 1.0 - 1.0 / p.tau;
        a.invtau = 1.0 / p.tau;
        layout(b, i, m);
        a.step = b->d_steps + i;
        a.nan_flag = b->d_flags + i;
        fill1<<<(p.Lx + 255) / 256, 256, 0, b->stream>>>(a.h, p.Lx, b->rb, 1.0);  // height = 1
        swb::count_launches(1);
        C1_TRY(cudaGetLastError());
    }
    C1_TRY(cudaStreamSynchronize(b->stream));
#undef C1_TRY
    *out = b;
    return SWB_OK;
}

int swb1d_destroy(swb1d *b) {
    delete b;
    return SWB_OK;
}

int swb1d_set_field(swb1d *b, int idx, int field, const double *host) {
    if (!b || idx < 0 || idx >= b->count) return d1fail(b ? &b->err : nullptr, SWB_ERR_ARG, "bad arguments");
    D1Args &a = b->args[idx];
    const int L = a.L;
    switch (field) {
        case SWB_FIELD_HEIGHT:
        case SWB_FIELD_VELX:
            if (!host) return d1fail(&b->err, SWB_ERR_ARG, "NULL field");
            return upload(b, field == SWB_FIELD_HEIGHT ? a.h : a.u, host, L);
        case SWB1D_FIELD_THETA: {
            if (!host) {
                a.kapF = nullptr;
                b->args_dirty = true;
                return SWB_OK;
            }
            std::vector<double> kap(L);
            const swb_params &p = b->params[idx];
            for (int i = 0; i < L; ++i) kap[i] = swb::host_kappa_shared(host[i], p.n, p.m, p.hmin);
            char *dst = field_ptr(b, idx, 0);
            int rc = upload(b, dst, kap.data(), L);
            if (rc) return rc;
            a.kapF = dst;
            b->args_dirty = true;
            return SWB_OK;
        }
        case SWB1D_FIELD_GAMMA: {
            if (!host) {
                a.gamF = a.dgF = nullptr;
                b->args_dirty = true;
                return SWB_OK;
            }
            char *g = field_ptr(b, idx, 1), *dg = field_ptr(b, idx, 2);
            int rc = upload(b, g, host, L);
            if (rc) return rc;
            if (b->rb == 8)
                swb::d1q3_gradgamma_kernel<double><<<(L + 255) / 256, 256, 0, b->stream>>>(
                    (const double *)g, (double *)dg, L);
            else
                swb::d1q3_gradgamma_kernel<float><<<(L + 255) / 256, 256, 0, b->stream>>>(
                    (const float *)g, (float *)dg, L);
            swb::count_launches(1);
            D1_TRY(b, cudaGetLastError());
            a.gamF = g;
            a.dgF = dg;
            b->args_dirty = true;
            return SWB_OK;
        }
        default:
            return d1fail(&b->err, SWB_ERR_ARG, "1D fields: height, vel, theta, gamma");
    }
}

int swb1d_get_field(swb1d *b, int idx, int field, double *host) {
    if (!b || !host || idx < 0 || idx >= b->count)
        return d1fail(b ? &b->err : nullptr, SWB_ERR_ARG, "bad arguments");
    D1Args &a = b->args[idx];
    long long t = 0;
    D1_TRY(b, cudaMemcpyAsync(&t, a.step, sizeof(long long), cudaMemcpyDeviceToHost, b->stream));
    D1_TRY(b, cudaStreamSynchronize(b->stream));
    switch (field) {
        case SWB_FIELD_HEIGHT: return download(b, a.h, host, (size_t)a.L);
        case SWB_FIELD_VELX: return download(b, a.u, host, (size_t)a.L);
        case SWB_FIELD_PRESSURE: return download(b, a.p, host, (size_t)a.L);
        case SWB_FIELD_FOUT: return download(b, (t & 1) ? a.fb : a.fa, host, (size_t)3 * a.L);
        default: return d1fail(&b->err, SWB_ERR_ARG, "1D fields: height, vel, pressure, fout");
    }
}

int swb1d_step(swb1d *b, int64_t nsteps) {
    if (!b || nsteps < 0) return d1fail(b ? &b->err : nullptr, SWB_ERR_ARG, "bad arguments");
    if (b->args_dirty) {
        D1_TRY(b, cudaMemcpyAsync(b->d_args, b->args.data(), sizeof(D1Args) * b->count,
                                  cudaMemcpyHostToDevice, b->stream));
        b->args_dirty = false;
    }
    while (nsteps > 0) {  // launches of at most 4096 iterations
        const int n = (int)(nsteps < 4096 ? nsteps : 4096);
        if (b->rb == 8)
            swb::d1q3_run_kernel<double><<<b->count, 256, 0, b->stream>>>(b->d_args, n);
        else
            swb::d1q3_run_kernel<float><<<b->count, 256, 0, b->stream>>>(b->d_args, n);
        swb::count_launches(1);
        D1_TRY(b, cudaGetLastError());
        nsteps -= n;
    }
    return SWB_OK;
}

int swb1d_sync(swb1d *b) {
    if (!b) return d1fail(nullptr, SWB_ERR_ARG, "NULL");
    D1_TRY(b, cudaStreamSynchronize(b->stream));
    std::vector<int> flags(b->count);
    D1_TRY(b, cudaMemcpy(flags.data(), b->d_flags, sizeof(int) * b->count, cudaMemcpyDeviceToHost));
    for (int i = 0; i < b->count; ++i)
        if (flags[i]) return d1fail(&b->err, SWB_ERR_NAN, "non-finite height in 1D lattice " + std::to_string(i));
    return SWB_OK;
}

int swb1d_get_measures(swb1d *b, int idx, swb_measure *out, int64_t cap, int64_t *count) {
    if (!b || !count || idx < 0 || idx >= b->count || (cap > 0 && !out))
        return d1fail(b ? &b->err : nullptr, SWB_ERR_ARG, "bad arguments");
    *count = 0;
    const D1Args &a = b->args[idx];
    if (!a.rec) return SWB_OK;
    long long t = 0;
    D1_TRY(b, cudaMemcpyAsync(&t, a.step, sizeof(long long), cudaMemcpyDeviceToHost, b->stream));
    D1_TRY(b, cudaStreamSynchronize(b->stream));
    long long n = t < a.rec_cap ? t : a.rec_cap;
    if (n > cap) n = cap;
    std::vector<Record> r((size_t)a.rec_cap);
    D1_TRY(b, cudaMemcpy(r.data(), a.rec, sizeof(Record) * a.rec_cap, cudaMemcpyDeviceToHost));
    for (long long k = 0; k < n; ++k) {  // the newest n iterations, oldest first
        const Record &x = r[(size_t)((t - n + k) % a.rec_cap)];
        out[k].t = x.t;
        out[k].mass = x.mass;
        out[k].wetted = (int64_t)x.wetted;
        out[k].hmax = x.hmax;
        out[k].hmin = x.hmin;
        out[k].area = 0.0;
        out[k].energy = 0.0;
    }
    *count = n;
    return SWB_OK;
}

}  // extern "C"
