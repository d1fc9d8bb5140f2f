// swb_api.cu -- host side of the C ABI (include/swalbe_gb300.h).
//
// A swb_state mirrors one `State` of the reference (src/initialize.jl:149-168):
// it owns the device buffers of one lattice and a CUDA stream.  Time steps
// are launched asynchronously; repeated launches are captured once into a
// CUDA graph and replayed (the step counter lives on the device, so the
// same graph serves every chunk of steps).
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_fp16.h>

#include "swb_internal.h"

using swb::Control;
using swb::PlainState;
using swb::Record;
using swb::StepArgs;
using swb::TileRef;

// ------------------------------------------------------------------ errors
namespace {
thread_local std::string g_err;

int fail(std::string *slot, int code, const std::string &msg) {
    g_err = msg;
    if (slot) *slot = msg;
    return code;
}

#define CUDA_TRY(slot, expr)                                                              \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(slot, e_ == cudaErrorMemoryAllocation ? SWB_ERR_OOM : SWB_ERR_CUDA, \
                        std::string(#expr) + ": " + cudaGetErrorString(e_));              \
    } while (0)

// cos(πx): exact at multiples of 1/2 (like Julia's Base.cospi), otherwise
// the argument is reduced exactly modulo 2 and cos evaluated in long double,
// then rounded once.
double host_cospi(double x) {
    if (!std::isfinite(x)) return NAN;
    double r = std::fmod(std::fabs(x), 2.0);
    if (r == 0.0) return 1.0;
    if (r == 1.0) return -1.0;
    if (r == 0.5 || r == 1.5) return 0.0;
    const long double PI_L = 3.141592653589793238462643383279502884L;
    return (double)cosl(PI_L * (long double)r);
}

// ((1 - cospi θ)(n-1)(m-1)) / ((n-m) hmin), left to right (src/pressure.jl:141-147)
double host_kappa(double theta, int n, int m, double hmin) {
    double a = 1.0 - host_cospi(theta);
    a = a * (double)(n - 1);
    a = a * (double)(m - 1);
    return a / ((double)(n - m) * hmin);
}

double incl_factor(long long t, long long tstart, long long tsmooth) {
    return 0.5 + 0.5 * std::tanh((double)(t - tstart) / (double)tsmooth);
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int real_bytes(int precision) { return precision == SWB_F64 || precision == SWB_PLAIN64 ? 8 : 4; }

// Population buffer bytes for `pitch` cells.
size_t fbuf_bytes(int precision, long long pitch) {
    switch (precision) {
        case SWB_F64: return (size_t)9 * pitch * 8;
        case SWB_F32: return (size_t)9 * pitch * 4;
        case SWB_F16: return (size_t)pitch * 4 + (size_t)8 * pitch * 2;
        default: return 0;
    }
}

long long pitch_of(long long N) { return (N + 63) / 64 * 64; }

int check_params(const swb_params *p, std::string *slot) {
    if (!p) return fail(slot, SWB_ERR_ARG, "params is NULL");
    if (p->Lx < 1 || p->Ly < 1) return fail(slot, SWB_ERR_ARG, "Lx and Ly must be >= 1");
    if (9LL * (((long long)p->Lx * p->Ly + 63) / 64 * 64) >= (1LL << 31))
        return fail(slot, SWB_ERR_ARG, "lattice too large: Lx*Ly*9 must be < 2^31");
    if (!(p->tau > 0.0)) return fail(slot, SWB_ERR_ARG, "tau must be > 0");
    if (p->n <= p->m || p->m < 1) return fail(slot, SWB_ERR_ARG, "need n > m >= 1");
    if (!(p->hmin > 0.0)) return fail(slot, SWB_ERR_ARG, "hmin must be > 0");
    if (!(p->kbt >= 0.0)) return fail(slot, SWB_ERR_ARG, "kbt must be >= 0");
    return SWB_OK;
}

// Static parts of the step arguments from the parameters.
void fill_args_from_params(StepArgs &a, const swb_params &p) {
    a.Lx = p.Lx;
    a.Ly = p.Ly;
    a.gamma = p.gamma;
    a.hmin = p.hmin;
    a.hcrit = p.hcrit;
    a.delta = p.delta;
    a.mu = p.mu;
    a.g = p.g;
    a.invtau = 1.0 / p.tau;
    a.omeg = 1.0 - 1.0 / p.tau;
    a.tau_is_one = (p.tau == 1.0);
    a.n = p.n;
    a.m = p.m;
    a.theta_mode = swb::THETA_SCALAR;
    a.kap = host_kappa(p.theta, p.n, p.m, p.hmin);
    a.cos_theta = host_cospi(p.theta);
    a.hthresh = 0.055;
    a.thermal = p.kbt > 0.0 ? 1 : 0;
    a.k6 = ((2.0 * p.kbt) * p.mu) * 6.0;  // src/forcing.jl:300-302, left to right
}

__global__ void fill_kernel(double *d, long long n, double v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        d[i] = v;
}
__global__ void fill_kernel_f(float *d, long long n, float v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        d[i] = v;
}
// Inverse of the pull fout_q(x) = fpost_q(x - c_q): fpost_q(x - c_q) = fout_q(x).
template <class T>
__global__ void push_kernel(const double *fout, void *fpost, int Lx, int Ly, long long pitch,
                            int precision) {
    const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
    const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    const long long N = (long long)Lx * Ly;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % Lx), j = (int)(c / Lx);
        for (int q = 0; q < 9; ++q) {
            int di = i - CX[q], dj = j - CY[q];
            di = (di % Lx + Lx) % Lx;
            dj = (dj % Ly + Ly) % Ly;
            const double v = fout[q * N + c];
            const long long d = (long long)dj * Lx + di;
            if (precision == SWB_F64) {
                ((double *)fpost)[q * pitch + d] = v;
            } else if (precision == SWB_F32) {
                ((float *)fpost)[q * pitch + d] = (float)v;
            } else {
                if (q == 0)
                    ((float *)fpost)[d] = (float)v;
                else
                    ((__half *)((float *)fpost + pitch))[(q - 1) * pitch + d] =
                        __float2half_rn((float)v * 1024.0f);
            }
        }
    }
}

int blocks_for(long long n) {
    long long b = (n + 255) / 256;
    if (b > 4096) b = 4096;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

// ------------------------------------------------------------------ dispatch
namespace swb {
void set_global_error(const char *msg) { g_err = msg; }
static std::atomic<unsigned long long> g_launches{0};
void count_launches(unsigned long long n) { g_launches += n; }
unsigned long long launches_so_far() { return g_launches.load(); }

bool launch_overlap() {
    static const bool on = [] {
        const char *v = getenv("SWB_LAUNCH_OVERLAP");
        return !(v && v[0] == '0');
    }();
    return on;
}

cudaError_t launch_fused_step(int precision, const StepArgs &a, int k, bool steady, cudaStream_t st) {
    count_launches(1);
    return precision == SWB_F64 ? launch_fused_step_f64(a, k, st)
                                : launch_fused_step_f32(precision, a, k, steady, st);
}
cudaError_t launch_moments(int precision, const StepArgs &a, cudaStream_t st) {
    count_launches(1);
    return precision == SWB_F64 ? launch_moments_f64(a, st) : launch_moments_f32(precision, a, st);
}
cudaError_t launch_fout(int precision, const StepArgs &a, double *out, cudaStream_t st) {
    count_launches(1);
    return precision == SWB_F64 ? launch_fout_f64(a, out, st) : launch_fout_f32(precision, a, out, st);
}
cudaError_t launch_thermal_field(int precision, const StepArgs &a, long long t, double *fx,
                                 double *fy, cudaStream_t st) {
    count_launches(1);
    return precision == SWB_F32 || precision == SWB_F16
               ? launch_thermal_field_f32(precision, a, t, fx, fy, st)
               : launch_thermal_field_f64(a, t, fx, fy, st);
}
cudaError_t launch_pressure_now(int precision, const StepArgs &a, double *out, cudaStream_t st) {
    count_launches(1);
    return precision == SWB_F64 ? launch_pressure_now_f64(a, out, st)
                                : launch_pressure_now_f32(precision, a, out, st);
}
cudaError_t launch_batch_step(int precision, int nt, bool gen, bool steady_tau1,
                              const StepArgs *d_args, const TileRef *d_tiles, int ntiles,
                              int grid, int k, cudaStream_t st, bool rare) {
    count_launches(1);
    return precision == SWB_F64
               ? launch_batch_step_f64(nt, gen, d_args, d_tiles, ntiles, grid, k, st)
               : launch_batch_step_f32(precision, nt, gen, steady_tau1, d_args, d_tiles, ntiles,
                                       grid, k, st, rare);
}
int batch_blocks_per_sm(int precision, int nt, bool wave) {
    return precision == SWB_F64 ? batch_blocks_per_sm_f64(nt) : batch_blocks_per_sm_f32(precision, nt, wave);
}

// Default strip geometry by lattice size (from sweeps on GB300): narrow
// strips (64 threads) and as many rows per strip as still leave ~1000 CTAs
// (FP16: at most 16 rows); FP16 small lattices prefer 128-thread strips.
// E.g. FP32 2048^2: 60x32 strips, 61.9 us per iteration against 64.0 at
// 60x16; 1024^2: 60x16.  (*nt == kTileGeom keeps the 2D tiles.)
int pair_rows(int Lx, int Ly, int precision, int nt) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
        sms = 1;
    const long long slots = (long long)pair_blocks_per_sm(precision, nt) * sms;
    const long long w = -2LL * nt - 4, tx = (Lx + w - 1) / w;
    long long best = -1;
    int bh = 8;
    for (int hh = 8; hh <= kMaxRows; ++hh) {
        const long long ctas = tx * ((Ly + hh - 1) / hh);
        const long long cost = (ctas + slots - 1) / slots * (hh + 4);
        if (best < 0 || cost < best) {
            best = cost;
            bh = hh;
        }
    }
    return bh < Ly ? bh : (Ly < kMinRows ? kMinRows : Ly);
}

void default_geometry(int Lx, int Ly, int precision, int *nt, int *h) {
    int n = *nt;
    if (n == kTileGeom) {
        *h = kTileY;
        return;
    }
    // Lattices whose populations exceed L2 (the HBM-bound ones) in FP32
    // arithmetic: pair strips of 64 threads, rows by the wave rule (FP32
    // 2048²: 124 x 24 strips, 53.5 us per iteration against 59.7 for 60 x 32
    // one-column strips, measured on GB300).
    if ((n == 0 || n < 0) && (precision == SWB_F32 || precision == SWB_F16) && Lx % 2 == 0 &&
        (long long)Lx * Ly >= (1LL << 21)) {
        *nt = n < 0 ? n : -64;
        *h = pair_rows(Lx, Ly, precision, *nt);
        return;
    }
    if (!n) n = (precision == SWB_F16 && (long long)Lx * Ly <= 512LL * 512) ? 128 : 64;
    const long long strips = (Lx + n - 5) / (n - 4);
    const long long want = precision == SWB_F64 ? 600 : 1000;
    int hh = 4;  // 2-row strips only through the tuner (faster at 256², slower at 512²)
    for (int cand : {32, 16, 8}) {
        if (precision == SWB_F16 && cand > 16) continue;
        if (strips * ((Ly + cand - 1) / cand) >= want) {
            hh = cand;
            break;
        }
    }
    if (hh > Ly) hh = Ly < kMinRows ? kMinRows : Ly;
    *nt = n;
    *h = hh;
}
}  // namespace swb

// ------------------------------------------------------------------ state
struct swb_state {
    swb_params p{};
    int precision = 0;
    long long N = 0, pitch = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;  // the state's own stream
    unsigned long long graph_launches = 0;  // kernels in the captured graph
    std::vector<void *> allocs;
    StepArgs a{};
    PlainState ps{};
    double *plain_kapF = nullptr;
    double *plain_cosF = nullptr;  // cospi(θ) of a θ field (the plain path's measures)
    // measures
    Record *rec = nullptr;     // ring of kRecCap
    Record *mrec = nullptr;    // slot for swb_measure_now
    double *mscratch = nullptr;
    unsigned int *mticket = nullptr;
    long long rec_read = 0;    // records consumed by the host
    long long rec_dropped = 0; // records overwritten before the host read them
    long long plain_rec_head = 0;
    int plain_meas_mask = 0;
    // host mirrors
    long long steps = 0;
    bool host_fresh = true;      // next step starts from the fields
    bool fields_current = true;  // fields equal the moments of the populations
    // inclination for the plain path
    int incl = 0, incl_loop_time = 0;
    double ax = 0, ay = 0;
    long long incl_t = 1000, incl_tstart = 0, incl_tsmooth = 1;
    // strip geometry: autotuned on the first long run unless set explicitly
    bool tuned = false;
    bool autotune = true;
    // launch form: SWB_STEP_AUTO (tuner / size rule) or a fixed one; persist
    // is the form in effect (multi-step cooperative kernel vs one launch per
    // iteration replayed from CUDA graphs)
    int mode = SWB_STEP_AUTO;
    bool persist = false;
    // graph cache
    cudaGraphExec_t gexec = nullptr;
    int gsteps = 0;
    bool gvalid = false;
    double *dtmp = nullptr;
    size_t dtmp_bytes = 0;
    // snapshots: device ring of snap_cap heights taken every snap_every iterations
    long long snap_every = 0, snap_cap = 0, snap_count = 0, snap_read = 0;
    double *snap = nullptr;
    std::vector<long long> snap_t;
    std::string err;

    int rb() const { return real_bytes(precision); }
    bool plain() const { return precision == SWB_PLAIN64; }

    cudaError_t alloc(void **ptr, size_t bytes) {
        cudaError_t e = cudaMalloc(ptr, bytes);
        if (e == cudaSuccess) allocs.push_back(*ptr);
        return e;
    }
    void invalidate_graph() {
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
        gvalid = false;
    }
    ~swb_state() {
        invalidate_graph();
        if (stream) cudaStreamSynchronize(stream);
        if (own_stream) cudaStreamSynchronize(own_stream);
        for (void *q : allocs) cudaFree(q);
        if (own_stream) cudaStreamDestroy(own_stream);
    }
};

namespace {

int ensure_tmp(swb_state *s, size_t bytes) {
    if (s->dtmp_bytes >= bytes) return SWB_OK;
    if (s->dtmp) {
        cudaFree(s->dtmp);
        for (auto &q : s->allocs)
            if (q == s->dtmp) q = nullptr;
    }
    s->dtmp = nullptr;
    s->dtmp_bytes = 0;
    CUDA_TRY(&s->err, s->alloc((void **)&s->dtmp, bytes));
    s->dtmp_bytes = bytes;
    return SWB_OK;
}

// Host Float64 column-major -> device field of the compute type.
__global__ void f2d_kernel(const float *src, double *dst, long long n);
__global__ void d2f_kernel(const double *src, float *dst, long long n);

// Host Float64 field -> device field of the compute type.  FP32 states copy
// the doubles into the staging buffer (one DMA; asynchronous from pinned host
// memory) and round them on the device.  Synchronous: the host buffer is only
// read during the call.
int upload_field(swb_state *s, void *dst, const double *host, long long n) {
    if (s->rb() == 8) {
        CUDA_TRY(&s->err, cudaMemcpyAsync(dst, host, n * 8, cudaMemcpyHostToDevice, s->stream));
    } else {
        int rc = ensure_tmp(s, (size_t)n * 8);
        if (rc) return rc;
        CUDA_TRY(&s->err, cudaMemcpyAsync(s->dtmp, host, n * 8, cudaMemcpyHostToDevice, s->stream));
        swb::count_launches(1);
        d2f_kernel<<<blocks_for(n), 256, 0, s->stream>>>(s->dtmp, (float *)dst, n);
        CUDA_TRY(&s->err, cudaGetLastError());
    }
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    return SWB_OK;
}

// Device field -> host Float64 field (widened on the device for FP32 states).
int download_field(swb_state *s, const void *src, double *host, long long n, int bytes) {
    if (bytes == 8) {
        CUDA_TRY(&s->err, cudaMemcpyAsync(host, src, n * 8, cudaMemcpyDeviceToHost, s->stream));
    } else {
        int rc = ensure_tmp(s, (size_t)n * 8);
        if (rc) return rc;
        swb::count_launches(1);
        f2d_kernel<<<blocks_for(n), 256, 0, s->stream>>>((const float *)src, s->dtmp, n);
        CUDA_TRY(&s->err, cudaGetLastError());
        CUDA_TRY(&s->err, cudaMemcpyAsync(host, s->dtmp, n * 8, cudaMemcpyDeviceToHost, s->stream));
    }
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    return SWB_OK;
}

// Fields <- moments of the populations (only needed after steps).
int materialize(swb_state *s) {
    if (s->plain() || s->host_fresh || s->fields_current) return SWB_OK;
    CUDA_TRY(&s->err, swb::launch_moments(s->precision, s->a, s->stream));
    s->fields_current = true;
    return SWB_OK;
}

// The next iteration takes h, u from the fields; the FP16 mass correction
// restarts from the mass of that iteration.
__global__ void set_fresh_kernel(Control *c) {
    c->fresh_step = c->step_base + 1;
    c->corr[0] = 0.0;
    c->corr[1] = 0.0;
}
__global__ void f2d_kernel(const float *src, double *dst, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}
__global__ void d2f_kernel(const double *src, float *dst, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

int set_fresh(swb_state *s) {
    set_fresh_kernel<<<1, 1, 0, s->stream>>>(s->a.ctl);
    swb::count_launches(1);
    CUDA_TRY(&s->err, cudaGetLastError());
    s->host_fresh = true;
    s->fields_current = true;
    return SWB_OK;
}

int check_nan(swb_state *s) {
    if (s->plain()) return SWB_OK;
    Control c{};
    CUDA_TRY(&s->err, cudaMemcpyAsync(&c, s->a.ctl, sizeof(Control), cudaMemcpyDeviceToHost,
                                      s->stream));
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    if (c.bar_err) {
        // a grid-barrier wait gave up: the iterations of that launch are not
        // valid.  Re-arm the barrier so that the state can be re-initialised.
        CUDA_TRY(&s->err, cudaMemsetAsync(s->a.bar, 0, swb::kBarWords * sizeof(unsigned int),
                                          s->stream));
        CUDA_TRY(&s->err, cudaMemsetAsync(&s->a.ctl->bar_err, 0, sizeof(int), s->stream));
        // the measures of the abandoned iterations were never reduced
        CUDA_TRY(&s->err, cudaMemsetAsync(s->a.ctl->acc, 0, sizeof(s->a.ctl->acc), s->stream));
        CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
        return fail(&s->err, SWB_ERR_CUDA, "multi-step kernel: grid barrier wait timed out");
    }
    if (c.nan_flag) return fail(&s->err, SWB_ERR_NAN, "non-finite height detected during a step");
    return SWB_OK;
}

// The θ source of surfacearea!'s energy term for the height that iteration
// t starts from: the scalar θ, the θ field at its offset of iteration t (a
// moving substrate), or the θ wave at t -- what the fused step's own measures
// of iteration t use.
swb::CosSrc cos_source(const swb_state *s, long long t) {
    swb::CosSrc cs{};
    cs.mode = s->a.theta_mode;
    cs.cos_theta = s->a.cos_theta;
    cs.cosF = s->plain() ? (const void *)s->plain_cosF : s->a.cosF;
    if (cs.mode == swb::THETA_FIELD) swb::substrate_shift(s->a, t, &cs.sx, &cs.sy);
    cs.theta0 = s->a.theta0;
    cs.dtheta = s->a.dtheta;
    cs.wave_v = s->a.wave_v;
    cs.t = t;
    return cs;
}

// One plain iteration: the reference's op sequence, one kernel per op.
int plain_iteration(swb_state *s) {
    const long long t = s->steps + 1;
    const swb_params &p = s->p;
    PlainState &ps = s->ps;
    if (s->plain_meas_mask) {
        CUDA_TRY(&s->err, swb::launch_measure(ps.h, 1, p.Lx, p.Ly, s->a.hthresh, cos_source(s, t),
                                              s->mscratch, s->mticket,
                                              s->rec + (t - 1) % swb::kRecCap, t, s->stream));
        s->plain_rec_head++;
    }
    const bool field = s->a.theta_mode == swb::THETA_FIELD;
    int sx = 0, sy = 0;
    swb::substrate_shift(s->a, t, &sx, &sy);
    CUDA_TRY(&s->err, swb::plain_filmpressure(ps, field ? s->plain_kapF : nullptr, s->a.kap,
                                              p.gamma, p.n, p.m, p.hmin, p.hcrit, sx, sy,
                                              s->stream));
    CUDA_TRY(&s->err, swb::plain_hgradp(ps, s->stream));
    CUDA_TRY(&s->err, swb::plain_slippage(ps, p.delta, p.mu, s->stream));
    CUDA_TRY(&s->err, swb::plain_force_sum(ps, s->stream));
    if (s->a.thermal)
        CUDA_TRY(&s->err, swb::plain_thermal(ps, s->a.k6, p.delta, s->a.seed, t, s->stream));
    if (s->incl) {
        const double fac = incl_factor(s->incl_loop_time ? t : s->incl_t, s->incl_tstart,
                                       s->incl_tsmooth);
        CUDA_TRY(&s->err, swb::plain_inclination(ps, s->ax, s->ay, fac, s->stream));
    }
    CUDA_TRY(&s->err, swb::plain_equilibrium(ps, p.g, s->stream));
    CUDA_TRY(&s->err, swb::plain_collide(ps, 1.0 - 1.0 / p.tau, 1.0 / p.tau, s->stream));
    CUDA_TRY(&s->err, swb::plain_stream(ps, s->stream));
    CUDA_TRY(&s->err, swb::plain_moments(ps, s->stream));
    s->steps++;
    return SWB_OK;
}

constexpr int kGraphSteps = 64;

// Geometries chosen by the autotuner, per (Lx, Ly, precision), process-wide.
std::mutex g_tune_mu;
std::vector<std::array<int, 7>> g_tuned;  // Lx, Ly, precision, mode, nt, h, persist

bool tuned_lookup(int Lx, int Ly, int prec, int mode, int *nt, int *h, bool *persist) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    for (auto &e : g_tuned)
        if (e[0] == Lx && e[1] == Ly && e[2] == prec && e[3] == mode) {
            *nt = e[4];
            *h = e[5];
            *persist = e[6] != 0;
            return true;
        }
    return false;
}

// Iterations per launch of the multi-step kernel (keeps launches short).
constexpr int kRunChunk = 1024;

// CTAs of the multi-step kernel for the state's geometry: one per strip plus
// the reducer, capped at what the GPU holds at once (0: not possible).
int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
        sms = 1;
    return sms;
}

// Rows of resident tiles for a lattice: the shortest tiles (the most CTAs)
// whose CTAs are all co-resident; 0 when even kResMaxTH rows do not fit.
int resident_rows(int Lx, int Ly, int precision, int nt = swb::kResGeom) {
    const long long tx = (Lx + swb::kResTW - 1) / swb::kResTW, sms = sm_count();
    for (int h = 1; h <= swb::kResMaxTH; ++h) {
        const long long tiles = tx * ((Ly + h - 1) / h);
        const int per_sm = swb::resident_blocks_per_sm(precision, h, nt);
        if (per_sm > 0 && tiles <= per_sm * sms) return h < Ly ? h : Ly;
    }
    return 0;
}

// CTAs of the multi-step kernel for the state's geometry: one per strip plus
// the reducer, capped at what the GPU holds at once; resident tiles: one per
// tile, all of which must be co-resident (0: not possible).
int run_grid(swb_state *s) {
    const long long tiles = (long long)s->a.tiles_x * s->a.tiles_y;
    if (swb::resident_geometry(s->a.march_nt)) {
        const int per_sm = swb::resident_blocks_per_sm(s->precision, s->a.march_h, s->a.march_nt);
        return (per_sm > 0 && tiles <= (long long)per_sm * sm_count()) ? (int)tiles : 0;
    }
    const int per_sm = swb::fused_run_blocks_per_sm(s->precision, s->a.march_nt);
    if (per_sm <= 0) return 0;
    const long long want = tiles + (swb::needs_partials(s->a) ? 1 : 0);
    const long long cap = (long long)per_sm * sm_count();
    return (int)(want < cap ? want : cap);
}

// Whether the state's iterations can run in its multi-step form now:
// strips / 2D tiles of FP32-arithmetic states, or resident tiles for the
// common steady τ = 1 step.
bool run_possible(const swb_state *s) {
    if (s->precision != SWB_F32 && s->precision != SWB_F16) return false;
    if (swb::resident_geometry(s->a.march_nt))
        return swb::resident_ok(s->a) && run_grid(const_cast<swb_state *>(s)) > 0;
    return s->a.march_nt == 64 || s->a.march_nt == 128 || s->a.march_nt == swb::kTileGeom;
}

// n iterations as multi-step launches of at most kRunChunk iterations.
cudaError_t run_sequence(swb_state *s, long long n) {
    const int grid = run_grid(s);
    if (grid <= 0) return cudaErrorInvalidConfiguration;
    while (n > 0) {
        const int c = (int)(n < kRunChunk ? n : kRunChunk);
        cudaError_t e = swb::resident_geometry(s->a.march_nt)
                            ? swb::launch_resident_run(s->precision, s->a, c, s->stream)
                            : swb::launch_fused_run(s->precision, s->a, c, grid, s->stream);
        if (e != cudaSuccess) return e;
        swb::count_launches(1);
        n -= c;
    }
    return cudaSuccess;
}

// Launch form without the tuner: one launch per iteration unless the
// multi-step kernel was asked for (on GB300 it measured 5-25 % slower than
// graph-replayed launches at 512^2..2048^2; the tuner times both) or the
// geometry is resident tiles (a multi-step form only).
bool persist_default(const swb_state *s) {
    return (s->mode == SWB_STEP_MULTI || swb::resident_geometry(s->a.march_nt)) && run_possible(s);
}

// n step launches (k = 0..n-1) and the advance kernel that closes them.
// Launch 0 is the first iteration after the fields were set when the state
// is fresh; fused_steps runs that one alone, so that every launch of a
// captured sequence is steady and the graph can be replayed at any time.
cudaError_t launch_sequence(swb_state *s, int n) {
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < n && e == cudaSuccess; ++k)
        e = swb::launch_fused_step(s->precision, s->a, k, !(s->host_fresh && k == 0), s->stream);
    if (e == cudaSuccess) e = swb::launch_advance(s->a, n, s->stream);
    return e;
}

// Autotuner: times a few geometries and launch forms on real steps (each
// probe is a complete launch sequence, so nothing is wasted) and keeps the
// fastest.  Every candidate first runs a short untimed sequence, which also
// loads its kernel (modules load lazily, on first launch).  Only for
// SWB_F64 / SWB_F32, whose results do not depend on the geometry.
constexpr int kTuneMinSteps = 512;
constexpr int kTuneProbe = 16;
constexpr int kPersistProbe = 4;

// One candidate's probe: a per-iteration sequence is captured into a graph
// (as it runs outside the tuner), a multi-step one is a single launch.
// Returns the GPU time of the second of two runs (the first loads the
// kernel) in ms, or a negative value on error.
float tune_probe(swb_state *s, cudaEvent_t e0, cudaEvent_t e1) {
    cudaGraphExec_t gx = nullptr;
    unsigned long long nodes = 0;
    if (!s->persist) {
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return -1.f;
        const unsigned long long c0 = swb::launches_so_far();
        cudaError_t le = launch_sequence(s, kTuneProbe);
        nodes = swb::launches_so_far() - c0;
        swb::count_launches(0ULL - nodes);  // captured, not run
        cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
        if (le != cudaSuccess || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return -1.f;
        }
        cudaError_t ie = cudaGraphInstantiate(&gx, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) return -1.f;
    }
    // a multi-step candidate runs kPersistProbe times the iterations in one
    // launch and is scaled back: outside the tuner it runs launches of up to
    // kRunChunk iterations, whose set-up (loading a resident tile's region,
    // the cooperative launch) a 16-iteration launch would overweight
    const int reps = gx ? 1 : kPersistProbe;
    float ms = -1.f;
    for (int rep = 0; rep < 2; ++rep) {
        cudaEventRecord(e0, s->stream);
        cudaError_t e;
        if (gx) {
            e = cudaGraphLaunch(gx, s->stream);
            swb::count_launches(nodes);
        } else {
            e = run_sequence(s, (long long)kTuneProbe * reps);
        }
        cudaEventRecord(e1, s->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            ms = -1.f;
            break;
        }
        s->steps += (long long)kTuneProbe * reps;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)reps;
    }
    if (gx) cudaGraphExecDestroy(gx);
    return ms;
}

int autotune_geometry(swb_state *s, long long &left) {
    int nt = 0, h = 0;
    bool pers = false;
    if (tuned_lookup(s->p.Lx, s->p.Ly, s->precision, s->mode, &nt, &h, &pers)) {
        swb::set_geometry(s->a, nt, h);
        s->persist = pers;
        s->invalidate_graph();
        s->tuned = true;
        return SWB_OK;
    }
    // {nt, h, multi-step}
    const int K = swb::kTileGeom;
    const int all[][3] = {{64, 2, 0},   {64, 4, 0},   {64, 8, 0},   {64, 16, 0},  {64, 32, 0},
                          {128, 4, 0},  {128, 16, 0}, {256, 16, 0}, {K, 16, 0},   {-32, 4, 0},
                          {-32, 8, 0},  {-64, 4, 0},  {-64, 8, 0},  {-64, 16, 0}, {-64, 32, 0},
                          {-128, 16, 0}, {64, 8, 1},  {64, 16, 1},  {128, 8, 1},  {K, 16, 1}};
    std::vector<std::array<int, 3>> cands;
    const bool multi_ok = s->precision == SWB_F32 || s->precision == SWB_F16;
    // pair strips: FP32 arithmetic, even Lx, and only the common steady τ = 1
    // step has that form (others would time the one-column fallback)
    const bool pair_ok = multi_ok && s->p.Lx % 2 == 0 && swb::pair_form_ok(s->a);
    std::vector<std::array<int, 3>> todo;
    for (auto &c : all) todo.push_back({c[0], c[1], c[2]});
    if (pair_ok && s->mode != SWB_STEP_MULTI) {  // and the wave rule's rows
        for (int pn : {-64, -32}) todo.push_back({pn, swb::pair_rows(s->p.Lx, s->p.Ly, s->precision, pn), 0});
    }
    // resident tiles (a multi-step form) where the lattice fits in the CTAs'
    // shared memory: the shortest co-resident tiles
    if (multi_ok && swb::resident_ok(s->a)) {
        for (int rg : {swb::kResGeom, swb::kResGeom2}) {
            const int res_h = resident_rows(s->p.Lx, s->p.Ly, s->precision, rg);
            if (res_h > 0) todo.push_back({rg, res_h, 1});
        }
    }
    for (auto &c : todo) {
        if (c[0] == K && !multi_ok) continue;
        if (c[0] < 0 && !pair_ok) continue;
        // the multi-step form only when asked for: it never won on GB300
        // (sweeps at 512^2..2048^2), and a 16-iteration probe can misjudge it
        if (c[2] && !swb::resident_geometry(c[0]) && (!multi_ok || s->mode != SWB_STEP_MULTI)) continue;
        if (!c[2] && s->mode == SWB_STEP_MULTI) continue;
        cands.push_back({c[0], c[1], c[2]});
    }
    cudaEvent_t e0, e1;
    CUDA_TRY(&s->err, cudaEventCreate(&e0));
    CUDA_TRY(&s->err, cudaEventCreate(&e1));
    float best = 1e30f;
    int bnt = s->a.march_nt, bh = s->a.march_h;
    bool bpers = s->persist;
    int rc = SWB_OK;
    for (auto &c : cands) {
        if (c[1] > s->p.Ly && c[1] != swb::kMinRows) continue;
        if (left < 2 * kTuneProbe) break;
        swb::set_geometry(s->a, c[0], c[1]);
        s->persist = c[2] != 0;
        if (s->persist && run_grid(s) <= 0) continue;
        if (s->persist && left < 2 * kTuneProbe * kPersistProbe) continue;
        const float ms = tune_probe(s, e0, e1);
        if (ms < 0.f) {
            rc = fail(&s->err, SWB_ERR_CUDA, "autotuner probe failed");
            break;
        }
        left -= 2 * kTuneProbe * (s->persist ? kPersistProbe : 1);
        if (ms < best) {
            best = ms;
            bnt = c[0];
            bh = c[1];
            bpers = s->persist;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    swb::set_geometry(s->a, bnt, bh);
    s->persist = bpers;
    s->invalidate_graph();
    s->tuned = true;
    if (rc == SWB_OK) {
        std::lock_guard<std::mutex> g(g_tune_mu);
        g_tuned.push_back({s->p.Lx, s->p.Ly, s->precision, s->mode, bnt, bh, bpers ? 1 : 0});
    }
    return rc;
}

int fused_steps(swb_state *s, long long nsteps) {
    long long left = nsteps;
    const long long steps0 = s->steps;
    const bool tune_now = !s->tuned && s->autotune && nsteps >= kTuneMinSteps;
    if (s->host_fresh && left > 0) {
        // the first iteration after the fields were set, alone (see launch_sequence)
        CUDA_TRY(&s->err, launch_sequence(s, 1));
        s->steps += 1;
        left -= 1;
        s->host_fresh = false;
        s->fields_current = false;
    }
    if (tune_now) {
        int rc = autotune_geometry(s, left);
        if (rc) return rc;
    }
    // (a resident-tile state whose θ, forces or τ changed since the form was
    // chosen runs one launch per iteration, on strips of the same rows)
    if (s->persist && run_possible(s)) {
        if (left > 0) CUDA_TRY(&s->err, run_sequence(s, left));
        left = 0;
    }
    if (left >= kGraphSteps) {
        if (!s->gvalid) {
            cudaGraph_t g = nullptr;
            CUDA_TRY(&s->err, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            const unsigned long long c0 = swb::launches_so_far();
            cudaError_t le = launch_sequence(s, kGraphSteps);
            s->graph_launches = swb::launches_so_far() - c0;
            swb::count_launches(0ULL - s->graph_launches);  // captured, not run
            cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
            if (le != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return fail(&s->err, SWB_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(le));
            }
            CUDA_TRY(&s->err, ce);
            cudaError_t ie = cudaGraphInstantiate(&s->gexec, g, 0);
            cudaGraphDestroy(g);
            CUDA_TRY(&s->err, ie);
            s->gvalid = true;
            s->gsteps = kGraphSteps;
        }
        while (left >= s->gsteps) {
            CUDA_TRY(&s->err, cudaGraphLaunch(s->gexec, s->stream));
            swb::count_launches(s->graph_launches);
            left -= s->gsteps;
        }
    }
    if (left > 0) CUDA_TRY(&s->err, launch_sequence(s, (int)left));
    s->steps = steps0 + nsteps;
    if (nsteps > 0) {
        s->host_fresh = false;
        s->fields_current = false;
    }
    return SWB_OK;
}

void record_to_measure(const Record &r, swb_measure *m) {
    m->t = r.t;
    m->mass = r.mass;
    m->wetted = (int64_t)r.wetted;
    m->hmax = r.hmax;
    m->hmin = r.hmin;
    m->area = r.area;
    m->energy = r.area - r.cos_sum;
}

}  // namespace

// ------------------------------------------------------------------ ABI
extern "C" {

int swb_abi_version(void) { return SWB_ABI_VERSION; }

const char *swb_last_error(const swb_state *s) {
    if (s && !s->err.empty()) return s->err.c_str();
    return g_err.c_str();
}

const char *swb_status_string(int st) {
    switch (st) {
        case SWB_OK: return "ok";
        case SWB_ERR_ARG: return "invalid argument";
        case SWB_ERR_OOM: return "out of device memory";
        case SWB_ERR_CUDA: return "CUDA error";
        case SWB_ERR_NAN: return "non-finite height";
        case SWB_ERR_UNSUPPORTED: return "unsupported in this mode";
        case SWB_ERR_CANCELLED: return "cancelled";
        case SWB_ERR_NOT_FOUND: return "not found";
        case SWB_ERR_BUSY: return "busy";
        default: return "unknown status";
    }
}

int swb_state_bytes(const swb_params *p, int precision, size_t *bytes) {
    int rc = check_params(p, nullptr);
    if (rc) return rc;
    if (!bytes) return fail(nullptr, SWB_ERR_ARG, "bytes is NULL");
    const long long N = (long long)p->Lx * p->Ly, pitch = pitch_of(N);
    const long long tiles = swb::max_tiles(p->Lx, p->Ly);
    size_t b = 0;
    if (precision == SWB_PLAIN64) {
        b = align256((size_t)27 * N * 8) + 11 * align256((size_t)N * 8);
    } else if (precision == SWB_F64 || precision == SWB_F32 || precision == SWB_F16) {
        b = 2 * align256(fbuf_bytes(precision, pitch)) + 3 * align256((size_t)N * real_bytes(precision)) +
            align256((size_t)2 * tiles * swb::kNPart * 8) + align256(sizeof(Control)) +
            align256(swb::kBarWords * sizeof(unsigned int));
    } else {
        return fail(nullptr, SWB_ERR_ARG, "unknown precision");
    }
    b += align256((size_t)swb::kRecCap * sizeof(Record)) + align256(sizeof(Record)) +
         align256((size_t)swb::measure_blocks(N) * swb::kNPart * 8) + 256;
    *bytes = b;
    return SWB_OK;
}

int swb_create(const swb_params *p, int precision, swb_state **out) {
    if (!out) return fail(nullptr, SWB_ERR_ARG, "out is NULL");
    *out = nullptr;
    int rc = check_params(p, nullptr);
    if (rc) return rc;
    if (precision < SWB_F64 || precision > SWB_PLAIN64) return fail(nullptr, SWB_ERR_ARG, "unknown precision");
    swb_state *s = new swb_state();
    s->p = *p;
    s->precision = precision;
    s->N = (long long)p->Lx * p->Ly;
    s->pitch = pitch_of(s->N);
    fill_args_from_params(s->a, *p);
    s->a.pitch = s->pitch;
    s->a.mass_fixed = (precision == SWB_F32 || precision == SWB_F16) ? 1 : 0;
    s->a.mass_corr = (precision == SWB_F16) ? 1 : 0;
    auto bad = [&](int code) {
        std::string m = s->err.empty() ? g_err : s->err;
        delete s;
        g_err = m;
        return code;
    };
#define CREATE_TRY(expr)                                                                   \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            s->err = std::string(#expr) + ": " + cudaGetErrorString(e_);                   \
            return bad(e_ == cudaErrorMemoryAllocation ? SWB_ERR_OOM : SWB_ERR_CUDA);      \
        }                                                                                  \
    } while (0)
    CREATE_TRY(cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking));
    s->stream = s->own_stream;
    const long long N = s->N;
    if (precision == SWB_PLAIN64) {
        PlainState &ps = s->ps;
        ps.Lx = p->Lx;
        ps.Ly = p->Ly;
        ps.N = N;
        double **nine[3] = {&ps.fout, &ps.ftemp, &ps.feq};
        for (auto q : nine) CREATE_TRY(s->alloc((void **)q, (size_t)9 * N * 8));
        double **one[11] = {&ps.h, &ps.ux, &ps.uy, &ps.vsq, &ps.p, &ps.Fx,
                            &ps.Fy, &ps.sx, &ps.sy, &ps.hgx, &ps.hgy};
        for (auto q : one) CREATE_TRY(s->alloc((void **)q, (size_t)N * 8));
        for (auto q : nine) CREATE_TRY(cudaMemsetAsync(*q, 0, (size_t)9 * N * 8, s->stream));
        for (auto q : one) CREATE_TRY(cudaMemsetAsync(*q, 0, (size_t)N * 8, s->stream));
        swb::count_launches(1);
        fill_kernel<<<blocks_for(N), 256, 0, s->stream>>>(ps.h, N, 1.0);
        CREATE_TRY(cudaGetLastError());
        s->a.hF = ps.h;
    } else {
        StepArgs &a = s->a;
        const size_t fb = fbuf_bytes(precision, s->pitch);
        CREATE_TRY(s->alloc(&a.fa, fb));
        CREATE_TRY(s->alloc(&a.fb, fb));
        CREATE_TRY(cudaMemsetAsync(a.fa, 0, fb, s->stream));
        CREATE_TRY(cudaMemsetAsync(a.fb, 0, fb, s->stream));
        const size_t fbytes = (size_t)N * s->rb();
        CREATE_TRY(s->alloc(&a.hF, fbytes));
        CREATE_TRY(s->alloc(&a.uxF, fbytes));
        CREATE_TRY(s->alloc(&a.uyF, fbytes));
        CREATE_TRY(cudaMemsetAsync(a.uxF, 0, fbytes, s->stream));
        CREATE_TRY(cudaMemsetAsync(a.uyF, 0, fbytes, s->stream));
        swb::count_launches(1);
        if (s->rb() == 8)
            fill_kernel<<<blocks_for(N), 256, 0, s->stream>>>((double *)a.hF, N, 1.0);
        else
            fill_kernel_f<<<blocks_for(N), 256, 0, s->stream>>>((float *)a.hF, N, 1.0f);
        CREATE_TRY(cudaGetLastError());
        int gnt = 0, gh = 0;
        swb::default_geometry(p->Lx, p->Ly, precision, &gnt, &gh);
        swb::set_geometry(a, gnt, gh);
        a.part_stride = (int)swb::max_tiles(p->Lx, p->Ly);
        CREATE_TRY(s->alloc((void **)&a.partials, (size_t)2 * a.part_stride * swb::kNPart * 8));
        CREATE_TRY(s->alloc((void **)&a.ctl, sizeof(Control)));
        CREATE_TRY(s->alloc((void **)&a.bar, swb::kBarWords * sizeof(unsigned int)));
        CREATE_TRY(cudaMemsetAsync(a.bar, 0, swb::kBarWords * sizeof(unsigned int), s->stream));
        Control c0{};
        c0.fresh_step = 1;
        CREATE_TRY(cudaMemcpyAsync(a.ctl, &c0, sizeof(Control), cudaMemcpyHostToDevice, s->stream));
    }
    CREATE_TRY(s->alloc((void **)&s->rec, (size_t)swb::kRecCap * sizeof(Record)));
    CREATE_TRY(s->alloc((void **)&s->mrec, sizeof(Record)));
    CREATE_TRY(s->alloc((void **)&s->mscratch, (size_t)swb::measure_blocks(N) * swb::kNPart * 8));
    CREATE_TRY(s->alloc((void **)&s->mticket, sizeof(unsigned int)));
    CREATE_TRY(cudaMemsetAsync(s->mticket, 0, sizeof(unsigned int), s->stream));
    s->a.records = s->rec;
    s->a.rec_cap = swb::kRecCap;
    s->persist = persist_default(s);
    CREATE_TRY(cudaStreamSynchronize(s->stream));
#undef CREATE_TRY
    *out = s;
    return SWB_OK;
}

int swb_destroy(swb_state *s) {
    delete s;
    return SWB_OK;
}

int swb_get_params(const swb_state *s, swb_params *p, int *precision) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (p) *p = s->p;
    if (precision) *precision = s->precision;
    return SWB_OK;
}

int swb_set_field(swb_state *s, int field, const double *host) {
    if (!s || !host) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    const long long N = s->N;
    if (s->plain()) {
        PlainState &ps = s->ps;
        double *dst = nullptr;
        long long n = N;
        switch (field) {
            case SWB_FIELD_HEIGHT: dst = ps.h; break;
            case SWB_FIELD_VELX: dst = ps.ux; break;
            case SWB_FIELD_VELY: dst = ps.uy; break;
            case SWB_FIELD_PRESSURE: dst = ps.p; break;
            case SWB_FIELD_FOUT: dst = ps.fout; n = 9 * N; break;
            case SWB_FIELD_FEQ: dst = ps.feq; n = 9 * N; break;
            case SWB_FIELD_FX: dst = ps.Fx; break;
            case SWB_FIELD_FY: dst = ps.Fy; break;
            case SWB_FIELD_SLIPX: dst = ps.sx; break;
            case SWB_FIELD_SLIPY: dst = ps.sy; break;
            case SWB_FIELD_HGRADPX: dst = ps.hgx; break;
            case SWB_FIELD_HGRADPY: dst = ps.hgy; break;
            case SWB_FIELD_VSQ: dst = ps.vsq; break;
            default: return fail(&s->err, SWB_ERR_ARG, "unknown field");
        }
        CUDA_TRY(&s->err, cudaMemcpyAsync(dst, host, n * 8, cudaMemcpyHostToDevice, s->stream));
        // the reference's fout and ftemp are equal between steps
        if (field == SWB_FIELD_FOUT)
            CUDA_TRY(&s->err, cudaMemcpyAsync(ps.ftemp, host, n * 8, cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
        return SWB_OK;
    }
    int rc = materialize(s);
    if (rc) return rc;
    StepArgs &a = s->a;
    switch (field) {
        case SWB_FIELD_HEIGHT: rc = upload_field(s, a.hF, host, N); break;
        case SWB_FIELD_VELX: rc = upload_field(s, a.uxF, host, N); break;
        case SWB_FIELD_VELY: rc = upload_field(s, a.uyF, host, N); break;
        case SWB_FIELD_FOUT: {
            rc = ensure_tmp(s, (size_t)9 * N * 8);
            if (rc) return rc;
            CUDA_TRY(&s->err, cudaMemcpyAsync(s->dtmp, host, (size_t)9 * N * 8, cudaMemcpyHostToDevice, s->stream));
            const long long step = s->steps;
            void *dst = (step & 1) ? a.fb : a.fa;  // the buffer the next step pulls from
            swb::count_launches(1);
            push_kernel<double><<<blocks_for(N), 256, 0, s->stream>>>(s->dtmp, dst, s->p.Lx, s->p.Ly,
                                                                      s->pitch, s->precision);
            CUDA_TRY(&s->err, cudaGetLastError());
            break;
        }
        default: return fail(&s->err, SWB_ERR_UNSUPPORTED, "field cannot be set in a fused mode");
    }
    if (rc) return rc;
    return set_fresh(s);
}

int swb_get_field(swb_state *s, int field, double *host) {
    if (!s || !host) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    const long long N = s->N;
    if (s->plain()) {
        PlainState &ps = s->ps;
        const double *src = nullptr;
        long long n = N;
        switch (field) {
            case SWB_FIELD_HEIGHT: src = ps.h; break;
            case SWB_FIELD_VELX: src = ps.ux; break;
            case SWB_FIELD_VELY: src = ps.uy; break;
            case SWB_FIELD_PRESSURE: src = ps.p; break;
            case SWB_FIELD_FOUT: src = ps.fout; n = 9 * N; break;
            case SWB_FIELD_FEQ: src = ps.feq; n = 9 * N; break;
            case SWB_FIELD_FX: src = ps.Fx; break;
            case SWB_FIELD_FY: src = ps.Fy; break;
            case SWB_FIELD_SLIPX: src = ps.sx; break;
            case SWB_FIELD_SLIPY: src = ps.sy; break;
            case SWB_FIELD_HGRADPX: src = ps.hgx; break;
            case SWB_FIELD_HGRADPY: src = ps.hgy; break;
            case SWB_FIELD_VSQ: src = ps.vsq; break;
            default: return fail(&s->err, SWB_ERR_ARG, "unknown field");
        }
        return download_field(s, src, host, n, 8);
    }
    int rc = materialize(s);
    if (rc) return rc;
    StepArgs &a = s->a;
    switch (field) {
        case SWB_FIELD_HEIGHT: return download_field(s, a.hF, host, N, s->rb());
        case SWB_FIELD_VELX: return download_field(s, a.uxF, host, N, s->rb());
        case SWB_FIELD_VELY: return download_field(s, a.uyF, host, N, s->rb());
        case SWB_FIELD_PRESSURE: {
            rc = ensure_tmp(s, (size_t)N * 8);
            if (rc) return rc;
            CUDA_TRY(&s->err, swb::launch_pressure_now(s->precision, a, s->dtmp, s->stream));
            return download_field(s, s->dtmp, host, N, 8);
        }
        case SWB_FIELD_FOUT: {
            rc = ensure_tmp(s, (size_t)9 * N * 8);
            if (rc) return rc;
            CUDA_TRY(&s->err, swb::launch_fout(s->precision, a, s->dtmp, s->stream));
            return download_field(s, s->dtmp, host, 9 * N, 8);
        }
        default: return fail(&s->err, SWB_ERR_UNSUPPORTED, "field not available in a fused mode");
    }
}

int swb_set_theta(swb_state *s, double theta) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (s->a.theta_mode == swb::THETA_SCALAR && s->p.theta == theta) return SWB_OK;
    s->p.theta = theta;
    s->a.theta_mode = swb::THETA_SCALAR;
    s->a.shift_tmove = 0;
    s->a.kap = host_kappa(theta, s->p.n, s->p.m, s->p.hmin);
    s->a.cos_theta = host_cospi(theta);
    s->invalidate_graph();
    return SWB_OK;
}

int swb_set_theta_field(swb_state *s, const double *theta) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (!theta) return swb_set_theta(s, s->p.theta);
    const long long N = s->N;
    std::vector<double> kap(N), cs(N);
    for (long long i = 0; i < N; ++i) {
        kap[i] = host_kappa(theta[i], s->p.n, s->p.m, s->p.hmin);
        cs[i] = host_cospi(theta[i]);
    }
    StepArgs &a = s->a;
    if (s->plain()) {
        if (!s->plain_kapF) CUDA_TRY(&s->err, s->alloc((void **)&s->plain_kapF, (size_t)N * 8));
        if (!s->plain_cosF) CUDA_TRY(&s->err, s->alloc((void **)&s->plain_cosF, (size_t)N * 8));
        CUDA_TRY(&s->err, cudaMemcpyAsync(s->plain_kapF, kap.data(), N * 8, cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(&s->err, cudaMemcpyAsync(s->plain_cosF, cs.data(), N * 8, cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    } else {
        if (!a.kapF) {
            void *k = nullptr, *c = nullptr;
            CUDA_TRY(&s->err, s->alloc(&k, (size_t)N * s->rb()));
            CUDA_TRY(&s->err, s->alloc(&c, (size_t)N * s->rb()));
            a.kapF = k;
            a.cosF = c;
        }
        int rc = upload_field(s, (void *)a.kapF, kap.data(), N);
        if (rc) return rc;
        rc = upload_field(s, (void *)a.cosF, cs.data(), N);
        if (rc) return rc;
    }
    a.theta_mode = swb::THETA_FIELD;
    a.shift_tmove = 0;  // a new field starts at rest
    s->invalidate_graph();
    return SWB_OK;
}

int swb_set_substrate_motion(swb_state *s, int64_t tmove, int dx, int dy) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (tmove < 0 || dx < 0 || dy < 0 || tmove > (int64_t)INT32_MAX)
        return fail(&s->err, SWB_ERR_ARG, "substrate motion: tmove, dx, dy must be >= 0");
    if (tmove > 0 && s->a.theta_mode != swb::THETA_FIELD)
        return fail(&s->err, SWB_ERR_UNSUPPORTED, "substrate motion moves a θ field: set one first");
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    s->a.shift_tmove = (int)tmove;
    s->a.shift_dx = dx % s->p.Lx;
    s->a.shift_dy = dy % s->p.Ly;
    s->a.shift_t0 = s->steps;
    s->invalidate_graph();
    return SWB_OK;
}

int swb_set_theta_wave(swb_state *s, double theta0, double dtheta, double v) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (s->plain()) return fail(&s->err, SWB_ERR_UNSUPPORTED, "moving wettability needs a fused mode");
    s->a.theta_mode = swb::THETA_WAVE;
    s->a.shift_tmove = 0;
    s->a.theta0 = theta0;
    s->a.dtheta = dtheta;
    s->a.wave_v = v;
    s->invalidate_graph();
    return SWB_OK;
}

int swb_set_inclination(swb_state *s, double ax, double ay, int loop_time, int64_t t,
                        int64_t tstart, int64_t tsmooth) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (tsmooth == 0) return fail(&s->err, SWB_ERR_ARG, "tsmooth must be nonzero");
    const int on = (ax != 0.0 || ay != 0.0);
    if (s->incl == on && s->ax == ax && s->ay == ay && s->incl_loop_time == loop_time &&
        s->incl_t == t && s->incl_tstart == tstart && s->incl_tsmooth == tsmooth)
        return SWB_OK;
    s->incl = on;
    s->ax = ax;
    s->ay = ay;
    s->incl_loop_time = loop_time;
    s->incl_t = t;
    s->incl_tstart = tstart;
    s->incl_tsmooth = tsmooth;
    StepArgs &a = s->a;
    a.incl = on;
    a.ax = ax;
    a.ay = ay;
    a.incl_loop_time = loop_time;
    a.incl_fixed = incl_factor(t, tstart, tsmooth);
    a.incl_tstart = tstart;
    a.incl_tsmooth = tsmooth;
    s->invalidate_graph();
    return SWB_OK;
}

int swb_set_geometry(swb_state *s, int nt, int h) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (s->plain()) return SWB_OK;
    if (nt == 0 && h == 0) {
        swb::default_geometry(s->p.Lx, s->p.Ly, s->precision, &nt, &h);  // nt == 0: choose
    } else if (nt == swb::kTileGeom) {
        if (s->precision == SWB_F64)
            return fail(&s->err, SWB_ERR_UNSUPPORTED, "2D tiles: FP32 and FP16 storage only");
        h = swb::kTileY;
    } else if (swb::resident_geometry(nt)) {
        if (s->precision != SWB_F32 && s->precision != SWB_F16)
            return fail(&s->err, SWB_ERR_UNSUPPORTED, "resident tiles: FP32 and FP16 storage only");
        if (h == 0) h = resident_rows(s->p.Lx, s->p.Ly, s->precision, nt);
        if (h < 1 || h > swb::kResMaxTH)
            return fail(&s->err, SWB_ERR_UNSUPPORTED,
                        "resident tiles: the lattice does not fit in the GPU's shared memory "
                        "(rows must be 1..40 with every tile co-resident)");
        const long long tiles = (long long)((s->p.Lx + swb::kResTW - 1) / swb::kResTW) *
                                ((s->p.Ly + h - 1) / h);
        if (tiles > (long long)swb::resident_blocks_per_sm(s->precision, h, nt) * sm_count())
            return fail(&s->err, SWB_ERR_UNSUPPORTED,
                        "resident tiles: more tiles than the GPU holds at once; use more rows");
    } else if (swb::pair_geometry(nt)) {
        if (s->precision == SWB_F64)
            return fail(&s->err, SWB_ERR_UNSUPPORTED, "pair strips: FP32 and FP16 storage only");
        if (s->p.Lx % 2)
            return fail(&s->err, SWB_ERR_UNSUPPORTED, "pair strips: Lx must be even");
        if (h < swb::kMinRows || h > swb::kMaxRows)
            return fail(&s->err, SWB_ERR_ARG, "geometry: 2 <= h <= 512");
    } else if ((nt != 64 && nt != 128 && nt != 256) || h < swb::kMinRows || h > swb::kMaxRows) {
        return fail(&s->err, SWB_ERR_ARG,
                    "geometry: nt must be 64, 128 or 256 and 2 <= h <= 512, nt = -32, -64 or "
                    "-128 (pair strips), or nt = 32 (2D tiles)");
    }
    if (s->mode == SWB_STEP_MULTI && (nt == 256 || nt < 0))
        return fail(&s->err, SWB_ERR_UNSUPPORTED, "multi-step kernel: nt must be 64, 128, 32 or 33");
    s->autotune = false;  // an explicit geometry (or the default) is kept
    s->tuned = true;
    if (s->a.march_nt != nt || s->a.march_h != h) {
        CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
        swb::set_geometry(s->a, nt, h);
        s->invalidate_graph();
    }
    s->persist = persist_default(s);
    return SWB_OK;
}

int swb_set_step_mode(swb_state *s, int mode) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (mode != SWB_STEP_AUTO && mode != SWB_STEP_PER_ITERATION && mode != SWB_STEP_MULTI)
        return fail(&s->err, SWB_ERR_ARG, "unknown step mode");
    if (s->plain())
        return mode == SWB_STEP_MULTI
                   ? fail(&s->err, SWB_ERR_UNSUPPORTED, "plain path: one kernel per op")
                   : SWB_OK;
    if (mode == SWB_STEP_MULTI && s->precision != SWB_F32 && s->precision != SWB_F16)
        return fail(&s->err, SWB_ERR_UNSUPPORTED, "multi-step kernel: FP32 and FP16 storage only");
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    s->mode = mode;
    if (mode == SWB_STEP_MULTI && (s->a.march_nt == 256 || s->a.march_nt < 0)) {
        int nt = 128, h = 0;
        swb::default_geometry(s->p.Lx, s->p.Ly, s->precision, &nt, &h);
        swb::set_geometry(s->a, nt, h);
    }
    if (mode == SWB_STEP_PER_ITERATION && swb::resident_geometry(s->a.march_nt)) {
        int nt = 0, h = 0;  // resident tiles are a multi-step form
        swb::default_geometry(s->p.Lx, s->p.Ly, s->precision, &nt, &h);
        swb::set_geometry(s->a, nt, h);
    }
    if (s->autotune) s->tuned = false;  // re-tune within the new form
    s->persist = persist_default(s);
    s->invalidate_graph();
    return SWB_OK;
}

int swb_get_step_mode(swb_state *s, int *mode) {
    if (!s || !mode) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    *mode = (!s->plain() && s->persist) ? SWB_STEP_MULTI : SWB_STEP_PER_ITERATION;
    return SWB_OK;
}

int swb_get_geometry(swb_state *s, int *nt, int *h) {
    if (!s || !nt || !h) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    *nt = s->a.march_nt;
    *h = s->a.march_h;
    return SWB_OK;
}

int swb_set_mass_correction(swb_state *s, int on) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    const int v = (on && (s->precision == SWB_F32 || s->precision == SWB_F16)) ? 1 : 0;
    if (s->a.mass_corr != v) {
        s->a.mass_corr = v;
        s->invalidate_graph();
    }
    return SWB_OK;
}

int swb_set_measures(swb_state *s, int mask, double hthresh) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (mask & ~SWB_MEAS_ALL) return fail(&s->err, SWB_ERR_ARG, "unknown measure bits");
    if (s->a.meas_mask == mask && s->a.hthresh == hthresh) return SWB_OK;
    s->a.meas_mask = mask;
    s->a.hthresh = hthresh;
    s->plain_meas_mask = mask;
    s->invalidate_graph();
    return SWB_OK;
}

namespace {
int run_steps(swb_state *s, long long n) {
    if (s->plain()) {
        for (long long k = 0; k < n; ++k) {
            int rc = plain_iteration(s);
            if (rc) return rc;
        }
        return SWB_OK;
    }
    return fused_steps(s, n);
}

// snapshot!(fluid, height, t) (src/measures.jl:99-105) of the height after
// the current iteration, into the next slot of the device ring.
int take_snapshot(swb_state *s) {
    int rc = materialize(s);
    if (rc) return rc;
    const long long N = s->N;
    double *dst = s->snap + (size_t)(s->snap_count % s->snap_cap) * N;
    if (s->plain()) {
        CUDA_TRY(&s->err, cudaMemcpyAsync(dst, s->ps.h, N * 8, cudaMemcpyDeviceToDevice, s->stream));
    } else if (s->rb() == 8) {
        CUDA_TRY(&s->err, cudaMemcpyAsync(dst, s->a.hF, N * 8, cudaMemcpyDeviceToDevice, s->stream));
    } else {
        f2d_kernel<<<blocks_for(N), 256, 0, s->stream>>>((const float *)s->a.hF, dst, N);
        swb::count_launches(1);
        CUDA_TRY(&s->err, cudaGetLastError());
    }
    s->snap_t[(size_t)(s->snap_count % s->snap_cap)] = s->steps;
    s->snap_count++;
    return SWB_OK;
}
}  // namespace

int swb_step(swb_state *s, int64_t nsteps) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (nsteps < 0) return fail(&s->err, SWB_ERR_ARG, "nsteps must be >= 0");
    if (s->snap_every <= 0) return run_steps(s, nsteps);
    // run to each multiple of the dump interval, then take the snapshot
    long long left = nsteps;
    while (left > 0) {
        const long long to_dump = s->snap_every - s->steps % s->snap_every;
        const long long n = left < to_dump ? left : to_dump;
        int rc = run_steps(s, n);
        if (rc) return rc;
        left -= n;
        if (s->steps % s->snap_every == 0) {
            rc = take_snapshot(s);
            if (rc) return rc;
        }
    }
    return SWB_OK;
}

int swb_set_snapshots(swb_state *s, int64_t dumping, int64_t capacity) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (dumping < 0 || (dumping > 0 && capacity < 1))
        return fail(&s->err, SWB_ERR_ARG, "snapshots: dumping >= 0 and capacity >= 1");
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    if (s->snap) {
        cudaFree(s->snap);
        for (auto &q : s->allocs)
            if (q == s->snap) q = nullptr;
        s->snap = nullptr;
    }
    s->snap_every = dumping;
    s->snap_cap = dumping > 0 ? capacity : 0;
    s->snap_count = s->snap_read = 0;
    s->snap_t.assign((size_t)s->snap_cap, 0);
    if (dumping > 0)
        CUDA_TRY(&s->err, s->alloc((void **)&s->snap, (size_t)capacity * s->N * 8));
    return SWB_OK;
}

int swb_get_snapshots(swb_state *s, double *out, int64_t cap, int64_t *count, int64_t *times) {
    if (!s || !count || (cap > 0 && !out)) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    *count = 0;
    if (!s->snap) return SWB_OK;
    long long first = s->snap_read;
    if (s->snap_count - first > s->snap_cap) first = s->snap_count - s->snap_cap;  // overwritten
    long long n = s->snap_count - first;
    if (n > cap) n = cap;
    const long long N = s->N;
    for (long long k = 0; k < n; ++k) {
        const long long slot = (first + k) % s->snap_cap;
        CUDA_TRY(&s->err, cudaMemcpyAsync(out + (size_t)k * N, s->snap + (size_t)slot * N, N * 8,
                                          cudaMemcpyDeviceToHost, s->stream));
        if (times) times[k] = s->snap_t[(size_t)slot];
    }
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    s->snap_read = first + n;
    *count = n;
    return SWB_OK;
}

int swb_sync(swb_state *s) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    return check_nan(s);
}

int swb_steps_done(swb_state *s, int64_t *t) {
    if (!s || !t) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    *t = s->steps;
    return SWB_OK;
}

int swb_get_measures(swb_state *s, swb_measure *out, int64_t cap, int64_t *count) {
    if (!s || !count) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    *count = 0;
    long long head = 0;
    if (s->plain()) {
        head = s->plain_rec_head;
    } else {
        CUDA_TRY(&s->err, cudaMemcpyAsync(&head, &s->a.ctl->rec_head, sizeof(long long),
                                          cudaMemcpyDeviceToHost, s->stream));
    }
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    long long first = s->rec_read;
    if (head - first > swb::kRecCap) {  // older ones overwritten
        s->rec_dropped += head - swb::kRecCap - first;
        first = head - swb::kRecCap;
        s->rec_read = first;
    }
    long long n = head - first;
    if (n > cap) n = cap;
    std::vector<Record> tmp(n);
    for (long long k = 0; k < n;) {
        const long long slot = (first + k) % swb::kRecCap;
        long long run = std::min<long long>(n - k, swb::kRecCap - slot);
        CUDA_TRY(&s->err, cudaMemcpyAsync(tmp.data() + k, s->rec + slot, run * sizeof(Record),
                                          cudaMemcpyDeviceToHost, s->stream));
        k += run;
    }
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    for (long long k = 0; k < n; ++k) record_to_measure(tmp[k], out + k);
    s->rec_read = first + n;
    *count = n;
    return check_nan(s);
}

int swb_measures_dropped(swb_state *s, int64_t *dropped) {
    if (!s || !dropped) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    long long head = 0;
    if (s->plain()) {
        head = s->plain_rec_head;
    } else {
        CUDA_TRY(&s->err, cudaMemcpyAsync(&head, &s->a.ctl->rec_head, sizeof(long long),
                                          cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    }
    const long long lost = head - s->rec_read - swb::kRecCap;
    *dropped = s->rec_dropped + (lost > 0 ? lost : 0);
    return SWB_OK;
}

int swb_measure_now(swb_state *s, double hthresh, swb_measure *out) {
    if (!s || !out) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    int rc = materialize(s);
    if (rc) return rc;
    // the current height is what iteration steps + 1 starts from: the θ of
    // a moving field or wave at that iteration, as in its own record
    const void *h = s->plain() ? (const void *)s->ps.h : s->a.hF;
    CUDA_TRY(&s->err, swb::launch_measure(h, s->rb() == 8, s->p.Lx, s->p.Ly, hthresh,
                                          cos_source(s, s->steps + 1), s->mscratch, s->mticket,
                                          s->mrec, s->steps, s->stream));
    Record r{};
    CUDA_TRY(&s->err, cudaMemcpyAsync(&r, s->mrec, sizeof(Record), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    record_to_measure(r, out);
    return SWB_OK;
}

int swb_set_thermal_seed(swb_state *s, uint64_t seed) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    if (s->a.seed != seed) {
        CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
        s->a.seed = seed;
        s->invalidate_graph();
    }
    return SWB_OK;
}

int swb_thermal_field(swb_state *s, int64_t t, double *fx, double *fy) {
    if (!s || !fx || !fy) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    int rc = materialize(s);
    if (rc) return rc;
    rc = ensure_tmp(s, (size_t)2 * s->N * 8);
    if (rc) return rc;
    StepArgs a = s->a;
    int prec = s->precision;
    if (s->plain()) {
        a.hF = s->ps.h;
        prec = SWB_F64;
    }
    CUDA_TRY(&s->err, swb::launch_thermal_field(prec, a, t, s->dtmp, s->dtmp + s->N, s->stream));
    CUDA_TRY(&s->err, cudaMemcpyAsync(fx, s->dtmp, s->N * 8, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(&s->err, cudaMemcpyAsync(fy, s->dtmp + s->N, s->N * 8, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
    return SWB_OK;
}

int swb_set_field_device(swb_state *s, int field, const double *dptr) {
    if (!s || !dptr) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    if (field != SWB_FIELD_HEIGHT && field != SWB_FIELD_VELX && field != SWB_FIELD_VELY)
        return fail(&s->err, SWB_ERR_UNSUPPORTED, "device upload supports height and velocities");
    const long long N = s->N;
    void *dst;
    if (s->plain()) {
        dst = field == SWB_FIELD_HEIGHT ? (void *)s->ps.h : field == SWB_FIELD_VELX ? (void *)s->ps.ux : (void *)s->ps.uy;
        CUDA_TRY(&s->err, cudaMemcpyAsync(dst, dptr, N * 8, cudaMemcpyDeviceToDevice, s->stream));
        return SWB_OK;
    }
    int rc = materialize(s);
    if (rc) return rc;
    dst = field == SWB_FIELD_HEIGHT ? s->a.hF : field == SWB_FIELD_VELX ? s->a.uxF : s->a.uyF;
    if (s->rb() == 8) {
        CUDA_TRY(&s->err, cudaMemcpyAsync(dst, dptr, N * 8, cudaMemcpyDeviceToDevice, s->stream));
    } else {
        d2f_kernel<<<blocks_for(N), 256, 0, s->stream>>>(dptr, (float *)dst, N);
        swb::count_launches(1);
        CUDA_TRY(&s->err, cudaGetLastError());
    }
    return set_fresh(s);
}

int swb_set_stream(swb_state *s, void *stream) {
    if (!s) return fail(nullptr, SWB_ERR_ARG, "state is NULL");
    cudaStream_t ns = stream ? (cudaStream_t)stream : s->own_stream;
    if (ns != s->stream) {
        CUDA_TRY(&s->err, cudaStreamSynchronize(s->stream));
        s->stream = ns;
    }
    return SWB_OK;
}

int swb_get_stream(swb_state *s, void **stream) {
    if (!s || !stream) return fail(s ? &s->err : nullptr, SWB_ERR_ARG, "NULL argument");
    *stream = (void *)s->stream;
    return SWB_OK;
}

int swb_launch_count(uint64_t *count) {
    if (!count) return fail(nullptr, SWB_ERR_ARG, "NULL argument");
    *count = swb::g_launches.load();
    return SWB_OK;
}

// ---------------------------------------------------------------- per-op API
#define PLAIN_ONLY(s)                                                                  \
    do {                                                                               \
        if (!(s)) return fail(nullptr, SWB_ERR_ARG, "state is NULL");                  \
        if (!(s)->plain())                                                             \
            return fail(&(s)->err, SWB_ERR_UNSUPPORTED, "per-op calls need SWB_PLAIN64"); \
    } while (0)

int swb_op_filmpressure(swb_state *s) {
    PLAIN_ONLY(s);
    const bool field = s->a.theta_mode == swb::THETA_FIELD;
    CUDA_TRY(&s->err, swb::plain_filmpressure(s->ps, field ? s->plain_kapF : nullptr, s->a.kap,
                                              s->p.gamma, s->p.n, s->p.m, s->p.hmin, s->p.hcrit,
                                              0, 0, s->stream));
    return SWB_OK;
}
int swb_op_hgradp(swb_state *s) {
    PLAIN_ONLY(s);
    CUDA_TRY(&s->err, swb::plain_hgradp(s->ps, s->stream));
    return SWB_OK;
}
int swb_op_slippage(swb_state *s) {
    PLAIN_ONLY(s);
    CUDA_TRY(&s->err, swb::plain_slippage(s->ps, s->p.delta, s->p.mu, s->stream));
    return SWB_OK;
}
int swb_op_force_sum(swb_state *s) {
    PLAIN_ONLY(s);
    CUDA_TRY(&s->err, swb::plain_force_sum(s->ps, s->stream));
    return SWB_OK;
}
int swb_op_thermal(swb_state *s, int64_t t) {
    PLAIN_ONLY(s);
    if (!s->a.thermal) return SWB_OK;
    CUDA_TRY(&s->err, swb::plain_thermal(s->ps, s->a.k6, s->p.delta, s->a.seed, t, s->stream));
    return SWB_OK;
}
int swb_op_inclination(swb_state *s, double ax, double ay, int64_t t, int64_t tstart,
                       int64_t tsmooth) {
    PLAIN_ONLY(s);
    if (tsmooth == 0) return fail(&s->err, SWB_ERR_ARG, "tsmooth must be nonzero");
    CUDA_TRY(&s->err, swb::plain_inclination(s->ps, ax, ay, incl_factor(t, tstart, tsmooth), s->stream));
    return SWB_OK;
}
int swb_op_equilibrium(swb_state *s) {
    PLAIN_ONLY(s);
    CUDA_TRY(&s->err, swb::plain_equilibrium(s->ps, s->p.g, s->stream));
    return SWB_OK;
}
int swb_op_bgk_stream(swb_state *s) {
    PLAIN_ONLY(s);
    CUDA_TRY(&s->err, swb::plain_collide(s->ps, 1.0 - 1.0 / s->p.tau, 1.0 / s->p.tau, s->stream));
    CUDA_TRY(&s->err, swb::plain_stream(s->ps, s->stream));
    return SWB_OK;
}
int swb_op_moments(swb_state *s) {
    PLAIN_ONLY(s);
    CUDA_TRY(&s->err, swb::plain_moments(s->ps, s->stream));
    return SWB_OK;
}

}  // extern "C"
