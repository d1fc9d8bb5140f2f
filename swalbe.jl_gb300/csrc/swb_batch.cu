// swb_batch.cu -- batched ensembles: many lattices of uneven size and
// parameters advanced together, one launch per time step over a packed tile
// table (persistent CTAs walk the table), replayed from a captured CUDA graph.
// The CTA count per launch is picked by timing the candidates on the first
// steps (the timed steps are real steps of the simulation).
#include <algorithm>
#include <array>
#include <chrono>
#include <string>
#include <vector>

#include "swb_lattice.h"

using swb::Control;
using swb::LatticeLayout;
using swb::StepArgs;
using swb::TileRef;

namespace swb {

namespace {
thread_local std::string b_err;
int bfail(std::string *slot, int code, const std::string &m) {
    b_err = m;
    set_global_error(m.c_str());
    if (slot) *slot = m;
    return code;
}

__global__ void fill_d(double *d, long long n, double v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        d[i] = v;
}
__global__ void fill_f(float *d, long long n, float v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        d[i] = v;
}
__global__ void d2f(const double *s, float *d, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        d[i] = (float)s[i];
}
__global__ void gather_nan(const StepArgs *args, int count, int *flags) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        flags[i] = args[i].ctl->nan_flag;
}

__global__ void set_fresh_k(Control *c) {
    c->fresh_step = c->step_base + 1;
    c->corr[0] = 0.0;
    c->corr[1] = 0.0;
}

int nblk(long long n) {
    long long b = (n + 255) / 256;
    return (int)std::min<long long>(std::max<long long>(b, 1), 2048);
}
}  // namespace

double host_cospi_shared(double x) {
    if (!std::isfinite(x)) return NAN;
    double r = std::fmod(std::fabs(x), 2.0);
    if (r == 0.0) return 1.0;
    if (r == 1.0) return -1.0;
    if (r == 0.5 || r == 1.5) return 0.0;
    const long double PI_L = 3.141592653589793238462643383279502884L;
    return (double)cosl(PI_L * (long double)r);
}

double host_kappa_shared(double theta, int n, int m, double hmin) {
    double a = 1.0 - host_cospi_shared(theta);
    a = a * (double)(n - 1);
    a = a * (double)(m - 1);
    return a / ((double)(n - m) * hmin);
}

cudaError_t lattice_init(const StepArgs &a, int precision, const LatticeLayout &L,
                         const double *h0_host, cudaStream_t st) {
    const long long N = (long long)a.Lx * a.Ly;
    cudaError_t e = cudaMemsetAsync(a.fa, 0, L.total, st);  // whole block is contiguous from fa
    if (e != cudaSuccess) return e;
    if (!h0_host) {
        count_launches(1);
        if (precision == SWB_F64)
            fill_d<<<nblk(N), 256, 0, st>>>((double *)a.hF, N, 1.0);
        else
            fill_f<<<nblk(N), 256, 0, st>>>((float *)a.hF, N, 1.0f);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    Control c0{};
    c0.fresh_step = 1;
    // c0 lives on this stack frame: a pageable-memory copy is staged before return
    e = cudaMemcpyAsync(a.ctl, &c0, sizeof(Control), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

cudaError_t lattice_upload_height(const StepArgs &a, int precision, const double *h_host,
                                  void *staging, cudaStream_t st) {
    const long long N = (long long)a.Lx * a.Ly;
    cudaError_t e;
    if (precision == SWB_F64) {
        e = cudaMemcpyAsync(a.hF, h_host, N * 8, cudaMemcpyHostToDevice, st);
    } else {
        e = cudaMemcpyAsync(staging, h_host, N * 8, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            count_launches(1);
            d2f<<<nblk(N), 256, 0, st>>>((const double *)staging, (float *)a.hF, N);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) return e;
    count_launches(1);
    set_fresh_k<<<1, 1, 0, st>>>(a.ctl);
    return cudaGetLastError();
}

cudaError_t lattice_download_height(const StepArgs &a, int precision, bool fields_current,
                                    double *h_host, cudaStream_t st) {
    const long long N = (long long)a.Lx * a.Ly;
    cudaError_t e = cudaSuccess;
    if (!fields_current) {
        e = launch_moments(precision, a, st);
        if (e != cudaSuccess) return e;
    }
    if (precision == SWB_F64) {
        e = cudaMemcpyAsync(h_host, a.hF, N * 8, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
        return cudaStreamSynchronize(st);
    }
    std::vector<float> tmp(N);
    e = cudaMemcpyAsync(tmp.data(), a.hF, N * 4, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    for (long long i = 0; i < N; ++i) h_host[i] = (double)tmp[i];
    return cudaSuccess;
}

}  // namespace swb

struct swb_batch {
    int count = 0, precision = 0;
    std::vector<swb_params> params;
    std::vector<LatticeLayout> layouts;
    std::vector<StepArgs> args;
    std::vector<char> fields_current;
    char *slab = nullptr;
    size_t slab_bytes = 0;
    double *staging = nullptr;
    StepArgs *d_args = nullptr;
    TileRef *d_tiles = nullptr;
    int *d_flags = nullptr;
    int ntiles = 0;
    // pair strips (nt < 0): the one-column strips (64 threads, same rows) of
    // the iterations the pair form leaves out, with their own table
    StepArgs *d_args_fb = nullptr;
    TileRef *d_tiles_fb = nullptr;
    int ntiles_fb = 0;
    size_t cap_tiles = 0, cap_tiles_fb = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int steps_per_graph = 32;
    int grid = 0;
    int nt = swb::kBatchNT, rows = swb::kBatchRows;  // strip geometry of every lattice
    bool tuned = false, args_dirty = true, gvalid = false;
    bool geometry_fixed = false;  // set by the caller: the tuner picks only the CTA count
    bool fresh_pending = true;  // a lattice's next iteration takes h, u from its fields
    long long steps = 0;
    std::string err;

    void invalidate() {
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
        gvalid = false;
    }
    ~swb_batch() {
        invalidate();
        if (stream) cudaStreamSynchronize(stream);
        cudaFree(slab);
        cudaFree(staging);
        cudaFree(d_args);
        cudaFree(d_tiles);
        cudaFree(d_flags);
        cudaFree(d_args_fb);
        cudaFree(d_tiles_fb);
        if (stream) cudaStreamDestroy(stream);
    }
};

#define B_TRY(b, expr)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return swb::bfail(&(b)->err, e_ == cudaErrorMemoryAllocation ? SWB_ERR_OOM : SWB_ERR_CUDA, \
                              std::string(#expr) + ": " + cudaGetErrorString(e_));        \
    } while (0)

namespace {

// Packed table of (lattice, strip) entries, the lattices' reducers first.
std::vector<TileRef> build_tiles(const std::vector<StepArgs> &args) {
    std::vector<TileRef> tiles, reducers;
    for (int i = 0; i < (int)args.size(); ++i) {
        const StepArgs &a = args[i];
        if (swb::needs_partials(a)) reducers.push_back({i, -1, 0});
        for (int ty = 0; ty < a.tiles_y; ++ty)
            for (int tx = 0; tx < a.tiles_x; ++tx) tiles.push_back({i, tx, ty});
    }
    tiles.insert(tiles.begin(), reducers.begin(), reducers.end());
    return tiles;
}

// Copies of the lattices' arguments with the one-column fallback strips.
std::vector<StepArgs> fallback_args(const swb_batch *b) {
    std::vector<StepArgs> fb = b->args;
    for (StepArgs &a : fb) a = swb::strip_fallback(a);
    return fb;
}

// Device copy of a tile table, growing its buffer when needed.
cudaError_t put_tiles(swb_batch *b, TileRef **d, size_t *cap, const std::vector<TileRef> &t) {
    if (t.size() > *cap) {
        cudaFree(*d);
        *d = nullptr;
        cudaError_t e = cudaMalloc((void **)d, sizeof(TileRef) * t.size());
        if (e != cudaSuccess) return e;
        *cap = t.size();
    }
    return cudaMemcpy(*d, t.data(), sizeof(TileRef) * t.size(), cudaMemcpyHostToDevice);
}

int upload_args(swb_batch *b) {
    if (!b->args_dirty) return SWB_OK;
    B_TRY(b, cudaMemcpyAsync(b->d_args, b->args.data(), b->args.size() * sizeof(StepArgs),
                             cudaMemcpyHostToDevice, b->stream));
    std::vector<StepArgs> fb;
    if (b->nt < 0) {
        fb = fallback_args(b);
        if (!b->d_args_fb) B_TRY(b, cudaMalloc((void **)&b->d_args_fb, sizeof(StepArgs) * b->count));
        B_TRY(b, cudaMemcpyAsync(b->d_args_fb, fb.data(), fb.size() * sizeof(StepArgs),
                                 cudaMemcpyHostToDevice, b->stream));
    }
    B_TRY(b, cudaStreamSynchronize(b->stream));
    b->args_dirty = false;
    b->invalidate();
    return SWB_OK;
}

// Strip geometry of every lattice (nt < 0: pair strips, which need FP32
// arithmetic and even Lx everywhere) and the tile tables.
int apply_geometry(swb_batch *b, int nt, int rows) {
    B_TRY(b, cudaStreamSynchronize(b->stream));
    b->nt = nt;
    b->rows = rows;
    for (int i = 0; i < b->count; ++i) {
        int h = rows < b->params[i].Ly ? rows : b->params[i].Ly;
        if (h < swb::kMinRows) h = swb::kMinRows;
        swb::set_geometry(b->args[i], nt, h);
    }
    const std::vector<TileRef> tiles = build_tiles(b->args);
    B_TRY(b, put_tiles(b, &b->d_tiles, &b->cap_tiles, tiles));
    b->ntiles = (int)tiles.size();
    if (nt < 0) {
        const std::vector<TileRef> fbt = build_tiles(fallback_args(b));
        B_TRY(b, put_tiles(b, &b->d_tiles_fb, &b->cap_tiles_fb, fbt));
        b->ntiles_fb = (int)fbt.size();
    }
    b->args_dirty = true;
    b->invalidate();
    return upload_args(b);
}

bool pair_possible(const swb_batch *b) {
    if (b->precision != SWB_F32 && b->precision != SWB_F16) return false;
    for (const swb_params &p : b->params)
        if (p.Lx % 2) return false;
    return true;
}

// n batched step launches (k = 0..n-1) and the advance kernel closing them.
// While a lattice is at its first iteration after its height was set
// (fresh_pending), swb_batch_step runs that iteration alone, so that the
// launches of a captured sequence are steady and the graph can be replayed
// at any time.
cudaError_t batch_sequence(swb_batch *b, int n, int grid) {
    cudaError_t e = cudaSuccess;
    bool gen = false, tau1 = true, pair = true, wave = false, rare = false;  // the general kernel if any lattice needs it
    for (const StepArgs &a : b->args) {
        gen = gen || swb::step_general(a);
        rare = rare || swb::step_rare(a);
        tau1 = tau1 && a.tau_is_one;
        pair = pair && swb::pair_form_ok(a);
        wave = wave || a.theta_mode == swb::THETA_WAVE;
    }
    for (int k = 0; k < n && e == cudaSuccess; ++k) {
        const bool steady = tau1 && !(b->fresh_pending && k == 0);
        if (b->nt < 0 && !(pair && steady))  // an iteration the pair form leaves out
            e = swb::launch_batch_step(b->precision, 64, gen, steady, b->d_args_fb, b->d_tiles_fb,
                                       b->ntiles_fb, grid, k, b->stream, rare);
        else if (b->nt < 0)
            e = swb::launch_batch_step(b->precision, b->nt, wave, steady, b->d_args, b->d_tiles,
                                       b->ntiles, grid, k, b->stream);
        else
            e = swb::launch_batch_step(b->precision, b->nt, gen, steady, b->d_args, b->d_tiles,
                                       b->ntiles, grid, k, b->stream, rare);
    }
    if (e == cudaSuccess && n > 0) e = swb::launch_batch_advance(b->d_args, b->count, n, b->stream);
    return e;
}

int launch_n(swb_batch *b, int n, int grid) {
    B_TRY(b, batch_sequence(b, n, grid));
    return SWB_OK;
}

// Autotuner: times real steps of a few strip geometries (one-column strips
// of 64 or 128 threads, and pair strips where every lattice allows them),
// each with a few CTA counts (persistent CTAs, k per SM, or one CTA per
// tile), and keeps the fastest.  Results do not depend on the choice (the
// per-cell arithmetic is the same and the measures are exact sums).
int autotune(swb_batch *b, long long &left) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    bool pair = true, wave = false;
    for (const StepArgs &a : b->args) {
        pair = pair && swb::pair_form_ok(a);
        wave = wave || a.theta_mode == swb::THETA_WAVE;
    }
    std::vector<std::array<int, 2>> geos = {{64, 32}, {64, 16}, {128, 16}};
    if (pair_possible(b) && pair) {
        geos.push_back({-64, 16});
        geos.push_back({-64, 32});
        geos.push_back({-64, 64});
        geos.push_back({-32, 16});
    }
    if (b->geometry_fixed) geos = {{b->nt, b->rows}};  // a geometry set by the caller
    const int probe = 2;
    struct Best {
        float ms = 1e30f;
        int nt = 0, rows = 0, grid = 0;
    } best;
    cudaEvent_t e0, e1;
    B_TRY(b, cudaEventCreate(&e0));
    B_TRY(b, cudaEventCreate(&e1));
    int rc = SWB_OK;
    for (auto &g : geos) {
        if (rc) break;
        if (g[0] != b->nt || g[1] != b->rows) {
            rc = apply_geometry(b, g[0], g[1]);
            if (rc) break;
        }
        const int occ = swb::batch_blocks_per_sm(b->precision, b->nt, wave);
        std::vector<int> grids = {b->ntiles, std::min(b->ntiles, sms * occ),
                                  std::min(b->ntiles, sms * std::max(1, occ / 2))};
        std::sort(grids.begin(), grids.end());
        grids.erase(std::unique(grids.begin(), grids.end()), grids.end());
        if (left < 1 + (long long)probe * (long long)grids.size()) break;
        rc = launch_n(b, 1, grids.back());  // loads the kernel (a real step)
        left -= 1;
        for (int gr : grids) {
            if (rc) break;
            cudaEventRecord(e0, b->stream);
            rc = launch_n(b, probe, gr);
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            left -= probe;
            if (ms < best.ms) best = {ms, b->nt, b->rows, gr};
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (best.nt == 0) {  // too few steps to probe: the default strips, persistent CTAs
        if (b->nt != swb::kBatchNT || b->rows != swb::kBatchRows) {
            rc = apply_geometry(b, swb::kBatchNT, swb::kBatchRows);
            if (rc) return rc;
        }
        b->grid = std::min(b->ntiles, sms * swb::batch_blocks_per_sm(b->precision, b->nt, wave));
    } else {
        if (best.nt != b->nt || best.rows != b->rows) {
            rc = apply_geometry(b, best.nt, best.rows);
            if (rc) return rc;
        }
        b->grid = best.grid;
    }
    b->tuned = true;
    return SWB_OK;
}

}  // namespace

extern "C" {

int swb_batch_create(const swb_params *params, int count, int precision, swb_batch **out) {
    if (!out || !params || count < 1) return swb::bfail(nullptr, SWB_ERR_ARG, "bad arguments");
    *out = nullptr;
    if (precision != SWB_F64 && precision != SWB_F32 && precision != SWB_F16)
        return swb::bfail(nullptr, SWB_ERR_ARG, "batch precision must be SWB_F64, SWB_F32 or SWB_F16");
    for (int i = 0; i < count; ++i) {
        const swb_params &p = params[i];
        if (p.Lx < 1 || p.Ly < 1 || 9LL * (((long long)p.Lx * p.Ly + 63) / 64 * 64) >= (1LL << 31) || !(p.tau > 0) ||
            p.n <= p.m || p.m < 1 || !(p.hmin > 0))
            return swb::bfail(nullptr, SWB_ERR_ARG, "invalid params for lattice " + std::to_string(i));
        if (!(p.kbt >= 0.0)) return swb::bfail(nullptr, SWB_ERR_ARG, "kbt must be >= 0");
    }
    swb_batch *b = new swb_batch();
    b->count = count;
    b->precision = precision;
    b->params.assign(params, params + count);
    size_t off = 0;
    long long maxN = 0;
    std::vector<size_t> offs;
    for (int i = 0; i < count; ++i) {
        LatticeLayout L = swb::lattice_layout(params[i], precision);
        b->layouts.push_back(L);
        offs.push_back(off);
        off += L.total;
        maxN = std::max<long long>(maxN, (long long)params[i].Lx * params[i].Ly);
    }
    auto bad = [&](int code) {
        std::string m = b->err;
        delete b;
        swb::b_err = m;
        swb::set_global_error(m.c_str());
        return code;
    };
#define BC_TRY(expr)                                                                       \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            b->err = std::string(#expr) + ": " + cudaGetErrorString(e_);                   \
            return bad(e_ == cudaErrorMemoryAllocation ? SWB_ERR_OOM : SWB_ERR_CUDA);      \
        }                                                                                  \
    } while (0)
    BC_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    b->slab_bytes = off;
    BC_TRY(cudaMalloc((void **)&b->slab, off));
    BC_TRY(cudaMalloc((void **)&b->staging, (size_t)maxN * 8));
    for (int i = 0; i < count; ++i) {
        StepArgs a = swb::lattice_args(params[i], precision, b->slab + offs[i], b->layouts[i],
                                       b->nt, b->rows);
        a.seed = (unsigned long long)i;  // thermal noise stream of lattice i
        b->args.push_back(a);
        BC_TRY(swb::lattice_init(a, precision, b->layouts[i], nullptr, b->stream));
    }
    const std::vector<TileRef> tiles = build_tiles(b->args);
    b->fields_current.assign(count, 1);
    b->ntiles = (int)tiles.size();
    BC_TRY(cudaMalloc((void **)&b->d_args, sizeof(StepArgs) * count));
    BC_TRY(cudaMalloc((void **)&b->d_flags, sizeof(int) * count));
    BC_TRY(cudaMalloc((void **)&b->d_tiles, sizeof(TileRef) * tiles.size()));
    BC_TRY(cudaMemcpy(b->d_tiles, tiles.data(), sizeof(TileRef) * tiles.size(), cudaMemcpyHostToDevice));
    b->cap_tiles = tiles.size();
#undef BC_TRY
    *out = b;
    return SWB_OK;
}

int swb_batch_destroy(swb_batch *b) {
    delete b;
    return SWB_OK;
}

int swb_batch_set_height(swb_batch *b, int idx, const double *host) {
    if (!b || !host || idx < 0 || idx >= b->count) return swb::bfail(b ? &b->err : nullptr, SWB_ERR_ARG, "bad arguments");
    StepArgs &a = b->args[idx];
    if (!b->fields_current[idx]) {  // keep the velocities current
        B_TRY(b, swb::launch_moments(b->precision, a, b->stream));
    }
    B_TRY(b, swb::lattice_upload_height(a, b->precision, host, b->staging, b->stream));
    B_TRY(b, cudaStreamSynchronize(b->stream));
    b->fields_current[idx] = 1;
    b->fresh_pending = true;
    return SWB_OK;
}

int swb_batch_get_height(swb_batch *b, int idx, double *host) {
    if (!b || !host || idx < 0 || idx >= b->count) return swb::bfail(b ? &b->err : nullptr, SWB_ERR_ARG, "bad arguments");
    B_TRY(b, swb::lattice_download_height(b->args[idx], b->precision, b->fields_current[idx], host, b->stream));
    b->fields_current[idx] = 1;
    return SWB_OK;
}

int swb_batch_set_theta_wave(swb_batch *b, int idx, double theta0, double dtheta, double v) {
    if (!b || idx < 0 || idx >= b->count) return swb::bfail(b ? &b->err : nullptr, SWB_ERR_ARG, "bad arguments");
    swb::set_wave(b->args[idx], theta0, dtheta, v);
    b->args_dirty = true;
    return SWB_OK;
}

int swb_batch_step(swb_batch *b, int64_t nsteps) {
    if (!b || nsteps < 0) return swb::bfail(b ? &b->err : nullptr, SWB_ERR_ARG, "bad arguments");
    if (nsteps == 0) return SWB_OK;
    int rc = upload_args(b);
    if (rc) return rc;
    long long left = nsteps;
    if (b->fresh_pending) {
        rc = launch_n(b, 1, b->grid > 0 ? b->grid : b->ntiles);
        if (rc) return rc;
        b->fresh_pending = false;
        left -= 1;
    }
    if (!b->tuned && left > 0) {
        rc = autotune(b, left);
        if (rc) return rc;
    }
    if (left >= b->steps_per_graph) {
        if (!b->gvalid) {
            cudaGraph_t g = nullptr;
            B_TRY(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t le = batch_sequence(b, b->steps_per_graph, b->grid);
            swb::count_launches(0ULL - (unsigned long long)(b->steps_per_graph + 1));
            cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
            if (le != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return swb::bfail(&b->err, SWB_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(le));
            }
            B_TRY(b, ce);
            cudaError_t ie = cudaGraphInstantiate(&b->gexec, g, 0);
            cudaGraphDestroy(g);
            B_TRY(b, ie);
            b->gvalid = true;
        }
        while (left >= b->steps_per_graph) {
            B_TRY(b, cudaGraphLaunch(b->gexec, b->stream));
            swb::count_launches(b->steps_per_graph + 1);
            left -= b->steps_per_graph;
        }
    }
    rc = launch_n(b, (int)left, b->grid);
    if (rc) return rc;
    b->steps += nsteps;
    std::fill(b->fields_current.begin(), b->fields_current.end(), 0);
    return SWB_OK;
}

int swb_batch_sync(swb_batch *b) {
    if (!b) return swb::bfail(nullptr, SWB_ERR_ARG, "batch is NULL");
    B_TRY(b, cudaStreamSynchronize(b->stream));
    if (b->args_dirty) return SWB_OK;  // no step since the arguments changed
    swb::count_launches(1);
    swb::gather_nan<<<(b->count + 255) / 256, 256, 0, b->stream>>>(b->d_args, b->count, b->d_flags);
    B_TRY(b, cudaGetLastError());
    std::vector<int> flags(b->count);
    B_TRY(b, cudaMemcpyAsync(flags.data(), b->d_flags, sizeof(int) * b->count,
                             cudaMemcpyDeviceToHost, b->stream));
    B_TRY(b, cudaStreamSynchronize(b->stream));
    for (int i = 0; i < b->count; ++i)
        if (flags[i])
            return swb::bfail(&b->err, SWB_ERR_NAN,
                              "non-finite height in lattice " + std::to_string(i));
    return SWB_OK;
}

int swb_batch_set_geometry(swb_batch *b, int nt, int rows) {
    if (!b || rows < swb::kMinRows || rows > swb::kMaxRows ||
        (nt != 64 && nt != 128 && nt != 256 && !swb::pair_geometry(nt)))
        return swb::bfail(b ? &b->err : nullptr, SWB_ERR_ARG,
                          "batch geometry: nt must be 64, 128, 256 or -32, -64, -128 (pair "
                          "strips) and 2 <= rows <= 512");
    if (nt < 0 && !pair_possible(b))
        return swb::bfail(&b->err, SWB_ERR_UNSUPPORTED,
                          "batch pair strips: FP32 or FP16 storage and even Lx in every lattice");
    const int rc = apply_geometry(b, nt, rows);
    if (rc) return rc;
    b->geometry_fixed = true;
    b->tuned = false;  // re-pick the CTA count (the tuner keeps this geometry)
    return SWB_OK;
}

int swb_batch_geometry(swb_batch *b, int *nt, int *rows, int *grid) {
    if (!b) return swb::bfail(nullptr, SWB_ERR_ARG, "batch is NULL");
    if (nt) *nt = b->nt;
    if (rows) *rows = b->rows;
    if (grid) *grid = b->grid;
    return SWB_OK;
}

int swb_batch_tile(swb_batch *b, int *tile_x, int *tile_y, int *steps_per_graph) {
    if (!b) return swb::bfail(nullptr, SWB_ERR_ARG, "batch is NULL");
    if (tile_x) *tile_x = b->tuned ? (b->nt < 0 ? -2 * b->nt - 4 : b->nt - 4) : 0;
    if (tile_y) *tile_y = b->tuned ? b->rows : 0;
    if (steps_per_graph) *steps_per_graph = b->tuned ? b->steps_per_graph : 0;
    return SWB_OK;
}

}  // extern "C"
