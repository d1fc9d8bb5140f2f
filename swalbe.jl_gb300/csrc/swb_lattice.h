// swb_lattice.h -- device memory of one lattice inside a batch or a server:
// layout, initialisation and host<->device field transfer.  Internal.
#pragma once
#include <cuda_fp16.h>

#include <cmath>
#include <string>
#include <vector>

#include "swb_internal.h"

namespace swb {

double host_cospi_shared(double x);
double host_kappa_shared(double theta, int n, int m, double hmin);

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
inline long long pitch_for(long long N) { return (N + 63) / 64 * 64; }
inline int real_bytes_of(int precision) { return precision == SWB_F64 ? 8 : 4; }
inline size_t fbuf_bytes_of(int precision, long long pitch) {
    switch (precision) {
        case SWB_F64: return (size_t)9 * pitch * 8;
        case SWB_F32: return (size_t)9 * pitch * 4;
        default: return (size_t)pitch * 4 + (size_t)8 * pitch * 2;
    }
}

// Byte offsets of one lattice's buffers inside a contiguous block.
struct LatticeLayout {
    size_t fa, fb, h, ux, uy, partials, ctl, total;
};

inline LatticeLayout lattice_layout(const swb_params &p, int precision) {
    const long long N = (long long)p.Lx * p.Ly, pitch = pitch_for(N);
    const long long tiles = max_tiles(p.Lx, p.Ly);
    LatticeLayout L{};
    size_t o = 0;
    const size_t fb = align256(fbuf_bytes_of(precision, pitch));
    const size_t fld = align256((size_t)N * real_bytes_of(precision));
    L.fa = o; o += fb;
    L.fb = o; o += fb;
    L.h = o; o += fld;
    L.ux = o; o += fld;
    L.uy = o; o += fld;
    L.partials = o; o += align256((size_t)2 * tiles * kNPart * 8);
    L.ctl = o; o += align256(sizeof(Control));
    L.total = o;
    return L;
}

// Strip rows of batched and served lattices: the batch has parallelism from
// its many lattices, so strips can be tall (fewer halo rows re-pulled; on
// GB300 the ensemble ran 26 GLUPS at 124x4 strips, 45 GLUPS at 60x32).
constexpr int kBatchRows = 32;

// Step arguments of a lattice whose buffers start at `base`; strips of
// nt threads and `rows` rows (capped at the lattice height).
inline StepArgs lattice_args(const swb_params &p, int precision, char *base, const LatticeLayout &L,
                             int nt = kBatchNT, int rows = kBatchRows) {
    StepArgs a{};
    a.Lx = p.Lx;
    a.Ly = p.Ly;
    a.pitch = pitch_for((long long)p.Lx * p.Ly);
    a.fa = base + L.fa;
    a.fb = base + L.fb;
    a.hF = base + L.h;
    a.uxF = base + L.ux;
    a.uyF = base + L.uy;
    a.partials = (double *)(base + L.partials);
    a.part_stride = (int)max_tiles(p.Lx, p.Ly);
    a.ctl = (Control *)(base + L.ctl);
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
    a.theta_mode = THETA_SCALAR;
    a.kap = host_kappa_shared(p.theta, p.n, p.m, p.hmin);
    a.cos_theta = host_cospi_shared(p.theta);
    int h = rows < p.Ly ? rows : p.Ly;  // one CTA width serves every lattice of a batch
    if (h < kMinRows) h = kMinRows;
    set_geometry(a, nt, h);
    a.hthresh = 0.055;
    a.thermal = p.kbt > 0.0 ? 1 : 0;
    a.k6 = ((2.0 * p.kbt) * p.mu) * 6.0;  // src/forcing.jl:300-302, left to right
    a.seed = 0;
    a.mass_fixed = (precision == SWB_F32 || precision == SWB_F16) ? 1 : 0;
    a.mass_corr = (precision == SWB_F16) ? 1 : 0;
    a.records = nullptr;
    a.rec_cap = 0;
    a.meas_mask = 0;
    a.stop_at = 0x7fffffffffffffffLL;  // runs until told otherwise
    return a;
}

inline void set_wave(StepArgs &a, double theta0, double dtheta, double v) {
    if (dtheta == 0.0 && v == 0.0) {
        a.theta_mode = THETA_SCALAR;
        a.kap = host_kappa_shared(theta0, a.n, a.m, a.hmin);
        a.cos_theta = host_cospi_shared(theta0);
    } else {
        a.theta_mode = THETA_WAVE;
        a.theta0 = theta0;
        a.dtheta = dtheta;
        a.wave_v = v;
    }
}

// Zero populations, h = 1 (or h0), u = 0, fresh control block.  Async on st.
cudaError_t lattice_init(const StepArgs &a, int precision, const LatticeLayout &L,
                         const double *h0_host, cudaStream_t st);
// Upload a host Float64 height into the field (converted to the compute type)
// and mark the lattice fresh.  Async on st; `staging` must stay alive until
// the stream passes this point (pinned or synchronised by the caller).
cudaError_t lattice_upload_height(const StepArgs &a, int precision, const double *h_host,
                                  void *staging, cudaStream_t st);
// Height of the lattice into host memory (runs the moments kernel first
// unless the fields are the current source).  Synchronises st.
cudaError_t lattice_download_height(const StepArgs &a, int precision, bool fields_current,
                                    double *h_host, cudaStream_t st);

}  // namespace swb
