// swb_internal.h -- definitions shared by the CUDA translation units of
// libswalbe_gb300.so.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/swalbe_gb300.h"

namespace swb {

// Fused-step tile: TX x TY interior cells per CTA, NTX x NTY threads.
// The pressure needs h at radius 1, the force p at radius 1, so a tile stages
// h on (TX+4) x (TY+4) and p on (TX+2) x (TY+2) in shared memory.
constexpr int kTX = 32;
constexpr int kTY = 16;
constexpr int kThreads = 256;

// Measure partials per block: mass, wetted, hmax, hmin, area, cos-sum.
constexpr int kNPart = 6;
// Capacity of the per-step measure ring of a single state (records).
constexpr int kRecCap = 65536;

// Device-side control block of one lattice.  The step counter lives on the
// device so that a captured CUDA graph can be replayed: each launch reads
// `step`, and the last CTA to finish (ticket) advances it.
struct Control {
    long long step;          // iterations completed
    unsigned int ticket;     // CTAs finished in the current launch
    int fresh;               // 1: next step takes h, u from the fields
    int nan_flag;            // set when a non-finite height is seen
    int pad0;
    double mass_target;      // FP32/FP16 mass correction: mass to hold
    double mass_last;        // mass of the height at the start of the last step
    double corr_last;        // correction added per cell in the last step
    long long rec_head;      // records written (monotone)
};

struct Record {              // one time_loop iteration
    long long t;
    double mass;
    double wetted;
    double hmax, hmin;
    double area;
    double cos_sum;
};

enum ThetaMode { THETA_SCALAR = 0, THETA_FIELD = 1, THETA_WAVE = 2 };

// Everything one fused step of one lattice needs.  Constant across steps,
// so launches can be captured in a CUDA graph.
struct StepArgs {
    int Lx, Ly;
    long long pitch;          // elements between population planes
    void *fa, *fb;            // post-collision populations, double buffered
    void *hF, *uxF, *uyF;     // macroscopic fields (compute type)
    const void *kapF;         // θ-field mode: kappa prefactor per cell
    const void *cosF;         // θ-field mode: cospi(θ) per cell
    double gamma, hmin, hcrit, kap, delta, mu, g, invtau, omeg;
    int n, m;
    int tau_is_one;
    int theta_mode;
    double theta0, dtheta, wave_v, cos_theta;
    int incl, incl_loop_time;
    double ax, ay, incl_fixed;    // incl_fixed: smoothing factor for fixed t
    long long incl_tstart, incl_tsmooth;
    int meas_mask;
    double hthresh;
    int mass_corr;
    double *partials;         // [blocks][kNPart]
    Record *records;          // ring of rec_cap records (may be null if meas_mask == 0)
    int rec_cap;
    Control *ctl;
    int tiles_x, tiles_y;     // tile grid of this lattice
};

// Entry in the packed tile table of a batch.
struct TileRef {
    int lattice;
    int tx, ty;
};

// Error text returned by swb_last_error(NULL) on the calling thread.
void set_global_error(const char *msg);
// Counts kernel launches issued by the library (swb_launch_count).
void count_launches(unsigned long long n);

// ---- launchers (defined in the .cu files) ----
// precision: SWB_F64 (swb_step_f64.cu) / SWB_F32, SWB_F16 (swb_step_f32.cu)
cudaError_t launch_fused_step(int precision, const StepArgs &a, cudaStream_t st);
cudaError_t launch_moments(int precision, const StepArgs &a, cudaStream_t st);
cudaError_t launch_fout(int precision, const StepArgs &a, double *out, cudaStream_t st);
cudaError_t launch_pressure_now(int precision, const StepArgs &a, double *out, cudaStream_t st);
cudaError_t launch_batch_step(int precision, const StepArgs *d_args, const TileRef *d_tiles,
                              int ntiles, int grid, cudaStream_t st);
int batch_blocks_per_sm(int precision);
cudaError_t launch_fused_step_f64(const StepArgs &a, cudaStream_t st);
cudaError_t launch_moments_f64(const StepArgs &a, cudaStream_t st);
cudaError_t launch_fout_f64(const StepArgs &a, double *out, cudaStream_t st);
cudaError_t launch_pressure_now_f64(const StepArgs &a, double *out, cudaStream_t st);
cudaError_t launch_batch_step_f64(const StepArgs *d_args, const TileRef *d_tiles, int ntiles,
                                  int grid, cudaStream_t st);
cudaError_t launch_fused_step_f32(int precision, const StepArgs &a, cudaStream_t st);
cudaError_t launch_moments_f32(int precision, const StepArgs &a, cudaStream_t st);
cudaError_t launch_fout_f32(int precision, const StepArgs &a, double *out, cudaStream_t st);
cudaError_t launch_pressure_now_f32(int precision, const StepArgs &a, double *out,
                                    cudaStream_t st);
cudaError_t launch_batch_step_f32(int precision, const StepArgs *d_args, const TileRef *d_tiles,
                                  int ntiles, int grid, cudaStream_t st);
int batch_blocks_per_sm_f64();
int batch_blocks_per_sm_f32(int precision);

// plain FP64 per-op kernels (reference operation order)
struct PlainState {
    int Lx, Ly;
    long long N;
    double *fout, *ftemp, *feq;
    double *h, *ux, *uy, *vsq, *p, *Fx, *Fy, *sx, *sy, *hgx, *hgy;
};
cudaError_t plain_filmpressure(const PlainState &s, const double *kapF, double kap, double gamma,
                               int n, int m, double hmin, double hcrit, cudaStream_t st);
cudaError_t plain_hgradp(const PlainState &s, cudaStream_t st);
cudaError_t plain_slippage(const PlainState &s, double delta, double mu, cudaStream_t st);
cudaError_t plain_force_sum(const PlainState &s, cudaStream_t st);
cudaError_t plain_inclination(const PlainState &s, double ax, double ay, double fac,
                              cudaStream_t st);
cudaError_t plain_equilibrium(const PlainState &s, double g, cudaStream_t st);
cudaError_t plain_collide(const PlainState &s, double omeg, double invtau, cudaStream_t st);
cudaError_t plain_stream(const PlainState &s, cudaStream_t st);
cudaError_t plain_moments(const PlainState &s, cudaStream_t st);

// Measures of a Float64/float height field: block partials + last-block
// reduction into `rec` (device).  `scratch` holds blocks*kNPart doubles,
// `ticket` one unsigned int (zero on entry, left zero).
int measure_blocks(long long N);
cudaError_t launch_measure(const void *h, int is_double, int Lx, int Ly, double hthresh,
                           const void *cosF, double cos_theta, double *scratch,
                           unsigned int *ticket, Record *rec, long long t, cudaStream_t st);

}  // namespace swb
