// swb_internal.h -- definitions shared by the CUDA translation units of
// libswalbe_gb300.so.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/swalbe_gb300.h"

namespace swb {

// Fused step geometry: a CTA of NT threads (64, 128 or 256) owns a strip of
// NT - 4 columns and H rows (kMinRows..kMaxRows).  Partial-measure buffers
// are sized for the finest decomposition (NT = 64, H = kMinRows).
constexpr int kMinRows = 2;
constexpr int kMaxRows = 512;
inline long long max_tiles(int Lx, int Ly) {  // per parity slot: strips or 2D tiles
    const long long strips = (long long)((Lx + 59) / 60) * ((Ly + kMinRows - 1) / kMinRows);
    const long long tiles = (long long)((Lx + 31) / 32) * ((Ly + 15) / 16);
    return strips > tiles ? strips : tiles;
}
// CTA width of batched and served lattices (all share one launch; 64 was
// the fastest on GB300 for the 128^2..1024x256 ensemble).
constexpr int kBatchNT = 64;
// Default geometry for a lattice.  *nt on entry: 0 to choose the width too,
// or a width (64, 128, 256) to keep; *h: rows per strip.
void default_geometry(int Lx, int Ly, int precision, int *nt, int *h);

// Measure partials per block: mass, wetted, hmax, hmin, area, cos-sum.
constexpr int kNPart = 6;
// Integer measure accumulators of FP32-arithmetic states: fixed-point mass,
// area and cos-sum (units of 2^-32 per cell), wetted count, and hmax / hmin
// as order-preserving keys (0: no cell), each in kAccLanes lanes.
enum { kAccMass, kAccWet, kAccHmax, kAccHmin, kAccArea, kAccCos, kAccFields };
constexpr int kAccLanes = 32;
// Capacity of the per-step measure ring of a single state (records).
constexpr int kRecCap = SWB_RECORD_CAPACITY;

// Device-side control block of one lattice.  A launch sequence of n steps
// is n step kernels (launch index k = 0..n-1, time_loop iteration
// t = step_base + k + 1) followed by an advance kernel that reduces the last
// step's measures and adds n to step_base; a captured CUDA graph replays such
// a sequence.  No CTA ever waits for another: the measures of iteration t are
// reduced by an extra CTA of launch t+1 (or by the advance kernel).
struct Control {
    long long step_base;     // iterations completed before the current sequence
    long long fresh_step;    // iteration that takes h, u from the fields (0: none)
    int nan_flag;            // set when a non-finite height is seen
    int pad0;
    double mass_target;      // FP16 mass correction: mass to hold
    double corr[2];          // correction per cell for iteration t in slot t & 1
    long long rec_head;      // records written (monotone)
    int bar_err;             // a grid-barrier wait of the multi-step kernel gave up
    int pad1;
    // FP32-arithmetic states: the per-iteration measures, accumulated by
    // integer atomics of every CTA into one of kAccLanes lanes (slot t & 1),
    // read and cleared by the reducer of iteration t (order-free, exact)
    unsigned long long acc[2][kAccFields][kAccLanes];
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
    int mass_fixed;           // FP32 arithmetic: block masses are fixed-point sums (kMassUnit)
    double *partials;         // [2][max_tiles][kNPart]: slot by iteration parity
    Record *records;          // ring of rec_cap records (may be null if meas_mask == 0)
    int rec_cap;
    Control *ctl;
    int part_stride;          // partial slots per parity (max_tiles of the lattice)
    int tiles_x, tiles_y;     // strip grid of this lattice: ceil(Lx/(NT-4)) x ceil(Ly/H)
    int march_nt, march_h;    // threads per CTA (strip width + 4) and rows per strip,
                              // or kTileGeom and kT2Y rows: 2D tiles of 32 x 16 cells
    unsigned int *bar;        // grid-barrier words of the multi-step kernel (kBarWords)
    int thermal;              // kbt > 0: thermal! forces (src/forcing.jl:297-320)
    double k6;                // ((2 kbt) mu) 6, the numerator's constant factor
    unsigned long long seed;  // noise stream: Philox key
    // moving substrate (θ field mode): the field moves by (shift_dx, shift_dy)
    // cells after every shift_tmove iterations counted from shift_t0
    long long shift_t0;
    int shift_tmove, shift_dx, shift_dy;
    // batches and the server: iterations after which the lattice stops (its
    // strips are skipped and its step counter stays there); a served
    // request's step count, so that ticks need not end when it does
    long long stop_at;
};

// Offset of the moving θ field at iteration t (1-based): it has moved
// k = (t - 1 - t0) / tmove times (move_substrate! runs at the end of every
// tmove-th iteration, scripts/Moving_wettability_structs.jl:139-152), and
// circshift by (dx, dy) means field(i, j) = original(i - k dx, j - k dy).
__host__ __device__ inline void substrate_shift(const StepArgs &a, long long t, int *sx, int *sy) {
    *sx = 0;
    *sy = 0;
    if (a.shift_tmove <= 0 || t - 1 - a.shift_t0 < a.shift_tmove) return;
    const long long k = (t - 1 - a.shift_t0) / a.shift_tmove;
    *sx = (int)((k % a.Lx) * a.shift_dx % a.Lx);
    *sy = (int)((k % a.Ly) * a.shift_dy % a.Ly);
}

// Geometry value of the 2D-tile form: CTAs of 256 threads own 32 x 16 cells.
constexpr int kTileGeom = 32;
constexpr int kTileX = 32, kTileY = 16, kTileThreads = 256;

// Pair strips (FP32 arithmetic, even Lx): geometry value -NT, CTAs of NT
// threads (32, 64 or 128) with two columns per thread own strips of
// 2 NT - 4 columns.  Only the common steady τ = 1 step has this form; the
// other iterations of such a state run as one-column strips of 64 threads
// with the same rows (pair_fallback).
inline bool pair_geometry(int nt) { return nt == -32 || nt == -64 || nt == -128; }
// Resident tiles (a multi-step launch form, SWB_F32 / SWB_F16): geometry
// value kResGeom, tiles of kResTW columns x h rows (1 <= h <= kResMaxTH), one
// CTA of kResThreads threads per tile holding the tile's populations in
// shared memory, all CTAs co-resident.  Only the common steady τ = 1 step
// has this form; other iterations run on strips (strip_fallback).
constexpr int kResGeom = 33;
// kResGeom2: the same with CTAs of kResThreads / 2 threads, two per SM (one
// CTA's phases run while the other waits at a barrier; tiles half as tall).
constexpr int kResGeom2 = 34;
constexpr int kResTW = 64, kResMaxTH = 40, kResThreads = 512;
inline bool resident_geometry(int nt) { return nt == kResGeom || nt == kResGeom2; }

inline void set_geometry(StepArgs &a, int nt, int h) {
    a.march_nt = nt;
    if (nt == kTileGeom) {
        a.march_h = kTileY;
        a.tiles_x = (a.Lx + kTileX - 1) / kTileX;
        a.tiles_y = (a.Ly + kTileY - 1) / kTileY;
        return;
    }
    if (resident_geometry(nt)) {
        a.march_h = h;
        a.tiles_x = (a.Lx + kResTW - 1) / kResTW;
        a.tiles_y = (a.Ly + h - 1) / h;
        return;
    }
    a.march_h = h;
    const int w = nt < 0 ? -2 * nt - 4 : nt - 4;  // strip width in columns
    a.tiles_x = (a.Lx + w - 1) / w;
    a.tiles_y = (a.Ly + h - 1) / h;
}
// Threads per CTA of a geometry.
inline int geometry_threads(int nt) {
    return nt == kTileGeom ? kTileThreads
                           : (nt == kResGeom ? kResThreads
                                             : (nt == kResGeom2 ? kResThreads / 2 : (nt < 0 ? -nt : nt)));
}
// The one-column strips (64 threads, the same rows) that run the iterations
// the pair-strip and resident-tile forms leave out.
inline StepArgs strip_fallback(const StepArgs &a) {
    StepArgs b = a;
    set_geometry(b, 64, a.march_h < kMinRows ? kMinRows : a.march_h);
    return b;
}
inline StepArgs pair_fallback(const StepArgs &a) { return strip_fallback(a); }

// Entry in the packed tile table of a batch (tx = -1: the lattice's reducer).
struct TileRef {
    int lattice;
    int tx, ty;
};

// Whether a lattice's step needs the general kernel (θ field or wave,
// thermal noise, inclination) rather than the common one.
inline bool step_general(const StepArgs &a) {
    return a.thermal || a.incl || a.theta_mode != THETA_SCALAR;
}
// Whether `a` needs the general kernel for more than the θ wave (θ field,
// thermal noise, inclination); steady iterations of wave-only lattices have
// a WAVE variant of the common kernels.
inline bool step_rare(const StepArgs &a) {
    return a.thermal || a.incl || a.theta_mode == THETA_FIELD;
}
// Whether a steady iteration of `a` has a pair-strip kernel: τ = 1, no rare
// forces, scalar θ or the θ wave (a per-column κ; the pair kernel's WAVE
// variant).
inline bool pair_form_ok(const StepArgs &a) {
    return a.tau_is_one && !a.thermal && !a.incl && a.theta_mode != THETA_FIELD;
}

// Whether the step kernels of a lattice produce per-step partial measures.
__host__ __device__ inline bool needs_partials(const StepArgs &a) { return a.meas_mask != 0 || a.mass_corr != 0; }

// Launch overlap of consecutive step kernels (programmatic dependent
// launch): on unless the environment sets SWB_LAUNCH_OVERLAP=0.  Read once.
bool launch_overlap();

// Error text returned by swb_last_error(NULL) on the calling thread.
void set_global_error(const char *msg);
// Counts kernel launches issued by the library (swb_launch_count).
void count_launches(unsigned long long n);
// Launches counted so far (to account for kernels captured into graphs).
unsigned long long launches_so_far();

// ---- launchers (defined in the .cu files) ----
// precision: SWB_F64 (swb_step_f64.cu) / SWB_F32, SWB_F16 (swb_step_f32.cu)
// Step kernel number k of a sequence, and the sequence's closing advance
// kernel (precision independent, defined in swb_step_f64.cu).
cudaError_t launch_fused_step(int precision, const StepArgs &a, int k, bool steady, cudaStream_t st);
cudaError_t launch_advance(const StepArgs &a, int n, cudaStream_t st);
cudaError_t launch_batch_advance(const StepArgs *d_args, int count, int n, cudaStream_t st);
// CTAs of step launch k of a single lattice: its strips, plus the reducer.
inline int step_grid(const StepArgs &a, int k) {
    return a.tiles_x * a.tiles_y + ((needs_partials(a) && k > 0) ? 1 : 0);
}
// Multi-step kernel: n iterations of a single F32/F16 lattice in one
// cooperative launch of `grid` CTAs (all co-resident), a grid barrier
// between iterations; closes the sequence itself (no advance kernel).
cudaError_t launch_fused_run(int precision, const StepArgs &a, int n, int grid, cudaStream_t st);
// CTAs of width nt one SM holds for the multi-step kernel (0: unsupported).
int fused_run_blocks_per_sm(int precision, int nt);
// Grid barrier of the multi-step kernel: a top counter, kBarGroups group
// counters and kBarGroups generation words, each on its own 128-byte line.
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ULL;  // one wait
constexpr unsigned int kBarGroups = 32;
constexpr unsigned int kBarStride = 32;  // words
constexpr unsigned int kBarWords = kBarStride * (1 + 2 * kBarGroups);
cudaError_t launch_moments(int precision, const StepArgs &a, cudaStream_t st);
cudaError_t launch_fout(int precision, const StepArgs &a, double *out, cudaStream_t st);
cudaError_t launch_pressure_now(int precision, const StepArgs &a, double *out, cudaStream_t st);
// thermal! forces of the current height field for iteration t (fx, fy: N doubles).
cudaError_t launch_thermal_field(int precision, const StepArgs &a, long long t, double *fx,
                                 double *fy, cudaStream_t st);
cudaError_t launch_thermal_field_f64(const StepArgs &a, long long t, double *fx, double *fy,
                                     cudaStream_t st);
cudaError_t launch_thermal_field_f32(int precision, const StepArgs &a, long long t, double *fx,
                                     double *fy, cudaStream_t st);
// gen: some lattice of the batch needs the general kernel (step_general);
// with pair strips (nt < 0): some lattice has the θ wave.
// steady_tau1: no lattice is at its first iteration after its fields were
// set and every lattice has τ = 1 (the steady batch form may run it)
cudaError_t launch_batch_step(int precision, int nt, bool gen, bool steady_tau1,
                              const StepArgs *d_args, const TileRef *d_tiles, int ntiles,
                              int grid, int k, cudaStream_t st, bool rare = true);
int batch_blocks_per_sm(int precision, int nt, bool wave = false);
cudaError_t launch_fused_step_f64(const StepArgs &a, int k, cudaStream_t st);
cudaError_t launch_moments_f64(const StepArgs &a, cudaStream_t st);
cudaError_t launch_fout_f64(const StepArgs &a, double *out, cudaStream_t st);
cudaError_t launch_pressure_now_f64(const StepArgs &a, double *out, cudaStream_t st);
cudaError_t launch_batch_step_f64(int nt, bool gen, const StepArgs *d_args, const TileRef *d_tiles,
                                  int ntiles, int grid, int k, cudaStream_t st);
// steady: the iteration is not the first after the fields were set (the
// steady kernel forms may run it)
cudaError_t launch_fused_step_f32(int precision, const StepArgs &a, int k, bool steady,
                                  cudaStream_t st);
cudaError_t launch_moments_f32(int precision, const StepArgs &a, cudaStream_t st);
cudaError_t launch_fout_f32(int precision, const StepArgs &a, double *out, cudaStream_t st);
cudaError_t launch_pressure_now_f32(int precision, const StepArgs &a, double *out,
                                    cudaStream_t st);
// rare: some lattice needs the general kernel for more than the θ wave
// (step_rare); otherwise steady τ = 1 launches of wave lattices take the
// WAVE variant of the steady kernel.
cudaError_t launch_batch_step_f32(int precision, int nt, bool gen, bool steady_tau1,
                                  const StepArgs *d_args, const TileRef *d_tiles, int ntiles,
                                  int grid, int k, cudaStream_t st, bool rare = true);
int batch_blocks_per_sm_f64(int nt);
// Resident tiles: dynamic shared memory of a tile of h rows, CTAs per SM
// that hold it (0: not possible), and n iterations in one cooperative launch
// of tiles_x * tiles_y CTAs (closes the sequence itself).
size_t resident_smem_bytes(int h, int nt = kResGeom);
int resident_blocks_per_sm(int precision, int h, int nt = kResGeom);
cudaError_t launch_resident_run(int precision, const StepArgs &a, int n, cudaStream_t st);
// Whether iterations of `a` may run as resident tiles (the common steady
// τ = 1 step with scalar θ of an FP32-arithmetic lattice).
inline bool resident_ok(const StepArgs &a) { return a.tau_is_one && !step_general(a); }
// Resident CTAs per SM of the pair-strip kernel (FP32 / FP16 storage).
int pair_blocks_per_sm(int precision, int nt);
// Rows per pair strip for a lattice: the strip march takes about the same
// time in every CTA, so a launch lasts (waves of resident CTAs) x (rows + 4
// halo rows); the rule takes the height that minimises that product.
int pair_rows(int Lx, int Ly, int precision, int nt);
int batch_blocks_per_sm_f32(int precision, int nt, bool wave = false);

// plain FP64 per-op kernels (reference operation order)
struct PlainState {
    int Lx, Ly;
    long long N;
    double *fout, *ftemp, *feq;
    double *h, *ux, *uy, *vsq, *p, *Fx, *Fy, *sx, *sy, *hgx, *hgy;
};
cudaError_t plain_filmpressure(const PlainState &s, const double *kapF, double kap, double gamma,
                               int n, int m, double hmin, double hcrit, int sx, int sy,
                               cudaStream_t st);
cudaError_t plain_hgradp(const PlainState &s, cudaStream_t st);
cudaError_t plain_slippage(const PlainState &s, double delta, double mu, cudaStream_t st);
cudaError_t plain_force_sum(const PlainState &s, cudaStream_t st);
cudaError_t plain_thermal(const PlainState &s, double k6, double delta, unsigned long long seed,
                          long long t, cudaStream_t st);
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
// Where cos θ of a wetted cell comes from (surfacearea!'s energy term): the
// scalar cos_theta, a θ field's cospi values (cosF, the height's type) moved
// by (sx, sy) cells, or the θ wave θ0 + Δθ sinpi(2 (x - v t) / Lx) at
// iteration t, evaluated like the fused step does.
struct CosSrc {
    int mode;  // ThetaMode
    const void *cosF;
    int sx, sy;
    double cos_theta;
    double theta0, dtheta, wave_v;
    long long t;
};
cudaError_t launch_measure(const void *h, int is_double, int Lx, int Ly, double hthresh,
                           const CosSrc &cs, double *scratch, unsigned int *ticket, Record *rec,
                           long long t, cudaStream_t st);
// Scalar θ (cosF null) or a fixed θ field.
cudaError_t launch_measure(const void *h, int is_double, int Lx, int Ly, double hthresh,
                           const void *cosF, double cos_theta, double *scratch,
                           unsigned int *ticket, Record *rec, long long t, cudaStream_t st);

}  // namespace swb
