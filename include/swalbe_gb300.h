/*
 * swalbe_gb300.h -- C ABI of the GB300-native thin-film lattice Boltzmann step.
 *
 * A drop-in for the time loop of Swalbe.jl.  The reference has no FFI: its
 * extension point is Julia multiple dispatch on `LBM_state_2D` plus the
 * `device` string of `Sys` (src/initialize.jl:4, 491-572).  Each entry point
 * below names the reference function it replaces (paths relative to the
 * Swalbe.jl project root).  The Julia binding is in
 * swalbe.jl_gb300/julia/SwalbeGB300.jl, the Python binding in
 * swalbe.jl_gb300/swalbe_gb300/.
 *
 * Conventions
 *  - Host arrays are Float64, column-major with x (i) fastest, exactly the
 *    memory of a Julia `Matrix{Float64}(undef, Lx, Ly)`; they are read or
 *    written only during the call.
 *  - Every function returns an int status: SWB_OK (0) or a negative error
 *    class.  No exception crosses the ABI.  swb_last_error() gives the text.
 *  - A handle owns its device memory and one CUDA stream; it is not
 *    thread-safe.  Use different handles from different threads.
 *  - Calls are asynchronous on the handle's stream unless they return host
 *    data (get_*), which synchronise.
 */
#ifndef SWALBE_GB300_H
#define SWALBE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWB_ABI_VERSION 1

/* ---- status codes ---- */
#define SWB_OK 0
#define SWB_ERR_ARG (-1)         /* invalid argument / size                       */
#define SWB_ERR_OOM (-2)         /* device allocation failed / over HBM budget     */
#define SWB_ERR_CUDA (-3)        /* CUDA runtime error (text in swb_last_error)   */
#define SWB_ERR_NAN (-4)         /* non-finite height detected during a step      */
#define SWB_ERR_UNSUPPORTED (-5) /* operation not available in this precision mode */
#define SWB_ERR_CANCELLED (-6)   /* request cancelled                              */
#define SWB_ERR_NOT_FOUND (-7)   /* unknown request id                             */
#define SWB_ERR_BUSY (-8)        /* request queue full                             */

/* ---- precision modes ---- */
#define SWB_F64 0     /* fused step, Float64 arithmetic in the reference's operation order */
#define SWB_F32 1     /* fused step, FP32 arithmetic and FP32 populations               */
#define SWB_F16 2     /* fused step, FP32 arithmetic; f0 FP32, f1..f8 FP16 (scaled 2^10) */
#define SWB_PLAIN64 3 /* one kernel per reference op, Float64, full State arrays        */

/* Taumucs{T} + SysConst{T} (src/initialize.jl:43-60, 76-81).  θ is in
 * multiples of π as in the reference (cospi(θ), src/pressure.jl:143). */
typedef struct swb_params {
    int32_t Lx, Ly;       /* lattice size                                  */
    int32_t Tmax, tdump;  /* time steps, dump interval                     */
    double tau, cs, mu;   /* relaxation time, sound speed, kinematic visc.  */
    double delta, kbt;    /* slip length, thermal energy (0: no fluctuations) */
    double gamma;         /* surface tension                                */
    int32_t n, m;         /* disjoining-pressure exponents                  */
    double hmin, hcrit;   /* Π(hmin) = 0, stabiliser                        */
    double theta, g;      /* contact angle (units of π), gravity            */
} swb_params;

/* Fields of a state (the arrays of `State`, src/initialize.jl:149-168). */
#define SWB_FIELD_HEIGHT 0
#define SWB_FIELD_VELX 1
#define SWB_FIELD_VELY 2
#define SWB_FIELD_PRESSURE 3 /* fused modes: film pressure of the current height */
#define SWB_FIELD_FOUT 4     /* Lx*Ly*9, the streamed populations (fout == ftemp) */
#define SWB_FIELD_FEQ 5      /* PLAIN64 only */
#define SWB_FIELD_FX 6       /* PLAIN64 only */
#define SWB_FIELD_FY 7       /* PLAIN64 only */
#define SWB_FIELD_SLIPX 8    /* PLAIN64 only */
#define SWB_FIELD_SLIPY 9    /* PLAIN64 only */
#define SWB_FIELD_HGRADPX 10 /* PLAIN64 only: h∇px */
#define SWB_FIELD_HGRADPY 11 /* PLAIN64 only: h∇py */
#define SWB_FIELD_VSQ 12     /* PLAIN64 only */

/* Per-step measures, recorded for time_loop iteration t on the height at
 * the start of that iteration -- where the reference takes them:
 * mass = sum(height) (src/simulate.jl:10), wetted = count(h > hthresh)
 * (src/measures.jl:13-17), hmax - hmin (src/simulate.jl:56), and the
 * liquid-vapour area of surfacearea! (src/measures.jl:126-168). */
#define SWB_MEAS_MASS 1
#define SWB_MEAS_WETTED 2
#define SWB_MEAS_MAXMIN 4
#define SWB_MEAS_AREA 8
#define SWB_MEAS_ALL 15

typedef struct swb_measure {
    int64_t t;       /* time_loop iteration (1-based)                     */
    double mass;     /* Σ h (FP64 accumulation in every precision mode)   */
    int64_t wetted;  /* #{h > hthresh}                                    */
    double hmax;     /* maximum(h)                                        */
    double hmin;     /* minimum(h)                                        */
    double area;     /* Σ_{h>hthresh} sqrt(1 + |∇h|²)                     */
    double energy;   /* area - Σ_{h>hthresh} cospi(θ)                      */
} swb_measure;

typedef struct swb_state swb_state;

/* ---------------------------------------------------------------------- */
/* Library                                                                 */
/* ---------------------------------------------------------------------- */
int swb_abi_version(void);
/* Text of the most recent error on this thread (state may be NULL). */
const char *swb_last_error(const swb_state *s);
const char *swb_status_string(int status);
/* Device memory a state of this size and mode needs, in bytes. */
int swb_state_bytes(const swb_params *p, int precision, size_t *bytes);

/* ---------------------------------------------------------------------- */
/* One simulation                                                          */
/* ---------------------------------------------------------------------- */
/* Sys(sysc, device; T) (src/initialize.jl:491-536): zero populations,
 * height = 1, velocities 0. */
int swb_create(const swb_params *p, int precision, swb_state **out);
int swb_destroy(swb_state *s);
int swb_get_params(const swb_state *s, swb_params *p, int *precision);

/* state.<field> .= values (host, column-major Float64).  Setting height or
 * a velocity makes the next step start from the fields, as the reference's
 * time_loop does after `state.height .= ...` (src/simulate.jl:240-242,
 * 384-397); the populations are kept (they are the reference's ftemp). */
int swb_set_field(swb_state *s, int field, const double *host);
/* Copies a field to the host (synchronises).  SWB_FIELD_FOUT is Lx*Ly*9. */
int swb_get_field(swb_state *s, int field, double *host);
/* As swb_set_field, from a Float64 column-major DEVICE array (e.g. the
 * memory of a CUDA.jl CuArray); asynchronous on the state's stream. */
int swb_set_field_device(swb_state *s, int field, const double *device_ptr);

/* Runs the state's work on `stream` (a cudaStream_t owned by the caller,
 * e.g. CUDA.jl's task stream); NULL returns to the state's own stream. */
int swb_set_stream(swb_state *s, void *stream);
int swb_get_stream(swb_state *s, void **stream);
/* Kernel launches issued by this library since load (all handles). */
int swb_launch_count(uint64_t *count);

/* θ for filmpressure!(state, sys; θ) (src/pressure.jl:119-147):
 *   set_theta       -- scalar θ (time_loop(sys, state, θ::Number));
 *   set_theta_field -- θ::Matrix (time_loop(sys, state, θ), src/simulate.jl:26-45);
 *   set_theta_wave  -- θ(x,t) = θ0 + Δθ·sin(2π(x - v t)/Lx), x = i-1, t the
 *                      time_loop iteration (moving wettability,
 *                      scripts/Moving_wettability_structs.jl:139-152 does a
 *                      discrete shift of such a pattern). */
int swb_set_theta(swb_state *s, double theta);
int swb_set_theta_field(swb_state *s, const double *theta);
int swb_set_theta_wave(swb_state *s, double theta0, double dtheta, double v);
/* Moving substrate: the θ field set by swb_set_theta_field moves by
 * (dx, dy) cells (periodically) after every tmove iterations, counted from
 * this call -- move_substrate!(θ, input, t, tmove; direction) called at the
 * end of each iteration (scripts/Moving_wettability_structs.jl:139-152;
 * direction "diagonal" = (1, 1), "x" = (1, 0), "y" = (0, 1)).  The field is
 * not copied: the step reads it at the moved index.  tmove = 0 stops it;
 * setting a θ (field, scalar or wave) resets it. */
int swb_set_substrate_motion(swb_state *s, int64_t tmove, int dx, int dy);

/* inclination!(α, state; t, tstart, tsmooth) as the time_loop callback
 * (src/forcing.jl:363-368, src/simulate.jl:89).  loop_time = 0 uses the
 * fixed `t` (the callback's default 1000); loop_time = 1 uses the
 * iteration.  ax = ay = 0 switches it off. */
int swb_set_inclination(swb_state *s, double ax, double ay, int loop_time, int64_t t,
                        int64_t tstart, int64_t tsmooth);

/* Geometry of the fused step: CTAs of nt threads (64, 128, 256) own strips
 * of nt-4 columns and h rows (2..512) that they march row by row; with
 * nt = -32, -64 or -128 (SWB_F32 / SWB_F16, even Lx) CTAs of -nt threads own
 * strips of 2|nt|-4 columns, two columns per thread with paired (vector)
 * population loads and stores (the common steady τ = 1 step; other
 * iterations run as 64-thread strips of the same rows); or, with
 * nt = 32 (SWB_F32 / SWB_F16 only; h is ignored), CTAs of 256 threads own
 * 2D tiles of 32 x 16 cells whose loads are all issued at once.  By default
 * states autotune it on their first swb_step of >= 512 steps (timing a few
 * geometries on those real steps; remembered per lattice size).  Setting it
 * (or (0, 0): a size rule) turns the autotuner off.  Results do not depend
 * on it: the per-cell arithmetic is the same in every form, and the mass that
 * drives the SWB_F32 / SWB_F16 mass correction is an exact fixed-point sum. */
int swb_set_geometry(swb_state *s, int nt, int h);
int swb_get_geometry(swb_state *s, int *nt, int *h);

/* Launch form of swb_step (no counterpart in the reference, whose time loop
 * runs each op as its own broadcast, src/simulate.jl:15-22).
 *   SWB_STEP_PER_ITERATION  one kernel per iteration, replayed from CUDA
 *                           graphs of 64 iterations;
 *   SWB_STEP_MULTI          SWB_F32 / SWB_F16 only: one cooperative launch
 *                           runs up to 1024 iterations, CTAs meeting at a
 *                           grid barrier between iterations (strip width 64
 *                           or 128);
 *   SWB_STEP_AUTO           (default) PER_ITERATION; the autotuner picks the
 *                           geometry.  (MULTI measured 5-25 % slower on
 *                           GB300; with SWB_STEP_MULTI the tuner picks the
 *                           geometry among the multi-step candidates.)
 * Both forms give identical results for the same geometry.
 * swb_get_step_mode reports the form in effect (PER_ITERATION or MULTI). */
#define SWB_STEP_AUTO 0
#define SWB_STEP_PER_ITERATION 1
#define SWB_STEP_MULTI 2
int swb_set_step_mode(swb_state *s, int mode);
int swb_get_step_mode(swb_state *s, int *mode);

/* SWB_F32 / SWB_F16: hold the total mass at its value when the fields were
 * last set, by a correction spread over the cells, two iterations behind
 * the measurement (default: on for SWB_F16, whose FP16 populations cannot
 * hold the rounding residues; off for SWB_F32, whose populations keep the
 * mass to ~1e-12 relative without it).  The mass is measured exactly (a
 * fixed-point sum in units of 2^-32 per cell), so the correction, and the
 * results, do not depend on the geometry.  It costs a reduction per
 * iteration.  No effect in SWB_F64, the reference's arithmetic. */
int swb_set_mass_correction(swb_state *s, int on);

/* Which measures swb_step records each iteration (SWB_MEAS_* mask). */
int swb_set_measures(swb_state *s, int mask, double hthresh);

/* `nsteps` iterations of the time_loop body (src/simulate.jl:15-22):
 * filmpressure!, h∇p!, slippage!, forces, equilibrium!, BGKandStream!,
 * moments!.  Asynchronous.  SWB_ERR_NAN is reported by the next
 * synchronising call after a non-finite height was seen. */
int swb_step(swb_state *s, int64_t nsteps);
/* snapshot!(fluid, height, t; dumping) (src/measures.jl:99-105) on the
 * device: after every iteration t with t % dumping == 0 the height is copied
 * into a device ring of `capacity` fields (Float64, column-major), without a
 * host round trip.  dumping = 0 turns it off (and frees the ring).
 * swb_get_snapshots copies the snapshots taken since the last call, oldest
 * first (each row Lx*Ly doubles, the reference's vec(h)), with their
 * iterations in `times` (may be NULL); if more than `capacity` were taken,
 * only the newest `capacity` remain. */
int swb_set_snapshots(swb_state *s, int64_t dumping, int64_t capacity);
int swb_get_snapshots(swb_state *s, double *out, int64_t cap, int64_t *count, int64_t *times);
int swb_sync(swb_state *s);
/* Number of iterations completed since swb_create. */
int swb_steps_done(swb_state *s, int64_t *t);
/* Drains the per-step measures recorded since the last call (oldest
 * first); at most `cap` records.  The device ring holds SWB_RECORD_CAPACITY
 * records: a caller that steps further than that between two drains loses
 * the oldest ones, and swb_measures_dropped counts them.  The reference
 * pushes Δh and wetted! every step (src/simulate.jl:56, src/measures.jl:13-17),
 * so time_loop drains at least every SWB_RECORD_CAPACITY steps. */
#define SWB_RECORD_CAPACITY 65536
int swb_get_measures(swb_state *s, swb_measure *out, int64_t cap, int64_t *count);
/* Records overwritten in the device ring before swb_get_measures read them,
 * since the state was created (0 when the host drained in time). */
int swb_measures_dropped(swb_state *s, int64_t *dropped);
/* Measures of the current height now (mass, wetted, max/min, area,
 * surfacearea!'s energy; src/measures.jl:126-168).  The energy's cos θ is
 * that of the iteration which starts from this height (steps done + 1): the
 * scalar θ, the θ field at that iteration's offset (a moving substrate), or
 * the θ wave at that time -- so it equals the step's own record of that
 * iteration. */
int swb_measure_now(swb_state *s, double hthresh, swb_measure *out);
/* The same measures of a caller's Float64 column-major DEVICE height field,
 * without any device allocation by the library.  No counterpart in the
 * reference: it serves callers that must not allocate (a host that has
 * committed its whole HBM budget, or whose own memory pool owns the device).
 * Scratch is a fixed 48 KiB array compiled into the library; lattices up to
 * 2^28 cells (larger: SWB_ERR_ARG).  d_cos_theta: per-cell cospi(θ) on the
 * device or NULL (then cos_theta is used for the energy).  Both fields must
 * be device memory of the CURRENT device (cudaSetDevice), which owns the
 * scratch copy the call uses; other pointers give SWB_ERR_ARG.  Runs on `stream`
 * (NULL: the default stream) and synchronises it.  The first call on each
 * device looks up the array's address, so make it before any stream capture.
 * All calls share the array: calls that overlap on the GPU race. */
int swb_measure_field_noalloc(const double *d_height, int Lx, int Ly, double hthresh,
                              const double *d_cos_theta, double cos_theta, void *stream,
                              swb_measure *out);

/* Thermal fluctuations (kbt > 0 in the params): every iteration adds
 * -thermal!(h) to the force, Fx .= -h∇px .- slipx .- kbtx as the reference's
 * thermal scripts do (src/forcing.jl:297-320, scripts/Rivulet_stability.jl:123).
 * The normals come from Philox-4x32-10 keyed by the seed with counter (cell,
 * iteration): reproducible, and the same stream in every precision mode and
 * launch form (Julia's randn! stream cannot be reproduced).  Default seed 0. */
int swb_set_thermal_seed(swb_state *s, uint64_t seed);
/* thermal!(kbtx, kbty, height, kbt, mu, delta) of the current height for
 * iteration t: the forces the step subtracts (host, column-major). */
int swb_thermal_field(swb_state *s, int64_t t, double *fx, double *fy);

/* Number of droplets in a host height field: connected components of the
 * cells with h > hthresh, 8-connected, periodic in x and y.  Host code, no
 * GPU.  No counterpart in the reference (its measures stop at wetted!,
 * src/measures.jl:13-17); used to compare spinodal dewetting across
 * precisions. */
int swb_count_droplets(const double *h, int Lx, int Ly, double hthresh, int64_t *count);

/* ---------------------------------------------------------------------- */
/* Per-op API, SWB_PLAIN64 only: one kernel per reference op on the full   */
/* State arrays, same Float64 operation order.                             */
/* ---------------------------------------------------------------------- */
int swb_op_filmpressure(swb_state *s);          /* src/pressure.jl:119-155 (uses the θ set) */
int swb_op_hgradp(swb_state *s);                /* src/forcing.jl:168-187 */
int swb_op_slippage(swb_state *s);              /* src/forcing.jl:42-56 */
int swb_op_force_sum(swb_state *s);             /* src/simulate.jl:18-19 */
int swb_op_thermal(swb_state *s, int64_t t);    /* Fx .-= kbtx, Fy .-= kbty: thermal! of iteration t
                                                   (src/forcing.jl:297-320); no-op when kbt == 0 */
int swb_op_inclination(swb_state *s, double ax, double ay, int64_t t, int64_t tstart,
                       int64_t tsmooth);        /* src/forcing.jl:363-368 */
int swb_op_equilibrium(swb_state *s);           /* src/equilibrium.jl:63-119 */
int swb_op_bgk_stream(swb_state *s);            /* src/collide.jl:70-105, 151-152 */
int swb_op_moments(swb_state *s);               /* src/moments.jl:43-64 */

/* ---------------------------------------------------------------------- */
/* Batched ensemble: many lattices of uneven size and parameters advanced  */
/* together by one launch per step over a packed tile table.  Replaces a   */
/* loop of independent `run_*` simulations (src/simulate.jl:236-503).      */
/* ---------------------------------------------------------------------- */
typedef struct swb_batch swb_batch;
int swb_batch_create(const swb_params *params, int count, int precision, swb_batch **out);
int swb_batch_destroy(swb_batch *b);
int swb_batch_set_height(swb_batch *b, int idx, const double *host);
int swb_batch_get_height(swb_batch *b, int idx, double *host);
int swb_batch_set_theta_wave(swb_batch *b, int idx, double theta0, double dtheta, double v);
int swb_batch_step(swb_batch *b, int64_t nsteps);
/* Waits for the batch; SWB_ERR_NAN (lattice index in swb_last_error) if a
 * lattice saw a non-finite height. */
int swb_batch_sync(swb_batch *b);
/* Strips of every lattice: nt threads (64, 128, 256; nt - 4 columns), or
 * pair strips of -nt threads (nt = -32, -64, -128; 2|nt| - 4 columns, two per
 * thread; SWB_F32 / SWB_F16 with even Lx in every lattice; iterations the
 * pair form has no kernel for run on 64-thread strips), and `rows` rows
 * (2..512, capped at each lattice's height).  By default the first
 * swb_batch_step with enough steps times a few geometries (one-column and,
 * where possible, pair strips) and CTA counts on real steps and keeps the
 * fastest; setting a geometry keeps it and tunes only the CTA count. */
int swb_batch_set_geometry(swb_batch *b, int nt, int rows);
/* The geometry in use (nt as above), and the CTAs per launch (0: not tuned yet). */
int swb_batch_geometry(swb_batch *b, int *nt, int *rows, int *grid);
/* Strip width in columns and rows, and iterations per captured graph (0 until tuned). */
int swb_batch_tile(swb_batch *b, int *tile_x, int *tile_y, int *steps_per_graph);

/* ---------------------------------------------------------------------- */
/* Serving: a request loop with HBM-footprint admission and continuous     */
/* batching of resident simulations.                                       */
/* ---------------------------------------------------------------------- */
typedef struct swb_server swb_server;
typedef struct swb_request_info {
    int64_t id;
    int32_t status;        /* 0 queued, 1 running, 2 done, <0 error        */
    int64_t steps_done;
    double t_submit;       /* seconds on the server's clock                */
    double t_admit;
    double t_done;
} swb_request_info;
typedef struct swb_server_stats {
    int64_t submitted, admitted, completed, rejected;
    int64_t queued, running;
    double lattice_updates; /* total lattice updates served              */
    double busy_seconds;    /* time with at least one resident request   */
    size_t hbm_in_use, hbm_budget;
    int64_t ticks;
    double device_seconds;  /* device time of the ticks (CUDA events)     */
} swb_server_stats;

/* hbm_budget: bytes of device memory the resident states may use.
 * steps_per_tick: time steps run per scheduling tick. */
int swb_server_create(size_t hbm_budget, int precision, int steps_per_tick, swb_server **out);
int swb_server_destroy(swb_server *sv);
/* At most `max_queued` requests wait for admission (each holds its initial
 * film in host memory); further submissions return SWB_ERR_BUSY and count
 * as rejected.  Default 1024. */
int swb_server_set_queue_limit(swb_server *sv, int64_t max_queued);
/* Scheduling.  Resident requests advance in lock step, so a request's
 * latency is its step count times one step of the whole resident set.
 *   SWB_SCHED_FIFO  admit in arrival order (default);
 *   SWB_SCHED_SJF   admit the queued request with the least work
 *                   (Lx*Ly*nsteps) first; a full queue then sheds its
 *                   largest request (status SWB_ERR_BUSY) for a smaller
 *                   newcomer.  Large requests can wait indefinitely under
 *                   sustained overload.
 * max_resident_cells > 0 also bounds the summed Lx*Ly of resident requests
 * (a request larger than the bound still runs when it would be alone). */
#define SWB_SCHED_FIFO 0
#define SWB_SCHED_SJF 1
int swb_server_set_policy(swb_server *sv, int policy, int64_t max_resident_cells);
/* Strip geometry of the resident set.  nt = 0 (default): chosen whenever the
 * set changes (pair strips of 60 or 124 columns, whichever processes fewer
 * cells, when every lattice allows pair strips; one-column strips of 64
 * threads otherwise), each lattice's rows balanced up to `rows` (0: 64).
 * nt = -32 or -64: those pair strips whenever every lattice allows them,
 * rows balanced up to `rows` (>= 2).  Results do not depend on the
 * geometry. */
int swb_server_set_geometry(swb_server *sv, int nt, int rows);
/* Queues a solve: params (Lx, Ly, γ, θ, g, ...), initial height (copied),
 * moving wettability (dtheta = 0 for none) and the step count. */
int swb_server_submit(swb_server *sv, const swb_params *p, const double *h0, double theta0,
                      double dtheta, double v, int64_t nsteps, int64_t *id);
/* 1 if done (height copied to h_out when not NULL), 0 if not yet. */
int swb_server_poll(swb_server *sv, int64_t id, double *h_out, swb_request_info *info);
int swb_server_cancel(swb_server *sv, int64_t id);
int swb_server_stats_get(swb_server *sv, swb_server_stats *st);
double swb_server_clock(swb_server *sv);

/* ---------------------------------------------------------------------- */
/* One dimension: the D1Q3 solver (src/collide.jl:179-212,                 */
/* src/simulate.jl:98-179), for one or many 1D lattices.                    */
/* ---------------------------------------------------------------------- */
/* Sys(sysc::SysConst_1D) (src/initialize.jl:587-599) for each of `count`
 * lattices: L = params[i].Lx (>= 3), params[i].Ly = 1; zero populations,
 * height 1, velocity 0.  SWB_F64 (the reference's arithmetic, bit for bit)
 * or SWB_F32.  rec_cap > 0 keeps the measures (mass, wetted count,
 * max/min) of the last rec_cap iterations of each lattice.  Every
 * swb1d_step runs all lattices together, one CTA each. */
typedef struct swb1d swb1d;
#define SWB1D_FIELD_THETA 20 /* θ field (time_loop(sys, state, θ::Vector))          */
#define SWB1D_FIELD_GAMMA 21 /* γ field and its ∇γ force (run_gamma, src/simulate.jl:518-556) */
int swb1d_create(const swb_params *params, int count, int precision, int rec_cap, swb1d **out);
int swb1d_destroy(swb1d *b);
/* height, vel (SWB_FIELD_HEIGHT, SWB_FIELD_VELX), SWB1D_FIELD_THETA and
 * SWB1D_FIELD_GAMMA (NULL clears them); host arrays of L doubles. */
int swb1d_set_field(swb1d *b, int idx, int field, const double *host);
/* height, vel, pressure (SWB_FIELD_PRESSURE) or the populations
 * (SWB_FIELD_FOUT, L x 3 column-major, the reference's fout).  Syncs. */
int swb1d_get_field(swb1d *b, int idx, int field, double *host);
int swb1d_step(swb1d *b, int64_t nsteps);
int swb1d_sync(swb1d *b);
int swb1d_get_measures(swb1d *b, int idx, swb_measure *out, int64_t cap, int64_t *count);

#ifdef __cplusplus
}
#endif
#endif /* SWALBE_GB300_H */
