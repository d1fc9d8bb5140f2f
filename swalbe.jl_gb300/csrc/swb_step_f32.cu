// swb_step_f32.cu -- FP32-arithmetic kernels: FP32 populations (SWB_F32) and
// FP32 f0 with FP16 f1..f8 (SWB_F16).  Compiled with --fmad=false so that the
// single-lattice and batch kernels, which inline the same step code, round
// identically; parity with the Float64 oracle is checked against stated
// tolerances.
#include <type_traits>

#include "swb_step_impl.cuh"

namespace swb {

namespace {
int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b > 152LL * 32) b = 152LL * 32;
    return (int)(b < 1 ? 1 : b);
}
}  // namespace

#define DISPATCH_STORE(precision, ...)          \
    do {                                        \
        if ((precision) == SWB_F16) {           \
            using S = StoreF16;                 \
            __VA_ARGS__;                        \
        } else {                                \
            using S = StoreF32;                 \
            __VA_ARGS__;                        \
        }                                       \
    } while (0)

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

// Strips of 64 or 128 threads (the widths the tuner and the size rule pick
// for single lattices) also exist in the steady forms.
#define DISPATCH_NT_NARROW(nt, ...)                \
    do {                                           \
        if ((nt) == 64) {                          \
            constexpr int NT = 64;                 \
            __VA_ARGS__;                           \
        } else {                                   \
            constexpr int NT = 128;                \
            __VA_ARGS__;                           \
        }                                          \
    } while (0)

cudaError_t launch_fused_step_f32(int precision, const StepArgs &a, int k, bool steady,
                                  cudaStream_t st) {
    if (resident_geometry(a.march_nt))  // one iteration at a time: strips of the same rows
        return launch_fused_step_f32(precision, strip_fallback(a), k, steady, st);
    if (a.march_nt < 0) {
        if (!(steady && pair_form_ok(a)))
            return launch_fused_step_f32(precision, pair_fallback(a), k, steady, st);
        const int grid = step_grid(a, k);
        cudaError_t e = cudaSuccess;
        auto go = [&](auto wave) {
            constexpr bool W = decltype(wave)::value;
            if (a.march_nt == -32)
                DISPATCH_STORE(precision, e = launch_step(pair_step_kernel<S, 32, W>, grid, 32, st, a, k));
            else if (a.march_nt == -128)
                DISPATCH_STORE(precision, e = launch_step(pair_step_kernel<S, 128, W>, grid, 128, st, a, k));
            else
                DISPATCH_STORE(precision, e = launch_step(pair_step_kernel<S, 64, W>, grid, 64, st, a, k));
        };
        if (a.theta_mode == THETA_WAVE)
            go(std::true_type{});
        else
            go(std::false_type{});
        return e;
    }
    const int grid = step_grid(a, k);
    cudaError_t e = cudaSuccess;
    if (a.march_nt == kTileGeom) {
        DISPATCH_STORE(precision, e = launch_step(fused_tile_kernel<S>, grid, kT2NT, st, a, k));
    } else if (step_general(a) && !(steady && !step_rare(a) && (a.march_nt == 64 || a.march_nt == 128))) {
        DISPATCH_STORE(precision, DISPATCH_NT(a.march_nt, e = launch_step(fused_step_kernel<S, NT, true>, grid, NT, st, a, k)));
    } else if (step_general(a)) {  // the θ wave alone: WAVE variant of the steady forms
        if (a.tau_is_one)
            DISPATCH_STORE(precision, DISPATCH_NT_NARROW(a.march_nt, e = launch_step(fused_step_kernel<S, NT, false, kFormSteadyTau1, true>, grid, NT, st, a, k)));
        else
            DISPATCH_STORE(precision, DISPATCH_NT_NARROW(a.march_nt, e = launch_step(fused_step_kernel<S, NT, false, kFormSteady, true>, grid, NT, st, a, k)));
    } else if (steady && (a.march_nt == 64 || a.march_nt == 128)) {
        if (a.tau_is_one)
            DISPATCH_STORE(precision, DISPATCH_NT_NARROW(a.march_nt, e = launch_step(fused_step_kernel<S, NT, false, kFormSteadyTau1>, grid, NT, st, a, k)));
        else
            DISPATCH_STORE(precision, DISPATCH_NT_NARROW(a.march_nt, e = launch_step(fused_step_kernel<S, NT, false, kFormSteady>, grid, NT, st, a, k)));
    } else {
        DISPATCH_STORE(precision, DISPATCH_NT(a.march_nt, e = launch_step(fused_step_kernel<S, NT, false>, grid, NT, st, a, k)));
    }
    return e;
}

cudaError_t launch_moments_f32(int precision, const StepArgs &a, cudaStream_t st) {
    const int g = grid_for((long long)a.Lx * a.Ly, 256);
    DISPATCH_STORE(precision, (moments_kernel<S><<<g, 256, 0, st>>>(a)));
    return cudaGetLastError();
}

cudaError_t launch_fout_f32(int precision, const StepArgs &a, double *out, cudaStream_t st) {
    const int g = grid_for((long long)a.Lx * a.Ly, 256);
    DISPATCH_STORE(precision, (fout_kernel<S><<<g, 256, 0, st>>>(a, out)));
    return cudaGetLastError();
}

cudaError_t launch_thermal_field_f32(int precision, const StepArgs &a, long long t, double *fx,
                                     double *fy, cudaStream_t st) {
    const int g = grid_for((long long)a.Lx * a.Ly, 256);
    DISPATCH_STORE(precision, (thermal_field_kernel<S><<<g, 256, 0, st>>>(a, t, fx, fy)));
    return cudaGetLastError();
}

cudaError_t launch_pressure_now_f32(int precision, const StepArgs &a, double *out,
                                    cudaStream_t st) {
    const int g = grid_for((long long)a.Lx * a.Ly, 256);
    DISPATCH_STORE(precision, (pressure_now_kernel<S><<<g, 256, 0, st>>>(a, out)));
    return cudaGetLastError();
}

cudaError_t launch_batch_step_f32(int precision, int nt, bool gen, bool steady_tau1,
                                  const StepArgs *d_args, const TileRef *d_tiles, int ntiles,
                                  int grid, int k, cudaStream_t st, bool rare) {
    cudaError_t e = cudaSuccess;
    if (nt < 0) {  // pair strips: the caller passes their table only for steady steps they have
        if (!steady_tau1) return cudaErrorInvalidValue;
        auto go = [&](auto wave) {
            constexpr bool W = decltype(wave)::value;
            if (nt == -32)
                DISPATCH_STORE(precision, e = launch_step(batch_pair_kernel<S, 32, W>, grid, 32, st, d_args, d_tiles, ntiles, k));
            else if (nt == -128)
                DISPATCH_STORE(precision, e = launch_step(batch_pair_kernel<S, 128, W>, grid, 128, st, d_args, d_tiles, ntiles, k));
            else
                DISPATCH_STORE(precision, e = launch_step(batch_pair_kernel<S, 64, W>, grid, 64, st, d_args, d_tiles, ntiles, k));
        };
        if (gen)
            go(std::true_type{});
        else
            go(std::false_type{});
        return e;
    }
    if (gen && !rare && steady_tau1 && nt == kBatchNT)  // the θ wave alone
        DISPATCH_STORE(precision, e = launch_step(batch_step_kernel<S, kBatchNT, false, kFormSteadyTau1, true>, grid, kBatchNT, st, d_args, d_tiles, ntiles, k));
    else if (gen)
        DISPATCH_STORE(precision, DISPATCH_NT(nt, e = launch_step(batch_step_kernel<S, NT, true>, grid, NT, st, d_args, d_tiles, ntiles, k)));
    else if (steady_tau1 && nt == kBatchNT)
        DISPATCH_STORE(precision, e = launch_step(batch_step_kernel<S, kBatchNT, false, kFormSteadyTau1>, grid, kBatchNT, st, d_args, d_tiles, ntiles, k));
    else
        DISPATCH_STORE(precision, DISPATCH_NT(nt, e = launch_step(batch_step_kernel<S, NT, false>, grid, NT, st, d_args, d_tiles, ntiles, k)));
    return e;
}

// Resident CTAs per SM of the pair-strip kernel of geometry nt (-32, -64, -128).
int pair_blocks_per_sm(int precision, int nt) {
    int n = 0;
    if (nt == -32)
        DISPATCH_STORE(precision, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pair_step_kernel<S, 32, false>, 32, 0));
    else if (nt == -128)
        DISPATCH_STORE(precision, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pair_step_kernel<S, 128, false>, 128, 0));
    else
        DISPATCH_STORE(precision, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pair_step_kernel<S, 64, false>, 64, 0));
    return n < 1 ? 1 : n;
}

// Resident CTAs per SM of the batch kernel most launches use (the steady
// form at the default width: fewer registers, so more CTAs).  The table walk
// needs no co-residency, so a grid sized for it is valid for every form.
int batch_blocks_per_sm_f32(int precision, int nt, bool wave) {
    int n = 0;
    if (nt < 0) {  // the pair kernel of the θ-wave form, or the plain one
        auto occ = [&](auto w) {
            constexpr bool W = decltype(w)::value;
            if (nt == -32)
                DISPATCH_STORE(precision, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_pair_kernel<S, 32, W>, 32, 0));
            else if (nt == -128)
                DISPATCH_STORE(precision, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_pair_kernel<S, 128, W>, 128, 0));
            else
                DISPATCH_STORE(precision, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_pair_kernel<S, 64, W>, 64, 0));
        };
        if (wave)
            occ(std::true_type{});
        else
            occ(std::false_type{});
        return n < 1 ? 1 : n;
    }
    if (nt == kBatchNT)
        DISPATCH_STORE(precision, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_step_kernel<S, kBatchNT, false, kFormSteadyTau1>, kBatchNT, 0));
    else
        DISPATCH_STORE(precision, DISPATCH_NT(nt, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_step_kernel<S, NT, false>, NT, 0)));
    return n < 1 ? 1 : n;
}

}  // namespace swb
