// swb_run_f32.cu -- the multi-step (cooperative) kernel for FP32 and
// FP16-storage lattices.  Same step code and flags as swb_step_f32.cu
// (--fmad=false), so a lattice advanced here rounds exactly as it does with
// one launch per step; only the population loads go through L2 (LdCG).
#include "swb_step_impl.cuh"

namespace swb {

// S: the store type with L2 loads; NT, T2D: the tile form of the geometry.
#define RUN_DISPATCH(precision, nt, ...)                          \
    do {                                                          \
        auto run_body = [&](auto store_tag) {                     \
            using S = decltype(store_tag);                        \
            if ((nt) == kTileGeom) {                              \
                constexpr int NT = kT2NT;                         \
                constexpr bool T2D = true;                        \
                __VA_ARGS__;                                      \
            } else if ((nt) == 64) {                              \
                constexpr int NT = 64;                            \
                constexpr bool T2D = false;                       \
                __VA_ARGS__;                                      \
            } else {                                              \
                constexpr int NT = 128;                           \
                constexpr bool T2D = false;                       \
                __VA_ARGS__;                                      \
            }                                                     \
        };                                                        \
        if ((precision) == SWB_F16)                               \
            run_body(StoreF16T<LdCG>{});                          \
        else                                                      \
            run_body(StoreF32T<LdCG>{});                          \
    } while (0)

bool run_geometry_ok(int nt) { return nt == 64 || nt == 128 || nt == kTileGeom; }

int fused_run_blocks_per_sm(int precision, int nt) {
    if (precision != SWB_F32 && precision != SWB_F16) return 0;
    if (!run_geometry_ok(nt)) return 0;
    int n = 0;
    RUN_DISPATCH(precision, nt,
                 cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fused_run_kernel<S, NT, T2D>,
                                                               NT, 0));
    return n;
}

cudaError_t launch_fused_run(int precision, const StepArgs &a, int n, int grid, cudaStream_t st) {
    if ((precision != SWB_F32 && precision != SWB_F16) || !run_geometry_ok(a.march_nt) || !a.bar)
        return cudaErrorInvalidValue;
    StepArgs args = a;
    int steps = n;
    void *params[] = {&args, &steps};
    cudaError_t e = cudaSuccess;
    RUN_DISPATCH(precision, a.march_nt,
                 e = cudaLaunchCooperativeKernel((const void *)fused_run_kernel<S, NT, T2D>,
                                                 dim3(grid), dim3(NT), params, 0, st));
    return e;
}

}  // namespace swb
