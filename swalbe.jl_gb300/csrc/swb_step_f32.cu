// swb_step_f32.cu -- FP32-arithmetic kernels: FP32 populations (SWB_F32) and
// FP32 f0 with FP16 f1..f8 (SWB_F16).  Contraction into FMA is allowed here;
// parity with the Float64 oracle is checked against stated tolerances.
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

cudaError_t launch_fused_step_f32(int precision, const StepArgs &a, cudaStream_t st) {
    dim3 grid(a.tiles_x, a.tiles_y);
    DISPATCH_STORE(precision, (fused_step_kernel<S><<<grid, kThreads, 0, st>>>(a)));
    return cudaGetLastError();
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

cudaError_t launch_pressure_now_f32(int precision, const StepArgs &a, double *out,
                                    cudaStream_t st) {
    const int g = grid_for((long long)a.Lx * a.Ly, 256);
    DISPATCH_STORE(precision, (pressure_now_kernel<S><<<g, 256, 0, st>>>(a, out)));
    return cudaGetLastError();
}

cudaError_t launch_batch_step_f32(int precision, const StepArgs *d_args, const TileRef *d_tiles,
                                  int ntiles, int grid, cudaStream_t st) {
    DISPATCH_STORE(precision, (batch_step_kernel<S><<<grid, kThreads, 0, st>>>(d_args, d_tiles, ntiles)));
    return cudaGetLastError();
}

int batch_blocks_per_sm_f32(int precision) {
    int n = 0;
    if (precision == SWB_F16)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_step_kernel<StoreF16>, kThreads, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_step_kernel<StoreF32>, kThreads, 0);
    return n < 1 ? 1 : n;
}

}  // namespace swb
