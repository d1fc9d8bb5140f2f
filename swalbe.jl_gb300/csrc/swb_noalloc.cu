// swb_noalloc.cu -- measures of a caller's height field without any device
// allocation by this library.
//
// Some callers cannot let a library call cudaMalloc: a serving loop that has
// already committed the whole HBM budget to resident simulations (it admits
// solves by their exact footprint, so an allocation behind its back can fail
// or break the accounting), or a host whose own memory pool owns the device
// (CUDA.jl's pool, PyTorch's caching allocator), where a foreign cudaMalloc
// fragments the pool and cudaFree synchronises the whole device.  For them,
// swb_measure_field_noalloc runs the same reduction kernel as
// swb_measure_now, with its scratch in a fixed array compiled into this file.
//
// The array is file-scope `static __device__` memory: every GPU that loads
// the library holds it (48 KiB) until the process exits.  Host code cannot
// use the symbol itself as a device address; the address is looked up once
// per device with cudaGetSymbolAddress and cached.
#include <mutex>
#include <string>

#include "swb_internal.h"

namespace {

// Scratch layout (in doubles): block partials for at most kMaxBlocks CTAs,
// then one Record, then the CTA ticket (an unsigned int in the last slot).
constexpr int kMaxBlocks = 1024;  // the measure kernel never launches more
constexpr int kPartialDoubles = kMaxBlocks * swb::kNPart;
constexpr int kRecordDoubles = (int)((sizeof(swb::Record) + 7) / 8);
constexpr int kScratchDoubles = kPartialDoubles + kRecordDoubles + 1;
// Largest lattice accepted: 2^28 cells (a 16384 x 16384 film, 2 GiB of Float64).
constexpr long long kMaxCells = 1LL << 28;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up on first
// use per device).
cudaError_t scratch_address(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = static_cast<double *>(p);
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

int nfail(int code, const std::string &m) {
    swb::set_global_error(m.c_str());
    return code;
}

// Whether p is device memory that the current device owns (the scratch
// address is that device's): cudaPointerGetAttributes allocates nothing.
bool on_current_device(const void *p) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
        cudaGetLastError();  // clear the error the query recorded
        return false;
    }
    return (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged) &&
           pa.device == dev;
}

}  // namespace

extern "C" int swb_measure_field_noalloc(const double *d_height, int Lx, int Ly, double hthresh,
                                         const double *d_cos_theta, double cos_theta,
                                         void *stream, swb_measure *out) {
    if (!d_height || !out) return nfail(SWB_ERR_ARG, "swb_measure_field_noalloc: NULL argument");
    if (Lx < 1 || Ly < 1) return nfail(SWB_ERR_ARG, "swb_measure_field_noalloc: Lx, Ly must be >= 1");
    if ((long long)Lx * Ly > kMaxCells)
        return nfail(SWB_ERR_ARG, "swb_measure_field_noalloc: lattice larger than the 2^28-cell "
                                  "limit of its fixed scratch");
    if (swb::measure_blocks((long long)Lx * Ly) > kMaxBlocks)
        return nfail(SWB_ERR_ARG, "swb_measure_field_noalloc: reduction grid exceeds the scratch");
    if (!on_current_device(d_height) || (d_cos_theta && !on_current_device(d_cos_theta)))
        return nfail(SWB_ERR_ARG, "swb_measure_field_noalloc: the height (and cos θ) field must "
                                  "be device memory of the current device");
    double *scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess)
        return nfail(SWB_ERR_CUDA, std::string("swb_measure_field_noalloc: scratch address: ") +
                                       cudaGetErrorString(e));
    cudaStream_t st = (cudaStream_t)stream;
    swb::Record *rec = reinterpret_cast<swb::Record *>(scratch + kPartialDoubles);
    unsigned int *ticket =
        reinterpret_cast<unsigned int *>(scratch + kPartialDoubles + kRecordDoubles);
    // the array keeps the previous call's contents: the ticket must start at 0
    e = cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st);
    if (e == cudaSuccess)
        e = swb::launch_measure(d_height, 1, Lx, Ly, hthresh, d_cos_theta, cos_theta, scratch,
                                ticket, rec, 0, st);
    swb::Record r{};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&r, rec, sizeof(r), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return nfail(SWB_ERR_CUDA, std::string("swb_measure_field_noalloc: ") + cudaGetErrorString(e));
    out->t = 0;
    out->mass = r.mass;
    out->wetted = (int64_t)r.wetted;
    out->hmax = r.hmax;
    out->hmin = r.hmin;
    out->area = r.area;
    out->energy = r.area - r.cos_sum;
    return SWB_OK;
}
