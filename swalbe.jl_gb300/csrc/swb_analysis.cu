// swb_analysis.cu -- host-side analysis of height fields: droplet count by
// periodic 8-connected labelling of the cells above a threshold.  The
// reference has no such function (its measures stop at wetted!,
// src/measures.jl:13-17, whose threshold 0.055 is the default here); the
// spinodal-dewetting comparison counts droplets with it.
#include <cstdint>
#include <numeric>
#include <vector>

#include "swb_internal.h"

namespace {

// Union-find with path halving over cell indices.
struct Forest {
    std::vector<int64_t> up;
    explicit Forest(int64_t n) : up(n) { std::iota(up.begin(), up.end(), 0); }
    int64_t find(int64_t a) {
        while (up[a] != a) {
            up[a] = up[up[a]];
            a = up[a];
        }
        return a;
    }
    void join(int64_t a, int64_t b) {
        a = find(a);
        b = find(b);
        if (a != b) up[a < b ? b : a] = a < b ? a : b;
    }
};

}  // namespace

extern "C" int swb_count_droplets(const double *h, int Lx, int Ly, double hthresh,
                                  int64_t *count) {
    if (!h || !count || Lx < 1 || Ly < 1) {
        swb::set_global_error("count_droplets: bad arguments");
        return SWB_ERR_ARG;
    }
    const int64_t N = (int64_t)Lx * Ly;
    Forest f(N);
    auto wet = [&](int64_t c) { return h[c] > hthresh; };
    for (int j = 0; j < Ly; ++j) {
        for (int i = 0; i < Lx; ++i) {
            const int64_t c = (int64_t)j * Lx + i;
            if (!wet(c)) continue;
            // four of the eight neighbours; the other four link back to this cell
            const int ip = i + 1 == Lx ? 0 : i + 1, im = i == 0 ? Lx - 1 : i - 1;
            const int jp = j + 1 == Ly ? 0 : j + 1;
            const int64_t nb[4] = {(int64_t)j * Lx + ip, (int64_t)jp * Lx + im,
                                   (int64_t)jp * Lx + i, (int64_t)jp * Lx + ip};
            for (int64_t n : nb)
                if (wet(n)) f.join(c, n);
        }
    }
    int64_t roots = 0;
    for (int64_t c = 0; c < N; ++c)
        if (wet(c) && f.find(c) == c) ++roots;
    *count = roots;
    return SWB_OK;
}
