// swb_server.cu -- serving: a request loop that admits thin-film solves by
// their HBM footprint, keeps their state resident, and advances every
// resident solve together (continuous batching: requests that arrive while
// others run are admitted at the next tick, and finished ones leave).
//
// One worker thread owns two streams.  A tick runs up to `steps_per_tick`
// time steps as one batched launch per step over the packed tile table of
// all resident lattices; every lattice carries its request's step count and
// stops there inside the tick, so one short request does not cut the tick
// for the others.  While a tick runs, the copy stream downloads the results
// of the requests that finished at the previous tick (and frees their pool
// memory) and initialises the newly admitted ones, which join at the next
// tick.  Each lattice's arithmetic is independent of which others share the
// launch, so a result is bit-identical alone and in the mix.  The strip
// geometry is chosen for the resident set whenever it changes
// (choose_geometry): pair strips when every lattice allows them, 60 or 124
// columns wide by the cells either would process.
//
// Resident requests advance in lock step, so a request's latency is its
// step count times the time of one step of the whole resident set.  The
// scheduler therefore bounds the resident set (HBM budget, and optionally a
// cell count) and orders the queue either first-come-first-served or
// shortest-job-first by work (cells x steps); under SJF a full queue sheds
// its largest job rather than refusing a smaller newcomer.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "swb_lattice.h"

using swb::LatticeLayout;
using swb::StepArgs;
using swb::TileRef;

namespace {

struct Req {
    int64_t id = 0;
    swb_params p{};
    std::vector<double> h0;
    double theta0 = 0, dtheta = 0, v = 0;
    int64_t nsteps = 0, done = 0;
    int status = 0;  // 0 queued, 1 running, 2 done, <0 error
    double t_submit = 0, t_admit = 0, t_done = 0;
    double work() const { return (double)p.Lx * p.Ly * (double)nsteps; }
    std::vector<double> result;
    char *dev = nullptr;
    LatticeLayout L{};
    StepArgs a{};
    size_t bytes = 0;
    bool cancel = false;
};

thread_local std::string s_err;
int sfail(int code, const std::string &m) {
    s_err = m;
    swb::set_global_error(m.c_str());
    return code;
}

}  // namespace

struct swb_server {
    size_t budget = 0, in_use = 0;
    int precision = SWB_F32;
    int steps_per_tick = 100;
    int64_t max_queued = 1024;
    int policy = SWB_SCHED_FIFO;
    int64_t max_cells = 0;       // resident cells (0: HBM budget only)
    int64_t resident_cells = 0;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<int64_t> queue;
    std::map<int64_t, std::unique_ptr<Req>> reqs;
    std::vector<Req *> active;
    std::thread worker;
    bool stop = false;
    int64_t next_id = 1;
    cudaStream_t stream = nullptr;  // the ticks
    cudaStream_t copy = nullptr;    // admissions and results, beside the ticks
    cudaMemPool_t pool = nullptr;
    int nt = swb::kBatchNT;         // strip geometry of the resident set (< 0: pair strips)
    int want_nt = 0, want_rows = 0; // swb_server_set_geometry (0: chosen per set), under mu
    bool geometry_dirty = false;    // under mu
    int geo_nt = 0, geo_rows = 0;   // the worker's copy of want_nt / want_rows
    bool fresh_pending = false;     // lattices that joined are at their first iteration
    StepArgs *d_args = nullptr;
    TileRef *d_tiles = nullptr;
    size_t cap_args = 0, cap_tiles = 0;
    int ntiles = 0;
    // pair strips: the one-column strips of the iterations the pair form
    // leaves out (a lattice's first iteration after it joined)
    StepArgs *d_args_fb = nullptr;
    TileRef *d_tiles_fb = nullptr;
    size_t cap_args_fb = 0, cap_tiles_fb = 0;
    int ntiles_fb = 0;
    double *staging = nullptr;
    size_t staging_elems = 0;
    swb_server_stats st{};
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    std::string err;

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

void set_error(swb_server *sv, const std::string &m) {
    std::lock_guard<std::mutex> g(sv->mu);
    sv->err = m;
}

// A failed admission gives the request's pool memory back, so that the
// budget accounting (which treats it as free again) stays true.
void release_device(swb_server *sv, Req *r) {
    if (r->dev) {
        cudaFreeAsync(r->dev, sv->copy);
        cudaStreamSynchronize(sv->copy);
        r->dev = nullptr;
    }
}

// Worker-side, on the copy stream (while a tick runs on the compute stream):
// allocate and initialise a newly admitted request.  Synchronises the copy
// stream, so the lattice is ready before it joins a tick.
bool admit_device(swb_server *sv, Req *r) {
    cudaError_t e = cudaMallocFromPoolAsync((void **)&r->dev, r->bytes, sv->pool, sv->copy);
    if (e != cudaSuccess) {
        r->dev = nullptr;
        set_error(sv, std::string("admit: ") + cudaGetErrorString(e));
        return false;
    }
    // the strip geometry is set again when the lattice joins (choose_geometry)
    r->a = swb::lattice_args(r->p, sv->precision, r->dev, r->L, swb::kBatchNT, swb::kBatchRows);
    r->a.seed = (unsigned long long)r->id;  // thermal noise stream of this request
    r->a.stop_at = r->nsteps;  // its strips stop there, whatever the tick length
    swb::set_wave(r->a, r->theta0, r->dtheta, r->v);
    const long long N = (long long)r->p.Lx * r->p.Ly;
    if ((size_t)N > sv->staging_elems) {
        cudaStreamSynchronize(sv->copy);
        cudaFree(sv->staging);
        sv->staging = nullptr;
        if (cudaMalloc((void **)&sv->staging, (size_t)N * 8) != cudaSuccess) {
            sv->staging = nullptr;
            sv->staging_elems = 0;
            release_device(sv, r);
            set_error(sv, "admit: staging allocation failed");
            return false;
        }
        sv->staging_elems = N;
    }
    e = swb::lattice_init(r->a, sv->precision, r->L, r->h0.data(), sv->copy);
    if (e == cudaSuccess) e = swb::lattice_upload_height(r->a, sv->precision, r->h0.data(), sv->staging, sv->copy);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sv->copy);
    if (e != cudaSuccess) {
        release_device(sv, r);
        set_error(sv, std::string("admit: ") + cudaGetErrorString(e));
        return false;
    }
    return true;
}

// Strip geometry of the resident set, chosen whenever it changes: pair
// strips when every lattice allows them (FP32 arithmetic, even Lx, the
// common τ = 1 step), else one-column strips of kBatchNT threads.  Pair
// strips are about 1.3x faster per cell.  Each strip recomputes 2 columns
// and 2 rows on each side, and the last strip of a lattice is partly empty,
// so the strip width is chosen for the set: 124 columns (64 threads) or 60
// (32 threads), whichever processes fewer cells in all (60-column strips
// waste less on the small lattices a shortest-job-first queue favours).
// Rows are set per lattice to the balanced height of at most 64 rows that
// covers it (a 64-row lattice is one strip, 100 rows two of 50).  Results
// do not depend on the geometry.
constexpr int kServePairRows = 64;
int balanced_rows(int Ly, int cap) {
    const int strips = (Ly + cap - 1) / cap;
    return (Ly + strips - 1) / strips;
}
double padded_cells(const std::vector<Req *> &set, int nt, int cap) {
    const int w = -2 * nt - 4;
    double n = 0.0;
    for (const Req *r : set) {
        const int h = balanced_rows(r->p.Ly, cap);
        n += (double)((r->p.Lx + w - 1) / w) * (w + 4) * (double)((r->p.Ly + h - 1) / h) * (h + 4);
    }
    return n;
}
void choose_geometry(swb_server *sv) {
    bool pair = sv->precision == SWB_F32 || sv->precision == SWB_F16;
    for (Req *r : sv->active) pair = pair && r->p.Lx % 2 == 0 && swb::pair_form_ok(r->a);
    sv->nt = swb::kBatchNT;
    const int cap = sv->geo_rows > 0 ? sv->geo_rows : kServePairRows;
    if (pair)
        sv->nt = sv->geo_nt != 0 ? sv->geo_nt
                                 : (padded_cells(sv->active, -32, cap) < padded_cells(sv->active, -64, cap)
                                        ? -32
                                        : -64);
    for (Req *r : sv->active) {
        const int h = pair ? balanced_rows(r->p.Ly, cap) : std::min(swb::kBatchRows, r->p.Ly);
        swb::set_geometry(r->a, sv->nt, std::max(h, swb::kMinRows));
    }
}

// Packed table of (lattice, strip) entries, the lattices' reducers first.
std::vector<TileRef> tile_table(const std::vector<StepArgs> &args) {
    std::vector<TileRef> tiles, reducers;
    for (size_t i = 0; i < args.size(); ++i) {
        const StepArgs &a = args[i];
        if (swb::needs_partials(a)) reducers.push_back({(int)i, -1, 0});
        for (int ty = 0; ty < a.tiles_y; ++ty)
            for (int tx = 0; tx < a.tiles_x; ++tx) tiles.push_back({(int)i, tx, ty});
    }
    tiles.insert(tiles.begin(), reducers.begin(), reducers.end());
    return tiles;
}

// Device copy of a table on the tick stream, growing its buffer when needed.
template <class T>
bool put_table(swb_server *sv, const std::vector<T> &v, T **d, size_t *cap) {
    if (v.size() > *cap) {
        cudaFree(*d);
        *d = nullptr;
        *cap = std::max<size_t>(v.size(), 2 * *cap);
        if (cudaMalloc((void **)d, *cap * sizeof(T)) != cudaSuccess) {
            *cap = 0;
            return false;
        }
    }
    return cudaMemcpyAsync(*d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, sv->stream) ==
           cudaSuccess;
}

// The tables of the resident set (and, for pair strips, of its one-column
// fallback strips), uploaded on the tick stream.
bool upload_table(swb_server *sv) {
    choose_geometry(sv);
    std::vector<StepArgs> args;
    for (Req *r : sv->active) args.push_back(r->a);
    const std::vector<TileRef> tiles = tile_table(args);
    std::vector<StepArgs> fb;
    std::vector<TileRef> fbt;
    if (sv->nt < 0) {
        for (const StepArgs &a : args) fb.push_back(swb::strip_fallback(a));
        fbt = tile_table(fb);
    }
    if (!put_table(sv, args, &sv->d_args, &sv->cap_args) ||
        !put_table(sv, tiles, &sv->d_tiles, &sv->cap_tiles))
        return false;
    sv->ntiles = (int)tiles.size();
    if (sv->nt < 0) {
        if (!put_table(sv, fb, &sv->d_args_fb, &sv->cap_args_fb) ||
            !put_table(sv, fbt, &sv->d_tiles_fb, &sv->cap_tiles_fb))
            return false;
        sv->ntiles_fb = (int)fbt.size();
    }
    // the copies read the host vectors: wait for them before they go
    return cudaStreamSynchronize(sv->stream) == cudaSuccess;
}

void worker_main(swb_server *sv) {
    cudaSetDevice(sv->device);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sv->device);
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // device time of a tick
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    const int occ1 = swb::batch_blocks_per_sm(sv->precision, swb::kBatchNT);
    std::vector<Req *> joining;  // initialised on the copy stream; join at the next tick
    std::vector<Req *> leaving;  // finished at the last tick; results still to download
    bool changed = false;
    for (;;) {
        std::vector<Req *> admitted;
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv.wait(lk, [&] {
                return sv->stop || !sv->queue.empty() || !sv->active.empty() || !joining.empty() ||
                       !leaving.empty();
            });
            if (sv->stop) break;
            // drop cancelled residents
            for (auto it = sv->active.begin(); it != sv->active.end();) {
                if ((*it)->cancel) {
                    (*it)->status = SWB_ERR_CANCELLED;
                    (*it)->t_done = sv->now();
                    cudaFreeAsync((*it)->dev, sv->stream);
                    (*it)->dev = nullptr;
                    sv->in_use -= (*it)->bytes;
                    sv->resident_cells -= (int64_t)(*it)->p.Lx * (*it)->p.Ly;
                    it = sv->active.erase(it);
                    changed = true;
                } else {
                    ++it;
                }
            }
            // admission: FIFO or shortest job first, while the HBM budget and
            // the resident-cell bound hold (one request may always run alone)
            for (;;) {
                auto pick = sv->queue.end();
                for (auto it = sv->queue.begin(); it != sv->queue.end(); ++it) {
                    Req *q = sv->reqs[*it].get();
                    if (q->cancel) {
                        pick = it;
                        break;
                    }
                    if (sv->policy == SWB_SCHED_FIFO) {
                        pick = it;
                        break;
                    }
                    if (pick == sv->queue.end() || q->work() < sv->reqs[*pick]->work()) pick = it;
                }
                if (pick == sv->queue.end()) break;
                Req *r = sv->reqs[*pick].get();
                if (r->cancel) {
                    r->status = SWB_ERR_CANCELLED;
                    r->t_done = sv->now();
                    sv->queue.erase(pick);
                    continue;
                }
                const int64_t cells = (int64_t)r->p.Lx * r->p.Ly;
                if (sv->in_use + r->bytes > sv->budget) break;
                const bool alone = sv->active.empty() && admitted.empty() && joining.empty();
                if (sv->max_cells > 0 && sv->resident_cells + cells > sv->max_cells && !alone) break;
                sv->queue.erase(pick);
                sv->in_use += r->bytes;
                sv->resident_cells += cells;
                r->status = 1;
                r->t_admit = sv->now();
                admitted.push_back(r);
                sv->st.admitted++;
            }
        }
        // 1. the tick: every resident request advances together (a request
        // whose steps run out stops inside the tick; the tick is as long as
        // the longest remaining request allows, at most steps_per_tick)
        {
            std::lock_guard<std::mutex> g(sv->mu);
            if (sv->geometry_dirty) changed = true;
            sv->geometry_dirty = false;
            sv->geo_nt = sv->want_nt;
            sv->geo_rows = sv->want_rows;
        }
        if (changed && !sv->active.empty() && !upload_table(sv)) {
            set_error(sv, "tile table upload failed");
            std::this_thread::sleep_for(std::chrono::milliseconds(10));
            continue;
        }
        changed = false;
        int64_t tick = 0;
        for (Req *r : sv->active) tick = std::max<int64_t>(tick, r->nsteps - r->done);
        tick = std::min<int64_t>(tick, sv->steps_per_tick);
        const double tb = sv->now();
        cudaError_t e = cudaSuccess;
        if (tick > 0) {
            // the general kernel if any resident request needs it
            bool gen = false, tau1 = true, rare = false, wave = false;
            for (Req *r : sv->active) {
                gen = gen || swb::step_general(r->a);
                rare = rare || swb::step_rare(r->a);
                tau1 = tau1 && r->a.tau_is_one;
                wave = wave || r->a.theta_mode == swb::THETA_WAVE;
            }
            // pair strips: one CTA per table entry (the hardware balances the
            // uneven strips; on GB300 faster than persistent CTAs walking the
            // table); one-column strips: persistent CTAs
            const int grid = sv->nt < 0 ? sv->ntiles : std::min(sv->ntiles, sms * occ1);
            const int grid_fb = std::min(sv->ntiles_fb, sms * occ1);
            cudaEventRecord(ev0, sv->stream);
            for (int64_t k = 0; k < tick && e == cudaSuccess; ++k) {
                const bool steady = tau1 && !(sv->fresh_pending && k == 0);
                if (sv->nt < 0 && !steady)  // an iteration the pair form leaves out
                    e = swb::launch_batch_step(sv->precision, swb::kBatchNT, gen, steady, sv->d_args_fb,
                                               sv->d_tiles_fb, sv->ntiles_fb, grid_fb, (int)k,
                                               sv->stream, rare);
                else if (sv->nt < 0)
                    e = swb::launch_batch_step(sv->precision, sv->nt, wave, steady, sv->d_args,
                                               sv->d_tiles, sv->ntiles, grid, (int)k, sv->stream);
                else
                    e = swb::launch_batch_step(sv->precision, sv->nt, gen, steady, sv->d_args,
                                               sv->d_tiles, sv->ntiles, grid, (int)k, sv->stream, rare);
            }
            if (e == cudaSuccess)
                e = swb::launch_batch_advance(sv->d_args, (int)sv->active.size(), (int)tick, sv->stream);
            cudaEventRecord(ev1, sv->stream);
            sv->fresh_pending = false;
        }
        // 2. while it runs, on the copy stream: the results of the requests
        // that finished at the previous tick, then the new admissions
        for (Req *r : leaving) {
            r->result.resize((size_t)r->p.Lx * r->p.Ly);
            cudaError_t de = swb::lattice_download_height(r->a, sv->precision, false, r->result.data(), sv->copy);
            cudaFreeAsync(r->dev, sv->copy);
            r->dev = nullptr;
            std::lock_guard<std::mutex> g(sv->mu);
            r->status = de == cudaSuccess ? 2 : SWB_ERR_CUDA;
            r->t_done = sv->now();
            sv->in_use -= r->bytes;
            sv->resident_cells -= (int64_t)r->p.Lx * r->p.Ly;
            sv->st.completed++;
            r->h0.clear();
            r->h0.shrink_to_fit();
        }
        leaving.clear();
        for (Req *r : admitted) {
            if (admit_device(sv, r)) {
                joining.push_back(r);
            } else {
                std::lock_guard<std::mutex> g(sv->mu);
                r->status = SWB_ERR_OOM;
                r->t_done = sv->now();
                sv->in_use -= r->bytes;
                sv->resident_cells -= (int64_t)r->p.Lx * r->p.Ly;
                sv->st.rejected++;
            }
        }
        // 3. the end of the tick
        if (tick > 0 && e == cudaSuccess) e = cudaStreamSynchronize(sv->stream);
        {
            std::lock_guard<std::mutex> g(sv->mu);
            double lu = 0.0;
            for (Req *r : sv->active) {
                const int64_t n = std::min<int64_t>(tick, r->nsteps - r->done);
                r->done += n;
                lu += (double)r->p.Lx * r->p.Ly * (double)n;
                if (r->done >= r->nsteps) {
                    leaving.push_back(r);
                    if (e != cudaSuccess) r->status = SWB_ERR_CUDA;
                }
            }
            if (!leaving.empty()) {
                sv->active.erase(std::remove_if(sv->active.begin(), sv->active.end(),
                                                [](Req *r) { return r->done >= r->nsteps; }),
                                 sv->active.end());
                changed = true;
            }
            if (!joining.empty()) {
                sv->active.insert(sv->active.end(), joining.begin(), joining.end());
                joining.clear();
                sv->fresh_pending = true;
                changed = true;
            }
            sv->st.lattice_updates += lu;
            if (tick > 0) {
                sv->st.busy_seconds += sv->now() - tb;
                sv->st.ticks++;
                float ms = 0.f;
                if (e == cudaSuccess && cudaEventElapsedTime(&ms, ev0, ev1) == cudaSuccess)
                    sv->st.device_seconds += ms * 1e-3;
            }
            if (e != cudaSuccess) sv->err = std::string("tick: ") + cudaGetErrorString(e);
        }
    }
    cudaStreamSynchronize(sv->stream);
    cudaStreamSynchronize(sv->copy);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
}

}  // namespace

extern "C" {

int swb_server_create(size_t hbm_budget, int precision, int steps_per_tick, swb_server **out) {
    if (!out || hbm_budget == 0 || steps_per_tick < 1) return sfail(SWB_ERR_ARG, "bad arguments");
    if (precision != SWB_F64 && precision != SWB_F32 && precision != SWB_F16)
        return sfail(SWB_ERR_ARG, "server precision must be SWB_F64, SWB_F32 or SWB_F16");
    *out = nullptr;
    swb_server *sv = new swb_server();
    sv->budget = hbm_budget;
    sv->precision = precision;
    sv->steps_per_tick = steps_per_tick;
    cudaGetDevice(&sv->device);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = sv->device;
    cudaError_t e = cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sv->copy, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMemPoolCreate(&sv->pool, &props);
    if (e == cudaSuccess) {
        uint64_t thr = UINT64_MAX;  // keep freed blocks cached in this pool
        e = cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    if (e != cudaSuccess) {
        if (sv->stream) cudaStreamDestroy(sv->stream);
        if (sv->copy) cudaStreamDestroy(sv->copy);
        delete sv;
        return sfail(SWB_ERR_CUDA, std::string("server create: ") + cudaGetErrorString(e));
    }
    sv->st.hbm_budget = hbm_budget;
    sv->worker = std::thread(worker_main, sv);
    *out = sv;
    return SWB_OK;
}

int swb_server_destroy(swb_server *sv) {
    if (!sv) return SWB_OK;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->stop = true;
    }
    sv->cv.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    cudaStreamSynchronize(sv->copy);
    for (auto &kv : sv->reqs)
        if (kv.second->dev) cudaFreeAsync(kv.second->dev, sv->stream);
    cudaStreamSynchronize(sv->stream);
    cudaFree(sv->d_args);
    cudaFree(sv->d_tiles);
    cudaFree(sv->d_args_fb);
    cudaFree(sv->d_tiles_fb);
    cudaFree(sv->staging);
    if (sv->pool) cudaMemPoolDestroy(sv->pool);
    cudaStreamDestroy(sv->stream);
    cudaStreamDestroy(sv->copy);
    delete sv;
    return SWB_OK;
}

int swb_server_submit(swb_server *sv, const swb_params *p, const double *h0, double theta0,
                      double dtheta, double v, int64_t nsteps, int64_t *id) {
    if (!sv || !p || !h0 || !id || nsteps < 1) return sfail(SWB_ERR_ARG, "bad arguments");
    if (p->Lx < 1 || p->Ly < 1 || 9LL * (((long long)p->Lx * p->Ly + 63) / 64 * 64) >= (1LL << 31) || !(p->tau > 0) ||
        p->n <= p->m || p->m < 1 || !(p->hmin > 0))
        return sfail(SWB_ERR_ARG, "invalid params");
    if (!(p->kbt >= 0.0)) return sfail(SWB_ERR_ARG, "kbt must be >= 0");
    const double work = (double)p->Lx * p->Ly * (double)nsteps;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        if ((int64_t)sv->queue.size() >= sv->max_queued) {
            // SJF sheds the largest queued job if the newcomer is smaller
            auto big = sv->queue.end();
            if (sv->policy == SWB_SCHED_SJF)
                for (auto it = sv->queue.begin(); it != sv->queue.end(); ++it)
                    if (big == sv->queue.end() || sv->reqs[*it]->work() > sv->reqs[*big]->work())
                        big = it;
            if (big == sv->queue.end() || sv->reqs[*big]->work() <= work) {
                sv->st.submitted++;
                sv->st.rejected++;
                return sfail(SWB_ERR_BUSY, "request queue full");
            }
            Req *victim = sv->reqs[*big].get();
            victim->status = SWB_ERR_BUSY;
            victim->t_done = sv->now();
            victim->h0.clear();
            victim->h0.shrink_to_fit();
            sv->st.rejected++;
            sv->queue.erase(big);
        }
    }
    auto r = std::make_unique<Req>();
    r->p = *p;
    r->h0.assign(h0, h0 + (size_t)p->Lx * p->Ly);
    r->theta0 = theta0;
    r->dtheta = dtheta;
    r->v = v;
    r->nsteps = nsteps;
    r->L = swb::lattice_layout(*p, sv->precision);
    r->bytes = r->L.total;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        r->t_submit = sv->now();
        r->id = sv->next_id++;
        *id = r->id;
        sv->st.submitted++;
        if (r->bytes > sv->budget) {
            r->status = SWB_ERR_OOM;
            r->t_done = r->t_submit;
            sv->st.rejected++;
        } else {
            sv->queue.push_back(r->id);
        }
        sv->reqs[r->id] = std::move(r);
    }
    sv->cv.notify_all();
    return SWB_OK;
}

int swb_server_set_queue_limit(swb_server *sv, int64_t max_queued) {
    if (!sv || max_queued < 1) return sfail(SWB_ERR_ARG, "bad arguments");
    std::lock_guard<std::mutex> g(sv->mu);
    sv->max_queued = max_queued;
    return SWB_OK;
}

int swb_server_set_geometry(swb_server *sv, int nt, int rows) {
    if (!sv || (nt != 0 && nt != -32 && nt != -64) || (rows != 0 && rows < swb::kMinRows) ||
        (nt != 0 && rows == 0))
        return sfail(SWB_ERR_ARG, "bad arguments");
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->want_nt = nt;
        sv->want_rows = rows;
        sv->geometry_dirty = true;
    }
    sv->cv.notify_all();
    return SWB_OK;
}

int swb_server_set_policy(swb_server *sv, int policy, int64_t max_resident_cells) {
    if (!sv || (policy != SWB_SCHED_FIFO && policy != SWB_SCHED_SJF) || max_resident_cells < 0)
        return sfail(SWB_ERR_ARG, "bad arguments");
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->policy = policy;
        sv->max_cells = max_resident_cells;
    }
    sv->cv.notify_all();
    return SWB_OK;
}

int swb_server_poll(swb_server *sv, int64_t id, double *h_out, swb_request_info *info) {
    if (!sv) return sfail(SWB_ERR_ARG, "server is NULL");
    std::lock_guard<std::mutex> g(sv->mu);
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return sfail(SWB_ERR_NOT_FOUND, "unknown request id");
    Req *r = it->second.get();
    if (info) {
        info->id = r->id;
        info->status = r->status;
        info->steps_done = r->done;
        info->t_submit = r->t_submit;
        info->t_admit = r->t_admit;
        info->t_done = r->t_done;
    }
    if (r->status == 2) {
        if (h_out) std::copy(r->result.begin(), r->result.end(), h_out);
        return 1;
    }
    if (r->status < 0) return r->status;
    return 0;
}

int swb_server_cancel(swb_server *sv, int64_t id) {
    if (!sv) return sfail(SWB_ERR_ARG, "server is NULL");
    {
        std::lock_guard<std::mutex> g(sv->mu);
        auto it = sv->reqs.find(id);
        if (it == sv->reqs.end()) return sfail(SWB_ERR_NOT_FOUND, "unknown request id");
        it->second->cancel = true;
    }
    sv->cv.notify_all();
    return SWB_OK;
}

int swb_server_stats_get(swb_server *sv, swb_server_stats *out) {
    if (!sv || !out) return sfail(SWB_ERR_ARG, "bad arguments");
    std::lock_guard<std::mutex> g(sv->mu);
    *out = sv->st;
    out->queued = (int64_t)sv->queue.size();
    out->running = (int64_t)sv->active.size();
    out->hbm_in_use = sv->in_use;
    out->hbm_budget = sv->budget;
    return SWB_OK;
}

double swb_server_clock(swb_server *sv) { return sv ? sv->now() : 0.0; }

}  // extern "C"
