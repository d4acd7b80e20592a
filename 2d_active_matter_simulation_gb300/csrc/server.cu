// Serving engine: simulation requests in, results out, with continuous
// batching on one GPU.
//
// The reference runs one simulation per process, start to finish
// (ActFlow_V3-2.cu:214-878).  A server takes requests -- grid, parameters,
// precision, seed or initial state, step count -- from any thread and runs
// many of them at once:
//
//  * admission (thread "admit"): pending requests are admitted in arrival
//    order (or shortest job first) while their device footprint fits the HBM
//    budget and an active slot is free.  FP64 and double-float requests
//    (about 20 and 5 times the GPU time of an FP32 request of the same size)
//    share a lane of their own: at most max_active_fp64 of them are active at
//    once, and a request waiting for that lane does not hold back the FP32
//    requests behind it.  Admission creates the request's
//    handle, builds its initial field (the seeded band-limited generator or
//    the caller's state) and loads it.  Finished handles are destroyed on this
//    thread too (stream-ordered frees: no wait for other requests' work).
//  * chunks: about 20 ms of estimated GPU time each (at most chunk_steps), so
//    a large FP64 request advances in short chunks like everything else.
//  * scheduling (thread "run"): every active request keeps up to two chunks of
//    steps in flight on its own stream (one CUDA graph replay per step), so
//    the kernels of different requests overlap on the device.  Streams carry
//    priorities by request size, so the blocks of small requests are
//    dispatched ahead of the queued blocks of large ones; a completed
//    chunk's energies and NaN probe are harvested, and the next chunk is
//    enqueued at once.  A request whose last chunk completed has its state
//    copied out and becomes a result.
//
// Requests that arrive while others run are admitted as soon as memory and a
// slot free up; nothing waits for a batch boundary.  Each request computes
// exactly what a lone handle computes: the same kernels, the same per-handle
// state and stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "actflow.h"
#include "handle_internal.h"
#include "step_kernels.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Chunk {
    int k = 0;
    double *energy = nullptr;      // pinned, chunk capacity
    af::Scalars *sc = nullptr;     // pinned
    cudaEvent_t done = nullptr;
    bool busy = false;
};

struct Job {
    long long id = 0;
    am_job spec{};
    std::vector<unsigned char> w0;  // caller's initial state (copied at submit) or empty
    long long footprint = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    am_handle *h = nullptr;
    cudaStream_t stream = nullptr;  // created by the server with the request's priority
    Chunk ch[2];
    int next = 0;                   // chunk slot to enqueue next
    long long enqueued = 0, harvested = 0;
    std::vector<double> energy;
    std::vector<unsigned char> state;
    double mean[2] = {0, 0};
    int chunk = 0;                  // steps per chunk for this request
    am_status status = AM_OK;
    std::string err;
    bool finished = false;
};

size_t state_bytes(const am_params &p)
{
    return (size_t)p.ny * (p.nx / 2 + 1) * (p.precision != AM_FP32 ? 16 : 8);
}

}  // namespace

struct am_server {
    am_server_config cfg{};
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_admit, cv_run, cv_done;
    std::deque<std::shared_ptr<Job>> pending;
    std::vector<std::shared_ptr<Job>> ready;       // admitted, not yet picked up by the scheduler
    std::vector<std::shared_ptr<Job>> reap;        // finished: handles to destroy
    std::map<long long, std::shared_ptr<Job>> results;
    long long next_id = 1;
    long long used = 0;                            // reserved device bytes
    int active = 0;                                // admitted and not yet reaped
    int active_fp64 = 0;                           // of which FP64 or double-float
    bool stop = false;
    long long gps_done = 0, jobs_done = 0, peak_used = 0;
    int peak_active = 0;
    std::vector<Chunk> chunk_pool;                 // pinned chunk buffers of finished requests
    std::thread admit_thr, run_thr;
    int device = 0;
    int prio_least = 0, prio_greatest = 0;   // cudaDeviceGetStreamPriorityRange

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void free_chunk(Chunk &c)
{
    if (c.energy) cudaFreeHost(c.energy);
    if (c.sc) cudaFreeHost(c.sc);
    if (c.done) cudaEventDestroy(c.done);
    c = Chunk{};
}

// Steps per chunk: about 20 ms of estimated GPU time (at most the configured
// chunk), so that a chunk of a large request never holds the host for long.
// Estimated step time per grid point on this GPU: 7e-8 ms FP32, 1.5e-6 ms FP64,
// 3.5e-7 ms double-float.
int chunk_steps_for(const am_server *s, const am_params &p)
{
    const double per = p.precision == AM_FP64 ? 1.5e-6 : p.precision == AM_DF64 ? 3.5e-7 : 7e-8;
    const double ms = (double)p.nx * p.ny * per;
    const double k = 20.0 / (ms > 0 ? ms : 1.0);
    return k >= s->cfg.chunk_steps ? s->cfg.chunk_steps : k < 1.0 ? 1 : (int)k;
}

// Work of a request in FP32 grid-point-steps (an FP64 step costs about 20
// FP32 steps of the same grid on this GPU, a double-float step about 5).
double work_of(const am_job &j)
{
    const double f = j.params.precision == AM_FP64 ? 20.0 : j.params.precision == AM_DF64 ? 5.0 : 1.0;
    return (double)j.params.nx * j.params.ny * (double)j.nsteps * f;
}

// Requests that take the FP64 lane: the 8-byte precisions.
bool in_fp64_lane(const am_params &p) { return p.precision != AM_FP32; }

// Stream priority of a request: one level per factor 10 of work above 1e8
// grid-point-steps, the least work on the greatest priority.  The block
// scheduler dispatches pending blocks of higher-priority streams first, so a
// small request's kernels do not queue behind the blocks of a large one.
int priority_of(const am_server *s, const am_job &j)
{
    const int levels = s->prio_least - s->prio_greatest;   // e.g. 0 - (-5) = 5
    double w = work_of(j);
    int lvl = 0;
    while (w > 1e8 && lvl < levels) {
        w /= 10.0;
        lvl++;
    }
    return s->prio_greatest + lvl;
}

// Create the handle on a stream of the request's priority, load the initial
// state and allocate the chunk buffers.
am_status prepare(am_server *s, Job &j)
{
    const am_params &p = j.spec.params;
    am_status st = am_create(&p, &j.h);
    if (st) {
        j.err = "am_create failed";
        return st;
    }
    if (cudaStreamCreateWithPriority(&j.stream, cudaStreamNonBlocking, priority_of(s, j.spec)) != cudaSuccess) {
        j.stream = nullptr;
        j.err = "stream creation failed";
        return AM_ERR_CUDA;
    }
    st = am_set_stream(j.h, j.stream);
    if (st) {
        j.err = am_last_error(j.h);
        return st;
    }
    if (!j.w0.empty()) {
        st = am_set_state(j.h, j.w0.data(), j.spec.mean);
        std::vector<unsigned char>().swap(j.w0);
    } else {
        std::vector<double> w((size_t)p.ny * (p.nx / 2 + 1) * 2);
        st = am_ic_bandlimited(p.nx, p.ny, j.spec.seed, j.spec.kmin, j.spec.kmax, j.spec.rms, w.data());
        if (!st) {
            if (p.precision != AM_FP32) {   // FP64, double-float: double on the host
                st = am_set_state(j.h, w.data(), j.spec.mean);
            } else {
                std::vector<float> f(w.size());
                for (size_t i = 0; i < w.size(); i++) f[i] = (float)w[i];
                st = am_set_state(j.h, f.data(), j.spec.mean);
            }
        }
    }
    if (st) {
        j.err = std::string("initial state: ") + am_last_error(j.h);
        return st;
    }
    // pinned chunk buffers: reused from finished requests, else allocated
    const int cap = s->cfg.chunk_steps;
    for (Chunk &c : j.ch) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (!s->chunk_pool.empty()) {
                c = s->chunk_pool.back();
                s->chunk_pool.pop_back();
                continue;
            }
        }
        if (cudaMallocHost((void **)&c.energy, cap * sizeof(double)) != cudaSuccess ||
            cudaMallocHost((void **)&c.sc, sizeof(af::Scalars)) != cudaSuccess ||
            cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming) != cudaSuccess) {
            j.err = "pinned host buffers";
            return AM_ERR_OOM;
        }
    }
    j.chunk = chunk_steps_for(s, p);
    if (j.spec.want_energy) j.energy.reserve((size_t)j.spec.nsteps);
    return AM_OK;
}

void admit_loop(am_server *s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        // destroy finished handles first: it frees memory for admission
        while (!s->reap.empty()) {
            std::shared_ptr<Job> j = s->reap.back();
            s->reap.pop_back();
            lk.unlock();
            if (j->h) am_destroy(j->h);
            j->h = nullptr;
            if (j->stream) cudaStreamDestroy(j->stream);
            j->stream = nullptr;
            lk.lock();
            for (Chunk &c : j->ch) {
                if (c.energy && c.sc && c.done) {
                    c.busy = false;
                    s->chunk_pool.push_back(c);
                } else {
                    free_chunk(c);
                }
                c = Chunk{};
            }
            s->used -= j->footprint;
            s->active--;
            if (in_fp64_lane(j->spec.params)) s->active_fp64--;
        }
        if (s->stop && s->pending.empty() && s->active == 0) return;
        // pick the next request that may be admitted
        // (FP64-lane requests are passed over while the lane is full; the first request
        // that may take a slot is then admitted only if its footprint fits,
        // so a large request is not overtaken indefinitely by smaller ones)
        auto pick = s->pending.end();
        if (!s->pending.empty() && s->active < s->cfg.max_active) {
            const bool lane64 = s->active_fp64 < s->cfg.max_active_fp64;
            auto eligible = [&](const std::shared_ptr<Job> &j) {
                return lane64 || !in_fp64_lane(j->spec.params);
            };
            if (s->cfg.order == AM_ORDER_SHORTEST_FIRST) {
                for (auto it = s->pending.begin(); it != s->pending.end(); ++it)
                    if (eligible(*it) && (pick == s->pending.end() || work_of((*it)->spec) < work_of((*pick)->spec)))
                        pick = it;
            } else {
                pick = std::find_if(s->pending.begin(), s->pending.end(), eligible);
            }
            if (pick != s->pending.end() && s->used + (*pick)->footprint > s->cfg.hbm_budget_bytes && s->active > 0)
                pick = s->pending.end();
        }
        if (pick == s->pending.end()) {
            s->cv_admit.wait(lk);
            continue;
        }
        std::shared_ptr<Job> j = *pick;
        s->pending.erase(pick);
        s->used += j->footprint;
        s->active++;
        if (in_fp64_lane(j->spec.params)) s->active_fp64++;
        s->peak_used = std::max(s->peak_used, s->used);
        s->peak_active = std::max(s->peak_active, s->active);
        lk.unlock();
        const am_status st = prepare(s, *j);
        lk.lock();
        j->t_admit = s->now();
        if (st) {
            j->status = st;
            j->finished = true;
            j->t_done = j->t_admit;
            s->results[j->id] = j;
            s->reap.push_back(j);
            s->cv_done.notify_all();
            continue;
        }
        s->ready.push_back(j);
        s->cv_run.notify_all();
    }
}

// Enqueue the next chunk of a job if it has steps left and a free chunk slot.
bool feed(am_server *s, Job &j)
{
    Chunk &c = j.ch[j.next];
    if (c.busy || j.enqueued >= j.spec.nsteps || j.status != AM_OK) return false;
    const int k = (int)std::min<long long>(j.chunk, j.spec.nsteps - j.enqueued);
    const am_status st = af::handle_enqueue_chunk(j.h, k, j.spec.want_energy ? c.energy : nullptr, c.sc, c.done);
    if (st) {
        j.status = st;
        j.err = am_last_error(j.h);
        return false;
    }
    c.busy = true;
    c.k = k;
    j.enqueued += k;
    j.next ^= 1;
    return true;
}

// Harvest the oldest chunk if it completed.  Returns true if it did.
bool harvest(Job &j)
{
    Chunk &c = j.ch[j.next];   // with two slots the oldest in flight is the one fed next
    Chunk &o = c.busy ? c : j.ch[j.next ^ 1];
    if (!o.busy) return false;
    if (cudaEventQuery(o.done) != cudaSuccess) return false;
    if (j.spec.want_energy) j.energy.insert(j.energy.end(), o.energy, o.energy + o.k);
    if (o.sc->nan_step >= 0 && j.status == AM_OK) {
        j.status = AM_ERR_NAN;
        j.err = "w(0,0) is NaN after step " + std::to_string(j.harvested + o.sc->nan_step);
    }
    if (o.sc->status != 0 && j.status == AM_OK) {
        j.status = AM_ERR_TIMEOUT;
        j.err = "a row pass's tensor-map copies did not complete in time";
    }
    j.harvested += o.k;
    o.busy = false;
    return true;
}

void run_loop(am_server *s)
{
    cudaSetDevice(s->device);
    std::vector<std::shared_ptr<Job>> act;
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (act.empty() && s->ready.empty()) {
                if (s->stop && s->pending.empty() && s->active == 0) return;
                s->cv_run.wait_for(lk, std::chrono::milliseconds(50));
            }
            for (auto &j : s->ready) act.push_back(j);
            s->ready.clear();
        }
        bool progress = false;
        for (auto &j : act) {
            progress |= feed(s, *j);
            progress |= feed(s, *j);
        }
        for (size_t i = 0; i < act.size();) {
            Job &j = *act[i];
            while (harvest(j)) {
                progress = true;
                feed(s, j);
            }
            const bool inflight = j.ch[0].busy || j.ch[1].busy;
            if (!inflight && (j.harvested >= j.spec.nsteps || j.status != AM_OK)) {
                if (j.status == AM_OK) {
                    if (j.spec.want_state) j.state.resize(state_bytes(j.spec.params));
                    const am_status st = am_get_state(j.h, j.spec.want_state ? j.state.data() : nullptr, j.mean);
                    if (st) {
                        j.status = st;
                        j.err = am_last_error(j.h);
                    }
                }
                std::lock_guard<std::mutex> lk(s->mu);
                j.t_done = s->now();
                j.finished = true;
                if (j.status == AM_OK) {
                    s->jobs_done++;
                    s->gps_done += (long long)j.spec.params.nx * j.spec.params.ny * j.spec.nsteps;
                }
                s->results[j.id] = act[i];
                s->reap.push_back(act[i]);
                s->cv_done.notify_all();
                s->cv_admit.notify_all();
                act.erase(act.begin() + i);
                progress = true;
                continue;
            }
            i++;
        }
        if (!progress && !act.empty()) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

}  // namespace

extern "C" {

am_status am_server_create(const am_server_config *cfg, am_server **out)
{
    if (!out) return AM_ERR_ARG;
    *out = nullptr;
    am_server_config c{};
    if (cfg) c = *cfg;
    if (c.hbm_budget_bytes <= 0) c.hbm_budget_bytes = 180LL << 30;
    if (c.max_active <= 0) c.max_active = 16;
    if (c.max_active_fp64 <= 0) c.max_active_fp64 = (c.max_active + 3) / 4;
    if (c.max_active_fp64 > c.max_active) c.max_active_fp64 = c.max_active;
    if (c.chunk_steps <= 0) c.chunk_steps = 256;
    if (c.chunk_steps > af::handle_ring_capacity()) c.chunk_steps = af::handle_ring_capacity();
    if (c.order != AM_ORDER_ARRIVAL && c.order != AM_ORDER_SHORTEST_FIRST) return AM_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return AM_ERR_CUDA;
    am_server *s = new (std::nothrow) am_server();
    if (!s) return AM_ERR_OOM;
    s->cfg = c;
    s->t0 = Clock::now();
    cudaGetDevice(&s->device);
    if (cudaDeviceGetStreamPriorityRange(&s->prio_least, &s->prio_greatest) != cudaSuccess)
        s->prio_least = s->prio_greatest = 0;
    s->admit_thr = std::thread(admit_loop, s);
    s->run_thr = std::thread(run_loop, s);
    *out = s;
    return AM_OK;
}

am_status am_server_submit(am_server *s, const am_job *job, long long *id)
{
    if (!s || !job) return AM_ERR_ARG;
    const am_params &p = job->params;
    const long long fp = am_footprint_bytes(&p);
    if (fp < 0 || p.nx < 8 || p.ny < 8 || p.nx > 4096 || p.ny > 4096) return AM_ERR_UNSUPPORTED;
    if (job->nsteps < 0 || (p.precision != AM_FP32 && p.precision != AM_FP64 && p.precision != AM_DF64))
        return AM_ERR_ARG;
    auto j = std::make_shared<Job>();
    j->spec = *job;
    j->footprint = fp;
    if (job->w_hat) {
        const unsigned char *src = static_cast<const unsigned char *>(job->w_hat);
        j->w0.assign(src, src + state_bytes(p));
        j->spec.w_hat = nullptr;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return AM_ERR_ARG;
    if (fp > s->cfg.hbm_budget_bytes) return AM_ERR_OOM;
    j->id = s->next_id++;
    j->t_submit = s->now();
    if (id) *id = j->id;
    s->pending.push_back(j);
    s->cv_admit.notify_all();
    return AM_OK;
}

am_status am_server_wait(am_server *s, long long id, double timeout_s, am_job_result *res, void *w_hat,
                         double *energy)
{
    if (!s) return AM_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (id <= 0 || id >= s->next_id) return AM_ERR_ARG;
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                             std::chrono::duration<double>(timeout_s < 0 ? 1e9 : timeout_s));
    for (;;) {
        auto it = s->results.find(id);
        if (it != s->results.end()) {
            std::shared_ptr<Job> j = it->second;
            s->results.erase(it);
            lk.unlock();
            if (res) {
                std::memset(res, 0, sizeof(*res));
                res->id = j->id;
                res->status = j->status;
                res->t_submit = j->t_submit;
                res->t_admit = j->t_admit;
                res->t_done = j->t_done;
                res->mean[0] = j->mean[0];
                res->mean[1] = j->mean[1];
                res->steps_done = j->harvested;
                std::strncpy(res->error, j->err.c_str(), sizeof(res->error) - 1);
            }
            if (w_hat && !j->state.empty()) std::memcpy(w_hat, j->state.data(), j->state.size());
            if (energy && !j->energy.empty()) std::memcpy(energy, j->energy.data(), j->energy.size() * sizeof(double));
            return j->status;
        }
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !s->results.count(id))
            return AM_ERR_TIMEOUT;
    }
}

am_status am_server_stats(am_server *s, am_server_info *out)
{
    if (!s || !out) return AM_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->elapsed_s = s->now();
    out->jobs_submitted = s->next_id - 1;
    out->jobs_done = s->jobs_done;
    out->jobs_pending = (long long)s->pending.size();
    out->jobs_active = s->active;
    out->grid_point_steps = s->gps_done;
    out->device_bytes_reserved = s->used;
    out->peak_device_bytes = s->peak_used;
    out->peak_active = s->peak_active;
    return AM_OK;
}

am_status am_server_destroy(am_server *s)
{
    if (!s) return AM_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_admit.notify_all();
        s->cv_run.notify_all();
    }
    if (s->run_thr.joinable()) s->run_thr.join();
    if (s->admit_thr.joinable()) s->admit_thr.join();
    for (Chunk &c : s->chunk_pool) free_chunk(c);
    delete s;
    return AM_OK;
}

}  // extern "C"
