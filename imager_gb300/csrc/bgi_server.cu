// Serving runtime: a request loop over the imager handles (no counterpart in the reference,
// whose imager images one block per call on the default stream).
//
// Callers register arrays once (their UVW, flags, cable lengths and frequencies stay resident
// on the device) and submit blocks of visibilities in host memory as they arrive.  One
// scheduler thread makes every CUDA call: it admits queued requests in arrival order while a
// slot (a stream with its own imager handles) is free and the request's device buffers fit
// both the byte budget and the device's free memory, then issues the upload, the imaging and
// the download on the slot's stream.  Requests on different slots overlap on the GPU; a
// request that arrives while others run is admitted as soon as a slot and memory free up
// (continuous batching rather than a queue drained one block at a time).  A host callback on
// the stream stamps each completion; latency is submit-to-completion.
#include <algorithm>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "bgi_internal.h"

using bgi::check_cuda;
using bgi::set_error;
using bgi::vis_blocks;

namespace {

using Clock = std::chrono::steady_clock;

struct ArrayState {  // host copy of an array's state, from which each slot makes its handle
    bgi_config cfg{};
    int n_ant = 0, n_uvw_sets = 0, n_channels = 0;
    long long n_baselines = 0;
    std::vector<float> u, v, w;
    std::vector<int> flags;
    std::vector<double> cable, freqs;
};

struct Request {
    uint64_t ticket = 0;
    int array_id = 0, format = BGI_VIS_C64, n_intervals = 0;
    unsigned flags = 0;
    const void *vis = nullptr;
    const float *scales = nullptr;
    float *images = nullptr;
    size_t vis_bytes = 0, scale_bytes = 0, img_bytes = 0;  // device bytes while running
    int n_images = 0;
    Clock::time_point t_submit, t_done;
    int status = 1;  // 1 pending/running, then BGI_OK or an error status
    std::string error;
    int slot = -1;
    void *d_vis = nullptr, *d_scales = nullptr, *d_img = nullptr;
    struct bgi_server *server = nullptr;
    std::shared_ptr<const ArrayState> array;  // the array's state, fixed at submission
    size_t device_bytes() const { return vis_bytes + scale_bytes + img_bytes; }
};

struct Slot {
    cudaStream_t stream = nullptr;
    bool busy = false;
    std::unordered_map<int, bgi_imager *> handles;  // array id -> this slot's handle
};

// pol planes a block-scaled request must upload (XX=0, XY=1, YX=2, YY=3)
int needed_planes(int pol, int planes[2]) {
    switch (pol) {
        case BGI_POL_XX: planes[0] = 0; return 1;
        case BGI_POL_YY: planes[0] = 3; return 1;
        case BGI_POL_I: planes[0] = 0, planes[1] = 3; return 2;
        default: planes[0] = 1, planes[1] = 2; return 2;
    }
}

}  // namespace

struct bgi_server {
    bgi_server_config cfg{};
    size_t budget = 0, in_use = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> requests;
    std::vector<std::shared_ptr<Request>> completed;  // stamped by stream callbacks, not yet retired
    std::vector<std::shared_ptr<const ArrayState>> arrays;  // appended under mu, never changed
    std::vector<Slot> slots;
    std::thread worker;
    bool stop = false;
    uint64_t next_ticket = 1;
    // statistics since the last reset
    std::vector<double> latencies_ms;
    uint64_t n_submitted = 0, n_completed = 0, n_failed = 0, n_images = 0, n_admission_waits = 0;
    uint64_t n_rejected = 0, n_cancelled = 0;
    Clock::time_point t_first_submit, t_last_done;
    bool any_submit = false;

    // ---- scheduler thread ---------------------------------------------------------------
    static void CUDART_CB on_stream_done(void *arg) {
        // runs on a CUDA callback thread: no CUDA calls here
        Request *r = static_cast<Request *>(arg);
        bgi_server *sv = r->server;
        std::lock_guard<std::mutex> lk(sv->mu);
        r->t_done = Clock::now();
        sv->completed.push_back(sv->requests.at(r->ticket));
        sv->cv_work.notify_one();
    }

    int free_slot() const {
        for (size_t i = 0; i < slots.size(); ++i)
            if (!slots[i].busy) return (int)i;
        return -1;
    }

    // true when the front request fits the budget (the caller also checks free device memory)
    bool front_fits() const { return !queue.empty() && in_use + queue.front()->device_bytes() <= budget; }

    void finish(const std::shared_ptr<Request> &r, int status, const char *msg) {
        // mu held
        r->status = status;
        if (status != BGI_OK) {
            r->error = msg ? msg : "";
            if (status != BGI_ERR_CANCELLED) ++n_failed;
        } else {
            latencies_ms.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
            n_images += (uint64_t)r->n_images;
            t_last_done = r->t_done;
        }
        ++n_completed;
        cv_done.notify_all();
    }

    bgi_imager *handle_for(Slot &slot, int array_id, const ArrayState &a, int *st) {
        auto it = slot.handles.find(array_id);
        if (it != slot.handles.end()) return it->second;
        bgi_imager *h = nullptr;
        *st = bgi_create(&a.cfg, &h);
        if (*st == BGI_OK)
            *st = bgi_set_array(h, a.n_ant, a.n_uvw_sets, a.u.data(), a.v.data(), a.w.empty() ? nullptr : a.w.data(),
                                a.flags.data(), a.cable.empty() ? nullptr : a.cable.data());
        if (*st == BGI_OK) *st = bgi_set_frequencies(h, a.n_channels, a.freqs.data());
        if (*st == BGI_OK) *st = bgi_set_deterministic(h, cfg.deterministic);
        if (*st != BGI_OK) {
            bgi_destroy(h);
            return nullptr;
        }
        slot.handles[array_id] = h;
        return h;
    }

    // Issues one admitted request on its slot's stream (outside mu).
    int launch(Request &r) {
        nvtxRangePushA("bgi_server request");
        const int st = launch_request(r);
        nvtxRangePop();
        return st;
    }

    int launch_request(Request &r) {
        Slot &slot = slots[(size_t)r.slot];
        cudaStream_t s = slot.stream;
        int st = BGI_OK;
        const ArrayState &a = *r.array;
        bgi_imager *h = handle_for(slot, r.array_id, a, &st);
        if (!h) return st;
        if ((st = check_cuda(cudaMallocAsync(&r.d_vis, r.vis_bytes, s), "server: visibility buffer"))) return st;
        if (r.scale_bytes && (st = check_cuda(cudaMallocAsync(&r.d_scales, r.scale_bytes, s), "server: scale buffer")))
            return st;
        if ((st = check_cuda(cudaMallocAsync(&r.d_img, r.img_bytes, s), "server: image buffer"))) return st;
        if (r.format == BGI_VIS_C64) {
            st = check_cuda(cudaMemcpyAsync(r.d_vis, r.vis, r.vis_bytes, cudaMemcpyHostToDevice, s), "server: H2D");
        } else {
            // only the pol planes this array's pol needs, and their scales
            const size_t nb = (size_t)a.n_baselines, nblk = (size_t)vis_blocks(a.n_baselines);
            const size_t rows = (size_t)r.n_intervals * a.n_channels;
            int planes[2];
            const int np = needed_planes(a.cfg.pol, planes);
            for (int q = 0; !st && q < np; ++q) {
                const size_t off = (size_t)planes[q] * nb * 4, soff = (size_t)planes[q] * nblk * 4;
                st = check_cuda(cudaMemcpy2DAsync(static_cast<char *>(r.d_vis) + off, 16 * nb,
                                                  static_cast<const char *>(r.vis) + off, 16 * nb, 4 * nb, rows,
                                                  cudaMemcpyHostToDevice, s),
                                "server: H2D planes");
                if (!st)
                    st = check_cuda(cudaMemcpy2DAsync(static_cast<char *>(r.d_scales) + soff, 16 * nblk,
                                                      reinterpret_cast<const char *>(r.scales) + soff, 16 * nblk,
                                                      4 * nblk, rows, cudaMemcpyHostToDevice, s),
                                    "server: H2D scales");
            }
        }
        if (st) return st;
        st = r.format == BGI_VIS_C64
                 ? bgi_image(h, static_cast<const float *>(r.d_vis), r.n_intervals, r.flags,
                             static_cast<float *>(r.d_img), s)
                 : bgi_image_compressed(h, r.format, r.d_vis, static_cast<const float *>(r.d_scales), r.n_intervals,
                                        r.flags, static_cast<float *>(r.d_img), s);
        if (st) return st;
        if ((st = check_cuda(cudaMemcpyAsync(r.images, r.d_img, r.img_bytes, cudaMemcpyDeviceToHost, s), "server: D2H")))
            return st;
        return check_cuda(cudaLaunchHostFunc(s, on_stream_done, &r), "server: completion callback");
    }

    void release_buffers(Request &r) {
        cudaStream_t s = slots[(size_t)r.slot].stream;
        if (r.d_vis) cudaFreeAsync(r.d_vis, s);
        if (r.d_scales) cudaFreeAsync(r.d_scales, s);
        if (r.d_img) cudaFreeAsync(r.d_img, s);
        r.d_vis = r.d_scales = r.d_img = nullptr;
    }

    void fail_running(const std::shared_ptr<Request> &r, int status, const std::string &msg,
                      std::unique_lock<std::mutex> &lk) {
        lk.unlock();
        release_buffers(*r);
        lk.lock();
        in_use -= r->device_bytes();
        slots[(size_t)r->slot].busy = false;
        r->t_done = Clock::now();
        finish(r, status, msg.c_str());
    }

    void run() {
        cudaSetDevice(cfg.device);
        std::unique_lock<std::mutex> lk(mu);
        bool blocked = false;  // the front request waits for memory held by running requests
        for (;;) {
            while (!completed.empty()) {
                std::shared_ptr<Request> r = completed.back();
                completed.pop_back();
                lk.unlock();
                release_buffers(*r);
                lk.lock();
                in_use -= r->device_bytes();
                slots[(size_t)r->slot].busy = false;
                finish(r, BGI_OK, nullptr);
                blocked = false;
            }
            while (!queue.empty() && !blocked) {
                const int si = free_slot();
                if (si < 0) break;
                std::shared_ptr<Request> r = queue.front();
                const bool running = in_use > 0;
                bool fits = in_use + r->device_bytes() <= budget;
                if (fits) {  // and the device has the memory now (other users included)
                    lk.unlock();
                    size_t free_b = 0, total_b = 0;
                    const bool ok = cudaMemGetInfo(&free_b, &total_b) == cudaSuccess;
                    lk.lock();
                    fits = ok && free_b >= r->device_bytes() + cfg.reserve_bytes;
                }
                if (!fits) {
                    if (running) {  // wait for a completion to free memory
                        ++n_admission_waits;
                        blocked = true;
                        break;
                    }
                    queue.pop_front();
                    r->t_done = Clock::now();
                    finish(r, BGI_ERR_ALLOC, "server: the request does not fit in device memory");
                    continue;
                }
                queue.pop_front();
                r->slot = si;
                slots[(size_t)si].busy = true;
                in_use += r->device_bytes();
                lk.unlock();
                const int st = launch(*r);
                const std::string msg = st ? bgi_last_error() : "";
                lk.lock();
                if (st) fail_running(r, st, msg, lk);
            }
            if (stop && queue.empty() && completed.empty() && in_use == 0) break;
            cv_work.wait(lk, [&] {
                return !completed.empty() || (!queue.empty() && !blocked && free_slot() >= 0) ||
                       (stop && queue.empty() && in_use == 0);
            });
        }
    }
};

extern "C" {

int bgi_server_create(const bgi_server_config *cfg, bgi_server **out) {
    if (!cfg || !out) return set_error(BGI_ERR_INVALID, "server_create: null argument");
    *out = nullptr;
    if (cfg->max_slots < 1 || cfg->max_slots > 64) return set_error(BGI_ERR_INVALID, "server_create: 1 <= max_slots <= 64");
    if (cfg->max_queued < 0) return set_error(BGI_ERR_INVALID, "server_create: max_queued >= 0");
    int n_dev = 0;
    int st = check_cuda(cudaGetDeviceCount(&n_dev), "server_create: device count");
    if (st) return st;
    if (cfg->device < 0 || cfg->device >= n_dev) return set_error(BGI_ERR_INVALID, "server_create: no device %d", cfg->device);
    int prev = 0;
    cudaGetDevice(&prev);
    if ((st = check_cuda(cudaSetDevice(cfg->device), "server_create: set device"))) return st;
    std::unique_ptr<bgi_server> sv(new bgi_server());
    sv->cfg = *cfg;
    size_t free_b = 0, total_b = 0;
    st = check_cuda(cudaMemGetInfo(&free_b, &total_b), "server_create: memory info");
    if (!st) {
        const size_t avail = free_b > cfg->reserve_bytes ? free_b - cfg->reserve_bytes : 0;
        sv->budget = cfg->hbm_budget_bytes ? std::min(cfg->hbm_budget_bytes, avail) : avail;
        // keep freed request buffers in the stream-ordered pool instead of returning them
        cudaMemPool_t pool;
        st = check_cuda(cudaDeviceGetDefaultMemPool(&pool, cfg->device), "server_create: memory pool");
        if (!st) {
            uint64_t keep = UINT64_MAX;
            st = check_cuda(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep), "server_create: pool");
        }
    }
    sv->slots.resize((size_t)cfg->max_slots);
    for (auto &slot : sv->slots)
        if (!st) st = check_cuda(cudaStreamCreateWithFlags(&slot.stream, cudaStreamNonBlocking), "server_create: stream");
    cudaSetDevice(prev);
    if (st) {
        for (auto &slot : sv->slots)
            if (slot.stream) cudaStreamDestroy(slot.stream);
        return st;
    }
    bgi_server *raw = sv.release();
    raw->worker = std::thread([raw] { raw->run(); });
    *out = raw;
    return BGI_OK;
}

int bgi_server_destroy(bgi_server *sv) {
    if (!sv) return BGI_OK;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    sv->worker.join();  // after every queued request has finished
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(sv->cfg.device);
    for (auto &slot : sv->slots) {
        if (slot.stream) cudaStreamSynchronize(slot.stream);
        for (auto &kv : slot.handles) bgi_destroy(kv.second);
        if (slot.stream) cudaStreamDestroy(slot.stream);
    }
    cudaSetDevice(prev);
    delete sv;
    return BGI_OK;
}

int bgi_server_add_array(bgi_server *sv, const bgi_config *cfg, int n_ant, int n_uvw_sets, const float *u,
                         const float *v, const float *w, const int *baseline_flags, const double *cable_lengths,
                         int n_channels, const double *freqs_hz, int *array_id) {
    if (!sv || !cfg || !u || !v || !baseline_flags || !freqs_hz || !array_id || n_ant < 1 || n_uvw_sets < 1 ||
        n_channels < 1)
        return set_error(BGI_ERR_INVALID, "server_add_array: bad arguments");
    if (cfg->device != sv->cfg.device) return set_error(BGI_ERR_INVALID, "server_add_array: config for another device");
    // check the state by building a handle from it (on the calling thread), then keep a host copy
    bgi_imager *probe = nullptr;
    int st = bgi_create(cfg, &probe);
    if (!st) st = bgi_set_array(probe, n_ant, n_uvw_sets, u, v, w, baseline_flags, cable_lengths);
    if (!st) st = bgi_set_frequencies(probe, n_channels, freqs_hz);
    bgi_destroy(probe);
    if (st) return st;
    auto a = std::make_shared<ArrayState>();
    const long long nb = (long long)n_ant * (n_ant + 1) / 2;
    a->cfg = *cfg;
    a->n_ant = n_ant;
    a->n_uvw_sets = n_uvw_sets;
    a->n_channels = n_channels;
    a->n_baselines = nb;
    a->u.assign(u, u + (size_t)n_uvw_sets * nb);
    a->v.assign(v, v + (size_t)n_uvw_sets * nb);
    if (w) a->w.assign(w, w + (size_t)n_uvw_sets * nb);  // empty: no geometric correction possible
    a->flags.assign(baseline_flags, baseline_flags + nb);
    if (cable_lengths) a->cable.assign(cable_lengths, cable_lengths + n_ant);
    a->freqs.assign(freqs_hz, freqs_hz + n_channels);
    std::lock_guard<std::mutex> lk(sv->mu);
    *array_id = (int)sv->arrays.size();
    sv->arrays.push_back(std::move(a));
    return BGI_OK;
}

int bgi_server_submit(bgi_server *sv, int array_id, int format, const void *vis_host, const float *scales_host,
                      int n_intervals, unsigned flags, float *images_host, uint64_t *ticket) {
    if (!sv || !vis_host || !images_host || !ticket || n_intervals < 1)
        return set_error(BGI_ERR_INVALID, "server_submit: bad arguments");
    if (format < BGI_VIS_C64 || format > BGI_VIS_FP16 || (format != BGI_VIS_C64 && !scales_host))
        return set_error(BGI_ERR_INVALID, "server_submit: bad format or missing scales");
    if (flags & ~(BGI_APPLY_GEOMETRIC | BGI_APPLY_CABLE | BGI_OUTPUT_REAL))
        return set_error(BGI_ERR_INVALID, "server_submit: unknown flags");
    auto r = std::make_shared<Request>();
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->stop) return set_error(BGI_ERR_STATE, "server_submit: the server is shutting down");
    if (array_id < 0 || array_id >= (int)sv->arrays.size())
        return set_error(BGI_ERR_INVALID, "server_submit: no array %d", array_id);
    const ArrayState &a = *sv->arrays[(size_t)array_id];
    if (a.n_uvw_sets != 1 && a.n_uvw_sets != n_intervals)
        return set_error(BGI_ERR_INVALID, "server_submit: array has %d UVW sets for %d intervals", a.n_uvw_sets, n_intervals);
    if (sv->cfg.max_queued > 0 && sv->queue.size() >= (size_t)sv->cfg.max_queued) {
        ++sv->n_rejected;
        return set_error(BGI_ERR_BUSY, "server_submit: %d requests already wait for admission", sv->cfg.max_queued);
    }
    const size_t imgs = (size_t)n_intervals * a.n_channels, n = (size_t)a.cfg.n_pixels;
    r->array = sv->arrays[(size_t)array_id];
    r->array_id = array_id;
    r->format = format;
    r->vis = vis_host;
    r->scales = scales_host;
    r->n_intervals = n_intervals;
    r->flags = flags;
    r->images = images_host;
    r->n_images = (int)imgs;
    r->vis_bytes = imgs * (size_t)a.n_baselines * (format == BGI_VIS_C64 ? 32 : 16);
    r->scale_bytes = format == BGI_VIS_C64 ? 0 : imgs * 16 * (size_t)vis_blocks(a.n_baselines);
    r->img_bytes = imgs * n * n * ((flags & BGI_OUTPUT_REAL) ? 4 : 8);
    r->server = sv;
    r->ticket = sv->next_ticket++;
    r->t_submit = Clock::now();
    if (!sv->any_submit) {
        sv->t_first_submit = r->t_submit;
        sv->any_submit = true;
    }
    ++sv->n_submitted;
    sv->requests[r->ticket] = r;
    sv->queue.push_back(r);
    *ticket = r->ticket;
    sv->cv_work.notify_one();
    return BGI_OK;
}

// Reports a finished request once: its status is returned through *status and the ticket is
// released.
static int collect(bgi_server *sv, uint64_t ticket, int *status, std::unique_lock<std::mutex> &lk, bool block,
                   int timeout_ms, int *done) {
    auto it = sv->requests.find(ticket);
    if (it == sv->requests.end()) return set_error(BGI_ERR_INVALID, "server: unknown or already collected ticket %llu",
                                                   (unsigned long long)ticket);
    std::shared_ptr<Request> r = it->second;
    if (block) {
        auto pred = [&] { return r->status != 1; };
        if (timeout_ms < 0) sv->cv_done.wait(lk, pred);
        else sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred);
    }
    if (done) *done = r->status != 1;
    if (r->status == 1) return block ? set_error(BGI_ERR_STATE, "server_wait: timed out") : BGI_OK;
    if (status) *status = r->status;
    if (r->status != BGI_OK) set_error(r->status, "%s", r->error.c_str());
    sv->requests.erase(it);
    return BGI_OK;
}

int bgi_server_wait(bgi_server *sv, uint64_t ticket, int timeout_ms, int *status) {
    if (!sv || !status) return set_error(BGI_ERR_INVALID, "server_wait: null argument");
    std::unique_lock<std::mutex> lk(sv->mu);
    return collect(sv, ticket, status, lk, true, timeout_ms, nullptr);
}

int bgi_server_cancel(bgi_server *sv, uint64_t ticket) {
    if (!sv) return set_error(BGI_ERR_INVALID, "server_cancel: null server");
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->requests.find(ticket);
    if (it == sv->requests.end())
        return set_error(BGI_ERR_INVALID, "server_cancel: unknown or already collected ticket %llu",
                         (unsigned long long)ticket);
    std::shared_ptr<Request> r = it->second;
    auto q = std::find(sv->queue.begin(), sv->queue.end(), r);
    if (q == sv->queue.end()) return set_error(BGI_ERR_STATE, "server_cancel: the request is already admitted");
    sv->queue.erase(q);
    r->t_done = Clock::now();
    ++sv->n_cancelled;
    sv->finish(r, BGI_ERR_CANCELLED, "server: the request was cancelled");
    sv->cv_work.notify_one();  // the next request may be admitted now
    return BGI_OK;
}

int bgi_server_poll(bgi_server *sv, uint64_t ticket, int *done, int *status) {
    if (!sv || !done || !status) return set_error(BGI_ERR_INVALID, "server_poll: null argument");
    std::unique_lock<std::mutex> lk(sv->mu);
    return collect(sv, ticket, status, lk, false, 0, done);
}

int bgi_server_get_stats(bgi_server *sv, bgi_server_stats *out) {
    if (!sv || !out) return set_error(BGI_ERR_INVALID, "server_get_stats: null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    bgi_server_stats s{};
    s.submitted = sv->n_submitted;
    s.completed = sv->n_completed;
    s.failed = sv->n_failed;
    s.images = sv->n_images;
    s.admission_waits = sv->n_admission_waits;
    s.queued = sv->queue.size();
    s.device_bytes_in_use = sv->in_use;
    s.device_budget_bytes = sv->budget;
    s.rejected = sv->n_rejected;
    s.cancelled = sv->n_cancelled;
    std::vector<double> lat = sv->latencies_ms;
    if (!lat.empty()) {
        std::sort(lat.begin(), lat.end());
        auto q = [&](double f) {  // nearest-rank percentile
            size_t k = (size_t)std::ceil(f * (double)lat.size());
            return lat[std::min(lat.size() - 1, k ? k - 1 : 0)];
        };
        s.p50_ms = q(0.50);
        s.p99_ms = q(0.99);
        s.max_ms = lat.back();
        double sum = 0;
        for (double x : lat) sum += x;
        s.mean_ms = sum / (double)lat.size();
    }
    if (sv->any_submit && sv->n_images)
        s.wall_s = std::chrono::duration<double>(sv->t_last_done - sv->t_first_submit).count();
    s.images_per_s = s.wall_s > 0 ? (double)s.images / s.wall_s : 0.0;
    *out = s;
    return BGI_OK;
}

int bgi_server_reset_stats(bgi_server *sv) {
    if (!sv) return set_error(BGI_ERR_INVALID, "server_reset_stats: null server");
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->latencies_ms.clear();
    sv->n_submitted = sv->n_completed = sv->n_failed = sv->n_images = sv->n_admission_waits = 0;
    sv->n_rejected = sv->n_cancelled = 0;
    sv->any_submit = false;
    return BGI_OK;
}

}  // extern "C"
