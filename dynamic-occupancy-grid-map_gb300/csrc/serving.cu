// Serving loop behind dogm_server_* (include/dogm_gb300.h): resident sensor streams, admission
// under an HBM budget and continuous batching of their frames.
//
// The reference has no serving layer: its demo owns one dogm::DOGM and calls updateGrid once
// per simulated frame (dogm/demo/main.cpp:81-92).  Here one worker thread per server owns the
// device side:
//   * completion: every launch in flight is polled (cudaEventQuery); a finished launch turns
//     into one result per frame and frees its streams for their next frame;
//   * closing and admission: closed streams free their handles; waiting streams are admitted
//     in opening order while the budget allows;
//   * launching: while a launch slot is free, the oldest pending frame of every stream with
//     nothing on the device (oldest first, at most max_batch) goes into one batched launch.
// Submitters only append to per-stream queues, so frames that arrive while launches run are
// picked up by the next free slot (continuous batching), and with two slots the tail of one
// launch overlaps the head of the next on the device.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "dogm_internal.h"

using namespace dogm_gb300;

namespace {

int64_t now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

dogm_status fail(dogm_status s, const char* msg) {
    set_last_error(msg);
    return s;
}

struct Frame {
    const dogm_measurement_cell* meas;
    int device;
    float x, y, yaw, dt;
    dogm_grid_cell* out;
    uint64_t tag;
    int64_t t_submit;
};

struct Stream {
    int id = -1;
    int state = DOGM_STREAM_WAITING;
    dogm_params params{};
    dogm_options opt{};
    size_t bytes = 0;
    dogm_handle* h = nullptr;
    std::deque<Frame> q;       // submitted, not launched
    bool inflight = false;     // one frame on the device
    Frame cur{};               // the frame on the device
    int64_t t_launch = 0;
    cudaEvent_t ev = nullptr;  // per-stream mode: the frame's completion
    bool closing = false;
};

struct Launch {
    BatchSlot* slot;
    std::vector<Stream*> streams;
    int64_t t_launch;
};

}  // namespace

struct dogm_server {
    dogm_server_config cfg{};
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_work;  // worker: new frames, streams, closes, stop
    std::condition_variable cv_out;   // callers: results, admission and close progress
    std::vector<Stream*> streams;     // by id (kept after close; state CLOSED)
    std::deque<Stream*> waiting;      // admission queue, opening order
    size_t resident = 0;
    std::vector<BatchSlot*> free_slots, all_slots;
    std::deque<Launch> launches_inflight;
    std::vector<Stream*> per_stream_inflight;
    std::deque<dogm_server_result> results;
    uint64_t submitted = 0, done = 0, launches = 0, launched_frames = 0;
    bool stop = false;
    bool paused = false;   // launches held back (frames keep queueing)
    std::thread worker;
    dogm_status worker_status = DOGM_OK;

    void run();
    bool complete();
    bool close_and_admit(std::unique_lock<std::mutex>& lk);
    bool launch(std::unique_lock<std::mutex>& lk);
    dogm_status admit(Stream* st, std::unique_lock<std::mutex>& lk);
    void push_result(Stream* st, const Frame& f, int status, int batch, int64_t t_launch, int64_t t_done);
    bool busy() const { return !launches_inflight.empty() || !per_stream_inflight.empty(); }
};

namespace {

// Allocates the stream's device state.  Called with the lock held; dogm_create runs unlocked
// (it allocates and initialises device memory), the budget is reserved before.
dogm_status create_handle(dogm_server* s, Stream* st, std::unique_lock<std::mutex>& lk) {
    dogm_options opt = st->opt;
    opt.sync_each_update = 0;  // the worker waits on events, never on the update call
    dogm_handle* h = nullptr;
    lk.unlock();
    dogm_status rc = dogm_create(&st->params, &opt, &h);
    cudaEvent_t ev = nullptr;
    const bool per_stream = s->cfg.mode == DOGM_SERVE_PER_STREAM || s->cfg.mode == DOGM_SERVE_PER_STREAM_PLAIN;
    if (rc == DOGM_OK && s->cfg.mode == DOGM_SERVE_PER_STREAM_PLAIN) rc = dogm_set_launch_mode(h, DOGM_LAUNCH_PLAIN);
    if (rc == DOGM_OK && per_stream && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
        dogm_destroy(h);
        h = nullptr;
        rc = fail(DOGM_ERR_CUDA, "cudaEventCreate failed");
    }
    lk.lock();
    if (rc != DOGM_OK) return rc;
    st->h = h;
    st->ev = ev;
    return DOGM_OK;
}

}  // namespace

dogm_status dogm_server::admit(Stream* st, std::unique_lock<std::mutex>& lk) {
    resident += st->bytes;  // reserved while the handle is being created
    dogm_status rc = create_handle(this, st, lk);
    if (rc != DOGM_OK) {
        resident -= st->bytes;
        st->state = DOGM_STREAM_CLOSED;
        // frames submitted while it waited cannot run
        const int64_t t = now_ns();
        while (!st->q.empty()) {
            push_result(st, st->q.front(), rc, 0, 0, t);
            st->q.pop_front();
        }
    } else {
        st->state = DOGM_STREAM_ACTIVE;
    }
    cv_out.notify_all();
    return rc;
}

void dogm_server::push_result(Stream* st, const Frame& f, int status, int batch, int64_t t_launch, int64_t t_done) {
    dogm_server_result r{};
    r.stream = st->id;
    r.status = status;
    r.tag = f.tag;
    r.iteration = st->h ? dogm_get_iteration(st->h) : 0;
    r.batch_size = batch;
    r.t_submit_ns = f.t_submit;
    r.t_launch_ns = t_launch;
    r.t_done_ns = t_done;
    results.push_back(r);
    done += 1;
}

// Turns finished launches into results.  Lock held.
bool dogm_server::complete() {
    bool any = false;
    for (auto it = launches_inflight.begin(); it != launches_inflight.end();) {
        if (!slot_done(it->slot)) { ++it; continue; }
        const dogm_status rc = slot_finish(it->slot);
        const int64_t t = now_ns();
        const int n = (int)it->streams.size();
        for (Stream* st : it->streams) {
            push_result(st, st->cur, rc, n, it->t_launch, t);
            st->inflight = false;
        }
        free_slots.push_back(it->slot);
        it = launches_inflight.erase(it);
        any = true;
    }
    for (size_t i = 0; i < per_stream_inflight.size();) {
        Stream* st = per_stream_inflight[i];
        if (cudaEventQuery(st->ev) == cudaErrorNotReady) { ++i; continue; }
        const dogm_status rc = dogm_synchronize(st->h);  // finished: returns the frame's status
        push_result(st, st->cur, rc, 1, st->t_launch, now_ns());
        st->inflight = false;
        per_stream_inflight[i] = per_stream_inflight.back();
        per_stream_inflight.pop_back();
        any = true;
    }
    if (any) cv_out.notify_all();
    return any;
}

// Frees closed streams and admits waiting ones.  Lock held.
bool dogm_server::close_and_admit(std::unique_lock<std::mutex>& lk) {
    bool any = false;
    // by index: the lock is dropped around dogm_destroy and open_stream may grow the vector
    for (size_t i = 0; i < streams.size(); ++i) {
        Stream* st = streams[i];
        if (!st->closing || st->state == DOGM_STREAM_CLOSED || st->inflight || !st->q.empty()) continue;
        if (st->state == DOGM_STREAM_WAITING) {
            waiting.erase(std::remove(waiting.begin(), waiting.end(), st), waiting.end());
        } else {
            dogm_handle* h = st->h;
            cudaEvent_t ev = st->ev;
            st->h = nullptr;
            st->ev = nullptr;
            lk.unlock();
            dogm_destroy(h);
            if (ev) cudaEventDestroy(ev);
            lk.lock();
            resident -= st->bytes;
        }
        st->state = DOGM_STREAM_CLOSED;
        any = true;
    }
    while (!waiting.empty() && resident + waiting.front()->bytes <= cfg.hbm_budget_bytes) {
        Stream* st = waiting.front();
        waiting.pop_front();
        admit(st, lk);
        any = true;
    }
    if (any) cv_out.notify_all();
    return any;
}

// Queues launches while slots (or, per stream, ready streams) are available.  Lock held.
bool dogm_server::launch(std::unique_lock<std::mutex>& lk) {
    if (paused) return false;
    std::vector<Stream*> ready;
    for (Stream* st : streams)
        if (st->state == DOGM_STREAM_ACTIVE && !st->inflight && !st->q.empty()) ready.push_back(st);
    if (ready.empty()) return false;
    std::sort(ready.begin(), ready.end(),
              [](const Stream* a, const Stream* b) { return a->q.front().t_submit < b->q.front().t_submit; });
    bool any = false;
    if (cfg.mode == DOGM_SERVE_PER_STREAM || cfg.mode == DOGM_SERVE_PER_STREAM_PLAIN) {
        const bool plain = cfg.mode == DOGM_SERVE_PER_STREAM_PLAIN;
        for (Stream* st : ready) {
            st->cur = st->q.front();
            st->q.pop_front();
            st->inflight = true;
            const Frame f = st->cur;
            lk.unlock();
            dogm_status rc = dogm_update(st->h, f.meas, f.x, f.y, f.yaw, f.dt, f.device);
            cudaStream_t cs = handle_stream(st->h);
            if (rc == DOGM_OK && f.out &&
                cudaMemcpyAsync(f.out, handle_cells(st->h), sizeof(dogm_grid_cell) * (size_t)handle_cell_count(st->h),
                                cudaMemcpyDeviceToHost, cs) != cudaSuccess)
                rc = fail(DOGM_ERR_CUDA, "readback copy failed");
            if (rc == DOGM_OK && cudaEventRecord(st->ev, cs) != cudaSuccess)
                rc = fail(DOGM_ERR_CUDA, "cudaEventRecord failed");
            // plain mode: the frame is waited for before the next one starts, as the reference
            if (rc == DOGM_OK && plain && cudaEventSynchronize(st->ev) != cudaSuccess)
                rc = fail(DOGM_ERR_CUDA, "cudaEventSynchronize failed");
            const int64_t t = now_ns();
            lk.lock();
            launches += 1;
            launched_frames += 1;
            st->t_launch = t;
            if (rc != DOGM_OK) {
                push_result(st, f, rc, 1, t, now_ns());
                st->inflight = false;
                cv_out.notify_all();
            } else {
                per_stream_inflight.push_back(st);
            }
            any = true;
        }
        return any;
    }
    size_t next = 0;
    while (next < ready.size() && !free_slots.empty()) {
        BatchSlot* slot = free_slots.back();
        free_slots.pop_back();
        const size_t n = std::min(ready.size() - next, (size_t)cfg.max_batch);
        Launch L{slot, std::vector<Stream*>(ready.begin() + next, ready.begin() + next + n), 0};
        next += n;
        std::vector<SlotFrame> fr(n);
        for (size_t i = 0; i < n; ++i) {
            Stream* st = L.streams[i];
            st->cur = st->q.front();
            st->q.pop_front();
            st->inflight = true;
            const Frame& f = st->cur;
            fr[i] = SlotFrame{st->h, f.meas, f.device, f.x, f.y, f.yaw, f.dt, f.out};
        }
        lk.unlock();
        const dogm_status rc = slot_launch(slot, fr.data(), (int)n);
        const int64_t t = now_ns();
        lk.lock();
        launches += 1;
        launched_frames += n;
        L.t_launch = t;
        if (rc != DOGM_OK) {
            for (Stream* st : L.streams) {
                push_result(st, st->cur, rc, (int)n, t, now_ns());
                st->inflight = false;
            }
            free_slots.push_back(slot);
            cv_out.notify_all();
        } else {
            launches_inflight.push_back(std::move(L));
        }
        any = true;
    }
    return any;
}

void dogm_server::run() {
    if (cudaSetDevice(device) != cudaSuccess) {
        std::lock_guard<std::mutex> g(mu);
        worker_status = DOGM_ERR_CUDA;
        return;
    }
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        bool progress = complete();
        progress |= close_and_admit(lk);
        progress |= launch(lk);
        if (stop && !busy()) {
            bool pending = false;
            for (Stream* st : streams) pending |= st->state == DOGM_STREAM_ACTIVE && !st->q.empty();
            if (!pending) break;
        }
        if (progress) continue;
        if (busy()) {
            // launches on the device: poll their events without holding the lock
            lk.unlock();
            std::this_thread::yield();
            lk.lock();
        } else {
            cv_work.wait(lk);
        }
    }
}

extern "C" {

int64_t dogm_server_now_ns(void) { return now_ns(); }

dogm_status dogm_server_default_config(dogm_server_config* cfg) {
    if (!cfg) return fail(DOGM_ERR_INVALID_ARGUMENT, "cfg is NULL");
    cfg->hbm_budget_bytes = (size_t)150 * 1000 * 1000 * 1000;
    cfg->mode = DOGM_SERVE_BATCHED;
    cfg->max_batch = 64;
    cfg->max_inflight = 2;
    cfg->queue_admission = 1;
    return DOGM_OK;
}

dogm_status dogm_server_create(const dogm_server_config* cfg, dogm_server** out) {
    if (!cfg || !out) return fail(DOGM_ERR_INVALID_ARGUMENT, "cfg/out is NULL");
    *out = nullptr;
    if (cfg->mode != DOGM_SERVE_BATCHED && cfg->mode != DOGM_SERVE_PER_STREAM &&
        cfg->mode != DOGM_SERVE_PER_STREAM_PLAIN)
        return fail(DOGM_ERR_INVALID_ARGUMENT, "unknown serve mode");
    if (cfg->max_batch < 1 || cfg->max_batch > kMaxBatch)
        return fail(DOGM_ERR_INVALID_ARGUMENT, "max_batch must be in [1, 256]");
    if (cfg->max_inflight < 1 || cfg->max_inflight > 4)
        return fail(DOGM_ERR_INVALID_ARGUMENT, "max_inflight must be in [1, 4]");
    if (cfg->hbm_budget_bytes == 0) return fail(DOGM_ERR_INVALID_ARGUMENT, "hbm_budget_bytes is 0");
    dogm_server* s = new dogm_server();
    s->cfg = *cfg;
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        delete s;
        return fail(DOGM_ERR_CUDA, "no CUDA device");
    }
    if (cfg->mode == DOGM_SERVE_BATCHED) {
        for (int i = 0; i < cfg->max_inflight; ++i) {
            BatchSlot* slot = nullptr;
            dogm_status rc = slot_create(s->device, &slot);
            if (rc == DOGM_OK) rc = slot_prewarm(slot, cfg->max_batch);  // no graph built mid-serving
            if (rc != DOGM_OK) {
                slot_destroy(slot);
                for (BatchSlot* b : s->all_slots) slot_destroy(b);
                delete s;
                return rc;
            }
            s->all_slots.push_back(slot);
            s->free_slots.push_back(slot);
        }
    }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return DOGM_OK;
}

dogm_status dogm_server_destroy(dogm_server* s) {
    if (!s) return DOGM_OK;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
        s->paused = false;
        for (Stream* st : s->streams) st->closing = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    const int prev = [] { int d = 0; cudaGetDevice(&d); return d; }();
    cudaSetDevice(s->device);
    for (Stream* st : s->streams) {
        if (st->h) dogm_destroy(st->h);
        if (st->ev) cudaEventDestroy(st->ev);
        delete st;
    }
    for (BatchSlot* b : s->all_slots) slot_destroy(b);
    cudaSetDevice(prev);
    const dogm_status ws = s->worker_status;
    delete s;
    return ws;
}

dogm_status dogm_server_open_stream(dogm_server* s, const dogm_params* params, const dogm_options* opt,
                                    int* stream_id) {
    if (!s || !params || !stream_id) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    *stream_id = -1;
    const size_t bytes = dogm_state_bytes(params);
    if (bytes == 0) return fail(DOGM_ERR_INVALID_ARGUMENT, "invalid stream parameters");
    if (bytes > s->cfg.hbm_budget_bytes)
        return fail(DOGM_ERR_BUDGET, "the stream's state alone exceeds the server's HBM budget");
    Stream* st = new Stream();
    st->params = *params;
    if (opt) st->opt = *opt; else dogm_default_options(&st->opt);
    st->bytes = bytes;
    std::unique_lock<std::mutex> lk(s->mu);
    const bool fits = s->waiting.empty() && s->resident + bytes <= s->cfg.hbm_budget_bytes;
    if (!fits && !s->cfg.queue_admission) {
        delete st;
        return fail(DOGM_ERR_BUDGET, "admission refused: the HBM budget is taken by admitted streams");
    }
    st->id = (int)s->streams.size();
    s->streams.push_back(st);
    *stream_id = st->id;
    if (!fits) {
        s->waiting.push_back(st);
        return DOGM_OK;
    }
    const int prev = [] { int d = 0; cudaGetDevice(&d); return d; }();
    cudaSetDevice(s->device);
    const dogm_status rc = s->admit(st, lk);
    cudaSetDevice(prev);
    lk.unlock();
    s->cv_work.notify_all();
    return rc;
}

dogm_status dogm_server_close_stream(dogm_server* s, int stream_id) {
    if (!s) return fail(DOGM_ERR_INVALID_ARGUMENT, "server is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    if (stream_id < 0 || stream_id >= (int)s->streams.size())
        return fail(DOGM_ERR_INVALID_ARGUMENT, "unknown stream id");
    Stream* st = s->streams[stream_id];
    if (st->state == DOGM_STREAM_CLOSED) return DOGM_OK;
    st->closing = true;
    s->cv_work.notify_all();
    s->cv_out.wait(lk, [&] { return st->state == DOGM_STREAM_CLOSED || s->worker_status != DOGM_OK; });
    return s->worker_status;
}

dogm_status dogm_server_submit(dogm_server* s, int stream_id, const dogm_measurement_cell* meas, int device,
                               float new_x, float new_y, float new_yaw, float dt, dogm_grid_cell* cells_out,
                               uint64_t tag) {
    if (!s) return fail(DOGM_ERR_INVALID_ARGUMENT, "server is NULL");
    Frame f{meas, device, new_x, new_y, new_yaw, dt, cells_out, tag, now_ns()};
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (stream_id < 0 || stream_id >= (int)s->streams.size())
            return fail(DOGM_ERR_INVALID_ARGUMENT, "unknown stream id");
        Stream* st = s->streams[stream_id];
        if (st->state == DOGM_STREAM_CLOSED || st->closing)
            return fail(DOGM_ERR_INVALID_ARGUMENT, "stream is closed");
        st->q.push_back(f);
        s->submitted += 1;
    }
    s->cv_work.notify_one();
    return DOGM_OK;
}

dogm_status dogm_server_pause(dogm_server* s, int paused) {
    if (!s) return fail(DOGM_ERR_INVALID_ARGUMENT, "server is NULL");
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->paused = paused != 0;
    }
    s->cv_work.notify_all();
    return DOGM_OK;
}

dogm_status dogm_server_poll(dogm_server* s, dogm_server_result* out, int max, int timeout_us, int* n_out) {
    if (!s || !n_out || (max > 0 && !out)) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    *n_out = 0;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->results.empty() && timeout_us > 0)
        s->cv_out.wait_for(lk, std::chrono::microseconds(timeout_us), [&] { return !s->results.empty(); });
    int n = 0;
    while (n < max && !s->results.empty()) {
        out[n++] = s->results.front();
        s->results.pop_front();
    }
    *n_out = n;
    return DOGM_OK;
}

dogm_status dogm_server_drain(dogm_server* s, int timeout_ms) {
    if (!s) return fail(DOGM_ERR_INVALID_ARGUMENT, "server is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cv_out.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                       [&] { return s->done == s->submitted || s->worker_status != DOGM_OK; });
    if (s->worker_status != DOGM_OK) return s->worker_status;
    return ok ? DOGM_OK : fail(DOGM_ERR_NOT_READY, "frames still pending after the drain timeout");
}

dogm_status dogm_server_get_stats(dogm_server* s, dogm_server_stats* out) {
    if (!s || !out) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> g(s->mu);
    out->frames_submitted = s->submitted;
    out->frames_done = s->done;
    out->launches = s->launches;
    out->streams_active = out->streams_waiting = 0;
    for (Stream* st : s->streams) {
        out->streams_active += st->state == DOGM_STREAM_ACTIVE;
        out->streams_waiting += st->state == DOGM_STREAM_WAITING;
    }
    out->resident_bytes = s->resident;
    out->budget_bytes = s->cfg.hbm_budget_bytes;
    out->mean_batch = s->launches ? (double)s->launched_frames / (double)s->launches : 0.0;
    return DOGM_OK;
}

int dogm_server_stream_state(dogm_server* s, int stream_id) {
    if (!s) return -1;
    std::lock_guard<std::mutex> g(s->mu);
    if (stream_id < 0 || stream_id >= (int)s->streams.size()) return -1;
    return s->streams[stream_id]->state;
}

dogm_status dogm_server_stream_handle(dogm_server* s, int stream_id, dogm_handle** out) {
    if (!s || !out) return fail(DOGM_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    std::lock_guard<std::mutex> g(s->mu);
    if (stream_id < 0 || stream_id >= (int)s->streams.size())
        return fail(DOGM_ERR_INVALID_ARGUMENT, "unknown stream id");
    Stream* st = s->streams[stream_id];
    if (st->state != DOGM_STREAM_ACTIVE) return fail(DOGM_ERR_NOT_READY, "stream is not admitted");
    *out = st->h;
    return DOGM_OK;
}

}  // extern "C"
