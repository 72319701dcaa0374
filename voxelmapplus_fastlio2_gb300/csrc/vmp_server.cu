// Multi-stream serving over vmp_process (host code).
//
// The reference has one LIOBuilder per ROS node and processes a node's
// packages one at a time (lio_node.cpp:167-182); a server runs many
// independent streams on one GPU.  Each stream keeps its map and filter on
// the device and has its own CUDA stream.  Worker threads take packages in
// submission order per stream (a stream runs one package at a time, as the
// reference's step is a dependency chain) and across streams by submission
// time; while a worker waits for its stream's result, the other workers'
// streams keep the GPU busy, so the kernels of different streams overlap.
// Admission: a stream is opened while the device memory of the open streams
// (each stream's footprint is what vmp_create allocated) stays within the
// HBM budget and a slot is free.
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "vmp.h"

namespace vmp {
void merge_set_throughput_mode(bool on);
}

namespace {

struct Package {
    long long cookie = 0;
    std::vector<vmp_point> pts;
    std::vector<vmp_imu> imus;
    // vmp_submit_device: the caller's device buffers
    const vmp_point* d_pts = nullptr;
    const vmp_imu* d_imus = nullptr;
    int n = 0, n_imu = 0;
    double t_start = 0.0, t_end = 0.0;
    double submit_ms = 0.0;
};

struct Slot {
    bool open = false;
    bool busy = false;    // a worker runs one of its packages
    bool closing = false;
    vmp_stream_t h = nullptr;
    long long bytes = 0;
    std::deque<Package> q;
};

}  // namespace

struct vmp_server_s {
    vmp_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work;  // workers: a package is ready / stop
    std::condition_variable cv_done;  // pollers, close / destroy: a package finished
    std::vector<Slot> slots;
    std::deque<vmp_server_result> done;
    std::vector<std::thread> workers;
    bool stop = false;
    long long used = 0;
    int running = 0;
    int queued = 0;
    std::string err;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    double now_ms() const {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }

    // the ready stream whose oldest package was submitted first (-1: none)
    int pick() const {
        int best = -1;
        double bt = 0.0;
        for (int i = 0; i < (int)slots.size(); ++i) {
            const Slot& s = slots[i];
            if (!s.open || s.busy || s.q.empty()) continue;
            if (best < 0 || s.q.front().submit_ms < bt) {
                best = i;
                bt = s.q.front().submit_ms;
            }
        }
        return best;
    }

    void worker() {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            int id = -1;
            cv_work.wait(lk, [&] { return stop || (id = pick()) >= 0; });
            if (stop) return;
            Slot& sl = slots[id];
            Package p = std::move(sl.q.front());
            sl.q.pop_front();
            sl.busy = true;
            --queued;
            ++running;
            vmp_stream_t h = sl.h;
            lk.unlock();
            vmp_server_result r;
            std::memset(&r, 0, sizeof(r));
            r.cookie = p.cookie;
            r.stream_id = id;
            r.submit_ms = p.submit_ms;
            r.start_ms = now_ms();
            if (p.d_pts) {
                r.status = vmp_process_device(h, p.d_pts, p.n, p.t_start, p.t_end, p.d_imus, p.n_imu, &r.result);
            } else {
                vmp_scan scan{p.pts.data(), (int)p.pts.size(), p.t_start, p.t_end};
                r.status = vmp_process(h, &scan, p.imus.data(), (int)p.imus.size(), &r.result);
            }
            r.end_ms = now_ms();
            lk.lock();
            sl.busy = false;
            --running;
            done.push_back(r);
            cv_done.notify_all();
            cv_work.notify_all();
        }
    }
};

extern "C" {

void vmp_server_config_default(vmp_server_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->hbm_budget_bytes = 150000000000ll;
    c->max_streams = 64;
    c->workers = 32;
    c->queue_depth = 64;
}

vmp_status vmp_server_create(const vmp_server_config* c, vmp_server_t* out) {
    if (!out) return VMP_ERR_INVALID_ARG;
    *out = nullptr;
    vmp_server_config cfg;
    if (c) cfg = *c; else vmp_server_config_default(&cfg);
    if (cfg.max_streams <= 0 || cfg.max_streams > 4096 || cfg.workers <= 0 || cfg.workers > 1024 ||
        cfg.queue_depth <= 0 || cfg.hbm_budget_bytes <= 0)
        return VMP_ERR_INVALID_ARG;
    // Many streams need more hardware work queues than the default 8, or
    // kernels of unrelated streams queue behind each other.  Effective only
    // if the process has not created its CUDA context yet; a caller's own
    // setting wins.
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
    vmp_server_t sv = new (std::nothrow) vmp_server_s();
    if (!sv) return VMP_ERR_OUT_OF_MEMORY;
    sv->cfg = cfg;
    sv->slots.resize(cfg.max_streams);
    sv->workers.reserve(cfg.workers);
    // cooperative merges of several streams at once: small grids, many in
    // flight (a one-worker server runs one package at a time: whole-device
    // merges, as a single stream)
    if (cfg.workers > 1) vmp::merge_set_throughput_mode(true);
    for (int i = 0; i < cfg.workers; ++i) sv->workers.emplace_back([sv] { sv->worker(); });
    *out = sv;
    return VMP_OK;
}

vmp_status vmp_server_destroy(vmp_server_t sv) {
    if (!sv) return VMP_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    for (auto& t : sv->workers) t.join();
    for (auto& s : sv->slots)
        if (s.h) vmp_destroy(s.h);
    if (sv->cfg.workers > 1) vmp::merge_set_throughput_mode(false);
    delete sv;
    return VMP_OK;
}

vmp_status vmp_server_open_stream(vmp_server_t sv, const vmp_config* cfg, int* stream_id) {
    if (!sv || !stream_id) return VMP_ERR_INVALID_ARG;
    *stream_id = -1;
    int id = -1;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        for (int i = 0; i < (int)sv->slots.size(); ++i)
            if (!sv->slots[i].open && !sv->slots[i].closing && !sv->slots[i].h) { id = i; break; }
        if (id < 0) {
            sv->err = "no free stream slot";
            return VMP_ERR_ADMISSION_DENIED;
        }
        sv->slots[id].closing = true;  // reserved while the stream is created
    }
    vmp_stream_t h = nullptr;
    vmp_status st = vmp_create(cfg, &h);
    std::lock_guard<std::mutex> lk(sv->mu);
    Slot& s = sv->slots[id];
    s.closing = false;
    if (st != VMP_OK) {
        sv->err = std::string("vmp_create: ") + vmp_last_error(nullptr);
        return st;
    }
    vmp_set_wait_mode(h, 1);
    const long long b = vmp_device_bytes(h);
    if (sv->used + b > sv->cfg.hbm_budget_bytes) {
        vmp_destroy(h);
        sv->err = "HBM budget: " + std::to_string(sv->used) + " + " + std::to_string(b) + " bytes > " +
                  std::to_string(sv->cfg.hbm_budget_bytes);
        return VMP_ERR_ADMISSION_DENIED;
    }
    sv->used += b;
    s.open = true;
    s.busy = false;
    s.h = h;
    s.bytes = b;
    s.q.clear();
    *stream_id = id;
    return VMP_OK;
}

vmp_status vmp_server_close_stream(vmp_server_t sv, int id) {
    if (!sv) return VMP_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(sv->mu);
    if (id < 0 || id >= (int)sv->slots.size() || !sv->slots[id].open) return VMP_ERR_INVALID_ARG;
    Slot& s = sv->slots[id];
    s.closing = true;  // no new packages
    sv->cv_done.wait(lk, [&] { return sv->stop || (s.q.empty() && !s.busy); });
    s.open = false;
    vmp_stream_t h = s.h;
    s.h = nullptr;
    sv->used -= s.bytes;
    s.bytes = 0;
    lk.unlock();
    vmp_destroy(h);
    lk.lock();
    s.closing = false;
    return VMP_OK;
}

static vmp_status enqueue(vmp_server_t sv, int id, Package&& p) {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (id < 0 || id >= (int)sv->slots.size() || !sv->slots[id].open || sv->slots[id].closing) {
        sv->err = "submit to a stream that is not open";
        return VMP_ERR_INVALID_ARG;
    }
    Slot& s = sv->slots[id];
    if ((int)s.q.size() >= sv->cfg.queue_depth) {
        sv->err = "stream queue full";
        return VMP_ERR_CAPACITY;
    }
    p.submit_ms = sv->now_ms();
    s.q.push_back(std::move(p));
    ++sv->queued;
    sv->cv_work.notify_one();
    return VMP_OK;
}

vmp_status vmp_submit(vmp_server_t sv, int id, const vmp_scan* scan, const vmp_imu* imus, int n_imu,
                      long long cookie) {
    if (!sv || !scan || (scan->n > 0 && !scan->points) || n_imu < 0 || (n_imu > 0 && !imus))
        return VMP_ERR_INVALID_ARG;
    Package p;
    p.cookie = cookie;
    p.pts.assign(scan->points, scan->points + (scan->n > 0 ? scan->n : 0));
    p.imus.assign(imus, imus + n_imu);
    p.t_start = scan->t_start;
    p.t_end = scan->t_end;
    return enqueue(sv, id, std::move(p));
}

vmp_status vmp_submit_device(vmp_server_t sv, int id, const vmp_point* d_pts, int n, double t_start, double t_end,
                             const vmp_imu* d_imus, int n_imu, long long cookie) {
    if (!sv || !d_pts || n <= 0 || !d_imus || n_imu <= 0) return VMP_ERR_INVALID_ARG;
    Package p;
    p.cookie = cookie;
    p.d_pts = d_pts;
    p.d_imus = d_imus;
    p.n = n;
    p.n_imu = n_imu;
    p.t_start = t_start;
    p.t_end = t_end;
    return enqueue(sv, id, std::move(p));
}

int vmp_poll(vmp_server_t sv, vmp_server_result* out, int max, int timeout_ms) {
    if (!sv || !out || max <= 0) return -1;
    std::unique_lock<std::mutex> lk(sv->mu);
    if (sv->done.empty() && timeout_ms > 0)
        sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !sv->done.empty() || sv->stop; });
    int n = 0;
    while (n < max && !sv->done.empty()) {
        out[n++] = sv->done.front();
        sv->done.pop_front();
    }
    return n;
}

vmp_status vmp_server_stream(vmp_server_t sv, int id, vmp_stream_t* out) {
    if (!sv || !out) return VMP_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(sv->mu);
    if (id < 0 || id >= (int)sv->slots.size() || !sv->slots[id].open) return VMP_ERR_INVALID_ARG;
    Slot& s = sv->slots[id];
    sv->cv_done.wait(lk, [&] { return sv->stop || (s.q.empty() && !s.busy); });
    *out = s.h;
    return VMP_OK;
}

vmp_status vmp_server_info(vmp_server_t sv, long long* budget_used, int* streams_open, int* queued, int* running) {
    if (!sv) return VMP_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (budget_used) *budget_used = sv->used;
    if (streams_open) {
        int n = 0;
        for (auto& s : sv->slots) n += s.open ? 1 : 0;
        *streams_open = n;
    }
    if (queued) *queued = sv->queued;
    if (running) *running = sv->running;
    return VMP_OK;
}

const char* vmp_server_last_error(vmp_server_t sv) {
    if (!sv) return "null server";
    std::lock_guard<std::mutex> lk(sv->mu);
    static thread_local std::string copy;
    copy = sv->err;
    return copy.c_str();
}

}  // extern "C"
