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
void merge_set_grid_divisor(int d);
}

namespace {

struct Package {
    long long cookie = 0;
    std::vector<vmp_point> pts;
    std::vector<vmp_imu> imus;
    // vmp_submit_livox: the raw message, decoded by the worker
    std::vector<vmp_livox_point> livox;
    bool is_livox = false;
    int filter_num = 1;
    double range_min = 0.0, range_max = 0.0;
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

// Online autotuner of the served merge launch shape, a hill climb over the
// grid divisors kCand: a window of completed packages at the current divisor
// (the first packages after a switch are not counted), then one at each
// neighbour; the fastest of the three becomes current.  When the current one
// wins, it is kept for kExploit windows before its neighbours are measured
// again (the stream mix may have changed).  It starts at 16 (measured best
// on 64 mixed streams) and climbs first after kFirst windows, so short runs
// pay nothing for the exploration.
struct MergeTuner {
    static constexpr int kWindow = 128, kSettle = 16, kExploit = 32, kN = 5;
    static constexpr int kCand[kN] = {4, 8, 16, 32, 64};
    static constexpr int kFirst = 8;  // windows at the starting divisor before the first climb
    int idx = 2;             // current candidate
    int probe = 3;           // 0: current, 1: idx + 1, 2: idx - 1, 3: exploiting
    int exploit_left = kFirst;
    int seen = 0;            // packages completed in the window (settling first)
    double t_begin = 0.0;
    double rate[3] = {};     // current, upper, lower
    long long windows = 0;
    double best = 0.0;

    int cur() const {
        const int i = probe == 1 ? idx + 1 : (probe == 2 ? idx - 1 : idx);
        return kCand[i];
    }
    // the next probe that has a candidate, from `p` on
    int next_probe(int p) const {
        if (p == 1 && idx + 1 >= kN) p = 2;
        if (p == 2 && idx - 1 < 0) p = 3;
        return p;
    }
    // called under the server lock at every completion; returns the divisor
    // to switch to, or 0
    int on_done(double now_ms) {
        ++seen;
        if (seen == kSettle) t_begin = now_ms;
        if (seen < kSettle + kWindow) return 0;
        const double r = kWindow / ((now_ms - t_begin) * 1e-3);
        seen = 0;
        ++windows;
        if (r > best) best = r;
        if (probe == 3) {
            if (--exploit_left > 0) return 0;
            rate[0] = r;  // the current one, freshly measured
            probe = next_probe(1);
            return probe == 3 ? 0 : cur();
        }
        rate[probe] = r;
        probe = next_probe(probe + 1);
        if (probe < 3) return cur();
        int pick = 0;  // decide among current / upper / lower
        if (idx + 1 < kN && rate[1] > rate[pick]) pick = 1;
        if (idx - 1 >= 0 && rate[2] > rate[pick]) pick = 2;
        if (pick == 0) {
            exploit_left = kExploit;
        } else {
            idx += pick == 1 ? 1 : -1;
            rate[0] = rate[pick];
            probe = next_probe(1);
            if (probe == 3) exploit_left = kExploit;
        }
        return cur();
    }
};
constexpr int MergeTuner::kCand[MergeTuner::kN];

struct vmp_server_s {
    vmp_server_config cfg{};
    MergeTuner tuner;
    int fixed_divisor = 16;
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
            if (p.is_livox) {
                int m = 0;
                float last_t = 0.f;
                r.status = vmp_livox_decode(h, p.livox.data(), (int)p.livox.size(), p.filter_num, p.range_min,
                                            p.range_max, nullptr, nullptr, &m, &last_t);
                if (r.status == VMP_OK && m <= 0) r.status = VMP_ERR_INVALID_ARG;
                if (r.status == VMP_OK) {
                    const double t_end = p.t_start + (double)last_t / 1000.0;  // lio_node.cpp:146
                    r.status = vmp_process_decoded(h, p.t_start, t_end, p.imus.data(), (int)p.imus.size(),
                                                   &r.result);
                }
            } else if (p.d_pts) {
                r.status = vmp_process_device(h, p.d_pts, p.n, p.t_start, p.t_end, p.d_imus, p.n_imu, &r.result);
            } else {
                vmp_scan scan{p.pts.data(), (int)p.pts.size(), p.t_start, p.t_end};
                r.status = vmp_process(h, &scan, p.imus.data(), (int)p.imus.size(), &r.result);
            }
            r.end_ms = now_ms();
            lk.lock();
            sl.busy = false;
            --running;
            if (cfg.autotune && cfg.workers > 1) {
                const int d = tuner.on_done(r.end_ms);
                if (d > 0) vmp::merge_set_grid_divisor(d);
            }
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
    c->autotune = 1;
    c->merge_grid_divisor = 16;
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
    if (cfg.workers > 1) {
        vmp::merge_set_throughput_mode(true);
        const int d0 = cfg.merge_grid_divisor > 0 ? cfg.merge_grid_divisor : 16;
        vmp::merge_set_grid_divisor(d0);
        if (cfg.autotune) {  // the climb starts at the candidate nearest the configured divisor
            int bi = 0;
            for (int i = 1; i < MergeTuner::kN; ++i)
                if (std::abs(MergeTuner::kCand[i] - d0) < std::abs(MergeTuner::kCand[bi] - d0)) bi = i;
            sv->tuner.idx = bi;
            vmp::merge_set_grid_divisor(sv->tuner.cur());
        }
        sv->fixed_divisor = d0;
    }
    for (int i = 0; i < cfg.workers; ++i) sv->workers.emplace_back([sv] { sv->worker(); });
    *out = sv;
    return VMP_OK;
}

vmp_status vmp_server_tuning(vmp_server_t sv, int* merge_grid_divisor, long long* windows, double* best_rate) {
    if (!sv) return VMP_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (merge_grid_divisor)
        *merge_grid_divisor = sv->cfg.autotune && sv->cfg.workers > 1 ? sv->tuner.cur() : sv->fixed_divisor;
    if (windows) *windows = sv->tuner.windows;
    if (best_rate) *best_rate = sv->tuner.best;
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

vmp_status vmp_submit_livox(vmp_server_t sv, int id, const vmp_livox_point* pts, int n, int filter_num,
                            double range_min, double range_max, double t_start, const vmp_imu* imus, int n_imu,
                            long long cookie) {
    if (!sv || n < 0 || (n > 0 && !pts) || filter_num < 1 || n_imu <= 0 || !imus) return VMP_ERR_INVALID_ARG;
    Package p;
    p.cookie = cookie;
    p.is_livox = true;
    p.livox.assign(pts, pts + n);
    p.imus.assign(imus, imus + n_imu);
    p.filter_num = filter_num;
    p.range_min = range_min;
    p.range_max = range_max;
    p.t_start = t_start;
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
