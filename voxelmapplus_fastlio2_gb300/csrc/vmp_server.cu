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
// HBM budget and a slot is free.  vmp_server_open_stream answers at once;
// vmp_server_open_stream_wait queues the request (arrival order) until a slot
// and the budget free up as streams close, or until its time limit.
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "vmp.h"

namespace vmp {
void merge_set_throughput_mode(bool on);
bool merge_throughput_mode();
void merge_set_grid_divisor(int d);
cudaError_t seg_set_grid_blocks(int blocks);
int seg_grid_blocks();
void residual_set_ctas_per_sm(int c);
int residual_ctas_per_sm();
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

// One knob of the online autotuner: a hill climb over its candidate values.
// From the current value (its rate measured), it measures one window at each
// neighbour; the fastest of the three becomes current, and the climb goes
// on from a new current until the current one wins ("settled").
struct KnobClimb {
    const char* name;
    std::vector<int> cand;
    std::function<void(int)> apply;
    int idx = 0;          // current candidate
    int probe = 3;        // 1: measuring idx + 1, 2: idx - 1, 3: not climbing
    double rate[3] = {};  // current, upper, lower

    int cur() const {
        const int i = probe == 1 ? idx + 1 : (probe == 2 ? idx - 1 : idx);
        return cand[i];
    }
    int next_probe(int p) const {
        if (p == 1 && idx + 1 >= (int)cand.size()) p = 2;
        if (p == 2 && idx - 1 < 0) p = 3;
        return p;
    }
    // starts a climb from the current value, whose rate is r; false: nothing
    // to probe
    bool start(double r) {
        rate[0] = r;
        probe = next_probe(1);
        return probe != 3;
    }
    // the rate of the window just measured at cur(); returns true once settled
    bool feed(double r) {
        rate[probe] = r;
        probe = next_probe(probe + 1);
        if (probe < 3) return false;
        int pick = 0;
        if (idx + 1 < (int)cand.size() && rate[1] > rate[pick]) pick = 1;
        if (idx - 1 >= 0 && rate[2] > rate[pick]) pick = 2;
        if (pick == 0) return true;
        idx += pick == 1 ? 1 : -1;
        rate[0] = rate[pick];
        probe = next_probe(1);
        return probe == 3;
    }
    void set_nearest(int v) {
        int bi = 0;
        for (int i = 1; i < (int)cand.size(); ++i)
            if (std::abs(cand[i] - v) < std::abs(cand[bi] - v)) bi = i;
        idx = bi;
    }
};

// Online autotuner of the served launch shapes: windows of kWindow completed
// packages (the first kSettle after a switch are not counted) measure the
// throughput of the current shapes; the knobs are climbed one after the
// other (coordinate-wise), then the shapes are kept for kExploit windows
// before the next round of climbs (the stream mix may have changed).  The
// first climb starts after kFirst windows (about 3 000 packages), so that
// short runs stay on the starting shapes, the best measured ones.  The
// knobs change scheduling only, never results, and none needs the streams'
// captured scan graphs to be captured again:
//   merge_grid_divisor  served merge launches use SMs / d CTAs;
//   max_inflight        packages on the GPU at once (of the workers' slots):
//                       fewer contend less for the hardware work queues,
//                       more overlap more;
//   seg_grid_blocks     blocks of the voxel-chain kernels that take work
//                       (a device-side value the captured launches read;
//                       they have 304 blocks while a server runs):
//                       fewer leave more SM slots to other streams' kernels,
//                       more run more of one scan's chains at once.
struct Autotuner {
    static constexpr int kWindow = 128, kSettle = 16, kExploit = 32, kFirst = 24;
    std::vector<KnobClimb> knobs;
    int active = -1;  // the knob being climbed (-1: exploiting)
    int exploit_left = kFirst;
    int seen = 0;
    double t_begin = 0.0;
    long long windows = 0;
    double best = 0.0;

    void apply_all() {
        for (auto& k : knobs) k.apply(k.cur());
    }
    // from knob `from` on, the first one with something to probe (rate r at
    // the current shapes); none: exploit
    void climb_from(int from, double r) {
        for (int k = from; k < (int)knobs.size(); ++k)
            if (knobs[k].start(r)) {
                active = k;
                knobs[k].apply(knobs[k].cur());
                return;
            }
        active = -1;
        exploit_left = kExploit;
    }
    // called at every completion (time in ms); applies the next shapes
    void on_done(double now_ms) {
        ++seen;
        if (seen == kSettle) t_begin = now_ms;
        if (seen < kSettle + kWindow) return;
        const double r = kWindow / ((now_ms - t_begin) * 1e-3);
        seen = 0;
        ++windows;
        if (r > best) best = r;
        if (active < 0) {
            if (--exploit_left > 0) return;
            climb_from(0, r);
            return;
        }
        KnobClimb& k = knobs[active];
        const bool settled = k.feed(r);
        k.apply(k.cur());
        if (settled) climb_from(active + 1, k.rate[0]);
    }
    int value(const char* name) const {
        for (const auto& k : knobs)
            if (std::strcmp(k.name, name) == 0) return k.cur();
        return -1;
    }
};

static void apply_merge_divisor(int d) { vmp::merge_set_grid_divisor(d); }
static void apply_seg_blocks(int b) { (void)vmp::seg_set_grid_blocks(b); }
// the launch shapes of vmp_test_autotune's model (one caller at a time)
static int g_model_d = 0, g_model_c = 0, g_model_s = 0;
static void model_set_d(int d) { g_model_d = d; }
static void model_set_c(int c) { g_model_c = c; }
static void model_set_s(int b) { g_model_s = b; }

constexpr int kDefaultSegBlocks = 152;  // 1 per SM: on the 64-stream mix 152 and 304 were the best of 152 .. 2432

static Autotuner make_tuner(int merge_divisor, int inflight, int seg_blocks, std::function<void(int)> set_d,
                            std::function<void(int)> set_c, std::function<void(int)> set_s) {
    Autotuner t;
    t.knobs.push_back(KnobClimb{"merge_grid_divisor", {4, 8, 16, 32, 64}, set_d});
    t.knobs.push_back(KnobClimb{"max_inflight", {8, 16, 24, 32}, set_c});
    t.knobs.push_back(KnobClimb{"seg_grid_blocks", {76, 152, 304}, set_s});
    t.knobs[0].set_nearest(merge_divisor);
    t.knobs[1].set_nearest(inflight);
    t.knobs[2].set_nearest(seg_blocks);
    return t;
}

struct vmp_server_s {
    vmp_server_config cfg{};
    Autotuner tuner;
    int fixed_divisor = 16;
    int fixed_seg_blocks = kDefaultSegBlocks;
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
    int max_inflight = 1 << 30;  // packages on the GPU at once (the autotuner's second knob)
    std::string err;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    // admission requests in arrival order (tickets); the front one is served
    std::condition_variable cv_admit;
    std::deque<unsigned long long> admit_q;
    unsigned long long admit_ticket = 0;
    unsigned long long closes = 0;  // streams closed so far (a create that ran out of memory retries after one)
    // measured device footprint of each stream configuration seen
    std::vector<std::pair<vmp_config, long long>> footprints;

    long long known_bytes(const vmp_config& c) const {
        for (const auto& f : footprints)
            if (std::memcmp(&f.first, &c, sizeof(vmp_config)) == 0) return f.second;
        return -1;
    }
    void remember_bytes(const vmp_config& c, long long b) {
        if (known_bytes(c) < 0) footprints.emplace_back(c, b);
    }
    int free_slot() const {
        for (int i = 0; i < (int)slots.size(); ++i)
            if (!slots[i].open && !slots[i].closing && !slots[i].h) return i;
        return -1;
    }

    double now_ms() const {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }

    // the ready stream whose oldest package was submitted first (-1: none, or
    // max_inflight packages running)
    int pick() const {
        if (running >= max_inflight) return -1;
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
            if (cfg.autotune && cfg.workers > 1) tuner.on_done(r.end_ms);
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
    c->seg_grid_blocks = kDefaultSegBlocks;
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
        const int s0 = cfg.seg_grid_blocks > 0 ? cfg.seg_grid_blocks : kDefaultSegBlocks;
        vmp::merge_set_grid_divisor(d0);
        apply_seg_blocks(s0);
        if (cfg.autotune) {  // the climbs start at the candidates nearest the configured shapes
            // (applied under the server lock: the tuner runs in on_done, called with it held)
            sv->tuner = make_tuner(d0, cfg.workers, s0, apply_merge_divisor, [sv](int c) {
                sv->max_inflight = c;
                sv->cv_work.notify_all();
            }, apply_seg_blocks);
            sv->tuner.apply_all();
        }
        sv->fixed_divisor = d0;
        sv->fixed_seg_blocks = s0;
    }
    for (int i = 0; i < cfg.workers; ++i) sv->workers.emplace_back([sv] { sv->worker(); });
    *out = sv;
    return VMP_OK;
}

vmp_status vmp_server_tuning(vmp_server_t sv, int* merge_grid_divisor, long long* windows, double* best_rate) {
    if (!sv) return VMP_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (merge_grid_divisor)
        *merge_grid_divisor =
            sv->cfg.autotune && sv->cfg.workers > 1 ? sv->tuner.value("merge_grid_divisor") : sv->fixed_divisor;
    if (windows) *windows = sv->tuner.windows;
    if (best_rate) *best_rate = sv->tuner.best;
    return VMP_OK;
}

vmp_status vmp_server_destroy(vmp_server_t sv) {
    if (!sv) return VMP_ERR_INVALID_ARG;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        sv->stop = true;
        sv->cv_admit.notify_all();
        // admission requests still waiting return VMP_ERR_STATE; wait until they left
        sv->cv_admit.wait(lk, [&] { return sv->admit_q.empty(); });
    }
    sv->cv_work.notify_all();
    for (auto& t : sv->workers) t.join();
    for (auto& s : sv->slots)
        if (s.h) vmp_destroy(s.h);
    if (sv->cfg.workers > 1) {
        vmp::merge_set_throughput_mode(false);
        if (!vmp::merge_throughput_mode()) apply_seg_blocks(0);  // the last server: every block works again
    }
    delete sv;
    return VMP_OK;
}

// Admission of one stream (timeout_ms: 0 answer at once, < 0 no limit).
static vmp_status open_stream(vmp_server_t sv, const vmp_config* cfg_in, int timeout_ms, int* stream_id) {
    if (!sv || !stream_id) return VMP_ERR_INVALID_ARG;
    *stream_id = -1;
    vmp_config cfg;
    if (cfg_in) cfg = *cfg_in; else vmp_config_default(&cfg);
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms > 0 ? timeout_ms : 0);
    std::unique_lock<std::mutex> lk(sv->mu);
    const unsigned long long ticket = sv->admit_ticket++;
    sv->admit_q.push_back(ticket);
    auto leave = [&](vmp_status st, const std::string& why) {
        for (auto it = sv->admit_q.begin(); it != sv->admit_q.end(); ++it)
            if (*it == ticket) { sv->admit_q.erase(it); break; }
        if (!why.empty()) sv->err = why;
        sv->cv_admit.notify_all();
        return st;
    };
    // waits for `pred`; false when the time limit passed first
    auto wait_for = [&](const std::function<bool()>& pred) {
        if (pred()) return true;
        if (timeout_ms == 0) return false;
        if (timeout_ms < 0) { sv->cv_admit.wait(lk, pred); return true; }
        return sv->cv_admit.wait_until(lk, deadline, pred);
    };
    const long long budget = sv->cfg.hbm_budget_bytes;
    for (;;) {
        const long long kb = sv->known_bytes(cfg);
        if (kb > budget)
            return leave(VMP_ERR_ADMISSION_DENIED, "stream footprint " + std::to_string(kb) + " bytes > HBM budget");
        const bool ready = wait_for([&] {
            if (sv->stop) return true;
            const long long k = sv->known_bytes(cfg);
            return sv->admit_q.front() == ticket && sv->free_slot() >= 0 && (k < 0 || sv->used + k <= budget);
        });
        if (sv->stop) return leave(VMP_ERR_STATE, "server is shutting down");
        if (!ready) {
            if (timeout_ms != 0) return leave(VMP_ERR_TIMEOUT, "admission wait ran out");
            const long long k = sv->known_bytes(cfg);
            if (sv->free_slot() < 0) return leave(VMP_ERR_ADMISSION_DENIED, "no free stream slot");
            return leave(VMP_ERR_ADMISSION_DENIED, "HBM budget: " + std::to_string(sv->used) + " + " +
                                                       std::to_string(k) + " bytes > " + std::to_string(budget));
        }
        const int id = sv->free_slot();
        sv->slots[id].closing = true;  // reserved while the stream is created
        const unsigned long long closes0 = sv->closes;
        lk.unlock();
        vmp_stream_t h = nullptr;
        const vmp_status st = vmp_create(&cfg, &h);
        const long long b = st == VMP_OK ? vmp_device_bytes(h) : 0;
        lk.lock();
        sv->slots[id].closing = false;
        if (st == VMP_ERR_OUT_OF_MEMORY && timeout_ms != 0) {
            // the device is full: try again once a stream has closed
            if (!wait_for([&] { return sv->stop || sv->closes != closes0; }))
                return leave(VMP_ERR_TIMEOUT, "admission wait ran out (device memory)");
            continue;
        }
        if (st != VMP_OK) return leave(st, std::string("vmp_create: ") + vmp_last_error(nullptr));
        if (sv->stop) {
            lk.unlock();
            vmp_destroy(h);
            lk.lock();
            return leave(VMP_ERR_STATE, "server is shutting down");
        }
        sv->remember_bytes(cfg, b);
        if (b > budget || sv->used + b > budget) {
            lk.unlock();
            vmp_destroy(h);
            lk.lock();
            if (b > budget || timeout_ms == 0)
                return leave(VMP_ERR_ADMISSION_DENIED, "HBM budget: " + std::to_string(sv->used) + " + " +
                                                           std::to_string(b) + " bytes > " + std::to_string(budget));
            continue;  // footprint now known: wait for the budget
        }
        vmp_set_wait_mode(h, 1);
        sv->used += b;
        Slot& sl = sv->slots[id];
        sl.open = true;
        sl.busy = false;
        sl.h = h;
        sl.bytes = b;
        sl.q.clear();
        *stream_id = id;
        return leave(VMP_OK, "");
    }
}

vmp_status vmp_server_open_stream(vmp_server_t sv, const vmp_config* cfg, int* stream_id) {
    return open_stream(sv, cfg, 0, stream_id);
}

vmp_status vmp_server_open_stream_wait(vmp_server_t sv, const vmp_config* cfg, int timeout_ms, int* stream_id) {
    return open_stream(sv, cfg, timeout_ms, stream_id);
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
    lk.unlock();
    vmp_destroy(h);
    lk.lock();
    sv->used -= s.bytes;  // released once its memory is freed
    s.bytes = 0;
    s.closing = false;
    ++sv->closes;
    sv->cv_admit.notify_all();
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

vmp_status vmp_server_knob(vmp_server_t sv, const char* name, int* value) {
    if (!sv || !name || !value) return VMP_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (std::strcmp(name, "merge_grid_divisor") == 0) {
        *value = sv->cfg.autotune && sv->cfg.workers > 1 ? sv->tuner.value(name) : sv->fixed_divisor;
        return VMP_OK;
    }
    if (std::strcmp(name, "seg_grid_blocks") == 0) {
        *value = sv->cfg.workers <= 1 ? vmp::seg_grid_blocks()
                 : sv->cfg.autotune  ? sv->tuner.value(name)
                                     : sv->fixed_seg_blocks;
        return VMP_OK;
    }
    if (std::strcmp(name, "max_inflight") == 0) {
        *value = sv->max_inflight < sv->cfg.workers ? sv->max_inflight : sv->cfg.workers;
        return VMP_OK;
    }
    if (std::strcmp(name, "residual_ctas_per_sm") == 0) {
        *value = vmp::residual_ctas_per_sm();
        return VMP_OK;
    }
    return VMP_ERR_INVALID_ARG;
}

// Test hook: the autotuner's climb on a model throughput instead of a GPU.
// rates[(i * 4 + j) * 3 + k]: packages/s with merge divisor candidate i (4,
// 8, 16, 32, 64), max_inflight candidate j (8, 16, 24, 32) and
// seg_grid_blocks candidate k (76, 152, 304); completions are spaced by
// 1 / rate.  trace[3 * w .. 3 * w + 2]: the three knobs after
// window w.
vmp_status vmp_test_autotune(int merge_divisor, int max_inflight, int seg_blocks, const double* rates, int windows,
                             int* trace) {
    if (!rates || !trace || windows < 0) return VMP_ERR_INVALID_ARG;
    Autotuner t = make_tuner(merge_divisor, max_inflight, seg_blocks, model_set_d, model_set_c, model_set_s);
    t.apply_all();
    double now = 0.0;
    for (int w = 0; w < windows;) {
        int di = 0;
        for (int i = 0; i < (int)t.knobs[0].cand.size(); ++i)
            if (t.knobs[0].cand[i] == g_model_d) di = i;
        int ci = 0;
        for (int i = 0; i < (int)t.knobs[1].cand.size(); ++i)
            if (t.knobs[1].cand[i] == g_model_c) ci = i;
        int si = 0;
        for (int i = 0; i < (int)t.knobs[2].cand.size(); ++i)
            if (t.knobs[2].cand[i] == g_model_s) si = i;
        const double r = rates[(di * 4 + ci) * 3 + si];
        if (!(r > 0.0)) return VMP_ERR_INVALID_ARG;
        now += 1000.0 / r;
        const long long before = t.windows;
        t.on_done(now);
        if (t.windows != before) {
            trace[3 * w] = g_model_d;
            trace[3 * w + 1] = g_model_c;
            trace[3 * w + 2] = g_model_s;
            ++w;
        }
    }
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
