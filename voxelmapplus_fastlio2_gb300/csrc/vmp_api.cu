// Host orchestration and the C ABI of libvmp (include/vmp.h).
//
// One vmp_stream owns a CUDA stream and every device buffer of one sensor
// stream.  vmp_process follows LIOBuilder::process (lio_builder.cpp:175-248):
//   IMU_INIT     accumulate IMU samples on the host until imu_init_num, then
//                k_imu_init on the device;
//   MAP_INIT     upload -> time sort -> IMU predict chain -> undistort ->
//                float world transform + covariances of the full cloud ->
//                VoxelMap::build;
//   LIO_MAPPING  upload -> time sort -> predict chain -> undistort ->
//                downsample -> calcBodyCov -> IESKF::update (ieskf_max_iter
//                residual launches; the last CTA of each runs the FP64 step,
//                later launches return at once after convergence) ->
//                covariance update -> world points -> VoxelMap::update.
// The scan's kernels are enqueued without host synchronisation; the call
// ends with one device->host copy of the result.  Two conditions add a host
// round trip: an IEKF-independent merge fixed point (one small read per
// round, k_merge.cu) and a batch that can overflow the LRU capacity (the
// eviction walk is read back to decide a split).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <new>
#include <string>
#include <vector>

#include "kernels.cuh"

using namespace vmp;

namespace {

struct DResult {
    DState x;
    double P[529];
    int iters;
    int effect_num;
    int no_effect;
    int n_down;
    Counters cnt;
};

__global__ void k_gather_result(const DFilter* f, const int* d_n_down, const Counters* c, DResult* r) {
    for (int e = threadIdx.x; e < 529; e += blockDim.x) r->P[e] = f->P[e];
    if (threadIdx.x == 0) {
        r->x = f->x;
        r->iters = f->iters;
        r->effect_num = f->effect_num;
        r->no_effect = f->no_effect;
        r->n_down = d_n_down ? *d_n_down : 0;
        r->cnt = *c;
    }
}
__global__ void k_clear_error(Counters* c) {
    if (threadIdx.x == 0) c->error = 0;
}
__global__ void k_set_int(int* p, int v) {
    if (threadIdx.x == 0) *p = v;
}
__global__ void k_copy_int(int* dst, const int* src) {
    if (threadIdx.x == 0) *dst = *src;
}
__global__ void k_floats_to_points(const float* pts, int n, float4* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = make_float4(pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2], 0.0f);
}
__global__ void k_reset_filter_iter(DFilter* f) {
    if (threadIdx.x == 0) { f->converged = 0; f->iters = 0; f->effect_num = 0; f->no_effect = 0; }
}
__global__ void k_read_hm(const DFilter* f, double* H, double* b, int* eff) {
    for (int e = threadIdx.x; e < 144; e += blockDim.x) H[e] = f->Hm[e];
    if (threadIdx.x < 12) b[threadIdx.x] = f->bm[threadIdx.x];
    if (threadIdx.x == 0) *eff = f->effect_num;
}

// Export of live records (device -> vmp_voxel).
__global__ void k_export(DMap m, vmp_voxel* out, int* d_count, int max) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m.rec_pool; r += gridDim.x * blockDim.x) {
        const RecHot& h = m.hot[r];
        if (!(h.flags & F_ALIVE)) continue;
        int pos = atomicAdd(d_count, 1);
        if (pos >= max) continue;
        const RecCold& c = m.cold[r];
        vmp_voxel& v = out[pos];
        int64_t x, y, z;
        unpack_key(c.key, x, y, z);
        v.key[0] = x; v.key[1] = y; v.key[2] = z;
        v.n = h.n;
        v.newly_add_point = c.newly;
        v.is_init = (h.flags & F_INIT) ? 1 : 0;
        v.is_plane = (h.flags & F_PLANE) ? 1 : 0;
        v.update_enable = (h.flags & F_UPDATE) ? 1 : 0;
        v.merged = (h.flags & F_MERGED) ? 1 : 0;
        v.group_id = h.group;
        v.lru_stamp = c.stamp;
        v.n_temp = (h.flags & F_DROPPED) ? h.n : c.nslab;
        v.pad = (int32_t)(r | ((h.flags & F_DROPPED) ? 0x40000000u : 0u));  // record id + "points not kept"
        for (int k = 0; k < 3; ++k) { v.mean[k] = h.mean[k]; v.norm[k] = h.norm[k]; v.center[k] = c.center[k]; }
        for (int k = 0; k < 9; ++k) v.ppt[k] = c.ppt[k];
        for (int k = 0; k < 36; ++k) v.cov[k] = c.cov[k];
    }
}
// Keys and LRU stamps of the live records (for vmp_map_keys).
__global__ void k_export_keys(DMap m, unsigned long long* out /* [max][2] */, int* d_count, int max) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m.rec_pool; r += gridDim.x * blockDim.x) {
        if (!(m.hot[r].flags & F_ALIVE)) continue;
        const int pos = atomicAdd(d_count, 1);
        if (pos >= max) continue;
        out[2 * (size_t)pos] = m.cold[r].stamp;
        out[2 * (size_t)pos + 1] = m.cold[r].key;
    }
}
// Test hook: the shared-divisor division against the FP64 division, per pair.
__global__ void k_div_check(const double* a, const double* b, int n, double* by_recip, double* by_div) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double y = 1.0 / b[i];
        by_recip[i] = div_recip_ok(b[i]) ? div_by_recip(a[i], b[i], y) : __ddiv_rn(a[i], b[i]);
        by_div[i] = __ddiv_rn(a[i], b[i]);
    }
}

// ---- voxel-map export for visualisation (voxel2MarkerArray, utils.cpp:154-208)
// Frozen planes (is_plane && !update_enable) with their LRU stamps, as sort
// keys that order the most recently touched first (complemented halves).
__global__ void k_plane_collect(DMap m, int* d_count, uint32_t* key_lo, uint32_t* key_hi, uint32_t* rec, int cap) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m.rec_pool; r += gridDim.x * blockDim.x) {
        const uint32_t f = m.hot[r].flags;
        if (!(f & F_ALIVE) || !(f & F_PLANE) || (f & F_UPDATE)) continue;
        const int pos = atomicAdd(d_count, 1);
        if (pos >= cap) continue;
        const uint64_t st = m.cold[r].stamp;
        key_lo[pos] = ~(uint32_t)st;
        key_hi[pos] = ~(uint32_t)(st >> 32);
        rec[pos] = (uint32_t)r;
    }
}
__global__ void k_iota_u32(uint32_t* v, const int* d_n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < *d_n; i += gridDim.x * blockDim.x) v[i] = (uint32_t)i;
}
__global__ void k_permute_pair(const uint32_t* perm, const uint32_t* a, const uint32_t* b, uint32_t* a2,
                               uint32_t* b2, const int* d_n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < *d_n; i += gridDim.x * blockDim.x) {
        a2[i] = a[perm[i]];
        b2[i] = b[perm[i]];
    }
}
// mapJet (utils.cpp:78-128) on v in [0, 1].
__device__ void map_jet(double v, uint8_t* rgb) {
    if (v < 0.0) v = 0.0;
    if (v > 1.0) v = 1.0;
    double dr, dg, db;
    if (v < 0.1242) { db = 0.504 + ((1. - 0.504) / 0.1242) * v; dg = dr = 0.; }
    else if (v < 0.3747) { db = 1.; dr = 0.; dg = (v - 0.1242) * (1. / (0.3747 - 0.1242)); }
    else if (v < 0.6253) { db = (0.6253 - v) * (1. / (0.6253 - 0.3747)); dg = 1.; dr = (v - 0.3747) * (1. / (0.6253 - 0.3747)); }
    else if (v < 0.8758) { db = 0.; dr = 1.; dg = (0.8758 - v) * (1. / (0.8758 - 0.6253)); }
    else { db = 0.; dg = 0.; dr = 1. - (v - 0.8758) * ((1. - 0.504) / (1. - 0.8758)); }
    rgb[0] = (uint8_t)(255 * dr);
    rgb[1] = (uint8_t)(255 * dg);
    rgb[2] = (uint8_t)(255 * db);
}
// Rotation taking (0, 0, 1) onto n (Quaternion::setFromTwoVectors as
// calcVectQuation uses it, utils.cpp:144-152), w x y z.  Antiparallel
// (c < -1 + 1e-12): a rotation by pi about the x axis.
__device__ void quat_from_z(const double* n0, double* q) {
    const double nn = sqrt(n0[0] * n0[0] + n0[1] * n0[1] + n0[2] * n0[2]);
    const double v1[3] = {n0[0] / nn, n0[1] / nn, n0[2] / nn};
    const double c = v1[2];
    if (c < -1.0 + 1e-12) {
        q[0] = 0.0; q[1] = 1.0; q[2] = 0.0; q[3] = 0.0;
        return;
    }
    // (0, 0, 1) x v1
    const double axis[3] = {-v1[1], v1[0], 0.0};
    const double sq = sqrt((1.0 + c) * 2.0);
    const double invs = 1.0 / sq;
    q[0] = sq * 0.5;
    for (int k = 0; k < 3; ++k) q[1 + k] = axis[k] * invs;
}
__global__ void k_plane_markers(DMap m, const uint32_t* rec_sorted, int n, vmp_plane_marker* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t r = rec_sorted[i];
        const RecHot& h = m.hot[r];
        const RecCold& c = m.cold[r];
        vmp_plane_marker o;
        for (int k = 0; k < 3; ++k) { o.center[k] = c.center[k]; o.norm[k] = h.norm[k]; }
        double trace = (c.cov[0] + c.cov[7]) + c.cov[14];
        o.trace = trace;
        if (trace >= 0.25) trace = 0.25;
        trace = trace * (1.0 / 0.25);
        trace = pow(trace, 0.2);
        map_jet(trace, o.rgb);
        o.merged = (h.flags & F_MERGED) ? 1 : 0;
        o.pad = 0;
        quat_from_z(o.norm, o.orientation);
        out[i] = o;
    }
}

// Buffered points of the given records (offsets = prefix of their counts).
__global__ void k_export_points(DMap m, const int* recs, const long long* offs, int nrec, double* pts, double* cov) {
    for (int q = blockIdx.x; q < nrec; q += gridDim.x) {
        const int r = recs[q];
        const RecCold& c = m.cold[r];
        const long long o = offs[q];
        for (int j = threadIdx.x; j < c.nslab; j += blockDim.x) {
            const double* s = m.slab + ((size_t)c.chunks[j / kChunkPts] * kChunkPts + (j % kChunkPts)) * kSlabStride;
            for (int k = 0; k < 3; ++k) pts[(o + j) * 3 + k] = s[k];
            for (int k = 0; k < 9; ++k) cov[(o + j) * 9 + k] = s[3 + k];
        }
    }
}
// Import: record q takes id q; LRU order given by the list (q = 0 most recent).
__global__ void k_import(DMap m, const vmp_voxel* vox, int n, const long long* offs, const double* pts,
                         const double* cov, unsigned long long stamp_top) {
    for (int q = blockIdx.x; q < n; q += gridDim.x) {
        const vmp_voxel& v = vox[q];
        const int r = q;
        RecHot& h = m.hot[r];
        RecCold& c = m.cold[r];
        int ncopy = v.n_temp;
        // buffered points that no refit can use any more are not kept: an
        // updating voxel at or over max_point_thresh freezes on its next point
        // before newly_add_point reaches update_size_thresh
        bool dropped = v.update_enable && v.is_init && v.n_temp >= m.max_thresh &&
                       v.newly_add_point + 1 < m.update_thresh;
        if (!dropped && ncopy > kMaxChunks * kChunkPts) {
            if (threadIdx.x == 0) set_error(m.cnt, E_CAPACITY);
            ncopy = kMaxChunks * kChunkPts;
        }
        if (threadIdx.x == 0) {
            for (int k = 0; k < 3; ++k) { h.mean[k] = v.mean[k]; h.norm[k] = v.norm[k]; c.center[k] = v.center[k]; }
            for (int k = 0; k < 9; ++k) c.ppt[k] = v.ppt[k];
            for (int k = 0; k < 36; ++k) c.cov[k] = v.cov[k];
            uint32_t fl = F_ALIVE;
            if (v.is_init) fl |= F_INIT;
            if (v.is_plane) fl |= F_PLANE;
            if (v.update_enable) fl |= F_UPDATE;
            if (v.merged) fl |= F_MERGED;
            if (dropped) fl |= F_DROPPED;
            h.flags = fl;
            h.n = v.n;
            h.group = v.group_id;
            c.key = pack_key(v.key[0], v.key[1], v.key[2]);
            c.stamp = stamp_top - (unsigned long long)q;
            c.create_g = 0;
            c.freeze_g = v.update_enable ? kNever : 0ull;
            c.evict_g = kNever;
            c.touch_first_g = kNever;
            c.newly = v.newly_add_point;
            c.nslab = 0;
            for (int k = 0; k < kMaxChunks; ++k) c.chunks[k] = -1;
            // slab chunks: ids taken from the end of the pool, record q -> a fixed range
            if (!dropped && ncopy > 0) {
                int nch = (ncopy + kChunkPts - 1) / kChunkPts;
                int base_chunk = atomicAdd(&m.cnt->chunk_freed_top, nch);  // bump counter (reset below)
                if (base_chunk + nch <= m.chunk_pool) {
                    for (int k = 0; k < nch; ++k) c.chunks[k] = m.chunk_pool - 1 - (base_chunk + k);
                    c.nslab = ncopy;
                } else {
                    set_error(m.cnt, E_CHUNKS);
                }
            }
            // hash insert
            uint64_t key = c.key;
            uint64_t hh = hash_key(key) & m.table_mask;
            for (uint64_t probe = 0; probe <= m.table_mask; ++probe) {
                unsigned long long prev = atomicCAS((unsigned long long*)&m.keys[hh], (unsigned long long)kEmptyKey,
                                                    (unsigned long long)key);
                if (prev == kEmptyKey) { m.vals[hh] = (uint32_t)r; break; }
                hh = (hh + 1) & m.table_mask;
            }
            // LRU queue: oldest first
            m.q_rec[n - 1 - q] = (uint32_t)r;
            m.q_stamp[n - 1 - q] = c.stamp;
        }
        __syncthreads();
        if (!dropped && c.nslab > 0) {
            const long long o = offs[q];
            for (int j = threadIdx.x; j < c.nslab; j += blockDim.x) {
                double* s = m.slab + ((size_t)c.chunks[j / kChunkPts] * kChunkPts + (j % kChunkPts)) * kSlabStride;
                for (int k = 0; k < 3; ++k) s[k] = pts[(o + j) * 3 + k];
                for (int k = 0; k < 9; ++k) s[3 + k] = cov[(o + j) * 9 + k];
            }
        }
    }
}
__global__ void k_import_counters(DMap m, int n, long long group_counter, unsigned long long stamp_top) {
    if (threadIdx.x != 0) return;
    Counters* c = m.cnt;
    int used_chunks = c->chunk_freed_top;
    if (used_chunks > m.chunk_pool) used_chunks = m.chunk_pool;
    c->chunk_freed_top = 0;
    c->chunk_free_top = m.chunk_pool - used_chunks;
    // records 0..n-1 are taken; the free stack holds n..pool-1 (pops give n, n+1, ...)
    for (int i = 0; i < m.rec_pool - n; ++i) m.rec_free[i] = (uint32_t)(m.rec_pool - 1 - i);
    c->rec_free_top = m.rec_pool - n;
    c->size = n;
    c->group_counter = group_counter;
    c->batch_base = stamp_top + 1;
    c->q_head = 0;
    c->q_tail = (unsigned long long)n;
    c->n_tomb = 0;
}

inline size_t next_pow2(size_t v) {
    size_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

}  // namespace

struct vmp_stream_s {
    vmp_config cfg{};
    cudaStream_t st = nullptr;
    std::string err;
    int lio_status = VMP_IMU_INIT;
    std::vector<vmp_imu> imu_cache;
    DFilter* f = nullptr;
    DScan s{};
    DMap m{};
    Counters* cnt = nullptr;
    MapScratch ms{};
    SortScratch ss{};
    ScanScratch sc{};
    vmp_point* h_pts = nullptr;
    vmp_imu* h_imus = nullptr;
    DResult* h_res = nullptr;
    DResult* d_res = nullptr;
    Counters* h_cnt = nullptr;
    int* h_int = nullptr;
    double sin_deg = 0.0;
    long long h_size = 0;
    unsigned long long h_qlen = 0;
    int h_tomb = 0;
    // LRU queue compaction scratch
    uint32_t* qc_flag = nullptr;
    uint32_t* qc_rank = nullptr;
    uint32_t* qc_rec = nullptr;
    uint64_t* qc_stamp = nullptr;
    int* qc_ints = nullptr;
    ScanScratch qsc{};
    std::vector<void*> allocs;
    bool broken = false;
    long long last_evicted_total = 0;
    long long dev_bytes = 0;  // device memory allocated by vmp_create
    long long eviction_splits = 0;  // batches split by the eviction walk
    DScanHdr* h_hdr = nullptr;      // pinned staging of the scan header
    // captured graphs of the steady-state scan, per size class: g1 = time
    // sort .. voxel state machine, g2 = LRU queue .. result copy (the merge
    // resolution runs between them)
    // g1 / g2: the steady scan around the merge resolution; g0: the scan
    // front alone (time sort to map batch), for scans whose map update may
    // evict and therefore runs its map part with host decisions
    struct ScanGraphs { int nb; cudaGraphExec_t g1, g2, g0; long long k1, k2, k0; long long epoch; };
    std::deque<ScanGraphs> graphs;
    bool use_graphs = true;
    // vmp_map_planes scratch (allocated by its first call)
    SortScratch vis_ss{};
    uint32_t* vis_buf = nullptr;  // 6 arrays of rec_pool + 16 u32, then the count
    int decoded_n = -1;  // points of a vmp_livox_decode cloud waiting for vmp_process_decoded
    int cloud_n = 0;     // points of the last processed scan's undistorted cloud
    bool blocking_wait = false;  // vmp_set_wait_mode
    cudaEvent_t done_ev = nullptr;
    // the IMU predict chain runs beside the time sort (they share no data):
    // forked onto st_side and joined before the undistortion
    cudaStream_t st_side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_cov = nullptr;
    // CUDA-event profiler (vmp_profile_enable): per pipeline phase, events on
    // the stream's own CUDA stream, resolved after the call's final sync
    struct ProfRec { int slot; int items_kind; cudaEvent_t a, b; };
    long long io_h2d = 0, io_d2h = 0;  // bytes copied host<->device by the library
    bool prof_on = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<ProfRec> prof_pending;
    cudaEvent_t prof_open = nullptr;
    double prof_ms[VMP_PROF_SLOTS] = {};
    long long prof_launches[VMP_PROF_SLOTS] = {};
    long long prof_items[VMP_PROF_SLOTS] = {};
    int cur_batch_kind = 1;

    cudaEvent_t ev() {
        if (ev_used == ev_pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev_pool.push_back(e);
        }
        return ev_pool[ev_used++];
    }
    void pbeg() {
        if (!prof_on) return;
        prof_open = ev();
        cudaEventRecord(prof_open, st);
    }
    // items_kind: 0 raw points, 1 downsampled points, 2 map batch points, -1 none
    void pend(int slot, int items_kind) {
        if (!prof_on || !prof_open) return;
        cudaEvent_t b = ev();
        cudaEventRecord(b, st);
        prof_pending.push_back(ProfRec{slot, items_kind, prof_open, b});
        prof_open = nullptr;
    }
    // after the stream is synchronised
    void pflush(int iters, int n_raw, int n_down, int n_batch) {
        if (!prof_on) { prof_pending.clear(); ev_used = 0; return; }
        int res_seen = 0;
        for (const ProfRec& r : prof_pending) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) { cudaGetLastError(); continue; }
            int slot = r.slot;
            if (slot == VMP_PROF_RESIDUAL) {
                if (res_seen >= iters) slot = VMP_PROF_RESIDUAL_IDLE;
                ++res_seen;
            } else if (slot == VMP_PROF_RESIDUAL_STEP && res_seen > iters) {
                slot = VMP_PROF_RESIDUAL_IDLE;  // the fold launch after convergence
            }
            prof_ms[slot] += ms;
            prof_launches[slot] += 1;
            long long it = r.items_kind == 0 ? n_raw : r.items_kind == 1 ? n_down : r.items_kind == 2 ? n_batch : 0;
            if (slot == VMP_PROF_RESIDUAL_IDLE) it = 0;
            prof_items[slot] += it;
        }
        prof_pending.clear();
        ev_used = 0;
    }
};

static thread_local std::string g_create_error;

static vmp_status fail(vmp_stream_t s, vmp_status code, const std::string& msg) {
    if (s) s->err = msg;
    return code;
}
static vmp_status cuda_fail(vmp_stream_t s, cudaError_t e, const char* where) {
    if (s) {
        s->err = std::string(where) + ": " + cudaGetErrorString(e);
        s->broken = true;
    }
    return VMP_ERR_CUDA;
}

#define VMP_TRY(expr, where)                          \
    do {                                              \
        cudaError_t e_ = (expr);                      \
        if (e_ != cudaSuccess) return cuda_fail(s, e_, where); \
    } while (0)

template <typename T>
static cudaError_t dalloc(vmp_stream_t s, T** p, size_t count) {
    cudaError_t e = dev_malloc(p, sizeof(T) * (count < 1 ? 1 : count));
    if (e == cudaSuccess) s->allocs.push_back(*p);
    return e;
}

static vmp_status validate(const vmp_config* c, std::string& why) {
    if (!(c->voxel_size > 0)) { why = "voxel_size must be > 0"; return VMP_ERR_INVALID_ARG; }
    if (!(c->scan_resolution >= 0)) { why = "scan_resolution must be >= 0"; return VMP_ERR_INVALID_ARG; }
    if (c->update_size_thresh < 2 || c->update_size_thresh > kMaxChunks * kChunkPts) {
        why = "update_size_thresh must be in [2, 256]";
        return VMP_ERR_INVALID_ARG;
    }
    if (c->max_point_thresh < 1 || c->max_point_thresh > kMaxChunks * kChunkPts) {
        why = "max_point_thresh must be in [1, 256]";
        return VMP_ERR_INVALID_ARG;
    }
    if (c->max_point_thresh < c->update_size_thresh) {
        why = "max_point_thresh must be >= update_size_thresh";
        return VMP_ERR_INVALID_ARG;
    }
    if (c->map_capacity < 1) { why = "map_capacity must be >= 1"; return VMP_ERR_INVALID_ARG; }
    if (c->ieskf_max_iter < 1 || c->ieskf_max_iter > 64) { why = "ieskf_max_iter must be in [1, 64]"; return VMP_ERR_INVALID_ARG; }
    if (c->max_scan_points < 1 || c->max_scan_points > (1 << 24)) { why = "max_scan_points must be in [1, 2^24]"; return VMP_ERR_INVALID_ARG; }
    if (c->max_imu_per_scan < 1 || c->max_imu_per_scan > 1000) { why = "max_imu_per_scan must be in [1, 1000]"; return VMP_ERR_INVALID_ARG; }
    if (c->imu_init_num < 1) { why = "imu_init_num must be >= 1"; return VMP_ERR_INVALID_ARG; }
    return VMP_OK;
}

extern "C" {

int vmp_abi_version(void) { return VMP_ABI_VERSION; }

void vmp_config_default(vmp_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->opti_max_iter = 5;
    c->na = 0.01; c->ng = 0.01; c->nba = 0.0001; c->nbg = 0.0001;
    c->imu_init_num = 20;
    c->r_il[0] = c->r_il[4] = c->r_il[8] = 1.0;
    c->gravity_align = 1;
    c->estimate_ext = 0;
    c->scan_resolution = 0.1;
    c->voxel_size = 0.5;
    c->update_size_thresh = 10;
    c->max_point_thresh = 100;
    c->plane_thresh = 0.01;
    c->ranging_cov = 0.04;
    c->angle_cov = 0.1;
    c->merge_thresh_for_angle = 0.1;
    c->merge_thresh_for_distance = 0.04;
    c->map_capacity = 100000;
    c->ieskf_max_iter = 5;
    c->ieskf_eps = 0.001;
    c->max_scan_points = 262144;
    c->max_imu_per_scan = 1000;
}

// With a null handle: the reason the calling thread's last vmp_create failed.
const char* vmp_last_error(vmp_stream_t s) { return s ? s->err.c_str() : g_create_error.c_str(); }

vmp_status vmp_destroy(vmp_stream_t s) {
    if (!s) return VMP_ERR_INVALID_ARG;
    if (s->st) cudaStreamSynchronize(s->st);
    for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
    for (void* p : s->allocs) cudaFree(p);
    map_scratch_free(s->ms);
    sort_scratch_free(s->ss);
    if (s->vis_buf) {
        sort_scratch_free(s->vis_ss);
        cudaFree(s->vis_buf);
    }
    scan_scratch_free(s->sc);
    scan_scratch_free(s->qsc);
    cudaFreeHost(s->h_pts);
    cudaFreeHost(s->h_imus);
    cudaFreeHost(s->h_res);
    cudaFreeHost(s->h_cnt);
    cudaFreeHost(s->h_int);
    for (auto& gp : s->graphs) {
        if (gp.g1) cudaGraphExecDestroy(gp.g1);
        if (gp.g2) cudaGraphExecDestroy(gp.g2);
        if (gp.g0) cudaGraphExecDestroy(gp.g0);
    }
    if (s->h_hdr) cudaFreeHost(s->h_hdr);
    if (s->done_ev) cudaEventDestroy(s->done_ev);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    if (s->ev_cov) cudaEventDestroy(s->ev_cov);
    if (s->st_side) cudaStreamDestroy(s->st_side);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
    return VMP_OK;
}

vmp_status vmp_create(const vmp_config* cfg_in, vmp_stream_t* out) {
    if (!out) return VMP_ERR_INVALID_ARG;
    *out = nullptr;
    vmp_config cfg;
    if (cfg_in) cfg = *cfg_in; else vmp_config_default(&cfg);
    if (cfg.max_imu_per_scan <= 0) cfg.max_imu_per_scan = 1000;
    if (cfg.max_scan_points <= 0) cfg.max_scan_points = 262144;
    std::string why;
    vmp_status v = validate(&cfg, why);
    g_create_error = why;
    if (v != VMP_OK) return v;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        g_create_error = "no CUDA device visible (libvmp has no CPU fallback)";
        return VMP_ERR_CUDA;
    }
    vmp_stream_t s = new (std::nothrow) vmp_stream_s();
    if (!s) return VMP_ERR_OUT_OF_MEMORY;
    s->cfg = cfg;
    const long long bytes0 = dev_bytes_counter();
    cudaError_t e;
#define CREATE_TRY(expr)                         \
    do {                                         \
        e = (expr);                              \
        if (e != cudaSuccess) {                  \
            g_create_error = std::string("device allocation / setup failed: ") + cudaGetErrorString(e); \
            vmp_destroy(s);                      \
            return e == cudaErrorMemoryAllocation ? VMP_ERR_OUT_OF_MEMORY : VMP_ERR_CUDA; \
        }                                        \
    } while (0)
    CREATE_TRY(residual_setup());
    CREATE_TRY(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
    CREATE_TRY(cudaEventCreateWithFlags(&s->done_ev, cudaEventBlockingSync | cudaEventDisableTiming));
    CREATE_TRY(cudaStreamCreateWithFlags(&s->st_side, cudaStreamNonBlocking));
    CREATE_TRY(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming));
    CREATE_TRY(cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming));
    CREATE_TRY(cudaEventCreateWithFlags(&s->ev_cov, cudaEventDisableTiming));
    const int max_pts = cfg.max_scan_points;
    const int max_imu = cfg.max_imu_per_scan;
    s->sin_deg = std::sin(cfg.angle_cov * 0.017453293);  // pcl_macros.h DEG2RAD
    // filter
    CREATE_TRY(dalloc(s, &s->f, 1));
    CREATE_TRY(cudaMemset(s->f, 0, sizeof(DFilter)));
    {
        DFilter hf;
        std::memset(&hf, 0, sizeof(hf));
        // kf::State defaults (ieskf.h:35-42)
        hf.x.rot[0] = hf.x.rot[4] = hf.x.rot[8] = 1.0;
        hf.x.rot_ext[0] = hf.x.rot_ext[4] = hf.x.rot_ext[8] = 1.0;
        hf.x.g[2] = -kGravity;
        // LIODataGroup::Q (lio_builder.cpp:9-12, lio_builder.h:52)
        for (int i = 0; i < 12; ++i) hf.Q[i * 13] = 1.0;
        for (int i = 0; i < 3; ++i) {
            hf.Q[i * 13] = cfg.ng;
            hf.Q[(3 + i) * 13] = cfg.na;
            hf.Q[(6 + i) * 13] = cfg.nbg;
            hf.Q[(9 + i) * 13] = cfg.nba;
        }
        CREATE_TRY(cudaMemcpy(s->f, &hf, sizeof(hf), cudaMemcpyHostToDevice));
    }
    // scan buffers
    DScan& sc = s->s;
    sc.max_pts = max_pts;
    sc.max_imu = max_imu;
    sc.res_blocks = 4 * 152;
    CREATE_TRY(dalloc(s, &sc.raw, max_pts));
    CREATE_TRY(dalloc(s, &sc.cloud, max_pts));
    CREATE_TRY(dalloc(s, &sc.raw_int, max_pts));
    CREATE_TRY(dalloc(s, &sc.cloud_int, max_pts));
    CREATE_TRY(dalloc(s, &sc.d_n_in, 4));
    CREATE_TRY(dalloc(s, &sc.sort_k, max_pts + 16));
    CREATE_TRY(dalloc(s, &sc.sort_v, max_pts + 16));
    CREATE_TRY(dalloc(s, &sc.flags, max_pts + 16));
    CREATE_TRY(dalloc(s, &sc.scan_out, max_pts + 16));
    CREATE_TRY(dalloc(s, &sc.hdr, 1));
    sc.d_n_raw = &sc.hdr->n_raw;
    CREATE_TRY(dalloc(s, &sc.down, max_pts));
    CREATE_TRY(dalloc(s, &sc.d_n_down, 4));
    CREATE_TRY(dalloc(s, &sc.minmax, 8));
    CREATE_TRY(dalloc(s, &sc.blk_minmax, kMinMaxBlocks * 6 + 8));
    CREATE_TRY(dalloc(s, &sc.ds_params, 32));
    CREATE_TRY(dalloc(s, &sc.run_start, max_pts + 16));
    CREATE_TRY(dalloc(s, &sc.pl, (size_t)max_pts * 3));
    CREATE_TRY(dalloc(s, &sc.covl, (size_t)max_pts * 9));
    CREATE_TRY(dalloc(s, &sc.rvalid, max_pts));
    CREATE_TRY(cudaMemset(sc.rvalid, 0, max_pts));
    CREATE_TRY(dalloc(s, &sc.rnorm, (size_t)max_pts * 3));
    CREATE_TRY(cudaMemset(sc.rnorm, 0, sizeof(double) * (size_t)max_pts * 3));
    CREATE_TRY(dalloc(s, &sc.rres, max_pts));
    CREATE_TRY(cudaMemset(sc.rres, 0, sizeof(double) * (size_t)max_pts));
    CREATE_TRY(dalloc(s, &sc.bpts, (size_t)max_pts * 3));
    CREATE_TRY(dalloc(s, &sc.bcov, (size_t)max_pts * 9));
    CREATE_TRY(dalloc(s, &sc.d_n_batch, 4));
    CREATE_TRY(dalloc(s, &sc.imus, max_imu + 8));
    CREATE_TRY(dalloc(s, &sc.poses, max_imu + 8));
    CREATE_TRY(dalloc(s, &sc.steps, max_imu + 8));
    CREATE_TRY(dalloc(s, &sc.partials, (size_t)sc.res_blocks * 160));
    CREATE_TRY(dalloc(s, &sc.done_ctr, 4));
    CREATE_TRY(cudaMemset(sc.done_ctr, 0, sizeof(unsigned int) * 4));
    CREATE_TRY(sort_scratch_alloc(s->ss, max_pts));
    CREATE_TRY(scan_scratch_alloc(s->sc, max_pts));
    // map
    DMap& m = s->m;
    const long long cap = cfg.map_capacity;
    const long long pool = cap + max_pts + 16;
    if (pool > 0x7FFFFFF0LL) { vmp_destroy(s); return VMP_ERR_INVALID_ARG; }
    m.rec_pool = (int)pool;
    const size_t tsize = next_pow2((size_t)(2 * pool) < 1024 ? 1024 : (size_t)(2 * pool));
    m.table_mask = tsize - 1;
    long long chunks = cfg.reserved[0] > 0 ? (long long)cfg.reserved[0] : 2 * pool + 1024;
    if (chunks > 0x7FFFFFF0LL) chunks = 0x7FFFFFF0LL;
    m.chunk_pool = (int)chunks;
    m.q_cap = (uint64_t)(2 * pool + 2 * (long long)max_pts);
    m.voxel_size = cfg.voxel_size;
    {
        int e = 0;
        const double mant = std::frexp(cfg.voxel_size, &e);
        m.voxel_inv = mant == 0.5 ? std::ldexp(1.0, 1 - e) : 0.0;  // 2^(e-1) -> 2^(1-e)
    }
    m.update_thresh = cfg.update_size_thresh;
    m.max_thresh = cfg.max_point_thresh;
    m.plane_thresh = cfg.plane_thresh;
    m.merge_angle = cfg.merge_thresh_for_angle;
    m.merge_dist = cfg.merge_thresh_for_distance;
    m.capacity = cap;
    CREATE_TRY(dalloc(s, &m.keys, tsize));
    CREATE_TRY(dalloc(s, &m.vals, tsize));
    CREATE_TRY(dalloc(s, &m.hot, pool));
    CREATE_TRY(dalloc(s, &m.cold, pool));
    CREATE_TRY(dalloc(s, &m.rec_free, pool));
    CREATE_TRY(dalloc(s, &m.slab, (size_t)chunks * kChunkPts * kSlabStride));
    CREATE_TRY(dalloc(s, &m.chunk_free, chunks));
    CREATE_TRY(dalloc(s, &m.chunk_freed, chunks));
    CREATE_TRY(dalloc(s, &m.q_rec, m.q_cap));
    CREATE_TRY(dalloc(s, &m.q_stamp, m.q_cap));
    CREATE_TRY(dalloc(s, &s->cnt, 1));
    m.cnt = s->cnt;
    CREATE_TRY(cudaMemset(s->cnt, 0, sizeof(Counters)));
    CREATE_TRY(map_scratch_alloc(s->ms, max_pts, m.rec_pool, cfg.reserved[1]));
    CREATE_TRY(map_recip_table_init());
    // queue compaction scratch
    const int qmax = (int)std::min<uint64_t>(m.q_cap, 0x7FFFFFF0ull);
    CREATE_TRY(dalloc(s, &s->qc_flag, qmax));
    CREATE_TRY(dalloc(s, &s->qc_rank, qmax));
    CREATE_TRY(dalloc(s, &s->qc_rec, qmax));
    CREATE_TRY(dalloc(s, &s->qc_stamp, qmax));
    CREATE_TRY(dalloc(s, &s->qc_ints, 8));
    CREATE_TRY(scan_scratch_alloc(s->qsc, qmax));
    // pinned host staging
    CREATE_TRY(cudaMallocHost(&s->h_pts, sizeof(vmp_point) * (size_t)max_pts));
    CREATE_TRY(cudaMallocHost(&s->h_imus, sizeof(vmp_imu) * (size_t)(max_imu + 8)));
    CREATE_TRY(cudaMallocHost(&s->h_res, sizeof(DResult)));
    CREATE_TRY(cudaMallocHost(&s->h_cnt, sizeof(Counters)));
    CREATE_TRY(cudaMallocHost(&s->h_int, sizeof(int) * 16));
    CREATE_TRY(cudaMallocHost(&s->h_hdr, sizeof(DScanHdr)));
    CREATE_TRY(dalloc(s, &s->d_res, 1));
    launch_map_reset(m, s->st);
    CREATE_TRY(cudaGetLastError());
    CREATE_TRY(cudaStreamSynchronize(s->st));
#undef CREATE_TRY
    s->dev_bytes = dev_bytes_counter() - bytes0;
    *out = s;
    return VMP_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ internals
static bool is_pinned_or_device(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static vmp_status read_counters(vmp_stream_t s) {
    VMP_TRY(cudaMemcpyAsync(s->h_cnt, s->cnt, sizeof(Counters), cudaMemcpyDeviceToHost, s->st), "read counters");
    s->io_d2h += (long long)sizeof(Counters);
    VMP_TRY(cudaStreamSynchronize(s->st), "sync");
    s->h_size = s->h_cnt->size;
    s->h_qlen = s->h_cnt->q_tail - s->h_cnt->q_head;
    s->h_tomb = s->h_cnt->n_tomb;
    return VMP_OK;
}

static void map_maintenance(vmp_stream_t s) {
    DMap& m = s->m;
    if ((size_t)s->h_tomb > (size_t)(m.table_mask + 1) / 8) {
        launch_rehash(m, s->st);
        s->h_tomb = 0;
    }
    if (s->h_qlen + 2ull * (unsigned long long)s->cfg.max_scan_points > m.q_cap) {
        // queue length is read on the device
        int* d_len = s->qc_ints;
        int* d_live = s->qc_ints + 1;
        VMP_NOTE_LAUNCH(); k_set_int<<<1, 32, 0, s->st>>>(d_len, (int)s->h_qlen);
        launch_queue_compact(m, s->qc_flag, s->qc_rank, s->qc_rec, s->qc_stamp, d_len, d_live,
                             (int)std::min<uint64_t>(m.q_cap, 0x7FFFFFF0ull), s->qsc, s->st);
        s->h_qlen = 0;  // refreshed at the next counter read
    }
}

// Applies batch points [0, n) of (bpts, bcov) where n is on the device
// (d_n_src) or on the host (n_host >= 0).  n_upper bounds n.
static vmp_status map_apply(vmp_stream_t s, const double* bpts, const double* bcov, const int* d_n_src, int n_host,
                            int n_upper, bool build) {
    DMap& m = s->m;
    MapScratch& ms = s->ms;
    map_maintenance(s);
    const bool evict_possible = s->h_size + (long long)n_upper > m.capacity;
    VMP_NOTE_LAUNCH();
    if (d_n_src) k_copy_int<<<1, 32, 0, s->st>>>(ms.d_n, d_n_src);
    else k_set_int<<<1, 32, 0, s->st>>>(ms.d_n, n_host);
    const int n_max = n_upper;
    if (!evict_possible) {
        s->pbeg();
        launch_map_phase_a(m, ms, bpts, n_max, s->st);
        launch_map_segments(m, ms, n_max, s->st);
        s->pend(VMP_PROF_MAP_GROUP, s->cur_batch_kind);
        s->pbeg();
        launch_map_state(m, ms, bpts, bcov, n_max, build, s->st);
        s->pend(VMP_PROF_MAP_STATE, s->cur_batch_kind);
        s->pbeg();
        launch_map_finish(m, ms, n_max, build, s->st);
        s->pend(VMP_PROF_MAP_FINISH, s->cur_batch_kind);
        VMP_TRY(cudaGetLastError(), "map update launch");
        s->h_size += n_upper;  // upper bound until the next counter read
        return VMP_OK;
    }
    // eviction possible: the walk runs on the device; its counters (a split?)
    // and the batch size come back in one read, the only host round trip of
    // a batch that does not split (the kernels take n from the device and
    // n_upper bounds their grids, as above)
    launch_map_phase_a(m, ms, bpts, n_upper, s->st);
    launch_map_segments(m, ms, n_upper, s->st);
    launch_map_walk(m, ms, s->st);
    VMP_TRY(cudaMemcpyAsync(s->h_int, ms.d_n, sizeof(int), cudaMemcpyDeviceToHost, s->st), "read n");
    s->io_d2h += (long long)sizeof(int);
    vmp_status st = read_counters(s);
    if (st != VMP_OK) return st;
    const int n = s->h_int[0];
    if (n <= 0) return VMP_OK;
    const int split = s->h_cnt->split_at;
    if (split < 0) {
        launch_map_phase_b(m, ms, bpts, bcov, n_upper, build, s->st);
        VMP_TRY(cudaGetLastError(), "map update launch");
        // at most the capacity once the walk evicted for it; every caller
        // reads the counters with its result
        s->h_size = m.capacity;
        return VMP_OK;
    }
    ++s->eviction_splits;
    launch_map_rollback(m, ms, n_upper, s->st);
    st = read_counters(s);
    if (st != VMP_OK) return st;
    if (split <= 0 || split >= n) return fail(s, VMP_ERR_STATE, "eviction split outside the batch");
    st = map_apply(s, bpts, bcov, nullptr, split, split, build);
    if (st != VMP_OK) return st;
    st = read_counters(s);
    if (st != VMP_OK) return st;
    return map_apply(s, bpts + (size_t)split * 3, bcov + (size_t)split * 9, nullptr, n - split, n - split, build);
}

static vmp_status upload_scan(vmp_stream_t s, const vmp_point* pts, int n, bool device_ptr) {
    if (pts == reinterpret_cast<const vmp_point*>(s->s.raw)) return VMP_OK;  // decoded on the device
    VMP_TRY(cudaMemsetAsync(s->s.raw_int, 0, sizeof(float) * (size_t)n, s->st), "intensity");
    if (!device_ptr) s->io_h2d += (long long)sizeof(vmp_point) * n;
    if (device_ptr) {
        VMP_TRY(cudaMemcpyAsync(s->s.raw, pts, sizeof(vmp_point) * (size_t)n, cudaMemcpyDeviceToDevice, s->st), "scan copy");
    } else if (is_pinned_or_device(pts)) {
        VMP_TRY(cudaMemcpyAsync(s->s.raw, pts, sizeof(vmp_point) * (size_t)n, cudaMemcpyDefault, s->st), "scan upload");
    } else {
        VMP_TRY(cudaStreamSynchronize(s->st), "sync");
        std::memcpy(s->h_pts, pts, sizeof(vmp_point) * (size_t)n);
        VMP_TRY(cudaMemcpyAsync(s->s.raw, s->h_pts, sizeof(vmp_point) * (size_t)n, cudaMemcpyHostToDevice, s->st), "scan upload");
    }
    return VMP_OK;
}

// The scan's scalars (point count, IMU count, package times) in one copy.
static vmp_status upload_header(vmp_stream_t s, int n, int n_imu, double t_start, double t_end) {
    s->h_hdr->n_raw = n;
    s->h_hdr->n_imu = n_imu;
    s->h_hdr->t_start = t_start;
    s->h_hdr->t_end = t_end;
    s->h_hdr->time_unsorted = 0;
    s->h_hdr->pad = 0;
    VMP_TRY(cudaMemcpyAsync(s->s.hdr, s->h_hdr, sizeof(DScanHdr), cudaMemcpyHostToDevice, s->st), "header");
    s->io_h2d += (long long)sizeof(DScanHdr);
    return VMP_OK;
}

// Grid sizes of a scan come from its size class (steps of a quarter octave,
// at least 1024 points, at most max_scan_points): a captured graph then
// serves every scan of the class, and graph and direct launches use the same
// grids (the reduction orders follow the grids).
static int size_class(int n, int max_pts) {
    const unsigned v = (unsigned)(n < 1024 ? 1024 : n);
    const int e = 31 - __builtin_clz(v);
    const unsigned step = (1u << e) >> 2;
    const unsigned c = (v + step - 1) / step * step;
    return (int)(c < (unsigned)max_pts ? c : (unsigned)max_pts);
}

static vmp_status upload_imus(vmp_stream_t s, const vmp_imu* imus, int n, bool device_ptr) {
    if (n <= 0) return VMP_OK;
    if (!device_ptr) s->io_h2d += (long long)sizeof(vmp_imu) * n;
    if (device_ptr) {
        VMP_TRY(cudaMemcpyAsync(s->s.imus, imus, sizeof(vmp_imu) * (size_t)n, cudaMemcpyDeviceToDevice, s->st), "imu copy");
    } else {
        VMP_TRY(cudaStreamSynchronize(s->st), "sync");
        std::memcpy(s->h_imus, imus, sizeof(vmp_imu) * (size_t)n);
        VMP_TRY(cudaMemcpyAsync(s->s.imus, s->h_imus, sizeof(vmp_imu) * (size_t)n, cudaMemcpyHostToDevice, s->st), "imu upload");
    }
    return VMP_OK;
}

// The result gathered on the device and copied to the pinned host mirror.
static vmp_status enqueue_result(vmp_stream_t s) {
    VMP_NOTE_LAUNCH(); k_gather_result<<<1, 256, 0, s->st>>>(s->f, s->s.d_n_down, s->cnt, s->d_res);
    VMP_TRY(cudaGetLastError(), "result launch");
    VMP_TRY(cudaMemcpyAsync(s->h_res, s->d_res, sizeof(DResult), cudaMemcpyDeviceToHost, s->st), "result copy");
    return VMP_OK;
}

static vmp_status finish_result_host(vmp_stream_t s, int n_raw, vmp_result* out);

static vmp_status finish_result(vmp_stream_t s, int n_raw, vmp_result* out) {
    s->pbeg();
    vmp_status v = enqueue_result(s);
    if (v != VMP_OK) return v;
    s->io_d2h += (long long)sizeof(DResult);
    s->pend(VMP_PROF_RESULT, -1);
    return finish_result_host(s, n_raw, out);
}

// Waits for the stream, then reads the result and the device error word.
static vmp_status finish_result_host(vmp_stream_t s, int n_raw, vmp_result* out) {
    if (s->blocking_wait && s->done_ev) {
        VMP_TRY(cudaEventRecord(s->done_ev, s->st), "scan");
        VMP_TRY(cudaEventSynchronize(s->done_ev), "scan");
    } else {
        VMP_TRY(cudaStreamSynchronize(s->st), "scan");
    }
    const DResult& r = *s->h_res;
    s->pflush(r.iters, n_raw, r.n_down, r.n_down);
    s->h_size = r.cnt.size;
    s->h_qlen = r.cnt.q_tail - r.cnt.q_head;
    s->h_tomb = r.cnt.n_tomb;
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->lio_status = s->lio_status;
        out->iters = r.iters;
        out->effect_num = r.effect_num;
        out->n_raw = n_raw;
        out->n_down = r.n_down;
        out->flags = r.no_effect ? 1 : 0;
        out->map_size = r.cnt.size;
        out->evicted = r.cnt.evicted_total - s->last_evicted_total;
        std::memcpy(&out->x, &r.x, sizeof(vmp_state));
        std::memcpy(out->P, r.P, sizeof(r.P));
    }
    s->last_evicted_total = r.cnt.evicted_total;
    if (r.cnt.error) {
        unsigned int e = r.cnt.error;
        VMP_NOTE_LAUNCH(); k_clear_error<<<1, 32, 0, s->st>>>(s->cnt);
        cudaStreamSynchronize(s->st);
        if (e & E_KEY_RANGE) return fail(s, VMP_ERR_KEY_RANGE, "a voxel index left the packed range [-2^20, 2^20)");
        if (e & E_HASH_FULL) return fail(s, VMP_ERR_HASH_FULL, "voxel hash table full");
        if (e & E_MERGE_WAIT)
            return fail(s, VMP_ERR_TIMEOUT, "merge fixed point: a grid barrier wait ran out (map state unreliable)");
        if (e & (E_RECORDS | E_CHUNKS | E_CAPACITY))
            return fail(s, VMP_ERR_CAPACITY, "voxel record / slab pool exhausted (error bits " + std::to_string(e) + ")");
    }
    return VMP_OK;
}

// The scan from the time sort to the map batch (LIOBuilder::process before
// VoxelMap::update, lio_builder.cpp:175-246); nb sizes the grids.  With
// map_init the undistorted cloud goes to the map batch (VoxelMap::build).
static void enqueue_scan_front(vmp_stream_t s, int nb, bool map_init) {
    const vmp_config& cfg = s->cfg;
    cudaStream_t st = s->st;
    if (s->prof_on) {  // one phase after the other, each timed on the stream
        s->pbeg();
        launch_time_sort(s->s, nb, s->ss, st);
        s->pend(VMP_PROF_TIME_SORT, 0);
        s->pbeg();
        launch_predict_chain2(s->f, s->s, st);
        s->pend(VMP_PROF_PREDICT, -1);
    } else {  // the predict chain beside the time sort; its covariance chain
              // beside everything up to the first reader of P (ev_cov)
        cudaEventRecord(s->ev_fork, st);
        cudaStreamWaitEvent(s->st_side, s->ev_fork, 0);
        launch_predict_state(s->f, s->s, s->st_side);
        cudaEventRecord(s->ev_join, s->st_side);
        launch_predict_cov(s->f, s->s, s->st_side);
        cudaEventRecord(s->ev_cov, s->st_side);
        launch_time_sort(s->s, nb, s->ss, st);
        cudaStreamWaitEvent(st, s->ev_join, 0);
    }
    s->pbeg();
    launch_undistort(s->f, s->s, nb, st);
    s->pend(VMP_PROF_UNDISTORT, 0);
    if (map_init) {
        if (!s->prof_on) cudaStreamWaitEvent(st, s->ev_cov, 0);
        s->pbeg();
        launch_map_batch(s->f, s->s, nb, true, cfg.ranging_cov, s->sin_deg, st);
        s->pend(VMP_PROF_MAP_BATCH, 0);
        return;
    }
    s->pbeg();
    if (cfg.scan_resolution > 0.0) launch_downsample(s->s, nb, cfg.scan_resolution, s->ss, s->sc, st);
    else launch_copy_down(s->s, nb, st);
    s->pend(VMP_PROF_DOWNSAMPLE, 0);
    s->pbeg();
    launch_body_cov(s->s, nb, cfg.ranging_cov, s->sin_deg, st);
    s->pend(VMP_PROF_BODY_COV, 1);
    if (!s->prof_on) cudaStreamWaitEvent(st, s->ev_cov, 0);
    s->pbeg();
    launch_update_begin(s->f, st);
    s->pend(VMP_PROF_UPDATE_OTHER, -1);
    for (int it = 0; it < cfg.ieskf_max_iter; ++it) {
        if (s->prof_on) {  // one phase after the other: the boxminus is timed with the step
            s->pbeg();
            launch_residual_points(s->f, s->s, s->m, nb, cfg.estimate_ext, st, 1);
            s->pend(VMP_PROF_RESIDUAL, 1);
            s->pbeg();
            launch_iekf_boxminus(s->f, st);
            launch_residual_step(s->f, s->s, nb, cfg.estimate_ext, cfg.ieskf_eps, st, 1);
            s->pend(VMP_PROF_RESIDUAL_STEP, -1);
        } else {  // the boxminus beside the point kernel, joined before the fold
            cudaEventRecord(s->ev_fork, st);
            cudaStreamWaitEvent(s->st_side, s->ev_fork, 0);
            launch_iekf_boxminus(s->f, s->st_side);
            cudaEventRecord(s->ev_join, s->st_side);
            launch_residual_points(s->f, s->s, s->m, nb, cfg.estimate_ext, st, 1);
            cudaStreamWaitEvent(st, s->ev_join, 0);
            launch_residual_step(s->f, s->s, nb, cfg.estimate_ext, cfg.ieskf_eps, st, 1);
        }
    }
    s->pbeg();
    launch_update_end(s->f, cfg.estimate_ext, st);
    s->pend(VMP_PROF_UPDATE_OTHER, -1);
    s->pbeg();
    launch_map_batch(s->f, s->s, nb, false, cfg.ranging_cov, s->sin_deg, st);
    s->pend(VMP_PROF_MAP_BATCH, 1);
}

// The graphs of size class nb (an empty entry on first use).
// Graphs captured before a launch shape changed (launch_shape_epoch) are
// dropped and captured again (an exec still running is freed when it ends).
static vmp_stream_s::ScanGraphs* graphs_for(vmp_stream_t s, int nb) {
    const long long ep = launch_shape_epoch();
    for (auto& g : s->graphs)
        if (g.nb == nb) {
            if (g.epoch != ep) {
                if (g.g1) cudaGraphExecDestroy(g.g1);
                if (g.g2) cudaGraphExecDestroy(g.g2);
                if (g.g0) cudaGraphExecDestroy(g.g0);
                g = vmp_stream_s::ScanGraphs{nb, nullptr, nullptr, nullptr, 0, 0, 0, ep};
            }
            return &g;
        }
    s->graphs.push_back(vmp_stream_s::ScanGraphs{nb, nullptr, nullptr, nullptr, 0, 0, 0, ep});
    return &s->graphs.back();
}

// The scan front (time sort to map batch) of size class nb as one graph
// launch; captured on first use.  The same kernels and grids as the direct
// launches.
static vmp_status launch_front_graph(vmp_stream_t s, int nb) {
    vmp_stream_s::ScanGraphs* gp = graphs_for(s, nb);
    if (!gp->g0) {
        long long launches = 0;
        set_capture_launch_counter(&launches);
        cudaError_t e = cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            enqueue_scan_front(s, nb, false);
            cudaGraph_t g = nullptr;
            e = cudaStreamEndCapture(s->st, &g);
            if (e == cudaSuccess) {
                e = cudaGraphInstantiate(&gp->g0, g, 0);
                cudaGraphDestroy(g);
                gp->k0 = launches;
            }
        }
        set_capture_launch_counter(nullptr);
        if (e != cudaSuccess) return cuda_fail(s, e, "scan front graph capture");
    }
    VMP_TRY(cudaGraphLaunch(gp->g0, s->st), "scan front graph");
    g_launch_count.fetch_add(gp->k0, std::memory_order_relaxed);
    return VMP_OK;
}

// Captures the two graphs of a steady-state scan of size class nb.
static vmp_status capture_scan_graphs(vmp_stream_t s, int nb, vmp_stream_s::ScanGraphs& gp) {
    cudaStream_t st = s->st;
    MapScratch& ms = s->ms;
    gp.nb = nb;
    for (int part = 0; part < 2; ++part) {
        long long launches = 0;
        set_capture_launch_counter(&launches);
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            if (part == 0) {
                enqueue_scan_front(s, nb, false);
                VMP_NOTE_LAUNCH(); k_copy_int<<<1, 32, 0, st>>>(ms.d_n, s->s.d_n_batch);
                launch_map_phase_a(s->m, ms, s->s.bpts, nb, st);
                launch_map_segments(s->m, ms, nb, st);
                launch_map_state(s->m, ms, s->s.bpts, s->s.bcov, nb, false, st);
                launch_map_finish_pre(s->m, ms, nb, false, st);
            } else {
                launch_map_finish_post(s->m, ms, nb, st);
                enqueue_result(s);
            }
            cudaGraph_t g = nullptr;
            e = cudaStreamEndCapture(st, &g);
            if (e == cudaSuccess) {
                cudaGraphExec_t x = nullptr;
                e = cudaGraphInstantiate(&x, g, 0);
                cudaGraphDestroy(g);
                if (part == 0) { gp.g1 = x; gp.k1 = launches; }
                else { gp.g2 = x; gp.k2 = launches; }
            }
        }
        set_capture_launch_counter(nullptr);
        if (e != cudaSuccess) return cuda_fail(s, e, "scan graph capture");
    }
    return VMP_OK;
}

// The steady-state scan (LIO_MAPPING, no eviction possible, profiler off)
// as two graph launches around the merge resolution: ~90 kernel launches
// per scan become 3.
static vmp_status process_graph(vmp_stream_t s, int n, int nb, vmp_result* out) {
    cudaStream_t st = s->st;
    map_maintenance(s);  // host-decided rehash / queue compaction, before the graph
    vmp_stream_s::ScanGraphs* gp = graphs_for(s, nb);
    if (!gp->g1) {
        vmp_status v = capture_scan_graphs(s, nb, *gp);
        if (v != VMP_OK) return v;
    }
    VMP_TRY(cudaGraphLaunch(gp->g1, st), "scan graph");
    g_launch_count.fetch_add(gp->k1, std::memory_order_relaxed);
    s->cur_batch_kind = 1;
    VMP_TRY(run_merge_events(s->m, s->ms, s->ms.merge, nb, s->ms.merge_mode, &s->ms.merge_rounds, st), "merges");
    VMP_TRY(cudaGraphLaunch(gp->g2, st), "scan graph");
    g_launch_count.fetch_add(gp->k2, std::memory_order_relaxed);
    s->h_size += n;  // upper bound until the result's counters arrive
    s->io_d2h += (long long)sizeof(DResult);
    return finish_result_host(s, n, out);
}

static vmp_status process_impl(vmp_stream_t s, const vmp_point* pts, int n, double t_start, double t_end,
                               const vmp_imu* imus, int n_imu, bool device_ptrs, vmp_result* out) {
    if (!s) return VMP_ERR_INVALID_ARG;
    if (s->broken) return fail(s, VMP_ERR_CUDA, "stream unusable after a CUDA error: " + s->err);
    if (pts != reinterpret_cast<const vmp_point*>(s->s.raw)) s->decoded_n = -1;  // its buffer is overwritten
    if (!pts || n <= 0) return fail(s, VMP_ERR_INVALID_ARG, "empty scan");
    if (n > s->cfg.max_scan_points) return fail(s, VMP_ERR_CAPACITY, "scan larger than max_scan_points");
    if (!imus || n_imu <= 0) return fail(s, VMP_ERR_INVALID_ARG, "package without IMU samples");
    if (n_imu > s->cfg.max_imu_per_scan) return fail(s, VMP_ERR_CAPACITY, "more IMU samples than max_imu_per_scan");
    const vmp_config& cfg = s->cfg;
    cudaStream_t st = s->st;
    if (s->lio_status == VMP_IMU_INIT) {
        // LIOBuilder::initializeImu: accumulate on the host, initialise on the device
        size_t old = s->imu_cache.size();
        s->imu_cache.resize(old + n_imu);
        if (device_ptrs) {
            VMP_TRY(cudaMemcpyAsync(s->imu_cache.data() + old, imus, sizeof(vmp_imu) * n_imu, cudaMemcpyDeviceToHost, st),
                    "imu read");
            VMP_TRY(cudaStreamSynchronize(st), "imu read");
        } else {
            std::memcpy(s->imu_cache.data() + old, imus, sizeof(vmp_imu) * n_imu);
        }
        if ((int)s->imu_cache.size() >= cfg.imu_init_num) {
            // all samples go to the device in one copy through the package
            // IMU buffers (max_imu_per_scan + 8 samples); a longer
            // initialisation window takes a stream-ordered temporary.  No
            // cudaMalloc / cudaFree: they would synchronise the whole device
            // and stall the other streams of a server.
            const size_t cnt = s->imu_cache.size();
            const size_t cap = (size_t)cfg.max_imu_per_scan + 8;
            vmp_imu* d_all = s->s.imus;
            vmp_imu* d_tmp = nullptr;
            VMP_TRY(cudaStreamSynchronize(st), "sync");
            if (cnt > cap) {
                VMP_TRY(cudaMallocAsync(&d_tmp, sizeof(vmp_imu) * cnt, st), "imu init alloc");
                d_all = d_tmp;
                VMP_TRY(cudaMemcpyAsync(d_all, s->imu_cache.data(), sizeof(vmp_imu) * cnt, cudaMemcpyHostToDevice, st),
                        "imu init upload");
                VMP_TRY(cudaStreamSynchronize(st), "sync");
            } else {
                std::memcpy(s->h_imus, s->imu_cache.data(), sizeof(vmp_imu) * cnt);
                VMP_TRY(cudaMemcpyAsync(d_all, s->h_imus, sizeof(vmp_imu) * cnt, cudaMemcpyHostToDevice, st),
                        "imu init upload");
            }
            launch_imu_init(s->f, d_all, (int)cnt, cfg, t_end, st);
            if (d_tmp) cudaFreeAsync(d_tmp, st);
            cudaError_t e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return cuda_fail(s, e, "imu init");
            s->imu_cache.clear();
            s->lio_status = VMP_MAP_INIT;
        }
        VMP_NOTE_LAUNCH(); k_set_int<<<1, 32, 0, st>>>(s->s.d_n_down, 0);
        s->cloud_n = 0;
        return finish_result(s, n, out);
    }
    s->cloud_n = n;
    const int nb = size_class(n, cfg.max_scan_points);
    s->pbeg();
    vmp_status v = upload_scan(s, pts, n, device_ptrs);
    if (v != VMP_OK) return v;
    v = upload_imus(s, imus, n_imu, device_ptrs);
    if (v != VMP_OK) return v;
    v = upload_header(s, n, n_imu, t_start, t_end);
    if (v != VMP_OK) return v;
    s->pend(VMP_PROF_UPLOAD, 0);
    if (s->lio_status == VMP_LIO_MAPPING && s->use_graphs && !s->prof_on && s->h_size + (long long)n <= s->m.capacity)
        return process_graph(s, n, nb, out);
    if (s->lio_status == VMP_MAP_INIT) {
        enqueue_scan_front(s, nb, true);
        VMP_NOTE_LAUNCH(); k_set_int<<<1, 32, 0, st>>>(s->s.d_n_down, 0);
        VMP_TRY(cudaGetLastError(), "map init launch");
        s->cur_batch_kind = 0;
        v = map_apply(s, s->s.bpts, s->s.bcov, s->s.d_n_batch, -1, nb, true);
        if (v != VMP_OK) return v;
        s->lio_status = VMP_LIO_MAPPING;
        return finish_result(s, n, out);
    }
    if (s->use_graphs && !s->prof_on) {  // the map update below may evict: only the front as a graph
        v = launch_front_graph(s, nb);
        if (v != VMP_OK) return v;
    } else {
        enqueue_scan_front(s, nb, false);
    }
    VMP_TRY(cudaGetLastError(), "scan launch");
    s->cur_batch_kind = 1;
    v = map_apply(s, s->s.bpts, s->s.bcov, s->s.d_n_batch, -1, nb, false);
    if (v != VMP_OK) return v;
    return finish_result(s, n, out);
}

extern "C" {

vmp_status vmp_process(vmp_stream_t s, const vmp_scan* scan, const vmp_imu* imus, int n_imu, vmp_result* out) {
    if (!s || !scan) return VMP_ERR_INVALID_ARG;
    return process_impl(s, scan->points, scan->n, scan->t_start, scan->t_end, imus, n_imu, false, out);
}

vmp_status vmp_process_device(vmp_stream_t s, const vmp_point* d_points, int n, double t_start, double t_end,
                              const vmp_imu* d_imus, int n_imu, vmp_result* out) {
    return process_impl(s, d_points, n, t_start, t_end, d_imus, n_imu, true, out);
}

vmp_status vmp_livox_decode(vmp_stream_t s, const vmp_livox_point* pts, int n, int filter_num, double range_min,
                            double range_max, vmp_point* out, float* intensity, int* n_out, float* last_t_ms) {
    if (!s || !n_out || n < 0 || (n > 0 && !pts)) return VMP_ERR_INVALID_ARG;
    if (s->broken) return fail(s, VMP_ERR_CUDA, "stream unusable after a CUDA error: " + s->err);
    if (filter_num < 1) return fail(s, VMP_ERR_INVALID_ARG, "filter_num must be >= 1");
    if (n > s->cfg.max_scan_points) return fail(s, VMP_ERR_CAPACITY, "more points than max_scan_points");
    *n_out = 0;
    if (last_t_ms) *last_t_ms = 0.0f;
    s->decoded_n = -1;
    if (n == 0) {
        s->decoded_n = 0;
        return VMP_OK;
    }
    // the raw Livox points are staged in the map-batch buffer (24 B per
    // point, free until the scan's map batch)
    vmp_livox_point* d_in = reinterpret_cast<vmp_livox_point*>(s->s.bpts);
    VMP_TRY(cudaMemcpyAsync(d_in, pts, sizeof(vmp_livox_point) * (size_t)n, cudaMemcpyDefault, s->st), "livox upload");
    s->io_h2d += (long long)sizeof(vmp_livox_point) * n;
    launch_livox_decode(s->s, d_in, n, filter_num, range_min, range_max, s->sc, s->st);
    VMP_TRY(cudaGetLastError(), "livox decode");
    // the count and the last kept point's time (written by the scatter) in one read
    VMP_TRY(cudaMemcpyAsync(s->h_int, s->s.d_n_raw, sizeof(int), cudaMemcpyDeviceToHost, s->st), "count");
    VMP_TRY(cudaMemcpyAsync(s->h_int + 1, s->s.d_n_in + 3, sizeof(int), cudaMemcpyDeviceToHost, s->st), "last time");
    VMP_TRY(cudaStreamSynchronize(s->st), "livox decode");
    const int m = s->h_int[0];
    *n_out = m;
    s->decoded_n = m;
    if (m > 0) {
        if (last_t_ms) std::memcpy(last_t_ms, s->h_int + 1, sizeof(float));
        if (!out && !intensity) return VMP_OK;
        if (out)
            VMP_TRY(cudaMemcpyAsync(out, s->s.raw, sizeof(vmp_point) * (size_t)m, cudaMemcpyDefault, s->st), "cloud");
        if (intensity)
            VMP_TRY(cudaMemcpyAsync(intensity, s->s.raw_int, sizeof(float) * (size_t)m, cudaMemcpyDefault, s->st),
                    "intensity");
        VMP_TRY(cudaStreamSynchronize(s->st), "livox decode");
    }
    return VMP_OK;
}

vmp_status vmp_process_decoded(vmp_stream_t s, double t_start, double t_end, const vmp_imu* imus, int n_imu,
                               vmp_result* out) {
    if (!s) return VMP_ERR_INVALID_ARG;
    if (s->decoded_n < 0) return fail(s, VMP_ERR_STATE, "no decoded cloud pending (call vmp_livox_decode first)");
    const int n = s->decoded_n;
    s->decoded_n = -1;
    return process_impl(s, reinterpret_cast<const vmp_point*>(s->s.raw), n, t_start, t_end, imus, n_imu, false, out);
}

vmp_status vmp_output_cloud_device(vmp_stream_t s, int frame, vmp_point* d_out, float* d_intensity, int max,
                                   int* n_out) {
    if (!s || !n_out || (frame != 0 && frame != 1) || max < 0 || (max > 0 && !d_out)) return VMP_ERR_INVALID_ARG;
    if (s->broken) return fail(s, VMP_ERR_CUDA, "stream unusable after a CUDA error: " + s->err);
    const int n = s->cloud_n < max ? s->cloud_n : max;
    *n_out = n;
    launch_output_cloud(s->f, s->s, n, frame, reinterpret_cast<float4*>(d_out), d_intensity, s->st);
    VMP_TRY(cudaGetLastError(), "output cloud");
    return VMP_OK;
}

vmp_status vmp_output_cloud(vmp_stream_t s, int frame, vmp_point* out, float* intensity, int max, int* n_out) {
    if (!s || !n_out || (frame != 0 && frame != 1) || max < 0 || (max > 0 && !out)) return VMP_ERR_INVALID_ARG;
    if (s->broken) return fail(s, VMP_ERR_CUDA, "stream unusable after a CUDA error: " + s->err);
    const int n = s->cloud_n;
    *n_out = n;
    const int m = n < max ? n : max;
    if (m <= 0) return VMP_OK;
    // staged in the map-batch buffer (24 B per point: 16 B point + 4 B intensity)
    float4* d_pts = reinterpret_cast<float4*>(s->s.bpts);
    float* d_int = reinterpret_cast<float*>(d_pts + s->s.max_pts);
    launch_output_cloud(s->f, s->s, m, frame, d_pts, d_int, s->st);
    VMP_TRY(cudaGetLastError(), "output cloud");
    VMP_TRY(cudaMemcpyAsync(out, d_pts, sizeof(vmp_point) * (size_t)m, cudaMemcpyDefault, s->st), "cloud");
    if (intensity)
        VMP_TRY(cudaMemcpyAsync(intensity, d_int, sizeof(float) * (size_t)m, cudaMemcpyDefault, s->st), "intensity");
    VMP_TRY(cudaStreamSynchronize(s->st), "output cloud");
    s->io_d2h += (long long)(sizeof(vmp_point) + (intensity ? sizeof(float) : 0)) * m;
    return VMP_OK;
}

// ------------------------------------------------------------- component API
static vmp_status stage_doubles(vmp_stream_t s, double* dst, const double* src, size_t count) {
    VMP_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyHostToDevice, s->st), "upload");
    return VMP_OK;
}

vmp_status vmp_map_index(vmp_stream_t s, const double* pts, int n, int64_t* keys) {
    if (!s || (!pts && n > 0) || (!keys && n > 0) || n < 0) return VMP_ERR_INVALID_ARG;
    if (n > s->cfg.max_scan_points) return fail(s, VMP_ERR_CAPACITY, "n larger than max_scan_points");
    if (n == 0) return VMP_OK;
    vmp_status v = stage_doubles(s, s->s.bpts, pts, (size_t)n * 3);
    if (v != VMP_OK) return v;
    int64_t* d_keys = reinterpret_cast<int64_t*>(s->s.bcov);
    launch_map_index(s->m, s->s.bpts, n, d_keys, s->st);
    VMP_TRY(cudaMemcpyAsync(keys, d_keys, sizeof(int64_t) * 3 * (size_t)n, cudaMemcpyDeviceToHost, s->st), "keys");
    VMP_TRY(cudaStreamSynchronize(s->st), "index");
    return VMP_OK;
}

static vmp_status map_component(vmp_stream_t s, const double* pts, const double* cov, int n, bool build) {
    if (!s || n < 0 || (n > 0 && (!pts || !cov))) return VMP_ERR_INVALID_ARG;
    if (s->broken) return fail(s, VMP_ERR_CUDA, "stream unusable after a CUDA error: " + s->err);
    if (n > s->cfg.max_scan_points) return fail(s, VMP_ERR_CAPACITY, "n larger than max_scan_points");
    if (build) {
        vmp_status v = read_counters(s);
        if (v != VMP_OK) return v;
        if (s->h_cnt->size != 0) return fail(s, VMP_ERR_STATE, "VoxelMap::build on a non-empty map");
    }
    if (n == 0) return VMP_OK;
    vmp_status v = stage_doubles(s, s->s.bpts, pts, (size_t)n * 3);
    if (v != VMP_OK) return v;
    v = stage_doubles(s, s->s.bcov, cov, (size_t)n * 9);
    if (v != VMP_OK) return v;
    v = map_apply(s, s->s.bpts, s->s.bcov, nullptr, n, n, build);
    if (v != VMP_OK) return v;
    VMP_NOTE_LAUNCH(); k_set_int<<<1, 32, 0, s->st>>>(s->s.d_n_down, 0);
    return finish_result(s, n, nullptr);
}

vmp_status vmp_map_build(vmp_stream_t s, const double* pts, const double* cov, int n) {
    return map_component(s, pts, cov, n, true);
}
vmp_status vmp_map_update(vmp_stream_t s, const double* pts, const double* cov, int n) {
    return map_component(s, pts, cov, n, false);
}

vmp_status vmp_map_info_get(vmp_stream_t s, vmp_map_info* info) {
    if (!s || !info) return VMP_ERR_INVALID_ARG;
    vmp_status v = read_counters(s);
    if (v != VMP_OK) return v;
    info->size = s->h_cnt->size;
    info->capacity = s->m.capacity;
    info->group_counter = s->h_cnt->group_counter;
    // buffered points: exported on demand
    std::vector<vmp_voxel> tmp;
    info->slab_points = -1;
    return VMP_OK;
}

static vmp_status export_all(vmp_stream_t s, std::vector<vmp_voxel>& out) {
    vmp_status v = read_counters(s);
    if (v != VMP_OK) return v;
    const long long n = s->h_cnt->size;
    out.resize((size_t)n);
    if (n == 0) return VMP_OK;
    vmp_voxel* d = nullptr;
    int* d_count = nullptr;
    VMP_TRY(cudaMalloc(&d, sizeof(vmp_voxel) * (size_t)n), "export alloc");
    VMP_TRY(cudaMalloc(&d_count, sizeof(int)), "export alloc");
    cudaMemsetAsync(d_count, 0, sizeof(int), s->st);
    VMP_NOTE_LAUNCH(); k_export<<<1216, 256, 0, s->st>>>(s->m, d, d_count, (int)n);
    cudaMemcpyAsync(out.data(), d, sizeof(vmp_voxel) * (size_t)n, cudaMemcpyDeviceToHost, s->st);
    cudaError_t e = cudaStreamSynchronize(s->st);
    cudaFree(d);
    cudaFree(d_count);
    if (e != cudaSuccess) return cuda_fail(s, e, "export");
    std::sort(out.begin(), out.end(), [](const vmp_voxel& a, const vmp_voxel& b) { return a.lru_stamp > b.lru_stamp; });
    return VMP_OK;
}

vmp_status vmp_map_export(vmp_stream_t s, vmp_voxel* out, long long max, long long* n_out) {
    if (!s || (!out && max > 0)) return VMP_ERR_INVALID_ARG;
    std::vector<vmp_voxel> all;
    vmp_status v = export_all(s, all);
    if (v != VMP_OK) return v;
    long long n = std::min<long long>(max, (long long)all.size());
    if (n > 0) std::memcpy(out, all.data(), sizeof(vmp_voxel) * (size_t)n);
    if (n_out) *n_out = (long long)all.size();
    return VMP_OK;
}

vmp_status vmp_map_keys(vmp_stream_t s, int64_t* keys, long long max, long long* n_out) {
    if (!s || max < 0 || (!keys && max > 0)) return VMP_ERR_INVALID_ARG;
    if (s->broken) return fail(s, VMP_ERR_CUDA, "stream unusable after a CUDA error: " + s->err);
    vmp_status v = read_counters(s);
    if (v != VMP_OK) return v;
    const long long n = s->h_cnt->size;
    if (n_out) *n_out = n;
    if (n == 0 || max == 0) return VMP_OK;
    unsigned long long* d = nullptr;
    VMP_TRY(cudaMallocAsync(&d, sizeof(unsigned long long) * (2 * (size_t)n + 1), s->st), "key export");
    int* d_count = reinterpret_cast<int*>(d + 2 * (size_t)n);
    std::vector<unsigned long long> h(2 * (size_t)n);
    cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(int), s->st);
    if (e == cudaSuccess) {
        VMP_NOTE_LAUNCH(); k_export_keys<<<1216, 256, 0, s->st>>>(s->m, d, d_count, (int)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h.data(), d, sizeof(unsigned long long) * 2 * (size_t)n, cudaMemcpyDeviceToHost, s->st);
    cudaFreeAsync(d, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) return cuda_fail(s, e, "key export");
    std::vector<size_t> ord((size_t)n);
    for (size_t i = 0; i < ord.size(); ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return h[2 * a] > h[2 * b]; });
    const long long m = std::min(max, n);
    for (long long i = 0; i < m; ++i) {
        int64_t x, y, z;
        unpack_key(h[2 * ord[(size_t)i] + 1], x, y, z);
        keys[3 * i] = x;
        keys[3 * i + 1] = y;
        keys[3 * i + 2] = z;
    }
    s->io_d2h += (long long)sizeof(unsigned long long) * 2 * n;
    return VMP_OK;
}

// Test hook: a[i] / b[i] by the reciprocal-and-correction path the kernels
// use for shared divisors and by the FP64 division (host arrays of n).
vmp_status vmp_test_division(const double* a, const double* b, int n, double* by_recip, double* by_div) {
    if (n < 0 || (n > 0 && (!a || !b || !by_recip || !by_div))) return VMP_ERR_INVALID_ARG;
    if (n == 0) return VMP_OK;
    double* d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * 4 * (size_t)n) != cudaSuccess) return VMP_ERR_OUT_OF_MEMORY;
    cudaError_t e = cudaMemcpy(d, a, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, b, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        VMP_NOTE_LAUNCH();
        k_div_check<<<std::min(1216, (n + 255) / 256), 256>>>(d, d + n, n, d + 2 * (size_t)n, d + 3 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(by_recip, d + 2 * (size_t)n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(by_div, d + 3 * (size_t)n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return VMP_ERR_CUDA;
    }
    return VMP_OK;
}

vmp_status vmp_map_planes(vmp_stream_t s, vmp_plane_marker* out, int max, int* n_out) {
    if (!s || !n_out || max < 0 || (max > 0 && !out)) return VMP_ERR_INVALID_ARG;
    if (s->broken) return fail(s, VMP_ERR_CUDA, "stream unusable after a CUDA error: " + s->err);
    *n_out = 0;
    if (max == 0) return VMP_OK;
    const int cap = s->m.rec_pool;
    const size_t stride = (size_t)cap + 16;
    if (!s->vis_buf) {
        VMP_TRY(cudaMalloc(&s->vis_buf, sizeof(uint32_t) * (6 * stride + 16)), "marker scratch");
        VMP_TRY(sort_scratch_alloc(s->vis_ss, cap), "marker scratch");
    }
    uint32_t* lo = s->vis_buf;
    uint32_t* hi = lo + stride;
    uint32_t* rec = hi + stride;
    uint32_t* perm = rec + stride;
    uint32_t* hi2 = perm + stride;
    uint32_t* rec2 = hi2 + stride;
    int* d_count = reinterpret_cast<int*>(rec2 + stride);
    cudaStream_t st = s->st;
    VMP_TRY(cudaMemsetAsync(d_count, 0, sizeof(int), st), "count");
    VMP_NOTE_LAUNCH(); k_plane_collect<<<1216, 256, 0, st>>>(s->m, d_count, lo, hi, rec, cap);
    const int g = std::max(1, std::min(1216, (cap + 255) / 256));
    VMP_NOTE_LAUNCH(); k_iota_u32<<<g, 256, 0, st>>>(perm, d_count);
    // LSD order: by the low stamp word, then stably by the high word
    radix_sort_pairs(lo, perm, d_count, 32, s->vis_ss, st);
    VMP_NOTE_LAUNCH(); k_permute_pair<<<g, 256, 0, st>>>(perm, hi, rec, hi2, rec2, d_count);
    radix_sort_pairs(hi2, rec2, d_count, 32, s->vis_ss, st);
    VMP_TRY(cudaMemcpyAsync(s->h_int, d_count, sizeof(int), cudaMemcpyDeviceToHost, st), "count");
    VMP_TRY(cudaStreamSynchronize(st), "markers");
    const int n = std::min(s->h_int[0], max);
    if (n <= 0) return VMP_OK;
    vmp_plane_marker* d_out = nullptr;
    VMP_TRY(cudaMallocAsync(&d_out, sizeof(vmp_plane_marker) * (size_t)n, st), "marker buffer");
    VMP_NOTE_LAUNCH(); k_plane_markers<<<std::max(1, std::min(1216, (n + 127) / 128)), 128, 0, st>>>(s->m, rec2, n, d_out);
    cudaError_t e = cudaMemcpyAsync(out, d_out, sizeof(vmp_plane_marker) * (size_t)n, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d_out, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(s, e, "markers");
    s->io_d2h += (long long)sizeof(vmp_plane_marker) * n;
    *n_out = n;
    return VMP_OK;
}

vmp_status vmp_map_export_points(vmp_stream_t s, double* pts, double* cov, long long max_points, long long* n_out) {
    if (!s) return VMP_ERR_INVALID_ARG;
    std::vector<vmp_voxel> all;
    vmp_status v = export_all(s, all);
    if (v != VMP_OK) return v;
    std::vector<int> recs;
    std::vector<long long> offs;
    long long total = 0;
    for (const vmp_voxel& x : all) {
        // voxels whose buffered points were not kept (no refit can use them)
        // contribute none
        const bool stored = !(x.pad & 0x40000000);
        const int cnt = stored ? x.n_temp : 0;
        recs.push_back(x.pad & 0x3FFFFFFF);
        offs.push_back(total);
        total += cnt;
    }
    if (n_out) *n_out = total;
    if (!pts || !cov || total == 0) return VMP_OK;
    if (total > max_points) return fail(s, VMP_ERR_CAPACITY, "max_points too small");
    int* d_recs = nullptr;
    long long* d_offs = nullptr;
    double *d_p = nullptr, *d_c = nullptr;
    VMP_TRY(cudaMalloc(&d_recs, sizeof(int) * recs.size()), "alloc");
    VMP_TRY(cudaMalloc(&d_offs, sizeof(long long) * offs.size()), "alloc");
    VMP_TRY(cudaMalloc(&d_p, sizeof(double) * 3 * (size_t)total), "alloc");
    VMP_TRY(cudaMalloc(&d_c, sizeof(double) * 9 * (size_t)total), "alloc");
    cudaMemcpyAsync(d_recs, recs.data(), sizeof(int) * recs.size(), cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(d_offs, offs.data(), sizeof(long long) * offs.size(), cudaMemcpyHostToDevice, s->st);
    VMP_NOTE_LAUNCH(); k_export_points<<<1216, 128, 0, s->st>>>(s->m, d_recs, d_offs, (int)recs.size(), d_p, d_c);
    cudaMemcpyAsync(pts, d_p, sizeof(double) * 3 * (size_t)total, cudaMemcpyDeviceToHost, s->st);
    cudaMemcpyAsync(cov, d_c, sizeof(double) * 9 * (size_t)total, cudaMemcpyDeviceToHost, s->st);
    cudaError_t e = cudaStreamSynchronize(s->st);
    cudaFree(d_recs); cudaFree(d_offs); cudaFree(d_p); cudaFree(d_c);
    if (e != cudaSuccess) return cuda_fail(s, e, "export points");
    return VMP_OK;
}

vmp_status vmp_map_import(vmp_stream_t s, const vmp_voxel* vox, long long n, const double* pts, const double* cov,
                          long long group_counter) {
    if (!s || n < 0 || (n > 0 && !vox)) return VMP_ERR_INVALID_ARG;
    if (n > s->m.capacity) return fail(s, VMP_ERR_CAPACITY, "more voxels than map_capacity");
    std::vector<long long> offs((size_t)n + 1, 0);
    long long total = 0;
    for (long long i = 0; i < n; ++i) {
        offs[(size_t)i] = total;
        total += vox[i].n_temp;
    }
    if (total > 0 && (!pts || !cov)) return VMP_ERR_INVALID_ARG;
    launch_map_reset(s->m, s->st);
    if (n > 0) {
        vmp_voxel* d_v = nullptr;
        long long* d_o = nullptr;
        double *d_p = nullptr, *d_c = nullptr;
        VMP_TRY(cudaMalloc(&d_v, sizeof(vmp_voxel) * (size_t)n), "alloc");
        VMP_TRY(cudaMalloc(&d_o, sizeof(long long) * (size_t)(n + 1)), "alloc");
        VMP_TRY(cudaMalloc(&d_p, sizeof(double) * 3 * (size_t)(total + 1)), "alloc");
        VMP_TRY(cudaMalloc(&d_c, sizeof(double) * 9 * (size_t)(total + 1)), "alloc");
        cudaMemcpyAsync(d_v, vox, sizeof(vmp_voxel) * (size_t)n, cudaMemcpyHostToDevice, s->st);
        cudaMemcpyAsync(d_o, offs.data(), sizeof(long long) * (size_t)(n + 1), cudaMemcpyHostToDevice, s->st);
        if (total > 0) {
            cudaMemcpyAsync(d_p, pts, sizeof(double) * 3 * (size_t)total, cudaMemcpyHostToDevice, s->st);
            cudaMemcpyAsync(d_c, cov, sizeof(double) * 9 * (size_t)total, cudaMemcpyHostToDevice, s->st);
        }
        const unsigned long long stamp_top = (unsigned long long)n + 1;
        VMP_NOTE_LAUNCH(); k_set_int<<<1, 32, 0, s->st>>>(&s->cnt->chunk_freed_top, 0);
        VMP_NOTE_LAUNCH(); k_import<<<1216, 128, 0, s->st>>>(s->m, d_v, (int)n, d_o, d_p, d_c, stamp_top);
        VMP_NOTE_LAUNCH(); k_import_counters<<<1, 32, 0, s->st>>>(s->m, (int)n, group_counter, stamp_top);
        cudaError_t e = cudaStreamSynchronize(s->st);
        cudaFree(d_v); cudaFree(d_o); cudaFree(d_p); cudaFree(d_c);
        if (e != cudaSuccess) return cuda_fail(s, e, "import");
    } else {
        VMP_NOTE_LAUNCH(); k_import_counters<<<1, 32, 0, s->st>>>(s->m, 0, group_counter, 1ull);
    }
    return read_counters(s);
}

vmp_status vmp_get_state(vmp_stream_t s, vmp_state* x, double* P) {
    if (!s) return VMP_ERR_INVALID_ARG;
    if (x) VMP_TRY(cudaMemcpyAsync(x, &s->f->x, sizeof(vmp_state), cudaMemcpyDeviceToHost, s->st), "state");
    if (P) VMP_TRY(cudaMemcpyAsync(P, s->f->P, sizeof(double) * 529, cudaMemcpyDeviceToHost, s->st), "P");
    VMP_TRY(cudaStreamSynchronize(s->st), "get state");
    return VMP_OK;
}

vmp_status vmp_set_state(vmp_stream_t s, const vmp_state* x, const double* P) {
    if (!s) return VMP_ERR_INVALID_ARG;
    if (x) VMP_TRY(cudaMemcpyAsync(&s->f->x, x, sizeof(vmp_state), cudaMemcpyHostToDevice, s->st), "state");
    if (P) VMP_TRY(cudaMemcpyAsync(s->f->P, P, sizeof(double) * 529, cudaMemcpyHostToDevice, s->st), "P");
    VMP_TRY(cudaStreamSynchronize(s->st), "set state");
    return VMP_OK;
}

vmp_status vmp_ieskf_predict(vmp_stream_t s, const double acc[3], const double gyro[3], double dt, const double* Q) {
    if (!s || !acc || !gyro) return VMP_ERR_INVALID_ARG;
    if (Q) VMP_TRY(cudaMemcpyAsync(s->f->Q, Q, sizeof(double) * 144, cudaMemcpyHostToDevice, s->st), "Q");
    launch_ieskf_predict_once(s->f, acc, gyro, dt, s->st);
    VMP_TRY(cudaGetLastError(), "predict");
    VMP_TRY(cudaStreamSynchronize(s->st), "predict");
    return VMP_OK;
}

vmp_status vmp_ieskf_update(vmp_stream_t s, const float* pts_l, int n, int* iters, int* effect_num) {
    if (!s || n < 0 || (n > 0 && !pts_l)) return VMP_ERR_INVALID_ARG;
    if (n > s->cfg.max_scan_points) return fail(s, VMP_ERR_CAPACITY, "n larger than max_scan_points");
    float* d_f = reinterpret_cast<float*>(s->s.bcov);
    VMP_TRY(cudaMemcpyAsync(d_f, pts_l, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, s->st), "upload");
    VMP_NOTE_LAUNCH(); k_floats_to_points<<<152, 256, 0, s->st>>>(d_f, n, s->s.down);
    VMP_NOTE_LAUNCH(); k_set_int<<<1, 32, 0, s->st>>>(s->s.d_n_down, n);
    launch_body_cov(s->s, n, s->cfg.ranging_cov, s->sin_deg, s->st);
    launch_update_begin(s->f, s->st);
    for (int it = 0; it < s->cfg.ieskf_max_iter; ++it)
        launch_residual_iter(s->f, s->s, s->m, n, s->cfg.estimate_ext, s->cfg.ieskf_eps, s->st, 1, 1);
    launch_update_end(s->f, s->cfg.estimate_ext, s->st);
    vmp_status v = finish_result(s, n, nullptr);
    if (v != VMP_OK) return v;
    if (iters) *iters = s->h_res->iters;
    if (effect_num) *effect_num = s->h_res->effect_num;
    return VMP_OK;
}

vmp_status vmp_residual_reduce(vmp_stream_t s, const vmp_state* x, const double* P, const double* pts_l,
                               const double* cov_l, int n, double* H, double* b, int* effect_num) {
    if (!s || !x || !P || n < 0 || (n > 0 && (!pts_l || !cov_l)) || !H || !b) return VMP_ERR_INVALID_ARG;
    if (n > s->cfg.max_scan_points) return fail(s, VMP_ERR_CAPACITY, "n larger than max_scan_points");
    VMP_TRY(cudaMemcpyAsync(&s->f->x, x, sizeof(vmp_state), cudaMemcpyHostToDevice, s->st), "state");
    VMP_TRY(cudaMemcpyAsync(s->f->P, P, sizeof(double) * 529, cudaMemcpyHostToDevice, s->st), "P");
    vmp_status v = stage_doubles(s, s->s.pl, pts_l, (size_t)n * 3);
    if (v != VMP_OK) return v;
    v = stage_doubles(s, s->s.covl, cov_l, (size_t)n * 9);
    if (v != VMP_OK) return v;
    VMP_NOTE_LAUNCH(); k_set_int<<<1, 32, 0, s->st>>>(s->s.d_n_down, n);
    VMP_NOTE_LAUNCH(); k_reset_filter_iter<<<1, 32, 0, s->st>>>(s->f);
    launch_residual_iter(s->f, s->s, s->m, n, s->cfg.estimate_ext, s->cfg.ieskf_eps, s->st, 0, 0);
    double* d_h = s->s.bcov;  // scratch
    int* d_e = reinterpret_cast<int*>(s->s.bcov + 160);
    VMP_NOTE_LAUNCH(); k_read_hm<<<1, 256, 0, s->st>>>(s->f, d_h, d_h + 144, d_e);
    VMP_TRY(cudaMemcpyAsync(H, d_h, sizeof(double) * 144, cudaMemcpyDeviceToHost, s->st), "H");
    VMP_TRY(cudaMemcpyAsync(b, d_h + 144, sizeof(double) * 12, cudaMemcpyDeviceToHost, s->st), "b");
    VMP_TRY(cudaMemcpyAsync(s->h_int, d_e, sizeof(int), cudaMemcpyDeviceToHost, s->st), "eff");
    VMP_TRY(cudaStreamSynchronize(s->st), "residual");
    if (effect_num) *effect_num = s->h_int[0];
    return VMP_OK;
}

vmp_status vmp_undistort(vmp_stream_t s, const vmp_scan* scan, const vmp_imu* imus, int n_imu, vmp_point* out) {
    if (!s || !scan || !out || !imus || n_imu <= 0 || scan->n <= 0) return VMP_ERR_INVALID_ARG;
    const int n = scan->n;
    if (n > s->cfg.max_scan_points) return fail(s, VMP_ERR_CAPACITY, "scan larger than max_scan_points");
    if (n_imu > s->cfg.max_imu_per_scan) return fail(s, VMP_ERR_CAPACITY, "too many IMU samples");
    vmp_status v = upload_scan(s, scan->points, n, false);
    if (v != VMP_OK) return v;
    v = upload_imus(s, imus, n_imu, false);
    if (v != VMP_OK) return v;
    v = upload_header(s, n, n_imu, scan->t_start, scan->t_end);
    if (v != VMP_OK) return v;
    const int nb = size_class(n, s->cfg.max_scan_points);
    launch_time_sort(s->s, nb, s->ss, s->st);
    launch_predict_chain2(s->f, s->s, s->st);
    launch_undistort(s->f, s->s, nb, s->st);
    VMP_TRY(cudaGetLastError(), "undistort");
    VMP_TRY(cudaMemcpyAsync(out, s->s.cloud, sizeof(vmp_point) * (size_t)n, cudaMemcpyDeviceToHost, s->st), "cloud");
    VMP_TRY(cudaStreamSynchronize(s->st), "undistort");
    return VMP_OK;
}

vmp_status vmp_downsample(vmp_stream_t s, const vmp_point* pts, int n, double leaf, vmp_point* out, int* n_out) {
    if (!s || n < 0 || (n > 0 && (!pts || !out)) || !n_out) return VMP_ERR_INVALID_ARG;
    if (n > s->cfg.max_scan_points) return fail(s, VMP_ERR_CAPACITY, "n larger than max_scan_points");
    if (!(leaf > 0)) return fail(s, VMP_ERR_INVALID_ARG, "leaf must be > 0");
    VMP_TRY(cudaMemcpyAsync(s->s.cloud, pts, sizeof(vmp_point) * (size_t)n, cudaMemcpyHostToDevice, s->st), "upload");
    VMP_NOTE_LAUNCH(); k_set_int<<<1, 32, 0, s->st>>>(s->s.d_n_raw, n);
    launch_downsample(s->s, n > 0 ? n : 1, leaf, s->ss, s->sc, s->st);
    VMP_TRY(cudaMemcpyAsync(s->h_int, s->s.d_n_down, sizeof(int), cudaMemcpyDeviceToHost, s->st), "n");
    VMP_TRY(cudaStreamSynchronize(s->st), "downsample");
    const int m = s->h_int[0];
    *n_out = m;
    if (m > 0) {
        VMP_TRY(cudaMemcpyAsync(out, s->s.down, sizeof(vmp_point) * (size_t)m, cudaMemcpyDeviceToHost, s->st), "down");
        VMP_TRY(cudaStreamSynchronize(s->st), "downsample");
    }
    return VMP_OK;
}

// Valid flags of the persistent residual records (test hook for the match set).
vmp_status vmp_residual_valid(vmp_stream_t s, unsigned char* valid, int n) {
    if (!s || !valid || n < 0 || n > s->cfg.max_scan_points) return VMP_ERR_INVALID_ARG;
    VMP_TRY(cudaMemcpyAsync(valid, s->s.rvalid, (size_t)n, cudaMemcpyDeviceToHost, s->st), "valid");
    VMP_TRY(cudaStreamSynchronize(s->st), "valid");
    return VMP_OK;
}

// The clouds of the last scan: kind 0 = undistorted (time-sorted) raw cloud,
// kind 1 = downsampled cloud.
vmp_status vmp_last_cloud(vmp_stream_t s, int kind, vmp_point* out, int max, int* n_out) {
    if (!s || !n_out) return VMP_ERR_INVALID_ARG;
    const int* d_n = kind == 0 ? s->s.d_n_raw : s->s.d_n_down;
    VMP_TRY(cudaMemcpyAsync(s->h_int, d_n, sizeof(int), cudaMemcpyDeviceToHost, s->st), "n");
    VMP_TRY(cudaStreamSynchronize(s->st), "n");
    const int n = s->h_int[0];
    *n_out = n;
    if (out && max > 0) {
        VMP_TRY(cudaMemcpyAsync(out, kind == 0 ? s->s.cloud : s->s.down, sizeof(vmp_point) * (size_t)std::min(n, max),
                                cudaMemcpyDeviceToHost, s->st), "cloud");
        VMP_TRY(cudaStreamSynchronize(s->st), "cloud");
    }
    return VMP_OK;
}

vmp_status vmp_profile_enable(vmp_stream_t s, int on) {
    if (!s) return VMP_ERR_INVALID_ARG;
    cudaStreamSynchronize(s->st);
    s->prof_on = on != 0;
    s->prof_pending.clear();
    s->ev_used = 0;
    for (int i = 0; i < VMP_PROF_SLOTS; ++i) { s->prof_ms[i] = 0; s->prof_launches[i] = 0; s->prof_items[i] = 0; }
    return VMP_OK;
}

vmp_status vmp_profile_read(vmp_stream_t s, double* ms, long long* launches, long long* items) {
    if (!s) return VMP_ERR_INVALID_ARG;
    for (int i = 0; i < VMP_PROF_SLOTS; ++i) {
        if (ms) ms[i] = s->prof_ms[i];
        if (launches) launches[i] = s->prof_launches[i];
        if (items) items[i] = s->prof_items[i];
    }
    return VMP_OK;
}

void* vmp_cuda_stream(vmp_stream_t s) { return s ? (void*)s->st : nullptr; }

vmp_status vmp_io_bytes(vmp_stream_t s, long long* h2d, long long* d2h) {
    if (!s) return VMP_ERR_INVALID_ARG;
    if (h2d) *h2d = s->io_h2d;
    if (d2h) *d2h = s->io_d2h + s->ms.merge_d2h;
    return VMP_OK;
}

long long vmp_launch_count(void) { return g_launch_count.load(std::memory_order_relaxed); }

// Selects the merge resolution: 0 = parallel fixed point (default),
// 1 = single-thread replay in point order (both exact).
vmp_status vmp_set_merge_mode(vmp_stream_t s, int mode) {
    if (!s || mode < 0 || mode > 1) return VMP_ERR_INVALID_ARG;
    s->ms.merge_mode = mode;
    return VMP_OK;
}
long long vmp_device_bytes(vmp_stream_t s) { return s ? s->dev_bytes : -1; }
vmp_status vmp_set_graphs(vmp_stream_t s, int on) {
    if (!s) return VMP_ERR_INVALID_ARG;
    s->use_graphs = on != 0;
    return VMP_OK;
}
long long vmp_eviction_splits(vmp_stream_t s) { return s ? s->eviction_splits : -1; }
vmp_status vmp_set_wait_mode(vmp_stream_t s, int blocking) {
    if (!s) return VMP_ERR_INVALID_ARG;
    s->blocking_wait = blocking != 0;
    return VMP_OK;
}
int vmp_last_merge_rounds(vmp_stream_t s) { return s ? merge_rounds_read(s->ms.merge, s->st) : -1; }
int vmp_last_merge_profile(vmp_stream_t s, double* us, int max) {
    if (!s || !us || max <= 0) return -1;
    return merge_profile_read(s->ms.merge, s->st, us, max);
}
vmp_status vmp_set_residual_ctas_per_sm(int ctas) {
    if (ctas != 3 && ctas != 4) return VMP_ERR_INVALID_ARG;
    residual_set_ctas_per_sm(ctas);
    return VMP_OK;
}
int vmp_last_merge_calls(vmp_stream_t s) {
    if (!s) return -1;
    int n = -1;
    if (cudaStreamSynchronize(s->st) != cudaSuccess ||
        cudaMemcpy(&n, s->ms.d_n_ev, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return n;
}

}  // extern "C"
