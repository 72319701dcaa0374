// VoxelGrid::merge (voxel_map.cpp:138-186) for every point of a batch that
// reached a frozen plane voxel, in point order.
//
// A merge call reads and writes frozen plane voxels only (the caller and its
// six face neighbours); nothing else in the batch changes a frozen voxel.  So
// the calls can be resolved after the per-voxel state machine, as a fixed
// point:
//   * every call is evaluated in parallel against "the state of each voxel as
//     of the call's point index" = the latest entry of a per-voxel write log
//     with a smaller point index, else the voxel's state after the state
//     machine;
//   * its writes (the caller's final plane and each merged neighbour's) form
//     the next log; a 64-bit signature per call detects change;
//   * when no call's outcome changes, the log equals the sequential
//     replay's: the earliest call always sees exact inputs, and by induction
//     every later one does once the calls before it have settled.
// If the fixed point is not reached in kMaxRounds rounds (long causal chains)
// or the log pool overflows, a single-thread replay in point order runs
// instead.  Both paths do the reference's arithmetic in its order.
#include <cstring>
#include "kernels.cuh"

namespace vmp {

constexpr int kMergeThreads = 256;
constexpr int kMaxRounds = 24;
constexpr uint32_t kNone = 0xFFFFFFFFu;

struct MState {
    double mean[3];
    double norm[3];
    double cov[36];
    uint64_t group;
    uint32_t merged;
    uint32_t pad;
};

struct MEntry {
    uint32_t rec;
    uint32_t t;      // batch-relative point index of the writing call
    uint32_t next;   // next entry of the same record
    uint32_t pad;
    MState s;
};

struct MergeCtl {
    int n_ent[2];
    int changed;
    int overflow;
};

struct MergeScratch {
    MEntry* ent[2];
    uint32_t* head[2];   // [rec_pool]
    uint64_t* sig;       // [max_batch] per call signature
    MergeCtl* ctl;
    MergeCtl* h_ctl;     // pinned host mirror
    int pool;
    int rec_pool;
};

__device__ inline void base_state(const DMap& m, uint32_t r, MState& s) {
    const RecHot& h = m.hot[r];
    const RecCold& c = m.cold[r];
    for (int k = 0; k < 3; ++k) { s.mean[k] = h.mean[k]; s.norm[k] = h.norm[k]; }
    for (int k = 0; k < 36; ++k) s.cov[k] = c.cov[k];
    s.group = h.group;
    s.merged = (h.flags & F_MERGED) ? 1u : 0u;
}

// State of record r as of batch point t (entries with a smaller t).
__device__ inline void state_at(const DMap& m, uint32_t r, uint32_t t, const MEntry* ent, const uint32_t* head,
                                MState& s) {
    uint32_t best = kNone, best_t = 0;
    if (head) {
        for (uint32_t e = head[r]; e != kNone; e = ent[e].next) {
            uint32_t et = ent[e].t;
            if (et < t && (best == kNone || et > best_t)) { best = e; best_t = et; }
        }
    }
    if (best == kNone) base_state(m, r, s);
    else s = ent[best].s;
}

__device__ inline double trace3(const double* cov, int off) {
    return (cov[off * 6 + off] + cov[(off + 1) * 6 + off + 1]) + cov[(off + 2) * 6 + off + 2];
}

__device__ inline uint64_t mix64(uint64_t h, uint64_t v) {
    h ^= v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 0xff51afd7ed558ccdull;
    return h ^ (h >> 29);
}
__device__ inline uint64_t sig_state(uint64_t h, uint32_t rec, const MState& s) {
    h = mix64(h, rec);
    for (int k = 0; k < 3; ++k) { h = mix64(h, __double_as_longlong(s.mean[k])); h = mix64(h, __double_as_longlong(s.norm[k])); }
    for (int k = 0; k < 36; ++k) h = mix64(h, __double_as_longlong(s.cov[k]));
    h = mix64(h, s.group);
    return mix64(h, s.merged);
}

// One merge() call by record a_rec at batch point t.  Outputs the written
// states (neighbours first, in probe order, then the caller) into out/out_rec;
// returns how many.
__device__ int merge_call(const DMap& m, uint32_t a_rec, uint32_t t, const MEntry* ent, const uint32_t* head,
                          MState* out, uint32_t* out_rec) {
    const unsigned long long T = m.cnt->batch_base + t;
    MState a;
    state_at(m, a_rec, t, ent, head, a);
    int64_t x, y, z;
    unpack_key(m.cold[a_rec].key, x, y, z);
    const int64_t nb[6][3] = {{x - 1, y, z}, {x, y - 1, z}, {x, y, z - 1}, {x + 1, y, z}, {x, y + 1, z}, {x, y, z + 1}};
    int nout = 0;
    bool any = false;
    for (int k = 0; k < 6; ++k) {
        if (!key_in_range(nb[k][0]) || !key_in_range(nb[k][1]) || !key_in_range(nb[k][2])) continue;
        uint32_t b_rec = map_find(m, pack_key(nb[k][0], nb[k][1], nb[k][2]));
        if (b_rec == kNoRec || b_rec >= (uint32_t)m.rec_pool) continue;
        const RecCold& bc = m.cold[b_rec];
        if (!(m.hot[b_rec].flags & F_ALIVE) && bc.evict_g == kNever) continue;
        if (!(bc.create_g < T && bc.evict_g > T)) continue;  // not in the map at this point
        const bool frozen = bc.freeze_g < T;
        const bool plane = (m.hot[b_rec].flags & F_PLANE) != 0;
        MState b;
        state_at(m, b_rec, t, ent, head, b);
        if (b.group == a.group || !frozen || !plane) continue;
        double norm_distance = 1.0 - dot3(b.norm, a.norm);
        double axis_distance = fabs(dot3(b.norm, b.mean) - dot3(a.norm, a.mean));
        if (norm_distance > m.merge_angle || axis_distance > m.merge_dist) continue;
        double tn0 = trace3(a.cov, 0), tm0 = trace3(a.cov, 3), tn1 = trace3(b.cov, 0), tm1 = trace3(b.cov, 3);
        double tc0 = tn0 + tm0, tc1 = tn1 + tm1;
        MState ns;
        for (int q = 0; q < 3; ++q) {
            ns.mean[q] = tm0 * b.mean[q] + tm1 * a.mean[q] / (tm0 + tm1);
            ns.norm[q] = tn0 * b.norm[q] + tn1 * a.norm[q] / (tn0 + tn1);
        }
        const double w0 = tc0 * tc0, w1 = tc1 * tc1, den = (tc0 + tc1) * (tc0 + tc1);
        for (int q = 0; q < 36; ++q) ns.cov[q] = (w0 * b.cov[q] + w1 * a.cov[q]) / den;
        if (-dot3(ns.mean, ns.norm) < 0.0) {
            for (int q = 0; q < 3; ++q) ns.norm[q] = -ns.norm[q];
        }
        b.group = a.group;
        a.merged = 1;
        b.merged = 1;
        for (int q = 0; q < 3; ++q) { a.mean[q] = ns.mean[q]; a.norm[q] = ns.norm[q]; b.mean[q] = ns.mean[q]; b.norm[q] = ns.norm[q]; }
        for (int q = 0; q < 36; ++q) { a.cov[q] = ns.cov[q]; b.cov[q] = ns.cov[q]; }
        out[nout] = b;
        out_rec[nout] = b_rec;
        ++nout;
        any = true;
    }
    if (any) {
        out[nout] = a;
        out_rec[nout] = a_rec;
        ++nout;
    }
    return nout;
}

__device__ inline void write_state(const DMap& m, uint32_t r, const MState& s) {
    RecHot& h = m.hot[r];
    RecCold& c = m.cold[r];
    for (int k = 0; k < 3; ++k) { h.mean[k] = s.mean[k]; h.norm[k] = s.norm[k]; }
    for (int k = 0; k < 36; ++k) c.cov[k] = s.cov[k];
    h.group = s.group;
    if (s.merged) h.flags |= F_MERGED;
}

// ------------------------------------------------------------ sequential replay
__global__ void k_merge_sequential(DMap m, const uint32_t* __restrict__ ev_list, const uint32_t* __restrict__ ev_rec,
                                   const int* d_n_ev) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int ne = *d_n_ev;
    MState out[7];
    uint32_t out_rec[7];
    for (int e = 0; e < ne; ++e) {
        uint32_t t = ev_list[e];
        int no = merge_call(m, ev_rec[t], t, nullptr, nullptr, out, out_rec);
        for (int k = 0; k < no; ++k) write_state(m, out_rec[k], out[k]);
    }
}

// ------------------------------------------------------------ fixed point
__global__ void k_merge_clear(MergeScratch ms, int cur) {
    const int n = ms.ctl->n_ent[cur];
    const int lim = n < ms.pool ? n : ms.pool;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < lim; e += gridDim.x * blockDim.x)
        ms.head[cur][ms.ent[cur][e].rec] = kNone;
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0) { ms.ctl->changed = 0; }
}
__global__ void k_merge_reset_count(MergeScratch ms, int cur) {
    if (threadIdx.x == 0 && blockIdx.x == 0) ms.ctl->n_ent[cur] = 0;
}
__global__ void k_merge_begin(MergeScratch ms) {
    if (threadIdx.x == 0 && blockIdx.x == 0) { ms.ctl->overflow = 0; ms.ctl->changed = 0; }
}

__global__ void __launch_bounds__(kMergeThreads) k_merge_round(DMap m, MergeScratch ms, const uint32_t* __restrict__ ev_list,
                                                               const uint32_t* __restrict__ ev_rec,
                                                               const int* d_n_ev, int cur, int first) {
    const int ne = *d_n_ev;
    const int prev = cur ^ 1;
    const MEntry* pent = ms.ent[prev];
    const uint32_t* phead = first ? nullptr : ms.head[prev];
    MState out[7];
    uint32_t out_rec[7];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const uint32_t t = ev_list[e];
        int no = merge_call(m, ev_rec[t], t, pent, phead, out, out_rec);
        uint64_t sg = 0x1234567ull + (uint64_t)no;
        for (int k = 0; k < no; ++k) sg = sig_state(sg, out_rec[k], out[k]);
        if (first || ms.sig[e] != sg) atomicAdd(&ms.ctl->changed, 1);
        ms.sig[e] = sg;
        if (no == 0) continue;
        int pos = atomicAdd(&ms.ctl->n_ent[cur], no);
        if (pos + no > ms.pool) { ms.ctl->overflow = 1; continue; }
        for (int k = 0; k < no; ++k) {
            MEntry& en = ms.ent[cur][pos + k];
            en.rec = out_rec[k];
            en.t = t;
            en.s = out[k];
            en.next = atomicExch(&ms.head[cur][out_rec[k]], (uint32_t)(pos + k));
        }
    }
}

// Final states: the latest entry of each written record.
__global__ void k_merge_apply(DMap m, MergeScratch ms, int cur) {
    const int n = ms.ctl->n_ent[cur];
    const MEntry* ent = ms.ent[cur];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const uint32_t r = ent[e].rec;
        // the entry is the record's latest if no other entry of r has a larger t
        bool latest = true;
        for (uint32_t o = ms.head[cur][r]; o != kNone; o = ent[o].next)
            if (ent[o].t > ent[e].t) { latest = false; break; }
        if (latest) write_state(m, r, ent[e].s);
    }
}

__global__ void k_flag_merge_fallback(DMap m) {
    if (threadIdx.x == 0 && blockIdx.x == 0) m.cnt->changed = 1;  // informational: the replay path ran
}
static void set_error_host_flag(DMap& m, cudaStream_t st) { VMP_NOTE_LAUNCH(); k_flag_merge_fallback<<<1, 32, 0, st>>>(m); }

static MergeScratch* g_unused = nullptr;

cudaError_t merge_scratch_alloc(void** out, int max_batch, int rec_pool) {
    MergeScratch* ms = new MergeScratch();
    std::memset(ms, 0, sizeof(*ms));
    ms->pool = max_batch / 2 + 1024;
    ms->rec_pool = rec_pool;
    cudaError_t e;
    for (int b = 0; b < 2; ++b) {
        if ((e = cudaMalloc(&ms->ent[b], sizeof(MEntry) * (size_t)ms->pool)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&ms->head[b], sizeof(uint32_t) * (size_t)rec_pool)) != cudaSuccess) return e;
        if ((e = cudaMemset(ms->head[b], 0xFF, sizeof(uint32_t) * (size_t)rec_pool)) != cudaSuccess) return e;
    }
    if ((e = cudaMalloc(&ms->sig, sizeof(uint64_t) * ((size_t)max_batch + 16))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&ms->ctl, sizeof(MergeCtl))) != cudaSuccess) return e;
    if ((e = cudaMemset(ms->ctl, 0, sizeof(MergeCtl))) != cudaSuccess) return e;
    if ((e = cudaMallocHost(&ms->h_ctl, sizeof(MergeCtl))) != cudaSuccess) return e;
    *out = ms;
    (void)g_unused;
    return cudaSuccess;
}
void merge_scratch_free(void* p) {
    MergeScratch* ms = (MergeScratch*)p;
    if (!ms) return;
    for (int b = 0; b < 2; ++b) { cudaFree(ms->ent[b]); cudaFree(ms->head[b]); }
    cudaFree(ms->sig);
    cudaFree(ms->ctl);
    cudaFreeHost(ms->h_ctl);
    delete ms;
}

// Host loop: rounds until no call changes (one small device->host read per
// round), then applies the log; sequential replay as the fallback.
cudaError_t run_merge_events(DMap& m, MapScratch& ms, void* scratch, int n_max, int mode, int* rounds_out,
                             cudaStream_t st) {
    MergeScratch& g = *(MergeScratch*)scratch;
    int grid = (n_max + kMergeThreads - 1) / kMergeThreads;
    if (grid > 152 * 4) grid = 152 * 4;
    if (grid < 1) grid = 1;
    if (rounds_out) *rounds_out = 0;
    if (mode == 1) {  // sequential replay only
        VMP_NOTE_LAUNCH(); k_merge_sequential<<<1, 32, 0, st>>>(m, ms.ev_list, ms.ev_rec, ms.d_n_ev);
        return cudaGetLastError();
    }
    cudaError_t e;
    VMP_NOTE_LAUNCH(); k_merge_begin<<<1, 32, 0, st>>>(g);
    // clear both logs (left over from the previous batch)
    for (int b = 0; b < 2; ++b) {
        VMP_NOTE_LAUNCH(); k_merge_clear<<<grid, kMergeThreads, 0, st>>>(g, b);
        VMP_NOTE_LAUNCH(); k_merge_reset_count<<<1, 32, 0, st>>>(g, b);
    }
    int cur = 0;
    bool converged = false;
    for (int r = 0; r < kMaxRounds; ++r) {
        VMP_NOTE_LAUNCH(); k_merge_clear<<<grid, kMergeThreads, 0, st>>>(g, cur);
        VMP_NOTE_LAUNCH(); k_merge_reset_count<<<1, 32, 0, st>>>(g, cur);
        VMP_NOTE_LAUNCH(); k_merge_round<<<grid, kMergeThreads, 0, st>>>(m, g, ms.ev_list, ms.ev_rec, ms.d_n_ev, cur, r == 0 ? 1 : 0);
        if ((e = cudaMemcpyAsync(g.h_ctl, g.ctl, sizeof(MergeCtl), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
        ms.merge_d2h += (long long)sizeof(MergeCtl);
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        if (rounds_out) *rounds_out = r + 1;
        if (g.h_ctl->overflow) break;
        if (g.h_ctl->n_ent[cur] == 0 && r == 0) { converged = true; break; }  // no call merges anything
        if (r > 0 && g.h_ctl->changed == 0) { converged = true; break; }
        cur ^= 1;
    }
    if (converged) {
        VMP_NOTE_LAUNCH(); k_merge_apply<<<grid, kMergeThreads, 0, st>>>(m, g, cur);
    } else {
        VMP_NOTE_LAUNCH(); k_merge_sequential<<<1, 32, 0, st>>>(m, ms.ev_list, ms.ev_rec, ms.d_n_ev);
        set_error_host_flag(m, st);
    }
    return cudaGetLastError();
}

}  // namespace vmp
