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
//     every later one does once the calls before it have settled (a fixed
//     point is therefore unique).
// All rounds run in one cooperative kernel (its CTAs are co-resident; rounds
// are separated by a grid barrier whose waits are bounded), so the host never
// waits on a round.  Per round, one thread per call tests whether the call
// merges anything (most do not: in the reference sequence the first call on a
// pair of voxels gives them one group id, and later calls see equal groups);
// the calls that merge are then re-run by one warp each, with the 36
// covariance entries and the 6 mean / normal components of the merge
// arithmetic on separate lanes.  Which neighbours can be merged at all (in
// the map at the call's point, frozen, plane) does not change during the
// merges, so it is decided once, in the first round.
// If the fixed point is not reached in kMaxRounds rounds, the log pool
// overflows or a barrier wait runs out, a single-thread replay in point order
// runs instead.  Both paths do the reference's arithmetic in its order.
#include <cstring>
#include <mutex>
#include <vector>
#include "kernels.cuh"

namespace vmp {

constexpr int kMergeThreads = 256;
constexpr int kMaxRounds = 24;
constexpr int kLogs = 3;  // round r writes log r % 3, reads log (r - 1) % 3, clears log (r + 1) % 3
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint64_t kSigNone = 0x1234567ull;
constexpr long long kBarrierSpinLimit = 20000000;  // x >= 64 ns sleeps: about a second or more
constexpr int kMaxMarks = 4 + 2 * kMaxRounds;

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
    int n_ent[kLogs];
    int overflow;
    int changed[kMaxRounds];
    int n_queue[kMaxRounds];
    int rounds;     // rounds run by the last batch
    int converged;  // 1: the final log is the sequential result
    int wait_error; // a grid barrier gave up waiting
    int pad;
    unsigned int bar_count;
    unsigned int bar_gen;
    unsigned int epoch;  // batches resolved so far (tags rec_round)
    int n_marks;
    // %globaltimer (ns) at the kernel's start and after each of its grid
    // barriers (for the per-round profile of the last batch)
    unsigned long long t_mark[kMaxMarks];
};

struct MergeScratch {
    MEntry* ent[kLogs];
    uint32_t* head[kLogs];  // [rec_pool]
    uint64_t* sig;          // [max_batch] per call signature
    uint32_t* cand;         // [max_batch * 6] mergeable neighbours per call (kNone: none)
    uint32_t* queue;        // [max_batch] calls that merge in the current round
    uint32_t* rec_round;    // [rec_pool] (epoch << 8) | the last round that wrote the record
    MergeCtl* ctl;
    int pool;
    int rec_pool;
    int coop_capacity;  // CTAs of k_merge_fixpoint the device holds at once
    int sms;
};

__device__ inline void base_state(const DMap& m, uint32_t r, MState& s) {
    const RecHot& h = m.hot[r];
    const RecCold& c = m.cold[r];
    for (int k = 0; k < 3; ++k) { s.mean[k] = h.mean[k]; s.norm[k] = h.norm[k]; }
    for (int k = 0; k < 36; ++k) s.cov[k] = c.cov[k];
    s.group = h.group;
    s.merged = (h.flags & F_MERGED) ? 1u : 0u;
}

// Latest log entry of record r written before batch point t (kNone: none).
__device__ inline uint32_t find_entry(uint32_t r, uint32_t t, const MEntry* ent, const uint32_t* head) {
    uint32_t best = kNone, best_t = 0;
    if (head) {
        for (uint32_t e = head[r]; e != kNone; e = ent[e].next) {
            const uint32_t et = ent[e].t;
            if (et < t && (best == kNone || et > best_t)) { best = e; best_t = et; }
        }
    }
    return best;
}

// State of record r as of batch point t.
__device__ inline void state_at(const DMap& m, uint32_t r, uint32_t t, const MEntry* ent, const uint32_t* head,
                                MState& s) {
    const uint32_t best = find_entry(r, t, ent, head);
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

// The static part of merge()'s neighbour test: neighbour k of the caller is
// in the map at point T, frozen and a plane (voxel_map.cpp:146-152).
__device__ inline uint32_t merge_candidate(const DMap& m, int64_t x, int64_t y, int64_t z, int k,
                                           unsigned long long T) {
    const int64_t nb[6][3] = {{x - 1, y, z}, {x, y - 1, z}, {x, y, z - 1}, {x + 1, y, z}, {x, y + 1, z}, {x, y, z + 1}};
    if (!key_in_range(nb[k][0]) || !key_in_range(nb[k][1]) || !key_in_range(nb[k][2])) return kNone;
    const uint32_t b_rec = map_find(m, pack_key(nb[k][0], nb[k][1], nb[k][2]));
    if (b_rec == kNoRec || b_rec >= (uint32_t)m.rec_pool) return kNone;
    const RecCold& bc = m.cold[b_rec];
    if (!(m.hot[b_rec].flags & F_ALIVE) && bc.evict_g == kNever) return kNone;
    if (!(bc.create_g < T && bc.evict_g > T)) return kNone;  // not in the map at this point
    if (!(bc.freeze_g < T)) return kNone;
    if (!(m.hot[b_rec].flags & F_PLANE)) return kNone;
    return b_rec;
}

// merge_candidate for all six neighbours at once, with the loads of the six
// lookups issued together (the first probe of each; a collision falls back to
// the probe loop) and then those of the six records: one memory round trip
// per step instead of six.
__device__ inline void merge_candidates6(const DMap& m, int64_t x, int64_t y, int64_t z, unsigned long long T,
                                         uint32_t out[6]) {
    const int64_t nb[6][3] = {{x - 1, y, z}, {x, y - 1, z}, {x, y, z - 1}, {x + 1, y, z}, {x, y + 1, z}, {x, y, z + 1}};
    uint64_t key[6], h[6], kk[6];
    bool ok[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        ok[k] = key_in_range(nb[k][0]) && key_in_range(nb[k][1]) && key_in_range(nb[k][2]);
        key[k] = ok[k] ? pack_key(nb[k][0], nb[k][1], nb[k][2]) : 0;
        h[k] = hash_key(key[k]) & m.table_mask;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) kk[k] = ok[k] ? __ldg(&m.keys[h[k]]) : kEmptyKey;
    uint32_t rec[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) rec[k] = (ok[k] && kk[k] == key[k]) ? __ldg(&m.vals[h[k]]) : kNoRec;
    for (int k = 0; k < 6; ++k)  // first slot taken by another key: probe on (rare)
        if (ok[k] && kk[k] != key[k] && kk[k] != kEmptyKey) rec[k] = map_find(m, key[k]);
    unsigned long long cg[6], eg[6], fg[6];
    uint32_t fl[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const bool v = rec[k] != kNoRec && rec[k] < (uint32_t)m.rec_pool;
        if (!v) rec[k] = kNoRec;
        const uint32_t r = v ? rec[k] : 0;
        fl[k] = v ? m.hot[r].flags : 0u;
        cg[k] = v ? m.cold[r].create_g : 0ull;
        eg[k] = v ? m.cold[r].evict_g : 0ull;
        fg[k] = v ? m.cold[r].freeze_g : 0ull;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        uint32_t r = rec[k];
        if (r != kNoRec) {
            if (!(fl[k] & F_ALIVE) && eg[k] == kNever) r = kNone;
            else if (!(cg[k] < T && eg[k] > T)) r = kNone;  // not in the map at this point
            else if (!(fg[k] < T)) r = kNone;
            else if (!(fl[k] & F_PLANE)) r = kNone;
        } else {
            r = kNone;
        }
        out[k] = r;
    }
}

// One merge() call by record a_rec at batch point t, one thread (the replay).
// Outputs the written states (neighbours first, in probe order, then the
// caller) into out/out_rec; returns how many.
__device__ int merge_call(const DMap& m, uint32_t a_rec, uint32_t t, MState* out, uint32_t* out_rec) {
    const unsigned long long T = m.cnt->batch_base + t;
    MState a;
    base_state(m, a_rec, a);
    int64_t x, y, z;
    unpack_key(m.cold[a_rec].key, x, y, z);
    int nout = 0;
    bool any = false;
    for (int k = 0; k < 6; ++k) {
        const uint32_t b_rec = merge_candidate(m, x, y, z, k, T);
        if (b_rec == kNone) continue;
        MState b;
        base_state(m, b_rec, b);
        if (b.group == a.group) continue;
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
// Every call in point order on one thread, writing the records in place
// (mode 1, and the fallback when the fixed point did not settle: `only_if`
// non-null makes it return when the fixed point converged).
__global__ void k_merge_sequential(DMap m, const uint32_t* __restrict__ ev_list, const uint32_t* __restrict__ ev_rec,
                                   const int* d_n_ev, const MergeCtl* only_if) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (only_if && only_if->converged) return;
    if (only_if) m.cnt->changed = 1;  // informational: the replay path ran
    const int ne = *d_n_ev;
    MState out[7];
    uint32_t out_rec[7];
    for (int e = 0; e < ne; ++e) {
        const uint32_t t = ev_list[e];
        const int no = merge_call(m, ev_rec[t], t, out, out_rec);
        for (int k = 0; k < no; ++k) write_state(m, out_rec[k], out[k]);
    }
}

// ------------------------------------------------------------ fixed point
// Grid barrier for the cooperative kernel (all CTAs co-resident).  A wait
// gives up after kBarrierSpinLimit polls, records the failure and lets every
// later barrier pass at once, so the kernel always ends; the replay then
// produces the result.
__device__ void grid_barrier(MergeCtl* c, long long spin_limit = kBarrierSpinLimit) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* vgen = &c->bar_gen;
        volatile int* verr = &c->wait_error;
        if (!*verr) {
            const unsigned int g = *vgen;
            __threadfence();
            if (atomicAdd(&c->bar_count, 1u) == gridDim.x - 1) {
                c->bar_count = 0;
                __threadfence();
                atomicAdd(&c->bar_gen, 1u);
            } else {
                long long spins = 0;
                while (*vgen == g) {
                    if (*verr) break;
                    __nanosleep(64);
                    if (++spins > spin_limit) {
                        atomicExch(&c->wait_error, 1);
                        break;
                    }
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
}

struct PlaneRef {
    double mean[3], norm[3];
    uint64_t group;
};
__device__ inline void plane_at(const DMap& m, uint32_t r, uint32_t t, const MEntry* ent, const uint32_t* head,
                                PlaneRef& p) {
    const uint32_t e = find_entry(r, t, ent, head);
    if (e == kNone) {
        const RecHot& h = m.hot[r];
        for (int k = 0; k < 3; ++k) { p.mean[k] = h.mean[k]; p.norm[k] = h.norm[k]; }
        p.group = h.group;
    } else {
        const MState& s = ent[e].s;
        for (int k = 0; k < 3; ++k) { p.mean[k] = s.mean[k]; p.norm[k] = s.norm[k]; }
        p.group = s.group;
    }
}

// Does the call merge anything?  merge()'s tests up to its first merge, with
// the caller's state as of the call (one thread).
// The group ids of the six neighbours are read first (independent loads and
// log walks, which overlap); a neighbour of the caller's group is skipped
// without reading its plane.
__device__ bool call_merges(const DMap& m, uint32_t a_rec, uint32_t t, const uint32_t* cand, const MEntry* ent,
                            const uint32_t* head) {
    PlaneRef a;
    plane_at(m, a_rec, t, ent, head, a);
    uint32_t eb[6];
    uint64_t gb[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        eb[k] = cand[k] != kNone ? find_entry(cand[k], t, ent, head) : kNone;
        gb[k] = cand[k] == kNone ? a.group : (eb[k] == kNone ? m.hot[cand[k]].group : ent[eb[k]].s.group);
    }
    for (int k = 0; k < 6; ++k) {
        const uint32_t b_rec = cand[k];
        if (b_rec == kNone || gb[k] == a.group) continue;
        PlaneRef b;
        if (eb[k] == kNone) {
            const RecHot& hb = m.hot[b_rec];
            for (int q = 0; q < 3; ++q) { b.mean[q] = hb.mean[q]; b.norm[q] = hb.norm[q]; }
        } else {
            const MState& sb = ent[eb[k]].s;
            for (int q = 0; q < 3; ++q) { b.mean[q] = sb.mean[q]; b.norm[q] = sb.norm[q]; }
        }
        double norm_distance = 1.0 - dot3(b.norm, a.norm);
        double axis_distance = fabs(dot3(b.norm, b.mean) - dot3(a.norm, a.mean));
        if (norm_distance > m.merge_angle || axis_distance > m.merge_dist) continue;
        return true;
    }
    return false;
}

// A voxel state spread over a warp: mean / normal / group on every lane,
// covariance entry `lane` in c0 and entry 32 + lane (lane < 4) in c1.
struct WState {
    double mean[3], norm[3];
    double c0, c1;
    uint64_t group;
    uint32_t merged;
};
__device__ inline void wstate_load(const DMap& m, uint32_t r, uint32_t e, const MEntry* ent, int lane, WState& s) {
    if (e == kNone) {
        const RecHot& h = m.hot[r];
        const RecCold& c = m.cold[r];
        for (int k = 0; k < 3; ++k) { s.mean[k] = h.mean[k]; s.norm[k] = h.norm[k]; }
        s.c0 = c.cov[lane];
        s.c1 = lane < 4 ? c.cov[32 + lane] : 0.0;
        s.group = h.group;
        s.merged = (h.flags & F_MERGED) ? 1u : 0u;
    } else {
        const MState& x = ent[e].s;
        for (int k = 0; k < 3; ++k) { s.mean[k] = x.mean[k]; s.norm[k] = x.norm[k]; }
        s.c0 = x.cov[lane];
        s.c1 = lane < 4 ? x.cov[32 + lane] : 0.0;
        s.group = x.group;
        s.merged = x.merged;
    }
}
// trace3(cov, 0) and trace3(cov, 3) of a warp-spread covariance
__device__ inline void wtraces(const WState& s, double& tn, double& tm) {
    const double d0 = __shfl_sync(0xffffffffu, s.c0, 0), d7 = __shfl_sync(0xffffffffu, s.c0, 7),
                 d14 = __shfl_sync(0xffffffffu, s.c0, 14), d21 = __shfl_sync(0xffffffffu, s.c0, 21),
                 d28 = __shfl_sync(0xffffffffu, s.c0, 28), d35 = __shfl_sync(0xffffffffu, s.c1, 3);
    tn = (d0 + d7) + d14;
    tm = (d21 + d28) + d35;
}
// Appends one output state to the log; returns its contribution to the
// call's signature (the same on every lane).
__device__ inline uint64_t wstate_emit(MergeScratch& g, int cur, uint32_t rec, uint32_t t, const WState& s, int lane,
                                       bool& overflow, uint32_t round_tag) {
    uint64_t h = mix64(0x51ull + lane, __double_as_longlong(s.c0));
    if (lane < 4) h = mix64(h, __double_as_longlong(s.c1));
    if (lane == 0) {
        h = mix64(h, rec);
        for (int k = 0; k < 3; ++k) { h = mix64(h, __double_as_longlong(s.mean[k])); h = mix64(h, __double_as_longlong(s.norm[k])); }
        h = mix64(h, s.group);
        h = mix64(h, s.merged);
    }
    for (int o = 16; o > 0; o >>= 1) h ^= __shfl_xor_sync(0xffffffffu, h, o);
    int pos = 0;
    if (lane == 0) pos = atomicAdd(&g.ctl->n_ent[cur], 1);
    pos = __shfl_sync(0xffffffffu, pos, 0);
    if (pos >= g.pool) {
        overflow = true;
        return h;
    }
    MEntry& en = g.ent[cur][pos];
    if (lane == 0) g.rec_round[rec] = round_tag;
    en.s.cov[lane] = s.c0;
    if (lane < 4) en.s.cov[32 + lane] = s.c1;
    if (lane == 0) {
        en.rec = rec;
        en.t = t;
        for (int k = 0; k < 3; ++k) { en.s.mean[k] = s.mean[k]; en.s.norm[k] = s.norm[k]; }
        en.s.group = s.group;
        en.s.merged = s.merged;
        __threadfence();
        en.next = atomicExch(&g.head[cur][rec], (uint32_t)pos);
    }
    return h;
}

// One merge() call on one warp, against the previous round's log; writes its
// outputs to log `cur` and returns the call's signature.
__device__ uint64_t warp_merge_call(const DMap& m, MergeScratch& g, uint32_t a_rec, uint32_t t, const uint32_t* cand,
                                    const MEntry* pent, const uint32_t* phead, int cur, bool& overflow,
                                    uint32_t round_tag) {
    const int lane = threadIdx.x & 31;
    // the log entries of the caller (lane 6) and of the six neighbours (lanes
    // 0-5) as of the call, and the neighbours' group ids: walked in parallel
    // (nothing the call writes changes a neighbour's state before it is read)
    uint32_t e_l = kNone;
    uint64_t g_l = 0;
    if (lane < 6 && cand[lane] != kNone) {
        e_l = find_entry(cand[lane], t, pent, phead);
        g_l = e_l == kNone ? m.hot[cand[lane]].group : pent[e_l].s.group;
    } else if (lane == 6) {
        e_l = find_entry(a_rec, t, pent, phead);
    }
    const uint32_t ea = __shfl_sync(0xffffffffu, e_l, 6);
    WState a;
    wstate_load(m, a_rec, ea, pent, lane, a);
    uint64_t sig = kSigNone;
    int nout = 0;
    for (int k = 0; k < 6; ++k) {
        const uint32_t b_rec = cand[k];
        const uint32_t eb = __shfl_sync(0xffffffffu, e_l, k);
        const uint64_t gbk = __shfl_sync(0xffffffffu, g_l, k);
        if (b_rec == kNone || gbk == a.group) continue;
        WState b;
        wstate_load(m, b_rec, eb, pent, lane, b);
        double norm_distance = 1.0 - dot3(b.norm, a.norm);
        double axis_distance = fabs(dot3(b.norm, b.mean) - dot3(a.norm, a.mean));
        if (norm_distance > m.merge_angle || axis_distance > m.merge_dist) continue;
        double tn0, tm0, tn1, tm1;
        wtraces(a, tn0, tm0);
        wtraces(b, tn1, tm1);
        const double tc0 = tn0 + tm0, tc1 = tn1 + tm1;
        // mean on lanes 0-2, normal on lanes 3-5 (the reference's precedence:
        // only the second product is divided)
        const int q = lane < 3 ? lane : (lane < 6 ? lane - 3 : 0);
        const bool is_mean = lane < 3;
        const double bv = is_mean ? (q == 0 ? b.mean[0] : q == 1 ? b.mean[1] : b.mean[2])
                                  : (q == 0 ? b.norm[0] : q == 1 ? b.norm[1] : b.norm[2]);
        const double av = is_mean ? (q == 0 ? a.mean[0] : q == 1 ? a.mean[1] : a.mean[2])
                                  : (q == 0 ? a.norm[0] : q == 1 ? a.norm[1] : a.norm[2]);
        const double wb = is_mean ? tm0 : tn0, wa = is_mean ? tm1 : tn1;
        const double v = wb * bv + wa * av / (wb + wa);
        double nmean[3], nnorm[3];
        for (int r = 0; r < 3; ++r) {
            nmean[r] = __shfl_sync(0xffffffffu, v, r);
            nnorm[r] = __shfl_sync(0xffffffffu, v, 3 + r);
        }
        const double w0 = tc0 * tc0, w1 = tc1 * tc1, den = (tc0 + tc1) * (tc0 + tc1);
        const double nc0 = (w0 * b.c0 + w1 * a.c0) / den;
        const double nc1 = lane < 4 ? (w0 * b.c1 + w1 * a.c1) / den : 0.0;
        if (-dot3(nmean, nnorm) < 0.0) {
            for (int r = 0; r < 3; ++r) nnorm[r] = -nnorm[r];
        }
        b.group = a.group;
        a.merged = 1;
        b.merged = 1;
        for (int r = 0; r < 3; ++r) { a.mean[r] = nmean[r]; a.norm[r] = nnorm[r]; b.mean[r] = nmean[r]; b.norm[r] = nnorm[r]; }
        a.c0 = nc0; a.c1 = nc1; b.c0 = nc0; b.c1 = nc1;
        sig = mix64(sig, wstate_emit(g, cur, b_rec, t, b, lane, overflow, round_tag));
        ++nout;
    }
    if (nout > 0) sig = mix64(sig, wstate_emit(g, cur, a_rec, t, a, lane, overflow, round_tag));
    return mix64(sig, (uint64_t)nout);
}

__device__ inline unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Thread 0 of CTA 0 notes the time (after a grid barrier: all CTAs passed it).
__device__ inline void mark(MergeCtl* c, int& k) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && k < kMaxMarks) {
        c->t_mark[k] = global_ns();
        c->n_marks = k + 1;
    }
    ++k;
}

// All rounds of the fixed point and the final write-back, one cooperative
// launch.
__global__ void __launch_bounds__(kMergeThreads, 3) k_merge_fixpoint(DMap m, MergeScratch g,
                                                                  const uint32_t* __restrict__ ev_list,
                                                                  const uint32_t* __restrict__ ev_rec,
                                                                  const int* d_n_ev) {
    MergeCtl* c = g.ctl;
    const int ne = *d_n_ev;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31, gw = tid >> 5, nw = nth >> 5;
    const uint64_t noop_sig = mix64(kSigNone, 0);
    int nm = 0;
    mark(c, nm);
    // the three logs still hold the previous batch's entries: unlink them
    int old_n[kLogs];
    for (int b = 0; b < kLogs; ++b) old_n[b] = min(c->n_ent[b], g.pool);
    const unsigned int epoch = (c->epoch + 1u) & 0xFFFFFFu;  // tags of this batch: (epoch << 8) | round
    grid_barrier(c);
    if (tid == 0) c->epoch = epoch;
    if (tid == 0) {
        for (int b = 0; b < kLogs; ++b) c->n_ent[b] = 0;
        c->overflow = 0;
        c->rounds = 0;
        for (int r = 0; r < kMaxRounds; ++r) { c->changed[r] = 0; c->n_queue[r] = 0; }
    }
    for (int b = 0; b < kLogs; ++b)
        for (int e = tid; e < old_n[b]; e += nth) g.head[b][g.ent[b][e].rec] = kNone;
    grid_barrier(c);
    mark(c, nm);

    int final_log = -1;
    for (int r = 0; r < kMaxRounds; ++r) {
        const int cur = r % kLogs, prev = (r + kLogs - 1) % kLogs, nxt = (r + 1) % kLogs;
        const bool first = r == 0;
        const MEntry* pent = g.ent[prev];
        const uint32_t* phead = first ? nullptr : g.head[prev];
        if (r >= 2) {  // the log the next round writes still holds round r - 2's entries
            const int nn = min(c->n_ent[nxt], g.pool);
            for (int e = tid; e < nn; e += nth) g.head[nxt][g.ent[nxt][e].rec] = kNone;
        }
        // one thread per call: does it merge anything?  A call that merged
        // nothing last time and none of whose records the last two logs
        // wrote sees the base states it saw then: the same no-op.
        const uint32_t cut = (epoch << 8) | (uint32_t)(r >= 2 ? r - 2 : 0);
        for (int e = tid; e < ne; e += nth) {
            const uint32_t t = ev_list[e];
            const uint32_t a_rec = ev_rec[t];
            uint32_t cl[6];
            if (!first && g.sig[e] == noop_sig) {
                bool dirty = g.rec_round[a_rec] >= cut && (g.rec_round[a_rec] >> 8) == epoch;
                for (int k = 0; k < 6 && !dirty; ++k) {
                    const uint32_t b = g.cand[(size_t)e * 6 + k];
                    if (b != kNone) dirty = g.rec_round[b] >= cut && (g.rec_round[b] >> 8) == epoch;
                }
                if (!dirty) continue;
            }
            if (first) {
                const unsigned long long T = m.cnt->batch_base + t;
                int64_t x, y, z;
                unpack_key(m.cold[a_rec].key, x, y, z);
                merge_candidates6(m, x, y, z, T, cl);
                for (int k = 0; k < 6; ++k) g.cand[(size_t)e * 6 + k] = cl[k];
            } else {
                for (int k = 0; k < 6; ++k) cl[k] = g.cand[(size_t)e * 6 + k];
            }
            if (call_merges(m, a_rec, t, cl, pent, phead)) {
                const int q = atomicAdd(&c->n_queue[r], 1);
                g.queue[q] = (uint32_t)e;
            } else {
                if (first || g.sig[e] != noop_sig) atomicAdd(&c->changed[r], 1);
                g.sig[e] = noop_sig;
            }
        }
        grid_barrier(c);
        mark(c, nm);
        if (tid == 0) c->n_ent[nxt] = 0;  // its unlinking above is done
        // one warp per call that merges: the whole call, lane-parallel
        const int nq = c->n_queue[r];
        bool ovf = false;
        for (int qi = gw; qi < nq; qi += nw) {
            const int e = (int)g.queue[qi];
            const uint32_t t = ev_list[e];
            const uint32_t a_rec = ev_rec[t];
            uint32_t cl[6];
            for (int k = 0; k < 6; ++k) cl[k] = g.cand[(size_t)e * 6 + k];
            const uint64_t sg = warp_merge_call(m, g, a_rec, t, cl, pent, phead, cur, ovf, (epoch << 8) | (uint32_t)r);
            if (lane == 0) {
                if (first || g.sig[e] != sg) atomicAdd(&c->changed[r], 1);
                g.sig[e] = sg;
            }
        }
        if (ovf && lane == 0) c->overflow = 1;
        grid_barrier(c);
        mark(c, nm);
        if (tid == 0) c->rounds = r + 1;
        if (c->wait_error || c->overflow) break;
        if (first && nq == 0) { final_log = cur; break; }  // no call merges anything
        if (!first && c->changed[r] == 0) { final_log = cur; break; }
    }
    if (final_log >= 0 && !c->wait_error) {
        const MEntry* fe = g.ent[final_log];
        const uint32_t* fh = g.head[final_log];
        const int nf = min(c->n_ent[final_log], g.pool);
        for (int e = tid; e < nf; e += nth) {
            const MEntry& en = fe[e];
            bool latest = true;
            for (uint32_t o = fh[en.rec]; o != kNone; o = fe[o].next)
                if (fe[o].t > en.t) { latest = false; break; }
            if (latest) write_state(m, en.rec, en.s);
        }
        if (tid == 0) c->converged = 1;
    }
    if (tid == 0 && c->wait_error) set_error(m.cnt, E_MERGE_WAIT);
    mark(c, nm);  // CTA 0's end of the write-back
}

cudaError_t merge_scratch_alloc(void** out, int max_batch, int rec_pool) {
    MergeScratch* ms = new MergeScratch();
    std::memset(ms, 0, sizeof(*ms));
    *out = ms;
    ms->pool = max_batch / 2 + 1024;
    ms->rec_pool = rec_pool;
    cudaError_t e;
    for (int b = 0; b < kLogs; ++b) {
        if ((e = dev_malloc(&ms->ent[b], sizeof(MEntry) * (size_t)ms->pool)) != cudaSuccess) return e;
        if ((e = dev_malloc(&ms->head[b], sizeof(uint32_t) * (size_t)rec_pool)) != cudaSuccess) return e;
        if ((e = cudaMemset(ms->head[b], 0xFF, sizeof(uint32_t) * (size_t)rec_pool)) != cudaSuccess) return e;
    }
    const size_t nb = (size_t)max_batch + 16;
    if ((e = dev_malloc(&ms->sig, sizeof(uint64_t) * nb)) != cudaSuccess) return e;
    if ((e = dev_malloc(&ms->cand, sizeof(uint32_t) * 6 * nb)) != cudaSuccess) return e;
    if ((e = dev_malloc(&ms->queue, sizeof(uint32_t) * nb)) != cudaSuccess) return e;
    if ((e = dev_malloc(&ms->rec_round, sizeof(uint32_t) * (size_t)rec_pool)) != cudaSuccess) return e;
    if ((e = cudaMemset(ms->rec_round, 0, sizeof(uint32_t) * (size_t)rec_pool)) != cudaSuccess) return e;
    if ((e = dev_malloc(&ms->ctl, sizeof(MergeCtl))) != cudaSuccess) return e;
    if ((e = cudaMemset(ms->ctl, 0, sizeof(MergeCtl))) != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_merge_fixpoint, kMergeThreads, 0)) != cudaSuccess)
        return e;
    ms->coop_capacity = sms * per_sm;
    ms->sms = sms;
    return cudaSuccess;
}
void merge_scratch_free(void* p) {
    MergeScratch* ms = (MergeScratch*)p;
    if (!ms) return;
    for (int b = 0; b < kLogs; ++b) { cudaFree(ms->ent[b]); cudaFree(ms->head[b]); }
    cudaFree(ms->sig);
    cudaFree(ms->cand);
    cudaFree(ms->queue);
    cudaFree(ms->rec_round);
    cudaFree(ms->ctl);
    delete ms;
}

constexpr int kMaxCoopSlots = 64;
static std::mutex g_coop_mu;
static std::vector<cudaEvent_t> g_coop_done;  // completion of the last launches, one per slot
static unsigned long long g_coop_next = 0;
static int g_coop_slots = 1;
static bool g_coop_throughput = false;
static int g_coop_throughput_refs = 0;
static int g_coop_divisor = 16;

void merge_set_grid_divisor(int d) {
    std::lock_guard<std::mutex> lk(g_coop_mu);
    g_coop_divisor = d < 1 ? 1 : (d > 1024 ? 1024 : d);
}

bool merge_throughput_mode() {
    std::lock_guard<std::mutex> lk(g_coop_mu);
    return g_coop_throughput;
}

void merge_set_throughput_mode(bool on) {
    std::lock_guard<std::mutex> lk(g_coop_mu);
    g_coop_throughput_refs += on ? 1 : -1;
    if (g_coop_throughput_refs < 0) g_coop_throughput_refs = 0;
    g_coop_throughput = g_coop_throughput_refs > 0;
}

// The merge calls of one batch: the cooperative fixed point, then the replay
// if it did not settle (the replay kernel returns at once when it did).
// Nothing waits on the host.
cudaError_t run_merge_events(DMap& m, MapScratch& ms, void* scratch, int n_max, int mode, int* rounds_out,
                             cudaStream_t st) {
    (void)n_max;
    MergeScratch& g = *(MergeScratch*)scratch;
    if (rounds_out) *rounds_out = -1;
    if (mode == 1) {  // sequential replay only
        VMP_NOTE_LAUNCH(); k_merge_sequential<<<1, 32, 0, st>>>(m, ms.ev_list, ms.ev_rec, ms.d_n_ev, nullptr);
        return cudaGetLastError();
    }
    cudaError_t e;
    // converged = 0; wait_error, pad, bar_count = 0 (bar_gen keeps counting)
    if ((e = cudaMemsetAsync(&g.ctl->converged, 0, sizeof(int) * 3 + sizeof(unsigned int), st)) != cudaSuccess) return e;
    if (g.coop_capacity > 0) {
        // Launch sizing (process-wide): alone, one launch at a time on the
        // whole device; once a server runs many streams, SMs / divisor CTAs
        // per launch (a batch's merge calls are few: small grids spend less
        // on grid barriers and leave the device to the other streams; the
        // server's autotuner picks the divisor, 16 by default) and at most capacity / grid
        // launches (<= 64) on the device at once (launch i waits for launch
        // i - slots; on a switch, for all earlier ones).  Their CTAs then
        // always fit co-resident, so no launch can wait for CTAs that the
        // others hold while they wait.
        std::lock_guard<std::mutex> lk(g_coop_mu);
        if (g_coop_done.empty()) {
            g_coop_done.assign(kMaxCoopSlots, nullptr);
            for (auto& ev : g_coop_done)
                if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
                    cudaGetLastError();
                    ev = nullptr;
                }
        }
        int grid = g.coop_capacity, slots = 1;
        if (g_coop_throughput) {
            grid = g.sms / g_coop_divisor > 0 ? g.sms / g_coop_divisor : 1;
            if (grid > g.coop_capacity) grid = g.coop_capacity;
            slots = g.coop_capacity / grid;
            if (slots < 1) slots = 1;
            if (slots > kMaxCoopSlots) slots = kMaxCoopSlots;
        }
        if (slots != g_coop_slots) {
            for (auto ev : g_coop_done)
                if (ev) cudaStreamWaitEvent(st, ev, 0);
            g_coop_slots = slots;
            g_coop_next = 0;
        } else {
            cudaEvent_t prev = g_coop_done[g_coop_next % slots];
            if (prev) cudaStreamWaitEvent(st, prev, 0);
        }
        cudaEvent_t mine = g_coop_done[g_coop_next % slots];
        ++g_coop_next;
        void* args[] = {(void*)&m, (void*)&g, (void*)&ms.ev_list, (void*)&ms.ev_rec, (void*)&ms.d_n_ev};
        VMP_NOTE_LAUNCH();
        e = cudaLaunchCooperativeKernel((const void*)k_merge_fixpoint, dim3(grid), dim3(kMergeThreads), args, 0, st);
        if (e != cudaSuccess) cudaGetLastError();  // the replay below produces the result
        if (mine) cudaEventRecord(mine, st);
    }
    VMP_NOTE_LAUNCH(); k_merge_sequential<<<1, 32, 0, st>>>(m, ms.ev_list, ms.ev_rec, ms.d_n_ev, g.ctl);
    return cudaGetLastError();
}

// Phase times of the last batch's fixed point (us): setup, then per round
// the call tests and the merging calls, then CTA 0's write-back; returns how
// many (0 when no fixed point ran).  Waits for the stream.
int merge_profile_read(void* scratch, cudaStream_t st, double* us, int max) {
    MergeScratch& g = *(MergeScratch*)scratch;
    MergeCtl h;
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    if (cudaMemcpy(&h, g.ctl, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    if (!h.converged) return 0;
    int n = 0;
    for (int k = 1; k < h.n_marks && k < kMaxMarks && n < max; ++k)
        us[n++] = (double)(h.t_mark[k] - h.t_mark[k - 1]) * 1e-3;
    return n;
}

// Rounds the last batch's fixed point ran (0 when the replay ran alone);
// waits for the stream.
int merge_rounds_read(void* scratch, cudaStream_t st) {
    MergeScratch& g = *(MergeScratch*)scratch;
    MergeCtl h;
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    if (cudaMemcpy(&h, g.ctl, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return h.converged ? h.rounds : 0;
}

}  // namespace vmp

// ------------------------------------------------------------ test hook
// The barrier's failure path without a fault: with skip set, CTA 1 returns
// without arriving, so CTA 0's wait runs out after spin_limit polls, records
// wait_error and returns; without skip both arrive (cooperative launch, so
// both CTAs are resident).  The kernel always ends.
namespace vmp {
namespace {
__global__ void k_barrier_probe(MergeCtl* c, int skip, long long spin_limit) {
    if (skip && blockIdx.x == 1) return;
    grid_barrier(c, spin_limit);
}
}  // namespace
}  // namespace vmp

extern "C" vmp_status vmp_test_barrier_timeout(int skip, long long spin_limit, int* timed_out, double* ms) {
    using namespace vmp;
    if (!timed_out || spin_limit < 1) return VMP_ERR_INVALID_ARG;
    MergeCtl* c = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaMalloc((void**)&c, sizeof(MergeCtl));
    if (e == cudaSuccess) e = cudaMemset(c, 0, sizeof(MergeCtl));
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    if (e == cudaSuccess) e = cudaEventRecord(a, 0);
    if (e == cudaSuccess) {
        void* args[] = {(void*)&c, (void*)&skip, (void*)&spin_limit};
        e = cudaLaunchCooperativeKernel((const void*)k_barrier_probe, dim3(2), dim3(32), args, 0, 0);
    }
    if (e == cudaSuccess) e = cudaEventRecord(b, 0);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    MergeCtl h{};
    if (e == cudaSuccess) e = cudaMemcpy(&h, c, sizeof(MergeCtl), cudaMemcpyDeviceToHost);
    float t = 0.f;
    if (e == cudaSuccess && ms) {
        cudaEventElapsedTime(&t, a, b);
        *ms = t;
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (c) cudaFree(c);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return VMP_ERR_CUDA;
    }
    *timed_out = h.wait_error;
    return VMP_OK;
}
