// Device-resident voxel plane map: VoxelMap::build / update with LRU
// (voxel_map.cpp:200-256), VoxelGrid::pushPoint / addPoint / updatePlane
// (voxel_map.cpp:29-136).
//
// One batch of N world points (in order) is applied as:
//   1. key + hash lookup / CAS insert per point; a new key's slot records the
//      smallest point index that reached it (atomicMin) = its creating point;
//   2. creating points are ranked by a prefix sum: rank = creation order, so
//      VoxelGrid::count (group_id) is assigned exactly as the sequential
//      loop would;
//   3. points are stably sorted by record -> one segment per touched voxel,
//      each in point order;
//   4. a warp per segment runs the pushPoint state machine in point order
//      (lane 0 carries the incremental mean / ppt; refits use all lanes: the
//      per-point J * cov * J^T terms are computed 32 at a time and each of the
//      36 plane-cov entries is summed by one lane in point order, so the sum
//      is the reference's sequential sum);
//   5. points that reach a frozen plane voxel become merge events, resolved in
//      point order in k_merge.cu (merges only read and write frozen voxels,
//      which no other step changes);
//   6. LRU: each touched voxel's stamp = global index of its last touching
//      point; evictions take the least recent untouched voxels in creation
//      order.
#include <mutex>
#include <vector>
#include "kernels.cuh"

namespace vmp {

constexpr int kMapThreads = 256;
constexpr int kSegThreads = 128;  // 4 warps: 4 x 32 x 36 doubles of refit staging

static int grid_for_map(int n) {
    int b = (n + kMapThreads - 1) / kMapThreads;
    if (b > 152 * 8) b = 152 * 8;
    return b < 1 ? 1 : served_grid(b);
}

// Blocks of k_seg_chain and k_seg_cov that take work.  The launches keep
// their full grids (the scan graphs hold them); blocks from this index on
// return at once.  Their warps take segments from a counter, so the number of
// working blocks changes only how many voxel chains run at once, never the
// results.  A server lowers it: a latency-bound chain of one stream then
// holds fewer SM slots that other streams' kernels could issue from.
__device__ int g_seg_blocks = 1 << 30;
static std::mutex g_seg_mu;
static int g_seg_blocks_host = 0;  // 0: every block works

cudaError_t seg_set_grid_blocks(int blocks) {
    std::lock_guard<std::mutex> lk(g_seg_mu);
    static cudaStream_t st = nullptr;
    cudaError_t e = cudaSuccess;
    if (!st && (e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) return e;
    const int v = blocks > 0 ? blocks : (1 << 30);
    e = cudaMemcpyToSymbolAsync(g_seg_blocks, &v, sizeof(int), 0, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) g_seg_blocks_host = blocks > 0 ? blocks : 0;
    return e;
}
int seg_grid_blocks() {
    std::lock_guard<std::mutex> lk(g_seg_mu);
    return g_seg_blocks_host;
}

// (k, RN(1 / k)) for k = 1 .. kRecipTable - 1 (the running mean's divisors
// n + 1), written once per device from the host's correctly rounded divisions.
constexpr int kRecipTable = 4096;
__device__ double2 g_div[kRecipTable];

cudaError_t map_recip_table_init() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(mu);
    if (done[dev]) return cudaSuccess;
    std::vector<double2> t(kRecipTable, make_double2(0.0, 0.0));
    for (int k = 1; k < kRecipTable; ++k) t[k] = make_double2((double)k, 1.0 / (double)k);
    e = cudaMemcpyToSymbol(g_div, t.data(), sizeof(double2) * kRecipTable);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

// ---------------------------------------------------------------- lookup / insert
__global__ void k_lookup_insert(DMap m, const double* __restrict__ bpts, const int* d_n, uint32_t* slot_out,
                                unsigned long long* keys_out) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double p[3] = {bpts[i * 3], bpts[i * 3 + 1], bpts[i * 3 + 2]};
        int64_t k[3];
        if (!voxel_index(p, m.voxel_size, m.voxel_inv, k)) {
            set_error(m.cnt, E_KEY_RANGE);
            slot_out[i] = kNoRec;
            continue;
        }
        uint64_t key = pack_key(k[0], k[1], k[2]);
        if (keys_out) keys_out[i] = key;
        uint64_t h = hash_key(key) & m.table_mask;
        bool placed = false;
        for (uint64_t probe = 0; probe <= m.table_mask; ++probe) {
            uint64_t cur = *((volatile unsigned long long*)&m.keys[h]);
            if (cur == key) { placed = true; break; }
            if (cur == kEmptyKey) {
                unsigned long long prev = atomicCAS((unsigned long long*)&m.keys[h], (unsigned long long)kEmptyKey,
                                                    (unsigned long long)key);
                if (prev == kEmptyKey || prev == key) { placed = true; break; }
            }
            h = (h + 1) & m.table_mask;
        }
        if (!placed) {
            set_error(m.cnt, E_HASH_FULL);
            slot_out[i] = kNoRec;
            continue;
        }
        uint32_t v = *((volatile uint32_t*)&m.vals[h]);
        if (v >= kPending) atomicMin(&m.vals[h], kPending | (uint32_t)i);
        slot_out[i] = (uint32_t)h;
    }
}

__global__ void k_creator_flags(DMap m, const uint32_t* __restrict__ slot, const int* d_n, uint32_t* flag) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t s = slot[i];
        flag[i] = (s != kNoRec && m.vals[s] == (kPending | (uint32_t)i)) ? 1u : 0u;
    }
}

__global__ void k_assign(DMap m, const uint32_t* __restrict__ slot, const uint32_t* __restrict__ flag,
                         const uint32_t* __restrict__ rank, const int* d_n, uint32_t* new_pos) {
    const int n = *d_n;
    const int top = m.cnt->rec_free_top;
    const long long gbase = m.cnt->group_counter;
    const unsigned long long base = m.cnt->batch_base;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!flag[i]) continue;
        uint32_t r = rank[i];
        uint32_t s = slot[i];
        if ((int)r >= top) {
            set_error(m.cnt, E_RECORDS);
            m.vals[s] = kNoRec;
            continue;
        }
        uint32_t rec = m.rec_free[top - 1 - (int)r];
        RecHot& h = m.hot[rec];
        for (int a = 0; a < 3; ++a) { h.mean[a] = 0.0; h.norm[a] = 0.0; }
        h.flags = F_UPDATE | F_ALIVE;
        h.n = 0;
        h.group = (uint64_t)(gbase + (long long)r);
        RecCold& c = m.cold[rec];
        for (int a = 0; a < 9; ++a) c.ppt[a] = 0.0;
        for (int a = 0; a < 36; ++a) c.cov[a] = 0.0;
        for (int a = 0; a < 3; ++a) c.center[a] = 0.0;
        c.key = m.keys[s];
        c.stamp = base + (unsigned long long)i;
        c.create_g = base + (unsigned long long)i;
        c.freeze_g = kNever;
        c.evict_g = kNever;
        c.touch_first_g = kNever;
        c.newly = 0;
        c.nslab = 0;
        for (int a = 0; a < kMaxChunks; ++a) c.chunks[a] = -1;
        new_pos[r] = (uint32_t)i;
        __threadfence();
        m.vals[s] = rec;
    }
}

__global__ void k_assign_counters(DMap m, const int* d_n_new) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int nn = *d_n_new;
        Counters* c = m.cnt;
        int take = nn <= c->rec_free_top ? nn : c->rec_free_top;
        c->rec_free_top -= take;
        c->group_counter += nn;
        c->size += take;
        c->n_new = nn;
        c->n_evict = 0;
        c->split_at = -1;
    }
}

__global__ void k_resolve(DMap m, const uint32_t* __restrict__ slot, const int* d_n, uint32_t* rec,
                          uint32_t* sk, uint32_t* sv) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t s = slot[i];
        uint32_t r = (s == kNoRec) ? kNoRec : m.vals[s];
        if (r >= kPending) r = kNoRec;
        rec[i] = r;
        sk[i] = r;
        sv[i] = (uint32_t)i;
    }
}

__global__ void k_seg_heads(const uint32_t* __restrict__ sk, const int* d_n, uint32_t* flag) {
    const int n = *d_n;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        flag[j] = (sk[j] != kNoRec && (j == 0 || sk[j] != sk[j - 1])) ? 1u : 0u;
}

// Segment bounds + LRU bookkeeping of the touched records.
__global__ void k_seg_bounds(DMap m, const uint32_t* __restrict__ sk, const uint32_t* __restrict__ sv,
                             const uint32_t* __restrict__ flag, const uint32_t* __restrict__ rank, const int* d_n,
                             uint32_t* seg_start, uint32_t* seg_end, uint32_t* seg_rec, uint32_t* last_touch) {
    const int n = *d_n;
    const unsigned long long base = m.cnt->batch_base;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        uint32_t r = sk[j];
        if (r == kNoRec) continue;
        uint32_t s = rank[j];  // segment index (exclusive scan of heads; valid for non-head too: rank of next head)
        if (flag[j]) {
            seg_start[s] = (uint32_t)j;
            seg_rec[s] = r;
            m.cold[r].touch_first_g = base + sv[j];
        }
        bool tail = (j == n - 1) || sk[j + 1] != r;
        if (tail) {
            uint32_t seg = flag[j] ? s : s - 1;
            seg_end[seg] = (uint32_t)(j + 1);
            last_touch[sv[j]] = 1u;
        }
    }
}

__global__ void k_fill_u32(uint32_t* p, const int* d_n, uint32_t v) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

// ---------------------------------------------------------------- eviction
// Walk over the creations of this batch that overflow the capacity (exact
// LRU semantics): the victim of a creation at point c is the
// least recently used voxel that no point before c touched in this batch.
// A victim that a later point of the batch touches would be re-created by the
// reference; the walk then reports the first such point (split_at) and the
// host applies the batch in two parts.
// The walk is a scan, 1024 queue entries per step in one CTA: an entry is
// stale (its voxel dead or touched again since), live and untouched in this
// batch, or live and touched in this batch.  Before the first split every
// victim is a live untouched entry, so the creation an entry meets is j0 plus
// the count of live untouched entries before it (a block prefix sum); a
// touched entry is skipped if its first touch precedes that creation and is
// the split point otherwise.  The assignments equal the one-entry-at-a-time
// walk's.
constexpr int kWalkThreads = 1024;
__global__ void __launch_bounds__(kWalkThreads) k_evict_walk(DMap m, const uint32_t* __restrict__ new_pos,
                                                              uint32_t* victims, const int* d_n) {
    __shared__ int s_wsum[kWalkThreads / 32];
    __shared__ int s_split_t, s_last_t;
    Counters* c = m.cnt;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const unsigned long long base = c->batch_base;
    const unsigned long long batch_end = base + (unsigned long long)*d_n;
    const int n_new = c->n_new;
    const long long size_before = c->size - n_new;
    const unsigned long long q_head = c->q_head, q_tail = c->q_tail;
    __syncthreads();  // every thread has read the counters before they change
    if (t == 0) {
        c->n_evict = 0;
        c->split_at = -1;
    }
    long long j0 = m.capacity - size_before;  // creations j >= j0 evict
    if (j0 < 0) j0 = 0;
    if (j0 >= n_new) return;  // uniform
    const int need = (int)(n_new - j0);
    unsigned long long q0 = q_head;
    int assigned = 0;  // victims assigned before q0
    int ne = -1;       // victims of the batch once known
    unsigned long long q_end = q_tail;
    for (;;) {
        const unsigned long long qi = q0 + (unsigned long long)t;
        int kind = 0;  // 0 stale or past the tail, 1 live untouched, 2 live touched in this batch
        uint32_t r = 0;
        uint64_t tf = kNever;
        if (qi < q_tail) {
            r = m.q_rec[qi % m.q_cap];
            const uint64_t st = m.q_stamp[qi % m.q_cap];
            if ((m.hot[r].flags & F_ALIVE) && m.cold[r].stamp == st) {
                tf = m.cold[r].touch_first_g;
                // a stamp past this batch's points is left by the rolled-back
                // first pass of a batch that was split: not a touch of this batch
                kind = (tf != kNever && tf >= base && tf < batch_end) ? 2 : 1;
            }
        }
        // exclusive prefix count of live untouched entries over the block
        const int f = kind == 1 ? 1 : 0;
        int inc = f;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) s_wsum[w] = inc;
        if (t == 0) {
            s_split_t = kWalkThreads;
            s_last_t = -1;
        }
        __syncthreads();
        if (w == 0) {
            int x = s_wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += v;
            }
            s_wsum[lane] = x;  // inclusive over warps
        }
        __syncthreads();
        const int total = s_wsum[kWalkThreads / 32 - 1];
        const int a = assigned + (w > 0 ? s_wsum[w - 1] : 0) + inc - f;  // creation offset this entry meets
        if (kind == 2 && a < need && tf >= base + new_pos[j0 + a]) atomicMin(&s_split_t, t);
        __syncthreads();
        const int ts = s_split_t;
        if (kind == 1 && t < ts && a < need) {
            victims[a] = r;
            if (a == need - 1) s_last_t = t;
        }
        __syncthreads();
        if (ts < kWalkThreads) {  // re-created later by the reference: split the batch here
            if (t == ts) c->split_at = (int)(tf - base);
            return;
        }
        if (s_last_t >= 0) {  // every creation has its victim
            ne = need;
            q_end = q0 + (unsigned long long)s_last_t + 1ull;
            break;
        }
        assigned += total;
        q0 += kWalkThreads;
        if (q0 >= q_tail) {  // the queue ran out before every creation had a victim
            if (t == 0) set_error(c, E_CAPACITY);
            ne = assigned;
            q_end = q_tail;
            break;
        }
        __syncthreads();  // s_wsum and the flags are reused by the next step
    }
    __syncthreads();  // the victims written above are visible to the block
    for (int v = t; v < ne; v += kWalkThreads) m.cold[victims[v]].evict_g = base + new_pos[j0 + v];
    if (t == 0) {
        c->q_head = q_end;
        c->n_evict = ne;
    }
}

// Undoes the creations of an aborted batch (the batch is split and re-applied).
__global__ void k_rollback(DMap m, const uint32_t* __restrict__ slot, const uint32_t* __restrict__ flag,
                           const int* d_n) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!flag[i]) continue;
        uint32_t s = slot[i];
        uint32_t r = m.vals[s];
        m.keys[s] = kTombKey;
        m.vals[s] = 0xFFFFFFFFu;
        if (r < kPending) m.hot[r].flags = 0;
    }
}
__global__ void k_rollback_counters(DMap m) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Counters* c = m.cnt;
    c->rec_free_top += c->n_new;
    c->group_counter -= c->n_new;
    c->size -= c->n_new;
    c->n_tomb += c->n_new;
    c->n_new = 0;
}

// ---------------------------------------------------------------- segments
__device__ inline double* slab_pt(const DMap& m, const int* chunks, int j) {
    return m.slab + ((size_t)chunks[j / kChunkPts] * kChunkPts + (j % kChunkPts)) * kSlabStride;
}

// Per-refit factors of VoxelGrid::updatePlane's J (voxel_map.cpp:115-130):
// J = [evecs * F; I / n], F row m = ((p - mean) / (n (l0 - lm)))^T (vm pn^T + pn vm^T).
struct RefitConst {
    double mean[3];
    double evecs[9];
    double M1[9], M2[9];
    double den1, den2, inv_n;
    double rden1, rden2;  // RN(1 / den1), RN(1 / den2)
    bool recip_ok;        // both divisors in the range where div_by_recip is exact
};
__device__ inline void refit_const(const double* mean, int n, const double* ev, const double* evecs, RefitConst& k) {
    const double pn[3] = {evecs[0], evecs[3], evecs[6]};
    for (int q = 0; q < 3; ++q) k.mean[q] = mean[q];
    for (int q = 0; q < 9; ++q) k.evecs[q] = evecs[q];
    for (int m = 1; m < 3; ++m) {
        const double vm[3] = {evecs[m], evecs[3 + m], evecs[6 + m]};
        double* M = m == 1 ? k.M1 : k.M2;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) M[i * 3 + j] = vm[i] * pn[j] + pn[i] * vm[j];
    }
    k.den1 = (double)n * (ev[0] - ev[1]);
    k.den2 = (double)n * (ev[0] - ev[2]);
    k.inv_n = 1.0 / (double)n;
    k.recip_ok = div_recip_ok(k.den1) && div_recip_ok(k.den2);
    k.rden1 = k.recip_ok ? 1.0 / k.den1 : 0.0;
    k.rden2 = k.recip_ok ? 1.0 / k.den2 : 0.0;
}

// J cov J^T is symmetric: its 21 upper-triangle entries (row-major over the
// 6x6, i <= j) are formed per point and mirrored when the voxel's covariance
// is written back, as the oracle does.
constexpr int kCovTerms = 21;
__device__ __constant__ unsigned char kUpper[kCovTerms] = {0,  1,  2,  3,  4,  5,  7,  8,  9,  10, 11,
                                                           14, 15, 16, 17, 21, 22, 23, 28, 29, 35};

// Per-point term of J * cov * J^T (its upper triangle), without the products
// with J's known zeros (row 0 of F, the off-diagonal of I / n): the same sums
// without their +-0 terms, as the oracle forms them.
__device__ inline void plane_cov_term(const double* p, const double* cov, const RefitConst& k, double* out21) {
    const double d[3] = {p[0] - k.mean[0], p[1] - k.mean[1], p[2] - k.mean[2]};
    double F1[3], F2[3];
    {
        // d / den, correctly rounded (the reference's division)
        double a[3], b[3];
        if (k.recip_ok) {
            for (int c = 0; c < 3; ++c) {
                a[c] = div_by_recip(d[c], k.den1, k.rden1);
                b[c] = div_by_recip(d[c], k.den2, k.rden2);
            }
        } else {
            for (int c = 0; c < 3; ++c) {
                a[c] = d[c] / k.den1;
                b[c] = d[c] / k.den2;
            }
        }
        for (int j = 0; j < 3; ++j) {
            F1[j] = (a[0] * k.M1[j] + a[1] * k.M1[3 + j]) + a[2] * k.M1[6 + j];
            F2[j] = (b[0] * k.M2[j] + b[1] * k.M2[3 + j]) + b[2] * k.M2[6 + j];
        }
    }
    double top[9], A[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) top[i * 3 + j] = k.evecs[i * 3 + 1] * F1[j] + k.evecs[i * 3 + 2] * F2[j];
    mm<3, 3, 3>(top, cov, A);
    int q = 0;
    for (int i = 0; i < 3; ++i)  // rows 0-2: (i, j >= i) then (i, 3 + j)
        for (int j = i; j < 3; ++j)
            out21[q++] = (A[i * 3] * top[j * 3] + A[i * 3 + 1] * top[j * 3 + 1]) + A[i * 3 + 2] * top[j * 3 + 2];
    // q == 6; the order below follows kUpper: row i's (i, 3 + j) entries come
    // after row i's (i, j <= 2) entries in row-major order
    double tr[9], br[6];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) tr[i * 3 + j] = A[i * 3 + j] * k.inv_n;
    int u = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) br[u++] = (k.inv_n * cov[i * 3 + j]) * k.inv_n;
    // assemble in kUpper order: row 0: (0,0..2) tl, (0,3..5) tr; row 1: (1,1..2) tl,
    // (1,3..5) tr; row 2: (2,2) tl, (2,3..5) tr; rows 3-5: br
    const double tl[6] = {out21[0], out21[1], out21[2], out21[3], out21[4], out21[5]};
    out21[0] = tl[0]; out21[1] = tl[1]; out21[2] = tl[2];
    out21[3] = tr[0]; out21[4] = tr[1]; out21[5] = tr[2];
    out21[6] = tl[3]; out21[7] = tl[4];
    out21[8] = tr[3]; out21[9] = tr[4]; out21[10] = tr[5];
    out21[11] = tl[5];
    out21[12] = tr[6]; out21[13] = tr[7]; out21[14] = tr[8];
    for (int v = 0; v < 6; ++v) out21[15 + v] = br[v];
}

// ---------------------------------------------------------------- voxel state machine
// VoxelGrid::pushPoint / addPoint / updatePlane (voxel_map.cpp:29-136) for
// every touched voxel of a batch, in three kernels:
//   k_seg_chain  three voxels per warp, ten lanes each: the points in order
//                -- addToPlane with the three coordinates of the mean and the
//                six distinct entries of ppt on separate lanes, slab
//                appends, the integer state machine --
//                recording a snapshot (n, mean, ppt, slab length) at every
//                updatePlane call that reaches the eigen decomposition;
//   k_refit_eig  one thread per snapshot: the 3x3 eigen decomposition and the
//                plane test, all refits of the batch at once;
//   k_seg_cov    one warp per voxel with snapshots: the plane covariance
//                terms of each plane refit (lanes over points) summed in
//                point order onto the voxel's cov, the normal and centre of
//                the last plane refit, and the merge calls of the points that
//                reached the voxel after it froze.
// Nothing in the state machine reads a refit's plane decision before the
// voxel freezes (the branches test is_init and update_enable only, and
// is_init follows from the count), so splitting the refits out keeps the
// reference's sequence exactly.
struct RefitSnap {
    int n;           // point count at the refit
    int npts;        // points the covariance terms run over
    int from_batch;  // build: the batch segment's points, else the slab prefix
    int plane;       // eigen test result
    int seg;         // segment index
    int toff;        // first of its npts covariance terms in the term buffer (-1: computed in k_seg_cov)
    double mean[3];
    double ppt[9];
    double ev[3];
    double evecs[9];
    double M1[9], M2[9];  // RefitConst of a plane refit
    double den1, den2, inv_n;
    double rden1, rden2;  // RN(1 / den): the divisions of the terms by the reciprocal (div_by_recip)
    int recip_ok;
    int pad2;
};
struct CovSeg {
    uint32_t seg;
    int nref;    // snapshots at seg_start[seg] .. + nref
    int mstart;  // first point index of the merge calls (seg_end: none)
    int pad;
    int32_t chunks[kMaxChunks];  // the slab before a freeze released it
};

__device__ inline void slab_release(const DMap& m, int* chunks, int& nslab) {
    int used = (nslab + kChunkPts - 1) / kChunkPts;
    for (int k = 0; k < used && k < kMaxChunks; ++k) {
        if (chunks[k] >= 0) {
            int pos = atomicAdd(&m.cnt->chunk_freed_top, 1);
            if (pos < m.chunk_pool) m.chunk_freed[pos] = chunks[k];
        }
        chunks[k] = -1;
    }
    nslab = 0;
}

struct SegScratch {
    RefitSnap* snaps;     // [max_batch], indexed like the sorted batch
    uint32_t* refit_list; // [max_batch] snapshot indices
    CovSeg* covsegs;      // [max_batch]
    int* seg_cov;         // [max_batch] covseg index of a segment with snapshots
    uint32_t* term_snap;  // [term_cap] snapshot of each covariance term (kNoRec: unused slot)
    double* terms;        // [term_cap][21] upper triangles
    int term_cap;
    int snap_cap;         // snapshots (max_batch + 16)
    int* d_n_refit;
    int* d_n_covseg;
    int* d_n_terms;
    int* d_work_chain;  // next segment group for k_seg_chain
    int* d_work_cov;    // next voxel-with-refits for k_seg_cov
};

// Three voxel chains per warp, ten lanes each: the nine ppt components on
// lanes 0-8 of a group (the three mean components on lanes 0-2), the integer
// state on every lane of the group.  A chain's steps stay lane-parallel (its
// latency as with a whole warp), and every FP64 instruction serves three
// voxels.  Collective steps (chunk allocation, the loop test) run on the
// whole warp with per-group predicates.
constexpr int kGroupLanes = 10;
// Lane 3 + e of a chain holds the distinct ppt entry e = (i, j), i <= j:
// i, j, i * 3 + j and j * 3 + i as 4-bit fields e of these constants.
constexpr unsigned kPptI = 0x211000u, kPptJ = 0x221210u, kPptIdx = 0x854210u, kPptMir = 0x874630u;
__device__ __forceinline__ int ppt_field(unsigned packed, int e) { return (int)((packed >> (4 * e)) & 15u); }
constexpr int kGroups = 3;

// Slab append for the groups with `app` (all lanes call it).  c0 / c1: this
// lane's covariance entries (lanes 3-9: entry q - 3; lanes 0-1: entry 7 + q).
__device__ inline void group_slab_append(const DMap& m, bool app, int* chunks, int& nslab, const double* p,
                                         double c0, double c1, int q, int gbase) {
    const int ci = nslab / kChunkPts;
    const bool fits = app && ci < kMaxChunks;
    const bool need = fits && (nslab % kChunkPts == 0);
    int got = 1;
    if (need && q == 0) {
        const int top = atomicSub(&m.cnt->chunk_free_top, 1);
        if (top <= 0) {
            atomicAdd(&m.cnt->chunk_free_top, 1);
            set_error(m.cnt, E_CHUNKS);
            got = 0;
        } else {
            chunks[ci] = m.chunk_free[top - 1];
        }
    }
    got = __shfl_sync(0xffffffffu, got, gbase);
    __syncwarp();
    if (fits && (!need || got)) {
        double* d = slab_pt(m, chunks, nslab);
        if (q < 3) d[q] = p[q];
        else d[q] = c0;  // covariance entries 0-6 on lanes 3-9
        if (q < 2) d[10 + q] = c1;
        nslab++;
    }
}

__global__ void __launch_bounds__(kSegThreads) k_seg_chain(DMap m, const uint32_t* __restrict__ seg_start,
                                                           const uint32_t* __restrict__ seg_end,
                                                           const uint32_t* __restrict__ seg_rec, const int* d_n_seg,
                                                           const uint32_t* __restrict__ sv,
                                                           const double* __restrict__ bpts,
                                                           const double* __restrict__ bcov, uint32_t* ev_rec,
                                                           SegScratch ss, int build) {
    __shared__ int s_chunks[kSegThreads / 32][kGroups][kMaxChunks];
    __shared__ int s_saved[kSegThreads / 32][kGroups][kMaxChunks];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int g = lane / kGroupLanes, q = lane - g * kGroupLanes;  // lanes 30, 31: g == kGroups, idle
    const int gi = g < kGroups ? g : 0;
    const int gbase = gi * kGroupLanes;
    const unsigned gmask = ((1u << kGroupLanes) - 1u) << gbase;
    const int pe = q >= 3 && q < 9 ? q - 3 : 0;
    const int p_i = ppt_field(kPptI, pe), p_j = ppt_field(kPptJ, pe);
    const int p_idx = ppt_field(kPptIdx, pe), p_mir = ppt_field(kPptMir, pe);
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    if ((int)blockIdx.x >= g_seg_blocks) return;  // uniform per block
    const int nseg = *d_n_seg;
    const unsigned long long base = m.cnt->batch_base;
    int* chunks = s_chunks[wib][gi];
    int* saved = s_saved[wib][gi];
    // segment groups are taken from a counter: a warp that finishes early
    // takes the next group instead of idling in its block
    (void)gw;
    (void)nw;
    for (;;) {
        int s0 = 0;
        if (lane == 0) s0 = atomicAdd(ss.d_work_chain, kGroups);
        s0 = __shfl_sync(0xffffffffu, s0, 0);
        if (s0 >= nseg) break;
        const int sidx = s0 + g;
        const bool mine = g < kGroups && sidx < nseg;
        uint32_t rec = 0, flags = 0;
        int b = 0, e = 0, n = 0, newly = 0, nslab = 0;
        double mean_l = 0.0, ppt_l = 0.0;
        if (mine) {
            rec = seg_rec[sidx];
            b = (int)seg_start[sidx];
            e = (int)seg_end[sidx];
            const RecHot& H = m.hot[rec];
            const RecCold& Cc = m.cold[rec];
            flags = H.flags;
            n = H.n;
            newly = Cc.newly;
            nslab = Cc.nslab;
            if (q < 3) mean_l = H.mean[q];
            if (q >= 3 && q < 9) ppt_l = Cc.ppt[p_idx];
            for (int k = q; k < kMaxChunks; k += kGroupLanes) chunks[k] = Cc.chunks[k];
        }
        __syncwarp();
        int nref = 0, mstart = e;
        bool have_saved = false, done = !mine;
        // updatePlane call (group-uniform): a snapshot when it reaches the eigen decomposition
        auto refit = [&](int npts, int from_batch) {
            if (n < m.update_thresh) return;
            flags |= F_INIT;
            RefitSnap& sn = ss.snaps[b + nref];
            if (q < 3) sn.mean[q] = mean_l;
            if (q >= 3 && q < 9) {  // ppt is symmetric: entry and mirror
                sn.ppt[p_idx] = ppt_l;
                sn.ppt[p_mir] = ppt_l;
            }
            if (q == 0) {
                sn.n = n;
                sn.npts = npts;
                sn.from_batch = from_batch;
                sn.seg = sidx;
                const int k = atomicAdd(ss.d_n_refit, 1);
                ss.refit_list[k] = (uint32_t)(b + nref);
            }
            ++nref;
        };
        auto add_point = [&](const double* p) {
            // addToPlane: lanes 0-2 mean += (p - mean) / (n + 1), the division
            // through the tabled RN(1 / (n + 1)) with Markstein's correction;
            // lanes 3-8 the six distinct entries of ppt += p p^T (p_i - 0 is
            // p_i exactly).  One FP64 instruction sequence serves both roles.
            const int np1 = n + 1;
            if (q < 9 && np1 < kRecipTable) {
                const bool ml = q < 3;
                const double2 dr = __ldg(g_div + np1);  // (n + 1, RN(1 / (n + 1)))
                const int pi = ml ? q : p_i, pj = p_j;
                const double a = p[pi] - (ml ? mean_l : 0.0);
                const double prod = a * (ml ? dr.y : p[pj]);
                const double r = __fma_rn(-prod, dr.x, a);
                const double q2 = __fma_rn(r, dr.y, prod);
                const double inc = ml ? (a == 0.0 ? prod : q2) : prod;
                const double v = (ml ? mean_l : ppt_l) + inc;
                if (ml) mean_l = v; else ppt_l = v;
            } else if (q < 9) {
                if (q < 3) mean_l = mean_l + (p[q] - mean_l) / ((double)n + 1.0);
                else ppt_l = ppt_l + p[p_i] * p[p_j];
            }
            n += 1;
        };
        // The point of step jj + 1 (index, coordinates, this lane's covariance
        // entries) is loaded during step jj, and the index of step jj + 2:
        // the two dependent loads leave the chain's critical path.
        uint32_t i_nx = 0, i_nx2 = 0;
        double p_nx[3] = {0.0, 0.0, 0.0}, c0_nx = 0.0, c1_nx = 0.0;
        auto fetch = [&](int j) {  // loads point j of the segment (j < e), index of j + 1
            i_nx = i_nx2;
            p_nx[0] = bpts[(size_t)i_nx * 3]; p_nx[1] = bpts[(size_t)i_nx * 3 + 1];
            p_nx[2] = bpts[(size_t)i_nx * 3 + 2];
            const double* c = bcov + (size_t)i_nx * 9;
            c0_nx = (q >= 3 && q < 10) ? c[q - 3] : 0.0;
            c1_nx = q < 2 ? c[7 + q] : 0.0;
            if (j + 1 < e) i_nx2 = sv[j + 1];
        };
        if (mine && b < e) {
            i_nx2 = sv[b];
            fetch(b);
        }
        if (build) {
            // VoxelMap::build: addPoint for every point, one updatePlane at the end.
            const int cnt = e - b;
            const bool store = mine && (nslab + cnt) < m.max_thresh && !(flags & F_DROPPED);
            for (int jj = 0;; ++jj) {
                const bool act = mine && b + jj < e;
                if (!__any_sync(0xffffffffu, act)) break;
                double p[3] = {0.0, 0.0, 0.0}, c0 = 0.0, c1 = 0.0;
                if (act) {
                    p[0] = p_nx[0]; p[1] = p_nx[1]; p[2] = p_nx[2];
                    c0 = c0_nx; c1 = c1_nx;
                    if (b + jj + 1 < e) fetch(b + jj + 1);
                    add_point(p);
                }
                group_slab_append(m, act && store, chunks, nslab, p, c0, c1, q, gbase);
            }
            if (mine) {
                if (!store) flags |= F_DROPPED;
                refit(cnt, 1);
                if (flags & F_DROPPED) {
                    __syncwarp(gmask);
                    if (q == 0) slab_release(m, chunks, nslab);
                    nslab = 0;
                }
            }
            __syncwarp();
        } else {
            for (int jj = 0;; ++jj) {
                bool act = !done && b + jj < e;
                bool init = (flags & F_INIT) != 0;
                if (act && init && !(flags & F_UPDATE)) {
                    // frozen: the remaining points only call merge() (if plane)
                    mstart = b + jj;
                    done = true;
                    act = false;
                }
                if (!__any_sync(0xffffffffu, act)) break;
                double p[3] = {0.0, 0.0, 0.0}, c0 = 0.0, c1 = 0.0;
                uint32_t i = 0;
                if (act) {
                    i = i_nx;
                    p[0] = p_nx[0]; p[1] = p_nx[1]; p[2] = p_nx[2];
                    c0 = c0_nx; c1 = c1_nx;
                    if (b + jj + 1 < e) fetch(b + jj + 1);
                    add_point(p);
                }
                group_slab_append(m, act && !(flags & F_DROPPED), chunks, nslab, p, c0, c1, q, gbase);
                if (act) {
                    if (!init) {
                        refit(nslab, 0);
                    } else {
                        newly++;
                        if (newly >= m.update_thresh) {
                            refit(nslab, 0);
                            newly = 0;
                        }
                        const int size_after = (flags & F_DROPPED) ? n : nslab;
                        if (size_after >= m.max_thresh) {
                            flags &= ~F_UPDATE;
                            flags &= ~F_DROPPED;
                            if (nref > 0 && !have_saved) {
                                for (int k = q; k < kMaxChunks; k += kGroupLanes) saved[k] = chunks[k];
                                have_saved = true;
                            }
                            __syncwarp(gmask);
                            if (q == 0) {
                                slab_release(m, chunks, nslab);
                                m.cold[rec].freeze_g = base + i;
                            }
                            nslab = 0;
                            __syncwarp(gmask);
                        }
                    }
                }
                __syncwarp();
            }
        }
        if (mine) {
            RecHot& H = m.hot[rec];
            RecCold& Cc = m.cold[rec];
            if (nref > 0) {
                int k = 0;
                if (q == 0) k = atomicAdd(ss.d_n_covseg, 1);
                k = __shfl_sync(gmask, k, gbase);
                CovSeg& cs = ss.covsegs[k];
                if (q == 0) {
                    cs.seg = (uint32_t)sidx;
                    cs.nref = nref;
                    cs.mstart = mstart;
                    ss.seg_cov[sidx] = k;
                }
                for (int t = q; t < kMaxChunks; t += kGroupLanes) cs.chunks[t] = have_saved ? saved[t] : chunks[t];
            } else if (flags & F_PLANE) {
                for (int j = mstart + q; j < e; j += kGroupLanes) ev_rec[sv[j]] = rec;  // merge() calls
            }
            if (q == 0) {
                H.flags = flags;
                H.n = n;
                Cc.newly = newly;
                Cc.nslab = nslab;
                Cc.stamp = base + sv[e - 1];
            }
            if (q < 3) H.mean[q] = mean_l;
            if (q >= 3 && q < 9) {
                Cc.ppt[p_idx] = ppt_l;
                Cc.ppt[p_mir] = ppt_l;
            }
            for (int t = q; t < kMaxChunks; t += kGroupLanes) Cc.chunks[t] = chunks[t];
        }
        __syncwarp();
    }
}

// Eigen decomposition of every refit snapshot (updatePlane, voxel_map.cpp:97-113);
// for a plane, the refit's J factors and a run of npts slots in the term
// buffer (one covariance term per buffered point).
__global__ void k_refit_eig(DMap m, SegScratch ss) {
    const int nr = *ss.d_n_refit;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nr; t += gridDim.x * blockDim.x) {
        const uint32_t si = ss.refit_list[t];
        RefitSnap& sn = ss.snaps[si];
        const double dn = (double)sn.n;
        double C[9], ev[3], evecs[9];
        // ppt / n - mean mean^T; the nine divisions by n share the divisor
        const double rn = 1.0 / dn;
        for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l)
                C[k * 3 + l] = div_by_recip(sn.ppt[k * 3 + l], dn, rn) - sn.mean[k] * sn.mean[l];
        eig_sym3<double>(C, ev, evecs);
        for (int k = 0; k < 3; ++k) sn.ev[k] = ev[k];
        for (int k = 0; k < 9; ++k) sn.evecs[k] = evecs[k];
        const int plane = ev[0] > m.plane_thresh ? 0 : 1;
        sn.plane = plane;
        sn.toff = -1;
        if (!plane) continue;
        RefitConst kc;
        refit_const(sn.mean, sn.n, ev, evecs, kc);
        for (int k = 0; k < 9; ++k) { sn.M1[k] = kc.M1[k]; sn.M2[k] = kc.M2[k]; }
        sn.den1 = kc.den1;
        sn.den2 = kc.den2;
        sn.inv_n = kc.inv_n;
        sn.rden1 = kc.rden1;
        sn.rden2 = kc.rden2;
        sn.recip_ok = kc.recip_ok ? 1 : 0;
        const int off = atomicAdd(ss.d_n_terms, sn.npts);
        if (off + sn.npts <= ss.term_cap) {  // else k_seg_cov forms these terms itself
            sn.toff = off;
            for (int j = 0; j < sn.npts; ++j) ss.term_snap[off + j] = si;
        }
    }
}

__device__ inline void snap_const(const RefitSnap& sn, RefitConst& k) {
    for (int q = 0; q < 3; ++q) k.mean[q] = sn.mean[q];
    for (int q = 0; q < 9; ++q) { k.evecs[q] = sn.evecs[q]; k.M1[q] = sn.M1[q]; k.M2[q] = sn.M2[q]; }
    k.den1 = sn.den1;
    k.den2 = sn.den2;
    k.inv_n = sn.inv_n;
    k.rden1 = sn.rden1;
    k.rden2 = sn.rden2;
    k.recip_ok = sn.recip_ok != 0;
}

// The point's source: batch segment (build) or slab prefix.
__device__ inline const double* term_point(const DMap& m, const RefitSnap& sn, int j, const int* chunks,
                                           const uint32_t* sv, const uint32_t* seg_start, const double* bpts,
                                           const double* bcov, double* pc) {
    if (sn.from_batch) {
        const uint32_t i = sv[seg_start[sn.seg] + j];
        for (int k = 0; k < 3; ++k) pc[k] = bpts[(size_t)i * 3 + k];
        for (int k = 0; k < 9; ++k) pc[3 + k] = bcov[(size_t)i * 9 + k];
        return pc;
    }
    return slab_pt(m, chunks, j);
}

constexpr int kTermThreads = 128;

// Every covariance term of every plane refit, one per thread (the terms of
// all refits of the batch packed densely over the lanes).  Register budget:
// 5 CTAs per SM (96 registers instead of 112).
__global__ void __launch_bounds__(kTermThreads, 5) k_cov_terms(DMap m, const uint32_t* __restrict__ seg_start,
                                                           const uint32_t* __restrict__ sv,
                                                           const double* __restrict__ bpts,
                                                           const double* __restrict__ bcov, SegScratch ss) {
    __shared__ double stage[kTermThreads * kCovTerms];
    int nt = *ss.d_n_terms;
    if (nt > ss.term_cap) nt = ss.term_cap;
    for (int t0 = blockIdx.x * kTermThreads; t0 < nt; t0 += gridDim.x * kTermThreads) {
        const int t = t0 + threadIdx.x;
        // a slot belongs to a refit only if that refit's whole run fitted;
        // the others keep the fill value of this batch (kNoRec)
        const uint32_t si = t < nt ? ss.term_snap[t] : kNoRec;
        if (si < (uint32_t)ss.snap_cap) {
            const RefitSnap& sn = ss.snaps[si];
            const int j = t - sn.toff;
            if (sn.toff >= 0 && j >= 0 && j < sn.npts) {
                RefitConst kc;
                snap_const(sn, kc);
                double pc[12];
                const int* chunks = ss.covsegs[ss.seg_cov[sn.seg]].chunks;
                const double* src = term_point(m, sn, j, chunks, sv, seg_start, bpts, bcov, pc);
                plane_cov_term(src, src + 3, kc, stage + threadIdx.x * kCovTerms);
            }
        }
        __syncthreads();
        const int cnt = min(kTermThreads, nt - t0);
        for (int q = threadIdx.x; q < cnt * kCovTerms; q += kTermThreads)
            ss.terms[(size_t)t0 * kCovTerms + q] = stage[q];
        __syncthreads();
    }
}

struct CovShared {
    double stage[kSegThreads / 32][32][kCovTerms];
    int chunks[kSegThreads / 32][kMaxChunks];
};

// Per voxel with refits: the plane covariance sums in point order (terms from
// the term buffer, or formed here when they did not fit), normal and centre
// of the last plane refit, merge calls.  Register budget: 6 CTAs per SM (80
// registers instead of 152; its warps mostly wait on a serial sum).
__global__ void __launch_bounds__(kSegThreads, 6) k_seg_cov(DMap m, const uint32_t* __restrict__ seg_start,
                                                         const uint32_t* __restrict__ seg_end,
                                                         const uint32_t* __restrict__ seg_rec,
                                                         const uint32_t* __restrict__ sv,
                                                         const double* __restrict__ bpts,
                                                         const double* __restrict__ bcov, uint32_t* ev_rec,
                                                         SegScratch ss) {
    __shared__ CovShared sh;
    if ((int)blockIdx.x >= g_seg_blocks) return;  // uniform per block
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int nc = *ss.d_n_covseg;
    int* chunks = sh.chunks[wib];
    double (*stage)[kCovTerms] = sh.stage[wib];
    (void)gw;
    (void)nw;
    for (;;) {
        int li = 0;
        if (lane == 0) li = atomicAdd(ss.d_work_cov, 1);
        li = __shfl_sync(0xffffffffu, li, 0);
        if (li >= nc) break;
        const CovSeg& cs = ss.covsegs[li];
        const uint32_t sidx = cs.seg;
        const int nref = cs.nref, mstart = cs.mstart;
        const uint32_t rec = seg_rec[sidx];
        const int b = (int)seg_start[sidx], e = (int)seg_end[sidx];
        RecHot& H = m.hot[rec];
        RecCold& Cc = m.cold[rec];
        uint32_t flags = H.flags;
        double norm[3] = {H.norm[0], H.norm[1], H.norm[2]};
        double center[3] = {Cc.center[0], Cc.center[1], Cc.center[2]};
        // lane q < 21 accumulates upper-triangle entry kUpper[q]
        const int ent = lane < kCovTerms ? kUpper[lane] : 0;
        double c0 = lane < kCovTerms ? Cc.cov[ent] : 0.0;
        if (lane < kMaxChunks) chunks[lane] = cs.chunks[lane];
        __syncwarp();
        for (int r = 0; r < nref; ++r) {
            const RefitSnap& sn = ss.snaps[b + r];
            if (!sn.plane) {
                flags &= ~F_PLANE;
                continue;
            }
            flags |= F_PLANE;
            const int npts = sn.npts;
            if (sn.toff >= 0) {
                const double* tp = ss.terms + (size_t)sn.toff * kCovTerms;
                if (lane < kCovTerms)
                    for (int j = 0; j < npts; ++j) c0 = c0 + tp[j * kCovTerms + lane];
            } else {
                RefitConst kc;
                snap_const(sn, kc);
                for (int base = 0; base < npts; base += 32) {
                    const int j = base + lane;
                    if (j < npts) {
                        double pc[12];
                        const double* src = term_point(m, sn, j, chunks, sv, seg_start, bpts, bcov, pc);
                        plane_cov_term(src, src + 3, kc, stage[lane]);
                    }
                    __syncwarp();
                    const int cnt = min(32, npts - base);
                    if (lane < kCovTerms)
                        for (int u = 0; u < cnt; ++u) c0 = c0 + stage[u][lane];
                    __syncwarp();
                }
            }
            double pn[3] = {sn.evecs[0], sn.evecs[3], sn.evecs[6]};
            const double axis_distance = -dot3(sn.mean, pn);
            if (axis_distance < 0.0) { pn[0] = -pn[0]; pn[1] = -pn[1]; pn[2] = -pn[2]; }
            for (int k = 0; k < 3; ++k) { norm[k] = pn[k]; center[k] = sn.mean[k]; }
        }
        if (flags & F_PLANE)
            for (int j = mstart + lane; j < e; j += 32) ev_rec[sv[j]] = rec;  // merge() calls
        if (lane == 0) {
            H.flags = flags;
            for (int k = 0; k < 3; ++k) { H.norm[k] = norm[k]; Cc.center[k] = center[k]; }
        }
        if (lane < kCovTerms) {  // the upper triangle and its mirror
            Cc.cov[ent] = c0;
            Cc.cov[(ent % 6) * 6 + ent / 6] = c0;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- finalize
__global__ void k_ev_flags(const uint32_t* __restrict__ ev_rec, const int* d_n, uint32_t* flag) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        flag[i] = ev_rec[i] != kNoRec ? 1u : 0u;
}
__global__ void k_compact_idx(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ rank, const int* d_n,
                              uint32_t* out) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (flag[i]) out[rank[i]] = (uint32_t)i;
}

// Appends the touched records to the LRU queue in last-touch order.
__global__ void k_queue_append(DMap m, const uint32_t* __restrict__ last_touch, const uint32_t* __restrict__ rank,
                               const uint32_t* __restrict__ rec, const int* d_n, const int* d_n_touch) {
    const int n = *d_n;
    const unsigned long long tail = m.cnt->q_tail;
    const unsigned long long base = m.cnt->batch_base;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!last_touch[i]) continue;
        unsigned long long q = tail + rank[i];
        m.q_rec[q % m.q_cap] = rec[i];
        m.q_stamp[q % m.q_cap] = base + (unsigned long long)i;
    }
    (void)d_n_touch;
}

// Evictions: remove the victims' keys (tombstones), return records and slab
// chunks to their free stacks.
__global__ void k_finalize(DMap m, const uint32_t* __restrict__ victims) {
    Counters* c = m.cnt;
    const int ne = c->n_evict;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < ne; v += gridDim.x * blockDim.x) {
        uint32_t r = victims[v];
        uint64_t key = m.cold[r].key;
        uint64_t h = hash_key(key) & m.table_mask;
        for (uint64_t probe = 0; probe <= m.table_mask; ++probe) {
            uint64_t k = m.keys[h];
            if (k == key && m.vals[h] == r) { m.keys[h] = kTombKey; m.vals[h] = 0xFFFFFFFFu; break; }
            if (k == kEmptyKey) break;
            h = (h + 1) & m.table_mask;
        }
        m.hot[r].flags = 0;
        int nsl = m.cold[r].nslab;
        slab_release(m, m.cold[r].chunks, nsl);
        m.cold[r].nslab = 0;
        m.rec_free[c->rec_free_top + v] = r;
    }
}
__global__ void k_finalize_chunks(DMap m) {
    Counters* c = m.cnt;
    int nf = c->chunk_freed_top;
    if (nf > m.chunk_pool) nf = m.chunk_pool;
    const int top = c->chunk_free_top;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nf; k += gridDim.x * blockDim.x)
        m.chunk_free[top + k] = m.chunk_freed[k];
}
__global__ void k_finalize_counters(DMap m, const int* d_n, const int* d_n_touch) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Counters* c = m.cnt;
    const int ne = c->n_evict;
    c->rec_free_top += ne;
    c->size -= ne;
    c->evicted_total += ne;
    c->n_tomb += ne;
    int nf = c->chunk_freed_top;
    if (nf > m.chunk_pool) nf = m.chunk_pool;
    c->chunk_free_top += nf;
    c->chunk_freed_top = 0;
    c->q_tail += (unsigned long long)(*d_n_touch);
    c->batch_base += (unsigned long long)(*d_n);
    c->n_evict = 0;
}

// ---------------------------------------------------------------- driver
// Phase A: keys, hash insert, creation ranking, records, segments.
void launch_map_phase_a(DMap& m, MapScratch& ms, const double* bpts, int n_max, cudaStream_t st) {
    const int g = grid_for_map(n_max);
    VMP_NOTE_LAUNCH(); k_lookup_insert<<<g, kMapThreads, 0, st>>>(m, bpts, ms.d_n, ms.slot, nullptr);
    VMP_NOTE_LAUNCH(); k_creator_flags<<<g, kMapThreads, 0, st>>>(m, ms.slot, ms.d_n, ms.flag);
    exclusive_scan_u32(ms.flag, ms.rank, ms.d_n, ms.d_n_new, ms.scan, st);
    VMP_NOTE_LAUNCH(); k_assign<<<g, kMapThreads, 0, st>>>(m, ms.slot, ms.flag, ms.rank, ms.d_n, ms.new_pos);
    VMP_NOTE_LAUNCH(); k_assign_counters<<<1, 32, 0, st>>>(m, ms.d_n_new);
}
// Eviction walk (only when the batch can overflow the capacity).
void launch_map_walk(DMap& m, MapScratch& ms, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_evict_walk<<<1, kWalkThreads, 0, st>>>(m, ms.new_pos, ms.victims, ms.d_n);
}
void launch_map_rollback(DMap& m, MapScratch& ms, int n_max, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_rollback<<<grid_for_map(n_max), kMapThreads, 0, st>>>(m, ms.slot, ms.flag, ms.d_n);
    VMP_NOTE_LAUNCH(); k_rollback_counters<<<1, 32, 0, st>>>(m);
}
// Segments are formed before the walk (the walk needs each touched record's
// first touch).
void launch_map_segments(DMap& m, MapScratch& ms, int n_max, cudaStream_t st) {
    const int g = grid_for_map(n_max);
    VMP_NOTE_LAUNCH(); k_resolve<<<g, kMapThreads, 0, st>>>(m, ms.slot, ms.d_n, ms.rec, ms.sk, ms.sv);
    int rec_bits = 1;
    while (rec_bits < 32 && (1ll << rec_bits) < (long long)m.rec_pool) ++rec_bits;
    radix_sort_pairs(ms.sk, ms.sv, ms.d_n, rec_bits, ms.sort, st);
    VMP_NOTE_LAUNCH(); k_seg_heads<<<g, kMapThreads, 0, st>>>(ms.sk, ms.d_n, ms.flag2);
    exclusive_scan_u32(ms.flag2, ms.rank2, ms.d_n, ms.d_n_seg, ms.scan, st);
    VMP_NOTE_LAUNCH(); k_fill_u32<<<g, kMapThreads, 0, st>>>(ms.last_touch, ms.d_n, 0u);
    VMP_NOTE_LAUNCH(); k_fill_u32<<<g, kMapThreads, 0, st>>>(ms.ev_rec, ms.d_n, kNoRec);
    VMP_NOTE_LAUNCH(); k_seg_bounds<<<g, kMapThreads, 0, st>>>(m, ms.sk, ms.sv, ms.flag2, ms.rank2, ms.d_n, ms.seg_start, ms.seg_end,
                                            ms.seg_rec, ms.last_touch);
}
// Phase B1: the per-voxel pushPoint / addPoint state machine.
void launch_map_state(DMap& m, MapScratch& ms, const double* bpts, const double* bcov, int n_max, bool build,
                      cudaStream_t st) {
    // warps take their work from counters; the grids keep enough warps for
    // the longest chains to start at once (of them, the first g_seg_blocks
    // blocks work)
    int sg = (n_max + (kSegThreads / 32) - 1) / (kSegThreads / 32);
    if (sg > 152 * 16) sg = 152 * 16;
    if (seg_grid_blocks() > 0 && sg > kSegServedBlocks) sg = kSegServedBlocks;  // blocks past it would return
    if (sg < 1) sg = 1;
    const int cg = sg;
    SegScratch ss{static_cast<RefitSnap*>(ms.seg_snaps), ms.refit_list, static_cast<CovSeg*>(ms.covsegs),
                  ms.seg_cov, ms.term_snap, ms.terms, ms.term_cap, ms.max_batch + 16, ms.d_scratch_int + 5,
                  ms.d_scratch_int + 6, ms.d_scratch_int + 7, ms.d_scratch_int + 8, ms.d_scratch_int + 9};
    cudaMemsetAsync(ms.d_scratch_int + 5, 0, 5 * sizeof(int), st);
    cudaMemsetAsync(ms.term_snap, 0xFF, sizeof(uint32_t) * (size_t)ms.term_cap, st);
    VMP_NOTE_LAUNCH();
    k_seg_chain<<<sg, kSegThreads, 0, st>>>(m, ms.seg_start, ms.seg_end, ms.seg_rec, ms.d_n_seg, ms.sv, bpts, bcov,
                                            ms.ev_rec, ss, build ? 1 : 0);
    // one warp per block so that the refits spread over all SMs
    int eg = (n_max + 255) / 256;
    if (eg > 152 * 8) eg = 152 * 8;
    if (eg < 1) eg = 1;
    eg = served_grid(eg);
    VMP_NOTE_LAUNCH();
    k_refit_eig<<<eg, 32, 0, st>>>(m, ss);
    int tg = (2 * n_max + kTermThreads - 1) / kTermThreads;
    if (tg > 152 * 8) tg = 152 * 8;
    if (tg < 1) tg = 1;
    tg = served_grid(tg);
    VMP_NOTE_LAUNCH();
    k_cov_terms<<<tg, kTermThreads, 0, st>>>(m, ms.seg_start, ms.sv, bpts, bcov, ss);
    VMP_NOTE_LAUNCH();
    k_seg_cov<<<cg, kSegThreads, 0, st>>>(m, ms.seg_start, ms.seg_end, ms.seg_rec, ms.sv, bpts, bcov, ms.ev_rec, ss);
}
// Phase B2: merges, LRU queue, evictions, counters.  In two halves around the
// merge resolution, so that a captured graph can hold each half.
void launch_map_finish_pre(DMap& m, MapScratch& ms, int n_max, bool build, cudaStream_t st) {
    const int g = grid_for_map(n_max);
    if (build) return;
    VMP_NOTE_LAUNCH(); k_ev_flags<<<g, kMapThreads, 0, st>>>(ms.ev_rec, ms.d_n, ms.flag2);
    exclusive_scan_u32(ms.flag2, ms.rank2, ms.d_n, ms.d_n_ev, ms.scan, st);
    VMP_NOTE_LAUNCH(); k_compact_idx<<<g, kMapThreads, 0, st>>>(ms.flag2, ms.rank2, ms.d_n, ms.ev_list);
}
void launch_map_finish_post(DMap& m, MapScratch& ms, int n_max, cudaStream_t st) {
    const int g = grid_for_map(n_max);
    exclusive_scan_u32(ms.last_touch, ms.rank2, ms.d_n, ms.d_n_touch, ms.scan, st);
    VMP_NOTE_LAUNCH(); k_queue_append<<<g, kMapThreads, 0, st>>>(m, ms.last_touch, ms.rank2, ms.rec, ms.d_n, ms.d_n_touch);
    VMP_NOTE_LAUNCH(); k_finalize<<<g, kMapThreads, 0, st>>>(m, ms.victims);
    VMP_NOTE_LAUNCH(); k_finalize_chunks<<<g, kMapThreads, 0, st>>>(m);
    VMP_NOTE_LAUNCH(); k_finalize_counters<<<1, 32, 0, st>>>(m, ms.d_n, ms.d_n_touch);
}
void launch_map_finish(DMap& m, MapScratch& ms, int n_max, bool build, cudaStream_t st) {
    launch_map_finish_pre(m, ms, n_max, build, st);
    if (!build) run_merge_events(m, ms, ms.merge, n_max, ms.merge_mode, &ms.merge_rounds, st);
    launch_map_finish_post(m, ms, n_max, st);
}
void launch_map_phase_b(DMap& m, MapScratch& ms, const double* bpts, const double* bcov, int n_max, bool build,
                        cudaStream_t st) {
    launch_map_state(m, ms, bpts, bcov, n_max, build, st);
    launch_map_finish(m, ms, n_max, build, st);
}

// Rebuilds the hash table from the live records (drops tombstones).
__global__ void k_clear_table(DMap m) {
    const size_t ts = (size_t)m.table_mask + 1;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ts; i += (size_t)gridDim.x * blockDim.x) {
        m.keys[i] = kEmptyKey;
        m.vals[i] = 0xFFFFFFFFu;
    }
}
__global__ void k_reinsert(DMap m) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m.rec_pool; r += gridDim.x * blockDim.x) {
        if (!(m.hot[r].flags & F_ALIVE)) continue;
        uint64_t key = m.cold[r].key;
        uint64_t h = hash_key(key) & m.table_mask;
        for (uint64_t probe = 0; probe <= m.table_mask; ++probe) {
            unsigned long long prev = atomicCAS((unsigned long long*)&m.keys[h], (unsigned long long)kEmptyKey,
                                                (unsigned long long)key);
            if (prev == kEmptyKey) { m.vals[h] = (uint32_t)r; break; }
            h = (h + 1) & m.table_mask;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) m.cnt->n_tomb = 0;
}
void launch_rehash(DMap& m, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_clear_table<<<1216, 256, 0, st>>>(m);
    VMP_NOTE_LAUNCH(); k_reinsert<<<1216, 256, 0, st>>>(m);
}

// LRU queue compaction: keeps the live entries, in order, from q_head.
__global__ void k_q_live(DMap m, uint32_t* flag, const int* d_len) {
    const int len = *d_len;
    const unsigned long long h = m.cnt->q_head;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        unsigned long long q = (h + i) % m.q_cap;
        uint32_t r = m.q_rec[q];
        flag[i] = ((m.hot[r].flags & F_ALIVE) && m.cold[r].stamp == m.q_stamp[q]) ? 1u : 0u;
    }
}
__global__ void k_q_gather(DMap m, const uint32_t* flag, const uint32_t* rank, const int* d_len, uint32_t* tr,
                           uint64_t* ts) {
    const int len = *d_len;
    const unsigned long long h = m.cnt->q_head;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        if (!flag[i]) continue;
        unsigned long long q = (h + i) % m.q_cap;
        tr[rank[i]] = m.q_rec[q];
        ts[rank[i]] = m.q_stamp[q];
    }
}
__global__ void k_q_scatter(DMap m, const uint32_t* tr, const uint64_t* ts, const int* d_live) {
    const int live = *d_live;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < live; i += gridDim.x * blockDim.x) {
        m.q_rec[i] = tr[i];
        m.q_stamp[i] = ts[i];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        m.cnt->q_head = 0;
        m.cnt->q_tail = (unsigned long long)live;
    }
}
void launch_queue_compact(DMap& m, uint32_t* flag, uint32_t* rank, uint32_t* tr, uint64_t* ts, int* d_len,
                          int* d_live, int len_max, ScanScratch& sc, cudaStream_t st) {
    const int g = grid_for_map(len_max);
    VMP_NOTE_LAUNCH(); k_q_live<<<g, kMapThreads, 0, st>>>(m, flag, d_len);
    exclusive_scan_u32(flag, rank, d_len, d_live, sc, st);
    VMP_NOTE_LAUNCH(); k_q_gather<<<g, kMapThreads, 0, st>>>(m, flag, rank, d_len, tr, ts);
    VMP_NOTE_LAUNCH(); k_q_scatter<<<g, kMapThreads, 0, st>>>(m, tr, ts, d_live);
}

__global__ void k_map_index(DMap m, const double* pts, int n, int64_t* keys) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double p[3] = {pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]};
        // VoxelMap::index, unbounded int64 (no packing here)
        for (int a = 0; a < 3; ++a) keys[i * 3 + a] = (int64_t)floor(__ddiv_rn(p[a], m.voxel_size));
    }
}
void launch_map_index(const DMap& m, const double* pts, int n, int64_t* keys, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_map_index<<<grid_for_map(n), kMapThreads, 0, st>>>(m, pts, n, keys);
}

__global__ void k_map_reset(DMap m) {
    const size_t ts = (size_t)m.table_mask + 1;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ts; i += (size_t)gridDim.x * blockDim.x) {
        m.keys[i] = kEmptyKey;
        m.vals[i] = 0xFFFFFFFFu;
    }
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)m.rec_pool;
         i += (size_t)gridDim.x * blockDim.x) {
        m.rec_free[i] = (uint32_t)(m.rec_pool - 1 - i);
        m.hot[i].flags = 0;
    }
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)m.chunk_pool;
         i += (size_t)gridDim.x * blockDim.x)
        m.chunk_free[i] = (int32_t)(m.chunk_pool - 1 - i);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Counters* c = m.cnt;
        c->size = 0;
        c->group_counter = 0;
        c->batch_base = 1;
        c->q_head = c->q_tail = 0;
        c->rec_free_top = m.rec_pool;
        c->chunk_free_top = m.chunk_pool;
        c->chunk_freed_top = 0;
        c->n_new = c->n_seg = c->n_events = c->n_evict = 0;
        c->error = 0;
        c->evicted_total = 0;
        c->split_at = -1;
        c->n_tomb = 0;
    }
}
void launch_map_reset(DMap& m, cudaStream_t st) { VMP_NOTE_LAUNCH(); k_map_reset<<<1216, 256, 0, st>>>(m); }

cudaError_t map_scratch_alloc(MapScratch& ms, int max_batch, int rec_pool, int term_cap) {
    ms.max_batch = max_batch;
    size_t nb = (size_t)max_batch + 16;
    cudaError_t e;
    uint32_t** u32s[] = {&ms.slot, &ms.rec, &ms.flag, &ms.rank, &ms.flag2, &ms.rank2, &ms.sk, &ms.sv, &ms.seg_start, &ms.seg_end,
                         &ms.seg_rec, &ms.ev_rec, &ms.ev_list, &ms.last_touch, &ms.victims, &ms.new_pos};
    for (auto pp : u32s)
        if ((e = dev_malloc(pp, sizeof(uint32_t) * nb)) != cudaSuccess) return e;
    if ((e = merge_scratch_alloc(&ms.merge, max_batch, rec_pool)) != cudaSuccess) return e;
    if ((e = dev_malloc(&ms.seg_snaps, sizeof(RefitSnap) * nb)) != cudaSuccess) return e;
    if ((e = dev_malloc(&ms.covsegs, sizeof(CovSeg) * nb)) != cudaSuccess) return e;
    if ((e = dev_malloc(&ms.refit_list, sizeof(uint32_t) * nb)) != cudaSuccess) return e;
    if ((e = dev_malloc(&ms.seg_cov, sizeof(int) * nb)) != cudaSuccess) return e;
    // refits re-read the slab, so a batch has more terms than points; terms
    // that do not fit are formed by k_seg_cov itself
    ms.term_cap = term_cap > 0 ? term_cap : 4 * max_batch + 65536;
    if ((e = dev_malloc(&ms.term_snap, sizeof(uint32_t) * (size_t)ms.term_cap)) != cudaSuccess) return e;
    if ((e = dev_malloc(&ms.terms, sizeof(double) * kCovTerms * (size_t)ms.term_cap)) != cudaSuccess) return e;
    ms.merge_mode = 0;
    ms.merge_rounds = 0;
    ms.merge_d2h = 0;
    if ((e = dev_malloc(&ms.d_scratch_int, sizeof(int) * 32)) != cudaSuccess) return e;
    ms.d_n = ms.d_scratch_int;
    ms.d_n_new = ms.d_scratch_int + 1;
    ms.d_n_seg = ms.d_scratch_int + 2;
    ms.d_n_ev = ms.d_scratch_int + 3;
    ms.d_n_touch = ms.d_scratch_int + 4;
    if ((e = sort_scratch_alloc(ms.sort, max_batch)) != cudaSuccess) return e;
    if ((e = scan_scratch_alloc(ms.scan, max_batch)) != cudaSuccess) return e;
    return cudaSuccess;
}
void map_scratch_free(MapScratch& ms) {
    uint32_t* u32s[] = {ms.slot, ms.rec, ms.flag, ms.rank, ms.flag2, ms.rank2, ms.sk, ms.sv, ms.seg_start, ms.seg_end, ms.seg_rec,
                        ms.ev_rec, ms.ev_list, ms.last_touch, ms.victims, ms.new_pos};
    for (auto p : u32s) cudaFree(p);
    merge_scratch_free(ms.merge);
    cudaFree(ms.seg_snaps);
    cudaFree(ms.covsegs);
    cudaFree(ms.refit_list);
    cudaFree(ms.seg_cov);
    cudaFree(ms.term_snap);
    cudaFree(ms.terms);
    cudaFree(ms.d_scratch_int);
    sort_scratch_free(ms.sort);
    scan_scratch_free(ms.scan);
}

}  // namespace vmp
