// Stable LSD radix sort (8-bit digits) and exclusive scan.
//
// Sort pass = histogram per 2048-element tile -> per-digit exclusive scan of
// the tile counts (one warp per digit) -> stable scatter, which adds the
// digit's base (an exclusive scan of the 256 digit totals, redone in every
// scatter CTA).  The scatter ranks equal digits inside a tile
// with __match_any_sync: warp w owns tile elements [256w, 256w + 256) and
// walks them 32 at a time in order, so the rank of an element is
// (earlier warps' count of its digit) + (its warp's running count) + (its
// rank among equal lanes of the same 32-element step) -- input order is kept.
#include "common.cuh"
#include "prims.cuh"

namespace vmp {

std::atomic<long long> g_launch_count{0};

static thread_local long long* t_capture_counter = nullptr;
long long* capture_launch_counter() { return t_capture_counter; }
void set_capture_launch_counter(long long* c) { t_capture_counter = c; }

long long& dev_bytes_counter() {
    static thread_local long long bytes = 0;
    return bytes;
}

__global__ void k_radix_hist(const uint32_t* __restrict__ keys, const int* __restrict__ d_n, int shift,
                             uint32_t* __restrict__ hist, int blocks, const int* need) {
    __shared__ uint32_t cnt[256];
    if (need && *need == 0) return;  // uniform
    const int n = *d_n;
    // the grid covers the largest n: tiles past this n hold nothing, and
    // k_radix_scan_rows / k_radix_scatter read only the tiles that do
    if (blockIdx.x > 0 && (long long)blockIdx.x * kSortTile >= n) return;
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += kSortThreads) {
        int e = base + i;
        if (e < n) atomicAdd(&cnt[(keys[e] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * blocks + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of each digit's tile counts, one warp per digit, in place;
// the digit totals go to row_total.
__global__ void k_radix_scan_rows(uint32_t* hist, int blocks, uint32_t* row_total, const int* need,
                                  const int* d_n) {
    if (need && *need == 0) return;  // uniform
    const int d = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (d >= 256) return;
    const int used = max(1, min(blocks, (*d_n + kSortTile - 1) / kSortTile));  // tiles that hold keys
    uint32_t* row = hist + (size_t)d * blocks;
    uint32_t carry = 0;
    for (int base = 0; base < used; base += 32) {
        const int i = base + lane;
        const uint32_t v = i < used ? row[i] : 0u;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (i < used) row[i] = carry + x - v;
        carry += __shfl_sync(0xffffffffu, x, 31);
    }
    if (lane == 0) row_total[d] = carry;
}

__device__ inline uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot, uint32_t& total);

__global__ void k_radix_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                const int* __restrict__ d_n, int shift, const uint32_t* __restrict__ hist,
                                const uint32_t* __restrict__ row_total, int blocks, const int* need) {
    constexpr int W = kSortThreads / 32;
    if (need && *need == 0) return;  // uniform
    if ((long long)blockIdx.x * kSortTile >= *d_n) return;  // a tile past the keys: nothing to place
    static_assert(kSortThreads == 256, "one thread per digit");
    __shared__ uint32_t wcnt[W][256];
    __shared__ uint32_t dbase[256];
    __shared__ uint32_t warp_tot[32];
    const int n = *d_n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < W * 256; i += kSortThreads) (&wcnt[0][0])[i] = 0;
    {
        uint32_t total;
        dbase[threadIdx.x] = block_exclusive_scan(row_total[threadIdx.x], warp_tot, total);
    }
    __syncthreads();
    const int base = blockIdx.x * kSortTile + warp * (32 * kSortItems);
    uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        int e = base + r * 32 + lane;
        bool ok = e < n;
        key[r] = ok ? kin[e] : 0u;
        val[r] = ok ? vin[e] : 0u;
        uint32_t d = ok ? ((key[r] >> shift) & 255u) : 0xFFFFFFFFu;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = __popc(peers & lt);
        uint32_t c = ok ? wcnt[warp][d] : 0u;
        rank[r] = c + before;
        __syncwarp();
        if (ok && before == 0) wcnt[warp][d] = c + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // exclusive prefix over warps, per digit
    for (int d = threadIdx.x; d < 256; d += kSortThreads) {
        uint32_t s = dbase[d] + hist[d * blocks + blockIdx.x];
        for (int w = 0; w < W; ++w) {
            uint32_t c = wcnt[w][d];
            wcnt[w][d] = s;
            s += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        int e = base + r * 32 + lane;
        if (e < n) {
            uint32_t d = (key[r] >> shift) & 255u;
            uint32_t pos = wcnt[warp][d] + rank[r];
            kout[pos] = key[r];
            vout[pos] = val[r];
        }
    }
}

cudaError_t sort_scratch_alloc(SortScratch& s, int n_max) {
    s.n_max = n_max;
    s.blocks = (n_max + kSortTile - 1) / kSortTile;
    if (s.blocks < 1) s.blocks = 1;
    cudaError_t e;
    if ((e = dev_malloc(&s.k_alt, sizeof(uint32_t) * (size_t)n_max + 16)) != cudaSuccess) return e;
    if ((e = dev_malloc(&s.v_alt, sizeof(uint32_t) * (size_t)n_max + 16)) != cudaSuccess) return e;
    if ((e = dev_malloc(&s.hist, sizeof(uint32_t) * 256 * (size_t)s.blocks)) != cudaSuccess) return e;
    if ((e = dev_malloc(&s.row_total, sizeof(uint32_t) * 256)) != cudaSuccess) return e;
    return cudaSuccess;
}
void sort_scratch_free(SortScratch& s) {
    cudaFree(s.k_alt); cudaFree(s.v_alt); cudaFree(s.hist); cudaFree(s.row_total);
    s.k_alt = s.v_alt = s.hist = s.row_total = nullptr;
}

__global__ void k_copy_pairs(const uint32_t* __restrict__ ks, const uint32_t* __restrict__ vs, uint32_t* kd,
                             uint32_t* vd, const int* d_n, const int* need) {
    if (need && *need == 0) return;  // uniform: the pairs never left keys / vals
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        kd[i] = ks[i];
        vd[i] = vs[i];
    }
}

void radix_sort_pairs(uint32_t* keys, uint32_t* vals, const int* d_n, int bits, SortScratch& s, cudaStream_t st,
                      const int* need) {
    int passes = (bits + 7) / 8;
    if (passes < 1) passes = 1;
    if (passes > 4) passes = 4;
    uint32_t *ka = keys, *va = vals, *kb = s.k_alt, *vb = s.v_alt;
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        VMP_NOTE_LAUNCH(); k_radix_hist<<<s.blocks, kSortThreads, 0, st>>>(ka, d_n, shift, s.hist, s.blocks, need);
        VMP_NOTE_LAUNCH(); k_radix_scan_rows<<<8, 1024, 0, st>>>(s.hist, s.blocks, s.row_total, need, d_n);
        VMP_NOTE_LAUNCH();
        k_radix_scatter<<<s.blocks, kSortThreads, 0, st>>>(ka, va, kb, vb, d_n, shift, s.hist, s.row_total, s.blocks,
                                                            need);
        uint32_t* t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    if (ka != keys) {  // odd pass count: the result is in the alternate buffers
        int g = (s.n_max + 255) / 256;
        if (g > 152 * 8) g = 152 * 8;
        VMP_NOTE_LAUNCH(); k_copy_pairs<<<g, 256, 0, st>>>(ka, va, keys, vals, d_n, need);
    }
}

// ------------------------------------------------------------------ scan
__device__ inline uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot, uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    total = warp_tot[(blockDim.x >> 5) - 1];
    uint32_t r = (warp > 0 ? warp_tot[warp - 1] : 0u) + x - v;
    __syncthreads();
    return r;
}

__global__ void k_scan_tiles(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, const int* d_n,
                             uint32_t* __restrict__ block_sums) {
    __shared__ uint32_t warp_tot[32];
    const int n = *d_n;
    // tiles past n: k_scan_top and k_scan_add read only the tiles that hold values
    if (blockIdx.x > 0 && (long long)blockIdx.x * kScanTile >= n) return;
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int r = 0; r < kScanItems; ++r) {
        int e = base + r;
        v[r] = e < n ? in[e] : 0u;
        s += v[r];
    }
    uint32_t total;
    uint32_t pre = block_exclusive_scan(s, warp_tot, total);
#pragma unroll
    for (int r = 0; r < kScanItems; ++r) {
        int e = base + r;
        if (e < n) out[e] = pre;
        pre += v[r];
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void k_scan_top(uint32_t* block_sums, int blocks, const int* d_n, int* d_total) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t carry;
    const int n = *d_n;
    const int used = (n + kScanTile - 1) / kScanTile;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < used; base += blockDim.x) {
        int i = base + threadIdx.x;
        uint32_t v = i < used ? block_sums[i] : 0u;
        uint32_t total;
        uint32_t pre = block_exclusive_scan(v, warp_tot, total);
        if (i < used) block_sums[i] = carry + pre;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0 && d_total) *d_total = (int)carry;
    (void)blocks;
}

__global__ void k_scan_add(uint32_t* __restrict__ out, const int* d_n, const uint32_t* __restrict__ block_sums) {
    const int n = *d_n;
    if ((long long)blockIdx.x * kScanTile >= n) return;
    const uint32_t add = block_sums[blockIdx.x];
    const int base = blockIdx.x * kScanTile;
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) {
        int e = base + i;
        if (e < n) out[e] += add;
    }
}

cudaError_t scan_scratch_alloc(ScanScratch& s, int n_max) {
    s.n_max = n_max;
    s.blocks = (n_max + kScanTile - 1) / kScanTile;
    if (s.blocks < 1) s.blocks = 1;
    return dev_malloc(&s.block_sums, sizeof(uint32_t) * (size_t)s.blocks + 16);
}
void scan_scratch_free(ScanScratch& s) {
    cudaFree(s.block_sums);
    s.block_sums = nullptr;
}

void exclusive_scan_u32(const uint32_t* in, uint32_t* out, const int* d_n, int* d_total, ScanScratch& s,
                        cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_scan_tiles<<<s.blocks, kScanThreads, 0, st>>>(in, out, d_n, s.block_sums);
    VMP_NOTE_LAUNCH(); k_scan_top<<<1, 1024, 0, st>>>(s.block_sums, s.blocks, d_n, d_total);
    VMP_NOTE_LAUNCH(); k_scan_add<<<s.blocks, kScanThreads, 0, st>>>(out, d_n, s.block_sums);
}

}  // namespace vmp
