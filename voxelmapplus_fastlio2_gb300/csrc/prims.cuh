// Device primitives used by the per-scan pipeline: a stable LSD radix sort of
// (u32 key, u32 value) pairs and an exclusive scan of u32 values.  Both take
// the element count from device memory (d_n) and size their grids for a
// host-side upper bound, so a scan pipeline needs no host synchronisation.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace vmp {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // 2048
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

struct SortScratch {
    uint32_t* k_alt = nullptr;
    uint32_t* v_alt = nullptr;
    uint32_t* hist = nullptr;       // [256][blocks]
    uint32_t* row_total = nullptr;  // [256] per-digit totals
    int n_max = 0;
    int blocks = 0;
};

struct ScanScratch {
    uint32_t* block_sums = nullptr;
    int n_max = 0;
    int blocks = 0;
};

cudaError_t sort_scratch_alloc(SortScratch& s, int n_max);
void sort_scratch_free(SortScratch& s);
cudaError_t scan_scratch_alloc(ScanScratch& s, int n_max);
void scan_scratch_free(ScanScratch& s);

// Sorts keys/vals (length *d_n <= s.n_max) by the low `bits` key bits,
// stably.  The result is left in keys/vals (in place; s holds the alternate
// buffers).  need (device, may be null): when it holds 0 the keys are known
// to be in non-decreasing order already, so the stable sort is the identity
// and every pass returns at once.
void radix_sort_pairs(uint32_t* keys, uint32_t* vals, const int* d_n, int bits, SortScratch& s, cudaStream_t st,
                      const int* need = nullptr);

// out[i] = sum_{j<i} in[i] for i < *d_n; *d_total = sum (may alias nothing).
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, const int* d_n, int* d_total, ScanScratch& s,
                        cudaStream_t st);

}  // namespace vmp
