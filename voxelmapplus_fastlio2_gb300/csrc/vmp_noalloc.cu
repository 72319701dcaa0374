// vmp_downsample_noalloc: the scan downsample (pcl::VoxelGrid leaf-centroid
// filter) for callers that cannot allocate device memory.
//
// Who needs it: a LiDAR driver or real-time control thread that must not call
// cudaMalloc / cudaFree (they can synchronise the whole device and have no
// latency bound), and host frameworks whose device memory is owned by their
// own allocator that reserved the GPU up front.  Such a caller hands in
// device buffers it already owns for the input cloud and the output; the
// working memory of the filter (sort keys and values, histograms, run bounds,
// grid parameters) lives in one fixed array of this library.
//
// The working memory is `g_noalloc_scratch`, a file-scope __device__ array of
// kNoAllocBytes (2 MiB), enough for kNoAllocMaxPoints (65536) input points.
// Every GPU that loads libvmp.so holds that array until the process exits.
// In host code the array's name is only a host-side handle, not a device
// address: the first call on each device (with that device current) resolves
// the device address with cudaGetSymbolAddress and caches it.  Every call
// ends by reading the output count back and synchronising its stream.  The
// cached address belongs to
// the device's context of that moment: cudaDeviceReset while libvmp is loaded
// is not supported.  All calls share the one array: two calls whose work
// overlaps on the GPU race on it and must be serialised by the caller (same
// stream, or events).  Each call writes every scratch word it reads before
// reading it, so nothing has to start at zero and no state survives from one
// call to the next.
//
// The input and output are read as float4, so both must be 16-byte aligned
// device (or managed) memory, and they must not overlap: the centroid pass
// reads input points across the whole cloud while other threads write output
// points.  All three are checked before anything is launched.
#include <mutex>

#include "kernels.cuh"

namespace vmp {

constexpr int kNoAllocMaxPoints = 65536;
constexpr size_t kNoAllocBytes = size_t(2) << 20;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

constexpr size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// Scratch layout (byte offsets into g_noalloc_scratch).
constexpr int kNaSortBlocks = (kNoAllocMaxPoints + kSortTile - 1) / kSortTile;
constexpr int kNaScanBlocks = (kNoAllocMaxPoints + kScanTile - 1) / kScanTile;
constexpr size_t kU32N = sizeof(uint32_t) * (kNoAllocMaxPoints + 16);
constexpr size_t kOffNRaw = 0;
constexpr size_t kOffNDown = align256(kOffNRaw + sizeof(int));
constexpr size_t kOffParams = align256(kOffNDown + sizeof(int));
constexpr size_t kOffMinMax = align256(kOffParams + 32 * sizeof(int));
constexpr size_t kOffSortK = align256(kOffMinMax + (kMinMaxBlocks * 6 + 8) * sizeof(float));
constexpr size_t kOffSortV = align256(kOffSortK + kU32N);
constexpr size_t kOffFlags = align256(kOffSortV + kU32N);
constexpr size_t kOffScan = align256(kOffFlags + kU32N);
constexpr size_t kOffRunStart = align256(kOffScan + kU32N);
constexpr size_t kOffKAlt = align256(kOffRunStart + kU32N);
constexpr size_t kOffVAlt = align256(kOffKAlt + kU32N);
constexpr size_t kOffHist = align256(kOffVAlt + kU32N);
constexpr size_t kOffRowTotal = align256(kOffHist + sizeof(uint32_t) * 256 * kNaSortBlocks);
constexpr size_t kOffBlockSums = align256(kOffRowTotal + sizeof(uint32_t) * 256);
constexpr size_t kOffEnd = align256(kOffBlockSums + sizeof(uint32_t) * (kNaScanBlocks + 16));
static_assert(kOffEnd <= kNoAllocBytes, "no-alloc scratch layout exceeds the static array");

std::mutex g_noalloc_mu;
unsigned char* g_noalloc_dev_ptr[kNoAllocMaxDevices] = {};

// Device or managed memory (cudaPointerGetAttributes allocates nothing).
bool is_device_pointer(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

__global__ void k_noalloc_set_n(int* p, int v) {
    if (threadIdx.x == 0) *p = v;
}

// Device address of g_noalloc_scratch on the current device (resolved once).
cudaError_t noalloc_scratch(unsigned char** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_dev_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_dev_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_dev_ptr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace vmp

using namespace vmp;

extern "C" vmp_status vmp_downsample_noalloc(const vmp_point* d_in, int n, double leaf, vmp_point* d_out,
                                             int* n_out, void* cuda_stream) {
    if (!n_out || n < 0 || !(leaf > 0.0) || (n > 0 && (!d_in || !d_out))) return VMP_ERR_INVALID_ARG;
    if (n > kNoAllocMaxPoints) return VMP_ERR_CAPACITY;  // more than 65536 input points
    if (n == 0) {
        *n_out = 0;
        return VMP_OK;
    }
    const uintptr_t in_a = reinterpret_cast<uintptr_t>(d_in), out_a = reinterpret_cast<uintptr_t>(d_out);
    const uintptr_t bytes = uintptr_t(n) * sizeof(vmp_point);
    if ((in_a | out_a) & 15) return VMP_ERR_INVALID_ARG;              // float4 loads and stores
    if (in_a < out_a + bytes && out_a < in_a + bytes) return VMP_ERR_INVALID_ARG;  // overlapping buffers
    if (!is_device_pointer(d_in) || !is_device_pointer(d_out)) return VMP_ERR_INVALID_ARG;
    unsigned char* base = nullptr;
    if (noalloc_scratch(&base) != cudaSuccess) {
        cudaGetLastError();
        return VMP_ERR_CUDA;
    }
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    DScan s{};
    s.raw = nullptr;
    s.cloud = reinterpret_cast<float4*>(const_cast<vmp_point*>(d_in));  // read only
    s.down = reinterpret_cast<float4*>(d_out);
    s.d_n_raw = reinterpret_cast<int*>(base + kOffNRaw);
    s.d_n_down = reinterpret_cast<int*>(base + kOffNDown);
    s.ds_params = reinterpret_cast<int*>(base + kOffParams);
    s.blk_minmax = reinterpret_cast<float*>(base + kOffMinMax);
    s.sort_k = reinterpret_cast<uint32_t*>(base + kOffSortK);
    s.sort_v = reinterpret_cast<uint32_t*>(base + kOffSortV);
    s.flags = reinterpret_cast<uint32_t*>(base + kOffFlags);
    s.scan_out = reinterpret_cast<uint32_t*>(base + kOffScan);
    s.run_start = reinterpret_cast<uint32_t*>(base + kOffRunStart);
    s.max_pts = kNoAllocMaxPoints;
    SortScratch ss{};
    ss.k_alt = reinterpret_cast<uint32_t*>(base + kOffKAlt);
    ss.v_alt = reinterpret_cast<uint32_t*>(base + kOffVAlt);
    ss.hist = reinterpret_cast<uint32_t*>(base + kOffHist);
    ss.row_total = reinterpret_cast<uint32_t*>(base + kOffRowTotal);
    ss.n_max = kNoAllocMaxPoints;
    ss.blocks = kNaSortBlocks;
    ScanScratch sc{};
    sc.block_sums = reinterpret_cast<uint32_t*>(base + kOffBlockSums);
    sc.n_max = kNoAllocMaxPoints;
    sc.blocks = kNaScanBlocks;
    VMP_NOTE_LAUNCH(); k_noalloc_set_n<<<1, 32, 0, st>>>(s.d_n_raw, n);
    launch_downsample(s, n, leaf, ss, sc, st);
    if (cudaGetLastError() != cudaSuccess) return VMP_ERR_CUDA;
    if (cudaMemcpyAsync(n_out, s.d_n_down, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return VMP_ERR_CUDA;
    }
    return VMP_OK;
}
