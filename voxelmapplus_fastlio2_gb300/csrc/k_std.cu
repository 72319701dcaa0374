// Plane voxels of a key cloud for the STD loop-closure descriptor
// (std_desc::STDManager::buildVoxels, std_matcher/src/std_manager/
// descriptor.cpp:70-122): voxelise the cloud (VoxelKey::index, floor of
// p / voxel_size, descriptor.cpp:44-49), accumulate per voxel the FP64 sum
// and sum of outer products in cloud order, and for voxels with more than
// voxel_min_point points form mean, C = ppt / n - mean mean^T, its eigen
// decomposition and the plane test lambda_min < voxel_plane_thresh.
//
// On the device: packed 63-bit keys, a stable LSD radix sort of the point
// indices by key (low word, then high word), run heads and a scan give the
// voxels in key order with their points in cloud order; one thread per voxel
// then sums its points in that order (the reference's sums, bit for bit) and
// decomposes C (the symmetric Jacobi solver: the reference's general
// EigenSolver returns the same eigenvalues of a symmetric matrix up to
// rounding, its eigenvectors up to sign).
#include <cmath>
#include <vector>

#include "kernels.cuh"

namespace vmp {
namespace {

__global__ void k_std_keys(const float* __restrict__ pts, int stride, int n, double vs, double inv,
                           uint32_t* key_lo, uint32_t* key_hi, uint32_t* idx, unsigned int* err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double p[3] = {(double)pts[(size_t)i * stride], (double)pts[(size_t)i * stride + 1],
                             (double)pts[(size_t)i * stride + 2]};
        int64_t k[3];
        if (!voxel_index(p, vs, inv, k)) atomicOr(err, 1u);
        const uint64_t pk = pack_key(k[0], k[1], k[2]);
        key_lo[i] = (uint32_t)pk;
        key_hi[i] = (uint32_t)(pk >> 32);
        idx[i] = (uint32_t)i;
    }
}
__global__ void k_std_permute(const uint32_t* perm, const uint32_t* hi, uint32_t* hi2, const int* d_n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < *d_n; i += gridDim.x * blockDim.x) hi2[i] = hi[perm[i]];
}
// Packed keys of the points in sorted order (for the run heads and the
// voxels' keys), re-derived from the points.
__global__ void k_std_heads(const float* __restrict__ pts, int stride, const uint32_t* order, const int* d_n,
                            double vs, double inv, uint64_t* skey) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t j = order[i];
        const double p[3] = {(double)pts[(size_t)j * stride], (double)pts[(size_t)j * stride + 1],
                             (double)pts[(size_t)j * stride + 2]};
        int64_t k[3];
        voxel_index(p, vs, inv, k);
        skey[i] = pack_key(k[0], k[1], k[2]);
    }
}
__global__ void k_std_flags(const uint64_t* skey, const int* d_n, uint32_t* head) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        head[i] = (i == 0 || skey[i] != skey[i - 1]) ? 1u : 0u;
}
__global__ void k_std_starts(const uint32_t* head, const uint32_t* rank, const int* d_n, uint32_t* start) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (head[i]) start[rank[i]] = (uint32_t)i;
}

// One voxel per thread: STDManager::buildVoxels' accumulation (in cloud
// order) and per-voxel step.
__global__ void k_std_fit(const float* __restrict__ pts, int stride, const uint32_t* order, const uint64_t* skey,
                          const uint32_t* start, const int* d_runs, int n, int min_point, double plane_thresh,
                          vmp_std_voxel* out) {
    const int nr = *d_runs;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nr; v += gridDim.x * blockDim.x) {
        const int s0 = (int)start[v];
        const int s1 = v + 1 < nr ? (int)start[v + 1] : n;
        vmp_std_voxel o;
        int64_t kx, ky, kz;
        unpack_key(skey[s0], kx, ky, kz);
        o.key[0] = kx;
        o.key[1] = ky;
        o.key[2] = kz;
        o.n = s1 - s0;
        double sum[3] = {0.0, 0.0, 0.0}, ppt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int q = s0; q < s1; ++q) {
            const uint32_t j = order[q];
            const double p[3] = {(double)pts[(size_t)j * stride], (double)pts[(size_t)j * stride + 1],
                                 (double)pts[(size_t)j * stride + 2]};
            for (int a = 0; a < 3; ++a) sum[a] += p[a];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) ppt[a * 3 + b] += p[a] * p[b];
        }
        for (int a = 0; a < 3; ++a) o.sum[a] = sum[a];
        for (int a = 0; a < 9; ++a) o.ppt[a] = ppt[a];
        o.valid = o.n > min_point ? 1 : 0;
        o.is_plane = 0;
        for (int a = 0; a < 3; ++a) o.mean[a] = 0.0, o.lamdas[a] = 0.0;
        for (int a = 0; a < 9; ++a) o.norms[a] = 0.0;
        if (o.valid) {
            const double dn = (double)o.n;
            double mean[3], C[9], ev[3], E[9];
            for (int a = 0; a < 3; ++a) mean[a] = sum[a] / dn;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) C[a * 3 + b] = ppt[a * 3 + b] / dn - mean[a] * mean[b];
            eig_sym3<double>(C, ev, E);
            for (int a = 0; a < 3; ++a) o.mean[a] = mean[a];
            if (ev[0] < plane_thresh) {
                o.is_plane = 1;
                for (int a = 0; a < 3; ++a) o.lamdas[a] = ev[a];
                for (int a = 0; a < 9; ++a) o.norms[a] = E[a];
            }
        }
        out[v] = o;
    }
}

int grid_for_n(int n) {
    int g = (n + 255) / 256;
    return g < 1 ? 1 : (g > 152 * 8 ? 152 * 8 : g);
}

}  // namespace
}  // namespace vmp

using namespace vmp;

extern "C" vmp_status vmp_std_plane_voxels(const float* pts, int stride, int n, double voxel_size, int voxel_min_point,
                                           double voxel_plane_thresh, vmp_std_voxel* out, int max, int* n_out) {
    if (!n_out || n < 0 || stride < 3 || (n > 0 && !pts) || max < 0 || (max > 0 && !out) || !(voxel_size > 0.0))
        return VMP_ERR_INVALID_ARG;
    *n_out = 0;
    if (n == 0) return VMP_OK;
    int e2 = 0;
    const double mant = std::frexp(voxel_size, &e2);
    const double inv = mant == 0.5 ? std::ldexp(1.0, 1 - e2) : 0.0;
    cudaStream_t st = nullptr;
    SortScratch ss{};
    ScanScratch sc{};
    unsigned char* buf = nullptr;
    vmp_status rc = VMP_OK;
    const size_t N = (size_t)n + 16;
    // layout: pts copy | key_lo | key_hi | idx | hi2 | head | rank | start | skey (u64) | out | ints
    const size_t pts_b = sizeof(float) * (size_t)stride * (size_t)n;
    const size_t off_u32 = (pts_b + 255) & ~size_t(255);
    const size_t off_skey = off_u32 + ((7 * N * sizeof(uint32_t) + 255) & ~size_t(255));
    const size_t off_out = off_skey + ((N * sizeof(uint64_t) + 255) & ~size_t(255));
    const size_t off_int = off_out + ((N * sizeof(vmp_std_voxel) + 255) & ~size_t(255));
    const size_t total = off_int + 256;
    do {
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) { rc = VMP_ERR_CUDA; break; }
        if (cudaMalloc(&buf, total) != cudaSuccess || sort_scratch_alloc(ss, n) != cudaSuccess ||
            scan_scratch_alloc(sc, n) != cudaSuccess) {
            rc = VMP_ERR_OUT_OF_MEMORY;
            break;
        }
        float* d_pts = reinterpret_cast<float*>(buf);
        uint32_t* key_lo = reinterpret_cast<uint32_t*>(buf + off_u32);
        uint32_t* key_hi = key_lo + N;
        uint32_t* idx = key_hi + N;
        uint32_t* hi2 = idx + N;
        uint32_t* head = hi2 + N;
        uint32_t* rank = head + N;
        uint32_t* start = rank + N;
        uint64_t* skey = reinterpret_cast<uint64_t*>(buf + off_skey);
        vmp_std_voxel* d_out = reinterpret_cast<vmp_std_voxel*>(buf + off_out);
        int* ints = reinterpret_cast<int*>(buf + off_int);  // [0] n, [1] runs, [2] error
        int h[3] = {n, 0, 0};
        cudaError_t e = cudaMemcpyAsync(d_pts, pts, pts_b, cudaMemcpyDefault, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ints, h, sizeof(h), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) { rc = VMP_ERR_CUDA; break; }
        const int g = grid_for_n(n);
        VMP_NOTE_LAUNCH();
        k_std_keys<<<g, 256, 0, st>>>(d_pts, stride, n, voxel_size, inv, key_lo, key_hi, idx,
                                      reinterpret_cast<unsigned int*>(ints + 2));
        // stable LSD order by the 64-bit key: low word, then high word
        radix_sort_pairs(key_lo, idx, ints, 32, ss, st);
        VMP_NOTE_LAUNCH(); k_std_permute<<<g, 256, 0, st>>>(idx, key_hi, hi2, ints);
        radix_sort_pairs(hi2, idx, ints, 32, ss, st);
        VMP_NOTE_LAUNCH(); k_std_heads<<<g, 256, 0, st>>>(d_pts, stride, idx, ints, voxel_size, inv, skey);
        VMP_NOTE_LAUNCH(); k_std_flags<<<g, 256, 0, st>>>(skey, ints, head);
        exclusive_scan_u32(head, rank, ints, ints + 1, sc, st);
        VMP_NOTE_LAUNCH(); k_std_starts<<<g, 256, 0, st>>>(head, rank, ints, start);
        VMP_NOTE_LAUNCH();
        k_std_fit<<<grid_for_n(n), 128, 0, st>>>(d_pts, stride, idx, skey, start, ints + 1, n, voxel_min_point,
                                                voxel_plane_thresh, d_out);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(h, ints, sizeof(h), cudaMemcpyDeviceToHost, st) !=
                                                     cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = VMP_ERR_CUDA;
            break;
        }
        if (h[2]) { rc = VMP_ERR_KEY_RANGE; break; }
        const int nr = h[1];
        *n_out = nr;
        const int m = nr < max ? nr : max;
        if (m > 0 && (cudaMemcpyAsync(out, d_out, sizeof(vmp_std_voxel) * (size_t)m, cudaMemcpyDeviceToHost, st) !=
                          cudaSuccess ||
                      cudaStreamSynchronize(st) != cudaSuccess)) {
            rc = VMP_ERR_CUDA;
            break;
        }
    } while (false);
    if (rc != VMP_OK) cudaGetLastError();
    if (st) cudaStreamSynchronize(st);
    if (buf) cudaFree(buf);
    sort_scratch_free(ss);
    scan_scratch_free(sc);
    if (st) cudaStreamDestroy(st);
    return rc;
}
