// Per-point stages of one scan:
//   k_time_keys / gather   std::sort of the package cloud by time   lio_builder.cpp:75-76
//   downsample             pcl::VoxelGrid leaf-centroid filter     lio_builder.cpp:215-223
//                          (PCL 1.10 VoxelGrid::applyFilter: float leaf grid,
//                          idx = i + j*div_x + k*div_x*div_y, sort by idx,
//                          per-leaf float sum in sorted order / count)
//   k_body_cov             lio::calcBodyCov                        commons.cpp:18-45
//   k_map_batch            lidarToWorld (float 4x4, PCL SSE se3 order) +
//                          the world covariance of each inserted point
//                                                                  lio_builder.cpp:155-163, 185-211, 231-246
// The sorts are stable, so equal keys keep their input order (the reference's
// std::sort leaves that order unspecified).
#include <cmath>

#include "kernels.cuh"

namespace vmp {

constexpr int kPtThreads = 256;

__device__ inline uint32_t float_order_key(float f) {
    uint32_t b = __float_as_uint(f);
    if (b == 0x80000000u) b = 0u;  // -0 sorts with +0
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Also records whether the keys are out of order anywhere: point clouds of
// spinning and Livox sensors come in time order, and then the stable time
// sort is the identity and its passes return at once.
__global__ void k_time_keys(const float4* __restrict__ raw, const int* d_n, uint32_t* k, uint32_t* v,
                            int* unsorted) {
    const int n = *d_n;
    bool down = false;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t ki = float_order_key(raw[i].w);
        k[i] = ki;
        v[i] = (uint32_t)i;
        if (i > 0 && ki < float_order_key(raw[i - 1].w)) down = true;
    }
    if (__any_sync(0xffffffffu, down) && (threadIdx.x & 31) == 0) *unsorted = 1;
}
// Applies the time-sort permutation to the points and their intensities.
__global__ void k_gather4(const float4* __restrict__ src, const float* __restrict__ src_int,
                          const uint32_t* __restrict__ perm, const int* d_n, float4* __restrict__ dst,
                          float* __restrict__ dst_int) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t j = perm[i];
        dst[i] = src[j];
        dst_int[i] = src_int[j];
    }
}

static int grid_for(int n_max) {
    int b = (n_max + kPtThreads - 1) / kPtThreads;
    if (b > 152 * 8) b = 152 * 8;
    return b < 1 ? 1 : served_grid(b);
}

void launch_time_sort(DScan& s, int n_max, SortScratch& ss, cudaStream_t st) {
    int g = grid_for(n_max);
    VMP_NOTE_LAUNCH();
    k_time_keys<<<g, kPtThreads, 0, st>>>(s.raw, s.d_n_raw, s.sort_k, s.sort_v, &s.hdr->time_unsorted);
    radix_sort_pairs(s.sort_k, s.sort_v, s.d_n_raw, 32, ss, st, &s.hdr->time_unsorted);
    VMP_NOTE_LAUNCH(); k_gather4<<<g, kPtThreads, 0, st>>>(s.raw, s.raw_int, s.sort_v, s.d_n_raw, s.cloud, s.cloud_int);
}

// ---------------------------------------------------------------- downsample

__global__ void k_minmax_partial(const float4* __restrict__ c, const int* d_n, float* blk) {
    __shared__ float red[6][kPtThreads];
    const int n = *d_n;
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = c[i];
        mn[0] = fminf(mn[0], p.x); mn[1] = fminf(mn[1], p.y); mn[2] = fminf(mn[2], p.z);
        mx[0] = fmaxf(mx[0], p.x); mx[1] = fmaxf(mx[1], p.y); mx[2] = fmaxf(mx[2], p.z);
    }
    for (int a = 0; a < 3; ++a) { red[a][threadIdx.x] = mn[a]; red[3 + a][threadIdx.x] = mx[a]; }
    __syncthreads();
    for (int o = kPtThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            for (int a = 0; a < 3; ++a) {
                red[a][threadIdx.x] = fminf(red[a][threadIdx.x], red[a][threadIdx.x + o]);
                red[3 + a][threadIdx.x] = fmaxf(red[3 + a][threadIdx.x], red[3 + a][threadIdx.x + o]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 6) blk[blockIdx.x * 6 + threadIdx.x] = red[threadIdx.x][0];
}

// params: [0] overflow flag, [1..3] min_b, [4..6] div_b, [7] mul1, [8] mul2,
// float bits: [9] inv
__global__ void k_ds_params(const float* blk, int nblk, float leaf_f, int* params, const int* d_n) {
    if (threadIdx.x != 0) return;
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int b = 0; b < nblk; ++b)
        for (int a = 0; a < 3; ++a) { mn[a] = fminf(mn[a], blk[b * 6 + a]); mx[a] = fmaxf(mx[a], blk[b * 6 + 3 + a]); }
    float inv = 1.0f / leaf_f;
    int64_t d[3];
    for (int a = 0; a < 3; ++a) d[a] = (int64_t)((mx[a] - mn[a]) * inv) + 1;
    params[0] = (*d_n == 0) ? 2 : ((d[0] * d[1] * d[2] > (int64_t)2147483647) ? 1 : 0);
    int minb[3], maxb[3];
    for (int a = 0; a < 3; ++a) {
        minb[a] = (int)floorf(mn[a] * inv);
        maxb[a] = (int)floorf(mx[a] * inv);
        params[1 + a] = minb[a];
        params[4 + a] = maxb[a] - minb[a] + 1;
    }
    params[7] = params[4];
    params[8] = (int)((uint32_t)params[4] * (uint32_t)params[5]);
    params[9] = __float_as_int(inv);
}

__global__ void k_leaf_idx(const float4* __restrict__ c, const int* d_n, const int* __restrict__ params,
                           uint32_t* k, uint32_t* v) {
    const int n = *d_n;
    if (params[0] != 0) return;
    const float inv = __int_as_float(params[9]);
    const float fb0 = (float)params[1], fb1 = (float)params[2], fb2 = (float)params[3];
    const uint32_t mul1 = (uint32_t)params[7], mul2 = (uint32_t)params[8];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = c[i];
        int i0 = (int)(floorf(p.x * inv) - fb0);
        int i1 = (int)(floorf(p.y * inv) - fb1);
        int i2 = (int)(floorf(p.z * inv) - fb2);
        k[i] = (uint32_t)i0 + (uint32_t)i1 * mul1 + (uint32_t)i2 * mul2;
        v[i] = (uint32_t)i;
    }
}

__global__ void k_run_heads(const uint32_t* __restrict__ k, const int* d_n, const int* params, uint32_t* flags) {
    const int n = *d_n;
    const bool grid_ok = params[0] == 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        flags[i] = (grid_ok && (i == 0 || k[i] != k[i - 1])) ? 1u : 0u;
}

__global__ void k_run_starts(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ rank, const int* d_n,
                             const int* params, uint32_t* run_start, int* d_runs) {
    const int n = (params[0] == 0) ? *d_n : 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (flags[i]) run_start[rank[i]] = (uint32_t)i;
    if (blockIdx.x == 0 && threadIdx.x == 0) run_start[*d_runs] = (uint32_t)n;
}

__global__ void k_centroid(const float4* __restrict__ c, const uint32_t* __restrict__ perm,
                           const uint32_t* __restrict__ run_start, const int* d_runs, const int* params,
                           const int* d_n, float4* down, int* d_n_down) {
    if (params[0] != 0) {
        // PCL: the leaf grid would overflow 32-bit indices -> output = input
        const int n = (params[0] == 1) ? *d_n : 0;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) down[i] = c[i];
        if (blockIdx.x == 0 && threadIdx.x == 0) *d_n_down = n;
        return;
    }
    const int runs = *d_runs;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < runs; r += gridDim.x * blockDim.x) {
        uint32_t s = run_start[r], e = run_start[r + 1];
        float sx = 0.f, sy = 0.f, sz = 0.f, stt = 0.f;
        for (uint32_t j = s; j < e; ++j) {
            float4 p = c[perm[j]];
            sx = sx + p.x; sy = sy + p.y; sz = sz + p.z; stt = stt + p.w;
        }
        float cnt = (float)(e - s);
        down[r] = make_float4(sx / cnt, sy / cnt, sz / cnt, stt / cnt);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_n_down = runs;
}

void launch_downsample(DScan& s, int n_max, double leaf, SortScratch& ss, ScanScratch& sc, cudaStream_t st) {
    int g = grid_for(n_max);
    VMP_NOTE_LAUNCH(); k_minmax_partial<<<kMinMaxBlocks, kPtThreads, 0, st>>>(s.cloud, s.d_n_raw, s.blk_minmax);
    VMP_NOTE_LAUNCH(); k_ds_params<<<1, 32, 0, st>>>(s.blk_minmax, kMinMaxBlocks, (float)leaf, s.ds_params, s.d_n_raw);
    VMP_NOTE_LAUNCH(); k_leaf_idx<<<g, kPtThreads, 0, st>>>(s.cloud, s.d_n_raw, s.ds_params, s.sort_k, s.sort_v);
    radix_sort_pairs(s.sort_k, s.sort_v, s.d_n_raw, 32, ss, st);
    VMP_NOTE_LAUNCH(); k_run_heads<<<g, kPtThreads, 0, st>>>(s.sort_k, s.d_n_raw, s.ds_params, s.flags);
    int* d_runs = s.ds_params + 12;
    exclusive_scan_u32(s.flags, s.scan_out, s.d_n_raw, d_runs, sc, st);
    VMP_NOTE_LAUNCH(); k_run_starts<<<g, kPtThreads, 0, st>>>(s.flags, s.scan_out, s.d_n_raw, s.ds_params, s.run_start, d_runs);
    VMP_NOTE_LAUNCH(); k_centroid<<<g, kPtThreads, 0, st>>>(s.cloud, s.sort_v, s.run_start, d_runs, s.ds_params, s.d_n_raw, s.down,
                                         s.d_n_down);
}

__global__ void k_copy_down(const float4* __restrict__ c, const int* d_n, float4* down, int* d_n_down) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) down[i] = c[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_n_down = n;
}
void launch_copy_down(DScan& s, int n_max, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_copy_down<<<grid_for(n_max), kPtThreads, 0, st>>>(s.cloud, s.d_n_raw, s.down, s.d_n_down);
}

// ---------------------------------------------------------------- calcBodyCov
__device__ inline void normalize3(double* v) {
    double n = dot3(v, v);
    if (n > 0.0) {
        double r = sqrt(n);
        if (div_recip_ok(r)) {  // the three divisions by r, correctly rounded
            const double y = 1.0 / r;
            v[0] = div_by_recip(v[0], r, y); v[1] = div_by_recip(v[1], r, y); v[2] = div_by_recip(v[2], r, y);
        } else {
            v[0] = v[0] / r; v[1] = v[1] / r; v[2] = v[2] / r;
        }
    }
}

// lio::calcBodyCov; pb is fixed in place when z == 0 (commons.cpp:20-23).
__device__ void calc_body_cov(double* pb, double range_inc, double s, double* cov) {
    if (pb[2] == 0) pb[2] = 0.001;
    double range = sqrt(pb[0] * pb[0] + pb[1] * pb[1] + pb[2] * pb[2]);
    double range_var = range_inc * range_inc;
    double dvar[4] = {s * s, 0.0, 0.0, s * s};
    double d[3] = {pb[0], pb[1], pb[2]};
    normalize3(d);
    double dh[9] = {0, -d[2], d[1], d[2], 0, -d[0], -d[1], d[0], 0};
    double b1[3] = {1, 1, -(d[0] + d[1]) / d[2]};
    normalize3(b1);
    double b2[3] = {b1[1] * d[2] - b1[2] * d[1], b1[2] * d[0] - b1[0] * d[2], b1[0] * d[1] - b1[1] * d[0]};
    normalize3(b2);
    double N[6] = {b1[0], b2[0], b1[1], b2[1], b1[2], b2[2]};
    // A = (range [d]x) N and A dvar without the products with the zero
    // diagonal of [d]x and the zero off-diagonal of dvar: the dense sums less
    // their +-0 terms (the oracle evaluates it alike)
    double A[6], AD[6], AT[6], C1[9], C2[9], dr[3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 2; ++j) {
            const int k0 = i == 0 ? 1 : 0, k1 = i == 2 ? 1 : 2;
            A[i * 2 + j] = (range * dh[i * 3 + k0]) * N[k0 * 2 + j] + (range * dh[i * 3 + k1]) * N[k1 * 2 + j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 2; ++j) AD[i * 2 + j] = A[i * 2 + j] * dvar[j * 3];
    tr<3, 2>(A, AT);
    mm<3, 2, 3>(AD, AT, C2);
    for (int i = 0; i < 3; ++i) dr[i] = d[i] * range_var;
    mm<3, 1, 3>(dr, d, C1);
    for (int i = 0; i < 9; ++i) cov[i] = C1[i] + C2[i];
}

__global__ void k_body_cov(const float4* __restrict__ down, const int* d_n, double range_inc, double sin_deg,
                           double* pl, double* covl) {
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = down[i];
        double pb[3] = {(double)q.x, (double)q.y, (double)q.z};
        double cov[9];
        calc_body_cov(pb, range_inc, sin_deg, cov);
        pl[i * 3] = pb[0]; pl[i * 3 + 1] = pb[1]; pl[i * 3 + 2] = pb[2];
#pragma unroll
        for (int k = 0; k < 9; ++k) covl[i * 9 + k] = cov[k];
    }
}
void launch_body_cov(DScan& s, int n_max, double range_inc, double sin_deg, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_body_cov<<<grid_for(n_max), kPtThreads, 0, st>>>(s.down, s.d_n_down, range_inc, sin_deg, s.pl, s.covl);
}

// Test hook: calcBodyCov on the device for explicit points.
__global__ void k_body_cov_check(const double* pts, int n, double range_inc, double sin_deg, double* pts_out,
                                 double* cov) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double pb[3] = {pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]};
        double c[9];
        calc_body_cov(pb, range_inc, sin_deg, c);
        for (int k = 0; k < 3; ++k) pts_out[i * 3 + k] = pb[k];
        for (int k = 0; k < 9; ++k) cov[i * 9 + k] = c[k];
    }
}

// Test hook: [p]x M [p]x^T (hat_sandwich) for explicit points and matrices.
__global__ void k_hat_sandwich_check(const double* pts, const double* M, int n, double* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double o[9];
        hat_sandwich(pts + 3 * (size_t)i, M + 9 * (size_t)i, o);
        for (int k = 0; k < 9; ++k) out[i * 9 + k] = o[k];
    }
}

// ---------------------------------------------------------------- map batch
// Register budget: 3 CTAs per SM (80 registers instead of 124), for the
// register file it leaves to other streams' kernels (served scans/s +1.4 %).
__global__ void __launch_bounds__(kPtThreads, 3) k_map_batch(const DFilter* __restrict__ f, const float4* __restrict__ pts, const int* d_n,
                            const double* __restrict__ pl, const double* __restrict__ covl, int full,
                            double range_inc, double sin_deg, double* bpts, double* bcov, int* d_n_batch) {
    __shared__ float sR[9], sT[3];
    __shared__ double rwl[9], prr[9], ppp[9];
    const int n = *d_n;
    if (blockIdx.x > 0 && (long long)blockIdx.x * blockDim.x >= n) return;  // past the points: no setup either
    // R_wl = rot rot_ext and p_wl = rot pos_ext + pos (one entry per
    // thread), their float casts, and the P blocks
    const int t = threadIdx.x;
    if (t < 9) {
        rwl[t] = mm3_entry(f->x.rot, f->x.rot_ext, t);
        sR[t] = (float)rwl[t];
    } else if (t < 12) {
        sT[t - 9] = (float)(m3v_entry(f->x.rot, f->x.pos_ext, t - 9) + f->x.pos[t - 9]);
    } else if (t >= 32 && t < 41) {
        const int i = (t - 32) / 3, j = (t - 32) % 3;
        prr[i * 3 + j] = f->P[(3 + i) * 23 + 3 + j];
        ppp[i * 3 + j] = f->P[i * 23 + j];
    }
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = pts[i];
        for (int r = 0; r < 3; ++r) {
            float w = q.x * sR[r * 3] + (q.y * sR[r * 3 + 1] + (q.z * sR[r * 3 + 2] + sT[r]));
            bpts[i * 3 + r] = (double)w;
        }
        double pb[3], cl[9];
        if (full) {
            pb[0] = (double)q.x; pb[1] = (double)q.y; pb[2] = (double)q.z;
            calc_body_cov(pb, range_inc, sin_deg, cl);
        } else {
            for (int a = 0; a < 3; ++a) pb[a] = pl[i * 3 + a];
            for (int a = 0; a < 9; ++a) cl[a] = covl[i * 9 + a];
        }
        double T1[9], T2[9], rT[9], T4[9];
        mm<3, 3, 3>(rwl, cl, T1);
        tr<3, 3>(rwl, rT);
        mm<3, 3, 3>(T1, rT, T2);
        hat_sandwich(pb, prr, T4);
        for (int k = 0; k < 9; ++k) bcov[i * 9 + k] = (T2[k] + T4[k]) + ppp[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_n_batch = n;
}

void launch_map_batch(DFilter* f, DScan& s, int n_max, bool from_full_cloud, double range_inc, double sin_deg,
                      cudaStream_t st) {
    VMP_NOTE_LAUNCH();
    if (from_full_cloud)
        k_map_batch<<<grid_for(n_max), kPtThreads, 0, st>>>(f, s.cloud, s.d_n_raw, nullptr, nullptr, 1, range_inc,
                                                             sin_deg, s.bpts, s.bcov, s.d_n_batch);
    else
        k_map_batch<<<grid_for(n_max), kPtThreads, 0, st>>>(f, s.down, s.d_n_down, s.pl, s.covl, 0, range_inc,
                                                             sin_deg, s.bpts, s.bcov, s.d_n_batch);
}

// ---------------------------------------------------------------- Livox decode
// livox2pcl (src/utils.cpp:3-28) as a stream compaction: a point passes the
// line / tag test, then every filter_num-th passing point (counted from 0)
// goes on to the range test, |p|^2 summed in float as in the reference and
// compared in double.
__device__ inline bool livox_line_tag_ok(const vmp_livox_point& p) {
    const unsigned t = p.tag & 0x30u;
    return p.line < 4 && (t == 0x10u || t == 0x00u);
}
__global__ void k_livox_valid(const vmp_livox_point* __restrict__ in, int n, uint32_t* __restrict__ valid,
                              int* d_n) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_n = n;  // count for the scans that follow
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        valid[i] = livox_line_tag_ok(in[i]) ? 1u : 0u;
}
__global__ void k_livox_keep(const vmp_livox_point* __restrict__ in, int n, const uint32_t* __restrict__ valid,
                             const uint32_t* __restrict__ rank, unsigned filter_num, double rmin2, double rmax2,
                             uint32_t* __restrict__ keep) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t k = 0;
        if (valid[i] && rank[i] % filter_num == 0u) {
            const vmp_livox_point p = in[i];
            const float sq = p.x * p.x + p.y * p.y + p.z * p.z;
            const double d = (double)sq;
            k = (d > rmin2 && d < rmax2) ? 1u : 0u;
        }
        keep[i] = k;
    }
}
// filter_num == 1 (every point that passes the line / tag test goes on to
// the range test): both tests in one pass, one scan instead of two.
__global__ void k_livox_keep1(const vmp_livox_point* __restrict__ in, int n, double rmin2, double rmax2,
                              uint32_t* __restrict__ keep, int* d_n) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_n = n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const vmp_livox_point p = in[i];
        uint32_t k = 0;
        if (livox_line_tag_ok(p)) {
            const float sq = p.x * p.x + p.y * p.y + p.z * p.z;
            const double d = (double)sq;
            k = (d > rmin2 && d < rmax2) ? 1u : 0u;
        }
        keep[i] = k;
    }
}
// The kept points in order; the thread of the last one also writes its time
// (ms, as float bits) to *last_t_bits, so the host reads count and time at once.
__global__ void k_livox_scatter(const vmp_livox_point* __restrict__ in, int n, const uint32_t* __restrict__ keep,
                                const uint32_t* __restrict__ pos, const int* __restrict__ d_total,
                                float4* __restrict__ raw, float* __restrict__ raw_int, int* last_t_bits) {
    const uint32_t total = (uint32_t)*d_total;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        const vmp_livox_point p = in[i];
        const uint32_t o = pos[i];
        const float t = (float)p.offset_time / 1000000.0f;  // ns -> ms
        raw[o] = make_float4(p.x, p.y, p.z, t);
        raw_int[o] = (float)p.reflectivity;
        if (o + 1u == total) *last_t_bits = __float_as_int(t);
    }
}

void launch_livox_decode(DScan& s, const vmp_livox_point* d_in, int n, int filter_num, double range_min,
                         double range_max, ScanScratch& sc, cudaStream_t st) {
    const int g = grid_for(n);
    if (filter_num == 1) {
        VMP_NOTE_LAUNCH();
        k_livox_keep1<<<g, kPtThreads, 0, st>>>(d_in, n, range_min * range_min, range_max * range_max, s.sort_k,
                                                s.d_n_in);
    } else {
        VMP_NOTE_LAUNCH(); k_livox_valid<<<g, kPtThreads, 0, st>>>(d_in, n, s.flags, s.d_n_in);
        exclusive_scan_u32(s.flags, s.scan_out, s.d_n_in, s.d_n_in + 1, sc, st);
        VMP_NOTE_LAUNCH();
        k_livox_keep<<<g, kPtThreads, 0, st>>>(d_in, n, s.flags, s.scan_out, (unsigned)filter_num,
                                               range_min * range_min, range_max * range_max, s.sort_k);
    }
    exclusive_scan_u32(s.sort_k, s.sort_v, s.d_n_in, s.d_n_raw, sc, st);
    VMP_NOTE_LAUNCH();
    k_livox_scatter<<<g, kPtThreads, 0, st>>>(d_in, n, s.sort_k, s.sort_v, s.d_n_raw, s.raw, s.raw_int,
                                              s.d_n_in + 3);
}

// ---------------------------------------------------------------- output clouds
// lidarToBody / lidarToWorld (lio_builder.cpp:155-173): the undistorted cloud
// under a float 4x4 transform, in pcl::transformPointCloud's operation order.
__global__ void k_output_cloud(const DFilter* __restrict__ f, const float4* __restrict__ cloud,
                               const float* __restrict__ cloud_int, int n, int frame, float4* __restrict__ out,
                               float* __restrict__ out_int) {
    __shared__ float sR[9], sT[3];
    if (threadIdx.x == 0) {
        const DState& x = f->x;
        if (frame == 0) {
            for (int a = 0; a < 9; ++a) sR[a] = (float)x.rot_ext[a];
            for (int a = 0; a < 3; ++a) sT[a] = (float)x.pos_ext[a];
        } else {
            double rwl[9], rp[3];
            mm<3, 3, 3>(x.rot, x.rot_ext, rwl);
            m3v(x.rot, x.pos_ext, rp);
            for (int a = 0; a < 9; ++a) sR[a] = (float)rwl[a];
            for (int a = 0; a < 3; ++a) sT[a] = (float)(rp[a] + x.pos[a]);
        }
    }
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 q = cloud[i];
        float w[3];
        for (int r = 0; r < 3; ++r) w[r] = q.x * sR[r * 3] + (q.y * sR[r * 3 + 1] + (q.z * sR[r * 3 + 2] + sT[r]));
        out[i] = make_float4(w[0], w[1], w[2], q.w);
        if (out_int) out_int[i] = cloud_int[i];
    }
}

void launch_output_cloud(const DFilter* f, const DScan& s, int n, int frame, float4* out, float* out_int,
                         cudaStream_t st) {
    if (n <= 0) return;
    VMP_NOTE_LAUNCH(); k_output_cloud<<<grid_for(n), kPtThreads, 0, st>>>(f, s.cloud, s.cloud_int, n, frame, out, out_int);
}

}  // namespace vmp

// Test hook (host arrays): lio::calcBodyCov (commons.cpp:18-45) of n points on
// the device, with the angle noise in degrees as vmp_config.angle_cov.
extern "C" vmp_status vmp_test_body_cov(const double* pts, int n, double range_inc, double degree_inc,
                                        double* pts_out, double* cov) {
    if (n < 0 || (n > 0 && (!pts || !pts_out || !cov))) return VMP_ERR_INVALID_ARG;
    if (n == 0) return VMP_OK;
    double* d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * 15 * (size_t)n) != cudaSuccess) return VMP_ERR_OUT_OF_MEMORY;
    const double sin_deg = std::sin(degree_inc * 0.017453293);  // as vmp_create forms it
    cudaError_t e = cudaMemcpy(d, pts, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        VMP_NOTE_LAUNCH();
        vmp::k_body_cov_check<<<(n + 255) / 256 < 1216 ? (n + 255) / 256 : 1216, 256>>>(
            d, n, range_inc, sin_deg, d + 3 * (size_t)n, d + 6 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(pts_out, d + 3 * (size_t)n, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(cov, d + 6 * (size_t)n, sizeof(double) * 9 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return VMP_ERR_CUDA;
    }
    return VMP_OK;
}

extern "C" vmp_status vmp_test_hat_sandwich(const double* pts, const double* M, int n, double* out) {
    if (n < 0 || (n > 0 && (!pts || !M || !out))) return VMP_ERR_INVALID_ARG;
    if (n == 0) return VMP_OK;
    double* d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * 21 * (size_t)n) != cudaSuccess) return VMP_ERR_OUT_OF_MEMORY;
    cudaError_t e = cudaMemcpy(d, pts, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + 3 * (size_t)n, M, sizeof(double) * 9 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        VMP_NOTE_LAUNCH();
        vmp::k_hat_sandwich_check<<<(n + 255) / 256 < 1216 ? (n + 255) / 256 : 1216, 256>>>(
            d, d + 3 * (size_t)n, n, d + 12 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + 12 * (size_t)n, sizeof(double) * 9 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return VMP_ERR_CUDA;
    }
    return VMP_OK;
}
