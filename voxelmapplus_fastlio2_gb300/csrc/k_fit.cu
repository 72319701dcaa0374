// Batched plane fitting (vmp_fit_planes): VoxelGrid::updatePlane
// (voxel_map.cpp:97-136) over every point of many voxels at once, as
// VoxelMap::build fits each voxel after adding all its points
// (voxel_map.cpp:200-230), in three arithmetic modes:
//   FP64   the reference's FP64 arithmetic, sums formed in parallel;
//   FP32   plain FP32 throughout, on world coordinates;
//   FP32C  FP32 with compensated covariance sums: each point is taken
//          relative to its voxel's first point (a float subtraction of two
//          nearby values, free of cancellation error) and the sums of the
//          coordinates and of their products are compensated (Kahan's
//          summation per lane, Knuth's error-free TwoSum where lanes
//          combine); the plane terms use the same relative coordinates.
//
// One launch per call (k_fit): a warp fits 32 consecutive voxels --
//   pass 1   voxel by voxel over all lanes: sums of p and p p^T
//            (lane-strided, four points per lane in flight), reduced across
//            the warp by a transpose reduction (16 shuffles for 9 sums
//            instead of 45) and handed to the lane that owns the voxel;
//   finalize one voxel per lane: mean, C = ppt / n - mean mean^T, the eigen
//            decomposition, the plane test, the normal's sign flip, the
//            per-voxel factors of J;
//   pass 2   voxel by voxel again for the planes: the per-point terms of
//            J cov J^T in factored form, reduced like the sums; lane e < 21
//            forms entry e of the 6x6 and writes it.
//
// Factored J cov J^T.  With evecs E = [n v1 v2], d = p - mean, a = n . d,
// b_m = v_m . d and k_m = 1 / (n_pts (l0 - l_m)), row m of updatePlane's F is
// f_m^T with f_m = k_m (a v_m + b_m n) (m = 1, 2; row 0 is zero), so the top
// block of J is A = E F = v1 f1^T + v2 f2^T and, with g_m = cov f_m and
// s_mk = f_m . g_k,
//   A cov A^T = s11 v1 v1^T + s12 (v1 v2^T + v2 v1^T) + s22 v2 v2^T,
//   A cov / n = (v1 g1^T + v2 g2^T) / n,      cov / n^2 (bottom right).
// Summed over the points, 15 numbers per voxel (S11 S12 S22, G1, G2 and the
// sum of the point covariances) give the whole 6x6: the reference's sums,
// regrouped (rounding-level differences in FP64).
#include <mutex>

#include "kernels.cuh"

namespace vmp {
namespace {

constexpr int FIT_FP64 = VMP_FIT_FP64, FIT_FP32 = VMP_FIT_FP32, FIT_FP32C = VMP_FIT_FP32C;
constexpr int kFitWarps = 8;  // warps per CTA in the warp-per-voxel kernels

struct FitArgs {
    const float* x;
    const float* y;
    const float* z;
    const float* c[6];  // point covariance: xx xy xz yy yz zz
    const long long* off;
    long long n_pts;
    int n_vox;
    int min_pts;
    double plane_thresh;
    vmp_fit_rec* out;
};

// A compensated float sum: value s plus the running error c.
struct F2 {
    float s, c;
};
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}
__device__ __forceinline__ float shx(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shx(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ F2 shx(F2 v, int o) { return {shx(v.s, o), shx(v.c, o)}; }
__device__ __forceinline__ float comb(float a, float b) { return a + b; }
__device__ __forceinline__ double comb(double a, double b) { return a + b; }
// Combines two Kahan sums (c holds the negated error): TwoSum of the values.
__device__ __forceinline__ F2 comb(F2 a, F2 b) {
    float s, e;
    two_sum(a.s, b.s, s, e);
    return {s, (a.c + b.c) - e};
}
// Kahan's compensated summation step: c carries the negated lost low part.
__device__ __forceinline__ void acc_add(F2& a, float v) {
    const float y = v - a.c;
    const float t = a.s + y;
    a.c = (t - a.s) - y;
    a.s = t;
}
__device__ __forceinline__ double as_double(float v) { return (double)v; }
__device__ __forceinline__ double as_double(double v) { return v; }
__device__ __forceinline__ double as_double(F2 v) { return (double)v.s - (double)v.c; }
template <class V> __device__ __forceinline__ V vzero() { return V(0); }
template <> __device__ __forceinline__ F2 vzero<F2>() { return {0.f, 0.f}; }

__device__ __forceinline__ float mad(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double mad(double a, double b, double c) { return __fma_rn(a, b, c); }

// Sum of 16 per-lane values over the warp in 16 shuffles: at each level a
// lane keeps half of its values and trades the other half with its partner.
// Afterwards lanes red_lane(k) and red_lane(k) + 1 hold the total of value k.
template <class V>
__device__ __forceinline__ void transpose_reduce16(V (&v)[16], int lane) {
#pragma unroll
    for (int lvl = 0; lvl < 4; ++lvl) {
        const int o = 16 >> lvl, half = 8 >> lvl;
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int k = 0; k < half; ++k) {
            const V send = up ? v[k] : v[k + half];
            const V keep = up ? v[k + half] : v[k];
            v[k] = comb(keep, shx(send, o));
        }
    }
    v[0] = comb(v[0], shx(v[0], 1));
}
__host__ __device__ constexpr int red_lane(int k) {
    return (((k >> 3) & 1) << 4) | (((k >> 2) & 1) << 3) | (((k >> 1) & 1) << 2) | ((k & 1) << 1);
}

template <int MODE> struct FitTypes;
template <> struct FitTypes<FIT_FP64> { using T = double; using Acc = double; };
template <> struct FitTypes<FIT_FP32> { using T = float; using Acc = float; };
template <> struct FitTypes<FIT_FP32C> { using T = float; using Acc = F2; };

__device__ __forceinline__ void voxel_range(const FitArgs& a, long long v, long long& p0, long long& p1) {
    // offsets are clamped into [0, n_pts]: a malformed list gives wrong
    // records, never an access outside the point arrays
    p0 = a.off[v];
    p1 = a.off[v + 1];
    p0 = p0 < 0 ? 0 : (p0 > a.n_pts ? a.n_pts : p0);
    p1 = p1 < p0 ? p0 : (p1 > a.n_pts ? a.n_pts : p1);
}

// ---------------------------------------------------------------- one voxel
// Pass 1 over voxel [p0, p1): sums of p and p p^T (FP32C: of p - anchor),
// lane-strided with four points per lane in flight, reduced across the
// warp; afterwards lanes red_lane(k) hold sum k (as a double).
template <int MODE>
__device__ __forceinline__ double voxel_sums(const FitArgs& a, long long p0, long long p1, float ax, float ay,
                                             float az, int lane) {
    using T = typename FitTypes<MODE>::T;
    using Acc = typename FitTypes<MODE>::Acc;
    Acc acc[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[k] = vzero<Acc>();
    auto add = [&](float px, float py, float pz) {
        if constexpr (MODE == FIT_FP32C) {
            const float dx = px - ax, dy = py - ay, dz = pz - az;
            acc_add(acc[0], dx);
            acc_add(acc[1], dy);
            acc_add(acc[2], dz);
            acc_add(acc[3], dx * dx);
            acc_add(acc[4], dx * dy);
            acc_add(acc[5], dx * dz);
            acc_add(acc[6], dy * dy);
            acc_add(acc[7], dy * dz);
            acc_add(acc[8], dz * dz);
        } else {
            const T x = (T)px, y = (T)py, z = (T)pz;
            acc[0] += x;
            acc[1] += y;
            acc[2] += z;
            acc[3] = mad(x, x, acc[3]);
            acc[4] = mad(x, y, acc[4]);
            acc[5] = mad(x, z, acc[5]);
            acc[6] = mad(y, y, acc[6]);
            acc[7] = mad(y, z, acc[7]);
            acc[8] = mad(z, z, acc[8]);
        }
    };
    // four points per lane in flight while a whole round of 128 remains,
    // then one at a time (no predicated-off work for small voxels)
    long long i = p0 + lane;
    for (; i + 96 < p1; i += 128) {
        float px[4], py[4], pz[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            px[u] = __ldg(a.x + i + 32 * u);
            py[u] = __ldg(a.y + i + 32 * u);
            pz[u] = __ldg(a.z + i + 32 * u);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) add(px[u], py[u], pz[u]);
    }
    for (; i < p1; i += 32) add(__ldg(a.x + i), __ldg(a.y + i), __ldg(a.z + i));
    transpose_reduce16(acc, lane);
    return as_double(acc[0]);
}

// The per-voxel step of updatePlane from the sums: mean, C, eigen
// decomposition, plane test, sign flip; writes the record's fields except
// the plane covariance of a plane, and returns the factors of J for pass 2
// in kc: the mean the points are taken relative to (FP32C: relative to the
// first point), the unflipped normal, v1, v2, k1, k2, 1 / n.
template <int MODE>
__device__ int voxel_finalize(const FitArgs& a, const double* S, int n, const float* anchor, vmp_fit_rec& r,
                              typename FitTypes<MODE>::T* kc) {
    using T = typename FitTypes<MODE>::T;
    r.n = n;
    for (int k = 0; k < 3; ++k) r.norm[k] = 0.0;
    for (int k = 0; k < 21; ++k) r.plane_cov[k] = 0.0;
    if (n <= 0) {
        for (int k = 0; k < 3; ++k) r.mean[k] = 0.0, r.evals[k] = 0.0;
        for (int k = 0; k < 6; ++k) r.cov[k] = 0.0;
        r.flags = 0;
        return 0;
    }
    const T tn = (T)n;
    T m[3];
    for (int k = 0; k < 3; ++k) m[k] = (T)S[k] / tn;
    double mean[3];
    for (int k = 0; k < 3; ++k) mean[k] = MODE == FIT_FP32C ? (double)anchor[k] + (double)m[k] : (double)m[k];
    for (int k = 0; k < 3; ++k) r.mean[k] = mean[k];
    if (n < a.min_pts) {
        for (int k = 0; k < 3; ++k) r.evals[k] = 0.0;
        for (int k = 0; k < 6; ++k) r.cov[k] = 0.0;
        r.flags = 0;
        return 0;
    }
    // C = ppt / n - mean mean^T (upper triangle mirrored)
    constexpr int kU[3][3] = {{3, 4, 5}, {4, 6, 7}, {5, 7, 8}};
    T C[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C[i * 3 + j] = (T)S[kU[i][j]] / tn - m[i] * m[j];
    T ev[3], E[9];
    eig_sym3<T>(C, ev, E);
    r.cov[0] = (double)C[0];
    r.cov[1] = (double)C[1];
    r.cov[2] = (double)C[2];
    r.cov[3] = (double)C[4];
    r.cov[4] = (double)C[5];
    r.cov[5] = (double)C[8];
    for (int k = 0; k < 3; ++k) r.evals[k] = (double)ev[k];
    int flags = VMP_FIT_FITTED;
    if ((double)ev[0] > a.plane_thresh) {
        r.flags = flags;
        return flags;
    }
    flags |= VMP_FIT_PLANE;
    const T pn[3] = {E[0], E[3], E[6]};
    // sign flip of updatePlane (voxel_map.cpp:131-133)
    bool flip;
    if (MODE == FIT_FP32) {
        flip = -(m[0] * pn[0] + m[1] * pn[1] + m[2] * pn[2]) < T(0);
    } else {
        flip = -(mean[0] * (double)pn[0] + mean[1] * (double)pn[1] + mean[2] * (double)pn[2]) < 0.0;
    }
    if (flip) flags |= VMP_FIT_FLIPPED;
    for (int k = 0; k < 3; ++k) r.norm[k] = flip ? -(double)pn[k] : (double)pn[k];
    for (int k = 0; k < 3; ++k) {
        kc[k] = m[k];
        kc[3 + k] = pn[k];
        kc[6 + k] = E[k * 3 + 1];
        kc[9 + k] = E[k * 3 + 2];
    }
    kc[12] = T(1) / (tn * (ev[0] - ev[1]));
    kc[13] = T(1) / (tn * (ev[0] - ev[2]));
    kc[14] = T(1) / tn;
    r.flags = flags;
    return flags;
}

// Pass 2 over a plane voxel: the factored J cov J^T terms, reduced across
// the warp; lane e < 21 forms entry e of the 6x6 and writes it.
template <int MODE>
__device__ __forceinline__ void voxel_terms(const FitArgs& a, long long p0, long long p1, float ax, float ay,
                                            float az, const typename FitTypes<MODE>::T* kc, int lane,
                                            double* plane_cov) {
    using T = typename FitTypes<MODE>::T;
    const T m[3] = {kc[0], kc[1], kc[2]};
    const T nn[3] = {kc[3], kc[4], kc[5]};
    const T v1[3] = {kc[6], kc[7], kc[8]};
    const T v2[3] = {kc[9], kc[10], kc[11]};
    const T k1 = kc[12], k2 = kc[13], inv_n = kc[14];
    T acc[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[k] = T(0);
    auto add = [&](float px, float py, float pz, const float* pc) {
        T d[3];
        if constexpr (MODE == FIT_FP32C) {
            d[0] = (px - ax) - m[0];
            d[1] = (py - ay) - m[1];
            d[2] = (pz - az) - m[2];
        } else {
            d[0] = (T)px - m[0];
            d[1] = (T)py - m[1];
            d[2] = (T)pz - m[2];
        }
        const T an = mad(nn[2], d[2], mad(nn[1], d[1], nn[0] * d[0]));
        const T b1 = mad(v1[2], d[2], mad(v1[1], d[1], v1[0] * d[0]));
        const T b2 = mad(v2[2], d[2], mad(v2[1], d[1], v2[0] * d[0]));
        T f1[3], f2[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            f1[q] = k1 * mad(an, v1[q], b1 * nn[q]);
            f2[q] = k2 * mad(an, v2[q], b2 * nn[q]);
        }
        const T c00 = (T)pc[0], c01 = (T)pc[1], c02 = (T)pc[2], c11 = (T)pc[3], c12 = (T)pc[4], c22 = (T)pc[5];
        T g1[3], g2[3];
        g1[0] = mad(c02, f1[2], mad(c01, f1[1], c00 * f1[0]));
        g1[1] = mad(c12, f1[2], mad(c11, f1[1], c01 * f1[0]));
        g1[2] = mad(c22, f1[2], mad(c12, f1[1], c02 * f1[0]));
        g2[0] = mad(c02, f2[2], mad(c01, f2[1], c00 * f2[0]));
        g2[1] = mad(c12, f2[2], mad(c11, f2[1], c01 * f2[0]));
        g2[2] = mad(c22, f2[2], mad(c12, f2[1], c02 * f2[0]));
        acc[0] += mad(f1[2], g1[2], mad(f1[1], g1[1], f1[0] * g1[0]));
        acc[1] += mad(f1[2], g2[2], mad(f1[1], g2[1], f1[0] * g2[0]));
        acc[2] += mad(f2[2], g2[2], mad(f2[1], g2[1], f2[0] * g2[0]));
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            acc[3 + q] += g1[q];
            acc[6 + q] += g2[q];
        }
        acc[9] += c00;
        acc[10] += c01;
        acc[11] += c02;
        acc[12] += c11;
        acc[13] += c12;
        acc[14] += c22;
    };
    long long i = p0 + lane;
    for (; i + 32 < p1; i += 64) {  // two points per lane in flight (9 floats each)
        float px[2], py[2], pz[2], pc[2][6];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const long long k = i + 32 * u;
            px[u] = __ldg(a.x + k);
            py[u] = __ldg(a.y + k);
            pz[u] = __ldg(a.z + k);
#pragma unroll
            for (int q = 0; q < 6; ++q) pc[u][q] = __ldg(a.c[q] + k);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) add(px[u], py[u], pz[u], pc[u]);
    }
    for (; i < p1; i += 32) {
        float pc[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) pc[q] = __ldg(a.c[q] + i);
        add(__ldg(a.x + i), __ldg(a.y + i), __ldg(a.z + i), pc);
    }
    transpose_reduce16(acc, lane);
    // lane e < 21 forms entry e = (i, j), i <= j, row by row
    int ei = 0, ej = 0;
    {
        int e = lane < 21 ? lane : 0, row = 0, len = 6;
        while (e >= len) { e -= len; ++row; --len; }
        ei = row;
        ej = row + e;
    }
    const T s11 = __shfl_sync(0xffffffffu, acc[0], red_lane(0));
    const T s12 = __shfl_sync(0xffffffffu, acc[0], red_lane(1));
    const T s22 = __shfl_sync(0xffffffffu, acc[0], red_lane(2));
    const int jc = ej >= 3 ? ej - 3 : ej;
    const T g1j = __shfl_sync(0xffffffffu, acc[0], red_lane(3 + jc));
    const T g2j = __shfl_sync(0xffffffffu, acc[0], red_lane(6 + jc));
    int ss = 0;
    if (ei >= 3) {
        const int a3 = ei - 3, b3 = ej - 3;  // index in xx xy xz yy yz zz
        ss = a3 == 0 ? b3 : (a3 == 1 ? 2 + b3 : 5);
    }
    const T sij = __shfl_sync(0xffffffffu, acc[0], red_lane(9 + ss));
    if (lane < 21) {
        T val;
        if (ej < 3) {
            val = s11 * v1[ei] * v1[ej] + s12 * (v1[ei] * v2[ej] + v2[ei] * v1[ej]) + s22 * v2[ei] * v2[ej];
        } else if (ei < 3) {
            val = (v1[ei] * g1j + v2[ei] * g2j) * inv_n;
        } else {
            val = sij * inv_n * inv_n;
        }
        plane_cov[lane] = (double)val;
    }
}

// ---------------------------------------------------------------- the fit
// One warp fits 32 consecutive voxels: their offsets and anchors are loaded
// by one lane each (coalesced), pass 1 runs voxel by voxel over all lanes and
// hands each voxel's sums to the lane that owns it, the 32 eigen
// decompositions run one per lane, and pass 2 runs voxel by voxel again
// (the points of the 32 voxels were just read: their xyz mostly comes from
// L2).
template <int MODE>
__global__ void __launch_bounds__(kFitWarps * 32, MODE == FIT_FP64 ? 1 : 4) k_fit(FitArgs a) {
    using T = typename FitTypes<MODE>::T;
    const int lane = threadIdx.x & 31;
    const long long v0 = ((long long)blockIdx.x * kFitWarps + (threadIdx.x >> 5)) * 32;
    if (v0 >= a.n_vox) return;  // uniform per warp
    const int nb = (int)(a.n_vox - v0 < 32 ? a.n_vox - v0 : 32);
    long long mp0 = 0, mp1 = 0;
    float anc[3] = {0.f, 0.f, 0.f};
    if (lane < nb) {
        voxel_range(a, v0 + lane, mp0, mp1);
        if (MODE == FIT_FP32C && mp1 > mp0) {
            anc[0] = a.x[mp0];
            anc[1] = a.y[mp0];
            anc[2] = a.z[mp0];
        }
    }
    double S[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) S[k] = 0.0;
    for (int j = 0; j < nb; ++j) {
        const long long p0 = __shfl_sync(0xffffffffu, mp0, j), p1 = __shfl_sync(0xffffffffu, mp1, j);
        const float ax = __shfl_sync(0xffffffffu, anc[0], j), ay = __shfl_sync(0xffffffffu, anc[1], j),
                    az = __shfl_sync(0xffffffffu, anc[2], j);
        const double tot = voxel_sums<MODE>(a, p0, p1, ax, ay, az, lane);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const double t = __shfl_sync(0xffffffffu, tot, red_lane(k));
            if (lane == j) S[k] = t;
        }
    }
    T kc[15];
#pragma unroll
    for (int k = 0; k < 15; ++k) kc[k] = T(0);
    int fl = 0;
    if (lane < nb) fl = voxel_finalize<MODE>(a, S, (int)(mp1 - mp0), anc, a.out[v0 + lane], kc);
    for (int j = 0; j < nb; ++j) {
        if (!(__shfl_sync(0xffffffffu, fl, j) & VMP_FIT_PLANE)) continue;  // uniform
        T kj[15];
#pragma unroll
        for (int k = 0; k < 15; ++k) kj[k] = __shfl_sync(0xffffffffu, kc[k], j);
        const long long p0 = __shfl_sync(0xffffffffu, mp0, j), p1 = __shfl_sync(0xffffffffu, mp1, j);
        const float ax = __shfl_sync(0xffffffffu, anc[0], j), ay = __shfl_sync(0xffffffffu, anc[1], j),
                    az = __shfl_sync(0xffffffffu, anc[2], j);
        voxel_terms<MODE>(a, p0, p1, ax, ay, az, kj, lane, a.out[v0 + j].plane_cov);
    }
}

// Measurement hook (vmp_fit_profile): CUDA events around the fit kernel; the
// call waits for them and adds up its device time.
struct FitProfile {
    std::mutex mu;
    bool on = false;
    cudaEvent_t ev[2] = {};
    double ms = 0.0;
    long long calls = 0;
};
FitProfile& fit_profile() {
    static FitProfile p;
    return p;
}

template <int MODE>
void launch_mode(const FitArgs& a, cudaStream_t st, cudaEvent_t* ev) {
    const unsigned grid = (unsigned)((a.n_vox + 32 * kFitWarps - 1) / (32 * kFitWarps));
    if (ev) cudaEventRecord(ev[0], st);
    VMP_NOTE_LAUNCH(); k_fit<MODE><<<grid, kFitWarps * 32, 0, st>>>(a);
    if (ev) cudaEventRecord(ev[1], st);
}

bool params_ok(const vmp_fit_params* p) {
    return p && p->mode >= VMP_FIT_FP64 && p->mode <= VMP_FIT_FP32C && p->update_point_thresh >= 1 &&
           p->plane_thresh == p->plane_thresh;
}

cudaError_t fit_enqueue(const float* xyz, const float* cov, const long long* offsets, int n_vox, long long n_pts,
                        const vmp_fit_params* p, vmp_fit_rec* out, cudaStream_t st) {
    FitArgs a;
    a.x = xyz;
    a.y = xyz + n_pts;
    a.z = xyz + 2 * n_pts;
    for (int q = 0; q < 6; ++q) a.c[q] = cov + q * n_pts;
    a.off = offsets;
    a.n_pts = n_pts;
    a.n_vox = n_vox;
    a.min_pts = p->update_point_thresh;
    a.plane_thresh = p->plane_thresh;
    a.out = out;
    FitProfile& prof = fit_profile();
    std::unique_lock<std::mutex> lk(prof.mu);
    cudaEvent_t* ev = nullptr;
    if (prof.on) {
        for (auto& e : prof.ev)
            if (!e && cudaEventCreate(&e) != cudaSuccess) return cudaGetLastError();
        ev = prof.ev;
    } else {
        lk.unlock();
    }
    switch (p->mode) {
        case VMP_FIT_FP64: launch_mode<FIT_FP64>(a, st, ev); break;
        case VMP_FIT_FP32: launch_mode<FIT_FP32>(a, st, ev); break;
        default: launch_mode<FIT_FP32C>(a, st, ev); break;
    }
    cudaError_t e = cudaGetLastError();
    if (ev && e == cudaSuccess && (e = cudaEventSynchronize(ev[1])) == cudaSuccess) {
        float t = 0.f;
        cudaEventElapsedTime(&t, ev[0], ev[1]);
        prof.ms += t;
        ++prof.calls;
    }
    return e;
}

}  // namespace
}  // namespace vmp

using namespace vmp;

extern "C" vmp_status vmp_fit_planes_device(const float* xyz, const float* cov, const long long* offsets,
                                            int n_vox, long long n_pts, const vmp_fit_params* params,
                                            vmp_fit_rec* out, void* cuda_stream) {
    if (!params_ok(params) || n_vox < 0 || n_pts < 0) return VMP_ERR_INVALID_ARG;
    if (n_vox == 0) return VMP_OK;
    if (!offsets || !out || (n_pts > 0 && (!xyz || !cov))) return VMP_ERR_INVALID_ARG;
    if (fit_enqueue(xyz, cov, offsets, n_vox, n_pts, params, out, (cudaStream_t)cuda_stream) != cudaSuccess)
        return VMP_ERR_CUDA;
    return VMP_OK;
}

namespace vmp {
namespace {
// Device buffers and streams of the host-buffer entry point, kept between
// calls (grown when a call needs more): the copies of one chunk of voxels
// overlap the fit of the previous chunk and the copy-back of the one before.
struct FitHostCache {
    std::mutex mu;
    float* d_pts = nullptr;
    long long* d_off = nullptr;
    vmp_fit_rec* d_out = nullptr;
    size_t cap_pts = 0, cap_vox = 0;
    cudaStream_t s_in = nullptr, s_fit = nullptr, s_out = nullptr;
    static constexpr int kChunks = 4;
    cudaEvent_t in_done[kChunks] = {}, fit_done[kChunks] = {};
    bool ready = false;
};
FitHostCache& fit_host_cache() {
    static FitHostCache c;
    return c;
}
cudaError_t fit_host_prepare(FitHostCache& c, size_t n_pts, size_t n_vox) {
    cudaError_t e = cudaSuccess;
    if (!c.ready) {
        for (cudaStream_t* st : {&c.s_in, &c.s_fit, &c.s_out})
            if ((e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking)) != cudaSuccess) return e;
        for (int k = 0; k < FitHostCache::kChunks; ++k) {
            if ((e = cudaEventCreateWithFlags(&c.in_done[k], cudaEventDisableTiming)) != cudaSuccess) return e;
            if ((e = cudaEventCreateWithFlags(&c.fit_done[k], cudaEventDisableTiming)) != cudaSuccess) return e;
        }
        c.ready = true;
    }
    if (n_pts > c.cap_pts) {
        if (c.d_pts) cudaFree(c.d_pts);
        c.d_pts = nullptr;
        c.cap_pts = 0;
        if ((e = cudaMalloc((void**)&c.d_pts, sizeof(float) * 9 * n_pts)) != cudaSuccess) return e;
        c.cap_pts = n_pts;
    }
    if (n_vox > c.cap_vox) {
        if (c.d_off) cudaFree(c.d_off);
        if (c.d_out) cudaFree(c.d_out);
        c.d_off = nullptr;
        c.d_out = nullptr;
        c.cap_vox = 0;
        if ((e = cudaMalloc((void**)&c.d_off, sizeof(long long) * (n_vox + 1))) != cudaSuccess) return e;
        if ((e = cudaMalloc((void**)&c.d_out, sizeof(vmp_fit_rec) * n_vox)) != cudaSuccess) return e;
        c.cap_vox = n_vox;
    }
    return e;
}
}  // namespace
}  // namespace vmp

extern "C" vmp_status vmp_fit_planes(const float* xyz, const float* cov, const long long* offsets, int n_vox,
                                     long long n_pts, const vmp_fit_params* params, vmp_fit_rec* out) {
    if (!params_ok(params) || n_vox < 0 || n_pts < 0) return VMP_ERR_INVALID_ARG;
    if (n_vox == 0) return VMP_OK;
    if (!offsets || !out || (n_pts > 0 && (!xyz || !cov))) return VMP_ERR_INVALID_ARG;
    if (offsets[0] != 0 || offsets[n_vox] != n_pts) return VMP_ERR_INVALID_ARG;
    for (int v = 0; v < n_vox; ++v)
        if (offsets[v + 1] < offsets[v]) return VMP_ERR_INVALID_ARG;
    FitHostCache& c = fit_host_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    cudaError_t e = fit_host_prepare(c, (size_t)(n_pts > 0 ? n_pts : 1), (size_t)n_vox);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? VMP_ERR_OUT_OF_MEMORY : VMP_ERR_CUDA;
    }
    const size_t N = (size_t)n_pts;
    float* d_xyz = c.d_pts;
    float* d_cov = c.d_pts + 3 * N;
    const int K = n_vox >= 4096 ? FitHostCache::kChunks : 1;
    // the chunk's voxels [v[k], v[k+1]) own points [offsets[v[k]], offsets[v[k+1]])
    int vb[FitHostCache::kChunks + 1];
    for (int k = 0; k <= K; ++k) vb[k] = (int)((long long)n_vox * k / K);
    e = cudaMemcpyAsync(c.d_off, offsets, sizeof(long long) * ((size_t)n_vox + 1), cudaMemcpyHostToDevice, c.s_in);
    for (int k = 0; k < K && e == cudaSuccess; ++k) {
        const size_t p0 = (size_t)offsets[vb[k]], p1 = (size_t)offsets[vb[k + 1]];
        for (int q = 0; q < 9 && e == cudaSuccess && p1 > p0; ++q) {
            const float* src = (q < 3 ? xyz + (size_t)q * N : cov + (size_t)(q - 3) * N) + p0;
            float* dst = (q < 3 ? d_xyz + (size_t)q * N : d_cov + (size_t)(q - 3) * N) + p0;
            e = cudaMemcpyAsync(dst, src, sizeof(float) * (p1 - p0), cudaMemcpyHostToDevice, c.s_in);
        }
        if (e == cudaSuccess) e = cudaEventRecord(c.in_done[k], c.s_in);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c.s_fit, c.in_done[k], 0);
        if (e == cudaSuccess)
            e = fit_enqueue(d_xyz, d_cov, c.d_off + vb[k], vb[k + 1] - vb[k], n_pts, params, c.d_out + vb[k], c.s_fit);
        if (e == cudaSuccess) e = cudaEventRecord(c.fit_done[k], c.s_fit);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c.s_out, c.fit_done[k], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(out + vb[k], c.d_out + vb[k], sizeof(vmp_fit_rec) * (size_t)(vb[k + 1] - vb[k]),
                                cudaMemcpyDeviceToHost, c.s_out);
    }
    const cudaError_t e2 = cudaStreamSynchronize(c.s_out);
    cudaStreamSynchronize(c.s_in);
    cudaStreamSynchronize(c.s_fit);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) {
        cudaGetLastError();
        return VMP_ERR_CUDA;
    }
    return VMP_OK;
}

extern "C" vmp_status vmp_fit_profile(int on) {
    FitProfile& p = fit_profile();
    std::lock_guard<std::mutex> lk(p.mu);
    p.on = on != 0;
    p.ms = 0.0;
    p.calls = 0;
    return VMP_OK;
}

extern "C" vmp_status vmp_fit_profile_read(double* ms, long long* calls) {
    FitProfile& p = fit_profile();
    std::lock_guard<std::mutex> lk(p.mu);
    if (ms) *ms = p.ms;
    if (calls) *calls = p.calls;
    return VMP_OK;
}
