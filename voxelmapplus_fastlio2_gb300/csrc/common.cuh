// Shared device definitions of libvmp: FP64 small-matrix algebra, SO(3) /
// S2 helpers, packed voxel keys and the device-resident data structures.
//
// Every FP64 expression on the decision path (voxel keys, residual gates,
// plane tests, float outputs) is written in the reference's evaluation order
// (left-to-right products, k = 0..K-1 sums) and the library is compiled with
// --fmad=false, so the device rounds exactly like the reference's x86-64
// build, which has no fused multiply-add.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "vmp.h"

namespace vmp {

// Host-side count of kernel launches issued by the library (all streams).
extern std::atomic<long long> g_launch_count;
// While this thread captures a CUDA graph its launches only record into the
// graph: they are counted here and added to g_launch_count at every replay.
long long* capture_launch_counter();
inline void note_launch() {
    long long* c = capture_launch_counter();
    if (c) ++*c;
    else g_launch_count.fetch_add(1, std::memory_order_relaxed);
}
#define VMP_NOTE_LAUNCH() ::vmp::note_launch()

constexpr double kGravity = 9.81;          // kf::GRAVITY (ieskf.h:6)
constexpr double kSophusEps = 1e-10;       // Sophus::Constants<double>::epsilon()
constexpr int kChunkPts = 16;              // points per slab chunk
constexpr int kMaxChunks = 16;             // chunks per voxel (max_point_thresh <= 256)
constexpr int kSlabStride = 12;            // doubles per buffered point: xyz + 3x3 cov
constexpr uint64_t kEmptyKey = ~0ull;
constexpr uint64_t kTombKey = ~0ull - 1;
constexpr uint32_t kPending = 0x80000000u;
constexpr uint32_t kNoRec = 0xFFFFFFFFu;
constexpr uint64_t kNever = ~0ull;
constexpr int kKeyBits = 21;
constexpr int64_t kKeyOff = 1ll << 20;     // packed axis range [-2^20, 2^20)

// record flag bits
constexpr uint32_t F_INIT = 1u, F_PLANE = 2u, F_UPDATE = 4u, F_MERGED = 8u, F_ALIVE = 16u, F_DROPPED = 32u;

// device error word bits
constexpr uint32_t E_KEY_RANGE = 1u, E_HASH_FULL = 2u, E_RECORDS = 4u, E_CHUNKS = 8u, E_CAPACITY = 16u,
                   E_NONFINITE = 32u, E_MERGE_ITER = 64u, E_MERGE_WAIT = 128u;

// --------------------------------------------------------------- data layout
// kf::State; identical layout to vmp_state.
struct DState {
    double pos[3];
    double rot[9];
    double rot_ext[9];
    double pos_ext[3];
    double vel[3];
    double bg[3];
    double ba[3];
    double g[3];
};
static_assert(sizeof(DState) == sizeof(vmp_state), "state layout");

// One entry of LIODataGroup::imu_poses_cache (commons.h:30-43).
struct DPose {
    double offset;
    double acc[3], gyro[3], vel[3], pos[3];
    double rot[9];
};

// Per-step terms of the IMU predict chain (k_predict.cu).
struct DStep {
    double dt, offset;
    double acc[3], gyro[3], ab[3];
    double E[9];     // Exp((gyro - bg) dt)
    double nJr[9];   // -Jr((gyro - bg) dt) dt
    double rot[9];   // rotation before the step
    double FRa[9];   // (-rot [acc - ba]x) dt
    double nRdt[9];  // -rot dt
    double Mxdt[6];  // Mx dt
    double B[24];    // G Q G^T: block 3-5, block 12-14, diagonal 15-20
    double vinc[3], velA[3], posA[3];
    int pose;
    int pad;
};

// Filter state + LIO bookkeeping that lives on the device between scans.
struct DFilter {
    DState x;
    double P[529];
    double Q[144];
    DState x_pred;
    double K[23 * 12];  // gain M_E S^-1 of the last iteration (ld 12)
    double Hinv[529];   // M = D P D^T of the last iteration
    double delta[23];
    double Hm[144];
    double bm[12];
    // x boxminus x_pred of the current IEKF iteration and its block-diagonal
    // inverse Jacobian (rot 3x3, rot_ext 3x3, S2 2x2), from k_iekf_boxminus
    double bmx_d[23];
    double bmx_D[22];
    double last_acc[3], last_gyro[3];
    double last_cloud_end_time;
    double gravity_norm;
    double last_imu_t, last_imu_acc[3], last_imu_gyro[3];
    double inp_acc[3], inp_gyro[3];
    int iters;
    int effect_num;
    int converged;
    int no_effect;
    int npose;
    int pad[3];
};

// Hot part of a voxel record: what the residual kernel reads (64 B).
struct __align__(64) RecHot {
    double mean[3];
    double norm[3];
    uint32_t flags;
    int32_t n;
    uint64_t group;
};

// Cold part of a voxel record.
struct RecCold {
    double ppt[9];
    double cov[36];
    double center[3];
    uint64_t key;
    uint64_t stamp;      // global index of the last touching point
    uint64_t create_g;   // global index of the creating point
    uint64_t freeze_g;   // global index of the point that froze it (kNever if not frozen)
    uint64_t evict_g;    // global index of the creation that evicted it (kNever if alive)
    uint64_t touch_first_g;  // first touching point of the current batch
    int32_t newly;
    int32_t nslab;       // temp_points.size()
    int32_t chunks[kMaxChunks];
};

struct DMap {
    // open-addressing hash, linear probing
    uint64_t* keys;
    uint32_t* vals;
    uint64_t table_mask;
    // records
    RecHot* hot;
    RecCold* cold;
    uint32_t* rec_free;   // stack of free record ids
    // point slabs
    double* slab;         // [chunk][kChunkPts][kSlabStride]
    int32_t* chunk_free;  // stack of free chunk ids
    int32_t* chunk_freed; // chunks released during a kernel (pushed back later)
    // LRU queue (append-only ring of (record, stamp))
    uint32_t* q_rec;
    uint64_t* q_stamp;
    uint64_t q_cap;
    // counters (device)
    struct Counters* cnt;
    double voxel_size;
    double voxel_inv;  // 1 / voxel_size when that is a power of two (then exact), else 0
    int update_thresh;
    int max_thresh;
    double plane_thresh;
    double merge_angle;
    double merge_dist;
    long long capacity;
    int rec_pool;
    int chunk_pool;
};

struct Counters {
    long long size;           // live voxels
    long long group_counter;  // VoxelGrid::count
    unsigned long long batch_base;  // global index of the next point
    unsigned long long q_head, q_tail;
    int rec_free_top;
    int chunk_free_top;
    int chunk_freed_top;
    int n_new;
    int n_seg;
    int n_events;
    int n_evict;
    unsigned int error;
    long long evicted_total;
    int n_writes;
    int changed;
    int split_at;             // batch-relative index to split at (-1: none)
    int n_tomb;               // tombstones in the hash table
};

// --------------------------------------------------------------- packed keys
__host__ __device__ inline bool key_in_range(int64_t k) { return k >= -kKeyOff && k < kKeyOff; }
__host__ __device__ inline uint64_t pack_key(int64_t x, int64_t y, int64_t z) {
    return (uint64_t)(x + kKeyOff) | ((uint64_t)(y + kKeyOff) << kKeyBits) | ((uint64_t)(z + kKeyOff) << (2 * kKeyBits));
}
__host__ __device__ inline void unpack_key(uint64_t k, int64_t& x, int64_t& y, int64_t& z) {
    const uint64_t m = (1ull << kKeyBits) - 1;
    x = (int64_t)(k & m) - kKeyOff;
    y = (int64_t)((k >> kKeyBits) & m) - kKeyOff;
    z = (int64_t)((k >> (2 * kKeyBits)) & m) - kKeyOff;
}
__host__ __device__ inline uint64_t hash_key(uint64_t k) {
    // 64-bit finaliser (MurmurHash3 fmix64); bucket placement only.
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

// Lookup of a packed key; returns the record id or kNoRec.
__device__ inline uint32_t map_find(const DMap& m, uint64_t key) {
    uint64_t h = hash_key(key) & m.table_mask;
    for (uint64_t probe = 0; probe <= m.table_mask; ++probe) {
        uint64_t k = m.keys[h];
        if (k == key) return m.vals[h];
        if (k == kEmptyKey) return kNoRec;
        h = (h + 1) & m.table_mask;
    }
    return kNoRec;
}

// VoxelMap::index (voxel_map.cpp:194-198): floor(p / voxel_size) in FP64.
// With a power-of-two voxel size (the 0.5 m default) the quotient is the
// product with the exact reciprocal -- the same correctly rounded value --
// and the FP64 division (a ~10-instruction sequence) is skipped.
__device__ inline bool voxel_index(const double p[3], double vs, double inv, int64_t k[3]) {
    bool ok = true;
    for (int a = 0; a < 3; ++a) {
        double f = floor(inv != 0.0 ? p[a] * inv : __ddiv_rn(p[a], vs));
        if (!(f >= -(double)kKeyOff && f < (double)kKeyOff)) { ok = false; f = 0.0; }
        k[a] = (int64_t)f;
    }
    return ok;
}

// --------------------------------------------------------------- division
// a / b, correctly rounded, from y = RN(1 / b) by Markstein's correction
// (P. W. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990): q = RN(a y) is
// within one ulp of a / b, the remainder r = a - b q is exact by FMA, and
// RN(q + r y) is RN(a / b).  Three FP64 instructions instead of a division
// sequence, for divisions that share a divisor.  Valid while a / b and y
// stay in the normal range (callers check the divisor with div_recip_ok);
// a zero dividend keeps the sign rule of a / b.
__host__ __device__ inline bool div_recip_ok(double b) {
    const double ab = b < 0 ? -b : b;
    return ab > 1e-290 && ab < 1e290;
}
__device__ __forceinline__ double div_by_recip(double a, double b, double y) {
    const double q = a * y;
    const double r = __fma_rn(-q, b, a);
    const double q2 = __fma_rn(r, y, q);
    return a == 0.0 ? q : q2;
}

// --------------------------------------------------------------- small FP64 algebra
// Row-major, products summed k = 0..K-1 left to right (no FMA).
template <int R, int K, int C>
__device__ inline void mm(const double* A, const double* B, double* O) {
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < C; ++j) {
            double s = __dmul_rn(A[i * K], B[j]);
            for (int k = 1; k < K; ++k) s = __dadd_rn(s, __dmul_rn(A[i * K + k], B[k * C + j]));
            O[i * C + j] = s;
        }
}
// O = A^T (A is R x C)
template <int R, int C>
__device__ inline void tr(const double* A, double* O) {
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < C; ++j) O[j * R + i] = A[i * C + j];
}
__device__ inline void m3v(const double* A, const double* v, double* o) { mm<3, 3, 1>(A, v, o); }
// Entry e = i * 3 + j of mm<3, 3, 3>(A, B, .) and entry i of m3v(A, v, .),
// the same operations in the same order (one thread per entry).
__device__ inline double mm3_entry(const double* A, const double* B, int e) {
    const int i = e / 3, j = e - 3 * (e / 3);
    double s = __dmul_rn(A[i * 3], B[j]);
    s = __dadd_rn(s, __dmul_rn(A[i * 3 + 1], B[3 + j]));
    return __dadd_rn(s, __dmul_rn(A[i * 3 + 2], B[6 + j]));
}
__device__ inline double m3v_entry(const double* A, const double* v, int i) {
    double s = __dmul_rn(A[i * 3], v[0]);
    s = __dadd_rn(s, __dmul_rn(A[i * 3 + 1], v[1]));
    return __dadd_rn(s, __dmul_rn(A[i * 3 + 2], v[2]));
}
__device__ inline double dot3(const double* a, const double* b) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}
__device__ inline void hat3(const double* w, double* m) {
    m[0] = 0; m[1] = -w[2]; m[2] = w[1];
    m[3] = w[2]; m[4] = 0; m[5] = -w[0];
    m[6] = -w[1]; m[7] = w[0]; m[8] = 0;
}
// [p]x M [p]x^T as ([p]x M) [p]x^T, products summed k = 0..2 left to right,
// without the products with [p]x's zero diagonal: the dense sums less their
// +-0 terms (the same values up to the sign of an exact zero).
__device__ inline void hat_sandwich(const double* p, const double* M, double* out) {
    double h[9], T[9];
    hat3(p, h);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const int k0 = i == 0 ? 1 : 0, k1 = i == 2 ? 1 : 2;  // the two k != i
            T[i * 3 + j] = h[i * 3 + k0] * M[k0 * 3 + j] + h[i * 3 + k1] * M[k1 * 3 + j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const int k0 = j == 0 ? 1 : 0, k1 = j == 2 ? 1 : 2;  // the two k != j
            out[i * 3 + j] = T[i * 3 + k0] * h[j * 3 + k0] + T[i * 3 + k1] * h[j * 3 + k1];
        }
}
__device__ inline void eye3(double* m) {
    for (int i = 0; i < 9; ++i) m[i] = (i % 4 == 0) ? 1.0 : 0.0;
}

// Eigen QuaternionBase::toRotationMatrix.
__device__ inline void quat_to_mat(double w, double x, double y, double z, double* r) {
    const double tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z;
    const double twx = tx * w, twy = ty * w, twz = tz * w;
    const double txx = tx * x, txy = ty * x, txz = tz * x;
    const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
    r[0] = 1.0 - (tyy + tzz); r[1] = txy - twz; r[2] = txz + twy;
    r[3] = txy + twz; r[4] = 1.0 - (txx + tzz); r[5] = tyz - twx;
    r[6] = txz - twy; r[7] = tyz + twx; r[8] = 1.0 - (txx + tyy);
}

// Sophus SO3::exp(w).matrix()
__device__ inline void so3_exp(const double* w, double* R) {
    double theta_sq = dot3(w, w);
    double imag, real;
    if (theta_sq < kSophusEps * kSophusEps) {
        double t4 = theta_sq * theta_sq;
        imag = 0.5 - (1.0 / 48.0) * theta_sq + (1.0 / 3840.0) * t4;
        real = 1.0 - (1.0 / 8.0) * theta_sq + (1.0 / 384.0) * t4;
    } else {
        double theta = sqrt(theta_sq);
        double half = 0.5 * theta;
        double s, c;
        sincos(half, &s, &c);
        imag = s / theta;
        real = c;
    }
    quat_to_mat(real, imag * w[0], imag * w[1], imag * w[2], R);
}

// Sophus SO3(R).log() through Eigen's matrix -> quaternion conversion.
__device__ inline void so3_log(const double* m, double* out) {
    double qw, qx, qy, qz;
    double t = m[0] + m[4] + m[8];
    if (t > 0.0) {
        t = sqrt(t + 1.0);
        qw = 0.5 * t;
        t = 0.5 / t;
        qx = (m[7] - m[5]) * t;
        qy = (m[2] - m[6]) * t;
        qz = (m[3] - m[1]) * t;
    } else {
        int i = 0;
        if (m[4] > m[0]) i = 1;
        if (m[8] > m[i * 4]) i = 2;
        int j = (i + 1) % 3, k = (j + 1) % 3;
        t = sqrt(m[i * 4] - m[j * 4] - m[k * 4] + 1.0);
        double c[3];
        c[i] = 0.5 * t;
        t = 0.5 / t;
        qw = (m[k * 3 + j] - m[j * 3 + k]) * t;
        c[j] = (m[j * 3 + i] + m[i * 3 + j]) * t;
        c[k] = (m[k * 3 + i] + m[i * 3 + k]) * t;
        qx = c[0]; qy = c[1]; qz = c[2];
    }
    double sq_n = qx * qx + qy * qy + qz * qz;
    double f;
    if (sq_n < kSophusEps * kSophusEps) {
        double sq_w = qw * qw;
        f = 2.0 / qw - (2.0 / 3.0) * sq_n / (qw * sq_w);
    } else {
        double n = sqrt(sq_n);
        double a = (qw < 0.0) ? atan2(-n, -qw) : atan2(n, qw);
        f = 2.0 * a / n;
    }
    out[0] = f * qx; out[1] = f * qy; out[2] = f * qz;
}

// Sophus SO3::leftJacobian
__device__ inline void so3_left_jac(const double* w, double* V) {
    double theta_sq = dot3(w, w);
    double O[9], O2[9];
    hat3(w, O);
    mm<3, 3, 3>(O, O, O2);
    if (theta_sq < kSophusEps * kSophusEps) {
        for (int i = 0; i < 9; ++i) V[i] = ((i % 4 == 0) ? 1.0 : 0.0) + 0.5 * O[i];
        return;
    }
    double theta = sqrt(theta_sq);
    double s, c;
    sincos(theta, &s, &c);
    double a = (1.0 - c) / theta_sq;
    double b = (theta - s) / (theta_sq * theta);
    for (int i = 0; i < 9; ++i) V[i] = (((i % 4 == 0) ? 1.0 : 0.0) + a * O[i]) + b * O2[i];
}
// kf::rightJacobian (ieskf.cpp:6-9) = leftJacobian^T
__device__ inline void so3_right_jac(const double* w, double* J) {
    double V[9];
    so3_left_jac(w, V);
    tr<3, 3>(V, J);
}

// ----- S2 gravity helpers (ieskf.cpp:69-95)
__device__ inline void s2_Bx(const double* g, double* r /*3x2*/) {
    r[0] = -g[1]; r[1] = -g[2];
    r[2] = kGravity - g[1] * g[1] / (kGravity + g[0]); r[3] = -g[2] * g[1] / (kGravity + g[0]);
    r[4] = -g[2] * g[1] / (kGravity + g[0]); r[5] = kGravity - g[2] * g[2] / (kGravity + g[0]);
    for (int i = 0; i < 6; ++i) r[i] /= kGravity;
}
__device__ inline void s2_Mx(const double* g, double* r /*3x2*/) {
    double H[9], Bx[6];
    hat3(g, H);
    for (int i = 0; i < 9; ++i) H[i] = -H[i];
    s2_Bx(g, Bx);
    mm<3, 3, 2>(H, Bx, r);
}
__device__ inline void s2_Mx_res(const double* g, const double* res, double* r /*3x2*/) {
    double bx[6], bu[3], E[9], H[9], Jl[9], JlT[9], T1[9], T2[9];
    s2_Bx(g, bx);
    mm<3, 2, 1>(bx, res, bu);
    so3_exp(bu, E);
    for (int i = 0; i < 9; ++i) E[i] = -E[i];
    hat3(g, H);
    mm<3, 3, 3>(E, H, T1);
    so3_left_jac(bu, Jl);
    tr<3, 3>(Jl, JlT);
    mm<3, 3, 3>(T1, JlT, T2);
    mm<3, 3, 2>(T2, bx, r);
}
__device__ inline void s2_Nx(const double* g, double* r /*2x3*/) {
    double bx[6], bxT[6], H[9];
    s2_Bx(g, bx);
    tr<3, 2>(bx, bxT);
    const double s = 1.0 / kGravity / kGravity;
    for (int i = 0; i < 6; ++i) bxT[i] = s * bxT[i];
    hat3(g, H);
    mm<2, 3, 3>(bxT, H, r);
}

// Boxplus pieces: R <- R Exp(d) and the S2 gravity update (ieskf.cpp:11-21).
__device__ inline void rot_plus(double* R, const double* d) {
    double E[9], T[9];
    so3_exp(d, E); mm<3, 3, 3>(R, E, T); for (int i = 0; i < 9; ++i) R[i] = T[i];
}
__device__ inline void s2_plus(double* g, const double* d) {
    double bx[6], w[3], E[9], g2[3];
    s2_Bx(g, bx);
    mm<3, 2, 1>(bx, d, w);
    so3_exp(w, E);
    m3v(E, g, g2);
    for (int i = 0; i < 3; ++i) g[i] = g2[i];
}
// State boxplus with a 23-vector (ieskf.cpp:11-21)
__device__ inline void state_plus23(DState& x, const double* d) {
    for (int i = 0; i < 3; ++i) x.pos[i] = x.pos[i] + d[i];
    rot_plus(x.rot, d + 3);
    rot_plus(x.rot_ext, d + 6);
    for (int i = 0; i < 3; ++i) {
        x.pos_ext[i] = x.pos_ext[i] + d[9 + i];
        x.vel[i] = x.vel[i] + d[12 + i];
        x.bg[i] = x.bg[i] + d[15 + i];
        x.ba[i] = x.ba[i] + d[18 + i];
    }
    s2_plus(x.g, d + 21);
}
// State boxplus with a 24-vector (ieskf.cpp:23-33)
__device__ inline void state_plus24(DState& x, const double* d) {
    double E[9], T[9];
    for (int i = 0; i < 3; ++i) x.pos[i] = x.pos[i] + d[i];
    so3_exp(d + 3, E); mm<3, 3, 3>(x.rot, E, T); for (int i = 0; i < 9; ++i) x.rot[i] = T[i];
    so3_exp(d + 6, E); mm<3, 3, 3>(x.rot_ext, E, T); for (int i = 0; i < 9; ++i) x.rot_ext[i] = T[i];
    for (int i = 0; i < 3; ++i) {
        x.pos_ext[i] = x.pos_ext[i] + d[9 + i];
        x.vel[i] = x.vel[i] + d[12 + i];
        x.bg[i] = x.bg[i] + d[15 + i];
        x.ba[i] = x.ba[i] + d[18 + i];
    }
    double g2[3];
    so3_exp(d + 21, E);
    m3v(E, x.g, g2);
    for (int i = 0; i < 3; ++i) x.g[i] = g2[i];
}
// Boxminus pieces (ieskf.cpp:35-67): Log(o^T x) and the S2 difference of
// two gravity vectors.
__device__ inline void rot_minus(const double* xr, const double* orr, double* d) {
    double RT[9], M[9];
    tr<3, 3>(orr, RT); mm<3, 3, 3>(RT, xr, M); so3_log(M, d);
}
__device__ inline void s2_minus(const double* xg, const double* og, double* d) {
    double H[9], hg[3];
    hat3(xg, H);
    m3v(H, og, hg);
    double v_sin = sqrt(dot3(hg, hg));
    double v_cos = dot3(xg, og);
    double theta = atan2(v_sin, v_cos);
    if (v_sin < 1e-11) {
        if (fabs(theta) > 1e-11) { d[0] = 3.1415926; d[1] = 0; }
        else { d[0] = 0; d[1] = 0; }
    } else {
        double bx[6], bxT[6], Ho[9], T1[6], T2[2];
        s2_Bx(og, bx);
        tr<3, 2>(bx, bxT);
        const double s = theta / v_sin;
        for (int i = 0; i < 6; ++i) bxT[i] = s * bxT[i];
        hat3(og, Ho);
        mm<2, 3, 3>(bxT, Ho, T1);
        mm<2, 3, 1>(T1, xg, T2);
        d[0] = T2[0]; d[1] = T2[1];
    }
}
// State boxminus (ieskf.cpp:35-67)
__device__ inline void state_minus(const DState& x, const DState& o, double* d) {
    for (int i = 0; i < 23; ++i) d[i] = 0.0;
    for (int i = 0; i < 3; ++i) d[i] = x.pos[i] - o.pos[i];
    rot_minus(x.rot, o.rot, d + 3);
    rot_minus(x.rot_ext, o.rot_ext, d + 6);
    for (int i = 0; i < 3; ++i) {
        d[9 + i] = x.pos_ext[i] - o.pos_ext[i];
        d[12 + i] = x.vel[i] - o.vel[i];
        d[15 + i] = x.bg[i] - o.bg[i];
        d[18 + i] = x.ba[i] - o.ba[i];
    }
    s2_minus(x.g, o.g, d + 21);
}

// ----- device allocations
// Bytes of device memory allocated through dev_malloc by the calling thread;
// vmp_create reads it around a stream's allocations (its footprint, which the
// server's HBM admission adds up).
long long& dev_bytes_counter();
template <class T>
inline cudaError_t dev_malloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n);
    if (e == cudaSuccess) dev_bytes_counter() += (long long)n;
    return e;
}

// ----- error reporting
__device__ inline void set_error(Counters* c, uint32_t bit) { atomicOr(&c->error, bit); }

// ----- warp helpers
__device__ inline double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Symmetric 3x3 eigen decomposition (cyclic Jacobi), the same operation
// sequence as the oracle's restatement of Eigen's SelfAdjointEigenSolver
// (ascending eigenvalues, eigenvectors as columns of evecs, row-major).  T is
// double on the odometry path; the float instance serves the FP32 plane-fit
// modes, with a stopping threshold suited to float.
template <class T> struct EigStop;
template <> struct EigStop<double> {
    static __device__ __forceinline__ double tiny() { return 1e-300; }
    static __device__ __forceinline__ double rel() { return 1e-18; }
};
template <> struct EigStop<float> {
    static __device__ __forceinline__ float tiny() { return 1e-37f; }
    static __device__ __forceinline__ float rel() { return 1e-12f; }
};
template <class T>
__device__ void eig_sym3(const T* A, T* evals, T* evecs) {
    T a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = A[i * 3 + j];
    for (int sweep = 0; sweep < 50; ++sweep) {
        T off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
        T scale = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]);
        if (off == T(0) || off <= EigStop<T>::tiny() || off < EigStop<T>::rel() * scale) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                T apq = a[p][q];
                if (apq == T(0)) continue;
                T theta = (a[q][q] - a[p][p]) / (T(2) * apq);
                T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
                T c = T(1) / sqrt(t * t + T(1)), s = t * c;
                for (int k = 0; k < 3; ++k) {
                    T akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    T apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    T vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    int idx[3] = {0, 1, 2};
    T d[3] = {a[0][0], a[1][1], a[2][2]};
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (d[idx[j]] < d[idx[i]]) { int t = idx[i]; idx[i] = idx[j]; idx[j] = t; }
    for (int c = 0; c < 3; ++c) {
        evals[c] = d[idx[c]];
        for (int r = 0; r < 3; ++r) evecs[r * 3 + c] = v[r][idx[c]];
    }
}

}  // namespace vmp
