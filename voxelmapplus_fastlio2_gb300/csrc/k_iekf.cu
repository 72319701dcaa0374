// IESKF::update (ieskf.cpp:125-156) with the measurement model of
// LIOBuilder::sharedUpdateFunc (lio_builder.cpp:250-311) and
// VoxelMap::buildResidual (voxel_map.cpp:258-276).
//
// k_residual: one thread per downsampled point (grid-stride over a fixed
// grid).  What decides a voxel key or the residual value is computed exactly
// as the reference does (FP64, its operation order, no FMA): the world point
// r_wl p + p_wl, floor(p / voxel_size) and r = n . (p_w - mean).  The gate's
// variance and the weight use the reduced forms
//     n^T (R S R^T + [p]x Prr [p]x^T + Ppp) n = u^T S u + v^T Prr v + n^T Ppp n,
//     u = R^T n, v = n x p,      r_cov = u^T S u,
// and the H / b accumulation uses FMA; these differ from the reference's
// dense evaluation only by rounding (relative 1e-16), which cannot move a gate
// decision except for a residual within that distance of its threshold.
// Accumulation: the valid points of a warp's 32 are compacted (ballot, lane
// order) into a shared-memory row per point -- J, J w, r, 1 -- and lane k of
// the warp then adds entry k of the upper triangle of H (then b, then the
// valid count) over those rows: one FMA per row and value, every lane busy,
// one accumulator per lane instead of 28 per thread.  Warps, then blocks are
// folded in a fixed order; the last CTA to finish folds the block partials
// (a fixed stripe-then-sum tree) and runs the filter step, so the result
// depends only on the grid, which depends only on the scan size bound.
//
// The filter step solves the reference's information-form normal equations
//     H = J^T P^-1 J + E Hm E^T,  b = J^T P^-1 d + E bm,  step = -H^-1 b
// (E selects the 6 -- or 12 -- measured coordinates) without a 23x23 inverse:
// with D = J^-1 (block diagonal: identity except the rot, rot_ext and S2
// blocks), M = D P D^T and d' = D d,
//     S = I + Hm M_EE,  K = M_E S^-1,  step = -d' + K (Hm d'_E - bm),
//     H^-1 = M - K Hm (E^T M),
// which is the same solution (Woodbury identity); it needs one NJ x NJ
// Gauss-Jordan solve and products with block-diagonal matrices, all spread
// over the lanes, with the transcendental functions of the boxminus / boxplus
// on separate lanes.
#include <atomic>
#include <cstdlib>

#include "kernels.cuh"

namespace vmp {

constexpr int kIekfThreads = 256;
constexpr int kPartStride2 = 96;  // >= NJ(NJ+1)/2 + NJ + 1 for NJ = 12

template <int NJ>
struct Red {
    static constexpr int NH = NJ * (NJ + 1) / 2;
    static constexpr int NV = NH + NJ + 1;  // H upper triangle, b, count
    static constexpr int VPL = (NV + 31) / 32;  // values per lane
    static constexpr int RW = 2 * NJ + 2;  // row: J, J w, r, 1
    static constexpr int STRIPES = kIekfThreads / NV;  // last-CTA fold
};

// ---------------------------------------------------------------- point part
// Gate of one point (buildResidual) and, for a valid one, its Jacobian row J,
// weight w and residual r (sharedUpdateFunc loop 2).  from_down: the LiDAR
// point is the downsampled float point (after calcBodyCov's z == 0 fix, as
// k_body_cov stores it), else the FP64 point of s.pl.
template <int NJ>
__device__ inline bool residual_row(int i, const DScan& s, const DMap& m, int from_down, const double* rwl,
                                    const double* pwl, const double* rot, const double* rext, const double* pext,
                                    const double* Prr, const double* Ppp, double* J, double& w, double& r) {
    double pl[3];
    if (from_down) {
        const float4 q = s.down[i];
        pl[0] = (double)q.x; pl[1] = (double)q.y; pl[2] = (double)q.z;
        if (pl[2] == 0) pl[2] = 0.001;
    } else {
        pl[0] = s.pl[i * 3]; pl[1] = s.pl[i * 3 + 1]; pl[2] = s.pl[i * 3 + 2];
    }
    double pw[3];
    m3v(rwl, pl, pw);
    for (int a = 0; a < 3; ++a) pw[a] = pw[a] + pwl[a];
    int64_t key[3];
    const bool inr = voxel_index(pw, m.voxel_size, m.voxel_inv, key);
    const uint32_t rec = inr ? map_find(m, pack_key(key[0], key[1], key[2])) : kNoRec;
    const double* cl = s.covl + (size_t)i * 9;
    // u = R^T n and r_cov = u^T S u of a plane found in this call: the
    // accumulation below uses the same values (same operations), so they are
    // formed once; a miss recomputes them from the stored normal
    double u[3], r_cov = 0.0, n[3];
    r = 0.0;
    bool fresh = false;
    int valid = 0;
    if (rec != kNoRec) {
        const RecHot hot = m.hot[rec];
        if (hot.flags & F_PLANE) {
            for (int c = 0; c < 3; ++c) n[c] = hot.norm[c];
            const double p2m[3] = {pw[0] - hot.mean[0], pw[1] - hot.mean[1], pw[2] - hot.mean[2]};
            r = dot3(n, p2m);
            // v = n x p_l
            double v[3], su[3], pv[3], pn[3];
            for (int c = 0; c < 3; ++c) u[c] = fma(rwl[6 + c], n[2], fma(rwl[3 + c], n[1], rwl[c] * n[0]));
            v[0] = fma(n[1], pl[2], -n[2] * pl[1]);
            v[1] = fma(n[2], pl[0], -n[0] * pl[2]);
            v[2] = fma(n[0], pl[1], -n[1] * pl[0]);
            for (int c = 0; c < 3; ++c) {
                su[c] = fma(cl[c * 3 + 2], u[2], fma(cl[c * 3 + 1], u[1], cl[c * 3] * u[0]));
                pv[c] = fma(Prr[c * 3 + 2], v[2], fma(Prr[c * 3 + 1], v[1], Prr[c * 3] * v[0]));
                pn[c] = fma(Ppp[c * 3 + 2], n[2], fma(Ppp[c * 3 + 1], n[1], Ppp[c * 3] * n[0]));
            }
            const double t1 = fma(u[2], su[2], fma(u[1], su[1], u[0] * su[0]));
            const double t2 = fma(v[2], pv[2], fma(v[1], pv[1], v[0] * pv[0]));
            const double t3 = fma(n[2], pn[2], fma(n[1], pn[1], n[0] * pn[0]));
            const double sigma = t1 + t2 + t3;
            r_cov = t1;
            fresh = true;
            valid = fabs(r) < 3.0 * sqrt(sigma) ? 1 : 0;
            s.rvalid[i] = valid;
            s.rnorm[i * 3] = n[0]; s.rnorm[i * 3 + 1] = n[1]; s.rnorm[i * 3 + 2] = n[2];
            s.rres[i] = r;
        } else {
            s.rvalid[i] = 0;
        }
    } else {
        // a miss keeps the record of the previous iteration / scan
        valid = s.rvalid[i];
        if (valid) {
            for (int c = 0; c < 3; ++c) n[c] = s.rnorm[i * 3 + c];
            r = s.rres[i];
        }
    }
    if (!valid) return false;
    if (!fresh) {
        double su[3];
        for (int c = 0; c < 3; ++c) u[c] = fma(rwl[6 + c], n[2], fma(rwl[3 + c], n[1], rwl[c] * n[0]));
        for (int c = 0; c < 3; ++c) su[c] = fma(cl[c * 3 + 2], u[2], fma(cl[c * 3 + 1], u[1], cl[c * 3] * u[0]));
        r_cov = fma(u[2], su[2], fma(u[1], su[1], u[0] * su[0]));
    }
    w = r_cov < 0.0002 ? 5000 : 1.0 / r_cov;
    // J = [n, (-rot^T n) x q, ...]  with q = rot_ext p_l + pos_ext
    double q[3], v1[3];
    for (int c = 0; c < 3; ++c) {
        q[c] = fma(rext[c * 3 + 2], pl[2], fma(rext[c * 3 + 1], pl[1], rext[c * 3] * pl[0])) + pext[c];
        v1[c] = -fma(rot[6 + c], n[2], fma(rot[3 + c], n[1], rot[c] * n[0]));
    }
    J[0] = n[0]; J[1] = n[1]; J[2] = n[2];
    J[3] = fma(v1[1], q[2], -v1[2] * q[1]);
    J[4] = fma(v1[2], q[0], -v1[0] * q[2]);
    J[5] = fma(v1[0], q[1], -v1[1] * q[0]);
    if (NJ == 12) {
        // (-(r_wl^T n)) x p_l and rot^T n
        J[6 % NJ] = -fma(u[1], pl[2], -u[2] * pl[1]);
        J[7 % NJ] = -fma(u[2], pl[0], -u[0] * pl[2]);
        J[8 % NJ] = -fma(u[0], pl[1], -u[1] * pl[0]);
        J[9 % NJ] = -v1[0]; J[10 % NJ] = -v1[1]; J[11 % NJ] = -v1[2];
    }
    return true;
}

// ---------------------------------------------------------------- filter step
// Block-diagonal factor with identity outside the rot (3-5), rot_ext (6-8) and
// S2 (21-22) blocks: D = J^-1 during the iterations, L at the end.
struct BlkDiag {
    double r[9], e[9], g[4];
};

struct IekfSm {
    double M[529];  // D P D^T
    double T[529];  // scratch
    double aug[12 * 24];
    double K[23 * 12];
    double prow[24], col[12];
    double d[23], dp[23], y[12], step[23];
    BlkDiag D;
    double ip;
    int piv;
};

__device__ inline void inv3(const double* A, double* o) {
    const double c00 = A[4] * A[8] - A[5] * A[7], c01 = A[5] * A[6] - A[3] * A[8], c02 = A[3] * A[7] - A[4] * A[6];
    const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
    const double id = 1.0 / det;
    o[0] = c00 * id; o[1] = (A[2] * A[7] - A[1] * A[8]) * id; o[2] = (A[1] * A[5] - A[2] * A[4]) * id;
    o[3] = c01 * id; o[4] = (A[0] * A[8] - A[2] * A[6]) * id; o[5] = (A[2] * A[3] - A[0] * A[5]) * id;
    o[6] = c02 * id; o[7] = (A[1] * A[6] - A[0] * A[7]) * id; o[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

__device__ inline int blk_of(int i) { return (i >= 3 && i < 6) ? 0 : (i >= 6 && i < 9) ? 1 : (i >= 21) ? 2 : -1; }

// (B X)(i, j), X with leading dimension ld
__device__ inline double bd_row(const BlkDiag& B, const double* X, int ld, int i, int j) {
    const int b = blk_of(i);
    if (b < 0) return X[i * ld + j];
    if (b == 2) {
        const int a = i - 21;
        return fma(B.g[a * 2 + 1], X[22 * ld + j], B.g[a * 2] * X[21 * ld + j]);
    }
    const double* Dm = b == 0 ? B.r : B.e;
    const int o = b == 0 ? 3 : 6, a = i - o;
    return fma(Dm[a * 3 + 2], X[(o + 2) * ld + j], fma(Dm[a * 3 + 1], X[(o + 1) * ld + j], Dm[a * 3] * X[o * ld + j]));
}
// (X B^T)(i, j), X 23 x 23
__device__ inline double bd_col(const BlkDiag& B, const double* X, int i, int j) {
    const int b = blk_of(j);
    const double* r = X + i * 23;
    if (b < 0) return r[j];
    if (b == 2) {
        const int a = j - 21;
        return fma(B.g[a * 2 + 1], r[22], B.g[a * 2] * r[21]);
    }
    const double* Dm = b == 0 ? B.r : B.e;
    const int o = b == 0 ? 3 : 6, a = j - o;
    return fma(Dm[a * 3 + 2], r[o + 2], fma(Dm[a * 3 + 1], r[o + 1], Dm[a * 3] * r[o]));
}

// out = B X B^T for a 23 x 23 X (global or shared), tmp 529 doubles; all threads.
__device__ void bd_sandwich(const BlkDiag& B, const double* X, double* tmp, double* out) {
    for (int e = threadIdx.x; e < 529; e += blockDim.x) tmp[e] = bd_row(B, X, 23, e / 23, e % 23);
    __syncthreads();
    for (int e = threadIdx.x; e < 529; e += blockDim.x) out[e] = bd_col(B, tmp, e / 23, e % 23);
    __syncthreads();
}

// Gauss-Jordan with partial pivoting on s.aug = [S | I] (nj x 2nj); S^-1 ends
// in the right half.  One warp (the caller's); the other warps wait at the
// caller's next __syncthreads.
__device__ void gauss_jordan_warp(IekfSm& s, int nj) {
    const int lane = threadIdx.x & 31;
    const int w = 2 * nj;
    for (int k = 0; k < nj; ++k) {
        // pivot: largest |a_ik|, i >= k; magnitudes of doubles order like the
        // integers of their high words (ties go to the lower row); the
        // butterfly leaves the winner on every lane
        const int i = k + lane;
        int key = -1;
        if (i < nj) key = __double2hiint(s.aug[i * w + k]) & 0x7fffffff;
        int best = i;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const int ok = __shfl_xor_sync(0xffffffffu, key, o);
            const int oi = __shfl_xor_sync(0xffffffffu, best, o);
            if (ok > key || (ok == key && oi < best)) { key = ok; best = oi; }
        }
        const int p = best;
        if (p != k && lane < w) {
            const double a = s.aug[k * w + lane];
            s.aug[k * w + lane] = s.aug[p * w + lane];
            s.aug[p * w + lane] = a;
        }
        __syncwarp();
        if (lane < w) s.prow[lane] = s.aug[k * w + lane] * (1.0 / s.aug[k * w + k]);
        if (lane < nj) s.col[lane] = s.aug[lane * w + k];
        __syncwarp();
        for (int e = lane; e < nj * w; e += 32) {
            const int r = e / w, j = e - r * w;
            s.aug[e] = (r == k) ? s.prow[j] : fma(-s.col[r], s.prow[j], s.aug[e]);
        }
        __syncwarp();
    }
}

// The 15 linear coordinates of the error state: pos (0-2) and pos_ext, vel,
// bg, ba (9-20); their offsets in DState (doubles) and in the 23-vector.
__device__ inline int lin_state_off(int u) { return u < 3 ? u : u + 18; }
__device__ inline int lin_delta_idx(int u) { return u < 3 ? u : u + 6; }

// One pass of the IESKF::update loop body after func_ (ieskf.cpp:135-148) in
// the information-form rewrite described at the top of this file, in two
// parts.  iekf_boxminus: delta = x boxminus x_pred and D = J^-1, the
// transcendental pieces on separate warps (thread `base`: rot, base + 32:
// rot_ext, base + 64: the S2 block, base + 96 .. 110: the linear
// coordinates); it needs nothing of the measurement, so it runs in its own
// kernel (k_iekf_boxminus) beside the iteration's point kernel.
// iekf_step_rest: the rest, in the fold kernel after its fold.  H / b of the
// measurement (nj x nj, nj) are in shared memory.  One CTA.
__device__ void iekf_boxminus(const DFilter* f, IekfSm& s, int base) {
    const int t = threadIdx.x;
    const DState& x = f->x;
    const DState& xp = f->x_pred;
    if (t == base) {
        double J[9];
        rot_minus(x.rot, xp.rot, s.d + 3);
        so3_right_jac(s.d + 3, J);
        inv3(J, s.D.r);
    } else if (t == base + 32) {
        double J[9];
        rot_minus(x.rot_ext, xp.rot_ext, s.d + 6);
        so3_right_jac(s.d + 6, J);
        inv3(J, s.D.e);
    } else if (t == base + 64) {
        double Nx[6], Mx[6], A[4];
        s2_minus(x.g, xp.g, s.d + 21);
        s2_Nx(x.g, Nx);
        s2_Mx_res(xp.g, s.d + 21, Mx);
        mm<2, 3, 2>(Nx, Mx, A);
        const double id = 1.0 / (A[0] * A[3] - A[1] * A[2]);
        s.D.g[0] = A[3] * id; s.D.g[1] = -A[1] * id;
        s.D.g[2] = -A[2] * id; s.D.g[3] = A[0] * id;
    } else if (t >= base + 96 && t < base + 111) {
        const int u = t - base - 96;
        const double* xs = reinterpret_cast<const double*>(&x);
        const double* ps = reinterpret_cast<const double*>(&xp);
        s.d[lin_delta_idx(u)] = xs[lin_state_off(u)] - ps[lin_state_off(u)];
    }
}
__device__ void iekf_step_rest(DFilter* f, IekfSm& s, const double* Hm, const double* bm, int nj, double eps) {
    const int t = threadIdx.x;
    if (t < 23) s.dp[t] = bd_row(s.D, s.d, 1, t, 0);
    bd_sandwich(s.D, f->P, s.T, s.M);  // M = D P D^T
    // S = I + Hm M_EE as [S | I];  y = Hm d'_E - bm
    const int w = 2 * nj;
    for (int e = t; e < nj * w; e += blockDim.x) {
        const int i = e / w, j = e - i * w;
        double v;
        if (j < nj) {
            double a = 0.0;
            for (int k = 0; k < nj; ++k) a = fma(Hm[i * 12 + k], s.M[k * 23 + j], a);
            v = (i == j ? 1.0 : 0.0) + a;
        } else {
            v = (j - nj == i) ? 1.0 : 0.0;
        }
        s.aug[e] = v;
    }
    if (t >= 224 && t - 224 < nj) {
        const int i = t - 224;
        double a = 0.0;
        for (int k = 0; k < nj; ++k) a = fma(Hm[i * 12 + k], s.dp[k], a);
        s.y[i] = a - bm[i];
    }
    __syncthreads();
    if (t < 32) gauss_jordan_warp(s, nj);
    __syncthreads();
    // K = M_E S^-1
    for (int e = t; e < 23 * nj; e += blockDim.x) {
        const int i = e / nj, j = e - i * nj;
        double a = 0.0;
        for (int k = 0; k < nj; ++k) a = fma(s.M[i * 23 + k], s.aug[k * w + nj + j], a);
        s.K[i * 12 + j] = a;
    }
    __syncthreads();
    if (t < 23) {
        double a = 0.0;
        for (int j = 0; j < nj; ++j) a = fma(s.K[t * 12 + j], s.y[j], a);
        s.step[t] = a - s.dp[t];
    }
    __syncthreads();
    // x = x boxplus step, again one warp per transcendental piece
    DState& xm = f->x;
    if (t == 0) {
        rot_plus(xm.rot, s.step + 3);
    } else if (t == 32) {
        rot_plus(xm.rot_ext, s.step + 6);
    } else if (t == 64) {
        s2_plus(xm.g, s.step + 21);
    } else if (t >= 96 && t < 111) {
        const int u = t - 96;
        double* xs = reinterpret_cast<double*>(&xm);
        xs[lin_state_off(u)] = xs[lin_state_off(u)] + s.step[lin_delta_idx(u)];
    } else if (t == 128) {
        double mx = s.step[0];
        for (int i = 1; i < 23; ++i) mx = fmax(mx, s.step[i]);
        f->iters = f->iters + 1;
        if (mx < eps) f->converged = 1;
    }
    for (int e = t; e < 529; e += blockDim.x) f->Hinv[e] = s.M[e];
    for (int e = t; e < 23 * 12; e += blockDim.x) f->K[e] = s.K[e];
    if (t < 23) f->delta[t] = s.step[t];
}

// ---------------------------------------------------------------- kernels
// The boxminus part of an iteration's step (x boxminus x_pred and D = J^-1),
// one CTA of 128 threads.  It reads only x and x_pred, so it runs beside the
// iteration's point kernel (on a side stream) and the fold kernel reads its
// result: its transcendentals leave the fold's critical path.
__global__ void __launch_bounds__(128) k_iekf_boxminus(DFilter* f) {
    __shared__ IekfSm sm;
    if (f->converged) return;  // uniform
    iekf_boxminus(f, sm, 0);
    __syncthreads();
    const int t = threadIdx.x;
    if (t < 23) f->bmx_d[t] = sm.d[t];
    else if (t < 32) f->bmx_D[t - 23] = sm.D.r[t - 23];
    else if (t < 41) f->bmx_D[9 + t - 32] = sm.D.e[t - 32];
    else if (t < 45) f->bmx_D[18 + t - 41] = sm.D.g[t - 41];
}

// IESKF::update entry (ieskf.cpp:125-130): predict_x = x, delta = 0.
__global__ void k_update_begin(DFilter* f) {
    const int t = threadIdx.x;
    const double* xs = reinterpret_cast<const double*>(&f->x);
    double* ps = reinterpret_cast<double*>(&f->x_pred);
    for (int e = t; e < (int)(sizeof(DState) / sizeof(double)); e += blockDim.x) ps[e] = xs[e];
    if (t < 23) f->delta[t] = 0.0;
    if (t == 0) {
        f->converged = 0;
        f->iters = 0;
        f->effect_num = 0;
        f->no_effect = 0;
    }
}

// Dynamic shared memory of k_residual<NJ>: the warps' row tiles, later reused
// for the block fold and the filter step's scratch.
template <int NJ>
constexpr size_t residual_smem_bytes() {
    using R = Red<NJ>;
    constexpr size_t rows = sizeof(double) * (kIekfThreads / 32) * 32 * R::RW;
    constexpr size_t fold = sizeof(double) * (kIekfThreads / 32) * 32 * R::VPL;
    return rows > fold ? rows : fold;
}
// ... and of k_residual_fold<NJ>: the filter step's scratch, then the stripes.
constexpr int kFoldThreads = kIekfThreads;
template <int NJ>
constexpr size_t fold_smem_bytes() {
    using R = Red<NJ>;
    return (sizeof(IekfSm) + 15) / 16 * 16 + sizeof(double) * (R::STRIPES + 1) * R::NV;
}

// func_ (sharedUpdateFunc) over all downsampled points: per block the sums of
// the upper triangle of H, of b and of the valid count (block partials).
template <int NJ, int MINB>
__global__ void __launch_bounds__(kIekfThreads, MINB) k_residual(DFilter* f, DScan s, DMap m, int from_down) {
    using R = Red<NJ>;
    constexpr int kWarps = kIekfThreads / 32;
    extern __shared__ __align__(16) unsigned char smem_dyn[];
    __shared__ double s_rwl[9], s_pwl[3], s_rot[9], s_rext[9], s_pext[3], s_prr[9], s_ppp[9];
    if (f->converged) return;  // written by the previous launch; uniform
    const int n = *s.d_n_down;
    // the grid is sized for the stream's largest scan: blocks past this
    // scan's points return (the fold reads the partials of the others; block
    // 0 always writes one)
    if (blockIdx.x > 0 && (long long)blockIdx.x * blockDim.x >= n) return;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // R_wl = rot rot_ext and p_wl = rot pos_ext + pos, one entry per thread
    if (t < 9) {
        s_rwl[t] = mm3_entry(f->x.rot, f->x.rot_ext, t);
    } else if (t < 12) {
        s_pwl[t - 9] = m3v_entry(f->x.rot, f->x.pos_ext, t - 9) + f->x.pos[t - 9];
    } else if (t >= 32 && t < 41) {
        const int a = t - 32;
        s_rot[a] = f->x.rot[a];
        s_rext[a] = f->x.rot_ext[a];
        s_prr[a] = f->P[(3 + a / 3) * 23 + 3 + a % 3];
        s_ppp[a] = f->P[(a / 3) * 23 + a % 3];
        if (a < 3) s_pext[a] = f->x.pos_ext[a];
    }
    // the values this lane accumulates: entry k = lane + 32 v is the product
    // of row slots oa[v] and ob[v] (H(a, b): J w [a] J[b]; b(a): J w [a] r;
    // the count: 1 * 1)
    int oa[R::VPL], ob[R::VPL];
#pragma unroll
    for (int v = 0; v < R::VPL; ++v) {
        const int k = lane + 32 * v;
        oa[v] = -1;
        ob[v] = 0;
        if (k < R::NH) {
            int a = 0, rem = k;
            while (rem >= NJ - a) { rem -= NJ - a; ++a; }
            oa[v] = NJ + a;
            ob[v] = a + rem;
        } else if (k < R::NH + NJ) {
            oa[v] = NJ + (k - R::NH);
            ob[v] = 2 * NJ;
        } else if (k == R::NH + NJ) {
            oa[v] = ob[v] = 2 * NJ + 1;
        }
    }
    double acc[R::VPL];
#pragma unroll
    for (int v = 0; v < R::VPL; ++v) acc[v] = 0.0;
    double* wrows = reinterpret_cast<double*>(smem_dyn) + (size_t)warp * 32 * R::RW;
    __syncthreads();
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int i = base + t;
        double J[NJ], w = 0.0, r = 0.0;
        const bool valid = i < n && residual_row<NJ>(i, s, m, from_down, s_rwl, s_pwl, s_rot, s_rext, s_pext, s_prr,
                                                     s_ppp, J, w, r);
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
        if (valid) {
            double* row = wrows + __popc(vm & ((1u << lane) - 1u)) * R::RW;
#pragma unroll
            for (int a = 0; a < NJ; ++a) {
                row[a] = J[a];
                row[NJ + a] = J[a] * w;
            }
            row[2 * NJ] = r;
            row[2 * NJ + 1] = 1.0;
        }
        __syncwarp();
        const int cnt = __popc(vm);
        for (int j = 0; j < cnt; ++j) {
            const double* row = wrows + j * R::RW;
#pragma unroll
            for (int v = 0; v < R::VPL; ++v)
                if (oa[v] >= 0) acc[v] = fma(row[oa[v]], row[ob[v]], acc[v]);
        }
        __syncwarp();
    }
    // warps -> block, in warp order
    __syncthreads();
    double* s_red = reinterpret_cast<double*>(smem_dyn);
#pragma unroll
    for (int v = 0; v < R::VPL; ++v) s_red[(warp * R::VPL + v) * 32 + lane] = acc[v];
    __syncthreads();
    for (int k = t; k < R::NV; k += blockDim.x) {
        const int v = k >> 5, l = k & 31;
        double x = s_red[v * 32 + l];
        for (int w2 = 1; w2 < kWarps; ++w2) x = x + s_red[(w2 * R::VPL + v) * 32 + l];
        s.partials[blockIdx.x * kPartStride2 + k] = x;
    }
}

// The grid's block partials folded in a fixed order -- thread (stripe q,
// value k) adds blocks q, q + STRIPES, ... in order, then the stripes are
// added in order -- and the filter step of this iteration.  One CTA.
template <int NJ>
__global__ void __launch_bounds__(kFoldThreads) k_residual_fold(DFilter* f, DScan s, int G, double eps, int do_step) {
    using R = Red<NJ>;
    extern __shared__ __align__(16) unsigned char smem_dyn[];
    __shared__ double sH[144], sb[12];
    if (f->converged) return;  // uniform
    const int t = threadIdx.x;
    IekfSm& sm = *reinterpret_cast<IekfSm*>(smem_dyn);
    double* s_red = reinterpret_cast<double*>(smem_dyn + (sizeof(IekfSm) + 15) / 16 * 16);
    if (do_step) {  // k_iekf_boxminus's result
        if (t < 23) sm.d[t] = f->bmx_d[t];
        else if (t < 32) sm.D.r[t - 23] = f->bmx_D[t - 23];
        else if (t < 41) sm.D.e[t - 32] = f->bmx_D[9 + t - 32];
        else if (t < 45) sm.D.g[t - 41] = f->bmx_D[18 + t - 41];
    }
    // the blocks of the grid that held points (k_residual's others return)
    const int Gw = max(1, min(G, (*s.d_n_down + kIekfThreads - 1) / kIekfThreads));
    if (t < R::STRIPES * R::NV) {
        const int q = t / R::NV, k = t - q * R::NV;
        double x = 0.0;
        for (int b = q; b < Gw; b += R::STRIPES) x = x + s.partials[b * kPartStride2 + k];
        s_red[q * R::NV + k] = x;
    }
    __syncthreads();
    double* s_sum = s_red + R::STRIPES * R::NV;
    for (int k = t; k < R::NV; k += blockDim.x) {
        double x = s_red[k];
        for (int q = 1; q < R::STRIPES; ++q) x = x + s_red[q * R::NV + k];
        s_sum[k] = x;
    }
    __syncthreads();
    for (int e = t; e < 144; e += blockDim.x) {
        const int r = e / 12, c = e % 12;
        double v = 0.0;
        if (r < NJ && c < NJ) {
            const int a = r < c ? r : c, b = r < c ? c : r;
            v = s_sum[a * NJ - a * (a - 1) / 2 + (b - a)];
        }
        sH[e] = v;
        f->Hm[e] = v;
    }
    if (t < 12) {
        sb[t] = t < NJ ? s_sum[R::NH + t] : 0.0;
        f->bm[t] = sb[t];
    }
    if (t == 0) {
        const int eff = (int)s_sum[R::NH + NJ];
        f->effect_num = eff;
        if (eff < 1) f->no_effect = 1;
    }
    __syncthreads();
    if (do_step) iekf_step_rest(f, sm, sH, sb, NJ, eps);
}

// P = L H^-1 L^T (ieskf.cpp:149-155) with H^-1 = M - K Hm (E^T M) of the last
// iteration.  P is not exactly symmetric after the reference's own recursion,
// and neither is M: the row block E^T M (not the transposed column block)
// keeps this the exact inverse of the nonsymmetric H.
__global__ void k_update_end(DFilter* f, int nj) {
    __shared__ double sM[529], sT[529], sKH[23 * 12];
    __shared__ BlkDiag L;
    const int t = threadIdx.x;
    if (f->iters == 0) return;  // uniform
    for (int e = t; e < 529; e += blockDim.x) sM[e] = f->Hinv[e];
    const double* d = f->delta;
    if (t == 0) {
        so3_right_jac(d + 3, L.r);
    } else if (t == 32) {
        so3_right_jac(d + 6, L.e);
    } else if (t == 64) {
        double Nx[6], Mx[6];
        s2_Nx(f->x.g, Nx);
        s2_Mx_res(f->x_pred.g, d + 21, Mx);
        mm<2, 3, 2>(Nx, Mx, L.g);
    }
    for (int e = t; e < 23 * nj; e += blockDim.x) {
        const int i = e / nj, j = e - i * nj;
        double a = 0.0;
        for (int k = 0; k < nj; ++k) a = fma(f->K[i * 12 + k], f->Hm[k * 12 + j], a);
        sKH[i * 12 + j] = a;
    }
    __syncthreads();
    for (int e = t; e < 529; e += blockDim.x) {
        const int i = e / 23, j = e - i * 23;
        double a = 0.0;
        for (int k = 0; k < nj; ++k) a = fma(sKH[i * 12 + k], sM[k * 23 + j], a);
        sT[e] = sM[e] - a;
    }
    __syncthreads();
    bd_sandwich(L, sT, sM, sT);
    for (int e = t; e < 529; e += blockDim.x) f->P[e] = sT[e];
}

// ---------------------------------------------------------------- launchers
void launch_update_begin(DFilter* f, cudaStream_t st) {
    VMP_NOTE_LAUNCH();
    k_update_begin<<<1, 64, 0, st>>>(f);
}
// Resident CTAs per SM that k_residual is compiled for (register budget):
// 3 (80 registers, no spills) or 4 (64 registers, a few spilled words); the
// arithmetic is the same either way.  4 by default: one stream runs as fast
// with either, and beside other streams' kernels the smaller budget leaves
// them register file.  VMP_RESIDUAL_CTAS_PER_SM (at load) and
// vmp_set_residual_ctas_per_sm set it; a change bumps the launch-shape epoch,
// so that captured scan graphs are captured again with the new kernel.
static std::atomic<int> g_residual_minb{4};
static std::atomic<long long> g_shape_epoch{0};

void residual_set_ctas_per_sm(int c) {
    const int v = c == 4 ? 4 : 3;
    if (g_residual_minb.exchange(v) != v) g_shape_epoch.fetch_add(1);
}
int residual_ctas_per_sm() { return g_residual_minb.load(); }
long long launch_shape_epoch() { return g_shape_epoch.load(); }

template <int NJ, int MINB>
static cudaError_t set_residual_smem() {
    return cudaFuncSetAttribute(k_residual<NJ, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)residual_smem_bytes<NJ>());
}
cudaError_t residual_setup() {
    static const bool from_env = [] {
        if (const char* v = std::getenv("VMP_RESIDUAL_CTAS_PER_SM")) g_residual_minb = std::atoi(v) == 3 ? 3 : 4;
        return true;
    }();
    (void)from_env;
    cudaError_t e = set_residual_smem<6, 3>();
    if (e == cudaSuccess) e = set_residual_smem<6, 4>();
    if (e == cudaSuccess) e = set_residual_smem<12, 3>();
    if (e == cudaSuccess) e = set_residual_smem<12, 4>();
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_residual_fold<6>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)fold_smem_bytes<6>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_residual_fold<12>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)fold_smem_bytes<12>());
    return e;
}
// one point per thread and tile; the fold and the reduction order follow the
// grid, which depends only on n_max (the bound of the downsampled count)
static int residual_grid(const DScan& s, int n_max) {
    int grid = (n_max + kIekfThreads - 1) / kIekfThreads;
    if (grid > s.res_blocks) grid = s.res_blocks;
    return grid < 1 ? 1 : grid;
}
void launch_residual_points(DFilter* f, DScan& s, const DMap& m, int n_max, int estimate_ext, cudaStream_t st,
                            int from_down) {
    const int grid = residual_grid(s, n_max);
    VMP_NOTE_LAUNCH();
    if (estimate_ext) {
        if (g_residual_minb == 4)
            k_residual<12, 4><<<grid, kIekfThreads, residual_smem_bytes<12>(), st>>>(f, s, m, from_down);
        else
            k_residual<12, 3><<<grid, kIekfThreads, residual_smem_bytes<12>(), st>>>(f, s, m, from_down);
    } else {
        if (g_residual_minb == 4)
            k_residual<6, 4><<<grid, kIekfThreads, residual_smem_bytes<6>(), st>>>(f, s, m, from_down);
        else
            k_residual<6, 3><<<grid, kIekfThreads, residual_smem_bytes<6>(), st>>>(f, s, m, from_down);
    }
}
void launch_residual_step(DFilter* f, DScan& s, int n_max, int estimate_ext, double eps, cudaStream_t st,
                          int do_step) {
    const int grid = residual_grid(s, n_max);
    VMP_NOTE_LAUNCH();
    if (estimate_ext)
        k_residual_fold<12><<<1, kFoldThreads, fold_smem_bytes<12>(), st>>>(f, s, grid, eps, do_step);
    else
        k_residual_fold<6><<<1, kFoldThreads, fold_smem_bytes<6>(), st>>>(f, s, grid, eps, do_step);
}
void launch_iekf_boxminus(DFilter* f, cudaStream_t st) {
    VMP_NOTE_LAUNCH();
    k_iekf_boxminus<<<1, 128, 0, st>>>(f);
}
void launch_residual_iter(DFilter* f, DScan& s, const DMap& m, int n_max, int estimate_ext, double eps,
                          cudaStream_t st, int do_step, int from_down) {
    if (do_step) launch_iekf_boxminus(f, st);
    launch_residual_points(f, s, m, n_max, estimate_ext, st, from_down);
    launch_residual_step(f, s, n_max, estimate_ext, eps, st, do_step);
}
void launch_update_end(DFilter* f, int estimate_ext, cudaStream_t st) {
    VMP_NOTE_LAUNCH();
    k_update_end<<<1, 256, 0, st>>>(f, estimate_ext ? 12 : 6);
}

}  // namespace vmp
