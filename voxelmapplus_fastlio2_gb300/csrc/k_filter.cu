// Small-state FP64 kernels of the iterated error-state Kalman filter and the
// per-point measurement model:
//   k_imu_init        LIOBuilder::initializeImu        lio_builder.cpp:28-63
//   k_predict_chain   undistortCloud's IMU loop        lio_builder.cpp:65-123
//                     + IESKF::predict                 ieskf.cpp:101-123
//   k_undistort       undistortCloud's point loop      lio_builder.cpp:125-152
//   k_update_begin / k_residual / k_update_end
//                     IESKF::update                    ieskf.cpp:125-156
//                     + sharedUpdateFunc               lio_builder.cpp:250-311
//                     + VoxelMap::buildResidual        voxel_map.cpp:258-276
// The residual kernel is the hot one: one thread per downsampled point
// (grid-stride over a fixed grid), FP64 world transform, hash probe, gate and
// Jacobian row, a warp-shuffle + per-block reduction of H / b, and the last
// CTA to finish folds the block partials in a fixed order (deterministic) and
// runs the 23x23 FP64 iteration step of the filter.
#include "kernels.cuh"

namespace vmp {

// ---------------------------------------------------------------- block algebra
// All matrices 23x23 row-major in shared memory; sums in k order so that the
// result equals the reference's dense Eigen products.
__device__ void blk_mm23(const double* A, const double* B, double* C) {
    for (int e = threadIdx.x; e < 529; e += blockDim.x) {
        int i = e / 23, j = e % 23;
        double s = A[i * 23] * B[j];
        for (int k = 1; k < 23; ++k) s = s + A[i * 23 + k] * B[k * 23 + j];
        C[e] = s;
    }
    __syncthreads();
}
// C = A^T * B
__device__ void blk_mm23_tn(const double* A, const double* B, double* C) {
    for (int e = threadIdx.x; e < 529; e += blockDim.x) {
        int i = e / 23, j = e % 23;
        double s = A[i] * B[j];
        for (int k = 1; k < 23; ++k) s = s + A[k * 23 + i] * B[k * 23 + j];
        C[e] = s;
    }
    __syncthreads();
}
// C = A * B^T
__device__ void blk_mm23_nt(const double* A, const double* B, double* C) {
    for (int e = threadIdx.x; e < 529; e += blockDim.x) {
        int i = e / 23, j = e % 23;
        double s = A[i * 23] * B[j * 23];
        for (int k = 1; k < 23; ++k) s = s + A[i * 23 + k] * B[j * 23 + k];
        C[e] = s;
    }
    __syncthreads();
}

// Inverse by LU with partial pivoting (first maximum), then per-column
// forward / back substitution -- the same operation sequence as the oracle's
// restatement of Eigen's PartialPivLU inverse.
__device__ void blk_inverse23(const double* A, double* inv, double* lu, int* perm) {
    for (int e = threadIdx.x; e < 529; e += blockDim.x) lu[e] = A[e];
    if (threadIdx.x < 23) perm[threadIdx.x] = threadIdx.x;
    __shared__ int s_piv;
    __syncthreads();
    for (int k = 0; k < 23; ++k) {
        if (threadIdx.x == 0) {
            int p = k;
            double best = fabs(lu[k * 23 + k]);
            for (int i = k + 1; i < 23; ++i) {
                double v = fabs(lu[i * 23 + k]);
                if (v > best) { best = v; p = i; }
            }
            s_piv = p;
            if (p != k) { int t = perm[k]; perm[k] = perm[p]; perm[p] = t; }
        }
        __syncthreads();
        int p = s_piv;
        if (p != k && threadIdx.x < 23) {
            double t = lu[k * 23 + threadIdx.x];
            lu[k * 23 + threadIdx.x] = lu[p * 23 + threadIdx.x];
            lu[p * 23 + threadIdx.x] = t;
        }
        __syncthreads();
        double piv = lu[k * 23 + k];
        if (threadIdx.x > k && threadIdx.x < 23) lu[threadIdx.x * 23 + k] = lu[threadIdx.x * 23 + k] / piv;
        __syncthreads();
        int rows = 22 - k;
        for (int e = threadIdx.x; e < rows * rows; e += blockDim.x) {
            int i = k + 1 + e / rows, j = k + 1 + e % rows;
            lu[i * 23 + j] = lu[i * 23 + j] - lu[i * 23 + k] * lu[k * 23 + j];
        }
        __syncthreads();
    }
    if (threadIdx.x < 23) {
        const int c = threadIdx.x;
        double x[23];
        for (int i = 0; i < 23; ++i) x[i] = (perm[i] == c) ? 1.0 : 0.0;
        for (int i = 0; i < 23; ++i)
            for (int j = 0; j < i; ++j) x[i] = x[i] - lu[i * 23 + j] * x[j];
        for (int i = 22; i >= 0; --i) {
            for (int j = i + 1; j < 23; ++j) x[i] = x[i] - lu[i * 23 + j] * x[j];
            x[i] = x[i] / lu[i * 23 + i];
        }
        for (int i = 0; i < 23; ++i) inv[i * 23 + c] = x[i];
    }
    __syncthreads();
}

__device__ inline void set_block3(double* M, int ld, int r0, int c0, const double* b) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) M[(r0 + i) * ld + c0 + j] = b[i * 3 + j];
}

// ---------------------------------------------------------------- IMU init
__global__ void k_imu_init(DFilter* f, const vmp_imu* imus, int n, int gravity_align, DState ext, double t_end) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double am[3] = {0, 0, 0}, gm[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) { am[a] = am[a] + imus[i].acc[a]; gm[a] = gm[a] + imus[i].gyro[a]; }
    for (int a = 0; a < 3; ++a) { am[a] = am[a] / (double)n; gm[a] = gm[a] / (double)n; }
    f->gravity_norm = sqrt(dot3(am, am));
    DState& x = f->x;
    for (int i = 0; i < 9; ++i) x.rot_ext[i] = ext.rot_ext[i];
    for (int i = 0; i < 3; ++i) { x.pos_ext[i] = ext.pos_ext[i]; x.bg[i] = gm[i]; }
    if (gravity_align) {
        // Eigen Quaternion::FromTwoVectors(normalized(-acc_mean), (0,0,-1))
        double a[3] = {-am[0], -am[1], -am[2]};
        double na = dot3(a, a);
        double v0[3], v1[3] = {0.0, 0.0, -1.0};
        for (int i = 0; i < 3; ++i) v0[i] = na > 0 ? a[i] / sqrt(na) : a[i];
        // FromTwoVectors normalises both inputs again
        double n0 = dot3(v0, v0);
        for (int i = 0; i < 3; ++i) v0[i] = n0 > 0 ? v0[i] / sqrt(n0) : v0[i];
        double n1 = dot3(v1, v1);
        for (int i = 0; i < 3; ++i) v1[i] = v1[i] / sqrt(n1);
        double c = dot3(v1, v0);
        double qw, qx, qy, qz;
        if (c < -1.0 + 1e-12) {
            double e[3] = {1, 0, 0};
            double ax[3] = {v0[1] * e[2] - v0[2] * e[1], v0[2] * e[0] - v0[0] * e[2], v0[0] * e[1] - v0[1] * e[0]};
            if (dot3(ax, ax) < 1e-12) {
                double e2[3] = {0, 1, 0};
                ax[0] = v0[1] * e2[2] - v0[2] * e2[1]; ax[1] = v0[2] * e2[0] - v0[0] * e2[2]; ax[2] = v0[0] * e2[1] - v0[1] * e2[0];
            }
            double nn = dot3(ax, ax);
            for (int i = 0; i < 3; ++i) ax[i] = ax[i] / sqrt(nn);
            c = fmax(c, -1.0);
            double w2 = (1.0 + c) * 0.5;
            qw = sqrt(w2);
            double s = sqrt(1.0 - w2);
            qx = ax[0] * s; qy = ax[1] * s; qz = ax[2] * s;
        } else {
            double ax[3] = {v0[1] * v1[2] - v0[2] * v1[1], v0[2] * v1[0] - v0[0] * v1[2], v0[0] * v1[1] - v0[1] * v1[0]};
            double s = sqrt((1.0 + c) * 2.0);
            double invs = 1.0 / s;
            qx = ax[0] * invs; qy = ax[1] * invs; qz = ax[2] * invs;
            qw = s * 0.5;
        }
        quat_to_mat(qw, qx, qy, qz, x.rot);
        double gd[3] = {0.0, 0.0, -1.0};
        double ng = dot3(gd, gd);
        for (int i = 0; i < 3; ++i) x.g[i] = (gd[i] / sqrt(ng)) * kGravity;
    } else {
        double gd[3] = {-am[0], -am[1], -am[2]};
        double ng = dot3(gd, gd);
        for (int i = 0; i < 3; ++i) x.g[i] = (ng > 0 ? gd[i] / sqrt(ng) : gd[i]) * kGravity;
    }
    for (int i = 0; i < 529; ++i) f->P[i] = (i % 24 == 0) ? 1.0 : 0.0;
    for (int i = 6; i < 12; ++i) f->P[i * 24] = 0.00001;
    for (int i = 15; i < 21; ++i) f->P[i * 24] = 0.0001;
    for (int i = 21; i < 23; ++i) f->P[i * 24] = 0.00001;
    const vmp_imu& last = imus[n - 1];
    f->last_imu_t = last.t;
    for (int a = 0; a < 3; ++a) { f->last_imu_acc[a] = last.acc[a]; f->last_imu_gyro[a] = last.gyro[a]; }
    f->last_cloud_end_time = t_end;
}

// ---------------------------------------------------------------- predict
struct PredSmem {
    double F[529];
    double G[23 * 12];
    double P[529];
    double FP[529];
    double GQ[23 * 12];
    double Q[144];
    DState x, xn;
};

// One IESKF::predict step, block-cooperative.  F and G are built by six
// threads in parallel from the pre-step state; the covariance product skips
// the structural zeros of F and G, which leaves every sum equal to the dense
// product's.
__device__ void predict_step(PredSmem& s, const double* acc, const double* gyro, double dt) {
    const int t = threadIdx.x;
    for (int e = t; e < 529; e += blockDim.x) s.F[e] = (e % 24 == 0) ? 1.0 : 0.0;
    for (int e = t; e < 23 * 12; e += blockDim.x) s.G[e] = 0.0;
    __syncthreads();
    const DState& x = s.x;
    double w[3];
    for (int i = 0; i < 3; ++i) w[i] = (gyro[i] - x.bg[i]) * dt;
    if (t == 0) {
        double wn[3] = {-(gyro[0] - x.bg[0]) * dt, -(gyro[1] - x.bg[1]) * dt, -(gyro[2] - x.bg[2]) * dt};
        double E[9];
        so3_exp(wn, E);
        set_block3(s.F, 23, 3, 3, E);
    } else if (t == 1) {
        double Jr[9], B[9];
        so3_right_jac(w, Jr);
        for (int i = 0; i < 9; ++i) B[i] = (-Jr[i]) * dt;
        set_block3(s.F, 23, 3, 15, B);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) s.G[(3 + i) * 12 + j] = B[i * 3 + j];
    } else if (t == 2) {
        double nr[9], H[9], T[9], ab[3];
        for (int i = 0; i < 9; ++i) nr[i] = -x.rot[i];
        for (int i = 0; i < 3; ++i) ab[i] = acc[i] - x.ba[i];
        hat3(ab, H);
        mm<3, 3, 3>(nr, H, T);
        for (int i = 0; i < 9; ++i) T[i] = T[i] * dt;
        set_block3(s.F, 23, 12, 3, T);
    } else if (t == 3) {
        double B[9];
        for (int i = 0; i < 9; ++i) B[i] = (-x.rot[i]) * dt;
        set_block3(s.F, 23, 12, 18, B);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) s.G[(12 + i) * 12 + 3 + j] = B[i * 3 + j];
        for (int i = 0; i < 3; ++i) {
            s.G[(15 + i) * 12 + 6 + i] = 1.0 * dt;
            s.G[(18 + i) * 12 + 9 + i] = 1.0 * dt;
            s.F[i * 23 + 12 + i] = 1.0 * dt;
        }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                if (i != j) { s.G[(15 + i) * 12 + 6 + j] = 0.0 * dt; s.G[(18 + i) * 12 + 9 + j] = 0.0 * dt; }
    } else if (t == 4) {
        double Mx[6], Nx[6], NM[4];
        s2_Mx(x.g, Mx);
        s2_Nx(x.g, Nx);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 2; ++j) s.F[(12 + i) * 23 + 21 + j] = Mx[i * 2 + j] * dt;
        mm<2, 3, 2>(Nx, Mx, NM);
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j) s.F[(21 + i) * 23 + 21 + j] = NM[i * 2 + j];
    } else if (t == 5) {
        double d[24];
        for (int i = 0; i < 24; ++i) d[i] = 0.0;
        for (int i = 0; i < 3; ++i) d[i] = x.vel[i] * dt;
        for (int i = 0; i < 3; ++i) d[3 + i] = (gyro[i] - x.bg[i]) * dt;
        double ab[3], ra[3];
        for (int i = 0; i < 3; ++i) ab[i] = acc[i] - x.ba[i];
        m3v(x.rot, ab, ra);
        for (int i = 0; i < 3; ++i) d[12 + i] = (ra[i] + x.g[i]) * dt;
        s.xn = x;
        state_plus24(s.xn, d);
    }
    __syncthreads();
    // FP = F * P ; GQ = G * Q   (zero terms of F / G skipped)
    for (int e = t; e < 529; e += blockDim.x) {
        int i = e / 23, j = e % 23;
        double acc_s = 0.0;
        bool first = true;
        for (int k = 0; k < 23; ++k) {
            double a = s.F[i * 23 + k];
            if (a == 0.0) continue;
            double p = a * s.P[k * 23 + j];
            acc_s = first ? p : acc_s + p;
            first = false;
        }
        s.FP[e] = acc_s;
    }
    for (int e = t; e < 23 * 12; e += blockDim.x) {
        int i = e / 12, j = e % 12;
        double acc_s = 0.0;
        bool first = true;
        for (int k = 0; k < 12; ++k) {
            double a = s.G[i * 12 + k];
            if (a == 0.0) continue;
            double p = a * s.Q[k * 12 + j];
            acc_s = first ? p : acc_s + p;
            first = false;
        }
        s.GQ[e] = acc_s;
    }
    __syncthreads();
    for (int e = t; e < 529; e += blockDim.x) {
        int i = e / 23, j = e % 23;
        double a1 = 0.0;
        bool first = true;
        for (int k = 0; k < 23; ++k) {
            double b = s.F[j * 23 + k];
            if (b == 0.0) continue;
            double p = s.FP[i * 23 + k] * b;
            a1 = first ? p : a1 + p;
            first = false;
        }
        double a2 = 0.0;
        first = true;
        for (int k = 0; k < 12; ++k) {
            double b = s.G[j * 12 + k];
            if (b == 0.0) continue;
            double p = s.GQ[i * 12 + k] * b;
            a2 = first ? p : a2 + p;
            first = false;
        }
        s.P[e] = a1 + a2;
    }
    __syncthreads();
    if (t == 0) s.x = s.xn;
    __syncthreads();
}

__global__ void k_predict_chain(DFilter* f, const vmp_imu* imus, int n_imu, double t_begin, double t_end,
                                DPose* poses) {
    __shared__ PredSmem s;
    __shared__ double s_in[6];
    __shared__ int s_go;
    const int t = threadIdx.x;
    for (int e = t; e < 529; e += blockDim.x) s.P[e] = f->P[e];
    for (int e = t; e < 144; e += blockDim.x) s.Q[e] = f->Q[e];
    if (t == 0) s.x = f->x;
    __syncthreads();
    const double last_end = f->last_cloud_end_time;
    if (t == 0) {
        DPose& p0 = poses[0];
        p0.offset = 0.0;
        for (int a = 0; a < 3; ++a) {
            p0.acc[a] = f->last_acc[a]; p0.gyro[a] = f->last_gyro[a];
            p0.vel[a] = s.x.vel[a]; p0.pos[a] = s.x.pos[a];
        }
        for (int a = 0; a < 9; ++a) p0.rot[a] = s.x.rot[a];
    }
    int npose = 1;
    double inp_acc[3] = {0, 0, 0}, inp_gyro[3] = {0, 0, 0};
    // imu_cache = [last_imu] + package imus
    for (int k = 0; k < n_imu; ++k) {
        double ht, hacc[3], hgyro[3];
        if (k == 0) {
            ht = f->last_imu_t;
            for (int a = 0; a < 3; ++a) { hacc[a] = f->last_imu_acc[a]; hgyro[a] = f->last_imu_gyro[a]; }
        } else {
            ht = imus[k - 1].t;
            for (int a = 0; a < 3; ++a) { hacc[a] = imus[k - 1].acc[a]; hgyro[a] = imus[k - 1].gyro[a]; }
        }
        const vmp_imu& tail = imus[k];
        if (tail.t < last_end) continue;
        double dt;
        if (t == 0) {
            for (int a = 0; a < 3; ++a) {
                double gv = 0.5 * (hgyro[a] + tail.gyro[a]);
                double av = 0.5 * (hacc[a] + tail.acc[a]);
                av = av * 9.81 / f->gravity_norm;
                s_in[a] = av;
                s_in[3 + a] = gv;
            }
        }
        __syncthreads();
        dt = (ht < last_end) ? tail.t - last_end : tail.t - ht;
        for (int a = 0; a < 3; ++a) { inp_acc[a] = s_in[a]; inp_gyro[a] = s_in[3 + a]; }
        predict_step(s, inp_acc, inp_gyro, dt);
        if (t == 0) {
            DPose& p = poses[npose];
            double ab[3], ra[3];
            for (int a = 0; a < 3; ++a) ab[a] = inp_acc[a] - s.x.ba[a];
            m3v(s.x.rot, ab, ra);
            for (int a = 0; a < 3; ++a) {
                f->last_gyro[a] = inp_gyro[a] - s.x.bg[a];
                f->last_acc[a] = ra[a] + s.x.g[a];
                p.acc[a] = f->last_acc[a];
                p.gyro[a] = f->last_gyro[a];
                p.vel[a] = s.x.vel[a];
                p.pos[a] = s.x.pos[a];
            }
            for (int a = 0; a < 9; ++a) p.rot[a] = s.x.rot[a];
            p.offset = tail.t - t_begin;
        }
        npose++;
        __syncthreads();
    }
    // final predict to the scan end with the last input
    {
        const double imu_time_end = n_imu > 0 ? imus[n_imu - 1].t : f->last_imu_t;
        double dt = t_end - imu_time_end;
        if (t == 0) s_go = 1;
        __syncthreads();
        predict_step(s, inp_acc, inp_gyro, dt);
    }
    for (int e = t; e < 529; e += blockDim.x) f->P[e] = s.P[e];
    if (t == 0) {
        f->x = s.x;
        f->npose = npose;
        if (n_imu > 0) {
            const vmp_imu& last = imus[n_imu - 1];
            f->last_imu_t = last.t;
            for (int a = 0; a < 3; ++a) { f->last_imu_acc[a] = last.acc[a]; f->last_imu_gyro[a] = last.gyro[a]; }
        }
        f->last_cloud_end_time = t_end;
        for (int a = 0; a < 3; ++a) { f->inp_acc[a] = inp_acc[a]; f->inp_gyro[a] = inp_gyro[a]; }
    }
}

// Single IESKF::predict (component entry point).
__global__ void k_predict_once(DFilter* f, double a0, double a1, double a2, double g0, double g1, double g2,
                               double dt) {
    __shared__ PredSmem s;
    for (int e = threadIdx.x; e < 529; e += blockDim.x) s.P[e] = f->P[e];
    for (int e = threadIdx.x; e < 144; e += blockDim.x) s.Q[e] = f->Q[e];
    if (threadIdx.x == 0) s.x = f->x;
    __syncthreads();
    double acc[3] = {a0, a1, a2}, gyro[3] = {g0, g1, g2};
    predict_step(s, acc, gyro, dt);
    for (int e = threadIdx.x; e < 529; e += blockDim.x) f->P[e] = s.P[e];
    if (threadIdx.x == 0) f->x = s.x;
}

// ---------------------------------------------------------------- undistort
__device__ void compensate(const DPose& head, const DPose& tail, double dt, const DState& cur, float4& q) {
    double point[3] = {(double)q.x, (double)q.y, (double)q.z};
    double wdt[3], E[9], point_rot[9];
    for (int a = 0; a < 3; ++a) wdt[a] = tail.gyro[a] * dt;
    so3_exp(wdt, E);
    mm<3, 3, 3>(head.rot, E, point_rot);
    double point_pos[3];
    for (int a = 0; a < 3; ++a) point_pos[a] = (head.pos[a] + head.vel[a] * dt) + ((0.5 * tail.acc[a]) * dt) * dt;
    double a1[3], b1[3], c1[3], d1[3], e1[3], pc[3], RT[9];
    m3v(cur.rot_ext, point, a1);
    for (int a = 0; a < 3; ++a) a1[a] = a1[a] + cur.pos_ext[a];
    m3v(point_rot, a1, b1);
    for (int a = 0; a < 3; ++a) c1[a] = (b1[a] + point_pos[a]) - cur.pos[a];
    tr<3, 3>(cur.rot, RT);
    m3v(RT, c1, d1);
    for (int a = 0; a < 3; ++a) e1[a] = d1[a] - cur.pos_ext[a];
    tr<3, 3>(cur.rot_ext, RT);
    m3v(RT, e1, pc);
    q.x = (float)pc[0]; q.y = (float)pc[1]; q.z = (float)pc[2];
}

__global__ void k_undistort(const DFilter* __restrict__ f, const DPose* __restrict__ poses, float4* cloud,
                            const int* d_n) {
    __shared__ double s_off[1024];
    __shared__ DState cur;
    const int n = *d_n;
    const int npose = f->npose;
    if (npose > 1024) return;  // bounded by max_imu (checked on the host)
    for (int i = threadIdx.x; i < npose; i += blockDim.x) s_off[i] = poses[i].offset;
    if (threadIdx.x == 0) cur = f->x;
    __syncthreads();
    if (npose < 2) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = cloud[i];
        double tau = (double)q.w / double(1000);
        // head = largest h in [0, npose-2] with offset[h] < tau
        int lo = 0, hi = npose - 2, h = -1;
        while (lo <= hi) {
            int mid = (lo + hi) >> 1;
            if (s_off[mid] < tau) { h = mid; lo = mid + 1; } else hi = mid - 1;
        }
        if (h < 0) continue;
        if (i == 0) {
            // the reference re-compensates its first point once per remaining
            // segment (its inner loop breaks at the first point, the outer
            // loop keeps going: lio_builder.cpp:138-151)
            for (int hh = h; hh >= 0; --hh) {
                double dt = tau - s_off[hh];
                compensate(poses[hh], poses[hh + 1], dt, cur, q);
            }
        } else {
            double dt = tau - s_off[h];
            compensate(poses[h], poses[h + 1], dt, cur, q);
        }
        cloud[i] = q;
    }
}

// ---------------------------------------------------------------- update
__global__ void k_update_begin(DFilter* f) {
    __shared__ double sP[529], sInv[529], lu[529];
    __shared__ int perm[23];
    for (int e = threadIdx.x; e < 529; e += blockDim.x) sP[e] = f->P[e];
    if (threadIdx.x == 0) {
        f->x_pred = f->x;
        f->converged = 0;
        f->iters = 0;
        f->effect_num = 0;
        f->no_effect = 0;
        for (int i = 0; i < 23; ++i) f->delta[i] = 0.0;
    }
    __syncthreads();
    blk_inverse23(sP, sInv, lu, perm);
    for (int e = threadIdx.x; e < 529; e += blockDim.x) f->Pinv[e] = sInv[e];
}

constexpr int kResThreads = 256;
constexpr int kPartStride = 160;  // >= 12*12 + 12 + 1

// IESKF::update loop body after func_ (ieskf.cpp:135-148), one CTA.
__device__ void ieskf_iteration_step(DFilter* f, double eps) {
    __shared__ double sJ[529], sA[529], sH[529], sInv[529], lu[529];
    __shared__ double sd[23], sb[23];
    __shared__ int perm[23];
    const int t = threadIdx.x;
    for (int e = t; e < 529; e += blockDim.x) { sJ[e] = (e % 24 == 0) ? 1.0 : 0.0; sInv[e] = f->Pinv[e]; }
    __syncthreads();
    if (t == 0) {
        state_minus(f->x, f->x_pred, sd);
        double Jr[9];
        so3_right_jac(sd + 3, Jr);
        set_block3(sJ, 23, 3, 3, Jr);
        so3_right_jac(sd + 6, Jr);
        set_block3(sJ, 23, 6, 6, Jr);
        double Nx[6], Mx[6], NM[4];
        s2_Nx(f->x.g, Nx);
        s2_Mx_res(f->x_pred.g, sd + 21, Mx);
        mm<2, 3, 2>(Nx, Mx, NM);
        sJ[21 * 23 + 21] = NM[0]; sJ[21 * 23 + 22] = NM[1];
        sJ[22 * 23 + 21] = NM[2]; sJ[22 * 23 + 22] = NM[3];
    }
    __syncthreads();
    blk_mm23_tn(sJ, sInv, sA);  // A = J^T P^-1
    // b = A * delta ; H = A * J
    if (t < 23) {
        double s = sA[t * 23] * sd[0];
        for (int k = 1; k < 23; ++k) s = s + sA[t * 23 + k] * sd[k];
        sb[t] = s;
    }
    blk_mm23(sA, sJ, sH);
    for (int e = t; e < 144; e += blockDim.x) {
        int r = e / 12, c = e % 12;
        sH[r * 23 + c] = sH[r * 23 + c] + f->Hm[e];
    }
    if (t < 12) sb[t] = sb[t] + f->bm[t];
    __syncthreads();
    blk_inverse23(sH, sInv, lu, perm);
    if (t < 23) {
        double s = sInv[t * 23] * sb[0];
        for (int k = 1; k < 23; ++k) s = s + sInv[t * 23 + k] * sb[k];
        sd[t] = -s;
    }
    __syncthreads();
    for (int e = t; e < 529; e += blockDim.x) f->Hinv[e] = sInv[e];
    if (t == 0) {
        state_plus23(f->x, sd);
        double mx = sd[0];
        for (int i = 1; i < 23; ++i) mx = fmax(mx, sd[i]);
        for (int i = 0; i < 23; ++i) f->delta[i] = sd[i];
        f->iters = f->iters + 1;
        if (mx < eps) f->converged = 1;
    }
}

template <int NJ>
__global__ void __launch_bounds__(kResThreads) k_residual(DFilter* f, DScan s, DMap m, double eps, int do_step) {
    constexpr int NV = NJ * NJ + NJ;
    __shared__ double s_red[kResThreads / 32][NV + 1];
    __shared__ double s_rwl[9], s_pwl[3], s_rot[9], s_rext[9], s_pext[3], s_prr[9], s_ppp[9];
    __shared__ int s_last;
    if (f->converged) return;  // written by the previous launch; uniform
    const int n = *s.d_n_down;
    const int t = threadIdx.x;
    if (t == 0) {
        const DState& x = f->x;
        mm<3, 3, 3>(x.rot, x.rot_ext, s_rwl);
        double rp[3];
        m3v(x.rot, x.pos_ext, rp);
        for (int a = 0; a < 3; ++a) s_pwl[a] = rp[a] + x.pos[a];
        for (int a = 0; a < 9; ++a) { s_rot[a] = x.rot[a]; s_rext[a] = x.rot_ext[a]; }
        for (int a = 0; a < 3; ++a) s_pext[a] = x.pos_ext[a];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                s_prr[i * 3 + j] = f->P[(3 + i) * 23 + 3 + j];
                s_ppp[i * 3 + j] = f->P[i * 23 + j];
            }
    }
    __syncthreads();
    double accH[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) accH[k] = 0.0;
    double cnt = 0.0;
    for (int i = blockIdx.x * blockDim.x + t; i < n; i += gridDim.x * blockDim.x) {
        double pl[3] = {s.pl[i * 3], s.pl[i * 3 + 1], s.pl[i * 3 + 2]};
        double cl[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) cl[k] = s.covl[i * 9 + k];
        double pw[3];
        m3v(s_rwl, pl, pw);
        for (int a = 0; a < 3; ++a) pw[a] = pw[a] + s_pwl[a];
        int64_t key[3];
        bool inr = voxel_index(pw, m.voxel_size, key);
        uint32_t rec = inr ? map_find(m, pack_key(key[0], key[1], key[2])) : kNoRec;
        if (rec != kNoRec) {
            const RecHot hot = m.hot[rec];
            if (hot.flags & F_PLANE) {
                // cov_world = r_wl cov_l r_wl^T + [p]x P_rr [p]x^T + P_pp
                double T1[9], T2[9], rT[9], cm[9], cmT[9], T3[9], T4[9], cw[9];
                mm<3, 3, 3>(s_rwl, cl, T1);
                tr<3, 3>(s_rwl, rT);
                mm<3, 3, 3>(T1, rT, T2);
                hat3(pl, cm);
                mm<3, 3, 3>(cm, s_prr, T3);
                tr<3, 3>(cm, cmT);
                mm<3, 3, 3>(T3, cmT, T4);
                for (int k = 0; k < 9; ++k) cw[k] = (T2[k] + T4[k]) + s_ppp[k];
                double p2m[3] = {pw[0] - hot.mean[0], pw[1] - hot.mean[1], pw[2] - hot.mean[2]};
                double r = dot3(hot.norm, p2m);
                double nc[3];
                for (int j = 0; j < 3; ++j) nc[j] = (hot.norm[0] * cw[j] + hot.norm[1] * cw[3 + j]) + hot.norm[2] * cw[6 + j];
                double sigma = dot3(nc, hot.norm);
                uint8_t valid = fabs(r) < 3.0 * sqrt(sigma) ? 1 : 0;
                s.rvalid[i] = valid;
                s.rnorm[i * 3] = hot.norm[0]; s.rnorm[i * 3 + 1] = hot.norm[1]; s.rnorm[i * 3 + 2] = hot.norm[2];
                s.rres[i] = r;
            } else {
                s.rvalid[i] = 0;
            }
        }
        if (s.rvalid[i]) {
            double nn[3] = {s.rnorm[i * 3], s.rnorm[i * 3 + 1], s.rnorm[i * 3 + 2]};
            double r = s.rres[i];
            // r_cov = n^T r_wl cov_l r_wl^T n
            double u1[3], u2[3], u3[3];
            for (int j = 0; j < 3; ++j) u1[j] = (nn[0] * s_rwl[j] + nn[1] * s_rwl[3 + j]) + nn[2] * s_rwl[6 + j];
            for (int j = 0; j < 3; ++j) u2[j] = (u1[0] * cl[j] + u1[1] * cl[3 + j]) + u1[2] * cl[6 + j];
            for (int j = 0; j < 3; ++j) u3[j] = (u2[0] * s_rwl[j * 3] + u2[1] * s_rwl[j * 3 + 1]) + u2[2] * s_rwl[j * 3 + 2];
            double r_cov = dot3(u3, nn);
            double w = r_cov < 0.0002 ? 5000 : 1.0 / r_cov;
            double J[NJ];
            J[0] = nn[0]; J[1] = nn[1]; J[2] = nn[2];
            double q[3], Hq[9], v1[3];
            m3v(s_rext, pl, q);
            for (int a = 0; a < 3; ++a) q[a] = q[a] + s_pext[a];
            hat3(q, Hq);
            for (int j = 0; j < 3; ++j) v1[j] = ((-nn[0]) * s_rot[j] + (-nn[1]) * s_rot[3 + j]) + (-nn[2]) * s_rot[6 + j];
            for (int j = 0; j < 3; ++j) J[3 + j] = (v1[0] * Hq[j] + v1[1] * Hq[3 + j]) + v1[2] * Hq[6 + j];
            if (NJ == 12) {
                double v2[3], Hp[9];
                for (int j = 0; j < 3; ++j) v2[j] = ((-nn[0]) * s_rwl[j] + (-nn[1]) * s_rwl[3 + j]) + (-nn[2]) * s_rwl[6 + j];
                hat3(pl, Hp);
                for (int j = 0; j < 3; ++j) J[(6 + j) % NJ] = (v2[0] * Hp[j] + v2[1] * Hp[3 + j]) + v2[2] * Hp[6 + j];
                for (int j = 0; j < 3; ++j) J[(9 + j) % NJ] = (nn[0] * s_rot[j] + nn[1] * s_rot[3 + j]) + nn[2] * s_rot[6 + j];
            }
#pragma unroll
            for (int a = 0; a < NJ; ++a) {
                double u = J[a] * w;
#pragma unroll
                for (int c = 0; c < NJ; ++c) accH[a * NJ + c] = accH[a * NJ + c] + u * J[c];
                accH[NJ * NJ + a] = accH[NJ * NJ + a] + u * r;
            }
            cnt = cnt + 1.0;
        }
    }
    // block reduction (fixed order)
    const int lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double v = warp_sum(accH[k]);
        if (lane == 0) s_red[warp][k] = v;
    }
    {
        double v = warp_sum(cnt);
        if (lane == 0) s_red[warp][NV] = v;
    }
    __syncthreads();
    for (int k = t; k <= NV; k += blockDim.x) {
        double v = s_red[0][k];
        for (int w = 1; w < kResThreads / 32; ++w) v = v + s_red[w][k];
        s.partials[blockIdx.x * kPartStride + k] = v;
    }
    __threadfence();
    __syncthreads();
    if (t == 0) {
        unsigned int ticket = atomicAdd(s.done_ctr, 1u);
        s_last = (ticket == gridDim.x - 1) ? 1 : 0;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // last CTA: fold block partials in block order -> H_meas (12x12), b_meas
    for (int k = t; k <= NV; k += blockDim.x) {
        double v = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) v = (b == 0) ? s.partials[k] : v + s.partials[b * kPartStride + k];
        s_red[0][k] = v;
    }
    __syncthreads();
    for (int e = t; e < 144; e += blockDim.x) {
        int r = e / 12, c = e % 12;
        f->Hm[e] = (r < NJ && c < NJ) ? s_red[0][r * NJ + c] : 0.0;
    }
    if (t < 12) f->bm[t] = t < NJ ? s_red[0][NJ * NJ + t] : 0.0;
    if (t == 0) {
        int eff = (int)s_red[0][NV];
        f->effect_num = eff;
        if (eff < 1) f->no_effect = 1;
        *s.done_ctr = 0;
    }
    __syncthreads();
    if (do_step) ieskf_iteration_step(f, eps);
}

// P = L H^-1 L^T (ieskf.cpp:151-155)
__global__ void k_update_end(DFilter* f) {
    __shared__ double sL[529], sI[529], sT[529];
    const int t = threadIdx.x;
    for (int e = t; e < 529; e += blockDim.x) { sL[e] = (e % 24 == 0) ? 1.0 : 0.0; sI[e] = f->Hinv[e]; }
    __syncthreads();
    if (f->iters == 0) return;
    if (t == 0) {
        const double* d = f->delta;
        double Jr[9];
        so3_right_jac(d + 3, Jr);
        set_block3(sL, 23, 3, 3, Jr);
        so3_right_jac(d + 6, Jr);
        set_block3(sL, 23, 6, 6, Jr);
        double Nx[6], Mx[6], NM[4];
        s2_Nx(f->x.g, Nx);
        s2_Mx_res(f->x_pred.g, d + 21, Mx);
        mm<2, 3, 2>(Nx, Mx, NM);
        sL[21 * 23 + 21] = NM[0]; sL[21 * 23 + 22] = NM[1];
        sL[22 * 23 + 21] = NM[2]; sL[22 * 23 + 22] = NM[3];
    }
    __syncthreads();
    blk_mm23(sL, sI, sT);
    blk_mm23_nt(sT, sL, sI);
    for (int e = t; e < 529; e += blockDim.x) f->P[e] = sI[e];
}

// ---------------------------------------------------------------- launchers
void launch_imu_init(DFilter* f, const vmp_imu* imus, int n, const vmp_config& cfg, double t_end, cudaStream_t st) {
    DState ext{};
    for (int i = 0; i < 9; ++i) ext.rot_ext[i] = cfg.r_il[i];
    for (int i = 0; i < 3; ++i) ext.pos_ext[i] = cfg.p_il[i];
    VMP_NOTE_LAUNCH(); k_imu_init<<<1, 32, 0, st>>>(f, imus, n, cfg.gravity_align, ext, t_end);
}
void launch_predict_chain(DFilter* f, DScan& s, int n_imu, double t_start, double t_end, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_predict_chain<<<1, 256, 0, st>>>(f, s.imus, n_imu, t_start, t_end, s.poses);
}
void launch_undistort(DFilter* f, DScan& s, int n_max, cudaStream_t st) {
    int blocks = (n_max + 255) / 256;
    if (blocks > 1216) blocks = 1216;
    if (blocks < 1) blocks = 1;
    VMP_NOTE_LAUNCH(); k_undistort<<<blocks, 256, 0, st>>>(f, s.poses, s.cloud, s.d_n_raw);
}
void launch_ieskf_predict_once(DFilter* f, const double* acc, const double* gyro, double dt, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_predict_once<<<1, 256, 0, st>>>(f, acc[0], acc[1], acc[2], gyro[0], gyro[1], gyro[2], dt);
}
void launch_update_begin(DFilter* f, cudaStream_t st) { VMP_NOTE_LAUNCH(); k_update_begin<<<1, 256, 0, st>>>(f); }
void launch_residual_iter(DFilter* f, DScan& s, const DMap& m, int n_max, int estimate_ext, double eps,
                          cudaStream_t st, int do_step) {
    (void)n_max;
    VMP_NOTE_LAUNCH();
    if (estimate_ext)
        k_residual<12><<<s.res_blocks, kResThreads, 0, st>>>(f, s, m, eps, do_step);
    else
        k_residual<6><<<s.res_blocks, kResThreads, 0, st>>>(f, s, m, eps, do_step);
}
void launch_update_end(DFilter* f, cudaStream_t st) { VMP_NOTE_LAUNCH(); k_update_end<<<1, 256, 0, st>>>(f); }

}  // namespace vmp
