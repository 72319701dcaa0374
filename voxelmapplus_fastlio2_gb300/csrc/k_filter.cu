// Small-state FP64 kernels of the iterated error-state Kalman filter and the
// per-point measurement model:
//   k_imu_init        LIOBuilder::initializeImu        lio_builder.cpp:28-63
//   k_predict_once    one IESKF::predict               ieskf.cpp:101-123
//   k_undistort       undistortCloud's point loop      lio_builder.cpp:125-152
// The IMU loop of undistortCloud is k_predict.cu; IESKF::update with the
// residual kernel is k_iekf.cu.
#include "kernels.cuh"

namespace vmp {

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

// Register budget: 3 CTAs per SM (80 registers, a few spilled words instead
// of 126).  Alone it runs as fast; beside other streams' kernels it leaves
// register file to them (served scans/s +0.7 %).
__global__ void __launch_bounds__(256, 3) k_undistort(const DFilter* __restrict__ f, const DPose* __restrict__ poses,
                                                      float4* cloud, const int* d_n) {
    __shared__ double s_off[1024];
    __shared__ DState cur;
    const int n = *d_n;
    if (blockIdx.x > 0 && (long long)blockIdx.x * blockDim.x >= n) return;  // past the points: no setup either
    const int npose = f->npose;
    if (npose > 1024) return;  // bounded by max_imu (checked on the host)
    for (int i = threadIdx.x; i < npose; i += blockDim.x) s_off[i] = poses[i].offset;
    if (threadIdx.x == 0) cur = f->x;
    __syncthreads();
    if (npose < 2) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = cloud[i];
        const double tau = div_by_recip((double)q.w, 1000.0, 1.0 / 1000.0);  // q.w / 1000, correctly rounded
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

// ---------------------------------------------------------------- launchers
void launch_imu_init(DFilter* f, const vmp_imu* imus, int n, const vmp_config& cfg, double t_end, cudaStream_t st) {
    DState ext{};
    for (int i = 0; i < 9; ++i) ext.rot_ext[i] = cfg.r_il[i];
    for (int i = 0; i < 3; ++i) ext.pos_ext[i] = cfg.p_il[i];
    VMP_NOTE_LAUNCH(); k_imu_init<<<1, 32, 0, st>>>(f, imus, n, cfg.gravity_align, ext, t_end);
}
void launch_undistort(DFilter* f, DScan& s, int n_max, cudaStream_t st) {
    int blocks = (n_max + 255) / 256;
    if (blocks > 1216) blocks = 1216;
    if (blocks < 1) blocks = 1;
    blocks = served_grid(blocks);
    VMP_NOTE_LAUNCH(); k_undistort<<<blocks, 256, 0, st>>>(f, s.poses, s.cloud, s.d_n_raw);
}
void launch_ieskf_predict_once(DFilter* f, const double* acc, const double* gyro, double dt, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_predict_once<<<1, 256, 0, st>>>(f, acc[0], acc[1], acc[2], gyro[0], gyro[1], gyro[2], dt);
}
}  // namespace vmp
