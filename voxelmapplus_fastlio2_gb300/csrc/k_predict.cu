// IMU predict chain of LIOBuilder::undistortCloud (lio_builder.cpp:65-123):
// one IESKF::predict (ieskf.cpp:101-123) per IMU pair plus the final predict
// to the scan end, with the pose cache the point compensation uses.
//
// The reference's arithmetic is kept bit for bit, but the chain is laid out
// for a GPU whose FP64 instructions cost the same for 1 or 32 lanes:
//   * during prediction bg, ba, g, rot_ext and pos_ext do not change (their
//     delta entries are zero and Exp(0) is the identity), so every step's
//     rotation increment Exp(w), right Jacobian and the F / G blocks that do
//     not involve the rotation are computed in parallel, one lane per step;
//     F's rotation block Exp(-w) equals Exp(w)^T exactly;
//   * only the rotation chain (lanes over the 9 entries) and the velocity /
//     position prefix sums (lanes over xyz) are sequential;
//   * the covariance chain P = F P F^T + G Q G^T computes only the 11 rows /
//     columns of F that are not identity rows, summing each entry's
//     structural non-zero terms in k order -- the same value as the dense
//     product -- one warp per row with the lanes over the other index;
//     the G Q G^T blocks (Q diagonal) are precomputed per step.
// Two kernels: k_predict_chain2 (the state chain, the per-step F / G data and
// the pose cache the undistortion needs) and k_predict_cov (the covariance
// chain over that per-step data).  Nothing reads P before the first residual
// kernel (its gate), so the second runs beside the undistortion,
// downsampling and body covariances.
#include "kernels.cuh"

namespace vmp {

constexpr int kPredThreads = 352;  // 11 warps: one per active F row / column of the covariance chain

// F row / column groups that are not identity: {0,1,2}, {3,4,5}, {12,13,14}, {21,22}.
__device__ inline bool f_row_active(int i) { return i < 6 || (i >= 12 && i < 15) || i >= 21; }

// Per-step F / G data staged in shared memory for the covariance chain.
struct StepSm {
    double dt;
    double E[9], nJr[9], FRa[9], nRdt[9], Mxdt[6], B[24];
};

__device__ inline void stage_step(StepSm& o, const DStep& d, int t) {
    // 67 doubles, one per thread
    if (t == 0) o.dt = d.dt;
    else if (t < 10) o.E[t - 1] = d.E[t - 1];
    else if (t < 19) o.nJr[t - 10] = d.nJr[t - 10];
    else if (t < 28) o.FRa[t - 19] = d.FRa[t - 19];
    else if (t < 37) o.nRdt[t - 28] = d.nRdt[t - 28];
    else if (t < 43) o.Mxdt[t - 37] = d.Mxdt[t - 37];
    else if (t < 67) o.B[t - 43] = d.B[t - 43];
}

// FP(i, j) = sum_k F(i, k) P(k, j) over F row i's structural non-zeros, k ascending.
__device__ inline double fp_entry_s(const StepSm& d, const double* NM, const double* P, int i, int j) {
    if (i < 3) return P[i * 23 + j] + d.dt * P[(12 + i) * 23 + j];
    if (i < 6) {
        const int a = i - 3;
        double s = d.E[0 * 3 + a] * P[3 * 23 + j];
        s = s + d.E[1 * 3 + a] * P[4 * 23 + j];
        s = s + d.E[2 * 3 + a] * P[5 * 23 + j];
        s = s + d.nJr[a * 3 + 0] * P[15 * 23 + j];
        s = s + d.nJr[a * 3 + 1] * P[16 * 23 + j];
        s = s + d.nJr[a * 3 + 2] * P[17 * 23 + j];
        return s;
    }
    if (i >= 12 && i < 15) {
        const int a = i - 12;
        double s = d.FRa[a * 3 + 0] * P[3 * 23 + j];
        s = s + d.FRa[a * 3 + 1] * P[4 * 23 + j];
        s = s + d.FRa[a * 3 + 2] * P[5 * 23 + j];
        s = s + P[i * 23 + j];
        s = s + d.nRdt[a * 3 + 0] * P[18 * 23 + j];
        s = s + d.nRdt[a * 3 + 1] * P[19 * 23 + j];
        s = s + d.nRdt[a * 3 + 2] * P[20 * 23 + j];
        s = s + d.Mxdt[a * 2 + 0] * P[21 * 23 + j];
        s = s + d.Mxdt[a * 2 + 1] * P[22 * 23 + j];
        return s;
    }
    const int a = i - 21;
    return NM[a * 2 + 0] * P[21 * 23 + j] + NM[a * 2 + 1] * P[22 * 23 + j];
}

// A(i, j) = sum_k FPf(i, k) F(j, k) over F row j's structural non-zeros;
// FPf(i, .) is FP's row i for the active rows and P's row i otherwise.
__device__ inline double fpft_entry_s(const StepSm& d, const double* NM, const double* FPf, int i, int j) {
    const double* r = FPf + i * 23;
    if (j < 3) return r[j] + r[12 + j] * d.dt;
    if (j < 6) {
        const int a = j - 3;
        double s = r[3] * d.E[0 * 3 + a];
        s = s + r[4] * d.E[1 * 3 + a];
        s = s + r[5] * d.E[2 * 3 + a];
        s = s + r[15] * d.nJr[a * 3 + 0];
        s = s + r[16] * d.nJr[a * 3 + 1];
        s = s + r[17] * d.nJr[a * 3 + 2];
        return s;
    }
    if (j >= 12 && j < 15) {
        const int a = j - 12;
        double s = r[3] * d.FRa[a * 3 + 0];
        s = s + r[4] * d.FRa[a * 3 + 1];
        s = s + r[5] * d.FRa[a * 3 + 2];
        s = s + r[j];
        s = s + r[18] * d.nRdt[a * 3 + 0];
        s = s + r[19] * d.nRdt[a * 3 + 1];
        s = s + r[20] * d.nRdt[a * 3 + 2];
        s = s + r[21] * d.Mxdt[a * 2 + 0];
        s = s + r[22] * d.Mxdt[a * 2 + 1];
        return s;
    }
    const int a = j - 21;
    return r[21] * NM[a * 2 + 0] + r[22] * NM[a * 2 + 1];
}

// Row (half 1) / column (half 2) of each warp: the 11 active indices, one per
// warp, so that a step's dependent chain is one entry's sum.
__constant__ int kGroupStart[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
__constant__ int kGroupIdx[11] = {12, 3, 13, 4, 14, 5, 0, 1, 2, 21, 22};

// B = G Q G^T entry (i, j) for the step, 0 where structurally zero.
__device__ inline bool b_entry(const StepSm& d, int i, int j, double& b) {
    if (i >= 3 && i < 6 && j >= 3 && j < 6) { b = d.B[(i - 3) * 3 + (j - 3)]; return true; }
    if (i >= 12 && i < 15 && j >= 12 && j < 15) { b = d.B[9 + (i - 12) * 3 + (j - 12)]; return true; }
    if (i == j && i >= 15 && i < 21) { b = d.B[18 + (i - 15)]; return true; }
    return false;
}

__device__ inline int inactive_index(int q) { return q < 6 ? 6 + q : 15 + (q - 6); }  // rows/cols 6..11, 15..20

__global__ void __launch_bounds__(kPredThreads) k_predict_chain2(DFilter* f, const vmp_imu* imus,
                                                                 const DScanHdr* __restrict__ hdr, DPose* poses,
                                                                 DStep* st) {
    const int n_imu = hdr->n_imu;
    const double t_begin = hdr->t_start, t_end = hdr->t_end;
    __shared__ double sMx[6], sQd[12];
    __shared__ double sBg[3], sBa[3], sG[3], sRot0[9], sVel0[3], sPos0[3], sRotF[9], sVelF[3], sPosF[3];
    __shared__ int sPosOf[1024];
    __shared__ int sS;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (n_imu > 1024) return;  // bounded by max_imu_per_scan (<= 1000) on the host
    const double last_end = f->last_cloud_end_time;
    const double gn = f->gravity_norm;
    if (t < 12) sQd[t] = f->Q[t * 13];
    if (t < 3) {
        sBg[t] = f->x.bg[t]; sBa[t] = f->x.ba[t]; sG[t] = f->x.g[t];
        sVel0[t] = f->x.vel[t]; sPos0[t] = f->x.pos[t];
    }
    if (t < 9) sRot0[t] = f->x.rot[t];
    __syncthreads();
    if (t == 64) s2_Mx(sG, sMx);  // beside warp 0's compaction below
    // ---- phase 0: active IMU pairs (tail at or after the last scan end), compacted in order
    if (warp == 0) {
        int running = 0;
        for (int base = 0; base < n_imu; base += 32) {
            const int k = base + lane;
            const bool act = k < n_imu && !(imus[k].t < last_end);
            const unsigned m = __ballot_sync(0xffffffffu, act);
            if (k < n_imu) sPosOf[k] = act ? running + __popc(m & ((1u << lane) - 1u)) : -1;
            running += __popc(m);
        }
        if (lane == 0) sS = running;
    }
    __syncthreads();
    const int S = sS, NS = S + 1;
    for (int k = t; k < n_imu; k += blockDim.x) {
        const int s = sPosOf[k];
        if (s < 0) continue;
        double ht, ha[3], hg[3];
        if (k == 0) {
            ht = f->last_imu_t;
            for (int a = 0; a < 3; ++a) { ha[a] = f->last_imu_acc[a]; hg[a] = f->last_imu_gyro[a]; }
        } else {
            ht = imus[k - 1].t;
            for (int a = 0; a < 3; ++a) { ha[a] = imus[k - 1].acc[a]; hg[a] = imus[k - 1].gyro[a]; }
        }
        const vmp_imu& tl = imus[k];
        DStep& d = st[s];
        for (int a = 0; a < 3; ++a) {
            d.gyro[a] = 0.5 * (hg[a] + tl.gyro[a]);
            const double av = 0.5 * (ha[a] + tl.acc[a]);
            d.acc[a] = av * 9.81 / gn;
        }
        d.dt = (ht < last_end) ? tl.t - last_end : tl.t - ht;
        d.offset = tl.t - t_begin;
        d.pose = 1;
    }
    __syncthreads();
    if (t == 0) {  // final predict to the scan end with the last input
        DStep& d = st[S];
        for (int a = 0; a < 3; ++a) {
            d.acc[a] = S > 0 ? st[S - 1].acc[a] : 0.0;
            d.gyro[a] = S > 0 ? st[S - 1].gyro[a] : 0.0;
        }
        const double imu_end = n_imu > 0 ? imus[n_imu - 1].t : f->last_imu_t;
        d.dt = t_end - imu_end;
        d.offset = 0.0;
        d.pose = 0;
    }
    __syncthreads();
    // ---- phase 1: per-step terms that do not involve the rotation, one lane
    // per step: Exp(w) on warps 0.., the right Jacobian and its products on
    // the warps after them (the two are independent)
    // threads per role: whole warps, at most half the block
    const int role = min(((NS + 31) / 32) * 32, (int)(blockDim.x / 64) * 32);
    {
        if (t < role) {
            for (int s = t; s < NS; s += role) {
                DStep& d = st[s];
                double w[3];
                for (int a = 0; a < 3; ++a) w[a] = (d.gyro[a] - sBg[a]) * d.dt;
                so3_exp(w, d.E);
                for (int a = 0; a < 3; ++a) d.ab[a] = d.acc[a] - sBa[a];
                for (int q = 0; q < 6; ++q) d.Mxdt[q] = sMx[q] * d.dt;
            }
        } else if (t < 2 * role) {
            for (int s = t - role; s < NS; s += role) {
                DStep& d = st[s];
                double w[3], Jr[9], GQ[9];
                for (int a = 0; a < 3; ++a) w[a] = (d.gyro[a] - sBg[a]) * d.dt;
                so3_right_jac(w, Jr);
                for (int q = 0; q < 9; ++q) d.nJr[q] = (-Jr[q]) * d.dt;
                for (int a = 0; a < 3; ++a)
                    for (int c = 0; c < 3; ++c) GQ[a * 3 + c] = d.nJr[a * 3 + c] * sQd[c];
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        d.B[a * 3 + b] = (GQ[a * 3] * d.nJr[b * 3] + GQ[a * 3 + 1] * d.nJr[b * 3 + 1]) + GQ[a * 3 + 2] * d.nJr[b * 3 + 2];
                for (int a = 0; a < 3; ++a) {
                    d.B[18 + a] = (d.dt * sQd[6 + a]) * d.dt;
                    d.B[21 + a] = (d.dt * sQd[9 + a]) * d.dt;
                }
            }
        }
    }
    __syncthreads();
    // ---- phase 2: rotation chain rot_{s+1} = rot_s Exp(w_s) (lanes over the 9 entries)
    if (warp == 0) {
        const int ri = (lane < 9 ? lane : 0) / 3, ci = (lane < 9 ? lane : 0) % 3;
        double r = lane < 9 ? sRot0[lane] : 0.0;
        double e0 = st[0].E[ci], e1 = st[0].E[3 + ci], e2 = st[0].E[6 + ci];
        for (int s = 0; s < NS; ++s) {
            double n0 = 0, n1 = 0, n2 = 0;
            if (s + 1 < NS) { n0 = st[s + 1].E[ci]; n1 = st[s + 1].E[3 + ci]; n2 = st[s + 1].E[6 + ci]; }
            if (lane < 9) st[s].rot[lane] = r;
            const double r0 = __shfl_sync(0xffffffffu, r, ri * 3 + 0);
            const double r1 = __shfl_sync(0xffffffffu, r, ri * 3 + 1);
            const double r2 = __shfl_sync(0xffffffffu, r, ri * 3 + 2);
            r = (r0 * e0 + r1 * e1) + r2 * e2;
            e0 = n0; e1 = n1; e2 = n2;
        }
        if (lane < 9) sRotF[lane] = r;
    }
    __syncthreads();
    // ---- phase 3: terms that involve the step's rotation, one lane per step.
    // The warps of the second role form the F / G blocks the covariance chain
    // needs (only k_predict_cov reads them); those of the first form the
    // velocity increments and go on, behind a barrier of their own, to the
    // velocity / position prefix and the pose cache the undistortion needs.
    if (t >= role && t < 2 * role) {
        for (int s = t - role; s < NS; s += role) {
            DStep& d = st[s];
            double nr[9], H[9], T[9], GQ[9];
            for (int q = 0; q < 9; ++q) nr[q] = -d.rot[q];
            hat3(d.ab, H);
            mm<3, 3, 3>(nr, H, T);
            for (int q = 0; q < 9; ++q) { d.FRa[q] = T[q] * d.dt; d.nRdt[q] = nr[q] * d.dt; }
            for (int a = 0; a < 3; ++a)
                for (int c = 0; c < 3; ++c) GQ[a * 3 + c] = d.nRdt[a * 3 + c] * sQd[3 + c];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    d.B[9 + a * 3 + b] =
                        (GQ[a * 3] * d.nRdt[b * 3] + GQ[a * 3 + 1] * d.nRdt[b * 3 + 1]) + GQ[a * 3 + 2] * d.nRdt[b * 3 + 2];
        }
    } else if (t < role) {
        for (int s = t; s < NS; s += role) {
            DStep& d = st[s];
            double ra[3];
            m3v(d.rot, d.ab, ra);
            for (int a = 0; a < 3; ++a) d.vinc[a] = (ra[a] + sG[a]) * d.dt;
        }
        asm volatile("bar.sync 1, %0;" ::"r"(role) : "memory");
        if (t < 3) {  // velocity / position prefix (pos uses the velocity before the step)
            double v = sVel0[t], p = sPos0[t];
            for (int s = 0; s < NS; ++s) {
                DStep& d = st[s];
                p = p + v * d.dt;
                v = v + d.vinc[t];
                d.velA[t] = v;
                d.posA[t] = p;
            }
            sVelF[t] = v;
            sPosF[t] = p;
        }
        asm volatile("bar.sync 1, %0;" ::"r"(role) : "memory");
        // pose cache (imu_poses_cache): pose 0 = state before the chain, pose s+1 after step s
        for (int s = t; s < S; s += role) {
            const DStep& d = st[s];
            const double* rotA = st[s + 1].rot;
            DPose& p = poses[s + 1];
            double ra[3];
            m3v(rotA, d.ab, ra);
            p.offset = d.offset;
            for (int a = 0; a < 3; ++a) {
                p.acc[a] = ra[a] + sG[a];
                p.gyro[a] = d.gyro[a] - sBg[a];
                p.vel[a] = d.velA[a];
                p.pos[a] = d.posA[a];
            }
            for (int q = 0; q < 9; ++q) p.rot[q] = rotA[q];
        }
        if (t == 0) {
            DPose& p0 = poses[0];
            p0.offset = 0.0;
            for (int a = 0; a < 3; ++a) {
                p0.acc[a] = f->last_acc[a]; p0.gyro[a] = f->last_gyro[a];
                p0.vel[a] = sVel0[a]; p0.pos[a] = sPos0[a];
            }
            for (int q = 0; q < 9; ++q) p0.rot[q] = sRot0[q];
        }
    }
    // ---- write back (the covariance chain is k_predict_cov)
    __syncthreads();
    if (t == 0) {
        DState& x = f->x;
        for (int q = 0; q < 9; ++q) x.rot[q] = sRotF[q];
        for (int a = 0; a < 3; ++a) { x.vel[a] = sVelF[a]; x.pos[a] = sPosF[a]; }
        f->npose = S + 1;
        if (S > 0) {
            for (int a = 0; a < 3; ++a) {
                f->last_acc[a] = poses[S].acc[a];
                f->last_gyro[a] = poses[S].gyro[a];
                f->inp_acc[a] = st[S - 1].acc[a];
                f->inp_gyro[a] = st[S - 1].gyro[a];
            }
        }
        const vmp_imu& last = imus[n_imu - 1];
        f->last_imu_t = last.t;
        for (int a = 0; a < 3; ++a) { f->last_imu_acc[a] = last.acc[a]; f->last_imu_gyro[a] = last.gyro[a]; }
        f->last_cloud_end_time = t_end;
    }
}

// The covariance chain P = F P F^T + G Q G^T over the steps k_predict_chain2
// wrote (f->npose of them), with the F / G data of each step staged in shared
// memory while the previous step runs.
__global__ void __launch_bounds__(kPredThreads) k_predict_cov(DFilter* f, const DStep* __restrict__ st) {
    __shared__ double sP[2][529];
    __shared__ double sFP[529];
    __shared__ StepSm sStep[2];
    __shared__ double sNM[4];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int NS = f->npose;
    for (int e = t; e < 529; e += blockDim.x) sP[0][e] = f->P[e];
    if (t == 0) {  // the S2 block of F: N(g) M(g) (g does not change while predicting)
        double Nx[6], Mx[6];
        s2_Mx(f->x.g, Mx);
        s2_Nx(f->x.g, Nx);
        mm<2, 3, 2>(Nx, Mx, sNM);
    }
    if (t < 67) stage_step(sStep[0], st[0], t);
    __syncthreads();
    int cur = 0;
    for (int s = 0; s < NS; ++s) {
        const StepSm& d = sStep[s & 1];
        const double* P = sP[cur];
        for (int g = kGroupStart[warp]; g < kGroupStart[warp + 1]; ++g) {
            const int i = kGroupIdx[g];
            if (lane < 23) sFP[i * 23 + lane] = fp_entry_s(d, sNM, P, i, lane);
        }
        for (int e = t; e < 12 * 23; e += blockDim.x) {
            const int r = inactive_index(e / 23), j = e % 23;
            sFP[r * 23 + j] = P[r * 23 + j];
        }
        if (s + 1 < NS && t < 67) stage_step(sStep[(s + 1) & 1], st[s + 1], t);
        __syncthreads();
        double* Pn = sP[cur ^ 1];
        for (int g = kGroupStart[warp]; g < kGroupStart[warp + 1]; ++g) {
            const int j = kGroupIdx[g];
            if (lane < 23) {
                double a = fpft_entry_s(d, sNM, sFP, lane, j), b;
                if (b_entry(d, lane, j, b)) a = a + b;
                Pn[lane * 23 + j] = a;
            }
        }
        for (int e = t; e < 23 * 12; e += blockDim.x) {
            const int i = e / 12, j = inactive_index(e % 12);
            double a = sFP[i * 23 + j], b;
            if (b_entry(d, i, j, b)) a = a + b;
            Pn[i * 23 + j] = a;
        }
        __syncthreads();
        cur ^= 1;
    }
    for (int e = t; e < 529; e += blockDim.x) f->P[e] = sP[cur][e];
}

void launch_predict_state(DFilter* f, DScan& s, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_predict_chain2<<<1, kPredThreads, 0, st>>>(f, s.imus, s.hdr, s.poses, s.steps);
}
void launch_predict_cov(DFilter* f, DScan& s, cudaStream_t st) {
    VMP_NOTE_LAUNCH(); k_predict_cov<<<1, kPredThreads, 0, st>>>(f, s.steps);
}
void launch_predict_chain2(DFilter* f, DScan& s, cudaStream_t st) {
    launch_predict_state(f, s, st);
    launch_predict_cov(f, s, st);
}

}  // namespace vmp
