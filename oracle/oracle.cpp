// ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into libvmp.so.
//
// A CPU restatement, in plain C++ on FP64, of the reference odometry hot path
// of liangheming/VoxelMapPlus_FASTLIO2 (package voxel_plus).  It is the
// checker for the GPU path: only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg may load it.
//
// PARITY UNPINNED: the reference ships no tests, fixtures or golden vectors
// for this path, and it cannot be compiled on this machine (Eigen3, Sophus,
// PCL and ROS are absent).  This restatement follows the reference source
// line by line (citations below) and restates the third-party arithmetic it
// relies on in mathkit.hpp.
//
// Every reference quirk is kept:
//   * VoxelGrid::updatePlane accumulates plane->cov across refits without a
//     reset (voxel_map.cpp:115-130);
//   * VoxelGrid::merge uses the reference's operator precedence and does not
//     normalise the merged normal (voxel_map.cpp:166-168);
//   * ResidualData::plane_cov is never assigned, so it stays zero
//     (voxel_map.cpp:258-276, lio_builder.cpp:25);
//   * sharedUpdateFunc never resets is_valid on a hash miss: the record at
//     index i keeps the previous iteration's / scan's values
//     (lio_builder.cpp:260-274);
//   * IESKF::update stops on the signed delta.maxCoeff() (ieskf.cpp:148) and
//     runs at most max_iter_ = 5 iterations (ieskf.h:101);
//   * calcBodyCov mutates its input when z == 0 (commons.cpp:20-23);
//   * the scan's world transform runs in float (lio_builder.cpp:155-163).
// Deviations (all documented as unpinned third-party behaviour):
//   * residual_info grows to the scan size instead of overflowing at 10000
//     (lio_builder.cpp:25);
//   * std::sort of points by time and PCL VoxelGrid's std::sort by leaf
//     index are restated as stable sorts (equal-key order is unspecified in
//     the reference);
//   * VoxelGrid::count (a process-wide static) is per map.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <list>
#include <tuple>
#include <map>
#include <memory>
#include <unordered_map>
#include <vector>
#include <algorithm>
#include <limits>
#include <functional>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mathkit.hpp"
#include "../include/vmp.h"

namespace orc {

constexpr double GRAVITY = 9.81;  // ieskf.h:6
typedef Mat<23, 23> M23;
typedef Mat<23, 1> V23;
typedef Mat<24, 1> V24;
typedef Mat<12, 12> M12;
typedef Mat<12, 1> V12;
typedef Mat<3, 2> M32;
typedef Mat<2, 3> M2x3;
typedef Mat<2, 2> M22;
typedef Mat<6, 6> M66;

template <int N>
inline V3 seg3(const Mat<N, 1>& d, int i) { return v3(d[i], d[i + 1], d[i + 2]); }
template <int N>
inline void setSeg3(Mat<N, 1>& d, int i, const V3& s) { d[i] = s[0]; d[i + 1] = s[1]; d[i + 2] = s[2]; }

// ---------------------------------------------------------------- kf::State
struct State {  // ieskf.h:31-62
    V3 pos = V3::Zero();
    M3 rot = M3::Identity();
    M3 rot_ext = M3::Identity();
    V3 pos_ext = V3::Zero();
    V3 vel = V3::Zero();
    V3 bg = V3::Zero();
    V3 ba = V3::Zero();
    V3 g = v3(0.0, 0.0, -GRAVITY);

    void initG(const V3& dir) { g = normalized(dir) * GRAVITY; }

    M32 getBx() const {  // ieskf.cpp:69-77
        M32 r;
        r(0, 0) = -g[1]; r(0, 1) = -g[2];
        r(1, 0) = GRAVITY - g[1] * g[1] / (GRAVITY + g[0]); r(1, 1) = -g[2] * g[1] / (GRAVITY + g[0]);
        r(2, 0) = -g[2] * g[1] / (GRAVITY + g[0]); r(2, 1) = GRAVITY - g[2] * g[2] / (GRAVITY + g[0]);
        r /= GRAVITY;
        return r;
    }
    M32 getMx() const { return -hat(g) * getBx(); }  // ieskf.cpp:79-83
    M32 getMx(const V2& res) const {                 // ieskf.cpp:85-90
        M32 bx = getBx();
        V3 bu = bx * res;
        return ((-Exp(bu)) * hat(g)) * T(leftJacobian(bu)) * bx;
    }
    M2x3 getNx() const { return (1.0 / GRAVITY / GRAVITY * T(getBx())) * hat(g); }  // ieskf.cpp:92-95

    void plus23(const V23& d) {  // ieskf.cpp:11-21
        pos += seg3(d, 0);
        rot = rot * Exp(seg3(d, 3));
        rot_ext = rot_ext * Exp(seg3(d, 6));
        pos_ext += seg3(d, 9);
        vel += seg3(d, 12);
        bg += seg3(d, 15);
        ba += seg3(d, 18);
        V2 dg; dg[0] = d[21]; dg[1] = d[22];
        g = Exp(getBx() * dg) * g;
    }
    void plus24(const V24& d) {  // ieskf.cpp:23-33
        pos += seg3(d, 0);
        rot = rot * Exp(seg3(d, 3));
        rot_ext = rot_ext * Exp(seg3(d, 6));
        pos_ext += seg3(d, 9);
        vel += seg3(d, 12);
        bg += seg3(d, 15);
        ba += seg3(d, 18);
        g = Exp(seg3(d, 21)) * g;
    }
    V23 minus(const State& o) const {  // ieskf.cpp:35-67
        V23 d = V23::Zero();
        setSeg3(d, 0, pos - o.pos);
        setSeg3(d, 3, Log(T(o.rot) * rot));
        setSeg3(d, 6, Log(T(o.rot_ext) * rot_ext));
        setSeg3(d, 9, pos_ext - o.pos_ext);
        setSeg3(d, 12, vel - o.vel);
        setSeg3(d, 15, bg - o.bg);
        setSeg3(d, 18, ba - o.ba);
        double v_sin = norm(hat(g) * o.g);
        double v_cos = dot(g, o.g);
        double theta = std::atan2(v_sin, v_cos);
        V2 res;
        if (v_sin < 1e-11) {
            if (std::fabs(theta) > 1e-11) { res[0] = 3.1415926; res[1] = 0; }
            else { res[0] = 0; res[1] = 0; }
        } else {
            res = (theta / v_sin * T(o.getBx())) * hat(o.g) * g;
        }
        d[21] = res[0]; d[22] = res[1];
        return d;
    }
};

struct SharedState { M12 H; V12 b; size_t iter_num = 0; };

// ---------------------------------------------------------------- kf::IESKF
struct IESKF {
    size_t max_iter_ = 5;  // ieskf.h:101
    double eps_ = 0.001;   // ieskf.h:102
    State x_;
    M23 P_ = M23::Zero();
    M23 H_, F_;
    V23 b_;
    Mat<23, 12> G_;
    std::function<void(State&, SharedState&)> func_;
    int last_iters = 0;

    void predict(const V3& acc, const V3& gyro, double dt, const M12& Q) {  // ieskf.cpp:101-123
        V24 delta = V24::Zero();
        setSeg3(delta, 0, x_.vel * dt);
        setSeg3(delta, 3, (gyro - x_.bg) * dt);
        setSeg3(delta, 12, (x_.rot * (acc - x_.ba) + x_.g) * dt);
        F_.setIdentity();
        F_.setBlock(0, 12, M3::Identity() * dt);
        F_.setBlock(3, 3, Exp(-(gyro - x_.bg) * dt));
        F_.setBlock(3, 15, -rightJacobian((gyro - x_.bg) * dt) * dt);
        F_.setBlock(12, 3, ((-x_.rot) * hat(acc - x_.ba)) * dt);
        F_.setBlock(12, 18, (-x_.rot) * dt);
        F_.setBlock(12, 21, x_.getMx() * dt);
        F_.setBlock(21, 21, x_.getNx() * x_.getMx());
        G_.setZero();
        G_.setBlock(3, 0, -rightJacobian((gyro - x_.bg) * dt) * dt);
        G_.setBlock(12, 3, (-x_.rot) * dt);
        G_.setBlock(15, 6, M3::Identity() * dt);
        G_.setBlock(18, 9, M3::Identity() * dt);
        x_.plus24(delta);
        P_ = F_ * P_ * T(F_) + G_ * Q * T(G_);
    }

    void update() {  // ieskf.cpp:125-156
        State predict_x = x_;
        SharedState shared;
        shared.iter_num = 0;
        V23 delta = V23::Zero();
        last_iters = 0;
        for (size_t i = 0; i < max_iter_; i++) {
            func_(x_, shared);
            H_.setZero();
            b_.setZero();
            delta = x_.minus(predict_x);
            M23 J = M23::Identity();
            J.setBlock(3, 3, rightJacobian(seg3(delta, 3)));
            J.setBlock(6, 6, rightJacobian(seg3(delta, 6)));
            V2 dg; dg[0] = delta[21]; dg[1] = delta[22];
            J.setBlock(21, 21, x_.getNx() * predict_x.getMx(dg));
            M23 Pinv = inverse(P_);
            b_ += (T(J) * Pinv * delta);
            H_ += (T(J) * Pinv * J);
            for (int r = 0; r < 12; ++r) {
                for (int c = 0; c < 12; ++c) H_(r, c) += shared.H(r, c);
                b_[r] += shared.b[r];
            }
            delta = -(inverse(H_) * b_);
            x_.plus23(delta);
            shared.iter_num += 1;
            last_iters = (int)shared.iter_num;
            if (delta.maxCoeff() < eps_) break;
        }
        M23 L = M23::Identity();
        L.setBlock(3, 3, rightJacobian(seg3(delta, 3)));
        L.setBlock(6, 6, rightJacobian(seg3(delta, 6)));
        V2 dg; dg[0] = delta[21]; dg[1] = delta[22];
        L.setBlock(21, 21, x_.getNx() * predict_x.getMx(dg));
        P_ = L * inverse(H_) * T(L);
    }
};

// ---------------------------------------------------------------- commons
// pcl_macros.h DEG2RAD(x) ((x)*0.017453293)
inline double deg2rad_pcl(double x) { return x * 0.017453293; }

// lio::calcBodyCov (commons.cpp:18-45); mutates pb when z == 0.
inline void calcBodyCov(V3& pb, double range_inc, double degree_inc, M3& cov) {
    if (pb[2] == 0) pb[2] = 0.001;
    double range = std::sqrt(pb[0] * pb[0] + pb[1] * pb[1] + pb[2] * pb[2]);
    double range_var = range_inc * range_inc;
    double s = std::sin(deg2rad_pcl(degree_inc));
    M22 dvar; dvar(0, 0) = s * s; dvar(0, 1) = 0; dvar(1, 0) = 0; dvar(1, 1) = s * s;
    V3 d = normalized(pb);
    M3 dh;
    dh(0, 0) = 0; dh(0, 1) = -d[2]; dh(0, 2) = d[1];
    dh(1, 0) = d[2]; dh(1, 1) = 0; dh(1, 2) = -d[0];
    dh(2, 0) = -d[1]; dh(2, 1) = d[0]; dh(2, 2) = 0;
    V3 b1 = normalized(v3(1, 1, -(d[0] + d[1]) / d[2]));
    V3 b2 = normalized(cross(b1, d));
    M32 N;
    N(0, 0) = b1[0]; N(0, 1) = b2[0];
    N(1, 0) = b1[1]; N(1, 1) = b2[1];
    N(2, 0) = b1[2]; N(2, 1) = b2[2];
    // A = range * direction_hat * N, cov = d range_var d^T + A dvar A^T
    // (commons.cpp:40-43) as written: (range [d]x) N and (A dvar) A^T, dense
    // left-to-right sums (the products with the zeros of [d]x and dvar
    // included)
    const M32 A = (range * dh) * N;
    cov = (d * range_var) * T(d) + (A * dvar) * T(A);
}

// ---------------------------------------------------------------- VoxelMap
struct VoxelKey {  // voxel_map.h:17-34
    int64_t x, y, z;
    bool operator==(const VoxelKey& o) const { return x == o.x && y == o.y && z == o.z; }
    struct Hasher {
        int64_t operator()(const VoxelKey& k) const {
            return ((((k.z) * 116101LL) % 10000000000LL + (k.y)) * 116101LL) % 10000000000LL + (k.x);
        }
    };
};

struct PointWithCov { V3 point; M3 cov; };

struct Plane {  // voxel_map.h:43-51 (make_shared value-initialises cov to 0)
    V3 mean = V3::Zero();
    M3 ppt = M3::Zero();
    V3 norm = V3::Zero();
    M66 cov = M66::Zero();
    int n = 0;
};

struct ResidualData {  // voxel_map.h:53-65, value-initialised
    V3 point_lidar = V3::Zero();
    V3 point_world = V3::Zero();
    V3 plane_mean = V3::Zero();
    V3 plane_norm = V3::Zero();
    M66 plane_cov = M66::Zero();
    M3 cov_lidar = M3::Zero();
    M3 cov_world = M3::Zero();
    bool is_valid = false;
    double residual = 0.0;
};

struct VoxelMap;

struct VoxelGrid {  // voxel_map.h:69-103, voxel_map.cpp:11-186
    int max_point_thresh, update_point_thresh;
    double plane_thresh;
    bool is_init = false, is_plane = false, update_enable = true;
    int newly_add_point = 0;
    bool merged = false;
    uint64_t group_id;
    std::vector<PointWithCov> temp_points;
    VoxelKey position;
    VoxelMap* map;
    Plane plane;
    V3 center = V3::Zero();
    std::list<VoxelKey>::iterator cache_it;

    VoxelGrid(int mpt, int upt, double pt, VoxelKey pos, VoxelMap* m, uint64_t gid)
        : max_point_thresh(mpt), update_point_thresh(upt), plane_thresh(pt), group_id(gid), position(pos), map(m) {
        temp_points.reserve(max_point_thresh);
    }
    void addToPlane(const PointWithCov& pv) {  // voxel_map.cpp:29-34
        plane.mean += (pv.point - plane.mean) / (plane.n + 1.0);
        plane.ppt += pv.point * T(pv.point);
        plane.n += 1;
    }
    void addPoint(const PointWithCov& pv) { addToPlane(pv); temp_points.push_back(pv); }
    void pushPoint(const PointWithCov& pv);
    void updatePlane();
    void merge();
};

struct VoxelMap {  // voxel_map.h:107-128
    int max_point_thresh, update_point_thresh;
    double plane_thresh, voxel_size;
    int capacity;
    double merge_thresh_for_angle = 0.1, merge_thresh_for_distance = 0.04;  // voxel_map.cpp:8-9
    uint64_t count = 0;  // VoxelGrid::count (voxel_map.cpp:6)
    std::unordered_map<VoxelKey, std::shared_ptr<VoxelGrid>, VoxelKey::Hasher> featmap;
    std::list<VoxelKey> cache;
    long long evicted = 0;

    VoxelKey index(const V3& p) const {  // voxel_map.cpp:194-198
        return VoxelKey{(int64_t)std::floor(p[0] / voxel_size), (int64_t)std::floor(p[1] / voxel_size),
                        (int64_t)std::floor(p[2] / voxel_size)};
    }
    std::shared_ptr<VoxelGrid> touch(const VoxelKey& k) {  // voxel_map.cpp:205-217 / 237-249
        auto it = featmap.find(k);
        if (it == featmap.end()) {
            auto g = std::make_shared<VoxelGrid>(max_point_thresh, update_point_thresh, plane_thresh, k, this, count++);
            featmap[k] = g;
            cache.push_front(k);
            g->cache_it = cache.begin();
            if ((long long)cache.size() > (long long)capacity) {
                featmap.erase(cache.back());
                cache.pop_back();
                evicted++;
            }
            return g;
        }
        cache.splice(cache.begin(), cache, it->second->cache_it);
        return it->second;
    }
    void build(std::vector<PointWithCov>& pvs) {  // voxel_map.cpp:200-230
        for (auto& pv : pvs) {
            VoxelKey k = index(pv.point);
            touch(k);
            featmap[k]->addPoint(pv);
        }
        for (auto& kv : featmap) kv.second->updatePlane();
    }
    void update(std::vector<PointWithCov>& pvs) {  // voxel_map.cpp:232-256
        for (auto& pv : pvs) {
            VoxelKey k = index(pv.point);
            touch(k);
            featmap[k]->pushPoint(pv);
        }
    }
    bool buildResidual(ResidualData& data, const std::shared_ptr<VoxelGrid>& vg) const {  // voxel_map.cpp:258-276
        data.is_valid = false;
        if (vg->is_plane) {
            V3 p2m = data.point_world - vg->plane.mean;
            data.plane_norm = vg->plane.norm;
            data.plane_mean = vg->plane.mean;
            data.residual = dot(data.plane_norm, p2m);
            Mat<1, 6> J_nq;
            J_nq(0, 0) = p2m[0]; J_nq(0, 1) = p2m[1]; J_nq(0, 2) = p2m[2];
            J_nq(0, 3) = -data.plane_norm[0]; J_nq(0, 4) = -data.plane_norm[1]; J_nq(0, 5) = -data.plane_norm[2];
            double sigma_l = (J_nq * data.plane_cov * T(J_nq))(0, 0);
            sigma_l += (T(data.plane_norm) * data.cov_world * data.plane_norm)(0, 0);
            if (std::fabs(data.residual) < 3.0 * std::sqrt(sigma_l)) data.is_valid = true;
        }
        return data.is_valid;
    }
};

void VoxelGrid::pushPoint(const PointWithCov& pv) {  // voxel_map.cpp:42-95
    if (!is_init) {
        addToPlane(pv);
        temp_points.push_back(pv);
        updatePlane();
    } else {
        if (is_plane) {
            if (update_enable) {
                addToPlane(pv);
                temp_points.push_back(pv);
                newly_add_point++;
                if (newly_add_point >= update_point_thresh) { updatePlane(); newly_add_point = 0; }
                if ((int)temp_points.size() >= max_point_thresh) {
                    update_enable = false;
                    std::vector<PointWithCov>().swap(temp_points);
                }
            } else {
                merge();
            }
        } else {
            if (update_enable) {
                addToPlane(pv);
                temp_points.push_back(pv);
                newly_add_point++;
                if (newly_add_point >= update_point_thresh) { updatePlane(); newly_add_point = 0; }
                if ((int)temp_points.size() >= max_point_thresh) {
                    update_enable = false;
                    std::vector<PointWithCov>().swap(temp_points);
                }
            }
        }
    }
}

void VoxelGrid::updatePlane() {  // voxel_map.cpp:97-136
    if (plane.n < update_point_thresh) return;
    is_init = true;
    M3 cov = plane.ppt / static_cast<double>(plane.n) - plane.mean * T(plane.mean);
    V3 evals; M3 evecs;
    eigSym3(cov, evals, evecs);
    if (evals[0] > plane_thresh) { is_plane = false; return; }
    is_plane = true;
    // J = [evecs * F; J_Q], J_Q = I / n, and plane.cov += J * pv.cov * J^T
    // (voxel_map.cpp:115-130) as written: F's row 0 stays zero, J_Q has its
    // zero off-diagonal, every product is the dense left-to-right sum
    // (J * pv.cov first, then (J * pv.cov) * J^T), and all 36 entries are
    // accumulated, the lower triangle with its own rounding.
    M3 J_Q = M3::Identity() / static_cast<double>(plane.n);
    V3 pn = v3(evecs(0, 0), evecs(1, 0), evecs(2, 0));
    for (PointWithCov& pv : temp_points) {
        M3 F = M3::Zero();
        for (int m = 1; m < 3; m++) {
            V3 vm = v3(evecs(0, m), evecs(1, m), evecs(2, m));
            Mat<1, 3> Fm = (T(pv.point - plane.mean) / ((plane.n) * (evals[0] - evals[m]))) * (vm * T(pn) + pn * T(vm));
            F(m, 0) = Fm(0, 0); F(m, 1) = Fm(0, 1); F(m, 2) = Fm(0, 2);
        }
        Mat<6, 3> J;
        J.setBlock(0, 0, evecs * F);
        J.setBlock(3, 0, J_Q);
        plane.cov += (J * pv.cov) * T(J);
    }
    double axis_distance = -dot(plane.mean, pn);
    if (axis_distance < 0.0) pn = -pn;
    plane.norm = pn;
    center = plane.mean;
}

void VoxelGrid::merge() {  // voxel_map.cpp:138-186
    VoxelKey near[6] = {{position.x - 1, position.y, position.z}, {position.x, position.y - 1, position.z},
                        {position.x, position.y, position.z - 1}, {position.x + 1, position.y, position.z},
                        {position.x, position.y + 1, position.z}, {position.x, position.y, position.z + 1}};
    for (VoxelKey& k : near) {
        auto it = map->featmap.find(k);
        if (it == map->featmap.end()) continue;
        VoxelGrid* nn = it->second.get();
        if (nn->group_id == group_id || nn->update_enable || !nn->is_plane) continue;
        double norm_distance = 1.0 - dot(nn->plane.norm, plane.norm);
        double axis_distance = std::fabs(dot(nn->plane.norm, nn->plane.mean) - dot(plane.norm, plane.mean));
        if (norm_distance > map->merge_thresh_for_angle || axis_distance > map->merge_thresh_for_distance) continue;
        double tn0 = plane.cov.block<3, 3>(0, 0).trace(), tm0 = plane.cov.block<3, 3>(3, 3).trace(),
               tn1 = nn->plane.cov.block<3, 3>(0, 0).trace(), tm1 = nn->plane.cov.block<3, 3>(3, 3).trace();
        double tc0 = tn0 + tm0, tc1 = tn1 + tm1;
        // Reference operator precedence: only the second term is divided.
        V3 new_mean = tm0 * nn->plane.mean + tm1 * plane.mean / (tm0 + tm1);
        V3 new_norm = tn0 * nn->plane.norm + tn1 * plane.norm / (tn0 + tn1);
        M66 new_cov = (tc0 * tc0 * nn->plane.cov + tc1 * tc1 * plane.cov) / ((tc0 + tc1) * (tc0 + tc1));
        nn->group_id = group_id;
        merged = true;
        nn->merged = true;
        if (-dot(new_mean, new_norm) < 0.0) new_norm = -new_norm;
        plane.mean = new_mean; plane.norm = new_norm; plane.cov = new_cov;
        nn->plane.mean = new_mean; nn->plane.norm = new_norm; nn->plane.cov = new_cov;
    }
}

// ---------------------------------------------------------------- clouds
struct CPoint { float x, y, z, intensity, t; };

// pcl::VoxelGrid<PointXYZINormal>::applyFilter (PCL 1.10, leaf-centroid,
// downsample_all_data_ = true), with a stable sort by leaf index.
void voxelGridFilter(const std::vector<CPoint>& in, double leaf_d, std::vector<CPoint>& out) {
    out.clear();
    if (in.empty()) return;
    float leaf = (float)leaf_d;
    float inv = 1.0f / leaf;
    float mn[3] = {in[0].x, in[0].y, in[0].z}, mx[3] = {in[0].x, in[0].y, in[0].z};
    for (const auto& p : in) {
        mn[0] = std::min(mn[0], p.x); mn[1] = std::min(mn[1], p.y); mn[2] = std::min(mn[2], p.z);
        mx[0] = std::max(mx[0], p.x); mx[1] = std::max(mx[1], p.y); mx[2] = std::max(mx[2], p.z);
    }
    int64_t dx = (int64_t)((mx[0] - mn[0]) * inv) + 1;
    int64_t dy = (int64_t)((mx[1] - mn[1]) * inv) + 1;
    int64_t dz = (int64_t)((mx[2] - mn[2]) * inv) + 1;
    if (dx * dy * dz > (int64_t)std::numeric_limits<int32_t>::max()) { out = in; return; }
    int minb[3], maxb[3], divb[3];
    for (int a = 0; a < 3; ++a) {
        minb[a] = (int)std::floor(mn[a] * inv);
        maxb[a] = (int)std::floor(mx[a] * inv);
        divb[a] = maxb[a] - minb[a] + 1;
    }
    uint32_t mul1 = (uint32_t)divb[0], mul2 = (uint32_t)divb[0] * (uint32_t)divb[1];
    std::vector<std::pair<uint32_t, uint32_t>> iv(in.size());
    for (size_t i = 0; i < in.size(); ++i) {
        const CPoint& p = in[i];
        int i0 = (int)(std::floor(p.x * inv) - (float)minb[0]);
        int i1 = (int)(std::floor(p.y * inv) - (float)minb[1]);
        int i2 = (int)(std::floor(p.z * inv) - (float)minb[2]);
        uint32_t idx = (uint32_t)i0 + (uint32_t)i1 * mul1 + (uint32_t)i2 * mul2;
        iv[i] = {idx, (uint32_t)i};
    }
    std::stable_sort(iv.begin(), iv.end(), [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) { return a.first < b.first; });
    size_t s = 0;
    while (s < iv.size()) {
        size_t e = s + 1;
        while (e < iv.size() && iv[e].first == iv[s].first) ++e;
        float sx = 0, sy = 0, sz = 0, si = 0, st = 0;
        for (size_t k = s; k < e; ++k) {
            const CPoint& p = in[iv[k].second];
            sx += p.x; sy += p.y; sz += p.z; si += p.intensity; st += p.t;
        }
        float c = (float)(e - s);
        out.push_back(CPoint{sx / c, sy / c, sz / c, si / c, st / c});
        s = e;
    }
}

// pcl::transformPointCloud with a float Matrix4f (PCL 1.10 SSE2 se3 order:
// x*c0 + (y*c1 + (z*c2 + c3))).
inline void transformFloat(const float R[9], const float t[3], const CPoint& p, float out[3]) {
    for (int r = 0; r < 3; ++r) out[r] = p.x * R[r * 3 + 0] + (p.y * R[r * 3 + 1] + (p.z * R[r * 3 + 2] + t[r]));
}

// ---------------------------------------------------------------- LIOBuilder
struct IMUData { V3 acc, gyro; double timestamp; };
struct Pose { double offset; V3 acc, gyro, vel, pos; M3 rot; };

struct LIOBuilder {  // lio_builder.h:56-83
    vmp_config config;
    IESKF kf;
    int status = VMP_IMU_INIT;
    // LIODataGroup (lio_builder.h:43-54)
    IMUData last_imu{};
    std::vector<IMUData> imu_cache;
    std::vector<Pose> imu_poses_cache;
    V3 last_acc = V3::Zero(), last_gyro = V3::Zero();
    double last_cloud_end_time = 0.0;
    double gravity_norm = 0.0;
    M12 Q = M12::Identity();
    std::vector<ResidualData> residual_info;
    std::vector<CPoint> cloud;        // package cloud (undistorted in place)
    std::vector<CPoint> lidar_cloud;  // downsampled
    std::unique_ptr<VoxelMap> map;
    int threads = 1;
    int last_effect = 0;
    int no_effect_flag = 0;
    long long last_evicted_total = 0;

    explicit LIOBuilder(const vmp_config& c) { loadConfig(c); }

    void loadConfig(const vmp_config& c) {  // lio_builder.cpp:5-26
        config = c;
        status = VMP_IMU_INIT;
        Q = M12::Identity();
        Q.setBlock(0, 0, M3::Identity() * config.ng);
        Q.setBlock(3, 3, M3::Identity() * config.na);
        Q.setBlock(6, 6, M3::Identity() * config.nbg);
        Q.setBlock(9, 9, M3::Identity() * config.nba);
        map.reset(new VoxelMap{config.max_point_thresh, config.update_size_thresh, config.plane_thresh,
                               config.voxel_size, config.map_capacity});
        map->merge_thresh_for_angle = config.merge_thresh_for_angle;
        map->merge_thresh_for_distance = config.merge_thresh_for_distance;
        kf.max_iter_ = (size_t)config.ieskf_max_iter;
        kf.eps_ = config.ieskf_eps;
        kf.func_ = [this](State& s, SharedState& d) { sharedUpdateFunc(s, d); };
        residual_info.resize(10000);
    }

    bool initializeImu(const std::vector<IMUData>& imus) {  // lio_builder.cpp:28-63
        imu_cache.insert(imu_cache.end(), imus.begin(), imus.end());
        if ((int)imu_cache.size() < config.imu_init_num) return false;
        V3 acc_mean = V3::Zero(), gyro_mean = V3::Zero();
        for (const auto& imu : imu_cache) { acc_mean += imu.acc; gyro_mean += imu.gyro; }
        acc_mean /= static_cast<double>(imu_cache.size());
        gyro_mean /= static_cast<double>(imu_cache.size());
        gravity_norm = norm(acc_mean);
        for (int i = 0; i < 9; ++i) kf.x_.rot_ext[i] = config.r_il[i];
        for (int i = 0; i < 3; ++i) kf.x_.pos_ext[i] = config.p_il[i];
        kf.x_.bg = gyro_mean;
        if (config.gravity_align) {
            kf.x_.rot = fromTwoVectors(normalized(-acc_mean), v3(0.0, 0.0, -1.0));
            kf.x_.initG(v3(0, 0, -1.0));
        } else {
            kf.x_.initG(-acc_mean);
        }
        kf.P_.setIdentity();
        kf.P_.setBlock(6, 6, M3::Identity() * 0.00001);
        kf.P_.setBlock(9, 9, M3::Identity() * 0.00001);
        kf.P_.setBlock(15, 15, M3::Identity() * 0.0001);
        kf.P_.setBlock(18, 18, M3::Identity() * 0.0001);
        kf.P_.setBlock(21, 21, M22::Identity() * 0.00001);
        last_imu = imus.back();
        return true;
    }

    void undistortCloud(const std::vector<IMUData>& pkg_imus, double cloud_time_begin, double cloud_time_end) {  // lio_builder.cpp:65-153
        imu_cache.clear();
        imu_cache.push_back(last_imu);
        imu_cache.insert(imu_cache.end(), pkg_imus.begin(), pkg_imus.end());
        const double imu_time_end = imu_cache.back().timestamp;
        std::stable_sort(cloud.begin(), cloud.end(), [](const CPoint& a, const CPoint& b) { return a.t < b.t; });
        imu_poses_cache.clear();
        imu_poses_cache.push_back(Pose{0.0, last_acc, last_gyro, kf.x_.vel, kf.x_.pos, kf.x_.rot});
        V3 acc_val, gyro_val;
        double dt = 0.0;
        V3 inp_acc = V3::Zero(), inp_gyro = V3::Zero();
        for (size_t k = 0; k + 1 < imu_cache.size(); ++k) {
            const IMUData& head = imu_cache[k];
            const IMUData& tail = imu_cache[k + 1];
            if (tail.timestamp < last_cloud_end_time) continue;
            gyro_val = 0.5 * (head.gyro + tail.gyro);
            acc_val = 0.5 * (head.acc + tail.acc);
            acc_val = acc_val * 9.81 / gravity_norm;
            if (head.timestamp < last_cloud_end_time) dt = tail.timestamp - last_cloud_end_time;
            else dt = tail.timestamp - head.timestamp;
            inp_acc = acc_val; inp_gyro = gyro_val;
            kf.predict(inp_acc, inp_gyro, dt, Q);
            last_gyro = gyro_val - kf.x_.bg;
            last_acc = kf.x_.rot * (acc_val - kf.x_.ba) + kf.x_.g;
            double offset = tail.timestamp - cloud_time_begin;
            imu_poses_cache.push_back(Pose{offset, last_acc, last_gyro, kf.x_.vel, kf.x_.pos, kf.x_.rot});
        }
        dt = cloud_time_end - imu_time_end;
        kf.predict(inp_acc, inp_gyro, dt, Q);
        last_imu = pkg_imus.back();
        last_cloud_end_time = cloud_time_end;
        M3 cur_rot = kf.x_.rot, cur_rot_ext = kf.x_.rot_ext;
        V3 cur_pos = kf.x_.pos, cur_pos_ext = kf.x_.pos_ext;
        if (cloud.empty()) return;
        long ip = (long)cloud.size() - 1;
        for (size_t kp = imu_poses_cache.size() - 1; kp != 0; --kp) {
            const Pose& head = imu_poses_cache[kp - 1];
            const Pose& tail = imu_poses_cache[kp];
            for (; cloud[ip].t / double(1000) > head.offset; ip--) {
                dt = cloud[ip].t / double(1000) - head.offset;
                V3 point = v3(cloud[ip].x, cloud[ip].y, cloud[ip].z);
                M3 point_rot = head.rot * Exp(tail.gyro * dt);
                V3 point_pos = head.pos + head.vel * dt + 0.5 * tail.acc * dt * dt;
                V3 pc = T(cur_rot_ext) * (T(cur_rot) * (point_rot * (cur_rot_ext * point + cur_pos_ext) + point_pos - cur_pos) - cur_pos_ext);
                cloud[ip].x = (float)pc[0]; cloud[ip].y = (float)pc[1]; cloud[ip].z = (float)pc[2];
                if (ip == 0) break;
            }
        }
    }

    void worldTransform(float R[9], float t[3]) const {  // lio_builder.cpp:155-163
        M3 r = kf.x_.rot * kf.x_.rot_ext;
        V3 p = kf.x_.rot * kf.x_.pos_ext + kf.x_.pos;
        for (int i = 0; i < 9; ++i) R[i] = (float)r[i];
        for (int i = 0; i < 3; ++i) t[i] = (float)p[i];
    }

    // lio_builder.cpp:200-203, 241-243; [p]x P_rr [p]x^T through hatSandwich
    M3 worldCov(const M3& r_wl, const M3& cov_l, const V3& p_l) const {
        return r_wl * cov_l * T(r_wl) + hatSandwich(p_l, kf.P_.block<3, 3>(3, 3)) + kf.P_.block<3, 3>(0, 0);
    }

    std::vector<float> next_intensity;  // intensities of the next package's points (else 0)

    void process(const vmp_scan& scan, const std::vector<IMUData>& imus) {  // lio_builder.cpp:175-248
        cloud.resize(scan.n);
        const bool has_int = (int)next_intensity.size() == scan.n;
        for (int i = 0; i < scan.n; ++i)
            cloud[i] = CPoint{scan.points[i].x, scan.points[i].y, scan.points[i].z,
                              has_int ? next_intensity[i] : 0.0f, scan.points[i].t_ms};
        next_intensity.clear();
        if (status == VMP_IMU_INIT) {
            if (initializeImu(imus)) {
                status = VMP_MAP_INIT;
                last_cloud_end_time = scan.t_end;
            }
        } else if (status == VMP_MAP_INIT) {
            undistortCloud(imus, scan.t_start, scan.t_end);
            float R[9], t[3];
            worldTransform(R, t);
            M3 r_wl = kf.x_.rot * kf.x_.rot_ext;
            std::vector<PointWithCov> pv_list;
            pv_list.reserve(cloud.size());
            for (size_t i = 0; i < cloud.size(); ++i) {
                float w[3];
                transformFloat(R, t, cloud[i], w);
                PointWithCov pv;
                pv.point = v3(w[0], w[1], w[2]);
                V3 pb = v3(cloud[i].x, cloud[i].y, cloud[i].z);
                M3 pc;
                calcBodyCov(pb, config.ranging_cov, config.angle_cov, pc);
                pv.cov = worldCov(r_wl, pc, pb);
                pv_list.push_back(pv);
            }
            map->build(pv_list);
            status = VMP_LIO_MAPPING;
        } else {
            undistortCloud(imus, scan.t_start, scan.t_end);
            if (config.scan_resolution > 0.0) voxelGridFilter(cloud, config.scan_resolution, lidar_cloud);
            else lidar_cloud = cloud;
            int size = (int)lidar_cloud.size();
            if ((int)residual_info.size() < size) residual_info.resize(size);
            for (int i = 0; i < size; i++) {
                residual_info[i].point_lidar = v3(lidar_cloud[i].x, lidar_cloud[i].y, lidar_cloud[i].z);
                calcBodyCov(residual_info[i].point_lidar, config.ranging_cov, config.angle_cov, residual_info[i].cov_lidar);
            }
            no_effect_flag = 0;
            kf.update();
            float R[9], t[3];
            worldTransform(R, t);
            M3 r_wl = kf.x_.rot * kf.x_.rot_ext;
            std::vector<PointWithCov> pv_list;
            pv_list.reserve(size);
            for (int i = 0; i < size; i++) {
                float w[3];
                transformFloat(R, t, lidar_cloud[i], w);
                PointWithCov pv;
                pv.point = v3(w[0], w[1], w[2]);
                pv.cov = worldCov(r_wl, residual_info[i].cov_lidar, residual_info[i].point_lidar);
                pv_list.push_back(pv);
            }
            map->update(pv_list);
        }
    }

    void sharedUpdateFunc(State& state, SharedState& shared) {  // lio_builder.cpp:250-311
        M3 r_wl = state.rot * state.rot_ext;
        V3 p_wl = state.rot * state.pos_ext + state.pos;
        int size = (int)lidar_cloud.size();
        M3 Prr = kf.P_.block<3, 3>(3, 3), Ppp = kf.P_.block<3, 3>(0, 0);
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static)
#endif
        for (int i = 0; i < size; i++) {
            ResidualData& rd = residual_info[i];
            rd.point_world = r_wl * rd.point_lidar + p_wl;
            M3 cm = hat(rd.point_lidar);
            rd.cov_world = r_wl * rd.cov_lidar * T(r_wl) + cm * Prr * T(cm) + Ppp;
            VoxelKey position = map->index(rd.point_world);
            auto iter = map->featmap.find(position);
            if (iter != map->featmap.end()) map->buildResidual(rd, iter->second);
        }
        shared.H.setZero();
        shared.b.setZero();
        int effect_num = 0;
        for (int i = 0; i < size; i++) {
            const ResidualData& rd = residual_info[i];
            if (!rd.is_valid) continue;
            effect_num++;
            Mat<1, 12> J = Mat<1, 12>::Zero();
            V3 pn = rd.plane_norm;
            Mat<1, 6> Jn;
            V3 pm = rd.point_world - rd.plane_mean;
            Jn(0, 0) = pm[0]; Jn(0, 1) = pm[1]; Jn(0, 2) = pm[2];
            Jn(0, 3) = -pn[0]; Jn(0, 4) = -pn[1]; Jn(0, 5) = -pn[2];
            double r_cov = (Jn * rd.plane_cov * T(Jn))(0, 0);
            r_cov += (T(pn) * r_wl * rd.cov_lidar * T(r_wl) * pn)(0, 0);
            double r_info = r_cov < 0.0002 ? 5000 : 1.0 / r_cov;
            J(0, 0) = pn[0]; J(0, 1) = pn[1]; J(0, 2) = pn[2];
            Mat<1, 3> j1 = (-T(pn)) * state.rot * hat(state.rot_ext * rd.point_lidar + state.pos_ext);
            J(0, 3) = j1(0, 0); J(0, 4) = j1(0, 1); J(0, 5) = j1(0, 2);
            if (config.estimate_ext) {
                Mat<1, 3> j2 = (-T(pn)) * r_wl * hat(rd.point_lidar);
                Mat<1, 3> j3 = T(pn) * state.rot;
                for (int k = 0; k < 3; ++k) { J(0, 6 + k) = j2(0, k); J(0, 9 + k) = j3(0, k); }
            }
            for (int a = 0; a < 12; ++a) {
                double u = J(0, a) * r_info;
                for (int c = 0; c < 12; ++c) shared.H(a, c) += u * J(0, c);
                shared.b[a] += u * rd.residual;
            }
        }
        last_effect = effect_num;
        if (effect_num < 1) no_effect_flag = 1;
    }
};

}  // namespace orc

// ====================================================================== C API
using namespace orc;

static void stateToC(const State& s, vmp_state* o) {
    for (int i = 0; i < 3; ++i) {
        o->pos[i] = s.pos[i]; o->pos_ext[i] = s.pos_ext[i]; o->vel[i] = s.vel[i];
        o->bg[i] = s.bg[i]; o->ba[i] = s.ba[i]; o->g[i] = s.g[i];
    }
    for (int i = 0; i < 9; ++i) { o->rot[i] = s.rot[i]; o->rot_ext[i] = s.rot_ext[i]; }
}
static void stateFromC(const vmp_state* o, State& s) {
    for (int i = 0; i < 3; ++i) {
        s.pos[i] = o->pos[i]; s.pos_ext[i] = o->pos_ext[i]; s.vel[i] = o->vel[i];
        s.bg[i] = o->bg[i]; s.ba[i] = o->ba[i]; s.g[i] = o->g[i];
    }
    for (int i = 0; i < 9; ++i) { s.rot[i] = o->rot[i]; s.rot_ext[i] = o->rot_ext[i]; }
}
static std::vector<IMUData> imusFromC(const vmp_imu* imus, int n) {
    std::vector<IMUData> v(n);
    for (int i = 0; i < n; ++i) {
        v[i].timestamp = imus[i].t;
        v[i].acc = v3(imus[i].acc[0], imus[i].acc[1], imus[i].acc[2]);
        v[i].gyro = v3(imus[i].gyro[0], imus[i].gyro[1], imus[i].gyro[2]);
    }
    return v;
}
static void voxelToC(const VoxelGrid& g, vmp_voxel* o) {
    std::memset(o, 0, sizeof(*o));
    o->key[0] = g.position.x; o->key[1] = g.position.y; o->key[2] = g.position.z;
    o->n = g.plane.n;
    o->newly_add_point = g.newly_add_point;
    o->is_init = g.is_init; o->is_plane = g.is_plane; o->update_enable = g.update_enable; o->merged = g.merged;
    o->group_id = g.group_id;
    o->n_temp = (int32_t)g.temp_points.size();
    for (int i = 0; i < 3; ++i) { o->mean[i] = g.plane.mean[i]; o->norm[i] = g.plane.norm[i]; o->center[i] = g.center[i]; }
    for (int i = 0; i < 9; ++i) o->ppt[i] = g.plane.ppt[i];
    for (int i = 0; i < 36; ++i) o->cov[i] = g.plane.cov[i];
}

extern "C" {

void* orc_create(const vmp_config* cfg) { return new LIOBuilder(*cfg); }
void orc_destroy(void* h) { delete (LIOBuilder*)h; }
void orc_set_threads(void* h, int n) { ((LIOBuilder*)h)->threads = n < 1 ? 1 : n; }

int orc_process(void* h, const vmp_scan* scan, const vmp_imu* imus, int n_imu, vmp_result* out) {
    LIOBuilder* b = (LIOBuilder*)h;
    b->process(*scan, imusFromC(imus, n_imu));
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->lio_status = b->status;
        out->iters = b->kf.last_iters;
        out->effect_num = b->last_effect;
        out->n_raw = scan->n;
        out->n_down = (int)b->lidar_cloud.size();
        out->flags = b->no_effect_flag;
        out->map_size = (long long)b->map->featmap.size();
        out->evicted = b->map->evicted - b->last_evicted_total;  // this scan's evictions
        stateToC(b->kf.x_, &out->x);
        for (int i = 0; i < 529; ++i) out->P[i] = b->kf.P_[i];
    }
    b->last_evicted_total = b->map->evicted;
    return 0;
}

void orc_get_state(void* h, vmp_state* x, double* P) {
    LIOBuilder* b = (LIOBuilder*)h;
    if (x) stateToC(b->kf.x_, x);
    if (P) for (int i = 0; i < 529; ++i) P[i] = b->kf.P_[i];
}
void orc_set_state(void* h, const vmp_state* x, const double* P) {
    LIOBuilder* b = (LIOBuilder*)h;
    if (x) stateFromC(x, b->kf.x_);
    if (P) for (int i = 0; i < 529; ++i) b->kf.P_[i] = P[i];
}
// Filter bookkeeping that the odometry loop carries between scans.
void orc_get_aux(void* h, double* aux /* 16 */) {
    LIOBuilder* b = (LIOBuilder*)h;
    for (int i = 0; i < 3; ++i) { aux[i] = b->last_acc[i]; aux[3 + i] = b->last_gyro[i]; }
    aux[6] = b->last_cloud_end_time; aux[7] = b->gravity_norm; aux[8] = b->status;
    aux[9] = b->last_imu.timestamp;
    for (int i = 0; i < 3; ++i) { aux[10 + i] = b->last_imu.acc[i]; aux[13 + i] = b->last_imu.gyro[i]; }
}
void orc_set_aux(void* h, const double* aux) {
    LIOBuilder* b = (LIOBuilder*)h;
    for (int i = 0; i < 3; ++i) { b->last_acc[i] = aux[i]; b->last_gyro[i] = aux[3 + i]; }
    b->last_cloud_end_time = aux[6]; b->gravity_norm = aux[7]; b->status = (int)aux[8];
    b->last_imu.timestamp = aux[9];
    for (int i = 0; i < 3; ++i) { b->last_imu.acc[i] = aux[10 + i]; b->last_imu.gyro[i] = aux[13 + i]; }
}

void orc_map_info(void* h, vmp_map_info* info) {
    LIOBuilder* b = (LIOBuilder*)h;
    info->size = (long long)b->map->featmap.size();
    info->capacity = b->map->capacity;
    info->group_counter = (long long)b->map->count;
    long long sp = 0;
    for (auto& kv : b->map->featmap) sp += (long long)kv.second->temp_points.size();
    info->slab_points = sp;
}

// LRU order (cache list front = most recently used).
long long orc_map_export(void* h, vmp_voxel* out, long long max) {
    LIOBuilder* b = (LIOBuilder*)h;
    long long n = 0;
    uint64_t stamp = b->map->cache.size();
    for (auto& k : b->map->cache) {
        if (n >= max) break;
        const VoxelGrid& g = *b->map->featmap[k];
        voxelToC(g, &out[n]);
        out[n].lru_stamp = stamp--;
        ++n;
    }
    return n;
}
// Keys of featmap in cache order (voxel_map.h:124-125), front first.
long long orc_map_keys(void* h, int64_t* keys, long long max) {
    LIOBuilder* b = (LIOBuilder*)h;
    long long n = 0;
    for (auto& k : b->map->cache) {
        if (n >= max) break;
        keys[3 * n] = k.x; keys[3 * n + 1] = k.y; keys[3 * n + 2] = k.z;
        ++n;
    }
    return (long long)b->map->cache.size();
}
// ResidualData::is_valid of the first n entries of residual_info
// (lio_builder.cpp:25, 260-274): the match set of the last iteration,
// stale entries included.
void orc_residual_valid(void* h, unsigned char* valid, int n) {
    LIOBuilder* b = (LIOBuilder*)h;
    for (int i = 0; i < n; ++i) valid[i] = i < (int)b->residual_info.size() ? b->residual_info[i].is_valid : 0;
}
long long orc_map_export_points(void* h, double* pts, double* cov, long long max_points) {
    LIOBuilder* b = (LIOBuilder*)h;
    long long n = 0;
    for (auto& k : b->map->cache) {
        const VoxelGrid& g = *b->map->featmap[k];
        for (const auto& pv : g.temp_points) {
            if (n >= max_points) return n;
            for (int i = 0; i < 3; ++i) pts[n * 3 + i] = pv.point[i];
            for (int i = 0; i < 9; ++i) cov[n * 9 + i] = pv.cov[i];
            ++n;
        }
    }
    return n;
}
void orc_map_import(void* h, const vmp_voxel* vox, long long n, const double* pts, const double* cov,
                    long long group_counter) {
    LIOBuilder* b = (LIOBuilder*)h;
    VoxelMap& m = *b->map;
    m.featmap.clear();
    m.cache.clear();
    long long off = 0;
    for (long long i = 0; i < n; ++i) {
        const vmp_voxel& v = vox[i];
        VoxelKey k{v.key[0], v.key[1], v.key[2]};
        auto g = std::make_shared<VoxelGrid>(m.max_point_thresh, m.update_point_thresh, m.plane_thresh, k, &m, v.group_id);
        g->plane.n = v.n;
        g->newly_add_point = v.newly_add_point;
        g->is_init = v.is_init; g->is_plane = v.is_plane; g->update_enable = v.update_enable; g->merged = v.merged;
        for (int j = 0; j < 3; ++j) { g->plane.mean[j] = v.mean[j]; g->plane.norm[j] = v.norm[j]; g->center[j] = v.center[j]; }
        for (int j = 0; j < 9; ++j) g->plane.ppt[j] = v.ppt[j];
        for (int j = 0; j < 36; ++j) g->plane.cov[j] = v.cov[j];
        for (int p = 0; p < v.n_temp; ++p, ++off) {
            PointWithCov pv;
            for (int j = 0; j < 3; ++j) pv.point[j] = pts[off * 3 + j];
            for (int j = 0; j < 9; ++j) pv.cov[j] = cov[off * 9 + j];
            g->temp_points.push_back(pv);
        }
        m.cache.push_back(k);
        g->cache_it = std::prev(m.cache.end());
        m.featmap[k] = g;
    }
    m.count = (uint64_t)group_counter;
}

static std::vector<PointWithCov> pvsFromC(const double* pts, const double* cov, int n) {
    std::vector<PointWithCov> v(n);
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < 3; ++j) v[i].point[j] = pts[i * 3 + j];
        for (int j = 0; j < 9; ++j) v[i].cov[j] = cov[i * 9 + j];
    }
    return v;
}
void orc_map_build(void* h, const double* pts, const double* cov, int n) {
    auto v = pvsFromC(pts, cov, n);
    ((LIOBuilder*)h)->map->build(v);
}
void orc_map_update(void* h, const double* pts, const double* cov, int n) {
    auto v = pvsFromC(pts, cov, n);
    ((LIOBuilder*)h)->map->update(v);
}
void orc_map_index(void* h, const double* pts, int n, int64_t* keys) {
    LIOBuilder* b = (LIOBuilder*)h;
    for (int i = 0; i < n; ++i) {
        VoxelKey k = b->map->index(v3(pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]));
        keys[i * 3] = k.x; keys[i * 3 + 1] = k.y; keys[i * 3 + 2] = k.z;
    }
}

// sharedUpdateFunc with an explicit state and points; residual_info persists.
int orc_residual_reduce(void* h, const vmp_state* x, const double* P, const double* pts_l, const double* cov_l,
                        int n, double* H, double* bvec, int* effect_num, unsigned char* valid_out) {
    LIOBuilder* b = (LIOBuilder*)h;
    stateFromC(x, b->kf.x_);
    for (int i = 0; i < 529; ++i) b->kf.P_[i] = P[i];
    b->lidar_cloud.resize(n);
    if ((int)b->residual_info.size() < n) b->residual_info.resize(n);
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < 3; ++j) b->residual_info[i].point_lidar[j] = pts_l[i * 3 + j];
        for (int j = 0; j < 9; ++j) b->residual_info[i].cov_lidar[j] = cov_l[i * 9 + j];
    }
    SharedState sh;
    b->sharedUpdateFunc(b->kf.x_, sh);
    for (int i = 0; i < 144; ++i) H[i] = sh.H[i];
    for (int i = 0; i < 12; ++i) bvec[i] = sh.b[i];
    *effect_num = b->last_effect;
    if (valid_out) for (int i = 0; i < n; ++i) valid_out[i] = b->residual_info[i].is_valid;
    return 0;
}

void orc_ieskf_predict(void* h, const double* acc, const double* gyro, double dt, const double* Q) {
    LIOBuilder* b = (LIOBuilder*)h;
    M12 q;
    for (int i = 0; i < 144; ++i) q[i] = Q[i];
    b->kf.predict(v3(acc[0], acc[1], acc[2]), v3(gyro[0], gyro[1], gyro[2]), dt, q);
}

void orc_ieskf_update(void* h, const float* pts_l, int n, int* iters, int* effect_num) {
    LIOBuilder* b = (LIOBuilder*)h;
    b->lidar_cloud.resize(n);
    for (int i = 0; i < n; ++i) b->lidar_cloud[i] = CPoint{pts_l[i * 3], pts_l[i * 3 + 1], pts_l[i * 3 + 2], 0.f, 0.f};
    if ((int)b->residual_info.size() < n) b->residual_info.resize(n);
    for (int i = 0; i < n; ++i) {
        b->residual_info[i].point_lidar = v3(pts_l[i * 3], pts_l[i * 3 + 1], pts_l[i * 3 + 2]);
        calcBodyCov(b->residual_info[i].point_lidar, b->config.ranging_cov, b->config.angle_cov, b->residual_info[i].cov_lidar);
    }
    b->kf.update();
    *iters = b->kf.last_iters;
    *effect_num = b->last_effect;
}

void orc_undistort(void* h, const vmp_scan* scan, const vmp_imu* imus, int n_imu, vmp_point* out) {
    LIOBuilder* b = (LIOBuilder*)h;
    b->cloud.resize(scan->n);
    for (int i = 0; i < scan->n; ++i)
        b->cloud[i] = CPoint{scan->points[i].x, scan->points[i].y, scan->points[i].z, 0.0f, scan->points[i].t_ms};
    b->undistortCloud(imusFromC(imus, n_imu), scan->t_start, scan->t_end);
    for (int i = 0; i < scan->n; ++i) out[i] = vmp_point{b->cloud[i].x, b->cloud[i].y, b->cloud[i].z, b->cloud[i].t};
}

int orc_downsample(const vmp_point* pts, int n, double leaf, vmp_point* out) {
    std::vector<CPoint> in(n), o;
    for (int i = 0; i < n; ++i) in[i] = CPoint{pts[i].x, pts[i].y, pts[i].z, 0.0f, pts[i].t_ms};
    voxelGridFilter(in, leaf, o);
    for (size_t i = 0; i < o.size(); ++i) out[i] = vmp_point{o[i].x, o[i].y, o[i].z, o[i].t};
    return (int)o.size();
}

// point_crossmat * P_rr * point_crossmat^T as written (lio_builder.cpp:199-202).
void orc_hat_sandwich(const double* pts, const double* M, int n, double* out) {
    for (int i = 0; i < n; ++i) {
        M3 m;
        for (int k = 0; k < 9; ++k) m[k] = M[i * 9 + k];
        const M3 o = hatSandwich(v3(pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]), m);
        for (int k = 0; k < 9; ++k) out[i * 9 + k] = o[k];
    }
}
void orc_calc_body_cov(const double* pts, int n, double range_inc, double degree_inc, double* pts_out, double* cov) {
    for (int i = 0; i < n; ++i) {
        V3 p = v3(pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]);
        M3 c;
        calcBodyCov(p, range_inc, degree_inc, c);
        for (int j = 0; j < 3; ++j) pts_out[i * 3 + j] = p[j];
        for (int j = 0; j < 9; ++j) cov[i * 9 + j] = c[j];
    }
}

// The clouds of the last process() call: kind 0 = undistorted package cloud,
// kind 1 = downsampled lidar_cloud.
int orc_last_cloud(void* h, int kind, vmp_point* out, int max) {
    LIOBuilder* b = (LIOBuilder*)h;
    const std::vector<CPoint>& c = kind == 0 ? b->cloud : b->lidar_cloud;
    int n = (int)c.size();
    for (int i = 0; i < n && i < max; ++i) out[i] = vmp_point{c[i].x, c[i].y, c[i].z, c[i].t};
    return n;
}

// Small-state helpers for unit tests of the SO(3)/S2 algebra.
void orc_so3_exp(const double* w, double* R) { M3 r = Exp(v3(w[0], w[1], w[2])); for (int i = 0; i < 9; ++i) R[i] = r[i]; }
void orc_so3_log(const double* R, double* w) { M3 r; for (int i = 0; i < 9; ++i) r[i] = R[i]; V3 v = Log(r); for (int i = 0; i < 3; ++i) w[i] = v[i]; }
void orc_eig_sym3(const double* A, double* evals, double* evecs) {
    M3 a; for (int i = 0; i < 9; ++i) a[i] = A[i];
    V3 e; M3 v; eigSym3(a, e, v);
    for (int i = 0; i < 3; ++i) evals[i] = e[i];
    for (int i = 0; i < 9; ++i) evecs[i] = v[i];
}

// Batched plane fit (vmp_fit_planes): per voxel, VoxelGrid::addPoint for each
// of its points in order, then one updatePlane -- what VoxelMap::build does
// for a voxel (voxel_map.cpp:200-230, 29-40, 97-136).  FP64; voxels are
// independent, so they are spread over `threads` OpenMP threads.
void orc_fit_planes(const float* xyz, const float* cov, const long long* off, int n_vox, long long n_pts,
                    int update_point_thresh, double plane_thresh, vmp_fit_rec* out, int threads) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads < 1 ? 1 : threads)
    for (int v = 0; v < n_vox; ++v) {
        const long long p0 = off[v], p1 = off[v + 1];
        const int n = (int)(p1 - p0);
        VoxelGrid g(n > 0 ? n : 1, update_point_thresh, plane_thresh, VoxelKey{0, 0, 0}, nullptr, 0);
        for (long long i = p0; i < p1; ++i) {
            PointWithCov pv;
            pv.point = v3(xyz[i], xyz[n_pts + i], xyz[2 * n_pts + i]);
            const double c[6] = {cov[i], cov[n_pts + i], cov[2 * n_pts + i], cov[3 * n_pts + i],
                                 cov[4 * n_pts + i], cov[5 * n_pts + i]};
            pv.cov(0, 0) = c[0]; pv.cov(0, 1) = c[1]; pv.cov(0, 2) = c[2];
            pv.cov(1, 0) = c[1]; pv.cov(1, 1) = c[3]; pv.cov(1, 2) = c[4];
            pv.cov(2, 0) = c[2]; pv.cov(2, 1) = c[4]; pv.cov(2, 2) = c[5];
            g.addPoint(pv);
        }
        g.updatePlane();
        vmp_fit_rec& r = out[v];
        std::memset(&r, 0, sizeof(r));
        r.n = n;
        for (int k = 0; k < 3; ++k) r.mean[k] = g.plane.mean[k];
        if (!g.is_init) continue;
        // C and its eigen decomposition as updatePlane formed them
        M3 C = g.plane.ppt / static_cast<double>(g.plane.n) - g.plane.mean * T(g.plane.mean);
        V3 ev; M3 E;
        eigSym3(C, ev, E);
        r.cov[0] = C(0, 0); r.cov[1] = C(0, 1); r.cov[2] = C(0, 2);
        r.cov[3] = C(1, 1); r.cov[4] = C(1, 2); r.cov[5] = C(2, 2);
        for (int k = 0; k < 3; ++k) r.evals[k] = ev[k];
        r.flags = VMP_FIT_FITTED;
        if (!g.is_plane) continue;
        r.flags |= VMP_FIT_PLANE;
        if (g.plane.norm[0] != E(0, 0) || g.plane.norm[1] != E(1, 0) || g.plane.norm[2] != E(2, 0))
            r.flags |= VMP_FIT_FLIPPED;
        for (int k = 0; k < 3; ++k) r.norm[k] = g.plane.norm[k];
        int e = 0;
        for (int i = 0; i < 6; ++i)
            for (int j = i; j < 6; ++j) r.plane_cov[e++] = g.plane.cov(i, j);
    }
}

// livox2pcl (src/utils.cpp:3-28): line / tag filter, 1-in-filter_num
// decimation of the passing points, range gate with |p|^2 summed in float.
int orc_livox_decode(const vmp_livox_point* in, int n, int filter_num, double range_min, double range_max,
                     vmp_point* out, float* intensity) {
    unsigned valid_num = 0;
    int m = 0;
    for (int i = 0; i < n; i++) {
        const vmp_livox_point& q = in[i];
        if ((q.line < 4) && ((q.tag & 0x30) == 0x10 || (q.tag & 0x30) == 0x00)) {
            if ((valid_num++) % (unsigned)filter_num != 0) continue;
            const float x = q.x, y = q.y, z = q.z;
            const float t = q.offset_time / float(1000000);
            const double sq_range = x * x + y * y + z * z;
            if (sq_range > (range_min * range_min) && sq_range < range_max * range_max) {
                out[m] = vmp_point{x, y, z, t};
                if (intensity) intensity[m] = q.reflectivity;
                ++m;
            }
        }
    }
    return m;
}

// Intensities of the points of the next orc_process package (n must match).
void orc_set_intensity(void* h, const float* v, int n) {
    ((LIOBuilder*)h)->next_intensity.assign(v, v + n);
}

// lidarToBody (frame 0) / lidarToWorld (frame 1) of the package cloud after
// process (lio_builder.cpp:155-173).
int orc_output_cloud(void* h, int frame, vmp_point* out, float* intensity, int max) {
    LIOBuilder* b = (LIOBuilder*)h;
    float R[9], t[3];
    if (frame == 0) {
        for (int i = 0; i < 9; ++i) R[i] = (float)b->kf.x_.rot_ext[i];
        for (int i = 0; i < 3; ++i) t[i] = (float)b->kf.x_.pos_ext[i];
    } else {
        b->worldTransform(R, t);
    }
    const int n = (int)b->cloud.size();
    for (int i = 0; i < n && i < max; ++i) {
        float w[3];
        transformFloat(R, t, b->cloud[i], w);
        out[i] = vmp_point{w[0], w[1], w[2], b->cloud[i].t};
        if (intensity) intensity[i] = b->cloud[i].intensity;
    }
    return n;
}

// voxel2MarkerArray (src/utils.cpp:154-208) without the ROS message: the
// frozen planes in LRU order, their trace colour (mapJet, utils.cpp:78-128)
// and the marker orientation (calcVectQuation -> Quaterniond::FromTwoVectors,
// utils.cpp:144-152; the antiparallel case picks the x axis, see mathkit).
static void mapJetRestated(double v, double vmin, double vmax, uint8_t& r, uint8_t& g, uint8_t& b) {
    if (v < vmin) v = vmin;
    if (v > vmax) v = vmax;
    double dr, dg, db;
    if (v < 0.1242) { db = 0.504 + ((1. - 0.504) / 0.1242) * v; dg = dr = 0.; }
    else if (v < 0.3747) { db = 1.; dr = 0.; dg = (v - 0.1242) * (1. / (0.3747 - 0.1242)); }
    else if (v < 0.6253) { db = (0.6253 - v) * (1. / (0.6253 - 0.3747)); dg = 1.; dr = (v - 0.3747) * (1. / (0.6253 - 0.3747)); }
    else if (v < 0.8758) { db = 0.; dr = 1.; dg = (0.8758 - v) * (1. / (0.8758 - 0.6253)); }
    else { db = 0.; dg = 0.; dr = 1. - (v - 0.8758) * ((1. - 0.504) / (1. - 0.8758)); }
    r = (uint8_t)(255 * dr);
    g = (uint8_t)(255 * dg);
    b = (uint8_t)(255 * db);
}
int orc_map_planes(void* h, vmp_plane_marker* out, int max) {
    LIOBuilder* b = (LIOBuilder*)h;
    VoxelMap& m = *b->map;
    const int size = std::min((int)m.cache.size(), max);
    int count = 0;
    for (auto& k : m.cache) {
        if (count >= size) break;
        VoxelGrid* g = m.featmap[k].get();
        if (!g->is_plane || g->update_enable) continue;
        vmp_plane_marker& o = out[count++];
        std::memset(&o, 0, sizeof(o));
        for (int i = 0; i < 3; ++i) { o.center[i] = g->center[i]; o.norm[i] = g->plane.norm[i]; }
        double trace = (g->plane.cov(0, 0) + g->plane.cov(1, 1)) + g->plane.cov(2, 2);
        o.trace = trace;
        if (trace >= 0.25) trace = 0.25;
        trace = trace * (1.0 / 0.25);
        trace = std::pow(trace, 0.2);
        mapJetRestated(trace, 0, 1, o.rgb[0], o.rgb[1], o.rgb[2]);
        o.merged = g->merged ? 1 : 0;
        quatFromTwoVectors(v3(0, 0, 1), g->plane.norm, o.orientation);
    }
    return count;
}

// std_desc::STDManager::buildVoxels (std_matcher/src/std_manager/
// descriptor.cpp:70-122): voxels of the cloud (VoxelKey::index with bias 0,
// descriptor.cpp:44-49), FP64 sum and outer-product sum in cloud order, and
// for voxels with more than min_point points the mean, the decomposition of
// C (eigSym3: the symmetric restatement; the reference's general EigenSolver
// gives the same eigenvalues of a symmetric matrix up to rounding) and the
// plane test.  Records in ascending (z, y, x) key order.
int orc_std_plane_voxels(const float* pts, int stride, int n, double voxel_size, int min_point, double plane_thresh,
                         vmp_std_voxel* out, int max) {
    struct Acc { int n = 0; V3 sum = V3::Zero(); M3 ppt = M3::Zero(); };
    std::map<std::tuple<int64_t, int64_t, int64_t>, Acc> vox;
    for (int i = 0; i < n; ++i) {
        const V3 p = v3(pts[(size_t)i * stride], pts[(size_t)i * stride + 1], pts[(size_t)i * stride + 2]);
        const int64_t kx = (int64_t)std::floor(p[0] / voxel_size + 0.0);
        const int64_t ky = (int64_t)std::floor(p[1] / voxel_size + 0.0);
        const int64_t kz = (int64_t)std::floor(p[2] / voxel_size + 0.0);
        Acc& a = vox[std::make_tuple(kz, ky, kx)];
        a.n += 1;
        a.sum += p;
        a.ppt += p * T(p);
    }
    int m = 0;
    for (auto& kv : vox) {
        if (m >= max) break;
        vmp_std_voxel& o = out[m++];
        std::memset(&o, 0, sizeof(o));
        o.key[0] = std::get<2>(kv.first);
        o.key[1] = std::get<1>(kv.first);
        o.key[2] = std::get<0>(kv.first);
        const Acc& a = kv.second;
        o.n = a.n;
        for (int k = 0; k < 3; ++k) o.sum[k] = a.sum[k];
        for (int k = 0; k < 9; ++k) o.ppt[k] = a.ppt[k];
        if (a.n <= min_point) continue;
        o.valid = 1;
        const V3 mean = a.sum / static_cast<double>(a.n);
        const M3 C = a.ppt / static_cast<double>(a.n) - mean * T(mean);
        V3 ev; M3 E;
        eigSym3(C, ev, E);
        for (int k = 0; k < 3; ++k) o.mean[k] = mean[k];
        if (ev[0] < plane_thresh) {
            o.is_plane = 1;
            for (int k = 0; k < 3; ++k) o.lamdas[k] = ev[k];
            for (int k = 0; k < 9; ++k) o.norms[k] = E[k];
        }
    }
    return (int)vox.size();
}

}  // extern "C"
