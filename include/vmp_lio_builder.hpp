// vmp_lio_builder.hpp -- header-only C++ adapter with the shape of
// lio::LIOBuilder (voxel_plus/src/map_builder/lio_builder.h:56-83) over the C
// ABI of libvmp.so, so that the node's LIONode::mainCB
// (voxel_plus/src/lio_node.cpp:167-182) keeps calling
//     map_builder.process(sync_pack); map_builder.status; map_builder.kf.x()
// while the odometry step runs on the GPU.
//
// It is templated on the package / point / IMU types instead of including PCL
// or Eigen: Package needs `cloud->points` (points with x, y, z, curvature),
// `imus` (elements with acc[0..2], gyro[0..2], timestamp) and
// `cloud_start_time`, `cloud_end_time` -- lio::SyncPackage (commons.h:22-28).
// The package cloud is written back time-sorted and motion-compensated, as
// LIOBuilder::undistortCloud leaves it (lio_builder.cpp:65-153), so the node's
// lidarToBody / lidarToWorld publishing works on it unchanged.
#pragma once
#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "vmp.h"

namespace vmp_adapter {

enum LIOStatus { IMU_INIT = VMP_IMU_INIT, MAP_INIT = VMP_MAP_INIT, LIO_MAPPING = VMP_LIO_MAPPING };

class LIOBuilder {
public:
    LIOBuilder() = default;
    LIOBuilder(const LIOBuilder&) = delete;
    LIOBuilder& operator=(const LIOBuilder&) = delete;
    ~LIOBuilder() {
        if (s_) vmp_destroy(s_);
    }

    // LIOBuilder::loadConfig (lio_builder.cpp:5-26): Cfg has lio::LIOConfig's
    // field names (r_il / p_il index like Eigen: r_il(i, j), p_il(i)).
    template <class Cfg>
    void loadConfig(const Cfg& c) {
        vmp_config v;
        vmp_config_default(&v);
        v.opti_max_iter = c.opti_max_iter;
        v.na = c.na; v.ng = c.ng; v.nba = c.nba; v.nbg = c.nbg;
        v.imu_init_num = c.imu_init_num;
        for (int i = 0; i < 3; ++i) {
            v.p_il[i] = c.p_il(i);
            for (int j = 0; j < 3; ++j) v.r_il[i * 3 + j] = c.r_il(i, j);
        }
        v.gravity_align = c.gravity_align ? 1 : 0;
        v.estimate_ext = c.estimate_ext ? 1 : 0;
        v.scan_resolution = c.scan_resolution;
        v.voxel_size = c.voxel_size;
        v.update_size_thresh = c.update_size_thresh;
        v.max_point_thresh = c.max_point_thresh;
        v.plane_thresh = c.plane_thresh;
        v.ranging_cov = c.ranging_cov;
        v.angle_cov = c.angle_cov;
        v.merge_thresh_for_angle = c.merge_thresh_for_angle;
        v.merge_thresh_for_distance = c.merge_thresh_for_distance;
        v.map_capacity = c.map_capacity;
        loadConfig(v);
    }
    void loadConfig(const vmp_config& v) {
        if (s_) vmp_destroy(s_);
        s_ = nullptr;
        vmp_status st = vmp_create(&v, &s_);
        if (st != VMP_OK) throw std::runtime_error(std::string("vmp_create: ") + vmp_last_error(nullptr));
        status = IMU_INIT;
    }

    // LIOBuilder::process (lio_builder.cpp:175-248).
    template <class Package>
    void process(Package& pkg) {
        auto& pts = pkg.cloud->points;
        const int n = static_cast<int>(pts.size());
        // stable time order on the host keeps per-point attributes (intensity)
        // aligned with the compensated coordinates written back below
        bool sorted = true;
        for (int i = 1; i < n && sorted; ++i) sorted = !(pts[i].curvature < pts[i - 1].curvature);
        if (!sorted)
            std::stable_sort(pts.begin(), pts.end(), [](const auto& a, const auto& b) { return a.curvature < b.curvature; });
        pts_.resize(static_cast<size_t>(n));
        for (int i = 0; i < n; ++i) pts_[i] = vmp_point{pts[i].x, pts[i].y, pts[i].z, pts[i].curvature};
        imus_.resize(pkg.imus.size());
        for (size_t i = 0; i < pkg.imus.size(); ++i) {
            const auto& m = pkg.imus[i];
            imus_[i].t = m.timestamp;
            for (int a = 0; a < 3; ++a) { imus_[i].acc[a] = m.acc[a]; imus_[i].gyro[a] = m.gyro[a]; }
        }
        vmp_scan scan{pts_.data(), n, pkg.cloud_start_time, pkg.cloud_end_time};
        vmp_status st = vmp_process(s_, &scan, imus_.data(), static_cast<int>(imus_.size()), &res_);
        if (st != VMP_OK) throw std::runtime_error(std::string("vmp_process: ") + vmp_last_error(s_));
        status = static_cast<LIOStatus>(res_.lio_status);
        if (res_.lio_status != VMP_IMU_INIT && n > 0) {
            int m = 0;
            vmp_last_cloud(s_, 0, pts_.data(), n, &m);
            for (int i = 0; i < n && i < m; ++i) { pts[i].x = pts_[i].x; pts[i].y = pts_[i].y; pts[i].z = pts_[i].z; }
        }
    }

    // LIOBuilder::lidarToBody / lidarToWorld (lio_builder.cpp:155-173) of the
    // last processed cloud, formed on the device from its undistorted copy.
    // PointVec: a vector of points with x, y, z, intensity, curvature
    // (pcl::PointXYZINormal); intensity is the decoded reflectivity after
    // vmp_livox_decode + vmp_process_decoded, else 0 (the package cloud
    // written back by process keeps the node's own intensities).
    template <class PointVec>
    void lidarToBody(PointVec& out) { outputCloud(0, out); }
    template <class PointVec>
    void lidarToWorld(PointVec& out) { outputCloud(1, out); }

    // kf::IESKF::x() / P() equivalents (ieskf.h:86-90), row-major.
    const vmp_state& x() const { return res_.x; }
    const double* P() const { return res_.P; }
    const vmp_result& last_result() const { return res_; }
    vmp_stream_t handle() const { return s_; }

    LIOStatus status = IMU_INIT;

private:
    template <class PointVec>
    void outputCloud(int frame, PointVec& out) {
        int n = 0;
        vmp_status st = vmp_output_cloud(s_, frame, nullptr, nullptr, 0, &n);
        if (st != VMP_OK) throw std::runtime_error(std::string("vmp_output_cloud: ") + vmp_last_error(s_));
        cloud_.resize(static_cast<size_t>(n));
        inten_.resize(static_cast<size_t>(n));
        if (n > 0) vmp_output_cloud(s_, frame, cloud_.data(), inten_.data(), n, &n);
        out.resize(static_cast<size_t>(n));
        for (int i = 0; i < n; ++i) {
            out[i].x = cloud_[i].x;
            out[i].y = cloud_[i].y;
            out[i].z = cloud_[i].z;
            out[i].intensity = inten_[i];
            out[i].curvature = cloud_[i].t_ms;
        }
    }

    vmp_stream_t s_ = nullptr;
    std::vector<vmp_point> cloud_;
    std::vector<float> inten_;
    vmp_result res_{};
    std::vector<vmp_point> pts_;
    std::vector<vmp_imu> imus_;
};

}  // namespace vmp_adapter
