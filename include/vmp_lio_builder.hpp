// vmp_lio_builder.hpp -- header-only C++ adapter with the shape of
// lio::LIOBuilder (voxel_plus/src/map_builder/lio_builder.h:56-83) over the C
// ABI of libvmp.so: the members the ROS node touches are here with the
// reference's names and types,
//     map_builder.loadConfig(lio_config);                 lio_node.cpp:44
//     map_builder.process(sync_pack);                     lio_node.cpp:171
//     map_builder.status != lio::LIOStatus::LIO_MAPPING   lio_node.cpp:172
//     state = map_builder.kf.x();                         lio_node.cpp:174
//     map_builder.lidarToBody(sync_pack.cloud)            lio_node.cpp:176 (and lidarToWorld, :178)
//     std::shared_ptr<lio::VoxelMap> m = map_builder.map; lio_node.cpp:185
//     map_builder.kf.P().block<6, 6>(0, 0)                lio_node.cpp:227
// while the odometry step runs on the GPU.  The drop-in headers under
// include/vmp_node/map_builder/ put these names into namespace lio in place of
// the reference's lio_builder.h and voxel_map.h, so that lio_node.cpp and
// utils.cpp compile unchanged.
//
// Needs Eigen (as the node does), not PCL, Sophus or ROS: the package, cloud
// and state types are template parameters.  Package needs `cloud->points`
// (points with x, y, z, curvature), `imus` (acc[0..2], gyro[0..2],
// timestamp), `cloud_start_time`, `cloud_end_time` -- lio::SyncPackage
// (commons.h:22-28).  The package cloud is written back time-sorted and
// motion-compensated, as LIOBuilder::undistortCloud leaves it
// (lio_builder.cpp:65-153).
#pragma once
#include <Eigen/Core>

#include <algorithm>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "vmp.h"

namespace vmp_adapter {

// lio::LIOStatus (lio_builder.h:10-16)
enum LIOStatus { IMU_INIT = VMP_IMU_INIT, MAP_INIT = VMP_MAP_INIT, LIO_MAPPING = VMP_LIO_MAPPING };

// lio::LIOConfig (lio_builder.h:17-42): same fields, same defaults.
struct LIOConfig {
    int opti_max_iter = 5;
    double na = 0.01;
    double ng = 0.01;
    double nba = 0.0001;
    double nbg = 0.0001;
    int imu_init_num = 20;
    Eigen::Matrix3d r_il = Eigen::Matrix3d::Identity();
    Eigen::Vector3d p_il = Eigen::Vector3d::Zero();
    bool gravity_align = true;
    bool estimate_ext = false;
    double scan_resolution = 0.1;
    double voxel_size = 0.5;
    int update_size_thresh = 10;
    int max_point_thresh = 100;
    double plane_thresh = 0.01;
    double ranging_cov = 0.04;
    double angle_cov = 0.1;
    double merge_thresh_for_angle = 0.1;
    double merge_thresh_for_distance = 0.04;
    int map_capacity = 100000;
};

inline void check(vmp_stream_t s, vmp_status st, const char* what) {
    if (st != VMP_OK) throw std::runtime_error(std::string(what) + ": " + vmp_last_error(s));
}

// ------------------------------------------------------------------- filter
// The filter state of the last processed scan, convertible to the node's
// kf::State (ieskf.h:31-44: Eigen members pos, rot, rot_ext, pos_ext, vel,
// bg, ba, g), so that `state = map_builder.kf.x();` compiles as before.
class StateView {
public:
    explicit StateView(const vmp_state& x) : x_(x) {}
    template <class State>
    operator State() const {
        State s;
        for (int i = 0; i < 3; ++i) {
            s.pos(i) = x_.pos[i];
            s.pos_ext(i) = x_.pos_ext[i];
            s.vel(i) = x_.vel[i];
            s.bg(i) = x_.bg[i];
            s.ba(i) = x_.ba[i];
            s.g(i) = x_.g[i];
            for (int j = 0; j < 3; ++j) {
                s.rot(i, j) = x_.rot[i * 3 + j];
                s.rot_ext(i, j) = x_.rot_ext[i * 3 + j];
            }
        }
        return s;
    }
    const vmp_state& raw() const { return x_; }

private:
    vmp_state x_;
};

// kf::IESKF's read side (ieskf.h:86-90): x() and P() after the last scan.
class KFView {
public:
    StateView x() const { return StateView(x_); }
    const Eigen::Matrix<double, 23, 23>& P() const { return P_; }
    void set(const vmp_result& r) {
        x_ = r.x;
        for (int i = 0; i < 23; ++i)
            for (int j = 0; j < 23; ++j) P_(i, j) = r.P[i * 23 + j];
    }

private:
    vmp_state x_{};
    Eigen::Matrix<double, 23, 23> P_ = Eigen::Matrix<double, 23, 23>::Zero();
};

// ---------------------------------------------------------------------- map
// lio::VoxelKey (voxel_map.h:11-34).
struct VoxelKey {
    int64_t x = 0, y = 0, z = 0;
    VoxelKey() = default;
    VoxelKey(int64_t a, int64_t b, int64_t c) : x(a), y(b), z(c) {}
    bool operator==(const VoxelKey& o) const { return x == o.x && y == o.y && z == o.z; }
    struct Hasher {
        int64_t operator()(const VoxelKey& k) const {
            const int64_t p = 116101, m = 10000000000LL;
            return ((((k.z) * p) % m + (k.y)) * p) % m + (k.x);
        }
    };
};

// lio::Plane (voxel_map.h:43-51) and the VoxelGrid fields a reader of the
// map uses (voxel_map.h:84-102), copied from the device.
struct PlaneView {
    Eigen::Vector3d mean = Eigen::Vector3d::Zero();
    Eigen::Matrix3d ppt = Eigen::Matrix3d::Zero();
    Eigen::Vector3d norm = Eigen::Vector3d::Zero();
    Eigen::Matrix<double, 6, 6> cov = Eigen::Matrix<double, 6, 6>::Zero();
    int n = 0;
};
struct GridView {
    VoxelKey position;
    bool is_init = false, is_plane = false, update_enable = true, merged = false;
    int newly_add_point = 0;
    uint64_t group_id = 0;
    Eigen::Vector3d center = Eigen::Vector3d::Zero();
    std::shared_ptr<PlaneView> plane = std::make_shared<PlaneView>();
};

// lio::VoxelMap's read side (voxel_map.h:106-128) over the device map: `cache`
// (keys, most recently used first) and `featmap` (key -> voxel) are fetched
// from the device when first read after a scan; `cache.size()` asks the
// device for the live count only.  For the node's voxel-map timer and
// voxel2MarkerArray (utils.cpp:154-208).  Not thread-safe: read it from the
// thread that calls process (the node's single-threaded spinner does).
class VoxelMapView {
public:
    class Cache {
    public:
        size_t size() const {
            vmp_map_info i{};
            check(m_->s_, vmp_map_info_get(m_->s_, &i), "vmp_map_info_get");
            return static_cast<size_t>(i.size);
        }
        bool empty() const { return size() == 0; }
        std::vector<VoxelKey>::const_iterator begin() const { return m_->keys().begin(); }
        std::vector<VoxelKey>::const_iterator end() const { return m_->keys().end(); }

    private:
        friend class VoxelMapView;
        VoxelMapView* m_ = nullptr;
    };
    class Featmap {
    public:
        typedef std::unordered_map<VoxelKey, std::shared_ptr<GridView>, VoxelKey::Hasher> Map;
        typename Map::const_iterator find(const VoxelKey& k) const { return m_->grids().find(k); }
        typename Map::const_iterator begin() const { return m_->grids().begin(); }
        typename Map::const_iterator end() const { return m_->grids().end(); }
        size_t size() const { return m_->grids().size(); }
        size_t count(const VoxelKey& k) const { return m_->grids().count(k); }
        // a key that is not in the map gives an empty pointer (the reference's
        // operator[] would insert one)
        std::shared_ptr<GridView> operator[](const VoxelKey& k) const {
            auto it = m_->grids().find(k);
            return it == m_->grids().end() ? std::shared_ptr<GridView>() : it->second;
        }

    private:
        friend class VoxelMapView;
        VoxelMapView* m_ = nullptr;
    };

    VoxelMapView(vmp_stream_t s, const vmp_config& c)
        : voxel_size(c.voxel_size), capacity(static_cast<int>(c.map_capacity)),
          max_point_thresh(c.max_point_thresh), update_point_thresh(c.update_size_thresh),
          plane_thresh(c.plane_thresh), s_(s) {
        cache.m_ = this;
        featmap.m_ = this;
    }
    VoxelMapView(const VoxelMapView&) = delete;
    VoxelMapView& operator=(const VoxelMapView&) = delete;

    // the device map changed (a scan was processed): snapshots are stale
    void invalidate() { ++version_; }

    double voxel_size;
    int capacity;
    int max_point_thresh;
    int update_point_thresh;
    double plane_thresh;
    Cache cache;
    Featmap featmap;

private:
    const std::vector<VoxelKey>& keys() {
        if (keys_version_ != version_) {
            long long n = 0;
            check(s_, vmp_map_keys(s_, nullptr, 0, &n), "vmp_map_keys");
            std::vector<int64_t> raw(static_cast<size_t>(3 * n));
            if (n > 0) check(s_, vmp_map_keys(s_, raw.data(), n, &n), "vmp_map_keys");
            keys_.resize(static_cast<size_t>(n));
            for (long long i = 0; i < n; ++i) keys_[i] = VoxelKey(raw[3 * i], raw[3 * i + 1], raw[3 * i + 2]);
            keys_version_ = version_;
        }
        return keys_;
    }
    const Featmap::Map& grids() {
        if (grids_version_ != version_) {
            long long n = 0;
            check(s_, vmp_map_export(s_, nullptr, 0, &n), "vmp_map_export");
            std::vector<vmp_voxel> v(static_cast<size_t>(n));
            if (n > 0) check(s_, vmp_map_export(s_, v.data(), n, &n), "vmp_map_export");
            grids_.clear();
            grids_.reserve(static_cast<size_t>(n));
            for (const vmp_voxel& x : v) {
                auto g = std::make_shared<GridView>();
                g->position = VoxelKey(x.key[0], x.key[1], x.key[2]);
                g->is_init = x.is_init != 0;
                g->is_plane = x.is_plane != 0;
                g->update_enable = x.update_enable != 0;
                g->merged = x.merged != 0;
                g->newly_add_point = x.newly_add_point;
                g->group_id = x.group_id;
                g->plane->n = x.n;
                for (int i = 0; i < 3; ++i) {
                    g->center(i) = x.center[i];
                    g->plane->mean(i) = x.mean[i];
                    g->plane->norm(i) = x.norm[i];
                    for (int j = 0; j < 3; ++j) g->plane->ppt(i, j) = x.ppt[i * 3 + j];
                }
                for (int i = 0; i < 6; ++i)
                    for (int j = 0; j < 6; ++j) g->plane->cov(i, j) = x.cov[i * 6 + j];
                grids_[g->position] = g;
            }
            grids_version_ = version_;
        }
        return grids_;
    }

    vmp_stream_t s_;
    long long version_ = 0, keys_version_ = -1, grids_version_ = -1;
    std::vector<VoxelKey> keys_;
    Featmap::Map grids_;
};

// ------------------------------------------------------------------ builder
class LIOBuilder {
public:
    LIOBuilder() = default;
    LIOBuilder(const LIOBuilder&) = delete;
    LIOBuilder& operator=(const LIOBuilder&) = delete;
    ~LIOBuilder() {
        map.reset();
        if (s_) vmp_destroy(s_);
    }

    // LIOBuilder::loadConfig (lio_builder.cpp:5-26); Cfg has lio::LIOConfig's
    // field names (r_il / p_il indexed like Eigen: r_il(i, j), p_il(i)).
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
    // The same from a vmp_config (device buffer sizes included).
    void loadConfig(const vmp_config& v) {
        map.reset();
        if (s_) vmp_destroy(s_);
        s_ = nullptr;
        vmp_status st = vmp_create(&v, &s_);
        if (st != VMP_OK) throw std::runtime_error(std::string("vmp_create: ") + vmp_last_error(nullptr));
        status = IMU_INIT;
        res_ = vmp_result{};
        kf.set(res_);
        map = std::make_shared<VoxelMapView>(s_, v);
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
        check(s_, vmp_process(s_, &scan, imus_.data(), static_cast<int>(imus_.size()), &res_), "vmp_process");
        status = static_cast<LIOStatus>(res_.lio_status);
        kf.set(res_);
        map->invalidate();
        if (res_.lio_status != VMP_IMU_INIT && n > 0) {
            int m = 0;
            check(s_, vmp_last_cloud(s_, 0, pts_.data(), n, &m), "vmp_last_cloud");
            for (int i = 0; i < n && i < m; ++i) { pts[i].x = pts_[i].x; pts[i].y = pts_[i].y; pts[i].z = pts_[i].z; }
        }
    }

    // LIOBuilder::lidarToBody / lidarToWorld (lio_builder.cpp:155-173): a new
    // cloud with the input's points and header whose coordinates are the
    // device's body / world transform of the last processed cloud.  `cloud`
    // is that cloud (the package cloud process wrote back); another size is an
    // error.
    template <class CloudPtr>
    CloudPtr lidarToBody(const CloudPtr cloud) { return outputCloud(0, cloud); }
    template <class CloudPtr>
    CloudPtr lidarToWorld(const CloudPtr cloud) { return outputCloud(1, cloud); }

    const vmp_result& last_result() const { return res_; }
    vmp_stream_t handle() const { return s_; }

    KFView kf;
    LIOStatus status = IMU_INIT;
    std::shared_ptr<VoxelMapView> map;

private:
    template <class CloudPtr>
    CloudPtr outputCloud(int frame, const CloudPtr& cloud) {
        int n = 0;
        check(s_, vmp_output_cloud(s_, frame, nullptr, nullptr, 0, &n), "vmp_output_cloud");
        if (!cloud || static_cast<int>(cloud->points.size()) != n)
            throw std::invalid_argument("lidarToBody / lidarToWorld: not the cloud of the last processed package");
        cloud_.resize(static_cast<size_t>(n));
        inten_.resize(static_cast<size_t>(n));
        if (n > 0) check(s_, vmp_output_cloud(s_, frame, cloud_.data(), inten_.data(), n, &n), "vmp_output_cloud");
        CloudPtr out(new typename CloudPtr::element_type(*cloud));
        for (int i = 0; i < n; ++i) {
            out->points[i].x = cloud_[i].x;
            out->points[i].y = cloud_[i].y;
            out->points[i].z = cloud_[i].z;
        }
        return out;
    }

    vmp_stream_t s_ = nullptr;
    std::vector<vmp_point> cloud_;
    std::vector<float> inten_;
    vmp_result res_{};
    std::vector<vmp_point> pts_;
    std::vector<vmp_imu> imus_;
};

}  // namespace vmp_adapter
