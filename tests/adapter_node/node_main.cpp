// TEST PROGRAM: a LIONode-like driver of the GPU adapter.  It includes the
// drop-in "map_builder/lio_builder.h" (include/vmp_node) as lio_node.cpp does
// and makes the node's calls on lio::LIOBuilder with the node's types and
// expressions:
//   map_builder.loadConfig(lio_config)                    lio_node.cpp:44
//   map_builder.process(sync_pack)                        lio_node.cpp:171
//   map_builder.status != lio::LIOStatus::LIO_MAPPING     lio_node.cpp:172
//   state = map_builder.kf.x()                            lio_node.cpp:174
//   map_builder.lidarToBody / lidarToWorld(sync_pack.cloud)   lio_node.cpp:176-178
//   std::shared_ptr<lio::VoxelMap> voxel_map = map_builder.map;
//   voxel_map->cache.size(), voxel_map->voxel_size        lio_node.cpp:185-190
//   Eigen::Map<Matrix<double, 6, 6, RowMajor>>(...) = map_builder.kf.P().block<6, 6>(0, 0)
//                                                         lio_node.cpp:227
// and the map walk of voxel2MarkerArray (utils.cpp:154-208): cache order,
// featmap[k], is_plane / update_enable, center, the trace of
// plane->cov.block<3, 3>(0, 0), merged, plane->norm.
//
// usage: node_main packages.bin results.bin
//   packages.bin: int32 count; per package int32 n, int32 n_imu, f64 t_start,
//     f64 t_end, n x (f32 x, y, z, t_ms), n_imu x (f64 t, acc[3], gyro[3]).
//   results.bin: per package int32 status; in LIO_MAPPING also f64 pos[3],
//     rot[9], the 6x6 pose covariance (row-major), the body and world clouds
//     (int32 n, n x f32 xyz each) and the plane markers (int32 n, n x (f64
//     center[3], f64 trace, f64 norm[3], int32 merged)).
// Exit status 3 (and "nogpu" on stdout) when no GPU can be used.
#include "map_builder/lio_builder.h"

#include <array>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

namespace {

struct Marker {
    double center[3];
    double trace;
    double norm[3];
    int merged;
};

// voxel2MarkerArray's walk over the map (utils.cpp:154-208), the markers'
// data without the ROS message.
std::vector<Marker> voxelMarkers(std::shared_ptr<lio::VoxelMap> map, int max_capacity) {
    std::vector<Marker> out;
    int size = std::min(static_cast<int>(map->cache.size()), max_capacity);
    int count = 0;
    for (auto& k : map->cache) {
        if (count >= size) break;
        std::shared_ptr<lio::VoxelGrid> grid = map->featmap[k];
        if (!grid->is_plane || grid->update_enable) continue;
        Eigen::Vector3d grid_center = grid->center;
        double trace = grid->plane->cov.block<3, 3>(0, 0).trace();
        Marker m;
        for (int i = 0; i < 3; ++i) { m.center[i] = grid_center(i); m.norm[i] = grid->plane->norm(i); }
        m.trace = trace;
        m.merged = grid->merged ? 1 : 0;
        out.push_back(m);
        ++count;
    }
    return out;
}

struct Node {
    lio::LIOConfig lio_config;
    lio::LIOBuilder map_builder;
    lio::SyncPackage sync_pack;
    kf::State state;
    FILE* out = nullptr;

    void write_cloud(const pcl::PointCloud<pcl::PointXYZINormal>::Ptr& c) {
        const int n = static_cast<int>(c->points.size());
        std::fwrite(&n, 4, 1, out);
        for (const auto& p : c->points) {
            const float v[3] = {p.x, p.y, p.z};
            std::fwrite(v, 4, 3, out);
        }
    }

    void mainCB() {
        map_builder.process(sync_pack);
        const int status = static_cast<int>(map_builder.status);
        std::fwrite(&status, 4, 1, out);
        if (map_builder.status != lio::LIOStatus::LIO_MAPPING) return;
        state = map_builder.kf.x();
        double pose[12];
        for (int i = 0; i < 3; ++i) pose[i] = state.pos(i);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) pose[3 + i * 3 + j] = state.rot(i, j);
        std::fwrite(pose, 8, 12, out);
        Eigen::Quaterniond q(state.rot);
        (void)q.w();
        std::array<double, 36> covariance;  // geometry_msgs::PoseWithCovariance::covariance
        Eigen::Map<Eigen::Matrix<double, 6, 6, Eigen::RowMajor>>(covariance.data()) = map_builder.kf.P().block<6, 6>(0, 0);
        std::fwrite(covariance.data(), 8, 36, out);
        pcl::PointCloud<pcl::PointXYZINormal>::Ptr body_cloud = map_builder.lidarToBody(sync_pack.cloud);
        write_cloud(body_cloud);
        pcl::PointCloud<pcl::PointXYZINormal>::Ptr world_cloud = map_builder.lidarToWorld(sync_pack.cloud);
        write_cloud(world_cloud);
        voxelTimerCB();
    }

    void voxelTimerCB() {
        std::shared_ptr<lio::VoxelMap> voxel_map = map_builder.map;
        std::vector<Marker> markers;
        if (voxel_map->cache.size() >= 10) markers = voxelMarkers(voxel_map, 1000000);
        const int n = static_cast<int>(markers.size());
        std::fwrite(&n, 4, 1, out);
        for (const Marker& m : markers) {
            std::fwrite(m.center, 8, 3, out);
            std::fwrite(&m.trace, 8, 1, out);
            std::fwrite(m.norm, 8, 3, out);
            std::fwrite(&m.merged, 4, 1, out);
        }
        (void)(voxel_map->voxel_size * 0.8);
    }
};

bool read_package(FILE* f, lio::SyncPackage& p) {
    int n = 0, n_imu = 0;
    double t[2];
    if (std::fread(&n, 4, 1, f) != 1 || std::fread(&n_imu, 4, 1, f) != 1 || std::fread(t, 8, 2, f) != 2) return false;
    p.cloud_start_time = t[0];
    p.cloud_end_time = t[1];
    p.cloud = std::make_shared<pcl::PointCloud<pcl::PointXYZINormal>>();
    p.cloud->points.resize(static_cast<size_t>(n));
    std::vector<float> buf(4 * static_cast<size_t>(n));
    if (n > 0 && std::fread(buf.data(), 4, buf.size(), f) != buf.size()) return false;
    for (int i = 0; i < n; ++i) {
        auto& q = p.cloud->points[i];
        q.x = buf[4 * i]; q.y = buf[4 * i + 1]; q.z = buf[4 * i + 2]; q.curvature = buf[4 * i + 3];
        q.intensity = static_cast<float>(i % 256);
    }
    p.cloud->width = static_cast<uint32_t>(n);
    p.imus.resize(static_cast<size_t>(n_imu));
    for (int i = 0; i < n_imu; ++i) {
        double r[7];
        if (std::fread(r, 8, 7, f) != 7) return false;
        p.imus[i].timestamp = r[0];
        p.imus[i].acc = Eigen::Vector3d(r[1], r[2], r[3]);
        p.imus[i].gyro = Eigen::Vector3d(r[4], r[5], r[6]);
    }
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    Node node;
    node.lio_config.scan_resolution = 0.2;
    try {
        node.map_builder.loadConfig(node.lio_config);
    } catch (const std::exception& e) {
        std::printf("nogpu %s\n", e.what());
        return 3;
    }
    FILE* in = std::fopen(argv[1], "rb");
    node.out = std::fopen(argv[2], "wb");
    if (!in || !node.out) return 2;
    int count = 0;
    if (std::fread(&count, 4, 1, in) != 1) return 2;
    for (int k = 0; k < count; ++k) {
        if (!read_package(in, node.sync_pack)) return 2;
        node.mainCB();
    }
    std::fclose(in);
    std::fclose(node.out);
    std::printf("ok %d\n", count);
    return 0;
}
