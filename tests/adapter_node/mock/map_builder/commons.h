// TEST MOCK of the types the node takes from voxel_plus' commons.h:
// lio::IMUData and lio::SyncPackage (commons.h:13-28).
#pragma once
#include <vector>
#include <Eigen/Eigen>
#include <pcl/point_cloud.h>
#include <pcl/point_types.h>
namespace lio {
struct IMUData {
    Eigen::Vector3d acc;
    Eigen::Vector3d gyro;
    double timestamp = 0.0;
};
struct SyncPackage {
    std::vector<lio::IMUData> imus;
    pcl::PointCloud<pcl::PointXYZINormal>::Ptr cloud;
    double cloud_start_time = 0.0;
    double cloud_end_time = 0.0;
};
}  // namespace lio
