// TEST MOCK: pcl::PointXYZINormal's fields (x, y, z, intensity, normal,
// curvature), enough for the GPU adapter and the node-like test program.
#pragma once
namespace pcl {
struct PointXYZINormal {
    float x = 0.f, y = 0.f, z = 0.f;
    float intensity = 0.f;
    float normal_x = 0.f, normal_y = 0.f, normal_z = 0.f;
    float curvature = 0.f;
};
}  // namespace pcl
