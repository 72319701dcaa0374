// TEST MOCK: pcl::PointCloud<T> with its header, points, width, height,
// is_dense and the shared_ptr alias Ptr.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>
namespace pcl {
struct PCLHeader {
    uint64_t stamp = 0;
    std::string frame_id;
};
template <class T>
struct PointCloud {
    typedef std::shared_ptr<PointCloud<T>> Ptr;
    PCLHeader header;
    std::vector<T> points;
    uint32_t width = 0, height = 1;
    bool is_dense = true;
    size_t size() const { return points.size(); }
};
}  // namespace pcl
