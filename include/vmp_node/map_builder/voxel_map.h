// Drop-in for voxel_plus/src/map_builder/voxel_map.h in a node build that runs
// the odometry step on the GPU: the map lives on the device, and lio::VoxelMap
// / lio::VoxelGrid / lio::VoxelKey name the read-side view of it
// (vmp_lio_builder.hpp) that the node's voxel-map timer (lio_node.cpp:183-191)
// and voxel2MarkerArray (utils.cpp:154-208) read: cache, featmap[k]->is_plane,
// update_enable, merged, center, plane->norm, plane->cov, voxel_size.
// Put include/vmp_node ahead of voxel_plus/src on the include path; the
// reference's voxel_map.cpp and lio_builder.cpp leave the target.
#pragma once
#include "vmp_lio_builder.hpp"

namespace lio {
using VoxelKey = vmp_adapter::VoxelKey;
using Plane = vmp_adapter::PlaneView;
using VoxelGrid = vmp_adapter::GridView;
using VoxelMap = vmp_adapter::VoxelMapView;
}  // namespace lio
