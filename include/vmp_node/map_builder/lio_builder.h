// Drop-in for voxel_plus/src/map_builder/lio_builder.h in a node build that
// runs the odometry step on the GPU through libvmp.so.  lio_node.cpp and
// utils.cpp compile unchanged against it:
//   lio::LIOConfig, lio::LIOStatus, lio::LIOBuilder (lio_builder.h:10-83)
// with loadConfig, process, status, kf.x(), kf.P(), map, lidarToBody,
// lidarToWorld as the node uses them (lio_node.cpp:44, 171-178, 185, 227).
// kf::State and lio::SyncPackage still come from the reference's ieskf.h and
// commons.h (their types only; nothing of the CPU filter runs).
// Put include/vmp_node ahead of voxel_plus/src on the include path, add
// include/ for vmp.h / vmp_lio_builder.hpp, drop voxel_map.cpp and
// lio_builder.cpp from the target and link libvmp.so.
#pragma once
#include "map_builder/ieskf.h"
#include "map_builder/commons.h"
#include "map_builder/voxel_map.h"
#include "vmp_lio_builder.hpp"

namespace lio {
using LIOStatus = vmp_adapter::LIOStatus;
using LIOConfig = vmp_adapter::LIOConfig;
using LIOBuilder = vmp_adapter::LIOBuilder;
}  // namespace lio
