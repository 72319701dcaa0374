// TEST MOCK of the types the node takes from voxel_plus' ieskf.h: kf::State's
// members (ieskf.h:31-44) with Eigen types; nothing of the CPU filter.
#pragma once
#include <Eigen/Core>
namespace kf {
const double GRAVITY = 9.81;
using Matrix23d = Eigen::Matrix<double, 23, 23>;
struct State {
    Eigen::Vector3d pos = Eigen::Vector3d::Zero();
    Eigen::Matrix3d rot = Eigen::Matrix3d::Identity();
    Eigen::Matrix3d rot_ext = Eigen::Matrix3d::Identity();
    Eigen::Vector3d pos_ext = Eigen::Vector3d::Zero();
    Eigen::Vector3d vel = Eigen::Vector3d::Zero();
    Eigen::Vector3d bg = Eigen::Vector3d::Zero();
    Eigen::Vector3d ba = Eigen::Vector3d::Zero();
    Eigen::Vector3d g = Eigen::Vector3d(0.0, 0.0, -GRAVITY);
};
}  // namespace kf
