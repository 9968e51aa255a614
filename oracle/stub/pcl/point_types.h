// Minimal stand-in for <pcl/point_types.h> and Eigen::aligned_allocator, used
// only to compile the unmodified ikd-Tree reference (ikd-Tree/ikd_Tree.h:11,
// :62 and ikd-Tree/ikd_Tree.cpp:1446-1449) inside the oracle build.  PCL and
// Eigen are not installed on this machine.  Test infrastructure only.
#pragma once
#include <memory>

namespace Eigen {
template <class T>
using aligned_allocator = std::allocator<T>;
}

namespace pcl {
struct PointXYZ {
    float x = 0.f, y = 0.f, z = 0.f, pad_ = 1.f;
};
struct PointXYZI {
    float x = 0.f, y = 0.f, z = 0.f, pad_ = 1.f;
    float intensity = 0.f, pad2_[3] = {0.f, 0.f, 0.f};
};
struct PointXYZINormal {
    float x = 0.f, y = 0.f, z = 0.f, pad_ = 1.f;
    float normal_x = 0.f, normal_y = 0.f, normal_z = 0.f, pad3_ = 0.f;
    float intensity = 0.f, curvature = 0.f, pad2_[2] = {0.f, 0.f};
};
}  // namespace pcl
