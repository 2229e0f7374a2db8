// Test-only stand-in for pcl::VoxelGrid (declarations only: the node's call
// sequence setInputCloud / setLeafSize / filter).
#pragma once
#include <pcl/point_cloud.h>

namespace pcl
{
template <typename PointT>
class VoxelGrid
{
public:
  void setInputCloud(const typename PointCloud<PointT>::ConstPtr&) {}
  void setLeafSize(float, float, float) {}
  void filter(PointCloud<PointT>&) {}
};
}  // namespace pcl
