// Test-only stand-in for pcl::toROSMsg (packs x, y, z, pad as 16-byte points).
#pragma once
#include <cstring>
#include <pcl/point_cloud.h>
#include <pcl/point_types.h>
#include <sensor_msgs/PointCloud2.h>
namespace pcl
{
template <typename PointT>
void toROSMsg(const PointCloud<PointT>& cloud, sensor_msgs::PointCloud2& msg)
{
  msg.height = 1;
  msg.width = static_cast<uint32_t>(cloud.size());
  msg.point_step = sizeof(PointT);
  msg.row_step = msg.point_step * msg.width;
  msg.data.resize(msg.row_step);
  if (!cloud.empty())
    std::memcpy(msg.data.data(), &cloud.points[0], msg.data.size());
  msg.is_dense = true;
}
}  // namespace pcl
