// Test-only stand-in: the filter core's pcl::toROSMsg plus the fromROSMsg the node
// calls on an incoming scan (declaration-level: the node check only compiles).
#pragma once
#include "../../stand_in/pcl_conversions/pcl_conversions.h"

namespace pcl
{
template <typename PointT>
void fromROSMsg(const sensor_msgs::PointCloud2& msg, PointCloud<PointT>& cloud)
{
  cloud.points.resize(msg.point_step ? msg.data.size() / msg.point_step : 0);
  cloud.width = static_cast<uint32_t>(cloud.points.size());
  cloud.height = 1;
}
}  // namespace pcl
