#include "VoxelGrid.h"

#include <ros/ros.h>

#include <vector>

namespace amcl3d
{
VoxelGrid::VoxelGrid()
{
  if (amcl_voxel_create(&voxel_, nullptr) != AMCL_OK)
  {
    ROS_ERROR("[%s] VoxelGrid: %s", ros::this_node::getName().data(), amcl_last_error());
    voxel_ = nullptr;
  }
}

VoxelGrid::~VoxelGrid()
{
  amcl_voxel_destroy(voxel_);
}

void VoxelGrid::setInputCloud(const pcl::PointCloud<pcl::PointXYZ>::Ptr& cloud)
{
  input_ = cloud;
}

void VoxelGrid::setLeafSize(const float lx, const float ly, const float lz)
{
  leaf_[0] = lx;
  leaf_[1] = ly;
  leaf_[2] = lz;
}

void VoxelGrid::filter(pcl::PointCloud<pcl::PointXYZ>& output)
{
  output.points.clear();
  output.width = 0;
  output.height = 1;
  if (!input_ || !voxel_)
    return;
  output.header = input_->header;
  const uint64_t n = input_->points.size();
  std::vector<float> out(static_cast<size_t>(n > 0 ? n : 1) * 4);
  uint64_t m = 0;
  const float* xyz = n ? &input_->points[0].x : nullptr;
  if (amcl_voxel_filter(voxel_, xyz, n, sizeof(pcl::PointXYZ) / sizeof(float), leaf_[0], leaf_[1], leaf_[2],
                        out.data(), n, &m) != AMCL_OK)
  {
    ROS_ERROR("[%s] VoxelGrid::filter: %s", ros::this_node::getName().data(), amcl_last_error());
    return;
  }
  output.points.resize(static_cast<size_t>(m));
  for (uint64_t i = 0; i < m; ++i)
  {
    output.points[i].x = out[4 * i + 0];
    output.points[i].y = out[4 * i + 1];
    output.points[i].z = out[4 * i + 2];
  }
  output.width = static_cast<uint32_t>(m);
  output.is_dense = true;
}
}  // namespace amcl3d
