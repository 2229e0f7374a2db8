/*
 * Drop-in for the scan filter amcl3d::Node applies to every accepted scan
 * (Node.cpp:130-137: pcl::VoxelGrid<pcl::PointXYZ> sor; sor.setInputCloud(cloud_src);
 * sor.setLeafSize(v, v, v); sor.filter(*cloud_down)), run on the GPU by the
 * amcl_voxel_* calls of include/amcl3d_gpu.h.  Replacing the type of `sor` with
 * amcl3d::VoxelGrid is the only change the node needs; the three calls keep their
 * meaning: one centroid per occupied leaf, in leaf-key order, non-finite points
 * skipped, the input returned unchanged when the leaf count overflows int32.
 */
#pragma once

#include <pcl/point_cloud.h>
#include <pcl/point_types.h>

#include "amcl3d_gpu.h"

namespace amcl3d
{
class VoxelGrid
{
public:
  VoxelGrid();
  virtual ~VoxelGrid();
  VoxelGrid(const VoxelGrid&) = delete;
  VoxelGrid& operator=(const VoxelGrid&) = delete;

  void setInputCloud(const pcl::PointCloud<pcl::PointXYZ>::Ptr& cloud);
  void setLeafSize(const float lx, const float ly, const float lz);
  /* Writes the filtered cloud into `output` (its header is the input's, as PCL's
   * Filter::filter sets it); on a GPU error `output` is left empty and the error logged. */
  void filter(pcl::PointCloud<pcl::PointXYZ>& output);

  amcl_voxel_t handle() const
  {
    return voxel_;
  }

private:
  amcl_voxel_t voxel_{ nullptr };
  pcl::PointCloud<pcl::PointXYZ>::Ptr input_;
  float leaf_[3]{ 0.f, 0.f, 0.f };
};
}  // namespace amcl3d
