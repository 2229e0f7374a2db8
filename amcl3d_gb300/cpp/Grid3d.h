/*
 * Drop-in amcl3d::Grid3d backed by the GB300 library (include/amcl3d_gpu.h).
 *
 * Same public interface as amcl3d/src/Grid3d.h:34-117, so amcl3d::Node
 * (Node.cpp:41,45,53) and ParticleFilter compile against it unchanged.  The grid
 * lives on the GPU; open() loads the octomap with the octomap library, builds the
 * distance field on the device (or loads the .grid cache) exactly as
 * Grid3d::open does (Grid3d.cpp:25-78).
 */
#pragma once

#include <geometry_msgs/PoseArray.h>
#include <nav_msgs/OccupancyGrid.h>
#include <octomap/OcTree.h>
#include <pcl/point_cloud.h>
#include <pcl/point_types.h>
#include <sensor_msgs/PointCloud2.h>
#include <tf/tf.h>

#include <memory>
#include <string>
#include <vector>

#include "amcl3d_gpu.h"

namespace amcl3d
{
class Grid3d
{
public:
  explicit Grid3d();
  virtual ~Grid3d();

  /* Grid3d::open (Grid3d.cpp:25-78): octomap -> occupied leaf centres -> .grid cache
   * or the GPU distance field (saved to the cache). */
  bool open(const std::string& map_path, const double sensor_dev);

  /* computeGrid under the name buildGridMap: builds the field from already extracted
   * occupied points and the octomap bounds. */
  bool buildGridMap(const pcl::PointCloud<pcl::PointXYZ>::Ptr& points, const double min[3], const double max[3],
                    const double resolution, const double sensor_dev);

  bool buildGridSliceMsg(const double z, nav_msgs::OccupancyGrid& msg) const;
  bool buildMapPointCloudMsg(sensor_msgs::PointCloud2& msg) const;
  float computeCloudWeight(const pcl::PointCloud<pcl::PointXYZ>::Ptr& cloud, const float tx, const float ty,
                           const float tz, const float roll, const float pitch, const float yaw) const;
  bool isIntoMap(const float x, const float y, const float z) const;

  /* The device grid used by amcl3d::ParticleFilter::update. */
  amcl_grid_t handle() const
  {
    return grid_;
  }

private:
  bool saveGrid(const std::string& grid_path);
  bool loadGrid(const std::string& grid_path, const double sensor_dev);

  amcl_grid_t grid_{ nullptr };
  bool built_{ false };
  double min_[3]{ 0, 0, 0 };
  double max_[3]{ 0, 0, 0 };
  double resol_{ 0 };
  pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_; /* map points, for buildMapPointCloudMsg */
};

}  // namespace amcl3d
