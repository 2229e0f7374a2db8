/*
 * Drop-in amcl3d::Grid3d over the GB300 library.  Error behaviour follows the
 * reference: failures are logged with ROS_ERROR / ROS_WARN and reported through
 * the bool results (Grid3d.cpp:27-48,62-70); nothing throws across the API.
 */
#include "Grid3d.h"

#include <pcl_conversions/pcl_conversions.h>

#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <sys/stat.h>

namespace amcl3d
{
namespace
{
bool ends_with(const std::string& s, const char* suf)
{
  const std::string t(suf);
  return s.size() >= t.size() && s.compare(s.size() - t.size(), t.size(), t) == 0;
}

bool file_exists(const std::string& p)
{
  struct stat st;
  return ::stat(p.c_str(), &st) == 0;
}

/* openOcTree + computePointCloud (PointCloudTools.cpp:26-82), through the octomap API. */
bool read_octomap(const std::string& path, pcl::PointCloud<pcl::PointXYZ>::Ptr& cloud, double mn[3], double mx[3],
                  double* res, std::string* err)
{
  if (!file_exists(path))
  {
    *err = "Cannot find file " + path;
    return false;
  }
  std::shared_ptr<octomap::OcTree> tree;
  if (ends_with(path, ".bt"))
  {
    tree.reset(new octomap::OcTree(0.1));
    if (!tree->readBinary(path))
    {
      *err = "OcTree cannot be read";
      return false;
    }
  }
  else if (ends_with(path, ".ot"))
    tree.reset(dynamic_cast<octomap::OcTree*>(octomap::AbstractOcTree::read(path)));
  if (!tree)
  {
    *err = "OcTree cannot be created from file " + path;
    return false;
  }
  if (tree->size() <= 1)
  {
    *err = "OcTree is empty";
    return false;
  }
  tree->getMetricMin(mn[0], mn[1], mn[2]);
  tree->getMetricMax(mx[0], mx[1], mx[2]);
  *res = tree->getResolution();
  cloud.reset(new pcl::PointCloud<pcl::PointXYZ>());
  for (auto it = tree->begin_leafs(); it != tree->end_leafs(); ++it)
    if (tree->isNodeOccupied(*it))
      cloud->push_back(pcl::PointXYZ(static_cast<float>(it.getX()), static_cast<float>(it.getY()),
                                     static_cast<float>(it.getZ())));
  return true;
}
}  // namespace

Grid3d::Grid3d()
{
  if (amcl_grid_create(&grid_, nullptr) != AMCL_OK)
    ROS_ERROR("[%s] amcl_grid_create: %s", ros::this_node::getName().data(), amcl_last_error());
}

Grid3d::~Grid3d()
{
  amcl_grid_destroy(grid_);
}

bool Grid3d::open(const std::string& map_path, const double sensor_dev)
{
  std::string err;
  pcl::PointCloud<pcl::PointXYZ>::Ptr cloud;
  double mn[3], mx[3], res = 0;
  if (!read_octomap(map_path, cloud, mn, mx, &res, &err))
  {
    ROS_ERROR("[%s] %s", ros::this_node::getName().data(), err.c_str());
    return false;
  }
  ROS_INFO("[%s] Octomap loaded", ros::this_node::getName().data());
  cloud_ = cloud;
  for (int a = 0; a < 3; ++a)
  {
    min_[a] = mn[a];
    max_[a] = mx[a];
  }
  resol_ = res;

  /* The .grid cache next to the map (Grid3d.cpp:50-58). */
  std::string grid_path;
  if (ends_with(map_path, ".bt"))
    grid_path = map_path.substr(0, map_path.find(".bt")) + ".grid";
  if (ends_with(map_path, ".ot"))
    grid_path = map_path.substr(0, map_path.find(".ot")) + ".grid";
  if (loadGrid(grid_path, sensor_dev))
    return true;

  ROS_INFO("[%s] Computing 3D occupancy grid on the GPU", ros::this_node::getName().data());
  if (!buildGridMap(cloud, mn, mx, res, sensor_dev))
    return false;
  saveGrid(grid_path);
  return true;
}

bool Grid3d::buildGridMap(const pcl::PointCloud<pcl::PointXYZ>::Ptr& points, const double min[3],
                          const double max[3], const double resolution, const double sensor_dev)
{
  const float* xyz = (points && !points->empty()) ? &points->points[0].x : nullptr;
  const uint64_t n = points ? points->size() : 0;
  const int rc = amcl_grid_build(grid_, xyz, n, sizeof(pcl::PointXYZ) / sizeof(float), min, max, resolution,
                                 sensor_dev);
  if (rc != AMCL_OK)
  {
    ROS_ERROR("[%s] %s", ros::this_node::getName().data(), amcl_last_error());
    built_ = false;
    return false;
  }
  if (points != cloud_)
    cloud_ = points;
  for (int a = 0; a < 3; ++a)
  {
    min_[a] = min[a];
    max_[a] = max[a];
  }
  resol_ = resolution;
  built_ = true;
  return true;
}

bool Grid3d::saveGrid(const std::string& grid_path)
{
  if (!built_)
    return false;
  if (amcl_grid_save(grid_, grid_path.c_str()) != AMCL_OK)
  {
    ROS_ERROR("[%s] Error opening file %s for writing", ros::this_node::getName().data(), grid_path.c_str());
    return false;
  }
  ROS_INFO("[%s] Grid map successfully saved on %s", ros::this_node::getName().data(), grid_path.c_str());
  return true;
}

bool Grid3d::loadGrid(const std::string& grid_path, const double sensor_dev)
{
  if (amcl_grid_load(grid_, grid_path.c_str(), min_, max_, resol_, sensor_dev) != AMCL_OK)
  {
    ROS_WARN("[%s] %s", ros::this_node::getName().data(), amcl_last_error());
    return false;
  }
  built_ = true;
  ROS_INFO("[%s] Grid map successfully loaded from %s", ros::this_node::getName().data(), grid_path.c_str());
  return true;
}

bool Grid3d::buildGridSliceMsg(const double z, nav_msgs::OccupancyGrid& msg) const
{
  if (!built_ || !cloud_)
    return false;
  uint64_t len = 0;
  uint32_t w = 0, h = 0;
  if (amcl_grid_slice(grid_, z, nullptr, 0, &len, &w, &h) != AMCL_OK)
    return false;
  msg.info.map_load_time = ros::Time::now();
  msg.info.resolution = resol_;
  msg.info.width = w;
  msg.info.height = h;
  msg.info.origin.position.x = 0.;
  msg.info.origin.position.y = 0.;
  msg.info.origin.position.z = z;
  msg.info.origin.orientation.x = 0.;
  msg.info.origin.orientation.y = 0.;
  msg.info.origin.orientation.z = 0.;
  msg.info.origin.orientation.w = 1.;
  msg.data.resize(len);
  if (len && amcl_grid_slice(grid_, z, msg.data.data(), len, &len, &w, &h) != AMCL_OK)
    return false;
  return true;
}

bool Grid3d::buildMapPointCloudMsg(sensor_msgs::PointCloud2& msg) const
{
  if (!cloud_)
    return false;
  pcl::toROSMsg(*cloud_, msg);
  return true;
}

float Grid3d::computeCloudWeight(const pcl::PointCloud<pcl::PointXYZ>::Ptr& cloud, const float tx, const float ty,
                                 const float tz, const float roll, const float pitch, const float yaw) const
{
  if (!built_ || !cloud)
    return 0;
  const float pose[4] = { tx, ty, tz, yaw };
  float out = 0;
  const float* xyz = cloud->empty() ? nullptr : &cloud->points[0].x;
  if (amcl_grid_cloud_weights(grid_, pose, 1, xyz, static_cast<uint32_t>(cloud->size()),
                              sizeof(pcl::PointXYZ) / sizeof(float), roll, pitch, &out) != AMCL_OK)
  {
    ROS_ERROR("[%s] %s", ros::this_node::getName().data(), amcl_last_error());
    return 0;
  }
  return out;
}

bool Grid3d::isIntoMap(const float x, const float y, const float z) const
{
  int inside = 0;
  if (!built_ || amcl_grid_is_into_map(grid_, x, y, z, &inside) != AMCL_OK)
    return false;
  return inside != 0;
}

}  // namespace amcl3d
