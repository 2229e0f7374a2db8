// Test-only stand-in for geometry_msgs::PoseWithCovarianceStamped.
#pragma once
#include "PoseArray.h"
namespace geometry_msgs
{
struct PoseWithCovariance
{
  Pose pose;
  double covariance[36]{};
};
struct PoseWithCovarianceStamped
{
  std_msgs::Header header;
  PoseWithCovariance pose;
};
}  // namespace geometry_msgs
