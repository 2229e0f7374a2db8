// Test-only stand-in for geometry_msgs::TransformStamped.
#pragma once
#include <boost/shared_ptr.hpp>
#include <geometry_msgs/PoseArray.h>
#include <string>

namespace geometry_msgs
{
struct Vector3
{
  double x{ 0 }, y{ 0 }, z{ 0 };
};
struct Transform
{
  Vector3 translation;
  Quaternion rotation;
};
struct TransformStamped
{
  std_msgs::Header header;
  std::string child_frame_id;
  Transform transform;
};
typedef boost::shared_ptr<const TransformStamped> TransformStampedConstPtr;
}  // namespace geometry_msgs
