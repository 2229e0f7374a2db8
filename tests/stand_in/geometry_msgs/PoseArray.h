// Test-only stand-in for geometry_msgs::PoseArray (plain structs, no serialisation).
#pragma once
#include <vector>
#include "../std_msgs_header.h"
namespace geometry_msgs
{
struct Point
{
  double x{ 0 }, y{ 0 }, z{ 0 };
};
struct Quaternion
{
  double x{ 0 }, y{ 0 }, z{ 0 }, w{ 0 };
};
struct Pose
{
  Point position;
  Quaternion orientation;
};
struct PoseArray
{
  std_msgs::Header header;
  std::vector<Pose> poses;
};
}  // namespace geometry_msgs
