// Test-only stand-in for visualization_msgs::Marker.
#pragma once
#include <geometry_msgs/PoseArray.h>
#include <string>
#include <vector>

namespace visualization_msgs
{
struct Marker
{
  enum
  {
    ARROW = 0,
    LINE_STRIP = 4,
    ADD = 0
  };
  std_msgs::Header header;
  std::string ns;
  int32_t id{ 0 };
  int32_t type{ 0 };
  int32_t action{ 0 };
  geometry_msgs::Point scale;
  struct
  {
    float r{ 0 }, g{ 0 }, b{ 0 }, a{ 0 };
  } color;
  std::vector<geometry_msgs::Point> points;
};
}  // namespace visualization_msgs
