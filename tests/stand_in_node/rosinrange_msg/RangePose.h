// Test-only stand-in for rosinrange_msg::RangePose (the radio-range message).
#pragma once
#include <boost/shared_ptr.hpp>
#include <geometry_msgs/PoseArray.h>
#include <stdint.h>

namespace rosinrange_msg
{
struct RangePose
{
  std_msgs::Header header;
  uint32_t source_id{ 0 };
  uint32_t destination_id{ 0 };
  double range{ 0 };
  geometry_msgs::Point position;
};
typedef boost::shared_ptr<const RangePose> RangePoseConstPtr;
}  // namespace rosinrange_msg
