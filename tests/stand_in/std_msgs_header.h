// Test-only stand-in for std_msgs::Header.
#pragma once
#include <stdint.h>
#include <string>
#include <ros/ros.h>
namespace std_msgs
{
struct Header
{
  uint32_t seq{ 0 };
  ros::Time stamp;
  std::string frame_id;
};
}  // namespace std_msgs
