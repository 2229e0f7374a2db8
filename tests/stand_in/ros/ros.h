// Test-only stand-in for <ros/ros.h>: just what the amcl3d filter core uses
// (log macros, node name, wall-clock time).  Logging goes to stderr only when
// AMCL_SHIM_VERBOSE is set in the environment.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include <stdint.h>

namespace ros
{
struct Time
{
  uint32_t sec{ 0 }, nsec{ 0 };
  static Time now() { return Time(); }
  static void init() {}
};
namespace this_node
{
inline std::string getName() { return "amcl3d_oracle"; }
}  // namespace this_node
inline bool shim_verbose()
{
  static int v = std::getenv("AMCL_SHIM_VERBOSE") ? 1 : 0;
  return v != 0;
}
}  // namespace ros

#define AMCL_SHIM_LOG(...)                 \
  do                                       \
  {                                        \
    if (ros::shim_verbose())               \
    {                                      \
      std::fprintf(stderr, __VA_ARGS__);   \
      std::fprintf(stderr, "\n");          \
    }                                      \
  } while (0)
#define ROS_INFO(...) AMCL_SHIM_LOG(__VA_ARGS__)
#define ROS_WARN(...) AMCL_SHIM_LOG(__VA_ARGS__)
#define ROS_ERROR(...) AMCL_SHIM_LOG(__VA_ARGS__)
#define ROS_DEBUG(...) AMCL_SHIM_LOG(__VA_ARGS__)
