// Test-only stand-in for sensor_msgs::PointCloud2 (xyz float32 fields only).
#pragma once
#include <stdint.h>
#include <vector>
#include "../std_msgs_header.h"
namespace sensor_msgs
{
struct PointCloud2
{
  std_msgs::Header header;
  uint32_t height{ 0 };
  uint32_t width{ 0 };
  uint32_t point_step{ 0 };
  uint32_t row_step{ 0 };
  std::vector<uint8_t> data;
  bool is_dense{ false };
};
}  // namespace sensor_msgs
