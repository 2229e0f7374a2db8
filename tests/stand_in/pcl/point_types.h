// Test-only stand-in for pcl::PointXYZ: 16-byte aligned x, y, z plus padding,
// the same layout PCL uses.
#pragma once
namespace pcl
{
struct alignas(16) PointXYZ
{
  float x{ 0 }, y{ 0 }, z{ 0 };
  float pad_{ 1.0f };
  PointXYZ() {}
  PointXYZ(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
};
}  // namespace pcl
