// Test-only stand-in for <sensor_msgs/point_cloud2_iterator.h> (the node includes it
// but uses nothing from it).
#pragma once
#include <sensor_msgs/PointCloud2.h>
