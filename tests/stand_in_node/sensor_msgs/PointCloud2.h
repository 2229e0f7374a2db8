// Test-only stand-in: the filter core's sensor_msgs::PointCloud2 plus the pointer
// type the node's subscriber callback takes.
#pragma once
#include "../../stand_in/sensor_msgs/PointCloud2.h"

#include <boost/shared_ptr.hpp>

namespace sensor_msgs
{
typedef boost::shared_ptr<const PointCloud2> PointCloud2ConstPtr;
}
