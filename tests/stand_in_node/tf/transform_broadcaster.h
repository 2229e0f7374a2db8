// Test-only stand-in for <tf/transform_broadcaster.h> (it brings in the transform
// message types, as the real header does).
#pragma once
#include <geometry_msgs/TransformStamped.h>
#include <tf/tf.h>

namespace tf
{
class TransformBroadcaster
{
public:
  void sendTransform(const StampedTransform&) {}
};
}  // namespace tf
