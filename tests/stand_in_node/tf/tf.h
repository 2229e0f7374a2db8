// Test-only stand-in: the filter core's <tf/tf.h> (math include set) plus the tf
// transform types amcl3d::Node uses (declarations enough for a syntax-only compile).
#pragma once
#include "../../stand_in/tf/tf.h"

#include <ros/ros.h>
#include <string>

namespace tf
{
class Vector3
{
public:
  Vector3() = default;
  Vector3(double x, double y, double z) : v_{ x, y, z } {}
  double getX() const { return v_[0]; }
  double getY() const { return v_[1]; }
  double getZ() const { return v_[2]; }
  double x() const { return v_[0]; }
  double y() const { return v_[1]; }
  double z() const { return v_[2]; }
  double length() const { return 0.0; }

private:
  double v_[3]{};
};
class Quaternion
{
public:
  Quaternion() = default;
  Quaternion(double x, double y, double z, double w) : q_{ x, y, z, w } {}
  void setRPY(double, double, double) {}
  double getX() const { return q_[0]; }
  double getY() const { return q_[1]; }
  double getZ() const { return q_[2]; }
  double getW() const { return q_[3]; }

private:
  double q_[4]{ 0, 0, 0, 1 };
};
class Matrix3x3
{
public:
  void getRPY(double& r, double& p, double& y) const { r = p = y = 0.0; }
};
class Transform
{
public:
  void setOrigin(const Vector3& o) { o_ = o; }
  void setRotation(const Quaternion& q) { q_ = q; }
  const Vector3& getOrigin() const { return o_; }
  Quaternion getRotation() const { return q_; }
  const Matrix3x3& getBasis() const { return b_; }
  Transform inverse() const { return *this; }
  Transform operator*(const Transform&) const { return *this; }

private:
  Vector3 o_;
  Quaternion q_;
  Matrix3x3 b_;
};
class StampedTransform : public Transform
{
public:
  StampedTransform(const Transform& t, const ros::Time&, const std::string&, const std::string&) : Transform(t) {}
};
}  // namespace tf
