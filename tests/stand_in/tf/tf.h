// Test-only stand-in for <tf/tf.h>.  The real header chain (LinearMath/Scalar.h)
// includes <math.h>, which makes the float overloads of sin/cos/exp/sqrt visible
// unqualified inside namespace amcl3d; this stand-in keeps that include set so the
// filter core picks the same overloads as in a ROS build.
#pragma once
#include <math.h>
#include <cmath>
