// Test-only stand-in: the filter core's <ros/ros.h> plus the node-side API that
// amcl3d::Node uses (declarations enough for a syntax-only compile).
#pragma once
#include "../../stand_in/ros/ros.h"

#include <ctime>
#include <string>
#include <unistd.h>

namespace ros
{
struct Duration
{
  double s{ 0 };
  Duration() = default;
  explicit Duration(double sec) : s(sec) {}
};
struct Rate
{
  double hz{ 0 };
  explicit Rate(double h) : hz(h) {}
  operator Duration() const { return Duration(hz > 0 ? 1.0 / hz : 0.0); }
};
inline Time operator+(const Time& t, const Duration&) { return t; }
inline bool operator<(const Time& a, const Time& b) { return a.sec < b.sec || (a.sec == b.sec && a.nsec < b.nsec); }
struct TimerEvent
{
};
struct Timer
{
};
struct Subscriber
{
};
struct Publisher
{
  template <typename M>
  void publish(const M&) const
  {
  }
};
class NodeHandle
{
public:
  explicit NodeHandle(const std::string& = std::string()) {}
  template <typename M>
  Publisher advertise(const std::string&, uint32_t, bool = false)
  {
    return Publisher();
  }
  template <typename T>
  Timer createTimer(Duration, void (T::*)(const TimerEvent&), T*)
  {
    return Timer();
  }
  template <typename M, typename T>
  Subscriber subscribe(const std::string&, uint32_t, void (T::*)(const M&), T*)
  {
    return Subscriber();
  }
  void shutdown() {}
};
inline bool ok() { return false; }
inline void spinOnce() {}
namespace param
{
template <typename T>
bool get(const std::string&, T&)
{
  return false;
}
}  // namespace param
}  // namespace ros
