// Test-only stand-in for pcl::PointCloud<T>.
#pragma once
#include <stdint.h>
#include <vector>
#include <boost/shared_ptr.hpp>
#include "../std_msgs_header.h"
namespace pcl
{
template <typename PointT>
class PointCloud
{
public:
  typedef boost::shared_ptr<PointCloud<PointT> > Ptr;
  typedef boost::shared_ptr<const PointCloud<PointT> > ConstPtr;
  typedef typename std::vector<PointT>::iterator iterator;
  typedef typename std::vector<PointT>::const_iterator const_iterator;

  std_msgs::Header header;
  std::vector<PointT> points;
  uint32_t width{ 0 };
  uint32_t height{ 1 };
  bool is_dense{ true };

  void push_back(const PointT& p)
  {
    points.push_back(p);
    width = static_cast<uint32_t>(points.size());
  }
  size_t size() const { return points.size(); }
  bool empty() const { return points.empty(); }
  iterator begin() { return points.begin(); }
  iterator end() { return points.end(); }
  const_iterator begin() const { return points.begin(); }
  const_iterator end() const { return points.end(); }
  PointT& operator[](size_t i) { return points[i]; }
  const PointT& operator[](size_t i) const { return points[i]; }
};
}  // namespace pcl
