// Test-only stand-in for pcl::KdTreeFLANN<PointXYZ>: an exact 1-nearest-neighbour
// search over a uniform bucket grid.  PCL's KdTreeFLANN runs FLANN's exact
// single kd-tree search with the L2_Simple metric, whose squared distance is
// accumulated in float as ((0 + dx*dx) + dy*dy) + dz*dz; this stand-in returns
// the minimum of that same float expression over all points, so the squared
// distance it reports is the one FLANN reports (ties between equidistant points
// are irrelevant because only the distance is used).
#pragma once
#include <algorithm>
#include <cmath>
#include <limits>
#include <stdint.h>
#include <vector>
#include <pcl/point_cloud.h>
#include <pcl/point_types.h>

namespace pcl
{
template <typename PointT>
class KdTreeFLANN
{
public:
  typedef typename PointCloud<PointT>::ConstPtr PointCloudConstPtr;

  void setInputCloud(const PointCloudConstPtr& cloud)
  {
    cloud_ = cloud;
    build();
  }

  int nearestKSearch(const PointT& q, int k, std::vector<int>& idx, std::vector<float>& sqd) const
  {
    if (k < 1 || !cloud_ || cloud_->empty())
      return 0;
    int best_i = -1;
    float best = std::numeric_limits<float>::infinity();
    const double qc[3] = { q.x, q.y, q.z };
    int c[3];
    for (int a = 0; a < 3; ++a)
    {
      long v = static_cast<long>(std::floor((qc[a] - lo_[a]) / h_));
      c[a] = static_cast<int>(std::min<long>(std::max<long>(v, 0), n_[a] - 1));
    }
    const int rmax = std::max(n_[0], std::max(n_[1], n_[2]));
    for (int r = 0; r <= rmax; ++r)
    {
      for (int bz = c[2] - r; bz <= c[2] + r; ++bz)
        for (int by = c[1] - r; by <= c[1] + r; ++by)
          for (int bx = c[0] - r; bx <= c[0] + r; ++bx)
          {
            if (std::max(std::abs(bx - c[0]), std::max(std::abs(by - c[1]), std::abs(bz - c[2]))) != r)
              continue;
            if (bx < 0 || by < 0 || bz < 0 || bx >= n_[0] || by >= n_[1] || bz >= n_[2])
              continue;
            const size_t b = (static_cast<size_t>(bz) * n_[1] + by) * n_[0] + bx;
            for (uint32_t j = start_[b]; j < start_[b + 1]; ++j)
            {
              const PointT& p = cloud_->points[order_[j]];
              float d = 0;
              float t = q.x - p.x;
              d += t * t;
              t = q.y - p.y;
              d += t * t;
              t = q.z - p.z;
              d += t * t;
              if (d < best || (d == best && static_cast<int>(order_[j]) < best_i))
              {
                best = d;
                best_i = static_cast<int>(order_[j]);
              }
            }
          }
      // Lower bound on the distance from q to any bucket outside the scanned cube.
      double bound = std::numeric_limits<double>::infinity();
      for (int a = 0; a < 3; ++a)
      {
        if (c[a] - r > 0)
          bound = std::min(bound, std::max(0.0, qc[a] - (lo_[a] + (c[a] - r) * h_)));
        if (c[a] + r < n_[a] - 1)
          bound = std::min(bound, std::max(0.0, (lo_[a] + (c[a] + r + 1) * h_) - qc[a]));
      }
      if (bound == std::numeric_limits<double>::infinity())
        break;
      if (best_i >= 0 && static_cast<double>(best) < bound * bound * (1.0 - 1e-6))
        break;
    }
    idx.assign(1, best_i);
    sqd.assign(1, best);
    return 1;
  }

private:
  void build()
  {
    const auto& pts = cloud_->points;
    const size_t n = pts.size();
    double hi[3];
    for (int a = 0; a < 3; ++a)
    {
      lo_[a] = std::numeric_limits<double>::infinity();
      hi[a] = -std::numeric_limits<double>::infinity();
    }
    for (size_t i = 0; i < n; ++i)
    {
      const float v[3] = { pts[i].x, pts[i].y, pts[i].z };
      for (int a = 0; a < 3; ++a)
      {
        lo_[a] = std::min(lo_[a], static_cast<double>(v[a]));
        hi[a] = std::max(hi[a], static_cast<double>(v[a]));
      }
    }
    if (n == 0)
      return;
    double vol = 1.0;
    for (int a = 0; a < 3; ++a)
      vol *= std::max(hi[a] - lo_[a], 1e-3);
    h_ = std::max(std::cbrt(vol / static_cast<double>(n)) * 2.0, 1e-3);
    size_t total = 1;
    for (int a = 0; a < 3; ++a)
    {
      n_[a] = static_cast<int>(std::floor((hi[a] - lo_[a]) / h_)) + 1;
      total *= static_cast<size_t>(n_[a]);
    }
    std::vector<uint32_t> cell(n);
    start_.assign(total + 1, 0);
    for (size_t i = 0; i < n; ++i)
    {
      const float v[3] = { pts[i].x, pts[i].y, pts[i].z };
      int c[3];
      for (int a = 0; a < 3; ++a)
        c[a] = std::min(n_[a] - 1, static_cast<int>(std::floor((v[a] - lo_[a]) / h_)));
      cell[i] = static_cast<uint32_t>((static_cast<size_t>(c[2]) * n_[1] + c[1]) * n_[0] + c[0]);
      start_[cell[i] + 1]++;
    }
    for (size_t b = 0; b < total; ++b)
      start_[b + 1] += start_[b];
    order_.resize(n);
    std::vector<uint32_t> fill(start_.begin(), start_.end() - 1);
    for (size_t i = 0; i < n; ++i)
      order_[fill[cell[i]]++] = static_cast<uint32_t>(i);
  }

  PointCloudConstPtr cloud_;
  double lo_[3]{ 0, 0, 0 };
  double h_{ 1.0 };
  int n_[3]{ 1, 1, 1 };
  std::vector<uint32_t> start_;
  std::vector<uint32_t> order_;
};
}  // namespace pcl
