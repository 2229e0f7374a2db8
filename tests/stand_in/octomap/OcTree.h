// Test-only stand-in for octomap::OcTree.  The octomap library is not available,
// so "map files" for the oracle are a plain point list written by the test
// harness ("AMCLPTS1" format: magic, resolution, metric min/max, point count,
// float xyz triples).  Every stored point is one occupied leaf, which is what
// amcl3d's computePointCloud extracts from a real octree.  Like the real
// header chain (octomap_types.h -> math/Vector3.h) it brings in <math.h> and
// <stdexcept>.
#pragma once
#include <math.h>
#include <cmath>
#include <stdexcept>
#include <cstdio>
#include <cstring>
#include <stdint.h>
#include <string>
#include <vector>

namespace octomap
{
struct OcTreeNode
{
  float x, y, z;
};

class AbstractOcTree
{
public:
  virtual ~AbstractOcTree() {}
  static AbstractOcTree* read(const std::string& path);
};

class OcTree : public AbstractOcTree
{
public:
  explicit OcTree(double res) : res_(res) {}

  bool readBinary(const std::string& path)
  {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f)
      return false;
    char magic[8];
    uint64_t n = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "AMCLPTS1", 8) == 0 &&
              std::fread(&res_, sizeof(double), 1, f) == 1 && std::fread(min_, sizeof(double), 3, f) == 3 &&
              std::fread(max_, sizeof(double), 3, f) == 3 && std::fread(&n, sizeof(uint64_t), 1, f) == 1;
    if (ok)
    {
      nodes_.resize(n);
      std::vector<float> xyz(3 * n);
      ok = std::fread(xyz.data(), sizeof(float), 3 * n, f) == 3 * n;
      for (uint64_t i = 0; ok && i < n; ++i)
      {
        nodes_[i].x = xyz[3 * i];
        nodes_[i].y = xyz[3 * i + 1];
        nodes_[i].z = xyz[3 * i + 2];
      }
    }
    std::fclose(f);
    return ok;
  }

  size_t size() const { return nodes_.empty() ? 0 : nodes_.size() + 1; }
  double getResolution() const { return res_; }
  void getMetricMin(double& x, double& y, double& z) const
  {
    x = min_[0];
    y = min_[1];
    z = min_[2];
  }
  void getMetricMax(double& x, double& y, double& z) const
  {
    x = max_[0];
    y = max_[1];
    z = max_[2];
  }
  bool isNodeOccupied(const OcTreeNode&) const { return true; }

  class leaf_iterator
  {
  public:
    leaf_iterator(const std::vector<OcTreeNode>* v, size_t i) : v_(v), i_(i) {}
    leaf_iterator& operator++()
    {
      ++i_;
      return *this;
    }
    bool operator!=(const leaf_iterator& o) const { return i_ != o.i_; }
    bool operator!=(std::nullptr_t) const { return true; }
    const OcTreeNode& operator*() const { return (*v_)[i_]; }
    double getX() const { return (*v_)[i_].x; }
    double getY() const { return (*v_)[i_].y; }
    double getZ() const { return (*v_)[i_].z; }

  private:
    const std::vector<OcTreeNode>* v_;
    size_t i_;
  };
  leaf_iterator begin_leafs() const { return leaf_iterator(&nodes_, 0); }
  leaf_iterator end_leafs() const { return leaf_iterator(&nodes_, nodes_.size()); }

private:
  double res_;
  double min_[3]{ 0, 0, 0 };
  double max_[3]{ 0, 0, 0 };
  std::vector<OcTreeNode> nodes_;
};

inline AbstractOcTree* AbstractOcTree::read(const std::string& path)
{
  OcTree* t = new OcTree(0.1);
  if (!t->readBinary(path))
  {
    delete t;
    return nullptr;
  }
  return t;
}
}  // namespace octomap
