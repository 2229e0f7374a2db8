// Drives the drop-in amcl3d::Grid3d / amcl3d::ParticleFilter the way amcl3d::Node
// does (Node.cpp:41-53 open + slice + map cloud, :387 init, :154 predict,
// :130-137 voxel filter, :162 update, :167 getMean, :181 resample,
// :104 buildParticlesPoseMsg) and dumps
// what the Python test compares with the oracle.
//
// usage: dropin_check <map.bt> <scan.f32 (n x 4 floats)> <ranges.f32 (b x 4)> <out dir>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "ParticleFilter.h"
#include "VoxelGrid.h"

using namespace amcl3d;

static std::vector<float> read_f32(const std::string& path)
{
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  const std::streamsize n = f.tellg();
  f.seekg(0);
  std::vector<float> v(static_cast<size_t>(n) / 4);
  f.read(reinterpret_cast<char*>(v.data()), n);
  return v;
}

static void write_particles(const std::string& path, const std::vector<Particle>& p)
{
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(p.data()), static_cast<std::streamsize>(p.size() * sizeof(Particle)));
}

int main(int argc, char** argv)
{
  if (argc != 5)
    return 2;
  const std::string map = argv[1], out = argv[4];
  const std::vector<float> s = read_f32(argv[2]), r = read_f32(argv[3]);
  pcl::PointCloud<pcl::PointXYZ>::Ptr cloud(new pcl::PointCloud<pcl::PointXYZ>());
  for (size_t i = 0; i + 4 <= s.size(); i += 4)
    cloud->push_back(pcl::PointXYZ(s[i], s[i + 1], s[i + 2]));
  std::vector<Range> ranges;
  for (size_t i = 0; i + 4 <= r.size(); i += 4)
    ranges.push_back(Range(r[i], r[i + 1], r[i + 2], r[i + 3]));

  Grid3d bad;
  std::printf("open_short %d\n", bad.open(".bt", 0.05) ? 1 : 0);
  std::printf("open_missing %d\n", bad.open(map + ".missing.bt", 0.05) ? 1 : 0);
  std::printf("weight_unopened %.9g\n", bad.computeCloudWeight(cloud, 1, 1, 1, 0, 0, 0));

  Grid3d grid;
  std::printf("open %d\n", grid.open(map, 0.05) ? 1 : 0);
  Grid3d cached;
  std::printf("open_cached %d\n", cached.open(map, 0.05) ? 1 : 0);
  nav_msgs::OccupancyGrid slice;
  std::printf("slice %d %u %u %zu\n", grid.buildGridSliceMsg(1.0, slice) ? 1 : 0, slice.info.width,
              slice.info.height, slice.data.size());
  sensor_msgs::PointCloud2 pc;
  std::printf("mapcloud %d %u\n", grid.buildMapPointCloudMsg(pc) ? 1 : 0, pc.width);
  std::printf("into %d %d\n", grid.isIntoMap(1, 1, 1) ? 1 : 0, grid.isIntoMap(-100, -100, -100) ? 1 : 0);

  ParticleFilter pf(42);
  std::printf("initialized_before %d\n", pf.isInitialized() ? 1 : 0);
  pf.init(600, 2.5f, 2.0f, 1.2f, 0.3f, 0.05f, 0.05f, 0.05f, 0.1f);
  const Particle m0 = pf.getMean();
  std::printf("init_mean %.9g %.9g %.9g %.9g %d\n", m0.x, m0.y, m0.z, m0.a, pf.isInitialized() ? 1 : 0);
  pf.predict(0.1, 0.1, 0.01, 0.3, 0.05, 0.0, 0.0, 0.01);
  write_particles(out + "/before_update.bin", pf.particles());
  pf.update(grid, cloud, ranges, 0.5, 0.1, 0.0, 0.0);
  const Particle m = pf.getMean();
  std::printf("mean %.9g %.9g %.9g %.9g\n", m.x, m.y, m.z, m.a);
  write_particles(out + "/after_update.bin", pf.particles());
  pf.resample();
  geometry_msgs::PoseArray msg;
  pf.buildParticlesPoseMsg(msg);
  std::printf("poses %zu %.9g\n", msg.poses.size(), msg.poses.empty() ? 0.0 : msg.poses[0].orientation.w);
  std::printf("weight %.9g\n", grid.computeCloudWeight(cloud, 2.5f, 2.0f, 1.2f, 0.0f, 0.0f, 0.3f));
  std::vector<Range> none;
  pf.update(none, 0.5, 0.1);  // range-only overload, no ranges: every weight 0
  std::printf("ranges_only_mean %.9g\n", pf.getMean().x);

  // Node.cpp:130-137: the scan filter, with the node's call sequence
  VoxelGrid sor;
  sor.setInputCloud(cloud);
  sor.setLeafSize(0.1f, 0.1f, 0.1f);
  pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_down(new pcl::PointCloud<pcl::PointXYZ>);
  sor.filter(*cloud_down);
  std::printf("voxel %zu %u\n", cloud_down->points.size(), cloud_down->width);
  {
    std::ofstream f(out + "/voxel.bin", std::ios::binary);
    for (const auto& p : cloud_down->points)
      f.write(reinterpret_cast<const char*>(&p.x), 3 * sizeof(float));
  }
  return 0;
}
